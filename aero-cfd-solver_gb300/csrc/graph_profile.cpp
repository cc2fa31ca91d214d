// graph_profile.cpp -- in-graph kernel times of the timed iterations (aero_profile_graph).
//
// The iterations run exactly as aero_time_iterations runs them (the same CUDA graphs, the
// controller on its side stream), while the CUPTI activity API records the start and end of
// every kernel the GPU executes, graph kernel nodes included, without serialising them.
// CUPTI is loaded at run time: the library itself does not depend on it, and without it
// aero_profile_graph reports AERO_ERR_STATE.
#include "../../include/aero_gb300.h"
#include "ctx.hpp"
#include "engine.hpp"

#include <cupti_activity.h>
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <cstdlib>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

namespace aero {
namespace {

struct CuptiApi {
  CUptiResult (*enable)(CUpti_ActivityKind) = nullptr;
  CUptiResult (*disable)(CUpti_ActivityKind) = nullptr;
  CUptiResult (*register_callbacks)(CUpti_BuffersCallbackRequestFunc, CUpti_BuffersCallbackCompleteFunc) = nullptr;
  CUptiResult (*flush_all)(uint32_t) = nullptr;
  CUptiResult (*next_record)(uint8_t*, size_t, CUpti_Activity**) = nullptr;
  bool ok = false;
};

const CuptiApi& cupti() {
  static const CuptiApi api = [] {
    CuptiApi a;
    const char* names[] = {"libcupti.so.13", "libcupti.so", "/usr/local/cuda/lib64/libcupti.so.13",
                           "/usr/local/cuda/extras/CUPTI/lib64/libcupti.so.13"};
    void* h = nullptr;
    for (const char* n : names) {
      h = dlopen(n, RTLD_NOW | RTLD_LOCAL);
      if (h) break;
    }
    if (!h) return a;
    a.enable = reinterpret_cast<decltype(a.enable)>(dlsym(h, "cuptiActivityEnable"));
    a.disable = reinterpret_cast<decltype(a.disable)>(dlsym(h, "cuptiActivityDisable"));
    a.register_callbacks =
        reinterpret_cast<decltype(a.register_callbacks)>(dlsym(h, "cuptiActivityRegisterCallbacks"));
    a.flush_all = reinterpret_cast<decltype(a.flush_all)>(dlsym(h, "cuptiActivityFlushAll"));
    a.next_record = reinterpret_cast<decltype(a.next_record)>(dlsym(h, "cuptiActivityGetNextRecord"));
    a.ok = a.enable && a.disable && a.register_callbacks && a.flush_all && a.next_record;
    return a;
  }();
  return api;
}

struct Span {
  int cls;
  uint64_t start, end;
};
std::mutex g_mu;       // the collected spans
std::mutex g_session;  // one profiling session at a time (CUPTI activity is process-wide)
std::vector<Span> g_spans;
bool g_registered = false;

int fail(aero_ctx* ctx, int code, const char* msg) {
  if (ctx) ctx->error = msg;
  return code;
}

// kernel class of a kernel name (the classes of aero_profile_kernels); -1: not ours
int kernel_class(const char* name) {
  if (name == nullptr) return -1;
  static const std::pair<const char*, int> table[] = {
      {"k_gradient", 0}, {"k_face_flux", 1}, {"k_gather", 1}, {"k_update", 2},
      {"k_srmax", 3},    {"k_symmetry", 4},  {"k_pjump", 4},  {"k_control", 5}};
  for (const auto& t : table) {
    if (std::strstr(name, t.first)) return t.second;
  }
  return -1;
}

void CUPTIAPI buffer_requested(uint8_t** buffer, size_t* size, size_t* max_records) {
  *size = size_t(8) << 20;
  *buffer = static_cast<uint8_t*>(std::aligned_alloc(8, *size));
  *max_records = 0;
}

void CUPTIAPI buffer_completed(CUcontext, uint32_t, uint8_t* buffer, size_t, size_t valid) {
  const CuptiApi& api = cupti();
  CUpti_Activity* rec = nullptr;
  std::lock_guard<std::mutex> lock(g_mu);
  while (valid > 0 && api.next_record(buffer, valid, &rec) == CUPTI_SUCCESS) {
    if (rec->kind == CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL || rec->kind == CUPTI_ACTIVITY_KIND_KERNEL) {
      const auto* k = reinterpret_cast<const CUpti_ActivityKernel10*>(rec);
      const int cls = kernel_class(k->name);
      if (cls >= 0) g_spans.push_back(Span{cls, k->start, k->end});
    }
  }
  std::free(buffer);
}

}  // namespace
}  // namespace aero

extern "C" {

int aero_profile_graph(aero_ctx* ctx, int n, int flush_l2, double* ms, int* launches, double* iteration_ms) {
  if (ctx == nullptr || n <= 0 || ms == nullptr || launches == nullptr || iteration_ms == nullptr)
    return aero::fail(ctx, AERO_ERR_INVALID, "aero_profile_graph: bad argument");
  const aero::CuptiApi& api = aero::cupti();
  if (!api.ok) return aero::fail(ctx, AERO_ERR_STATE, "aero_profile_graph: the CUPTI library is not available");
  std::lock_guard<std::mutex> session(aero::g_session);
  {
    std::lock_guard<std::mutex> lock(aero::g_mu);
    aero::g_spans.clear();
  }
  if (!aero::g_registered) {
    if (api.register_callbacks(aero::buffer_requested, aero::buffer_completed) != CUPTI_SUCCESS)
      return aero::fail(ctx, AERO_ERR_STATE, "aero_profile_graph: CUPTI refused the activity buffers");
    aero::g_registered = true;
  }
  if (api.enable(CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL) != CUPTI_SUCCESS)
    return aero::fail(ctx, AERO_ERR_STATE, "aero_profile_graph: CUPTI kernel activity could not be enabled");
  double total = 0.0;
  const int rc = ctx->engine->time_iterations(n, 1, flush_l2, &total);
  cudaDeviceSynchronize();
  api.flush_all(1);
  api.disable(CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL);
  api.flush_all(1);
  if (rc != AERO_OK) return aero::fail(ctx, rc, "aero_profile_graph: the timed iterations failed");
  for (int k = 0; k < 6; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  {
    std::lock_guard<std::mutex> lock(aero::g_mu);
    for (const auto& s : aero::g_spans) {
      ms[s.cls] += static_cast<double>(s.end - s.start) * 1e-6;
      ++launches[s.cls];
    }
    aero::g_spans.clear();
  }
  *iteration_ms = total;
  return AERO_OK;
}

}  // extern "C"
