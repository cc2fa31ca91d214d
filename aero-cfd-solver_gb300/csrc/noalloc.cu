// noalloc.cu -- aero_residual_noalloc: one residual evaluation on caller-owned device buffers
// that allocates nothing. Its working arrays live in a file-scope __device__ array of fixed
// size instead of memory obtained from cudaMalloc.
//
// Who needs this: code that evaluates the residual where device allocation is not allowed or
// not wanted -- under another framework's memory pool that owns all device memory, or in a
// time-stepping loop whose memory budget is fixed up front (cudaMalloc/cudaFree can
// synchronise the device and fragment memory).
//
// Limits and sharing: the scratch array is sized for kNoallocMaxCells cells and
// kNoallocMaxFaces faces (about 16.8 MB); every CUDA context that loads this library (one per
// GPU for the runtime's primary context) holds its own copy until the process exits. All
// calls made in one context share that copy and it keeps the last call's contents; the
// kernels clear what must start at zero. Two calls whose work overlaps on the GPU in the
// same context (different streams) race on the shared array and must be ordered by the caller.
#include "aero_face_kernels.cuh"
#include "ctx.hpp"

#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <utility>
#include <vector>

namespace aero {
namespace {

constexpr int kNoallocMaxCells = 65536;
constexpr int kNoallocMaxFaces = 3 * 65536;
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kCtrlBytes = align_up(sizeof(Ctrl));
// sized for double: per cell W, gx, gy, R (4 reals each) and SR; per face F (4 reals) and FS
constexpr size_t kScratchBytes = kCtrlBytes + 4 * align_up(size_t(kNoallocMaxCells) * 32) +
                                 align_up(size_t(kNoallocMaxCells) * 8) + align_up(size_t(kNoallocMaxFaces) * 32) +
                                 align_up(size_t(kNoallocMaxFaces) * 8);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The array's device address is looked up once per CUDA context, at the first call made in
// that context, and cached under the context's ID (unique for the life of the process, so a
// context created after cudaDeviceReset, or another context on the same device, gets its own
// lookup). The driver calls that name the current context are fetched through the runtime,
// so the library needs no link to the driver library.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct DriverCalls {
  CtxGetCurrentFn get_current = nullptr;
  CtxGetIdFn get_id = nullptr;
};

const DriverCalls& driver_calls() {
  static const DriverCalls calls = [] {
    DriverCalls d;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      d.get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      d.get_id = reinterpret_cast<CtxGetIdFn>(f);
    cudaGetLastError();
    return d;
  }();
  return calls;
}

// ID of the context the runtime uses on this thread (0 when none is current).
unsigned long long current_context_id() {
  const DriverCalls& d = driver_calls();
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (d.get_current == nullptr || d.get_id == nullptr || d.get_current(&c) != CUDA_SUCCESS || c == nullptr) return 0;
  return d.get_id(c, &id) == CUDA_SUCCESS ? id : 0;
}

std::mutex g_scratch_mu;
std::vector<std::pair<unsigned long long, void*>> g_scratch_addr;  // (context ID, address)

// Device address of the scratch array in the current context (the context's device must be
// current). The host-side name g_noalloc_scratch is only a stand-in; kernels must be given
// this address.
cudaError_t scratch_address(void** out) {
  unsigned long long id = current_context_id();
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (id != 0) {
    for (const auto& e : g_scratch_addr) {
      if (e.first == id) {
        *out = e.second;
        return cudaSuccess;
      }
    }
  }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  if (id == 0) id = current_context_id();  // the lookup above made the runtime's context current
  if (id != 0) g_scratch_addr.emplace_back(id, p);
  *out = p;
  return cudaSuccess;
}

// Gathers the caller's state (original order, AoS [N][5] double) into the bulk primitive
// state and resets the per-call fields of the scratch controller block.
template <class T>
__global__ void k_na_prepare(int n, const int* __restrict__ perm, const double* __restrict__ u,
                             typename Vec<T>::v4* __restrict__ W, double gamma, Ctrl* __restrict__ ctrl,
                             double stab, int as_fix, double as_fmin, double as_ramp) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c == 0) {
    ctrl->done = 0;
    ctrl->fo_fallback = 0;
    ctrl->diff_fallback = 0;
    set_eval_schedule(ctrl, stab, as_fix, as_fmin, as_ramp);
    ctrl->sr_max = 0.0;
  }
  if (c >= n) return;
  const double* s = u + 5 * static_cast<size_t>(perm[c]);
  const Prim<T> w = cons_to_prim(Cons<T>{T(s[0]), T(s[1]), T(s[2]), T(s[4])}, T(gamma));
  typename Vec<T>::v4 o;
  o.x = w.r; o.y = w.u; o.z = w.v; o.w = w.p;
  W[c] = o;
}

// Scatters the residual and spectral radius back to the caller's original order.
template <class T>
__global__ void k_na_store(int n, const int* __restrict__ perm, const typename Vec<T>::v4* __restrict__ R,
                           const T* __restrict__ SR, double* __restrict__ res, double* __restrict__ sr) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int o = perm[c];
  const auto r = R[c];
  double* d = res + 5 * static_cast<size_t>(o);
  d[0] = double(r.x);
  d[1] = double(r.y);
  d[2] = double(r.z);
  d[3] = 0.0;
  d[4] = double(r.w);
  sr[o] = double(SR[c]);
}

template <class T>
cudaError_t run_na(const EngineView& v, unsigned char* base, const double* u, int second, double stab,
                   int as_fix, double as_fmin, double as_ramp, double* res, double* sr, cudaStream_t st) {
  using V4 = typename Vec<T>::v4;
  const DevMesh<T>& dm = *static_cast<const DevMesh<T>*>(v.dm);
  const int n = v.n, ntot = v.ntot;
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(base);
  unsigned char* p = base + kCtrlBytes;
  auto take = [&](size_t bytes) {
    unsigned char* q = p;
    p += align_up(bytes);
    return q;
  };
  V4* W = reinterpret_cast<V4*>(take(sizeof(V4) * ntot));
  V4* gx = reinterpret_cast<V4*>(take(sizeof(V4) * ntot));
  V4* gy = reinterpret_cast<V4*>(take(sizeof(V4) * ntot));
  V4* R = reinterpret_cast<V4*>(take(sizeof(V4) * ntot));
  T* SR = reinterpret_cast<T*>(take(sizeof(T) * ntot));
  V4* F = reinterpret_cast<V4*>(take(sizeof(V4) * v.nf));
  T* FS = reinterpret_cast<T*>(take(sizeof(T) * v.nf));
  const int block = v.block;
  const FaceParams<T>* fps = static_cast<const FaceParams<T>*>(v.fps);
  const PrecondD* pcs = static_cast<const PrecondD*>(v.pcs);
  const MonitorConsts* mcs = static_cast<const MonitorConsts*>(v.mcs);
  const Cases<T> cells{v.cblk, ctrl, fps, pcs, mcs};
  const Cases<T> faces{v.fblk, ctrl, fps, pcs, mcs};
  k_na_prepare<T><<<v.cblocks, block, 0, st>>>(n, v.perm_dev, u, W, v.gamma, ctrl, stab, as_fix, as_fmin, as_ramp);
  if (second) k_gradient<T><<<v.cblocks, block, 0, st>>>(dm, W, gx, gy, cells);
  ResidualLaunch<T> a;
  a.block = block;
  a.st = st;
  a.faces = *static_cast<const DevFaces<T>*>(v.df);
  a.gather = *static_cast<const DevGather<T>*>(v.dg);
  a.face_cases = faces;
  a.cell_cases = cells;
  a.W = W;
  a.gx = gx;
  a.gy = gy;
  a.F = F;
  a.FS = FS;
  a.R = R;
  a.SR = SR;
  a.part = Partials{};
  a.fb = &ctrl->fo_fallback;
  a.global_dt = 0;
  launch_residual_passes(a, v.flux, second != 0, v.lm != 0, false);
  k_na_store<T><<<v.cblocks, block, 0, st>>>(n, v.perm_dev, R, SR, res, sr);
  return cudaGetLastError();
}

}  // namespace
}  // namespace aero

extern "C" {

int aero_residual_noalloc(aero_ctx* ctx, const double* conserved_dev, int second_order, double stab_mach_floor,
                          int all_speed_flux_fix, double all_speed_f_min, double all_speed_ramp_weight,
                          double* residual_dev, double* spectral_radius_dev, void* stream) {
  if (ctx == nullptr) return AERO_ERR_INVALID;
  if (conserved_dev == nullptr || residual_dev == nullptr || spectral_radius_dev == nullptr) {
    ctx->error = "aero_residual_noalloc: null device pointer";
    return AERO_ERR_INVALID;
  }
  const aero::EngineView v = ctx->engine->view();
  if (ctx->engine->n_cases() != 1) {
    ctx->error = "aero_residual_noalloc: batched context";
    return AERO_ERR_INVALID;
  }
  if (v.ntot > aero::kNoallocMaxCells || v.nf > aero::kNoallocMaxFaces) {
    ctx->error = "aero_residual_noalloc: the mesh has " + std::to_string(v.n) + " cells and " +
                 std::to_string(v.nf) + " faces; the allocation-free residual supports at most " +
                 std::to_string(aero::kNoallocMaxCells) + " cells and " +
                 std::to_string(aero::kNoallocMaxFaces) + " faces";
    return AERO_ERR_INVALID;
  }
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) {
    cudaGetLastError();
    ctx->error = "aero_residual_noalloc: no current CUDA device";
    return AERO_ERR_CUDA;
  }
  if (prev != ctx->device && cudaSetDevice(ctx->device) != cudaSuccess) {
    cudaGetLastError();
    ctx->error = "aero_residual_noalloc: cannot select the context's device";
    return AERO_ERR_CUDA;
  }
  void* base = nullptr;
  cudaError_t e = aero::scratch_address(&base);
  if (e == cudaSuccess) {
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : v.stream;
    unsigned char* b = static_cast<unsigned char*>(base);
    e = v.precision == AERO_PRECISION_FP32
            ? aero::run_na<float>(v, b, conserved_dev, second_order, stab_mach_floor, all_speed_flux_fix,
                                  all_speed_f_min, all_speed_ramp_weight, residual_dev, spectral_radius_dev, st)
            : aero::run_na<double>(v, b, conserved_dev, second_order, stab_mach_floor, all_speed_flux_fix,
                                   all_speed_f_min, all_speed_ramp_weight, residual_dev, spectral_radius_dev, st);
  }
  if (prev != ctx->device) cudaSetDevice(prev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ctx->error = std::string("aero_residual_noalloc: ") + cudaGetErrorString(e);
    return AERO_ERR_CUDA;
  }
  return AERO_OK;
}

}  // extern "C"
