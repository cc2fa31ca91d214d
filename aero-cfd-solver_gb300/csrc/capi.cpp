// capi.cpp -- extern "C" entry points of libaero_gb300.so (include/aero_gb300.h).
#include "../../include/aero_adjoint.h"
#include "../../include/aero_batch.h"
#include "../../include/aero_gb300.h"
#include "../../include/aero_mesh.h"
#include "engine.hpp"
#include "mesh_prep.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <new>
#include <string>

#include "ctx.hpp"

namespace {

thread_local std::string g_error;

int fail(aero_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->error = msg;
  g_error = msg;
  return code;
}

int cuda_status(aero_ctx* ctx) {
  const cudaError_t e = ctx->engine->last_cuda_error();
  if (e == cudaSuccess) return AERO_OK;
  return fail(ctx, e == cudaErrorMemoryAllocation ? AERO_ERR_NOMEM : AERO_ERR_CUDA,
              std::string("CUDA error: ") + cudaGetErrorString(e));
}

// Host resolution of the case (euler_solver.cpp:340-357, 120-140, 493-526, 543-566).
aero::Resolved resolve(const aero_case_desc& c) {
  aero::Resolved r{};
  const double pi = 3.14159265358979323846;
  const double gamma = c.gamma;
  double rho_inf = c.rho_inf;
  if (rho_inf <= 0.0) rho_inf = c.p_inf / (c.gas_constant * c.t_inf);
  const double alpha = c.aoa_deg * (pi / 180.0);
  const double a_inf = std::sqrt(gamma * c.p_inf / rho_inf);
  const double v_inf = std::max(c.mach, 0.0) * a_inf;
  const double u = v_inf * std::cos(alpha), v = v_inf * std::sin(alpha);
  // primitive_to_conservative (euler_flux.cpp:101-113)
  const double rho = std::max(rho_inf, 1.0e-8);
  const double ke = 0.5 * rho * (u * u + v * v);
  const double p = std::max(c.p_inf, 1.0e-8);
  r.gamma = gamma;
  r.cons_inf[0] = rho;
  r.cons_inf[1] = rho * u;
  r.cons_inf[2] = rho * v;
  r.cons_inf[3] = p / (gamma - 1.0) + ke;
  r.p_inf = c.p_inf;
  r.rho_inf = rho_inf;
  r.v_inf = v_inf;
  r.a_inf = a_inf;
  r.q_inf = 0.5 * rho_inf * v_inf * v_inf + 1.0e-12;
  r.pressure_ref = std::max(rho_inf * a_inf * a_inf, 1.0e-12);
  r.cos_a = std::cos(alpha);
  r.sin_a = std::sin(alpha);
  const double minf = std::max(c.mach, 1.0e-4);
  const double auto_bmin = std::max(1.0e-4, std::min(1.0e-3, 0.1 * minf));
  r.pc_mach_ref = std::max(c.precond_mach_ref > 0.0 ? c.precond_mach_ref : minf, 1.0e-4);
  r.pc_mach_min = std::max(c.precond_mach_min > 0.0 ? c.precond_mach_min : 1.0e-6, 1.0e-6);
  r.pc_beta_min = std::max(c.precond_beta_min > 0.0 ? c.precond_beta_min : auto_bmin, 1.0e-4);
  r.pc_beta_max = std::max(c.precond_beta_max, r.pc_beta_min);
  const double ks = c.stab_floor_k_start >= 0.0 ? c.stab_floor_k_start : c.stab_floor_start / minf;
  const double kt = c.stab_floor_k_target >= 0.0 ? c.stab_floor_k_target : c.stab_floor_target / minf;
  r.stab_start = std::clamp(std::max(ks, 0.0) * minf, 0.0, 1.0);
  r.stab_target = std::clamp(std::max(kt, 0.0) * minf, 0.0, 1.0);
  r.as_fmin = std::clamp(c.all_speed_f_min, 1.0e-6, 1.0);
  r.st_fmin_high = std::clamp(c.all_speed_stage_f_min_high, 1.0e-6, 1.0);
  r.st_fmin_mid = std::clamp(std::min(c.all_speed_stage_f_min_mid, r.st_fmin_high), 1.0e-6, 1.0);
  r.st_fmin_low = std::clamp(std::min(c.all_speed_stage_f_min_low, r.st_fmin_mid), 1.0e-6, 1.0);
  const double autopj = std::clamp(1.6e-2 * minf * minf * minf * minf, 1.0e-9, 2.0e-6);
  r.pj_target = c.all_speed_pjump_wall_target <= 0.0 ? autopj : c.all_speed_pjump_wall_target;
  r.pj_spike = std::max(c.all_speed_pjump_spike_factor, 1.0);
  r.cfl_drop = std::clamp(c.all_speed_cfl_drop_factor, 0.05, 1.0);
  r.cfl_restore = std::clamp(c.all_speed_cfl_restore_factor, 1.0, 1.2);
  r.cfl_min_scale = std::clamp(c.all_speed_cfl_min_scale, 0.01, 1.0);
  r.lm = (c.precond_on || c.low_mach_fix || c.all_speed_flux_fix) ? 1 : 0;
  return r;
}

bool device_ok(int dev) {
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return false;
  return prop.major == 10 && prop.minor == 3;
}

}  // namespace

extern "C" {

int aero_abi_version(void) { return AERO_ABI_VERSION; }

const char* aero_version(void) { return "0.1.0-gb300"; }

int aero_cuda_available(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  for (int i = 0; i < n; ++i) {
    if (device_ok(i)) return 1;
  }
  return 0;
}

void aero_case_defaults(aero_case_desc* c) {
  if (c == nullptr) return;
  std::memset(c, 0, sizeof(*c));
  auto f = [](float x) { return static_cast<double>(x); };
  c->gamma = f(1.4f);
  c->gas_constant = f(287.05f);
  c->mach = f(0.15f);
  c->aoa_deg = f(2.0f);
  c->p_inf = f(101325.0f);
  c->t_inf = f(288.15f);
  c->rho_inf = 0.0;
  c->chord = 1.0;
  c->x_ref = f(0.25f);
  c->y_ref = 0.0;
  c->flux = AERO_FLUX_RUSANOV;
  c->limiter = AERO_LIMITER_MINMOD;
  c->iterations = 400;
  c->min_iterations = 40;
  c->cfl_ramp_iters = 120;
  c->cfl_start = f(0.2f);
  c->cfl_max = f(1.2f);
  c->residual_reduction_target = f(1.0e-3f);
  c->force_stability_tol = f(2.0e-5f);
  c->force_mean_drift_tol = f(2.0e-5f);
  c->force_stability_window = 6;
  c->startup_first_order_iters = 25;
  c->rk_stages = 3;
  c->local_time_stepping = 1;
  c->precond_on = 0;
  c->precond_mach_ref = f(0.15f);
  c->precond_mach_min = f(1.0e-3f);
  c->precond_beta_min = f(0.2f);
  c->precond_beta_max = 1.0;
  c->precond_farfield_bc = 0;
  c->stab_floor_start = f(0.1f);
  c->stab_floor_target = f(0.02f);
  c->stab_floor_k_start = -1.0;
  c->stab_floor_k_target = -1.0;
  c->stab_ramp_iters = 400;
  c->low_mach_fix = 0;
  c->mach_cutoff = f(0.3f);
  c->all_speed_flux_fix = 0;
  c->all_speed_mach_cutoff = f(0.25f);
  c->all_speed_f_min = f(0.05f);
  c->all_speed_ramp_start_iter = 0;
  c->all_speed_ramp_iters = 0;
  c->all_speed_staged_controller = 0;
  c->all_speed_stage_a_min_iters = 600;
  c->all_speed_stage_a_max_iters = 0;
  c->all_speed_stage_f_min_high = f(0.2f);
  c->all_speed_stage_f_min_mid = f(0.1f);
  c->all_speed_stage_f_min_low = f(0.05f);
  c->all_speed_pjump_wall_target = 0.0;
  c->all_speed_pjump_spike_factor = f(1.5f);
  c->all_speed_pjump_hold_iters = 120;
  c->all_speed_freeze_iters = 120;
  c->all_speed_cfl_drop_factor = f(0.8f);
  c->all_speed_cfl_restore_factor = f(1.02f);
  c->all_speed_cfl_min_scale = f(0.1f);
  c->aoa0_symmetry_enforce = 0;
  c->aoa0_symmetry_enforce_interval = 0;
  c->precision = AERO_PRECISION_FP64;
  c->ordering = AERO_ORDER_MORTON;
  c->block_size = 0;
  c->diagnostics = 0;
  c->density_l2_target = 0.0;
  c->cells_per_thread = 0;
  c->precond_fp64 = 0;
}

}  // extern "C"

namespace {

int check_case(const aero_case_desc* cfg) {
  if (cfg->rk_stages != 1 && cfg->rk_stages != 3)
    return fail(nullptr, AERO_ERR_INVALID, "Euler pseudo-time rk_stages must be 1 or 3.");
  if (cfg->flux != AERO_FLUX_RUSANOV && cfg->flux != AERO_FLUX_HLLC)
    return fail(nullptr, AERO_ERR_INVALID, "unknown flux scheme");
  if (cfg->limiter != AERO_LIMITER_MINMOD && cfg->limiter != AERO_LIMITER_VENKAT)
    return fail(nullptr, AERO_ERR_INVALID, "unknown limiter");
  if (cfg->precision != AERO_PRECISION_FP64 && cfg->precision != AERO_PRECISION_FP32)
    return fail(nullptr, AERO_ERR_INVALID, "unknown precision");
  if (cfg->precond_fp64 < -1 || cfg->precond_fp64 > 2)
    return fail(nullptr, AERO_ERR_INVALID, "precond_fp64 must be -1, 0, 1 or 2");
  double rho_inf = cfg->rho_inf;
  if (rho_inf <= 0.0) rho_inf = cfg->p_inf / (cfg->gas_constant * cfg->t_inf);
  if (!(rho_inf > 0.0))
    return fail(nullptr, AERO_ERR_INVALID, "Invalid freestream density. Set rho_inf or p_inf/T_inf.");
  return AERO_OK;
}

// One context over n cases (n = 1: aero_create).
int create_ctx(int n, const aero_mesh_desc* meshes, const aero_case_desc* cfgs, aero_ctx** out) {
  if (out == nullptr || meshes == nullptr || cfgs == nullptr || n < 1)
    return fail(nullptr, AERO_ERR_INVALID, "aero_create: null argument");
  *out = nullptr;
  for (int k = 0; k < n; ++k) {
    const int rc = check_case(&cfgs[k]);
    if (rc != AERO_OK) return rc;
  }
  try {
    std::unique_ptr<aero_ctx> ctx(new aero_ctx());
    ctx->cfg = cfgs[0];
    // the meshes are checked and prepared on the host first, so that an invalid mesh is
    // reported as such on any machine
    std::vector<aero::HostSlots> hv(static_cast<size_t>(n));
    std::vector<aero_case_desc> cv(cfgs, cfgs + n);
    std::vector<aero::Resolved> rv;
    std::string err;
    for (int k = 0; k < n; ++k) {
      if (!aero::build_slots(meshes[k], cfgs[k].ordering, &hv[k], &err)) {
        return fail(nullptr, AERO_ERR_INVALID, n > 1 ? "case " + std::to_string(k) + ": " + err : err);
      }
      rv.push_back(resolve(cfgs[k]));
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || !device_ok(dev)) {
      cudaGetLastError();
      return fail(nullptr, AERO_ERR_CUDA, "no usable CUDA device of compute capability 10.3");
    }
    ctx->device = dev;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      return fail(nullptr, AERO_ERR_CUDA, "cudaStreamCreate failed");
    }
    aero::Engine* e = cfgs[0].precision == AERO_PRECISION_FP32 ? aero::make_engine_f32(hv, cv, rv, ctx->stream)
                                                               : aero::make_engine_f64(hv, cv, rv, ctx->stream);
    ctx->engine.reset(e);
    if (!e->init(&err)) {
      ctx->engine.reset();
      cudaStreamDestroy(ctx->stream);
      ctx->stream = nullptr;
      const int code = err.find("allocation") != std::string::npos ? AERO_ERR_NOMEM
                       : err.find("must share") != std::string::npos ? AERO_ERR_INVALID
                                                                      : AERO_ERR_CUDA;
      return fail(nullptr, code, err);
    }
    *out = ctx.release();
    return AERO_OK;
  } catch (const std::bad_alloc&) {
    return fail(nullptr, AERO_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception& ex) {
    return fail(nullptr, AERO_ERR_CUDA, ex.what());
  }
}

}  // namespace

extern "C" {

int aero_create(const aero_mesh_desc* mesh, const aero_case_desc* cfg, aero_ctx** out) {
  return create_ctx(1, mesh, cfg, out);
}

int aero_batch_create(int n_cases, const aero_mesh_desc* meshes, const aero_case_desc* cases, aero_ctx** out) {
  return create_ctx(n_cases, meshes, cases, out);
}

int aero_batch_size(const aero_ctx* ctx) { return ctx ? ctx->engine->n_cases() : 0; }

int aero_batch_run(aero_ctx* ctx, int n, aero_iter_record* records, int* n_done) {
  if (ctx == nullptr || n < 0) return fail(ctx, AERO_ERR_INVALID, "aero_batch_run: bad argument");
  const int rc = ctx->engine->run(n, records, n_done);
  const int cs = cuda_status(ctx);
  if (cs != AERO_OK) return cs;
  if (rc == AERO_ERR_NONFINITE) return fail(ctx, rc, "non-finite state trapped in a case");
  return rc;
}

int aero_batch_set_state(aero_ctx* ctx, int case_index, const double* conserved) {
  if (ctx == nullptr || conserved == nullptr || case_index < 0 || case_index >= ctx->engine->n_cases())
    return fail(ctx, AERO_ERR_INVALID, "aero_batch_set_state: bad argument");
  ctx->engine->set_state(case_index, conserved);
  return cuda_status(ctx);
}

int aero_batch_get_state(aero_ctx* ctx, int case_index, double* conserved) {
  if (ctx == nullptr || conserved == nullptr || case_index < 0 || case_index >= ctx->engine->n_cases())
    return fail(ctx, AERO_ERR_INVALID, "aero_batch_get_state: bad argument");
  ctx->engine->get_state(case_index, conserved);
  return cuda_status(ctx);
}

int aero_batch_get_last_residual(aero_ctx* ctx, int case_index, double* residual, double* spectral_radius) {
  if (ctx == nullptr || residual == nullptr || case_index < 0 || case_index >= ctx->engine->n_cases())
    return fail(ctx, AERO_ERR_INVALID, "aero_batch_get_last_residual: bad argument");
  ctx->engine->last_residual(case_index, residual, spectral_radius);
  return cuda_status(ctx);
}

void aero_destroy(aero_ctx* ctx) {
  if (ctx == nullptr) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->engine.reset();
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* aero_last_error(const aero_ctx* ctx) {
  if (ctx == nullptr) return g_error.c_str();
  return ctx->error.c_str();
}

int aero_set_state(aero_ctx* ctx, const double* conserved) {
  if (ctx == nullptr || conserved == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_set_state: null argument");
  ctx->engine->set_state(0, conserved);
  return cuda_status(ctx);
}

int aero_get_state(aero_ctx* ctx, double* conserved) {
  if (ctx == nullptr || conserved == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_get_state: null argument");
  ctx->engine->get_state(0, conserved);
  return cuda_status(ctx);
}

int aero_get_primitive(aero_ctx* ctx, double* rho, double* u, double* v, double* p) {
  if (ctx == nullptr || !rho || !u || !v || !p) return fail(ctx, AERO_ERR_INVALID, "aero_get_primitive: null argument");
  ctx->engine->get_primitive(0, rho, u, v, p);
  return cuda_status(ctx);
}

int aero_residual(aero_ctx* ctx, const double* conserved, int second_order, double stab_mach_floor,
                  int all_speed_flux_fix, double all_speed_f_min, double all_speed_ramp_weight,
                  double* residual, double* spectral_radius, double* gradients) {
  if (ctx == nullptr || conserved == nullptr || residual == nullptr || spectral_radius == nullptr)
    return fail(ctx, AERO_ERR_INVALID, "aero_residual: null argument");
  if (ctx->engine->n_cases() != 1) return fail(ctx, AERO_ERR_INVALID, "aero_residual: batched context");
  ctx->engine->residual(conserved, second_order, stab_mach_floor, all_speed_flux_fix, all_speed_f_min,
                        all_speed_ramp_weight, residual, spectral_radius, gradients);
  return cuda_status(ctx);
}

int aero_run(aero_ctx* ctx, int n, aero_iter_record* records, int* n_done) {
  if (ctx == nullptr || n < 0) return fail(ctx, AERO_ERR_INVALID, "aero_run: bad argument");
  if (ctx->engine->n_cases() != 1) return fail(ctx, AERO_ERR_INVALID, "aero_run: batched context (use aero_batch_run)");
  const int rc = ctx->engine->run(n, records, n_done);
  const int cs = cuda_status(ctx);
  if (cs != AERO_OK) return cs;
  if (rc == AERO_ERR_NONFINITE) return fail(ctx, rc, "non-finite state trapped");
  return rc;
}

int aero_reset_run(aero_ctx* ctx) {
  if (ctx == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_reset_run: null context");
  ctx->engine->reset_run();
  return cuda_status(ctx);
}

int aero_get_last_residual(aero_ctx* ctx, double* residual, double* spectral_radius) {
  if (ctx == nullptr || residual == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_get_last_residual: null argument");
  ctx->engine->last_residual(0, residual, spectral_radius);
  return cuda_status(ctx);
}

int aero_time_iterations(aero_ctx* ctx, int n, int use_graph, int flush_l2, double* device_ms) {
  if (ctx == nullptr || n <= 0 || device_ms == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_time_iterations: bad argument");
  const int rc = ctx->engine->time_iterations(n, use_graph, flush_l2, device_ms);
  const int cs = cuda_status(ctx);
  return cs != AERO_OK ? cs : rc;
}

int aero_profile_kernels(aero_ctx* ctx, int n, int flush_l2, double* ms, int* launches) {
  if (ctx == nullptr || n <= 0 || ms == nullptr || launches == nullptr)
    return fail(ctx, AERO_ERR_INVALID, "aero_profile_kernels: bad argument");
  const int rc = ctx->engine->profile_kernels(n, flush_l2, ms, launches);
  const int cs = cuda_status(ctx);
  return cs != AERO_OK ? cs : rc;
}

int aero_select_device(int device) {
  if (!device_ok(device)) return fail(nullptr, AERO_ERR_CUDA, "device is not a usable compute capability 10.3 GPU");
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return fail(nullptr, AERO_ERR_CUDA, "cudaSetDevice failed");
  }
  return AERO_OK;
}

int aero_get_info(aero_ctx* ctx, long long* info, int n_info) {
  if (ctx == nullptr || info == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_get_info: null argument");
  ctx->engine->info(info, n_info);
  return AERO_OK;
}

int aero_set_wait_limit(aero_ctx* ctx, int polls) {
  if (ctx == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_set_wait_limit: null context");
  const int rc = ctx->engine->set_wait_limit(polls);
  const int cs = cuda_status(ctx);
  return cs != AERO_OK ? cs : rc;
}

int aero_autotune(const aero_mesh_desc* mesh, const aero_case_desc* c, int iters, aero_case_desc* best,
                  double* ms_out) {
  if (mesh == nullptr || c == nullptr || best == nullptr || iters <= 0)
    return fail(nullptr, AERO_ERR_INVALID, "aero_autotune: bad argument");
  const int orders[2] = {AERO_ORDER_MORTON, AERO_ORDER_RCM};
  const int blocks[3] = {64, 128, 256};
  const int cpts[2] = {1, 2};
  double best_ms = 0.0;
  int k = 0;
  *best = *c;
  for (int n = 0; n < 2 * 3 * 2; ++n) {  // ordering-major, then block size, then cells per thread
    const int o = orders[n / 6], b = blocks[(n / 2) % 3], t = cpts[n % 2];
    aero_case_desc v = *c;
    v.ordering = o;
    v.block_size = b;
    v.cells_per_thread = t;
    aero_ctx* ctx = nullptr;
    int rc = create_ctx(1, mesh, &v, &ctx);
    if (rc != AERO_OK) return rc;
    double ms = 0.0;
    const int warm = std::max(c->startup_first_order_iters, 0);
    if (warm > 0) rc = ctx->engine->time_iterations(warm, 1, 0, &ms);  // first-order start-up
    if (rc == AERO_OK) rc = ctx->engine->time_iterations(2, 1, 0, &ms);  // graphs instantiated
    if (rc == AERO_OK) rc = ctx->engine->time_iterations(iters, 1, 0, &ms);
    const int cs = cuda_status(ctx);
    aero_destroy(ctx);
    if (cs != AERO_OK) return cs;
    if (rc != AERO_OK && rc != AERO_ERR_NONFINITE) return fail(nullptr, rc, "aero_autotune: timing failed");
    if (ms_out) ms_out[k] = ms;
    if (k == 0 || ms < best_ms) {
      best_ms = ms;
      best->ordering = o;
      best->block_size = b;
      best->cells_per_thread = t;
    }
    ++k;
  }
  return AERO_OK;
}

}  // extern "C"

// ---- discrete adjoint (include/aero_adjoint.h)

namespace {
int adjoint_status(aero_ctx* ctx, int rc, const char* what) {
  const int cs = cuda_status(ctx);
  if (cs != AERO_OK) return cs;
  if (rc == AERO_ERR_INVALID)
    return fail(ctx, rc, std::string(what) + ": needs a single-case FP64 context linearised by aero_adjoint_linearize");
  return rc;
}
}  // namespace

extern "C" {

int aero_adjoint_linearize(aero_ctx* ctx, double w_cd, double w_cl, int second_order) {
  if (ctx == nullptr || second_order < -1 || second_order > 1)
    return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_linearize: bad argument");
  if (ctx->engine->n_cases() != 1) return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_linearize: batched context");
  const int rc = ctx->engine->adjoint_linearize(w_cd, w_cl, second_order);
  const int cs = cuda_status(ctx);
  if (cs != AERO_OK) return cs;
  if (rc == AERO_ERR_INVALID)
    return fail(ctx, rc, "aero_adjoint_linearize: needs a single-case FP64 context and finite weights");
  return rc;
}

int aero_adjoint_vjp(aero_ctx* ctx, const double* v, double* out) {
  if (ctx == nullptr || v == nullptr || out == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_vjp: null argument");
  return adjoint_status(ctx, ctx->engine->adjoint_vjp(v, out), "aero_adjoint_vjp");
}

int aero_adjoint_objective_gradient(aero_ctx* ctx, double* g) {
  if (ctx == nullptr || g == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_objective_gradient: null argument");
  return adjoint_status(ctx, ctx->engine->adjoint_objective_gradient(g), "aero_adjoint_objective_gradient");
}

int aero_adjoint_solve(aero_ctx* ctx, int iters, double cfl, double* history) {
  if (ctx == nullptr || iters < 0 || !(cfl > 0.0) || !std::isfinite(cfl))
    return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_solve: bad argument");
  return adjoint_status(ctx, ctx->engine->adjoint_solve(iters, cfl, history), "aero_adjoint_solve");
}

int aero_adjoint_solve_krylov(aero_ctx* ctx, int max_iters, int restart, int smooth_iters, double cfl,
                              double rel_tol, double* history, int* iters_done) {
  if (ctx == nullptr || max_iters < 0 || restart < 1 || restart > 512 || smooth_iters < 0 || !(cfl > 0.0) ||
      !std::isfinite(cfl) || !(rel_tol >= 0.0))
    return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_solve_krylov: bad argument");
  return adjoint_status(
      ctx, ctx->engine->adjoint_solve_krylov(max_iters, restart, smooth_iters, cfl, rel_tol, history, iters_done),
      "aero_adjoint_solve_krylov");
}

int aero_adjoint_set_lambda(aero_ctx* ctx, const double* lam) {
  if (ctx == nullptr || lam == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_set_lambda: null argument");
  return adjoint_status(ctx, ctx->engine->adjoint_set_lambda(lam), "aero_adjoint_set_lambda");
}

int aero_adjoint_get_lambda(aero_ctx* ctx, double* lam) {
  if (ctx == nullptr || lam == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_get_lambda: null argument");
  return adjoint_status(ctx, ctx->engine->adjoint_lambda(lam), "aero_adjoint_get_lambda");
}

int aero_adjoint_dalpha(aero_ctx* ctx, double* dj_dalpha_deg) {
  if (ctx == nullptr || dj_dalpha_deg == nullptr) return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_dalpha: null argument");
  return adjoint_status(ctx, ctx->engine->adjoint_dalpha(dj_dalpha_deg), "aero_adjoint_dalpha");
}

int aero_adjoint_geometry(aero_ctx* ctx, const aero_mesh_desc* tangent, double* dj) {
  if (ctx == nullptr || tangent == nullptr || dj == nullptr)
    return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_geometry: null argument");
  return adjoint_status(ctx, ctx->engine->adjoint_geometry(*tangent, dj), "aero_adjoint_geometry");
}

int aero_adjoint_geometry_vjp(aero_ctx* ctx, double* d_normal, double* d_center, double* d_area, double* d_volume,
                              double* d_cell_center) {
  if (ctx == nullptr || !d_normal || !d_center || !d_area || !d_volume || !d_cell_center)
    return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_geometry_vjp: null argument");
  return adjoint_status(ctx, ctx->engine->adjoint_geometry_vjp(d_normal, d_center, d_area, d_volume, d_cell_center),
                        "aero_adjoint_geometry_vjp");
}

int aero_adjoint_node_vjp(aero_ctx* ctx, const aero_mesh* mesh, double* dj_dpoints) {
  if (ctx == nullptr || mesh == nullptr || dj_dpoints == nullptr)
    return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_node_vjp: null argument");
  aero_mesh_sizes sz{};
  if (aero_mesh_get_sizes(mesh, &sz) != AERO_OK)
    return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_node_vjp: bad mesh");
  long long info[2] = {0, 0};
  ctx->engine->info(info, 2);
  if (info[0] != sz.num_cells || info[1] != sz.num_faces)
    return fail(ctx, AERO_ERR_INVALID, "aero_adjoint_node_vjp: the mesh is not the context's");
  std::vector<double> bn(3 * static_cast<size_t>(sz.num_faces)), bc(bn.size()), ba(sz.num_faces),
      bv(sz.num_cells), bcc(3 * static_cast<size_t>(sz.num_cells));
  const int rc = aero_adjoint_geometry_vjp(ctx, bn.data(), bc.data(), ba.data(), bv.data(), bcc.data());
  if (rc != AERO_OK) return rc;
  if (aero_mesh_geometry_vjp(mesh, bn.data(), bc.data(), ba.data(), bv.data(), bcc.data(), dj_dpoints) != AERO_OK)
    return fail(ctx, AERO_ERR_INVALID, std::string("aero_adjoint_node_vjp: ") + aero_mesh_last_error());
  return AERO_OK;
}

}  // extern "C"
