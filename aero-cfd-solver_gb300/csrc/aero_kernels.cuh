// aero_kernels.cuh -- sm_103a kernels of one pseudo-time iteration.
//
// Data layout in HBM (N cells after renumbering, D face slots per cell, ELL):
//   slot (k, c) lives at k*N + c, so a warp reading slot k of 32 consecutive cells reads
//   one contiguous segment of every slot array.
//   link[k*N+c]  int   (other << 1 | side) for an interior face, side 0 when c owns the face
//                      and 1 when c is its neighbour; -1 far field, -2 slip wall; kPad.
//   nrm [k*N+c]  double2  unit normal of the face, pointing out of its OWNER (canonical)
//   area[k*N+c]  double   face length
//   doff/noff    T2       face centre minus owner / neighbour cell centre
//   vol[c]       double
// Each cell sums its own faces' fluxes (cell-owned gather): an interior face is evaluated
// by both of its cells with identical inputs in the owner->neighbour orientation, so both
// see the same flux bits and the update is conservative, deterministic and atomic-free.
// Slots of a cell are in ascending original face order, the order in which the reference's
// face loop (residual_assembly.cpp:97-180, reconstruction.cpp:87-109) accumulates into it.
//
// Per-iteration values that the device controller changes (CFL, floors, all-speed weights)
// are read from the Ctrl block in device memory, so one iteration is a fixed sequence of
// launches that can be captured once in a CUDA graph and replayed.
#pragma once

#include "aero_numerics.cuh"

#include <cstdint>

namespace aero {

constexpr int kPad = -0x7fffffff;
constexpr int kMaxForceWindow = 64;

struct alignas(32) d4 {
  double x, y, z, w;
};

template <class T>
struct Vec;
template <>
struct Vec<float> {
  using v4 = float4;
  using v2 = float2;
};
template <>
struct Vec<double> {
  using v4 = d4;
  using v2 = double2;
};

template <class T>
__device__ __forceinline__ typename Vec<T>::v4 ld4(const typename Vec<T>::v4* p) {
  return *p;
}

// Controller and per-iteration state (device memory, one per context).
struct Ctrl {
  int iter;        // index of the next iteration to run
  int done;        // converged or trapped: kernels return immediately
  int nonfinite;   // set by the last-stage update when the state is not finite
  int rec_base;    // iteration number stored at records[0] of the current chunk
  int second;      // second order in the current iteration
  int as_fix;      // all-speed fix effective in the current iteration
  int fo_fallback; // per-iteration counters (summed over stages)
  int diff_fallback;
  double cfl, stab_floor, as_fmin, as_ramp;  // current-iteration schedule values
  double cfl_scale, prev_l2, initial_l2;
  int has_prev, hist_count, hist_head, stage;  // stage: 0 single, 1 A, 2 B
  double prev_cl, prev_cd, prev_cm;
  double hist[3 * 2 * kMaxForceWindow];
  double stage_b_fmin;
  int stage_b_progress, pjump_below, freeze, pad0;
  double sr_max;  // global max of max(SR, floor) for global time stepping
};

// Run constants of the controller (euler_solver.cpp:463-566 resolved on the host).
struct CtrlConfig {
  int n_cells, n_wall, rk_stages, local_dt;
  int cfl_ramp, stab_ramp, as_ramp_start, as_ramp_iters;
  int startup_first_order, min_iterations, window, staged;
  int st_a_min, st_a_max, pj_hold, freeze_iters;
  int as_fix_cfg, n_blocks, pjump_blocks, pad;
  double cfl_start, cfl_max, stab_start, stab_target, as_fmin;
  double residual_target, stab_tol, drift_tol;
  double st_fmin_high, st_fmin_mid, st_fmin_low;
  double pj_target, pj_spike, cfl_drop, cfl_restore, cfl_min_scale;
  double p_inf, q_inf, s_ref, chord, cos_a, sin_a, x_ref, y_ref, pressure_ref, gamma;
  double rho_inf, u_inf, v_inf;
};

// Precondition constants in double for the residual preconditioner (preconditioning.cpp:51-76).
struct PrecondD {
  int enabled;
  double gamma, mach_ref, mach_min, beta_min, beta_max;
};

// Schedule of iteration s->iter (euler_solver.cpp:69-112 and 772-797): order switch,
// CFL ramp times the adaptive scale, stabilization-floor ramp, all-speed weights. Used by
// the controller for the next iteration and by the host for iteration 0.
__host__ __device__ inline void apply_schedule(const CtrlConfig& cc, Ctrl* sp) {
  Ctrl& s = *sp;
  const int it = s.iter;
  s.second = it >= (cc.startup_first_order > 0 ? cc.startup_first_order : 0);
  {
    double base;
    if (cc.cfl_ramp <= 0) {
      base = cc.cfl_max;
    } else {
      const double t = smin(1.0, double(it + 1) / double(cc.cfl_ramp > 1 ? cc.cfl_ramp : 1));
      base = cc.cfl_start + t * (cc.cfl_max - cc.cfl_start);
    }
    s.cfl = base * s.cfl_scale;
  }
  {
    const double m0s = sclamp(cc.stab_start, 0.0, 1.0), m0t = sclamp(cc.stab_target, 0.0, 1.0);
    if (cc.stab_ramp <= 0) {
      s.stab_floor = m0t;
    } else {
      const double t =
          sclamp(double(it > 0 ? it : 0) / double(cc.stab_ramp > 1 ? cc.stab_ramp : 1), 0.0, 1.0);
      s.stab_floor = m0s + t * (m0t - m0s);
    }
  }
  if (!cc.staged) {
    s.as_fix = cc.as_fix_cfg;
    s.as_fmin = cc.as_fmin;
    if (cc.as_ramp_iters <= 0) {
      s.as_ramp = (it >= cc.as_ramp_start) ? 1.0 : 0.0;
    } else {
      s.as_ramp = sclamp(double(it - cc.as_ramp_start) / double(cc.as_ramp_iters > 1 ? cc.as_ramp_iters : 1),
                         0.0, 1.0);
    }
  } else if (s.stage == 1) {
    s.as_fix = 0;
    s.as_fmin = cc.st_fmin_high;
    s.as_ramp = 0.0;
  } else {
    s.as_fix = cc.as_fix_cfg;
    s.as_fmin = sclamp(s.stage_b_fmin, cc.st_fmin_low, cc.st_fmin_high);
    s.as_ramp = (cc.as_ramp_iters <= 0)
                    ? 1.0
                    : sclamp(double(s.stage_b_progress) / double(cc.as_ramp_iters > 1 ? cc.as_ramp_iters : 1),
                             0.0, 1.0);
  }
}

template <class T>
struct DevMesh {
  int n, d;
  const int* link;
  const double2* nrm;
  const double* area;
  const typename Vec<T>::v2* doff;
  const typename Vec<T>::v2* noff;
  const double* vol;
};

// Per-block partial results reduced by the control kernel in a fixed order.
struct Partials {
  double* norms;   // [3 * blocks]: l1, l2 sum, linf
  double* dp;      // [2 * blocks]: max |p - p_inf| domain, wall-adjacent
  double* pjump;   // [4 * blocks]: sum dp^2, count, wall sum, wall count
  double* srmax;   // [blocks * warps per block]: max of max(SR, floor)
};

// ---------------------------------------------------------------------------------------
// warp/block reductions
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ double warp_max(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = smax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}
__device__ __forceinline__ float warp_maxf(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = smax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// Block sum of K doubles per thread; result valid in thread 0. shm holds 32*K doubles.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* shm) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) shm[wid * K + k] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = (lane < nw) ? shm[lane * K + k] : 0.0;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
  }
  __syncthreads();
}

__device__ __forceinline__ double block_max(double v, double* shm) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) shm[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = (lane < nw) ? shm[lane] : 0.0;
    v = warp_max(v);
  }
  __syncthreads();
  return v;
}

// ---------------------------------------------------------------------------------------
// Gradient: Green-Gauss primitive gradients (reconstruction.cpp:73-119), gathered per cell.
// ---------------------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_gradient(DevMesh<T> m, const typename Vec<T>::v4* __restrict__ W,
                                                  typename Vec<T>::v4* __restrict__ gx,
                                                  typename Vec<T>::v4* __restrict__ gy,
                                                  const Ctrl* __restrict__ ctrl) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n || ctrl->done) return;
  const auto wc = W[c];
  T ax0 = 0, ax1 = 0, ax2 = 0, ax3 = 0, ay0 = 0, ay1 = 0, ay2 = 0, ay3 = 0;
  for (int k = 0; k < m.d; ++k) {
    const int s = k * m.n + c;
    const int link = m.link[s];
    if (link == kPad) break;
    const double2 nd = m.nrm[s];
    const T a = T(m.area[s]);
    const T nax = T(nd.x) * a, nay = T(nd.y) * a;
    T q0 = wc.x, q1 = wc.y, q2 = wc.z, q3 = wc.w;
    bool minus = false;
    if (link >= 0) {
      const auto wo = W[link >> 1];
      q0 = T(0.5) * (q0 + wo.x);
      q1 = T(0.5) * (q1 + wo.y);
      q2 = T(0.5) * (q2 + wo.z);
      q3 = T(0.5) * (q3 + wo.w);
      minus = (link & 1) != 0;
    }
    if (minus) {
      ax0 -= q0 * nax; ay0 -= q0 * nay;
      ax1 -= q1 * nax; ay1 -= q1 * nay;
      ax2 -= q2 * nax; ay2 -= q2 * nay;
      ax3 -= q3 * nax; ay3 -= q3 * nay;
    } else {
      ax0 += q0 * nax; ay0 += q0 * nay;
      ax1 += q1 * nax; ay1 += q1 * nay;
      ax2 += q2 * nax; ay2 += q2 * nay;
      ax3 += q3 * nax; ay3 += q3 * nay;
    }
  }
  const T inv = T(1) / smax(T(m.vol[c]), Kn<T>::vol_floor);
  typename Vec<T>::v4 ox, oy;
  ox.x = ax0 * inv; ox.y = ax1 * inv; ox.z = ax2 * inv; ox.w = ax3 * inv;
  oy.x = ay0 * inv; oy.y = ay1 * inv; oy.z = ay2 * inv; oy.w = ay3 * inv;
  gx[c] = ox;
  gy[c] = oy;
}

// MUSCL on one variable (reconstruction.cpp:183-193)
template <class T>
__device__ __forceinline__ void muscl_var(int lim, T qo, T qn, T gox, T goy, T gnx, T gny, T dox,
                                          T doy, T dnx, T dny, T* ql, T* qr) {
  const T dc = qn - qo;
  T d_o = T(0), d_n = T(0);
  d_o += gox * dox;
  d_n += gnx * dnx;
  d_o += goy * doy;
  d_n += gny * dny;
  *ql = qo + limit(lim, d_o, dc);
  *qr = qn + limit(lim, d_n, -dc);
}

// ---------------------------------------------------------------------------------------
// Residual: reconstruction + face flux + gather (residual_assembly.cpp:73-182).
// FLUX 0 Rusanov / 1 HLLC; SECOND: MUSCL with gradients; LM: any low-Mach feature on
// (preconditioning, low-Mach dissipation fix, all-speed flux fix); NORMS: last RK stage,
// also writes the residual-norm partials (euler_solver.cpp:309-339).
// ---------------------------------------------------------------------------------------
template <class T, int FLUX, bool SECOND, bool LM, bool NORMS>
__global__ void __launch_bounds__(256) k_residual(DevMesh<T> m, FaceParams<T> fp,
                                                  const typename Vec<T>::v4* __restrict__ W,
                                                  const typename Vec<T>::v4* __restrict__ gx,
                                                  const typename Vec<T>::v4* __restrict__ gy,
                                                  typename Vec<T>::v4* __restrict__ R, T* __restrict__ SR,
                                                  Partials part, Ctrl* __restrict__ ctrl, int global_dt) {
  __shared__ double shm[32 * 3];
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (ctrl->done) return;
  if (LM) {
    fp.stab_floor = T(ctrl->stab_floor);
    fp.as_fix = ctrl->as_fix;
    fp.as_fmin = T(ctrl->as_fmin);
    fp.as_ramp = T(ctrl->as_ramp);
  }
  double nl1 = 0.0, nl2 = 0.0, nlinf = 0.0;
  double srm = 0.0;
  int fo = 0, df = 0;
  if (c < m.n) {
    const auto wc4 = W[c];
    const Prim<T> wc{wc4.x, wc4.y, wc4.z, wc4.w};
    typename Vec<T>::v4 gcx{}, gcy{};
    if (SECOND) {
      gcx = gx[c];
      gcy = gy[c];
    }
    T r0 = 0, r1 = 0, r2 = 0, r3 = 0, sr = 0;
    for (int k = 0; k < m.d; ++k) {
      const int s = k * m.n + c;
      const int link = m.link[s];
      if (link == kPad) break;
      const double2 nd = m.nrm[s];
      const T nx = T(nd.x), ny = T(nd.y);
      const T area = T(m.area[s]);
      Flux<T> f;
      T mws;
      bool fb = false;
      bool minus = false;
      if (link >= 0) {
        const int o = link >> 1;
        minus = (link & 1) != 0;
        const auto wo4 = W[o];
        const Prim<T> wo{wo4.x, wo4.y, wo4.z, wo4.w};
        const Prim<T>& pown = minus ? wo : wc;
        const Prim<T>& pnb = minus ? wc : wo;
        Prim<T> L = pown, Rt = pnb;
        if (SECOND) {
          const auto gox4 = gx[o];
          const auto goy4 = gy[o];
          const auto& gOx = minus ? gox4 : gcx;
          const auto& gOy = minus ? goy4 : gcy;
          const auto& gNx = minus ? gcx : gox4;
          const auto& gNy = minus ? gcy : goy4;
          const auto dO = m.doff[s];
          const auto dN = m.noff[s];
          muscl_var(fp.limiter, pown.r, pnb.r, gOx.x, gOy.x, gNx.x, gNy.x, dO.x, dO.y, dN.x, dN.y, &L.r, &Rt.r);
          muscl_var(fp.limiter, pown.u, pnb.u, gOx.y, gOy.y, gNx.y, gNy.y, dO.x, dO.y, dN.x, dN.y, &L.u, &Rt.u);
          muscl_var(fp.limiter, pown.v, pnb.v, gOx.z, gOy.z, gNx.z, gNy.z, dO.x, dO.y, dN.x, dN.y, &L.v, &Rt.v);
          muscl_var(fp.limiter, pown.p, pnb.p, gOx.w, gOy.w, gNx.w, gNy.w, dO.x, dO.y, dN.x, dN.y, &L.p, &Rt.p);
          L.r = smax(L.r, Kn<T>::rho_floor);
          Rt.r = smax(Rt.r, Kn<T>::rho_floor);
          L.p = smax(L.p, Kn<T>::p_floor);
          Rt.p = smax(Rt.p, Kn<T>::p_floor);
          if (!valid_prim(L) || !valid_prim(Rt)) {
            L = pown;
            Rt = pnb;
            if (!minus) ++fo;
          }
        }
        const Cons<T> cl = prim_to_cons(L, fp.gamma), cr = prim_to_cons(Rt, fp.gamma);
        const T as = face_acoustic_scale<T, LM>(cl, cr, fp);
        f = face_flux<T, FLUX, LM>(cl, cr, nx, ny, fp, as, &mws, &fb);
        if (minus) fb = false;  // count each face once, on its owner side
      } else {
        const Cons<T> in = prim_to_cons(wc, fp.gamma);
        if (link == -2) {
          const T as = face_acoustic_scale<T, LM>(in, in, fp);
          const Prim<T> w = cons_to_prim(in, fp.gamma);
          const T un = w.u * nx + w.v * ny;
          const T a = sound_speed(w, fp.gamma);
          f = {T(0), w.p * nx, w.p * ny, T(0)};
          mws = precond_speeds(un, a, as).sr;
        } else {
          const T as = face_acoustic_scale<T, LM>(in, fp.farfield, fp);
          const Cons<T> bs = fp.precond_farfield_bc ? precond_farfield_state(in, nx, ny, fp, as) : fp.farfield;
          f = face_flux<T, FLUX, LM>(in, bs, nx, ny, fp, as, &mws, &fb);
        }
      }
      if (fb) ++df;
      sr += mws * area;
      const T f0 = f.m * area, f1 = f.fx * area, f2 = f.fy * area, f3 = f.e * area;
      if (minus) {
        r0 -= f0; r1 -= f1; r2 -= f2; r3 -= f3;
      } else {
        r0 += f0; r1 += f1; r2 += f2; r3 += f3;
      }
    }
    typename Vec<T>::v4 out;
    out.x = r0; out.y = r1; out.z = r2; out.w = r3;
    R[c] = out;
    SR[c] = sr;
    if (global_dt) srm = double(smax(sr, Kn<T>::wave_floor));
    if (NORMS) {
      const double inv = 1.0 / smax(m.vol[c], 1.0e-12);
      const double v[4] = {double(r0) * inv, double(r1) * inv, double(r2) * inv, double(r3) * inv};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const double a = fabs(v[k]);
        nl1 += a;
        nl2 += a * a;
        nlinf = smax(nlinf, a);
      }
    }
  }
  // fallback counters: one atomic per warp when any lane counted something
  const unsigned any = __ballot_sync(0xffffffffu, (fo | df) != 0);
  if (any) {
    const int sfo = __reduce_add_sync(0xffffffffu, fo);
    const int sdf = __reduce_add_sync(0xffffffffu, df);
    if ((threadIdx.x & 31) == __ffs(any) - 1) {
      if (sfo) atomicAdd(&ctrl->fo_fallback, sfo);
      if (sdf) atomicAdd(&ctrl->diff_fallback, sdf);
    }
  }
  if (global_dt) {
    srm = warp_max(srm);
    if ((threadIdx.x & 31) == 0) part.srmax[blockIdx.x * ((blockDim.x + 31) >> 5) + (threadIdx.x >> 5)] = srm;
  }
  if (NORMS) {
    double v3[3] = {nl1, nl2, 0.0};
    block_sum<3>(v3, shm);
    const double mx = block_max(nlinf, shm);
    if (threadIdx.x == 0) {
      part.norms[3 * blockIdx.x + 0] = v3[0];
      part.norms[3 * blockIdx.x + 1] = v3[1];
      part.norms[3 * blockIdx.x + 2] = mx;
    }
  }
}

// Global time step (time_integrator.cpp:45-56): maximum over per-warp maxima of max(SR, floor).
static __global__ void k_srmax(const double* __restrict__ srmax, int n, Ctrl* ctrl) {
  __shared__ double shm[32];
  if (ctrl->done) return;
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = smax(m, srmax[i]);
  m = block_max(m, shm);
  if (threadIdx.x == 0) ctrl->sr_max = m;
}

// ---------------------------------------------------------------------------------------
// Update: low-Mach residual preconditioning (preconditioning.cpp:51-76, in double), local
// time step (time_integrator.cpp:31-59) and SSP-RK3 stage (time_integrator.cpp:61-104) on
// the double conserved state; writes the bulk primitive state for the next stage.
// The last stage also forms max |p - p_inf| partials and the non-finite trap
// (euler_solver.cpp:908-946) from the new state.
// ---------------------------------------------------------------------------------------
template <class T, bool PRECOND, bool LAST>
__global__ void __launch_bounds__(256) k_update(int n, int stage, PrecondD pc,
                                                const typename Vec<T>::v4* __restrict__ R,
                                                const T* __restrict__ SR, typename Vec<T>::v4* __restrict__ W,
                                                d4* __restrict__ Un, d4* __restrict__ Us,
                                                const unsigned char* __restrict__ wall_adj, double p_inf,
                                                Partials part, Ctrl* __restrict__ ctrl, int global_dt) {
  __shared__ double shm[32];
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (ctrl->done) return;
  double dpd = 0.0, dpw = 0.0;
  bool bad = false;
  if (c < n) {
    const auto r4 = R[c];
    double r0 = double(r4.x), r1 = double(r4.y), r2 = double(r4.z), r3 = double(r4.w);
    if (PRECOND) {
      const auto w4 = W[c];
      const Prim<double> w{double(w4.x), double(w4.y), double(w4.z), double(w4.w)};
      FaceParams<double> fpd;
      fpd.gamma = pc.gamma;
      fpd.pc_mach_ref = pc.mach_ref;
      fpd.pc_mach_min = pc.mach_min;
      fpd.pc_beta_min = pc.beta_min;
      fpd.pc_beta_max = pc.beta_max;
      const double beta = cell_beta(w, fpd);
      const double b2 = beta * beta;
      const double inv_rho = 1.0 / smax(w.r, 1.0e-8);
      const double ud = w.u * r1 + w.v * r2;
      r3 = b2 * r3 + (b2 - 1.0) * inv_rho * ud;
    }
    const T cfl = T(ctrl->cfl);
    T dt;
    if (global_dt) {
      dt = cfl / T(ctrl->sr_max);
      if (!sfinite(dt)) dt = T(0);
    } else {
      dt = cfl / smax(SR[c], Kn<T>::wave_floor);
    }
    const double d = double(dt);
    const d4 un = Un[c];
    const d4 us = (stage == 0) ? un : Us[c];
    Cons<double> s{us.x - d * r0, us.y - d * r1, us.z - d * r2, us.w - d * r3};
    if (stage == 1) {
      s.r = 0.75 * un.x + 0.25 * s.r;
      s.ru = 0.75 * un.y + 0.25 * s.ru;
      s.rv = 0.75 * un.z + 0.25 * s.rv;
      s.rE = 0.75 * un.w + 0.25 * s.rE;
    } else if (stage >= 2) {
      const double a = 1.0 / 3.0, b = 2.0 / 3.0;
      s.r = a * un.x + b * s.r;
      s.ru = a * un.y + b * s.ru;
      s.rv = a * un.z + b * s.rv;
      s.rE = a * un.w + b * s.rE;
    }
    enforce_physical(&s, pc.gamma);
    const d4 o{s.r, s.ru, s.rv, s.rE};
    if (LAST) {
      Un[c] = o;
    } else {
      Us[c] = o;
    }
    const Cons<T> ct{T(s.r), T(s.ru), T(s.rv), T(s.rE)};
    const Prim<T> w = cons_to_prim(ct, T(pc.gamma));
    typename Vec<T>::v4 wo;
    wo.x = w.r; wo.y = w.u; wo.z = w.v; wo.w = w.p;
    W[c] = wo;
    if (LAST) {
      const Prim<double> wd = cons_to_prim(s, pc.gamma);
      bad = !finite4(s.r, s.ru, s.rv, s.rE) || !finite4(wd.r, wd.u, wd.v, wd.p);
      dpd = fabs(wd.p - p_inf);
      if (wall_adj[c]) dpw = dpd;
    }
  }
  if (LAST) {
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&ctrl->nonfinite, 1);
    dpd = block_max(dpd, shm);
    dpw = block_max(dpw, shm);
    if (threadIdx.x == 0) {
      part.dp[2 * blockIdx.x] = dpd;
      part.dp[2 * blockIdx.x + 1] = dpw;
    }
  }
}

// AoA-0 symmetry (euler_solver.cpp:418-450): every `interval` iterations the new state's
// v is zeroed through the primitive variables. Applied after the last stage; it redoes the
// last stage's max |p - p_inf| partials and non-finite check on the symmetrised state.
template <class T>
__global__ void __launch_bounds__(256) k_symmetry(int n, int interval, double gamma, d4* __restrict__ Un,
                                                  typename Vec<T>::v4* __restrict__ W,
                                                  const unsigned char* __restrict__ wall_adj, double p_inf,
                                                  Partials part, Ctrl* __restrict__ ctrl) {
  __shared__ double shm[32];
  if (ctrl->done) return;
  if (((ctrl->iter + 1) % interval) != 0) return;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double dpd = 0.0, dpw = 0.0;
  bool bad = false;
  if (c < n) {
    const d4 u = Un[c];
    Prim<double> w = cons_to_prim(Cons<double>{u.x, u.y, u.z, u.w}, gamma);
    w.v = 0.0;
    const Cons<double> s = prim_to_cons(w, gamma);
    Un[c] = d4{s.r, s.ru, s.rv, s.rE};
    const Prim<T> wt = cons_to_prim(Cons<T>{T(s.r), T(s.ru), T(s.rv), T(s.rE)}, T(gamma));
    typename Vec<T>::v4 wo;
    wo.x = wt.r; wo.y = wt.u; wo.z = wt.v; wo.w = wt.p;
    W[c] = wo;
    const Prim<double> wd = cons_to_prim(s, gamma);
    bad = !finite4(s.r, s.ru, s.rv, s.rE) || !finite4(wd.r, wd.u, wd.v, wd.p);
    dpd = fabs(wd.p - p_inf);
    if (wall_adj[c]) dpw = dpd;
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&ctrl->nonfinite, 1);
  dpd = block_max(dpd, shm);
  dpw = block_max(dpw, shm);
  if (threadIdx.x == 0) {
    part.dp[2 * blockIdx.x] = dpd;
    part.dp[2 * blockIdx.x + 1] = dpw;
  }
}

// Pressure-jump energy over interior faces (euler_solver.cpp:1027-1063), per owning cell.
template <class T>
__global__ void __launch_bounds__(256) k_pjump(DevMesh<T> m, const d4* __restrict__ Un,
                                               const unsigned char* __restrict__ wall_adj, double gamma,
                                               Partials part, const Ctrl* __restrict__ ctrl) {
  __shared__ double shm[32 * 4];
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (ctrl->done) return;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  if (c < m.n) {
    const d4 uc = Un[c];
    const double pc = cons_to_prim(Cons<double>{uc.x, uc.y, uc.z, uc.w}, gamma).p;
    for (int k = 0; k < m.d; ++k) {
      const int link = m.link[k * m.n + c];
      if (link == kPad) break;
      if (link < 0 || (link & 1)) continue;  // interior faces owned by c
      const int o = link >> 1;
      const d4 uo = Un[o];
      const double po = cons_to_prim(Cons<double>{uo.x, uo.y, uo.z, uo.w}, gamma).p;
      const double dp = pc - po;
      v[0] += dp * dp;
      v[1] += 1.0;
      if (wall_adj[c] || wall_adj[o]) {
        v[2] += dp * dp;
        v[3] += 1.0;
      }
    }
  }
  block_sum<4>(v, shm);
  if (threadIdx.x == 0) {
    for (int k = 0; k < 4; ++k) part.pjump[4 * blockIdx.x + k] = v[k];
  }
}

// Wall faces for forces (forces.cpp:208-294), in wall-patch order.
struct WallSet {
  const int* cell;     // new index of the owner cell
  const double* nx;    // unit normal out of the owner
  const double* ny;
  const double* area;
  const double* x;     // face centre
  const double* y;
};

// Host-visible iteration record (mirrors aero_iter_record of include/aero_gb300.h).
struct Record {
  int iter, flags, fo, df;
  double l1, l2, linf, ratio;
  double cl, cd, cm, lift, drag, moment;
  double cl_abs, cd_abs, cm_abs;
  double fx_g, fy_g, fx_a, fy_a, snx, sny;
  double dcl, dcd, dcm, mdcl, mdcd, mdcm;
  double cfl, cfl_scale;
  double stab, as_fmin, as_ramp;
  double dp_dom, dp_wall;
  double pj, pj_wall;
  double wall_un, wall_mass_flux, cp_min, cp_max;
  double ff_dp, ff_drho, ff_du, ff_dv;
  int cp_nonfinite, action;
};

// Owner cells of the far-field faces, for the far-field deviation monitors.
struct FarSet {
  const int* cell;
  int n;
};

// Controller (one block): norms, forces, convergence monitor, adaptive CFL, staged all-speed
// controller and the next iteration's schedule (euler_solver.cpp:948-1208, 772-797;
// convergence_monitor.cpp:13-127).
static __global__ void __launch_bounds__(1024) k_control(CtrlConfig cc, WallSet ws, FarSet fs,
                                                  const d4* __restrict__ Un, Partials part,
                                                  Ctrl* __restrict__ ctrl, Record* __restrict__ recs,
                                                  int rec_cap) {
  __shared__ double shm[32 * 8];
  if (ctrl->done) return;
  const int tid = threadIdx.x;
  // residual norms
  double a[3] = {0.0, 0.0, 0.0};
  double lmax = 0.0;
  for (int b = tid; b < cc.n_blocks; b += blockDim.x) {
    a[0] += part.norms[3 * b];
    a[1] += part.norms[3 * b + 1];
    lmax = smax(lmax, part.norms[3 * b + 2]);
  }
  block_sum<3>(a, shm);
  lmax = block_max(lmax, shm);
  double dpd = 0.0, dpw = 0.0;
  for (int b = tid; b < cc.n_blocks; b += blockDim.x) {
    dpd = smax(dpd, part.dp[2 * b]);
    dpw = smax(dpw, part.dp[2 * b + 1]);
  }
  dpd = block_max(dpd, shm);
  dpw = block_max(dpw, shm);
  double pj[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = tid; b < cc.pjump_blocks; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < 4; ++k) pj[k] += part.pjump[4 * b + k];
  }
  block_sum<4>(pj, shm);
  // forces (forces.cpp:208-294) and wall monitors (euler_solver.cpp:976-1006)
  double fsum[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // snx sny fxa fya fxg fyg ma mg
  double un_max = 0.0, cp_hi = -1.0e308, cp_lo_neg = -1.0e308, cp_bad = 0.0;
  for (int i = tid; i < cc.n_wall; i += blockDim.x) {
    const d4 u = Un[ws.cell[i]];
    const Prim<double> w = cons_to_prim(Cons<double>{u.x, u.y, u.z, u.w}, cc.gamma);
    const double p = w.p;
    const double nax = -ws.nx[i] * ws.area[i];
    const double nay = -ws.ny[i] * ws.area[i];
    const double gp = p - cc.p_inf;
    const double x = ws.x[i] - cc.x_ref, y = ws.y[i] - cc.y_ref;
    fsum[0] += nax;
    fsum[1] += nay;
    fsum[2] -= p * nax;
    fsum[3] -= p * nay;
    fsum[4] -= gp * nax;
    fsum[5] -= gp * nay;
    fsum[6] += x * (-p * nay) - y * (-p * nax);
    fsum[7] += x * (-gp * nay) - y * (-gp * nax);
    un_max = smax(un_max, fabs(w.u * ws.nx[i] + w.v * ws.ny[i]));
    const double cp = (p - cc.p_inf) / cc.q_inf;
    if (isfinite(cp)) {
      cp_hi = smax(cp_hi, cp);
      cp_lo_neg = smax(cp_lo_neg, -cp);
    } else {
      cp_bad += 1.0;
    }
  }
  block_sum<8>(fsum, shm);
  un_max = block_max(un_max, shm);
  cp_hi = block_max(cp_hi, shm);
  cp_lo_neg = block_max(cp_lo_neg, shm);
  {
    double b1[1] = {cp_bad};
    block_sum<1>(b1, shm);
    cp_bad = b1[0];
  }
  // far-field monitors (euler_solver.cpp:1013-1026)
  double ffm[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = tid; i < fs.n; i += blockDim.x) {
    const d4 u = Un[fs.cell[i]];
    const Prim<double> w = cons_to_prim(Cons<double>{u.x, u.y, u.z, u.w}, cc.gamma);
    ffm[0] = smax(ffm[0], fabs(w.p - cc.p_inf));
    ffm[1] = smax(ffm[1], fabs(w.r - cc.rho_inf));
    ffm[2] = smax(ffm[2], fabs(w.u - cc.u_inf));
    ffm[3] = smax(ffm[3], fabs(w.v - cc.v_inf));
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) ffm[k] = block_max(ffm[k], shm);
  if (tid != 0) return;

  Ctrl& s = *ctrl;
  Record r;
  r.iter = s.iter;
  r.flags = (s.second ? 8 : 0) | (s.as_fix ? 32 : 0) | (s.stage == 1 ? 64 : 0) | (s.stage == 2 ? 128 : 0);
  r.fo = s.fo_fallback;
  r.df = s.diff_fallback;
  r.cfl = s.cfl;
  r.stab = s.stab_floor;
  r.as_fmin = s.as_fmin;
  r.as_ramp = s.as_ramp;
  r.dp_dom = dpd;
  r.dp_wall = dpw;
  r.wall_un = un_max;
  r.wall_mass_flux = 0.0;  // the slip-wall flux has no mass component (boundary_conditions.cpp:97-110)
  r.cp_min = cc.n_wall > 0 ? -cp_lo_neg : 0.0;
  r.cp_max = cc.n_wall > 0 ? cp_hi : 0.0;
  if (cc.n_wall > 0 && cp_bad == double(cc.n_wall)) {
    r.cp_min = 3.402823466e38;  // no finite sample: the reference keeps its float sentinels
    r.cp_max = -3.402823466e38;
  }
  r.cp_nonfinite = int(cp_bad);
  r.ff_dp = ffm[0];
  r.ff_drho = ffm[1];
  r.ff_du = ffm[2];
  r.ff_dv = ffm[3];
  r.action = 0;
  const bool nonfinite = s.nonfinite != 0;

  const double l1 = a[0];
  const double l2 = sqrt(a[1] / double(cc.n_cells > 0 ? 5 * cc.n_cells : 1));
  const double linf = lmax;
  r.l1 = l1;
  r.l2 = l2;
  r.linf = linf;
  // ConvergenceMonitor::update_residual
  const double bl2 = smax(l2, 1.0e-20);
  if (s.initial_l2 < 0.0) s.initial_l2 = bl2;
  const double ratio = bl2 / smax(s.initial_l2, 1.0e-20);
  r.ratio = ratio;
  if (s.prev_l2 > 0.0) {
    if (l2 > s.prev_l2 * 1.05) {
      s.cfl_scale = smax(s.cfl_scale * 0.65, 0.05);
    } else if (l2 < s.prev_l2 * 0.90) {
      s.cfl_scale = smin(s.cfl_scale * 1.03, 1.0);
    }
  }
  s.prev_l2 = l2;
  // integrate_pressure_forces (gauge -> reported, abs -> *_abs)
  const double qs = cc.q_inf * cc.s_ref;
  const double fxg = fsum[4], fyg = fsum[5], fxa = fsum[2], fya = fsum[3];
  r.fx_g = fxg; r.fy_g = fyg; r.fx_a = fxa; r.fy_a = fya; r.snx = fsum[0]; r.sny = fsum[1];
  r.drag = fxg * cc.cos_a + fyg * cc.sin_a;
  r.lift = -fxg * cc.sin_a + fyg * cc.cos_a;
  r.moment = fsum[7];
  r.cd = r.drag / qs;
  r.cl = r.lift / qs;
  r.cm = fsum[7] / (qs * cc.chord);
  r.cd_abs = (fxa * cc.cos_a + fya * cc.sin_a) / qs;
  r.cl_abs = (-fxa * cc.sin_a + fya * cc.cos_a) / qs;
  r.cm_abs = fsum[6] / (qs * cc.chord);
  // ConvergenceMonitor::update_forces
  r.dcl = r.dcd = r.dcm = 0.0;
  if (s.has_prev) {
    r.dcl = fabs(r.cl - s.prev_cl);
    r.dcd = fabs(r.cd - s.prev_cd);
    r.dcm = fabs(r.cm - s.prev_cm);
  }
  s.prev_cl = r.cl; s.prev_cd = r.cd; s.prev_cm = r.cm;
  s.has_prev = 1;
  const int req = cc.window < 1 ? 1 : cc.window;
  const int cap = 2 * req;
  {
    const int slot = (s.hist_head + s.hist_count) % cap;
    s.hist[3 * slot] = r.cl;
    s.hist[3 * slot + 1] = r.cd;
    s.hist[3 * slot + 2] = r.cm;
    if (s.hist_count < cap) {
      ++s.hist_count;
    } else {
      s.hist_head = (s.hist_head + 1) % cap;
    }
  }
  auto H = [&](int i, int k) { return s.hist[3 * ((s.hist_head + i) % cap) + k]; };
  bool stable = false;
  if (s.hist_count >= req) {
    const int b = s.hist_count - req;
    double lo[3], hi[3];
    for (int k = 0; k < 3; ++k) lo[k] = hi[k] = H(b, k);
    for (int i = b; i < s.hist_count; ++i) {
      for (int k = 0; k < 3; ++k) {
        lo[k] = smin(lo[k], H(i, k));
        hi[k] = smax(hi[k], H(i, k));
      }
    }
    stable = (hi[0] - lo[0]) <= cc.stab_tol && (hi[1] - lo[1]) <= cc.stab_tol && (hi[2] - lo[2]) <= cc.stab_tol;
  }
  bool dstable = false;
  r.mdcl = r.mdcd = r.mdcm = 0.0;
  if (s.hist_count >= cap) {
    double pa[3] = {0, 0, 0}, ca[3] = {0, 0, 0};
    for (int i = 0; i < req; ++i)
      for (int k = 0; k < 3; ++k) pa[k] += H(i, k);
    for (int i = req; i < cap; ++i)
      for (int k = 0; k < 3; ++k) ca[k] += H(i, k);
    const double inv = 1.0 / double(req);
    r.mdcl = fabs(ca[0] * inv - pa[0] * inv);
    r.mdcd = fabs(ca[1] * inv - pa[1] * inv);
    r.mdcm = fabs(ca[2] * inv - pa[2] * inv);
    dstable = r.mdcl <= cc.drift_tol && r.mdcd <= cc.drift_tol && r.mdcm <= cc.drift_tol;
  }
  // pressure-jump energies
  const double pr2 = cc.pressure_ref * cc.pressure_ref + 1.0e-24;
  r.pj = pj[1] > 0.0 ? (pj[0] / pj[1]) / pr2 : 0.0;
  r.pj_wall = pj[3] > 0.0 ? (pj[2] / pj[3]) / pr2 : 0.0;
  // staged all-speed controller (euler_solver.cpp:1068-1139)
  if (cc.staged) {
    if (s.stage == 1) {
      const bool ready = (s.iter + 1 >= cc.st_a_min) && stable;
      const bool timeout = (cc.st_a_max > 0) && (s.iter + 1 >= cc.st_a_max);
      if ((ready || timeout) && cc.as_fix_cfg) {
        s.stage = 2;
        s.stage_b_fmin = cc.st_fmin_high;
        s.stage_b_progress = 0;
        s.pjump_below = 0;
        s.freeze = 0;
        r.action = ready ? 10 : 11;
      }
    } else {
      const double thr = (cc.pj_target > 0.0) ? cc.pj_target * cc.pj_spike : 1.0e308;
      const bool spike = r.pj_wall > thr;
      const bool good = (cc.pj_target <= 0.0) || (r.pj_wall <= cc.pj_target);
      if (spike) {
        s.freeze = cc.freeze_iters;
        s.pjump_below = 0;
        s.stage_b_fmin = smin(cc.st_fmin_high, s.stage_b_fmin + 0.05);
        s.cfl_scale = smax(s.cfl_scale * cc.cfl_drop, cc.cfl_min_scale);
        r.action = 20;
      } else {
        if (s.freeze > 0) --s.freeze;
        s.pjump_below = good ? s.pjump_below + 1 : 0;
        if (s.freeze == 0) {
          if (s.stage_b_fmin > cc.st_fmin_mid + 1.0e-6 && s.pjump_below >= cc.pj_hold) {
            s.stage_b_fmin = cc.st_fmin_mid;
            s.pjump_below = 0;
            r.action = 31;
          } else if (s.stage_b_fmin > cc.st_fmin_low + 1.0e-6 && s.pjump_below >= cc.pj_hold) {
            s.stage_b_fmin = cc.st_fmin_low;
            s.pjump_below = 0;
            r.action = 32;
          } else if (s.stage_b_fmin <= cc.st_fmin_low + 1.0e-6 && good) {
            ++s.stage_b_progress;
            if (r.action == 0) r.action = 33;
          }
          if (good) {
            s.cfl_scale = smin(s.cfl_scale * cc.cfl_restore, 1.0);
          } else if (cc.pj_target > 0.0 && r.pj_wall > cc.pj_target) {
            s.cfl_scale = smax(s.cfl_scale * cc.cfl_drop, cc.cfl_min_scale);
            if (r.action == 0) r.action = 21;
          }
        }
      }
    }
  }
  r.cfl_scale = s.cfl_scale;
  if (stable) r.flags |= 1;
  if (dstable) r.flags |= 2;
  const bool conv = (s.iter + 1 >= cc.min_iterations) && !(ratio > cc.residual_target) && stable && dstable;
  if (conv) r.flags |= 4;
  if (nonfinite) r.flags |= 16;
  const int slot = s.iter - s.rec_base;
  if (slot >= 0 && slot < rec_cap) recs[slot] = r;
  if (conv || nonfinite) s.done = 1;
  // next iteration's schedule
  s.iter = s.iter + 1;
  s.fo_fallback = 0;
  s.diff_fallback = 0;
  apply_schedule(cc, &s);
}

// Bulk primitive state from the conserved state (start of a run or after aero_set_state).
template <class T>
__global__ void k_refresh_prim(int n, const d4* __restrict__ Un, typename Vec<T>::v4* __restrict__ W, double gamma) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const d4 u = Un[c];
  const Cons<T> ct{T(u.x), T(u.y), T(u.z), T(u.w)};
  const Prim<T> w = cons_to_prim(ct, T(gamma));
  typename Vec<T>::v4 o;
  o.x = w.r; o.y = w.u; o.z = w.v; o.w = w.p;
  W[c] = o;
}

}  // namespace aero
