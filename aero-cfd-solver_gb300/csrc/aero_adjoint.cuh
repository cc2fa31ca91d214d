// aero_adjoint.cuh -- discrete adjoint of the FP64 residual R(U) = sum over faces of F*A
// (the residual the face pass and cell gather compute; no reference counterpart: AeroCFD has
// no adjoint).
//
// Linearisation: for every face, eval_face is run in dual numbers seeded on the two cells'
// primitive states and Green-Gauss gradients, giving the exact local Jacobian of F*A with
// respect to (W_o, W_n, G_o, G_n) for the branches the converged state takes (limiter,
// floors, first-order fallback, HLLC wave pattern, low-Mach scalings). It is stored per face
// (4 x 24 doubles).
//
// Transpose product (dR/dU)^T v, as four deterministic passes:
//   face pass    per face, a = v_o - v_n; the face's adjoint contributions J^T a to the two
//                cells' primitive states and gradients;
//   cell gather  per cell, its faces' contributions in ascending original face order;
//   Green-Gauss  per cell, the gradient adjoints of the cell and its neighbours mapped back
//                onto the cell's primitive state (the transpose of reconstruction.cpp:73-119);
//   primitive    per cell, (dW/dU)^T from cons_to_prim in dual numbers.
#pragma once

#include "aero_dual.cuh"
#include "aero_face_kernels.cuh"

namespace aero {

constexpr int kJac = 24;  // columns of a face Jacobian: W_o, W_n, G_o (x, y), G_n (x, y)
// Columns stored per scheme: first order has no gradient inputs.
template <bool SECOND>
constexpr int jac_cols() {
  return SECOND ? kJac : 8;
}

template <int N>
__device__ __forceinline__ FaceParams<ad::Dual<N>> dual_params(const FaceParams<double>& f) {
  using D = ad::Dual<N>;
  FaceParams<D> d;
  d.gamma = D(f.gamma);
  d.farfield = Cons<D>{D(f.farfield.r), D(f.farfield.ru), D(f.farfield.rv), D(f.farfield.rE)};
  d.limiter = f.limiter;
  d.precond = f.precond;
  d.low_mach_fix = f.low_mach_fix;
  d.precond_farfield_bc = f.precond_farfield_bc;
  d.as_fix = f.as_fix;
  d.mach_cutoff = D(f.mach_cutoff);
  d.pc_mach_ref = D(f.pc_mach_ref);
  d.pc_mach_min = D(f.pc_mach_min);
  d.pc_beta_min = D(f.pc_beta_min);
  d.pc_beta_max = D(f.pc_beta_max);
  d.stab_floor = D(f.stab_floor);
  d.as_cutoff = D(f.as_cutoff);
  d.as_fmin = D(f.as_fmin);
  d.as_ramp = D(f.as_ramp);
  d.inv_gm1 = D(f.inv_gm1);
  return d;
}

// The schedule-dependent face parameters at the linearisation point.
__device__ __forceinline__ FaceParams<double> scheduled_params(FaceParams<double> fp, const Ctrl* ctrl, bool lm) {
  if (lm) {
    fp.as_fix = ctrl->as_fix;
    fp.stab_floor = ctrl->stab_floor;
    fp.as_fmin = ctrl->as_fmin;
    fp.as_ramp = ctrl->as_ramp;
  }
  return fp;
}

// Local Jacobian of face i: d(F_k A) / d(input j), inputs W_o(4), W_n(4), G_o(8: x then y of
// rho, u, v, p), G_n(8) (second order; the first 8 only for first order). Stored by column
// across faces, J[(k * NC + j) * nf + i], so that a warp's loads are coalesced. Three dual
// passes of 8 seeds each.
template <int FLUX, bool SECOND, bool LM>
__global__ void __launch_bounds__(256) k_adj_face_jac(DevFaces<double> f, const int2* __restrict__ fblk,
                                                      const FaceParams<double>* __restrict__ fps,
                                                      const Ctrl* __restrict__ ctrl, const d4* __restrict__ W,
                                                      const d4* __restrict__ gx, const d4* __restrict__ gy,
                                                      double* __restrict__ J) {
  using D = ad::Dual<8>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int2 bd = fblk[blockIdx.x];
  if (i >= bd.y) return;
  const FaceParams<D> fp = dual_params<8>(scheduled_params(fps[bd.x], ctrl, LM));
  const int2 oc = f.cells[i];
  const int o = oc.x, b = oc.y;
  const double2 nd = f.nrm[i];
  const double area = f.area[i];
  const d4 w0 = W[o];
  const d4 w1 = b >= 0 ? W[b] : w0;
  double go[8], gn[8];
  double dox = 0.0, doy = 0.0, dnx = 0.0, dny = 0.0;
  if (b >= 0 && SECOND) {
    const d4 a = gx[o], c = gy[o], e = gx[b], h = gy[b];
    const double g0[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
    const double g1[8] = {e.x, e.y, e.z, e.w, h.x, h.y, h.z, h.w};
    for (int k = 0; k < 8; ++k) {
      go[k] = g0[k];
      gn[k] = g1[k];
    }
    dox = f.doff[i].x;
    doy = f.doff[i].y;
    dnx = f.noff[i].x;
    dny = f.noff[i].y;
  } else {
    for (int k = 0; k < 8; ++k) go[k] = gn[k] = 0.0;
  }
  constexpr int NC = jac_cols<SECOND>();
  const size_t nf = static_cast<size_t>(f.nf);
  if (SECOND && b < 0) {  // no gradient inputs at a boundary face
    for (int k = 0; k < 4; ++k) {
      for (int j = 8; j < NC; ++j) J[(k * NC + j) * nf + i] = 0.0;
    }
  }
  const int passes = (b >= 0 && SECOND) ? 3 : 1;
  for (int pass = 0; pass < passes; ++pass) {
    D wo[4] = {D(w0.x), D(w0.y), D(w0.z), D(w0.w)};
    D wn[4] = {D(w1.x), D(w1.y), D(w1.z), D(w1.w)};
    D gO[8], gN[8];
    for (int k = 0; k < 8; ++k) {
      gO[k] = D(go[k]);
      gN[k] = D(gn[k]);
    }
    if (pass == 0) {
      for (int k = 0; k < 4; ++k) {
        wo[k].d[k] = 1.0;
        if (b >= 0) wn[k].d[4 + k] = 1.0;
      }
    } else if (pass == 1) {
      for (int k = 0; k < 8; ++k) gO[k].d[k] = 1.0;
    } else {
      for (int k = 0; k < 8; ++k) gN[k].d[k] = 1.0;
    }
    Flux<D> fl;
    D mws;
    bool fo = false, df = false;
    eval_face<D, FLUX, SECOND, LM>(fp, b, Prim<D>{wo[0], wo[1], wo[2], wo[3]}, Prim<D>{wn[0], wn[1], wn[2], wn[3]},
                                   gO, gN, D(nd.x), D(nd.y), D(dox), D(doy), D(dnx), D(dny), &fl, &mws, &fo, &df);
    const D fk[4] = {fl.m, fl.fx, fl.fy, fl.e};
    for (int k = 0; k < 4; ++k) {
      for (int j = 0; j < 8; ++j) J[(k * NC + pass * 8 + j) * nf + i] = fk[k].d[j] * area;
    }
  }
}

// Face pass of the transpose product: per face, a = v_o - v_n (v_o at a boundary face) and
// its NC contributions J^T a, face-contiguous: [0,4) to W_o, [4,8) W_n, [8,16) G_o,
// [16,24) G_n.
template <int NC>
__global__ void __launch_bounds__(256) k_adj_face_vjp(DevFaces<double> f, const int2* __restrict__ fblk,
                                                      const double* __restrict__ J, const d4* __restrict__ v,
                                                      double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= fblk[blockIdx.x].y) return;
  const int2 oc = f.cells[i];
  const d4 vo = v[oc.x];
  d4 a = vo;
  if (oc.y >= 0) {
    const d4 vn = v[oc.y];
    a = d4{vo.x - vn.x, vo.y - vn.y, vo.z - vn.z, vo.w - vn.w};
  }
  const size_t nf = static_cast<size_t>(f.nf);
  double* o = out + static_cast<size_t>(i) * NC;
#pragma unroll
  for (int j = 0; j < NC; ++j) {
    o[j] = J[j * nf + i] * a.x + J[(NC + j) * nf + i] * a.y + J[(2 * NC + j) * nf + i] * a.z +
           J[(3 * NC + j) * nf + i] * a.w;
  }
}

// Cell gather of the face contributions, in the cell's face order: mw (4) and, for second
// order, mg (8) per cell.
template <int NC>
__global__ void __launch_bounds__(256) k_adj_gather(DevGather<double> g, const int2* __restrict__ cblk,
                                                    const double* __restrict__ out, d4* __restrict__ mw,
                                                    d4* __restrict__ mgx, d4* __restrict__ mgy) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cblk[blockIdx.x].y) return;
  double w[4] = {0, 0, 0, 0}, q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < g.d; ++k) {
    const int s = g.slot[k * g.n + c];
    if (s == kPad) break;
    const double* o = out + static_cast<size_t>(s >> 1) * NC;
    const int wo = (s & 1) ? 4 : 0, go = (s & 1) ? 16 : 8;
    for (int j = 0; j < 4; ++j) w[j] += o[wo + j];
    if (NC > 8) {
      for (int j = 0; j < 8; ++j) q[j] += o[go + j];
    }
  }
  mw[c] = d4{w[0], w[1], w[2], w[3]};
  if (NC > 8) {
    mgx[c] = d4{q[0], q[1], q[2], q[3]};
    mgy[c] = d4{q[4], q[5], q[6], q[7]};
  }
}

// Transpose of the Green-Gauss gradient (cell_gradient): G_c = (1/V_c) sum_s sgn_s q_s n_s A_s,
// q_s = (W_c + W_o)/2 across an interior face, W_c at a boundary face. Adds to mw_c the
// adjoints of the cell's own gradient and of its neighbours' gradients.
static __global__ void k_adj_green_gauss(DevMesh<double> m, const int2* __restrict__ cblk, const d4* __restrict__ mgx,
                                  const d4* __restrict__ mgy, d4* __restrict__ mw) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cblk[blockIdx.x].y) return;
  const d4 gxc = mgx[c], gyc = mgy[c];
  const double invc = m.inv_vol[c];
  double w[4] = {0, 0, 0, 0};
  for (int k = 0; k < m.d; ++k) {
    const int s = k * m.n + c;
    const int link = m.link[s];
    if (link == kPad) break;
    const double2 nd = m.nrm[s];
    const double a = m.area[s];
    const double sgn = (link >= 0 && (link & 1)) ? -1.0 : 1.0;
    const double nax = nd.x * a * sgn, nay = nd.y * a * sgn;  // outward from c
    const double wt = link >= 0 ? 0.5 : 1.0;
    w[0] += wt * invc * (nax * gxc.x + nay * gyc.x);
    w[1] += wt * invc * (nax * gxc.y + nay * gyc.y);
    w[2] += wt * invc * (nax * gxc.z + nay * gyc.z);
    w[3] += wt * invc * (nax * gxc.w + nay * gyc.w);
    if (link >= 0) {  // the neighbour's gradient: its outward normal is -n
      const int o = link >> 1;
      const d4 gxo = mgx[o], gyo = mgy[o];
      const double invo = m.inv_vol[o];
      w[0] -= 0.5 * invo * (nax * gxo.x + nay * gyo.x);
      w[1] -= 0.5 * invo * (nax * gxo.y + nay * gyo.y);
      w[2] -= 0.5 * invo * (nax * gxo.z + nay * gyo.z);
      w[3] -= 0.5 * invo * (nax * gxo.w + nay * gyo.w);
    }
  }
  const d4 cur = mw[c];
  mw[c] = d4{cur.x + w[0], cur.y + w[1], cur.z + w[2], cur.w + w[3]};
}

// (dW/dU)^T per cell: out = J_c^T mw with J_c the Jacobian of cons_to_prim at U_c.
static __global__ void k_adj_prim(const int2* __restrict__ cblk, const d4* __restrict__ U, double gamma,
                           const d4* __restrict__ mw, d4* __restrict__ out) {
  using D = ad::Dual<4>;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cblk[blockIdx.x].y) return;
  const d4 u = U[c];
  const Prim<D> w = cons_to_prim(Cons<D>{ad::seed<4>(u.x, 0), ad::seed<4>(u.y, 1), ad::seed<4>(u.z, 2),
                                         ad::seed<4>(u.w, 3)},
                                 D(gamma));
  const d4 m = mw[c];
  double r[4];
  for (int j = 0; j < 4; ++j) r[j] = w.r.d[j] * m.x + w.u.d[j] * m.y + w.v.d[j] * m.z + w.p.d[j] * m.w;
  out[c] = d4{r[0], r[1], r[2], r[3]};
}

// dJ/dU of a force coefficient (forces.cpp:208-294): J = (e_x Fx + e_y Fy) / (q S) with the
// gauge force F = sum over the wall patch of (p_owner - p_inf) n A; per cell the sum over its
// patch faces, through p = p(U).
static __global__ void k_adj_objective(const int2* __restrict__ cblk, const d4* __restrict__ U, double gamma,
                                MonitorSet ms, double ex, double ey, double inv_qs, d4* __restrict__ g) {
  using D = ad::Dual<4>;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cblk[blockIdx.x].y) return;
  const unsigned char fl = ms.flags[c];
  double s = 0.0;
  if (fl >= 4) {
    const int first = ms.wall_first[c], cnt = fl >> 2;
    for (int j = first; j < first + cnt; ++j) {
      if (ms.wkind[j] & 1) s += (ex * ms.wnx[j] + ey * ms.wny[j]) * ms.warea[j];
    }
  }
  if (s == 0.0) {
    g[c] = d4{0.0, 0.0, 0.0, 0.0};
    return;
  }
  const d4 u = U[c];
  const Prim<D> w = cons_to_prim(Cons<D>{ad::seed<4>(u.x, 0), ad::seed<4>(u.y, 1), ad::seed<4>(u.z, 2),
                                         ad::seed<4>(u.w, 3)},
                                 D(gamma));
  const double f = s * inv_qs;
  g[c] = d4{f * w.p.d[0], f * w.p.d[1], f * w.p.d[2], f * w.p.d[3]};
}

// One pseudo-time stage of the adjoint (the primal's SSP-RK3 with local steps,
// time_integrator.cpp:31-104): r = (dR/dU)^T lam + g; stage s sets
// lam_s = c_n lam_n + c_s (lam_prev - dt r) with (c_n, c_s) = (0, 1), (3/4, 1/4), (1/3, 2/3).
// partial (may be null): per block, the sum of |r|^2 over its cells (fixed reduction order).
static __global__ void __launch_bounds__(256) k_adj_stage(const int2* __restrict__ cblk, int stage, double cfl,
                                                          const double* __restrict__ SR, const d4* __restrict__ r,
                                                          const d4* __restrict__ g, const d4* __restrict__ lam_n,
                                                          d4* __restrict__ lam, double* __restrict__ partial) {
  __shared__ double warp_sum[8];
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double e2 = 0.0;
  if (c < cblk[blockIdx.x].y) {
    const double dt = cfl / smax(SR[c], 1.0e-8);
    const d4 rr = r[c], gg = g[c], ln = lam_n[c], lp = lam[c];
    const double e[4] = {rr.x + gg.x, rr.y + gg.y, rr.z + gg.z, rr.w + gg.w};
    const double p[4] = {lp.x, lp.y, lp.z, lp.w}, q[4] = {ln.x, ln.y, ln.z, ln.w};
    double o[4];
    for (int k = 0; k < 4; ++k) {
      const double s = p[k] - dt * e[k];
      o[k] = stage == 0 ? s : (stage == 1 ? 0.75 * q[k] + 0.25 * s : q[k] / 3.0 + 2.0 * s / 3.0);
    }
    lam[c] = d4{o[0], o[1], o[2], o[3]};
    e2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2] + e[3] * e[3];
  }
  if (partial == nullptr) return;
  for (int off = 16; off > 0; off >>= 1) e2 += __shfl_down_sync(0xffffffffu, e2, off);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = e2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += warp_sum[w];
    partial[blockIdx.x] = s;
  }
}

// RMS over n cells of the adjoint residual from the block partials, into hist[*counter];
// the counter advances (one entry per iteration of a captured graph).
static __global__ void k_adj_norm(const double* __restrict__ partial, int nblocks, int n, double* __restrict__ hist,
                                  int* __restrict__ counter, int cap) {
  __shared__ double s[256];
  double a = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) a += partial[b];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int k = *counter;
    if (k < cap) hist[k] = sqrt(s[0] / double(n > 0 ? n : 1));
    *counter = k + 1;
  }
}

// d(F A)/d(alpha) of the far-field faces through the free-stream state (one dual direction;
// dfar is d(farfield conserved state)/d(alpha)), dotted with the owner's adjoint: per face.
template <int FLUX, bool LM>
__global__ void k_adj_dalpha(DevFaces<double> f, const int2* __restrict__ fblk, const FaceParams<double>* __restrict__ fps,
                             const Ctrl* __restrict__ ctrl, const d4* __restrict__ W, d4 dfar,
                             const d4* __restrict__ lam, double* __restrict__ out) {
  using D = ad::Dual<1>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= fblk[blockIdx.x].y) return;
  const int2 oc = f.cells[i];
  if (oc.y != -1) {
    out[i] = 0.0;
    return;
  }
  FaceParams<D> fp = dual_params<1>(scheduled_params(fps[fblk[blockIdx.x].x], ctrl, LM));
  fp.farfield.r.d[0] = dfar.x;
  fp.farfield.ru.d[0] = dfar.y;
  fp.farfield.rv.d[0] = dfar.z;
  fp.farfield.rE.d[0] = dfar.w;
  const d4 w0 = W[oc.x];
  const Prim<D> wo{D(w0.x), D(w0.y), D(w0.z), D(w0.w)};
  D g[8];
  for (int k = 0; k < 8; ++k) g[k] = D(0.0);
  const double2 nd = f.nrm[i];
  Flux<D> fl;
  D mws;
  bool fo = false, df = false;
  eval_face<D, FLUX, false, LM>(fp, -1, wo, wo, g, g, D(nd.x), D(nd.y), D(0.0), D(0.0), D(0.0), D(0.0), &fl, &mws,
                                &fo, &df);
  const d4 l = lam[oc.x];
  out[i] = f.area[i] * (l.x * fl.m.d[0] + l.y * fl.fx.d[0] + l.z * fl.fy.d[0] + l.w * fl.e.d[0]);
}

// ---- vector kernels of the Krylov adjoint solve. Vectors are d4 per cell, n cells; a set
// of vectors is contiguous with stride `ld` cells. Reductions are two-stage with a fixed
// order (per-block partials, then one block per row), so results are deterministic.

__device__ __forceinline__ double dot4(const d4& a, const d4& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}

template <int BS>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < BS / 32; ++w) s += sh[w];
  }
  return s;
}

// partial[r * gridDim.x + block] = sum over the block's cells of V_r . w, r = blockIdx.y.
static __global__ void __launch_bounds__(256) k_vdot_rows(const d4* __restrict__ V, size_t ld, const d4* __restrict__ w,
                                                          int n, double* __restrict__ partial) {
  __shared__ double sh[8];
  const int c = blockIdx.x * 256 + threadIdx.x;
  const int r = blockIdx.y;
  const double v = c < n ? dot4(V[static_cast<size_t>(r) * ld + c], w[c]) : 0.0;
  const double s = block_sum<256>(v, sh);
  if (threadIdx.x == 0) partial[static_cast<size_t>(r) * gridDim.x + blockIdx.x] = s;
}

// out[r] = sum of partial[r][0 .. nb), one block per row.
static __global__ void __launch_bounds__(256) k_rows_sum(const double* __restrict__ partial, int nb,
                                                         double* __restrict__ out) {
  __shared__ double sh[8];
  double a = 0.0;
  for (int b = threadIdx.x; b < nb; b += 256) a += partial[static_cast<size_t>(blockIdx.x) * nb + b];
  const double s = block_sum<256>(a, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// w = alpha * w + sum_{r < rows} coef[r] V_r   (cells c < n)
static __global__ void __launch_bounds__(256) k_vcombine(d4* __restrict__ w, double alpha, const d4* __restrict__ V,
                                                         size_t ld, const double* __restrict__ coef, int rows, int n) {
  const int c = blockIdx.x * 256 + threadIdx.x;
  if (c >= n) return;
  d4 a{0.0, 0.0, 0.0, 0.0};
  if (alpha != 0.0) {  // alpha = 0 does not read w
    a = w[c];
    a = d4{alpha * a.x, alpha * a.y, alpha * a.z, alpha * a.w};
  }
  for (int r = 0; r < rows; ++r) {
    const double k = coef[r];
    const d4 v = V[static_cast<size_t>(r) * ld + c];
    a.x += k * v.x;
    a.y += k * v.y;
    a.z += k * v.z;
    a.w += k * v.w;
  }
  w[c] = a;
}

// y = a * x + b * y   (cells c < n); b = 0 does not read y
static __global__ void __launch_bounds__(256) k_vaxpby(double a, const d4* __restrict__ x, double b,
                                                       d4* __restrict__ y, int n) {
  const int c = blockIdx.x * 256 + threadIdx.x;
  if (c >= n) return;
  const d4 u = x[c];
  if (b == 0.0) {
    y[c] = d4{a * u.x, a * u.y, a * u.z, a * u.w};
    return;
  }
  const d4 v = y[c];
  y[c] = d4{a * u.x + b * v.x, a * u.y + b * v.y, a * u.z + b * v.z, a * u.w + b * v.w};
}

// ---- geometry sensitivities: tangents of the residual along a mesh perturbation dX

template <int N>
__device__ __forceinline__ ad::Dual<N> dual1(double v, double d) {
  ad::Dual<N> r(v);
  r.d[0] = d;
  return r;
}

// Tangent of the Green-Gauss gradients along the geometry tangent (dnrm, darea per slot;
// dinv per cell) at fixed primitives.
static __global__ void k_adj_geo_grad(DevMesh<double> m, const double2* __restrict__ dnrm,
                                      const double* __restrict__ darea, const double* __restrict__ dinv,
                                      const int2* __restrict__ cblk, const d4* __restrict__ W, d4* __restrict__ dgx,
                                      d4* __restrict__ dgy) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cblk[blockIdx.x].y) return;
  const d4 wc = W[c];
  double sx[4] = {0, 0, 0, 0}, sy[4] = {0, 0, 0, 0}, tx[4] = {0, 0, 0, 0}, ty[4] = {0, 0, 0, 0};
  for (int k = 0; k < m.d; ++k) {
    const int s = k * m.n + c;
    const int link = m.link[s];
    if (link == kPad) break;
    const double2 nd = m.nrm[s], dn = dnrm[s];
    const double a = m.area[s], da = darea[s];
    double q[4] = {wc.x, wc.y, wc.z, wc.w};
    double sgn = 1.0;
    if (link >= 0) {
      const d4 wo = W[link >> 1];
      q[0] = 0.5 * (q[0] + wo.x);
      q[1] = 0.5 * (q[1] + wo.y);
      q[2] = 0.5 * (q[2] + wo.z);
      q[3] = 0.5 * (q[3] + wo.w);
      if (link & 1) sgn = -1.0;
    }
    const double nax = nd.x * a, nay = nd.y * a;
    const double dnax = dn.x * a + nd.x * da, dnay = dn.y * a + nd.y * da;
    for (int j = 0; j < 4; ++j) {
      sx[j] += sgn * q[j] * nax;
      sy[j] += sgn * q[j] * nay;
      tx[j] += sgn * q[j] * dnax;
      ty[j] += sgn * q[j] * dnay;
    }
  }
  const double inv = m.inv_vol[c], di = dinv[c];
  dgx[c] = d4{di * sx[0] + inv * tx[0], di * sx[1] + inv * tx[1], di * sx[2] + inv * tx[2], di * sx[3] + inv * tx[3]};
  dgy[c] = d4{di * sy[0] + inv * ty[0], di * sy[1] + inv * ty[1], di * sy[2] + inv * ty[2], di * sy[3] + inv * ty[3]};
}

// Per face: (lam_o - lam_n) . d(F A) along the geometry tangent (normal, length, MUSCL
// offsets, and the gradients' tangent dgx / dgy) at fixed primitives.
template <int FLUX, bool SECOND, bool LM>
__global__ void k_adj_geo_face(DevFaces<double> f, const double2* __restrict__ dfn, const double* __restrict__ dfa,
                               const double2* __restrict__ ddoff, const double2* __restrict__ dnoff,
                               const int2* __restrict__ fblk, const FaceParams<double>* __restrict__ fps,
                               const Ctrl* __restrict__ ctrl, const d4* __restrict__ W, const d4* __restrict__ gx,
                               const d4* __restrict__ gy, const d4* __restrict__ dgx, const d4* __restrict__ dgy,
                               const d4* __restrict__ lam, double* __restrict__ out) {
  using D = ad::Dual<1>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int2 bd = fblk[blockIdx.x];
  if (i >= bd.y) return;
  const FaceParams<D> fp = dual_params<1>(scheduled_params(fps[bd.x], ctrl, LM));
  const int2 oc = f.cells[i];
  const int o = oc.x, b = oc.y;
  const d4 w0 = W[o];
  const d4 w1 = b >= 0 ? W[b] : w0;
  D gO[8], gN[8];
  for (int k = 0; k < 8; ++k) gO[k] = gN[k] = D(0.0);
  D dox(0.0), doy(0.0), dnx(0.0), dny(0.0);
  if (b >= 0 && SECOND) {
    const d4 a = gx[o], c = gy[o], e = gx[b], h = gy[b];
    const d4 da = dgx[o], dc = dgy[o], de = dgx[b], dh = dgy[b];
    const double g0[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
    const double g1[8] = {e.x, e.y, e.z, e.w, h.x, h.y, h.z, h.w};
    const double t0[8] = {da.x, da.y, da.z, da.w, dc.x, dc.y, dc.z, dc.w};
    const double t1[8] = {de.x, de.y, de.z, de.w, dh.x, dh.y, dh.z, dh.w};
    for (int k = 0; k < 8; ++k) {
      gO[k] = dual1<1>(g0[k], t0[k]);
      gN[k] = dual1<1>(g1[k], t1[k]);
    }
    dox = dual1<1>(f.doff[i].x, ddoff[i].x);
    doy = dual1<1>(f.doff[i].y, ddoff[i].y);
    dnx = dual1<1>(f.noff[i].x, dnoff[i].x);
    dny = dual1<1>(f.noff[i].y, dnoff[i].y);
  }
  const double2 nd = f.nrm[i], dn = dfn[i];
  Flux<D> fl;
  D mws;
  bool fo = false, df = false;
  eval_face<D, FLUX, SECOND, LM>(fp, b, Prim<D>{D(w0.x), D(w0.y), D(w0.z), D(w0.w)},
                                 Prim<D>{D(w1.x), D(w1.y), D(w1.z), D(w1.w)}, gO, gN, dual1<1>(nd.x, dn.x),
                                 dual1<1>(nd.y, dn.y), dox, doy, dnx, dny, &fl, &mws, &fo, &df);
  const d4 lo = lam[o];
  d4 a = lo;
  if (b >= 0) {
    const d4 ln = lam[b];
    a = d4{lo.x - ln.x, lo.y - ln.y, lo.z - ln.z, lo.w - ln.w};
  }
  const double A = f.area[i], dA = dfa[i];
  out[i] = a.x * (fl.m.d[0] * A + fl.m.v * dA) + a.y * (fl.fx.d[0] * A + fl.fx.v * dA) +
           a.z * (fl.fy.d[0] * A + fl.fy.v * dA) + a.w * (fl.e.d[0] * A + fl.e.v * dA);
}

// Reverse products of the geometry: the transposes of k_adj_geo_face and k_adj_geo_grad, so
// that dJ/d(every face normal, length and centre, cell volume and centre) comes from one pass
// instead of one tangent per geometry perturbation.
//
// Per face i, with a = lam_o - lam_n (lam_o at a boundary face): the derivatives of a . (F A)
// at fixed primitives and gradients with respect to the face's unit normal (x, y), its length,
// and the MUSCL offsets of the face centre from the owner's and the neighbour's centres:
// out[7 i + 0..6] = (nx, ny, length, dox, doy, dnx, dny). One pass in six-way dual numbers.
template <int FLUX, bool SECOND, bool LM>
__global__ void k_adj_geo_face_vjp(DevFaces<double> f, const int2* __restrict__ fblk,
                                   const FaceParams<double>* __restrict__ fps, const Ctrl* __restrict__ ctrl,
                                   const d4* __restrict__ W, const d4* __restrict__ gx, const d4* __restrict__ gy,
                                   const d4* __restrict__ lam, double* __restrict__ out) {
  using D = ad::Dual<6>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int2 bd = fblk[blockIdx.x];
  if (i >= bd.y) return;
  const FaceParams<D> fp = dual_params<6>(scheduled_params(fps[bd.x], ctrl, LM));
  const int2 oc = f.cells[i];
  const int o = oc.x, b = oc.y;
  const d4 w0 = W[o];
  const d4 w1 = b >= 0 ? W[b] : w0;
  D gO[8], gN[8];
  for (int k = 0; k < 8; ++k) gO[k] = gN[k] = D(0.0);
  D dox(0.0), doy(0.0), dnx(0.0), dny(0.0);
  if (b >= 0 && SECOND) {
    const d4 a = gx[o], c = gy[o], e = gx[b], h = gy[b];
    const double g0[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
    const double g1[8] = {e.x, e.y, e.z, e.w, h.x, h.y, h.z, h.w};
    for (int k = 0; k < 8; ++k) {
      gO[k] = D(g0[k]);
      gN[k] = D(g1[k]);
    }
    dox = ad::seed<6>(f.doff[i].x, 2);
    doy = ad::seed<6>(f.doff[i].y, 3);
    dnx = ad::seed<6>(f.noff[i].x, 4);
    dny = ad::seed<6>(f.noff[i].y, 5);
  }
  const double2 nd = f.nrm[i];
  Flux<D> fl;
  D mws;
  bool fo = false, df = false;
  eval_face<D, FLUX, SECOND, LM>(fp, b, Prim<D>{D(w0.x), D(w0.y), D(w0.z), D(w0.w)},
                                 Prim<D>{D(w1.x), D(w1.y), D(w1.z), D(w1.w)}, gO, gN, ad::seed<6>(nd.x, 0),
                                 ad::seed<6>(nd.y, 1), dox, doy, dnx, dny, &fl, &mws, &fo, &df);
  const d4 lo = lam[o];
  d4 a = lo;
  if (b >= 0) {
    const d4 ln = lam[b];
    a = d4{lo.x - ln.x, lo.y - ln.y, lo.z - ln.z, lo.w - ln.w};
  }
  const double A = f.area[i];
  double dk[6];
  for (int k = 0; k < 6; ++k) dk[k] = A * (a.x * fl.m.d[k] + a.y * fl.fx.d[k] + a.z * fl.fy.d[k] + a.w * fl.e.d[k]);
  double* r = out + 7 * static_cast<size_t>(i);
  r[0] = dk[0];
  r[1] = dk[1];
  r[2] = a.x * fl.m.v + a.y * fl.fx.v + a.z * fl.fy.v + a.w * fl.e.v;
  r[3] = dk[2];
  r[4] = dk[3];
  r[5] = dk[4];
  r[6] = dk[5];
}

// With (mgx, mgy) the adjoint of the Green-Gauss gradients (cell_gradient: G_c = (1/V_c)
// sum_s sgn_s q_s n_s A_s), per slot s = k * n + c the derivatives of mg . G with respect to
// the slot's unit normal (x, y) and length, out_slot[3 s + 0..2], and per cell the derivative
// with respect to 1 / V_c, out_inv[c], at fixed primitives.
static __global__ void k_adj_geo_grad_vjp(DevMesh<double> m, const int2* __restrict__ cblk, const d4* __restrict__ W,
                                          const d4* __restrict__ mgx, const d4* __restrict__ mgy,
                                          double* __restrict__ out_slot, double* __restrict__ out_inv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cblk[blockIdx.x].y) return;
  const d4 wc = W[c], bx = mgx[c], by = mgy[c];
  const double inv = m.inv_vol[c];
  double binv = 0.0;
  for (int k = 0; k < m.d; ++k) {
    const int s = k * m.n + c;
    const int link = m.link[s];
    if (link == kPad) break;
    const double2 nd = m.nrm[s];
    const double a = m.area[s];
    double q[4] = {wc.x, wc.y, wc.z, wc.w};
    double sgn = 1.0;
    if (link >= 0) {
      const d4 wo = W[link >> 1];
      q[0] = 0.5 * (q[0] + wo.x);
      q[1] = 0.5 * (q[1] + wo.y);
      q[2] = 0.5 * (q[2] + wo.z);
      q[3] = 0.5 * (q[3] + wo.w);
      if (link & 1) sgn = -1.0;
    }
    const double px = bx.x * q[0] + bx.y * q[1] + bx.z * q[2] + bx.w * q[3];
    const double py = by.x * q[0] + by.y * q[1] + by.z * q[2] + by.w * q[3];
    const double bnax = inv * sgn * px, bnay = inv * sgn * py;  // d/d(n_x A), d/d(n_y A)
    double* r = out_slot + 3 * static_cast<size_t>(s);
    r[0] = bnax * a;
    r[1] = bnay * a;
    r[2] = bnax * nd.x + bnay * nd.y;
    binv += sgn * (px * nd.x * a + py * nd.y * a);
  }
  out_inv[c] = binv;
}

}  // namespace aero
