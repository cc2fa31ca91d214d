// aero_face_kernels.cuh -- the residual as two passes over a face table: the face pass
// reconstructs, evaluates the flux of every face exactly once (residual_assembly.cpp:73-182)
// and stores F*A and the wave-speed term; the cell pass gathers them. Each cell sums its
// faces in ascending original face order, owner side +, neighbour side -, so the residual is
// the same whatever the cell numbering or block size, and the flux arithmetic is half that
// of evaluating every interior face from both of its cells.
#pragma once

#include "../../include/aero_gb300.h"
#include "aero_kernels.cuh"

namespace aero {

// The arithmetic of one face (residual_assembly.cpp:73-182): MUSCL reconstruction of an
// interior face from the two cells' primitive states and gradients (gO / gN: x then y
// gradients of rho, u, v, p; dO / dN: offsets of the face centre from the cell centres), or
// the boundary state of a boundary face (b = -1 far field, -2 slip wall), then the face
// flux *f and wave-speed term *mws (per unit length). *fo: first-order fallback taken, *df:
// diffusive fallback taken. Templated on the real type: the face pass runs it in float or
// double and the adjoint linearisation in dual numbers.
//
// Interior, far-field and wall faces share one face-state setup, one acoustic-scale call and
// one flux call: a warp holding faces of several kinds runs the flux once, not once per kind.
// Each face's arithmetic is the reference's, operation for operation.
template <class T, int FLUX, bool SECOND, bool LM>
__device__ __forceinline__ void eval_face(const FaceParams<T>& fp, int b, const Prim<T>& wo, const Prim<T>& wn,
                                          const T (&gO)[8], const T (&gN)[8], T nx, T ny, T dox, T doy, T dnx,
                                          T dny, Flux<T>* f, T* mws, bool* fo, bool* df) {
  Prim<T> L = wo, Rt = wn;
  if (SECOND && b >= 0) {
    muscl_var(fp.limiter, wo.r, wn.r, gO[0], gO[4], gN[0], gN[4], dox, doy, dnx, dny, &L.r, &Rt.r);
    muscl_var(fp.limiter, wo.u, wn.u, gO[1], gO[5], gN[1], gN[5], dox, doy, dnx, dny, &L.u, &Rt.u);
    muscl_var(fp.limiter, wo.v, wn.v, gO[2], gO[6], gN[2], gN[6], dox, doy, dnx, dny, &L.v, &Rt.v);
    muscl_var(fp.limiter, wo.p, wn.p, gO[3], gO[7], gN[3], gN[7], dox, doy, dnx, dny, &L.p, &Rt.p);
    L.r = smax(L.r, Kn<T>::rho_floor);
    Rt.r = smax(Rt.r, Kn<T>::rho_floor);
    L.p = smax(L.p, Kn<T>::p_floor);
    Rt.p = smax(Rt.p, Kn<T>::p_floor);
    if (!valid_prim(L) || !valid_prim(Rt)) {
      L = wo;
      Rt = wn;
      *fo = true;
    }
  }
  // owner side: the reconstructed state (interior) or the cell state (boundary); the other
  // side: the neighbour's, the free stream (far field) or the owner's own (slip wall)
  const Cons<T> cl = prim_to_cons_face(L, fp);
  Cons<T> cr = cl;
  if (b >= 0) {
    cr = prim_to_cons_face(Rt, fp);
  } else if (b != -2) {
    cr = fp.farfield;
  }
  // both sides in primitive form, converted once for the acoustic scale and the flux
  FaceSides<T> sd = face_sides(cl, cr, nx, ny, fp.gamma);
  SideMach<T> sm{};
  if (LM) sm = side_mach(sd);
  const T as = face_acoustic_scale<T, LM>(sd, sm, fp);
  if (b == -2) {  // slip wall: pressure-only flux (boundary_conditions.cpp:97-110)
    const Prim<T>& w = sd.pl;
    *f = Flux<T>{T(0), w.p * nx, w.p * ny, T(0)};
    *mws = face_speeds<T, LM>(sd.unl, sd.al, as).sr;
  } else {
    if (b < 0 && fp.precond_farfield_bc) {  // the characteristic state replaces the free stream
      cr = precond_farfield_state(cl, nx, ny, fp, as);
      sd.pr = cons_to_prim(cr, fp.gamma, &sd.ir);
      sd.unr = sd.pr.u * nx + sd.pr.v * ny;
      sd.ar = sound_speed_inv(sd.pr, sd.ir, fp.gamma);
      if (LM) sm = side_mach(sd);
    }
    *f = face_flux<T, FLUX, LM>(cl, cr, sd, sm, nx, ny, fp, as, mws, df);
  }
}

// Face pass. FLUX 0 Rusanov / 1 HLLC; SECOND: MUSCL with the cell gradients; LM: any
// low-Mach feature on. fb[0] / fb[1] count first-order and diffusive fallbacks.
template <class T, int FLUX, bool SECOND, bool LM>
__global__ void __launch_bounds__(256) k_face_flux(DevFaces<T> f, Cases<T> cs,
                                                   const typename Vec<T>::v4* __restrict__ W,
                                                   const typename Vec<T>::v4* __restrict__ gx,
                                                   const typename Vec<T>::v4* __restrict__ gy,
                                                   typename Vec<T>::v4* __restrict__ F, T* __restrict__ FS,
                                                   int* __restrict__ fb_all, const LmSched* __restrict__ lms,
                                                   int parity, int pf) {
  if (pf > 0 && threadIdx.x < 5 && blockIdx.x + pf < gridDim.x) {
    // the face table of the block pf blocks ahead (every block's range is inside the
    // block-padded table): one array per thread
    const size_t f0 = static_cast<size_t>(blockIdx.x + pf) * blockDim.x;
    const unsigned nb = blockDim.x;
    if (threadIdx.x == 0) l2_prefetch(f.cells + f0, nb * sizeof(int2));
    if (threadIdx.x == 1) l2_prefetch(f.nrm + f0, nb * sizeof(f.nrm[0]));
    if (threadIdx.x == 2) l2_prefetch(f.area + f0, nb * sizeof(T));
    if (SECOND && threadIdx.x == 3) l2_prefetch(f.doff + f0, nb * sizeof(f.doff[0]));
    if (SECOND && threadIdx.x == 4) l2_prefetch(f.noff + f0, nb * sizeof(f.noff[0]));
  }
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  // The face's table entries before the case lookup, so that their latency overlaps it
  // (every block lies inside the block-padded table; padding entries go unused). The MUSCL
  // offsets do not depend on the cell ids: loaded with them, not after.
  const int2 oc = f.cells[i];
  const auto nd = f.nrm[i];
  const T area = f.area[i];
  typename Vec<T>::v2 dO{}, dN{};
  if (SECOND) {
    dO = f.doff[i];
    dN = f.noff[i];
  }
  const int2 bd = cs.blk[blockIdx.x];  // face blocks: (case, end of the case's faces)
  pdl_trigger();
  pdl_wait();  // the cells' states and gradients, the controller's flags
  const Ctrl* ctrl = cs.ctrl + bd.x;
  int* fb = fb_all + 4 * bd.x;
  if (ctrl->done) return;
  FaceParams<T> fp = cs.fp[bd.x];
  if (LM && lms) {  // the parity slot of this iteration's low-Mach weights
    const LmSched& q = lms[2 * bd.x + parity];
    fp.as_fix = q.as_fix;
    if constexpr (sizeof(T) == 4) {
      fp.stab_floor = q.stab_f;
      fp.as_fmin = q.as_fmin_f;
      fp.as_ramp = q.as_ramp_f;
    } else {
      fp.stab_floor = q.stab_floor;
      fp.as_fmin = q.as_fmin;
      fp.as_ramp = q.as_ramp;
    }
  } else if (LM) {
    fp.as_fix = ctrl->as_fix;
    if constexpr (sizeof(T) == 4) {
      fp.stab_floor = ctrl->stab_f;
      fp.as_fmin = ctrl->as_fmin_f;
      fp.as_ramp = ctrl->as_ramp_f;
    } else {
      fp.stab_floor = ctrl->stab_floor;
      fp.as_fmin = ctrl->as_fmin;
      fp.as_ramp = ctrl->as_ramp;
    }
  }
  int fo = 0, df = 0;
  if (i < bd.y) {
    const int o = oc.x, b = oc.y;
    const T nx = nd.x, ny = nd.y;
    const auto wo4 = W[o];
    const Prim<T> wo{wo4.x, wo4.y, wo4.z, wo4.w};
    Prim<T> wn = wo;
    T gO[8], gN[8];
    T dox = T(0), doy = T(0), dnx = T(0), dny = T(0);
    if (b >= 0) {
      const auto wn4 = W[b];
      wn = Prim<T>{wn4.x, wn4.y, wn4.z, wn4.w};
      if (SECOND) {
        const auto gOx = gx[o], gOy = gy[o], gNx = gx[b], gNy = gy[b];
        gO[0] = gOx.x; gO[1] = gOx.y; gO[2] = gOx.z; gO[3] = gOx.w;
        gO[4] = gOy.x; gO[5] = gOy.y; gO[6] = gOy.z; gO[7] = gOy.w;
        gN[0] = gNx.x; gN[1] = gNx.y; gN[2] = gNx.z; gN[3] = gNx.w;
        gN[4] = gNy.x; gN[5] = gNy.y; gN[6] = gNy.z; gN[7] = gNy.w;
        dox = dO.x; doy = dO.y; dnx = dN.x; dny = dN.y;
      }
    }
    Flux<T> fl;
    T mws;
    bool fbo = false, fbk = false;
    eval_face<T, FLUX, SECOND, LM>(fp, b, wo, wn, gO, gN, nx, ny, dox, doy, dnx, dny, &fl, &mws, &fbo, &fbk);
    if (fbo) ++fo;
    if (fbk) ++df;
    typename Vec<T>::v4 out;
    out.x = fl.m * area;
    out.y = fl.fx * area;
    out.z = fl.fy * area;
    out.w = fl.e * area;
    F[i] = out;
    FS[i] = mws * area;
  }
  // fallback counters: one atomic per warp when any lane counted something
  const unsigned any = __ballot_sync(0xffffffffu, (fo | df) != 0);
  if (any) {
    const int sfo = __reduce_add_sync(0xffffffffu, fo);
    const int sdf = __reduce_add_sync(0xffffffffu, df);
    if ((threadIdx.x & 31) == __ffs(any) - 1) {
      if (sfo) atomicAdd(&fb[0], sfo);
      if (sdf) atomicAdd(&fb[1], sdf);
    }
  }
}

// Cell pass: R = sum of +-F*A over the cell's faces, SR = sum of the wave-speed terms.
// NORMS (last RK stage): also the residual-norm block partials (euler_solver.cpp:309-339).
// global_dt: per-warp maxima of max(SR, floor) for the global time step.
template <class T, bool NORMS>
__global__ void __launch_bounds__(256) k_gather(DevGather<T> g, const typename Vec<T>::v4* __restrict__ F,
                                                const T* __restrict__ FS, typename Vec<T>::v4* __restrict__ R,
                                                T* __restrict__ SR, Partials part, Cases<T> cs, int global_dt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  // the cell's first slots before the case lookup (every block lies inside the padded table)
  int first[kGatherBatch];
  gather_slots(g, c, 0, first);
  const int2 bd = cs.blk[blockIdx.x];  // cell blocks
  if (cs.ctrl[bd.x].done) return;
  T nq[kNorm] = {T(0), T(0), T(0), T(0)};
  double srm = 0.0;
  if (c < bd.y) {
    T r[4], sr;
    gather_cell<T>(g, F, FS, c, first, r, &sr);
    typename Vec<T>::v4 out;
    out.x = r[0]; out.y = r[1]; out.z = r[2]; out.w = r[3];
    R[c] = out;
    SR[c] = sr;
    if (global_dt) srm = double(smax(sr, Kn<T>::wave_floor));
    if (NORMS) norm_terms<T>(r, g.inv_vol[c], nq);
  }
  if (global_dt) {
    srm = warp_max(srm);
    if ((threadIdx.x & 31) == 0) part.srmax[blockIdx.x * ((blockDim.x + 31) >> 5) + (threadIdx.x >> 5)] = srm;
  }
  if (NORMS) block_norms<T>(nq, part);
}

// Launch geometry and buffers of one residual evaluation. faces.nf and gather.n are the
// packed (block-padded) face and cell counts of all cases.
template <class T>
struct ResidualLaunch {
  int block;
  cudaStream_t st;
  DevFaces<T> faces;
  DevGather<T> gather;
  Cases<T> face_cases;  // blk over face blocks
  Cases<T> cell_cases;  // blk over cell blocks
  const typename Vec<T>::v4 *W, *gx, *gy;
  typename Vec<T>::v4* F;  // per face
  T* FS;                   // per face
  typename Vec<T>::v4* R;  // per cell
  T* SR;                   // per cell
  Partials part;
  int* fb;                 // [case][2]: fallback counters, stride 4 per case
  int global_dt;
  const LmSched* lms = nullptr;  // parity slots of the low-Mach weights (null: read the controller)
  int parity = 0;
  bool pdl = false;  // launch the face pass with programmatic stream serialization
};

template <class T, int FLUX, bool SECOND, bool LM>
void launch_face_flux_t(const ResidualLaunch<T>& a) {
  const int grid = (a.faces.nf + a.block - 1) / a.block;
  auto kern = k_face_flux<T, FLUX, SECOND, LM>;
  const int pf = resident_blocks(kern, a.block);
  launch_kernel(kern, grid, a.block, 0, a.st, a.pdl, a.faces, a.face_cases, a.W, a.gx, a.gy, a.F, a.FS, a.fb, a.lms,
                a.parity, pf);
}

// Face pass, dispatched on the flux, order and low-Mach switches.
template <class T>
void launch_face_pass(const ResidualLaunch<T>& a, int flux, bool second, bool lm) {
  if (flux == AERO_FLUX_HLLC) {
    if (second) {
      if (lm) launch_face_flux_t<T, 1, true, true>(a);
      else launch_face_flux_t<T, 1, true, false>(a);
    } else {
      if (lm) launch_face_flux_t<T, 1, false, true>(a);
      else launch_face_flux_t<T, 1, false, false>(a);
    }
  } else {
    if (second) {
      if (lm) launch_face_flux_t<T, 0, true, true>(a);
      else launch_face_flux_t<T, 0, true, false>(a);
    } else {
      if (lm) launch_face_flux_t<T, 0, false, true>(a);
      else launch_face_flux_t<T, 0, false, false>(a);
    }
  }
}

// Cell pass into a.R / a.SR (with the norm partials when `norms`).
template <class T>
void launch_gather_pass(const ResidualLaunch<T>& a, bool norms) {
  const int grid = (a.gather.n + a.block - 1) / a.block;
  if (norms) {
    k_gather<T, true><<<grid, a.block, 0, a.st>>>(a.gather, a.F, a.FS, a.R, a.SR, a.part, a.cell_cases,
                                                   a.global_dt);
  } else {
    k_gather<T, false><<<grid, a.block, 0, a.st>>>(a.gather, a.F, a.FS, a.R, a.SR, a.part, a.cell_cases,
                                                    a.global_dt);
  }
}

// Face pass then cell pass.
template <class T>
void launch_residual_passes(const ResidualLaunch<T>& a, int flux, bool second, bool lm, bool norms) {
  launch_face_pass(a, flux, second, lm);
  launch_gather_pass(a, norms);
}

}  // namespace aero
