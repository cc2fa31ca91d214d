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
#include <mutex>
#include <utility>
#include <vector>

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

// Hint to bring [p, p + bytes) into L2: one bulk prefetch with no completion to wait for
// (p 16-byte aligned, bytes a multiple of 16). The streaming kernels issue it for the block
// that will run `pf` blocks later, the blocks resident on the whole GPU at once, so that the
// block's coalesced loads, issued before its gathers can start, hit L2 instead of DRAM.
__device__ __forceinline__ void l2_prefetch(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "r"(bytes)
               : "memory");
}

// Programmatic dependent launch (opt-in per context: AERO_PDL=1). The iteration's gradient,
// face and update kernels may be launched with programmatic stream serialization: such a
// kernel starts while its
// predecessor in the stream is still running, once every block of the predecessor has
// called pdl_trigger() (each does so on entry, so the successor's blocks take the SM slots
// the predecessor's last wave frees). Before pdl_wait() a kernel reads only tables no kernel
// writes (face and slot tables, geometry, case blocks); pdl_wait() returns once the
// predecessor grids have completed and their writes are visible. Both are no-ops in a kernel
// launched without the attribute.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launches kernel<<<grid, block, smem, st>>>(args...), with programmatic stream serialization
// when `pdl` is set.
template <class... P, class... A>
inline cudaError_t launch_kernel(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl,
                                 A&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  if (pdl) {
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

// Blocks of `kernel` at `block` threads resident on the whole device at once (occupancy x
// SM count): the prefetch distance of the streaming kernels. Host side; the answer is kept
// per kernel, block size and device, so a launch queries the runtime once.
template <class K>
inline int resident_blocks(K kernel, int block) {
  struct Entry {
    const void* k;
    int block, dev, blocks;
  };
  static std::mutex mu;
  static std::vector<Entry> seen;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const void* key = reinterpret_cast<const void*>(kernel);
  {
    std::lock_guard<std::mutex> lock(mu);
    for (const Entry& e : seen) {
      if (e.k == key && e.block == block && e.dev == dev) return e.blocks;
    }
  }
  int per_sm = 0, sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  std::lock_guard<std::mutex> lock(mu);
  seen.push_back(Entry{key, block, dev, per_sm * sms});
  return per_sm * sms;
}

// Controller and per-iteration state (device memory, one per context).
struct alignas(16) Ctrl {
  int iter;        // index of the next iteration to run
  int done;        // converged or trapped: kernels return immediately
  int nonfinite;   // set by the last-stage update when the state is not finite
  int rec_base;    // iteration number stored at records[0] of the current chunk
  int second;      // second order in the current iteration
  int as_fix;      // all-speed fix effective in the current iteration
  int fo_fallback; // fallback counters of a single residual evaluation (the iteration loop
  int diff_fallback;  // counts into a separate per-parity array, see k_residual)
  double cfl, stab_floor, as_fmin, as_ramp;  // current-iteration schedule values
  double cfl_scale, prev_l2, initial_l2;
  int has_prev, hist_count, hist_head, stage;  // stage: 0 single, 1 A, 2 B
  double prev_cl, prev_cd, prev_cm;
  double hist[3 * 2 * kMaxForceWindow];
  double stage_b_fmin;
  int stage_b_progress, pjump_below, freeze;
  int wait_stop;   // set by the updates of an iteration whose gradient pass gave up a wait
  float cfl_f, stab_f, as_fmin_f, as_ramp_f;  // float copies of the schedule values (FP32 kernels)
  double sr_max;  // global max of max(SR, floor) for global time stepping
  double initial_l2rho;  // first density-residual L2 (< 0: not yet seen)
  double pad1;
};

// Run constants of the controller (euler_solver.cpp:463-566 resolved on the host).
struct CtrlConfig {
  int n_cells, n_wall, rk_stages, local_dt;
  int cfl_ramp, stab_ramp, as_ramp_start, as_ramp_iters;
  int startup_first_order, min_iterations, window, staged;
  int st_a_min, st_a_max, pj_hold, freeze_iters;
  int as_fix_cfg, n_blocks, pjump_blocks, n_wall_blocks;
  int bulk_f32;    // partials hold float norms and float monitor bits
  int block_base;  // the case's first cell block (its partials are blocks [base, base + n_blocks))
  int wall_base;   // the case's first slot in Partials::wall / wall_f
  double cfl_start, cfl_max, stab_start, stab_target, as_fmin;
  double residual_target, stab_tol, drift_tol;
  double st_fmin_high, st_fmin_mid, st_fmin_low;
  double pj_target, pj_spike, cfl_drop, cfl_restore, cfl_min_scale;
  double p_inf, q_inf, s_ref, chord, cos_a, sin_a, x_ref, y_ref, pressure_ref, gamma;
  double rho_inf, u_inf, v_inf;
  double rho_l2_target;  // > 0: also stop when the density-residual L2 ratio falls to it
};

// Precondition constants in double for the residual preconditioner (preconditioning.cpp:51-76).
struct PrecondD {
  int enabled;
  int fp64;  // FP32 contexts: energy row 0 float, 1 IEEE double (beta too), 2 double-float
  double gamma, mach_ref, mach_min, beta_min, beta_max;
  float gamma_f, gm1_f;  // float(gamma), float(gamma - 1)
  double pfe;            // p_floor / (gamma - 1) in double: the energy floor of enforce_physical
  float mach_ref_f, mach_min_f, beta_min_f, beta_max_f;  // float copies (FP32 update)
};

// Schedule of iteration s->iter (euler_solver.cpp:69-112 and 772-797): order switch,
// CFL ramp times the adaptive scale, stabilization-floor ramp, all-speed weights. Used by
// the controller for the next iteration and by the host for iteration 0. SchedBase is the
// part that depends on the iteration index alone.
struct SchedBase {
  int second;
  double cfl_base, stab_floor, as_ramp;  // as_ramp: the non-staged all-speed ramp
};
__host__ __device__ inline SchedBase schedule_base(const CtrlConfig& cc, int it) {
  SchedBase b;
  b.second = it >= (cc.startup_first_order > 0 ? cc.startup_first_order : 0);
  if (cc.cfl_ramp <= 0) {
    b.cfl_base = cc.cfl_max;
  } else {
    const double t = smin(1.0, double(it + 1) / double(cc.cfl_ramp > 1 ? cc.cfl_ramp : 1));
    b.cfl_base = cc.cfl_start + t * (cc.cfl_max - cc.cfl_start);
  }
  {
    const double m0s = sclamp(cc.stab_start, 0.0, 1.0), m0t = sclamp(cc.stab_target, 0.0, 1.0);
    if (cc.stab_ramp <= 0) {
      b.stab_floor = m0t;
    } else {
      const double t =
          sclamp(double(it > 0 ? it : 0) / double(cc.stab_ramp > 1 ? cc.stab_ramp : 1), 0.0, 1.0);
      b.stab_floor = m0s + t * (m0t - m0s);
    }
  }
  if (cc.as_ramp_iters <= 0) {
    b.as_ramp = (it >= cc.as_ramp_start) ? 1.0 : 0.0;
  } else {
    b.as_ramp = sclamp(double(it - cc.as_ramp_start) / double(cc.as_ramp_iters > 1 ? cc.as_ramp_iters : 1),
                       0.0, 1.0);
  }
  return b;
}

// Schedule of iteration s->iter from its iteration-only part b = schedule_base(cc, s->iter).
__host__ __device__ inline void apply_schedule_from(const CtrlConfig& cc, const SchedBase& b, Ctrl* sp) {
  Ctrl& s = *sp;
  s.second = b.second;
  s.cfl = b.cfl_base * s.cfl_scale;
  s.stab_floor = b.stab_floor;
  if (!cc.staged) {
    s.as_fix = cc.as_fix_cfg;
    s.as_fmin = cc.as_fmin;
    s.as_ramp = b.as_ramp;
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
  s.cfl_f = float(s.cfl);
  s.stab_f = float(s.stab_floor);
  s.as_fmin_f = float(s.as_fmin);
  s.as_ramp_f = float(s.as_ramp);
}

__host__ __device__ inline void apply_schedule(const CtrlConfig& cc, Ctrl* sp) {
  apply_schedule_from(cc, schedule_base(cc, sp->iter), sp);
}

// Low-Mach weights of one iteration's face passes under a schedule without the staged
// controller (they then depend on the iteration index alone): the values apply_schedule
// gives, kept per iteration parity so that an iteration's face passes can read them while
// the previous iteration's controller is still running.
struct alignas(16) LmSched {
  int as_fix, pad;
  double stab_floor, as_fmin, as_ramp;
  float stab_f, as_fmin_f, as_ramp_f, pad_f;
};
__host__ __device__ inline LmSched lm_sched_of(const CtrlConfig& cc, int it) {
  const SchedBase b = schedule_base(cc, it);
  LmSched q;
  q.as_fix = cc.as_fix_cfg;
  q.pad = 0;
  q.stab_floor = b.stab_floor;
  q.as_fmin = cc.as_fmin;
  q.as_ramp = b.as_ramp;
  q.stab_f = float(q.stab_floor);
  q.as_fmin_f = float(q.as_fmin);
  q.as_ramp_f = float(q.as_ramp);
  q.pad_f = 0.0f;
  return q;
}

// Schedule values of a single residual evaluation (aero_residual and its no-allocation form).
__host__ __device__ inline void set_eval_schedule(Ctrl* s, double stab, int as_fix, double as_fmin, double as_ramp) {
  s->stab_floor = stab;
  s->as_fix = as_fix;
  s->as_fmin = as_fmin;
  s->as_ramp = as_ramp;
  s->stab_f = float(stab);
  s->as_fmin_f = float(as_fmin);
  s->as_ramp_f = float(as_ramp);
}

// Per-cell slot table of the gradient and pressure-jump passes, in the bulk type T: the
// normals and areas are exact conversions of the mesh's double geometry and inv_vol =
// 1/max(V, 1e-12) is formed in T on the host, so FP32 kernels do neither double loads nor
// double conversions or divides.
template <class T>
struct DevMesh {
  int n, d;
  const int* link;
  const typename Vec<T>::v2* nrm;
  const T* area;
  const T* inv_vol;
  // per gradient slot, the face vector n * A formed in T as nrm * area, halved for a slot with
  // a neighbour: the Green-Gauss sums multiply the two cells' sum by it, which is exactly the
  // product of their average and n * A (halving is exact)
  const typename Vec<T>::v2* gvec;
};

// Faces sorted by the new index of their owner. cells = (owner, neighbour) new indices, the
// neighbour -1 for a far-field face and -2 for a slip wall. Geometry in the bulk type T:
// unit normal out of the owner, length, and the offsets of the face centre from the owner's
// and the neighbour's centres (MUSCL).
template <class T>
struct DevFaces {
  int nf;
  const int2* cells;
  const typename Vec<T>::v2* nrm;
  const T* area;
  const typename Vec<T>::v2* doff;
  const typename Vec<T>::v2* noff;
};

// Per-cell gather table (ELL, slot (k, c) at k*n + c): (face << 1) | (cell is the
// neighbour), kPad after the last face of the cell.
template <class T>
struct DevGather {
  int n, d;
  const int* slot;
  const T* inv_vol;
};

// Per-block partial results reduced by the control kernel in a fixed order. Quantity-major
// ([k][block]) so that the control warp reads them coalesced.
struct Partials {
  double* norms;   // [kNorm][nb]: l1, l2 sum, linf, density l2 sum (FP64)
  float* norms_f;  // [kNorm][nb]: the same in float (FP32)
  long long* mon;  // [kMon][nb]: maxima of |p - p_inf| (domain, wall-adjacent) and the far-field
                   // deviations |dp|, |drho|, |du|, |dv|, formed in the bulk type; stored as bit
                   // patterns (double, or float zero-extended) so that maxima are integer maxima
  double* wall;    // [kWall][nwb]: force sums and wall monitors of blocks holding wall cells (FP64)
  float* wall_f;   // [kWall][nwb]: the same in float (FP32)
  double* pjump;   // [4][nb]: sum dp^2, count, wall sum, wall count
  double* srmax;   // [blocks * warps per block]: max of max(SR, floor)
  int nb, nwb;     // blocks of the cell grid, blocks holding wall cells
};
constexpr int kNorm = 4;
constexpr int kMon = 6;
constexpr int kWall = 12;  // snx sny fxa fya fxg fyg ma mg | un_max cp_hi -cp_lo cp_bad

// End-of-iteration monitors (euler_solver.cpp:923-1026, forces.cpp:208-294) computed by the
// cells that own wall or far-field faces, while the new state is in registers.
struct MonitorSet {
  const unsigned char* flags;  // per cell: bit 0 owns slip-wall faces, bit 1 owns far-field
                               // faces, bits 2..7 number of wall entries
  const int* wall_first;       // per cell: its first wall entry
  const unsigned char* wkind;  // wall entries sorted by owner: bit 0 force patch face, bit 1
                               // slip-wall face (wall monitors);
  const double* wnx;           // unit normal out of the owner, length and centre
  const double* wny;
  const double* warea;
  const double* wx;
  const double* wy;
  const int* block_slot;       // per cell block: its slot in Partials::wall, or -1
  const float *wnx_f, *wny_f, *warea_f, *wx_f, *wy_f;  // float copies (FP32)
};

// Free-stream and reference constants of one case for the monitors and forces.
struct MonitorConsts {
  double p_inf, rho_inf, u_inf, v_inf, q_inf, x_ref, y_ref, gamma;
  float p_inf_f, rho_inf_f, u_inf_f, v_inf_f, q_inf_f, x_ref_f, y_ref_f;  // float copies (FP32)
  int sym_interval;  // AoA-0 symmetry every this many iterations, 0 = off
};

// The cases of a launch. Cases are packed one after another, each padded to whole blocks,
// so every block belongs to one case: blk[blockIdx.x] = (case, end of that case's range)
// over cells or faces. Per-case parameters are arrays indexed by the case. A single case
// is a batch of one.
template <class T>
struct Cases {
  const int2* blk;
  Ctrl* ctrl;
  const FaceParams<T>* fp;
  const PrecondD* pc;
  const MonitorConsts* mc;
  // wait[0]: nonzero once a kernel of the iteration gave up a bounded wait (its outputs are
  // then incomplete); wait[1]: the poll limit of those waits. Null outside the iterations.
  const int* wait = nullptr;
};

// Conserved state of the cells. FP64 holds it as double4; FP32 as a float-float pair: hi is
// the float image and lo the remainder (|lo| <= ulp(hi)/2), so that the state accumulates to
// about 2^-47 relative across iterations with float arithmetic only (a GB300 SM runs double
// arithmetic, and float<->double conversions even more so, at a small fraction of the float
// rate).
struct StateRef {
  d4* un;      // FP64
  float4* hi;  // FP32
  float4* lo;  // FP32
};

// Error-free float sum (Knuth's two-sum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float* s, float* e) {
  const float x = __fadd_rn(a, b);
  const float bb = __fsub_rn(x, a);
  *e = __fadd_rn(__fsub_rn(a, __fsub_rn(x, bb)), __fsub_rn(b, bb));
  *s = x;
}
// (hi, lo) + d as a renormalised float-float pair.
__device__ __forceinline__ void ff_add(float hi, float lo, float d, float* nh, float* nl) {
  float s, e;
  two_sum(hi, d, &s, &e);
  two_sum(s, __fadd_rn(lo, e), nh, nl);
}
// (ah, al) + (bh, bl) as a renormalised float-float pair.
__device__ __forceinline__ void ff_add2(float ah, float al, float bh, float bl, float* nh, float* nl) {
  float s, e;
  two_sum(ah, bh, &s, &e);
  two_sum(s, __fadd_rn(__fadd_rn(al, bl), e), nh, nl);
}
__device__ __forceinline__ void ff_split(double u, float* hi, float* lo) {
  *hi = float(u);
  *lo = float(u - double(*hi));
}

template <class T>
__device__ __forceinline__ Cons<double> load_state(const StateRef& u, int c) {
  if constexpr (sizeof(T) == 4) {
    const float4 h = u.hi[c], l = u.lo[c];
    return Cons<double>{double(h.x) + double(l.x), double(h.y) + double(l.y), double(h.z) + double(l.z),
                        double(h.w) + double(l.w)};
  } else {
    const d4 x = u.un[c];
    return Cons<double>{x.x, x.y, x.z, x.w};
  }
}
template <class T>
__device__ __forceinline__ void store_state(const StateRef& u, int c, const Cons<double>& s) {
  if constexpr (sizeof(T) == 4) {
    float4 h, l;
    ff_split(s.r, &h.x, &l.x);
    ff_split(s.ru, &h.y, &l.y);
    ff_split(s.rv, &h.z, &l.z);
    ff_split(s.rE, &h.w, &l.w);
    u.hi[c] = h;
    u.lo[c] = l;
  } else {
    u.un[c] = d4{s.r, s.ru, s.rv, s.rE};
  }
}

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
template <class T>
__device__ __forceinline__ T warp_sum_t(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
template <class T>
__device__ __forceinline__ T warp_max_t(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = smax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}
// Warp maximum of values that are >= 0 (or NaN): for float one warp-reduce instruction on the
// bit patterns, which order like the values; a NaN lane makes the result NaN.
template <class T>
__device__ __forceinline__ T warp_max_nonneg(T x) {
  if constexpr (sizeof(T) == 4) {
    return __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(x)));
  } else {
    return warp_max_t(x);
  }
}

// The first kGatherBatch gather slots of cell c (kPad beyond the table's d).
constexpr int kGatherBatch = 4;
template <class T>
__device__ __forceinline__ void gather_slots(const DevGather<T>& g, int c, int k0, int (&sl)[kGatherBatch]) {
#pragma unroll
  for (int u = 0; u < kGatherBatch; ++u) sl[u] = (k0 + u < g.d) ? g.slot[(k0 + u) * g.n + c] : kPad;
}

// Residual of cell c from the per-face fluxes: +-F*A over its faces in ascending original
// face order, and the sum of the faces' wave-speed terms. The slots are read first so the
// flux loads of one cell are in flight together; `first`, when given, holds the first batch
// of slots, loaded by the caller (gather_slots(g, c, 0, first)) ahead of its other work.
template <class T>
__device__ __forceinline__ void gather_cell(const DevGather<T>& g, const typename Vec<T>::v4* __restrict__ F,
                                            const T* __restrict__ FS, int c, const int* first, T (&r)[4], T* sr) {
  constexpr int kU = kGatherBatch;
  r[0] = r[1] = r[2] = r[3] = T(0);
  *sr = T(0);
  for (int k0 = 0; k0 < g.d; k0 += kU) {
    int sl[kU];
    if (k0 == 0 && first != nullptr) {
#pragma unroll
      for (int u = 0; u < kU; ++u) sl[u] = first[u];
    } else {
      gather_slots(g, c, k0, sl);
    }
    typename Vec<T>::v4 fv[kU];
    T fs[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if (sl[u] != kPad) {
        fv[u] = F[sl[u] >> 1];
        fs[u] = FS[sl[u] >> 1];
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if (sl[u] == kPad) break;
      if (sl[u] & 1) {
        r[0] -= fv[u].x; r[1] -= fv[u].y; r[2] -= fv[u].z; r[3] -= fv[u].w;
      } else {
        r[0] += fv[u].x; r[1] += fv[u].y; r[2] += fv[u].z; r[3] += fv[u].w;
      }
      *sr += fs[u];
    }
    if (sl[kU - 1] == kPad) break;
  }
}

// Residual-norm terms of one cell (euler_solver.cpp:309-339): |R|/V summed, squared, max;
// q[3] is the density component squared (the batched sweep's stop rule).
template <class T>
__device__ __forceinline__ void norm_terms(const T (&r)[4], T inv, T (&q)[kNorm]) {
  const T v0 = r[0] * inv, v1 = r[1] * inv, v2 = r[2] * inv, v3 = r[3] * inv;
  const T a0 = fabs(v0), a1 = fabs(v1), a2 = fabs(v2), a3 = fabs(v3);
  q[0] = ((a0 + a1) + a2) + a3;
  q[1] = ((v0 * v0 + v1 * v1) + v2 * v2) + v3 * v3;
  q[2] = smax(smax(smax(a0, a1), a2), a3);
  q[3] = v0 * v0;
}

// Block partials of the norm terms in T into Partials::norms / norms_f; the control kernel
// sums the blocks in double (FP32: float-float). Called by every thread of the block.
template <class T>
__device__ void block_norms(T (&q)[kNorm], Partials part) {
  __shared__ T shn[kNorm][32];
  q[0] = warp_sum_t(q[0]);
  q[1] = warp_sum_t(q[1]);
  q[2] = warp_max_nonneg(q[2]);
  q[3] = warp_sum_t(q[3]);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < kNorm; ++k) shn[k][wid] = q[k];
  }
  __syncthreads();
  // one term per thread, each over the warps in order
  if (threadIdx.x < kNorm) {
    const int k = threadIdx.x;
    T a = T(0);
    for (int i = 0; i < nw; ++i) a = (k == 2) ? smax(a, shn[2][i]) : a + shn[k][i];
    T* out;
    if constexpr (sizeof(T) == 4) {
      out = part.norms_f;
    } else {
      out = part.norms;
    }
    out[k * part.nb + blockIdx.x] = a;
  }
}

// Monitors of one cell after the last stage (euler_solver.cpp:923-1026, forces.cpp:208-294),
// from the bulk primitive state w in the bulk type T, reduced per block: maxima into
// Partials::mon (every block), force sums and wall monitors into Partials::wall / wall_f
// (only blocks holding wall cells). FP32 forms all of it in float: a GB300 SM runs double
// arithmetic at a small fraction of its float rate, and the blocks are combined in double by
// the control kernel. Must be called by every thread of the block; `valid` is false past the
// mesh.
template <class T>
__device__ void block_monitors(bool valid, const Prim<T>& w, int c, const MonitorSet& ms, const MonitorConsts& mc,
                               Partials part) {
  constexpr bool kF = sizeof(T) == 4;
  constexpr T kLow = kF ? T(-3.0e38f) : T(-1.0e308);
  __shared__ T shf[kMon][32];
  __shared__ T shd[kWall][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const T p_inf = kF ? T(mc.p_inf_f) : T(mc.p_inf);
  T mon[kMon] = {T(0), T(0), T(0), T(0), T(0), T(0)};
  unsigned char fl = 0;
  if (valid) {
    fl = ms.flags[c];
    const T dp = fabs(w.p - p_inf);
    mon[0] = dp;
    if (fl & 1) mon[1] = dp;
    if (fl & 2) {
      mon[2] = dp;
      mon[3] = fabs(w.r - (kF ? T(mc.rho_inf_f) : T(mc.rho_inf)));
      mon[4] = fabs(w.u - (kF ? T(mc.u_inf_f) : T(mc.u_inf)));
      mon[5] = fabs(w.v - (kF ? T(mc.v_inf_f) : T(mc.v_inf)));
    }
  }
#pragma unroll
  for (int k = 0; k < kMon; ++k) mon[k] = warp_max_nonneg(mon[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < kMon; ++k) shf[k][wid] = mon[k];
  }
  const int slot = ms.block_slot[blockIdx.x];
  if (slot >= 0) {
    // snx sny fxa fya fxg fyg ma mg | un_max cp_hi -cp_lo cp_bad
    T v[kWall] = {T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0), kLow, kLow, T(0)};
    if (valid && fl >= 4) {
      const T* wnx = kF ? reinterpret_cast<const T*>(ms.wnx_f) : reinterpret_cast<const T*>(ms.wnx);
      const T* wny = kF ? reinterpret_cast<const T*>(ms.wny_f) : reinterpret_cast<const T*>(ms.wny);
      const T* wa = kF ? reinterpret_cast<const T*>(ms.warea_f) : reinterpret_cast<const T*>(ms.warea);
      const T* wx = kF ? reinterpret_cast<const T*>(ms.wx_f) : reinterpret_cast<const T*>(ms.wx);
      const T* wy = kF ? reinterpret_cast<const T*>(ms.wy_f) : reinterpret_cast<const T*>(ms.wy);
      const T x_ref = kF ? T(mc.x_ref_f) : T(mc.x_ref), y_ref = kF ? T(mc.y_ref_f) : T(mc.y_ref);
      const T q_inf = kF ? T(mc.q_inf_f) : T(mc.q_inf);
      const int first = ms.wall_first[c], cnt = fl >> 2;
      const T p = w.p, gp = w.p - p_inf;
      for (int j = first; j < first + cnt; ++j) {
        const unsigned char kind = ms.wkind[j];
        if (kind & 1) {  // forces.cpp:208-294
          const T nax = -wnx[j] * wa[j];
          const T nay = -wny[j] * wa[j];
          const T x = wx[j] - x_ref, y = wy[j] - y_ref;
          v[0] += nax;
          v[1] += nay;
          v[2] -= p * nax;
          v[3] -= p * nay;
          v[4] -= gp * nax;
          v[5] -= gp * nay;
          v[6] += x * (-p * nay) - y * (-p * nax);
          v[7] += x * (-gp * nay) - y * (-gp * nax);
        }
        if (kind & 2) {  // euler_solver.cpp:976-1006
          v[8] = smax(v[8], fabs(w.u * wnx[j] + w.v * wny[j]));
          const T cp = sdiv(gp, q_inf);
          if (isfinite(cp)) {
            v[9] = smax(v[9], cp);
            v[10] = smax(v[10], -cp);
          } else {
            v[11] += T(1);
          }
        }
      }
    }
    if (__any_sync(0xffffffffu, valid && fl >= 4)) {
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = warp_sum_t(v[k]);
#pragma unroll
      for (int k = 8; k < 11; ++k) v[k] = warp_max_t(v[k]);
      v[11] = warp_sum_t(v[11]);
    }
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < kWall; ++k) shd[k][wid] = v[k];
    }
  }
  __syncthreads();
  // one quantity per thread, each over the warps in order: the maxima on threads
  // 0..kMon-1, the wall sums and maxima on threads 32..32+kWall-1
  const int t = threadIdx.x;
  if (t < kMon) {
    T m = T(0);
    for (int i = 0; i < nw; ++i) m = smax(m, shf[t][i]);
    if constexpr (kF) {
      part.mon[t * part.nb + blockIdx.x] = static_cast<long long>(__float_as_uint(m));
    } else {
      part.mon[t * part.nb + blockIdx.x] = __double_as_longlong(m);
    }
  }
  const int k = t - 32;
  if (slot >= 0 && k >= 0 && k < kWall) {
    T* out;
    if constexpr (kF) {
      out = part.wall_f;
    } else {
      out = part.wall;
    }
    T a = (k == 9 || k == 10) ? kLow : T(0);
    for (int i = 0; i < nw; ++i) a = (k >= 8 && k <= 10) ? smax(a, shd[k][i]) : a + shd[k][i];
    out[k * part.nwb + slot] = a;
  }
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
// Green-Gauss gradient of cell c (reconstruction.cpp:73-119): the face averages of the
// primitive state times the outward face vectors, over 1/V. sW (may be null) holds W of the
// cells [base, base + nsw): neighbours in that range are read from shared memory.
// One batch of a cell's gradient slots: links and face vectors (DevMesh::gvec) of slots
// k0 .. k0 + 3. The slot geometry does not depend on the links (padding slots hold zeros), so
// its loads go out with the links' and only the neighbour states wait for them.
constexpr int kGradBatch = 4;
template <class T>
struct GradSlots {
  int lk[kGradBatch];
  typename Vec<T>::v2 gv[kGradBatch];
};
template <class T>
__device__ __forceinline__ void grad_slots(const DevMesh<T>& m, int c, int k0, GradSlots<T>* sb) {
#pragma unroll
  for (int u = 0; u < kGradBatch; ++u) {
    sb->lk[u] = kPad;
    sb->gv[u] = typename Vec<T>::v2{};
    if (k0 + u < m.d) {
      const int s = (k0 + u) * m.n + c;
      sb->lk[u] = m.link[s];
      sb->gv[u] = m.gvec[s];
    }
  }
}
// One slot's terms of the Green-Gauss sums: q is the cell's state, plus the neighbour's for a
// slot with one (g is then half the face vector), times the face vector; subtracted when the
// cell is the face's neighbour.
template <class T>
__device__ __forceinline__ void grad_slot_terms(int link, const typename Vec<T>::v4& wc, const typename Vec<T>::v4& wo,
                                                const typename Vec<T>::v2& g, T (&ax)[4], T (&ay)[4]) {
  const T gx = g.x, gy = g.y;
  T q0 = wc.x, q1 = wc.y, q2 = wc.z, q3 = wc.w;
  bool minus = false;
  if (link >= 0) {
    q0 = q0 + wo.x;
    q1 = q1 + wo.y;
    q2 = q2 + wo.z;
    q3 = q3 + wo.w;
    minus = (link & 1) != 0;
  }
  if (minus) {
    ax[0] -= q0 * gx; ay[0] -= q0 * gy;
    ax[1] -= q1 * gx; ay[1] -= q1 * gy;
    ax[2] -= q2 * gx; ay[2] -= q2 * gy;
    ax[3] -= q3 * gx; ay[3] -= q3 * gy;
  } else {
    ax[0] += q0 * gx; ay[0] += q0 * gy;
    ax[1] += q1 * gx; ay[1] += q1 * gy;
    ax[2] += q2 * gx; ay[2] += q2 * gy;
    ax[3] += q3 * gx; ay[3] += q3 * gy;
  }
}

template <class T>
__device__ __forceinline__ void cell_gradient(const DevMesh<T>& m, const typename Vec<T>::v4* __restrict__ W, int c,
                                              typename Vec<T>::v4* gxo, typename Vec<T>::v4* gyo,
                                              const typename Vec<T>::v4* sW = nullptr, int base = 0, int nsw = 0) {
  const auto wc = sW ? sW[c - base] : W[c];
  T ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0};
  // slots in batches of kU: the links first, then every load of the batch, then the sums in
  // slot order, so the neighbour loads of one cell are in flight together
  constexpr int kU = kGradBatch;
  for (int k0 = 0; k0 < m.d; k0 += kU) {
    GradSlots<T> sb;
    grad_slots(m, c, k0, &sb);
    const int(&lk)[kU] = sb.lk;
    typename Vec<T>::v4 wo[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if (lk[u] >= 0) {
        const int o = lk[u] >> 1;
        const unsigned off = static_cast<unsigned>(o - base);
        wo[u] = (sW && off < static_cast<unsigned>(nsw)) ? sW[off] : W[o];
      } else {
        wo[u] = wc;
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if (lk[u] == kPad) break;
      grad_slot_terms<T>(lk[u], wc, wo[u], sb.gv[u], ax, ay);
    }
    if (lk[kU - 1] == kPad) break;
  }
  const T inv = m.inv_vol[c];
  typename Vec<T>::v4& ox = *gxo;
  typename Vec<T>::v4& oy = *gyo;
  ox.x = ax[0] * inv; ox.y = ax[1] * inv; ox.z = ax[2] * inv; ox.w = ax[3] * inv;
  oy.x = ay[0] * inv; oy.y = ay[1] * inv; oy.z = ay[2] * inv; oy.w = ay[3] * inv;
}

// The Green-Gauss gradients of CPT cells per thread (cell_gradient's arithmetic, same order
// per cell), their slot and neighbour loads issued together. on[j]: cell c[j] is computed.
template <class T, int CPT>
__device__ __forceinline__ void cell_gradients(const DevMesh<T>& m, const typename Vec<T>::v4* __restrict__ W,
                                               const int (&c)[CPT], const bool (&on)[CPT],
                                               typename Vec<T>::v4 (&gxo)[CPT], typename Vec<T>::v4 (&gyo)[CPT],
                                               const typename Vec<T>::v4* sW, int base, int nsw) {
  using V2 = typename Vec<T>::v2;
  using V4 = typename Vec<T>::v4;
  V4 wc[CPT];
  T ax[CPT][4], ay[CPT][4];
  bool live[CPT];
#pragma unroll
  for (int j = 0; j < CPT; ++j) {
    live[j] = on[j];
    if (on[j]) wc[j] = sW[c[j] - base];
#pragma unroll
    for (int v = 0; v < 4; ++v) ax[j][v] = ay[j][v] = T(0);
  }
  constexpr int kU = 4;
  for (int k0 = 0; k0 < m.d; k0 += kU) {
    int lk[CPT][kU];
    V2 gv[CPT][kU];
    V4 wo[CPT][kU];
#pragma unroll
    for (int j = 0; j < CPT; ++j)
#pragma unroll
      for (int u = 0; u < kU; ++u) lk[j][u] = (live[j] && k0 + u < m.d) ? m.link[(k0 + u) * m.n + c[j]] : kPad;
#pragma unroll
    for (int j = 0; j < CPT; ++j)
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        if (live[j] && k0 + u < m.d) {
          const int s = (k0 + u) * m.n + c[j];
          gv[j][u] = m.gvec[s];
        }
      }
#pragma unroll
    for (int j = 0; j < CPT; ++j)
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        if (lk[j][u] >= 0) {
          const int o = lk[j][u] >> 1;
          const unsigned off = static_cast<unsigned>(o - base);
          wo[j][u] = off < static_cast<unsigned>(nsw) ? sW[off] : W[o];
        } else {
          wo[j][u] = wc[j];
        }
      }
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int link = lk[j][u];
        if (link == kPad) break;
        grad_slot_terms<T>(link, wc[j], wo[j][u], gv[j][u], ax[j], ay[j]);
      }
      if (lk[j][kU - 1] == kPad) live[j] = false;
    }
    bool more = false;
#pragma unroll
    for (int j = 0; j < CPT; ++j) more = more || live[j];
    if (!more) break;
  }
#pragma unroll
  for (int j = 0; j < CPT; ++j) {
    if (!on[j]) continue;
    const T inv = m.inv_vol[c[j]];
    gxo[j].x = ax[j][0] * inv; gxo[j].y = ax[j][1] * inv; gxo[j].z = ax[j][2] * inv; gxo[j].w = ax[j][3] * inv;
    gyo[j].x = ay[j][0] * inv; gyo[j].y = ay[j][1] * inv; gyo[j].z = ay[j][2] * inv; gyo[j].w = ay[j][3] * inv;
  }
}

// Gradient pass. CPT (cells per thread, 1 or 2): a block of B threads covers CPT cell blocks
// (nblk: cell blocks in all, for CPT > 1); thread t computes cells t, t + B, ... of them.
template <class T, int CPT = 1>
__global__ void __launch_bounds__(256) k_gradient(DevMesh<T> m, const typename Vec<T>::v4* __restrict__ W,
                                                  typename Vec<T>::v4* __restrict__ gx,
                                                  typename Vec<T>::v4* __restrict__ gy, Cases<T> cs, int nblk = 0) {
  if constexpr (CPT == 1) {
    pdl_trigger();
    pdl_wait();
    const int base = blockIdx.x * blockDim.x;
    const int c = base + threadIdx.x;
    // No shared-memory staging of the block's own cells: their neighbour loads hit L1 and L2
    // as well, and the staging's store and barrier cost more than they saved (131k cells:
    // 4.64 -> 4.39 us per launch without them; 524k: 14.96 -> 13.0 us).
    const int2 bd = cs.blk[blockIdx.x];
    if (cs.ctrl[bd.x].done) return;  // uniform over the block (one case per block)
    if (c >= bd.y) return;
    typename Vec<T>::v4 ox, oy;
    cell_gradient<T>(m, W, c, &ox, &oy);
    gx[c] = ox;
    gy[c] = oy;
  } else {
    // the covered blocks' own cells' W staged in shared memory: with the cells in Morton /
    // RCM order most neighbours fall inside them
    __shared__ typename Vec<T>::v4 sW[256 * CPT];
    pdl_trigger();
    pdl_wait();
    const int B = blockDim.x, lb0 = blockIdx.x * CPT;
    const int base = lb0 * B;
    const int nlb = min(CPT, nblk - lb0);
    // every cell of the covered blocks (padding included: in bounds, never a neighbour)
    const int nsw = nlb * B;
    for (int i = threadIdx.x; i < nsw; i += B) sW[i] = W[base + i];
    __syncthreads();
    int c[CPT];
    bool on[CPT];
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
      c[j] = base + j * B + static_cast<int>(threadIdx.x);
      on[j] = false;
      if (j < nlb) {
        const int2 bd = cs.blk[lb0 + j];
        on[j] = c[j] < bd.y && !cs.ctrl[bd.x].done;
      }
    }
    typename Vec<T>::v4 ox[CPT], oy[CPT];
    cell_gradients<T, CPT>(m, W, c, on, ox, oy, sW, base, nsw);
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
      if (on[j]) {
        gx[c[j]] = ox[j];
        gy[c[j]] = oy[j];
      }
    }
  }
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

// Global time step (time_integrator.cpp:45-56): maximum over per-warp maxima of max(SR, floor).
// One block per case; case k's warps are [first[k], first[k+1]).
static __global__ void k_srmax(const double* __restrict__ srmax, const int* __restrict__ first, Ctrl* ctrls) {
  __shared__ double shm[32];
  Ctrl* ctrl = ctrls + blockIdx.x;
  if (ctrl->done) return;
  double m = 0.0;
  for (int i = first[blockIdx.x] + threadIdx.x; i < first[blockIdx.x + 1]; i += blockDim.x) m = smax(m, srmax[i]);
  m = block_max(m, shm);
  if (threadIdx.x == 0) ctrl->sr_max = m;
}

// Positivity screen in float: true when enforce_physical (euler_flux.cpp:129-144) is provably
// the identity on the double state s, judged from its float image f = float(s): the density
// is above twice its floor and the internal energy is a resolved fraction (>1e-3) of the
// total and above twice the pressure floor, so the double clamp can be skipped. NaN fails.
__device__ __forceinline__ bool positivity_safe(const Cons<float>& f, float gm1) {
  if (!(f.r > 2.0e-8f)) return false;
  const float inv = sdiv(1.0f, f.r);
  const float u = f.ru * inv, v = f.rv * inv;
  const float ke = 0.5f * f.r * (u * u + v * v);
  const float e = f.rE - ke;
  return e > 1.0e-3f * f.rE && gm1 * e > 2.0e-8f;
}

// ---------------------------------------------------------------------------------------
// Update: low-Mach residual preconditioning (preconditioning.cpp:51-76, in double), local
// time step (time_integrator.cpp:31-59) and SSP-RK3 stage (time_integrator.cpp:61-104);
// writes the bulk primitive state for the next stage.
//   FP64: the stage state Us is a double state, combined as the reference does.
//   FP32: delta form. Us holds the stage increment delta in float; since the RK3 weights sum
//         to one, stage k sets delta' = b_k (delta - dt R) with b = 1, 1/4, 2/3. Intermediate
//         stage states are float: hi + delta' with hi the float image of U_n, clamped in float
//         as the reference's float path clamps. The last stage adds delta' to the float-float
//         pair (hi, lo) of U_n, so the conserved state accumulates beyond float precision with
//         float arithmetic only; the double clamp runs only when the float screen fails.
// The last stage also runs the non-finite trap (euler_solver.cpp:908-946) and the monitors.
// GATHER (local time stepping): the cell's residual is gathered here from the face pass's
// fluxes instead of read from R/SR; the last stage stores it in R/SR (the run's last
// residual) and forms the residual-norm partials.
// ---------------------------------------------------------------------------------------
template <class T, bool PRECOND, bool LAST, bool GATHER>
__global__ void __launch_bounds__(256) k_update(int stage, Cases<T> cs, typename Vec<T>::v4* __restrict__ R,
                                                T* __restrict__ SR, DevGather<T> g,
                                                const typename Vec<T>::v4* __restrict__ F, const T* __restrict__ FS,
                                                typename Vec<T>::v4* __restrict__ W, StateRef U,
                                                typename Vec<T>::v4* __restrict__ Us, MonitorSet ms, Partials part,
                                                int global_dt, int pf) {
  if (pf > 0 && blockIdx.x + pf < gridDim.x) {
    // the cell streams of the block pf blocks ahead (inside the block-padded arrays): the
    // state, the stage increment, the primitive state and the gather slots, one per thread
    const size_t c0 = static_cast<size_t>(blockIdx.x + pf) * blockDim.x;
    const unsigned nb = blockDim.x;
    const int t = threadIdx.x;
    if constexpr (sizeof(T) == 4) {
      if (t == 0) l2_prefetch(U.hi + c0, nb * sizeof(float4));
      if (LAST && t == 1) l2_prefetch(U.lo + c0, nb * sizeof(float4));
    } else {
      if (t == 0) l2_prefetch(U.un + c0, nb * sizeof(d4));
    }
    if (stage > 0 && t == 2) l2_prefetch(Us + c0, nb * sizeof(Us[0]));
    if (PRECOND && t == 3) l2_prefetch(W + c0, nb * sizeof(W[0]));
    if (GATHER && t >= 4 && t < 4 + g.d) l2_prefetch(g.slot + static_cast<size_t>(t - 4) * g.n + c0, nb * sizeof(int));
  }
  pdl_trigger();
  pdl_wait();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  // The cell's own state and first gather slots, loaded before the case lookup so that their
  // latency overlaps it (every block lies inside the block-padded arrays; padding cells'
  // values go unused). The preconditioned last stage, and the FP64 kernels, load them after
  // the checks: held across them, they take the float stage from 64 to 80 registers per
  // thread and the FP64 kernels from 80 to 100.
  constexpr bool kEarly = sizeof(T) == 4 && !(PRECOND && LAST);
  typename Vec<T>::v4 st_hi{}, st_lo{}, st_us{}, st_w{};
  d4 st_un{};
  int first[kGatherBatch];
  auto load_own = [&] {
    if constexpr (sizeof(T) == 4) {
      st_hi = U.hi[c];
      if (LAST) st_lo = U.lo[c];
    } else {
      st_un = U.un[c];
    }
    if (stage > 0) st_us = Us[c];
    if (PRECOND) st_w = W[c];
    if (GATHER && kEarly) gather_slots(g, c, 0, first);
  };
  if (kEarly) load_own();
  const int2 bd = cs.blk[blockIdx.x];
  Ctrl* ctrl = cs.ctrl + bd.x;
  const PrecondD& pc = cs.pc[bd.x];
  const int n = bd.y;
  if (ctrl->done) return;
  if (cs.wait != nullptr && cs.wait[0] != 0) {
    // The gradient pass of this iteration gave up a wait and left gradients unwritten: no
    // stage of the iteration is applied (the conserved state is written by the last stage
    // only), and the controller stops the run without recording the iteration.
    if (threadIdx.x == 0) ctrl->wait_stop = 1;
    return;
  }
  bool bad = false;
  Cons<double> s{1.0, 0.0, 0.0, 1.0};
  Prim<T> w{T(1), T(0), T(0), T(1)};
  T nq[kNorm] = {T(0), T(0), T(0), T(0)};
  if (c < n) {
    if (!kEarly) load_own();
    T r0, r1, r2, r3, src;
    if (GATHER) {
      T rr[4];
      gather_cell<T>(g, F, FS, c, kEarly ? first : nullptr, rr, &src);
      r0 = rr[0];
      r1 = rr[1];
      r2 = rr[2];
      r3 = rr[3];
      if (LAST) {
        typename Vec<T>::v4 o;
        o.x = r0; o.y = r1; o.z = r2; o.w = r3;
        R[c] = o;
        SR[c] = src;
        norm_terms<T>(rr, g.inv_vol[c], nq);
      }
    } else {
      const auto r4 = R[c];
      r0 = r4.x;
      r1 = r4.y;
      r2 = r4.z;
      r3 = r4.w;
      if (!global_dt) src = SR[c];
    }
    if (PRECOND && sizeof(T) == 4 && pc.fp64 != 1) {
      // FP32 contexts: beta from the float state (preconditioning.cpp:9-32 in float); the
      // energy row (:51-76) in float, or with fp64 == 2 (by default below Mach 0.1) as the
      // double-float sum N = b2 (r3 rho) + (b2 - 1)(u r1 + v r2): every product split
      // error-free with a fused multiply-add, every sum with two-sum (Knuth), so N carries
      // about 44 significant bits on the float pipe, where the float row loses digits to the
      // cancellation between its two terms at low Mach. r3 = N / rho in float.
      const auto w4 = st_w;
      const Prim<float> w{float(w4.x), float(w4.y), float(w4.z), float(w4.w)};
      FaceParams<float> fpf;
      fpf.gamma = pc.gamma_f;
      fpf.pc_mach_ref = pc.mach_ref_f;
      fpf.pc_mach_min = pc.mach_min_f;
      fpf.pc_beta_min = pc.beta_min_f;
      fpf.pc_beta_max = pc.beta_max_f;
      const float beta = cell_beta(w, fpf);
      if (pc.fp64 == 0) {
        const float b2 = beta * beta;
        const float inv_rho = sdiv(1.0f, smax(w.r, 1.0e-8f));
        const float ud = fmaf(w.u, float(r1), w.v * float(r2));
        r3 = T(fmaf(b2, float(r3), (b2 - 1.0f) * inv_rho * ud));
      } else {
        const float rho = smax(w.r, 1.0e-8f);
        float bh, bl, dh, dl, ph, pl, qh, ql, uh, ul, th, tl, mh, ml, gh, gl, nh, nl, e;
        bh = __fmul_rn(beta, beta);  // b2 = bh + bl exactly
        bl = __fmaf_rn(beta, beta, -bh);
        two_sum(bh, -1.0f, &dh, &e);  // b2 - 1
        dl = __fadd_rn(e, bl);
        ph = __fmul_rn(w.u, float(r1));  // u r1 + v r2
        pl = __fmaf_rn(w.u, float(r1), -ph);
        qh = __fmul_rn(w.v, float(r2));
        ql = __fmaf_rn(w.v, float(r2), -qh);
        two_sum(ph, qh, &uh, &e);
        ul = __fadd_rn(e, __fadd_rn(pl, ql));
        th = __fmul_rn(dh, uh);  // (b2 - 1)(u r1 + v r2)
        tl = __fadd_rn(__fmaf_rn(dh, uh, -th), __fmaf_rn(dh, ul, __fmul_rn(dl, uh)));
        mh = __fmul_rn(float(r3), rho);  // r3 rho
        ml = __fmaf_rn(float(r3), rho, -mh);
        gh = __fmul_rn(bh, mh);  // b2 (r3 rho)
        gl = __fadd_rn(__fmaf_rn(bh, mh, -gh), __fmaf_rn(bh, ml, __fmul_rn(bl, mh)));
        two_sum(gh, th, &nh, &e);
        nl = __fadd_rn(e, __fadd_rn(gl, tl));
        r3 = T(sdiv(__fadd_rn(nh, nl), rho));
      }
    } else if (PRECOND) {
      // the preconditioned energy row in double, beta included: FP64 contexts, and FP32
      // contexts with fp64 == 1 (GB300 runs double at a small fraction of the float rate)
      const auto w4 = st_w;
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
      const double ud = w.u * double(r1) + w.v * double(r2);
      r3 = T(b2 * double(r3) + (b2 - 1.0) * inv_rho * ud);
    }
    const T cfl = (sizeof(T) == 4) ? T(ctrl->cfl_f) : T(ctrl->cfl);
    T dt;
    if (global_dt) {
      dt = sdiv(cfl, T(ctrl->sr_max));
      if (!sfinite(dt)) dt = T(0);
    } else {
      dt = sdiv(cfl, smax(src, Kn<T>::wave_floor));
    }
    if constexpr (sizeof(T) == 4) {
      float d0, d1, d2, d3;
      if (stage == 0) {
        d0 = -(dt * r0);
        d1 = -(dt * r1);
        d2 = -(dt * r2);
        d3 = -(dt * r3);
      } else {
        const float b = (stage == 1) ? 0.25f : (2.0f / 3.0f);
        const float4 dl = st_us;
        d0 = b * (dl.x - dt * r0);
        d1 = b * (dl.y - dt * r1);
        d2 = b * (dl.z - dt * r2);
        d3 = b * (dl.w - dt * r3);
      }
      const float4 uh = st_hi;
      if (!LAST) {
        Cons<float> f{uh.x + d0, uh.y + d1, uh.z + d2, uh.w + d3};
        const float fr = f.r, fe = f.rE;
        enforce_physical(&f, pc.gamma_f);  // changes only rho and rhoE
        if (f.r != fr) d0 = f.r - uh.x;
        if (f.rE != fe) d3 = f.rE - uh.w;
        Us[c] = make_float4(d0, d1, d2, d3);
        w = cons_to_prim(f, pc.gamma_f);
      } else {
        const float4 ul = st_lo;
        float4 h, l;
        ff_add(uh.x, ul.x, d0, &h.x, &l.x);
        ff_add(uh.y, ul.y, d1, &h.y, &l.y);
        ff_add(uh.z, ul.z, d2, &h.z, &l.z);
        ff_add(uh.w, ul.w, d3, &h.w, &l.w);
        Cons<float> f{h.x, h.y, h.z, h.w};
        if (!positivity_safe(f, pc.gm1_f)) {
          s = Cons<double>{double(h.x) + double(l.x), double(h.y) + double(l.y), double(h.z) + double(l.z),
                           double(h.w) + double(l.w)};
          enforce_physical(&s, pc.gamma);
          ff_split(s.r, &h.x, &l.x);
          ff_split(s.ru, &h.y, &l.y);
          ff_split(s.rv, &h.z, &l.z);
          ff_split(s.rE, &h.w, &l.w);
          f = Cons<float>{h.x, h.y, h.z, h.w};
        }
        U.hi[c] = h;
        U.lo[c] = l;
        w = cons_to_prim(f, pc.gamma_f);
        bad = !finite4(h.x, h.y, h.z, h.w) || !finite4(l.x, l.y, l.z, l.w) || !finite4(w.r, w.u, w.v, w.p);
      }
    } else {
      const d4 un = st_un;
      const double d = double(dt);
      const d4 us = (stage == 0) ? un : st_us;
      s = Cons<double>{us.x - d * r0, us.y - d * r1, us.z - d * r2, us.w - d * r3};
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
      // the case's energy floor and the floored rho's reciprocal reused by the primitive
      // refresh: the same quotients as enforce_physical and cons_to_prim form, two FP64
      // divisions fewer per cell
      const double inv = enforce_physical_pf(&s, pc.gamma, pc.pfe);
      const d4 o{s.r, s.ru, s.rv, s.rE};
      if (LAST) {
        U.un[c] = o;
      } else {
        Us[c] = o;
      }
      w = cons_to_prim_from(Cons<T>{T(s.r), T(s.ru), T(s.rv), T(s.rE)}, T(pc.gamma), T(s.r), T(inv));
      if (LAST) bad = !finite4(s.r, s.ru, s.rv, s.rE) || !finite4(w.r, w.u, w.v, w.p);
    }
    typename Vec<T>::v4 wo;
    wo.x = w.r; wo.y = w.u; wo.z = w.v; wo.w = w.p;
    W[c] = wo;
  }
  if (LAST) {
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&ctrl->nonfinite, 1);
    if (GATHER) block_norms<T>(nq, part);
    block_monitors<T>(c < n, w, c, ms, cs.mc[bd.x], part);
  }
}

// AoA-0 symmetry (euler_solver.cpp:418-450): every `interval` iterations the new state's
// v is zeroed through the primitive variables. Applied after the last stage; it redoes the
// last stage's max |p - p_inf| partials and non-finite check on the symmetrised state.
template <class T>
__global__ void __launch_bounds__(256) k_symmetry(Cases<T> cs, StateRef U, typename Vec<T>::v4* __restrict__ W,
                                                  MonitorSet ms, Partials part) {
  const int2 bd = cs.blk[blockIdx.x];
  Ctrl* ctrl = cs.ctrl + bd.x;
  const double gamma = cs.mc[bd.x].gamma;
  const int interval = cs.mc[bd.x].sym_interval;
  const int n = bd.y;
  if (ctrl->done || interval <= 0) return;
  if (((ctrl->iter + 1) % interval) != 0) return;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  bool bad = false;
  Cons<double> s{1.0, 0.0, 0.0, 1.0};
  Prim<T> wt{T(1), T(0), T(0), T(1)};
  if (c < n) {
    Prim<double> w = cons_to_prim(load_state<T>(U, c), gamma);
    w.v = 0.0;
    s = prim_to_cons(w, gamma);
    store_state<T>(U, c, s);
    wt = cons_to_prim(Cons<T>{T(s.r), T(s.ru), T(s.rv), T(s.rE)}, T(gamma));
    typename Vec<T>::v4 wo;
    wo.x = wt.r; wo.y = wt.u; wo.z = wt.v; wo.w = wt.p;
    W[c] = wo;
    bad = !finite4(s.r, s.ru, s.rv, s.rE) || !finite4(wt.r, wt.u, wt.v, wt.p);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&ctrl->nonfinite, 1);
  block_monitors<T>(c < n, wt, c, ms, cs.mc[bd.x], part);
}

// Pressure-jump energy over interior faces (euler_solver.cpp:1027-1063), per owning cell.
template <class T>
__global__ void __launch_bounds__(256) k_pjump(DevMesh<T> m, StateRef U,
                                               const unsigned char* __restrict__ flags, Cases<T> cs,
                                               Partials part) {
  __shared__ double shm[32 * 4];
  const int2 bd = cs.blk[blockIdx.x];
  const double gamma = cs.mc[bd.x].gamma;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (cs.ctrl[bd.x].done) return;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  if (c < bd.y) {
    const double pc = cons_to_prim(load_state<T>(U, c), gamma).p;
    for (int k = 0; k < m.d; ++k) {
      const int link = m.link[k * m.n + c];
      if (link == kPad) break;
      if (link < 0 || (link & 1)) continue;  // interior faces owned by c
      const int o = link >> 1;
      const double po = cons_to_prim(load_state<T>(U, o), gamma).p;
      const double dp = pc - po;
      v[0] += dp * dp;
      v[1] += 1.0;
      if ((flags[c] | flags[o]) & 1) {  // bit 0: the cell owns wall faces
        v[2] += dp * dp;
        v[3] += 1.0;
      }
    }
  }
  block_sum<4>(v, shm);
  if (threadIdx.x == 0) {
    for (int k = 0; k < 4; ++k) part.pjump[k * part.nb + blockIdx.x] = v[k];
  }
}

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
  double rho_ratio;
};

// The controller's serial work, split over the four warps (each warp on its own SM
// sub-partition, so their double arithmetic proceeds side by side) in two phases:
//   phase 1  ctl_forces_lane  force coefficients and their stability window (lanes 0-2 of
//                          warp 0, one coefficient each)
//            ctl_residual  residual monitor, adaptive CFL, the iteration-only part of the
//                          next schedule
//            ctl_side      density-residual ratio, wall pressure-jump energy
//            ctl_report    the record's reporting-only fields, fallback counters
//   phase 2  ctl_decide    staged all-speed controller, stop rule, next schedule
// Every value is formed by the same expression as in one serial pass
// (euler_solver.cpp:948-1208, convergence_monitor.cpp:13-127, forces.cpp:208-294); the
// threads write disjoint fields of the shared record and controller state.
struct CtlIn {  // the block partials combined
  double a[kNorm], mon[kMon], pj[4], wv[kWall];
};

__device__ inline void ctl_report(const CtrlConfig& cc, const CtlIn& in, const Ctrl& s, Record& r, int* fb) {
  const double* fsum = in.wv;
  const double un_max = in.wv[8], cp_hi = in.wv[9], cp_lo_neg = in.wv[10], cp_bad = in.wv[11];
  r.iter = s.iter;
  r.flags = (s.second ? 8 : 0) | (s.as_fix ? 32 : 0) | (s.stage == 1 ? 64 : 0) | (s.stage == 2 ? 128 : 0);
  r.fo = fb[0];
  r.df = fb[1];
  fb[0] = 0;
  fb[1] = 0;
  r.cfl = s.cfl;
  r.stab = s.stab_floor;
  r.as_fmin = s.as_fmin;
  r.as_ramp = s.as_ramp;
  r.dp_dom = in.mon[0];
  r.dp_wall = in.mon[1];
  r.wall_un = un_max;
  r.wall_mass_flux = 0.0;  // the slip-wall flux has no mass component (boundary_conditions.cpp:97-110)
  r.cp_min = cc.n_wall > 0 ? -cp_lo_neg : 0.0;
  r.cp_max = cc.n_wall > 0 ? cp_hi : 0.0;
  if (cc.n_wall > 0 && cp_bad == double(cc.n_wall)) {
    r.cp_min = 3.402823466e38;  // no finite sample: the reference keeps its float sentinels
    r.cp_max = -3.402823466e38;
  }
  r.cp_nonfinite = int(cp_bad);
  r.ff_dp = in.mon[2];
  r.ff_drho = in.mon[3];
  r.ff_du = in.mon[4];
  r.ff_dv = in.mon[5];
  r.action = 0;
  r.l1 = in.a[0];
  r.linf = in.a[2];
  // integrate_pressure_forces: gauge and absolute force components, absolute coefficients
  const double qs = cc.q_inf * cc.s_ref;
  const double fxg = fsum[4], fyg = fsum[5], fxa = fsum[2], fya = fsum[3];
  r.fx_g = fxg; r.fy_g = fyg; r.fx_a = fxa; r.fy_a = fya; r.snx = fsum[0]; r.sny = fsum[1];
  r.cd_abs = (fxa * cc.cos_a + fya * cc.sin_a) / qs;
  r.cl_abs = (-fxa * cc.sin_a + fya * cc.cos_a) / qs;
  r.cm_abs = fsum[6] / (qs * cc.chord);
  // domain pressure-jump energy
  const double pr2 = cc.pressure_ref * cc.pressure_ref + 1.0e-24;
  r.pj = in.pj[1] > 0.0 ? (in.pj[0] / in.pj[1]) / pr2 : 0.0;
}

__device__ inline void ctl_side(const CtrlConfig& cc, const CtlIn& in, Ctrl& s, Record& r, LmSched* lms) {
  // the low-Mach weights of iteration iter + 2, read by that iteration's face passes
  if (lms) lms[(s.iter + 2) & 1] = lm_sched_of(cc, s.iter + 2);
  // density-residual L2 ratio (the batched sweep's per-case stop rule)
  const double l2rho = smax(sqrt(in.a[3] / double(cc.n_cells > 0 ? cc.n_cells : 1)), 1.0e-20);
  if (s.initial_l2rho < 0.0) s.initial_l2rho = l2rho;
  r.rho_ratio = l2rho / smax(s.initial_l2rho, 1.0e-20);
  // wall pressure-jump energy (the staged controller's input)
  const double pr2 = cc.pressure_ref * cc.pressure_ref + 1.0e-24;
  r.pj_wall = in.pj[3] > 0.0 ? (in.pj[2] / in.pj[3]) / pr2 : 0.0;
}

__device__ inline void ctl_residual(const CtrlConfig& cc, const CtlIn& in, Ctrl& s, Record& r, SchedBase* next) {
  *next = schedule_base(cc, s.iter + 1);
  const double l2 = sqrt(in.a[1] / double(cc.n_cells > 0 ? 5 * cc.n_cells : 1));
  r.l2 = l2;
  // ConvergenceMonitor::update_residual
  const double bl2 = smax(l2, 1.0e-20);
  if (s.initial_l2 < 0.0) s.initial_l2 = bl2;
  r.ratio = bl2 / smax(s.initial_l2, 1.0e-20);
  if (s.prev_l2 > 0.0) {
    if (l2 > s.prev_l2 * 1.05) {
      s.cfl_scale = smax(s.cfl_scale * 0.65, 0.05);
    } else if (l2 < s.prev_l2 * 0.90) {
      s.cfl_scale = smin(s.cfl_scale * 1.03, 1.0);
    }
  }
  s.prev_l2 = l2;
}

// Forces and the force-window tests on lanes k = 0, 1, 2 of one warp (CL, CD, CM): each lane
// forms its coefficient, its column of the history ring and its window tests, every
// quantity with the operations, in the order, of the one-lane form; the three stability and
// drift tests are combined across the lanes. A GB300 SM runs double arithmetic at a small
// fraction of its float rate, so the three coefficients' chains run side by side.
__device__ inline void ctl_forces_lane(const CtrlConfig& cc, const CtlIn& in, Ctrl& s, Record& r, int k,
                                       bool* stable_out, bool* dstable_out) {
  constexpr unsigned kLanes = 0x7u;
  const double* fsum = in.wv;
  // integrate_pressure_forces (gauge -> reported)
  const double qs = cc.q_inf * cc.s_ref;
  const double fxg = fsum[4], fyg = fsum[5];
  double coef, prev;
  if (k == 0) {
    r.lift = -fxg * cc.sin_a + fyg * cc.cos_a;
    coef = r.lift / qs;
    r.cl = coef;
    prev = s.prev_cl;
  } else if (k == 1) {
    r.drag = fxg * cc.cos_a + fyg * cc.sin_a;
    coef = r.drag / qs;
    r.cd = coef;
    prev = s.prev_cd;
  } else {
    r.moment = fsum[7];
    coef = fsum[7] / (qs * cc.chord);
    r.cm = coef;
    prev = s.prev_cm;
  }
  // ConvergenceMonitor::update_forces
  const double dc = s.has_prev ? fabs(coef - prev) : 0.0;
  const int req = cc.window < 1 ? 1 : cc.window;
  const int cap = 2 * req;
  int count = s.hist_count, head = s.hist_head;
  const int slot = (head + count) % cap;
  s.hist[3 * slot + k] = coef;  // each lane reads and writes its own column only
  if (count < cap) {
    ++count;
  } else {
    head = (head + 1) % cap;
  }
  auto H = [&](int i) {  // entry i of the ring (0 = oldest); head < cap, i < cap
    const int j = head + i;
    return s.hist[3 * (j >= cap ? j - cap : j) + k];
  };
  bool st = false;
  if (count >= req) {
    const int b = count - req;
    double lo = H(b), hi = lo;
    for (int i = b; i < count; ++i) {
      lo = smin(lo, H(i));
      hi = smax(hi, H(i));
    }
    st = (hi - lo) <= cc.stab_tol;
  }
  bool dst = false;
  double mdc = 0.0;
  if (count >= cap) {
    double pa = 0, ca = 0;
    for (int i = 0; i < req; ++i) pa += H(i);
    for (int i = req; i < cap; ++i) ca += H(i);
    const double inv = 1.0 / double(req);
    mdc = fabs(ca * inv - pa * inv);
    dst = mdc <= cc.drift_tol;
  }
  if (k == 0) {
    r.dcl = dc;
    r.mdcl = mdc;
  } else if (k == 1) {
    r.dcd = dc;
    r.mdcd = mdc;
  } else {
    r.dcm = dc;
    r.mdcm = mdc;
  }
  *stable_out = __ballot_sync(kLanes, st) == kLanes;
  *dstable_out = __ballot_sync(kLanes, dst) == kLanes;
  __syncwarp(kLanes);  // every lane has read the ring's head, count and has_prev
  if (k == 0) {
    s.prev_cl = coef;
    s.has_prev = 1;
    s.hist_count = count;
    s.hist_head = head;
  } else if (k == 1) {
    s.prev_cd = coef;
  } else {
    s.prev_cm = coef;
  }
}

__device__ inline void ctl_decide(const CtrlConfig& cc, Ctrl& s, Record& r, bool stable, bool dstable,
                                  const SchedBase& next) {
  const bool nonfinite = s.nonfinite != 0;
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
  const bool conv = (s.iter + 1 >= cc.min_iterations) &&
                    ((!(r.ratio > cc.residual_target) && stable && dstable) ||
                     (cc.rho_l2_target > 0.0 && !(r.rho_ratio > cc.rho_l2_target)));
  if (conv) r.flags |= 4;
  if (nonfinite) r.flags |= 16;
  if (conv || nonfinite) s.done = 1;
  // next iteration's schedule (its iteration-only part formed in phase 1)
  s.iter = s.iter + 1;
  apply_schedule_from(cc, next, &s);
}


// Maximum of two non-negative doubles through their bit patterns, on the integer pipe.
__device__ __forceinline__ long long max_bits(long long a, long long b) { return a > b ? a : b; }
__device__ __forceinline__ long long warp_max_bits(long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = max_bits(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// Controller (one block of kCtlThreads): combines the per-block partials of the norms,
// monitors, forces and pressure jumps in a fixed order, then runs the convergence monitor,
// adaptive CFL, staged all-speed controller and the next iteration's schedule in the two
// phases of ctl_monitor / ctl_side / ctl_report and ctl_decide (euler_solver.cpp:948-1208,
// 772-797; convergence_monitor.cpp:13-127; forces.cpp:208-294). The record is assembled in
// shared memory and stored by the whole block.
// The serial part works on a shared-memory copy of the controller state, loaded and stored
// by the whole block, so that thread 0 pays no chain of global-memory round trips. Maxima
// of non-negative quantities are taken on the integer pipe: a GB300 SM runs double
// arithmetic at a small fraction of its float rate.
// 256 threads: the block-partial loops take four blocks per thread at 131k cells (128
// threads: 16.4 us in the iteration graph, 256: 15.3 us, 512: 16.1 us).
constexpr int kCtlThreads = 256;
static_assert(sizeof(Ctrl) % 16 == 0, "Ctrl is copied in 16-byte words");
// One block per case: ccs[case], ctrls[case], records recs[case * rec_cap ...], fallback
// counters fb[4 * case + 0/1] (fb already offset by the iteration's parity).
// lms_all (may be null): per case, the two parity slots of LmSched.
static __global__ void __launch_bounds__(kCtlThreads) k_control(const CtrlConfig* __restrict__ ccs, Partials part,
                                                                Ctrl* __restrict__ ctrls,
                                                                Record* __restrict__ recs_all, int rec_cap,
                                                                int* __restrict__ fb_all,
                                                                LmSched* __restrict__ lms_all) {
  constexpr int kWarps = kCtlThreads / 32;
  const CtrlConfig cc = ccs[blockIdx.x];
  Ctrl* ctrl = ctrls + blockIdx.x;
  Record* recs = recs_all + static_cast<size_t>(blockIdx.x) * rec_cap;
  int* fb = fb_all + 4 * blockIdx.x;
  __shared__ Ctrl sc;
  __shared__ double s_sum[kWarps][3 + 4];   // l1, l2 sum, density l2 sum, pressure-jump sums
  __shared__ long long s_max[kWarps][1 + kMon];  // linf, monitors (bit patterns)
  __shared__ double s_wall[kWarps][kWall];
  // The controller state is copied to shared memory and the block partials are read before
  // the done / wait-stop checks, which then come from the shared copy: the loads do not wait
  // for a round trip on the flags, and nothing is written before the checks.
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  constexpr int kWords = int(sizeof(Ctrl) / 16);
  {
    const int4* src = reinterpret_cast<const int4*>(ctrl);
    int4* dst = reinterpret_cast<int4*>(&sc);
    for (int i = tid; i < kWords; i += kCtlThreads) dst[i] = src[i];
  }
  const int nb = cc.n_blocks;      // this case's blocks: bb .. bb + nb - 1
  const int bb = cc.block_base;
  const int st = part.nb;          // quantity stride of the block partials
  double s1 = 0.0, s2 = 0.0, s3 = 0.0;
  long long mx[1 + kMon] = {0, 0, 0, 0, 0, 0, 0};
  if (cc.bulk_f32) {
    // float block partials summed in float-float, then one conversion per warp
    float h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f, h3 = 0.f, l3 = 0.f;
#pragma unroll 4
    for (int b = bb + tid; b < bb + nb; b += kCtlThreads) {
      ff_add(h1, l1, part.norms_f[b], &h1, &l1);
      ff_add(h2, l2, part.norms_f[st + b], &h2, &l2);
      ff_add(h3, l3, part.norms_f[3 * st + b], &h3, &l3);
      mx[0] = max_bits(mx[0], static_cast<long long>(__float_as_uint(part.norms_f[2 * st + b])));
#pragma unroll
      for (int k = 0; k < kMon; ++k) mx[k + 1] = max_bits(mx[k + 1], part.mon[k * st + b]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float a = __shfl_xor_sync(0xffffffffu, h1, o), b = __shfl_xor_sync(0xffffffffu, l1, o);
      const float c = __shfl_xor_sync(0xffffffffu, h2, o), d = __shfl_xor_sync(0xffffffffu, l2, o);
      const float e = __shfl_xor_sync(0xffffffffu, h3, o), f = __shfl_xor_sync(0xffffffffu, l3, o);
      ff_add2(h1, l1, a, b, &h1, &l1);
      ff_add2(h2, l2, c, d, &h2, &l2);
      ff_add2(h3, l3, e, f, &h3, &l3);
    }
    if (lane == 0) {
      s1 = double(h1) + double(l1);
      s2 = double(h2) + double(l2);
      s3 = double(h3) + double(l3);
    }
  } else {
#pragma unroll 2
    for (int b = bb + tid; b < bb + nb; b += kCtlThreads) {
      s1 += part.norms[b];
      s2 += part.norms[st + b];
      s3 += part.norms[3 * st + b];
      mx[0] = max_bits(mx[0], __double_as_longlong(part.norms[2 * st + b]));
#pragma unroll
      for (int k = 0; k < kMon; ++k) mx[k + 1] = max_bits(mx[k + 1], part.mon[k * st + b]);
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    s3 = warp_sum(s3);
  }
#pragma unroll
  for (int k = 0; k < 1 + kMon; ++k) mx[k] = warp_max_bits(mx[k]);
  double pj[4] = {0.0, 0.0, 0.0, 0.0};
  if (cc.pjump_blocks > 0) {
    for (int b = bb + tid; b < bb + cc.pjump_blocks; b += kCtlThreads) {
#pragma unroll
      for (int k = 0; k < 4; ++k) pj[k] += part.pjump[k * st + b];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) pj[k] = warp_sum(pj[k]);
  }
  // wall partials (snx sny fxa fya fxg fyg ma mg | un_max cp_hi -cp_lo cp_bad): with the
  // wall-owning cells numbered first these come from a few blocks, summed per quantity by
  // one thread each; otherwise by the whole block
  const int nwb = cc.n_wall_blocks;
  auto wall_init = [](int k) { return (k == 9 || k == 10) ? -1.0e308 : 0.0; };
  auto wall_comb = [](int k, double acc, double x) { return (k >= 8 && k <= 10) ? smax(acc, x) : acc + x; };
  const int wb = cc.wall_base, wst = part.nwb;
  auto wall_at = [&](int k, int b) {
    const int i = k * wst + wb + b;
    return cc.bulk_f32 ? double(part.wall_f[i]) : part.wall[i];
  };
  if (nwb <= 32) {
    // every (quantity, block) value loaded at once, then combined over the blocks in order
    __shared__ double s_wload[kWall][32];
    for (int i = tid; i < kWall * nwb; i += kCtlThreads) s_wload[i / nwb][i % nwb] = wall_at(i / nwb, i % nwb);
    __syncthreads();
    if (tid < kWall) {
      double acc = wall_init(tid);
      for (int b = 0; b < nwb; ++b) acc = wall_comb(tid, acc, s_wload[tid][b]);
      s_wall[0][tid] = acc;
    }
  } else {
    double wv[kWall];
#pragma unroll
    for (int k = 0; k < kWall; ++k) wv[k] = wall_init(k);
    for (int b = tid; b < nwb; b += kCtlThreads) {
#pragma unroll
      for (int k = 0; k < kWall; ++k) wv[k] = wall_comb(k, wv[k], wall_at(k, b));
    }
#pragma unroll
    for (int k = 0; k < kWall; ++k) wv[k] = (k >= 8 && k <= 10) ? warp_max(wv[k]) : warp_sum(wv[k]);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < kWall; ++k) s_wall[wid][k] = wv[k];
    }
  }
  if (lane == 0) {
    s_sum[wid][0] = s1;
    s_sum[wid][1] = s2;
    s_sum[wid][2] = s3;
#pragma unroll
    for (int k = 0; k < 4; ++k) s_sum[wid][3 + k] = pj[k];
#pragma unroll
    for (int k = 0; k < 1 + kMon; ++k) s_max[wid][k] = mx[k];
  }
  __syncthreads();
  if (sc.done) return;  // uniform over the block
  if (sc.wait_stop) {   // the iteration was not applied: stop without a record
    if (tid == 0) {
      fb[0] = 0;  // its face passes' fallback counts are dropped with it
      fb[1] = 0;
      ctrl->done = 1;
    }
    return;
  }
  __shared__ CtlIn s_in;
  __shared__ Record srec;
  __shared__ SchedBase snext;
  __shared__ int s_slot;
  // the warps' partials combined one quantity per lane of warp 0, each over the warps in
  // order: sums (lanes 0-6), maxima (7-13), wall quantities (14-25)
  if (tid < 7) {
    double v = 0.0;
    for (int w = 0; w < kWarps; ++w) v += s_sum[w][tid];
    if (tid == 0) s_in.a[0] = v;
    else if (tid == 1) s_in.a[1] = v;
    else if (tid == 2) s_in.a[3] = v;
    else s_in.pj[tid - 3] = v;
  } else if (tid < 7 + 1 + kMon) {
    const int k = tid - 7;
    long long m = 0;
    for (int w = 0; w < kWarps; ++w) m = max_bits(m, s_max[w][k]);
    const double v = cc.bulk_f32 ? double(__uint_as_float(static_cast<unsigned>(m))) : __longlong_as_double(m);
    if (k == 0) s_in.a[2] = v;
    else s_in.mon[k - 1] = v;
  } else if (tid < 8 + kMon + kWall) {
    const int k = tid - (8 + kMon);
    double v = s_wall[0][k];
    if (nwb > 32) {
      for (int w = 1; w < kWarps; ++w) v = wall_comb(k, v, s_wall[w][k]);
    }
    s_in.wv[k] = v;
  } else if (tid == 8 + kMon + kWall) {
    s_slot = sc.iter - sc.rec_base;  // the record slot of this iteration
  }
  __syncthreads();
  // phase 1: independent chains on warps 0..3 (the force coefficients on lanes 0-2 of warp 0)
  static_assert(kCtlThreads >= 128, "the controller's phase 1 uses four warps");
  bool stable = false, dstable = false;
  if (tid < 3) {
    ctl_forces_lane(cc, s_in, sc, srec, tid, &stable, &dstable);
  } else if (tid == 32) {
    ctl_residual(cc, s_in, sc, srec, &snext);
  } else if (tid == 64) {
    ctl_side(cc, s_in, sc, srec, lms_all ? lms_all + 2 * blockIdx.x : nullptr);
  } else if (tid == 96) {
    ctl_report(cc, s_in, sc, srec, fb);
  }
  __syncthreads();
  // phase 2: the decisions
  if (tid == 0) ctl_decide(cc, sc, srec, stable, dstable, snext);
  __syncthreads();
  if (s_slot >= 0 && s_slot < rec_cap) {
    static_assert(sizeof(Record) % 8 == 0, "Record is copied in 8-byte words");
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&srec);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(recs + s_slot);
    for (int i = tid; i < int(sizeof(Record) / 8); i += kCtlThreads) dst[i] = src[i];
  }
  {
    const int4* src = reinterpret_cast<const int4*>(&sc);
    int4* dst = reinterpret_cast<int4*>(ctrl);
    for (int i = tid; i < kWords; i += kCtlThreads) dst[i] = src[i];
  }
}

// Bulk primitive state from a double conserved state (FP64 state, or a state given to
// aero_residual).
template <class T>
__global__ void k_refresh_prim(int n, const d4* __restrict__ Un, typename Vec<T>::v4* __restrict__ W, double gamma) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const d4 u = Un[c];
  const Prim<T> w = cons_to_prim(Cons<T>{T(u.x), T(u.y), T(u.z), T(u.w)}, T(gamma));
  typename Vec<T>::v4 o;
  o.x = w.r; o.y = w.u; o.z = w.v; o.w = w.p;
  W[c] = o;
}

// FP32 state: split a double state into float-float pairs, combine the pairs back into
// doubles, and the bulk primitive state from the float image.
static __global__ void k_split_state(int n, const d4* __restrict__ Un, float4* __restrict__ hi,
                                     float4* __restrict__ lo) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const d4 u = Un[c];
  float4 h, l;
  ff_split(u.x, &h.x, &l.x);
  ff_split(u.y, &h.y, &l.y);
  ff_split(u.z, &h.z, &l.z);
  ff_split(u.w, &h.w, &l.w);
  hi[c] = h;
  lo[c] = l;
}
// State exchange with a caller's host array, read and written by the GPU in place where the
// device shares the host's page tables (Grace: NVLink-C2C with address translation): u is
// AoS [N][5] in the original cell order, and iperm maps an original cell to its device cell.
// A block moves kXferCells consecutive original cells. Their 5 * kXferCells doubles cross the
// host link as consecutive words, 256 contiguous bytes per warp and instruction, and are
// regrouped per cell in shared memory. The device side takes the scattered accesses.
constexpr int kXferCells = 256;
static __global__ void __launch_bounds__(kXferCells) k_state_from_host(int n, const double* __restrict__ u,
                                                                       const int* __restrict__ iperm,
                                                                       d4* __restrict__ Un) {
  __shared__ double buf[5 * kXferCells];
  const int c0 = blockIdx.x * kXferCells;
  const int cnt = min(kXferCells, n - c0);
  const double* src = u + 5 * static_cast<size_t>(c0);
  for (int i = threadIdx.x; i < 5 * cnt; i += kXferCells) buf[i] = src[i];
  __syncthreads();
  const int t = threadIdx.x;
  if (t < cnt) {
    const double* s = buf + 5 * t;
    Un[iperm[c0 + t]] = d4{s[0], s[1], s[2], s[4]};
  }
}
static __global__ void __launch_bounds__(kXferCells) k_state_to_host(int n, const d4* __restrict__ Un,
                                                                     const int* __restrict__ iperm,
                                                                     double* __restrict__ u) {
  __shared__ double buf[5 * kXferCells];
  const int c0 = blockIdx.x * kXferCells;
  const int cnt = min(kXferCells, n - c0);
  const int t = threadIdx.x;
  if (t < cnt) {
    const d4 v = Un[iperm[c0 + t]];
    double* s = buf + 5 * t;
    s[0] = v.x;
    s[1] = v.y;
    s[2] = v.z;
    s[3] = 0.0;
    s[4] = v.w;
  }
  __syncthreads();
  double* dst = u + 5 * static_cast<size_t>(c0);
  for (int i = t; i < 5 * cnt; i += kXferCells) dst[i] = buf[i];
}

static __global__ void k_combine_state(int n, const float4* __restrict__ hi, const float4* __restrict__ lo,
                                       d4* __restrict__ Un) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const float4 h = hi[c], l = lo[c];
  Un[c] = d4{double(h.x) + double(l.x), double(h.y) + double(l.y), double(h.z) + double(l.z),
             double(h.w) + double(l.w)};
}
static __global__ void k_prim_from_image(int n, const float4* __restrict__ hi, float4* __restrict__ W, float gamma) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const float4 h = hi[c];
  const Prim<float> w = cons_to_prim(Cons<float>{h.x, h.y, h.z, h.w}, gamma);
  W[c] = make_float4(w.r, w.u, w.v, w.p);
}

}  // namespace aero
