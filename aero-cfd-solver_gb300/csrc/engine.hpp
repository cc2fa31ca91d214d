// engine.hpp -- precision-independent interface of the device solver behind the C ABI.
#pragma once

#include "../../include/aero_gb300.h"
#include "mesh_prep.hpp"

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace aero {

// Case settings resolved on the host (euler_solver.cpp:340-357, 120-140, 493-566), in double.
struct Resolved {
  double gamma;
  double cons_inf[4];  // rho, rho*u, rho*v, rho*E of the freestream
  double p_inf, rho_inf, v_inf, a_inf, q_inf, pressure_ref;
  double pc_mach_ref, pc_mach_min, pc_beta_min, pc_beta_max;
  double stab_start, stab_target;
  double as_fmin;
  double st_fmin_high, st_fmin_mid, st_fmin_low;
  double pj_target, pj_spike, cfl_drop, cfl_restore, cfl_min_scale;
  double cos_a, sin_a;
  int lm;  // any low-Mach feature on
};

// Read-only device view of a single-case context for launches issued outside the engine.
// dm / df / dg point at the engine's DevMesh<T> / DevFaces<T> / DevGather<T>; fps, pcs, mcs
// at its device arrays of FaceParams<T> / PrecondD / MonitorConsts (T per `precision`);
// cblk / fblk are the block -> (case, end) tables of the cell and face kernels.
struct EngineView {
  int n;      // cells
  int ntot;   // cells padded to whole blocks (the stride of the per-cell arrays)
  int nf;     // faces padded to whole blocks
  int cblocks, fblocks;
  int precision;  // enum aero_precision
  int flux;
  int lm;
  int block;
  int device;
  double gamma;  // case 0
  const void* dm;
  const void* df;
  const void* dg;
  const void* fps;
  const void* pcs;
  const void* mcs;
  const int2* cblk;
  const int2* fblk;
  const int* perm_dev;  // new -> original cell, on the device
  cudaStream_t stream;
};

// Device solver for one or more cases packed into one set of arrays. Cases of one engine
// share the numerics that select kernel variants (flux, limiter, low-Mach switches, RK
// stages, time-step mode, start-up length, precision, block size); the flow conditions,
// CFL schedules and stop rules are per case. Single-case functions address case 0.
class Engine {
 public:
  virtual ~Engine() = default;
  virtual EngineView view() const = 0;
  virtual bool init(std::string* err) = 0;
  virtual int n_cases() const = 0;
  virtual void set_state(int cs, const double* u_orig) = 0;
  virtual void get_state(int cs, double* u_orig) = 0;
  virtual void get_primitive(int cs, double* rho, double* u, double* v, double* p) = 0;
  virtual void residual(const double* u_orig, int second, double stab, int as_fix, double as_fmin,
                        double as_ramp, double* res, double* sr, double* grad) = 0;
  // records: case k's records at recs + k * n (may be null); n_done[k] iterations run
  virtual int run(int n, aero_iter_record* recs, int* n_done) = 0;
  virtual void reset_run() = 0;
  virtual void last_residual(int cs, double* res, double* sr) = 0;
  virtual int time_iterations(int n, int use_graph, int flush_l2, double* ms) = 0;
  virtual int profile_kernels(int n, int flush_l2, double* ms, int* launches) = 0;
  virtual void info(long long* out, int n) = 0;
  virtual cudaError_t last_cuda_error() = 0;
  virtual int set_wait_limit(int polls) = 0;
  virtual bool uses_bulk_copy_gradient() const = 0;

  // Discrete adjoint at the current state (single-case FP64 contexts; others return
  // AERO_ERR_INVALID). Objective J = w_cd CD + w_cl CL; second_order -1: the run's scheme at
  // the current iteration. Host arrays are [N][5] in the original order.
  virtual int adjoint_linearize(double w_cd, double w_cl, int second_order) = 0;
  virtual int adjoint_vjp(const double* v, double* out) = 0;
  virtual int adjoint_objective_gradient(double* g) = 0;
  virtual int adjoint_solve(int iters, double cfl, double* history) = 0;
  virtual int adjoint_lambda(double* lam) = 0;
  virtual int adjoint_set_lambda(const double* lam) = 0;
  virtual int adjoint_solve_krylov(int max_iters, int restart, int smooth, double cfl, double rtol,
                                   double* history, int* done) = 0;
  virtual int adjoint_dalpha(double* dj_dalpha_deg) = 0;
  virtual int adjoint_geometry(const aero_mesh_desc& tangent, double* dj) = 0;
  virtual int adjoint_geometry_vjp(double* d_normal, double* d_center, double* d_area, double* d_volume,
                                   double* d_cell_center) = 0;
};

Engine* make_engine_f32(const std::vector<HostSlots>& hs, const std::vector<aero_case_desc>& cfg,
                        const std::vector<Resolved>& rs, cudaStream_t stream);
Engine* make_engine_f64(const std::vector<HostSlots>& hs, const std::vector<aero_case_desc>& cfg,
                        const std::vector<Resolved>& rs, cudaStream_t stream);

}  // namespace aero
