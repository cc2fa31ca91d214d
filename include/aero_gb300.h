/* aero_gb300.h -- C ABI of the GB300 (sm_103a) Euler residual-and-update path.
 *
 * This library replaces the device seam of AeroCFD's CUDA backend
 * (src/cfd_core/include/cfd_core/cuda_backend.hpp:44-52:
 *  init_euler_device_buffers / euler_residual_cuda / free_euler_device_buffers)
 * and the stage loop of run_euler_airfoil_case
 * (src/cfd_core/solvers/euler_solver.cpp:771-1208) with a device-resident solver.
 * Paths in citations are relative to the AeroCFD project root.
 *
 * Conventions
 *  - Plain C types only: pointers, sizes, ints and doubles. Every call returns an int
 *    status (AERO_OK = 0); aero_last_error(ctx) gives a message for the last failure
 *    on that context (the reference returns bool + std::string, euler_backend.cu:11-19).
 *  - Arrays passed in or out are host arrays in the reference layout and the
 *    reference's ORIGINAL cell/face numbering: conserved state is AoS [cell][5]
 *    = (rho, rho*u, rho*v, rho*w, rho*E); geometry is AoS xyz. The library renumbers
 *    internally and converts to its device layout (SoA, cell-owned face slots).
 *  - One context per host thread. A context owns its device memory and a private
 *    CUDA stream; calls on it are synchronous with respect to the host unless the
 *    function says otherwise.
 *  - The library has no CPU fallback: aero_create fails with AERO_ERR_CUDA when no
 *    CUDA device is usable.
 */
#ifndef AERO_GB300_H
#define AERO_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* 3: aero_case_desc gained cells_per_thread; aero_autotune writes 12 timings */
#define AERO_ABI_VERSION 4

#if defined(__GNUC__)
#define AERO_API __attribute__((visibility("default")))
#else
#define AERO_API
#endif

enum aero_status {
  AERO_OK = 0,
  AERO_ERR_INVALID = 1,   /* bad argument (std::invalid_argument in the reference) */
  AERO_ERR_CUDA = 2,      /* CUDA runtime error or no device */
  AERO_ERR_NONFINITE = 3, /* non-finite state trapped (euler_solver.cpp:908-946) */
  AERO_ERR_STATE = 4,     /* call not valid in the context's current state */
  AERO_ERR_TIMEOUT = 5,   /* a bounded device wait gave up */
  AERO_ERR_NOMEM = 6      /* device allocation failed */
};

/* Boundary type per face (mesh_geometry.hpp:9-13). */
enum aero_bc { AERO_BC_INTERIOR = 0, AERO_BC_FARFIELD = 1, AERO_BC_WALL = 2 };
/* euler_flux.hpp:22-25 and reconstruction.hpp:10-13 */
enum aero_flux { AERO_FLUX_RUSANOV = 0, AERO_FLUX_HLLC = 1 };
enum aero_limiter { AERO_LIMITER_MINMOD = 0, AERO_LIMITER_VENKAT = 1 };
/* Arithmetic of the residual (bulk) path.
 *  FP64: everything in double ("plain FP64").
 *  FP32: gradients, reconstruction, fluxes and residual in float; face normals and
 *        volumes stored in double; the conserved state across RK stages, the
 *        preconditioned residual, residual norms and force sums in double. */
enum aero_precision { AERO_PRECISION_FP64 = 0, AERO_PRECISION_FP32 = 1 };
/* Cell renumbering applied inside the library. */
enum aero_ordering { AERO_ORDER_NONE = 0, AERO_ORDER_MORTON = 1, AERO_ORDER_RCM = 2 };

/* Mesh in the reference's UnstructuredMesh layout (src/cfd_core/include/cfd_core/
 * mesh.hpp:14-35), geometry widened to double (float geometry converts exactly). */
typedef struct aero_mesh_desc {
  int num_cells;
  int num_faces;
  const int* face_owner;     /* [F] */
  const int* face_neighbor;  /* [F]; -1 on boundary faces */
  const int* face_bc;        /* [F]; enum aero_bc (0 on interior faces) */
  const double* face_normal; /* [3F] unit normal pointing out of the owner */
  const double* face_center; /* [3F] */
  const double* face_area;   /* [F] face length in 2D */
  const double* cell_volume; /* [N] cell area in 2D */
  const double* cell_center; /* [3N] */
  int num_wall_faces;        /* faces of the "wall" patch used for forces and Cp */
  const int* wall_faces;     /* [num_wall_faces] in patch order (forces.cpp:152-175) */
} aero_mesh_desc;

/* Case settings: the fields of EulerAirfoilCaseConfig that the path reads
 * (src/cfd_core/include/cfd_core/solvers/euler_solver.hpp:14-74). Real-valued
 * fields carry the case file's float values widened to double. Flags are 0/1.
 * aero_case_defaults() fills the reference's defaults. */
typedef struct aero_case_desc {
  double gamma, gas_constant, mach, aoa_deg, p_inf, t_inf, rho_inf;
  double chord, x_ref, y_ref;
  int flux;    /* enum aero_flux */
  int limiter; /* enum aero_limiter */
  int iterations, min_iterations;
  int cfl_ramp_iters;
  double cfl_start, cfl_max;
  double residual_reduction_target, force_stability_tol, force_mean_drift_tol;
  int force_stability_window;
  int startup_first_order_iters;
  int rk_stages; /* 1 or 3 */
  int local_time_stepping;
  int precond_on; /* effective flag: the caller applies any environment gating */
  double precond_mach_ref, precond_mach_min, precond_beta_min, precond_beta_max;
  int precond_farfield_bc;
  double stab_floor_start, stab_floor_target, stab_floor_k_start, stab_floor_k_target;
  int stab_ramp_iters;
  int low_mach_fix;
  double mach_cutoff;
  int all_speed_flux_fix;
  double all_speed_mach_cutoff, all_speed_f_min;
  int all_speed_ramp_start_iter, all_speed_ramp_iters;
  int all_speed_staged_controller;
  int all_speed_stage_a_min_iters, all_speed_stage_a_max_iters;
  double all_speed_stage_f_min_high, all_speed_stage_f_min_mid, all_speed_stage_f_min_low;
  double all_speed_pjump_wall_target, all_speed_pjump_spike_factor;
  int all_speed_pjump_hold_iters, all_speed_freeze_iters;
  double all_speed_cfl_drop_factor, all_speed_cfl_restore_factor, all_speed_cfl_min_scale;
  int aoa0_symmetry_enforce, aoa0_symmetry_enforce_interval;
  int precision; /* enum aero_precision */
  int ordering;  /* enum aero_ordering */
  int block_size; /* threads per block of the cell kernels (64, 128 or 256); 0 = default */
  int diagnostics; /* 1: also form the pressure-jump energies of every iteration */
  /* > 0: the run also stops (converged) once min_iterations are done and the density
   * residual's L2 norm has fallen to this fraction of its first value (the per-case mask of
   * a batched sweep); 0: the reference's stop rule only. No reference counterpart. */
  double density_l2_target;
  /* cells per thread of the gradient pass's gather kernel (1 or 2; 0 = 1): with 2, each thread
   * computes two cells of adjacent blocks and issues their loads together. Results are the
   * same bit for bit. The bulk-copy gradient keeps one cell per thread. No reference
   * counterpart (picked by aero_autotune). */
  int cells_per_thread;
  /* FP32-bulk contexts with the residual preconditioner on: arithmetic of the preconditioned
   * energy row (preconditioning.cpp:51-76, the cell beta of :9-32).
   *  -1: float;
   *   1: IEEE double, beta included (the FP64 contexts' arithmetic);
   *   2: beta in float, the row in double-float arithmetic (error-free products and sums on
   *      the float pipe, about 44 significant bits);
   *   0: 2 when the free-stream Mach number is below 0.1, else -1 (default).
   * FP64 contexts always form it in double. No reference counterpart (the reference computes
   * it in float). */
  int precond_fp64;
} aero_case_desc;

/* One record per pseudo-time iteration: the rows of residuals.csv and forces.csv
 * (euler_solver.cpp:1161-1175) plus the controller state. */
typedef struct aero_iter_record {
  int iter;
  int flags; /* AERO_REC_* bits */
  int first_order_fallback_faces, diffusive_fallback_faces;
  double residual_l1, residual_l2, residual_linf, residual_ratio;
  double cl, cd, cm, lift, drag, moment;
  double cl_abs, cd_abs, cm_abs;
  double fx_gauge, fy_gauge, fx_abs, fy_abs, sum_nax, sum_nay;
  double dcl, dcd, dcm, mean_dcl, mean_dcd, mean_dcm;
  double cfl, cfl_scale;
  double stab_mach_floor, all_speed_f_min, all_speed_ramp_weight;
  double max_abs_dp_domain, max_abs_dp_wall;
  double p_jump_energy_nd, p_jump_energy_wall_nd;
  /* wall and far-field monitors (euler_solver.cpp:976-1026) */
  double max_wall_un, max_wall_mass_flux, wall_cp_min, wall_cp_max;
  double max_farfield_abs_dp, max_farfield_abs_drho, max_farfield_abs_du, max_farfield_abs_dv;
  int wall_cp_nonfinite;
  int controller_action; /* all-speed controller action code (euler_solver.cpp:1068-1139) */
  /* L2 norm of the density residual / its first value (no reference counterpart) */
  double residual_rho_ratio;
} aero_iter_record;

enum aero_record_flags {
  AERO_REC_FORCE_WINDOW_STABLE = 1,
  AERO_REC_FORCE_DRIFT_STABLE = 2,
  AERO_REC_CONVERGED = 4,
  AERO_REC_SECOND_ORDER = 8,
  AERO_REC_NONFINITE = 16,
  AERO_REC_ALL_SPEED_FIX = 32,
  AERO_REC_STAGE_A = 64,
  AERO_REC_STAGE_B = 128
};

typedef struct aero_ctx aero_ctx;

/* Library identity. */
AERO_API int aero_abi_version(void);
AERO_API const char* aero_version(void);
/* 1 when a CUDA device of compute capability 10.x is usable (the reference's
 * cuda_available(), residual_stub.cpp:300-306). */
AERO_API int aero_cuda_available(void);

/* Fill *c with the reference's defaults (euler_solver.hpp:14-74). */
AERO_API void aero_case_defaults(aero_case_desc* c);

/* Replaces init_euler_device_buffers (cuda_backend.hpp:44-46): validates and copies
 * the mesh, renumbers cells, builds the cell-owned face slots, allocates all device
 * state and sets the conserved state to the freestream. */
AERO_API int aero_create(const aero_mesh_desc* mesh, const aero_case_desc* cfg, aero_ctx** out);
/* Replaces free_euler_device_buffers (cuda_backend.hpp:47). Null is a no-op. */
AERO_API void aero_destroy(aero_ctx* ctx);
AERO_API const char* aero_last_error(const aero_ctx* ctx);

/* Conserved state, AoS [N][5], original cell order. */
AERO_API int aero_set_state(aero_ctx* ctx, const double* conserved);
AERO_API int aero_get_state(aero_ctx* ctx, double* conserved);
/* Primitive fields of the current state (rho, u, v, p), each [N] original order. */
AERO_API int aero_get_primitive(aero_ctx* ctx, double* rho, double* u, double* v, double* p);

/* One residual evaluation on the given conserved state (replaces euler_residual_cuda,
 * cuda_backend.hpp:49-52, and covers the gradient and MUSCL steps the reference
 * runs on the CPU). residual [N][5] and spectral_radius [N] in original order;
 * gradients may be null, else [N][5][2] primitive gradients (rho,u,v,w,p x,y).
 * stab_mach_floor, all_speed_f_min and all_speed_ramp_weight are the per-iteration
 * controller values (euler_solver.cpp:772-797). The context's state is unchanged. */
AERO_API int aero_residual(aero_ctx* ctx, const double* conserved, int second_order,
                  double stab_mach_floor, int all_speed_flux_fix, double all_speed_f_min,
                  double all_speed_ramp_weight, double* residual, double* spectral_radius,
                  double* gradients);

/* Run up to n pseudo-time iterations on the device (iteration loop of
 * euler_solver.cpp:771-1208: CFL ramp, adaptive CFL scale, first-order startup,
 * stabilization-floor ramp, all-speed ramp, RK stages, norms, forces, convergence
 * monitor). records may be null, else receives one record per executed iteration.
 * *n_done receives the number executed (fewer than n when the monitor converged or
 * the non-finite trap fired; then AERO_ERR_NONFINITE is returned). Calls continue
 * the same run: the iteration counter and controller state persist in the context. */
AERO_API int aero_run(aero_ctx* ctx, int n, aero_iter_record* records, int* n_done);
/* Restart the iteration counter and controller state (state is kept). */
AERO_API int aero_reset_run(aero_ctx* ctx);

/* Last residual (pre-preconditioning, last RK stage) and spectral radius of the
 * last executed iteration (EulerRunResult::last_residual / last_spectral_radius). */
AERO_API int aero_get_last_residual(aero_ctx* ctx, double* residual, double* spectral_radius);

/* Timing helper: run n iterations with no records copied out and report the device
 * time between CUDA events recorded on the context's stream around them. Uses the
 * CUDA graph of one iteration when use_graph is 1. With flush_l2 = 1 a 256 MiB buffer
 * is overwritten before every iteration (outside the timed intervals) so that no
 * iteration starts with its working set in L2. */
AERO_API int aero_time_iterations(aero_ctx* ctx, int n, int use_graph, int flush_l2,
                                  double* device_ms);
/* Per-kernel profile of n iterations, every launch between its own CUDA events.
 * ms[6] receives summed device time and launches[6] the launch count of the kernel
 * classes 0 gradient, 1 residual face pass (and, with global time stepping, its cell
 * pass), 2 update (which gathers the cell residual itself under local time stepping),
 * 3 global-time-step reduction, 4 symmetry/pressure-jump, 5 controller. */
AERO_API int aero_profile_kernels(aero_ctx* ctx, int n, int flush_l2, double* ms, int* launches);

/* In-graph attribution of n iterations (no reference counterpart): the iterations run exactly
 * as aero_time_iterations runs them with use_graph = 1 (the same CUDA graphs; the controller
 * on its side stream beside the next iteration's first kernels) while the CUPTI activity API
 * records every kernel's start and end on the GPU, without serialising them. ms[6] /
 * launches[6]: summed kernel time and launches per class as in aero_profile_kernels (class 5,
 * the controller, overlaps other kernels); *iteration_ms: the device time of the n
 * iterations between CUDA events. CUPTI is loaded at run time; without it the call returns
 * AERO_ERR_STATE. One profiling session runs at a time in a process. */
AERO_API int aero_profile_graph(aero_ctx* ctx, int n, int flush_l2, double* ms, int* launches,
                                double* iteration_ms);

/* Make `device` the current device of the library's CUDA runtime for this host thread
 * (contexts created afterwards on this thread live there). */
AERO_API int aero_select_device(int device);

/* Allocation-free residual. No counterpart in the reference: an addition for callers that
 * cannot allocate device memory while they evaluate the residual -- code running under
 * another framework's memory pool, which owns all device memory, or solver loops whose memory
 * is fixed up front (cudaMalloc/cudaFree may synchronise the device).
 * Computes what aero_residual computes (gradients only internally), but takes DEVICE
 * pointers owned by the caller: conserved_dev [N][5] and residual_dev [N][5] double in the
 * original cell order, spectral_radius_dev [N] double. It allocates nothing: its working
 * arrays live in one fixed device array of the library (about 16.8 MB, held by every CUDA
 * context that loads the library -- one per GPU for the runtime's primary context -- until
 * exit), so meshes above 65,536 cells or 196,608 faces are rejected with AERO_ERR_INVALID.
 * The work is queued on `stream` (null: the context's stream) and the call returns without
 * waiting. The first call in each CUDA context looks up that array's address; make it before
 * any stream capture. All calls in one CUDA context share the array and it keeps the last
 * call's contents: calls whose work overlaps on the GPU race and must be ordered by the
 * caller (one stream, or events). */
AERO_API int aero_residual_noalloc(aero_ctx* ctx, const double* conserved_dev, int second_order,
                                   double stab_mach_floor, int all_speed_flux_fix,
                                   double all_speed_f_min, double all_speed_ramp_weight,
                                   double* residual_dev, double* spectral_radius_dev, void* stream);

/* Sizes and kernel-launch counts of the context, for roofline accounting:
 * info[0] cells, [1] faces, [2] slots per cell (padded), [3] kernel launches per
 * iteration, [4] bytes of device memory held, [5] precision, [6] block size, [7] cell
 * blocks, [8] cases, [9] 1 when the iterations' gradient pass streams its tiles through
 * shared memory with bulk copies (bounded waits), 0 for the plain gather kernel. */
AERO_API int aero_get_info(aero_ctx* ctx, long long* info, int n_info);

/* Poll limit of the bounded waits the iterations' kernels make on their bulk copies (no
 * reference counterpart; the reference has no device waits). polls < 0 restores the default,
 * about one second. A wait that runs out makes its kernel stop issuing copies, wait for the
 * copies it has in flight and return; the iteration it belonged to is then not applied (the
 * conserved state keeps its previous value, no record is written for it), aero_run and the
 * timing calls return AERO_ERR_TIMEOUT, and the next aero_run continues from the last applied
 * iteration. */
AERO_API int aero_set_wait_limit(aero_ctx* ctx, int polls);

/* Autotuner (no reference counterpart): times `iters` second-order iterations of the case on
 * this mesh for every cell ordering (Morton, RCM), block size (64, 128, 256) and number of
 * cells per thread of the gradient pass (1, 2), each in its own context after the case's
 * first-order start-up, and writes the case with the fastest combination into *best (all
 * other fields copied from *c). ms_out (may be NULL) receives the 12 device times in ms,
 * ordering-major, then block size, then cells per thread: [Morton 64/1, 64/2, 128/1, 128/2,
 * 256/1, 256/2, RCM 64/1, ...]. */
AERO_API int aero_autotune(const aero_mesh_desc* mesh, const aero_case_desc* c, int iters, aero_case_desc* best,
                           double* ms_out);

#ifdef __cplusplus
}
#endif

#endif /* AERO_GB300_H */
