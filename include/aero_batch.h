/* aero_batch.h -- batched sweep: many cases (meshes of uneven size, different flow
 * conditions) advanced together in one set of device arrays and one CUDA graph per
 * iteration.
 *
 * Replaces the reference's serial sweep loop (python/cfd/sweep.py:41-56, one
 * run_case_native call per angle of attack) for the Euler airfoil path. A batched context
 * is an aero_ctx: aero_destroy, aero_time_iterations, aero_profile_kernels, aero_get_info and
 * aero_reset_run apply to all its cases; aero_run, aero_residual and the other single-case
 * calls refuse a context of more than one case.
 *
 * Cases of one batch must share the settings that select kernel variants: flux, limiter,
 * precision, rk_stages, local_time_stepping, startup_first_order_iters, precond_on, the
 * low-Mach switches and block_size. Everything else (Mach, angle of attack, free stream,
 * CFL schedule, iteration limits, stop rules including density_l2_target) is per case.
 * Each case's results equal those of running it alone in a single-case context.
 */
#ifndef AERO_BATCH_H
#define AERO_BATCH_H

#include "aero_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Create a context over n_cases cases: meshes[k] and cases[k] as for aero_create. */
AERO_API int aero_batch_create(int n_cases, const aero_mesh_desc* meshes, const aero_case_desc* cases,
                               aero_ctx** out);

/* Number of cases of a context (1 for aero_create contexts). */
AERO_API int aero_batch_size(const aero_ctx* ctx);

/* Run up to n iterations of every case that has not stopped; a case stops at its own
 * convergence (the reference's rule, or density_l2_target) or non-finite trap while the
 * others continue. records (may be NULL): n_cases * n records, case k's at records + k * n;
 * n_done[k]: iterations case k ran. AERO_ERR_NONFINITE when any case trapped. */
AERO_API int aero_batch_run(aero_ctx* ctx, int n, aero_iter_record* records, int* n_done);

/* State of case k in its original cell order, AoS [N_k][5] double. */
AERO_API int aero_batch_set_state(aero_ctx* ctx, int case_index, const double* conserved);
AERO_API int aero_batch_get_state(aero_ctx* ctx, int case_index, double* conserved);

/* Residual [N_k][5] and spectral radius [N_k] of case k's last RK stage. */
AERO_API int aero_batch_get_last_residual(aero_ctx* ctx, int case_index, double* residual,
                                          double* spectral_radius);

#ifdef __cplusplus
}
#endif

#endif /* AERO_BATCH_H */
