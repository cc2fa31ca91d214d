/* aero_adjoint.h -- discrete adjoint of the FP64 Euler residual for force objectives.
 *
 * No reference counterpart: AeroCFD computes no sensitivities. The adjoint is of the
 * residual the device path evaluates (aero_residual: gradients, MUSCL with the case's
 * limiter, the Rusanov or HLLC flux with its fallbacks, slip wall and far field, the
 * low-Mach scalings at the schedule values of the linearisation point), so that at a
 * converged state dJ/dp = dJ/dp|_U + lam^T dR/dp with (dR/dU)^T lam = -dJ/dU.
 *
 * Objective: J = w_cd * CD + w_cl * CL with CD, CL the gauge-pressure force coefficients
 * the run reports (post/forces.cpp:208-294 restated).
 *
 * Contexts: single-case FP64 contexts (aero_create with precision AERO_PRECISION_FP64).
 * Others answer AERO_ERR_INVALID. The linearisation point is the context's state when
 * aero_adjoint_linearize is called; later aero_run / aero_set_state / aero_residual calls do
 * not change it. Host arrays are AoS [N][5] in the mesh's original cell order (component 3,
 * the z momentum, is 0 on output and ignored on input).
 */
#ifndef AERO_ADJOINT_H
#define AERO_ADJOINT_H

#include "aero_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Linearise at the current state: primitives, gradients, the per-face flux Jacobians
 * (exact forward-mode derivatives of the flux code), dJ/dU, and lam = 0.
 * second_order: 1 MUSCL, 0 first order, -1 the run's scheme at the current iteration. */
AERO_API int aero_adjoint_linearize(aero_ctx* ctx, double w_cd, double w_cl, int second_order);

/* out = (dR/dU)^T v at the linearisation point. */
AERO_API int aero_adjoint_vjp(aero_ctx* ctx, const double* v, double* out);

/* dJ/dU at the linearisation point. */
AERO_API int aero_adjoint_objective_gradient(aero_ctx* ctx, double* g);

/* Advance lam by `iters` pseudo-time iterations of (dR/dU)^T lam + dJ/dU = 0 with the
 * primal's three-stage SSP Runge-Kutta smoother and local steps cfl / SR (SR the spectral
 * radius at the linearisation point). history (may be NULL): per iteration the RMS over
 * cells of (dR/dU)^T lam + dJ/dU before the iteration. Continues from the current lam. */
AERO_API int aero_adjoint_solve(aero_ctx* ctx, int iters, double cfl, double* history);

/* Restarted GMRES(restart) on (dR/dU)^T lam = -dJ/dU from the current lam, right-
 * preconditioned by smooth_iters iterations of the smoother above from zero (0: no
 * preconditioner). Needed where the smoother alone diverges: a primal that stalls in a
 * limiter limit cycle leaves a few growing modes in the linearisation. Stops when the
 * residual estimate falls to rel_tol * |dJ/dU| or after max_iters Arnoldi steps.
 * history (may be NULL, max_iters entries): residual estimate / |dJ/dU| per step;
 * iters_done (may be NULL): steps taken. */
AERO_API int aero_adjoint_solve_krylov(aero_ctx* ctx, int max_iters, int restart, int smooth_iters,
                                       double cfl, double rel_tol, double* history, int* iters_done);

/* Current adjoint state lam; set it (a warm start, or a given lam for the dalpha and
 * geometry products). */
AERO_API int aero_adjoint_get_lambda(aero_ctx* ctx, double* lam);
AERO_API int aero_adjoint_set_lambda(aero_ctx* ctx, const double* lam);

/* dJ/d(alpha) per degree with the current lam: the force-rotation term plus lam^T dR/dalpha
 * through the far-field state. */
AERO_API int aero_adjoint_dalpha(aero_ctx* ctx, double* dj_dalpha_deg);

/* dJ/dX . dX with the current lam for a geometry perturbation dX of the mesh: `tangent`
 * has the connectivity of the context's mesh and holds, in face_normal, face_center,
 * face_area, cell_volume and cell_center, the derivatives of those arrays along the
 * perturbation (aero_mesh_geometry_tangent computes them from node displacements). The
 * free stream and the reference length are held fixed. */
AERO_API int aero_adjoint_geometry(aero_ctx* ctx, const aero_mesh_desc* tangent, double* dj);

/* Reverse product with respect to the geometry, the transpose of aero_adjoint_geometry (no
 * reference counterpart): with the current lam, dJ/d(geometry) for every face normal
 * d_normal [3F], face centre d_center [3F], face length d_area [F], cell volume d_volume [N]
 * and cell centre d_cell_center [3N] in the mesh's original numbering (z entries 0), the
 * objective's own dependence through the force patch included. For every geometry tangent
 * t, aero_adjoint_geometry(t) equals the sum of these arrays times t's. */
AERO_API int aero_adjoint_geometry_vjp(aero_ctx* ctx, double* d_normal, double* d_center, double* d_area,
                                       double* d_volume, double* d_cell_center);

/* dJ/dX for every node of the generator mesh the context's mesh was described from
 * (aero_mesh_describe of `mesh`): aero_adjoint_geometry_vjp followed by
 * aero_mesh_geometry_vjp, dj_dpoints [3P] (z entries 0). One reverse pass whatever the
 * number of nodes: dJ/d(any shape parameter p) = sum of dj_dpoints * dX/dp. */
struct aero_mesh;
AERO_API int aero_adjoint_node_vjp(aero_ctx* ctx, const struct aero_mesh* mesh, double* dj_dpoints);

#ifdef __cplusplus
}
#endif

#endif /* AERO_ADJOINT_H */
