"""Generate the golden vectors under tests/golden/ from the reference AeroCFD library.

The reference is compiled from its own sources by `make -C oracle ref` (into
oracle/_ref/, never committed) and driven through oracle/ref_shim.cpp. Run from the
repository root on a machine where the reference sources are mounted:

    python tests/golden/make_golden.py --ref-root <AeroCFD source root>

Outputs (all values exactly as the reference computed them, in float32):
  meshes.npz     reference meshes: demo 2x2 (src/cfd_core/mesh/mesh.cpp:44) and
                 O-grids from make_airfoil_ogrid_mesh (airfoil_mesh.cpp:459)
  residuals.npz  gradients, residuals, spectral radii and fallback counters of one
                 assemble_euler_residual_cpu call (residual_assembly.cpp:73) per
                 numerics combination, on seeded states of the 32x4 O-grid
  histories.npz  per-iteration (iter, l1, l2, linf, cl, cd, cm), final conserved state
                 and last residual of run_euler_airfoil_case_cpu for the case settings of
                 the reference's own C++ tests and a few added numerics combinations
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "aero-cfd-solver_gb300" / "python"))

from aero_gb300 import capi  # noqa: E402
from oracle import oracle_py as op  # noqa: E402
from oracle import oracle_types as ot  # noqa: E402

OUT = Path(__file__).resolve().parent
_dp = C.POINTER(C.c_double)

OGRIDS = {  # name: (n_circ, n_radial, farfield_radius, stretch)
    "ogrid_32x4": (32, 4, 10.0, 1.25),
    "ogrid_40x8": (40, 8, 10.0, 1.25),
    "ogrid_48x10": (48, 10, 10.0, 1.25),
    "ogrid_64x14": (64, 14, 12.0, 1.35),
    "ogrid_72x18": (72, 18, 12.0, 1.35),
}

# Numerics combinations of the residual fixtures. Precondition values are fixed points of
# build_precondition_config (euler_solver.cpp:340-357), so the shim can use them as given.
RESIDUAL_COMBOS = []
for flux in (capi.FLUX_RUSANOV, capi.FLUX_HLLC):
    for lim in (capi.LIMITER_MINMOD, capi.LIMITER_VENKAT):
        for lowmach in (0, 1):
            RESIDUAL_COMBOS.append(dict(flux=flux, limiter=lim, precond_on=lowmach,
                                        low_mach_fix=lowmach, all_speed_flux_fix=lowmach,
                                        precond_farfield_bc=lowmach))
RESIDUAL_CASE_BASE = dict(mach=0.3, aoa_deg=2.0, gas_constant=1.0, p_inf=1.0, t_inf=1.0, rho_inf=1.0)

# Whole-run settings. The first five are the case settings of the reference's C++ tests
# (tests/cpp/test_euler_parity.cpp:15-35, test_euler_regression.cpp:9-30,
#  test_euler_aoa0_regression.cpp:11-30, test_euler_wall_sanity.cpp:13-35,
#  test_euler_low_mach_asymptotic.cpp:135-197 with the CI thresholds of
#  tests/data/baselines/low_mach_euler/expected.yaml).
LOW_MACH = dict(iterations=1200, min_iterations=300, cfl_start=0.10, cfl_max=0.6, cfl_ramp_iters=180,
                residual_reduction_target=1e-3, force_stability_tol=3e-3, force_stability_window=6,
                force_mean_drift_tol=3e-3, startup_first_order_iters=30, rk_stages=3,
                precond_mach_ref=0.01, precond_mach_min=1e-3, precond_beta_min=1e-4,
                stab_floor_k_start=5.0, stab_floor_k_target=1.0, stab_ramp_iters=700,
                flux=capi.FLUX_HLLC, limiter=capi.LIMITER_MINMOD, mach_cutoff=0.3,
                all_speed_mach_cutoff=0.25, all_speed_f_min=0.05, all_speed_ramp_start_iter=100,
                all_speed_ramp_iters=200, all_speed_stage_a_min_iters=0,
                all_speed_pjump_hold_iters=160, all_speed_freeze_iters=160,
                all_speed_cfl_drop_factor=0.7, all_speed_cfl_min_scale=0.05, mach=0.01, aoa_deg=0.0)
RUNS = {
    "parity": ("ogrid_48x10", dict(gas_constant=1.0, p_inf=0.05, t_inf=1.0, rho_inf=1.0, iterations=26,
                                   min_iterations=26, cfl_start=0.0, cfl_max=0.0, cfl_ramp_iters=1,
                                   residual_reduction_target=0.0, force_stability_tol=0.0, rk_stages=1,
                                   startup_first_order_iters=1000), False),
    "regression": ("ogrid_72x18", dict(iterations=80, min_iterations=20, cfl_start=0.15, cfl_max=0.7,
                                       cfl_ramp_iters=80, residual_reduction_target=1e-2,
                                       force_stability_tol=5e-4, force_stability_window=6,
                                       startup_first_order_iters=25, mach=0.15, aoa_deg=2.0), False),
    "aoa0": ("ogrid_64x14", dict(iterations=12, min_iterations=12, cfl_start=0.15, cfl_max=0.7,
                                 cfl_ramp_iters=12, residual_reduction_target=1e-2,
                                 force_stability_tol=5e-4, startup_first_order_iters=25, mach=0.15,
                                 aoa_deg=0.0), False),
    "wall_sanity": ("ogrid_40x8", dict(iterations=1, min_iterations=1, cfl_start=0.0, cfl_max=0.0,
                                       cfl_ramp_iters=1, residual_reduction_target=0.0,
                                       force_stability_tol=0.0, flux=capi.FLUX_HLLC,
                                       limiter=capi.LIMITER_VENKAT, precond_on=1, mach=0.2,
                                       aoa_deg=0.0), False),
    "low_mach_off": ("ogrid_72x18", dict(LOW_MACH, all_speed_flux_fix=0), False),
    "low_mach_on": ("ogrid_72x18", dict(LOW_MACH, all_speed_flux_fix=1), False),
    # Added combinations: HLLC + venkat with the characteristic far field; the low-Mach
    # preconditioner path (enabled through AERO_ENABLE_EXPERIMENTAL_PRECOND); the staged
    # all-speed controller (stage A times out into stage B); global time stepping, RK1.
    "hllc_venkat": ("ogrid_48x10", dict(iterations=60, min_iterations=60, flux=capi.FLUX_HLLC,
                                        limiter=capi.LIMITER_VENKAT, startup_first_order_iters=10,
                                        mach=0.5, aoa_deg=1.25, precond_farfield_bc=1), False),
    "precond": ("ogrid_40x8", dict(iterations=40, min_iterations=40, flux=capi.FLUX_HLLC,
                                   limiter=capi.LIMITER_VENKAT, precond_on=1, low_mach_fix=1,
                                   all_speed_flux_fix=1, precond_farfield_bc=1,
                                   startup_first_order_iters=5, mach=0.05, aoa_deg=3.0,
                                   precond_mach_ref=0.05, precond_beta_min=1e-4), True),
    "staged": ("ogrid_48x10", dict(iterations=150, min_iterations=150, flux=capi.FLUX_HLLC,
                                   limiter=capi.LIMITER_MINMOD, all_speed_flux_fix=1,
                                   all_speed_staged_controller=1, all_speed_stage_a_min_iters=1000,
                                   all_speed_stage_a_max_iters=40, all_speed_ramp_iters=30,
                                   all_speed_pjump_hold_iters=10, all_speed_freeze_iters=5,
                                   startup_first_order_iters=20, mach=0.05, aoa_deg=1.0,
                                   aoa0_symmetry_enforce=1, aoa0_symmetry_enforce_interval=7), False),
    "global_dt_rk1": ("ogrid_40x8", dict(iterations=50, min_iterations=50, rk_stages=1,
                                         local_time_stepping=0, cfl_start=0.5, cfl_max=0.9,
                                         flux=capi.FLUX_RUSANOV, limiter=capi.LIMITER_VENKAT,
                                         startup_first_order_iters=10, mach=0.3, aoa_deg=4.0), False),
}


def export_mesh(name: str) -> dict:
    ref = op.ref_lib()
    if name == "demo_2x2":
        ref.ref_demo_mesh_build()
    else:
        nc, nr, radius, stretch = OGRIDS[name]
        if ref.ref_ogrid_build(b"0012", nc, nr, radius, stretch, 1.0) != 0:
            raise RuntimeError(ref.ref_last_error().decode())
    return op.ref_current_mesh()


def to_mesh(m: dict) -> capi.Mesh:
    return capi.Mesh(m["owner"], m["neighbor"], m["bc"], m["normal"], m["center"], m["area"],
                     m["volume"], m["cell_center"], m["wall_faces"])


def seeded_state(mesh: capi.Mesh, case, seed: int, stress: bool) -> np.ndarray:
    """Freestream plus smooth and random perturbations, rounded to float32."""
    sol = op.OracleSolver(op.MODE_FLOAT, mesh, case)
    u = sol.get_state().copy()
    sol.close()
    rng = np.random.default_rng(seed)
    x = mesh.cell_center.reshape(-1, 3)
    smooth = 0.1 * np.sin(1.3 * x[:, 0]) * np.cos(0.7 * x[:, 1])
    for k in (0, 1, 2, 4):
        u[:, k] *= 1.0 + smooth + 0.05 * rng.standard_normal(len(u))
    u[:, 3] = 0.0
    if stress:  # near-vacuum cells force MUSCL fallbacks and HLLC edge cases
        idx = rng.choice(len(u), size=max(2, len(u) // 40), replace=False)
        ke = 0.5 * (u[idx, 1] ** 2 + u[idx, 2] ** 2) / u[idx, 0]
        u[idx, 4] = ke + 1e-6
        u[idx[:1], 0] = 1e-7
    return u.astype(np.float32).astype(np.float64)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", required=True, help="root of the AeroCFD sources to compile")
    args = ap.parse_args()
    op.build(ref_root=args.ref_root)

    meshes = {"demo_2x2": export_mesh("demo_2x2")}
    for name in OGRIDS:
        meshes[name] = export_mesh(name)
    flat = {}
    for name, m in meshes.items():
        for key, val in m.items():
            flat[f"{name}/{key}"] = val
    np.savez_compressed(OUT / "meshes.npz", **flat)

    # --- single residual evaluations ---------------------------------------------------
    res = {}
    meta = []
    mesh = to_mesh(meshes["ogrid_32x4"])
    for ci, combo in enumerate(RESIDUAL_COMBOS):
        case = capi.make_case(**RESIDUAL_CASE_BASE, **combo)
        for stress in (False, True):
            u = seeded_state(mesh, case, seed=100 + ci, stress=stress)
            for second in (0, 1):
                key = f"c{ci}_s{int(stress)}_o{second}"
                r, s, g, diag = op.ref_residual(mesh, case, u, second, stab=0.02, as_fix=combo["all_speed_flux_fix"],
                                                as_fmin=0.05, as_ramp=0.7)
                res[key + "/u"] = u.astype(np.float32)
                res[key + "/r"] = r.astype(np.float32)
                res[key + "/sr"] = s.astype(np.float32)
                res[key + "/g"] = g.astype(np.float32)
                res[key + "/diag"] = np.array(diag, np.int32)
                meta.append(dict(key=key, mesh="ogrid_32x4", case={**RESIDUAL_CASE_BASE, **combo},
                                 second_order=second, stab=0.02, as_fix=combo["all_speed_flux_fix"],
                                 as_fmin=0.05, as_ramp=0.7))
    np.savez_compressed(OUT / "residuals.npz", meta=np.array(json.dumps(meta)), **res)

    # --- whole runs ------------------------------------------------------------------------
    hist = {}
    hmeta = {}
    ref = op.ref_lib()
    for name, (mesh_name, kw, precond_env) in RUNS.items():
        nc, nr, radius, stretch = OGRIDS[mesh_name]
        case = capi.make_case(**kw)
        n_cells = 2 * nc * nr
        maxh = case.iterations
        h = np.zeros(maxh * 7)
        nd = C.c_int(0)
        consv = np.zeros(n_cells * 5)
        lr = np.zeros(n_cells * 5)
        ls = np.zeros(n_cells)
        mw = C.c_double(0)
        if precond_env:
            os.environ["AERO_ENABLE_EXPERIMENTAL_PRECOND"] = "1"
        else:
            os.environ.pop("AERO_ENABLE_EXPERIMENTAL_PRECOND", None)
        with tempfile.TemporaryDirectory() as d:
            rc = ref.ref_run_case(C.byref(ot.case_desc(case)), b"0012", nc, nr, radius, stretch, d.encode(),
                                  h.ctypes.data_as(_dp), maxh, C.byref(nd), consv.ctypes.data_as(_dp),
                                  lr.ctypes.data_as(_dp), ls.ctypes.data_as(_dp), C.byref(mw))
        os.environ.pop("AERO_ENABLE_EXPERIMENTAL_PRECOND", None)
        if rc != 0:
            raise RuntimeError(ref.ref_last_error().decode())
        n = nd.value
        hist[name + "/history"] = h[: 7 * n].reshape(n, 7)
        hist[name + "/conserved"] = consv.reshape(-1, 5).astype(np.float32)
        hist[name + "/last_residual"] = lr.reshape(-1, 5).astype(np.float32)
        hist[name + "/last_sr"] = ls.astype(np.float32)
        hmeta[name] = dict(mesh=mesh_name, case=kw, precond_env=precond_env,
                           max_wall_mass_flux=mw.value, iterations_done=n)
        print(f"{name}: {n} iterations, final cl={h[7 * (n - 1) + 4]:.6g} cd={h[7 * (n - 1) + 5]:.6g}")
    np.savez_compressed(OUT / "histories.npz", meta=np.array(json.dumps(hmeta)), **hist)
    for f in ("meshes.npz", "residuals.npz", "histories.npz"):
        print(f, (OUT / f).stat().st_size, "bytes")


if __name__ == "__main__":
    main()
