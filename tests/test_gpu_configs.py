"""Parity of the sm_103a path with the CPU oracle at the benchmark configurations' own mesh
sizes, and the configurations the benchmark measures run end to end against the oracle.

* Single residual evaluations on the 512x128 (131,072 triangles, HLLC + MUSCL venkat) and
  1024x256 (524,288 triangles, preconditioning + low-Mach fix + all-speed fix, HLLC + minmod,
  M = 0.05) triangulated, jittered, permuted O-grids:
    FP64 path vs FP64 oracle: |dR| <= 1e-12 S per cell and component, S = sum over the cell's
    faces of |F_k A| (the oracle's flux scale); spectral radius to 1e-12 relative.
    FP32 path: float-class agreement. The reference's own float arithmetic (the oracle's float
    mode, pinned bit for bit to the compiled reference) deviates from FP64 by e_ref = max
    |dR| / S; the device's float path must stay within max(5e-5, 2 e_ref) of FP64, and within
    the same bound of the reference's float residual.
* The plain-FP64 quad configuration: NACA 0012, 128x32 quad O-grid (4,096 cells, cosine
  clustering at the leading and trailing edges, first wall spacing 0.005 c, geometric growth
  to a far field at 20 c), M = 0.5, alpha = 2 deg, first-order Rusanov, local time stepping
  at CFL 0.8, 2,000 iterations: the whole CL / CD / CM and residual history against the FP64
  oracle's run of the same case.
* Per-iteration diagnostics (pressure-deviation maxima, wall normal velocity and Cp range,
  far-field deviations, wall mass flux) against the oracle's, and the reference's own
  wall-mass-flux assertions (tests/cpp/test_euler_aoa0_regression.cpp:88, <= 1e-8, and
  tests/cpp/test_euler_wall_sanity.cpp:37, <= 1e-4) on the device.
"""

import numpy as np
import pytest

import aero_gb300
from aero_gb300 import capi
from conftest import golden_mesh
from oracle import oracle_py as op

pytestmark = pytest.mark.gpu

GAMMA = 1.4


@pytest.fixture(scope="module", autouse=True)
def _device():
    lib = aero_gb300.load(build_if_missing=True)
    assert lib.aero_cuda_available(), "GPU tests need an sm_103 device"
    op.build()


def flux_err(a, b, fscale):
    return float(np.max(np.abs(a - b) / (fscale + 1e-300)))


def perturbed_state(mesh, case, seed):
    """A smooth plus random departure from the free stream sized by the flow itself: density
    by 1%, velocity by 5% of the free-stream speed, pressure by 5% of the dynamic pressure, so
    that the state is physical at any Mach number."""
    u0 = op.OracleSolver(op.MODE_DOUBLE, mesh, case).get_state()
    rho0 = u0[:, 0]
    vx, vy = u0[:, 1] / rho0, u0[:, 2] / rho0
    p0 = (GAMMA - 1.0) * (u0[:, 4] - 0.5 * rho0 * (vx * vx + vy * vy))
    speed = np.sqrt(vx * vx + vy * vy)
    q = 0.5 * rho0 * speed * speed
    x = mesh.cell_center.reshape(-1, 3)
    smooth = 0.1 * np.sin(1.3 * x[:, 0]) * np.cos(0.7 * x[:, 1])
    rng = np.random.default_rng(seed)
    n = len(rho0)
    rho = rho0 * (1.0 + 0.1 * smooth + 0.01 * rng.standard_normal(n))
    ux = vx * (1.0 + smooth) + 0.05 * speed * rng.standard_normal(n)
    uy = vy + 0.05 * speed * rng.standard_normal(n)
    p = p0 + q * (smooth + 0.05 * rng.standard_normal(n))
    u = np.zeros_like(u0)
    u[:, 0] = rho
    u[:, 1] = rho * ux
    u[:, 2] = rho * uy
    u[:, 4] = p / (GAMMA - 1.0) + 0.5 * rho * (ux * ux + uy * uy)
    return u


C2_CASE = dict(mach=0.8, aoa_deg=1.25, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT, precond_farfield_bc=1)
C3_CASE = dict(mach=0.05, aoa_deg=3.0, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_MINMOD, precond_on=1,
               low_mach_fix=1, all_speed_flux_fix=1, precond_farfield_bc=1)
# (n_circ, n_radial, seed, case, residual arguments: second order, stabilization floor,
#  all-speed fix, all-speed f_min, all-speed ramp weight)
FULL_SIZE = {
    "512x128_hllc_venkat": (512, 128, 2, C2_CASE, (1, 0.0, 0, 0.05, 1.0)),
    "1024x256_low_mach": (1024, 256, 3, C3_CASE, (1, 0.02, 1, 0.05, 0.7)),
}


@pytest.mark.parametrize("name", sorted(FULL_SIZE))
def test_residual_at_benchmark_mesh_size(name):
    nc, nr, seed, kw, args = FULL_SIZE[name]
    mesh = aero_gb300.ogrid_synthetic(nc, nr, cell_type=3, permute=True, jitter=0.1, seed=seed,
                                      wall_spacing=0.005, farfield_radius=20.0)
    assert mesh.num_cells == 2 * nc * nr and mesh.num_faces == nc * (3 * nr + 1)
    case64 = capi.make_case(**kw, precision=capi.PRECISION_FP64)
    case32 = capi.make_case(**kw, precision=capi.PRECISION_FP32)
    u = perturbed_state(mesh, case64, seed=7)
    ro, sro, go, diag_o, fs = op.OracleSolver(op.MODE_DOUBLE, mesh, case64).residual(u, *args, with_scale=True)
    rf = op.OracleSolver(op.MODE_FLOAT, mesh, case32).residual(u, *args)[0]
    with aero_gb300.Solver(mesh, case64) as s:
        r, sr, g = s.residual(u, *args)
    e64 = flux_err(r, ro, fs)
    assert e64 <= 1e-12, e64
    np.testing.assert_allclose(sr, sro, rtol=1e-12)
    assert np.max(np.abs(g - go)) / (np.abs(go).max() + 1e-300) < 1e-12
    with aero_gb300.Solver(mesh, case32) as s:
        r32, sr32, _ = s.residual(u, *args)
    e_ref = flux_err(rf, ro, fs)
    bound = max(5e-5, 2.0 * e_ref)
    e32 = flux_err(r32, ro, fs)
    assert e32 <= bound, (e32, e_ref)
    assert flux_err(r32, rf, fs) <= bound
    np.testing.assert_allclose(sr32, sro, rtol=1e-5)
    print(f"{name}: FP64 {e64:.2e}, FP32 {e32:.2e}, reference float {e_ref:.2e}")


def c1_mesh():
    return aero_gb300.ogrid_synthetic(128, 32, cell_type=4, permute=False, jitter=0.0, seed=1,
                                      wall_spacing=0.005, farfield_radius=20.0)


def c1_case(precision=capi.PRECISION_FP64, iterations=2000):
    return capi.make_case(mach=0.5, aoa_deg=2.0, flux=capi.FLUX_RUSANOV, limiter=capi.LIMITER_MINMOD,
                          cfl_start=0.8, cfl_max=0.8, startup_first_order_iters=10 ** 9, iterations=iterations,
                          min_iterations=iterations, residual_reduction_target=0.0, precision=precision)


def test_plain_fp64_quad_configuration_matches_the_oracle():
    mesh = c1_mesh()
    assert mesh.num_cells == 4096 and mesh.num_faces == 128 * (2 * 32 + 1)
    case = c1_case()
    with aero_gb300.Solver(mesh, case) as s:
        _, rec = s.run(2000)
        state = s.get_state()
    o = op.OracleSolver(op.MODE_DOUBLE, mesh, case)
    _, orec = o.run(2000)
    assert len(rec) == len(orec) == 2000
    assert not np.any(rec["flags"] & capi.REC_SECOND_ORDER)
    for key in ("cl", "cd", "cm"):
        assert np.max(np.abs(rec[key] - orec[key])) <= 1e-9, key
    l2 = orec["residual_l2"]
    assert np.max(np.abs(rec["residual_l2"] - l2) / l2) <= 1e-8
    ostate = o.get_state()
    assert np.max(np.abs(state - ostate) / (np.abs(ostate).max(axis=0) + 1e-300)) <= 1e-9
    assert rec["residual_ratio"][-1] < 1e-3  # the first-order case converges


def test_low_mach_configuration_run_tracks_the_oracle():
    """The low-Mach configuration's numerics (M = 0.05, alpha = 3 deg, preconditioning,
    low-Mach fix, all-speed flux fix, characteristic far field, HLLC + minmod, second order
    after 25 first-order iterations) on the 128x32 grid of its family, 1,500 iterations in FP64
    against the FP64 oracle's run: the histories agree to round-off growth, including the
    residual ratio's climb above 1. The case converges in neither, so that climb is the
    scheme's, not the device's."""
    mesh = aero_gb300.ogrid_synthetic(128, 32, cell_type=3, permute=True, jitter=0.1, seed=3)
    case = capi.make_case(mach=0.05, aoa_deg=3.0, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_MINMOD, precond_on=1,
                          low_mach_fix=1, all_speed_flux_fix=1, precond_farfield_bc=1, iterations=1500,
                          min_iterations=1500, cfl_start=0.2, cfl_max=0.8, cfl_ramp_iters=120,
                          startup_first_order_iters=25, precision=capi.PRECISION_FP64)
    with aero_gb300.Solver(mesh, case) as s:
        _, rec = s.run(1500)
    _, orec = op.OracleSolver(op.MODE_DOUBLE, mesh, case).run(1500)
    assert len(rec) == len(orec) == 1500
    for key in ("cl", "cd", "cm"):
        assert np.max(np.abs(rec[key] - orec[key])) <= 1e-9, key
    assert np.max(np.abs(rec["residual_ratio"] - orec["residual_ratio"]) / orec["residual_ratio"]) <= 1e-8
    assert np.max(orec["residual_ratio"][1000:]) > 0.5  # no convergence in the oracle either


# each diagnostic with the free-stream quantity it is a deviation of (0: a plain maximum)
DIAG_KEYS = {"max_abs_dp_domain": "p", "max_abs_dp_wall": "p", "max_wall_un": "speed", "wall_cp_min": 0,
             "wall_cp_max": 0, "max_farfield_abs_dp": "p", "max_farfield_abs_drho": "rho",
             "max_farfield_abs_du": "speed", "max_farfield_abs_dv": "speed"}


def freestream(mesh, case):
    u = op.OracleSolver(op.MODE_DOUBLE, mesh, case).get_state()[0]
    rho, vx, vy = u[0], u[1] / u[0], u[2] / u[0]
    return {"rho": rho, "speed": np.hypot(vx, vy), "p": (GAMMA - 1.0) * (u[4] - 0.5 * rho * (vx * vx + vy * vy)), 0: 0.0}


@pytest.mark.parametrize("name", ["parity", "regression", "aoa0", "hllc_venkat", "precond", "staged"])
def test_run_diagnostics_vs_oracle(name, golden_meshes, golden_histories):
    """The per-iteration diagnostics of euler_diagnostics.csv (euler_solver.cpp:923-1026)
    against the FP64 oracle on the reference's test cases. Each is a maximum over cells of a
    state quantity, compared within 1e-9 of the largest value it takes over the run; those
    that are deviations from the free stream (|p - p_inf| and the like) lose the digits of
    the free-stream value to cancellation, so they also get 1e-12 of that value."""
    _, meta = golden_histories
    m = meta[name]
    kw = dict(m["case"])
    if kw.get("precond_on") and not m["precond_env"]:
        kw["precond_on"] = 0
    mesh = golden_mesh(golden_meshes, m["mesh"])
    case = capi.make_case(**kw, precision=capi.PRECISION_FP64, diagnostics=1)
    with aero_gb300.Solver(mesh, case) as s:
        _, rec = s.run(case.iterations)
    _, orec = op.OracleSolver(op.MODE_DOUBLE, mesh, case).run(case.iterations)
    assert len(rec) == len(orec)
    base = freestream(mesh, case)
    for key, of in DIAG_KEYS.items():
        ref = orec[key]
        tol = 1e-9 * np.max(np.abs(ref)) + 1e-12 * base[of] + 1e-300
        assert np.max(np.abs(rec[key] - ref)) < tol, key
    np.testing.assert_array_equal(rec["wall_cp_nonfinite"], orec["wall_cp_nonfinite"])
    np.testing.assert_allclose(rec["p_jump_energy_nd"], orec["p_jump_energy_nd"], rtol=1e-8, atol=1e-30)
    np.testing.assert_allclose(rec["p_jump_energy_wall_nd"], orec["p_jump_energy_wall_nd"], rtol=1e-8, atol=1e-30)
    np.testing.assert_array_equal(rec["max_wall_mass_flux"], orec["max_wall_mass_flux"])


@pytest.mark.parametrize("precision", [capi.PRECISION_FP64, capi.PRECISION_FP32])
def test_reference_wall_mass_flux_assertions_on_device(precision, golden_meshes, golden_histories):
    """test_euler_aoa0_regression.cpp:88 (wall mass flux <= 1e-8 after the AoA-0 run) and
    test_euler_wall_sanity.cpp:37 (<= 1e-4 after one HLLC/venkat preconditioned iteration),
    with the device's records; the wall's normal velocity and Cp range match the oracle."""
    _, meta = golden_histories
    for name, limit in (("aoa0", 1e-8), ("wall_sanity", 1e-4)):
        m = meta[name]
        kw = dict(m["case"])
        if kw.get("precond_on") and not m["precond_env"]:
            kw["precond_on"] = 0
        mesh = golden_mesh(golden_meshes, m["mesh"])
        case = capi.make_case(**kw, precision=precision)
        with aero_gb300.Solver(mesh, case) as s:
            _, rec = s.run(case.iterations)
        assert len(rec) == case.iterations
        assert np.all(np.isfinite(rec["max_wall_mass_flux"])) and rec["max_wall_mass_flux"][-1] <= limit, name
        mode = op.MODE_DOUBLE if precision == capi.PRECISION_FP64 else op.MODE_MIXED
        _, orec = op.OracleSolver(mode, mesh, case).run(case.iterations)
        tol = 1e-9 if precision == capi.PRECISION_FP64 else 1e-4
        for key in ("max_wall_un", "wall_cp_min", "wall_cp_max"):
            scale = np.max(np.abs(orec[key])) + 1e-12
            assert np.max(np.abs(rec[key] - orec[key])) / scale < tol, (name, key)
