"""Pin the CPU oracle to the reference: every golden vector in tests/golden/ (produced by
the reference AeroCFD library itself, see tests/golden/make_golden.py) must be reproduced
bit for bit by the oracle's float mode, and to float accuracy by its double mode."""

import numpy as np
import pytest

from aero_gb300 import capi
from conftest import golden_mesh
from oracle import oracle_py as op


@pytest.fixture(scope="module", autouse=True)
def _build():
    op.build()


def _residual_cases(golden_residuals):
    data, meta = golden_residuals
    return [(m, data) for m in meta]


def test_residuals_float_bitwise(golden_meshes, golden_residuals):
    data, meta = golden_residuals
    mesh = golden_mesh(golden_meshes, "ogrid_32x4")
    assert len(meta) == 32
    for m in meta:
        case = capi.make_case(**m["case"])
        sol = op.OracleSolver(op.MODE_FLOAT, mesh, case)
        u = data[m["key"] + "/u"].astype(np.float64)
        r, s, g, diag = sol.residual(u, m["second_order"], m["stab"], m["as_fix"], m["as_fmin"], m["as_ramp"])
        np.testing.assert_array_equal(r.astype(np.float32), data[m["key"] + "/r"], err_msg=m["key"])
        np.testing.assert_array_equal(s.astype(np.float32), data[m["key"] + "/sr"], err_msg=m["key"])
        if m["second_order"]:
            np.testing.assert_array_equal(g.astype(np.float32), data[m["key"] + "/g"], err_msg=m["key"])
        assert tuple(diag) == tuple(data[m["key"] + "/diag"]), m["key"]


def test_residuals_double_close(golden_meshes, golden_residuals):
    """FP64 oracle vs the float reference: differences are float round-off, measured
    against the per-cell flux magnitude scale (|R| itself cancels)."""
    data, meta = golden_residuals
    mesh = golden_mesh(golden_meshes, "ogrid_32x4")
    for m in meta:
        if "_s1_" in m["key"]:
            continue  # near-vacuum stress states amplify float round-off without bound
        case = capi.make_case(**m["case"])
        sol = op.OracleSolver(op.MODE_DOUBLE, mesh, case)
        u = data[m["key"] + "/u"].astype(np.float64)
        r, s, _, _ = sol.residual(u, m["second_order"], m["stab"], m["as_fix"], m["as_fmin"], m["as_ramp"])
        ref_r = data[m["key"] + "/r"].astype(np.float64)
        scale = np.abs(s)[:, None] * np.abs(u).max(axis=1, keepdims=True) + 1e-30
        assert np.max(np.abs(r - ref_r) / scale) < 2e-4, m["key"]
        np.testing.assert_allclose(s, data[m["key"] + "/sr"], rtol=2e-5)


@pytest.mark.parametrize("name", ["parity", "regression", "aoa0", "wall_sanity", "hllc_venkat",
                                  "precond", "staged", "global_dt_rk1", "low_mach_off", "low_mach_on"])
def test_history_float_bitwise(name, golden_meshes, golden_histories):
    data, meta = golden_histories
    m = meta[name]
    mesh = golden_mesh(golden_meshes, m["mesh"])
    case_kw = dict(m["case"])
    if case_kw.get("precond_on") and not m["precond_env"]:
        case_kw["precond_on"] = 0  # forced off by the reference without the experimental flag
    case = capi.make_case(**case_kw)
    sol = op.OracleSolver(op.MODE_FLOAT, mesh, case)
    status, recs = sol.run(case.iterations)
    hist = data[name + "/history"]
    mine = np.stack([recs["iter"], recs["residual_l1"], recs["residual_l2"], recs["residual_linf"],
                     recs["cl"], recs["cd"], recs["cm"]], axis=1)
    assert mine.shape == hist.shape
    np.testing.assert_array_equal(mine, hist)
    np.testing.assert_array_equal(sol.get_state().astype(np.float32), data[name + "/conserved"])
    r, s = sol.last_residual()
    np.testing.assert_array_equal(r.astype(np.float32), data[name + "/last_residual"])
    np.testing.assert_array_equal(s.astype(np.float32), data[name + "/last_sr"])


def test_reference_test_thresholds_hold_on_golden(golden_histories):
    """The golden runs satisfy the reference's own C++ test assertions
    (test_euler_regression.cpp:40-61, test_euler_aoa0_regression.cpp:78-88,
    test_euler_wall_sanity.cpp:37, test_euler_low_mach_asymptotic.cpp:315-316)."""
    data, meta = golden_histories
    reg = data["regression/history"]
    assert reg[-1, 2] <= reg[0, 2] * 1.2
    assert 0.16 <= reg[-1, 4] <= 0.30 and abs(reg[-1, 5]) <= 0.25
    a0 = data["aoa0/history"]
    assert abs(a0[-1, 4]) < 0.05 and abs(a0[-1, 5]) < 0.06
    assert meta["aoa0"]["max_wall_mass_flux"] <= 1e-8
    assert meta["wall_sanity"]["max_wall_mass_flux"] <= 1e-4
    off = data["low_mach_off/history"][-1, 5] * np.float32(0.01)
    on = data["low_mach_on/history"][-1, 5] * np.float32(0.01)
    assert abs(on) < 0.95 * abs(off)


def test_mixed_mode_tracks_double(golden_meshes):
    """FP32-bulk/FP64-accumulate oracle stays close to the FP64 oracle over a short run."""
    mesh = golden_mesh(golden_meshes, "ogrid_48x10")
    case = capi.make_case(iterations=40, min_iterations=40, flux=capi.FLUX_HLLC,
                          limiter=capi.LIMITER_VENKAT, startup_first_order_iters=5, mach=0.5,
                          aoa_deg=1.25, precond_farfield_bc=1)
    a = op.OracleSolver(op.MODE_MIXED, mesh, case)
    b = op.OracleSolver(op.MODE_DOUBLE, mesh, case)
    _, ra = a.run(40)
    _, rb = b.run(40)
    assert np.max(np.abs(ra["cl"] - rb["cl"])) < 1e-4
    ua, ub = a.get_state(), b.get_state()
    mom = np.abs(ub[:, 1:3]).max()
    scale = np.array([np.abs(ub[:, 0]).max(), mom, mom, 1.0, np.abs(ub[:, 4]).max()])
    assert np.max(np.abs(ua - ub) / scale) < 1e-5
