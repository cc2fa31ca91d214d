"""Batched sweep (include/aero_batch.h): cases of uneven mesh size and different flow
conditions advanced together must reproduce single-case runs bit for bit, stop independently
and refuse mixed kernel variants. Replaces the reference's serial sweep loop
(python/cfd/sweep.py:41-56)."""

import numpy as np
import pytest

import aero_gb300
from aero_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device():
    lib = aero_gb300.load(build_if_missing=True)
    assert lib.aero_cuda_available(), "GPU tests need an sm_103 device"


SIZES = [(64, 16), (48, 12), (96, 24)]
FLOWS = [dict(mach=0.5, aoa_deg=2.0), dict(mach=0.7, aoa_deg=-1.0), dict(mach=0.3, aoa_deg=4.0)]


def _cases(precision, **extra):
    meshes = [aero_gb300.ogrid_synthetic(nc, nr, cell_type=3, permute=True, jitter=0.1, seed=31 + i)
              for i, (nc, nr) in enumerate(SIZES)]
    cases = [capi.make_case(**f, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT, startup_first_order_iters=4,
                            cfl_max=0.8, precision=precision, **extra) for f in FLOWS]
    return meshes, cases


@pytest.mark.parametrize("precision", [capi.PRECISION_FP32, capi.PRECISION_FP64])
def test_batch_reproduces_single_runs(precision):
    meshes, cases = _cases(precision)
    n = 30
    with aero_gb300.Batch(meshes, cases) as b:
        assert b.info()["cases"] == 3
        _, recs = b.run(n)
        states = [b.get_state(k) for k in range(3)]
        last = [b.last_residual(k) for k in range(3)]
    for k in range(3):
        with aero_gb300.Solver(meshes[k], cases[k]) as s:
            _, rec = s.run(n)
            np.testing.assert_array_equal(states[k], s.get_state())
            r, sr = s.last_residual()
        assert len(recs[k]) == len(rec) == n
        for key in ("residual_l2", "residual_l1", "cl", "cd", "cm", "cfl", "flags", "max_abs_dp_domain",
                    "first_order_fallback_faces", "residual_rho_ratio"):
            np.testing.assert_array_equal(recs[k][key], rec[key], err_msg=f"case {k} {key}")
        np.testing.assert_array_equal(last[k][0], r)
        np.testing.assert_array_equal(last[k][1], sr)


def test_batch_cases_stop_independently():
    """A density-residual target stops each case at its own iteration; the others run on."""
    meshes, cases = _cases(capi.PRECISION_FP32)
    cases[1].density_l2_target = 0.5
    cases[1].min_iterations = 5
    with aero_gb300.Batch(meshes, cases) as b:
        _, recs = b.run(60)
        ran = [len(r) for r in recs]
    assert ran[0] == ran[2] == 60
    assert 5 <= ran[1] < 60
    assert recs[1]["flags"][-1] & capi.REC_CONVERGED
    assert recs[1]["residual_rho_ratio"][-1] <= 0.5 < recs[1]["residual_rho_ratio"][-2]
    with aero_gb300.Solver(meshes[1], cases[1]) as s:
        _, rec = s.run(60)
    assert len(rec) == ran[1]
    np.testing.assert_array_equal(rec["cl"], recs[1]["cl"])


def test_batch_refuses_mixed_kernel_variants():
    meshes, cases = _cases(capi.PRECISION_FP32)
    cases[2].flux = capi.FLUX_RUSANOV
    with pytest.raises(aero_gb300.AeroError) as e:
        aero_gb300.Batch(meshes, cases)
    assert e.value.code == capi.AERO_ERR_INVALID


def test_batch_context_refuses_single_case_calls():
    meshes, cases = _cases(capi.PRECISION_FP32)
    with aero_gb300.Batch(meshes, cases) as b:
        recs = (capi.IterRecord * 1)()
        done = aero_gb300.C.c_int(0)
        assert b.lib.aero_run(b.h, 1, recs, aero_gb300.C.byref(done)) == capi.AERO_ERR_INVALID


def test_autotune_picks_the_fastest_measured_variant():
    mesh = aero_gb300.ogrid_synthetic(96, 24, cell_type=3, permute=True, jitter=0.1, seed=7)
    case = capi.make_case(mach=0.6, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT, startup_first_order_iters=3,
                          precision=capi.PRECISION_FP32)
    best, table = aero_gb300.autotune(mesh, case, iters=10)
    assert len(table) == 12 and all(v > 0 for v in table.values())
    assert (best.ordering, best.block_size, best.cells_per_thread) == min(table, key=table.get)
    assert best.mach == case.mach and best.flux == case.flux
    with aero_gb300.Solver(mesh, best) as s:  # the tuned case runs and matches the default's results
        _, rec = s.run(8)
    with aero_gb300.Solver(mesh, case) as s:
        _, rec0 = s.run(8)
    np.testing.assert_allclose(rec["cl"], rec0["cl"], rtol=1e-5, atol=1e-7)
