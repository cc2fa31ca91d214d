"""The allocation-free residual entry point, aero_residual_noalloc.

It exists for callers that cannot allocate device memory while they evaluate the
residual: code running under another framework's memory pool, or solver loops whose device
memory is fixed up front. Such a caller owns the input and output buffers; the library
supplies its working arrays from one fixed device array. This test allocates the buffers with
PyTorch (standing in for such a caller), calls the entry point through the C ABI, and checks
it against the existing aero_residual entry point on two calls in a row (different states),
plus a repeat of the first state, with the tolerance of the other parity tests: |dR| <= 1e-12
(FP64) or 2e-5 (FP32) times the per-cell sum over faces of |F_k A|; every result is also
checked against the FP64 oracle, at 1e-12 (FP64) or 5e-5 (FP32) of the same scale. The device's free memory is the same just before
and just after every call once the first has loaded the kernels. It also checks that meshes
above the array's limit are refused. It runs on its own in a fresh process as well as after the other tests.
"""

import ctypes as C

import numpy as np
import pytest

import aero_gb300
from aero_gb300 import capi
from oracle import oracle_py as op

pytestmark = pytest.mark.gpu

_dp = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def lib():
    lib = aero_gb300.load(build_if_missing=True)
    assert lib.aero_cuda_available(), "GPU test needs an sm_103 device"
    lib.aero_residual_noalloc.restype = C.c_int
    lib.aero_residual_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_double,
                                          C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    op.build()
    return lib


def _states(mesh, case, seeds):
    base = op.OracleSolver(op.MODE_DOUBLE, mesh, case).get_state()
    out = []
    for seed in seeds:
        rng = np.random.default_rng(seed)
        u = base.copy()
        x = mesh.cell_center.reshape(-1, 3)
        for k in (0, 1, 2, 4):
            u[:, k] *= 1.0 + 0.05 * np.sin(1.1 * x[:, 0] + seed) + 0.03 * rng.standard_normal(len(u))
        u[:, 3] = 0.0
        out.append(u)
    return out


def _noalloc(lib, solver, u, args):
    """One call on caller-owned device buffers; returns the residual, the spectral radius and
    the device's free memory just before and just after the call."""
    torch = pytest.importorskip("torch")
    n = solver.n
    u_dev = torch.from_numpy(np.ascontiguousarray(u)).to("cuda")
    r_dev = torch.full((n, 5), float("nan"), dtype=torch.float64, device="cuda")
    s_dev = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()  # inputs written before the library's stream reads them
    free_before = torch.cuda.mem_get_info()[0]
    rc = lib.aero_residual_noalloc(solver.h, u_dev.data_ptr(), *args, r_dev.data_ptr(), s_dev.data_ptr(), None)
    assert rc == 0, lib.aero_last_error(solver.h).decode()
    torch.cuda.synchronize()  # device-wide: also waits for the library's own stream
    free_after = torch.cuda.mem_get_info()[0]
    return r_dev.cpu().numpy(), s_dev.cpu().numpy(), (free_before, free_after)


@pytest.mark.parametrize("precision,tol", [(capi.PRECISION_FP64, 1e-12), (capi.PRECISION_FP32, 2e-5)])
@pytest.mark.parametrize("numerics", [
    dict(flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT, precond_farfield_bc=1),
    dict(flux=capi.FLUX_RUSANOV, limiter=capi.LIMITER_MINMOD, precond_on=1, low_mach_fix=1, all_speed_flux_fix=1),
])
def test_noalloc_matches_existing_entry_point(lib, precision, tol, numerics):
    mesh = aero_gb300.ogrid_synthetic(64, 16, cell_type=3, permute=True, jitter=0.1, seed=21)
    case = capi.make_case(mach=0.4, aoa_deg=2.0, precision=precision, **numerics)
    u1, u2 = _states(mesh, case, (1, 2))
    args = (1, 0.02, int(numerics.get("all_speed_flux_fix", 0)), 0.05, 0.7)
    oracle = op.OracleSolver(op.MODE_DOUBLE, mesh, case)
    with aero_gb300.Solver(mesh, case) as solver:
        results = []
        for call, u in enumerate((u1, u2, u1)):  # two calls in a row on different states, then the first again
            r, s, (free_before, free_after) = _noalloc(lib, solver, u, args)
            if call > 0:  # after the first call has loaded the kernels, no call takes device memory
                assert free_after == free_before, (call, free_before - free_after)
            r_ref, s_ref, _ = solver.residual(u, *args)
            r_or, _, _, _, fscale = oracle.residual(u, *args, with_scale=True)
            assert np.all(np.isfinite(r)) and np.all(np.isfinite(s))
            assert np.max(np.abs(r - r_ref) / (fscale + 1e-300)) <= tol
            # against the FP64 oracle: 1e-12 in FP64, float-class (the bound of the FP32 parity
            # tests, which the reference's own float residual meets) in FP32
            assert np.max(np.abs(r - r_or) / (fscale + 1e-300)) <= (1e-12 if precision == capi.PRECISION_FP64 else 5e-5)
            np.testing.assert_allclose(s, s_ref, rtol=tol)
            results.append(r)
        # the shared array keeps the previous call's contents; results must not depend on it
        np.testing.assert_array_equal(results[0], results[2])


def test_noalloc_refuses_meshes_above_its_limit(lib):
    mesh = aero_gb300.ogrid_synthetic(512, 128, cell_type=3, permute=False, jitter=0.0, seed=0)
    assert mesh.num_cells > 65536
    case = capi.make_case(mach=0.5, precision=capi.PRECISION_FP32)
    with aero_gb300.Solver(mesh, case) as solver:
        dummy = C.c_double(0.0)
        rc = lib.aero_residual_noalloc(solver.h, C.addressof(dummy), 1, 0.0, 0, 0.05, 1.0, C.addressof(dummy),
                                       C.addressof(dummy), None)
        assert rc == capi.AERO_ERR_INVALID
        assert "65536" in lib.aero_last_error(solver.h).decode()
