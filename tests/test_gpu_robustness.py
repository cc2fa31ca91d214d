"""Bounded device waits and shared-memory limits of the iteration kernels.

* The gradient pass that streams cell tiles through shared memory with bulk copies waits on
  each tile's copies with a bounded poll loop. With the poll limit set to 0 every such wait
  runs out at once (no fault, no hang: the kernel then waits, bounded, for the copies it has
  in flight and returns). The run must report AERO_ERR_TIMEOUT, leave the conserved state of
  the failed iteration untouched and write no record for it; after the limit is restored the
  same context continues, and its records and state agree with a run that never timed out.
* Meshes with many faces per cell: the bulk-copy pass's two tile buffers (per slot a link
  and a face vector) outgrow a CTA's shared memory at FP64 and block size 256 for cells of
  24 faces. Such a context must still
  be created (the plain gather gradient runs) and match the FP64 oracle; forcing the
  bulk-copy pass there is refused with a clear error.
"""

import numpy as np
import pytest

import aero_gb300
from aero_gb300 import capi
from oracle import oracle_py as op

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device():
    lib = aero_gb300.load(build_if_missing=True)
    assert lib.aero_cuda_available(), "GPU tests need an sm_103 device"
    op.build()


@pytest.mark.parametrize("precision", [capi.PRECISION_FP64, capi.PRECISION_FP32])
def test_expired_copy_wait_discards_the_iteration_and_the_context_continues(precision, monkeypatch):
    monkeypatch.setenv("AERO_BULK_COPY", "1")
    mesh = aero_gb300.ogrid_synthetic(96, 24, cell_type=3, permute=True, jitter=0.1, seed=31)
    case = capi.make_case(mach=0.7, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT, startup_first_order_iters=3,
                          precision=precision)
    with aero_gb300.Solver(mesh, case) as s:
        _, ref = s.run(10)
        ref_state = s.get_state()
    with aero_gb300.Solver(mesh, case) as s:
        assert s.info()["bulk_copy_gradient"] == 1
        _, first = s.run(5)  # iterations 0-4; 3 and 4 are second order and use the bulk copies
        u5 = s.get_state()
        s.set_wait_limit(0)
        rc, rec = s.run(3, raise_on_nonfinite=False)
        assert rc == capi.AERO_ERR_TIMEOUT
        assert len(rec) == 0  # iteration 5 was not applied and nothing after it ran
        np.testing.assert_array_equal(s.get_state(), u5)
        s.set_wait_limit(-1)
        _, rest = s.run(5)  # iterations 5-9 from the last applied state
        assert list(rest["iter"]) == [5, 6, 7, 8, 9]
        state = s.get_state()
    got = np.concatenate([first, rest])
    tol = 1e-12 if precision == capi.PRECISION_FP64 else 1e-5
    for key in ("residual_l2", "cl", "cd"):
        assert np.max(np.abs(got[key] - ref[key]) / (np.abs(ref[key]) + 1e-300)) <= tol, key
    if precision == capi.PRECISION_FP64:
        np.testing.assert_array_equal(got["first_order_fallback_faces"], ref["first_order_fallback_faces"])
    assert np.max(np.abs(state - ref_state) / (np.abs(ref_state).max(axis=0) + 1e-300)) <= tol


def flower_mesh(petals: int = 16):
    """One regular polygon of `petals` faces surrounded by one triangle on each of its edges;
    the triangles' outer edges are far field, four of them wall."""
    th = 2.0 * np.pi * np.arange(petals) / petals
    ring = np.stack([np.cos(th), np.sin(th)], 1)
    apex = 1.6 * np.stack([np.cos(th + np.pi / petals), np.sin(th + np.pi / petals)], 1)
    pts = np.concatenate([ring, apex])
    cells = [list(range(petals))] + [[k, petals + k, (k + 1) % petals] for k in range(petals)]

    def area2(v):
        x, y = pts[v, 0], pts[v, 1]
        return float(np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y))

    cells = [c if area2(c) > 0 else c[::-1] for c in cells]
    faces, index = [], {}
    for ci, v in enumerate(cells):
        for a, b in zip(v, v[1:] + v[:1]):
            key = (min(a, b), max(a, b))
            if key in index:
                faces[index[key]][1] = ci
            else:
                index[key] = len(faces)
                faces.append([ci, -1, a, b])
    nf = len(faces)
    owner = np.array([f[0] for f in faces], np.int32)
    neighbor = np.array([f[1] for f in faces], np.int32)
    bc = np.where(neighbor >= 0, capi.BC_INTERIOR, capi.BC_FARFIELD).astype(np.int32)
    walls = [i for i, f in enumerate(faces) if f[1] < 0 and min(f[2], f[3]) < 4][:4]
    bc[walls] = capi.BC_WALL
    d = np.array([pts[f[3]] - pts[f[2]] for f in faces])
    length = np.hypot(d[:, 0], d[:, 1])
    normal = np.zeros((nf, 3))
    normal[:, 0], normal[:, 1] = d[:, 1] / length, -d[:, 0] / length
    center = np.zeros((nf, 3))
    center[:, :2] = np.array([0.5 * (pts[f[2]] + pts[f[3]]) for f in faces])
    vol = np.array([0.5 * area2(v) for v in cells])
    cc = np.zeros((len(cells), 3))
    for ci, v in enumerate(cells):
        x, y = pts[v, 0], pts[v, 1]
        cr = x * np.roll(y, -1) - np.roll(x, -1) * y
        cc[ci, 0] = np.sum((x + np.roll(x, -1)) * cr) / (6.0 * vol[ci])
        cc[ci, 1] = np.sum((y + np.roll(y, -1)) * cr) / (6.0 * vol[ci])
    return capi.Mesh(owner, neighbor, bc, normal, center, length, vol, cc, np.array(walls, np.int32))


def test_cells_with_many_faces_at_block_256(monkeypatch):
    mesh = flower_mesh(24)
    case64 = capi.make_case(mach=0.5, aoa_deg=2.0, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT,
                            precision=capi.PRECISION_FP64, block_size=256)
    o = op.OracleSolver(op.MODE_DOUBLE, mesh, case64)
    u = o.get_state().copy()
    rng = np.random.default_rng(4)
    for k in (0, 1, 2, 4):
        u[:, k] *= 1.0 + 0.02 * rng.standard_normal(len(u))
    with aero_gb300.Solver(mesh, case64) as s:
        info = s.info()
        assert info["slots_per_cell"] >= 24 and info["bulk_copy_gradient"] == 0
        for second in (0, 1):
            r, sr, _ = s.residual(u, second, 0.0, 0, 0.05, 1.0)
            ro, sro, _, _, fs = o.residual(u, second, 0.0, 0, 0.05, 1.0, with_scale=True)
            assert np.max(np.abs(r - ro) / (fs + 1e-300)) <= 1e-12
            np.testing.assert_allclose(sr, sro, rtol=1e-12)
        _, rec = s.run(5)
        assert len(rec) == 5 and np.all(np.isfinite(rec["residual_l2"]))
    monkeypatch.setenv("AERO_BULK_COPY", "1")
    with pytest.raises(aero_gb300.AeroError, match="shared memory"):
        aero_gb300.Solver(mesh, case64)
    case32 = capi.make_case(mach=0.5, aoa_deg=2.0, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT,
                            precision=capi.PRECISION_FP32, block_size=256)
    with aero_gb300.Solver(mesh, case32) as s:  # two float tile buffers of 24 slots fit
        assert s.info()["bulk_copy_gradient"] == 1
        _, rec = s.run(5)
        assert np.all(np.isfinite(rec["residual_l2"]))
