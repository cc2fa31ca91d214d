"""Host-side shape machinery of the adjoint (include/aero_mesh.h): geometry recomputation from
node coordinates, its tangent, and the Hicks-Henne / inverse-distance-weighting modes. No
reference counterpart (AeroCFD has no shape parameterisation); checked against the
synthetic generator's own geometry and central differences."""

import numpy as np
import pytest

import aero_gb300


@pytest.fixture(scope="module")
def mesh():
    aero_gb300.load(build_if_missing=True)
    return aero_gb300.ogrid_synthetic(48, 12, cell_type=3, permute=True, jitter=0.1, seed=5)


@pytest.fixture(scope="module")
def quad_mesh():
    aero_gb300.load(build_if_missing=True)
    return aero_gb300.ogrid_synthetic(32, 8, cell_type=4, permute=True, jitter=0.1, seed=6)


@pytest.mark.parametrize("name", ["mesh", "quad_mesh"])
def test_set_points_reproduces_generator_geometry(name, request):
    m = request.getfixturevalue(name)
    d = aero_gb300.deform(m, m.points.reshape(-1, 3))
    for k in ("normal", "center", "area", "volume", "cell_center"):
        np.testing.assert_array_equal(getattr(d, k), getattr(m, k), err_msg=k)


@pytest.mark.parametrize("name", ["mesh", "quad_mesh"])
def test_geometry_tangent_matches_central_differences(name, request):
    m = request.getfixturevalue(name)
    rng = np.random.default_rng(1)
    pts = m.points.reshape(-1, 3)
    dp = np.zeros_like(pts)
    dp[:, :2] = rng.standard_normal((pts.shape[0], 2)) * 1e-3
    t = aero_gb300.geometry_tangent(m, dp)
    h = 1e-4
    a = aero_gb300.deform(m, pts + h * dp)
    b = aero_gb300.deform(m, pts - h * dp)
    for k in ("normal", "center", "area", "volume", "cell_center"):
        fd = (getattr(a, k) - getattr(b, k)) / (2 * h)
        scale = np.abs(fd).max()
        assert np.abs(getattr(t, k) - fd).max() <= 1e-6 * scale + 1e-15, k


def test_hicks_henne_modes(mesh):
    peaks = np.array([0.1, 0.3, 0.5, 0.8])
    upper = np.array([1, 1, 0, 0])
    modes = aero_gb300.hicks_henne_modes(mesh, peaks, upper, width=3.0)
    pts = mesh.points.reshape(-1, 3)
    assert modes.shape == (4, pts.shape[0], 3)
    assert not modes[:, :, 0].any() and not modes[:, :, 2].any()  # y displacements only
    fv = mesh.face_vertices.reshape(-1, 2)
    wall = np.unique(fv[mesh.wall_faces].ravel())
    far = np.unique(fv[mesh.bc == aero_gb300.capi.BC_FARFIELD].ravel())
    x0, x1 = pts[wall, 0].min(), pts[wall, 0].max()
    xi = (pts[wall, 0] - x0) / (x1 - x0)
    for k, (pk, up) in enumerate(zip(peaks, upper)):
        on = pts[wall, 1] > 0 if up else pts[wall, 1] < 0
        e = np.log(0.5) / np.log(pk)
        with np.errstate(invalid="ignore"):
            want = np.where(on & (xi > 0) & (xi < 1), np.sin(np.pi * np.clip(xi, 0, 1) ** e) ** 3, 0.0)
        np.testing.assert_allclose(modes[k, wall, 1], want, rtol=1e-12, atol=1e-15)
        assert np.abs(modes[k, far, 1]).max() == 0.0
        # the peak of the bump is 1 at xi = peak; interior nodes stay within the wall's range
        assert np.abs(modes[k, :, 1]).max() <= np.abs(modes[k, wall, 1]).max() + 1e-15
    # a deformed mesh stays valid for amplitudes of 1e-3 chord
    a = np.array([1e-3, -1e-3, 5e-4, -5e-4])
    d = aero_gb300.deform(mesh, pts + np.tensordot(a, modes, axes=1))
    assert (d.volume > 0).all()


def test_set_points_refuses_inverted_cells(mesh):
    pts = mesh.points.reshape(-1, 3).copy()
    pts[:, 0] *= -1.0  # mirror: every cell turns clockwise
    with pytest.raises(aero_gb300.AeroError):
        aero_gb300.deform(mesh, pts)


@pytest.mark.parametrize("name", ["mesh", "quad_mesh"])
def test_geometry_vjp_is_the_transpose_of_the_tangent(name, request):
    """Dot-product test of the reverse geometry pass: for random node displacements dX and
    random geometry derivatives b, sum(b * tangent(dX)) = sum(vjp(b) * dX)."""
    m = request.getfixturevalue(name)
    rng = np.random.default_rng(7)
    pts = m.points.reshape(-1, 3)
    nf, nc = m.num_faces, m.num_cells
    for trial in range(3):
        dp = np.zeros_like(pts)
        dp[:, :2] = rng.standard_normal((pts.shape[0], 2))
        t = aero_gb300.geometry_tangent(m, dp)
        b = {k: rng.standard_normal(n) for k, n in (("normal", 3 * nf), ("center", 3 * nf), ("area", nf),
                                                     ("volume", nc), ("cell_center", 3 * nc))}
        for k in ("normal", "center"):
            b[k].reshape(-1, 3)[:, 2] = 0.0
        b["cell_center"].reshape(-1, 3)[:, 2] = 0.0
        bars = aero_gb300.capi.Mesh(m.owner, m.neighbor, m.bc, b["normal"], b["center"], b["area"], b["volume"],
                                    b["cell_center"], m.wall_faces)
        bp = aero_gb300.geometry_vjp(m, bars)
        lhs = sum(float(np.dot(b[k], getattr(t, k))) for k in b)
        rhs = float(np.sum(bp * dp))
        assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + abs(rhs)), (trial, lhs, rhs)
        assert not bp[:, 2].any()
