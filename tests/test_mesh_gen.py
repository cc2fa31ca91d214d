"""Mesh generators of libaero_gb300.so.

The reference O-grid restatement must reproduce make_airfoil_ogrid_mesh
(src/cfd_core/mesh/airfoil_mesh.cpp:459-544) bit for bit: the golden meshes in
tests/golden/meshes.npz were exported from the reference library itself. The synthetic
benchmark O-grid is checked through its geometric properties."""

import numpy as np
import pytest

import aero_gb300
from aero_gb300 import capi

OGRIDS = {
    "ogrid_32x4": (32, 4, 10.0, 1.25),
    "ogrid_40x8": (40, 8, 10.0, 1.25),
    "ogrid_48x10": (48, 10, 10.0, 1.25),
    "ogrid_64x14": (64, 14, 12.0, 1.35),
    "ogrid_72x18": (72, 18, 12.0, 1.35),
}


@pytest.fixture(scope="module", autouse=True)
def _lib():
    aero_gb300.load(build_if_missing=True)


@pytest.mark.parametrize("name", list(OGRIDS))
def test_reference_ogrid_bitwise(name, golden_meshes):
    nc, nr, radius, stretch = OGRIDS[name]
    m = aero_gb300.ogrid_reference("0012", nc, nr, radius, stretch, 1.0)
    g = lambda k: golden_meshes[f"{name}/{k}"]  # noqa: E731
    np.testing.assert_array_equal(m.owner, g("owner"))
    np.testing.assert_array_equal(m.neighbor, g("neighbor"))
    np.testing.assert_array_equal(m.bc, g("bc"))
    np.testing.assert_array_equal(m.face_vertices, g("face_vertices"))
    np.testing.assert_array_equal(m.wall_faces, g("wall_faces"))
    for key, mine in (("normal", m.normal), ("center", m.center), ("area", m.area),
                      ("volume", m.volume), ("cell_center", m.cell_center), ("points", m.points)):
        np.testing.assert_array_equal(mine.astype(np.float32), g(key), err_msg=key)
        np.testing.assert_array_equal(mine, g(key).astype(np.float64), err_msg=key)
    np.testing.assert_array_equal(m.cell_conn, g("cell_conn"))


def test_reference_ogrid_rejects_bad_sizes():
    with pytest.raises(aero_gb300.AeroError):
        aero_gb300.ogrid_reference(n_circ=16, n_radial=8)
    with pytest.raises(aero_gb300.AeroError):
        aero_gb300.ogrid_reference(n_circ=32, n_radial=2)


def _closure(m: capi.Mesh) -> np.ndarray:
    """Per-cell sum of outward n*A (geometric conservation)."""
    n = m.normal.reshape(-1, 3)[:, :2] * m.area[:, None]
    s = np.zeros((m.num_cells, 2))
    np.add.at(s, m.owner, n)
    inner = m.neighbor >= 0
    np.add.at(s, m.neighbor[inner], -n[inner])
    return s


@pytest.mark.parametrize("cell_type", [3, 4])
def test_synthetic_ogrid_properties(cell_type):
    nt, nr = 64, 16
    m = aero_gb300.ogrid_synthetic(nt, nr, cell_type=cell_type, permute=True, jitter=0.1, seed=7)
    if cell_type == 3:
        assert m.num_cells == 2 * nt * nr and m.num_faces == nt * (3 * nr + 1)
    else:
        assert m.num_cells == nt * nr and m.num_faces == nt * (2 * nr + 1)
    assert len(m.wall_faces) == nt
    assert np.all(m.volume > 0)
    assert np.allclose(np.linalg.norm(m.normal.reshape(-1, 3), axis=1), 1.0, atol=1e-14)
    # contiguous patches: interior, then wall, then far field
    nint = int(np.sum(m.neighbor >= 0))
    assert np.all(m.neighbor[:nint] >= 0) and np.all(m.neighbor[nint:] < 0)
    assert np.array_equal(m.wall_faces, np.arange(nint, nint + nt))
    assert np.all(m.bc[m.wall_faces] == capi.BC_WALL)
    assert np.all(m.bc[nint + nt:] == capi.BC_FARFIELD)
    # geometric closure to round-off in double
    scale = np.sqrt(m.volume)
    assert np.max(np.abs(_closure(m)) / scale[:, None]) < 1e-12
    # outward normals: owner centre lies behind its faces
    fc = m.center.reshape(-1, 3)[:, :2]
    oc = m.cell_center.reshape(-1, 3)[m.owner, :2]
    assert np.all(np.sum((fc - oc) * m.normal.reshape(-1, 3)[:, :2], axis=1) > 0)
    # first wall spacing: wall-adjacent cells are thin
    wall_cells = m.owner[m.wall_faces]
    thickness = 2.0 * m.volume[wall_cells] / m.area[m.wall_faces] / (2 if cell_type == 3 else 1)
    assert 0.001 < np.median(thickness) < 0.01


def test_synthetic_ogrid_deterministic_and_seeded():
    a = aero_gb300.ogrid_synthetic(48, 12, seed=3)
    b = aero_gb300.ogrid_synthetic(48, 12, seed=3)
    c = aero_gb300.ogrid_synthetic(48, 12, seed=4)
    np.testing.assert_array_equal(a.owner, b.owner)
    np.testing.assert_array_equal(a.points, b.points)
    assert not np.array_equal(a.points, c.points)
    # the far field is a circle of radius 20 chords around mid-chord
    p = a.points.reshape(-1, 3)[-48:]
    assert np.allclose(np.hypot(p[:, 0] - 0.5, p[:, 1]), 20.0, atol=1e-9)


@pytest.mark.parametrize("spec", [(512, 128, 3, True, 0.1, 2), (128, 32, 4, False, 0.0, 1), (64, 16, 3, True, 0.1, 100),
                                  (96, 24, 4, True, 0.1, 11)])
def test_oracle_generator_builds_the_same_mesh(spec):
    """The oracle's own synthetic O-grid generator (used by the reference arm of the benchmark,
    which must not load the product) builds the product generator's mesh bit for bit."""
    from oracle import oracle_py as op

    nc, nr, ct, perm, jit, seed = spec
    kw = dict(cell_type=ct, permute=perm, jitter=jit, seed=seed, wall_spacing=0.005, farfield_radius=20.0)
    a = aero_gb300.ogrid_synthetic(nc, nr, **kw)
    b = op.ogrid_synthetic(nc, nr, **kw)
    for key in ("owner", "neighbor", "bc", "normal", "center", "area", "volume", "cell_center", "wall_faces"):
        np.testing.assert_array_equal(getattr(a, key), getattr(b, key), err_msg=key)
