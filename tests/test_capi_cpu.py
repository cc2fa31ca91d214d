"""C-ABI library checks that need no GPU: it loads, exports every symbol the public
headers declare, its defaults match the reference's, and it refuses to run without a
device instead of falling back to the CPU."""

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import aero_gb300
from aero_gb300 import capi

REPO = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    return aero_gb300.load(build_if_missing=True)


def declared_symbols():
    names = []
    for header in sorted((REPO / "include").glob("*.h")):
        text = header.read_text()
        names += re.findall(r"^AERO_API\s+[\w\s\*]+?\b(aero_\w+)\s*\(", text, flags=re.M)
    return names


def test_headers_declare_symbols():
    names = declared_symbols()
    assert "aero_create" in names and "aero_run" in names and "aero_mesh_ogrid_reference" in names
    assert len(names) == len(set(names))


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_identity(lib):
    assert lib.aero_abi_version() == capi.ABI_VERSION == 4
    assert lib.aero_version().decode().endswith("gb300")


def test_case_defaults_match_reference(lib):
    c = capi.CaseDesc()
    lib.aero_case_defaults(C.byref(c))
    got = capi.case_to_dict(c)
    for key, val in capi.CASE_DEFAULTS.items():
        assert got[key] == val, key


def test_no_cpu_fallback_without_device(lib):
    if lib.aero_cuda_available():
        pytest.skip("a CUDA device is present")
    mesh = aero_gb300.ogrid_reference(n_circ=32, n_radial=4, farfield_radius=10.0, radial_stretch=1.25)
    with pytest.raises(aero_gb300.AeroError) as exc:
        aero_gb300.Solver(mesh, capi.make_case())
    assert exc.value.code == capi.AERO_ERR_CUDA


def test_invalid_arguments_are_rejected(lib):
    mesh = aero_gb300.ogrid_reference(n_circ=32, n_radial=4, farfield_radius=10.0, radial_stretch=1.25)
    with pytest.raises(aero_gb300.AeroError) as exc:
        aero_gb300.Solver(mesh, capi.make_case(rk_stages=2))
    assert exc.value.code == capi.AERO_ERR_INVALID
    with pytest.raises(aero_gb300.AeroError) as exc:
        aero_gb300.Solver(mesh, capi.make_case(rho_inf=-1.0, p_inf=-1.0))
    assert exc.value.code == capi.AERO_ERR_INVALID
    with pytest.raises(aero_gb300.AeroError) as exc:
        aero_gb300.Solver(mesh, capi.make_case(precond_fp64=3))
    assert exc.value.code == capi.AERO_ERR_INVALID


def _corrupted(mesh, what):
    """A copy of `mesh` with one defect."""
    m = capi.Mesh(mesh.owner.copy(), mesh.neighbor.copy(), mesh.bc.copy(), mesh.normal.copy(), mesh.center.copy(),
                  mesh.area.copy(), mesh.volume.copy(), mesh.cell_center.copy(), mesh.wall_faces.copy())
    interior = int(np.flatnonzero(m.neighbor >= 0)[0])
    boundary = int(np.flatnonzero(m.neighbor < 0)[0])
    if what == "owner out of range":
        m.owner[interior] = m.num_cells
    elif what == "neighbour equals owner":
        m.neighbor[interior] = m.owner[interior]
    elif what == "neighbour below -1":
        m.neighbor[boundary] = -2
    elif what == "boundary face without a type":
        m.bc[boundary] = capi.BC_INTERIOR
    elif what == "non-finite normal":
        m.normal[3 * interior] = np.nan
    elif what == "non-finite length":
        m.area[interior] = np.inf
    elif what == "non-finite volume":
        m.volume[0] = np.nan
    elif what == "interior face in the wall list":
        m.wall_faces[0] = interior
    elif what == "wall face out of range":
        m.wall_faces[0] = m.num_faces
    return m


@pytest.mark.parametrize("what, message", [
    ("owner out of range", "invalid owner/neighbour"),
    ("neighbour equals owner", "invalid owner/neighbour"),
    ("neighbour below -1", "invalid owner/neighbour"),
    ("boundary face without a type", "no far-field/wall type"),
    ("non-finite normal", "non-finite geometry"),
    ("non-finite length", "non-finite geometry"),
    ("non-finite volume", "non-finite volume"),
    ("interior face in the wall list", "wall face list"),
    ("wall face out of range", "wall face list"),
])
def test_invalid_meshes_are_refused(lib, what, message):
    """aero_create checks the mesh on the host before it looks for a device: each defect is
    refused with AERO_ERR_INVALID and a message naming it, on any machine."""
    mesh = aero_gb300.ogrid_reference(n_circ=32, n_radial=4, farfield_radius=10.0, radial_stretch=1.25)
    with pytest.raises(aero_gb300.AeroError) as exc:
        aero_gb300.Solver(_corrupted(mesh, what), capi.make_case())
    assert exc.value.code == capi.AERO_ERR_INVALID
    assert message in str(exc.value)


def test_empty_mesh_is_refused(lib):
    mesh = aero_gb300.ogrid_reference(n_circ=32, n_radial=4, farfield_radius=10.0, radial_stretch=1.25)
    empty = capi.Mesh(np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0), np.zeros(0),
                      np.zeros(0), mesh.volume, mesh.cell_center, np.zeros(0, np.int32))
    with pytest.raises(aero_gb300.AeroError) as exc:
        aero_gb300.Solver(empty, capi.make_case())
    assert exc.value.code == capi.AERO_ERR_INVALID and "cells and faces" in str(exc.value)


def test_record_struct_size_matches_header():
    # aero_iter_record: 4 ints + 42 doubles + 2 ints + 1 double
    assert C.sizeof(capi.IterRecord) == 4 * 4 + 42 * 8 + 2 * 4 + 8
    assert np.dtype(capi.RECORD_DTYPE).itemsize == C.sizeof(capi.IterRecord)


@pytest.mark.parametrize("c_name,py_struct", [
    ("aero_case_desc", capi.CaseDesc), ("aero_mesh_desc", capi.MeshDesc), ("aero_iter_record", capi.IterRecord),
    ("aero_ogrid_spec", aero_gb300.OgridSpec), ("aero_mesh_sizes", aero_gb300.MeshSizes)])
def test_struct_layouts_match_the_headers(c_name, py_struct, tmp_path):
    """Every field offset and the size of the ctypes mirrors equal what a C compiler lays out
    from include/*.h, so a field added on one side only fails here instead of shifting the
    fields after it."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f[0] for f in py_struct._fields_]
    src = ["#include <stddef.h>", "#include <stdio.h>", '#include "aero_gb300.h"', '#include "aero_mesh.h"',
           "int main(void) {", f'  printf("size %zu\\n", sizeof({c_name}));']
    src += [f'  printf("{f} %zu\\n", offsetof({c_name}, {f}));' for f in fields]
    src += ["  return 0;", "}"]
    (tmp_path / "layout.c").write_text("\n".join(src) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(REPO / "include"), str(tmp_path / "layout.c"), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    assert int(out["size"]) == C.sizeof(py_struct)
    for f in fields:
        assert int(out[f]) == getattr(py_struct, f).offset, f
