"""TEST INFRASTRUCTURE ONLY: ctypes loaders for the CPU oracle (oracle/_build/liboracle.so)
and, where it was built, the compiled reference (oracle/_ref/libaero_ref.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU arms import this module. It needs
nothing from the product package: structures come from oracle_types (read from the C
header), and the benchmark's synthetic meshes from the oracle's own generator.
"""

from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from . import oracle_types as ot
from .oracle_types import OracleMesh, make_case  # noqa: F401

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libaero_ref.so"

MODE_FLOAT, MODE_DOUBLE, MODE_MIXED = 0, 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_oracle = None
_ref = None


def build(ref_root: str | None = None) -> None:
    """Compile the oracle; with ref_root (the AeroCFD source root) also the reference library."""
    targets = ["all"] + (["ref", f"REF_ROOT={ref_root}"] if ref_root else [])
    subprocess.run(["make", "-s", "-C", str(HERE), *targets], check=True)


def oracle_lib():
    global _oracle
    if _oracle is None:
        if not ORACLE_LIB.exists():
            build()
        lib = C.CDLL(str(ORACLE_LIB))
        lib.oracle_solver_create.restype = C.c_void_p
        lib.oracle_solver_create.argtypes = [C.c_int, C.POINTER(ot.MeshDesc), C.POINTER(ot.CaseDesc)]
        lib.oracle_solver_destroy.argtypes = [C.c_void_p]
        lib.oracle_solver_set_state.argtypes = [C.c_void_p, _dp]
        lib.oracle_solver_get_state.argtypes = [C.c_void_p, _dp]
        lib.oracle_solver_last_residual.argtypes = [C.c_void_p, _dp, _dp]
        lib.oracle_solver_reset_run.argtypes = [C.c_void_p]
        lib.oracle_solver_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(ot.IterRecord), _ip]
        lib.oracle_solver_residual.argtypes = [C.c_void_p, _dp, C.c_int, C.c_double, C.c_int,
                                               C.c_double, C.c_double, _dp, _dp, _dp, _ip, _dp]
        lib.oracle_mesh_ogrid.restype = C.c_void_p
        lib.oracle_mesh_ogrid.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_double, C.c_ulonglong]
        lib.oracle_mesh_sizes.argtypes = [C.c_void_p, _ip]
        lib.oracle_mesh_copy.argtypes = [C.c_void_p, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _ip]
        lib.oracle_mesh_free.argtypes = [C.c_void_p]
        _oracle = lib
    return _oracle


def ref_lib():
    """The compiled reference, or None when it was not built (e.g. on a host without the
    reference sources)."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            return None
        lib = C.CDLL(str(REF_LIB))
        lib.ref_last_error.restype = C.c_char_p
        lib.ref_ogrid_build.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double]
        lib.ref_mesh_sizes.argtypes = [_ip]
        fp = C.POINTER(C.c_float)
        lib.ref_mesh_get.argtypes = [_ip, _ip, _ip, _ip, fp, fp, fp, fp, fp, fp, _ip, _ip]
        lib.ref_residual.argtypes = [C.POINTER(ot.MeshDesc), C.POINTER(ot.CaseDesc), _dp, C.c_int,
                                     C.c_double, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, _ip]
        lib.ref_run_case.argtypes = [C.POINTER(ot.CaseDesc), C.c_char_p, C.c_int, C.c_int, C.c_double,
                                     C.c_double, C.c_char_p, _dp, C.c_int, _ip, _dp, _dp, _dp, _dp]
        _ref = lib
    return _ref


class OracleSolver:
    """One oracle solver instance on an injected mesh."""

    def __init__(self, mode: int, mesh, case):
        self.lib = oracle_lib()
        self.mesh = OracleMesh.of(mesh)
        self._mdesc = self.mesh.desc()
        self._case = ot.case_desc(case)
        self.h = self.lib.oracle_solver_create(mode, C.byref(self._mdesc), C.byref(self._case))
        if not self.h:
            raise RuntimeError("oracle_solver_create failed")
        self.n = self.mesh.num_cells

    def close(self):
        if self.h:
            self.lib.oracle_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_state(self, u: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        self.lib.oracle_solver_set_state(self.h, u.ctypes.data_as(_dp))

    def get_state(self) -> np.ndarray:
        u = np.empty(self.n * 5, np.float64)
        self.lib.oracle_solver_get_state(self.h, u.ctypes.data_as(_dp))
        return u.reshape(self.n, 5)

    def last_residual(self):
        r = np.empty(self.n * 5, np.float64)
        s = np.empty(self.n, np.float64)
        self.lib.oracle_solver_last_residual(self.h, r.ctypes.data_as(_dp), s.ctypes.data_as(_dp))
        return r.reshape(self.n, 5), s

    def reset_run(self):
        self.lib.oracle_solver_reset_run(self.h)

    def run(self, n: int):
        recs = (ot.IterRecord * max(n, 1))()
        done = C.c_int(0)
        status = self.lib.oracle_solver_run(self.h, n, recs, C.byref(done))
        return status, ot.records_to_array(recs, done.value)

    def residual(self, u, second_order=True, stab=0.0, as_fix=False, as_fmin=0.05, as_ramp=1.0,
                 with_scale=False):
        """Residual [N,5], spectral radius [N], gradients [N,5,2], fallback counters; with
        with_scale also the per-cell, per-component sum over faces of |F_k A| [N,5]."""
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        r = np.empty(self.n * 5, np.float64)
        s = np.empty(self.n, np.float64)
        g = np.empty(self.n * 10, np.float64)
        fs = np.empty(self.n * 5, np.float64)
        diag = (C.c_int * 3)()
        self.lib.oracle_solver_residual(self.h, u.ctypes.data_as(_dp), int(second_order), float(stab),
                                        int(as_fix), float(as_fmin), float(as_ramp),
                                        r.ctypes.data_as(_dp), s.ctypes.data_as(_dp),
                                        g.ctypes.data_as(_dp), diag, fs.ctypes.data_as(_dp))
        out = (r.reshape(self.n, 5), s, g.reshape(self.n, 5, 2), tuple(diag))
        return out + (fs.reshape(self.n, 5),) if with_scale else out


def ref_residual(mesh, case, u, second_order=True, stab=0.0, as_fix=False, as_fmin=0.05, as_ramp=1.0):
    lib = ref_lib()
    n = mesh.num_cells
    u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
    r = np.empty(n * 5, np.float64)
    s = np.empty(n, np.float64)
    g = np.empty(n * 10, np.float64)
    diag = (C.c_int * 3)()
    md = OracleMesh.of(mesh).desc()
    cd = ot.case_desc(case)
    rc = lib.ref_residual(C.byref(md), C.byref(cd), u.ctypes.data_as(_dp), int(second_order),
                          float(stab), int(as_fix), float(as_fmin), float(as_ramp),
                          r.ctypes.data_as(_dp), s.ctypes.data_as(_dp), g.ctypes.data_as(_dp), diag)
    if rc != 0:
        raise RuntimeError(lib.ref_last_error().decode())
    return r.reshape(n, 5), s, g.reshape(n, 5, 2), tuple(diag)


def ref_current_mesh():
    """Copy the shim's current mesh into numpy arrays (float32 geometry as in the reference)."""
    lib = ref_lib()
    sizes = (C.c_int * 4)()
    lib.ref_mesh_sizes(sizes)
    nc, nf, npnt, npatch = list(sizes)
    owner = np.empty(nf, np.int32)
    nb = np.empty(nf, np.int32)
    bc = np.empty(nf, np.int32)
    fv = np.empty(2 * nf, np.int32)
    normal = np.empty(3 * nf, np.float32)
    center = np.empty(3 * nf, np.float32)
    area = np.empty(nf, np.float32)
    vol = np.empty(nc, np.float32)
    cc = np.empty(3 * nc, np.float32)
    pts = np.empty(3 * npnt, np.float32)
    conn = np.empty(3 * nc, np.int32)
    patches = np.empty(3 * max(npatch, 1), np.int32)
    fp = C.POINTER(C.c_float)
    lib.ref_mesh_get(owner.ctypes.data_as(_ip), nb.ctypes.data_as(_ip), bc.ctypes.data_as(_ip),
                     fv.ctypes.data_as(_ip), normal.ctypes.data_as(fp), center.ctypes.data_as(fp),
                     area.ctypes.data_as(fp), vol.ctypes.data_as(fp), cc.ctypes.data_as(fp),
                     pts.ctypes.data_as(fp), conn.ctypes.data_as(_ip), patches.ctypes.data_as(_ip))
    patches = patches[: 3 * npatch].reshape(npatch, 3)
    wall = []
    for start, count, is_wall in patches:
        if is_wall:
            wall.extend(range(start, start + count))
    return dict(owner=owner, neighbor=nb, bc=bc, face_vertices=fv, normal=normal, center=center,
                area=area, volume=vol, cell_center=cc, points=pts, cell_conn=conn,
                patches=patches, wall_faces=np.array(wall, np.int32))


def ogrid_synthetic(n_circ: int, n_radial: int, cell_type: int = 3, permute: bool = True, chord: float = 1.0,
                    thickness: float = 0.12, wall_spacing: float = 0.005, farfield_radius: float = 20.0,
                    jitter: float = 0.0, seed: int = 1) -> OracleMesh:
    """The benchmark's synthetic O-grid from the oracle's own generator (oracle_mesh.hpp),
    the same mesh as the product generator builds from the same arguments."""
    lib = oracle_lib()
    h = lib.oracle_mesh_ogrid(n_circ, n_radial, cell_type, int(permute), chord, thickness, wall_spacing,
                              farfield_radius, jitter, seed)
    if not h:
        raise ValueError("oracle_mesh_ogrid: invalid O-grid specification")
    try:
        sizes = (C.c_int * 3)()
        lib.oracle_mesh_sizes(h, sizes)
        nc, nf, nw = list(sizes)
        a = dict(owner=np.empty(nf, np.int32), neighbor=np.empty(nf, np.int32), bc=np.empty(nf, np.int32),
                 normal=np.empty(3 * nf), center=np.empty(3 * nf), area=np.empty(nf), volume=np.empty(nc),
                 cell_center=np.empty(3 * nc), wall_faces=np.empty(nw, np.int32))
        ptr = {k: v.ctypes.data_as(_ip if v.dtype == np.int32 else _dp) for k, v in a.items()}
        lib.oracle_mesh_copy(h, ptr["owner"], ptr["neighbor"], ptr["bc"], ptr["normal"], ptr["center"],
                             ptr["area"], ptr["volume"], ptr["cell_center"], ptr["wall_faces"])
    finally:
        lib.oracle_mesh_free(h)
    return OracleMesh(**a)
