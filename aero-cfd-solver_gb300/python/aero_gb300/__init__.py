"""Python side of the GB300 Euler residual-and-update path: ctypes over libaero_gb300.so.

The library is the product; this module only binds it. There is no CPU fallback: every
solver call goes to the CUDA path, and Solver() raises when no sm_103 device is usable.
"""

from __future__ import annotations

import ctypes as C
import weakref
from pathlib import Path

import numpy as np

from . import capi
from .capi import CaseDesc, IterRecord, Mesh, MeshDesc, make_case  # noqa: F401

_lib = None
_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_llp = C.POINTER(C.c_longlong)


class OgridSpec(C.Structure):
    _fields_ = [
        ("n_circ", C.c_int), ("n_radial", C.c_int), ("cell_type", C.c_int), ("permute", C.c_int),
        ("chord", C.c_double), ("thickness", C.c_double), ("wall_spacing", C.c_double),
        ("farfield_radius", C.c_double), ("jitter", C.c_double), ("seed", C.c_ulonglong),
    ]


class MeshSizes(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("num_cells", "num_faces", "num_points", "num_wall_faces",
                                       "num_farfield_faces", "conn_length")]


class AeroError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"aero error {code}: {msg}")
        self.code = code


def library_path() -> Path:
    return capi.LIB_PATH


def load(build_if_missing: bool = False):
    """Load libaero_gb300.so (built in-tree by aero-cfd-solver_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    path = capi.LIB_PATH
    if not path.exists():
        if not build_if_missing:
            raise FileNotFoundError(f"{path} is missing: run aero-cfd-solver_gb300/build.py")
        import importlib.util

        spec = importlib.util.spec_from_file_location("aero_build", capi.PKG_ROOT / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = C.CDLL(str(path))
    sig = {
        "aero_abi_version": (C.c_int, []),
        "aero_version": (C.c_char_p, []),
        "aero_cuda_available": (C.c_int, []),
        "aero_case_defaults": (None, [C.POINTER(CaseDesc)]),
        "aero_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(CaseDesc), C.POINTER(C.c_void_p)]),
        "aero_destroy": (None, [C.c_void_p]),
        "aero_last_error": (C.c_char_p, [C.c_void_p]),
        "aero_set_state": (C.c_int, [C.c_void_p, _dp]),
        "aero_get_state": (C.c_int, [C.c_void_p, _dp]),
        "aero_get_primitive": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
        "aero_residual": (C.c_int, [C.c_void_p, _dp, C.c_int, C.c_double, C.c_int, C.c_double,
                                    C.c_double, _dp, _dp, _dp]),
        "aero_run": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(IterRecord), _ip]),
        "aero_reset_run": (C.c_int, [C.c_void_p]),
        "aero_get_last_residual": (C.c_int, [C.c_void_p, _dp, _dp]),
        "aero_time_iterations": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp]),
        "aero_profile_kernels": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _ip]),
        "aero_profile_graph": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _ip, _dp]),
        "aero_select_device": (C.c_int, [C.c_int]),
        "aero_get_info": (C.c_int, [C.c_void_p, _llp, C.c_int]),
        "aero_set_wait_limit": (C.c_int, [C.c_void_p, C.c_int]),
        "aero_batch_create": (C.c_int, [C.c_int, C.POINTER(MeshDesc), C.POINTER(CaseDesc), C.POINTER(C.c_void_p)]),
        "aero_autotune": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(CaseDesc), C.c_int, C.POINTER(CaseDesc), _dp]),
        "aero_batch_size": (C.c_int, [C.c_void_p]),
        "aero_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(IterRecord), _ip]),
        "aero_batch_set_state": (C.c_int, [C.c_void_p, C.c_int, _dp]),
        "aero_batch_get_state": (C.c_int, [C.c_void_p, C.c_int, _dp]),
        "aero_batch_get_last_residual": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp]),
        "aero_mesh_ogrid_reference": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double,
                                                C.c_double, C.POINTER(C.c_void_p)]),
        "aero_mesh_ogrid_synthetic": (C.c_int, [C.POINTER(OgridSpec), C.POINTER(C.c_void_p)]),
        "aero_mesh_free": (None, [C.c_void_p]),
        "aero_mesh_last_error": (C.c_char_p, []),
        "aero_mesh_get_sizes": (C.c_int, [C.c_void_p, C.POINTER(MeshSizes)]),
        "aero_mesh_describe": (C.c_int, [C.c_void_p, C.POINTER(MeshDesc)]),
        "aero_mesh_get_aux": (C.c_int, [C.c_void_p, _dp, _ip, _ip, _ip, C.POINTER(C.c_ubyte), _ip]),
        "aero_mesh_clone": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
        "aero_mesh_set_points": (C.c_int, [C.c_void_p, _dp]),
        "aero_mesh_geometry_tangent": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]),
        "aero_mesh_hicks_henne_modes": (C.c_int, [C.c_void_p, C.c_int, _dp, _ip, C.c_double, _dp]),
        "aero_adjoint_linearize": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int]),
        "aero_adjoint_vjp": (C.c_int, [C.c_void_p, _dp, _dp]),
        "aero_adjoint_objective_gradient": (C.c_int, [C.c_void_p, _dp]),
        "aero_adjoint_solve": (C.c_int, [C.c_void_p, C.c_int, C.c_double, _dp]),
        "aero_adjoint_get_lambda": (C.c_int, [C.c_void_p, _dp]),
        "aero_adjoint_set_lambda": (C.c_int, [C.c_void_p, _dp]),
        "aero_adjoint_solve_krylov": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _dp,
                                                _ip]),
        "aero_adjoint_dalpha": (C.c_int, [C.c_void_p, _dp]),
        "aero_adjoint_geometry": (C.c_int, [C.c_void_p, C.POINTER(MeshDesc), _dp]),
        "aero_adjoint_geometry_vjp": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp]),
        "aero_adjoint_node_vjp": (C.c_int, [C.c_void_p, C.c_void_p, _dp]),
        "aero_mesh_geometry_vjp": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.aero_abi_version() != capi.ABI_VERSION:  # a stale build: its structures differ
        raise ImportError(f"{path} has ABI {lib.aero_abi_version()}, these bindings ABI {capi.ABI_VERSION}: "
                          "rebuild with aero-cfd-solver_gb300/build.py")
    _lib = lib
    return lib


def cuda_available() -> bool:
    return bool(load().aero_cuda_available())


def select_device(device: int) -> None:
    rc = load().aero_select_device(device)
    if rc != 0:
        raise AeroError(rc, load().aero_last_error(None).decode())


# --------------------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------------------
def _mesh_from_handle(h) -> Mesh:
    """Copy a generated mesh into numpy arrays; the Mesh keeps the handle (freed with it)
    for the node-based operations (deform, geometry_tangent, hicks_henne_modes)."""
    lib = load()
    sz = MeshSizes()
    lib.aero_mesh_get_sizes(h, C.byref(sz))
    d = MeshDesc()
    lib.aero_mesh_describe(h, C.byref(d))
    nf, nc = sz.num_faces, sz.num_cells

    def arr(ptr, n, dtype):
        return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)

    points = np.empty(3 * sz.num_points, np.float64)
    fv = np.empty(2 * nf, np.int32)
    conn = np.empty(sz.conn_length, np.int32)
    offs = np.empty(nc, np.int32)
    types = np.empty(nc, np.uint8)
    ff = np.empty(max(sz.num_farfield_faces, 1), np.int32)
    lib.aero_mesh_get_aux(h, points.ctypes.data_as(_dp), fv.ctypes.data_as(_ip), conn.ctypes.data_as(_ip),
                          offs.ctypes.data_as(_ip), types.ctypes.data_as(C.POINTER(C.c_ubyte)),
                          ff.ctypes.data_as(_ip))
    m = Mesh(arr(d.face_owner, nf, np.int32), arr(d.face_neighbor, nf, np.int32), arr(d.face_bc, nf, np.int32),
             arr(d.face_normal, 3 * nf, np.float64), arr(d.face_center, 3 * nf, np.float64),
             arr(d.face_area, nf, np.float64), arr(d.cell_volume, nc, np.float64),
             arr(d.cell_center, 3 * nc, np.float64),
             arr(d.wall_faces, sz.num_wall_faces, np.int32) if sz.num_wall_faces else np.zeros(0, np.int32),
             points=points, face_vertices=fv, cell_conn=conn, cell_offsets=offs,
             farfield_faces=ff[: sz.num_farfield_faces])
    m.cell_types = types
    m._handle = h
    weakref.finalize(m, lib.aero_mesh_free, h)
    return m


def _handle(mesh: Mesh):
    h = getattr(mesh, "_handle", None)
    if h is None:
        raise ValueError("mesh has no node data: generate it with ogrid_synthetic / ogrid_reference")
    return h


def deform(mesh: Mesh, points: np.ndarray) -> Mesh:
    """A copy of `mesh` with its nodes moved to points [P, 3] and the geometry recomputed
    (aero_mesh_set_points)."""
    lib = load()
    h = C.c_void_p()
    rc = lib.aero_mesh_clone(_handle(mesh), C.byref(h))
    if rc != 0:
        raise AeroError(rc, lib.aero_mesh_last_error().decode())
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1)
    rc = lib.aero_mesh_set_points(h, pts.ctypes.data_as(_dp))
    if rc != 0:
        msg = lib.aero_mesh_last_error().decode()
        lib.aero_mesh_free(h)
        raise AeroError(rc, msg)
    return _mesh_from_handle(h)


def geometry_tangent(mesh: Mesh, dpoints: np.ndarray) -> Mesh:
    """The derivative of the mesh geometry along a node displacement dpoints [P, 3], as a
    Mesh with the connectivity of `mesh` and the derivatives in its geometry arrays (the
    input of Solver.adjoint_geometry)."""
    lib = load()
    dp = np.ascontiguousarray(dpoints, dtype=np.float64).reshape(-1)
    nf, nc = mesh.num_faces, mesh.num_cells
    dn, dc, da = np.empty(3 * nf), np.empty(3 * nf), np.empty(nf)
    dv, dcc = np.empty(nc), np.empty(3 * nc)
    rc = lib.aero_mesh_geometry_tangent(_handle(mesh), dp.ctypes.data_as(_dp), dn.ctypes.data_as(_dp),
                                        dc.ctypes.data_as(_dp), da.ctypes.data_as(_dp), dv.ctypes.data_as(_dp),
                                        dcc.ctypes.data_as(_dp))
    if rc != 0:
        raise AeroError(rc, lib.aero_mesh_last_error().decode())
    return Mesh(mesh.owner, mesh.neighbor, mesh.bc, dn, dc, da, dv, dcc, mesh.wall_faces)


def geometry_vjp(mesh: Mesh, bars: Mesh) -> np.ndarray:
    """The transpose of geometry_tangent: `bars` carries, in its geometry arrays, derivatives of
    a scalar with respect to the mesh geometry (Solver.adjoint_geometry_vjp); returns the
    derivatives with respect to the node coordinates [P, 3]."""
    lib = load()
    out = np.empty(mesh.points.size, np.float64)
    arrays = [np.ascontiguousarray(a, dtype=np.float64) for a in
              (bars.normal, bars.center, bars.area, bars.volume, bars.cell_center)]
    rc = lib.aero_mesh_geometry_vjp(_handle(mesh), *[a.ctypes.data_as(_dp) for a in arrays], out.ctypes.data_as(_dp))
    if rc != 0:
        raise AeroError(rc, lib.aero_mesh_last_error().decode())
    return out.reshape(-1, 3)


def hicks_henne_modes(mesh: Mesh, peaks, upper, width: float = 3.0) -> np.ndarray:
    """Node displacement modes [n, P, 3] of Hicks-Henne bumps with unit amplitude, carried
    into the volume by inverse-distance weighting (aero_mesh_hicks_henne_modes)."""
    lib = load()
    pk = np.ascontiguousarray(peaks, dtype=np.float64)
    up = np.ascontiguousarray(upper, dtype=np.int32)
    assert pk.shape == up.shape
    npts = mesh.points.size // 3
    modes = np.empty((pk.size, npts, 3), np.float64)
    rc = lib.aero_mesh_hicks_henne_modes(_handle(mesh), pk.size, pk.ctypes.data_as(_dp), up.ctypes.data_as(_ip),
                                         float(width), modes.ctypes.data_as(_dp))
    if rc != 0:
        raise AeroError(rc, lib.aero_mesh_last_error().decode())
    return modes


def ogrid_reference(naca: str = "0012", n_circ: int = 160, n_radial: int = 48,
                    farfield_radius: float = 15.0, radial_stretch: float = 1.4, chord: float = 1.0) -> Mesh:
    """The reference's triangulated O-grid (make_airfoil_ogrid_mesh, airfoil_mesh.cpp:459)."""
    lib = load()
    h = C.c_void_p()
    rc = lib.aero_mesh_ogrid_reference(naca.encode(), n_circ, n_radial, farfield_radius, radial_stretch,
                                       chord, C.byref(h))
    if rc != 0:
        raise AeroError(rc, lib.aero_mesh_last_error().decode())
    return _mesh_from_handle(h)


def ogrid_synthetic(n_circ: int, n_radial: int, cell_type: int = 3, permute: bool = True,
                    chord: float = 1.0, thickness: float = 0.12, wall_spacing: float = 0.005,
                    farfield_radius: float = 20.0, jitter: float = 0.1, seed: int = 0) -> Mesh:
    """Benchmark O-grid: NACA 00xx closed TE, cosine clustering, first wall spacing, geometric
    growth, quads (cell_type 4) or seeded-diagonal triangles (3), jitter, permutations."""
    lib = load()
    spec = OgridSpec(n_circ, n_radial, cell_type, int(permute), chord, thickness, wall_spacing,
                     farfield_radius, jitter, seed)
    h = C.c_void_p()
    rc = lib.aero_mesh_ogrid_synthetic(C.byref(spec), C.byref(h))
    if rc != 0:
        raise AeroError(rc, lib.aero_mesh_last_error().decode())
    return _mesh_from_handle(h)


def autotune(mesh: Mesh, case: CaseDesc, iters: int = 20):
    """Fastest cell ordering, block size and cells per thread for this mesh and case
    (aero_autotune). Returns (case with them set, {(ordering, block, cells_per_thread): device
    ms of `iters` iterations})."""
    lib = load()
    md = mesh.desc()
    best = CaseDesc()
    ms = (C.c_double * 12)()
    rc = lib.aero_autotune(C.byref(md), C.byref(case), iters, C.byref(best), ms)
    if rc != 0:
        raise AeroError(rc, lib.aero_last_error(None).decode())
    table = {}
    k = 0
    for o in (capi.ORDER_MORTON, capi.ORDER_RCM):
        for b in (64, 128, 256):
            for t in (1, 2):
                table[(o, b, t)] = ms[k]
                k += 1
    return best, table


# --------------------------------------------------------------------------------------
# solver
# --------------------------------------------------------------------------------------
class Solver:
    """One device context (aero_create) on a mesh and a case."""

    def __init__(self, mesh: Mesh, case: CaseDesc):
        self.lib = load()
        self.mesh = mesh
        self.case = case
        self._mdesc = mesh.desc()
        h = C.c_void_p()
        rc = self.lib.aero_create(C.byref(self._mdesc), C.byref(case), C.byref(h))
        if rc != 0:
            raise AeroError(rc, self.lib.aero_last_error(None).decode())
        self.h = h
        self.n = mesh.num_cells

    def close(self):
        if getattr(self, "h", None):
            self.lib.aero_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc != 0:
            raise AeroError(rc, self.lib.aero_last_error(self.h).decode())

    def set_state(self, u: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        assert u.size == 5 * self.n
        self._check(self.lib.aero_set_state(self.h, u.ctypes.data_as(_dp)))

    def get_state(self, out: np.ndarray | None = None) -> np.ndarray:
        """The conserved state [N, 5] in the original cell order; `out` (float64, C-contiguous,
        N*5 values) is filled and returned instead of a new array when given."""
        if out is None:
            out = np.empty((self.n, 5), np.float64)
        if not (out.dtype == np.float64 and out.flags.c_contiguous and out.flags.writeable and out.size == 5 * self.n):
            raise ValueError("get_state: out must be a writable C-contiguous float64 array of N*5 values")
        self._check(self.lib.aero_get_state(self.h, out.ctypes.data_as(_dp)))
        return out.reshape(self.n, 5)

    def get_primitive(self):
        out = [np.empty(self.n, np.float64) for _ in range(4)]
        self._check(self.lib.aero_get_primitive(self.h, *[a.ctypes.data_as(_dp) for a in out]))
        return out

    def residual(self, u, second_order=True, stab=0.0, as_fix=False, as_fmin=0.05, as_ramp=1.0):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        r = np.empty(5 * self.n, np.float64)
        s = np.empty(self.n, np.float64)
        g = np.empty(10 * self.n, np.float64)
        self._check(self.lib.aero_residual(self.h, u.ctypes.data_as(_dp), int(second_order), float(stab),
                                           int(as_fix), float(as_fmin), float(as_ramp), r.ctypes.data_as(_dp),
                                           s.ctypes.data_as(_dp), g.ctypes.data_as(_dp)))
        return r.reshape(self.n, 5), s, g.reshape(self.n, 5, 2)

    def run(self, n: int, raise_on_nonfinite: bool = True):
        recs = (IterRecord * max(n, 1))()
        done = C.c_int(0)
        rc = self.lib.aero_run(self.h, n, recs, C.byref(done))
        out = capi.records_to_array(recs, done.value)
        if rc in (capi.AERO_ERR_NONFINITE, capi.AERO_ERR_TIMEOUT) and not raise_on_nonfinite:
            return rc, out
        self._check(rc)
        return rc, out

    def reset_run(self):
        self._check(self.lib.aero_reset_run(self.h))

    def last_residual(self):
        r = np.empty(5 * self.n, np.float64)
        s = np.empty(self.n, np.float64)
        self._check(self.lib.aero_get_last_residual(self.h, r.ctypes.data_as(_dp), s.ctypes.data_as(_dp)))
        return r.reshape(self.n, 5), s

    def time_iterations(self, n: int, use_graph: bool = True, flush_l2: bool = False) -> float:
        """Device milliseconds of n iterations (CUDA events on the context's stream)."""
        ms = C.c_double(0.0)
        self._check(self.lib.aero_time_iterations(self.h, n, int(use_graph), int(flush_l2), C.byref(ms)))
        return ms.value

    # face_pass: the residual face pass (and its cell pass under global time stepping);
    # update: the RK update, which gathers the cell residual itself under local time stepping
    KERNEL_CLASSES = ("gradient", "face_pass", "update", "global_dt", "symmetry_pjump", "control")

    def profile_kernels(self, n: int, flush_l2: bool = False) -> dict:
        """Summed device ms and launch counts per kernel class over n iterations."""
        ms = (C.c_double * 6)()
        launches = (C.c_int * 6)()
        self._check(self.lib.aero_profile_kernels(self.h, n, int(flush_l2), ms, launches))
        return {k: (ms[i], launches[i]) for i, k in enumerate(self.KERNEL_CLASSES)}

    def profile_graph(self, n: int, flush_l2: bool = False) -> tuple[dict, float]:
        """Kernel times of n iterations inside the timed iteration graphs (recorded through
        CUPTI): ({class: (ms, launches)}, device ms of the n iterations)."""
        ms = (C.c_double * 6)()
        launches = (C.c_int * 6)()
        total = C.c_double(0.0)
        self._check(self.lib.aero_profile_graph(self.h, n, int(flush_l2), ms, launches, C.byref(total)))
        names = ("gradient", "face_pass", "update", "global_dt", "symmetry_pjump", "control")
        return {names[k]: (ms[k], launches[k]) for k in range(6)}, total.value

    def info(self) -> dict:
        v = (C.c_longlong * 10)()
        self._check(self.lib.aero_get_info(self.h, v, 10))
        keys = ("cells", "faces", "slots_per_cell", "launches_per_iteration", "device_bytes", "precision",
                "block_size", "blocks", "cases", "bulk_copy_gradient")
        return dict(zip(keys, list(v)))

    def set_wait_limit(self, polls: int) -> None:
        """Poll limit of the iterations' bounded waits on bulk copies (< 0: the default)."""
        self._check(self.lib.aero_set_wait_limit(self.h, int(polls)))

    # ---- discrete adjoint (include/aero_adjoint.h; FP64 contexts)
    def adjoint_linearize(self, w_cd: float = 1.0, w_cl: float = 0.0, second_order: int = -1):
        """Linearise at the current state for J = w_cd CD + w_cl CL; lam starts at 0."""
        self._check(self.lib.aero_adjoint_linearize(self.h, float(w_cd), float(w_cl), int(second_order)))

    def adjoint_vjp(self, v: np.ndarray) -> np.ndarray:
        """(dR/dU)^T v at the linearisation point, [N, 5] in and out."""
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        assert v.size == 5 * self.n
        out = np.empty(5 * self.n, np.float64)
        self._check(self.lib.aero_adjoint_vjp(self.h, v.ctypes.data_as(_dp), out.ctypes.data_as(_dp)))
        return out.reshape(self.n, 5)

    def adjoint_objective_gradient(self) -> np.ndarray:
        g = np.empty(5 * self.n, np.float64)
        self._check(self.lib.aero_adjoint_objective_gradient(self.h, g.ctypes.data_as(_dp)))
        return g.reshape(self.n, 5)

    def adjoint_solve(self, iters: int, cfl: float = 0.8) -> np.ndarray:
        """Pseudo-time iterations of the adjoint; returns the RMS adjoint residual per iteration."""
        hist = np.empty(max(iters, 1), np.float64)
        self._check(self.lib.aero_adjoint_solve(self.h, int(iters), float(cfl), hist.ctypes.data_as(_dp)))
        return hist[:iters]

    def adjoint_solve_krylov(self, max_iters: int = 2000, restart: int = 40, smooth: int = 10, cfl: float = 0.8,
                             rtol: float = 1e-10) -> np.ndarray:
        """Restarted GMRES on the adjoint system, preconditioned by `smooth` smoother
        iterations; returns the relative residual estimate per Arnoldi step."""
        hist = np.empty(max(max_iters, 1), np.float64)
        done = C.c_int(0)
        self._check(self.lib.aero_adjoint_solve_krylov(self.h, int(max_iters), int(restart), int(smooth), float(cfl),
                                                       float(rtol), hist.ctypes.data_as(_dp), C.byref(done)))
        return hist[: done.value]

    def adjoint_set_lambda(self, lam: np.ndarray):
        lam = np.ascontiguousarray(lam, dtype=np.float64).reshape(-1)
        assert lam.size == 5 * self.n
        self._check(self.lib.aero_adjoint_set_lambda(self.h, lam.ctypes.data_as(_dp)))

    def adjoint_lambda(self) -> np.ndarray:
        lam = np.empty(5 * self.n, np.float64)
        self._check(self.lib.aero_adjoint_get_lambda(self.h, lam.ctypes.data_as(_dp)))
        return lam.reshape(self.n, 5)

    def adjoint_dalpha(self) -> float:
        """dJ/d(alpha) per degree."""
        out = C.c_double(0.0)
        self._check(self.lib.aero_adjoint_dalpha(self.h, C.byref(out)))
        return out.value

    def adjoint_geometry(self, tangent: Mesh) -> float:
        """dJ/dX . dX for a geometry tangent (geometry_tangent(mesh, dpoints))."""
        d = tangent.desc()
        out = C.c_double(0.0)
        self._check(self.lib.aero_adjoint_geometry(self.h, C.byref(d), C.byref(out)))
        return out.value

    def adjoint_geometry_vjp(self) -> Mesh:
        """dJ/d(geometry) with the current lam, as a Mesh with this solver's connectivity whose
        geometry arrays hold the derivatives (the transpose of adjoint_geometry)."""
        m = self.mesh
        nf, nc = m.num_faces, m.num_cells
        dn, dc, da, dv, dcc = np.empty(3 * nf), np.empty(3 * nf), np.empty(nf), np.empty(nc), np.empty(3 * nc)
        self._check(self.lib.aero_adjoint_geometry_vjp(self.h, dn.ctypes.data_as(_dp), dc.ctypes.data_as(_dp),
                                                       da.ctypes.data_as(_dp), dv.ctypes.data_as(_dp),
                                                       dcc.ctypes.data_as(_dp)))
        return Mesh(m.owner, m.neighbor, m.bc, dn, dc, da, dv, dcc, m.wall_faces)

    def adjoint_node_vjp(self) -> np.ndarray:
        """dJ/dX for every node of this solver's (generated) mesh [P, 3], one reverse pass."""
        out = np.empty(self.mesh.points.size, np.float64)
        self._check(self.lib.aero_adjoint_node_vjp(self.h, _handle(self.mesh), out.ctypes.data_as(_dp)))
        return out.reshape(-1, 3)


class Batch(Solver):
    """Many cases advanced together in one device context (aero_batch_create): meshes of
    uneven size and per-case flow conditions, one set of packed arrays, one CUDA graph per
    iteration. Each case's results equal a single-case run of it."""

    def __init__(self, meshes, cases):
        assert len(meshes) == len(cases) and len(meshes) > 0
        self.lib = load()
        self.meshes = list(meshes)
        self.cases = list(cases)
        self._mdescs = (MeshDesc * len(meshes))(*[m.desc() for m in self.meshes])
        self._cdescs = (CaseDesc * len(cases))(*self.cases)
        h = C.c_void_p()
        rc = self.lib.aero_batch_create(len(meshes), self._mdescs, self._cdescs, C.byref(h))
        if rc != 0:
            raise AeroError(rc, self.lib.aero_last_error(None).decode())
        self.h = h
        self.k = len(meshes)
        self.sizes = [m.num_cells for m in self.meshes]

    def set_state(self, k: int, u: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        assert u.size == 5 * self.sizes[k]
        self._check(self.lib.aero_batch_set_state(self.h, k, u.ctypes.data_as(_dp)))

    def get_state(self, k: int) -> np.ndarray:
        u = np.empty(5 * self.sizes[k], np.float64)
        self._check(self.lib.aero_batch_get_state(self.h, k, u.ctypes.data_as(_dp)))
        return u.reshape(self.sizes[k], 5)

    def run(self, n: int, raise_on_nonfinite: bool = True):
        """Returns (status, [records of case k]) with each case's records as a structured array."""
        recs = (IterRecord * max(n * self.k, 1))()
        done = (C.c_int * self.k)()
        rc = self.lib.aero_batch_run(self.h, n, recs, done)
        base = capi.records_to_array(recs, n * self.k) if n > 0 else None
        out = [base[k * n: k * n + done[k]].copy() if n > 0 else capi.records_to_array(recs, 0)
               for k in range(self.k)]
        if rc in (capi.AERO_ERR_NONFINITE, capi.AERO_ERR_TIMEOUT) and not raise_on_nonfinite:
            return rc, out
        self._check(rc)
        return rc, out

    def last_residual(self, k: int):
        n = self.sizes[k]
        r = np.empty(5 * n, np.float64)
        s = np.empty(n, np.float64)
        self._check(self.lib.aero_batch_get_last_residual(self.h, k, r.ctypes.data_as(_dp), s.ctypes.data_as(_dp)))
        return r.reshape(n, 5), s

    def residual(self, *args, **kw):
        raise NotImplementedError("single residual evaluations need a single-case Solver")

    def get_primitive(self):
        raise NotImplementedError("use get_state(k)")
