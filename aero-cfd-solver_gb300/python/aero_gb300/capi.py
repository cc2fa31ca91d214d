"""ctypes mirror of include/aero_gb300.h and include/aero_mesh.h.

The structures below have exactly the field order and types of the C declarations;
tests check their sizes against the library's own sizeof values.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_ROOT = Path(__file__).resolve().parents[2]  # .../aero-cfd-solver_gb300
REPO_ROOT = PKG_ROOT.parent
LIB_PATH = PKG_ROOT / "lib" / "libaero_gb300.so"
ABI_VERSION = 4  # AERO_ABI_VERSION of include/aero_gb300.h that these structures mirror

AERO_OK = 0
AERO_ERR_INVALID = 1
AERO_ERR_CUDA = 2
AERO_ERR_NONFINITE = 3
AERO_ERR_STATE = 4
AERO_ERR_TIMEOUT = 5
AERO_ERR_NOMEM = 6

BC_INTERIOR, BC_FARFIELD, BC_WALL = 0, 1, 2
FLUX_RUSANOV, FLUX_HLLC = 0, 1
LIMITER_MINMOD, LIMITER_VENKAT = 0, 1
PRECISION_FP64, PRECISION_FP32 = 0, 1
ORDER_NONE, ORDER_MORTON, ORDER_RCM = 0, 1, 2

REC_FORCE_WINDOW_STABLE = 1
REC_FORCE_DRIFT_STABLE = 2
REC_CONVERGED = 4
REC_SECOND_ORDER = 8
REC_NONFINITE = 16

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


class MeshDesc(C.Structure):
    _fields_ = [
        ("num_cells", C.c_int),
        ("num_faces", C.c_int),
        ("face_owner", _ip),
        ("face_neighbor", _ip),
        ("face_bc", _ip),
        ("face_normal", _dp),
        ("face_center", _dp),
        ("face_area", _dp),
        ("cell_volume", _dp),
        ("cell_center", _dp),
        ("num_wall_faces", C.c_int),
        ("wall_faces", _ip),
    ]


_CASE_FIELDS = [
    ("gamma", C.c_double), ("gas_constant", C.c_double), ("mach", C.c_double),
    ("aoa_deg", C.c_double), ("p_inf", C.c_double), ("t_inf", C.c_double),
    ("rho_inf", C.c_double),
    ("chord", C.c_double), ("x_ref", C.c_double), ("y_ref", C.c_double),
    ("flux", C.c_int), ("limiter", C.c_int),
    ("iterations", C.c_int), ("min_iterations", C.c_int),
    ("cfl_ramp_iters", C.c_int),
    ("cfl_start", C.c_double), ("cfl_max", C.c_double),
    ("residual_reduction_target", C.c_double), ("force_stability_tol", C.c_double),
    ("force_mean_drift_tol", C.c_double),
    ("force_stability_window", C.c_int),
    ("startup_first_order_iters", C.c_int),
    ("rk_stages", C.c_int),
    ("local_time_stepping", C.c_int),
    ("precond_on", C.c_int),
    ("precond_mach_ref", C.c_double), ("precond_mach_min", C.c_double),
    ("precond_beta_min", C.c_double), ("precond_beta_max", C.c_double),
    ("precond_farfield_bc", C.c_int),
    ("stab_floor_start", C.c_double), ("stab_floor_target", C.c_double),
    ("stab_floor_k_start", C.c_double), ("stab_floor_k_target", C.c_double),
    ("stab_ramp_iters", C.c_int),
    ("low_mach_fix", C.c_int),
    ("mach_cutoff", C.c_double),
    ("all_speed_flux_fix", C.c_int),
    ("all_speed_mach_cutoff", C.c_double), ("all_speed_f_min", C.c_double),
    ("all_speed_ramp_start_iter", C.c_int), ("all_speed_ramp_iters", C.c_int),
    ("all_speed_staged_controller", C.c_int),
    ("all_speed_stage_a_min_iters", C.c_int), ("all_speed_stage_a_max_iters", C.c_int),
    ("all_speed_stage_f_min_high", C.c_double), ("all_speed_stage_f_min_mid", C.c_double),
    ("all_speed_stage_f_min_low", C.c_double),
    ("all_speed_pjump_wall_target", C.c_double), ("all_speed_pjump_spike_factor", C.c_double),
    ("all_speed_pjump_hold_iters", C.c_int), ("all_speed_freeze_iters", C.c_int),
    ("all_speed_cfl_drop_factor", C.c_double), ("all_speed_cfl_restore_factor", C.c_double),
    ("all_speed_cfl_min_scale", C.c_double),
    ("aoa0_symmetry_enforce", C.c_int), ("aoa0_symmetry_enforce_interval", C.c_int),
    ("precision", C.c_int),
    ("ordering", C.c_int),
    ("block_size", C.c_int),
    ("diagnostics", C.c_int),
    ("density_l2_target", C.c_double),
    ("cells_per_thread", C.c_int),
    ("precond_fp64", C.c_int),
]


class CaseDesc(C.Structure):
    _fields_ = _CASE_FIELDS


_REC_FIELDS = [
    ("iter", C.c_int), ("flags", C.c_int),
    ("first_order_fallback_faces", C.c_int), ("diffusive_fallback_faces", C.c_int),
] + [(name, C.c_double) for name in (
    "residual_l1", "residual_l2", "residual_linf", "residual_ratio",
    "cl", "cd", "cm", "lift", "drag", "moment",
    "cl_abs", "cd_abs", "cm_abs",
    "fx_gauge", "fy_gauge", "fx_abs", "fy_abs", "sum_nax", "sum_nay",
    "dcl", "dcd", "dcm", "mean_dcl", "mean_dcd", "mean_dcm",
    "cfl", "cfl_scale",
    "stab_mach_floor", "all_speed_f_min", "all_speed_ramp_weight",
    "max_abs_dp_domain", "max_abs_dp_wall",
    "p_jump_energy_nd", "p_jump_energy_wall_nd",
    "max_wall_un", "max_wall_mass_flux", "wall_cp_min", "wall_cp_max",
    "max_farfield_abs_dp", "max_farfield_abs_drho", "max_farfield_abs_du", "max_farfield_abs_dv",
)] + [("wall_cp_nonfinite", C.c_int), ("controller_action", C.c_int), ("residual_rho_ratio", C.c_double)]


class IterRecord(C.Structure):
    _fields_ = _REC_FIELDS


RECORD_DTYPE = np.dtype([(n, np.int32 if t is C.c_int else np.float64) for n, t in _REC_FIELDS])
assert RECORD_DTYPE.itemsize == C.sizeof(IterRecord)

# EulerAirfoilCaseConfig defaults (src/cfd_core/include/cfd_core/solvers/euler_solver.hpp:14-74),
# as float values widened to double.
_F = lambda x: float(np.float32(x))  # noqa: E731
CASE_DEFAULTS = dict(
    gamma=_F(1.4), gas_constant=_F(287.05), mach=_F(0.15), aoa_deg=_F(2.0),
    p_inf=_F(101325.0), t_inf=_F(288.15), rho_inf=0.0,
    chord=1.0, x_ref=_F(0.25), y_ref=0.0,
    flux=FLUX_RUSANOV, limiter=LIMITER_MINMOD,
    iterations=400, min_iterations=40, cfl_ramp_iters=120,
    cfl_start=_F(0.2), cfl_max=_F(1.2),
    residual_reduction_target=_F(1.0e-3), force_stability_tol=_F(2.0e-5),
    force_mean_drift_tol=_F(2.0e-5), force_stability_window=6,
    startup_first_order_iters=25, rk_stages=3, local_time_stepping=1,
    precond_on=0, precond_mach_ref=_F(0.15), precond_mach_min=_F(1.0e-3),
    precond_beta_min=_F(0.2), precond_beta_max=1.0, precond_farfield_bc=0,
    stab_floor_start=_F(0.1), stab_floor_target=_F(0.02),
    stab_floor_k_start=-1.0, stab_floor_k_target=-1.0, stab_ramp_iters=400,
    low_mach_fix=0, mach_cutoff=_F(0.3),
    all_speed_flux_fix=0, all_speed_mach_cutoff=_F(0.25), all_speed_f_min=_F(0.05),
    all_speed_ramp_start_iter=0, all_speed_ramp_iters=0,
    all_speed_staged_controller=0, all_speed_stage_a_min_iters=600,
    all_speed_stage_a_max_iters=0,
    all_speed_stage_f_min_high=_F(0.2), all_speed_stage_f_min_mid=_F(0.1),
    all_speed_stage_f_min_low=_F(0.05),
    all_speed_pjump_wall_target=0.0, all_speed_pjump_spike_factor=_F(1.5),
    all_speed_pjump_hold_iters=120, all_speed_freeze_iters=120,
    all_speed_cfl_drop_factor=_F(0.8), all_speed_cfl_restore_factor=_F(1.02),
    all_speed_cfl_min_scale=_F(0.1),
    aoa0_symmetry_enforce=0, aoa0_symmetry_enforce_interval=0,
    precision=PRECISION_FP64, ordering=ORDER_MORTON, block_size=0, diagnostics=0,
    density_l2_target=0.0, cells_per_thread=0, precond_fp64=0,
)


def make_case(**overrides) -> CaseDesc:
    """CaseDesc with the reference defaults, float-valued overrides rounded to float32
    (the reference parses every real setting with std::stof)."""
    values = dict(CASE_DEFAULTS)
    for key, val in overrides.items():
        if key not in values:
            raise KeyError(f"unknown case field {key!r}")
        if isinstance(values[key], float):
            values[key] = _F(val)
        else:
            values[key] = int(val)
    desc = CaseDesc()
    for key, val in values.items():
        setattr(desc, key, val)
    return desc


def case_to_dict(desc: CaseDesc) -> dict:
    return {name: getattr(desc, name) for name, _ in _CASE_FIELDS}


class Mesh:
    """Reference-layout mesh held in numpy arrays (geometry in float64).

    Fields follow UnstructuredMesh (src/cfd_core/include/cfd_core/mesh.hpp:14-35);
    ``bc`` is the per-face boundary type and ``wall_faces`` the wall patch in order.
    Optional ``points``, ``cell_conn``/``cell_offsets`` and ``face_vertices`` serve the
    VTU and Cp outputs.
    """

    def __init__(self, owner, neighbor, bc, normal, center, area, volume, cell_center,
                 wall_faces, points=None, face_vertices=None, cell_conn=None,
                 cell_offsets=None, farfield_faces=None):
        self.owner = np.ascontiguousarray(owner, dtype=np.int32)
        self.neighbor = np.ascontiguousarray(neighbor, dtype=np.int32)
        self.bc = np.ascontiguousarray(bc, dtype=np.int32)
        self.normal = np.ascontiguousarray(normal, dtype=np.float64).reshape(-1)
        self.center = np.ascontiguousarray(center, dtype=np.float64).reshape(-1)
        self.area = np.ascontiguousarray(area, dtype=np.float64)
        self.volume = np.ascontiguousarray(volume, dtype=np.float64)
        self.cell_center = np.ascontiguousarray(cell_center, dtype=np.float64).reshape(-1)
        self.wall_faces = np.ascontiguousarray(wall_faces, dtype=np.int32)
        self.points = None if points is None else np.asarray(points, dtype=np.float64)
        self.face_vertices = None if face_vertices is None else np.asarray(face_vertices, np.int32)
        self.cell_conn = None if cell_conn is None else np.asarray(cell_conn, np.int32)
        self.cell_offsets = None if cell_offsets is None else np.asarray(cell_offsets, np.int32)
        self.farfield_faces = farfield_faces

    @property
    def num_cells(self) -> int:
        return int(self.volume.shape[0])

    @property
    def num_faces(self) -> int:
        return int(self.owner.shape[0])

    def desc(self) -> MeshDesc:
        d = MeshDesc()
        d.num_cells = self.num_cells
        d.num_faces = self.num_faces
        d.face_owner = self.owner.ctypes.data_as(_ip)
        d.face_neighbor = self.neighbor.ctypes.data_as(_ip)
        d.face_bc = self.bc.ctypes.data_as(_ip)
        d.face_normal = self.normal.ctypes.data_as(_dp)
        d.face_center = self.center.ctypes.data_as(_dp)
        d.face_area = self.area.ctypes.data_as(_dp)
        d.cell_volume = self.volume.ctypes.data_as(_dp)
        d.cell_center = self.cell_center.ctypes.data_as(_dp)
        d.num_wall_faces = int(self.wall_faces.shape[0])
        d.wall_faces = self.wall_faces.ctypes.data_as(_ip)
        d._keepalive = self  # the arrays must outlive the descriptor
        return d

    @classmethod
    def from_npz(cls, data, prefix: str = "") -> "Mesh":
        g = lambda k: data[prefix + k] if (prefix + k) in data else None  # noqa: E731
        return cls(g("owner"), g("neighbor"), g("bc"), g("normal"), g("center"), g("area"),
                   g("volume"), g("cell_center"), g("wall_faces"), points=g("points"),
                   face_vertices=g("face_vertices"), cell_conn=g("cell_conn"))


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def records_to_array(recs, n: int) -> np.ndarray:
    raw = np.frombuffer(C.string_at(C.addressof(recs), n * C.sizeof(IterRecord)),
                        dtype=RECORD_DTYPE, count=n)
    return raw.copy()


def env_flag_on(name: str) -> bool:
    """The reference's env_flag_on (src/cfd_core/solvers/euler_solver.cpp:37-44)."""
    return os.environ.get(name) in ("1", "true", "TRUE", "on", "ON")
