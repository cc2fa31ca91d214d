"""TEST INFRASTRUCTURE ONLY: ctypes structures of the oracle's C interface, read from the C
header the oracle is compiled against (include/aero_gb300.h), so that the oracle's Python
side needs nothing from the product package.

The header's structures are plain C (ints, doubles and pointers to them); this module reads
their field declarations, in order, and builds the matching ctypes.Structure classes. A CPU
test checks them field by field against the product's own ctypes mirror.
"""

from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np

HEADER = Path(__file__).resolve().parents[1] / "include" / "aero_gb300.h"

_CTYPES = {"int": C.c_int, "double": C.c_double, "const int*": C.POINTER(C.c_int),
           "const double*": C.POINTER(C.c_double)}


def _struct_fields(text: str, name: str):
    body = re.search(r"typedef\s+struct\s+" + name + r"\s*\{(.*?)\}\s*" + name + r"\s*;", text, re.S)
    if body is None:
        raise LookupError(f"struct {name} not found in {HEADER}")
    fields = []
    for decl in body.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"((?:const\s+)?(?:int|double))\s*(\*?)\s*(.*)", decl, re.S)
        if m is None:
            raise ValueError(f"unsupported declaration in {name}: {decl!r}")
        ctype = _CTYPES[m.group(1) + m.group(2)]
        for ident in m.group(3).split(","):
            fields.append((ident.strip(), ctype))
    return fields


def _header_text() -> str:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


_TEXT = _header_text()


class MeshDesc(C.Structure):
    _fields_ = _struct_fields(_TEXT, "aero_mesh_desc")


class CaseDesc(C.Structure):
    _fields_ = _struct_fields(_TEXT, "aero_case_desc")


class IterRecord(C.Structure):
    _fields_ = _struct_fields(_TEXT, "aero_iter_record")


RECORD_DTYPE = np.dtype([(n, np.int32 if t is C.c_int else np.float64) for n, t in IterRecord._fields_])
assert RECORD_DTYPE.itemsize == C.sizeof(IterRecord)

CASE_FIELDS = [n for n, _ in CaseDesc._fields_]


def case_desc(case) -> CaseDesc:
    """The oracle's CaseDesc with every field of `case` (any object carrying the header's
    field names as attributes, or a dict of them)."""
    out = CaseDesc()
    get = case.get if isinstance(case, dict) else (lambda k: getattr(case, k))
    for name in CASE_FIELDS:
        setattr(out, name, get(name))
    return out


class OracleMesh:
    """Reference-layout mesh arrays (geometry in float64) with the attribute names of the
    C descriptor's arrays; also accepts any object carrying them."""

    def __init__(self, owner, neighbor, bc, normal, center, area, volume, cell_center, wall_faces):
        self.owner = np.ascontiguousarray(owner, dtype=np.int32)
        self.neighbor = np.ascontiguousarray(neighbor, dtype=np.int32)
        self.bc = np.ascontiguousarray(bc, dtype=np.int32)
        self.normal = np.ascontiguousarray(normal, dtype=np.float64).reshape(-1)
        self.center = np.ascontiguousarray(center, dtype=np.float64).reshape(-1)
        self.area = np.ascontiguousarray(area, dtype=np.float64)
        self.volume = np.ascontiguousarray(volume, dtype=np.float64)
        self.cell_center = np.ascontiguousarray(cell_center, dtype=np.float64).reshape(-1)
        self.wall_faces = np.ascontiguousarray(wall_faces, dtype=np.int32)

    @classmethod
    def of(cls, mesh) -> "OracleMesh":
        if isinstance(mesh, cls):
            return mesh
        return cls(mesh.owner, mesh.neighbor, mesh.bc, mesh.normal, mesh.center, mesh.area, mesh.volume,
                   mesh.cell_center, mesh.wall_faces)

    @property
    def num_cells(self) -> int:
        return int(self.volume.shape[0])

    @property
    def num_faces(self) -> int:
        return int(self.owner.shape[0])

    def desc(self) -> MeshDesc:
        ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
        d = MeshDesc()
        d.num_cells = self.num_cells
        d.num_faces = self.num_faces
        d.face_owner = self.owner.ctypes.data_as(ip)
        d.face_neighbor = self.neighbor.ctypes.data_as(ip)
        d.face_bc = self.bc.ctypes.data_as(ip)
        d.face_normal = self.normal.ctypes.data_as(dp)
        d.face_center = self.center.ctypes.data_as(dp)
        d.face_area = self.area.ctypes.data_as(dp)
        d.cell_volume = self.volume.ctypes.data_as(dp)
        d.cell_center = self.cell_center.ctypes.data_as(dp)
        d.num_wall_faces = int(self.wall_faces.shape[0])
        d.wall_faces = self.wall_faces.ctypes.data_as(ip)
        d._keepalive = self  # the arrays must outlive the descriptor
        return d


def records_to_array(recs, n: int) -> np.ndarray:
    raw = np.frombuffer(C.string_at(C.addressof(recs), n * C.sizeof(IterRecord)), dtype=RECORD_DTYPE, count=n)
    return raw.copy()


def _f32(x: float) -> float:
    return float(np.float32(x))


# EulerAirfoilCaseConfig defaults (src/cfd_core/include/cfd_core/solvers/euler_solver.hpp:14-74),
# float fields widened to double, under the descriptor's field names; the fields with no
# reference counterpart (precision, ordering, block size, diagnostics, density target, cells
# per thread) take their neutral values.
REFERENCE_DEFAULTS = dict(
    gamma=_f32(1.4), gas_constant=_f32(287.05), mach=_f32(0.15), aoa_deg=_f32(2.0), p_inf=_f32(101325.0),
    t_inf=_f32(288.15), rho_inf=0.0, chord=1.0, x_ref=_f32(0.25), y_ref=0.0, flux=0, limiter=0,
    iterations=400, min_iterations=40, cfl_ramp_iters=120, cfl_start=_f32(0.2), cfl_max=_f32(1.2),
    residual_reduction_target=_f32(1.0e-3), force_stability_tol=_f32(2.0e-5), force_mean_drift_tol=_f32(2.0e-5),
    force_stability_window=6, startup_first_order_iters=25, rk_stages=3, local_time_stepping=1, precond_on=0,
    precond_mach_ref=_f32(0.15), precond_mach_min=_f32(1.0e-3), precond_beta_min=_f32(0.2), precond_beta_max=1.0,
    precond_farfield_bc=0, stab_floor_start=_f32(0.1), stab_floor_target=_f32(0.02), stab_floor_k_start=-1.0,
    stab_floor_k_target=-1.0, stab_ramp_iters=400, low_mach_fix=0, mach_cutoff=_f32(0.3), all_speed_flux_fix=0,
    all_speed_mach_cutoff=_f32(0.25), all_speed_f_min=_f32(0.05), all_speed_ramp_start_iter=0,
    all_speed_ramp_iters=0, all_speed_staged_controller=0, all_speed_stage_a_min_iters=600,
    all_speed_stage_a_max_iters=0, all_speed_stage_f_min_high=_f32(0.2), all_speed_stage_f_min_mid=_f32(0.1),
    all_speed_stage_f_min_low=_f32(0.05), all_speed_pjump_wall_target=0.0, all_speed_pjump_spike_factor=_f32(1.5),
    all_speed_pjump_hold_iters=120, all_speed_freeze_iters=120, all_speed_cfl_drop_factor=_f32(0.8),
    all_speed_cfl_restore_factor=_f32(1.02), all_speed_cfl_min_scale=_f32(0.1), aoa0_symmetry_enforce=0,
    aoa0_symmetry_enforce_interval=0, precision=0, ordering=0, block_size=0, diagnostics=0, density_l2_target=0.0,
    cells_per_thread=0, precond_fp64=0,
)


def make_case(**overrides) -> CaseDesc:
    """The reference defaults with overrides; real-valued settings rounded to float32 as the
    reference's case parser (std::stof) does."""
    values = dict(REFERENCE_DEFAULTS)
    for key, val in overrides.items():
        if key not in values:
            raise KeyError(f"unknown case field {key!r}")
        values[key] = _f32(val) if isinstance(values[key], float) else int(val)
    return case_desc(values)
