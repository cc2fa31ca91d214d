"""Case-level drop-in: the key=value case file, backend normalisation, and (on a GPU) a full
run_case through the cfd_core mirror with the reference's output files."""

import csv
import ctypes as C

import numpy as np
import pytest

import aero_gb300
import cfd_core
from aero_gb300 import capi


class MeshCfg(C.Structure):
    _fields_ = [("naca_code", C.c_char * 16), ("num_circumferential", C.c_int), ("num_radial", C.c_int),
                ("farfield_radius", C.c_double), ("radial_stretch", C.c_double), ("chord", C.c_double)]


def write_cfg(path, **kv):
    lines = ["case_type=euler_airfoil_2d"] + [f"{k}={v}" for k, v in kv.items()]
    path.write_text("\n".join(lines) + "\n")
    return path


def parse(path):
    lib = aero_gb300.load()
    lib.aero_parse_case.argtypes = [C.c_char_p, C.POINTER(capi.CaseDesc), C.POINTER(MeshCfg), C.c_char_p, C.c_int]
    c, m, t = capi.CaseDesc(), MeshCfg(), C.create_string_buffer(64)
    assert lib.aero_parse_case(str(path).encode(), C.byref(c), C.byref(m), t, 64) == 0
    return c, m, t.value.decode()


def test_parse_case_maps_reference_keys(tmp_path):
    p = write_cfg(tmp_path / "native_case.cfg", num_circumferential=72, num_radial=18, farfield_radius=12,
                  radial_stretch=1.35, mach=0.15, aoa_deg=2, iterations=80, flux="HLLC", limiter="venkat",
                  local_time_stepping="off", low_mach_fix="on", mach_ref=0.2, all_speed_f_min=0)
    c, m, t = parse(p)
    assert t == "euler_airfoil_2d"
    assert (m.num_circumferential, m.num_radial) == (72, 18)
    assert m.farfield_radius == np.float32(12.0) and m.radial_stretch == float(np.float32(1.35))
    assert c.mach == float(np.float32(0.15)) and c.iterations == 80
    assert c.flux == capi.FLUX_HLLC and c.limiter == capi.LIMITER_VENKAT and c.local_time_stepping == 0
    # precond follows low_mach_fix when no precond key is given (residual_stub.cpp:438-450)
    assert c.low_mach_fix == 1 and c.precond_on == 1
    assert c.precond_mach_ref == float(np.float32(0.2))  # mach_ref alias
    assert c.all_speed_f_min == float(np.float32(0.05))  # non-positive -> 0.05
    assert c.precision == capi.PRECISION_FP32


def test_parse_case_colon_separator_and_comments(tmp_path):
    p = tmp_path / "c.cfg"
    p.write_text("# comment\ncase_type: euler_airfoil_2d\n  mach :  0.5 \nprecond=off\nlow_mach_fix=on\nprecision=fp64\n")
    c, _, t = parse(p)
    assert t == "euler_airfoil_2d" and c.mach == float(np.float32(0.5))
    assert c.precond_on == 0 and c.low_mach_fix == 1 and c.precision == capi.PRECISION_FP64


def test_backend_normalisation_errors(tmp_path):
    p = write_cfg(tmp_path / "c.cfg", iterations=1)
    with pytest.raises(ValueError):
        cfd_core.run_case(str(p), str(tmp_path / "out"), "metal")
    with pytest.raises(ValueError):
        cfd_core.run_case(str(p), str(tmp_path / "out"), "CPU")  # the CPU path is the reference's
    if not cfd_core.cuda_available():
        with pytest.raises(RuntimeError):
            cfd_core.run_case(str(p), str(tmp_path / "out"), "cuda")


@pytest.mark.gpu
def test_run_case_cuda_writes_reference_outputs(tmp_path, golden_histories):
    data, meta = golden_histories
    # the regression case of tests/cpp/test_euler_regression.cpp:9-30
    p = write_cfg(tmp_path / "native_case.cfg", naca_code="0012", num_circumferential=72, num_radial=18,
                  farfield_radius=12, radial_stretch=1.35, iterations=80, min_iterations=20, cfl_start=0.15,
                  cfl_max=0.7, cfl_ramp_iters=80, residual_reduction_target=0.01, force_stability_tol=0.0005,
                  force_stability_window=6, flux="rusanov", limiter="minmod", precond="off",
                  startup_first_order_iters=25, mach=0.15, aoa_deg=2)
    out = tmp_path / "out"
    res = cfd_core.run_case(str(p), str(out), "cuda")
    assert res["status"] == "ok" and res["backend"] == "cuda" and res["case_type"] == "euler_airfoil_2d"
    assert set(res) == {"status", "backend", "case_type", "run_log", "iterations", "residual_l1", "residual_l2",
                        "residual_linf", "cl", "cd", "cm"}
    for f in ("residuals.csv", "forces.csv", "euler_diagnostics.csv", "cp_wall.csv", "wall_flux.csv",
              "dissipation_debug.csv", "boundary_faces_debug.txt", "effective_config_snapshot.txt",
              "field_0000.vtu", "run.log"):
        assert (out / f).exists(), f
    rows = list(csv.DictReader(open(out / "residuals.csv")))
    assert list(rows[0]) == ["iter", "residual_l1", "residual_l2", "residual_linf", "residual_ratio"]
    frows = list(csv.DictReader(open(out / "forces.csv")))
    assert len(frows) == res["iterations"] == len(rows)
    ref = data["regression/history"]
    assert len(rows) == len(ref)
    cl = np.array([float(r["cl"]) for r in frows])
    assert np.max(np.abs(cl - ref[:, 4])) < 1e-3
    assert 0.16 <= res["cl"] <= 0.30
    cp = list(csv.DictReader(open(out / "cp_wall.csv")))
    assert len(cp) == 72 and list(cp[0]) == ["s", "x", "y", "Cp"]
    drow = list(csv.DictReader(open(out / "euler_diagnostics.csv")))
    assert len(drow[0]) == 64 and None not in drow[0]  # header and rows both have 64 columns
    log = dict(line.split("=", 1) for line in open(out / "run.log").read().splitlines()[1:] if "=" in line)
    assert log["backend"] == "cuda" and int(log["num_cells"]) == 2 * 72 * 18
