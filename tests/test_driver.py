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


def _state_fns():
    lib = aero_gb300.load()
    lib.aero_state_write.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_double)]
    lib.aero_state_read.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_double)]
    lib.aero_driver_last_error.restype = C.c_char_p
    return lib


def test_state_file_round_trip_and_checks(tmp_path):
    lib = _state_fns()
    dp = C.POINTER(C.c_double)
    u = np.random.default_rng(3).standard_normal((37, 5))
    path = str(tmp_path / "s.state").encode()
    assert lib.aero_state_write(path, 37, u.ctypes.data_as(dp)) == 0
    v = np.empty_like(u)
    assert lib.aero_state_read(path, 37, v.ctypes.data_as(dp)) == 0
    np.testing.assert_array_equal(u, v)
    assert lib.aero_state_read(path, 36, v.ctypes.data_as(dp)) == capi.AERO_ERR_INVALID  # wrong mesh
    assert b"37 cells" in lib.aero_driver_last_error()
    raw = (tmp_path / "s.state").read_bytes()
    (tmp_path / "t.state").write_bytes(raw[:-8])
    assert lib.aero_state_read(str(tmp_path / "t.state").encode(), 37, v.ctypes.data_as(dp)) == capi.AERO_ERR_INVALID
    (tmp_path / "m.state").write_bytes(b"X" + raw[1:])
    assert lib.aero_state_read(str(tmp_path / "m.state").encode(), 37, v.ctypes.data_as(dp)) == capi.AERO_ERR_INVALID
    assert lib.aero_state_read(str(tmp_path / "none").encode(), 37, v.ctypes.data_as(dp)) == capi.AERO_ERR_INVALID


@pytest.mark.gpu
def test_run_case_rejects_unknown_vtu_format(tmp_path):
    p = write_cfg(tmp_path / "c.cfg", iterations=1, vtu_format="hdf5")
    with pytest.raises(ValueError):
        cfd_core.run_case(str(p), str(tmp_path / "o"), "cuda")


def _read_vtu_appended(path):
    """Arrays of a raw-appended VTU (UInt32 byte count before each array)."""
    import re

    blob = path.read_bytes()
    head, _, tail = blob.partition(b'<AppendedData encoding="raw">')
    data = tail[tail.index(b"_") + 1:]
    types = {"Float32": np.float32, "Int32": np.int32, "UInt8": np.uint8}
    out = {}
    for m in re.finditer(rb'<DataArray type="(\w+)"(?: Name="(\w+)")?[^>]*offset="(\d+)"', head):
        t, name, off = m.group(1).decode(), (m.group(2) or b"Points").decode(), int(m.group(3))
        nb = int(np.frombuffer(data[off:off + 4], np.uint32)[0])
        out[name] = np.frombuffer(data[off + 4:off + 4 + nb], types[t])
    return out


def _read_vtu_ascii(path):
    import re

    text = path.read_text()
    out = {}
    for m in re.finditer(r'<DataArray type="(\w+)"(?: Name="(\w+)")?[^>]*format="ascii">([^<]*)</DataArray>', text):
        out[m.group(2) or "Points"] = np.array(m.group(3).split(), dtype=np.float64)
    return out


@pytest.mark.gpu
def test_restart_dump_and_binary_vtu(tmp_path):
    base = dict(naca_code="0012", num_circumferential=48, num_radial=12, farfield_radius=12, radial_stretch=1.35,
                min_iterations=100, residual_reduction_target=1e-9, flux="hllc", limiter="venkat", precond="off",
                startup_first_order_iters=0, cfl_ramp_iters=0, cfl_start=0.8, cfl_max=0.8, mach=0.5, aoa_deg=2,
                precision="fp64")
    p1 = write_cfg(tmp_path / "a.cfg", iterations=30, restart_out="a.state", **base)
    cfd_core.run_case(str(p1), str(tmp_path / "a"), "cuda")
    assert (tmp_path / "a" / "a.state").exists()
    # restart_in replaces the free-stream start: 30 + 10 iterations from the dump follow the
    # state, so the first restarted residual continues the first run's history
    p2 = write_cfg(tmp_path / "b.cfg", iterations=10, restart_in="a/a.state", vtu_format="binary", **base)
    r2 = cfd_core.run_case(str(p2), str(tmp_path / "b"), "cuda")
    p3 = write_cfg(tmp_path / "c.cfg", iterations=10, **base)
    r3 = cfd_core.run_case(str(p3), str(tmp_path / "c"), "cuda")
    l2_a = [float(r["residual_l2"]) for r in csv.DictReader(open(tmp_path / "a" / "residuals.csv"))]
    l2_b = [float(r["residual_l2"]) for r in csv.DictReader(open(tmp_path / "b" / "residuals.csv"))]
    assert l2_b[0] < 0.9 * l2_a[0] and r2["residual_l2"] != r3["residual_l2"]
    # the binary VTU holds the same arrays as the ASCII one of the same state (ASCII carries
    # the reference writer's default 6 significant digits)
    p4 = write_cfg(tmp_path / "d.cfg", iterations=10, restart_in="a/a.state", **base)
    cfd_core.run_case(str(p4), str(tmp_path / "d"), "cuda")
    vb = _read_vtu_appended(tmp_path / "b" / "field_0000.vtu")
    va = _read_vtu_ascii(tmp_path / "d" / "field_0000.vtu")
    assert set(va) == set(vb) and len(va) == 10
    for k in va:
        np.testing.assert_allclose(vb[k].astype(np.float64), va[k], rtol=1e-5, atol=1e-12, err_msg=k)


SMALL = dict(naca_code="0012", num_circumferential=48, num_radial=12, farfield_radius=12, radial_stretch=1.35,
             min_iterations=40, residual_reduction_target=1e-9, flux="hllc", limiter="venkat", precond="off",
             startup_first_order_iters=10, cfl_ramp_iters=20, cfl_start=0.3, cfl_max=0.8, mach=0.5)


def _csv_text(path):
    return path.read_text()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sweep_writes_each_case_like_run_case(tmp_path, precision):
    """The batched sweep entry (python/cfd/sweep.py:14-59 as one batch) writes, for each angle,
    the files run_case writes for the case file at that angle: forces, residuals, diagnostics
    and Cp identical to the byte."""
    base = write_cfg(tmp_path / "base.cfg", iterations=40, aoa_deg=0.0, precision=precision, **SMALL)
    sweep = tmp_path / "sweep.cfg"
    sweep.write_text("base_case = base.cfg\naoa_deg = -2, 1.5, 4\n")
    res = cfd_core.run_sweep(str(sweep), jobs=3, backend="cuda", out_dir=str(tmp_path / "sw"))
    assert res["status"] == "ok" and res["jobs_requested"] == 3 and len(res["runs"]) == 3
    summary = list(csv.DictReader(open(tmp_path / "sw" / "sweep_summary.csv")))
    assert [float(r["aoa_deg"]) for r in summary] == [-2.0, 1.5, 4.0]
    for k, aoa in enumerate((-2.0, 1.5, 4.0)):
        single = write_cfg(tmp_path / f"single{k}.cfg", iterations=40, aoa_deg=aoa, precision=precision, **SMALL)
        one = cfd_core.run_case(str(single), str(tmp_path / f"one{k}"), "cuda")
        run = res["runs"][k]
        assert run["aoa_deg"] == aoa and run["iterations"] == one["iterations"]
        for key in ("cl", "cd", "cm", "residual_l2"):
            assert run[key] == one[key], key
        for f in ("forces.csv", "residuals.csv", "euler_diagnostics.csv", "cp_wall.csv", "wall_flux.csv"):
            assert _csv_text(tmp_path / "sw" / f"run_{k:03d}" / f) == _csv_text(tmp_path / f"one{k}" / f), f
        assert float(summary[k]["cl"]) == pytest.approx(one["cl"], rel=1e-6)
    # lift grows with incidence across the sweep
    assert res["runs"][0]["cl"] < res["runs"][1]["cl"] < res["runs"][2]["cl"]


@pytest.mark.gpu
def test_sweep_over_mach_numbers(tmp_path):
    base = write_cfg(tmp_path / "base.cfg", iterations=20, aoa_deg=2.0, precision="fp64", **SMALL)
    runs = cfd_core.run_case_sweep(str(base), str(tmp_path / "sw"), [2.0, 2.0], "cuda", mach=[0.3, 0.6])
    assert [r["mach"] for r in runs] == [0.3, 0.6]
    snap = dict(line.split("=", 1) for line in
                open(tmp_path / "sw" / "run_001" / "effective_config_snapshot.txt").read().split())
    assert float(snap["mach_inf"]) == pytest.approx(0.6)
    with pytest.raises(ValueError):
        cfd_core.run_case_sweep(str(base), str(tmp_path / "x"), [1.0, 2.0], "cuda", mach=[0.3])


@pytest.mark.gpu
def test_run_case_outputs_match_the_oracle(tmp_path):
    """forces.csv, residuals.csv and cp_wall.csv of an FP64 run_case against the FP64 oracle's
    run of the same case on the same mesh (run_euler_airfoil_case, euler_solver.cpp:1161-1175,
    and extract_wall_cp, forces.cpp:177-206). The files hold the reference writer's float
    values at its default 6 significant digits."""
    from oracle import oracle_py as op

    op.build()
    p = write_cfg(tmp_path / "c.cfg", iterations=60, aoa_deg=2.0, precision="fp64", **SMALL)
    out = tmp_path / "out"
    cfd_core.run_case(str(p), str(out), "cuda")
    case, mcfg, _ = parse(p)
    case.diagnostics = 1
    mesh = aero_gb300.ogrid_reference(mcfg.naca_code.decode(), mcfg.num_circumferential, mcfg.num_radial,
                                      mcfg.farfield_radius, mcfg.radial_stretch, mcfg.chord)
    o = op.OracleSolver(op.MODE_DOUBLE, mesh, case)
    _, orec = o.run(case.iterations)
    frows = list(csv.DictReader(open(out / "forces.csv")))
    rrows = list(csv.DictReader(open(out / "residuals.csv")))
    assert len(frows) == len(rrows) == len(orec)
    for key in ("cl", "cd", "cm"):
        got = np.array([float(r[key]) for r in frows])
        np.testing.assert_allclose(got, orec[key], rtol=1e-5, atol=1e-7, err_msg=key)
    for key in ("residual_l1", "residual_l2", "residual_linf"):
        got = np.array([float(r[key]) for r in rrows])
        np.testing.assert_allclose(got, orec[key], rtol=1e-5, err_msg=key)
    # wall Cp of the final state, matched to the wall faces by their centres
    u = o.get_state()
    g = case.gamma
    rho = u[:, 0]
    pres = (g - 1.0) * (u[:, 4] - 0.5 * (u[:, 1] ** 2 + u[:, 2] ** 2) / rho)
    rho_inf = case.p_inf / (case.gas_constant * case.t_inf)
    v_inf = case.mach * np.sqrt(g * case.p_inf / rho_inf)
    q_inf = 0.5 * rho_inf * v_inf * v_inf + 1e-12
    wall = mesh.wall_faces
    centres = mesh.center.reshape(-1, 3)[wall, :2]
    want = (pres[mesh.owner[wall]] - case.p_inf) / q_inf
    cp = list(csv.DictReader(open(out / "cp_wall.csv")))
    assert len(cp) == len(wall)
    seen = set()
    for r in cp:  # the file's centres carry 6 significant digits: take the nearest wall face
        d = np.hypot(centres[:, 0] - float(r["x"]), centres[:, 1] - float(r["y"]))
        k = int(np.argmin(d))
        assert d[k] < 1e-5 and k not in seen
        seen.add(k)
        assert float(r["Cp"]) == pytest.approx(want[k], rel=1e-5, abs=1e-6)
