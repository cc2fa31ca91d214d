"""Drop-in for AeroCFD's ``cfd_core`` pybind11 module (src/cfd_core/bindings/pybind_module.cpp:9-38)
serving the ``cuda`` backend from libaero_gb300.so.

Same functions, argument meanings and result dict as the reference module:
    version() -> str, hello() -> str, cuda_available() -> bool,
    run_case(case_path, out_dir, backend="cpu") -> dict with keys
        status, backend, case_type, run_log, iterations, residual_l1, residual_l2,
        residual_linf, cl, cd, cm
and the sweep of the reference's python/cfd/sweep.py as one batched device run:
    run_sweep(sweep_path, jobs=1, backend="cpu", out_dir=None) -> dict
    run_case_sweep(case_path, out_dir, aoa_deg, backend="cpu", mach=None) -> list of dicts
``case_path`` is the flat key=value file written by python/cfd/case.py. Errors follow the
reference's exception types: std::invalid_argument surfaces as ValueError, other failures
as RuntimeError. backend="cpu" is the reference library's own CPU path and is rejected here.
"""

from __future__ import annotations

import ctypes as C

import aero_gb300


class _Summary(C.Structure):
    _fields_ = [("status", C.c_char * 16), ("backend", C.c_char * 16), ("case_type", C.c_char * 64),
                ("run_log", C.c_char * 1024), ("iterations", C.c_int),
                ("residual_l1", C.c_double), ("residual_l2", C.c_double), ("residual_linf", C.c_double),
                ("cl", C.c_double), ("cd", C.c_double), ("cm", C.c_double)]


def _lib():
    lib = aero_gb300.load()
    if not getattr(lib, "_driver_bound", False):
        lib.aero_run_case.restype = C.c_int
        lib.aero_run_case.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(_Summary)]
        lib.aero_driver_last_error.restype = C.c_char_p
        lib.aero_driver_last_error.argtypes = []
        lib._driver_bound = True
    return lib


def version() -> str:
    return "0.1.1"


def hello() -> str:
    return "cfd_core bindings ok"


def cuda_available() -> bool:
    return aero_gb300.cuda_available()


def run_case(case_path: str, out_dir: str, backend: str = "cpu") -> dict:
    lib = _lib()
    s = _Summary()
    rc = lib.aero_run_case(str(case_path).encode(), str(out_dir).encode(), str(backend).encode(), C.byref(s))
    if rc != 0:
        msg = lib.aero_driver_last_error().decode()
        if rc == 1:
            raise ValueError(msg)
        raise RuntimeError(msg)
    return _summary_dict(s)


def _sweep_lib():
    lib = _lib()
    if not getattr(lib, "_sweep_bound", False):
        lib.aero_run_sweep.restype = C.c_int
        lib.aero_run_sweep.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_char_p,
                                       C.c_char_p, C.POINTER(_Summary)]
        lib._sweep_bound = True
    return lib


def _summary_dict(s: _Summary) -> dict:
    return {
        "status": s.status.decode(), "backend": s.backend.decode(), "case_type": s.case_type.decode(),
        "run_log": s.run_log.decode(), "iterations": s.iterations, "residual_l1": s.residual_l1,
        "residual_l2": s.residual_l2, "residual_linf": s.residual_linf, "cl": s.cl, "cd": s.cd, "cm": s.cm,
    }


def run_case_sweep(case_path: str, out_dir: str, aoa_deg, backend: str = "cpu", mach=None) -> list[dict]:
    """The flat case file run at each angle of attack (and Mach number, when given), all cases
    in one batched device run; case k's outputs go to out_dir/run_kkk as run_case writes them.
    Returns the run_case dict of every case with its aoa_deg (and mach)."""
    lib = _sweep_lib()
    aoa = [float(a) for a in aoa_deg]
    n = len(aoa)
    if mach is not None and len(mach) != n:
        raise ValueError("mach must give one value per angle of attack")
    a = (C.c_double * max(n, 1))(*aoa)
    m = (C.c_double * n)(*[float(x) for x in mach]) if mach is not None else None
    out = (_Summary * max(n, 1))()
    rc = lib.aero_run_sweep(str(case_path).encode(), n, a, m, str(out_dir).encode(), str(backend).encode(), out)
    if rc != 0:
        msg = lib.aero_driver_last_error().decode()
        raise (ValueError if rc == 1 else RuntimeError)(msg)
    runs = []
    for k in range(n):
        d = _summary_dict(out[k])
        d["aoa_deg"] = aoa[k]
        if mach is not None:
            d["mach"] = float(mach[k])
        runs.append(d)
    return runs


def run_sweep(sweep_path: str, jobs: int = 1, backend: str = "cpu", out_dir: str | None = None) -> dict:
    """The reference's run_sweep (python/cfd/sweep.py:14-59) over a flat key=value sweep file:
    base_case = <flat case file, relative to the sweep file>, aoa_deg = <comma-separated
    angles> (default: the base case's), and optionally mach = <comma-separated Mach numbers>.
    The base case is resolved relative to the sweep file and that resolved file is what runs
    (the reference passes the unresolved YAML path to the native solver, sweep.py:51). All
    angles run as one batched device run instead of one after another; jobs is recorded
    only, as in the reference. Returns {status, jobs_requested, output_root, runs}."""
    from pathlib import Path

    sweep_file = Path(sweep_path)
    if not sweep_file.exists():
        raise FileNotFoundError(f"Sweep file not found: {sweep_file}")
    kv = {}
    for line in sweep_file.read_text().splitlines():
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        sep = "=" if "=" in line else ":"
        key, _, val = line.partition(sep)
        kv[key.strip()] = val.strip()
    if not kv.get("base_case"):
        raise ValueError("Sweep file must define 'base_case'.")
    base = (sweep_file.parent / kv["base_case"]).resolve()
    if "aoa_deg" in kv:
        aoa = [float(x) for x in kv["aoa_deg"].replace(" ", "").split(",") if x]
    else:
        case_kv = dict(line.split("=", 1) for line in base.read_text().splitlines() if "=" in line)
        aoa = [float(case_kv.get("aoa_deg", "0"))]
    mach = [float(x) for x in kv["mach"].replace(" ", "").split(",") if x] if "mach" in kv else None
    root = Path(out_dir) if out_dir is not None else sweep_file.parent / "sweep_output"
    runs = run_case_sweep(str(base), str(root), aoa, backend, mach)
    return {"status": "ok", "jobs_requested": int(jobs), "output_root": str(root), "runs": runs}
