"""Drop-in for AeroCFD's ``cfd_core`` pybind11 module (src/cfd_core/bindings/pybind_module.cpp:9-38)
serving the ``cuda`` backend from libaero_gb300.so.

Same functions, argument meanings and result dict as the reference module:
    version() -> str, hello() -> str, cuda_available() -> bool,
    run_case(case_path, out_dir, backend="cpu") -> dict with keys
        status, backend, case_type, run_log, iterations, residual_l1, residual_l2,
        residual_linf, cl, cd, cm
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
    return {
        "status": s.status.decode(), "backend": s.backend.decode(), "case_type": s.case_type.decode(),
        "run_log": s.run_log.decode(), "iterations": s.iterations, "residual_l1": s.residual_l1,
        "residual_l2": s.residual_l2, "residual_linf": s.residual_linf, "cl": s.cl, "cd": s.cd, "cm": s.cm,
    }
