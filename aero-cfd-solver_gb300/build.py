"""Build libaero_gb300.so in-tree (aero-cfd-solver_gb300/lib/).

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), host C++ with g++ -std=c++20; the objects
are compiled in parallel and linked by nvcc with the static CUDA runtime.

    python aero-cfd-solver_gb300/build.py [--ptxas-v] [--force]
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "lib" / "libaero_gb300.so"

CU_SOURCES = ["engine_f32.cu", "engine_f64.cu", "noalloc.cu"]
# Float division and square root by the hardware approximations (at most 2 ulp) in the units
# holding FP32 kernels: the FP32 residual stays within twice the reference float path's own
# deviation from FP64 either way, and the correctly rounded sequences cost the face pass
# about a tenth of its time. Float subnormals (below 1.2e-38) flush to zero there: the
# solver's floored densities, pressures and wave speeds never come near them, and the square
# roots and quotients then skip their subnormal scaling (face pass 12.7 -> 11.6 us at 131k
# cells). Double arithmetic is unaffected by these flags.
FAST_FLOAT_DIV_SQRT = ("engine_f32.cu", "noalloc.cu")
CPP_SOURCES = ["capi.cpp", "mesh_prep.cpp", "mesh_gen.cpp", "driver.cpp", "graph_profile.cpp"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _deps_mtime() -> float:
    files = list(CSRC.glob("*")) + list((REPO / "include").glob("*.h")) + [Path(__file__)]
    return max(f.stat().st_mtime for f in files if f.is_file())


def _run(cmd: list[str]) -> tuple[list[str], subprocess.CompletedProcess]:
    return cmd, subprocess.run(cmd, capture_output=True, text=True)


def build(force: bool = False, ptxas_v: bool = False, verbose: bool = False) -> Path:
    cuda = cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    OBJ.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    deps = _deps_mtime()
    if not force and LIB.exists() and LIB.stat().st_mtime > deps:
        return LIB
    inc = [f"-I{REPO / 'include'}", f"-I{CSRC}", f"-I{cuda / 'include'}"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = OBJ / (src + ".o")
        objs.append(obj)
        cmd = [nvcc, GENCODE, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", *inc,
               "-c", str(CSRC / src), "-o", str(obj)]
        if ptxas_v:
            cmd.insert(3, "-Xptxas=-v")
        if src in FAST_FLOAT_DIV_SQRT:
            cmd[3:3] = ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
        cmd[3:3] = os.environ.get("AERO_NVCC_FLAGS", "").split()  # extra nvcc flags (experiments)
        jobs.append(cmd)
    for src in CPP_SOURCES:
        obj = OBJ / (src + ".o")
        objs.append(obj)
        jobs.append(["g++", "-std=c++20", "-O2", "-fPIC", "-fvisibility=hidden", "-Wall",
                     "-ffp-contract=off", *inc, "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(_run, jobs))
    failed = False
    for cmd, res in results:
        if verbose or ptxas_v or res.returncode != 0:
            sys.stderr.write(res.stdout + res.stderr)
        if res.returncode != 0:
            sys.stderr.write("FAILED: " + " ".join(cmd) + "\n")
            failed = True
    if failed:
        raise RuntimeError("libaero_gb300 compilation failed")
    tmp = LIB.with_suffix(".so.tmp")
    link = [nvcc, GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fPIC", "-ldl"]
    _, res = _run(link)
    if res.returncode != 0:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError("libaero_gb300 link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-v", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, ptxas_v=a.ptxas_v, verbose=a.verbose))
