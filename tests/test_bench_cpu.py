"""bench.py's contract on the CPU: the reference arm's JSON line (the oracle float port timed
on host cores), the algorithmic-byte model the roofline divides by, and the warm-up rule."""

import argparse
import json
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO))

import bench  # noqa: E402


def test_face_pass_algorithmic_bytes():
    # W and gradients of every cell (12 floats) + per face cell ids, normal, length, offsets
    # (8 B + 7 floats) and the F*A and wave-speed outputs (5 floats)
    assert bench.algorithmic_bytes("face", 131072, 3, "fp32", 197120) == 131072 * 48 + 197120 * 56 == 17330176
    assert bench.algorithmic_bytes("face", 131072, 3, "fp64", 197120) == 131072 * 96 + 197120 * 104


def test_warmup_below_three_is_refused():
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--warmup", "2"],
                       capture_output=True, text=True, cwd=REPO)
    assert r.returncode != 0 and "warmup" in r.stderr


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "3",
                        "--cpu-procs", "2"], capture_output=True, text=True, cwd=REPO, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["metric"] == bench.METRIC and line["unit"] == "Mcell-iter/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 3 and line["vs_baseline"] is None
    # the same config object as the GPU arm's line: the workload, L2 treatment and replication
    assert line["config"] == bench.workload_config(argparse.Namespace(mesh=None, no_flush=False), 2 * 512 * 128,
                                                   512 * (3 * 128 + 1), 1)
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 2 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


_PROBE = r"""
import sys, queue
sys.path.insert(0, {repo!r})
import bench
from oracle import oracle_py as op
q = queue.Queue()
bench._cpu_worker(dict(bench.WORKLOAD, n_circ=32, n_radial=8), dict(bench.CASE, startup_first_order_iters=0),
                  1, 1, None, q)
assert q.get() > 0
maps = open("/proc/self/maps").read()
print("PRODUCT_IMPORTED" if any(m.startswith("aero_gb300") for m in sys.modules) else "NO_PRODUCT_IMPORT")
print("PRODUCT_MAPPED" if "libaero_gb300" in maps else "NO_PRODUCT_MAPPED")
print("ORACLE_MAPPED" if "liboracle" in maps else "NO_ORACLE")
"""


def test_reference_arm_worker_neither_imports_nor_maps_the_product():
    """The reference arm's replicas build their mesh with the oracle's own generator and run
    the oracle: no module of the product package is imported and libaero_gb300.so is never
    mapped into the process."""
    r = subprocess.run([sys.executable, "-c", _PROBE.format(repo=str(REPO))], capture_output=True, text=True,
                       cwd=REPO, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.split()
    assert "NO_PRODUCT_IMPORT" in out and "NO_PRODUCT_MAPPED" in out and "ORACLE_MAPPED" in out


def test_reference_arm_reports_the_gpu_arm_workload():
    class A:
        mesh = None
        no_flush = False

    cfg = bench.workload_config(A(), 131072, 197120, 1)
    assert cfg == {"workload": cfg["workload"], "cells": 131072, "faces": 197120,
                   "l2": "flushed before every timed iteration (256 MiB write)", "parallelism": "replicas x1"}
    assert "512x128" in cfg["workload"] and "HLLC+MUSCL venkat" in cfg["workload"]
