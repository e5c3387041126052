"""GB300 microbenchmarks behind the factorization's design: FP64 latencies and issue limits,
the pivot reciprocal's accuracy, and the diagonal-tile LDL^T variants (tests/microbench/*.cu,
built here with nvcc for sm_103a).  Run with -s to see the tables; the assertions are the facts
the design relies on, with wide margins."""

from __future__ import annotations

import re
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent / "microbench"


def _run(name: str, tmp_path: Path) -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / name
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-o", str(exe),
                    str(HERE / f"{name}.cu")], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=300).stdout
    print(out)
    assert "status no error" in out
    return out


def _num(out: str, pattern: str) -> float:
    m = re.search(pattern, out)
    assert m, pattern
    return float(m.group(1))


def test_fp64_facts(tmp_path):
    out = _run("fp64_facts", tmp_path)
    # a dependent FP64 multiply-add costs tens of cycles per warp instruction
    assert _num(out, r"latency  32 thr fma\.f64\s+([\d.]+)") > 30
    # one warp cannot issue FP64 faster with independent chains ...
    assert _num(out, r"issue ILP4  1 warp\s+([\d.]+)") > 0.8 * _num(out, r"issue chain 1 warp\s+([\d.]+)")
    # ... and the limit of several warps is the SM's, not the sub-partition's
    two_one = _num(out, r"issue chain 2 warps, 1 sub-partition\s+([\d.]+)")
    assert two_one < 1.3 * _num(out, r"issue chain 2 warps, 2 sub-partitions\s+([\d.]+)")
    # the pivot reciprocal (approximation + two Newton steps) is exact to rounding
    assert _num(out, r"two Newton steps max rel err ([\d.e+-]+)") < 2.3e-16


def test_tile_ldlt_variants(tmp_path):
    out = _run("tile_ldlt", tmp_path)
    ff = _num(out, r"b=16 fraction-free, 1 barrier\s+grid\s+1:\s+([\d.]+)")
    rc = _num(out, r"b=16 reciprocal, 2 barriers\s+grid\s+1:\s+([\d.]+)")
    assert ff < rc
    cta = _num(out, r"b=32 CTA-wide, rcp\.approx\s+grid\s+1:\s+([\d.]+)")
    warp = _num(out, r"b=32 one warp, rows in registers\s+grid\s+1:\s+([\d.]+)")
    assert cta < warp
