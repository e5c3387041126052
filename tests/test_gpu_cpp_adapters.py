"""The compiled C++ drop-ins for SymForce's plug points (include/sfgpu_sym.h) on the GPU: the
driver tests/cpp/adapter_driver.cpp runs GpuSparseCholeskySolver (LinearSolver concept: solve
residual and L D L^T == P A P^T), GpuSparseSchurSolver, and GpuLevenbergMarquardtSolver driven the
way sym::Optimizer drives a NonlinearSolverType on the reference's robot_2d example (9 records,
initial error 6.39636, best below 2.2003e-4, SUCCESS, pose at 1e-6), plus ComputeCovariance."""

from __future__ import annotations

import subprocess

import pytest

from test_library_cpu import _build_cpp_driver

pytestmark = pytest.mark.gpu


def test_cpp_adapters_on_gpu(tmp_path):
    exe = _build_cpp_driver(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout
