"""Host-side checks of the GPU library that run without a GPU: it builds, loads, exports every
symbol include/sfgpu.h declares, reports the reference defaults, and refuses to run without a
device (there is no CPU fallback)."""

from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from symforce_gb300 import _build
from symforce_gb300 import _cabi as A
from symforce_gb300 import synth

ROOT = Path(__file__).resolve().parents[1]


def _lib():
    return C.CDLL(str(_build.build()))


def _gpu_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_exports_every_declared_symbol():
    header = (ROOT / "include" / "sfgpu.h").read_text()
    declared = set(re.findall(r"\b(sfg_[a-z_]+)\s*\(", header))
    out = subprocess.run(["nm", "-D", "--defined-only", str(_build.build())], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert declared, "no declarations parsed"
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    L = _lib()
    for name in declared:
        getattr(L, name)


def test_default_params_match_reference():
    L = _lib()
    p = A.OptimizerParams()
    L.sfg_default_optimizer_params(C.byref(p))
    ref = A.default_optimizer_params()
    for f, _ in A.OptimizerParams._fields_:
        assert getattr(p, f) == getattr(ref, f), f
    assert L.sfg_abi_version() == 3
    f = A.FormParams()
    L.sfg_default_form_params(C.byref(f))
    for k, _ in A.FormParams._fields_:
        assert getattr(f, k) == getattr(A.default_form_params(), k), k


def test_dims_tables():
    L = _lib()
    s, t = C.c_int32(), C.c_int32()
    for kt, (sd, td) in A.KEY_DIMS.items():
        assert L.sfg_key_dims(kt, C.byref(s), C.byref(t)) == 0
        assert (s.value, t.value) == (sd, td)
    nk, nc, rd = C.c_int32(), C.c_int32(), C.c_int32()
    for kind, (k, c, r, _) in A.FACTOR_DIMS.items():
        assert L.sfg_factor_dims(kind, C.byref(nk), C.byref(nc), C.byref(rd)) == 0
        assert (nk.value, nc.value, rd.value) == (k, c, r)
    assert L.sfg_factor_dims(99, None, None, None) == 1


@pytest.mark.skipif(_gpu_present(), reason="checks the no-device path")
def test_create_without_device_fails_loudly():
    from symforce_gb300.optimizer import Optimizer, SfgError
    p = synth.bundle_adjustment(num_cameras=4, num_points=20, num_observations=80, seed=0)
    with pytest.raises(SfgError) as e:
        Optimizer(p)
    assert e.value.code == 3  # SFG_ERR_NO_DEVICE


def test_graft_entry_build_imports():
    import __graft_entry__ as g
    g.build()


def test_csc_lower_to_dense_matches_scipy():
    """The DenseLinearizer adapter's conversion of the exported CSC hessian_lower."""
    sparse = pytest.importorskip("scipy.sparse")
    from symforce_gb300.optimizer import csc_lower_to_dense

    M = sparse.random(40, 40, density=0.2, random_state=1, format="csc")
    L = sparse.tril(M + M.T + sparse.eye(40), format="csc")
    L.sort_indices()
    H = csc_lower_to_dense(L.indptr, L.indices, L.data, 40)
    np.testing.assert_array_equal(H, L.toarray())
    assert np.count_nonzero(np.triu(H, 1)) == 0


def _build_cpp_driver(out_dir: Path) -> Path:
    """Compile tests/cpp/adapter_driver.cpp (the C++ adapters of include/sfgpu_sym.h over the
    Eigen / SymForce stand-ins) and link it against the in-tree libsfgpu.so."""
    import shutil
    import subprocess
    from symforce_gb300 import _build
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ is not available")
    lib = _build.build()
    exe = out_dir / "adapter_driver"
    subprocess.run([gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'tests' / 'cpp'}",
                    f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "adapter_driver.cpp"),
                    f"-L{lib.parent}", "-lsfgpu", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    return exe


def test_cpp_adapters_compile_and_link(tmp_path):
    """The header-only drop-ins for SymForce's plug points (GpuSparseCholeskySolver,
    GpuSparseSchurSolver, GpuLevenbergMarquardtSolver) compile warning-free against the interfaces
    they use and link against the C ABI; without a GPU the driver fails loudly, never falls back."""
    import subprocess
    exe = _build_cpp_driver(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, env={"CUDA_VISIBLE_DEVICES": ""})
    assert r.returncode != 0
    assert "no CUDA device" in r.stderr + r.stdout


def test_cc_sym_binding_builds_and_fails_loudly_without_device():
    """The compiled cc_sym-shaped binding (symforce/pybind/cc_optimizer.cc:29-170) imports, reports
    DefaultOptimizerParams, and refuses to construct an Optimizer without a GPU."""
    from symforce_gb300 import cc_sym
    d = cc_sym.default_optimizer_params()
    p = A.default_optimizer_params()
    for k, v in d.items():
        assert getattr(p, k) == pytest.approx(v), k
    prob = synth.robot_2d(num_poses=20, num_landmarks=5, seed=1)
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(RuntimeError, match="sfgpu error 3"):
        cc_sym.Optimizer(d, prob)
