"""Build the in-tree CUDA library libsfgpu.so for sm_103a (nvcc, no cmake).

Translation units compile in parallel; the shared library lands in symforce_gb300/lib/ (git-ignored).
Rebuilds only when a source is newer than the library.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT_DIR = PKG / "lib"
BUILD_DIR = PKG / "_build"
LIB = OUT_DIR / "libsfgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["kernels_lin.cu", "kernels_lm.cu", "kernels_solve.cu", "kernels_pcg.cu",
                "kernels_mlp.cu", "kernels_batch.cu", "kernels_tc.cu", "api.cu", "api_solvers.cu", "api_noalloc.cu",
                "api_learned.cu", "api_batch.cu"]
HOST_SOURCES = ["host_structure.cpp", "host_layout.cpp", "host_pcg.cpp", "device_plan.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [CSRC / s for s in CUDA_SOURCES + HOST_SOURCES]


def _deps():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _sources() + _deps() + [Path(__file__)])


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        build_python_binding(verbose)
        return LIB
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", f"-I{INCLUDE}", f"-I{CSRC}"]

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.name + ".o")
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, *common, "-c", str(src), "-o", str(obj)]
        else:
            cmd = [nvcc, *common, "-x", "c++", "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt",
           "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_python_binding(verbose)
    return LIB


def python_binding_path() -> Path:
    import sysconfig
    return PKG / ("_cc_sym_gpu" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def build_python_binding(verbose: bool = False) -> Path:
    """The compiled cc_sym-shaped binding (csrc/py_cc_sym.cpp, CPython C API) next to the package,
    linked against lib/libsfgpu.so."""
    import sysconfig
    out = python_binding_path()
    src = CSRC / "py_cc_sym.cpp"
    if out.exists() and out.stat().st_mtime > max(src.stat().st_mtime, LIB.stat().st_mtime):
        return out
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for the Python binding")
    cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", f"-I{sysconfig.get_paths()['include']}", f"-I{INCLUDE}",
           str(src), f"-L{OUT_DIR}", "-lsfgpu", "-Wl,-rpath,$ORIGIN/lib", "-o", str(out) + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"binding build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr)
    os.replace(str(out) + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(force=True, verbose=True))
