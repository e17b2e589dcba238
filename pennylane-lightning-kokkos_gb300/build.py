"""Build the GB300 state-vector core in-tree.

Produces, inside ``pennylane_lightning_kokkos/``:
  * ``libplk_gb300.so`` — the CUDA kernels and the C ABI declared in
    ``include/plk_gb300.h`` (nvcc, ``-gencode arch=compute_103a,code=sm_103a``);
  * ``lightning_kokkos_qubit_ops<EXT_SUFFIX>`` — the pybind11 module with the
    reference's class surface, linked against the library (pybind11 headers
    come from the installed PyTorch, so no extra package is needed).

Translation units compile in parallel; unchanged outputs are kept.  Usage:
``python pennylane-lightning-kokkos_gb300/build.py [--force] [--jobs N]``.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
PKG = os.path.join(HERE, "pennylane_lightning_kokkos")
OBJ = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

CUDA_SOURCES = ["state.cu", "gates.cu", "expval.cu", "measure.cu", "adjoint.cu", "noalloc.cu", "batch.cu", "windows.cu", "windows_df.cu", "windows_df_fwd.cu", "adjoint_kinds2.cu", "adjoint_kinds3.cu", "dense_tc.cu", "windows_sms.cu"]
BIND_SOURCES = ["bindings/Bindings.cpp"]
LIB_NAME = "libplk_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the GB300 core needs the CUDA toolkit")


def _headers(dirpath):
    out = []
    for d, _, files in os.walk(dirpath):
        out += [os.path.join(d, f) for f in files if f.endswith((".cuh", ".hpp", ".h"))]
    return out


def _stale(target, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _pybind_include() -> str:
    import torch  # PyTorch ships pybind11's headers

    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    if not os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
        raise RuntimeError("pybind11 headers not found under " + inc)
    return inc


def module_path() -> str:
    return os.path.join(PKG, "lightning_kokkos_qubit_ops" + sysconfig.get_config_var("EXT_SUFFIX"))


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> None:
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers(CSRC) + _headers(INCLUDE)
    common = ["-std=c++17", "-O3", "-I", INCLUDE, "-I", CSRC]
    cu_flags = common + ARCH + ["-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                                "-Xcompiler", "-fvisibility=hidden", "-Xptxas", "-warn-spills"]
    jobs = jobs or min(8, os.cpu_count() or 4)

    def compile_cu(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, os.path.splitext(os.path.basename(src))[0] + ".o")
        if force or _stale(o, [s] + hdrs):
            out = _run([nvcc, "-c", s, "-o", o] + cu_flags)
            if verbose and out.strip():
                print(out)
        return o

    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(compile_cu, CUDA_SOURCES))
    lib = os.path.join(PKG, LIB_NAME)
    if force or _stale(lib, objs):
        _run([nvcc, "-shared", "-o", lib] + objs + ARCH + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])

    # pybind11 module (host C++ only; talks to the library through the C ABI)
    mod = module_path()
    bind_src = [os.path.join(CSRC, b) for b in BIND_SOURCES]
    if force or _stale(mod, bind_src + hdrs + [lib]):
        py_inc = sysconfig.get_paths()["include"]
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-shared", "-fPIC", "-O2", "-std=c++17", "-fvisibility=hidden", "-I", INCLUDE, "-I", CSRC,
              "-I", _pybind_include(), "-I", py_inc] + bind_src +
             ["-o", mod, "-L", PKG, "-l:" + LIB_NAME, "-Wl,-rpath,$ORIGIN"])


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    build(force=a.force, jobs=a.jobs, verbose=a.verbose)
    print("built", os.path.join(PKG, LIB_NAME), "and", module_path())


if __name__ == "__main__":
    sys.exit(main())
