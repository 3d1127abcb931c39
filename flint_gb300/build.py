"""Build the in-tree CUDA library flint_gb300/_lib/libflint_gb300.so for sm_103a.

nvcc compiles the translation units in parallel and links one shared object
with only the CUDA runtime; no torch symbol is involved.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["flint_abi.cu", "flint_kernels.cu", "flint_reactor.cu", "flint_table.cu", "flint_mlp.cu",
           "flint_surrogate.cu", "flint_files.cu", "flint_ir.cu", "flint_umma.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-v"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build_all(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    objs = []
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "flint_gpu.h")]
    newest_dep = max(os.path.getmtime(d) for d in deps)

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
            return obj, ""
        cmd = [nvcc, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    for obj, log in results:
        objs.append(obj)
        if verbose and log:
            sys.stderr.write(log)
    so = os.path.join(OUT, "libflint_gb300.so")
    if not os.path.exists(so) or any(os.path.getmtime(o) > os.path.getmtime(so) for o in objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", so, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return so


if __name__ == "__main__":
    print(build_all(verbose=True))
