"""In-tree build of the CUDA library libfvm_gb300.so for sm_103a (nvcc only).

Translation units are compiled in parallel, then linked into
fvm_gb300/_build/libfvm_gb300.so.  Rebuilds only when a source is newer than the
library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfvm_gb300.so")
SOURCES = ["fvm_setup.cu", "fvm_step.cu", "fvm_mixed.cu", "fvm_resident.cu", "fvm_capi.cu", "fvm_static.cu",
           "fvm_batch.cu", "fvm_adjoint.cu", "fvm3d.cu", "fvm_post.cu"]
HEADERS = ["fvm_internal.cuh", "fvm_ops.cuh", "fvm_df.cuh", os.path.join("..", "..", "include", "fvm.h"),
           os.path.join("..", "..", "include", "fvm3d.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# FP32 subnormals flushed in the translation units whose FP32 arithmetic is the
# correction sweeps of the mixed path (far-field residuals reach the subnormal range,
# which measured slower); FP64 is unaffected, and fvm3d.cu keeps them for its
# double-float arithmetic.
FTZ_SOURCES = {"fvm_mixed.cu", "fvm_resident.cu", "fvm_adjoint.cu"}


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    hdrs = [os.path.join(CSRC, h) for h in HEADERS]
    if not force and not _stale(LIB, srcs + hdrs + [__file__]):
        return LIB
    nvcc = _nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, "-c", src, "-o", obj]
        if os.path.basename(src) in FTZ_SOURCES:
            cmd.insert(-4, "-ftz=true")
        if ptxas_v:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose or ptxas_v:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv))
