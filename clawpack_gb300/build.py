"""Build recipe for libgclaw.so (sm_103a).

    python -m clawpack_gb300.build

Produces, next to this file:
  libgclaw.so         the product library (nvcc default contraction of
                      multiply-adds into FMA)
  libgclaw_strict.so  the same sources with -fmad=false and GCLAW_STRICT:
                      every FP64 multiply and add rounded separately and every
                      quotient and square root taken as the reference writes
                      it, for bit-for-bit comparison with the CPU oracle in
                      the parity tests
Every (library, source) pair compiles to an object in parallel under
_build/, then each library is linked.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = [os.path.join(HERE, "csrc", n) for n in ("gclaw_step.cu", "gclaw_batch.cu",
                                                 "gclaw_adjoint.cu", "gclaw3.cu")]
BUILD_DIR = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


# -prec-div/-prec-sqrt/-ftz only change single-precision arithmetic (the
# FP32-bulk fluxes: approximate divide and square root, denormals flushed);
# the FP64 step is compiled with IEEE divide and square root either way.
FP32_FLAGS = ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]


def _compile_cmd(src, obj, extra):
    return [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            f"-I{INCLUDE}", *FP32_FLAGS, *extra, "-c", "-o", obj, src]


def targets():
    return [
        (os.path.join(HERE, "libgclaw.so"), []),
        (os.path.join(HERE, "libgclaw_strict.so"), ["-fmad=false", "-DGCLAW_STRICT"]),
    ]


def build(verbose=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    jobs = []
    for out, extra in targets():
        tag = os.path.splitext(os.path.basename(out))[0]
        for src in SRC:
            obj = os.path.join(BUILD_DIR, f"{tag}__{os.path.basename(src)}.o")
            jobs.append((src, obj, extra))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(lambda j: run(_compile_cmd(*j)), jobs))
    built = []
    for out, extra in targets():
        tag = os.path.splitext(os.path.basename(out))[0]
        objs = [os.path.join(BUILD_DIR, f"{tag}__{os.path.basename(src)}.o") for src in SRC]
        tmp = out + ".tmp"
        run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs])
        os.replace(tmp, out)
        built.append(out)
    return built


if __name__ == "__main__":
    for p in build(verbose="-v" in sys.argv):
        print("built", p)
