"""Build recipe for libgclaw.so (sm_103a).

    python -m clawpack_gb300.build

Produces, next to this file:
  libgclaw.so         the product library (nvcc default contraction of
                      multiply-adds into FMA)
  libgclaw_strict.so  the same sources with -fmad=false: every FP64 multiply
                      and add rounded separately, for bit-for-bit comparison
                      with the CPU oracle in the parity tests
Both builds run in parallel; each is one translation unit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = [os.path.join(HERE, "csrc", "gclaw_step.cu")]
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


def _cmd(out, extra):
    return [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
            f"-I{INCLUDE}", *FP32_FLAGS, *extra, "-o", out, *SRC]


def targets():
    return [
        (os.path.join(HERE, "libgclaw.so"), []),
        (os.path.join(HERE, "libgclaw_strict.so"), ["-fmad=false"]),
    ]


def build(verbose=False):
    jobs = targets()

    def run(job):
        out, extra = job
        tmp = out + ".tmp"
        cmd = _cmd(tmp, extra)
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {out}:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, out)
        return out

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        return list(ex.map(run, jobs))


if __name__ == "__main__":
    for p in build(verbose="-v" in sys.argv):
        print("built", p)
