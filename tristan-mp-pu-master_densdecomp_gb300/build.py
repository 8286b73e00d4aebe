"""Build recipe for libtristan_gpu.so (the C-ABI library), in-tree.

nvcc compiles every csrc/*.cu for sm_103a only, in parallel, with
-fmad=false (no FMA contraction) and IEEE division / square root so the
kernels round exactly like the reference's single-precision arithmetic,
then links one shared library into lib/. No cmake, no torch extension.
"""
from __future__ import annotations

import glob
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(LIBDIR, "libtristan_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
           "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off",
           "-I", INCLUDE]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    # objects built on another host architecture are never reused
    stamp = os.path.join(LIBDIR, "host_arch")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        for f in glob.glob(os.path.join(OBJDIR, "*.o")) + [LIB]:
            if os.path.exists(f):
                os.remove(f)
        with open(stamp, "w") as fh:
            fh.write(arch + "\n")
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")) + [__file__]
    cc = nvcc()
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(OBJDIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            extra = os.environ.get("TG_NVCC_EXTRA", "").split()
            cmd = [cc] + ARCH + NVFLAGS + extra + (["-Xptxas", "-v"] if ptxas_v else []) + ["-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_v or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if jobs or not os.path.exists(LIB):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_v="-v" in sys.argv))
