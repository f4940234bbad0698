"""Builds libsdfcontact.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each translation unit is compiled in parallel with nvcc, then linked into
``_build/libsdfcontact.so`` next to this file.  Sources are the ``csrc/*.cu``
files; the public header is ``include/sdfc.h`` at the repository root.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsdfcontact.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsdfcontact")


def _flags():
    f = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                "-I", CSRC]
    # force_kernel's resident CTAs per SM on the FP32 path (a tuning knob; see sdfc_kernels.cuh)
    mb = os.environ.get("SDFC_FORCE_MIN_BLOCKS")
    if mb:
        f.append(f"-DSDFC_FORCE_MIN_BLOCKS={int(mb)}")
    # further compile-time variants, e.g. SDFC_DEFINES="SDFC_COLD=inline" (measurement only)
    for d in os.environ.get("SDFC_DEFINES", "").split():
        f.append("-D" + d)
    return f


# Per-file flags.  The level-set builder reproduces the reference's FP32 distances bit for bit;
# the reference is compiled without contraction, so no multiply-add may be fused there.  (The
# batched evaluation keeps IEEE FP32 divides and square roots: the hardware's approximate forms
# made its force pass 4.5% faster, but the simulations' Newton iterations, which run to |g| <
# 1e-8 on stiff contacts, then needed up to 53% more evaluations.)
FILE_FLAGS = {"sdfc_levelset.cu": ["-fmad=false"]}


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        # (this file too: its flags are part of every object)
        if force or _stale(o, [s] + headers + [os.path.abspath(__file__)]):
            jobs.append([nvcc()] + _flags() + FILE_FLAGS.get(os.path.basename(s), []) + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
