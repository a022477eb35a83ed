"""Build the GB300 MAC-projection library (CUDA, sm_103a) in-tree.

Compiles every ``csrc/*.cu`` translation unit with nvcc for ``sm_103a`` in parallel and links
``maestro_gb300/_lib/libmaestro_mac.so`` (C ABI declared in ``include/maestro_mac.h``).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libmaestro_mac.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                   "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
                   *extra]


def _needs(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(ROOT, "include", "maestro_mac.h")]
    exe = nvcc()
    jobs = []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        if force or _needs(o, [s] + hdrs):
            extra = ["-Xptxas", "-v"] if ptxas_verbose else []
            jobs.append((s, o, [exe, *_flags(extra), "-c", s, "-o", o]))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): (s, o) for s, o, cmd in jobs}
        for fu in cf.as_completed(futs):
            r = fu.result()
            s, _ = futs[fu]
            logs.append((s, r.stdout + r.stderr))
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {s}:\n{r.stdout}{r.stderr}")
    if verbose or ptxas_verbose:
        for s, log in logs:
            if log.strip():
                print(f"== {os.path.basename(s)}\n{log}", file=sys.stderr)
    objs = [os.path.join(OBJ, os.path.basename(s)[:-3] + ".o") for s in srcs]
    if force or jobs or _needs(LIB, objs):
        cmd = [exe, *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
