"""Build libcnv.so in-tree for GB300 (sm_103a) with nvcc.

Every translation unit under csrc/ is compiled in parallel to an object in _build/, then
linked into libcnv.so beside this file. Host code is compiled with -ffp-contract=off so that
host-side constants (dx*dx*dy*dy, 2*(dx*dx+dy*dy), ...) round exactly as the reference's do on
every host, aarch64 included. Device code that must match the reference bit for bit uses the
round-to-nearest intrinsics, which nvcc never contracts.

Then the two host-only pieces on top of libcnv, with gcc:
    libcnv_compat.so   the reference's poisson*/euler entry points (compat/cnv_compat.c)
    cnavier_gpu        the reference program's command line and outputs (app/cnavier_gpu.c)
both linked against libcnv.so with rpath $ORIGIN.

    python fluid-dynamics1_gb300/build.py [--verbose-ptxas] [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcnv.so")
COMPAT_LIB = os.path.join(HERE, "libcnv_compat.so")
APP = os.path.join(HERE, "cnavier_gpu")
CC = os.environ.get("CC", "gcc")
CFLAGS = ["-O2", "-std=gnu99", "-fPIC", "-ffp-contract=off", "-I", os.path.join(HERE, "..", "include")]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(HERE, "..", "include")]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(HERE, "..", "include", "*.h")))


def _compile(src: str, verbose_ptxas: bool) -> tuple[str, str]:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [NVCC, *ARCH, *COMMON, "-lineinfo", "-c", src, "-o", obj]
    if src.endswith(".cu"):
        cmd[1:1] = ["-x", "cu"]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _host_parts(force: bool) -> None:
    """libcnv_compat.so and cnavier_gpu (gcc, linked against libcnv.so)."""
    link = ["-L", HERE, "-lcnv", "-Wl,-rpath,$ORIGIN", "-lm", "-lpthread"]
    jobs = [(os.path.join(HERE, "compat", "cnv_compat.c"), COMPAT_LIB, ["-shared"]),
            (os.path.join(HERE, "app", "cnavier_gpu.c"), APP, [])]
    for src, out, extra in jobs:
        newest = max(os.path.getmtime(p) for p in [src, LIB, __file__] + _headers())
        if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        tmp = out + ".tmp"
        r = subprocess.run([CC, *CFLAGS, *extra, src, "-o", tmp, *link], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"gcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, out)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile (if stale) and return the path of libcnv.so."""
    _build_lib(force, verbose_ptxas)
    _host_parts(force)
    return LIB


def _build_lib(force: bool, verbose_ptxas: bool) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    newest_input = max(os.path.getmtime(p) for p in srcs + _headers() + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest_input and not verbose_ptxas:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    if verbose_ptxas:
        for _, log in results:
            if log.strip():
                print(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--verbose-ptxas" in sys.argv))
