"""Builds libsst_gb300.so (the C-ABI CUDA library) in-tree for sm_103a.

Each translation unit is compiled by its own nvcc process (in parallel), then
linked into ``serstacker_gb300/_build/libsst_gb300.so``. No cmake, no
host-architecture flags: the same command builds on x86_64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsst_gb300.so")
SOURCES = ["sst_capi.cu", "sst_ecc.cu", "sst_pyramid.cu", "sst_stack.cu", "sst_noalloc.cu", "sst_bayer.cu", "sst_replicas.cu", "sst_roi.cu", "sst_flow.cu", "sst_adjoint.cu", "sst_weights.cu", "sst_inpaint.cu", "sst_calib.cu", "sst_registration.cu", "sst_lpg.cu", "sst_accum.cu", "sst_focus.cu", "sst_ser.cpp"]
HEADERS = ["sst_internal.cuh", "sst_model.cuh", "sst_engine.cuh", "sst_stack.cuh", "sst_host.h", "sst_kernels.cuh", "sst_tma.cuh", "sst_taps.h", "sst_resample.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "serstacker_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA source for sm_103a and link the shared library."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        cmd = [cc, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"{src}:\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcufft", "-lcudart"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
