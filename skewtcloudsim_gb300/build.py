"""Build libskewt_gb300.so in-tree with nvcc for sm_103a, and the skt_run driver over it.

The translation units are compiled in parallel, then linked with ``nvcc -shared`` (static
cudart). Output: ``skewtcloudsim_gb300/_build/libskewt_gb300.so`` and
``skewtcloudsim_gb300/_build/skt_run`` (host C++ against the C ABI and the C++ adapter).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libskewt_gb300.so")
DRIVER = os.path.join(BUILD, "skt_run")
ROOT = os.path.dirname(HERE)

SOURCES = ["skt_api.cu", "skt_stencil.cu", "skt_project.cu", "skt_micro.cu", "skt_mg.cu", "skt_edit.cu",
           "skt_sounding.cu", "skt_export.cu", "skt_tune.cu"]
# host arithmetic that must round like the reference's (no fused multiply-add contraction)
PER_SOURCE = {"skt_sounding.cu": ["-Xcompiler", "-ffp-contract=off"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "skewt.h")]
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    nv = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nv, *ARCH, *NVCC_FLAGS, *PER_SOURCE.get(src, []), *extra_flags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_driver(force: bool = False) -> str:
    """skt_run: g++ over csrc/skt_run.cpp, linked against the library (rpath: its own folder)."""
    lib = build()
    src = os.path.join(CSRC, "skt_run.cpp")
    hdrs = [os.path.join(ROOT, "include", h) for h in ("skewt.h", "skewt_env.hpp")]
    if not force and os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= max(os.path.getmtime(f) for f in [src, lib, *hdrs]):
        return DRIVER
    cxx = shutil.which("g++") or "g++"
    tmp = DRIVER + f".tmp{os.getpid()}"
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", src, "-I", os.path.join(ROOT, "include"), "-L", BUILD, "-lskewt_gb300",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for skt_run.cpp:\n{r.stderr}")
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
    print(build_driver(force="--force" in sys.argv))
