"""ORACLE — test infrastructure only.

Builds the reference's own CUDA kernels, unmodified, from the reference checkout into
``oracle/_ref/`` (git-ignored), and the driver-API harness that runs them.

* ``build_cubins()`` needs the reference checkout (``SKT_REFERENCE_DIR``, default
  ``/root/reference``). For each grid size it writes a wrapper translation unit that includes
  Game/config.h first (it is ``#pragma once``), overrides the compile-time grid and voxel size,
  defines the ``ConstantsGPU`` values by extracting Game/environment.cu:28-60, and includes
  Game/kernelMaths.cu, Game/kernelGround.cu, Game/kernelSky.cu and Game/microPhysics.cu as they
  are. Shim headers map the reference's ``<CUDA/include/...>`` and ``<CUDA/cmath>`` includes to
  the CUDA toolkit. Output: ``oracle/_ref/ref_<X>x<Y>x<Z>.cubin`` (sm_103a).
* ``build_harness()`` compiles ``oracle/ref_harness.cpp`` (driver API) into
  ``oracle/_ref/libref_harness.so``; it needs only g++ and the CUDA headers, so it also runs on
  a machine without the reference checkout, given the prebuilt cubins.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("SKT_REFERENCE_DIR", "/root/reference")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")

# (X, Y vertical, Z, voxel): reference-layout grids the tests pin against
GRIDS = [(16, 32, 16, 100.0), (32, 32, 32, 100.0), (64, 32, 64, 100.0)]


def cubin_path(X, Y, Z):
    return os.path.join(OUT, f"ref_{X}x{Y}x{Z}.cubin")


def harness_path():
    return os.path.join(OUT, "libref_harness.so")


def reference_available() -> bool:
    return os.path.exists(os.path.join(REF, "Game", "kernelSky.cu"))


def _shims():
    sh = os.path.join(OUT, "shim")
    os.makedirs(os.path.join(sh, "CUDA", "include"), exist_ok=True)
    files = {
        os.path.join(sh, "CUDA", "include", "cuda_runtime.h"): "#include <cuda_runtime.h>\n",
        os.path.join(sh, "CUDA", "include", "cuda.h"): "#include <cuda.h>\n",
        os.path.join(sh, "CUDA", "cmath"): "#include <cuda/std/cmath>\n#include <cmath>\n",
        os.path.join(sh, "force.h"): "#define __debugbreak() __builtin_trap()\n",
    }
    for p, txt in files.items():
        with open(p, "w") as f:
            f.write(txt)
    return sh


def _constants():
    """Game/environment.cu:28-60, the ConstantsGPU definitions, copied at build time."""
    with open(os.path.join(REF, "Game", "environment.cu"), encoding="utf-8", errors="replace") as f:
        lines = f.read().splitlines()
    block = lines[27:60]
    if not block[0].startswith("namespace ConstantsGPU") or not block[-1].startswith("}"):
        raise RuntimeError("unexpected Game/environment.cu layout")
    p = os.path.join(OUT, "constants.inc")
    with open(p, "w") as f:
        f.write("\n".join(block) + "\n")
    return p


def build_cubins(force: bool = False):
    if not reference_available():
        return []
    os.makedirs(OUT, exist_ok=True)
    sh = _shims()
    _constants()
    g = os.path.join(REF, "Game")
    nvcc = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    outs = []
    for X, Y, Z, vox in GRIDS:
        cub = cubin_path(X, Y, Z)
        outs.append(cub)
        if os.path.exists(cub) and not force:
            continue
        wrap = os.path.join(OUT, f"wrap_{X}x{Y}x{Z}.cu")
        with open(wrap, "w") as f:
            f.write(f'#include "{g}/config.h"\n')
            for n, v in (("GRIDSIZESKYX", X), ("GRIDSIZESKYY", Y), ("GRIDSIZESKYZ", Z)):
                f.write(f"#undef {n}\n#define {n} {v}\n")
            f.write(f"#undef VOXELSIZE\n#define VOXELSIZE {vox}f\n")
            f.write(f"static_assert(GRIDSIZESKY == {X * Y * Z}, \"grid override\");\n")
            f.write(f'#include "{g}/meteoconstants.cuh"\n#include "constants.inc"\n')
            for src in ("kernelMaths.cu", "kernelGround.cu", "kernelSky.cu", "microPhysics.cu"):
                f.write(f'#include "{g}/{src}"\n')
        cmd = [nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-cubin", "-w",
               "-I", OUT, "-I", sh, "-I", os.path.join(REF, "Engine", "external"), "-I", os.path.join(REF, "Engine", "include"),
               "-I", g, "-include", os.path.join(sh, "force.h"), wrap, "-o", cub + ".tmp"]
        subprocess.run(cmd, check=True, capture_output=True)
        os.replace(cub + ".tmp", cub)
    return outs


def build_harness(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    so = harness_path()
    src = os.path.join(HERE, "ref_harness.cpp")
    if os.path.exists(so) and not force and os.path.getmtime(so) >= os.path.getmtime(src):
        return so
    inc = os.path.join(CUDA_HOME, "include")
    libdirs = [os.path.join(CUDA_HOME, "lib64", "stubs"), os.path.join(CUDA_HOME, "lib64"),
               os.path.join(CUDA_HOME, "targets", "sbsa-linux", "lib", "stubs"),
               os.path.join(CUDA_HOME, "targets", "x86_64-linux", "lib", "stubs")]
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", src, "-I", inc, "-o", so + ".tmp"]
    for d in libdirs:
        if os.path.isdir(d):
            cmd += ["-L", d]
    cmd += ["-lcuda"]
    subprocess.run(cmd, check=True)
    os.replace(so + ".tmp", so)
    return so


# (X, Y vertical, Z, voxel): compile-time grids of the reference's sounding reader builds. The
# first is the reference's own Game/config.h; 37.5 m makes the level heights non-integer.
READTABLE_GRIDS = [(32, 32, 32, 64.0), (6, 40, 4, 100.0), (5, 24, 3, 37.5)]


def readtable_path(X, Y, Z, voxel):
    return os.path.join(OUT, f"libreadtable_{X}x{Y}x{Z}_{voxel:g}.so")


def build_readtable(force: bool = False):
    """The reference's sounding reader (Game/readTable.cpp with Engine/source/math/meteoformulas.cpp),
    unmodified, as one shared library per compile-time grid, with the harness
    ``oracle/ref_readtable.cpp`` appended. Host code only (g++), x86 or Arm."""
    if not os.path.exists(os.path.join(REF, "Game", "readTable.cpp")):
        return []
    os.makedirs(OUT, exist_ok=True)
    g = os.path.join(REF, "Game")
    inc = ["-I", os.path.join(HERE, "readtable_stubs"), "-I", os.path.join(REF, "Engine", "include"),
           "-I", os.path.join(REF, "Engine", "external"), "-I", g, "-I", os.path.join(CUDA_HOME, "include")]
    # -fpermissive: zip_file.hpp passes a uint64_t callback where miniz wants mz_uint64, the
    # same width under a different name on LP64 Linux
    flags = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-w", "-fpermissive"]
    meteo = os.path.join(OUT, "meteoformulas.o")
    harness = os.path.join(HERE, "ref_readtable.cpp")
    if force or not os.path.exists(meteo):
        subprocess.run(["g++", *flags, *inc, "-c", os.path.join(REF, "Engine", "source", "math", "meteoformulas.cpp"),
                        "-o", meteo + ".tmp"], check=True, capture_output=True, text=True)
        os.replace(meteo + ".tmp", meteo)
    outs = []
    for X, Y, Z, vox in READTABLE_GRIDS:
        so = readtable_path(X, Y, Z, vox)
        outs.append(so)
        if os.path.exists(so) and not force and os.path.getmtime(so) >= os.path.getmtime(harness):
            continue
        wrap = os.path.join(OUT, f"wrap_readtable_{X}x{Y}x{Z}_{vox:g}.cpp")
        with open(wrap, "w") as f:
            f.write(f'#include "{g}/config.h"\n')
            for n, v in (("GRIDSIZESKYX", X), ("GRIDSIZESKYY", Y), ("GRIDSIZESKYZ", Z)):
                f.write(f"#undef {n}\n#define {n} {v}\n")
            f.write(f"#undef VOXELSIZE\n#define VOXELSIZE {vox}f\n")
            # the reference was written against MSVC's headers: std::memset/strlen without
            # <cstring>, std::sinf/cosf, which libstdc++ leaves in the global namespace
            f.write("#include <cstring>\n#include <cmath>\nnamespace std { using ::sinf; using ::cosf; }\n")
            f.write(f'#include "{g}/readTable.cpp"\n#include "{harness}"\n')
        r = subprocess.run(["g++", *flags, "-shared", *inc, wrap, meteo, "-o", so + ".tmp"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference sounding reader build failed:\n{r.stderr[-4000:]}")
        os.replace(so + ".tmp", so)
    return outs


def colors_path():
    return os.path.join(OUT, "libref_colors.so")


def _setcolors_body():
    """The statements of editor::setColors (Game/editor.cpp:53-112), copied at build time."""
    with open(os.path.join(REF, "Game", "editor.cpp"), encoding="utf-8", errors="replace") as f:
        lines = f.read().splitlines()
    start = next(i for i, ln in enumerate(lines) if ln.strip() == "void editor::setColors()")
    if lines[start + 1].strip() != "{":
        raise RuntimeError("unexpected Game/editor.cpp layout")
    end = next(i for i in range(start + 2, len(lines)) if lines[i].rstrip() == "}")
    p = os.path.join(OUT, "setcolors_body.inc")
    with open(p, "w") as f:
        f.write("\n".join(lines[start + 2:end]) + "\n")
    return p


def build_colors(force: bool = False):
    """The reference's colour schemes: editor::setColors' statements and
    Engine/source/rendering/colors.cpp, unmodified, with oracle/ref_colors.cpp (g++, host code)."""
    src = os.path.join(REF, "Engine", "source", "rendering", "colors.cpp")
    if not os.path.exists(src) or not os.path.exists(os.path.join(REF, "Game", "editor.cpp")):
        return None
    os.makedirs(OUT, exist_ok=True)
    so = colors_path()
    harness = os.path.join(HERE, "ref_colors.cpp")
    if os.path.exists(so) and not force and os.path.getmtime(so) >= os.path.getmtime(harness):
        return so
    _setcolors_body()
    inc = ["-I", os.path.join(HERE, "colors_stubs"), "-I", OUT, "-I", os.path.join(REF, "Engine", "include"),
           "-I", os.path.join(REF, "Engine", "external")]
    force_inc = ["-include", os.path.join(HERE, "colors_stubs", "std_headers.hpp")]
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w", *force_inc, *inc, harness, src,
                        "-o", so + ".tmp"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference colour schemes build failed:\n{r.stderr[-4000:]}")
    os.replace(so + ".tmp", so)
    return so


if __name__ == "__main__":
    print(build_cubins(force=True))
    print(build_harness(force=True))
    print(build_readtable(force=True))
    print(build_colors(force=True))
