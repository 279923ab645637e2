"""Build libtfv.so (the C-ABI CUDA library) in-tree for sm_103a.

    python -m torch_gb300.build

Each translation unit is compiled by nvcc in parallel; the double-precision
kernels are built with -fmad=false so that they keep NumPy's rounding, the
single-precision kernels with FMA contraction, flush-to-zero and fast
division/square root.  Output: torch_gb300/_build/libtfv.so; with --checked,
the checked build torch_gb300/_build/checked/libtfv.so (kernel indexes
tested against their buffers, for debugging).
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libtfv.so"
CHECKED_LIB = BUILD / "checked" / "libtfv.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + str(INCLUDE),
          "-I" + str(CSRC)]
F32 = ["-fmad=true", "-ftz=true", "-prec-div=false", "-prec-sqrt=false"]
UNITS = {
    "tfv_f64.cu": ["-fmad=false"],
    "tfv_f32_3d.cu": F32,
    "tfv_f32_2d.cu": F32,
    "tfv_host.cu": [],
    "tfv_metric_f64.cu": ["-fmad=false"],
    "tfv_metric_f32.cu": F32,
    "tfv_metric_host.cu": [],
}


def nvcc_path():
    nvcc = shutil.which("nvcc")
    if nvcc is None:
        cand = Path("/usr/local/cuda/bin/nvcc")
        if cand.exists():
            return str(cand)
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtfv")
    return nvcc


def _sources_newer(target):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def library(checked=False):
    """Path of the library: the release build, or the checked build (every
    kernel index tested against its buffer, each launch waited for)."""
    return CHECKED_LIB if checked else LIB


def build(force=False, verbose=False, checked=False):
    """Compile every unit and link libtfv.so; returns its path."""
    lib = library(checked)
    if not force and not _sources_newer(lib):
        return lib
    out = lib.parent
    out.mkdir(parents=True, exist_ok=True)
    nvcc = nvcc_path()
    extra = ["-DTFV_CHECKED=1"] if checked else []

    def compile_unit(item):
        src, flags = item
        obj = out / (Path(src).stem + ".o")
        cmd = [nvcc, *ARCH, *COMMON, *extra, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as pool:
        objs = list(pool.map(compile_unit, UNITS.items()))
    tmp = out / "libtfv.so.tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv))
