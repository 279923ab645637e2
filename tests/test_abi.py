"""C-ABI checks that need no GPU: the library builds, loads and exports every
function include/tfv.h declares, and the ctypes structs match the C layout."""

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from torch_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "tfv.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tfv_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.library_path())],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (tfv_[a-z0-9_]+)", out))
    assert set(names) <= exported
    assert lib.tfv_version().decode().startswith("tfv")


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "tfv.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(tfv_config),"
        " sizeof(tfv_tile), sizeof(tfv_report), offsetof(tfv_config, spacing),"
        " offsetof(tfv_report, steps), sizeof(tfv_metric_face), sizeof(tfv_metric_config),"
        " offsetof(tfv_metric_config, max_steps), offsetof(tfv_metric_config, faces));"
        "return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == [C.sizeof(_lib.Config), C.sizeof(_lib.Tile), C.sizeof(_lib.Report),
                   _lib.Config.spacing.offset, _lib.Report.steps.offset,
                   C.sizeof(_lib.MetricFace), C.sizeof(_lib.MetricConfig),
                   _lib.MetricConfig.max_steps.offset, _lib.MetricConfig.faces.offset]


def test_invalid_arguments_are_rejected_without_a_gpu():
    lib = _lib.load()
    handle = C.c_void_p()
    cfg = _lib.Config()
    cfg.dim = 3
    for k in range(3):
        cfg.counts[k] = 1  # fewer than two cells
        cfg.lengths[k] = 1.0
    cfg.gamma, cfg.cfl, cfg.t_end, cfg.max_steps = 1.4, 0.4, 1.0, 10
    code = lib.tfv_batch_create(3, 0, 1, C.byref(cfg), None, C.byref(handle))
    assert code == _lib.TFV_EINVAL
    assert "cells" in _lib.last_error()
    with pytest.raises(ValueError):
        _lib.check(code)


def _weak_symbols(obj):
    out = subprocess.run(["nm", "--defined-only", str(obj)], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines()
            if len(line.split()) == 3 and line.split()[1] in ("W", "V") and "3tfv" in line}


def test_precision_units_share_no_mergeable_symbols():
    """The double and single precision units compile the same sources with a
    different REAL.  A weak (mergeable) tfv symbol defined in both would be
    linked once and run one precision's kernels on the other's buffers."""
    from torch_gb300 import build
    build.build()
    objs = {name: build.BUILD / (Path(name).stem + ".o") for name in build.UNITS}
    for double_unit in ("tfv_f64.cu", "tfv_metric_f64.cu"):
        f64 = _weak_symbols(objs[double_unit])
        for unit in ("tfv_f32_2d.cu", "tfv_f32_3d.cu", "tfv_metric_f32.cu"):
            shared = f64 & _weak_symbols(objs[unit])
            assert not shared, (double_unit, unit, sorted(shared)[:5])


def test_metric_and_rusanov_arguments_are_rejected_without_a_gpu():
    lib = _lib.load()
    cfg = _lib.MetricConfig()
    cfg.dim = 2
    cfg.n[0], cfg.n[1] = 8, 4
    cfg.lengths[0], cfg.lengths[1] = 1.0, 1.0
    cfg.geometry = _lib.GEOMETRIES["annular"]
    cfg.cfl, cfg.gamma, cfg.t_end, cfg.max_steps = 0.4, 1.4, 1.0, 10
    cfg.faces[2].type = _lib.FACE_TYPES["periodic"]  # y_min periodic, y_max not
    count = lib.tfv_metric_factor_count(C.byref(cfg))
    assert count == 8 + 4 + (9 + 4) + (8 + 5)
    factors = (C.c_double * count)(*([1.0] * count))
    handle = C.c_void_p()
    code = lib.tfv_metric_create(_lib.TFV_FP64, C.byref(cfg), factors, C.byref(handle))
    assert code == _lib.TFV_EINVAL and "Periodic" in _lib.last_error()
    cfg.faces[2].type = _lib.FACE_TYPES["outflow"]
    cfg.dim = 4
    assert lib.tfv_metric_create(_lib.TFV_FP64, C.byref(cfg), factors,
                                 C.byref(handle)) == _lib.TFV_EINVAL
    cfg.dim = 2
    code = lib.tfv_metric_create(_lib.TFV_FP64, C.byref(cfg), factors, C.byref(handle))
    assert code == _lib.TFV_OK  # a valid configuration needs no device until bind
    size = C.c_size_t()
    assert lib.tfv_metric_workspace_size(handle, C.byref(size)) == _lib.TFV_OK and size.value > 0
    lib.tfv_metric_destroy(handle)
    assert lib.tfv_rusanov_flux(0, 6, 10, 0, None, None, None, None, None,
                                None) == _lib.TFV_EINVAL
    assert lib.tfv_rusanov_flux(0, 4, 10, 2, None, None, None, None, None,
                                None) == _lib.TFV_EINVAL
