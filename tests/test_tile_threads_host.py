"""Threads per CTA of the step kernel for a tile shape (step_threads in
torch_gb300/csrc/tfv_types.h), compiled on the host with g++: tiles that are
whole warps of cells keep one thread per cell; single-precision 2D / 3D tiles
that are not get their ring cells on the lanes after the owners, rounded up to
whole warps, when that fits 256 threads; double precision never does."""

import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "torch_gb300" / "csrc"

# (dim, exact, tx, ty, expected threads)
CASES = [
    (3, False, 16, 16, 256),   # whole warps: one thread per cell
    (3, False, 32, 8, 256),
    (3, False, 16, 12, 192),
    (3, False, 12, 12, 224),   # 144 cells + 52 ring -> 196 -> 224
    (3, False, 12, 10, 192),   # 120 + 48 -> 168 -> 192
    (3, False, 20, 12, 240),   # 240 + 68 > 256: no ring lanes (not whole warps either)
    (3, True, 12, 12, 144),    # double precision: one thread per cell
    (3, True, 32, 4, 128),
    (2, False, 128, 1, 128),
    (2, False, 124, 1, 128),   # 124 + 2 -> 128
    (2, False, 100, 1, 128),
    (2, False, 252, 1, 256),
    (2, False, 256, 1, 256),
    (2, True, 124, 1, 124),
    (1, False, 100, 1, 100),   # 1D tubes keep one thread per cell
]

PROGRAM = r"""
#include <cstdio>
#include "tfv_types.h"
int main() {
  int d, e, tx, ty;
  while (std::scanf("%d %d %d %d", &d, &e, &tx, &ty) == 4)
    std::printf("%d\n", tfv::step_threads(d, e != 0, tx, ty));
  return 0;
}
"""


def test_step_threads(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("needs g++")
    src = tmp_path / "threads.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "threads"
    subprocess.run([gxx, "-O1", "-std=c++17", "-I" + str(CSRC), str(src), "-o", str(exe)],
                   check=True)
    feed = "".join(f"{d} {int(e)} {tx} {ty}\n" for d, e, tx, ty, _ in CASES)
    out = subprocess.run([str(exe)], input=feed, capture_output=True, text=True, check=True)
    got = [int(v) for v in out.stdout.split()]
    assert got == [c[-1] for c in CASES]
    for (d, e, tx, ty, want), n in zip(CASES, got):
        cells = tx * (ty if d == 3 else 1)
        assert n >= cells and n <= max(cells, 256)
