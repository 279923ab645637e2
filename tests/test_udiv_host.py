"""The invariant-divisor constants of the metric kernels' index decode
(torch_gb300/csrc/tfv_metric.h, make_udiv): the header is compiled on the
host with g++, and the quotient formula the kernels evaluate,
(mulhi(m, n) + n) >> l, is checked against exact division for divisors
1 .. 4096, every power of two and its neighbours, large divisors, and
dividends at 0, near multiples of d and at the 2^31 - 1 limit of the decode."""

import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "torch_gb300" / "csrc"

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <vector>
#include "tfv_metric.h"

static uint32_t quotient(uint32_t n, const tfv::UDiv& v) {
  const uint32_t hi = (uint32_t)(((uint64_t)n * v.m) >> 32);
  return (uint32_t)(((uint64_t)hi + n) >> v.l);
}

int main() {
  std::vector<uint32_t> ds;
  for (uint32_t d = 1; d <= 4096; ++d) ds.push_back(d);
  for (int k = 12; k < 31; ++k)
    for (int e = -1; e <= 1; ++e) ds.push_back((uint32_t)((1u << k) + e));
  const uint32_t big[] = {65537u, 100003u, 1000003u, 46341u, 2147483647u, 2147483648u};
  for (uint32_t d : big) ds.push_back(d);
  uint64_t bad = 0, checked = 0;
  uint32_t x = 12345u;
  for (uint32_t d : ds) {
    const tfv::UDiv v = tfv::make_udiv(d);
    std::vector<uint32_t> ns = {0u, 1u, d - 1u, d, d + 1u, 2147483647u, 2147483646u};
    for (uint32_t q = 1; q < 64; ++q) {
      const uint64_t base = (uint64_t)q * d;
      if (base < 2147483648ull) {
        ns.push_back((uint32_t)base);
        ns.push_back((uint32_t)(base - 1));
      }
    }
    for (int r = 0; r < 200; ++r) {
      x = x * 1664525u + 1013904223u;
      ns.push_back(x & 0x7fffffffu);
    }
    for (uint32_t n : ns) {
      if (n > 2147483647u) continue;
      ++checked;
      if (quotient(n, v) != n / d) {
        if (bad < 5) std::printf("d=%u n=%u got %u want %u\n", d, n, quotient(n, v), n / d);
        ++bad;
      }
    }
  }
  std::printf("checked %llu bad %llu\n", (unsigned long long)checked, (unsigned long long)bad);
  return bad != 0;
}
"""


def test_invariant_divisor_quotients_are_exact(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("needs g++")
    src = tmp_path / "udiv.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "udiv"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I" + str(CSRC), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "bad 0" in out.stdout
