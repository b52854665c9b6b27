"""FastDiv (laps_gb300/csrc/engine.cuh), the multiply-high division by an invariant divisor that
splits the flat element index of the elementwise update kernels, checked on the host against
the C++ division: every divisor 1..70000 (the kept kx and ky counts of grids up to 65536
points per axis) at the edges of each quotient step and at random numerators below 2^31.
The device evaluates the same formula with __umulhi."""
import shutil
import subprocess

import pytest

from laps_gb300.build import CSRC, PKG

ROOT = PKG.parent

PROG = r"""
#include <cstdio>
#include <random>
#include "engine.cuh"
using namespace laps;
int main() {
  std::mt19937 rng(5);
  long bad = 0, cases = 0;
  const unsigned top = 0x7fffffffu;
  for (unsigned d = 1; d <= 70000; d++) {
    const FastDiv f(d);
    auto check = [&](unsigned n) {
      cases++;
      if (f.div(n) != n / d) bad++;
    };
    for (unsigned n : {0u, 1u, d - 1, d, d + 1, 2 * d - 1, 2 * d, top, top - 1, top - d, top / d * d, top / d * d - 1})
      if (n <= top) check(n);
    for (int i = 0; i < 40; i++) check(rng() & top);
    for (int i = 0; i < 8; i++) {  // around a random multiple
      const unsigned q = (rng() & top) / d;
      check(q * d);
      if (q) check(q * d - 1);
    }
  }
  printf("%ld %ld\n", cases, bad);
  return bad != 0;
}
"""


def test_fast_div_matches_integer_division(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not shutil.which(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "fd.cu"
    src.write_text(PROG)
    exe = tmp_path / "fd"
    # device code for the library's architecture (its headers use sm_100-family intrinsics);
    # only the host functions run
    subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{CSRC}",
                    f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    cases, bad = map(int, r.stdout.split())
    assert cases > 4_000_000 and bad == 0, r.stdout
