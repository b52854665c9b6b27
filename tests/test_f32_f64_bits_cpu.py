"""The FP32 <-> FP64 conversions on the IEEE bit fields (laps_gb300/csrc/arith.cuh), which
the FP32-increment RK update uses instead of the FP64-pipe conversions, checked on the host
against the compiler's casts: float -> double exact for every normal float, zeros,
infinities and NaN; double -> float equal to the compiler's round-to-nearest-even cast for
every value in the FP32 normal range (ties included), zeros and infinities preserved, NaN
kept NaN, values below the FP32 normal range flushed to a signed zero."""
import shutil
import subprocess

import pytest

from laps_gb300.build import CSRC, PKG

ROOT = PKG.parent

PROG = r"""
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <limits>
#include "arith.cuh"
using namespace laps;
static uint64_t s = 88172645463325252ull;
static uint64_t rnd() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
int main() {
  long bad = 0, n = 0;
  // every float exponent with random significands and signs
  for (int i = 0; i < 4000000; i++) {
    uint32_t b = (uint32_t)rnd();
    float f; memcpy(&f, &b, 4);
    double d = f32_to_f64_bits(f);
    n++;
    if (std::isnan(f)) { if (!std::isnan(d)) bad++; continue; }
    if (std::fpclassify(f) == FP_SUBNORMAL) { if (d != 0.0 || std::signbit(d) != std::signbit(f)) bad++; continue; }
    if (d != (double)f) bad++;
  }
  // doubles across and beyond the float range
  for (int i = 0; i < 4000000; i++) {
    uint64_t b = rnd();
    int e = 1023 - 160 + (int)(rnd() % 320);  // exponents 2^-160 .. 2^160
    b = (b & 0x800fffffffffffffull) | ((uint64_t)e << 52);
    double d; memcpy(&d, &b, 8);
    if (i % 4 == 0) b = (b & ~0x1fffffffull) | 0x10000000ull;  // exact ties of the 29 dropped bits
    memcpy(&d, &b, 8);
    float t = f64_to_f32_rn(d);
    n++;
    const double a = std::fabs(d);
    if (a < (double)std::numeric_limits<float>::min()) { if (t != 0.0f || std::signbit(t) != std::signbit(d)) bad++; continue; }
    const float ref = (float)d;  // round to nearest even, overflow to infinity
    if (memcmp(&t, &ref, 4) != 0) bad++;
  }
  const double sp[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1.0, -2.5, 3.4028234663852886e38};
  for (double d : sp) {
    float t = f64_to_f32_rn(d);
    double back = f32_to_f64_bits(t);
    n++;
    if (std::isnan(d)) { if (!std::isnan(t) || !std::isnan(back)) bad++; }
    else if (t != (float)d || back != (double)(float)d || std::signbit(t) != std::signbit(d)) bad++;
  }
  printf("%ld %ld\n", n, bad);
  return bad != 0;
}
"""


def test_bit_field_conversions(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not shutil.which(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "cv.cu"
    src.write_text(PROG)
    exe = tmp_path / "cv"
    # device code for the library's architecture (its headers use sm_100-family intrinsics);
    # only the host functions run
    subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{CSRC}",
                    f"-I{ROOT / 'include'}", str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    n, bad = map(int, r.stdout.split())
    assert n > 8_000_000 and bad == 0 and r.returncode == 0
