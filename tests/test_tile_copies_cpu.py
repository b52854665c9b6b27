"""The kept-row tile copies of passes A and B, checked on the host.

``KeptCopies`` (laps_gb300/csrc/engine.cuh) decides which boxes of rows the TMA copies fetch
for a column whose kept rows are [0, lo) U [hi, n).  A wrong box either misses kept rows or
writes past the shared-memory tile, so every case the engine can meet is enumerated here, on
the CPU, by compiling the header for the host: every kept row covered exactly once, no box
outside the line, no two boxes overlapping, every destination on a 128-byte boundary, boxes of
at most 256 rows.
"""
import shutil
import subprocess

import pytest

from laps_gb300.build import CSRC, PKG

ROOT = PKG.parent

PROG = r"""
#include <cstdio>
#include <vector>
#include "engine.cuh"
using namespace laps;
int main() {
  long bad = 0, cases = 0;
  for (int n : {8, 16, 32, 64, 128, 256, 512, 1024})
    for (int bytes : {8, 16})
      for (int lo = 1; lo <= n; lo++)
        for (int hi = lo; hi <= n; hi++) {
          KeptCopies kc(lo, hi, n, tile_gran(bytes));
          cases++;
          std::vector<int> cov(n, 0);
          if (kc.box < 1 || kc.box > 256 || kc.box > n) { bad++; continue; }
          bool ok = true;
          for (int i = 0; i < kc.count(n) && ok; i++) {
            const int s = kc.start(i, n);
            if (s < 0 || s + kc.box > n || (s * TX * bytes) % 128) { ok = false; break; }
            for (int r = s; r < s + kc.box; r++) cov[r]++;
          }
          for (int r = 0; r < n && ok; r++)
            if (cov[r] > 1 || ((r < lo || r >= hi) && cov[r] != 1)) ok = false;
          if (!ok) bad++;
        }
  printf("%ld %ld\n", cases, bad);
  return bad != 0;
}
"""


def test_kept_row_copies_cover_every_case(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not shutil.which(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "kc.cu"
    src.write_text(PROG)
    exe = tmp_path / "kc"
    # device code for the library's architecture (its headers use sm_100-family intrinsics);
    # only the host functions run
    subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{CSRC}",
                    f"-I{ROOT / 'include'}", str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    cases, bad = map(int, r.stdout.split())
    assert cases > 1_000_000 and bad == 0 and r.returncode == 0
