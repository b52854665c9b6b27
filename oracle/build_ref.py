"""Build the reference's own offline statistics tool as a shared library (test infrastructure).

The reference's post-processing C tool (data_process/3D_C) computes its angle statistics in
``statistics.c`` with helpers from ``mathlib.c``; those two files compile on their own.  This
recipe compiles them, where they lie in the reference tree, into ``oracle/_ref/libangle_ref.so``
(git-ignored) so that the oracle restatement and the golden fixtures can be checked against
the reference itself.  It does not use the reference's makefile, copies no source, and does
nothing when the reference tree is absent.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

# the reference tree: LAPS_REFERENCE_DIR, else a checkout named "reference" beside this repository
REF = Path(os.environ.get("LAPS_REFERENCE_DIR") or Path(__file__).resolve().parents[2] / "reference")
OUT = Path(__file__).resolve().parent / "_ref"
LIB = OUT / "libangle_ref.so"


def build(force: bool = False) -> Path | None:
    src = REF / "data_process" / "3D_C"
    files = [src / "statistics.c", src / "mathlib.c"]
    if not all(f.exists() for f in files):
        return None
    if LIB.exists() and not force and LIB.stat().st_mtime > max(f.stat().st_mtime for f in files):
        return LIB
    OUT.mkdir(exist_ok=True)
    # mean() (mathlib.c:6-22) adds into a local it never initialises; zero-initialising
    # automatic variables gives it the start value the tool means, without touching the source
    cmd = ["gcc", "-O2", "-shared", "-fPIC", "-ftrivial-auto-var-init=zero", "-I", str(src), *map(str, files), "-lm",
           "-o", str(LIB)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))


def run_angle_statistics(prim, axis: int, nt: int = 0):
    """Run the reference's theta_ub_zpm_perp_only (statistics.c:10-356) on primitive fields
    ``prim[8, nz, ny, nx]`` for one axis, in a scratch directory (it writes its results to
    ./output/), and return the four arrays it wrote: ub method 1, ub method 2, zpm method 1,
    zpm method 2 (n_axis doubles each)."""
    import ctypes
    import tempfile

    import numpy as np

    lib_path = build()
    if lib_path is None:
        raise FileNotFoundError("the reference tree is not available")
    lib = ctypes.CDLL(str(lib_path))
    f = lib.theta_ub_zpm_perp_only
    f.restype = None
    f.argtypes = [ctypes.POINTER(ctypes.c_double)] + [ctypes.c_int] * 7
    nvar, nz, ny, nx = prim.shape
    uu = np.ascontiguousarray(np.transpose(prim, (0, 3, 2, 1)))  # the tool's [v][x][y][z]
    tag = "xyz"[axis]
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "output"))
        os.chdir(d)
        libc = ctypes.CDLL(None)
        saved = os.dup(1)
        log = os.open(os.path.join(d, "tool.log"), os.O_WRONLY | os.O_CREAT)
        os.dup2(log, 1)  # the tool reports its progress on stdout
        try:
            f(uu.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nt, 1, nx, ny, nz, nvar, axis)
        finally:
            libc.fflush(None)
            os.dup2(saved, 1)
            os.close(saved)
            os.close(log)
            os.chdir(cwd)
        out = []
        for kind in ("ub", "zpm"):
            for m in (1, 2):
                name = os.path.join(d, "output", f"theta_{kind}_perp_only_l{tag}_method{m}_{nt:03d}.dat")
                out.append(np.fromfile(name, dtype=np.float64))
    return out
