"""ctypes host of the C++/OpenMP restatement (oracle O2, ``oracle/laps3d_omp.cpp``).

TEST AND BASELINE INFRASTRUCTURE ONLY: the CPU baseline of the benchmark and a second
restatement the CPU tests check against ``oracle/laps3d.py``.  ``build()`` compiles the
source with g++ and OpenMP into ``oracle/_build/`` (git-ignored); nothing in the GPU path
loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "laps3d_omp.cpp"
LIB = HERE / "_build" / "liblaps3d_omp.so"
_lib = None


def build(force: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime > SRC.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-shared", "-fPIC", str(SRC), "-o", str(LIB)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        d, i, vp = C.c_double, C.c_int, C.c_void_p
        dp = C.POINTER(C.c_double)
        lib.o2_create.restype = vp
        lib.o2_create.argtypes = [i, i, i, d, i, d, i, d, d, i, d, d, i, d]
        lib.o2_destroy.argtypes = [vp]
        lib.o2_set_state.argtypes = [vp, dp, d]
        lib.o2_step.argtypes = [vp, i, dp, dp]
        lib.o2_get_state.argtypes = [vp, dp]
        lib.o2_threads.restype = i
        _lib = lib
    return _lib


def threads() -> int:
    return load().o2_threads()


class Run:
    """One 3-D compressible run: implicit viscosity / resistivity, the 2/3 sphere, Hall term
    and expanding box without corotation (the options the benchmark case uses)."""

    def __init__(self, shape, kw):
        nx, ny, nz = (shape,) * 3 if np.isscalar(shape) else shape
        unsupported = [k for k in ("if_resis_exp", "if_visc_exp", "if_corotating", "if_conserve_background")
                       if kw.get(k)]
        if kw.get("dealias_option", 2) != 1 or unsupported:
            raise ValueError(f"O2 covers dealias option 1 with implicit diffusion only ({unsupported})")
        self.lib = load()
        self.shape = (nz, ny, nx)
        self.h = self.lib.o2_create(nx, ny, nz, float(kw.get("adiabatic_index", 5.0 / 3.0)), int(kw.get("if_resis", 0)),
                                    float(kw.get("resistivity", 0.0)), int(kw.get("if_visc", 0)),
                                    float(kw.get("viscosity", 0.0)), float(kw.get("cfl", 0.5)), int(kw.get("if_AEB", 0)),
                                    float(kw.get("radius0", 30.0)), float(kw.get("Ur0", 0.0)), int(kw.get("if_Hall", 0)),
                                    float(kw.get("ion_inertial_length", 0.0)))
        if not self.h:
            raise ValueError("O2: grid sizes must be powers of two")

    def set_state(self, prim: np.ndarray, t0: float = 0.0):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        self.lib.o2_set_state(self.h, prim.ctypes.data_as(C.POINTER(C.c_double)), t0)

    def step(self, n: int = 1):
        t, dt = C.c_double(), C.c_double()
        self.lib.o2_step(self.h, n, C.byref(t), C.byref(dt))
        return t.value, dt.value

    def state(self) -> np.ndarray:
        out = np.empty((8,) + self.shape)
        self.lib.o2_get_state(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def close(self):
        if self.h:
            self.lib.o2_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
