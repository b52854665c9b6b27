"""ctypes binding of ``include/laps_gpu.h`` (the C-ABI of ``liblaps_gpu.so``).

This is the Python host's view of the drop-in boundary: the same entry points a Fortran
host binds through ``iso_c_binding`` (``fortran/laps_gpu.f90``).  Arrays cross as float64
in the reference's Fortran order ``uu(ix,iy,iz,ivar)``, i.e. numpy ``[ivar, iz, iy, ix]``.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "liblaps_gpu.so"
HEADER = PKG.parent / "include" / "laps_gpu.h"

LAPS_OK = 0
LAPS_EINVAL = -1
LAPS_ENOMEM = -2
LAPS_ECUDA = -3
LAPS_ETIMEDOUT = -4
LAPS_ESTATE = -5
LAPS_STATUS_NAN = 1
LAPS_STATUS_DT_FLOOR = 2
LAPS_STATUS_DEVICE_TIMEOUT = 4
VARIANT_3DC, VARIANT_3DI, VARIANT_2DC = 0, 1, 2
PREC_FP64, PREC_DD, PREC_FP32, PREC_FP32_F64 = 0, 1, 2, 3
LAYOUT_PRIMITIVE, LAYOUT_CONSERVED = 0, 1
SCHED_PERSISTENT_B, SCHED_NO_PREFETCH_E, SCHED_INLINE_MASS, SCHED_ALL = 1, 2, 4, 7


class laps_params(C.Structure):
    _fields_ = [
        ("variant", C.c_int), ("precision", C.c_int),
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
        ("adiabatic_index", C.c_double),
        ("if_resis", C.c_int), ("if_resis_exp", C.c_int), ("resistivity", C.c_double),
        ("if_visc", C.c_int), ("if_visc_exp", C.c_int), ("viscosity", C.c_double),
        ("if_conserve_background", C.c_int),
        ("dealias_option", C.c_int), ("afx", C.c_double), ("afy", C.c_double), ("afz", C.c_double),
        ("cfl", C.c_double),
        ("if_AEB", C.c_int), ("radius0", C.c_double), ("Ur0", C.c_double),
        ("if_corotating", C.c_int), ("corotating_angle", C.c_double),
        ("if_Hall", C.c_int), ("ion_inertial_length", C.c_double),
        ("rho0", C.c_double), ("if_z_radial", C.c_int), ("if_limit_dt_increase", C.c_int),
        ("dstep_calcdt", C.c_int),
        ("device", C.c_int), ("timeout_ms", C.c_int), ("mem_cap_bytes", C.c_longlong),
        ("reserved", C.c_int * 8),
    ]


class laps_diag(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("dt", C.c_double), ("radius", C.c_double),
        ("uu_ave", C.c_double * 8), ("uu_rms", C.c_double * 8), ("rho_u2", C.c_double * 3),
        ("max_divB", C.c_double), ("max_divB_real", C.c_double), ("max_divV_real", C.c_double),
        ("e_kin", C.c_double), ("e_mag", C.c_double),
        ("h_cross", C.c_double), ("h_mag", C.c_double),
    ]


class laps_ic(C.Structure):
    _fields_ = [
        ("ifield", C.c_int), ("ipert", C.c_int),
        ("T0", C.c_double), ("rho0", C.c_double), ("B0", C.c_double), ("a0", C.c_double),
        ("U_fast", C.c_double), ("U_slow", C.c_double), ("n_fast", C.c_double), ("n_slow", C.c_double),
        ("press0", C.c_double), ("shear_width", C.c_double),
        ("bx0", C.c_double), ("by0", C.c_double), ("bz0", C.c_double), ("db0", C.c_double),
        ("in_out_ratio", C.c_double), ("dv0", C.c_double), ("drho0", C.c_double),
        ("nmodex", C.c_int), ("nmodey", C.c_int), ("nmodez", C.c_int), ("wave_number_jet", C.c_int),
        ("jet_width", C.c_double), ("Vjet", C.c_double),
        ("B0_SB", C.c_double), ("dB_SB", C.c_double), ("R0_SB", C.c_double), ("R1_SB", C.c_double),
        ("H_SB", C.c_double), ("Rm_SB", C.c_double), ("Rd_SB", C.c_double),
    ]


def ic_params(**kw) -> laps_ic:
    """Initial-condition parameters: the reference's defaults (``laps_ic_default``) overridden
    by keyword arguments (the namelist names of mhdinit.f90)."""
    lib = load()
    ic = laps_ic()
    lib.laps_ic_default(C.byref(ic))
    for k, v in kw.items():
        if not hasattr(ic, k):
            raise KeyError(k)
        setattr(ic, k, v)
    return ic


class laps_info(C.Structure):
    _fields_ = [
        ("device_bytes", C.c_longlong), ("kx_keep", C.c_int), ("ky_keep", C.c_int), ("kz_keep", C.c_int),
        ("kernels_per_step", C.c_int), ("graph", C.c_int),
    ]


_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load ``liblaps_gpu.so`` (building it first when it is missing); ``LAPS_GPU_LIB`` in the
    environment names another build of the library."""
    global _lib
    if _lib is not None:
        return _lib
    env = os.environ.get("LAPS_GPU_LIB")
    p = Path(path) if path else (Path(env) if env else LIB_PATH)
    if not p.exists():
        from . import build as _b
        _b.build()
    lib = C.CDLL(str(p))
    P = C.POINTER
    vp = C.c_void_p
    dp = P(C.c_double)
    sig = {
        "laps_params_default": (C.c_int, [P(laps_params)]),
        "laps_create": (C.c_int, [P(laps_params), P(vp)]),
        "laps_destroy": (None, [vp]),
        "laps_upload_state": (C.c_int, [vp, dp, C.c_int]),
        "laps_ic_default": (C.c_int, [P(laps_ic)]),
        "laps_ic_nphases": (C.c_longlong, [P(laps_ic)]),
        "laps_init_fields": (C.c_int, [vp, P(laps_ic), dp, C.c_longlong]),
        "laps_angle_statistics": (C.c_int, [vp, C.c_int, dp]),
        "laps_set_time": (C.c_int, [vp, C.c_double]),
        "laps_vardt": (C.c_int, [vp, dp]),
        "laps_step": (C.c_int, [vp, C.c_int, dp, dp, P(C.c_int)]),
        "laps_rk_stage": (C.c_int, [vp, C.c_int]),
        "laps_step_profiled": (C.c_int, [vp, C.c_int, dp, dp, P(C.c_int)]),
        "laps_download_state": (C.c_int, [vp, dp, dp]),
        "laps_download_spectral": (C.c_int, [vp, dp]),
        "laps_upload_spectral": (C.c_int, [vp, dp]),
        "laps_diagnostics": (C.c_int, [vp, P(laps_diag)]),
        "laps_spectrum": (C.c_int, [vp, C.c_int, dp, dp]),
        "laps_write_output": (C.c_int, [vp, C.c_char_p, C.c_int]),
        "laps_calc_flux": (C.c_int, [vp, dp]),
        "laps_transform_flux": (C.c_int, [vp, dp]),
        "laps_calc_rhs": (C.c_int, [vp, dp]),
        "laps_dealias": (C.c_int, [vp]),
        "laps_transform_uu_k2r": (C.c_int, [vp, dp]),
        "laps_update_prim": (C.c_int, [vp, dp]),
        "laps_read_restart": (C.c_int, [vp, C.c_char_p, dp]),
        "laps_wait": (C.c_int, [vp, C.c_int]),
        "laps_get_time": (C.c_int, [vp, dp, dp]),
        "laps_get_info": (C.c_int, [vp, P(laps_info)]),
        "laps_last_error": (C.c_char_p, [vp]),
        "laps_set_schedule": (C.c_int, [vp, C.c_int]),
        "laps_get_schedule": (C.c_int, [vp, P(C.c_int)]),
        "laps_batch_create": (C.c_int, [P(laps_params), C.c_int, P(vp)]),
        "laps_batch_size": (C.c_int, [vp]),
        "laps_batch_member": (C.c_int, [vp, C.c_int, P(vp)]),
        "laps_batch_step": (C.c_int, [vp, C.c_int, dp, dp, P(C.c_int)]),
        "laps_batch_destroy": (None, [vp]),
        "laps_batch_last_error": (C.c_char_p, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class LapsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"laps error {code}: {msg}")
        self.code = code


def params(**kw) -> laps_params:
    """Reference defaults (``laps_params_default``) overridden by keyword arguments."""
    lib = load()
    p = laps_params()
    lib.laps_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Laps:
    """One GPU run: the reference's hot-path subroutines as methods over a context."""

    def __init__(self, p: laps_params, handle=None):
        self.lib = load()
        self.p = p
        self.owned = handle is None
        if handle is None:
            h = C.c_void_p()
            rc = self.lib.laps_create(C.byref(p), C.byref(h))
            if rc != LAPS_OK:
                raise LapsError(rc, self.lib.laps_last_error(None).decode())
            handle = h
        self.h = handle
        self.shape = (p.nz, p.ny, p.nx)

    def _ck(self, rc):
        if rc != LAPS_OK:
            raise LapsError(rc, self.lib.laps_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            if self.owned:
                self.lib.laps_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- reference routines
    def upload_state(self, uu: np.ndarray, primitive: bool = True):
        a = np.ascontiguousarray(uu, dtype=np.float64)
        assert a.shape == (8,) + self.shape
        self._ck(self.lib.laps_upload_state(self.h, _dptr(a), LAYOUT_PRIMITIVE if primitive else LAYOUT_CONSERVED))

    def init_fields(self, ic: "laps_ic", phases=None):
        """Generate the fresh-start state on the device (background + perturbation +
        conserved form + forward transform); ``phases`` (radians) for ipert 6 and 7."""
        n = self.lib.laps_ic_nphases(C.byref(ic))
        if n:
            a = np.ascontiguousarray(phases, dtype=np.float64).ravel()
            self._ck(self.lib.laps_init_fields(self.h, C.byref(ic), _dptr(a), int(a.size)))
        else:
            self._ck(self.lib.laps_init_fields(self.h, C.byref(ic), None, 0))

    def angle_statistics(self, axis: int) -> np.ndarray:
        """Perpendicular angle statistics of the increments along ``axis`` (0 x, 1 y, 2 z):
        rows ub method 1, ub method 2, zpm method 1, zpm method 2; column l = lag l."""
        n = (self.p.nx, self.p.ny, self.p.nz)[axis]
        out = np.zeros((4, n))
        self._ck(self.lib.laps_angle_statistics(self.h, int(axis), _dptr(out)))
        return out

    def set_time(self, t: float):
        self._ck(self.lib.laps_set_time(self.h, float(t)))

    def vardt(self) -> float:
        d = C.c_double()
        self._ck(self.lib.laps_vardt(self.h, C.byref(d)))
        return d.value

    def step(self, n: int = 1):
        t, d, s = C.c_double(), C.c_double(), C.c_int()
        self._ck(self.lib.laps_step(self.h, int(n), C.byref(t), C.byref(d), C.byref(s)))
        return t.value, d.value, s.value

    def step_profiled(self, n: int):
        """n steps with per-pass CUDA-event timing: (pass_ms[6], total_ms, status)."""
        pm = (C.c_double * 6)()
        tot, s = C.c_double(), C.c_int()
        self._ck(self.lib.laps_step_profiled(self.h, int(n), pm, C.byref(tot), C.byref(s)))
        return np.array(pm[:]), tot.value, s.value

    def rk_stage(self, irk: int):
        self._ck(self.lib.laps_rk_stage(self.h, int(irk)))

    def download_state(self):
        uu = np.empty((8,) + self.shape)
        prim = np.empty((4,) + self.shape)
        self._ck(self.lib.laps_download_state(self.h, _dptr(uu), _dptr(prim)))
        return uu, prim

    def download_spectral(self):
        nz, ny, nx = self.shape
        uf = np.empty((8, nz, ny, nx // 2 + 1), np.complex128)
        self._ck(self.lib.laps_download_spectral(self.h, uf.ctypes.data_as(C.POINTER(C.c_double))))
        return uf

    def upload_spectral(self, uf: np.ndarray):
        a = np.ascontiguousarray(uf, dtype=np.complex128)
        self._ck(self.lib.laps_upload_spectral(self.h, a.ctypes.data_as(C.POINTER(C.c_double))))

    def diagnostics(self) -> laps_diag:
        d = laps_diag()
        self._ck(self.lib.laps_diagnostics(self.h, C.byref(d)))
        return d

    def spectrum(self, nshell: int):
        """Shell spectra (e_u, e_b) of the current state, nshell shells of width 2 pi / max(L)."""
        eu = np.zeros(nshell)
        eb = np.zeros(nshell)
        self._ck(self.lib.laps_spectrum(self.h, int(nshell), _dptr(eu), _dptr(eb)))
        return eu, eb

    # -- granular path (the reference's subroutines one at a time)
    def nflux(self) -> int:
        return 18 + (1 if self.p.if_AEB else 0)

    def calc_flux(self) -> np.ndarray:
        out = np.empty((self.nflux(),) + self.shape)
        self._ck(self.lib.laps_calc_flux(self.h, _dptr(out)))
        return out

    def transform_flux(self) -> np.ndarray:
        out = np.empty((self.nflux(),) + self.shape[:2] + (self.shape[2] // 2 + 1,), dtype=np.complex128)
        self._ck(self.lib.laps_transform_flux(self.h, _dptr(out.view(np.float64))))
        return out

    def calc_rhs(self) -> np.ndarray:
        out = np.empty((8,) + self.shape[:2] + (self.shape[2] // 2 + 1,), dtype=np.complex128)
        self._ck(self.lib.laps_calc_rhs(self.h, _dptr(out.view(np.float64))))
        return out

    def dealias(self):
        self._ck(self.lib.laps_dealias(self.h))

    def write_output(self, path, primitive: bool = True):
        """Write the state as the reference's outNNN.dat."""
        self._ck(self.lib.laps_write_output(self.h, os.fsencode(path), LAYOUT_PRIMITIVE if primitive else LAYOUT_CONSERVED))

    def read_restart(self, path) -> float:
        """Read an outNNN.dat (primitive), upload it and set the time; returns the time."""
        t = C.c_double()
        self._ck(self.lib.laps_read_restart(self.h, os.fsencode(path), C.byref(t)))
        return t.value

    def time(self):
        t, d = C.c_double(), C.c_double()
        self._ck(self.lib.laps_get_time(self.h, C.byref(t), C.byref(d)))
        return t.value, d.value

    def set_schedule(self, bits: int):
        """Execution schedule bits (SCHED_*): bit-identical results, different launch plans."""
        self._ck(self.lib.laps_set_schedule(self.h, int(bits)))

    def schedule(self) -> int:
        v = C.c_int()
        self._ck(self.lib.laps_get_schedule(self.h, C.byref(v)))
        return v.value

    def info(self) -> laps_info:
        i = laps_info()
        self._ck(self.lib.laps_get_info(self.h, C.byref(i)))
        return i

    def wait(self, timeout_ms: int = 600000):
        self._ck(self.lib.laps_wait(self.h, int(timeout_ms)))


class Batch:
    """An ensemble of independent runs advanced together (laps_batch_*); members[i] is a Laps
    view of member i (upload, download, diagnostics), owned by the batch."""

    def __init__(self, plist):
        self.lib = load()
        arr = (laps_params * len(plist))(*plist)
        h = C.c_void_p()
        rc = self.lib.laps_batch_create(arr, len(plist), C.byref(h))
        if rc != LAPS_OK:
            raise LapsError(rc, self.lib.laps_batch_last_error(None).decode())
        self.h = h
        self.n = len(plist)
        self.members = []
        for i, p in enumerate(plist):
            m = C.c_void_p()
            self._ck(self.lib.laps_batch_member(self.h, i, C.byref(m)))
            self.members.append(Laps(p, handle=m))

    def _ck(self, rc):
        if rc != LAPS_OK:
            raise LapsError(rc, self.lib.laps_batch_last_error(self.h).decode())

    def step(self, nsteps: int = 1):
        """Advance every member by nsteps; returns arrays (time, dt, status)."""
        t = np.zeros(self.n)
        d = np.zeros(self.n)
        s = (C.c_int * self.n)()
        self._ck(self.lib.laps_batch_step(self.h, int(nsteps), _dptr(t), _dptr(d), s))
        return t, d, np.array(list(s), dtype=np.int32)

    def close(self):
        if getattr(self, "h", None):
            for m in self.members:
                m.h = None
            self.lib.laps_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
