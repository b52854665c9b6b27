"""The allocation-free forward transform against the context-owning path.

laps_transform_uu_real_to_fourier_noalloc serves callers that cannot call cudaMalloc
(device memory owned by their own pool or framework, or allocation forbidden after start-up):
they pass device buffers they already own and the library keeps its one intermediate
spectrum in a fixed device array.  Here its output must equal what laps_upload_state +
laps_download_spectral produce for the same fields, within the transform tolerance the other
tests use (1e-14 of the largest coefficient), on calls in a row that share that array - the
shapes cover every row-transform length it accepts up to 512 points (the 256- and 512-point
rows take the paired-row and 16-lines-per-batch paths).  A host that resets the device
between calls (cudaDeviceReset, as Fortran hosts do between runs) must get correct results
after the reset too: that case runs in a fresh process that owns the device alone.
Device buffers come from torch, or from the CUDA runtime in the reset case.  This file is
named so that pytest collects it last.
"""
import ctypes
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

from laps_gb300 import ffi

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def _fn():
    lib = ffi.load()
    f = lib.laps_transform_uu_real_to_fourier_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_void_p]
    return lib, f


def _reference_path(fields, shape):
    """The existing entry points: upload the fields as a conserved state, read the spectrum."""
    nx, ny, nz = shape
    state = np.zeros((8, nz, ny, nx))
    state[: fields.shape[0]] = fields
    run = ffi.Laps(ffi.params(nx=nx, ny=ny, nz=nz, precision=ffi.PREC_FP64))
    run.upload_state(state, primitive=False)
    uf = run.download_spectral()
    run.close()
    return uf[: fields.shape[0]]


def _noalloc(f, fields, shape):
    torch = pytest.importorskip("torch")
    nx, ny, nz = shape
    nf = fields.shape[0]
    d_in = torch.from_numpy(np.ascontiguousarray(fields)).cuda()
    d_out = torch.empty((nf, nz, ny, nx // 2 + 1), dtype=torch.complex128, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = f(d_in.data_ptr(), d_out.data_ptr(), nx, ny, nz, nf, stream)
    torch.cuda.synchronize()
    return rc, d_out.cpu().numpy()


@pytest.mark.parametrize("shapes", [
    (((32, 16, 8), 8), ((64, 32, 32), 3)),
    (((256, 64, 16), 3), ((512, 16, 8), 2)),
    (((128, 128, 128), 1), ((16, 256, 512), 2)),
], ids=["short", "x256_x512", "128cube_yz_long"])
def test_two_calls_match_the_context_path(shapes):
    lib, f = _fn()
    rng = np.random.default_rng(42)
    for shape, nf in shapes:  # two calls in a row on the shared scratch array
        nx, ny, nz = shape
        fields = rng.standard_normal((nf, nz, ny, nx))
        rc, got = _noalloc(f, fields, shape)
        assert rc == 0, lib.laps_last_error(None)
        ref = _reference_path(fields, shape)
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max(), shape


def test_rejects_grids_beyond_the_fixed_scratch():
    lib, f = _fn()
    torch = pytest.importorskip("torch")
    buf = torch.empty(16, dtype=torch.float64, device="cuda")
    rc = f(buf.data_ptr(), buf.data_ptr(), 512, 512, 512, 1, None)
    assert rc == ffi.LAPS_EINVAL
    assert b"scratch" in lib.laps_last_error(None)


_RESET_SCRIPT = textwrap.dedent(r"""
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    from laps_gb300 import ffi
    lib = ffi.load()
    rt = ctypes.CDLL("libcudart.so.13")  # the runtime the library itself is linked against
    f = lib.laps_transform_uu_real_to_fourier_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_int] * 4 + [ctypes.c_void_p]
    for fn in ("cudaMalloc", "cudaMemcpy", "cudaFree", "cudaDeviceSynchronize", "cudaDeviceReset"):
        getattr(rt, fn).restype = ctypes.c_int
    rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    rt.cudaFree.argtypes = [ctypes.c_void_p]

    def call(fields):
        nf, nz, ny, nx = fields.shape
        out = np.empty((nf, nz, ny, nx // 2 + 1), np.complex128)
        din, dout = ctypes.c_void_p(), ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(din), fields.nbytes) == 0
        assert rt.cudaMalloc(ctypes.byref(dout), out.nbytes) == 0
        assert rt.cudaMemcpy(din, fields.ctypes.data, fields.nbytes, 1) == 0
        rc = f(din, dout, nx, ny, nz, nf, None)
        assert rc == 0, lib.laps_last_error(None)
        assert rt.cudaDeviceSynchronize() == 0
        assert rt.cudaMemcpy(out.ctypes.data, dout, out.nbytes, 2) == 0
        assert rt.cudaFree(din) == 0 and rt.cudaFree(dout) == 0
        return out

    rng = np.random.default_rng(7)
    fields = rng.standard_normal((2, 16, 32, 64))
    # the transform's definition: x r2c, y and z c2c, each axis divided by its length
    ref = np.fft.fftn(np.fft.rfft(fields, axis=-1), axes=(-3, -2)) / fields[0].size
    first = call(fields)
    assert rt.cudaDeviceReset() == 0
    second = call(fields)
    for got in (first, second):
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.array_equal(first, second)
    print("reset ok")
""")


def test_correct_after_a_device_reset():
    """cudaDeviceReset between two calls: the second call must use the arrays of the new
    context (the library looks their addresses up on every call, never from a cache)."""
    ffi.load()  # built before the child starts
    r = subprocess.run([sys.executable, "-c", _RESET_SCRIPT, str(ROOT)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "reset ok" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
