"""The allocation-free forward transform against the context-owning path.

laps_transform_uu_real_to_fourier_noalloc serves callers that cannot call cudaMalloc
(device memory owned by their own pool or framework, or allocation forbidden after start-up):
they pass device buffers they already own and the library keeps its one intermediate
spectrum in a fixed device array.  Here its output must equal what laps_upload_state +
laps_download_spectral produce for the same fields, within the transform tolerance the other
tests use (1e-14 of the largest coefficient), on two calls in a row that share that array.
Device buffers come from torch.  This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from laps_gb300 import ffi

pytestmark = pytest.mark.gpu


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


def test_two_calls_match_the_context_path():
    lib, f = _fn()
    rng = np.random.default_rng(42)
    for shape, nf in (((32, 16, 8), 8), ((64, 32, 32), 3)):
        nx, ny, nz = shape
        fields = rng.standard_normal((nf, nz, ny, nx))
        rc, got = _noalloc(f, fields, shape)
        assert rc == 0, lib.laps_last_error(None)
        ref = _reference_path(fields, shape)
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()


def test_rejects_grids_beyond_the_fixed_scratch():
    lib, f = _fn()
    torch = pytest.importorskip("torch")
    buf = torch.empty(16, dtype=torch.float64, device="cuda")
    rc = f(buf.data_ptr(), buf.data_ptr(), 512, 512, 512, 1, None)
    assert rc == ffi.LAPS_EINVAL
    assert b"scratch" in lib.laps_last_error(None)
