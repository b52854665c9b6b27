"""Host side of the learned subgrid closure's convolutions (``laps_conv3_*`` in the C-ABI).

The layers run in ``liblaps_gpu.so`` (tcgen05 BF16 kernels); torch supplies device memory and
the stream.  Activations live in the kernels' layout: channels-last BF16 with a one-voxel
periodic halo on x, shape ``(nz, ny, nx + 2, C)`` with C = 16 or 32.
"""
from __future__ import annotations

import ctypes as C

from . import ffi

_bound = False


def _lib():
    global _bound
    lib = ffi.load()
    if not _bound:
        vp, i = C.c_void_p, C.c_int
        lib.laps_conv3_pack.restype = i
        lib.laps_conv3_pack.argtypes = [vp, vp, i, i, i, i, i, vp]
        lib.laps_conv3_forward.restype = i
        lib.laps_conv3_forward.argtypes = [vp, vp, vp, vp, vp, vp, i, i, i, i, i, i, vp]
        lib.laps_conv3_wgrad.restype = i
        lib.laps_conv3_wgrad.argtypes = [vp, vp, vp, i, i, i, i, i, vp]
        lib.laps_conv3_status.restype = i
        lib.laps_conv3_status.argtypes = [vp, C.POINTER(i)]
        _bound = True
    return lib


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def _ck(rc):
    if rc != ffi.LAPS_OK:
        raise ffi.LapsError(rc, ffi.load().laps_last_error(None).decode())


def padded_channels(c: int) -> int:
    if c > 32:
        raise ValueError("at most 32 channels")
    return 16 if c <= 16 else 32


def to_padded(x):
    """(C, nz, ny, nx) tensor -> the kernels' layout (nz, ny, nx + 2, Cp) in BF16."""
    import torch

    c, nz, ny, nx = x.shape
    cp = padded_channels(c)
    out = torch.zeros((nz, ny, nx + 2, cp), dtype=torch.bfloat16, device=x.device)
    v = x.permute(1, 2, 3, 0).to(torch.bfloat16)
    out[:, :, 1:nx + 1, :c] = v
    out[:, :, 0, :c] = v[:, :, nx - 1]
    out[:, :, nx + 1, :c] = v[:, :, 0]
    return out


def from_padded(y, c: int):
    """The kernels' layout -> (c, nz, ny, nx) float32 (interior only)."""
    nx = y.shape[2] - 2
    return y[:, :, 1:nx + 1, :c].permute(3, 0, 1, 2).float()


def pack(w, cin_p: int, cout_p: int, flip: bool = False):
    """Weights (cout, cin, 3, 3, 3) float32 -> packed BF16 operand of one layer."""
    import torch

    w = w.detach().float().contiguous()
    cout, cin = w.shape[:2]
    out = torch.empty(27 * cin_p * cout_p, dtype=torch.bfloat16, device=w.device)
    _ck(_lib().laps_conv3_pack(w.data_ptr(), out.data_ptr(), cin, cout, cin_p, cout_p, int(flip), _stream()))
    return out


def conv3(x, wpk, cout_p: int, bias=None, act: int = 0, zpre=None, gate=None, out=None):
    """One layer on padded activations x (nz, ny, nx + 2, Cin_p): act 0 linear, 1 GELU (the
    pre-activation into zpre when given), 2 times GELU'(gate).  Returns y (nz, ny, nx + 2, cout_p)."""
    import torch

    nz, ny, nxp, cin_p = x.shape
    nx = nxp - 2
    y = out if out is not None else torch.empty((nz, ny, nxp, cout_p), dtype=torch.bfloat16, device=x.device)
    b = None
    if bias is not None:  # the kernels read cout_p entries: zeros past the layer's channels
        b = torch.zeros(cout_p, dtype=torch.float32, device=x.device)
        b[: bias.numel()] = bias.float()
    _ck(_lib().laps_conv3_forward(x.data_ptr(), wpk.data_ptr(), b.data_ptr() if b is not None else None, y.data_ptr(),
                                  zpre.data_ptr() if zpre is not None else None,
                                  gate.data_ptr() if gate is not None else None, nx, ny, nz, cin_p, cout_p, act,
                                  _stream()))
    return y


def wgrad(x, dz, cin: int, cout: int):
    """Weight gradient of a layer y = conv(x): x (nz, ny, nx + 2, Cin_p) its input, dz the
    gradient at its pre-activation output (nz, ny, nx + 2, Cout_p).  Returns (cout, cin, 3, 3, 3)
    float32 in torch's Conv3d order."""
    import torch

    nz, ny, nxp, cin_p = x.shape
    cout_p = dz.shape[3]
    dw = torch.empty((27, cout_p, cin_p), dtype=torch.float32, device=x.device)
    _ck(_lib().laps_conv3_wgrad(x.data_ptr(), dz.data_ptr(), dw.data_ptr(), nxp - 2, ny, nz, cin_p, cout_p, _stream()))
    return dw[:, :cout, :cin].permute(1, 2, 0).reshape(cout, cin, 3, 3, 3)


def status() -> int:
    """Wait for the stream; 1 when a bounded wait inside a convolution ran out (error word cleared)."""
    e = C.c_int(0)
    _ck(_lib().laps_conv3_status(_stream(), C.byref(e)))
    return e.value
