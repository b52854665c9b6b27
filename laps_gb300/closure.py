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
        d = C.c_double
        lib.laps_closure_filter.restype = i
        lib.laps_closure_filter.argtypes = [vp, i, i, vp, vp, vp]
        lib.laps_closure_pack_input.restype = i
        lib.laps_closure_pack_input.argtypes = [vp, vp, i, d, d, vp]
        lib.laps_closure_unpack_output.restype = i
        lib.laps_closure_unpack_output.argtypes = [vp, vp, i, d, vp]
        lib.laps_closure_forcing.restype = i
        lib.laps_closure_forcing.argtypes = [vp, vp, i, vp]
        lib.laps_state_real_device.restype = i
        lib.laps_state_real_device.argtypes = [vp, vp]
        lib.laps_add_spectral_device.restype = i
        lib.laps_add_spectral_device.argtypes = [vp, vp, d]
        lib.laps_transform_uu_real_to_fourier_noalloc.restype = i
        lib.laps_transform_uu_real_to_fourier_noalloc.argtypes = [vp, vp, i, i, i, i, vp]
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


# ------------------------------------------------------------------------------ the net
LAYERS = ((6, 32, 1), (32, 32, 1), (32, 32, 1), (32, 12, 0))  # (in, out, GELU) per layer


class ClosureNet:
    """The subgrid-stress net: 4 periodic 3x3x3 convolutions (6 -> 32 -> 32 -> 32 -> 12,
    GELU between them) run by the tcgen05 kernels in BF16 with FP32 accumulation.  Master
    weights and biases are FP32 torch tensors; `forward` keeps what `backward` needs (the
    layer inputs and pre-activations, in the kernels' padded layout) and `backward` returns
    the FP32 gradients of every weight and bias for the gradient at the output."""

    def __init__(self, device="cuda", seed=0, layers=LAYERS):
        import torch

        g = torch.Generator().manual_seed(seed)
        self.layers = layers
        self.w, self.b = [], []
        for cin, cout, _ in layers:
            w = torch.randn((cout, cin, 3, 3, 3), generator=g) * (2.0 / (27 * cin)) ** 0.5
            self.w.append(w.to(device).requires_grad_(True))
            self.b.append(torch.zeros(cout, device=device).requires_grad_(True))
        self.device = device
        self.repack()

    def parameters(self):
        return self.w + self.b

    def repack(self):
        """BF16 operands of the current master weights (forward and input-gradient forms)."""
        self.pk, self.pkf = [], []
        for (cin, cout, _), w in zip(self.layers, self.w):
            ci, co = padded_channels(cin), padded_channels(cout)
            self.pk.append(pack(w, ci, co))
            self.pkf.append(pack(w, ci, co, flip=True))

    def forward(self, x, keep=True):
        """x: (nz, ny, nx + 2, 16) padded BF16 input.  Returns the padded output (16 channels,
        12 used).  keep=False (inference) skips the pre-activations backward needs."""
        import torch

        self.acts, self.pre = [x], []
        a = x
        for l, (cin, cout, act) in enumerate(self.layers):
            co = padded_channels(cout)
            z = torch.empty(a.shape[:3] + (co,), dtype=torch.bfloat16, device=a.device) if act and keep else None
            a = conv3(a, self.pk[l], co, bias=self.b[l].detach(), act=act, zpre=z)
            self.pre.append(z)
            self.acts.append(a)
        return a

    def backward(self, dy):
        """dy: gradient at the output, padded layout (halo filled).  Sets .grad of every
        weight and bias (FP32)."""
        g = dy
        for l in range(len(self.layers) - 1, -1, -1):
            cin, cout, _ = self.layers[l]
            nx = g.shape[2] - 2
            self.w[l].grad = wgrad(self.acts[l], g, cin, cout).contiguous()
            self.b[l].grad = g[:, :, 1:nx + 1, :cout].float().sum(dim=(0, 1, 2))
            if l > 0:  # through this layer's input and the previous activation's GELU
                ci = padded_channels(cin)
                g = conv3(g, self.pkf[l], ci, act=2, gate=self.pre[l - 1])
        return g


# ------------------------------------------------------------------------------ the study
def state_real(run, out=None):
    """The conserved real state of a run, (8, n, n, n) float64 on the device."""
    import torch

    nz, ny, nx = run.shape
    out = out if out is not None else torch.empty((8, nz, ny, nx), dtype=torch.float64, device="cuda")
    run._ck(_lib().laps_state_real_device(run.h, out.data_ptr()))
    return out


def filter_state(fine, ratio):
    """Box filter + sampling of a fine (8, n, n, n) state: (coarse state (8, m, m, m) float64,
    targets (12, m, m, m) float32), m = n / ratio."""
    import torch

    n = fine.shape[-1]
    m = n // ratio
    coarse = torch.empty((8, m, m, m), dtype=torch.float64, device=fine.device)
    tgt = torch.empty((12, m, m, m), dtype=torch.float32, device=fine.device)
    _ck(_lib().laps_closure_filter(fine.data_ptr(), n, ratio, coarse.data_ptr(), tgt.data_ptr(), _stream()))
    return coarse, tgt


def pack_input(state, su, sb, out=None):
    import torch

    n = state.shape[-1]
    x = out if out is not None else torch.zeros((n, n, n + 2, 16), dtype=torch.bfloat16, device=state.device)
    _ck(_lib().laps_closure_pack_input(state.data_ptr(), x.data_ptr(), n, su, sb, _stream()))
    return x


class Closure:
    """A trained net with its normalisation: inputs u / su and b / sb, outputs times st."""

    def __init__(self, net, su, sb, st):
        self.net, self.su, self.sb, self.st = net, su, sb, st

    def forcing(self, state, n):
        """The closure's right-hand side (8 spectral fields, laps_download_spectral layout) of a
        coarse state (8, n, n, n) on the device."""
        import torch

        lib = _lib()
        x = pack_input(state, self.su, self.sb)
        y = self.net.forward(x, keep=False)
        tau = torch.empty((12, n, n, n), dtype=torch.float64, device=state.device)
        _ck(lib.laps_closure_unpack_output(y.data_ptr(), tau.data_ptr(), n, self.st, _stream()))
        ts = torch.empty((12, n, n, n // 2 + 1), dtype=torch.complex128, device=state.device)
        _ck(lib.laps_transform_uu_real_to_fourier_noalloc(tau.data_ptr(), ts.data_ptr(), n, n, n, 12, _stream()))
        f = torch.empty((8, n, n, n // 2 + 1), dtype=torch.complex128, device=state.device)
        _ck(lib.laps_closure_forcing(ts.data_ptr(), f.data_ptr(), n, _stream()))
        return f


def closed_step(run, closure, n, buf=None):
    """One step of a coarse run with the closure: the solver's step (laps_step), then the
    closure's right-hand side of the new state added over the step's dt (operator splitting,
    explicit), followed by the dealias mask.  Returns (time, dt, status)."""
    import torch

    t, dt, st = run.step(1)
    if st != 0:
        return t, dt, st
    state = state_real(run, buf)
    f = closure.forcing(state, n)
    torch.cuda.current_stream().synchronize()  # the engine's stream reads f next
    run._ck(_lib().laps_add_spectral_device(run.h, f.data_ptr(), dt))
    return t, dt, st
