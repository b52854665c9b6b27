"""The closure's tensor-core convolutions against a float64 PyTorch conv3d on the CPU.

laps_conv3_forward runs a 3x3x3 periodic convolution in BF16 on tcgen05 with FP32
accumulation; the reference here is torch.nn.functional.conv3d on circularly padded inputs
in float64, fed the same BF16-rounded inputs and weights, so the only differences are the
FP32 accumulation order and the BF16 rounding of the output.  Bound: every element within
2^-7 of its reference value relative to (|ref| + 1e-2 rms(ref)) - one BF16 rounding is 2^-9.
Shapes cover the first layer (6 -> 32 channels, GELU), the hidden layers (32 -> 32), the
output layer (32 -> 12, linear), the input-gradient pass (flipped weights, GELU' gate) and
grids with many tiles per block (persistent blocks, alternating accumulators).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
F = torch.nn.functional

from laps_gb300 import closure  # noqa: E402

TOL = 2.0 ** -7


def _bf(t):
    return t.to(torch.bfloat16).to(torch.float64)


def _conv_ref(x, w, b=None):
    """float64 periodic cross-correlation: x (C, nz, ny, nx), w (co, ci, 3, 3, 3)."""
    xp = F.pad(x[None], (1, 1, 1, 1, 1, 1), mode="circular")
    y = F.conv3d(xp, w)[0]
    if b is not None:
        y = y + b[:, None, None, None]
    return y


def _gelu(z):
    return 0.5 * z * (1.0 + torch.erf(z / np.sqrt(2.0)))


def _check(got, ref):
    scale = ref.abs() + 1e-2 * ref.pow(2).mean().sqrt()
    err = ((got - ref).abs() / scale).max().item()
    assert err <= TOL, err


def _inputs(cin, cout, shape, seed):
    g = torch.Generator().manual_seed(seed)
    nx, ny, nz = shape
    x = _bf(torch.randn((cin, nz, ny, nx), generator=g, dtype=torch.float64))
    w = _bf(torch.randn((cout, cin, 3, 3, 3), generator=g, dtype=torch.float64) / np.sqrt(27 * cin))
    b = torch.randn(cout, generator=g, dtype=torch.float64) * 0.1
    return x, w, b


@pytest.mark.parametrize("cin,cout,act", [(6, 32, 1), (32, 32, 1), (32, 12, 0), (16, 16, 1)],
                         ids=["first_6_32_gelu", "hidden_32_32_gelu", "out_32_12_linear", "16_16_gelu"])
@pytest.mark.parametrize("shape", [(128, 8, 4), (256, 4, 6)], ids=["128x8x4", "256x4x6"])
def test_forward_matches_conv3d(cin, cout, act, shape):
    x, w, b = _inputs(cin, cout, shape, seed=cin * 100 + cout)
    cin_p, cout_p = closure.padded_channels(cin), closure.padded_channels(cout)
    dev = "cuda"
    xd = closure.to_padded(x.to(dev))
    wpk = closure.pack(w.to(dev).float(), cin_p, cout_p)
    zpre = torch.zeros((shape[2], shape[1], shape[0] + 2, cout_p), dtype=torch.bfloat16, device=dev)
    y = closure.conv3(xd, wpk, cout_p, bias=b.to(dev).float(), act=act, zpre=zpre if act == 1 else None)
    assert closure.status() == 0
    zref = _conv_ref(x, w, b.float().double())
    ref = _gelu(zref) if act == 1 else zref
    _check(closure.from_padded(y, cout).double().cpu(), ref)
    # the periodic halo holds the wrapped columns, the padded channels are zero
    yc = y.cpu()
    nx = shape[0]
    assert torch.equal(yc[:, :, 0], yc[:, :, nx]) and torch.equal(yc[:, :, nx + 1], yc[:, :, 1])
    assert (yc[..., cout:] == 0).all()
    if act == 1:
        _check(closure.from_padded(zpre, cout).double().cpu(), zref)


@pytest.mark.parametrize("cin,cout", [(32, 32), (32, 12), (6, 32)], ids=["32_32", "32_12", "6_32"])
def test_input_gradient_matches_autograd(cin, cout):
    """Flipped weights with the GELU' gate: d loss / d z_prev for y = conv(gelu(z_prev))."""
    shape = (128, 6, 5)
    nx, ny, nz = shape
    g = torch.Generator().manual_seed(7 + cin + cout)
    zprev = _bf(torch.randn((cin, nz, ny, nx), generator=g, dtype=torch.float64))
    w = _bf(torch.randn((cout, cin, 3, 3, 3), generator=g, dtype=torch.float64) / np.sqrt(27 * cin))
    up = _bf(torch.randn((cout, nz, ny, nx), generator=g, dtype=torch.float64))
    zr = zprev.clone().requires_grad_(True)
    y = _conv_ref(_gelu(zr), w)
    y.backward(up)
    ref = zr.grad.detach()
    cin_p, cout_p = closure.padded_channels(cin), closure.padded_channels(cout)
    dev = "cuda"
    wflip = closure.pack(w.to(dev).float(), cin_p, cout_p, flip=True)
    dz = closure.conv3(closure.to_padded(up.to(dev)), wflip, cin_p, act=2, gate=closure.to_padded(zprev.to(dev)))
    assert closure.status() == 0
    _check(closure.from_padded(dz, cin).double().cpu(), ref)


@pytest.mark.parametrize("cin,cout", [(32, 32), (32, 12), (6, 32), (16, 16)], ids=["32_32", "32_12", "6_32", "16_16"])
@pytest.mark.parametrize("shape", [(128, 6, 5), (64, 16, 4)], ids=["128x6x5", "64x16x4"])
def test_weight_gradient_matches_autograd(cin, cout, shape):
    """dW of y = conv(x) for an upstream gradient g, against torch's autograd in float64.
    The sum runs over every voxel in FP32 (several blocks adding partial sums), so the bound
    is relative to the largest entry: 1e-4."""
    nx, ny, nz = shape
    g = torch.Generator().manual_seed(3 + cin + cout)
    x = _bf(torch.randn((cin, nz, ny, nx), generator=g, dtype=torch.float64))
    w = torch.randn((cout, cin, 3, 3, 3), generator=g, dtype=torch.float64).requires_grad_(True)
    up = _bf(torch.randn((cout, nz, ny, nx), generator=g, dtype=torch.float64))
    _conv_ref(x, w).backward(up)
    ref = w.grad.detach()
    dev = "cuda"
    dw = closure.wgrad(closure.to_padded(x.to(dev)), closure.to_padded(up.to(dev)), cin, cout)
    assert closure.status() == 0
    err = ((dw.double().cpu() - ref).abs().max() / ref.abs().max()).item()
    assert err < 1e-4, err


def test_many_tiles_per_block():
    """A 128 x 128 x 24 grid: 3072 tiles, so every persistent block runs many tiles through
    both accumulators and wraps the stage ring many times; two calls in a row agree bitwise."""
    shape = (128, 128, 24)
    x, w, b = _inputs(32, 32, shape, seed=11)
    dev = "cuda"
    xd = closure.to_padded(x.to(dev))
    wpk = closure.pack(w.to(dev).float(), 32, 32)
    y1 = closure.conv3(xd, wpk, 32, bias=b.to(dev).float(), act=1)
    y2 = closure.conv3(xd, wpk, 32, bias=b.to(dev).float(), act=1)
    assert closure.status() == 0
    assert torch.equal(y1, y2)
    ref = _gelu(_conv_ref(x, w, b.float().double()))
    _check(closure.from_padded(y1, 32).double().cpu(), ref)


def test_rejects_bad_shapes():
    from laps_gb300 import ffi

    dev = "cuda"
    x = torch.zeros((4, 4, 66, 32), dtype=torch.bfloat16, device=dev)
    wpk = torch.zeros(27 * 32 * 32, dtype=torch.bfloat16, device=dev)
    with pytest.raises(ffi.LapsError):
        closure.conv3(x, wpk, 32)  # nx = 64 is not a multiple of 128


def test_net_gradients_match_autograd():
    """The whole 4-layer net (6 -> 32 -> 32 -> 32 -> 12, GELU) forward and backward through
    the C-ABI kernels against torch autograd of the same net in float64 on BF16-rounded
    inputs: output errors within 5e-3 of the output rms in rms (3e-2 at most), every weight and bias gradient within 3e-2 of the
    largest entry of its tensor (gradients pass through three BF16-rounded activations)."""
    shape = (128, 8, 6)
    nx, ny, nz = shape
    dev = "cuda"
    net = closure.ClosureNet(device=dev, seed=5)
    g = torch.Generator().manual_seed(9)
    x = _bf(torch.randn((6, nz, ny, nx), generator=g, dtype=torch.float64))
    target = torch.randn((12, nz, ny, nx), generator=g, dtype=torch.float64) * 0.1
    # reference: float64 autograd of the same net on the BF16-rounded weights
    ws = [_bf(w.detach().double().cpu()).requires_grad_(True) for w in net.w]
    bs = [b.detach().double().cpu().requires_grad_(True) for b in net.b]
    a = x
    for l, (cin, cout, act) in enumerate(closure.LAYERS):
        z = _conv_ref(a, ws[l], bs[l])
        a = _gelu(z) if act else z
    loss = ((a - target) ** 2).sum() / 2
    loss.backward()
    y = net.forward(closure.to_padded(x.to(dev)))
    yo = closure.from_padded(y, 12).double().cpu()
    # four layers of BF16-rounded activations: the error's rms within 5e-3 of the output's
    # rms, and its largest value over the ~7e4 outputs (a ~4.5 sigma tail) within 3e-2
    ref = a.detach()
    rms = ref.pow(2).mean().sqrt()
    assert ((yo - ref).pow(2).mean().sqrt() / rms).item() <= 5e-3
    assert ((yo - ref).abs().max() / rms).item() <= 3e-2
    dy = closure.to_padded((yo - target).to(dev))  # d loss / d y, BF16 padded with its halo
    net.backward(dy)
    assert closure.status() == 0
    for l in range(4):
        for got, ref in ((net.w[l].grad, ws[l].grad), (net.b[l].grad, bs[l].grad)):
            err = ((got.double().cpu() - ref).abs().max() / ref.abs().max()).item()
            assert err < 3e-2, (l, err)


def test_training_reduces_the_loss():
    """A few Adam steps on a fixed input/target pair through the tcgen05 kernels lower the loss."""
    shape = (128, 8, 4)
    nx, ny, nz = shape
    dev = "cuda"
    net = closure.ClosureNet(device=dev, seed=6)
    g = torch.Generator().manual_seed(10)
    x = closure.to_padded(torch.randn((6, nz, ny, nx), generator=g).to(dev))
    t = torch.randn((12, nz, ny, nx), generator=g).to(dev) * 0.3
    opt = torch.optim.Adam(net.parameters(), lr=3e-3)
    losses = []
    for _ in range(30):
        y = net.forward(x)
        r = closure.from_padded(y, 12) - t
        losses.append(float((r ** 2).mean()))
        net.backward(closure.to_padded(2 * r / r.numel()))
        opt.step()
        net.repack()
    assert closure.status() == 0
    assert losses[-1] < 0.7 * losses[0], losses
