"""The closure's data path on the device against numpy definitions, through the C-ABI.

laps_closure_filter (box means and the subgrid stress / electromotive force), the net's
input packing and output unpacking, laps_closure_forcing (-(i k . tau) projected, i k x eps),
laps_add_spectral_device (uu_fourier += scale f, then the 2/3 mask) and a few closed steps of
a coarse incompressible run.  Tolerances: float64 results 1e-12 relative to the largest
value; float32 targets 1e-6; BF16 packing one BF16 rounding (2^-8 relative).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from laps_gb300 import closure, ffi  # noqa: E402
from laps_gb300.ic import turbulence_ic  # noqa: E402
from oracle.laps3d import Laps3DC, Params3D  # noqa: E402


def _random_state(n, seed):
    rng = np.random.default_rng(seed)
    s = rng.standard_normal((8, n, n, n))
    s[0] = 1.0 + 0.2 * rng.random((n, n, n))  # a positive density
    return s


def test_filter_matches_numpy():
    nf, r = 16, 4
    m = nf // r
    s = _random_state(nf, 1)
    coarse, tgt = closure.filter_state(torch.from_numpy(s).cuda(), r)
    coarse, tgt = coarse.cpu().numpy(), tgt.cpu().numpy()
    blk = lambda a: a.reshape(m, r, m, r, m, r).mean(axis=(1, 3, 5))
    ref = np.stack([blk(s[f]) for f in range(8)])
    assert np.abs(coarse - ref).max() <= 1e-12 * np.abs(ref).max()
    u = s[1:4] / s[0]
    b = s[4:7]
    ub, bb = [blk(x) for x in u], [blk(x) for x in b]
    want = []
    for a in range(3):
        for e in range(a, 3):
            want.append((blk(u[a] * u[e]) - ub[a] * ub[e]) - (blk(b[a] * b[e]) - bb[a] * bb[e]))
    cr = np.cross(u, b, axis=0)
    cb = np.cross(np.stack(ub), np.stack(bb), axis=0)
    for a in range(3):
        want.append(blk(cr[a]) - cb[a])
    want = np.stack(want)
    assert np.abs(tgt[:9] - want).max() <= 1e-6 * np.abs(want).max()
    assert (tgt[9:] == 0).all()


def test_pack_and_unpack():
    n = 8
    s = _random_state(n, 2)
    su, sb = 0.7, 1.3
    x = closure.pack_input(torch.from_numpy(s).cuda(), su, sb)
    got = closure.from_padded(x, 6).double().cpu().numpy()
    want = np.concatenate([s[1:4] / s[0] / su, s[4:7] / sb])
    assert np.abs(got - want).max() <= 2.0 ** -8 * np.abs(want).max()
    xc = x.cpu()
    assert torch.equal(xc[:, :, 0], xc[:, :, n]) and torch.equal(xc[:, :, n + 1], xc[:, :, 1])
    assert (xc[..., 6:] == 0).all()
    y = torch.randn((n, n, n + 2, 16), device="cuda").to(torch.bfloat16)
    tau = torch.empty((12, n, n, n), dtype=torch.float64, device="cuda")
    assert closure._lib().laps_closure_unpack_output(y.data_ptr(), tau.data_ptr(), n, 2.5, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(tau.cpu(), 2.5 * closure.from_padded(y, 12).double().cpu())


def test_forcing_matches_numpy():
    n = 16
    nh = n // 2 + 1
    rng = np.random.default_rng(3)
    ts = rng.standard_normal((12, n, n, nh)) + 1j * rng.standard_normal((12, n, n, nh))
    f = torch.empty((8, n, n, nh), dtype=torch.complex128, device="cuda")
    tsd = torch.from_numpy(ts).cuda()
    assert closure._lib().laps_closure_forcing(tsd.data_ptr(), f.data_ptr(), n, None) == 0
    got = f.cpu().numpy()
    m = np.arange(n)
    kk = np.where(m <= n // 2, m, m - n).astype(float)
    kx = kk[:nh][None, None, :]
    ky = kk[None, :, None]
    kz = kk[:, None, None]
    k = [kx, ky, kz]
    T = [[ts[0], ts[1], ts[2]], [ts[1], ts[3], ts[4]], [ts[2], ts[4], ts[5]]]
    fm = [-1j * (k[0] * T[a][0] + k[1] * T[a][1] + k[2] * T[a][2]) for a in range(3)]
    k2 = kx**2 + ky**2 + kz**2
    with np.errstate(invalid="ignore", divide="ignore"):
        d = (k[0] * fm[0] + k[1] * fm[1] + k[2] * fm[2]) / k2
    fm = [np.where(k2 > 0, fm[a] - k[a] * d, 0) for a in range(3)]
    e = [ts[6 + a] + ts[9 + a] for a in range(3)]
    g = [1j * (k[1] * e[2] - k[2] * e[1]), 1j * (k[2] * e[0] - k[0] * e[2]), 1j * (k[0] * e[1] - k[1] * e[0])]
    want = np.stack([np.zeros_like(ts[0])] + fm + g + [np.zeros_like(ts[0])])
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_add_spectral_device_then_mask():
    n = 16
    kw = dict(if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4, dealias_option=1, cfl=0.4, rho0=1.0)
    prim = turbulence_ic(n, seed=4, kmax=3, rms_u=0.3, rms_b=0.3, p0=1.0)
    g = ffi.Laps(ffi.params(nx=n, ny=n, nz=n, variant=ffi.VARIANT_3DI, precision=ffi.PREC_FP64, **kw))
    g.upload_state(prim, primitive=True)
    uf0 = g.download_spectral()
    rng = np.random.default_rng(5)
    f = rng.standard_normal(uf0.shape) + 1j * rng.standard_normal(uf0.shape)
    fd = torch.from_numpy(np.ascontiguousarray(f)).cuda()
    assert closure._lib().laps_add_spectral_device(g.h, fd.data_ptr(), 0.25) == 0
    uf1 = g.download_spectral()
    g.close()
    p = Params3D(nx=n, ny=n, nz=n, dealias_option=1)
    keep = Laps3DC(p).keep
    want = np.where(keep[None], uf0 + 0.25 * f, 0)
    assert np.abs(uf1 - want).max() <= 1e-13 * np.abs(want).max()


def test_closed_steps_stay_finite():
    """An untrained closure with a small output scale: three closed steps of a 128^3 run, the
    state finite and within 1e-3 of the unclosed run's."""
    n = 128
    kw = dict(if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4, dealias_option=1, cfl=0.4, rho0=1.0)
    prim = turbulence_ic(n, seed=6, kmax=6, rms_u=0.5, rms_b=0.5, p0=1.0)
    model = closure.Closure(closure.ClosureNet(device="cuda", seed=1), 0.5, 1.0, 1e-4)
    out = {}
    for name in ("closed", "plain"):
        g = ffi.Laps(ffi.params(nx=n, ny=n, nz=n, variant=ffi.VARIANT_3DI, precision=ffi.PREC_FP64, **kw))
        g.upload_state(prim, primitive=True)
        g.set_time(0.0)
        for _ in range(3):
            t, dt, st = closure.closed_step(g, model, n) if name == "closed" else g.step(1)
            assert st == 0
        out[name] = g.download_spectral()
        g.close()
    assert closure.status() == 0
    assert np.isfinite(out["closed"]).all()
    d = np.abs(out["closed"] - out["plain"]).max() / np.abs(out["plain"]).max()
    assert 0 < d < 1e-3, d
