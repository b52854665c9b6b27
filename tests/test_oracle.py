"""The oracle (CPU restatement of the reference) checked against definitions, known answers
and the committed golden fixtures.  No GPU."""
import math
from pathlib import Path

import numpy as np
import pytest

from laps_gb300.ic import alfven_wave_ic, turbulence_ic
from oracle import laps3d
from oracle.laps3d import Laps3DC, Params3D, forward_3d, inverse_3d, wave_numbers

GOLDEN = Path(__file__).resolve().parent / "golden"


def direct_forward(u):
    """O(N^2) DFT with the reference's per-axis 1/n normalisation, no FFT library."""
    nz, ny, nx = u.shape
    ex = np.exp(-2j * np.pi * np.outer(np.arange(nx // 2 + 1), np.arange(nx)) / nx) / nx
    ey = np.exp(-2j * np.pi * np.outer(np.arange(ny), np.arange(ny)) / ny) / ny
    ez = np.exp(-2j * np.pi * np.outer(np.arange(nz), np.arange(nz)) / nz) / nz
    w = np.einsum("kx,zyx->zyk", ex, u)
    w = np.einsum("ly,zyk->zlk", ey, w)
    return np.einsum("mz,zlk->mlk", ez, w)


def test_forward_matches_direct_dft():
    rng = np.random.default_rng(0)
    u = rng.standard_normal((8, 4, 16))
    assert np.abs(forward_3d(u) - direct_forward(u)).max() < 1e-15


def test_inverse_is_unnormalised_and_ignores_nyquist_imag():
    rng = np.random.default_rng(1)
    u = rng.standard_normal((8, 8, 16))
    w = forward_3d(u)
    assert np.abs(inverse_3d(w, 16) - u).max() < 1e-14
    w2 = w.copy()
    w2[0, 0, 0] += 3j  # c2r ignores Im of the kx = 0 and kx = nx/2 planes' (0,0) entries
    w2[0, 0, -1] += 5j
    assert np.abs(inverse_3d(w2, 16) - u).max() < 1e-14


def test_wave_numbers_nyquist_positive():
    k = wave_numbers(8, 2 * math.pi)
    assert list(k) == [0, 1, 2, 3, 4, -3, -2, -1]


def test_single_mode_coefficient():
    n = 16
    x = np.arange(n) * 2 * math.pi / n
    u = np.broadcast_to(np.cos(3 * x)[None, None, :], (n, n, n)).copy()
    w = forward_3d(u)
    assert abs(w[0, 0, 3] - 0.5) < 1e-15
    w[0, 0, 3] = 0
    assert np.abs(w).max() < 1e-15


def test_dealias_sphere():
    p = Params3D(nx=16, ny=16, nz=16, dealias_option=1)
    o = Laps3DC(p)
    mx = np.arange(9)[None, None, :]
    my = np.abs(np.fft.fftfreq(16, 1 / 16))[None, :, None]  # the Nyquist row has |m| = 8 either way
    mz = np.abs(np.fft.fftfreq(16, 1 / 16))[:, None, None]
    keep = (mx**2 + my**2 + mz**2) / 256.0 <= 1.0 / 9.0
    assert np.array_equal(o.keep, keep)


def test_rk_coefficients():
    o = Laps3DC(Params3D(nx=16, ny=8, nz=8))
    o.rkt_init(0.3)
    assert np.allclose(o.cc1, [8 / 15 * 0.3, 5 / 12 * 0.3, 0.75 * 0.3], rtol=0, atol=1e-17)
    assert np.allclose(o.dd1, [0, -17 / 60 * 0.3, -5 / 12 * 0.3], rtol=0, atol=1e-17)
    assert np.allclose(o.time_step, [8 / 15 * 0.3, 2 / 15 * 0.3, 1 / 3 * 0.3], rtol=0, atol=1e-17)


def test_vardt_hysteresis():
    prim = turbulence_ic(16, seed=2)
    o = laps3d.restart(16, dict(cfl=0.4), prim)
    d0 = o.vardt()
    o.dt = d0 * 1.015  # within +-2 %: kept
    assert o.vardt() == d0 * 1.015
    o.dt = d0 * 1.03  # outside: replaced
    assert o.vardt() == d0


def test_alfven_wave_known_answer():
    """ipert=1 (mhdinit.f90:328-342) is an exact nonlinear solution: it travels at v_A and
    decays as exp(-eta k^2 t) when eta = nu."""
    n, eta = 16, 1e-2
    kw = dict(if_resis=1, resistivity=eta, if_visc=1, viscosity=eta, dealias_option=1, cfl=0.05)
    o = laps3d.restart(n, kw, alfven_wave_ic(n, db0=0.1))
    for _ in range(40):
        o.vardt(); o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    x = np.arange(n) * (2 * math.pi / n)
    dec = math.exp(-eta * o.time)
    assert np.abs(o.uu[6] + 0.1 * np.sin(x - o.time) * dec).max() < 1e-5
    assert np.abs(o.uu[5] + 0.1 * np.cos(x - o.time) * dec).max() < 1e-5


def test_force_free_field_decays_by_the_implicit_factor():
    """A Beltrami field B = (sin z, cos z, 0) with u = 0 is force-free (J = B) and keeps a
    uniform total pressure, so only resistivity acts: every RK stage divides the k = 1 modes by
    1 + ts_i eta k^2 with ts = (8/15, 2/15, 1/3) dt (rktmod.f90:34-62, implicit branch), and the
    field after the steps is the initial one times the product of those factors, to round-off.
    The flow stays at rest."""
    n, eta = 16, 0.05
    z = np.arange(n) * (2 * math.pi / n)
    prim = np.zeros((8, n, n, n))
    prim[0] = 1.0
    prim[4] = np.sin(z)[:, None, None]
    prim[5] = np.cos(z)[:, None, None]
    prim[7] = 0.5
    kw = dict(if_resis=1, resistivity=eta, dealias_option=1, cfl=0.3)
    o = laps3d.restart(n, kw, prim)
    amp = 1.0
    for _ in range(10):
        o.vardt()
        for ts in (8.0 / 15.0, 2.0 / 15.0, 1.0 / 3.0):
            amp /= 1.0 + ts * o.dt * eta
        o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    assert amp < 0.99
    assert np.abs(o.uu[4] - amp * prim[4]).max() < 1e-13
    assert np.abs(o.uu[5] - amp * prim[5]).max() < 1e-13
    assert np.abs(o.uu[1:4]).max() < 1e-13


def test_beltrami_flow_decays_by_the_implicit_viscous_factor():
    """u = (sin z, cos z, 0) with B = 0 and uniform density: no advection (u . grad u = 0),
    a uniform |u| and total energy, hence a uniform pressure, so viscosity is all that acts on
    the momentum: each RK stage divides its k = 1 modes by 1 + ts_i nu k^2 (rktmod.f90:34-62),
    to round-off."""
    n, nu = 16, 0.05
    z = np.arange(n) * (2 * math.pi / n)
    prim = np.zeros((8, n, n, n))
    prim[0] = 1.0
    prim[1] = np.sin(z)[:, None, None]
    prim[2] = np.cos(z)[:, None, None]
    prim[7] = 0.5
    o = laps3d.restart(n, dict(if_visc=1, viscosity=nu, dealias_option=1, cfl=0.3), prim)
    amp = 1.0
    for _ in range(10):
        o.vardt()
        for ts in (8.0 / 15.0, 2.0 / 15.0, 1.0 / 3.0):
            amp /= 1.0 + ts * o.dt * nu
        o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    assert amp < 0.99
    assert np.abs(o.uu[1] - amp * prim[1]).max() < 1e-13
    assert np.abs(o.uu[2] - amp * prim[2]).max() < 1e-13
    assert np.abs(o.uu[3]).max() < 1e-13 and np.abs(o.uu[4:7]).max() < 1e-13
    assert np.abs(o.uu[0] - 1.0).max() < 1e-13


def test_conservation_ideal():
    """Mean density, momentum, field and total energy are invariants of the ideal equations."""
    prim = turbulence_ic(16, seed=4, rms_u=0.3, rms_b=0.3, kmax=3)
    o = laps3d.restart(16, dict(dealias_option=1, cfl=0.3), prim)
    m0 = o.uu.mean(axis=(1, 2, 3))
    for _ in range(5):
        o.vardt(); o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    m1 = o.uu.mean(axis=(1, 2, 3))
    assert np.abs(m1 - m0).max() < 1e-13
    assert o.calc_max_divB() < 1e-13


def test_expanding_box_scalings():
    """<rho> ~ (R0/R)^2, <Bx> ~ (R0/R)^2, <By>,<Bz> ~ R0/R: the checks of the reference's own
    rms reader (data_process/3D_Python/read_rms.py:58-66).  The k = 0 modes evolve linearly
    (d/dt = -c / tau with tau frozen at the step start, mhdrhs.f90:235-247), so each step
    multiplies them by RK3's amplification 1 + z + z^2/2 + z^3/6, z = -c dt / tau_n: exact to
    round-off.  Against the continuous law the scheme is first order in dt Ur / R."""
    prim = turbulence_ic(16, seed=5, rms_u=0.1, rms_b=0.1, kmax=3, B0=(1.0, 0.5, 0.2))
    kw = dict(if_AEB=1, radius0=30.0, Ur0=3.0, dealias_option=1, cfl=0.3)
    o = laps3d.restart(16, kw, prim)
    r0 = o.uu[[0, 4, 5, 6]].mean(axis=(1, 2, 3))
    c = np.array([2.0, 2.0, 1.0, 1.0])
    amp = np.ones(4)
    bound = 0.0
    for _ in range(10):
        tau = o.tau_exp
        o.vardt()
        z = -c * o.dt / tau
        amp *= 1 + z + z**2 / 2 + z**3 / 6
        bound += 2 * (o.dt * 3.0 / o.radius) ** 2
        o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    r1 = o.uu[[0, 4, 5, 6]].mean(axis=(1, 2, 3))
    assert np.abs(r1 / (r0 * amp) - 1).max() < 1e-13
    ratio = 30.0 / o.radius
    expect = r0 * np.array([ratio**2, ratio**2, ratio, ratio])
    assert np.abs(r1 / expect - 1).max() < 1.5 * bound


@pytest.mark.parametrize("path", sorted(GOLDEN.glob("c*.npz")), ids=lambda p: p.stem)
def test_golden_fixture(path):
    g = np.load(path)
    shape = tuple(int(v) for v in g["shape"])
    kw = eval(str(g["params"]))  # a dict literal written by make_golden.py
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    o = mg.start(shape, kw, g["prim"])
    for _ in range(int(g["steps"])):
        o.step()
    assert abs(o.time - float(g["time"])) <= 1e-13 * o.time
    for f in range(8):
        assert np.linalg.norm(o.uu[f] - g["uu"][f]) <= 1e-12 * max(np.linalg.norm(g["uu"][f]), 1e-300)
    assert np.allclose(o.invariants(), g["inv"], rtol=1e-11, atol=1e-15)


def test_shell_spectra_parseval_and_single_mode():
    """The shells of the oracle's spectrum sum to <u^2>/2 and <B^2>/2 (Parseval, half
    spectrum weights), and a single Fourier mode lands in its own shell."""
    from laps_gb300.ic import turbulence_ic
    from oracle import laps3d

    prim = turbulence_ic((16, 8, 4), seed=5)
    o = laps3d.restart((16, 8, 4), {}, prim)
    eu, eb = laps3d.shell_spectra(o.uu, 2 * np.pi, 2 * np.pi, 2 * np.pi, 32)
    u = o.uu[1:4] / o.uu[0]
    assert abs(eu.sum() - 0.5 * np.mean(np.sum(u ** 2, axis=0))) < 1e-14
    assert abs(eb.sum() - 0.5 * np.mean(np.sum(o.uu[4:7] ** 2, axis=0))) < 1e-14
    n = 16
    x = np.arange(n) * 2 * np.pi / n
    uu = np.zeros((8, n, n, n))
    uu[0] = 1.0
    uu[4] = np.cos(3 * x)[None, None, :]            # |k| = 3, energy 1/4
    uu[5] = np.sin(4 * x)[None, :, None]            # |k| = 4, energy 1/4
    _, eb = laps3d.shell_spectra(uu, 2 * np.pi, 2 * np.pi, 2 * np.pi, 8)
    assert np.allclose(eb, [0, 0, 0, 0.25, 0.25, 0, 0, 0], atol=1e-15)


def test_output_file_layout(tmp_path):
    """The restated outNNN.dat: 12-byte time record (markers 4, float32), then float64 data in
    Fortran order; a read gives back the array and the time rounded to float32."""
    from oracle import outfile

    rng = np.random.default_rng(3)
    uu = rng.standard_normal((8, 4, 3, 16))
    raw = outfile.write_output(tmp_path / outfile.output_name(7), uu, 1.2345678901)
    assert outfile.output_name(7) == "out007.dat" and outfile.output_name(123) == "out123.dat"
    assert len(raw) == 12 + 8 * uu.size
    assert raw[:4] == b"\x04\x00\x00\x00" and raw[8:12] == b"\x04\x00\x00\x00"
    assert np.frombuffer(raw[12:20], "<f8")[0] == uu[0, 0, 0, 0]   # x fastest
    assert np.frombuffer(raw[20:28], "<f8")[0] == uu[0, 0, 0, 1]
    t, back = outfile.read_output(tmp_path / "out007.dat", (16, 3, 4))
    assert np.array_equal(back, uu) and t == float(np.float32(1.2345678901))
