"""Execution schedules (laps_set_schedule) on the GPU: every schedule gives bit-identical
states (the schedules change launch plans, not arithmetic), the autotuner picks one of them
and caches it, and an ensemble whose member changes schedule between steps recaptures its
graph and still equals the member advanced alone."""
import numpy as np
import pytest

from laps_gb300 import autotune, ffi

from pairs import CONFIG2, turb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [ffi.PREC_FP32_F64, ffi.PREC_FP32, ffi.PREC_DD], ids=["fp32_f64", "fp32_dd", "dd"])
def test_every_schedule_gives_the_same_state(prec):
    shape = (64, 128, 32)
    prim = turb(shape, seed=51, kmax=4, rms_u=0.3, rms_b=0.3)
    out = {}
    for bits in autotune.CANDIDATES:
        g = ffi.Laps(ffi.params(nx=shape[0], ny=shape[1], nz=shape[2], precision=prec, **CONFIG2))
        g.upload_state(prim, primitive=True)
        g.set_time(0.0)
        g.set_schedule(bits)
        assert g.schedule() == bits
        t, dt, st = g.step(4)
        assert st == 0
        out[bits] = (g.download_spectral(), t)
        g.close()
    for bits in autotune.CANDIDATES:
        assert np.array_equal(out[bits][0], out[0][0]), bits
        assert out[bits][1] == out[0][1]


def test_autotune_picks_and_caches(tmp_path):
    prim = turb(64, seed=52, kmax=4, rms_u=0.3, rms_b=0.3)
    g = ffi.Laps(ffi.params(nx=64, ny=64, nz=64, precision=ffi.PREC_FP32_F64, **CONFIG2))
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    g.step(1)
    cache = {}
    r = autotune.tune(g, steps=2, cache=cache)
    assert r["bits"] in autotune.CANDIDATES and g.schedule() == r["bits"] and not r["from_cache"]
    assert len(r["times_ms"]) == len(autotune.CANDIDATES) and all(v > 0 for v in r["times_ms"].values())
    r2 = autotune.tune(g, cache=cache)
    assert r2["from_cache"] and r2["bits"] == r["bits"]
    with pytest.raises(ffi.LapsError):
        g.set_schedule(99)
    g.close()


def test_batch_recaptures_after_a_schedule_change():
    prim = turb(32, seed=53, kmax=4, rms_u=0.3, rms_b=0.3)
    p = ffi.params(nx=32, ny=32, nz=32, precision=ffi.PREC_FP32_F64, **CONFIG2)
    b = ffi.Batch([p, p])
    for m in b.members:
        m.upload_state(prim, primitive=True)
        m.set_time(0.0)
    b.step(3)
    b.members[1].set_schedule(ffi.SCHED_ALL)
    t, dt, st = b.step(3)
    assert (st == 0).all()
    solo = ffi.Laps(p)
    solo.upload_state(prim, primitive=True)
    solo.set_time(0.0)
    solo.step(6)
    for m in b.members:
        assert np.array_equal(m.download_spectral(), solo.download_spectral())
    solo.close()
    b.close()
