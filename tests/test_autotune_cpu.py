"""The schedule autotuner's host logic without a GPU: the cache key, the choice (fastest,
ties to the smaller bit pattern), the on-disk cache round trip, and a tuning pass over a
stand-in run that times candidates once and then answers from the cache."""
import numpy as np

from laps_gb300 import autotune, ffi


class FakeRun:
    """Duck-typed run: each schedule's 'step time' from a table."""

    def __init__(self, ms):
        self.p = ffi.laps_params()
        self.p.nx, self.p.ny, self.p.nz, self.p.precision = 256, 256, 256, ffi.PREC_FP32_F64
        self.ms = ms
        self.bits = 0
        self.profiled = 0

    def set_schedule(self, b):
        self.bits = b

    def step(self, n):
        return 0.0, 0.0, 0

    def step_profiled(self, n):
        self.profiled += 1
        return np.zeros(6), self.ms[self.bits] * n, 0


def test_choose_prefers_fastest_then_default():
    assert autotune.choose({0: 5.0, 1: 4.0, 2: 4.5}) == 1
    assert autotune.choose({3: 4.0, 0: 4.0}) == 0


def test_tune_times_once_then_uses_the_cache(tmp_path):
    path = tmp_path / "s.json"
    ms = {b: 5.0 + 0.1 * b for b in autotune.CANDIDATES}
    ms[4] = 4.2
    run = FakeRun(ms)
    cache = autotune.load_cache(path)
    r = autotune.tune(run, steps=2, cache=cache, name="GB300-test")
    autotune.save_cache(cache, path)
    assert r["bits"] == 4 and run.bits == 4 and not r["from_cache"]
    assert run.profiled == len(autotune.CANDIDATES)
    run2 = FakeRun(ms)
    r2 = autotune.tune(run2, cache=autotune.load_cache(path), name="GB300-test")
    assert r2["from_cache"] and r2["bits"] == 4 and run2.bits == 4 and run2.profiled == 0
    assert autotune.key(run.p, "other") != r["key"]
