"""Bounded host waits: a call whose device work outlasts the run's timeout_ms returns
LAPS_ETIMEDOUT at about the timeout instead of blocking until the work ends; the queued work
still completes, laps_wait drains it, and the run continues with a clean status.  (Nothing on
the device is made to fail: the steps simply take longer than the timeout.)"""
import time

import pytest

from laps_gb300 import ffi
from laps_gb300.ic import turbulence_ic

from pairs import CONFIG2

pytestmark = pytest.mark.gpu


def test_step_times_out_promptly_and_the_run_continues():
    n = 128
    tmo = 300  # ms; 128^3 FP64 steps take ~10 ms each, the upload well under the timeout
    g = ffi.Laps(ffi.params(nx=n, ny=n, nz=n, precision=ffi.PREC_FP64, timeout_ms=tmo, **CONFIG2))
    g.upload_state(turbulence_ic(n, kmin=1, kmax=8, alpha=-1.0, rms_u=0.3, rms_b=0.3, seed=5), primitive=True)
    g.set_time(0.0)
    t0 = time.perf_counter()
    with pytest.raises(ffi.LapsError) as ei:
        g.step(100)  # about a second of device work
    el = time.perf_counter() - t0
    assert ei.value.code == ffi.LAPS_ETIMEDOUT
    assert el < tmo / 1000 + 1.0, el
    g.wait(600000)  # the queued steps finish
    t, dt, status = g.step(1)
    assert status == 0 and dt > 0 and t > 0
    g.close()
