"""GPU runs of the committed golden cases (tests/golden/c*.npz, made by make_golden.py from
the oracle) through the C-ABI: every field within 1e-11 relative L2, time within 1e-12."""
from pathlib import Path

import numpy as np
import pytest

from laps_gb300 import ffi

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("prec", [ffi.PREC_FP64, ffi.PREC_DD], ids=["fp64", "dd"])
@pytest.mark.parametrize("path", sorted(GOLDEN.glob("c*.npz")), ids=lambda p: p.stem)
def test_golden_case(path, prec):
    g = np.load(path)
    nx, ny, nz = (int(v) for v in g["shape"])
    kw = eval(str(g["params"]))  # a dict literal written by make_golden.py
    run = ffi.Laps(ffi.params(nx=nx, ny=ny, nz=nz, precision=prec, **kw))  # kw may carry "variant"
    run.upload_state(g["prim"], primitive=True)
    run.set_time(0.0)
    t, dt, status = run.step(int(g["steps"]))
    assert status == 0
    assert abs(t - float(g["time"])) <= 1e-12 * t
    assert abs(dt - float(g["dts"][-1])) <= 1e-12 * dt
    uu, _ = run.download_state()
    for f in range(8):
        ref = g["uu"][f]
        assert np.linalg.norm(uu[f] - ref) <= 1e-11 * max(np.linalg.norm(ref), 1e-300)
    d = run.diagnostics()
    assert np.allclose([d.e_kin, d.e_mag, d.h_cross, d.h_mag], g["inv"], rtol=1e-10, atol=1e-14)
    assert np.allclose(np.array(d.uu_ave[:]), g["ave"], rtol=1e-11, atol=1e-14)
