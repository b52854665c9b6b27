"""laps_write_output / laps_read_restart against the restated outNNN.dat format.

The file the GPU writes must be byte-identical to the restated writer applied to the state
the GPU downloads (primitive and conserved layouts, all three variants); a file made by the
restated writer, read back with laps_read_restart, must give the state an upload of the same
array gives, at the time rounded to a 4-byte real; a write -> read -> write cycle reproduces the
bytes of the first write.
"""
import numpy as np
import pytest

from laps_gb300 import ffi
from laps_gb300.ic import turbulence_ic
from oracle import outfile

pytestmark = pytest.mark.gpu

CASES = {
    "3dc": (dict(nx=32, ny=16, nz=8, dealias_option=1, if_Hall=1, ion_inertial_length=0.05), 0.1),
    "3di": (dict(nx=16, ny=16, nz=16, variant=ffi.VARIANT_3DI, dealias_option=1), 1.0),
    "2dc": (dict(nx=64, ny=32, nz=1, variant=ffi.VARIANT_2DC, dealias_option=1), 0.1),
}


@pytest.mark.parametrize("prec", [ffi.PREC_FP64, ffi.PREC_DD], ids=["fp64", "dd"])
@pytest.mark.parametrize("case", list(CASES))
def test_write_matches_restated_writer(tmp_path, prec, case):
    kw, p0 = CASES[case]
    g = ffi.Laps(ffi.params(precision=prec, **kw))
    prim = turbulence_ic((kw["nx"], kw["ny"], kw["nz"]), seed=41, kmax=4, p0=p0)
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    t, dt, st = g.step(3)
    uu, pr = g.download_state()
    inc = kw.get("variant") == ffi.VARIANT_3DI
    for primitive in (True, False):
        path = tmp_path / outfile.output_name(3 if primitive else 4)
        g.write_output(path, primitive=primitive)
        ref = outfile.primitive_layout(uu, pr, inc) if primitive else uu
        want = tmp_path / "want.dat"
        raw = outfile.write_output(want, ref, t)
        assert path.read_bytes() == raw
    g.close()


@pytest.mark.parametrize("case", list(CASES))
def test_restart_reads_restated_file(tmp_path, case):
    kw, p0 = CASES[case]
    shape = (kw["nx"], kw["ny"], kw["nz"])
    prim = turbulence_ic(shape, seed=42, kmax=4, p0=p0)
    path = tmp_path / outfile.output_name(12)
    outfile.write_output(path, prim, 0.7)
    a = ffi.Laps(ffi.params(precision=ffi.PREC_FP64, **kw))
    t = a.read_restart(path)
    assert t == float(np.float32(0.7)) and a.time()[0] == t
    b = ffi.Laps(ffi.params(precision=ffi.PREC_FP64, **kw))
    b.upload_state(prim, primitive=True)
    ua, _ = a.download_state()
    ub, _ = b.download_state()
    assert np.array_equal(ua, ub)
    # write -> read -> write reproduces the bytes
    p1, p2 = tmp_path / "a.dat", tmp_path / "b.dat"
    a.write_output(p1)
    c = ffi.Laps(ffi.params(precision=ffi.PREC_FP64, **kw))
    c.read_restart(p1)
    c.write_output(p2)
    t1, x1 = outfile.read_output(p1, shape)
    t2, x2 = outfile.read_output(p2, shape)
    assert t1 == t2 and np.abs(x1 - x2).max() <= 1e-13 * np.abs(x1).max()


def test_output_errors(tmp_path):
    g = ffi.Laps(ffi.params(nx=16, ny=16, nz=16))
    with pytest.raises(ffi.LapsError):
        g.write_output(tmp_path / "x.dat")  # no state
    (tmp_path / "bad.dat").write_bytes(b"\x08\x00\x00\x00" + b"\x00" * 20)
    with pytest.raises(ffi.LapsError):
        g.read_restart(tmp_path / "bad.dat")
    outfile.write_output(tmp_path / "small.dat", np.zeros((8, 8, 8, 16)), 0.0)
    with pytest.raises(ffi.LapsError):
        g.read_restart(tmp_path / "small.dat")  # too short for 16^3
