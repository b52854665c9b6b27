"""The reference's output / restart file, restated in numpy (test infrastructure: the oracle
of laps_write_output / laps_read_restart).

``outNNN.dat`` (``src_compressible/mhdoutput.f90:72-131``, ``restart.f90:17-63``; the 2-D and
incompressible codes use the same layout): rank 0 writes the time with a Fortran unformatted
sequential ``write(10) real(time,4)`` (a 4-byte length marker, the 4-byte real, the marker
again: 12 bytes), then ``mpi_file_write_all`` writes ``uu(nx,ny,nz,nvar)`` from byte 12
(``displacement = 12``) as ``mpi_double_precision`` (the code is built with ``-r8``) in
Fortran order.  With ``output_primitive`` slots 2:4 hold u instead of rho u and, in the
compressible codes, slot 8 holds p instead of e (``:90-97``).
"""
from __future__ import annotations

import numpy as np


def output_name(iout: int) -> str:
    """File name of output number iout (``mhdoutput.f90:80-83``): out000 .. out999."""
    return f"out{iout:03d}.dat"


def write_output(path, uu: np.ndarray, time: float) -> bytes:
    """Write ``uu`` ([8, nz, ny, nx] float64, already in the layout to be written) and the
    time; returns the bytes written."""
    head = np.array([4], "<i4").tobytes() + np.array([time], "<f4").tobytes() + np.array([4], "<i4").tobytes()
    data = np.ascontiguousarray(uu, dtype="<f8").tobytes()  # [var, z, y, x] = Fortran (x, y, z, var)
    raw = head + data
    with open(path, "wb") as f:
        f.write(raw)
    return raw


def read_output(path, shape):
    """(time as read back through the 4-byte real, uu [8, nz, ny, nx]) of an output file."""
    nx, ny, nz = shape
    raw = open(path, "rb").read()
    m0, = np.frombuffer(raw[0:4], "<i4")
    t, = np.frombuffer(raw[4:8], "<f4")
    m1, = np.frombuffer(raw[8:12], "<i4")
    assert m0 == 4 and m1 == 4, "not an output file"
    uu = np.frombuffer(raw[12:12 + 8 * 8 * nx * ny * nz], "<f8").reshape(8, nz, ny, nx).copy()
    return float(t), uu


def primitive_layout(uu_cons: np.ndarray, prim: np.ndarray, incompressible: bool = False) -> np.ndarray:
    """The array output_uu writes with output_primitive: rho u -> u (prim 0:3) and, except in
    the incompressible code, e -> p (prim 3)."""
    out = uu_cons.copy()
    out[1:4] = prim[0:3]
    if not incompressible:
        out[7] = prim[3]
    return out
