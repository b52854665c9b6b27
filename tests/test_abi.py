"""CPU checks of the C-ABI boundary: the library loads, exports every entry point the
header declares, its structs have the C layout, and argument validation fails with the
documented codes before any device call."""
import ctypes
import re
import subprocess
import tempfile
from pathlib import Path

import pytest

from laps_gb300 import ffi

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    txt = (ROOT / "include" / "laps_gpu.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(laps_[a-z_0-9]+)\s*\(", txt)))


def test_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 16
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "sz.c"
    fields = [f[0] for f in ffi.laps_params._fields_]
    body = "\n".join(f'printf("%zu ", offsetof(laps_params, {f}));' for f in fields)
    src.write_text(
        "#include <stdio.h>\n#include <stddef.h>\n#include \"laps_gpu.h\"\nint main(){"
        + body
        + 'printf("%zu %zu %zu\\n", sizeof(laps_params), sizeof(laps_diag), sizeof(laps_info));return 0;}'
    )
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    offs = [getattr(ffi.laps_params, f).offset for f in fields]
    assert [int(x) for x in out[: len(fields)]] == offs
    assert int(out[-3]) == ctypes.sizeof(ffi.laps_params)
    assert int(out[-2]) == ctypes.sizeof(ffi.laps_diag)
    assert int(out[-1]) == ctypes.sizeof(ffi.laps_info)


def test_defaults_are_reference_initialisers(lib):
    p = ffi.params()
    assert (p.nx, p.ny, p.nz) == (128, 128, 64)  # mhdinit.f90:5
    assert p.dealias_option == 2 and p.afx == 0.495  # dealiasing.f90:11-12
    assert p.cfl == 0.5 and p.radius0 == 30.0
    assert abs(p.adiabatic_index - 5.0 / 3.0) < 1e-15


@pytest.mark.parametrize(
    "kw,code",
    [
        (dict(nx=100), ffi.LAPS_EINVAL),
        (dict(nx=64, ny=48, nz=64), ffi.LAPS_EINVAL),
        (dict(nx=64, ny=64, nz=64, precision=7), ffi.LAPS_EINVAL),
        (dict(nx=64, ny=64, nz=64, variant=5), ffi.LAPS_EINVAL),
        (dict(nx=64, ny=64, nz=8, variant=2), ffi.LAPS_EINVAL),  # 2-D needs nz = 1
        (dict(nx=64, ny=64, nz=1, variant=0), ffi.LAPS_EINVAL),  # 3-D needs nz >= 8
        (dict(nx=64, ny=64, nz=1, variant=2, if_AEB=1, if_z_radial=1, if_corotating=1), ffi.LAPS_EINVAL),
        (dict(nx=1024, ny=64, nz=64), ffi.LAPS_EINVAL),
        (dict(nx=64, ny=64, nz=64, variant=1, rho0=0.0), ffi.LAPS_EINVAL),
        (dict(nx=64, ny=64, nz=64, cfl=0.0), ffi.LAPS_EINVAL),
        (dict(nx=64, ny=64, nz=64, mem_cap_bytes=1 << 20), ffi.LAPS_ENOMEM),
    ],
)
def test_create_rejects_bad_parameters(lib, kw, code):
    with pytest.raises(ffi.LapsError) as e:
        ffi.Laps(ffi.params(**kw))
    assert e.value.code == code
    assert lib.laps_last_error(None)


def test_null_context_is_an_error(lib):
    assert lib.laps_step(None, 1, None, None, None) == ffi.LAPS_EINVAL
    assert lib.laps_wait(None, 10) == ffi.LAPS_EINVAL


def _c_struct_fields(name):
    txt = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "laps_gpu.h").read_text(), flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), txt, flags=re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r"^(unsigned\s+)?(long long|int|double|char)\s+", "", decl)
        out += [re.sub(r"\[.*\]", "", v).strip() for v in decl.split(",")]
    return out


def _fortran_type_fields(name):
    txt = (ROOT / "fortran" / "laps_gpu.f90").read_text()
    body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type %s" % (name, name), txt, flags=re.S).group(1)
    out = []
    for line in body.splitlines():
        if "::" in line:
            out += [re.sub(r"\(.*\)", "", v).strip() for v in line.split("::")[1].split(",")]
    return out


@pytest.mark.parametrize("name,cls", [("laps_params", ffi.laps_params), ("laps_ic", ffi.laps_ic),
                                      ("laps_diag", ffi.laps_diag), ("laps_info", ffi.laps_info)])
def test_struct_fields_agree_across_bindings(name, cls):
    """The header's struct, the ctypes mirror and the Fortran bind(C) type list the same
    fields in the same order."""
    c = _c_struct_fields(name)
    assert [f[0] for f in cls._fields_] == c
    assert [v.lower() for v in _fortran_type_fields(name)] == [v.lower() for v in c]


def test_fortran_module_binds_the_stepping_entry_points():
    txt = (ROOT / "fortran" / "laps_gpu.f90").read_text()
    bound = set(re.findall(r"name='(laps_[a-z_0-9]+)'", txt))
    for fn in ("laps_create", "laps_upload_state", "laps_init_fields", "laps_step", "laps_vardt", "laps_download_state",
               "laps_diagnostics", "laps_calc_flux", "laps_calc_rhs", "laps_write_output", "laps_read_restart"):
        assert fn in bound, fn
    assert bound <= set(header_functions())
    # every entry point a Fortran host can use; the closure's convolution and data-path calls
    # take BF16 tensors of the training framework and are bound from Python only
    torch_side = {f for f in header_functions() if f.startswith(("laps_conv3_", "laps_closure_"))}
    assert set(header_functions()) - torch_side <= bound, sorted(set(header_functions()) - torch_side - bound)
    assert ctypes.sizeof(ffi.laps_ic) == 2 * 4 + 17 * 8 + 4 * 4 + 9 * 8


def test_ic_defaults_and_phase_counts(lib):
    """laps_ic_default holds the reference's initialisers and laps_ic_nphases the phase counts
    of the random-phase cases, as the oracle states them (no device needed)."""
    from oracle import ic as oic

    ic = ffi.ic_params()
    ref = oic.ic_default()
    for name, _ in ffi.laps_ic._fields_:
        assert getattr(ic, name) == ref[name], name
    for ipert in (0, 1, 6, 7, 8):
        for m in ((1, 0, 0), (3, 2, 1), (16, 16, 16)):
            kw = dict(ipert=ipert, nmodex=m[0], nmodey=m[1], nmodez=m[2])
            d = dict(ref, **kw)
            assert lib.laps_ic_nphases(ctypes.byref(ffi.ic_params(**kw))) == oic.nphases(d)
    assert lib.laps_ic_nphases(None) == 0


def test_post_processing_calls_need_a_context(lib):
    ic = ffi.ic_params(ifield=3)
    assert lib.laps_init_fields(None, ctypes.byref(ic), None, 0) == ffi.LAPS_EINVAL
    assert lib.laps_angle_statistics(None, 0, None) == ffi.LAPS_EINVAL


def _c_prototypes():
    """name -> [(type, is_pointer)] of every function the header declares."""
    txt = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "laps_gpu.h").read_text(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(laps_[a-z_0-9]+)\s*\(([^)]*)\)\s*;", txt):
        args = [a.strip() for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
        out[m.group(1)] = [("*" in a, a) for a in args]
    return out


def _fortran_interfaces():
    """name -> {argument: passed by value} of every interface body in the Fortran module."""
    txt = (ROOT / "fortran" / "laps_gpu.f90").read_text().replace("&\n", " ")
    out = {}
    for m in re.finditer(r"(?:function|subroutine)\s+(\w+)\(([^)]*)\)\s*bind\(C, name='(laps_\w+)'\)(.*?)end (?:function|subroutine)",
                         txt, flags=re.S):
        args = [a.strip().lower() for a in m.group(2).split(",") if a.strip()]
        by_value = {}
        for line in m.group(4).splitlines():
            line = line.split("!", 1)[0]
            if "::" not in line or line.strip().lower().startswith("import"):
                continue
            attrs, names = line.split("::", 1)
            for v in names.split(","):
                by_value[re.sub(r"\(.*\)", "", v).strip().lower()] = "value" in attrs.lower()
        out[m.group(3)] = (args, by_value)
    return out


def test_fortran_interfaces_match_the_c_prototypes():
    """Every Fortran interface has the C function's argument count, passes by value exactly
    the arguments the C prototype takes by value, and declares every argument."""
    protos = _c_prototypes()
    for name, (args, by_value) in _fortran_interfaces().items():
        c = protos[name]
        assert len(args) == len(c), name
        for a, (is_ptr, decl) in zip(args, c):
            assert a in by_value, (name, a)
            # a C pointer is passed by reference, or as type(c_ptr) by value (device / opaque)
            if not is_ptr:
                assert by_value[a], (name, a, decl)
