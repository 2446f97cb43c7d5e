"""The C-ABI library loads, exports every symbol include/mflbm.h declares, and validates
parameters the way the reference's read_parameter does -- all without a GPU."""
import ctypes as C
import os
import re

import pytest

from mflbm import _capi
from mflbm.solver import make_params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "mflbm.h")).read()
    return sorted(set(re.findall(r"\b(mflbm_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = _capi.load()
    syms = header_symbols()
    assert len(syms) >= 16
    for name in syms:
        assert hasattr(lib, name), name
    assert set(syms) == set(_capi.SIGNATURES), "ctypes binding and header disagree"
    assert lib.mflbm_version() == _capi.MFLBM_ABI_VERSION


def test_struct_layouts_match_fortran_types():
    assert C.sizeof(_capi.SolidBnd) == 96     # 4 int + 18 int + 1 double
    assert C.sizeof(_capi.FluidBnd) == 48     # 3 int + pad + 4 double
    assert _capi.FluidBnd.nwx.offset == 16
    assert _capi.SolidBnd.la_weight.offset == 88


def _create(**kw):
    lib = _capi.load()
    p = make_params(**kw)
    h = C.c_void_p()
    rc = lib.mflbm_create(C.byref(p), C.byref(h))
    if rc == 0:
        lib.mflbm_destroy(h)
    return rc, lib.mflbm_last_error(None).decode()


@pytest.mark.parametrize("kw,needle", [
    (dict(multiphase=1, iper=1, wall_x_min=0, wall_x_max=0), "X direction periodic"),
    (dict(multiphase=1, wall_x_min=0), "x = xmin or x = xmax"),
    (dict(jper=0, wall_y_min=0), "y = ymin"),
    (dict(jper=1, wall_y_min=1, wall_y_max=1), "y direction periodic BC enabled"),
    (dict(kper=1, wall_z_min=1), "z direction periodic BC enabled"),
    (dict(inlet_bc=2, outlet_bc=1), "Inlet pressure + outlet convective"),
    (dict(multiphase=1, mrt=7), "mrt"),
    (dict(nx=2), "dimensions"),
    (dict(precision=5), "precision"),
    (dict(multiphase=1, precision=2), "FP16 deviations cannot hold a vanishing species"),
])
def test_invalid_parameters_rejected_before_any_device_work(kw, needle):
    rc, msg = _create(**kw)
    assert rc == _capi.MFLBM_EINVAL
    assert needle in msg


def test_abi_version_checked():
    lib = _capi.load()
    p = make_params()
    p.abi_version = 99
    h = C.c_void_p()
    assert lib.mflbm_create(C.byref(p), C.byref(h)) == _capi.MFLBM_EINVAL


def test_null_context_calls_fail_cleanly():
    lib = _capi.load()
    assert lib.mflbm_step(None, 0) == _capi.MFLBM_EINVAL
    assert lib.mflbm_synchronize(None) == _capi.MFLBM_EINVAL
    lib.mflbm_destroy(None)


def test_header_constants_match_the_binding():
    """Every integer #define MFLBM_* of include/mflbm.h has the same value in the Python
    binding (the layout constants are bound as LAYOUT_*)."""
    import re
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "mflbm.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"^#define (MFLBM_[A-Z0-9_]+)\s+(-?\d+)\b", hdr, re.M)}
    assert "MFLBM_FP64FF" in defs and "MFLBM_FF" in defs
    for name, value in defs.items():
        py = name.replace("MFLBM_LAYOUT_", "LAYOUT_")
        assert hasattr(_capi, py), name
        assert getattr(_capi, py) == value, name
