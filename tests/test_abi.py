"""The C-ABI library without a GPU: it loads, exports every entry point the
public header declares, rejects bad arguments before touching a device, and
its host-only column builders reproduce the reference's columns bit for bit."""
import os
import re

import numpy as np
import pytest

from model_gb300 import abi, anelastic
from tests import fixtures as fx

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "ga_anelastic.h")


def _declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^GA_API\s+[^(]*?\b(ga_\w+)\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from model_gb300 import build
    build.build()
    return anelastic.load_library()


def test_header_declares_entry_points():
    names = _declared()
    assert "ga_create" in names and "ga_step" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.ga_abi_version() == 1


def test_null_arguments_are_rejected(lib):
    import ctypes as C
    assert lib.ga_create(None, None, None) == abi.GA_ERR_ARG
    assert "null" in anelastic.last_error()
    assert lib.ga_destroy(None) == abi.GA_ERR_ARG
    assert lib.ga_step(None, 1) == abi.GA_ERR_ARG
    assert lib.ga_op(None, 0, 1.0) == abi.GA_ERR_ARG
    assert lib.ga_launch_count(None) == -1
    assert lib.ga_tlm_step(None, 1) == abi.GA_ERR_ARG
    assert lib.ga_adjoint(None, 1, 1) == abi.GA_ERR_ARG
    assert lib.ga_lin_set_field(None, 0, 0, None, 0) == abi.GA_ERR_ARG
    assert lib.ga_lin_get_field(None, 0, 0, None, 0) == abi.GA_ERR_ARG
    store = abi.GaColumnStore()
    tb = np.zeros(4)
    rc = lib.ga_columns_build(4, 100.0, 100.0, tb.ctypes.data_as(C.POINTER(C.c_double)),
                              tb.ctypes.data_as(C.POINTER(C.c_double)), C.byref(store))
    assert rc == abi.GA_ERR_ARG


def test_bad_config_rejected_before_device(lib):
    import ctypes as C
    from model_gb300 import configs
    wl = configs.moist_blob()
    cols = anelastic.build_columns(wl)
    keep = {n: np.ascontiguousarray(v) for n, v in cols.items()}
    gc = abi.GaColumns()
    for n in abi.COLUMN_NAMES + ["f"]:
        setattr(gc, n, keep[n].ctypes.data_as(C.POINTER(C.c_double)))
    h = C.c_void_p()
    for change, code in [({"nx": 8}, abi.GA_ERR_CONFIG), ({"nz": 200}, abi.GA_ERR_CONFIG),
                         ({"microphysics_option": 3}, abi.GA_ERR_CONFIG),
                         ({"microphysics_option": 2, "linear_model": 1}, abi.GA_ERR_UNSUPPORTED),
                         ({"dt": -1.0}, abi.GA_ERR_CONFIG), ({"rain_fallout": 3}, abi.GA_ERR_CONFIG),
                         ({"use_explicit_diffusion": 1, "diffusion_order": 3}, abi.GA_ERR_CONFIG),
                         ({"turbulence_option": 2}, abi.GA_ERR_CONFIG),
                         ({"linear_model": 1, "turbulence_option": 1}, abi.GA_ERR_UNSUPPORTED),
                         ({"hydrostatic": 1, "periodic_ew_boundaries": 1}, abi.GA_ERR_UNSUPPORTED),
                         ({"hydrostatic": 1, "turbulence_option": 1}, abi.GA_ERR_UNSUPPORTED),
                         ({"hydrostatic": 2}, abi.GA_ERR_CONFIG)]:
        s = wl.settings()
        s.update(change)
        cfg = abi.make_config(s)
        assert lib.ga_create(C.byref(cfg), C.byref(gc), C.byref(h)) == code, change


@pytest.mark.parametrize("name", fx.run_names())
def test_library_columns_match_reference(lib, name):
    d = fx.load(name)
    wl = fx.workload(d)
    cols = anelastic.build_columns(wl)
    for n in abi.COLUMN_NAMES + ["f"]:
        np.testing.assert_array_equal(cols[n], d["out_" + n], err_msg=n)
