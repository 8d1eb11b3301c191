"""The CPU oracle against golden vectors produced by the reference itself.

The fixtures in tests/golden/ hold the output of the reference's own serial
step (built from its sources with oracle/build_ref.sh and
tests/golden/make_golden.py).  The oracle restatement must reproduce them bit
for bit: both use the same DFT, and neither contracts multiply-adds.
"""
import numpy as np
import pytest

from model_gb300 import abi
from oracle import oracle as O
from tests import fixtures as fx


@pytest.mark.parametrize("name", fx.run_names())
def test_columns_match_reference(name):
    d = fx.load(name)
    wl = fx.workload(d)
    cols = O.build_columns(wl)
    for n in abi.COLUMN_NAMES + ["f"]:
        np.testing.assert_array_equal(cols[n], d["out_" + n], err_msg=n)


@pytest.mark.parametrize("name", fx.run_names())
def test_full_steps_bit_exact(name):
    d = fx.load(name)
    wl = fx.workload(d)
    o = O.Oracle(wl, fx.columns(d))
    if "bigcounter0" in wl.fields:  # a run later in the model's life
        o.set_counters(int(np.ravel(wl.fields["bigcounter0"])[0]), float(np.ravel(wl.fields["mtime0"])[0]))
    assert o.step(wl.nsteps) == 0
    st = o.state()
    checked = 0
    for k, v in st.items():
        if "out_" + k not in d:
            continue
        np.testing.assert_array_equal(v, d["out_" + k], err_msg=f"{name}:{k}")
        checked += 1
    assert checked >= 13
    if wl.turbulence_option:  # the tendencies of the last step's calculate_diff_tend
        turb = [k for k in abi.TURB_NAMES if "out_" + k in d]
        assert len(turb) >= 6
        for k in turb:
            np.testing.assert_array_equal(o.get(abi.TURB_NAMES[k]), d["out_" + k], err_msg=f"{name}:{k}")


@pytest.mark.parametrize("name", fx.ops_names())
@pytest.mark.parametrize("op", ["advect_uvw", "solve_pressure", "integrate_non_hydro",
                                "advect_theta", "advect_micro", "zero_moisture", "bc",
                                "bc_micro", "kessler", "rayleigh"])
def test_single_operator_bit_exact(name, op):
    d = fx.load(name)
    wl = fx.workload(d)
    o = O.Oracle(wl)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        o.set(f, slot, v)
    assert o.op(op, float(d[f"step_{op}"])) == 0
    outs = [k for k in d if k.startswith(op + "__")]
    assert outs, "fixture has no output for this operator"
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        np.testing.assert_array_equal(o.get(f, slot), d[k], err_msg=f"{op}:{key}")


@pytest.mark.parametrize("name", fx.turb_names())
@pytest.mark.parametrize("op", ["turbulence", "kessler"])
def test_turbulence_operator_bit_exact(name, op):
    """calculate_diff_tend (mixing coefficients, stress and flux tendencies)
    of a state with differing rotation slots and a seeded saturation record,
    and the saturation record Kessler leaves"""
    d = fx.load(name)
    wl = fx.workload(d)
    if op == "kessler" and not wl.microphysics_option:
        pytest.skip("dry case")
    o = O.Oracle(wl)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        o.set(f, slot, v)
    assert o.op(op, float(d[f"step_{op}"])) == 0
    outs = [k for k in d if k.startswith(op + "__")]
    assert len(outs) >= (6 if op == "turbulence" else 5)
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        np.testing.assert_array_equal(o.get(f, slot), d[k], err_msg=f"{op}:{key}")


@pytest.mark.parametrize("name", fx.linop_names())
@pytest.mark.parametrize("op", ["advect_uvw", "advect_theta", "advect_micro", "integrate_non_hydro"])
def test_linear_operator_bit_exact(name, op):
    """the linearised model's operators against the reference's ISLINEAR
    build (advect_micro of a linearised context is advect_qv)"""
    d = fx.load(name)
    wl = fx.workload(d)
    assert wl.linear_model
    o = O.Oracle(wl)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        o.set(f, slot, v)
    assert o.op(op, float(d[f"step_{op}"])) == 0
    outs = [k for k in d if k.startswith(op + "__")]
    assert outs
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        np.testing.assert_array_equal(o.get(f, slot), d[k], err_msg=f"{op}:{key}")


@pytest.mark.parametrize("name", fx.hydop_names())
@pytest.mark.parametrize("op", ["advect_uvw", "solve_pressure", "integrate_non_hydro", "kessler", "bc", "rayleigh"])
def test_hydrostatic_operator_bit_exact(name, op):
    """the operators of the hydrostatic set against the reference's
    HYDROSTATIC build (advect_uvw is advect_uv_velocity, integrate_non_hydro
    integrate_hydro; the boundary conditions and damping act on the current
    w)"""
    d = fx.load(name)
    wl = fx.workload(d)
    assert wl.hydrostatic
    o = O.Oracle(wl)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        o.set(f, slot, v)
    assert o.op(op, float(d[f"step_{op}"])) == 0
    outs = [k for k in d if k.startswith(op + "__")]
    assert outs
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        np.testing.assert_array_equal(o.get(f, slot), d[k], err_msg=f"{op}:{key}")


@pytest.mark.parametrize("name", fx.iceop_names())
@pytest.mark.parametrize("op", ["advect_uvw", "advect_micro", "advect_ice", "kessler", "bc_micro", "zero_moisture",
                                "explicit_diffusion"])
def test_ice_operator_bit_exact(name, op):
    """the operators of the ice scheme (microphysics_option 2) against the
    reference build: the buoyancy with snow and ice, the Rutledge rain fall
    speed, advect_ice_cell, run_rutledge_microphysics (with semi-Lagrangian
    fallout and the saturation record in the periodic case), the boundary
    conditions, zero_moisture and explicit diffusion of snow and ice"""
    d = fx.load(name)
    if f"step_{op}" not in d:
        pytest.skip("operator not in this fixture")
    wl = fx.workload(d)
    assert wl.microphysics_option == 2
    o = O.Oracle(wl)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        o.set(f, slot, v)
    assert o.op(op, float(d[f"step_{op}"])) == 0
    outs = [k for k in d if k.startswith(op + "__")]
    assert outs
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        np.testing.assert_array_equal(o.get(f, slot), d[k], err_msg=f"{op}:{key}")
