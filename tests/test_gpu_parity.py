"""GPU parity: the CUDA path against the reference's own outputs (golden
fixtures) and against the CPU oracle.

Tolerances (relative L2 over a whole field, FP64):
  - operators without transcendental functions or transforms: bit exact
    (the FP64 kernels are compiled without FMA contraction and keep the
    reference's evaluation order);
  - operators with CUDA pow/exp (Kessler, fall speed) or the FFT: 1e-12;
  - full steps: 1e-10 (the benchmark spec bound for the plain FP64 path).
"""
import numpy as np
import pytest

from model_gb300 import abi, anelastic
from tests import fixtures as fx

pytestmark = pytest.mark.gpu

EXACT_OPS = {"advect_uvw", "advect_theta", "zero_moisture", "bc", "bc_micro", "rayleigh"}


@pytest.fixture(scope="module", autouse=True)
def _built():
    from model_gb300 import build
    build.build()


@pytest.mark.parametrize("name", fx.run_names())
def test_full_steps_match_reference(name):
    d = fx.load(name)
    wl = fx.workload(d)
    m = anelastic.Model(wl, abi.GA_PREC_F64, columns=fx.columns(d))
    m.step(wl.nsteps)
    st = m.state()
    worst = 0.0
    for k, v in st.items():
        if "out_" + k not in d:
            continue
        e = fx.rel_l2(v, d["out_" + k])
        worst = max(worst, e)
        assert e <= 1e-10, f"{name}:{k} rel L2 {e:.3e}"
    print(f"{name}: worst rel L2 {worst:.3e}")
    assert m.counters()[0] == wl.nsteps


@pytest.mark.parametrize("name", fx.ops_names())
@pytest.mark.parametrize("op", ["advect_uvw", "solve_pressure", "integrate_non_hydro", "advect_theta",
                                "advect_micro", "zero_moisture", "bc", "bc_micro", "kessler", "rayleigh"])
def test_single_operator_matches_reference(name, op):
    d = fx.load(name)
    wl = fx.workload(d)
    m = anelastic.Model(wl, abi.GA_PREC_F64)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        if f < abi.GA_NPROG and f >= (7 if wl.microphysics_option else 4):
            continue
        m.set(f, slot, v)
    m.op(op, float(d[f"step_{op}"]))
    outs = [k for k in d if k.startswith(op + "__")]
    assert outs
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        got = m.get(f, slot)
        if op in EXACT_OPS:
            np.testing.assert_array_equal(got, d[k], err_msg=f"{op}:{key}")
        else:
            e = fx.rel_l2(got, d[k])
            assert e <= 1e-12, f"{op}:{key} rel L2 {e:.3e}"
