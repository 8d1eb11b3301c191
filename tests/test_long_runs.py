"""Whole-run parity: the GPU step against the reference's own serial FP64 build
after each benchmark configuration's full step count.

The fixtures tests/golden/long_*.npz hold digests (model_gb300/digest.py) of
the reference build's end state (tests/golden/make_long.py): per field, 32 or
64 random +-1 projections (an estimate of the whole field's relative L2
error), level norms and a seeded point sample.  Every prognostic field and pi
must agree to 1e-10 relative L2 in FP64 (estimate, sample, level norms and
norm), the bound for the plain FP64 path:

  thunderstorm     128x128x48 Kessler, 600 steps
  monsoon_vortex   192x128x32 dry ITCZ shear + vortex, 500 steps
  member_small     ensemble member 0, 96x96x40 Kessler, 300 steps
  member_large     ensemble member 64, 160x160x48 Kessler, 300 steps
  squall_line      512x512x64 Kessler, 10 of its 400 steps (one host core
                   needs about 40 s per step of the reference)

The two ensemble members also run inside one batched FP64 ensemble, and the
FP32 thunderstorm must stay within 1e-4 of the reference after 600 steps.
"""
import json

import numpy as np
import pytest

from model_gb300 import abi, anelastic, configs, digest
from tests import fixtures as fx

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10
TOL_FP32 = 1e-4
CASES = ["long_thunderstorm", "long_monsoon_vortex", "long_member_small", "long_member_large",
         "long_squall_line"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    from model_gb300 import build
    build.build()


def _workload(d):
    gen = str(d["generator"])
    kw = json.loads(str(d["kwargs"]))
    wl = getattr(configs, gen)(**kw)
    names = json.loads(str(d["input_names"]))
    assert names == sorted(wl.fields)
    norms = np.array([np.linalg.norm(np.asarray(wl.fields[k], dtype=np.float64)) for k in names])
    ref = d["input_norms"]
    scale = np.where(ref > 0, ref, 1.0)
    assert np.all(np.abs(norms - ref) <= 1e-13 * scale), "initial state differs from the fixture's"
    return wl


def _end_fields(m, wl):
    out = {n: m.get(f) for f, n in enumerate(abi.PROG_NAMES[:7 if wl.microphysics_option else 4])}
    out["pi"] = m.get(abi.GA_PI)
    return out


def _check(res, tol, label):
    for k, e in res.items():
        worst = max(e.values())
        assert worst <= tol, f"{label}: {k} {e}"


@pytest.mark.parametrize("name", CASES)
def test_fp64_whole_run_matches_reference(name):
    d = fx.load(name)
    wl = _workload(d)
    steps = int(d["steps"])
    m = anelastic.Model(wl, abi.GA_PREC_F64)
    m.step(steps)
    res = digest.compare(_end_fields(m, wl), d)
    m.close()
    print(name, steps, {k: f"{max(v.values()):.2e}" for k, v in res.items()})
    _check(res, TOL_FP64, name)


def test_fp64_batched_ensemble_members_match_reference():
    ds = [fx.load("long_member_small"), fx.load("long_member_large")]
    wls = [_workload(d) for d in ds]
    steps = int(ds[0]["steps"])
    assert steps == int(ds[1]["steps"])
    # a third member between them, so that the two pinned ones are not alone
    extra = configs.ensemble_member(1, 96, 96, 40, nsteps=steps)
    members = [wls[0], extra, wls[1]]
    cols = [anelastic.build_columns(w) for w in members]
    ens = anelastic.Ensemble(members, abi.GA_PREC_F64, columns=cols)
    for i, w in enumerate(members):
        ens.load_member(i, w.fields)
    ens.step(steps)
    for i, d in ((0, ds[0]), (2, ds[1])):
        w = members[i]
        fields = {n: ens.get(i, f) for f, n in enumerate(abi.PROG_NAMES)}
        fields["pi"] = ens.get(i, abi.GA_PI)
        res = digest.compare(fields, d)
        _check(res, TOL_FP64, f"ensemble member {i} ({w.nx}x{w.ny}x{w.nz})")
    ens.close()


def test_fp32_thunderstorm_within_1e4_of_reference_after_600_steps():
    d = fx.load("long_thunderstorm")
    wl = _workload(d)
    m = anelastic.Model(wl, abi.GA_PREC_F32)
    m.step(int(d["steps"]))
    res = digest.compare(_end_fields(m, wl), d)
    m.close()
    print("fp32", {k: f"{v['proj']:.2e}" for k, v in res.items()})
    for k, e in res.items():
        assert e["proj"] <= TOL_FP32 and e["sample"] <= TOL_FP32, f"fp32 {k} {e}"
