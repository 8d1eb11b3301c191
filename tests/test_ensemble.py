"""Uneven ensembles: every member advanced by the batched kernels must equal a
standalone context run of the same member bit for bit (both use the same
device bodies), in FP64 and FP32."""
import numpy as np
import pytest

from model_gb300 import abi, anelastic, configs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tune,x_solve", [(abi.GA_PREC_F64, False, "fused"),
                                                    (abi.GA_PREC_F32, False, "fused"),
                                                    (abi.GA_PREC_F32, True, "fused"),
                                                    (abi.GA_PREC_F64, False, "unfused"),
                                                    (abi.GA_PREC_F32, False, "unfused")])
def test_ensemble_members_equal_standalone_runs(monkeypatch, precision, tune, x_solve):
    """tune: the autotuner runs mid-run; tiles change nothing bit for bit.
    x_solve "unfused": the ensemble's x solve as batched x FFTs and Thomas
    blocks, against standalone contexts that use the fused x kernel."""
    members = [configs.moist_blob(nx=24, ny=22, nz=16, seed=3000),
               configs.moist_blob(nx=36, ny=30, nz=20, seed=3100, qc=2e-3),
               configs.moist_blob(nx=40, ny=24, nz=12, seed=3200, dt=3.0)]
    if x_solve == "unfused":
        monkeypatch.setenv("GA_SPECTRAL_X", "unfused")
    ens = anelastic.Ensemble(members, precision)
    monkeypatch.delenv("GA_SPECTRAL_X", raising=False)
    for m, wl in enumerate(members):
        ens.load_member(m, wl.fields)
    nsteps = 5
    if tune:
        ens.step(2)
        assert "advect tile" in ens.tune()
        ens.step(nsteps - 2)
    else:
        ens.step(nsteps)
    for m, wl in enumerate(members):
        solo = anelastic.Model(wl, precision)
        solo.step(nsteps)
        for f in range(7):
            for slot in (abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M):
                np.testing.assert_array_equal(ens.get(m, f, slot), solo.get(f, slot), err_msg=f"member {m} f{f} s{slot}")
        np.testing.assert_array_equal(ens.get(m, abi.GA_PI), solo.get(abi.GA_PI))
        np.testing.assert_array_equal(ens.get(m, abi.GA_ACCRAIN), solo.get(abi.GA_ACCRAIN))
        assert ens.counters(m)[0] == nsteps
        solo.close()
    ens.close()



def test_ensemble_member_too_tall_for_the_fused_x_kernel():
    """a member whose levels of one y-wavenumber exceed shared memory (FP32:
    200 x 70 spectral points) runs the batched unfused x solve; every member
    still equals its standalone context bit for bit"""
    members = [configs.moist_blob(nx=200, ny=20, nz=72, seed=3300),
               configs.moist_blob(nx=36, ny=30, nz=20, seed=3100, qc=2e-3)]
    ens = anelastic.Ensemble(members, abi.GA_PREC_F32)
    for m, wl in enumerate(members):
        ens.load_member(m, wl.fields)
    ens.step(3)
    for m, wl in enumerate(members):
        solo = anelastic.Model(wl, abi.GA_PREC_F32)
        solo.step(3)
        for f in range(7):
            np.testing.assert_array_equal(ens.get(m, f), solo.get(f), err_msg=f"member {m} f{f}")
        np.testing.assert_array_equal(ens.get(m, abi.GA_PI), solo.get(abi.GA_PI))
        solo.close()
    ens.close()

def test_ensemble_rejects_mixed_precision():
    a, b = configs.moist_blob(), configs.moist_blob(seed=9)
    cols = [anelastic.build_columns(a), anelastic.build_columns(b)]
    import ctypes as C
    L = anelastic.load_library()
    cfgs = (abi.GaConfig * 2)(abi.make_config(a.settings(), abi.GA_PREC_F64),
                              abi.make_config(b.settings(), abi.GA_PREC_F32))
    keep = [{k: np.ascontiguousarray(v) for k, v in c.items()} for c in cols]
    gcs = (abi.GaColumns * 2)()
    for m in range(2):
        for name in abi.COLUMN_NAMES + ["f"]:
            setattr(gcs[m], name, keep[m][name].ctypes.data_as(C.POINTER(C.c_double)))
    h = C.c_void_p()
    assert L.ga_ensemble_create(cfgs, gcs, 2, C.byref(h)) == abi.GA_ERR_CONFIG
