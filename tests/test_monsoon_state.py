"""The monsoon-vortex initial state against the reference's own initialisers.

model_gb300/monsoon.py restates initialize_basic_state_ITCZ_shear2 and
initialize_vortex (data_initializer.cpp:298-568, 862-1064).  The fixtures
tests/golden/itcz_*.npz come from the reference's code itself
(oracle/ref/itcz_harness.cpp, tests/golden/make_itcz.py) on grids of at least
39 levels; one of them has a second-pass vorticity (hor_shear != 1e-4) and a
vortex away from the base column.  Columns must agree to 1e-13 and the 3-D
fields to 1e-12 relative (numpy's FFT and transcendentals against the
reference's DFT and libm).
"""
import numpy as np
import pytest

from model_gb300 import configs, digest, monsoon
from tests import fixtures as fx

CASES = ["itcz_default", "itcz_strong"]


def _state(d):
    p = {k[6:]: float(d[k]) for k in d if k.startswith("param_")}
    nx, ny, nz = int(p["nx"]), int(p["ny"]), int(p["nz"])
    st = monsoon.itcz_shear_state(nx, ny, nz, p["dx"], p["dz"], p["corner_lat"], p["corner_lon"], p["hor_shear"],
                                  p["vert_shear0"], p["vert_shear1"])
    xpos = monsoon._nearest(st["lons"], p["vortex_longitude"])
    ypos = monsoon._nearest(st["lats"], p["vortex_latitude"])
    u, v, th = monsoon.vortex(st, nx, ny, nz, p["dx"], p["dz"], p["vortex_radius"], p["vortex_height_wind_max"],
                              p["vortex_vertical_extent"], p["vortex_upper_warm_anomaly"],
                              p["vortex_lower_cold_anomaly"], xpos, ypos)
    st.update(u=u, v=v, th=th, vortex_ij=np.array([xpos, ypos], dtype=np.float64))
    return st


@pytest.mark.parametrize("name", CASES)
def test_itcz_columns_match_reference(name):
    d = fx.load(name)
    st = _state(d)
    for k in ("tb", "qb", "tbv", "pib", "rhou", "rhow", "lats", "lons", "f", "vortex_ij"):
        e = fx.rel_l2(st[k], d["col_" + k])
        assert e <= 1e-13, f"{name}: {k} rel L2 {e:.3e}"


@pytest.mark.parametrize("name", CASES)
def test_itcz_fields_match_reference(name):
    d = fx.load(name)
    st = _state(d)
    fields = {k: st[k] for k in ("ubar", "vbar", "wbar", "thbar", "qbar", "pbar", "u", "v", "th")}
    res = digest.compare(fields, d)
    for k, e in res.items():
        worst = max(e.values())
        assert worst <= 1e-12, f"{name}: {k} {e}"


def test_monsoon_vortex_config_is_the_c3_state():
    """192 x 128 x 32 at 40 km: the shear profile's ktrop clamped to 30, the
    vortex's maximum wind 5 m/s about 500 km from its centre at about 4 km."""
    wl = configs.monsoon_vortex(nsteps=1)
    f = wl.fields
    for k in ("ubar", "thbar", "qbar", "pbar", "u", "v", "th"):
        assert np.all(np.isfinite(f[k])), k
    sp = np.maximum(np.abs(f["u"]), np.abs(f["v"]))
    i, j, k = np.unravel_index(np.argmax(sp), sp.shape)
    assert abs(sp.max() - 5.0) < 0.01
    assert abs(np.hypot(i - 96, j - 64) * 40.0 - 500.0) <= 40.0
    assert abs((k - 0.5) * 600.0 - 4000.0) <= 300.0
    # zonally uniform jet: the strip spans every longitude
    assert np.array_equal(f["ubar"][3], f["ubar"][100])
    assert float(np.abs(f["ubar"]).max()) > 10.0
