"""The oracle against the reference build on seeded random configurations.

Each case draws a grid (odd and even, prime transform lengths, stretched
levels), the boundary options (sponge widths, periodic east-west), the rain
fallout, the optional physics (explicit diffusion of each order, the
turbulence scheme with and without the ocean fluxes) and the equation set
(nonlinear, linearised, hydrostatic), runs the reference's own serial step
(oracle/_ref, built from the reference sources by oracle/build_ref.sh) and
the oracle on the same state for a few steps, and requires every field of
the dump bit for bit.  Runs where the reference build exists (this
container); skipped elsewhere.
"""
import numpy as np
import pytest

from model_gb300 import abi, configs
from oracle import oracle as O

pytestmark = pytest.mark.skipif(not O.reference_available(), reason="reference build not present")

NCASES = 48


def _case(seed: int):
    rng = np.random.default_rng(seed)
    nx = int(rng.choice([12, 13, 16, 17, 19, 24, 29]))
    ny = int(rng.choice([12, 14, 15, 18, 23]))
    nz = int(rng.choice([6, 7, 9, 12, 16]))
    kind = int(rng.integers(0, 4))  # 0 dry bubble, 1 moist blob, 2 dry jet, 3 moist jet
    eq = int(rng.choice([0, 0, 0, 1, 2]))  # nonlinear (most), linearised, hydrostatic
    periodic = int(rng.integers(0, 2)) if eq == 0 and nx >= 13 else 0
    if kind == 0:
        wl = configs.dry_bubble(nx=nx, ny=ny, nz=nz, dx=600.0, dz=450.0, amp=2.5, radius=2200.0, zc=1300.0,
                                noise=0.2)
    elif kind == 1:
        wl = configs.moist_blob(nx=nx, ny=ny, nz=nz, dz=5000.0 / nz, periodic=periodic,
                                rain_fallout=int(rng.integers(1, 3)) if eq == 0 else 1)
    else:
        wl = configs.jet_vortex(nx=nx, ny=ny, nz=nz, dx=20000.0, dz=6400.0 / nz, dt=30.0, rmax=60000.0, vmax=8.0,
                                moist=kind == 3, noise=0.3, extra_basic=1.0)
    if kind != 1:
        wl.periodic_ew_boundaries = 0
    for side in ("north", "south", "east", "west"):
        setattr(wl, "boundary_width_" + side, int(rng.integers(0, 4)))
    # the first damped level; NZ-1 itself would divide by zero in the
    # reference's coefficient (damping.cpp:1158-1159)
    wl.rayleigh_damping_z = int(rng.integers(max(1, nz - 5), nz - 1))
    if rng.random() < 0.4:
        wl.use_explicit_diffusion, wl.diffusion_order = 1, int(rng.choice([2, 4, 6]))
        wl.kdiffh = wl.kdiffv = float(rng.uniform(0.001, 0.01))
    if eq == 0 and rng.random() < 0.4:
        wl.turbulence_option = 1
        wl.use_surface_heat_flux = int(rng.integers(0, 2))
        wl.water_temp = float(rng.uniform(24.0, 30.0))
    if eq == 1:
        wl.linear_model = 1
    elif eq == 2:
        wl.hydrostatic, wl.periodic_ew_boundaries = 1, 0
    return wl, int(rng.integers(2, 4))


@pytest.mark.parametrize("seed", range(NCASES))
def test_random_configuration_bit_exact(seed):
    wl, nsteps = _case(7000 + seed)
    ref = O.run_reference(wl, "run", nsteps)
    cols = {k: ref[k] for k in abi.COLUMN_NAMES}
    cols["f"] = ref["f"]
    o = O.Oracle(wl, cols)
    assert o.step(nsteps) == 0
    st = o.state()
    checked = 0
    for k, v in st.items():
        if k in ref:
            np.testing.assert_array_equal(v, ref[k], err_msg=f"seed {seed}: {k}")
            assert np.isfinite(v).all(), (seed, k)  # equal NaNs would pass the comparison
            checked += 1
    assert checked >= 13
    if wl.turbulence_option:
        for k, f in abi.TURB_NAMES.items():
            if k in ref:
                np.testing.assert_array_equal(o.get(f), ref[k], err_msg=f"seed {seed}: {k}")


NICE = 16


def _ice_case(seed: int):
    """a seeded ice-scheme configuration: grid, sponge widths, periodic east-
    west, fallout, explicit diffusion, turbulence with or without the ocean
    fluxes, the blob's height and its snow and ice"""
    rng = np.random.default_rng(seed)
    nx = int(rng.choice([13, 15, 16, 19, 24]))
    ny = int(rng.choice([12, 14, 17]))
    nz = int(rng.choice([8, 12, 16, 20]))
    rf = int(rng.integers(1, 3))
    periodic = int(rng.integers(0, 2))
    wl = configs.ice_cloud(nx=nx, ny=ny, nz=nz, dz=12000.0 / nz, rain_fallout=rf, periodic=periodic,
                           zc=float(rng.uniform(3000.0, 8000.0)), qi=float(rng.uniform(1e-4, 8e-4)),
                           qs=float(rng.uniform(2e-4, 2e-3)), seed=3000 + seed)
    for side in ("north", "south", "east", "west"):
        setattr(wl, "boundary_width_" + side, int(rng.integers(0, 4)))
    wl.rayleigh_damping_z = int(rng.integers(max(1, nz - 5), nz - 1))
    if rng.random() < 0.4:
        wl.use_explicit_diffusion, wl.diffusion_order = 1, int(rng.choice([2, 4, 6]))
        wl.kdiffh = wl.kdiffv = float(rng.uniform(0.001, 0.01))
    if rng.random() < 0.4:
        wl.turbulence_option = 1
        wl.use_surface_heat_flux = int(rng.integers(0, 2))
        wl.water_temp = float(rng.uniform(24.0, 30.0))
    return wl, int(rng.integers(2, 4))


@pytest.mark.parametrize("seed", range(NICE))
def test_random_ice_configuration_bit_exact(seed):
    """the ice scheme on seeded configurations: every field of the dump,
    the snow intercept and (with turbulence) the saturation record"""
    wl, nsteps = _ice_case(8000 + seed)
    ref = O.run_reference(wl, "run", nsteps)
    cols = {k: ref[k] for k in abi.COLUMN_NAMES}
    cols["f"] = ref["f"]
    o = O.Oracle(wl, cols)
    assert o.step(nsteps) == 0
    st = o.state()
    checked = 0
    for k, v in st.items():
        if k in ref:
            np.testing.assert_array_equal(v, ref[k], err_msg=f"seed {seed}: {k}")
            assert np.isfinite(v).all(), (seed, k)
            checked += 1
    assert checked >= 24
    if wl.turbulence_option:
        for k, f in abi.TURB_NAMES.items():
            if k in ref:
                np.testing.assert_array_equal(o.get(f), ref[k], err_msg=f"seed {seed}: {k}")


@pytest.mark.parametrize("seed", range(6))
def test_random_hydrostatic_ice_bit_exact(seed):
    """the ice scheme in the hydrostatic set (the oracle only; the library
    builds the ice scheme for the non-hydrostatic step): the hydrostatic
    pressure's buoyancy less snow and ice (pressure.cpp:459-475) and the ice
    scheme's Exner pressure, against the reference's HYDROSTATIC build"""
    wl, nsteps = _ice_case(8100 + seed)
    wl.hydrostatic, wl.periodic_ew_boundaries, wl.turbulence_option = 1, 0, 0
    wl.dx = wl.dy = 2000.0
    ref = O.run_reference(wl, "run", nsteps)
    cols = {k: ref[k] for k in abi.COLUMN_NAMES}
    cols["f"] = ref["f"]
    o = O.Oracle(wl, cols)
    assert o.step(nsteps) == 0
    checked = 0
    for k, v in o.state().items():
        if k in ref:
            np.testing.assert_array_equal(v, ref[k], err_msg=f"seed {seed}: {k}")
            assert np.isfinite(v).all(), (seed, k)
            checked += 1
    assert checked >= 24
