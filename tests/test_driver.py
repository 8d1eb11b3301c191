"""The C++ run driver (model_gb300/ga_driver, csrc/ga_driver.cpp) on the C ABI.

  - a moist run of 6 steps written every 3 steps, against the CPU oracle
    (1e-10 relative L2, the bound of the FP64 path);
  - the optional physics settings (explicit diffusion, turbulence with
    surface fluxes) against the oracle;
  - restart: 3 steps, then 3 more from the written state file, against the
    6-step run: every record of the state file (all rotation slots, pi, fall
    speed, rain, the saturation record, counters) bit for bit, in FP64 and
    in FP32, with and without the turbulence scheme;
  - the ice scheme: a run against the oracle (snow, ice, their fall speeds,
    snow accumulation and the snow intercept) and its restart;
  - a missing input field is an error, reported before any context exists
    (runs without a GPU).
"""
import os
import subprocess

import numpy as np
import pytest

from model_gb300 import abi, configs
from tests import fixtures as fx


@pytest.fixture(scope="module")
def driver():
    from model_gb300 import build
    build.build()
    assert os.path.exists(build.DRIVER)
    return build.DRIVER


def _bundle(wl):
    from oracle import oracle as O
    return O.workload_bundle(wl)


def _run(driver, inp, prefix, *args):
    r = subprocess.run([driver, inp, prefix, *args], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r.stdout


@pytest.mark.gpu
def test_driver_run_matches_oracle(driver, tmp_path):
    from oracle import oracle as O
    from oracle.ga_bundle import read_bundle, write_bundle
    wl = configs.moist_blob(nx=24, ny=22, nz=16, nsteps=6)
    inp = str(tmp_path / "in.bin")
    write_bundle(inp, _bundle(wl))
    out = _run(driver, inp, str(tmp_path / "run"), "--steps", "6", "--every", "3")
    assert "step 3:" in out and "step 6:" in out
    st = read_bundle(str(tmp_path / "run_6.bin"))
    o = O.Oracle(wl)
    assert o.step(6) == 0
    for f, name in enumerate(abi.PROG_NAMES):
        e = fx.rel_l2(st[name], o.get(f))
        assert e <= 1e-10, f"{name}: rel L2 {e:.3e}"
    assert fx.rel_l2(st["pi"], o.get(abi.GA_PI)) <= 1e-10
    assert st["bigcounter"][0] == 6 and st["mtime"][0] == 6 * wl.dt


@pytest.mark.gpu
def test_driver_physics_switches_match_oracle(driver, tmp_path):
    """explicit diffusion and the turbulence scheme with surface fluxes,
    switched on through the input's optional settings"""
    from oracle import oracle as O
    from oracle.ga_bundle import read_bundle, write_bundle
    wl = configs.moist_blob(nx=24, ny=22, nz=16, nsteps=4)
    wl.use_explicit_diffusion, wl.diffusion_order, wl.kdiffh = 1, 6, 0.003
    wl.turbulence_option, wl.use_surface_heat_flux, wl.water_temp = 1, 1, 27.0
    inp = str(tmp_path / "in.bin")
    write_bundle(inp, _bundle(wl))
    _run(driver, inp, str(tmp_path / "run"), "--steps", "4")
    st = read_bundle(str(tmp_path / "run_4.bin"))
    o = O.Oracle(wl)
    assert o.step(4) == 0
    for f, name in enumerate(abi.PROG_NAMES):
        e = fx.rel_l2(st[name], o.get(f))
        assert e <= 1e-10, f"{name}: rel L2 {e:.3e}"
    np.testing.assert_array_equal(st["is_saturated"], o.get(abi.GA_SATURATED))


@pytest.mark.gpu
def test_driver_ice_run_matches_oracle(driver, tmp_path):
    """the ice scheme through the driver: every prognostic field including
    snow and ice, the ice fall speed, the accumulations and the snow
    intercept against the oracle after 6 steps written every 3"""
    from oracle import oracle as O
    from oracle.ga_bundle import read_bundle, write_bundle
    wl = configs.ice_cloud(nx=24, ny=22, nz=20, nsteps=6)
    inp = str(tmp_path / "in.bin")
    write_bundle(inp, _bundle(wl))
    _run(driver, inp, str(tmp_path / "run"), "--steps", "6", "--every", "3")
    st = read_bundle(str(tmp_path / "run_6.bin"))
    o = O.Oracle(wl)
    assert o.step(6) == 0
    ref = o.state()
    for k in ("u", "v", "w", "th", "qv", "qc", "qr", "qs", "qi", "qs_m", "qi_m", "pi", "its", "accrain",
              "accsnow", "n0s"):
        e = fx.rel_l2(st[k], ref[k])
        assert e <= 1e-10, f"{k}: rel L2 {e:.3e}"


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("turbulence", [0, 1])
@pytest.mark.parametrize("scheme", ["kessler", "ice"])
def test_driver_restart_is_exact(driver, tmp_path, precision, turbulence, scheme):
    from oracle.ga_bundle import read_bundle, write_bundle
    if scheme == "ice":
        wl = configs.ice_cloud(nx=24, ny=22, nz=20, nsteps=6)
    else:
        wl = configs.moist_blob(nx=24, ny=22, nz=16, nsteps=6)
    wl.turbulence_option = turbulence
    inp = str(tmp_path / "in.bin")
    write_bundle(inp, _bundle(wl))
    _run(driver, inp, str(tmp_path / "full"), "--steps", "6", "--every", "3", "--precision", precision)
    _run(driver, inp, str(tmp_path / "cont"), "--steps", "3", "--restart", str(tmp_path / "full_3.bin"),
         "--precision", precision)
    a = read_bundle(str(tmp_path / "full_6.bin"))
    b = read_bundle(str(tmp_path / "cont_6.bin"))
    assert sorted(a) == sorted(b)
    for k in a:
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)


def test_driver_rejects_missing_input(driver, tmp_path):
    from oracle.ga_bundle import write_bundle
    wl = configs.moist_blob(nx=24, ny=22, nz=16, nsteps=2)
    b = _bundle(wl)
    del b["qc"]
    inp = str(tmp_path / "in.bin")
    write_bundle(inp, b)
    r = subprocess.run([driver, inp, str(tmp_path / "x"), "--steps", "2"], capture_output=True, text=True)
    assert r.returncode != 0 and "qc" in r.stderr
    b = _bundle(configs.ice_cloud(nx=24, ny=22, nz=12, nsteps=2))
    del b["qs"]
    write_bundle(inp, b)
    r = subprocess.run([driver, inp, str(tmp_path / "x"), "--steps", "2"], capture_output=True, text=True)
    assert r.returncode != 0 and "qs" in r.stderr
