"""The FP32 four-level advection kernel (k_advect_quad) against the per-level
tile kernel (k_advect_tile) on the same inputs.

Both evaluate the same face and tendency expressions level by level, so a
single advection operator must agree bit for bit; whole steps are compared
to a relative L2 of 1e-6 (the pressure solve's FFT runs the same code on
both sides, so any difference would come from the advection alone).
GA_ADVECT selects the kernel when a context is created.
"""
import numpy as np
import pytest

from model_gb300 import abi, anelastic, configs
from tests import fixtures as fx

pytestmark = pytest.mark.gpu

ADVECT_OPS = {
    "advect_uvw": (abi.PROG_NAMES.index("u"), abi.PROG_NAMES.index("v"), abi.PROG_NAMES.index("w")),
    "advect_theta": (abi.PROG_NAMES.index("th"),),
    "advect_micro": (abi.PROG_NAMES.index("qv"), abi.PROG_NAMES.index("qc"), abi.PROG_NAMES.index("qr")),
}


@pytest.fixture(scope="module", autouse=True)
def _built():
    from model_gb300 import build
    build.build()


def _pair(monkeypatch, wl, blocks=3, tile="4x8", faces="single"):
    """a per-level tile context and a four-level one (tile TIxTJ) whose
    registers are sized for `blocks` blocks per SM; faces "rows" evaluates the
    east and north faces by sliding rows"""
    ms = []
    for mode in ("tile", "quad"):
        monkeypatch.setenv("GA_ADVECT", mode)
        monkeypatch.setenv("GA_ADVECT_BLOCKS", str(blocks))
        monkeypatch.setenv("GA_ADVECT_TILE", tile)
        monkeypatch.setenv("GA_ADVECT_FACES", faces)
        ms.append(anelastic.Model(wl, abi.GA_PREC_F32))
    for v in ("GA_ADVECT", "GA_ADVECT_BLOCKS", "GA_ADVECT_TILE", "GA_ADVECT_FACES"):
        monkeypatch.delenv(v)
    return ms


def _perturb(ms, wl, seed):
    """random current and start-of-step states, the same in every model;
    moisture straddles zero so that clipping takes both branches"""
    rng = np.random.default_rng(seed)
    n = wl.nx * wl.ny * wl.nz
    nprog = 7 if wl.microphysics_option else 4
    scale = [2.0, 2.0, 0.5, 0.3, 1e-3, 4e-4, 4e-4]
    for f in range(nprog):
        for slot in (abi.GA_SLOT_CUR, abi.GA_SLOT_M):
            x = rng.standard_normal(n) * scale[f]
            if f >= 5:
                x = x + 2e-4
            for m in ms:
                m.set(f, slot, x)


@pytest.mark.parametrize("faces", ["single", "rows"])
@pytest.mark.parametrize("tile", ["4x8", "4x4", "8x4", "2x8", "8x8"])
@pytest.mark.parametrize("blocks", [3, 4])
@pytest.mark.parametrize("case", ["moist_rf1", "moist_rf2", "dry"])
def test_single_advection_operator_bit_identical(monkeypatch, case, blocks, tile, faces):
    if case == "dry":
        wl = configs.dry_bubble(nx=30, ny=26, nz=20, nsteps=2)
    else:
        wl = configs.moist_blob(nx=30, ny=26, nz=16, rain_fallout=1 if case == "moist_rf1" else 2)
    ms = _pair(monkeypatch, wl, blocks, tile, faces)
    _perturb(ms, wl, 11)
    for op, fields in ADVECT_OPS.items():
        if op == "advect_micro" and not wl.microphysics_option:
            continue
        for m in ms:
            m.op(op, 0.5)
        for f in fields:
            a, b = (m.get(f, abi.GA_SLOT_P) for m in ms)
            np.testing.assert_array_equal(b, a, err_msg=f"{case} {op} field {abi.PROG_NAMES[f]}")


@pytest.mark.parametrize("faces", ["single", "rows"])
@pytest.mark.parametrize("blocks", [3, 4])
@pytest.mark.parametrize("case", ["moist_blob", "thunderstorm_small", "dry_bubble", "nz_not_multiple_of_4"])
def test_steps_match_tile_kernel(monkeypatch, case, blocks, faces):
    if case == "moist_blob":
        wl = configs.moist_blob(nx=30, ny=26, nz=16, nsteps=6)
    elif case == "thunderstorm_small":
        wl = configs.thunderstorm(nx=44, ny=38, nsteps=6)
    elif case == "dry_bubble":
        wl = configs.dry_bubble(nx=34, ny=30, nz=20, nsteps=6)
    else:  # falls back to the tile kernel: both contexts run the same code
        wl = configs.moist_blob(nx=30, ny=26, nz=18, nsteps=6)
    ms = _pair(monkeypatch, wl, blocks, faces=faces)
    for m in ms:
        m.step(wl.nsteps)
    nprog = 7 if wl.microphysics_option else 4
    worst = 0.0
    for f in list(range(nprog)) + [abi.GA_PI]:
        a, b = (m.get(f) for m in ms)
        e = fx.rel_l2(b, a)
        worst = max(worst, e)
        assert e <= 1e-6, f"{case} field {f}: rel L2 {e:.3e}"
    print(case, f"worst rel L2 {worst:.2e}")


def test_autotuner_reports_the_kernel(monkeypatch):
    wl = configs.thunderstorm(nx=44, ny=38, nsteps=2)
    monkeypatch.setenv("GA_ADVECT", "quad")
    m = anelastic.Model(wl, abi.GA_PREC_F32)
    info = m.tune()
    assert "four levels per thread" in info, info
    monkeypatch.setenv("GA_ADVECT", "tile")
    m2 = anelastic.Model(wl, abi.GA_PREC_F32)
    info2 = m2.tune()
    assert "four levels per thread" not in info2, info2


@pytest.mark.parametrize("case", ["moist_blob", "periodic_rf2", "dry_bubble", "thunderstorm_small"])
def test_post_quad_matches_column_kernel(monkeypatch, case):
    """k_post_quad against k_post (GA_POST=column): whole steps, every
    prognostic field, pi and the accumulated rain bit for bit"""
    if case == "moist_blob":
        wl = configs.moist_blob(nx=30, ny=26, nz=16, nsteps=4)
    elif case == "periodic_rf2":
        wl = configs.moist_blob(nx=30, ny=24, nz=16, nsteps=4, periodic=1, rain_fallout=2)
    elif case == "dry_bubble":
        wl = configs.dry_bubble(nx=34, ny=30, nz=20, nsteps=4)
    else:
        wl = configs.thunderstorm(nx=44, ny=38, nsteps=4)
    ms = []
    for mode in ("column", "quad"):
        monkeypatch.setenv("GA_POST", mode)
        ms.append(anelastic.Model(wl, abi.GA_PREC_F32))
    monkeypatch.delenv("GA_POST")
    for m in ms:
        m.step(wl.nsteps)
    nprog = 7 if wl.microphysics_option else 4
    fields = list(range(nprog)) + [abi.GA_PI] + ([abi.GA_ACCRAIN] if wl.microphysics_option else [])
    for f in fields:
        for slot in ((abi.GA_SLOT_CUR, abi.GA_SLOT_M) if f < nprog else (abi.GA_SLOT_CUR,)):
            a, b = (m.get(f, slot) for m in ms)
            np.testing.assert_array_equal(b, a, err_msg=f"{case} field {f} slot {slot}")


@pytest.mark.parametrize("case", ["moist_blob", "turbulence", "hydrostatic"])
def test_fused_kessler_matches_separate_kernel(monkeypatch, case):
    """Kessler inside the step's last four-level pass against the separate
    k_kessler (GA_KESSLER=separate): every field, pi, the rain total and the
    turbulence scheme's saturation record bit for bit, on a raining blob"""
    wl = configs.moist_blob(nx=36, ny=30, nz=16, nsteps=5)
    if case == "turbulence":
        wl.turbulence_option, wl.use_surface_heat_flux = 1, 1
    elif case == "hydrostatic":
        wl.hydrostatic, wl.dx, wl.dy = 1, 2000.0, 2000.0
    ms = []
    for mode in ("separate", "fused"):
        monkeypatch.setenv("GA_KESSLER", mode)
        ms.append(anelastic.Model(wl, abi.GA_PREC_F32))
    monkeypatch.delenv("GA_KESSLER")
    for m in ms:
        m.step(wl.nsteps)
    fields = list(range(7)) + [abi.GA_PI, abi.GA_ACCRAIN] + ([abi.GA_SATURATED] if wl.turbulence_option else [])
    for f in fields:
        a, b = (m.get(f) for m in ms)
        np.testing.assert_array_equal(b, a, err_msg=f"{case} field {f}")
    assert np.abs(ms[1].get(abi.GA_ACCRAIN)).max() > 0


@pytest.mark.parametrize("form", ["pair", "1024"])
@pytest.mark.parametrize("case", ["thunderstorm_small", "moist_blob_odd"])
def test_spectral_x_pair_matches_single_cta(monkeypatch, case, form):
    """the fused x kernel as CTA pairs (GA_SPECTRAL_X=pair) or as one block
    of 1024 threads (GA_SPECTRAL_X=1024) against one 256-thread CTA per
    y-wavenumber: whole steps bit for bit (an odd interior size splits the
    lines and the columns unevenly)"""
    if case == "thunderstorm_small":
        wl = configs.thunderstorm(nx=44, ny=38, nsteps=4)
    else:
        wl = configs.moist_blob(nx=31, ny=27, nz=17, nsteps=4)
    ms = []
    for mode in ("single", form):
        monkeypatch.setenv("GA_SPECTRAL_X", mode)
        ms.append(anelastic.Model(wl, abi.GA_PREC_F32))
    monkeypatch.delenv("GA_SPECTRAL_X")
    for m in ms:
        m.step(wl.nsteps)
    nprog = 7 if wl.microphysics_option else 4
    for f in list(range(nprog)) + [abi.GA_PI]:
        a, b = (m.get(f) for m in ms)
        np.testing.assert_array_equal(b, a, err_msg=f"{case} field {f}")


def _staged_pair(monkeypatch, wl, cand):
    """a four-level context reading the fields from global memory and one
    staging them into shared memory by the tensor memory accelerator
    (candidate `cand` of the staged kernel: tile, level slab, blocks per SM)"""
    ms = []
    for mode in ("quad", "tma"):
        monkeypatch.setenv("GA_ADVECT", mode)
        monkeypatch.setenv("GA_ADVECT_TMA", str(cand))
        ms.append(anelastic.Model(wl, abi.GA_PREC_F32))
    monkeypatch.delenv("GA_ADVECT")
    monkeypatch.delenv("GA_ADVECT_TMA")
    return ms


@pytest.mark.parametrize("cand", [0, 1, 2, 3])
@pytest.mark.parametrize("case", ["moist_rf1", "moist_rf2", "dry", "tall_slabs"])
def test_staged_advection_operator_bit_identical(monkeypatch, case, cand):
    """k_advect_tma (halo boxes in shared memory) against k_advect_quad on
    one advection operator: every forecast field bit for bit.  tall_slabs
    has 20 levels, so the last 8- or 16-level slab is cut at NZ and the
    slabs above the bottom need the top faces of the quad below them."""
    if case == "dry":
        wl = configs.dry_bubble(nx=30, ny=26, nz=20, nsteps=2)
    elif case == "tall_slabs":
        wl = configs.moist_blob(nx=27, ny=29, nz=20)
    else:
        wl = configs.moist_blob(nx=30, ny=26, nz=16, rain_fallout=1 if case == "moist_rf1" else 2)
    ms = _staged_pair(monkeypatch, wl, cand)
    _perturb(ms, wl, 13)
    for op, fields in ADVECT_OPS.items():
        if op == "advect_micro" and not wl.microphysics_option:
            continue
        for m in ms:
            m.op(op, 0.5)
        for f in fields:
            a, b = (m.get(f, abi.GA_SLOT_P) for m in ms)
            np.testing.assert_array_equal(b, a, err_msg=f"{case} cand {cand} {op} field {abi.PROG_NAMES[f]}")


@pytest.mark.parametrize("cand", [0, 1, 2, 3])
@pytest.mark.parametrize("case", ["thunderstorm_small", "dry_bubble"])
def test_staged_advection_steps_bit_identical(monkeypatch, case, cand):
    """whole steps (the mirror copies ride in the advection launch) with the
    staged kernel against the four-level kernel: every field bit for bit"""
    if case == "thunderstorm_small":
        wl = configs.thunderstorm(nx=44, ny=38, nsteps=4)
    else:
        wl = configs.dry_bubble(nx=34, ny=30, nz=20, nsteps=4)
    ms = _staged_pair(monkeypatch, wl, cand)
    for m in ms:
        m.step(wl.nsteps)
    nprog = 7 if wl.microphysics_option else 4
    for f in list(range(nprog)) + [abi.GA_PI]:
        for slot in (abi.GA_SLOT_CUR, abi.GA_SLOT_M):
            if f == abi.GA_PI and slot != abi.GA_SLOT_CUR:
                continue
            a, b = (m.get(f, slot) for m in ms)
            np.testing.assert_array_equal(b, a, err_msg=f"{case} cand {cand} field {f} slot {slot}")


def test_autotuner_races_the_staged_kernel(monkeypatch):
    wl = configs.thunderstorm(nx=44, ny=38, nsteps=2)
    monkeypatch.setenv("GA_ADVECT", "tma")
    m = anelastic.Model(wl, abi.GA_PREC_F32)
    info = m.tune()
    assert "staged by TMA" in info, info


@pytest.mark.parametrize("faces", ["single", "rows"])
@pytest.mark.parametrize("rf", [1, 2])
def test_ice_step_four_level_matches_tile(monkeypatch, faces, rf):
    """the ice scheme's FP32 step with the four-level kernel (ice buoyancy,
    the stored Rutledge rain fall speed, the snow and ice pass) against the
    per-level kernels (k_advect_tile and k_advect_ice): every prognostic
    field, snow and ice within 1e-5 relative L2 after 4 steps.  The two
    snow and ice advections contract their multiply-adds differently, and
    the microphysics' thresholds let last-bit differences grow: cloud ice
    differs by 1.1e-6 with semi-Lagrangian fallout."""
    wl = configs.ice_cloud(nx=40, ny=36, nz=32, dz=375.0, rain_fallout=rf)
    ms = _pair(monkeypatch, wl, tile="4x8", faces=faces)
    for m in ms:
        m.step(4)
    for f in list(range(7)) + [abi.GA_QS, abi.GA_QI]:
        a, b = ms[0].get(f), ms[1].get(f)
        assert np.isfinite(b).all(), f
        e = fx.rel_l2(b, a)
        assert e <= 1e-5, (f, e)
