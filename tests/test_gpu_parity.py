"""GPU parity: the CUDA path against the reference's own outputs (golden
fixtures) and against the CPU oracle.

Tolerances (relative L2 over a whole field, FP64):
  - operators without transcendental functions or transforms: bit exact
    (the FP64 kernels are compiled without FMA contraction and keep the
    reference's evaluation order);
  - operators with CUDA pow/exp (Kessler, fall speed) or the FFT: 1e-12;
  - full steps: 1e-10 (the bound for the plain FP64 path).
"""
import numpy as np
import pytest

from model_gb300 import abi, anelastic
from tests import fixtures as fx

pytestmark = pytest.mark.gpu

EXACT_OPS = {"advect_uvw", "advect_theta", "zero_moisture", "bc", "bc_micro", "rayleigh", "explicit_diffusion"}
# the turbulence scheme: operator fixtures turb_*.npz (test_turbulence_operator_matches_reference)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from model_gb300 import build
    build.build()


@pytest.mark.parametrize("name", fx.run_names())
def test_full_steps_match_reference(name):
    d = fx.load(name)
    wl = fx.workload(d)
    m = anelastic.Model(wl, abi.GA_PREC_F64, columns=fx.columns(d))
    bc0 = 0
    if "bigcounter0" in wl.fields:  # a run later in the model's life
        bc0 = int(np.ravel(wl.fields["bigcounter0"])[0])
        m.set_counters(bc0, float(np.ravel(wl.fields["mtime0"])[0]))
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
    assert m.counters()[0] == bc0 + wl.nsteps
    if wl.turbulence_option:  # the last step's coefficients, tendencies and saturation record
        for k, f in abi.TURB_NAMES.items():
            if "out_" + k not in d:
                continue
            got = m.get(f)
            if k == "is_saturated":
                np.testing.assert_array_equal(got, d["out_" + k], err_msg=f"{name}:{k}")
            else:
                e = fx.rel_l2(got, d["out_" + k])
                assert e <= 1e-10, f"{name}:{k} rel L2 {e:.3e}"


@pytest.mark.parametrize("name", fx.ops_names())
@pytest.mark.parametrize("op", ["advect_uvw", "solve_pressure", "integrate_non_hydro", "advect_theta",
                                "advect_micro", "zero_moisture", "bc", "bc_micro", "kessler", "rayleigh",
                                "explicit_diffusion"])
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


@pytest.mark.parametrize("name", fx.turb_names())
@pytest.mark.parametrize("op", ["turbulence", "kessler"])
def test_turbulence_operator_matches_reference(name, op):
    """calculate_diff_tend on a state whose rotation slots differ, with a
    seeded saturation record: bit exact for the dry scheme (no pow or exp),
    1e-12 relative L2 where the saturated Brunt-Vaisala frequency or the
    surface fluxes call pow and exp; Kessler's saturation record bit exact"""
    d = fx.load(name)
    wl = fx.workload(d)
    if op == "kessler" and not wl.microphysics_option:
        pytest.skip("dry case")
    m = anelastic.Model(wl, abi.GA_PREC_F64)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        if f < abi.GA_NPROG and f >= (7 if wl.microphysics_option else 4):
            continue
        m.set(f, slot, v)
    m.op(op, float(d[f"step_{op}"]))
    outs = [k for k in d if k.startswith(op + "__")]
    assert len(outs) >= (6 if op == "turbulence" else 5)
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        got = m.get(f, slot)
        if not wl.microphysics_option or key == "is_saturated":
            np.testing.assert_array_equal(got, d[k], err_msg=f"{op}:{key}")
        else:
            e = fx.rel_l2(got, d[k])
            assert e <= 1e-12, f"{op}:{key} rel L2 {e:.3e}"


@pytest.mark.parametrize("name", fx.linop_names())
@pytest.mark.parametrize("op", ["advect_uvw", "advect_theta", "advect_micro", "integrate_non_hydro"])
def test_linear_operator_matches_reference(name, op):
    """the linearised model's operators against the reference's ISLINEAR
    build: bit exact without the FFT, 1e-12 with it"""
    d = fx.load(name)
    wl = fx.workload(d)
    m = anelastic.Model(wl, abi.GA_PREC_F64)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        m.set(f, slot, v)
    m.op(op, float(d[f"step_{op}"]))
    outs = [k for k in d if k.startswith(op + "__")]
    assert outs
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        got = m.get(f, slot)
        if op != "integrate_non_hydro":
            np.testing.assert_array_equal(got, d[k], err_msg=f"{op}:{key}")
        else:
            e = fx.rel_l2(got, d[k])
            assert e <= 1e-12, f"{op}:{key} rel L2 {e:.3e}"


@pytest.mark.parametrize("name", fx.hydop_names())
@pytest.mark.parametrize("op", ["advect_uvw", "solve_pressure", "integrate_non_hydro", "kessler", "bc", "rayleigh"])
def test_hydrostatic_operator_matches_reference(name, op):
    """the operators of the hydrostatic set against the reference's
    HYDROSTATIC build: bit exact for the advection, boundary conditions and
    damping; 1e-12 with the FFT or pow/exp"""
    d = fx.load(name)
    wl = fx.workload(d)
    m = anelastic.Model(wl, abi.GA_PREC_F64)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        m.set(f, slot, v)
    m.op(op, float(d[f"step_{op}"]))
    outs = [k for k in d if k.startswith(op + "__")]
    assert outs
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        got = m.get(f, slot)
        if op in ("advect_uvw", "bc", "rayleigh"):
            np.testing.assert_array_equal(got, d[k], err_msg=f"{op}:{key}")
        else:
            e = fx.rel_l2(got, d[k])
            assert e <= 1e-12, f"{op}:{key} rel L2 {e:.3e}"


@pytest.mark.parametrize("moist", [False, True])
def test_hydrostatic_thunderstorm_size_vs_oracle(moist):
    """the hydrostatic set at 128x128x48 (dx = 2 km): FP64 against the
    oracle after 6 steps, with explicit diffusion; FP32 against FP64"""
    from model_gb300 import configs
    wl = configs.thunderstorm(dx=2000.0) if moist else configs.dry_bubble(nx=128, ny=128, nz=48, dx=2000.0,
                                                                          dz=400.0, dt=4.0, radius=8000.0)
    wl.hydrostatic = 1
    wl.use_explicit_diffusion, wl.diffusion_order, wl.kdiffh, wl.kdiffv = 1, 4, 0.002, 0.002
    _oracle_compare(wl, 6, 1e-10)
    a = anelastic.Model(wl, abi.GA_PREC_F32)
    b = anelastic.Model(wl, abi.GA_PREC_F64)
    a.step(6)
    b.step(6)
    for f in range(7 if moist else 4):
        e = fx.rel_l2(a.get(f), b.get(f))
        assert e <= 1e-3, (abi.PROG_NAMES[f], e)


def _oracle_compare(wl, nsteps, tol, counters=None):
    from oracle import oracle as O
    cols = anelastic.build_columns(wl)
    m = anelastic.Model(wl, abi.GA_PREC_F64, columns=cols)
    o = O.Oracle(wl, cols)
    if counters:
        m.set_counters(*counters)
        o.set_counters(*counters)
    m.step(nsteps)
    assert o.step(nsteps) == 0
    worst = {}
    nprog = 7 if wl.microphysics_option else 4
    extra = [abi.GA_QS, abi.GA_QI, abi.GA_VTI] if wl.microphysics_option == 2 else []
    for f in list(range(nprog)) + [abi.GA_PI] + extra:
        worst[f] = fx.rel_l2(m.get(f), o.get(f))
    print(wl.name, nsteps, {k: f"{v:.2e}" for k, v in worst.items()})
    for f, e in worst.items():
        assert e <= tol, f"field {f}: rel L2 {e:.3e}"
    return worst


def test_dry_bubble_full_config_fp64_vs_oracle():
    """Dry warm bubble, 64x64x40, 100 steps: every prognostic field within
    1e-10 relative L2 of the oracle."""
    from model_gb300 import configs
    _oracle_compare(configs.dry_bubble(), 100, 1e-10)


def test_thunderstorm_fp64_vs_oracle_short():
    """Kessler thunderstorm at full size (128x128x48), 8 steps (the oracle
    needs about 2 s per step)."""
    from model_gb300 import configs
    _oracle_compare(configs.thunderstorm(), 8, 1e-10)


def test_periodic_rf2_fp64_vs_oracle():
    from model_gb300 import configs
    _oracle_compare(configs.moist_blob(nx=30, ny=24, nz=16, periodic=1, rain_fallout=2), 12, 1e-10)


def test_fp32_error_against_fp64():
    """FP32 path: relative L2 error against FP64 after 60 thunderstorm steps."""
    from model_gb300 import configs
    wl = configs.thunderstorm()
    a = anelastic.Model(wl, abi.GA_PREC_F32)
    b = anelastic.Model(wl, abi.GA_PREC_F64)
    a.step(60)
    b.step(60)
    errs = {abi.PROG_NAMES[f]: fx.rel_l2(a.get(f), b.get(f)) for f in range(7)}
    print("fp32 vs fp64 after 60 steps", {k: f"{v:.2e}" for k, v in errs.items()})
    for k in ("u", "v", "w", "th", "qv"):
        assert errs[k] <= 1e-4, (k, errs[k])


@pytest.mark.parametrize("order", [2, 4, 6])
def test_explicit_diffusion_thunderstorm_vs_oracle(order):
    """full-size thunderstorm with explicit diffusion of each order: FP64
    against the oracle after 6 steps, and FP32 against FP64"""
    from model_gb300 import configs
    wl = configs.thunderstorm()
    wl.use_explicit_diffusion, wl.diffusion_order, wl.kdiffh, wl.kdiffv = 1, order, 0.004, 0.004
    _oracle_compare(wl, 6, 1e-10)
    a = anelastic.Model(wl, abi.GA_PREC_F32)
    b = anelastic.Model(wl, abi.GA_PREC_F64)
    a.step(6)
    b.step(6)
    for f in range(7):
        e = fx.rel_l2(a.get(f), b.get(f))
        assert e <= 1e-4, (abi.PROG_NAMES[f], e)


@pytest.mark.parametrize("sfc", [0, 1])
def test_turbulence_thunderstorm_vs_oracle(sfc):
    """full-size thunderstorm with the turbulence scheme (and the ocean
    surface fluxes): FP64 against the oracle after 6 steps, FP32 against
    FP64"""
    from model_gb300 import configs
    wl = configs.thunderstorm()
    wl.turbulence_option, wl.use_surface_heat_flux, wl.water_temp = 1, sfc, 29.0
    _oracle_compare(wl, 6, 1e-10)
    a = anelastic.Model(wl, abi.GA_PREC_F32)
    b = anelastic.Model(wl, abi.GA_PREC_F64)
    a.step(6)
    b.step(6)
    for f in range(7):
        e = fx.rel_l2(a.get(f), b.get(f))
        assert e <= 1e-4, (abi.PROG_NAMES[f], e)
    assert fx.rel_l2(b.get(abi.GA_KMIX), a.get(abi.GA_KMIX)) <= 1e-3


def test_turbulence_dry_jet_vs_oracle():
    from model_gb300 import configs
    wl = configs.jet_vortex(nx=64, ny=48, nz=24, dx=20000.0, dz=800.0, dt=30.0, rmax=200000.0, vmax=12.0,
                            noise=0.3, extra_basic=1.0)
    wl.turbulence_option = 1
    _oracle_compare(wl, 10, 1e-10)


@pytest.mark.parametrize("moist", [False, True])
def test_linear_model_monsoon_size_vs_oracle(moist):
    """the linearised model about the 192x128x32 jet basic state (dt = 120 s,
    a rescaling every 360 steps): FP64 against the oracle over 4 steps that
    cross a rescaling, with explicit diffusion in every stage; FP32 against
    FP64 within 1e-3 (on this state the FP32 step, nonlinear or linearised,
    differs from FP64 by 4e-4 after one step and 2.6e-4 after four, in the
    largest field)"""
    from model_gb300 import configs
    wl = configs.jet_vortex(noise=0.3, extra_basic=1.0, moist=moist)
    wl.linear_model = 1
    wl.use_explicit_diffusion, wl.diffusion_order, wl.kdiffh, wl.kdiffv = 1, 4, 0.002, 0.002
    _oracle_compare(wl, 4, 1e-10, counters=(358, 358 * wl.dt))
    a = anelastic.Model(wl, abi.GA_PREC_F32)
    b = anelastic.Model(wl, abi.GA_PREC_F64)
    for m in (a, b):
        m.set_counters(358, 358 * wl.dt)
        m.step(4)
    for f in range(7 if moist else 4):
        e = fx.rel_l2(a.get(f), b.get(f))
        assert e <= 1e-3, (abi.PROG_NAMES[f], e)


def test_linear_model_rejects_turbulence():
    from model_gb300 import configs
    wl = configs.moist_blob(nx=20, ny=18, nz=12)
    wl.linear_model, wl.turbulence_option = 1, 1
    with pytest.raises(anelastic.GaError):
        anelastic.Model(wl, abi.GA_PREC_F64)


@pytest.mark.parametrize("name", [n for n in fx.run_names() if n.startswith("run_edge_")])
def test_edge_sizes_fp32_against_fp64(name):
    """the edge-size golden cases (12x12x6, prime transform lengths with an
    odd level count, the smallest periodic domain, 128 levels) in FP32 (the
    per-level column kernels where NZ is not a multiple of 4, the four-level
    ones where it is) against FP64"""
    d = fx.load(name)
    wl = fx.workload(d)
    a = anelastic.Model(wl, abi.GA_PREC_F32, columns=fx.columns(d))
    b = anelastic.Model(wl, abi.GA_PREC_F64, columns=fx.columns(d))
    a.step(wl.nsteps)
    b.step(wl.nsteps)
    for f in range(7):
        e = fx.rel_l2(a.get(f), b.get(f))
        assert e <= 1e-4, (name, abi.PROG_NAMES[f], e)


@pytest.mark.parametrize("seed", range(48))
def test_random_configuration_vs_oracle(seed):
    """the GPU's FP64 step against the oracle on the seeded random
    configurations of tests/test_oracle_random.py (grids with prime
    transform lengths and odd level counts, sponge widths, periodic domains,
    rain fallout, explicit diffusion, turbulence, the linearised and
    hydrostatic sets), whose oracle runs equal the reference build's bit for
    bit: every prognostic field and pi within 1e-10"""
    from oracle import oracle as O
    from tests.test_oracle_random import _case
    wl, nsteps = _case(7000 + seed)
    cols = anelastic.build_columns(wl)
    m = anelastic.Model(wl, abi.GA_PREC_F64, columns=cols)
    m.step(nsteps)
    o = O.Oracle(wl, cols)
    assert o.step(nsteps) == 0
    nprog = 7 if wl.microphysics_option else 4
    for f in list(range(nprog)) + [abi.GA_PI]:
        for slot in ((abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M) if f < nprog else (0,)):
            e = fx.rel_l2(m.get(f, slot), o.get(f, slot))
            assert e <= 1e-10, (seed, f, slot, e)


@pytest.mark.parametrize("seed", range(48))
def test_random_configuration_fp32(seed):
    """FP32 (the four-level kernels where NZ is a multiple of 4 and the basic
    state a function of height, the per-level ones elsewhere) against FP64 on
    the seeded random configurations, within 3e-3 relative L2 after their 2-3
    steps (the jets' small w sets the bound: on case 7, a moist jet, the FP32
    step's w differs from FP64's by 1.2e-3 after the second step with or
    without the turbulence scheme, and by 2.2e-4 after the sixth)"""
    from tests.test_oracle_random import _case
    wl, nsteps = _case(7000 + seed)
    cols = anelastic.build_columns(wl)
    a = anelastic.Model(wl, abi.GA_PREC_F32, columns=cols)
    b = anelastic.Model(wl, abi.GA_PREC_F64, columns=cols)
    a.step(nsteps)
    b.step(nsteps)
    for f in range(7 if wl.microphysics_option else 4):
        x, y = a.get(f), b.get(f)
        assert np.isfinite(x).all(), (seed, f)
        e = fx.rel_l2(x, y)
        assert e <= 3e-3, (seed, abi.PROG_NAMES[f], e)


def test_step_is_deterministic():
    from model_gb300 import configs
    wl = configs.moist_blob(nx=40, ny=36, nz=20, nsteps=5)
    outs = []
    for _ in range(2):
        m = anelastic.Model(wl, abi.GA_PREC_F32)
        m.step(5)
        outs.append([m.get(f) for f in range(7)] + [m.get(abi.GA_ACCRAIN)])
    for x, y in zip(*outs):
        np.testing.assert_array_equal(x, y)


@pytest.mark.gpu
def test_autotuner_keeps_state_and_results(_built):
    """ga_tune leaves the state untouched; a tuned context steps to the same
    result (bit-identical tiles; FFT factor orders agree to rounding)."""
    from model_gb300 import configs
    wl = configs.moist_blob(nx=30, ny=26, nz=20)
    a = anelastic.Model(wl, abi.GA_PREC_F64)
    b = anelastic.Model(wl, abi.GA_PREC_F64)
    a.step(3)
    b.step(3)
    before = b.state()
    info = b.tune()
    assert "advect tile" in info and "FFT order" in info
    after = b.state()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    a.step(4)
    b.step(4)
    sa, sb = a.state(), b.state()
    for k in sa:
        assert fx.rel_l2(sb[k], sa[k]) <= 1e-12, k


ICE_EXACT = {"advect_uvw", "bc_micro", "zero_moisture", "explicit_diffusion"}


@pytest.mark.parametrize("name", fx.iceop_names())
@pytest.mark.parametrize("op", ["advect_uvw", "advect_micro", "advect_ice", "kessler", "bc_micro", "zero_moisture",
                                "explicit_diffusion"])
def test_ice_operator_matches_reference(name, op):
    """the ice scheme's operators against the reference build: bit exact
    where no pow or exp enters (the buoyancy with snow and ice, boundary
    conditions, clipping, diffusion), 1e-12 relative L2 for the fall speeds,
    the advection with them and run_rutledge_microphysics; its saturation
    record and the snow intercept's source point exact"""
    d = fx.load(name)
    if f"step_{op}" not in d:
        pytest.skip("operator not in this fixture")
    wl = fx.workload(d)
    m = anelastic.Model(wl, abi.GA_PREC_F64)
    for k, v in fx.slot_extra(d).items():
        f, slot = fx.FIELD_OF[k]
        m.set(f, slot, v)
    m.op(op, float(d[f"step_{op}"]))
    outs = [k for k in d if k.startswith(op + "__")]
    assert outs
    for k in outs:
        key = k.split("__", 1)[1]
        f, slot = fx.FIELD_OF[key]
        got = m.get(f, slot)
        if op in ICE_EXACT or key == "is_saturated":
            np.testing.assert_array_equal(got, d[k], err_msg=f"{name} {op}:{key}")
        else:
            e = fx.rel_l2(got, d[k])
            assert e <= 1e-12, f"{name} {op}:{key} rel L2 {e:.3e}"


@pytest.mark.parametrize("rf", [1, 2])
def test_ice_cloud_thunderstorm_size_vs_oracle(rf):
    """the ice scheme at the thunderstorm grid (128x128x48, 400 m levels): a
    12 km deep cloud of water, rain, ice and snow, 4 steps, every prognostic
    field, pi and the ice fall speed within 1e-10 of the oracle; then FP32
    against FP64"""
    from model_gb300 import configs
    wl = configs.ice_cloud(nx=128, ny=128, nz=48, dz=400.0, rain_fallout=rf)
    _oracle_compare(wl, 4, 1e-10)
    a = anelastic.Model(wl, abi.GA_PREC_F32)
    b = anelastic.Model(wl, abi.GA_PREC_F64)
    a.step(4)
    b.step(4)
    for f in list(range(7)) + [abi.GA_QS, abi.GA_QI]:
        x = a.get(f)
        assert np.isfinite(x).all(), f
        e = fx.rel_l2(x, b.get(f))
        print("fp32", f, f"{e:.2e}")
        assert e <= 1e-3, (f, e)


@pytest.mark.parametrize("seed", range(16))
def test_random_ice_configuration_vs_oracle(seed):
    """the GPU's FP64 step with the ice scheme against the oracle on the
    seeded configurations of tests/test_oracle_random.py (whose oracle runs
    equal the reference build's bit for bit): every prognostic field in
    every slot, pi, the ice fall speed and the snow intercept within 1e-10"""
    from oracle import oracle as O
    from tests.test_oracle_random import _ice_case
    wl, nsteps = _ice_case(8000 + seed)
    cols = anelastic.build_columns(wl)
    m = anelastic.Model(wl, abi.GA_PREC_F64, columns=cols)
    m.step(nsteps)
    o = O.Oracle(wl, cols)
    assert o.step(nsteps) == 0
    for f in list(range(7)) + [abi.GA_QS, abi.GA_QI]:
        for slot in (abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M):
            e = fx.rel_l2(m.get(f, slot), o.get(f, slot))
            assert e <= 1e-10, (seed, f, slot, e)
    for f in (abi.GA_PI, abi.GA_VTI, abi.GA_VTS, abi.GA_VT, abi.GA_ACCRAIN, abi.GA_ACCSNOW, abi.GA_N0S):
        e = fx.rel_l2(m.get(f), o.get(f))
        assert e <= 1e-10, (seed, f, e)


@pytest.mark.parametrize("case", ["kessler", "ice", "hydrostatic", "linear", "turbulence"])
@pytest.mark.parametrize("prec", [abi.GA_PREC_F32, abi.GA_PREC_F64])
def test_overlapped_step_is_bit_identical(monkeypatch, case, prec):
    """the θ and moisture advection on the second stream beside the pressure
    solve (GA_OVERLAP=1) and the one-stream step (GA_OVERLAP=0) leave every
    slot of every prognostic field bit for bit equal: no field is written by
    both streams, and each kernel's arithmetic is the same"""
    from model_gb300 import configs
    if case == "ice":
        wl = configs.ice_cloud(nx=40, ny=36, nz=32, dz=375.0)
    elif case == "hydrostatic":
        wl = configs.moist_blob(nx=40, ny=36, nz=16, dx=2000.0)
        wl.hydrostatic = 1
    elif case == "linear":
        wl = configs.jet_vortex(nx=40, ny=36, nz=16, dx=20000.0, dz=800.0, dt=30.0, rmax=60000.0, vmax=8.0,
                                moist=True, noise=0.3, extra_basic=1.0)
        wl.linear_model = 1
    else:
        wl = configs.moist_blob(nx=40, ny=36, nz=16)
        if case == "turbulence":
            wl.turbulence_option, wl.use_surface_heat_flux = 1, 1
    ms = []
    for ov in ("1", "0"):
        monkeypatch.setenv("GA_OVERLAP", ov)
        ms.append(anelastic.Model(wl, prec))
    monkeypatch.delenv("GA_OVERLAP")
    for m in ms:
        m.step(5)  # two captured pairs and one eager step
    fields = list(range(7)) + ([abi.GA_QS, abi.GA_QI] if case == "ice" else [])
    for f in fields:
        for slot in (abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M):
            np.testing.assert_array_equal(ms[0].get(f, slot), ms[1].get(f, slot), err_msg=f"{case} {f} {slot}")
    np.testing.assert_array_equal(ms[0].get(abi.GA_PI), ms[1].get(abi.GA_PI))
