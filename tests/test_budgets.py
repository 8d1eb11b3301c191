"""FP64 domain budgets on the GPU (ga_budget) and the conservation laws they
check.

  - the budgets of an FP64 run against the same sums of the CPU oracle's
    state (1e-12 relative);
  - an FP32 context's budgets against FP64 sums of its own fields: the
    accumulation is FP64 (1e-13 relative; an FP32 accumulation would miss by
    about 1e-7);
  - flux-form conservation (advection.cpp:349-498 with the face fluxes of
    fluxes.cpp:582-784): with every perturbation confined away from the
    lateral boundaries and w' = 0, one advection operator leaves the
    rho-weighted integrals of theta', qv, qc and qr unchanged; with w' != 0
    those of qc and qr (no base-state term);
  - Kessler conserves the total water of every point (kessler.cpp:25-213).
Conservation is checked to 1e-13 of the integral of rho |s| dV.
"""
import numpy as np
import pytest

from model_gb300 import abi, anelastic, configs

pytestmark = pytest.mark.gpu

NAMES = abi.BUDGET_NAMES


@pytest.fixture(scope="module", autouse=True)
def _built():
    from model_gb300 import build
    build.build()


def _weights(wl, cols):
    return np.asarray(cols["rhou"]) * wl.dx * wl.dy * wl.dz / np.asarray(cols["mu"])


def _np_budget(wl, cols, fields, accrain=None, accsnow=None):
    """The same sums in numpy (FP64)."""
    wk = _weights(wl, cols)
    sl = (slice(1, wl.nx - 1), slice(1, wl.ny - 1), slice(1, wl.nz - 1))
    g = lambda a: np.asarray(a, dtype=np.float64).reshape(wl.nx, wl.ny, wl.nz)[sl]  # noqa: E731
    w = wk[1:-1][None, None, :]
    out = {"theta": float(np.sum(w * g(fields["th"])))}
    for q in ("qv", "qc", "qr", "qi", "qs"):
        out[q] = float(np.sum(w * g(fields[q]))) if q in fields else 0.0
    out["water"] = out["qv"] + out["qc"] + out["qr"] + out["qi"] + out["qs"]
    out["ke"] = float(np.sum(w * 0.5 * (g(fields["u"]) ** 2 + g(fields["v"]) ** 2 + g(fields["w"]) ** 2)))
    out["rain"] = 0.0 if accrain is None else float(
        np.sum(np.asarray(accrain).reshape(wl.nx, wl.ny)[1:-1, 1:-1]) * wl.dx * wl.dy)
    out["mass"] = float(np.sum(w * np.ones_like(g(fields["th"]))))
    out["snow"] = 0.0 if accsnow is None else float(
        np.sum(np.asarray(accsnow).reshape(wl.nx, wl.ny)[1:-1, 1:-1]) * wl.dx * wl.dy)
    return out


def _close(a, b, tol, what):
    for k in NAMES:
        scale = max(abs(b[k]), 1e-300)
        assert abs(a[k] - b[k]) <= tol * scale or (b[k] == 0 and abs(a[k]) < 1e-300), \
            f"{what}: {k} {a[k]!r} vs {b[k]!r}"


def test_fp64_budgets_match_oracle_state():
    from oracle import oracle as O
    wl = configs.moist_blob(nx=30, ny=26, nz=16, nsteps=4)
    cols = anelastic.build_columns(wl)
    m = anelastic.Model(wl, abi.GA_PREC_F64, columns=cols)
    m.step(wl.nsteps)
    got = m.budget(abi.GA_SLOT_CUR)
    o = O.Oracle(wl, cols)
    assert o.step(wl.nsteps) == 0
    fields = {n: o.get(f) for f, n in enumerate(abi.PROG_NAMES)}
    ref = _np_budget(wl, cols, fields, o.get(abi.GA_ACCRAIN))
    _close(got, ref, 1e-12, "fp64 vs oracle")
    assert got["rain"] > 0 and got["qr"] > 0


@pytest.mark.parametrize("prec", [abi.GA_PREC_F64, abi.GA_PREC_F32])
def test_ice_budgets_match_state(prec):
    """the ice scheme's budgets: cloud ice, snow, accumulated snow, and the
    total water with them, against numpy sums of the oracle's state (FP64)
    or of the context's own fields (FP32, accumulated in FP64); a caller
    passing the first 8 entries gets them"""
    import ctypes as C
    from oracle import oracle as O
    wl = configs.ice_cloud(nx=30, ny=26, nz=16, dz=750.0, nsteps=4)
    cols = anelastic.build_columns(wl)
    m = anelastic.Model(wl, prec, columns=cols)
    m.step(wl.nsteps)
    got = m.budget(abi.GA_SLOT_CUR)
    names = list(abi.PROG_NAMES) + ["qs", "qi"]
    fids = list(range(7)) + [abi.GA_QS, abi.GA_QI]
    if prec == abi.GA_PREC_F64:
        o = O.Oracle(wl, cols)
        assert o.step(wl.nsteps) == 0
        fields = {n: o.get(f) for f, n in zip(fids, names)}
        ref = _np_budget(wl, cols, fields, o.get(abi.GA_ACCRAIN), o.get(abi.GA_ACCSNOW))
        _close(got, ref, 1e-12, "ice fp64 vs oracle")
    else:
        fields = {n: m.get(f) for f, n in zip(fids, names)}
        ref = _np_budget(wl, cols, fields, m.get(abi.GA_ACCRAIN), m.get(abi.GA_ACCSNOW))
        _close(got, ref, 1e-13, "ice fp32")
    assert got["qi"] > 0 and got["qs"] > 0 and got["snow"] > 0
    assert got["water"] == got["qv"] + got["qc"] + got["qr"] + got["qi"] + got["qs"]
    short = (C.c_double * 8)()
    assert m.L.ga_budget(m.h, abi.GA_SLOT_CUR, short, 8) == 0
    assert list(short) == [got[n] for n in abi.BUDGET_NAMES[:8]]


def test_fp32_budgets_accumulate_in_fp64():
    wl = configs.thunderstorm(nx=44, ny=38, nsteps=3)
    cols = anelastic.build_columns(wl)
    m = anelastic.Model(wl, abi.GA_PREC_F32, columns=cols)
    m.step(wl.nsteps)
    for slot in (abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M):
        got = m.budget(slot)
        fields = {n: m.get(f, slot) for f, n in enumerate(abi.PROG_NAMES)}
        ref = _np_budget(wl, cols, fields, m.get(abi.GA_ACCRAIN))
        _close(got, ref, 1e-13, f"fp32 slot {slot}")
    # the same bits on a repeated call
    assert m.budget(abi.GA_SLOT_CUR) == m.budget(abi.GA_SLOT_CUR)


def _compact_state(wl, seed, w_on):
    """perturbations that vanish within 6 points of the lateral boundaries and
    below level 3 and above NZ-4; positive moisture"""
    n3 = (wl.nx, wl.ny, wl.nz)
    rng = np.random.default_rng(seed)
    mask = np.zeros(n3)
    mask[8:wl.nx - 8, 8:wl.ny - 8, 3:wl.nz - 4] = 1.0
    st = {}
    for f, name in enumerate(abi.PROG_NAMES):
        scale = {"u": 3.0, "v": 3.0, "w": 0.5 if w_on else 0.0, "th": 1.0,
                 "qv": 1e-3, "qc": 1e-3, "qr": 1e-3}[name]
        x = rng.random(n3) if name in ("qc", "qr") else rng.standard_normal(n3)
        st[name] = (scale * x * mask).ravel()
    return st


@pytest.mark.parametrize("prec", [abi.GA_PREC_F64, abi.GA_PREC_F32])
@pytest.mark.parametrize("w_on", [False, True])
def test_advection_conserves_rho_weighted_integrals(prec, w_on):
    wl = configs.moist_blob(nx=40, ny=36, nz=20)
    cols = anelastic.build_columns(wl)
    m = anelastic.Model(wl, prec, columns=cols, init_state=False)
    for b, name in enumerate(abi.BAR_NAMES):
        m.set(abi.GA_UBAR + b, 0, wl.fields[name])
    cur, start = _compact_state(wl, 21, w_on), _compact_state(wl, 22, w_on)
    for f, name in enumerate(abi.PROG_NAMES):
        m.set(f, abi.GA_SLOT_CUR, cur[name])
        m.set(f, abi.GA_SLOT_M, start[name])
        m.set(f, abi.GA_SLOT_P, start[name])  # cells the operator does not write keep M
    before = m.budget(abi.GA_SLOT_M)
    m.op("advect_theta", 0.5)
    m.op("advect_micro", 0.5)
    after = m.budget(abi.GA_SLOT_P)
    wk = _weights(wl, cols)
    conserved = ("theta", "qv", "qc", "qr") if not w_on else ("qc", "qr")
    tol = 1e-13 if prec == abi.GA_PREC_F64 else 1e-6
    field_of = {"theta": "th", "qv": "qv", "qc": "qc", "qr": "qr"}
    for name in conserved:
        s = np.abs(np.asarray(start[field_of[name]]).reshape(wl.nx, wl.ny, wl.nz))
        norm = float(np.sum(wk[None, None, :] * s))
        assert abs(after[name] - before[name]) <= tol * norm, (name, after[name], before[name], norm)
    # the advection did change the fields
    assert not np.array_equal(m.get(abi.GA_QC, abi.GA_SLOT_P), np.asarray(start["qc"]))


def test_kessler_conserves_total_water():
    wl = configs.moist_blob(nx=30, ny=26, nz=16, nsteps=1)
    m = anelastic.Model(wl, abi.GA_PREC_F64)
    m.step(1)
    # Kessler acts on the forecast slot: copy the current state there
    for f in range(7):
        m.set(f, abi.GA_SLOT_P, m.get(f, abi.GA_SLOT_CUR))
    before = m.budget(abi.GA_SLOT_P)
    th_before = m.get(abi.GA_TH, abi.GA_SLOT_P)
    m.op("kessler", 1.0)
    after = m.budget(abi.GA_SLOT_P)
    assert abs(after["water"] - before["water"]) <= 1e-13 * abs(before["water"]) + 1e-300
    assert not np.array_equal(th_before, m.get(abi.GA_TH, abi.GA_SLOT_P))  # latent heating happened
