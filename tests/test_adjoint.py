"""Tangent-linear model and adjoint of the dry step.

The reference has no linearisation, so its checks are mathematical:
  - the TLM against central finite differences of the forward step;
  - the adjoint against the TLM by the dot-product test <L x, y> = <x, L^T y>
    (to 1e-8 in FP64);
  - the GPU TLM / adjoint (gather form) against the oracle's (scatter form,
    oracle/ga_oracle_lin.c), whose forward step is pinned to the reference;
  - checkpointing changes nothing: the recomputed trajectory is bit-identical;
  - the gradient of the 850 hPa domain-mean vorticity (the monsoon-vortex cost
    function) against finite differences along random directions.
The trajectory carries small noise in every slot so that no upwind sign is
decided at an exact zero (there the flux is a kink and central differences
average the two one-sided derivatives).  The moist cases (Kessler, Eulerian
rain fallout) freeze zero_moisture's clipping and Kessler's branches at the
trajectory; their finite-difference check keeps cloud and rain above zero.
"""
from __future__ import annotations

import numpy as np
import pytest

from model_gb300 import abi, configs
from oracle import oracle as O

LIN = [(f, s) for f in (abi.GA_U, abi.GA_V, abi.GA_W, abi.GA_TH)
       for s in (abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M)]
SCALE = {abi.GA_U: 1.0, abi.GA_V: 1.0, abi.GA_W: 0.1, abi.GA_TH: 0.5}


def small_vortex(**kw):
    """Dry sheared vortex on a general (horizontally varying) basic state."""
    args = dict(nx=16, ny=14, nz=10, dx=20000.0, dz=800.0, dt=30.0, rmax=60000.0, vmax=8.0, noise=0.3,
                extra_basic=1.0)
    args.update(kw)
    return configs.jet_vortex(**args)


def trajectory_state(wl, seed=77):
    """Initial state of every slot: the workload's perturbation plus noise."""
    rng = np.random.default_rng(seed)
    st = {}
    for f, s in LIN:
        base = np.asarray(wl.fields[abi.PROG_NAMES[f]], dtype=np.float64).ravel()
        st[(f, s)] = base * (0.9 if s == abi.GA_SLOT_P else 1.0) + 0.05 * rng.standard_normal(wl.points)
    return st


def random_dirs(wl, seed, with_pi=True):
    rng = np.random.default_rng(seed)
    d = {(f, s): SCALE[f] * rng.standard_normal(wl.points) for f, s in LIN}
    if with_pi:
        d[(abi.GA_PI, 0)] = rng.standard_normal(wl.points)
    return d


def dot(a: dict, b: dict) -> float:
    return float(sum(np.dot(a[k], b[k]) for k in a if k in b))


def rel(a: dict, b: dict) -> float:
    num = sum(np.sum((a[k] - b[k]) ** 2) for k in b)
    den = sum(np.sum(b[k] ** 2) for k in b)
    return float(np.sqrt(num / den))


# ---------------------------------------------------------------------------
# oracle (CPU)
# ---------------------------------------------------------------------------
def _oracle(wl, st, pert=None, eps=0.0):
    o = O.Oracle(wl)
    for (f, s), v in st.items():
        p = v if pert is None else v + eps * pert[(f, s)]
        o.set(f, s, p)
    return o


def _oracle_state(o):
    d = {(f, s): o.get(f, s) for f, s in LIN}
    d[(abi.GA_PI, 0)] = o.get(abi.GA_PI)
    return d


def test_oracle_tlm_matches_finite_differences():
    wl = small_vortex()
    st = trajectory_state(wl)
    dx = random_dirs(wl, 1)
    o = _oracle(wl, st)
    T = O.OracleLin(o)
    T.set_all(dx)
    T.tlm(2)
    dy = T.get_all()
    eps = 1e-4
    op = _oracle(wl, st, dx, eps); op.step(2)
    om = _oracle(wl, st, dx, -eps); om.step(2)
    yp, ym = _oracle_state(op), _oracle_state(om)
    fd = {k: (yp[k] - ym[k]) / (2 * eps) for k in dy}
    assert rel(fd, dy) < 1e-7


def test_oracle_adjoint_dot_product():
    wl = small_vortex()
    st = trajectory_state(wl)
    x, y = random_dirs(wl, 2), random_dirs(wl, 3)
    T = O.OracleLin(_oracle(wl, st))
    T.set_all(x)
    T.tlm(3)
    Lx = T.get_all()
    A = O.OracleLin(_oracle(wl, st))
    A.set_all(y)
    A.adjoint(3)
    LTy = A.get_all()
    lhs, rhs = dot(Lx, y), dot(x, LTy)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    assert np.all(LTy[(abi.GA_PI, 0)] == 0)  # the step never reads pi


def test_oracle_lin_is_dry_nonperiodic_only():
    o = O.Oracle(configs.moist_blob(nx=14, ny=13, nz=10))
    with pytest.raises(RuntimeError):
        O.OracleLin(o)


# ---------------------------------------------------------------------------
# cost function of the monsoon-vortex case: mean relative vorticity at the
# level nearest 850 hPa, zeta = dv/dx - du/dy at cell corners, over the
# corners inside the lateral boundary zone (MARGIN points).  Over the whole
# domain the mean telescopes to the outermost ring, which no step changes.
# ---------------------------------------------------------------------------
MARGIN = 4
def level_850(wl, cols=None) -> int:
    cols = cols if cols is not None else O.build_columns(wl)
    p = 100000.0 * np.asarray(cols["pib"]) ** (1004.0 / 287.0)
    k = int(np.argmin(np.abs(p[1:-1] - 85000.0))) + 1
    return k


def vorticity_cost(u, v, wl, k):
    U = u.reshape(wl.nx, wl.ny, wl.nz)[:, :, k]
    V = v.reshape(wl.nx, wl.ny, wl.nz)[:, :, k]
    a, bx, by = MARGIN, wl.nx - MARGIN, wl.ny - MARGIN
    z = (V[a:bx, a:by] - V[a - 1:bx - 1, a:by]) / wl.dx - (U[a:bx, a:by] - U[a:bx, a - 1:by - 1]) / wl.dy
    return float(z.mean())


def vorticity_cost_grad(wl, k):
    """(dJ/du, dJ/dv) of vorticity_cost (it is linear)."""
    a, bx, by = MARGIN, wl.nx - MARGIN, wl.ny - MARGIN
    n = (bx - a) * (by - a)
    gu = np.zeros((wl.nx, wl.ny, wl.nz))
    gv = np.zeros((wl.nx, wl.ny, wl.nz))
    gv[a:bx, a:by, k] += 1.0 / (wl.dx * n)
    gv[a - 1:bx - 1, a:by, k] -= 1.0 / (wl.dx * n)
    gu[a:bx, a:by, k] -= 1.0 / (wl.dy * n)
    gu[a:bx, a - 1:by - 1, k] += 1.0 / (wl.dy * n)
    return gu.ravel(), gv.ravel()


def test_vorticity_cost_gradient_is_exact():
    wl = small_vortex()
    k = level_850(wl)
    rng = np.random.default_rng(5)
    u, v = rng.standard_normal(wl.points), rng.standard_normal(wl.points)
    gu, gv = vorticity_cost_grad(wl, k)
    assert abs(vorticity_cost(u, v, wl, k) - (gu @ u + gv @ v)) < 1e-15


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _model(wl, st, prec=abi.GA_PREC_F64, pert=None, eps=0.0):
    from model_gb300 import anelastic
    m = anelastic.Model(wl, prec)
    for (f, s), v in st.items():
        m.set(f, s, v if pert is None else v + eps * pert[(f, s)])
    return m


def _model_state(m):
    d = {(f, s): m.get(f, s) for f, s in LIN}
    d[(abi.GA_PI, 0)] = m.get(abi.GA_PI)
    return d


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()


@pytest.mark.gpu
def test_gpu_tlm_matches_oracle(built):
    wl = small_vortex()
    st = trajectory_state(wl)
    dx = random_dirs(wl, 11)
    T = O.OracleLin(_oracle(wl, st))
    T.set_all(dx)
    T.tlm(3)
    ref = T.get_all()
    m = _model(wl, st)
    m.lin_set_all(dx)
    m.tlm_step(3)
    got = m.lin_get_all()
    for k in ref:
        a, b = got[k], ref[k]
        nb = np.linalg.norm(b)
        assert np.linalg.norm(a - b) <= 1e-10 * max(nb, 1e-300), k
    # the state advanced exactly as by ga_step
    m2 = _model(wl, st)
    m2.step(3)
    for f, s in LIN:
        assert np.array_equal(m.get(f, s), m2.get(f, s))


@pytest.mark.gpu
def test_gpu_adjoint_matches_oracle(built):
    wl = small_vortex()
    st = trajectory_state(wl)
    y = random_dirs(wl, 12)
    A = O.OracleLin(_oracle(wl, st))
    A.set_all(y)
    A.adjoint(3)
    ref = A.get_all()
    m = _model(wl, st)
    m.lin_set_all(y)
    m.adjoint(3, 2)
    got = m.lin_get_all()
    for k in LIN:
        a, b = got[k], ref[k]
        assert np.linalg.norm(a - b) <= 1e-10 * max(np.linalg.norm(b), 1e-300), k
    assert np.all(got[(abi.GA_PI, 0)] == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(abi.GA_PREC_F64, 1e-8), (abi.GA_PREC_F32, 1e-4)])
def test_gpu_dot_product(built, prec, tol):
    wl = small_vortex(nx=24, ny=20, nz=12)
    st = trajectory_state(wl)
    x, y = random_dirs(wl, 21), random_dirs(wl, 22)
    m = _model(wl, st, prec)
    m.lin_set_all(x)
    m.tlm_step(5)
    Lx = m.lin_get_all()
    m = _model(wl, st, prec)
    m.lin_set_all(y)
    m.adjoint(5, 2)
    LTy = m.lin_get_all()
    lhs, rhs = dot(Lx, y), dot(x, LTy)
    assert abs(lhs - rhs) <= tol * abs(lhs), (lhs, rhs)


@pytest.mark.gpu
def test_gpu_checkpointing_is_exact(built, monkeypatch):
    """any checkpoint interval, with every segment recomputed but the last
    (GA_ADJ_RESIDENT=1) or as many kept on the tape as memory allows (all of
    them on this grid), gives the same adjoint bit for bit"""
    wl = small_vortex()
    st = trajectory_state(wl)
    y = random_dirs(wl, 31)
    outs = []
    for K, res in ((1, "1"), (2, "1"), (5, "1"), (0, "1"), (2, None), (2, "2")):
        if res is None:
            monkeypatch.delenv("GA_ADJ_RESIDENT", raising=False)
        else:
            monkeypatch.setenv("GA_ADJ_RESIDENT", res)
        m = _model(wl, st)
        m.lin_set_all(y)
        m.adjoint(5, K)
        outs.append(m.lin_get_all())
        assert m.counters()[0] == 5
    monkeypatch.delenv("GA_ADJ_RESIDENT", raising=False)
    for o in outs[1:]:
        for k in LIN:
            assert np.array_equal(o[k], outs[0][k]), k


@pytest.mark.gpu
def test_gpu_tlm_matches_finite_differences(built):
    wl = small_vortex(nx=20, ny=18, nz=12)
    st = trajectory_state(wl)
    dx = random_dirs(wl, 41, with_pi=False)
    m = _model(wl, st)
    m.lin_set_all(dx)
    m.tlm_step(4)
    dy = m.lin_get_all()
    eps = 1e-4
    mp = _model(wl, st, pert=dx, eps=eps); mp.step(4)
    mm = _model(wl, st, pert=dx, eps=-eps); mm.step(4)
    yp, ym = _model_state(mp), _model_state(mm)
    fd = {k: (yp[k] - ym[k]) / (2 * eps) for k in dy}
    assert rel(fd, dy) < 1e-6


@pytest.mark.gpu
def test_gpu_vorticity_gradient_matches_finite_differences(built):
    """dJ/d(theta', u', v')_0 of the 850 hPa mean vorticity by the adjoint,
    checked by central differences along seeded directions."""
    wl = small_vortex(nx=24, ny=20, nz=12, dt=60.0)
    nsteps, K = 6, 3
    k = level_850(wl)
    st = trajectory_state(wl)
    # the initial state convention: current = M = x0, P = 0
    for f in (abi.GA_U, abi.GA_V, abi.GA_W, abi.GA_TH):
        st[(f, abi.GA_SLOT_M)] = st[(f, abi.GA_SLOT_CUR)]
        st[(f, abi.GA_SLOT_P)] = np.zeros(wl.points)
    gu, gv = vorticity_cost_grad(wl, k)
    m = _model(wl, st)
    zero = np.zeros(wl.points)
    for f, s in LIN:
        m.lin_set(f, s, zero)
    m.lin_set(abi.GA_PI, 0, zero)
    m.lin_set(abi.GA_U, abi.GA_SLOT_CUR, gu)
    m.lin_set(abi.GA_V, abi.GA_SLOT_CUR, gv)
    m.adjoint(nsteps, K)
    grad = {f: m.lin_get(f, abi.GA_SLOT_CUR) + m.lin_get(f, abi.GA_SLOT_M)
            for f in (abi.GA_U, abi.GA_V, abi.GA_TH)}

    def J(d, eps):
        s2 = dict(st)
        for f, v in d.items():
            s2[(f, abi.GA_SLOT_CUR)] = st[(f, abi.GA_SLOT_CUR)] + eps * v
            s2[(f, abi.GA_SLOT_M)] = s2[(f, abi.GA_SLOT_CUR)]
        mm = _model(wl, s2)
        mm.step(nsteps)
        return vorticity_cost(mm.get(abi.GA_U), mm.get(abi.GA_V), wl, k)

    rng = np.random.default_rng(51)
    for _ in range(3):
        d = {f: SCALE[f] * rng.standard_normal(wl.points) for f in grad}
        eps = 1e-4
        fd = (J(d, eps) - J(d, -eps)) / (2 * eps)
        ad = sum(float(grad[f] @ d[f]) for f in d)
        assert abs(fd - ad) <= 1e-5 * abs(ad), (fd, ad)


@pytest.mark.gpu
def test_gpu_adjoint_rejects_explicit_diffusion(built):
    from model_gb300 import anelastic
    wl = configs.moist_blob(nx=20, ny=18, nz=12)
    wl.use_explicit_diffusion, wl.diffusion_order = 1, 4
    m = anelastic.Model(wl, abi.GA_PREC_F64)
    with pytest.raises(anelastic.GaError):
        m.lin_set(abi.GA_U, abi.GA_SLOT_CUR, np.zeros(wl.points))
    assert "diffusion" in anelastic.last_error()


@pytest.mark.gpu
def test_gpu_adjoint_rejects_turbulence(built):
    from model_gb300 import anelastic
    wl = configs.moist_blob(nx=20, ny=18, nz=12)
    wl.turbulence_option = 1
    m = anelastic.Model(wl, abi.GA_PREC_F64)
    with pytest.raises(anelastic.GaError):
        m.adjoint(1, 1)
    assert "turbulence" in anelastic.last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [dict(rain_fallout=2), dict(periodic=1)])
def test_gpu_adjoint_rejects_unsupported(built, kw):
    """Semi-Lagrangian rain fallout and periodic boundaries are not linearised."""
    from model_gb300 import anelastic
    m = anelastic.Model(configs.moist_blob(nx=18, ny=13, nz=10, **kw), abi.GA_PREC_F64)
    with pytest.raises(anelastic.GaError):
        m.tlm_step(1)
    with pytest.raises(anelastic.GaError):
        m.adjoint(1, 1)


# ---------------------------------------------------------------------------
# moist (Kessler, Eulerian rain fallout): the clipping of zero_moisture and
# the branches of Kessler are frozen at the trajectory
# ---------------------------------------------------------------------------
MOIST = [(f, s) for f in range(7) for s in (abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M)]
MSCALE = {0: 1.0, 1: 1.0, 2: 0.1, 3: 0.5, 4: 1e-5, 5: 1e-5, 6: 1e-5}


def moist_state(wl, positive, seed=77):
    """Every slot: the workload's state plus noise; positive: cloud and rain
    above zero everywhere, so that no clipping decision sits at a kink."""
    rng = np.random.default_rng(seed)
    st = {}
    for f, s in MOIST:
        v = np.asarray(wl.fields[abi.PROG_NAMES[f]], dtype=np.float64).ravel() * (0.9 if s == abi.GA_SLOT_P else 1.0)
        if f < 4:
            v = v + 0.05 * rng.standard_normal(wl.points)
        elif positive:
            v = np.abs(v) + 4e-4 * (1.0 + 0.2 * rng.standard_normal(wl.points))
        st[(f, s)] = v
    return st


def moist_dirs(wl, seed, with_pi=True):
    rng = np.random.default_rng(seed)
    d = {(f, s): MSCALE[f] * rng.standard_normal(wl.points) for f, s in MOIST}
    if with_pi:
        d[(abi.GA_PI, 0)] = rng.standard_normal(wl.points)
    return d


def _moist_model_state(m):
    d = {(f, s): m.get(f, s) for f, s in MOIST}
    d[(abi.GA_PI, 0)] = m.get(abi.GA_PI)
    return d


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(abi.GA_PREC_F64, 1e-8), (abi.GA_PREC_F32, 1e-4)])
@pytest.mark.parametrize("positive", [False, True])
def test_gpu_moist_dot_product(built, prec, tol, positive):
    wl = configs.moist_blob(nx=24, ny=22, nz=16)
    st = moist_state(wl, positive)
    x, y = moist_dirs(wl, 21), moist_dirs(wl, 22)
    m = _model(wl, st, prec)
    m.lin_set_all(x)
    m.tlm_step(4)
    Lx = m.lin_get_all()
    m = _model(wl, st, prec)
    m.lin_set_all(y)
    m.adjoint(4, 2)
    LTy = m.lin_get_all()
    lhs, rhs = dot(Lx, y), dot(x, LTy)
    assert abs(lhs - rhs) <= tol * abs(lhs), (lhs, rhs)


@pytest.mark.gpu
def test_gpu_moist_tlm_matches_finite_differences(built):
    wl = configs.moist_blob(nx=24, ny=22, nz=16)
    st = moist_state(wl, True)
    dx = moist_dirs(wl, 41, with_pi=False)
    m = _model(wl, st)
    m.lin_set_all(dx)
    m.tlm_step(3)
    dy = m.lin_get_all()
    eps = 1e-5
    mp = _model(wl, st, pert=dx, eps=eps); mp.step(3)
    mm = _model(wl, st, pert=dx, eps=-eps); mm.step(3)
    yp, ym = _moist_model_state(mp), _moist_model_state(mm)
    fd = {k: (yp[k] - ym[k]) / (2 * eps) for k in dy}
    assert rel(fd, dy) < 1e-6


@pytest.mark.gpu
def test_gpu_moist_checkpointing_is_exact(built, monkeypatch):
    wl = configs.moist_blob(nx=24, ny=22, nz=16)
    st = moist_state(wl, False)
    y = moist_dirs(wl, 31)
    outs = []
    for K, res in ((1, "1"), (2, "1"), (0, "1"), (1, None), (1, "3")):
        if res is None:
            monkeypatch.delenv("GA_ADJ_RESIDENT", raising=False)
        else:
            monkeypatch.setenv("GA_ADJ_RESIDENT", res)
        m = _model(wl, st)
        m.lin_set_all(y)
        m.adjoint(4, K)
        outs.append(m.lin_get_all())
        assert m.counters()[0] == 4
    monkeypatch.delenv("GA_ADJ_RESIDENT", raising=False)
    for o in outs[1:]:
        for k in MOIST:
            assert np.array_equal(o[k], outs[0][k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["dry_varying_base", "dry_uniform_base", "moist"])
def test_gpu_adjoint_quad_kernel_matches_level_kernel(built, monkeypatch, case):
    """FP32: the four-level adjoint advection and, for a basic state of height
    only, the four-level coefficient pass (the defaults when NZ % 4 == 0)
    against the per-level kernels (GA_ADJ=level), bit for bit.  The grids are
    ragged against the 16 x 8 x 8 tiles; NZ = 12 leaves a half level tile."""
    if case == "moist":
        wl = configs.moist_blob(nx=24, ny=22, nz=16)
        st, y = moist_state(wl, False), moist_dirs(wl, 31)
    else:
        wl = small_vortex(nx=24, ny=20, nz=12, extra_basic=1.0 if case == "dry_varying_base" else 0.0)
        st, y = trajectory_state(wl), random_dirs(wl, 22)
    outs = []
    for mode in ("level", "quad"):
        monkeypatch.setenv("GA_ADJ", mode)
        m = _model(wl, st, abi.GA_PREC_F32)
        m.lin_set_all(y)
        m.adjoint(4, 2)
        outs.append(m.lin_get_all())
    monkeypatch.delenv("GA_ADJ")
    for k in outs[0]:
        np.testing.assert_array_equal(outs[1][k], outs[0][k], err_msg=str(k))



@pytest.mark.gpu
def test_gpu_adjoint_after_1024_thread_forward_x_solve(built, monkeypatch):
    """a context whose fused forward x solve runs 1024-thread blocks
    (GA_SPECTRAL_X=1024, an autotuner candidate) runs its adjoint x solve in
    blocks the adjoint kernel's registers allow, with the same gradient bit
    for bit"""
    wl = small_vortex(nx=24, ny=20, nz=12)
    st, y = trajectory_state(wl), random_dirs(wl, 22)
    outs = []
    for mode in ("single", "1024"):
        monkeypatch.setenv("GA_SPECTRAL_X", mode)
        m = _model(wl, st, abi.GA_PREC_F32)
        m.lin_set_all(y)
        m.adjoint(4, 2)
        outs.append(m.lin_get_all())
    monkeypatch.delenv("GA_SPECTRAL_X")
    for k in outs[0]:
        np.testing.assert_array_equal(outs[1][k], outs[0][k], err_msg=str(k))
