"""The monsoon-vortex sensitivity at full size: the adjoint gradient of the
850 hPa mean relative vorticity after 500 steps with respect to the initial
theta', u' and v', on the 192 x 128 x 32 ITCZ-shear state (dx = dy = 40 km,
dz = 600 m, dt = 120 s), state checkpoints every 50 steps, checked against
central finite differences along 16 seeded random directions in FP64.

The directional derivatives of random directions d (each field scaled by
s_f) spread about zero with standard deviation sigma = (sum_f s_f^2
|dJ/dx_f|^2)^(1/2); the difference between the adjoint's and the central
differences' derivative is bounded by 3e-5 sigma (a direction whose
derivative happens to be near zero is not held to a relative bound).

Every slot of u, v, w and theta gets seeded noise (0.05 standard deviation,
scaled per field), so that no advecting velocity of the trajectory is exactly
zero: there the upwind sign is decided at a kink, and central differences
would average its two one-sided derivatives.
"""
import numpy as np
import pytest

from model_gb300 import abi, anelastic, configs
from tests.test_adjoint import LIN, SCALE, MARGIN, vorticity_cost, vorticity_cost_grad

pytestmark = pytest.mark.gpu

# central differences of 500 FP64 steps: along the first two directions the
# difference to the adjoint was 3.1e-5 and 1.0e-5 of the derivative at
# eps = 1e-4 (truncation), 2.3e-6 and 7.0e-6 at 1e-5, and about 3e-6 at 1e-6
# (the roundoff of the runs); eps = 1e-5 with a bound of 3e-5 sigma
STEPS, EVERY, NDIR, EPS = 500, 50, 16, 1e-5
TOL = 3e-5


@pytest.fixture(scope="module", autouse=True)
def _built():
    from model_gb300 import build
    build.build()


def _level_850(cols):
    p = 100000.0 * np.asarray(cols["pib"]) ** (1004.0 / 287.0)
    return int(np.argmin(np.abs(p[1:-1] - 85000.0))) + 1


def test_c3_vorticity_gradient_16_directions_500_steps():
    wl = configs.monsoon_vortex(nsteps=STEPS)
    assert (wl.nx, wl.ny, wl.nz) == (192, 128, 32)
    cols = anelastic.build_columns(wl)
    k = _level_850(cols)
    rng = np.random.default_rng(1003)
    x0 = {}
    for f in (abi.GA_U, abi.GA_V, abi.GA_W, abi.GA_TH):
        base = np.asarray(wl.fields[abi.PROG_NAMES[f]], dtype=np.float64).ravel()
        x0[f] = base + 0.05 * SCALE[f] * rng.standard_normal(wl.points)

    def model(pert=None, eps=0.0):
        m = anelastic.Model(wl, abi.GA_PREC_F64, columns=cols, init_state=False)
        for b, name in enumerate(abi.BAR_NAMES):
            m.set(abi.GA_UBAR + b, 0, wl.fields[name])
        for f, v in x0.items():
            x = v if pert is None or f not in pert else v + eps * pert[f]
            m.set(f, abi.GA_SLOT_CUR, x)
            m.set(f, abi.GA_SLOT_M, x)
            m.set(f, abi.GA_SLOT_P, np.zeros(wl.points))
        return m

    gu, gv = vorticity_cost_grad(wl, k)
    m = model()
    zero = np.zeros(wl.points)
    for f, s in LIN:
        m.lin_set(f, s, zero)
    m.lin_set(abi.GA_PI, 0, zero)
    m.lin_set(abi.GA_U, abi.GA_SLOT_CUR, gu)
    m.lin_set(abi.GA_V, abi.GA_SLOT_CUR, gv)
    m.adjoint(STEPS, EVERY)
    # the initial state enters both the current and the start-of-step slot
    grad = {f: m.lin_get(f, abi.GA_SLOT_CUR) + m.lin_get(f, abi.GA_SLOT_M) for f in (abi.GA_U, abi.GA_V, abi.GA_TH)}
    m.close()

    def J(d, eps):
        mm = model(d, eps)
        mm.step(STEPS)
        j = vorticity_cost(mm.get(abi.GA_U), mm.get(abi.GA_V), wl, k)
        mm.close()
        return j

    sigma = float(np.sqrt(sum(SCALE[f] ** 2 * float(grad[f] @ grad[f]) for f in grad)))
    drng = np.random.default_rng(16)
    worst = 0.0
    for n in range(NDIR):
        d = {f: SCALE[f] * drng.standard_normal(wl.points) for f in grad}
        fd = (J(d, EPS) - J(d, -EPS)) / (2 * EPS)
        ad = sum(float(grad[f] @ d[f]) for f in d)
        e = abs(fd - ad) / sigma
        worst = max(worst, e)
        print(f"direction {n}: adjoint {ad:.12e} central difference {fd:.12e} "
              f"difference/sigma {e:.2e} difference/derivative {abs(fd - ad) / abs(ad):.2e}")
        assert e <= TOL, (n, fd, ad, sigma)
    print(f"level {k} (850 hPa), margin {MARGIN}, sigma {sigma:.3e}, worst difference/sigma {worst:.2e}")
