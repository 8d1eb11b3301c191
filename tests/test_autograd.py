"""ga_step and ga_adjoint behind torch.autograd.Function (test harness only).

Step.apply(z) runs `nsteps` model steps from the initial state x0 + S z (S:
one scale per field, so that a unit perturbation is physically small) and
returns the final prognostic fields; its backward maps the gradient of the
final fields to the gradient with respect to z through ga_adjoint (state
checkpoints every `every` steps).  The initial state enters the current and
the start-of-step rotation slots alike, so the gradient is the sum of the two
adjoint slots.  torch.autograd.gradcheck (fast mode: random directions on
both sides, central differences in FP64) checks the pair, dry and moist
(Kessler, Eulerian rain fallout), and a scalar loss's .backward() is checked
against central differences along seeded directions.
"""
import numpy as np
import pytest

from model_gb300 import abi, anelastic, configs
from tests.test_adjoint import moist_state, trajectory_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SCALES = {abi.GA_U: 1.0, abi.GA_V: 1.0, abi.GA_W: 0.1, abi.GA_TH: 0.5, abi.GA_QV: 1e-5, abi.GA_QC: 1e-5,
          abi.GA_QR: 1e-5}


@pytest.fixture(scope="module", autouse=True)
def _built():
    from model_gb300 import build
    build.build()


class Trajectory:
    """The map z -> final fields of an FP64 run, and its adjoint."""

    def __init__(self, wl, base: dict, nsteps: int, every: int):
        self.wl, self.base, self.nsteps, self.every = wl, base, nsteps, every
        self.fields = list(range(7 if wl.microphysics_option else 4))
        self.m = anelastic.Model(wl, abi.GA_PREC_F64)
        self.n = wl.points

    def _load(self, z: np.ndarray):
        z = z.reshape(len(self.fields), self.n)
        for (f, s), v in self.base.items():
            x = v
            if s in (abi.GA_SLOT_CUR, abi.GA_SLOT_M) and f in self.fields:
                x = v + SCALES[f] * z[self.fields.index(f)]
            self.m.set(f, s, x)

    def forward(self, z: np.ndarray) -> np.ndarray:
        self._load(z)
        self.m.step(self.nsteps)
        return np.concatenate([self.m.get(f) for f in self.fields])

    def vjp(self, z: np.ndarray, gy: np.ndarray) -> np.ndarray:
        self._load(z)
        gy = gy.reshape(len(self.fields), self.n)
        zero = np.zeros(self.n)
        for f in self.fields:
            for s in (abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M):
                self.m.lin_set(f, s, zero)
        self.m.lin_set(abi.GA_PI, 0, zero)
        for i, f in enumerate(self.fields):
            self.m.lin_set(f, abi.GA_SLOT_CUR, gy[i])
        self.m.adjoint(self.nsteps, self.every)
        return np.concatenate([SCALES[f] * (self.m.lin_get(f, abi.GA_SLOT_CUR) + self.m.lin_get(f, abi.GA_SLOT_M))
                               for f in self.fields])


class Step(torch.autograd.Function):
    @staticmethod
    def forward(ctx, z, traj):
        ctx.traj = traj
        ctx.save_for_backward(z)
        return torch.from_numpy(traj.forward(z.detach().cpu().numpy()))

    @staticmethod
    def backward(ctx, gy):
        (z,) = ctx.saved_tensors
        g = ctx.traj.vjp(z.detach().cpu().numpy(), gy.detach().cpu().numpy().astype(np.float64))
        return torch.from_numpy(g), None


def _case(name):
    if name == "dry":
        wl = configs.jet_vortex(nx=16, ny=14, nz=10, dx=20000.0, dz=800.0, dt=30.0, rmax=60000.0, vmax=8.0,
                                noise=0.3, extra_basic=1.0)
        st = trajectory_state(wl)
    else:
        wl = configs.moist_blob(nx=24, ny=22, nz=16)
        st = moist_state(wl, True)
    nf = 7 if wl.microphysics_option else 4
    return wl, st, nf


@pytest.mark.parametrize("name", ["dry", "moist"])
def test_gradcheck_fast_mode(name):
    wl, st, nf = _case(name)
    traj = Trajectory(wl, st, nsteps=4, every=2)
    z0 = torch.zeros(nf * wl.points, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda z: Step.apply(z, traj), (z0,), eps=1e-6, atol=1e-9, rtol=1e-5,
                                    fast_mode=True)


@pytest.mark.parametrize("name", ["dry", "moist"])
def test_loss_backward_matches_central_differences(name):
    wl, st, nf = _case(name)
    traj = Trajectory(wl, st, nsteps=4, every=2)
    rng = np.random.default_rng(7)
    wout = torch.from_numpy(rng.standard_normal(nf * wl.points))
    z = torch.zeros(nf * wl.points, dtype=torch.float64, requires_grad=True)
    loss = (wout * Step.apply(z, traj)).sum()
    loss.backward()
    g = z.grad.numpy().copy()
    for seed in (1, 2, 3):
        d = np.random.default_rng(100 + seed).standard_normal(nf * wl.points)
        eps = 1e-6
        lp = float((wout.numpy() * traj.forward(eps * d)).sum())
        lm = float((wout.numpy() * traj.forward(-eps * d)).sum())
        fd = (lp - lm) / (2 * eps)
        ad = float(g @ d)
        assert abs(fd - ad) <= 1e-6 * abs(ad), (seed, fd, ad)
