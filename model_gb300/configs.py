"""Seeded synthetic initial states for the benchmark and test workloads.

The reference initialises from NetCDF files written by its Python tools
(initialize.py:52-111, sample_initializations.py:371-492); no such file ships
with it and NetCDF is not available here, so these generators build the same
kinds of state in memory: a horizontally uniform basic state from an analytic
sounding (theta, humidity, wind profiles), and a perturbation (warm bubble,
line thermal, vortex) plus seeded uniform noise.  Values are produced once on
the host and fed bit-identically to the CPU oracle and to the GPU.

Random numbers come from splitmix64 (integer arithmetic, so identical on every
platform), seeded with 1000 + workload id (+ 7919 * member for ensembles).

Layout of every 3-D array: [i][j][k], k fastest (reference INDEX, model.h:50).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# physical constants of the reference (include/model.h:248-259)
RD = 287.0
CP = 1004.0
P0 = 100000.0
GRAV = 9.8
PRESSFC = 100200.0

# theta anomalies (K) of the monsoon vortex, in the ratio of the reference's
# example call (2.5, -2.05; data_initializer.cpp:809), scaled once (by 1.55105)
# so that the maximum wind of the 192 x 128 x 32 state is 5.0 m/s, found 520 km
# from the centre at 3.9 km
VORTEX_TMAX = 3.8776
VORTEX_TMIN = -3.1796

_SM_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_SM_M1 = np.uint64(0xBF58476D1CE4E5B9)
_SM_M2 = np.uint64(0x94D049BB133111EB)


def splitmix_uniform(seed: int, n: int) -> np.ndarray:
    """n doubles uniform in [0, 1) from the splitmix64 stream of `seed`."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + idx * _SM_GAMMA
        z = (z ^ (z >> np.uint64(30))) * _SM_M1
        z = (z ^ (z >> np.uint64(27))) * _SM_M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclasses.dataclass
class Workload:
    """One initial state plus the runtime settings the step reads."""

    name: str
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    dt: float
    nsteps: int
    microphysics_option: int = 0
    rain_fallout: int = 1
    periodic_ew_boundaries: int = 0
    boundary_width_north: int = 5
    boundary_width_south: int = 5
    boundary_width_east: int = 5
    boundary_width_west: int = 5
    rayleigh_damping_z: int = -1  # default NZ - 5
    height_lowest_level: float = -1.0  # default dz (uniform grid)
    corner_lat: float = 120.0
    # explicit diffusion (apply_explicit_diffusion, damping.cpp:1125); off by default
    use_explicit_diffusion: int = 0
    diffusion_order: int = 4
    kdiffh: float = 0.005
    kdiffv: float = 0.005
    # turbulence (calculate_diff_tend, turbulence.cpp:158); off by default
    turbulence_option: int = 0
    use_surface_heat_flux: int = 0
    water_temp: float = 28.0
    # the linearised model (linear_integrate_rk3, driver_serial.cpp:83); off by default
    linear_model: int = 0
    # the hydrostatic equation set (integrate_hydro, solver.cpp:33); off by default
    hydrostatic: int = 0
    fields: dict = dataclasses.field(default_factory=dict)

    def __post_init__(self):
        if self.rayleigh_damping_z < 0:
            self.rayleigh_damping_z = self.nz - 5
        if self.height_lowest_level < 0:
            self.height_lowest_level = self.dz

    @property
    def points(self) -> int:
        return self.nx * self.ny * self.nz

    def settings(self) -> dict:
        keys = ("nx", "ny", "nz", "dx", "dy", "dz", "dt", "microphysics_option", "rain_fallout",
                "periodic_ew_boundaries", "boundary_width_north", "boundary_width_south",
                "boundary_width_east", "boundary_width_west", "rayleigh_damping_z",
                "height_lowest_level", "corner_lat", "use_explicit_diffusion", "diffusion_order", "kdiffh",
                "kdiffv", "turbulence_option", "use_surface_heat_flux", "water_temp", "linear_model", "hydrostatic")
        return {k: getattr(self, k) for k in keys}


# ---------------------------------------------------------------------------
# soundings
# ---------------------------------------------------------------------------
def _levels(nz: int, dz: float) -> np.ndarray:
    """Heights of the scalar levels of the uniform grid: zu[k] = (k-0.5) dz
    (initializer.cpp:843)."""
    return (np.arange(nz, dtype=np.float64) - 0.5) * dz


def _exner_profile(theta_v: np.ndarray, zu: np.ndarray) -> np.ndarray:
    """Hydrostatic Exner function on the scalar levels, integrated upward
    from the surface value (same recurrence as initializer.cpp:887-893)."""
    nz = zu.size
    pib = np.zeros(nz)
    pisfc = (PRESSFC / P0) ** (RD / CP)
    pib[1] = pisfc - GRAV * zu[1] / (CP * theta_v[1])
    pib[0] = pisfc + GRAV * (0 - zu[0]) / (CP * theta_v[0])
    for k in range(2, nz):
        pib[k] = pib[k - 1] - GRAV * (zu[k] - zu[k - 1]) / (CP * 0.5 * (theta_v[k] + theta_v[k - 1]))
    return pib


def _qvsat(temperature, pressure):
    esl = 611.2 * np.exp(17.67 * (temperature - 273.15) / (temperature - 29.65))
    return 0.62197 * esl / (pressure - esl)


def thunderstorm_sounding(nz: int, dz: float, u_top: float = 15.0, shear_depth: float = 6000.0):
    """Weisman-Klemp style sounding: theta 300 K at the surface rising as
    (z/12 km)^1.25 to 343 K at a 12 km tropopause, isothermal (213 K) above
    (shape of sample_initializations.py:422-427); relative humidity 0.95 at
    the surface falling linearly to 0.25 at 12 km, vapour capped at 14 g/kg;
    u rising linearly from 0 to u_top over shear_depth, constant above."""
    zu = _levels(nz, dz)
    z = np.maximum(zu, 0.0)
    ztr, ttr, tsurf, temptr = 12000.0, 343.0, 300.0, 213.0
    theta = np.where(z < ztr, tsurf + (ttr - tsurf) * (z / ztr) ** 1.25,
                     ttr * np.exp(GRAV * (z - ztr) / (CP * temptr)))
    rh = np.where(z < ztr, 0.95 - (0.95 - 0.25) * z / ztr, 0.25)
    qv = np.zeros(nz)
    for _ in range(4):  # fixed point: Exner depends on theta_v
        pib = _exner_profile(theta * (1.0 + 0.61 * qv), zu)
        temp = theta * pib
        pres = P0 * pib ** (CP / RD)
        qv = np.minimum(rh * _qvsat(temp, pres), 0.014)
    ubar = u_top * np.minimum(z / shear_depth, 1.0)
    return theta, qv, ubar


def stable_sounding(nz: int, dz: float, theta0: float = 300.0, bv: float = 0.01):
    """Constant Brunt-Vaisala frequency: theta = theta0 exp(N^2 z / g)."""
    z = np.maximum(_levels(nz, dz), 0.0)
    return theta0 * np.exp(bv * bv * z / GRAV)


def _grid_xyz(nx, ny, nz, dx, dy, dz):
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dy
    z = _levels(nz, dz)
    return x, y, z


def _basic_state(wl: Workload, theta_col, qv_col, u_col):
    n3 = (wl.nx, wl.ny, wl.nz)
    f = wl.fields
    f["tb_in"] = np.array(theta_col, dtype=np.float64)
    f["qb_in"] = np.array(qv_col, dtype=np.float64)
    f["ubar"] = np.broadcast_to(u_col, n3).copy()
    f["vbar"] = np.zeros(n3)
    f["wbar"] = np.zeros(n3)
    f["thbar"] = np.zeros(n3)
    f["qbar"] = np.zeros(n3)
    # basic-state Exner pressure, full value (PBAR, model.h:91): the 1-D
    # profile of the column builder broadcast horizontally
    tb = np.array(theta_col, dtype=np.float64)
    qb = np.array(qv_col, dtype=np.float64)
    tb[0], tb[-1], qb[0], qb[-1] = tb[1], tb[-2], qb[1], qb[-2]
    pib = _exner_profile(tb * (1.0 + 0.61 * qb), _levels(wl.nz, wl.dz))
    pib[0], pib[-1] = pib[1], pib[-2]
    f["pbar"] = np.broadcast_to(pib, n3).copy()


def _zero_perturbation(wl: Workload):
    n3 = (wl.nx, wl.ny, wl.nz)
    for k in ("u", "v", "w", "th", "qv", "qc", "qr") + (("qs", "qi") if wl.microphysics_option == 2 else ()):
        wl.fields[k] = np.zeros(n3)


def _add_noise(wl: Workload, seed: int, amp: float):
    """U(-amp, amp) on theta' at every interior level k = 1..NZ-2."""
    r = splitmix_uniform(seed, wl.points).reshape(wl.nx, wl.ny, wl.nz)
    noise = amp * (2.0 * r - 1.0)
    noise[:, :, 0] = 0.0
    noise[:, :, -1] = 0.0
    wl.fields["th"] += noise


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def dry_bubble(nx=64, ny=64, nz=40, dx=500.0, dz=250.0, dt=2.0, nsteps=100, seed=1001,
               amp=2.0, radius=2000.0, zc=2000.0, noise=0.01) -> Workload:
    """Dry warm bubble: basic state at rest, theta 300 K at the surface with
    N = 0.01 1/s; theta' = amp exp(-r^2/radius^2) centred at (domain centre,
    zc) plus U(+-noise) everywhere."""
    wl = Workload("dry_bubble", nx, ny, nz, dx, dx, dz, dt, nsteps, microphysics_option=0)
    _basic_state(wl, stable_sounding(nz, dz), np.zeros(nz), np.zeros(nz))
    _zero_perturbation(wl)
    x, y, z = _grid_xyz(nx, ny, nz, dx, dx, dz)
    xc, yc = 0.5 * nx * dx, 0.5 * ny * dx
    r2 = ((x[:, None, None] - xc) ** 2 + (y[None, :, None] - yc) ** 2
          + (z[None, None, :] - zc) ** 2) / radius ** 2
    wl.fields["th"] += amp * np.exp(-r2)
    _add_noise(wl, seed, noise)
    return wl


def thunderstorm(nx=128, ny=128, nz=48, dx=1000.0, dz=400.0, dt=4.0, nsteps=600, seed=1002,
                 amp=3.0, rh=10000.0, rz=1500.0, zc=1500.0, noise=0.05, u_top=15.0,
                 shear_depth=6000.0, rain_fallout=1, name="thunderstorm", microphysics_option=1) -> Workload:
    """Moist thunderstorm (Kessler; microphysics_option 2 for the ice scheme
    of the reference's own thunderstorm inputs): thunderstorm_sounding basic
    state; theta' = amp * (1 + cos(pi r))/2 for r <= 1 with r the distance
    from (domain centre, zc) scaled by rh horizontally and rz vertically
    (shape of sample_initializations.py:349-362), plus U(+-noise)."""
    wl = Workload(name, nx, ny, nz, dx, dx, dz, dt, nsteps, microphysics_option=microphysics_option,
                  rain_fallout=rain_fallout)
    th, qv, u = thunderstorm_sounding(nz, dz, u_top, shear_depth)
    _basic_state(wl, th, qv, u)
    _zero_perturbation(wl)
    x, y, z = _grid_xyz(nx, ny, nz, dx, dx, dz)
    xc, yc = 0.5 * nx * dx, 0.5 * ny * dx
    r = np.sqrt(((x[:, None, None] - xc) / rh) ** 2 + ((y[None, :, None] - yc) / rh) ** 2
                + ((z[None, None, :] - zc) / rz) ** 2)
    wl.fields["th"] += np.where(r <= 1.0, amp * 0.5 * (1.0 + np.cos(math.pi * r)), 0.0)
    _add_noise(wl, seed, noise)
    return wl


def squall_line(nx=512, ny=512, nz=64, dx=1000.0, dz=300.0, dt=3.0, nsteps=400, seed=1005,
                amp=2.0, half_width=5000.0, depth=3000.0, mod=0.15) -> Workload:
    """Squall line: thunderstorm sounding with 0 -> 20 m/s shear over 0-2.5 km;
    a line thermal of amp K with a half-cosine of half-width `half_width`
    across x, extending along y with a seeded, y-smoothed +-mod amplitude
    modulation, and a half-cosine in z up to `depth`."""
    wl = Workload("squall_line", nx, ny, nz, dx, dx, dz, dt, nsteps, microphysics_option=1)
    th, qv, u = thunderstorm_sounding(nz, dz, 20.0, 2500.0)
    _basic_state(wl, th, qv, u)
    _zero_perturbation(wl)
    x, y, z = _grid_xyz(nx, ny, nz, dx, dx, dz)
    x0 = 0.5 * nx * dx
    xi = 2.0 * splitmix_uniform(seed, ny) - 1.0
    kern = np.ones(9) / 9.0
    xi = np.convolve(np.pad(xi, 4, mode="wrap"), kern, mode="valid")
    xi = xi / max(np.abs(xi).max(), 1e-12)
    sx = 0.5 * (1.0 + np.cos(math.pi * np.minimum(np.abs(x - x0) / half_width, 1.0)))
    sz = np.where((z > 0) & (z < depth), 0.5 * (1.0 + np.cos(math.pi * (z / depth - 0.5) * 2.0)) , 0.0)
    wl.fields["th"] += (amp * (1.0 + mod * xi)[None, :, None]) * sx[:, None, None] * sz[None, None, :]
    _add_noise(wl, seed + 1, 0.01)
    return wl


def moist_blob(nx=24, ny=22, nz=16, dx=1000.0, dz=500.0, dt=4.0, nsteps=3, seed=2001,
               rain_fallout=1, periodic=0, qc=1.5e-3, qr=2.0e-3) -> Workload:
    """Small moist test case that exercises every Kessler branch from the
    first step: a warm, cloudy, rainy blob (theta' 2 K, qc and qr set) in the
    thunderstorm sounding, with seeded noise on all perturbation fields."""
    wl = Workload("moist_blob", nx, ny, nz, dx, dx, dz, dt, nsteps, microphysics_option=1,
                  rain_fallout=rain_fallout, periodic_ew_boundaries=periodic,
                  boundary_width_north=3, boundary_width_south=3, boundary_width_east=3,
                  boundary_width_west=3)
    th, qv, u = thunderstorm_sounding(nz, dz, 12.0, 4000.0)
    _basic_state(wl, th, qv, u)
    _zero_perturbation(wl)
    x, y, z = _grid_xyz(nx, ny, nz, dx, dx, dz)
    xc, yc = 0.5 * nx * dx, 0.5 * ny * dx
    r = np.sqrt(((x[:, None, None] - xc) / (0.3 * nx * dx)) ** 2
                + ((y[None, :, None] - yc) / (0.3 * ny * dx)) ** 2
                + ((z[None, None, :] - 2500.0) / 2000.0) ** 2)
    blob = np.where(r <= 1.0, 0.5 * (1.0 + np.cos(math.pi * r)), 0.0)
    f = wl.fields
    n3 = (nx, ny, nz)
    rnd = [2.0 * splitmix_uniform(seed + s, wl.points).reshape(n3) - 1.0 for s in range(6)]
    f["th"] += 2.0 * blob + 0.3 * rnd[0]
    f["u"] += 2.0 * rnd[1]
    f["v"] += 2.0 * rnd[2]
    f["w"] += 0.5 * rnd[3] * blob
    f["qv"] += 1.0e-3 * blob
    f["qc"] += qc * blob * (1.0 + 0.5 * rnd[4])
    f["qr"] += qr * blob * (1.0 + 0.5 * rnd[5])
    return wl


def ice_cloud(nx=24, ny=22, nz=20, dx=1000.0, dz=600.0, dt=4.0, nsteps=3, seed=2101, rain_fallout=1,
              periodic=0, qc=1.0e-3, qr=1.0e-3, qi=4.0e-4, qs=1.0e-3, zc=5000.0) -> Workload:
    """Small ice-microphysics case (microphysics_option 2) that reaches the
    warm, mixed-phase and ice-only branches from the first step: a cloudy,
    supersaturated blob centred at zc in the thunderstorm sounding (0 C near
    4 km, -30 C near 8.5 km), 5 km deep in half-width, carrying cloud water,
    rain, cloud ice and snow, with seeded noise on all perturbation fields.
    Outside the blob snow is exactly zero, as the snow intercept's update
    distinguishes."""
    wl = Workload("ice_cloud", nx, ny, nz, dx, dx, dz, dt, nsteps, microphysics_option=2,
                  rain_fallout=rain_fallout, periodic_ew_boundaries=periodic,
                  boundary_width_north=3, boundary_width_south=3, boundary_width_east=3,
                  boundary_width_west=3)
    th, qv, u = thunderstorm_sounding(nz, dz, 12.0, 4000.0)
    _basic_state(wl, th, qv, u)
    _zero_perturbation(wl)
    x, y, z = _grid_xyz(nx, ny, nz, dx, dx, dz)
    xc, yc = 0.5 * nx * dx, 0.5 * ny * dx
    r = np.sqrt(((x[:, None, None] - xc) / (0.3 * nx * dx)) ** 2
                + ((y[None, :, None] - yc) / (0.3 * ny * dx)) ** 2
                + ((z[None, None, :] - zc) / 5000.0) ** 2)
    blob = np.where(r <= 1.0, 0.5 * (1.0 + np.cos(math.pi * r)), 0.0)
    f = wl.fields
    n3 = (nx, ny, nz)
    rnd = [2.0 * splitmix_uniform(seed + s, wl.points).reshape(n3) - 1.0 for s in range(8)]
    f["th"] += 2.0 * blob + 0.3 * rnd[0]
    f["u"] += 2.0 * rnd[1]
    f["v"] += 2.0 * rnd[2]
    f["w"] += 0.5 * rnd[3] * blob
    f["qv"] += 1.0e-3 * blob
    f["qc"] += qc * blob * (1.0 + 0.5 * rnd[4])
    f["qr"] += qr * blob * (1.0 + 0.5 * rnd[5])
    f["qi"] = qi * blob * (1.0 + 0.5 * rnd[6])
    f["qs"] = qs * blob * (1.0 + 0.5 * rnd[7])
    return wl


def jet_vortex(nx=192, ny=128, nz=32, dx=40000.0, dz=600.0, dt=120.0, nsteps=500, seed=1003,
               vort=1.0e-4, upper_shear=-2.0e-3, lower_shear=-1.0e-3, vmax=5.0, rmax=500000.0,
               zmax=4000.0, corner_lat=95.0, noise=0.0, moist=False, extra_basic=0.0) -> Workload:
    """Analytic sheared jet with a vortex (small test cases of the general
    basic-state path): a zonal jet u(y, z) whose relative vorticity peaks at
    `vort` (1/s) at the domain's centre latitude, with vertical shear
    `lower_shear` below and `upper_shear` above the jet level (1/s), theta in
    thermal-wind balance with it on the stable sounding, and an axisymmetric
    vortex (max wind `vmax` at radius `rmax`, peaking at height `zmax`).
    extra_basic > 0 adds smooth horizontally varying VBAR, WBAR and QBAR of
    that relative size.  The benchmark's monsoon state is monsoon_vortex."""
    wl = Workload("jet_vortex", nx, ny, nz, dx, dx, dz, dt, nsteps, microphysics_option=1 if moist else 0,
                  corner_lat=corner_lat)
    theta = stable_sounding(nz, dz)
    qv = thunderstorm_sounding(nz, dz)[1] if moist else np.zeros(nz)
    x, y, z = _grid_xyz(nx, ny, nz, dx, dx, dz)
    yc = 0.5 * ny * dx
    ly = 0.15 * ny * dx
    eta = (y - yc) / ly
    # u = -vort * ly * eta * exp(-eta^2 / 2) / e^-0 ... scaled so that
    # -du/dy peaks at `vort` on the axis
    shape_y = -vort * ly * eta * np.exp(-0.5 * eta * eta)
    zj = 0.35 * nz * dz
    zz = np.maximum(z, 0.0)
    prof_z = 1.0 + np.where(zz < zj, lower_shear * (zz - zj) / (vort * ly), upper_shear * (zz - zj) / (vort * ly))
    u = shape_y[:, None] * prof_z[None, :]  # [y][z]
    # thermal wind: f du/dz = -(g/theta0) dtheta/dy  ->  dtheta/dy = -(f theta0 / g) du/dz
    f0 = 2 * 7.292e-5 * math.sin(math.radians(20.0))
    dudz = np.gradient(u, z, axis=1)
    dthdy = -(f0 * 300.0 / GRAV) * dudz
    th = np.cumsum(dthdy, axis=0) * dx
    th -= th.mean(axis=0, keepdims=True)
    n3 = (nx, ny, nz)
    f = wl.fields
    f["tb_in"] = theta.copy()
    f["qb_in"] = qv.copy()
    f["ubar"] = np.broadcast_to(u[None, :, :], n3).copy()
    f["vbar"] = np.zeros(n3)
    f["wbar"] = np.zeros(n3)
    f["thbar"] = np.broadcast_to(th[None, :, :], n3).copy()
    f["qbar"] = np.zeros(n3)
    tb = theta.copy(); qb = qv.copy()
    tb[0], tb[-1], qb[0], qb[-1] = tb[1], tb[-2], qb[1], qb[-2]
    pib = _exner_profile(tb * (1.0 + 0.61 * qb), _levels(nz, dz))
    pib[0], pib[-1] = pib[1], pib[-2]
    f["pbar"] = np.broadcast_to(pib, n3).copy()
    _zero_perturbation(wl)
    # vortex: v_t(r, z) = vmax (r/rmax) exp(1 - r/rmax) exp(-((z - zmax)/(0.6 zmax))^2)
    xc, ycv = 0.5 * nx * dx, 0.5 * ny * dx
    X, Y = np.meshgrid(x - xc, y - ycv, indexing="ij")
    r = np.sqrt(X * X + Y * Y) + 1e-9
    vt = vmax * (r / rmax) * np.exp(1.0 - r / rmax)
    vz = np.exp(-(((zz - zmax) / (0.6 * zmax)) ** 2))
    f["u"] = (-vt * Y / r)[:, :, None] * vz[None, None, :]
    f["v"] = (vt * X / r)[:, :, None] * vz[None, None, :]
    if extra_basic > 0:
        X3 = (x[:, None, None] / (nx * dx)) * 2 * math.pi
        Y3 = (y[None, :, None] / (ny * dx)) * 2 * math.pi
        Z3 = np.maximum(z, 0)[None, None, :] / (nz * dz)
        f["vbar"] = extra_basic * 3.0 * np.sin(X3) * np.cos(Y3) * np.ones((1, 1, nz))
        f["wbar"] = extra_basic * 0.05 * np.cos(X3 + Y3) * np.sin(math.pi * Z3)
        if moist:
            f["qbar"] = extra_basic * 1e-3 * np.sin(X3 - Y3) * np.exp(-3 * Z3)
    if noise > 0:
        _add_noise(wl, seed, noise)
    return wl


def monsoon_vortex(nx=192, ny=128, nz=32, dx=40000.0, dz=600.0, dt=120.0, nsteps=500, seed=1003,
                   corner_lat=86.0, corner_lon=53.0, hor_shear=1.0e-4, vert_shear0=-2.0e-3,
                   vert_shear1=-1.0e-3, vortex_lat=20.0, vortex_lon=88.0, r_end=2.0e6, zm=4000.0, zt=11000.0,
                   tmax=VORTEX_TMAX, tmin=VORTEX_TMIN, noise=0.0) -> Workload:
    """Sheared monsoon-depression state (dry): the reference's ITCZ-shear
    basic state (initialize_basic_state_ITCZ_shear2(hor_shear, vert_shear0,
    vert_shear1), data_initializer.cpp:298-568: vorticity strip at 18-21 N,
    streamfunction inversion, vertical shear about a 4 km level, geostrophic
    pressure and hydrostatic theta from the 20 N / 88 E column) and the
    reference's axisymmetric vortex (initialize_vortex, :862-1064) at
    (vortex_lat, vortex_lon) with radius r_end, its wind maximum at zm and
    theta anomalies tmax (warm, above zm) and tmin (cold, below); restated in
    model_gb300/monsoon.py.  corner_lat / corner_lon place the domain (the
    reference's latoffset / lonoffset, initializer.cpp:181-182): with the
    defaults 192 x 128 points of 40 km span 53.4-122.6 E and 3.1 S-42.7 N,
    centred on the 20 N / 88 E column.  The default anomalies give a maximum
    wind of 5 m/s at about 500 km from the centre, at 4 km."""
    from model_gb300 import monsoon
    wl = Workload("monsoon_vortex", nx, ny, nz, dx, dx, dz, dt, nsteps, microphysics_option=0,
                  corner_lat=corner_lat)
    st = monsoon.itcz_shear_state(nx, ny, nz, dx, dz, corner_lat, corner_lon, hor_shear, vert_shear0, vert_shear1)
    f = wl.fields
    f["tb_in"] = st["tb"].copy()
    f["qb_in"] = st["qb"].copy()
    for k in ("ubar", "vbar", "wbar", "thbar", "qbar", "pbar"):
        f[k] = st[k]
    _zero_perturbation(wl)
    xpos = monsoon._nearest(st["lons"], vortex_lon)
    ypos = monsoon._nearest(st["lats"], vortex_lat)
    f["u"], f["v"], f["th"] = monsoon.vortex(st, nx, ny, nz, dx, dz, r_end, zm, zt, tmax, tmin, xpos, ypos)
    if noise > 0:
        _add_noise(wl, seed, noise)
    return wl


def ensemble_member(m: int, nx: int, ny: int, nz: int = 48, dz: float = 400.0, nsteps: int = 300,
                    base_seed: int = 1004) -> Workload:
    """Member m of the uneven ensemble: the thunderstorm sounding and bubble
    with a seeded amplitude drawn from U(1.5, 3.5) K and U(+-0.1 K) noise
    (seed = base_seed + 7919 m)."""
    seed = base_seed + 7919 * m
    amp = 1.5 + 2.0 * float(splitmix_uniform(seed, 1)[0])
    wl = thunderstorm(nx=nx, ny=ny, nz=nz, dz=dz, nsteps=nsteps, seed=seed + 1, amp=amp, noise=0.1,
                      name=f"ensemble_member_{m}")
    return wl


def ensemble_layout(n_small: int = 64, n_large: int = 32):
    """Grid sizes of the uneven ensemble: n_small members at 96x96x40 and
    n_large at 160x160x48 (both with the thunderstorm spacing)."""
    return [(96, 96, 40)] * n_small + [(160, 160, 48)] * n_large


WORKLOADS = {
    "dry_bubble": dry_bubble,
    "thunderstorm": thunderstorm,
    "squall_line": squall_line,
    "moist_blob": moist_blob,
    "ice_cloud": ice_cloud,
    "monsoon_vortex": monsoon_vortex,
    "jet_vortex": jet_vortex,
}


def make(name: str, **kw) -> Workload:
    return WORKLOADS[name](**kw)
