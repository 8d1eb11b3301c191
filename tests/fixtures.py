"""Helpers that turn the golden .npz fixtures back into workloads."""
from __future__ import annotations

import os

import numpy as np

from model_gb300 import abi, configs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

_INT_KEYS = ("nx", "ny", "nz", "microphysics_option", "rain_fallout", "periodic_ew_boundaries",
             "boundary_width_north", "boundary_width_south", "boundary_width_east",
             "boundary_width_west", "rayleigh_damping_z")
_FLOAT_KEYS = ("dx", "dy", "dz", "dt", "height_lowest_level", "corner_lat")


def load(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def workload(d: dict) -> configs.Workload:
    kw = {k: int(d[k]) for k in _INT_KEYS}
    kw.update({k: float(d[k]) for k in _FLOAT_KEYS})
    for k in ("use_explicit_diffusion", "diffusion_order", "turbulence_option",
              "use_surface_heat_flux", "linear_model", "hydrostatic"):  # optional: fixtures with these physics
        if k in d:
            kw[k] = int(d[k])
    for k in ("kdiffh", "kdiffv", "water_temp"):
        if k in d:
            kw[k] = float(d[k])
    wl = configs.Workload(name="golden", nsteps=int(d["nsteps"]), **kw)
    n3 = (wl.nx, wl.ny, wl.nz)
    for k in list(d):
        if k.startswith("in_"):
            v = d[k]
            wl.fields[k[3:]] = v.reshape(n3) if v.size == wl.points else v
    return wl


def columns(d: dict) -> dict:
    cols = {n: d["out_" + n] for n in abi.COLUMN_NAMES}
    cols["f"] = d["out_f"]
    return cols


def run_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("run_") and f.endswith(".npz"))


def ops_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("ops_") and f.endswith(".npz"))


def linop_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("linop_") and f.endswith(".npz"))


def iceop_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("iceop_") and f.endswith(".npz"))


def hydop_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("hydop_") and f.endswith(".npz"))


def turb_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("turb_") and f.endswith(".npz"))


def slot_extra(d: dict) -> dict:
    """Per-slot input arrays of an ops fixture (u_p, u_m, ..., pi, vt)."""
    out = {}
    for k in d:
        if k.startswith("in_") and (k.endswith("_p") or k.endswith("_m") or k in (
                "in_pi", "in_vt", "in_is_saturated", "in_sts", "in_its", "in_n0s")):
            out[k[3:]] = d[k]
    return out


FIELD_OF = {}
for _f, _n in enumerate(abi.PROG_NAMES):
    for _slot, _suf in abi.SLOT_SUFFIX.items():
        FIELD_OF[_n + _suf] = (_f, _slot)
FIELD_OF["pi"] = (abi.GA_PI, 0)
FIELD_OF["vt"] = (abi.GA_VT, 0)
FIELD_OF["accrain"] = (abi.GA_ACCRAIN, 0)
for _n, _f in abi.TURB_NAMES.items():
    FIELD_OF[_n] = (_f, 0)
for _n, _f in abi.ICE_PROG.items():
    for _slot, _suf in abi.SLOT_SUFFIX.items():
        FIELD_OF[_n + _suf] = (_f, _slot)
for _n, _f in abi.ICE_NAMES.items():
    FIELD_OF[_n] = (_f, 0)


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    n = np.linalg.norm(b)
    d = np.linalg.norm(a - b)
    return float(d / n) if n > 0 else float(d)
