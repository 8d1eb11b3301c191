"""Generate tests/golden/itcz_*.npz from the reference's own monsoon initialisers.

Runs oracle/_ref/itcz_harness (the reference's initialize_basic_state_ITCZ_shear2
and initialize_vortex, built by oracle/build_ref.sh) on small grids and stores
the column arrays in full and the 3-D basic state and vortex as digests
(model_gb300/digest.py).  The grids have at least 39 levels, where the
reference's shear profile stays inside its arrays; tests/test_monsoon_state.py
checks model_gb300/monsoon.py against them.

Usage (where the reference sources exist):  python tests/golden/make_itcz.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from model_gb300 import digest  # noqa: E402
from oracle.ga_bundle import read_bundle, write_bundle  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "itcz_harness")

# grid and parameters; 80 km spacing keeps 5-30 N inside 52 rows
CASES = {
    "default": dict(nx=48, ny=52, nz=40, dx=80000.0, dz=600.0, corner_lat=85.7, corner_lon=71.5, hor_shear=1.0e-4,
                    vert_shear0=-2.0e-3, vert_shear1=-1.0e-3, vortex_radius=1.0e6, vortex_height_wind_max=4000.0,
                    vortex_vertical_extent=11000.0, vortex_upper_warm_anomaly=3.8776,
                    vortex_lower_cold_anomaly=-3.1796, vortex_latitude=20.0, vortex_longitude=88.0),
    "strong": dict(nx=40, ny=56, nz=42, dx=80000.0, dz=500.0, corner_lat=85.0, corner_lon=74.0, hor_shear=1.6e-4,
                   vert_shear0=-1.0e-3, vert_shear1=-2.5e-3, vortex_radius=1.4e6, vortex_height_wind_max=3000.0,
                   vortex_vertical_extent=12000.0, vortex_upper_warm_anomaly=2.0,
                   vortex_lower_cold_anomaly=-2.5, vortex_latitude=17.0, vortex_longitude=86.0),
}
COLUMNS = ("tb", "qb", "tbv", "pib", "rhou", "rhow", "lats", "lons", "f", "vortex_ij")
FIELDS = ("ubar", "vbar", "wbar", "thbar", "qbar", "pbar", "u", "v", "th")


def run(params: dict) -> dict:
    b = {k: np.array([float(v)]) for k, v in params.items()}
    b["dy"] = b["dx"]
    b["dt"] = np.array([60.0])
    b["height_lowest_level"] = b["dz"]
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_bundle(fi, b)
        subprocess.run([HARNESS, fi, fo], check=True, stdout=subprocess.DEVNULL)
        return read_bundle(fo)


def main():
    for name, p in CASES.items():
        out = run(p)
        shape = (p["nx"], p["ny"], p["nz"])
        d = digest.digest({k: out[k] for k in FIELDS}, shape, m=64, samples=4096)
        for k in COLUMNS:
            d["col_" + k] = np.asarray(out[k], dtype=np.float64)
        for k, v in p.items():
            d["param_" + k] = np.float64(v)
        path = os.path.join(HERE, f"itcz_{name}.npz")
        np.savez_compressed(path, **d)
        print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    main()
