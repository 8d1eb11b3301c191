"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference's own serial step (oracle/_ref/ref_harness, built from the
reference sources by oracle/build_ref.sh) on small seeded states and stores
inputs and outputs as compressed .npz files:

  run_<case>.npz   full steps (s_integrate_rk3, driver_serial.cpp:178-286)
  ops_<case>.npz   single operators applied to one state whose three rotation
                   buffers all hold different data
  turb_<case>.npz  the turbulence tendencies (calculate_diff_tend) of such a
                   state, and Kessler's saturation record
  linop_<case>.npz the linearised model's operators (the ISLINEAR build)
  iceop_<case>.npz the operators of the ice microphysics (microphysics_option 2)

Usage (where the reference sources exist):  python tests/golden/make_golden.py
The fixtures are then read by tests/test_golden_oracle.py (CPU) and
tests/test_gpu_parity.py (GPU) without needing the reference.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from model_gb300 import abi, configs  # noqa: E402
from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

def _diffusing(wl, order, kdiffh):
    wl.use_explicit_diffusion, wl.diffusion_order, wl.kdiffh = 1, order, kdiffh
    return wl


def _turbulent(wl, surface_flux=0, water_temp=28.0):
    wl.turbulence_option, wl.use_surface_heat_flux, wl.water_temp = 1, surface_flux, water_temp
    return wl


def _linear(wl, bigcounter0=0):
    wl.linear_model = 1
    if bigcounter0:  # dt = 30 s: the rescaling falls on every 1440th step
        wl.fields["bigcounter0"] = np.float64(bigcounter0)
        wl.fields["mtime0"] = np.float64(bigcounter0 * wl.dt)
    return wl


def _hydro(wl):
    wl.hydrostatic = 1
    return wl


def _ice(nx=15, ny=14, nz=16, **kw):
    return configs.ice_cloud(nx=nx, ny=ny, nz=nz, dz=750.0, **kw)


def _jet(moist):
    return configs.jet_vortex(nx=16, ny=14, nz=10, dx=20000.0, dz=800.0, dt=30.0, rmax=60000.0, vmax=8.0,
                              moist=moist, noise=0.3, extra_basic=1.0)


RUN_CASES = {
    "dry": (lambda: configs.dry_bubble(nx=16, ny=14, nz=10, dx=500.0, dz=400.0, amp=3.0,
                                       radius=2000.0, zc=1500.0, noise=0.2), 4),
    "moist": (lambda: configs.moist_blob(nx=14, ny=13, nz=10), 4),
    "moist_rf2": (lambda: configs.moist_blob(nx=14, ny=13, nz=10, rain_fallout=2), 4),
    "moist_periodic": (lambda: configs.moist_blob(nx=18, ny=13, nz=10, periodic=1), 3),
    # horizontally varying basic state (jet + balanced theta), moist: the general path
    # explicit diffusion once per step (apply_explicit_diffusion), each order
    "diffusion2_dry": (lambda: _diffusing(configs.dry_bubble(nx=16, ny=14, nz=10, dx=500.0, dz=400.0, amp=3.0,
                                                             radius=2000.0, zc=1500.0, noise=0.2), 2, 0.02), 3),
    "diffusion4_moist": (lambda: _diffusing(configs.moist_blob(nx=15, ny=14, nz=10), 4, 0.004), 3),
    "diffusion6_moist": (lambda: _diffusing(configs.moist_blob(nx=16, ny=15, nz=12), 6, 0.002), 3),
    "jet": (lambda: configs.jet_vortex(nx=16, ny=14, nz=10, dx=20000.0, dz=800.0, dt=30.0, rmax=60000.0,
                                           vmax=8.0, moist=True, noise=0.3, extra_basic=1.0), 3),
    # turbulence (calculate_diff_tend once per step, applied in every RK stage)
    "turbulence_dry": (lambda: _turbulent(configs.dry_bubble(nx=16, ny=14, nz=10, dx=500.0, dz=400.0, amp=3.0,
                                                             radius=2000.0, zc=1500.0, noise=0.2)), 4),
    "turbulence_jet_dry": (lambda: _turbulent(_jet(False)), 3),
    "turbulence_moist": (lambda: _turbulent(configs.moist_blob(nx=15, ny=14, nz=10)), 4),
    "turbulence_moist_sfc": (lambda: _turbulent(configs.moist_blob(nx=18, ny=14, nz=10, periodic=1), 1, 30.0), 4),
    "turbulence_jet_sfc": (lambda: _turbulent(_jet(True), 1, 26.0), 3),
    # the linearised model (linear_integrate_rk3): dry and moist jets, with
    # explicit diffusion in every stage, and across a 12-hour rescaling
    "linear_dry": (lambda: _linear(_jet(False)), 4),
    "linear_moist": (lambda: _linear(_jet(True)), 4),
    "linear_diffusion": (lambda: _linear(_diffusing(_jet(True), 4, 0.004)), 3),
    "linear_rescale": (lambda: _linear(_jet(False), bigcounter0=1438), 4),
    # edge sizes: the smallest grid the library takes (12x12x6), odd prime
    # transform lengths (31, 29) with an odd level count, the smallest periodic
    # domain (13: an x transform of 7), and the largest level count (128)
    "edge_min": (lambda: configs.moist_blob(nx=12, ny=12, nz=6, dz=1500.0), 4),
    "edge_prime": (lambda: configs.moist_blob(nx=31, ny=29, nz=7, dz=1200.0), 3),
    "edge_periodic_min": (lambda: configs.moist_blob(nx=13, ny=12, nz=8, dz=1000.0, periodic=1), 3),
    "edge_tall": (lambda: configs.moist_blob(nx=12, ny=13, nz=128, dz=100.0), 2),
    # the hydrostatic equation set (integrate_hydro, w diagnosed)
    "hydro_dry": (lambda: _hydro(configs.dry_bubble(nx=16, ny=14, nz=10, dx=2000.0, dz=500.0, dt=4.0, amp=3.0,
                                                    radius=6000.0, zc=1500.0, noise=0.2)), 4),
    "hydro_moist": (lambda: _hydro(configs.moist_blob(nx=15, ny=14, nz=10, dx=2000.0)), 4),
    "hydro_jet": (lambda: _hydro(_jet(True)), 3),
    "hydro_diffusion": (lambda: _hydro(_diffusing(configs.moist_blob(nx=16, ny=14, nz=12, dx=2000.0), 4, 0.004)), 3),
    # ice microphysics (run_rutledge_microphysics): Eulerian and semi-
    # Lagrangian fallout, periodic, with turbulence and ocean fluxes, with
    # explicit diffusion; 16 levels of 750 m reach the ice-only temperatures
    "ice": (lambda: _ice(), 3),
    "ice_rf2": (lambda: _ice(rain_fallout=2), 3),
    "ice_periodic": (lambda: _ice(nx=18, periodic=1), 3),
    "ice_turbulence": (lambda: _turbulent(_ice(nx=16), 1, 29.0), 3),
    "ice_diffusion": (lambda: _diffusing(_ice(nx=16, ny=15), 4, 0.004), 3),
    "hydro_ice": (lambda: _hydro(_ice(dx=2000.0)), 3),
}

OP_NAMES = ["advect_uvw", "solve_pressure", "integrate_non_hydro", "advect_theta",
            "advect_micro", "zero_moisture", "bc", "bc_micro", "kessler", "rayleigh", "explicit_diffusion"]


def _inputs(wl) -> dict:
    d = {k: np.asarray(v, dtype=np.float64) for k, v in wl.settings().items()}
    for k, v in wl.fields.items():
        d["in_" + k] = np.asarray(v, dtype=np.float64).ravel()
    d["nsteps"] = np.float64(wl.nsteps)
    return d


def make_runs():
    for name, (mk, nsteps) in RUN_CASES.items():
        wl = mk()
        wl.nsteps = nsteps
        out = O.run_reference(wl, "run", nsteps)
        d = _inputs(wl)
        for k, v in out.items():
            d["out_" + k] = v
        path = os.path.join(HERE, f"run_{name}.npz")
        np.savez_compressed(path, **d)
        print("wrote", path, os.path.getsize(path))


def _ops_state(wl, seed: int) -> dict:
    """Extra slot data so that current, P and M buffers all differ."""
    n3 = (wl.nx, wl.ny, wl.nz)
    extra = {}
    s = seed
    for f, name in enumerate(abi.PROG_NAMES):
        base = wl.fields[name]
        scale = {"u": 1.0, "v": 1.0, "w": 0.3, "th": 0.5, "qv": 2e-4, "qc": 4e-4, "qr": 4e-4}[name]
        for suf in ("_p", "_m"):
            r = 2.0 * configs.splitmix_uniform(s, wl.points).reshape(n3) - 1.0
            s += 1
            v = base + scale * r
            if name in ("qc", "qr"):
                v = np.abs(v) if suf == "_m" else v  # P may hold negatives for zero_moisture
            extra[name + suf] = v
    if wl.microphysics_option == 2:  # snow and ice: every slot non-negative
        for name in ("qs", "qi"):
            for suf in ("_p", "_m"):
                r = 2.0 * configs.splitmix_uniform(s, wl.points).reshape(n3) - 1.0
                s += 1
                extra[name + suf] = np.abs(wl.fields[name] + 4e-4 * r)
        extra["sts"] = np.zeros(n3)
        # a fall speed that the Eulerian ice update keeps where pi is small
        extra["its"] = 0.3 * configs.splitmix_uniform(s, wl.points).reshape(n3)
        s += 1
        extra["n0s"] = np.array([5.0e7])
    r = 2.0 * configs.splitmix_uniform(s, wl.points).reshape(n3) - 1.0
    extra["pi"] = 20.0 * r
    extra["vt"] = np.zeros(n3)
    return extra


def make_ops():
    cases = {
        "jet": configs.jet_vortex(nx=16, ny=14, nz=10, dx=20000.0, dz=800.0, dt=30.0, rmax=60000.0,
                                      vmax=8.0, moist=True, noise=0.3, extra_basic=1.0),
        "moist": configs.moist_blob(nx=14, ny=13, nz=10),
        "moist_periodic_rf2": configs.moist_blob(nx=18, ny=13, nz=10, periodic=1, rain_fallout=2),
    }
    for cname, wl in cases.items():
        # the reference allocates the diffusion work array only with the flag on
        _diffusing(wl, 4, 0.005)
        extra = _ops_state(wl, 5000)
        d = _inputs(wl)
        for k, v in extra.items():
            d["in_" + k] = v.ravel()
        steps = {"advect_uvw": 1.0 / 3.0, "solve_pressure": 0.5, "integrate_non_hydro": 1.0,
                 "advect_theta": 0.5, "advect_micro": 1.0 / 3.0}
        for op in OP_NAMES:
            st = steps.get(op, 1.0)
            out = O.run_reference(wl, "op", op=op, step=st, extra=extra)
            d[f"step_{op}"] = np.float64(st)
            for k, v in out.items():
                if k in abi.COLUMN_NAMES or k in ("f", "bigcounter", "mtime"):
                    continue
                ref_in = extra.get(k, wl.fields.get(k))
                if ref_in is not None and np.array_equal(np.asarray(ref_in).ravel(), v):
                    continue  # unchanged by this operator
                d[f"{op}__{k}"] = v
        path = os.path.join(HERE, f"ops_{cname}.npz")
        np.savez_compressed(path, **d)
        print("wrote", path, os.path.getsize(path))


TURB_OPS = ["turbulence", "kessler"]


def make_turb():
    """turb_<case>.npz: calculate_diff_tend on a state whose rotation slots
    differ, with a seeded saturation record (both Brunt-Vaisala branches of
    get_Kmix), and Kessler's saturation record of the same state"""
    cases = {
        "moist": _turbulent(configs.moist_blob(nx=14, ny=13, nz=10)),
        "moist_sfc": _turbulent(configs.moist_blob(nx=15, ny=13, nz=10), 1, 29.0),
        "jet_dry": _turbulent(_jet(False)),
        "jet_sfc": _turbulent(_jet(True), 1, 27.0),
    }
    for cname, wl in cases.items():
        extra = _ops_state(wl, 7000)
        if wl.microphysics_option:
            extra["is_saturated"] = (configs.splitmix_uniform(7100, wl.points) < 0.5).astype(np.float64).reshape(
                wl.nx, wl.ny, wl.nz)
        else:
            for q in ("qv", "qc", "qr"):
                extra.pop(q + "_p"), extra.pop(q + "_m")
        d = _inputs(wl)
        for k, v in extra.items():
            d["in_" + k] = v.ravel()
        ops = TURB_OPS if wl.microphysics_option else TURB_OPS[:1]
        for op in ops:
            out = O.run_reference(wl, "op", op=op, step=1.0, extra=extra)
            d[f"step_{op}"] = np.float64(1.0)
            for k, v in out.items():
                if k in abi.COLUMN_NAMES or k in ("f", "bigcounter", "mtime"):
                    continue
                if (op == "turbulence") != (k in abi.TURB_NAMES) or k == "is_saturated" and op == "turbulence":
                    if not (op == "kessler" and k == "is_saturated"):
                        continue
                ref_in = extra.get(k, wl.fields.get(k))
                if op != "turbulence" and ref_in is not None and np.array_equal(np.asarray(ref_in).ravel(), v):
                    continue  # unchanged by this operator
                d[f"{op}__{k}"] = v
        path = os.path.join(HERE, f"turb_{cname}.npz")
        np.savez_compressed(path, **d)
        print("wrote", path, os.path.getsize(path))


HYDRO_OPS = {"advect_uvw": "advect_uv", "solve_pressure": "solve_pressure", "integrate_non_hydro": "integrate_hydro",
             "kessler": "kessler", "bc": "bc", "rayleigh": "rayleigh"}

LINEAR_OPS = {"advect_uvw": "advect_uvw", "advect_theta": "advect_theta", "advect_micro": "advect_qv",
              "integrate_non_hydro": "integrate_non_hydro"}


ICE_OPS = {"advect_uvw": "advect_uvw", "advect_micro": "advect_micro", "advect_ice": "advect_ice",
           "kessler": "kessler", "bc_micro": "bc_micro", "zero_moisture": "zero_moisture",
           "explicit_diffusion": "explicit_diffusion"}


def make_ice_ops():
    """iceop_<case>.npz: the operators of the ice scheme on a state whose
    rotation slots differ (run_microphysics is run_rutledge_microphysics);
    the periodic case with turbulence also records saturation_adjustment's
    saturation record.  A third case puts negative snow and ice into the
    forecast slot for zero_moisture and the boundary conditions (the
    microphysics would take roots of them)."""
    cases = {"cloud": _diffusing(_ice(), 4, 0.005),
             "periodic_sat": _turbulent(_diffusing(_ice(nx=18, periodic=1, rain_fallout=2), 6, 0.003), 1, 28.0)}
    _variant_ops("iceop", cases, ICE_OPS, step=1.0 / 3.0)
    wl = _diffusing(_ice(nx=16, ny=13), 2, 0.01)
    neg = _ops_state(wl, 9500)
    for name in ("qs_p", "qi_p"):
        r = 2.0 * configs.splitmix_uniform(9600 + len(name), wl.points).reshape(wl.nx, wl.ny, wl.nz) - 1.0
        neg[name] = neg[name] + 3e-4 * r
    _variant_ops("iceop", {"negative": wl}, {"zero_moisture": "zero_moisture", "bc_micro": "bc_micro"},
                 extra=neg)


def make_linear_ops():
    """linop_<case>.npz: the linearised operators (the ISLINEAR build) on a
    state whose rotation slots differ; the moisture operator of the
    linearised model is advect_qv.  hydop_<case>.npz: the operators of the
    hydrostatic set (the HYDROSTATIC build)"""
    _variant_ops("linop", {"jet": _linear(_jet(True))}, LINEAR_OPS)
    _variant_ops("hydop", {"moist": _hydro(configs.moist_blob(nx=15, ny=14, nz=10, dx=2000.0))}, HYDRO_OPS)


def _variant_ops(prefix, cases, ops, step=0.5, extra=None):
    for cname, wl in cases.items():
        if extra is None or len(cases) > 1:
            extra = _ops_state(wl, 9000)
        if wl.turbulence_option and wl.microphysics_option:
            extra["is_saturated"] = (configs.splitmix_uniform(9900, wl.points) < 0.5).astype(np.float64).reshape(
                wl.nx, wl.ny, wl.nz)
        d = _inputs(wl)
        for k, v in extra.items():
            d["in_" + k] = v.ravel()
        for op, ref_op in ops.items():
            st = step
            out = O.run_reference(wl, "op", op=ref_op, step=st, extra=extra)
            d[f"step_{op}"] = np.float64(st)
            for k, v in out.items():
                if k in abi.COLUMN_NAMES or k in ("f", "bigcounter", "mtime"):
                    continue
                if k in abi.TURB_NAMES and k != "is_saturated":
                    continue  # the turbulence tendencies: calculate_diff_tend only
                ref_in = extra.get(k, wl.fields.get(k))
                if ref_in is not None and np.array_equal(np.asarray(ref_in).ravel(), v):
                    continue
                d[f"{op}__{k}"] = v
        path = os.path.join(HERE, f"{prefix}_{cname}.npz")
        np.savez_compressed(path, **d)
        print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    if not O.reference_available():
        subprocess_rc = os.system(os.path.join(ROOT, "oracle", "build_ref.sh"))
        if subprocess_rc != 0:
            sys.exit("reference build failed")
    make_runs()
    make_ops()
    make_turb()
    make_linear_ops()
    make_ice_ops()
