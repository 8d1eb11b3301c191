#!/usr/bin/env python
"""Benchmark of the GB300 anelastic dynamical core.

Metric: gridpoint-steps/s = NX*NY*NZ*steps / seconds of stepping, for the
forward RK3 step (s_integrate_rk3, driver_serial.cpp:178-286) of the Kessler
thunderstorm workload, 128x128x48, dx=dy=1 km, dz=400 m, dt=4 s (seeded
synthetic state: analytic sounding + warm bubble + noise), FP32 storage and
arithmetic with FP64 islands; FP64 beside it; each result's error against the
FP64 path (itself checked against the CPU oracle in tests/) stated.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Timing: K model steps, each bracketed by CUDA events recorded on the
library's stream, with a 256 MiB L2 flush (write) between steps outside the
events; a barrier + synchronize on both sides of the loop; the max over ranks.
Under torchrun (N>1) every rank integrates its own domain (replicas: the
single-domain step does not shard) and `value` is the sum over ranks.

--impl reference times the reference's CPU step: the oracle restatement,
which matches the reference's own serial build bit for bit (tests/golden), on
every host core of this machine (the serial step is single-threaded, so one
independent replica per core, stepping at the same time), over a bounded
sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "gridpoint-steps/s (fwd, fwd+adjoint) FP32 vs FP64 at stated err; %HBM peak"
UNIT = "gridpoint-steps/s"
WORKLOAD_DESC = ("Kessler thunderstorm 128x128x48, dx=dy=1 km, dz=400 m, dt=4 s; value: --steps steps from the "
                 "initial state; e2e and accuracy: whole 600-step runs")
DATA = "synthetic: seeded thunderstorm sounding (theta 300->343 K, RH 0.95->0.25, u 0->15 m/s) + 3 K warm bubble + U(+-0.05 K) noise"
L2_FLUSH_BYTES = 256 << 20

# algorithmic field passes (one read or write of an N-point field) per launch
# of each kernel group; spectral passes count complex values as two fields.
# Advection with a basic state of height only (every bench workload): the
# current and start-of-step fields in, the forecast (and the fall speed) out;
# the basic state is a per-level table.
PASSES_DRY = {"advect": 12, "div_fft_y": 5, "fft_x": 4, "thomas": 4, "ifft_y_pi": 3, "post": 9,
              "kessler": 0}
PASSES_MOIST = {"advect": 22, "div_fft_y": 5, "fft_x": 4, "thomas": 4, "ifft_y_pi": 3, "post": 16,
                "kessler": 12}
# DRAM bytes per launch (read + write) of the dominant kernel, copied from one
# ncu capture of the bench command (cold cache) into this table; a run does not
# measure it.  workload -> (kernel group, kernel, bytes, summary)
TRAFFIC_NCU = {"thunderstorm": ("advect", "k_advect_quad<4,8,4>", 50.01e6,
                                "profiles/forward_kernels_thunderstorm_128x128x48_fp32.md")}
# compulsory bytes per gridpoint-step of an ideally fused step (FP32 moist)
STEP_BYTES_FP32_MOIST = 540.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fp:
            d = json.load(fp)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"ga_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fp = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fp.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allreduce_max(dist, x: float, device) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_result(dist, ms_local: float, world: int, points: int, steps: int, device):
    """Replicas: every rank integrates its own domain, so the job advanced
    world x points x steps gridpoint-steps in the slowest rank's time.
    Returns (max over ranks of the timed ms, whole-job gridpoint-steps/s)."""
    ms = allreduce_max(dist, float(ms_local), device)
    return ms, world * points * steps / (ms * 1e-3)


# ---------------------------------------------------------------------------
def time_steps(model, torch, steps, flush, profile=False):
    """Per-step CUDA-event times (ms) on the library's stream, with an L2
    flush between steps outside the events."""
    ext = torch.cuda.ExternalStream(model.stream_handle())
    evs = []
    for _ in range(steps):
        with torch.cuda.stream(ext):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(ext)
        model.step_async(1)
        b.record(ext)
        evs.append((a, b))
    model.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


def profile_groups(model, torch, steps, flush):
    from model_gb300 import anelastic
    import ctypes as C
    L = anelastic.load_library()
    L.ga_profile_enable.argtypes = [C.c_void_p, C.c_int]
    L.ga_profile_get.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_size_t, C.POINTER(C.c_double),
                                 C.POINTER(C.c_longlong)]
    L.ga_profile_enable(model.h, 1)
    time_steps(model, torch, steps, flush)
    out = {}
    for i in range(L.ga_profile_count(model.h)):
        name = C.create_string_buffer(32)
        ms, n = C.c_double(), C.c_longlong()
        L.ga_profile_get(model.h, i, name, 32, C.byref(ms), C.byref(n))
        if n.value:
            out[name.value.decode()] = {"ms": ms.value, "launches": n.value}
    L.ga_profile_enable(model.h, 0)
    return out


def roofline(groups, wl, prec_bytes, peak_gbs, peak_kind, workload=None):
    passes = PASSES_MOIST if wl.microphysics_option else PASSES_DRY
    dom = max((g for g in groups if g in passes and passes[g] > 0), key=lambda g: groups[g]["ms"])
    g = groups[dom]
    per_launch_ms = g["ms"] / g["launches"]
    spec_pts = wl.nx * wl.ny * (wl.nz - 2)
    pts = spec_pts if dom in ("div_fft_y", "fft_x", "thomas", "ifft_y_pi") else wl.points
    nbytes = passes[dom] * pts * prec_bytes
    achieved = nbytes / (per_launch_ms * 1e-3) / 1e9
    table = {k: {"ms_per_launch": round(v["ms"] / v["launches"], 5), "share": round(v["ms"] / sum(
        x["ms"] for x in groups.values()), 4)} for k, v in groups.items()}
    tr = TRAFFIC_NCU.get(workload)
    traffic, source = (tr[2], f"ncu capture of {tr[1]} summarised in {tr[3]}, copied into bench.py; "
                       "not measured by this run") if tr and tr[0] == dom and prec_bytes == 4 else (None, None)
    out = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak_gbs, "unit": "GB/s",
           "frac": round(achieved / peak_gbs, 4), "peak_source": peak_kind,
           "algorithmic_bytes_per_launch": int(nbytes), "ms_per_launch": round(per_launch_ms, 5),
           "traffic": traffic, "groups": table}
    if source:
        out["traffic_source"] = source
    return out


def e2e_jobs(model_cls, wl, prec, torch, jobs, job_steps, device):
    """Whole runs through the C ABI with pinned host buffers: upload the
    initial state, integrate job_steps, download the prognostic fields."""
    from model_gb300 import abi
    m = model_cls(wl, prec, device=device, init_state=False)
    n = wl.points
    nprog = 7 if wl.microphysics_option else 4

    def pinned(arr):
        t = torch.empty(arr.size, dtype=torch.float64, pin_memory=True)
        t.numpy()[:] = np.asarray(arr, dtype=np.float64).ravel()
        return t

    host_in = []
    for b, name in enumerate(abi.BAR_NAMES):
        host_in.append((abi.GA_UBAR + b, 0, pinned(wl.fields[name])))
    zeros = pinned(np.zeros(n))
    for f in range(nprog):
        a = pinned(wl.fields[abi.PROG_NAMES[f]])
        host_in += [(f, abi.GA_SLOT_CUR, a), (f, abi.GA_SLOT_M, a), (f, abi.GA_SLOT_P, zeros)]
    host_out = [torch.empty(n, dtype=torch.float64, pin_memory=True) for _ in range(nprog + 1)]
    import ctypes as C
    L = m.L
    dp = C.POINTER(C.c_double)

    def one_job():
        for f, slot, t in host_in:
            rc = L.ga_set_field(m.h, f, slot, C.cast(t.data_ptr(), dp), n)
            assert rc == 0
        rc = L.ga_step(m.h, job_steps)
        assert rc == 0, rc
        for f in range(nprog):
            assert L.ga_get_field(m.h, f, 0, C.cast(host_out[f].data_ptr(), dp), n) == 0
        assert L.ga_get_field(m.h, abi.GA_PI, 0, C.cast(host_out[nprog].data_ptr(), dp), n) == 0

    one_job()  # warm-up; it leaves a real state for the autotuner
    tuning = m.tune()  # once per context, as a user of ga_tune would
    one_job()
    t0 = time.perf_counter()
    for _ in range(jobs):
        one_job()
    el = time.perf_counter() - t0
    h2d = len(host_in) * n * 8
    d2h = (nprog + 1) * n * 8
    m.close()
    return {"value": round(n * job_steps * jobs / el, 1), "unit": UNIT,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "step": f"one {job_steps}-step run: upload initial state, integrate, download fields",
            "jobs": jobs, "seconds_per_run": round(el / jobs, 4), "tuning": tuning}


def ensemble_bench(torch, device, steps, warmup, n_small=64, n_large=32):
    """Uneven ensemble: n_small members at 96x96x40 and n_large at
    160x160x48, FP32, Kessler, batched kernels + CUDA graph.  The state
    (about 8 GB) is far larger than L2, so no flush is needed."""
    from model_gb300 import abi, anelastic, configs
    layout = configs.ensemble_layout(n_small, n_large)
    members = [configs.Workload(f"m{m}", nx, ny, nz, 1000.0, 1000.0, 400.0, 4.0, 300, microphysics_option=1)
               for m, (nx, ny, nz) in enumerate(layout)]
    cols_by_size, cols = {}, []
    for m, (nx, ny, nz) in enumerate(layout):
        if (nx, ny, nz) not in cols_by_size:
            cols_by_size[(nx, ny, nz)] = anelastic.build_columns(configs.ensemble_member(m, nx, ny, nz))
        cols.append(cols_by_size[(nx, ny, nz)])
    t0 = time.perf_counter()
    ens = anelastic.Ensemble(members, abi.GA_PREC_F32, device=device, columns=cols)
    for m, (nx, ny, nz) in enumerate(layout):
        ens.load_member(m, configs.ensemble_member(m, nx, ny, nz).fields)
    setup = time.perf_counter() - t0
    t1 = time.perf_counter()
    tuning = ens.tune()
    t_tune = time.perf_counter() - t1
    ens.step(max(2, warmup))
    ext = torch.cuda.ExternalStream(ens.stream_handle())
    l0 = ens.launch_count()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    ens.synchronize()
    a.record(ext)
    ens.step_async(steps)
    b.record(ext)
    ens.synchronize()
    ms = a.elapsed_time(b)
    pts = sum(nx * ny * nz for nx, ny, nz in layout)
    out = {"value": round(pts * steps / (ms * 1e-3), 1), "unit": UNIT, "members": len(layout),
           "layout": f"{n_small} x 96x96x40 + {n_large} x 160x160x48", "points": pts, "steps": steps,
           "ms_per_step": round(ms / steps, 4), "launches_per_step": (ens.launch_count() - l0) / steps,
           "setup_s": round(setup, 1), "precision": "fp32",
           "tuning": {"choice": tuning, "seconds": round(t_tune, 2)},
           "note": "one launch per kernel phase over all members; two-step CUDA graph"}
    peak, peak_kind = load_peaks()
    out["hbm_fraction"] = round(out["value"] * STEP_BYTES_FP32_MOIST / 1e9 / peak, 4)
    out["hbm_peak"] = {"gbs": peak, "source": peak_kind, "bytes_per_gridpoint_step": STEP_BYTES_FP32_MOIST}
    ens.close()
    return out


def adjoint_bench(torch, device, steps, every, moist=False, size=512):
    """Forward vs forward+adjoint: `steps` steps from the initial state, then
    the adjoint of the whole run back to it with the state checkpointed every
    `every` steps.  The library keeps the trajectories of as many of the last
    segments as device memory holds and recomputes the others; the
    `*_one_resident` figures force one (every segment but the last
    recomputed).  Dry: the monsoon vortex
    (192x128x32, dx=dy=40 km, dz=600 m, dt=120 s), FP32 and FP64.  Moist: the
    Kessler squall line (size x size x 64, dx=dy=1 km, dz=300 m, dt=3 s), FP32.
    One job per timing, bracketed by CUDA events on the library stream, L2
    flushed before each job."""
    from model_gb300 import abi, anelastic, configs
    if moist:
        wl = configs.squall_line(nx=size, ny=size, nsteps=steps)
        desc = f"Kessler squall line {wl.nx}x{wl.ny}x{wl.nz}, dx=dy=1 km, dz=300 m, dt=3 s"
        precs = (("fp32", abi.GA_PREC_F32),)
        mem = "checkpoints: steps/every+1 states of 21 fields; trajectory: every x (26 fields + 3 clipping records)"
    else:
        wl = configs.monsoon_vortex(nsteps=steps)
        desc = f"dry monsoon vortex {wl.nx}x{wl.ny}x{wl.nz}, dx=dy=40 km, dz=600 m, dt=120 s"
        precs = (("fp32", abi.GA_PREC_F32), ("fp64", abi.GA_PREC_F64))
        mem = "checkpoints: steps/every+1 states of 12 fields; trajectory: every x 12 fields"
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")
    out = {"workload": desc, "steps": steps, "checkpoint_every": every, "memory": mem}
    nprog = 7 if moist else 4
    for name, prec in precs:
        m = anelastic.Model(wl, prec, device=device)
        m.tune()
        ext = torch.cuda.ExternalStream(m.stream_handle())
        zero = np.zeros(wl.points)

        def reset():
            # initial state (current = M = perturbation, P = 0); the basic
            # state is left alone so no graph is rebuilt inside a timing
            for f in range(nprog):
                init = wl.fields[abi.PROG_NAMES[f]]
                m.set(f, abi.GA_SLOT_CUR, init)
                m.set(f, abi.GA_SLOT_P, zero)
                m.set(f, abi.GA_SLOT_M, init)
            for f in range(nprog):
                for s in m.LIN_SLOTS:
                    m.lin_set(f, s, zero)
            m.lin_set(abi.GA_PI, 0, zero)
            m.lin_set(abi.GA_U, abi.GA_SLOT_CUR, np.full(wl.points, 1.0 / wl.points))

        def timed(fn):
            reset()
            flush.fill_(1.0)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(ext)
            fn()
            b.record(ext)
            torch.cuda.synchronize()
            return a.elapsed_time(b)

        reset()
        m.adjoint(steps, every)  # warm-up; sizes the checkpoint and trajectory buffers
        m.step(2)  # captures the two-step graphs of both rotation parities
        m.step(1)
        m.step(2)
        t_fwd = timed(lambda: m.step_async(steps))
        l1 = m.launch_count()
        t_adj = timed(lambda: m.adjoint(steps, every))
        l2 = m.launch_count()
        free, total = torch.cuda.mem_get_info(device)
        os.environ["GA_ADJ_RESIDENT"] = "1"
        try:
            t_adj1 = timed(lambda: m.adjoint(steps, every))
        finally:
            del os.environ["GA_ADJ_RESIDENT"]
        pts = wl.points * steps
        out[name] = {"fwd_ms": round(t_fwd, 2), "fwd_adj_ms": round(t_adj, 2),
                     "fwd_adj_over_fwd": round(t_adj / t_fwd, 3),
                     "value_fwd": round(pts / (t_fwd * 1e-3), 1), "value_fwd_adj": round(pts / (t_adj * 1e-3), 1),
                     "unit": UNIT, "launches_fwd_adj": int(l2 - l1),
                     "device_gb_in_use": round((total - free) / 1e9, 1),
                     "fwd_adj_ms_one_resident": round(t_adj1, 2),
                     "fwd_adj_over_fwd_one_resident": round(t_adj1 / t_fwd, 3)}
        if moist and prec == abi.GA_PREC_F32:
            # the forward against the HBM roofline by the 540 B/gridpoint-step model
            peak, peak_kind = load_peaks()
            out[name]["hbm_fraction_fwd"] = round(pts / (t_fwd * 1e-3) * STEP_BYTES_FP32_MOIST / 1e9 / peak, 4)
            out[name]["hbm_peak"] = {"gbs": peak, "source": peak_kind}
        m.close()
    return out


# field passes per step of the optional physics (moist, FP32 fields): the
# turbulence coefficients (14 fields in, 2 out), the tendencies (9 in, 7 out)
# and three stage additions (14 in, 7 out each); explicit diffusion's one
# pass (7 in, 7 out)
PHYSICS_PASSES = {"turbulence": 16 + 16 + 3 * 21, "diffusion": 14}


def physics_bench(torch, device, steps, accuracy_steps):
    """The C2 thunderstorm with the optional physics of the step switched on:
    explicit diffusion (4th order), the turbulence scheme with ocean surface
    fluxes, and both; FP32 tuned, per-group event times, the groups' HBM
    fraction by their algorithmic passes, FP64 beside the combined case and
    its FP32 error after accuracy_steps steps."""
    from model_gb300 import abi, anelastic, configs
    peak, peak_kind = load_peaks()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")
    variants = {"none": {}, "explicit_diffusion": {"use_explicit_diffusion": 1, "diffusion_order": 4},
                "turbulence": {"turbulence_option": 1, "use_surface_heat_flux": 1},
                "both": {"use_explicit_diffusion": 1, "diffusion_order": 4, "turbulence_option": 1,
                         "use_surface_heat_flux": 1}}
    out = {"workload": "Kessler thunderstorm 128x128x48 with the optional physics", "steps": steps,
           "kdiffh": 0.005, "kdiffv": 0.005, "water_temp_c": 28.0}
    for name, kw in variants.items():
        wl = configs.thunderstorm()
        for k, v in kw.items():
            setattr(wl, k, v)
        m = anelastic.Model(wl, abi.GA_PREC_F32, device=device)
        m.tune()
        for _ in range(3):
            m.step(1)
        per = time_steps(m, torch, steps, flush)
        ms = sum(per) / steps
        groups = profile_groups(m, torch, min(steps, 10), flush)
        nprof = min(steps, 10)
        r = {"ms_per_step": round(ms, 4), "value": round(wl.points / (ms * 1e-3), 1), "unit": UNIT}
        for g, passes in PHYSICS_PASSES.items():
            if g in groups:
                gms = groups[g]["ms"] / nprof
                gbs = passes * wl.points * 4 / (gms * 1e-3) / 1e9
                r[g] = {"ms_per_step": round(gms, 4), "launches_per_step": groups[g]["launches"] / nprof,
                        "algorithmic_passes": passes, "achieved_gbs": round(gbs, 1),
                        "hbm_frac": round(gbs / peak, 4)}
        m.close()
        out[name] = r
    base = out["none"]["ms_per_step"]
    for name in variants:
        out[name]["over_none"] = round(out[name]["ms_per_step"] / base, 3)
    wl = configs.thunderstorm()
    for k, v in variants["both"].items():
        setattr(wl, k, v)
    m64 = anelastic.Model(wl, abi.GA_PREC_F64, device=device)
    for _ in range(2):
        m64.step(1)
    per64 = time_steps(m64, torch, max(2, steps // 2), flush)
    out["both"]["fp64_ms_per_step"] = round(sum(per64) / len(per64), 4)
    out["both"]["fp32_over_fp64"] = round(out["both"]["fp64_ms_per_step"] / out["both"]["ms_per_step"], 2)
    m64.close()
    if accuracy_steps > 0:
        a = anelastic.Model(wl, abi.GA_PREC_F32, device=device)
        b = anelastic.Model(wl, abi.GA_PREC_F64, device=device)
        a.step(accuracy_steps)
        b.step(accuracy_steps)
        errs = {}
        for f in range(7):
            x, y = a.get(f), b.get(f)
            errs[abi.PROG_NAMES[f]] = float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))
        out["both"]["accuracy"] = {"steps": accuracy_steps, "rel_l2_fp32_vs_fp64": {k: float(f"{v:.4g}") for k, v
                                                                                   in errs.items()},
                                   "max": float(f"{max(errs.values()):.4g}")}
        a.close()
        b.close()
    out["hbm_peak"] = {"gbs": peak, "source": peak_kind}
    return out


def variants_bench(torch, device, steps, accuracy_steps):
    """The reference's other equation sets and its ice scheme: the
    linearised model about the C3 jet basic state (192x128x32, dt = 120 s),
    the hydrostatic set on the C2 thunderstorm at dx = 2 km, and the ice
    microphysics on a cloud at the C2 grid; FP32 and FP64 ms/step (tuned
    FP32, L2 written over between steps) and the FP32 error after
    accuracy_steps."""
    from model_gb300 import abi, anelastic, configs
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")
    cases = {"linear_model": (lambda: configs.jet_vortex(noise=0.3, extra_basic=1.0), {"linear_model": 1},
                              "linearised model about the 192x128x32 jet, dt=120 s"),
             "hydrostatic": (lambda: configs.thunderstorm(dx=2000.0), {"hydrostatic": 1},
                             "hydrostatic set, Kessler thunderstorm 128x128x48, dx=dy=2 km, dt=4 s"),
             "ice": (lambda: configs.ice_cloud(nx=128, ny=128, nz=48, dz=400.0), {},
                     "ice microphysics (microphysics_option 2), a 10 km deep cloud of water, rain, ice and "
                     "snow on the thunderstorm grid 128x128x48, dx=dy=1 km, dt=4 s")}
    out = {"steps": steps}
    for name, (mk, kw, desc) in cases.items():
        wl = mk()
        for k, v in kw.items():
            setattr(wl, k, v)
        r = {"workload": desc}
        for prec, tag in ((abi.GA_PREC_F32, "fp32"), (abi.GA_PREC_F64, "fp64")):
            m = anelastic.Model(wl, prec, device=device)
            if prec == abi.GA_PREC_F32:
                m.tune()
            for _ in range(3):
                m.step(1)
            n = steps if prec == abi.GA_PREC_F32 else max(2, steps // 4)
            per = time_steps(m, torch, n, flush)
            ms = sum(per) / n
            r[tag] = {"ms_per_step": round(ms, 4), "value": round(wl.points / (ms * 1e-3), 1), "unit": UNIT}
            m.close()
        r["fp32_over_fp64"] = round(r["fp64"]["ms_per_step"] / r["fp32"]["ms_per_step"], 2)
        if accuracy_steps > 0:
            a = anelastic.Model(wl, abi.GA_PREC_F32, device=device)
            b = anelastic.Model(wl, abi.GA_PREC_F64, device=device)
            a.step(accuracy_steps)
            b.step(accuracy_steps)
            nf = 7 if wl.microphysics_option else 4
            fids = {abi.PROG_NAMES[f]: f for f in range(nf)}
            if wl.microphysics_option == 2:
                fids.update(abi.ICE_PROG)
            errs = {name: float(np.linalg.norm(a.get(f) - b.get(f)) / max(np.linalg.norm(b.get(f)), 1e-300))
                    for name, f in fids.items()}
            r["accuracy"] = {"steps": accuracy_steps,
                             "rel_l2_fp32_vs_fp64": {k: float(f"{v:.4g}") for k, v in errs.items()},
                             "max": float(f"{max(errs.values()):.4g}")}
            a.close()
            b.close()
        out[name] = r
    return out


def cpu_baseline(wl, steps):
    """The reference's CPU step (oracle restatement, 1 core) on a bounded
    sample of the same workload."""
    from oracle import oracle as O
    O.build()
    o = O.Oracle(wl)
    t0 = time.perf_counter()
    rc = o.step(steps)
    el = time.perf_counter() - t0
    assert rc == 0
    return {"value": round(wl.points * steps / el, 1), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{steps} steps of the {wl.nx}x{wl.ny}x{wl.nz} workload from its initial state "
                      f"({el:.1f} s on 1 host core)",
            "cpu": cpu_model()}


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip() + f", nproc={os.cpu_count()}"
    except Exception:
        pass
    return f"nproc={os.cpu_count()}"


REFERENCE_DIGEST = os.path.join(ROOT, "tests", "golden", "long_{}.npz")


def accuracy(model_cls, wl, torch, device, steps, workload="thunderstorm"):
    """FP32 and FP64 after `steps` steps: relative L2 per field of FP32
    against the GPU FP64 path (whole fields), and of both against the
    reference's own serial FP64 build (the digest of its end state made by
    tests/golden/make_long.py: the random-projection estimate of the whole
    field's relative L2 error), where a digest of this run exists."""
    from model_gb300 import abi, digest
    out = {}
    m64 = model_cls(wl, abi.GA_PREC_F64, device=device)
    m32 = model_cls(wl, abi.GA_PREC_F32, device=device)
    t0 = time.perf_counter()
    m64.step(steps)
    t64 = time.perf_counter() - t0
    m32.step(steps)
    nprog = 7 if wl.microphysics_option else 4
    ends = {"fp32": {}, "fp64": {}}
    for f in range(nprog):
        a, b = m32.get(f), m64.get(f)
        nb = np.linalg.norm(b)
        out[abi.PROG_NAMES[f]] = float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a))
        ends["fp32"][abi.PROG_NAMES[f]], ends["fp64"][abi.PROG_NAMES[f]] = a, b
    ends["fp32"]["pi"], ends["fp64"]["pi"] = m32.get(abi.GA_PI), m64.get(abi.GA_PI)
    m64.close()
    m32.close()
    res = {"steps": steps, "rel_l2_fp32_vs_fp64": {k: float(f"{v:.3e}") for k, v in out.items()},
           "max": float(f"{max(out.values()):.3e}"), "fp64_wall_s": round(t64, 2)}
    path = REFERENCE_DIGEST.format(workload)
    if os.path.exists(path):
        with np.load(path) as z:
            ref = {k: z[k] for k in z.files}
        if int(ref["steps"]) == steps:
            for prec in ("fp32", "fp64"):
                cmp = digest.compare(ends[prec], ref)
                est = {k: float(f"{v['proj']:.3e}") for k, v in cmp.items()}
                res[f"rel_l2_{prec}_vs_reference"] = est
                res[f"max_{prec}_vs_reference"] = max(est.values())
            res["reference"] = ("the reference's serial FP64 build (PARALLEL 0) on the same initial state; "
                                "relative L2 estimated from 64 random +-1 projections of each end-state field")
    return res


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    from model_gb300 import abi, anelastic, configs

    world, rank, local, dist = dist_setup()
    device = local
    torch.cuda.set_device(device)
    wl = configs.make(args.workload)
    prec = abi.GA_PREC_F32 if args.precision == "f32" else abi.GA_PREC_F64
    model = anelastic.Model(wl, prec, device=device)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")
    t_tune = time.perf_counter()
    tuning = model.tune()
    t_tune = time.perf_counter() - t_tune
    # warm-up
    for _ in range(args.warmup):
        model.step(1)
    torch.cuda.synchronize()
    barrier(dist)
    sampler = ClockSampler(device)
    sampler.start()
    time.sleep(0.3)  # nvidia-smi's first samples, before the timed region opens
    l0 = model.launch_count()
    torch.cuda.synchronize()
    barrier(dist)
    per = time_steps(model, torch, args.steps, flush)
    torch.cuda.synchronize()
    barrier(dist)
    clocks = sampler.stop()
    launches = model.launch_count() - l0
    ms_total, value = replica_result(dist, float(sum(per)), world, wl.points, args.steps, f"cuda:{device}")
    rc = model.check_finite()
    if rc != 0:
        raise RuntimeError("non-finite state after the timed steps")

    if rank != 0:
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return
    prec_bytes = 4 if prec == abi.GA_PREC_F32 else 8
    peak, peak_kind = load_peaks()
    groups = profile_groups(model, torch, min(args.steps, 10), flush)
    roof = roofline(groups, wl, prec_bytes, peak, peak_kind, args.workload)
    line = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_total / args.steps, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.precision, "data": DATA,
            "config": {"workload": WORKLOAD_DESC if args.workload == "thunderstorm" else args.workload,
                       "grid": [wl.nx, wl.ny, wl.nz], "precision": args.precision,
                       "physics": "Kessler, rain_fallout 1, 5-point sponges, Rayleigh from NZ-5",
                       "l2": "256 MiB written between timed steps, outside the events",
                       "parallelism": f"replicas x{world}" if world > 1 else "single domain"},
            "roofline": roof, "gpu_launches": int(launches), "clocks": clocks,
            "tuning": {"choice": tuning, "seconds": round(t_tune, 2)}}
    line["hbm_fraction_step"] = round(value / world * STEP_BYTES_FP32_MOIST / 1e9 / peak, 4) \
        if prec == abi.GA_PREC_F32 else None
    if not args.no_fp64 and prec == abi.GA_PREC_F32:
        m64 = anelastic.Model(wl, abi.GA_PREC_F64, device=device)
        m64.tune()
        for _ in range(2):
            m64.step(1)
        per64 = time_steps(m64, torch, args.fp64_steps, flush)
        v64 = wl.points * args.fp64_steps / (sum(per64) * 1e-3)
        line["fp64"] = {"value": round(v64, 1), "unit": UNIT, "steps": args.fp64_steps,
                        "ms_per_step": round(sum(per64) / args.fp64_steps, 4),
                        "fp32_over_fp64": round(value / world / v64, 2)}
        m64.close()
    model.close()
    if args.accuracy_steps > 0:
        line["accuracy"] = accuracy(anelastic.Model, wl, torch, device, args.accuracy_steps, args.workload)
    if args.e2e_jobs > 0:
        line["e2e"] = e2e_jobs(anelastic.Model, wl, prec, torch, args.e2e_jobs, args.e2e_steps, device)
    if args.ensemble_steps > 0:
        line["ensemble"] = ensemble_bench(torch, device, args.ensemble_steps, 2)
    if args.adjoint_steps > 0:
        line["adjoint"] = adjoint_bench(torch, device, args.adjoint_steps, args.adjoint_every)
    if args.adjoint_moist_steps > 0:
        line["adjoint_moist"] = adjoint_bench(torch, device, args.adjoint_moist_steps, args.adjoint_moist_every,
                                              moist=True, size=args.adjoint_moist_size)
    if args.physics_steps > 0:
        line["physics"] = physics_bench(torch, device, args.physics_steps, args.physics_accuracy_steps)
    if args.variant_steps > 0:
        line["variants"] = variants_bench(torch, device, args.variant_steps, args.variant_accuracy_steps)
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(wl, args.cpu_steps)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


_REF_BARRIER = None


def _ref_init(barrier):
    global _REF_BARRIER
    _REF_BARRIER = barrier


def _ref_replica(job):
    """one replica of the reference's serial step: build the state, wait
    for every replica, then time the steps"""
    from model_gb300 import configs
    from oracle import oracle as O
    steps, kw = job
    wl = configs.thunderstorm(**kw)
    o = O.Oracle(wl)
    o.step(1)  # warm-up
    _REF_BARRIER.wait()
    t0 = time.perf_counter()
    rc = o.step(steps)
    return time.perf_counter() - t0, rc


def cpu_all_cores(steps: int, ncores: int = 0, **kw):
    """the reference's CPU step on every host core (or ncores): one replica
    per core in spawned processes, all stepping at once; aggregate
    gridpoint-steps/s = replicas x points x steps / the slowest replica's
    time.  kw: thunderstorm settings (the full workload by default)"""
    import multiprocessing as mp
    from model_gb300 import configs
    from oracle import oracle as O
    O.build()
    n = ncores or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(n)
    with ctx.Pool(n, initializer=_ref_init, initargs=(barrier,)) as pool:
        res = pool.map(_ref_replica, [(steps, kw)] * n)
    assert all(rc == 0 for _, rc in res)
    slow = max(el for el, _ in res)
    wl = configs.thunderstorm(**kw)
    return {"value": round(n * wl.points * steps / slow, 1), "unit": UNIT, "cores": n, "kind": "port",
            "sample": f"{n} replicas (one per host core) of {steps} steps of the {wl.nx}x{wl.ny}x{wl.nz} "
                      f"workload after one warm-up step, stepping at once ({slow:.1f} s for the slowest; "
                      f"{wl.points * steps / slow:.0f} gridpoint-steps/s per core)",
            "slowest_replica_s": slow, "cpu": cpu_model()}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from model_gb300 import configs
    wl = configs.thunderstorm()
    steps = max(1, min(args.steps, args.cpu_steps))
    base = cpu_all_cores(steps)
    line = {"metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": 0, "steps": steps,
            "warmup": args.warmup, "ms_per_step": round(wl.points / base["value"] * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "impl": "reference",
            "config": {"workload": WORKLOAD_DESC, "grid": [wl.nx, wl.ny, wl.nz], "precision": "fp64",
                       "implementation": "CPU restatement of the reference's serial step, bit-identical to "
                                         "the reference build on the golden fixtures; single-threaded like "
                                         "the reference, one replica per host core"},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"])
    ap.add_argument("--workload", default="thunderstorm",
                    choices=["thunderstorm", "dry_bubble", "squall_line", "moist_blob"])
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--accuracy-steps", type=int, default=600)
    ap.add_argument("--e2e-jobs", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=600)
    ap.add_argument("--cpu-steps", type=int, default=5)
    ap.add_argument("--ensemble-steps", type=int, default=10)
    ap.add_argument("--adjoint-steps", type=int, default=500)
    ap.add_argument("--adjoint-every", type=int, default=50)
    ap.add_argument("--adjoint-moist-steps", type=int, default=400)
    ap.add_argument("--adjoint-moist-every", type=int, default=40)
    ap.add_argument("--adjoint-moist-size", type=int, default=512, help="NX = NY of the moist adjoint case")
    ap.add_argument("--physics-steps", type=int, default=20,
                    help="timed steps of each optional-physics variant (0: skip)")
    ap.add_argument("--physics-accuracy-steps", type=int, default=600)
    ap.add_argument("--variant-steps", type=int, default=20,
                    help="timed steps of the linearised and hydrostatic sets (0: skip)")
    ap.add_argument("--variant-accuracy-steps", type=int, default=100)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        log("warning: fewer than 3 warm-up steps")
    if args.impl == "reference":
        run_reference(args)
    else:
        from model_gb300 import build
        build.build()
        run_ours(args)


if __name__ == "__main__":
    main()
