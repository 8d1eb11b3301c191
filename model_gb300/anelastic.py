"""Python host mirror of the C ABI in include/ga_anelastic.h.

The reference drives its step through global C++ functions on global arrays
(s_integrate_rk3, driver_serial.cpp:178; integrate_non_hydro, solver.cpp:87;
solve_pressure, pressure.cpp:142; ...).  `Model` exposes the same operations
on a GPU context: `step(n)` is n calls of s_integrate_rk3 plus the counter
updates of s_run_model, and the methods named after the reference functions
run one operator each, so parity tests read like calls into the reference.

There is no CPU fallback: if libga_anelastic.so is missing or no CUDA device
is present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libga_anelastic.so")
_DP = C.POINTER(C.c_double)
_lib = None


class GaError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what} failed with code {code}: {last_error()}")
        self.code = code


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load the in-tree CUDA library (built by model_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library {path} is missing: run model_gb300/build.py "
                           "(there is no CPU fallback)")
    L = C.CDLL(path)
    L.ga_abi_version.restype = C.c_int
    L.ga_last_error.restype = C.c_char_p
    abi.declare(L, "ga_")
    L.ga_create.argtypes = [C.POINTER(abi.GaConfig), C.POINTER(abi.GaColumns), C.POINTER(C.c_void_p)]
    L.ga_destroy.argtypes = [C.c_void_p]
    L.ga_set_field.argtypes = [C.c_void_p, C.c_int, C.c_int, _DP, C.c_size_t]
    L.ga_get_field.argtypes = [C.c_void_p, C.c_int, C.c_int, _DP, C.c_size_t]
    L.ga_step.argtypes = [C.c_void_p, C.c_int]
    L.ga_step_async.argtypes = [C.c_void_p, C.c_int]
    L.ga_synchronize.argtypes = [C.c_void_p]
    L.ga_op.argtypes = [C.c_void_p, C.c_int, C.c_double]
    L.ga_get_counters.argtypes = [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_double)]
    L.ga_set_counters.argtypes = [C.c_void_p, C.c_longlong, C.c_double]
    L.ga_budget.argtypes = [C.c_void_p, C.c_int, _DP, C.c_int]
    L.ga_check_finite.argtypes = [C.c_void_p]
    L.ga_launch_count.argtypes = [C.c_void_p]
    L.ga_launch_count.restype = C.c_longlong
    L.ga_stream.argtypes = [C.c_void_p]
    L.ga_stream.restype = C.c_void_p
    L.ga_field_device_ptr.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.ga_field_device_ptr.restype = C.c_void_p
    L.ga_ensemble_tune.argtypes = [C.c_void_p]
    L.ga_ensemble_tuning.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    L.ga_tune.argtypes = [C.c_void_p]
    L.ga_tuning.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    L.ga_lin_set_field.argtypes = [C.c_void_p, C.c_int, C.c_int, _DP, C.c_size_t]
    L.ga_lin_get_field.argtypes = [C.c_void_p, C.c_int, C.c_int, _DP, C.c_size_t]
    L.ga_tlm_step.argtypes = [C.c_void_p, C.c_int]
    L.ga_adjoint.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.ga_ensemble_create.argtypes = [C.POINTER(abi.GaConfig), C.POINTER(abi.GaColumns), C.c_int,
                                     C.POINTER(C.c_void_p)]
    L.ga_ensemble_destroy.argtypes = [C.c_void_p]
    L.ga_ensemble_size.argtypes = [C.c_void_p]
    L.ga_ensemble_set_field.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _DP, C.c_size_t]
    L.ga_ensemble_get_field.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _DP, C.c_size_t]
    L.ga_ensemble_step.argtypes = [C.c_void_p, C.c_int]
    L.ga_ensemble_step_async.argtypes = [C.c_void_p, C.c_int]
    L.ga_ensemble_synchronize.argtypes = [C.c_void_p]
    L.ga_ensemble_stream.argtypes = [C.c_void_p]
    L.ga_ensemble_stream.restype = C.c_void_p
    L.ga_ensemble_launch_count.argtypes = [C.c_void_p]
    L.ga_ensemble_launch_count.restype = C.c_longlong
    L.ga_ensemble_get_counters.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_double)]
    if L.ga_abi_version() != 1:
        raise RuntimeError("ABI version mismatch")
    _lib = L
    return L


def last_error() -> str:
    if _lib is None:
        return ""
    return (_lib.ga_last_error() or b"").decode(errors="replace")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def build_columns(workload) -> dict:
    """Vertical columns and Coriolis parameter of `workload` (host only):
    ga_columns_build + ga_coriolis_build."""
    L = load_library()
    store = abi.GaColumnStore()
    tb = np.ascontiguousarray(workload.fields["tb_in"], dtype=np.float64)
    qb = np.ascontiguousarray(workload.fields["qb_in"], dtype=np.float64)
    rc = L.ga_columns_build(workload.nz, workload.dz, workload.height_lowest_level, _ptr(tb), _ptr(qb),
                            C.byref(store))
    if rc:
        raise GaError(rc, "ga_columns_build")
    cols = {n: np.array(getattr(store, n)[: workload.nz]) for n in abi.COLUMN_NAMES}
    f = np.zeros(workload.ny)
    rc = L.ga_coriolis_build(workload.ny, workload.dy, workload.corner_lat, _ptr(f))
    if rc:
        raise GaError(rc, "ga_coriolis_build")
    cols["f"] = f
    return cols


class Model:
    """One GPU context: the anelastic step of one domain."""

    def __init__(self, workload, precision: int = abi.GA_PREC_F64, device: int = 0,
                 columns: dict | None = None, init_state: bool = True):
        self.L = load_library()
        self.wl = workload
        self.precision = precision
        self.cols = columns if columns is not None else build_columns(workload)
        self._keep = {n: np.ascontiguousarray(v, dtype=np.float64) for n, v in self.cols.items()}
        gc = abi.GaColumns()
        for n in abi.COLUMN_NAMES + ["f"]:
            setattr(gc, n, _ptr(self._keep[n]))
        cfg = abi.make_config(workload.settings(), precision, device)
        h = C.c_void_p()
        rc = self.L.ga_create(C.byref(cfg), C.byref(gc), C.byref(h))
        if rc:
            raise GaError(rc, "ga_create")
        self.h = h
        self.n3 = workload.points
        if init_state:
            self.load_initial_state(workload.fields)

    def close(self):
        if getattr(self, "h", None):
            self.L.ga_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc:
            raise GaError(rc, what)

    # ---- fields ---------------------------------------------------------
    def set(self, field: int, slot: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        self._check(self.L.ga_set_field(self.h, field, slot, _ptr(a), a.size), "ga_set_field")

    def get(self, field: int, slot: int = 0) -> np.ndarray:
        n = self.wl.nx * self.wl.ny if field in (abi.GA_ACCRAIN, abi.GA_ACCSNOW) else \
            1 if field == abi.GA_N0S else self.n3
        a = np.zeros(n)
        self._check(self.L.ga_get_field(self.h, field, slot, _ptr(a), n), "ga_get_field")
        return a

    def load_initial_state(self, fields: dict) -> None:
        """current = M = the given perturbation, P = 0, as the reference's
        initialize_from_output_serial (initializer.cpp:1918-1935)."""
        for b, name in enumerate(abi.BAR_NAMES):
            self.set(abi.GA_UBAR + b, 0, fields[name])
        nprog = 7 if self.wl.microphysics_option else 4
        for f in range(nprog):
            arr = fields[abi.PROG_NAMES[f]]
            self.set(f, abi.GA_SLOT_CUR, arr)
            self.set(f, abi.GA_SLOT_M, arr)
        if "accrain" in fields:
            self.set(abi.GA_ACCRAIN, 0, fields["accrain"])
        if self.wl.microphysics_option == 2:  # snow and cloud ice (initializer.cpp:1920-1926)
            for name, fid in abi.ICE_PROG.items():
                self.set(fid, abi.GA_SLOT_CUR, fields[name])
                self.set(fid, abi.GA_SLOT_M, fields[name])
            if "accsnow" in fields:
                self.set(abi.GA_ACCSNOW, 0, fields["accsnow"])

    def state(self) -> dict:
        out = {}
        nprog = 7 if self.wl.microphysics_option else 4
        for f in range(nprog):
            for slot, suf in abi.SLOT_SUFFIX.items():
                out[abi.PROG_NAMES[f] + suf] = self.get(f, slot)
        out["pi"] = self.get(abi.GA_PI)
        if self.wl.microphysics_option:
            out["vt"] = self.get(abi.GA_VT)
            out["accrain"] = self.get(abi.GA_ACCRAIN)
        if self.wl.microphysics_option == 2:
            for name, fid in abi.ICE_PROG.items():
                for slot, suf in abi.SLOT_SUFFIX.items():
                    out[name + suf] = self.get(fid, slot)
            for name, fid in abi.ICE_NAMES.items():
                out[name] = self.get(fid)
        return out

    # ---- stepping -------------------------------------------------------
    def step(self, n: int = 1) -> None:
        """n x s_integrate_rk3 (driver_serial.cpp:178-286)."""
        self._check(self.L.ga_step(self.h, n), "ga_step")

    def step_async(self, n: int = 1) -> None:
        self._check(self.L.ga_step_async(self.h, n), "ga_step_async")

    def synchronize(self) -> None:
        self._check(self.L.ga_synchronize(self.h), "ga_synchronize")

    def op(self, name: str, step: float = 1.0) -> None:
        self._check(self.L.ga_op(self.h, abi.OPS[name], step), f"ga_op({name})")

    # reference-named single operators
    def integrate_non_hydro(self, step):  # solver.cpp:87
        self.op("integrate_non_hydro", step)

    def advect_uvw_velocity(self, step):  # advection.cpp:304
        self.op("advect_uvw", step)

    def solve_pressure(self, step):  # pressure.cpp:142
        self.op("solve_pressure", step)

    def advect_theta(self, step):  # advection.cpp:349
        self.op("advect_theta", step)

    def advect_microphysics_cell(self, step):  # advection.cpp:451
        self.op("advect_micro", step)

    def zero_moisture(self):  # microphysics.cpp:675
        self.op("zero_moisture")

    def apply_boundary_condition(self):  # boundaries.cpp:119
        self.op("bc")

    def apply_boundary_condition_microphysics(self):  # boundaries.cpp:200
        self.op("bc_micro")

    def run_microphysics(self):  # microphysics.cpp:97 (Kessler or the ice scheme)
        self.op("kessler")

    def advect_ice_cell(self, step):  # advection.cpp:508
        self.op("advect_ice", step)

    def rayleigh_damping(self):  # damping.cpp:1148
        self.op("rayleigh")

    def apply_explicit_diffusion(self, step=1.0):  # damping.cpp:1125
        self.op("explicit_diffusion", step)

    def calculate_diff_tend(self):  # turbulence.cpp:158
        self.op("turbulence")

    def counters(self):
        bc, mt = C.c_longlong(), C.c_double()
        self._check(self.L.ga_get_counters(self.h, C.byref(bc), C.byref(mt)), "ga_get_counters")
        return bc.value, mt.value

    def set_counters(self, bigcounter: int, mtime: float) -> None:
        self._check(self.L.ga_set_counters(self.h, bigcounter, mtime), "ga_set_counters")

    def budget(self, slot: int = abi.GA_SLOT_CUR) -> dict:
        """FP64 domain budgets of one rotation slot (ga_budget), by name."""
        out = (C.c_double * abi.GA_NBUDGET)()
        self._check(self.L.ga_budget(self.h, slot, out, abi.GA_NBUDGET), "ga_budget")
        return {n: out[b] for b, n in enumerate(abi.BUDGET_NAMES)}

    def check_finite(self) -> int:
        return self.L.ga_check_finite(self.h)

    def launch_count(self) -> int:
        return self.L.ga_launch_count(self.h)

    def stream_handle(self) -> int:
        return self.L.ga_stream(self.h) or 0

    def device_ptr(self, field: int, slot: int = 0) -> int:
        return self.L.ga_field_device_ptr(self.h, field, slot) or 0

    # ---- autotuner -------------------------------------------------------
    def tune(self) -> str:
        """Time the candidate tile shapes and FFT plans, keep the fastest."""
        self._check(self.L.ga_tune(self.h), "ga_tune")
        return self.tuning()

    def tuning(self) -> str:
        buf = C.create_string_buffer(512)
        self._check(self.L.ga_tuning(self.h, buf, 512), "ga_tuning")
        return buf.value.decode()

    # ---- tangent-linear model and adjoint (dry, non-periodic) -------------
    LIN_FIELDS = (abi.GA_U, abi.GA_V, abi.GA_W, abi.GA_TH)
    LIN_SLOTS = (abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M)

    def lin_set(self, field: int, slot: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        self._check(self.L.ga_lin_set_field(self.h, field, slot, _ptr(a), a.size), "ga_lin_set_field")

    def lin_get(self, field: int, slot: int = 0) -> np.ndarray:
        a = np.zeros(self.n3)
        self._check(self.L.ga_lin_get_field(self.h, field, slot, _ptr(a), self.n3), "ga_lin_get_field")
        return a

    def lin_set_all(self, d: dict) -> None:
        """d maps (field, slot) -> array; (GA_PI, 0) for pi."""
        for (f, s), v in d.items():
            self.lin_set(f, s, v)

    def lin_fields(self):
        """The linearised prognostic fields of this context."""
        return tuple(range(7)) if self.wl.microphysics_option else self.LIN_FIELDS

    def lin_get_all(self) -> dict:
        d = {(f, s): self.lin_get(f, s) for f in self.lin_fields() for s in self.LIN_SLOTS}
        d[(abi.GA_PI, 0)] = self.lin_get(abi.GA_PI)
        return d

    def tlm_step(self, n: int = 1) -> None:
        """Advance the state and the perturbation buffers together."""
        self._check(self.L.ga_tlm_step(self.h, n), "ga_tlm_step")

    def adjoint(self, n: int, checkpoint_every: int = 0) -> None:
        """Advance the state n steps, then map the adjoint of the final state
        held in the perturbation buffers to that of the initial state."""
        self._check(self.L.ga_adjoint(self.h, n, checkpoint_every), "ga_adjoint")


class Ensemble:
    """Independent domains of uneven sizes advanced together by batched
    kernels (one launch per kernel phase over all members).  The reference
    farms such members out as separate serial runs (ensemble.cpp:45-144)."""

    def __init__(self, members, precision: int = abi.GA_PREC_F32, device: int = 0, columns=None):
        """members: list of Workload (their fields may be empty; load them
        later with load_member).  columns: optional list of column dicts."""
        self.L = load_library()
        self.members = list(members)
        n = len(self.members)
        self.cols = columns if columns is not None else [build_columns(w) for w in self.members]
        self._keep = []
        cfgs = (abi.GaConfig * n)()
        gcs = (abi.GaColumns * n)()
        for m, (wl, cols) in enumerate(zip(self.members, self.cols)):
            keep = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in cols.items()}
            self._keep.append(keep)
            cfgs[m] = abi.make_config(wl.settings(), precision, device)
            for name in abi.COLUMN_NAMES + ["f"]:
                setattr(gcs[m], name, _ptr(keep[name]))
        h = C.c_void_p()
        rc = self.L.ga_ensemble_create(cfgs, gcs, n, C.byref(h))
        if rc:
            raise GaError(rc, "ga_ensemble_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.ga_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, member: int, field: int, slot: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        rc = self.L.ga_ensemble_set_field(self.h, member, field, slot, _ptr(a), a.size)
        if rc:
            raise GaError(rc, "ga_ensemble_set_field")

    def get(self, member: int, field: int, slot: int = 0) -> np.ndarray:
        wl = self.members[member]
        n = wl.nx * wl.ny if field == abi.GA_ACCRAIN else wl.points
        a = np.zeros(n)
        rc = self.L.ga_ensemble_get_field(self.h, member, field, slot, _ptr(a), n)
        if rc:
            raise GaError(rc, "ga_ensemble_get_field")
        return a

    def load_member(self, member: int, fields: dict) -> None:
        for b, name in enumerate(abi.BAR_NAMES):
            self.set(member, abi.GA_UBAR + b, 0, fields[name])
        nprog = 7 if self.members[member].microphysics_option else 4
        for f in range(nprog):
            arr = fields[abi.PROG_NAMES[f]]
            self.set(member, f, abi.GA_SLOT_CUR, arr)
            self.set(member, f, abi.GA_SLOT_M, arr)

    def step(self, n: int = 1) -> None:
        rc = self.L.ga_ensemble_step(self.h, n)
        if rc:
            raise GaError(rc, "ga_ensemble_step")

    def step_async(self, n: int = 1) -> None:
        rc = self.L.ga_ensemble_step_async(self.h, n)
        if rc:
            raise GaError(rc, "ga_ensemble_step_async")

    def synchronize(self) -> None:
        rc = self.L.ga_ensemble_synchronize(self.h)
        if rc:
            raise GaError(rc, "ga_ensemble_synchronize")

    def stream_handle(self) -> int:
        return self.L.ga_ensemble_stream(self.h) or 0

    def launch_count(self) -> int:
        return self.L.ga_ensemble_launch_count(self.h)

    def tune(self) -> str:
        """Time the batched kernels' tile candidates over all members, keep the fastest."""
        rc = self.L.ga_ensemble_tune(self.h)
        if rc:
            raise GaError(rc, "ga_ensemble_tune")
        buf = C.create_string_buffer(512)
        rc = self.L.ga_ensemble_tuning(self.h, buf, 512)
        if rc:
            raise GaError(rc, "ga_ensemble_tuning")
        return buf.value.decode()

    def counters(self, member: int):
        bc, mt = C.c_longlong(), C.c_double()
        rc = self.L.ga_ensemble_get_counters(self.h, member, C.byref(bc), C.byref(mt))
        if rc:
            raise GaError(rc, "ga_ensemble_get_counters")
        return bc.value, mt.value
