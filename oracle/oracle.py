"""ctypes wrapper of the CPU oracle (liboracle.so) and of the reference build.

TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker or the
timed CPU baseline.  The product path (model_gb300) never imports this file.

  Oracle(workload)          the FP64 restatement (oracle/ga_oracle.c)
  run_reference(...)        the reference's own serial step, built by
                            oracle/build_ref.sh into oracle/_ref/ (only where
                            the reference sources exist)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

from model_gb300 import abi
from oracle.ga_bundle import read_bundle, write_bundle

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")
REF_HARNESS_LIN = os.path.join(HERE, "_ref", "ref_harness_lin")  # the ISLINEAR build
REF_HARNESS_HYD = os.path.join(HERE, "_ref", "ref_harness_hyd")  # the HYDROSTATIC build

_lib = None
_DP = C.POINTER(C.c_double)


def build(quiet: bool = True) -> str:
    subprocess.run(["make", "-C", HERE, "liboracle.so"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.ora_create.argtypes = [C.POINTER(abi.GaConfig), C.POINTER(abi.GaColumns)]
        L.ora_create.restype = C.c_void_p
        L.ora_destroy.argtypes = [C.c_void_p]
        L.ora_set_field.argtypes = [C.c_void_p, C.c_int, C.c_int, _DP, C.c_long]
        L.ora_get_field.argtypes = [C.c_void_p, C.c_int, C.c_int, _DP, C.c_long]
        L.ora_op.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.ora_step.argtypes = [C.c_void_p, C.c_int]
        L.ora_bigcounter.argtypes = [C.c_void_p]
        L.ora_bigcounter.restype = C.c_longlong
        L.ora_set_counters.argtypes = [C.c_void_p, C.c_longlong, C.c_double]
        L.ora_set_counters.restype = None
        L.ora_error.argtypes = [C.c_void_p]
        L.ora_lin_create.argtypes = [C.c_void_p]
        L.ora_lin_create.restype = C.c_void_p
        L.ora_lin_destroy.argtypes = [C.c_void_p]
        L.ora_lin_set.argtypes = [C.c_void_p, C.c_int, C.c_int, _DP, C.c_long]
        L.ora_lin_get.argtypes = [C.c_void_p, C.c_int, C.c_int, _DP, C.c_long]
        L.ora_tlm_step.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.ora_adj_run.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        abi.declare(L, "ora_")
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def build_columns(workload, builder=None) -> dict:
    """Column arrays of `workload` from the oracle's own builder."""
    L = lib()
    store = abi.GaColumnStore()
    tb = np.ascontiguousarray(workload.fields["tb_in"], dtype=np.float64)
    qb = np.ascontiguousarray(workload.fields["qb_in"], dtype=np.float64)
    rc = L.ora_columns_build(workload.nz, workload.dz, workload.height_lowest_level,
                             _ptr(tb), _ptr(qb), C.byref(store))
    if rc != 0:
        raise RuntimeError(f"ora_columns_build failed: {rc}")
    cols = {n: np.array(getattr(store, n)[: workload.nz]) for n in abi.COLUMN_NAMES}
    f = np.zeros(workload.ny)
    L.ora_coriolis_build(workload.ny, workload.dy, workload.corner_lat, _ptr(f))
    cols["f"] = f
    return cols


class Oracle:
    """FP64 CPU restatement of the step, driven like the GPU context."""

    def __init__(self, workload, columns: dict | None = None, init_state: bool = True):
        self.wl = workload
        self.cols = columns if columns is not None else build_columns(workload)
        self._keep = {n: np.ascontiguousarray(v, dtype=np.float64) for n, v in self.cols.items()}
        gc = abi.GaColumns()
        for n in abi.COLUMN_NAMES + ["f"]:
            setattr(gc, n, _ptr(self._keep[n]))
        cfg = abi.make_config(workload.settings())
        self.h = lib().ora_create(C.byref(cfg), C.byref(gc))
        if not self.h:
            raise RuntimeError("ora_create failed")
        self.n3 = workload.points
        if init_state:
            self.load_initial_state(workload.fields)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().ora_destroy(h)
            self.h = None

    def set(self, field: int, slot: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        rc = lib().ora_set_field(self.h, field, slot, _ptr(a), a.size)
        if rc != 0:
            raise RuntimeError(f"ora_set_field({field},{slot}) -> {rc}")

    def get(self, field: int, slot: int = 0) -> np.ndarray:
        n = self.wl.nx * self.wl.ny if field in (abi.GA_ACCRAIN, abi.GA_ACCSNOW) else \
            1 if field == abi.GA_N0S else self.n3
        a = np.zeros(n)
        rc = lib().ora_get_field(self.h, field, slot, _ptr(a), n)
        if rc != 0:
            raise RuntimeError(f"ora_get_field({field},{slot}) -> {rc}")
        return a

    def load_initial_state(self, fields: dict) -> None:
        """Initial state as the reference's initialize_from_output_serial
        leaves it: current = M = the given perturbation, P = 0."""
        for b, name in enumerate(abi.BAR_NAMES):
            self.set(abi.GA_UBAR + b, 0, fields[name])
        nprog = 7 if self.wl.microphysics_option else 4
        for f in range(nprog):
            arr = fields[abi.PROG_NAMES[f]]
            self.set(f, abi.GA_SLOT_CUR, arr)
            self.set(f, abi.GA_SLOT_M, arr)
        if "accrain" in fields:
            self.set(abi.GA_ACCRAIN, 0, fields["accrain"])
        if self.wl.microphysics_option == 2:
            for name, fid in abi.ICE_PROG.items():
                self.set(fid, abi.GA_SLOT_CUR, fields[name])
                self.set(fid, abi.GA_SLOT_M, fields[name])
            if "accsnow" in fields:
                self.set(abi.GA_ACCSNOW, 0, fields["accsnow"])

    def step(self, n: int = 1) -> int:
        return lib().ora_step(self.h, n)

    def set_counters(self, bigcounter: int, mtime: float) -> None:
        lib().ora_set_counters(self.h, bigcounter, mtime)

    def op(self, name: str, step: float = 1.0) -> int:
        return lib().ora_op(self.h, abi.OPS[name], step)

    def state(self) -> dict:
        """All fields, keyed like the reference harness' dump."""
        out = {}
        for f, name in enumerate(abi.PROG_NAMES):
            for slot, suf in abi.SLOT_SUFFIX.items():
                out[name + suf] = self.get(f, slot)
        out["pi"] = self.get(abi.GA_PI)
        out["vt"] = self.get(abi.GA_VT)
        out["accrain"] = self.get(abi.GA_ACCRAIN)
        if self.wl.microphysics_option == 2:
            for name, fid in abi.ICE_PROG.items():
                for slot, suf in abi.SLOT_SUFFIX.items():
                    out[name + suf] = self.get(fid, slot)
            for name, fid in abi.ICE_NAMES.items():
                out[name] = self.get(fid)
        return out


LIN_FIELDS = (abi.GA_U, abi.GA_V, abi.GA_W, abi.GA_TH)
LIN_SLOTS = (abi.GA_SLOT_CUR, abi.GA_SLOT_P, abi.GA_SLOT_M)


class OracleLin:
    """Perturbation or adjoint buffers of an Oracle's dry state (current, P,
    M of u, v, w, theta, and pi), rotating with it (ga_oracle_lin.c)."""

    def __init__(self, oracle: Oracle):
        self.o = oracle
        self.h = lib().ora_lin_create(oracle.h)
        if not self.h:
            raise RuntimeError("ora_lin_create failed (dry, non-periodic only)")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().ora_lin_destroy(h)
            self.h = None

    def set(self, field: int, slot: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        if lib().ora_lin_set(self.h, field, slot, _ptr(a), a.size) != 0:
            raise RuntimeError("ora_lin_set")

    def get(self, field: int, slot: int = 0) -> np.ndarray:
        a = np.zeros(self.o.n3)
        if lib().ora_lin_get(self.h, field, slot, _ptr(a), a.size) != 0:
            raise RuntimeError("ora_lin_get")
        return a

    def set_all(self, d: dict) -> None:
        """d maps (field, slot) -> array; (GA_PI, 0) for pi."""
        for (f, s), v in d.items():
            self.set(f, s, v)

    def get_all(self) -> dict:
        d = {(f, s): self.get(f, s) for f in LIN_FIELDS for s in LIN_SLOTS}
        d[(abi.GA_PI, 0)] = self.get(abi.GA_PI)
        return d

    def tlm(self, nsteps: int) -> None:
        """Advance the oracle's state and these perturbations together."""
        rc = lib().ora_tlm_step(self.o.h, self.h, nsteps)
        if rc != 0:
            raise RuntimeError(f"ora_tlm_step -> {rc}")

    def adjoint(self, nsteps: int) -> None:
        """Advance the oracle's state nsteps; map the adjoint of the final state
        held here to the adjoint of the initial state."""
        rc = lib().ora_adj_run(self.o.h, self.h, nsteps)
        if rc != 0:
            raise RuntimeError(f"ora_adj_run -> {rc}")


# ---------------------------------------------------------------------------
# the reference's own serial step (oracle/_ref/ref_harness)
# ---------------------------------------------------------------------------
def reference_available() -> bool:
    return os.path.exists(REF_HARNESS)


def workload_bundle(workload, extra: dict | None = None) -> dict:
    b = {k: np.array([float(v)]) for k, v in workload.settings().items()}
    for k, v in workload.fields.items():
        b[k] = np.asarray(v, dtype=np.float64).ravel()
    if extra:
        for k, v in extra.items():
            b[k] = np.asarray(v, dtype=np.float64).ravel()
    return b


def run_reference(workload, mode: str = "run", nsteps: int = 1, op: str = "", step: float = 1.0,
                  extra: dict | None = None) -> dict:
    """Run the reference harness on `workload` and return its dump."""
    if not reference_available():
        raise RuntimeError("reference build missing: run oracle/build_ref.sh")
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_bundle(fin, workload_bundle(workload, extra))
        exe = REF_HARNESS_LIN if getattr(workload, "linear_model", 0) else \
            REF_HARNESS_HYD if getattr(workload, "hydrostatic", 0) else REF_HARNESS
        args = [exe, fin, fout, mode]
        args += [str(nsteps)] if mode == "run" else [op, repr(step)]
        subprocess.run(args, check=True, stdout=subprocess.DEVNULL)
        return read_bundle(fout)
