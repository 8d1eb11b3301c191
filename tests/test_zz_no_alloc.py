"""The allocation-free pressure solve against the reference and the context path.

ga_solve_pressure_noalloc exists for callers that cannot allocate device
memory: a host model that hands out all GPU memory from its own pool, or a
plugin whose host process forbids foreign cudaMalloc calls.  It keeps its
scratch in a fixed file-scope device array.  Here it runs twice in a row on
caller-owned device arrays and must agree, within the tolerance the parity
tests use for the pressure solve (1e-12 relative L2):
  - with the reference's own solve_pressure outputs (the golden ops_*
    fixtures, made by the reference's serial build);
  - with the context entry point (ga_op GA_OP_SOLVE_PRESSURE), which shares
    every kernel; only the twiddle and wavenumber tables are formed on the
    device here instead of on the host.
A call must also leave the device's free memory unchanged, and grids beyond
the scratch array or the transforms' shared memory are rejected.

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from model_gb300 import abi, anelastic, configs
from tests import fixtures as fx

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def lib():
    from model_gb300 import build
    build.build()
    L = anelastic.load_library()
    L.ga_solve_pressure_noalloc.argtypes = [C.POINTER(abi.GaConfig), C.POINTER(abi.GaColumns), C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    L.ga_solve_pressure_noalloc.restype = C.c_int
    return L


def _columns_struct(cols):
    keep = {n: np.ascontiguousarray(v, dtype=np.float64) for n, v in cols.items()}
    gc = abi.GaColumns()
    for n in abi.COLUMN_NAMES + ["f"]:
        setattr(gc, n, keep[n].ctypes.data_as(C.POINTER(C.c_double)))
    return gc, keep


def _inputs(wl, seed):
    n3 = (wl.nx, wl.ny, wl.nz)
    r = [2.0 * configs.splitmix_uniform(seed + s, wl.points).reshape(n3) - 1.0 for s in range(3)]
    return 3.0 * r[0], 3.0 * r[1], 0.5 * r[2]


def _context_solve(wl, cols, up, vp, wp, step):
    m = anelastic.Model(wl, abi.GA_PREC_F64, columns=cols, init_state=False)
    m.set(abi.GA_U, abi.GA_SLOT_P, up)
    m.set(abi.GA_V, abi.GA_SLOT_P, vp)
    m.set(abi.GA_W, abi.GA_SLOT_P, wp)
    m.solve_pressure(step)
    out = (m.get(abi.GA_PI), m.get(abi.GA_U, abi.GA_SLOT_P), m.get(abi.GA_V, abi.GA_SLOT_P),
           m.get(abi.GA_W, abi.GA_SLOT_P))
    m.close()
    return out


@pytest.mark.parametrize("periodic", [0, 1])
def test_noalloc_matches_context_twice(lib, periodic):
    torch = pytest.importorskip("torch")
    wl = configs.moist_blob(nx=40, ny=36, nz=24, periodic=periodic)
    cols = anelastic.build_columns(wl)
    gc, keep = _columns_struct(cols)
    cfg = abi.make_config(wl.settings(), abi.GA_PREC_F64, 0)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    for call, (seed, step) in enumerate([(7000, 0.5), (7100, 1.0 / 3.0)]):
        up, vp, wp = _inputs(wl, seed)
        ref = _context_solve(wl, cols, up, vp, wp, step)
        d = [torch.tensor(a.ravel(), dtype=torch.float64, device=dev) for a in (up, vp, wp)]
        pi = torch.full((wl.points,), float("nan"), dtype=torch.float64, device=dev)
        rc = lib.ga_solve_pressure_noalloc(C.byref(cfg), C.byref(gc), d[0].data_ptr(), d[1].data_ptr(),
                                           d[2].data_ptr(), pi.data_ptr(), step, stream.cuda_stream)
        assert rc == 0, anelastic.last_error()
        torch.cuda.synchronize(dev)
        got = (pi.cpu().numpy(), d[0].cpu().numpy(), d[1].cpu().numpy(), d[2].cpu().numpy())
        for name, g, r in zip(("pi", "up", "vp", "wp"), got, ref):
            e = fx.rel_l2(g, r)
            assert np.all(np.isfinite(g)), f"call {call}: {name} has non-finite values"
            assert e <= TOL, f"call {call}: {name} rel L2 {e:.3e}"


def _call(lib, wl, cols, up, vp, wp, step, torch, dev):
    gc, keep = _columns_struct(cols)
    cfg = abi.make_config(wl.settings(), abi.GA_PREC_F64, 0)
    d = [torch.tensor(np.asarray(a).ravel(), dtype=torch.float64, device=dev) for a in (up, vp, wp)]
    pi = torch.full((wl.points,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.ga_solve_pressure_noalloc(C.byref(cfg), C.byref(gc), d[0].data_ptr(), d[1].data_ptr(),
                                       d[2].data_ptr(), pi.data_ptr(), step, stream.cuda_stream)
    assert rc == 0, anelastic.last_error()
    torch.cuda.synchronize(dev)
    return pi, d


@pytest.mark.parametrize("name", fx.ops_names())
def test_noalloc_matches_reference_solve_pressure_twice(lib, name):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    d = fx.load(name)
    wl = fx.workload(d)
    cols = anelastic.build_columns(wl)
    step = float(d["step_solve_pressure"])
    for call in range(2):
        pi, out = _call(lib, wl, cols, d["in_u_p"], d["in_v_p"], d["in_w_p"], step, torch, dev)
        got = {"pi": pi, "u_p": out[0], "v_p": out[1], "w_p": out[2]}
        for key, g in got.items():
            g = g.cpu().numpy()
            assert np.all(np.isfinite(g)), f"{name} call {call}: {key} has non-finite values"
            e = fx.rel_l2(g, d["solve_pressure__" + key])
            assert e <= TOL, f"{name} call {call}: {key} rel L2 {e:.3e}"


def test_noalloc_leaves_free_device_memory_unchanged(lib):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    wl = configs.moist_blob(nx=40, ny=36, nz=24)
    cols = anelastic.build_columns(wl)
    up, vp, wp = _inputs(wl, 7200)
    _call(lib, wl, cols, up, vp, wp, 0.5, torch, dev)  # first call: once-per-device set-up
    gc, keep = _columns_struct(cols)
    cfg = abi.make_config(wl.settings(), abi.GA_PREC_F64, 0)
    d = [torch.tensor(a.ravel(), dtype=torch.float64, device=dev) for a in (up, vp, wp)]
    pi = torch.zeros(wl.points, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    free_before = torch.cuda.mem_get_info(dev)[0]
    rc = lib.ga_solve_pressure_noalloc(C.byref(cfg), C.byref(gc), d[0].data_ptr(), d[1].data_ptr(),
                                       d[2].data_ptr(), pi.data_ptr(), 0.5, stream.cuda_stream)
    torch.cuda.synchronize(dev)
    free_after = torch.cuda.mem_get_info(dev)[0]
    assert rc == 0, anelastic.last_error()
    assert free_after == free_before, f"free device memory changed by {free_before - free_after} bytes"


def test_noalloc_rejects_grids_beyond_the_shared_memory(lib):
    # 12 x 6500 x 6 fits the scratch array (7.5 MB) but one y line of the
    # transform needs 2 * 6500 * 16 bytes of shared memory, above 200 KiB
    wl = configs.Workload("long_y", 12, 6500, 6, 1000.0, 1000.0, 500.0, 4.0, 1, boundary_width_north=3,
                          boundary_width_south=3, boundary_width_east=3, boundary_width_west=3)
    cfg = abi.make_config(wl.settings(), abi.GA_PREC_F64, 0)
    cols = {n: np.ones(wl.nz) for n in abi.COLUMN_NAMES}
    cols["f"] = np.zeros(wl.ny)
    gc, keep = _columns_struct(cols)
    rc = lib.ga_solve_pressure_noalloc(C.byref(cfg), C.byref(gc), 1, 1, 1, 1, 0.5, None)
    assert rc == abi.GA_ERR_ARG
    assert "shared memory" in anelastic.last_error()


def test_noalloc_rejects_grids_beyond_the_scratch(lib):
    wl = configs.moist_blob(nx=512, ny=512, nz=64)
    cfg = abi.make_config(wl.settings(), abi.GA_PREC_F64, 0)
    cols = {n: np.ones(wl.nz) for n in abi.COLUMN_NAMES}
    cols["f"] = np.zeros(wl.ny)
    gc, keep = _columns_struct(cols)
    rc = lib.ga_solve_pressure_noalloc(C.byref(cfg), C.byref(gc), 1, 1, 1, 1, 0.5, None)
    assert rc == abi.GA_ERR_ARG
    assert "scratch" in anelastic.last_error()
