"""ctypes mirror of include/ga_anelastic.h (constants, structs, signatures).

Shared by the product wrapper (model_gb300.anelastic) and the oracle wrapper
used by the tests, so both read the same ga_config / ga_columns layout.
"""
from __future__ import annotations

import ctypes as C

GA_OK = 0
GA_ERR_ARG = -1
GA_ERR_CUDA = -2
GA_ERR_NOMEM = -3
GA_ERR_CONFIG = -4
GA_ERR_NONFINITE = -5
GA_ERR_KESSLER = -6
GA_ERR_UNSUPPORTED = -7

GA_PREC_F64 = 0
GA_PREC_F32 = 1

GA_U, GA_V, GA_W, GA_TH, GA_QV, GA_QC, GA_QR = range(7)
GA_NPROG = 7
GA_PI, GA_UBAR, GA_VBAR, GA_WBAR, GA_THBAR, GA_QBAR, GA_PBAR, GA_VT = range(7, 15)
GA_NFIELDS = 15
GA_ACCRAIN = 15
# turbulence diagnostics (contexts with turbulence_option set)
GA_KMIX, GA_KHMIX, GA_UFRIC, GA_VFRIC, GA_WFRIC, GA_THDIFF, GA_QVDIFF, GA_QCDIFF, GA_QRDIFF, GA_SATURATED = \
    range(16, 26)
# bundle names of the turbulence diagnostics (turbulence.cpp:23-31)
TURB_NAMES = {"kmix": GA_KMIX, "khmix": GA_KHMIX, "u_friction": GA_UFRIC, "v_friction": GA_VFRIC,
              "w_friction": GA_WFRIC, "t_diffusion": GA_THDIFF, "qv_diffusion": GA_QVDIFF,
              "qc_diffusion": GA_QCDIFF, "qr_diffusion": GA_QRDIFF, "is_saturated": GA_SATURATED}

# ice microphysics (microphysics_option 2): snow and cloud ice with three
# rotation slots each, their fall speeds, accumulated snow, the snow intercept
GA_QS, GA_QI, GA_VTS, GA_VTI, GA_ACCSNOW, GA_N0S = range(26, 32)
# bundle names of the ice fields (microphysics.h:18-25, rutledge.cpp:90)
ICE_PROG = {"qs": GA_QS, "qi": GA_QI}
ICE_NAMES = {"sts": GA_VTS, "its": GA_VTI, "accsnow": GA_ACCSNOW, "n0s": GA_N0S}

GA_SLOT_CUR, GA_SLOT_P, GA_SLOT_M = 0, 1, 2

OPS = {
    "sign_cells": 0, "advect_uvw": 1, "solve_pressure": 2, "project": 3,
    "integrate_non_hydro": 4, "advect_theta": 5, "advect_micro": 6, "zero_moisture": 7,
    "bc": 8, "bc_micro": 9, "kessler": 10, "rayleigh": 11, "advance_inner": 12,
    "advance_outer": 13, "explicit_diffusion": 14, "turbulence": 15, "advect_ice": 16,
}

# names used in bundles / fixtures
PROG_NAMES = ["u", "v", "w", "th", "qv", "qc", "qr"]
BAR_NAMES = ["ubar", "vbar", "wbar", "thbar", "qbar", "pbar"]
SLOT_SUFFIX = {GA_SLOT_CUR: "", GA_SLOT_P: "_p", GA_SLOT_M: "_m"}
# ga_budget entries (GA_BUDGET_*)
BUDGET_NAMES = ["theta", "qv", "qc", "qr", "water", "ke", "rain", "mass", "qi", "qs", "snow"]
GA_NBUDGET = len(BUDGET_NAMES)
COLUMN_NAMES = ["zu", "zw", "zsu", "zsw", "mu", "mw", "rhou", "rhow", "one_d_rhou",
                "one_d_rhow", "tb", "tbv", "tbw", "qb", "pib"]

_DP = C.POINTER(C.c_double)


class GaConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
        ("microphysics_option", C.c_int), ("rain_fallout", C.c_int),
        ("periodic_ew_boundaries", C.c_int),
        ("boundary_width_north", C.c_int), ("boundary_width_south", C.c_int),
        ("boundary_width_east", C.c_int), ("boundary_width_west", C.c_int),
        ("rayleigh_damping_z", C.c_int), ("precision", C.c_int), ("device", C.c_int),
        ("use_explicit_diffusion", C.c_int), ("diffusion_order", C.c_int),
        ("kdiffh", C.c_double), ("kdiffv", C.c_double),
        ("turbulence_option", C.c_int), ("use_surface_heat_flux", C.c_int), ("water_temp", C.c_double),
        ("linear_model", C.c_int), ("hydrostatic", C.c_int),
    ]


class GaColumns(C.Structure):
    _fields_ = [(n, _DP) for n in COLUMN_NAMES] + [("f", _DP)]


class GaColumnStore(C.Structure):
    _fields_ = [(n, C.c_double * 512) for n in COLUMN_NAMES]


def make_config(settings: dict, precision: int = GA_PREC_F64, device: int = 0) -> GaConfig:
    c = GaConfig()
    for name, _ in GaConfig._fields_:
        if name in settings:
            setattr(c, name, settings[name])
    c.precision = precision
    c.device = device
    return c


def declare(lib: C.CDLL, prefix: str) -> None:
    """Attach argtypes/restype to the column builders exported as
    <prefix>columns_build / <prefix>coriolis_build."""
    fn = getattr(lib, prefix + "columns_build")
    fn.argtypes = [C.c_int, C.c_double, C.c_double, _DP, _DP, C.POINTER(GaColumnStore)]
    fn.restype = C.c_int
    fn = getattr(lib, prefix + "coriolis_build")
    fn.argtypes = [C.c_int, C.c_double, C.c_double, _DP]
    fn.restype = C.c_int
