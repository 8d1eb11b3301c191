/*
 * ga_anelastic.h - C ABI of the GB300 anelastic dynamical core.
 *
 * The reference model (michaeldiaz0/Model) has no plugin layer: its per-step
 * "operator API" is a set of global C++ functions that read and write global
 * arrays.  This header replaces that surface with a context object.  Each
 * entry point below names the reference function (file:line) it stands in for.
 *
 * Conventions
 *   - 3-D fields are double precision on the host side, laid out [i][j][k]
 *     with k fastest, exactly as the reference's INDEX(i,j,k) =
 *     i*NY*NZ + j*NZ + k (include/model.h:50).
 *   - Every prognostic field keeps the reference's three rotation buffers
 *     (current, forecast "P", start-of-step "M"; solver.cpp:229-263,
 *     microphysics.cpp:642-669).  Slots are addressed with GA_SLOT_*.
 *   - The library owns all device memory.  Host pointers are borrowed for the
 *     duration of a call only.  Calls are synchronous (they return after the
 *     GPU work has finished) unless the name ends in _async.
 *   - Every entry point returns GA_OK (0) or a negative GA_ERR_* code.  The
 *     reference prints and calls exit(0) instead (kessler.cpp:83-88); this
 *     library never exits the process.  ga_last_error() gives the text of the
 *     most recent error on the calling thread.
 *   - One context per host thread.  A context is bound to one CUDA device and
 *     one CUDA stream, created by ga_create.
 */
#ifndef GA_ANELASTIC_H
#define GA_ANELASTIC_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GA_API __attribute__((visibility("default")))
#else
#define GA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GA_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define GA_OK               0
#define GA_ERR_ARG         -1   /* bad argument (null pointer, bad id, size) */
#define GA_ERR_CUDA        -2   /* a CUDA runtime call failed                 */
#define GA_ERR_NOMEM       -3   /* device allocation failed                   */
#define GA_ERR_CONFIG      -4   /* configuration rejected (grid too small...) */
#define GA_ERR_NONFINITE   -5   /* NaN/Inf found by ga_check_finite           */
#define GA_ERR_KESSLER     -6   /* microphysics instability where the
                                   reference calls exit(0): evaporation E>100
                                   (kessler.cpp:83-88, rutledge.cpp:252-258)
                                   or snow melting |psmlt|>100 (:370-376)     */
#define GA_ERR_UNSUPPORTED -7   /* option not built in this library           */

/* ---- precision of a context ------------------------------------------- */
#define GA_PREC_F64 0   /* FP64 storage and arithmetic: the parity path     */
#define GA_PREC_F32 1   /* FP32 storage and arithmetic with FP64 islands    */

/* ---- field ids ---------------------------------------------------------- */
/* prognostic fields (three rotation slots each) */
#define GA_U      0   /* us/ups/ums     model.h:63-65   */
#define GA_V      1   /* vs/vps/vms                      */
#define GA_W      2   /* ws/wps/wms                      */
#define GA_TH     3   /* ths/thps/thms                   */
#define GA_QV     4   /* qvs/qvps/qvms  microphysics.h:18 */
#define GA_QC     5   /* qcs/qcps/qcms                   */
#define GA_QR     6   /* qrs/qrps/qrms                   */
#define GA_NPROG  7
/* single-buffer fields */
#define GA_PI     7   /* pis: perturbation Exner pressure (diagnostic)       */
#define GA_UBAR   8   /* m_ubar .. m_pbar: basic state (model.h:84-91)       */
#define GA_VBAR   9
#define GA_WBAR  10
#define GA_THBAR 11
#define GA_QBAR  12
#define GA_PBAR  13
#define GA_VT    14   /* vts: rain fall speed (microphysics.h:24)            */
#define GA_NFIELDS 15
/* 2-D field: accumulated rain accRain[NX][NY] (microphysics.h:25)           */
#define GA_ACCRAIN 15
/* turbulence diagnostics of a context with turbulence_option set, as of the
 * last calculate_diff_tend (turbulence.cpp:23-31); read-only through
 * ga_get_field (ga_set_field accepts them for operator tests)               */
#define GA_KMIX    16  /* Kmix: vertical mixing coefficient (w levels)        */
#define GA_KHMIX   17  /* KHmix: horizontal mixing coefficient                */
#define GA_UFRIC   18  /* u_friction: stress divergence of u (m s^-2)        */
#define GA_VFRIC   19  /* v_friction                                          */
#define GA_WFRIC   20  /* w_friction                                          */
#define GA_THDIFF  21  /* t_diffusion: flux divergence of theta (K s^-1)     */
#define GA_QVDIFF  22  /* qv_diffusion (moist contexts)                       */
#define GA_QCDIFF  23  /* qc_diffusion                                        */
#define GA_QRDIFF  24  /* qr_diffusion                                        */
#define GA_SATURATED 25 /* isSaturated of the last microphysics call, as 0 / 1 */
/* ice microphysics (microphysics_option 2: run_rutledge_microphysics,
 * rutledge.cpp:150-452; arrays of microphysics.h:18-24)                     */
#define GA_QS      26  /* qss/qsps/qsms: snow, three rotation slots           */
#define GA_QI      27  /* qis/qips/qims: cloud ice, three rotation slots      */
#define GA_VTS     28  /* sts: snow fall speed                                */
#define GA_VTI     29  /* its: cloud-ice fall speed; state: the Eulerian
                        * update keeps it where it is not recomputed
                        * (rutledge.cpp:580-600)                              */
#define GA_ACCSNOW 30  /* accSnow[NX][NY]: accumulated snow (2-D)             */
#define GA_N0S     31  /* N0S: the snow intercept that the last microphysics
                        * pass left (one value; the snow fall speed reads it,
                        * rutledge.cpp:197-205, 503-520)                      */

/* rotation slots */
#define GA_SLOT_CUR 0  /* us  : middle of the RK stage                        */
#define GA_SLOT_P   1  /* ups : forecast value                                */
#define GA_SLOT_M   2  /* ums : value at the beginning of the step            */

/* ---- per-operator entry ids for ga_op ---------------------------------- */
#define GA_OP_SIGN_CELLS        0  /* compute_sign_cells        fluxes.cpp:316  (no-op: signs are taken on the fly) */
#define GA_OP_ADVECT_UVW        1  /* advect_uvw_velocity       advection.cpp:304 (+ buoyancy overwrite :329-337) */
#define GA_OP_SOLVE_PRESSURE    2  /* solve_pressure            pressure.cpp:142 */
#define GA_OP_PROJECT           3  /* gradient loop of integrate_non_hydro  solver.cpp:120-135 */
#define GA_OP_INTEGRATE_NON_HYDRO 4 /* integrate_non_hydro      solver.cpp:87    */
#define GA_OP_ADVECT_THETA      5  /* advect_theta              advection.cpp:349 */
#define GA_OP_ADVECT_MICRO      6  /* advect_microphysics_cell  advection.cpp:451 (linear_model: advect_qv :577) */
#define GA_OP_ZERO_MOISTURE     7  /* zero_moisture             microphysics.cpp:675 */
#define GA_OP_BC                8  /* apply_boundary_condition  boundaries.cpp:119 */
#define GA_OP_BC_MICRO          9  /* apply_boundary_condition_microphysics boundaries.cpp:200 */
#define GA_OP_KESSLER          10  /* run_microphysics microphysics.cpp:97: run_kessler_microphysics kessler.cpp:25, or run_rutledge_microphysics rutledge.cpp:150 */
#define GA_OP_RAYLEIGH         11  /* rayleigh_damping          damping.cpp:1148 */
#define GA_OP_ADVANCE_INNER    12  /* advance_inner + microphysics_advance_inner solver.cpp:241, microphysics.cpp:642 */
#define GA_OP_ADVANCE_OUTER    13  /* advance_outer + microphysics_advance       solver.cpp:254, microphysics.cpp:657 */
#define GA_OP_EXPLICIT_DIFFUSION 14 /* apply_explicit_diffusion  damping.cpp:1125 (on the start-of-step slot) */
#define GA_OP_TURBULENCE       15  /* calculate_diff_tend(1,NX-1,1,NY-1) turbulence.cpp:158 (needs turbulence_option) */
#define GA_OP_ADVECT_ICE       16  /* advect_ice_cell           advection.cpp:508 (microphysics_option 2) */
#define GA_OP_COUNT            17

/*
 * Runtime configuration: the subset of the reference's struct input_params
 * (include/stdafx.h:126-203) that the step reads, after initialize_globals
 * (initializer.cpp:160-245) has copied it into globals.  The compile-time
 * choices of the reference build (5th/3rd order advection, non-hydrostatic,
 * nonlinear, stretched-grid code path) are fixed in the kernels.
 */
typedef struct ga_config {
    int    nx, ny, nz;              /* NX, NY, NZ                                   */
    double dx, dy, dz, dt;          /* grid spacing (m) and time step (s)           */
    int    microphysics_option;     /* 0 none, 1 Kessler, 2 Rutledge-Hobbs ice      */
    int    rain_fallout;            /* 1 Eulerian, 2 semi-Lagrangian (PPM)          */
    int    periodic_ew_boundaries;  /* 0 sponge on all sides, 1 periodic east-west  */
    int    boundary_width_north;    /* jnbuffer  (boundaries.cpp:23-26)             */
    int    boundary_width_south;    /* jsbuffer                                     */
    int    boundary_width_east;     /* iebuffer                                     */
    int    boundary_width_west;     /* iwbuffer                                     */
    int    rayleigh_damping_z;      /* raydampheight: first damped level            */
    int    precision;               /* GA_PREC_F64 or GA_PREC_F32                   */
    int    device;                  /* CUDA device ordinal                           */
    /* explicit diffusion of the start-of-step fields, once per step before the
     * RK stages (apply_explicit_diffusion, damping.cpp:1125-1146, called at
     * driver_serial.cpp:188); 0 (a zeroed struct) leaves it off */
    int    use_explicit_diffusion;  /* USE_EXPLICIT_DIFFUSION                        */
    int    diffusion_order;         /* DIFFUSION_ORDER: 2, 4 or 6                    */
    double kdiffh, kdiffv;          /* horizontal / vertical coefficients (kmixh*,   */
                                    /* kmixv*, damping.cpp:122-129)                  */
    /* turbulence: mixing coefficients and stress / scalar flux tendencies from
     * the start-of-step fields once per step (calculate_diff_tend,
     * turbulence.cpp:158-292, called at driver_serial.cpp:194), added in every
     * RK stage (apply_velocity/scalar/moisture_diffusion, :233-290); flat ground
     * and an all-ocean surface (the reference's land-sea mask without a file,
     * :370-375) */
    int    turbulence_option;       /* USE_TURBULENT_STRESS: 0 or 1                  */
    int    use_surface_heat_flux;   /* SURFACE_HEAT_FLUX: surface heat and vapour    */
                                    /* fluxes of a moist run                         */
    double water_temp;              /* WATER_TEMP_C: sea-surface temperature (C)     */
    /* the linearised model about the basic state (ISLINEAR: linear_integrate_rk3,
     * driver_serial.cpp:83-171): perturbation faces advected by the basic-state
     * velocity alone (fluxes.cpp:328-337, 594-650, 1204-1357), vapour advected
     * without microphysics, explicit diffusion in every stage, the
     * perturbation rescaled every 12 hours of model time */
    int    linear_model;            /* 0 or 1                                        */
    /* the hydrostatic equation set (HYDROSTATIC: integrate_hydro, solver.cpp:
     * 33-80): u and v advected, pressure from a lid-pressure Poisson solve and
     * hydrostatic integration (pressure.cpp:229-298, 453-537), w diagnosed
     * from continuity each stage (w_velocity_LH, solver.cpp:144-163);
     * non-periodic domains */
    int    hydrostatic;             /* 0 or 1                                        */
} ga_config;

/*
 * Vertical columns and the other small arrays the step reads.  The caller
 * fills them (ga_columns_build does it from tb/qb exactly as the reference's
 * initialize_vertical_basic_state2, initializer.cpp:858-928) and the library
 * copies them.  All arrays are double.
 */
typedef struct ga_columns {
    const double *zu, *zw;            /* [NZ] unstretched heights (initializer.cpp:840-849) */
    const double *zsu, *zsw;          /* [NZ] stretched heights (stretched_grid :1340)      */
    const double *mu, *mw;            /* [NZ] grid-stretching factors                       */
    const double *rhou, *rhow;        /* [NZ] base-state density at u and w levels          */
    const double *one_d_rhou, *one_d_rhow;
    const double *tb, *tbv, *tbw, *qb, *pib;   /* [NZ] base-state theta, theta_v, q, Exner */
    const double *f;                  /* [NY] Coriolis parameter (initializer.cpp:826)      */
} ga_columns;

/* Owned storage for a ga_columns, filled by ga_columns_build. */
typedef struct ga_column_store {
    double zu[512], zw[512], zsu[512], zsw[512], mu[512], mw[512];
    double rhou[512], rhow[512], one_d_rhou[512], one_d_rhow[512];
    double tb[512], tbv[512], tbw[512], qb[512], pib[512];
} ga_column_store;

typedef struct ga_ctx ga_ctx;

/* ---- library ----------------------------------------------------------- */
GA_API int ga_abi_version(void);
GA_API const char *ga_last_error(void);

/*
 * Build the vertical column arrays from the base-state theta tb[NZ] and
 * humidity qb[NZ] profiles.  Replaces setup_vertical_height_levels
 * (initializer.cpp:840), stretched_grid (:1340) and
 * initialize_vertical_basic_state2 (:858-928), including their in-place edits
 * of tb/qb (tb[0]=tb[1] etc.).  height_lowest_level is the reference input of
 * the same name.  Host-only; needs no GPU.
 */
GA_API int ga_columns_build(int nz, double dz, double height_lowest_level,
                     const double *tb_in, const double *qb_in,
                     ga_column_store *out);

/*
 * Coriolis parameter f[j] for a domain whose south-west corner is given by the
 * reference's corner_lat input: setup_coordinates(0,-89.462997)
 * (initializer.cpp:1948-1967) then initialize_coriolis_parameter (:826-833).
 * Host-only.
 */
GA_API int ga_coriolis_build(int ny, double dy, double corner_lat, double *f_out);

/* ---- context ------------------------------------------------------------ */
/* Replaces initialize_serial's solver set-up: initialize_pressure_solver
 * (pressure.cpp:99), init_boundaries (boundaries.cpp:44), init_microphysics
 * (microphysics.cpp:41).  Allocates every device buffer (zeroed, as the
 * reference's calloc) and precomputes the spectral and sponge tables. */
GA_API int ga_create(const ga_config *cfg, const ga_columns *cols, ga_ctx **out);
GA_API int ga_destroy(ga_ctx *ctx);

/* Copy one field between host and device.  For prognostic fields `slot` picks
 * the rotation buffer; for the others it is ignored.  n must equal NX*NY*NZ
 * (NX*NY for GA_ACCRAIN).  Values are converted to/from FP32 for FP32
 * contexts. */
GA_API int ga_set_field(ga_ctx *ctx, int field, int slot, const double *host, size_t n);
GA_API int ga_get_field(ga_ctx *ctx, int field, int slot, double *host, size_t n);

/* Advance nsteps full RK3 steps: nsteps calls of s_integrate_rk3
 * (driver_serial.cpp:178-286), each followed by the counter updates of
 * s_run_model (bigcounter++, mtime += dt; driver_serial.cpp:366-369). */
GA_API int ga_step(ga_ctx *ctx, int nsteps);
/* Same, queued on the context's stream without a final synchronize. */
GA_API int ga_step_async(ga_ctx *ctx, int nsteps);
GA_API int ga_synchronize(ga_ctx *ctx);

/* Run a single operator (GA_OP_*) with RK fraction `step`, for per-operator
 * parity tests.  Mirrors calling the reference global function directly. */
GA_API int ga_op(ga_ctx *ctx, int op, double step);

/* Number of completed steps (reference: bigcounter) and model time (mtime). */
GA_API int ga_get_counters(ga_ctx *ctx, long long *bigcounter, double *mtime);

/* FP64 domain budgets of one rotation slot (GA_SLOT_*), summed on the GPU in
 * FP64 whatever the context's precision, over the physical cells
 * i in [1, NX-1), j in [1, NY-1), k in [1, NZ-1) with the density-times-volume
 * weight rhou[k] dx dy dz / mu[k]:
 *   GA_BUDGET_THETA  sum of rho theta' dV      GA_BUDGET_WATER  QV + QC + QR
 *   GA_BUDGET_QV / _QC / _QR  rho q dV          (+ QI + QS with the ice scheme)
 *   GA_BUDGET_KE     0.5 rho |u'|^2 dV
 *   GA_BUDGET_RAIN   accumulated surface rain times dx dy (GA_ACCRAIN)
 *   GA_BUDGET_MASS   sum of rho dV
 *   GA_BUDGET_QI / _QS  rho q dV of cloud ice and snow, GA_BUDGET_SNOW the
 *   accumulated snow times dx dy (GA_ACCSNOW); 0 without the ice scheme
 * The flux form of the advection (advection.cpp:304-498) conserves the
 * theta, moisture and water integrals up to the fluxes through the domain's
 * boundary and the base-state terms; Kessler (kessler.cpp:25-213) conserves
 * the total water of every point.  The blocks' partial sums are added in a
 * fixed order, so repeated calls on the same state give the same bits.  The
 * reference computes no budget on its step path (its energy diagnostics,
 * energy.cpp, are out of this library's scope).  n must be at least 8 (the
 * entries up to GA_BUDGET_MASS); min(n, GA_NBUDGET) entries are written. */
#define GA_BUDGET_THETA 0
#define GA_BUDGET_QV    1
#define GA_BUDGET_QC    2
#define GA_BUDGET_QR    3
#define GA_BUDGET_WATER 4
#define GA_BUDGET_KE    5
#define GA_BUDGET_RAIN  6
#define GA_BUDGET_MASS  7
#define GA_BUDGET_QI    8
#define GA_BUDGET_QS    9
#define GA_BUDGET_SNOW  10
#define GA_NBUDGET      11
GA_API int ga_budget(ga_ctx *ctx, int slot, double *out, int n);

/* Set the step counter and model time (a restart: bigcounter and mtime as
 * ga_get_counters returned them when the state was saved). */
GA_API int ga_set_counters(ga_ctx *ctx, long long bigcounter, double mtime);

/* Scan the prognostic forecast buffers for NaN/Inf on the device.
 * Returns GA_OK or GA_ERR_NONFINITE.  The reference has no such check. */
GA_API int ga_check_finite(ga_ctx *ctx);

/* Number of kernel launches issued by this context since creation. */
GA_API long long ga_launch_count(ga_ctx *ctx);

/* CUDA stream the context runs on (a cudaStream_t, as void*). */
GA_API void *ga_stream(ga_ctx *ctx);

/* Device pointer of a field buffer (FP64 or FP32 per the precision), for
 * callers that keep state resident on the GPU. */
GA_API void *ga_field_device_ptr(ga_ctx *ctx, int field, int slot);

/*
 * Autotuner.  No counterpart in the reference.  ga_tune times the candidate
 * kernels, tile shapes and FFT plans of this context on its current state and
 * keeps the fastest: the advection kernel and tile (per-level tiles 4x4, 2x4,
 * 4x2, 4x8, 8x4; in FP32 with NZ % 4 == 0 the four-level kernel with tiles
 * 4x4, 4x8, 8x4, 2x8, 8x8, each at two register budgets, with east and north
 * faces per work item or by sliding row segments); the level tile of the y
 * transforms; the factor order of the x and y FFTs; the fused x solve's block
 * (256, 512 or 1024 threads; FP32: also as CTA pairs) against the unfused x
 * transforms and solve with each x level tile.  L2 is written over before each
 * candidate's timed launches, as a step that starts from DRAM sees it.  The
 * state is unchanged.  Every kernel and tile gives bit-identical results; the
 * FFT factor orders round differently (FP64: ~1e-15).  ga_tuning writes the
 * current choice as text (NUL-terminated, truncated to n bytes).
 */
GA_API int ga_tune(ga_ctx *ctx);
GA_API int ga_tuning(ga_ctx *ctx, char *buf, size_t n);

/*
 * Tangent-linear model and adjoint of the step.  No counterpart in the
 * reference, which has no linearisation; this differentiates exactly the step
 * ga_step runs, for non-periodic contexts, dry or with Kessler microphysics
 * and Eulerian rain fallout (rain_fallout 1); GA_ERR_UNSUPPORTED otherwise.
 * Arithmetic is in the context's precision.
 *
 * The context holds one set of perturbation buffers shaped like the state:
 * current, P and M slots of the prognostic fields (GA_U .. GA_TH, and GA_QV ..
 * GA_QR when moist), plus GA_PI (slot ignored), rotating with the state.
 * Upwind signs, zero_moisture clipping and the branches of Kessler are
 * frozen at the trajectory (recorded on the forward pass: clipping bits per
 * point and stage, Kessler's inputs per step).
 *
 * ga_tlm_step advances the state and the perturbations together nsteps.
 *
 * ga_adjoint advances the state nsteps from its current value (it ends there,
 * with the counters advanced) and maps the adjoint held in the perturbation
 * buffers, taken as the gradient of a function of the final state, to the
 * gradient with respect to the initial state.  The state is checkpointed every
 * `checkpoint_every` steps (<= 0: one segment).  A segment's adjoint runs on
 * its trajectory (the stage-start fields: 12 fields a step dry, 26 fields + 3
 * clipping records moist): the first sweep records the trajectories of the
 * last segments, as many as device memory holds beside the checkpoints with a
 * tenth of the GPU's memory to spare (at least one), and every earlier segment
 * is recomputed from its checkpoint, recording, before its adjoint runs.  The
 * environment variable GA_ADJ_RESIDENT=n fixes that count.  Results do not
 * depend on it or on checkpoint_every.  The trajectory buffer is kept for
 * later calls and released by ga_destroy.
 * The adjoint kernels are in gather form (no atomics).  The GA_PI entry is
 * zero on return: the step never reads pi.
 */
GA_API int ga_lin_set_field(ga_ctx *ctx, int field, int slot, const double *host, size_t n);
GA_API int ga_lin_get_field(ga_ctx *ctx, int field, int slot, double *host, size_t n);
GA_API int ga_tlm_step(ga_ctx *ctx, int nsteps);
GA_API int ga_adjoint(ga_ctx *ctx, int nsteps, int checkpoint_every);

/*
 * Ensembles.  The reference runs ensemble members as separate serial models
 * farmed out over MPI tasks (run_ensemble, ensemble.cpp:45-144).  Here the
 * members (independent domains; grids, spacings and time steps may differ)
 * advance together: every kernel phase of the step is one launch over all
 * members, from a packed member table, and the two-step cycle is captured in
 * a CUDA graph.  Each member computes exactly what a standalone context with
 * its configuration computes.  Members share precision, device and
 * microphysics option; periodic members and semi-Lagrangian rain fallout are
 * not batched (GA_ERR_UNSUPPORTED).  The x solve of the pressure equation is
 * one fused kernel per y-wavenumber, or, when a member's levels do not fit in
 * shared memory (or ga_ensemble_tune finds it faster), batched x FFTs, Thomas
 * blocks and inverse x FFTs.  Fields are set and read per member with the
 * same ids and slots as ga_set_field / ga_get_field.
 */
typedef struct ga_ens ga_ens;
GA_API int ga_ensemble_create(const ga_config *cfgs, const ga_columns *cols, int nmembers, ga_ens **out);
GA_API int ga_ensemble_destroy(ga_ens *ens);
GA_API int ga_ensemble_size(ga_ens *ens);
GA_API int ga_ensemble_set_field(ga_ens *ens, int member, int field, int slot, const double *host, size_t n);
GA_API int ga_ensemble_get_field(ga_ens *ens, int member, int field, int slot, double *host, size_t n);
GA_API int ga_ensemble_step(ga_ens *ens, int nsteps);
GA_API int ga_ensemble_step_async(ga_ens *ens, int nsteps);
GA_API int ga_ensemble_synchronize(ga_ens *ens);
GA_API void *ga_ensemble_stream(ga_ens *ens);
GA_API long long ga_ensemble_launch_count(ga_ens *ens);
GA_API int ga_ensemble_get_counters(ga_ens *ens, int member, long long *bigcounter, double *mtime);
/* Autotuner of the batched step (advection kernel and tile, y level tile, fused or
 * unfused x solve), as ga_tune, over all members. */
GA_API int ga_ensemble_tune(ga_ens *ens);
GA_API int ga_ensemble_tuning(ga_ens *ens, char *buf, size_t n);

/*
 * Pressure solve without device allocation.  No counterpart in the reference:
 * it is for callers that cannot allocate GPU memory themselves or through
 * this library: a host model that owns every byte of device memory in its
 * own pool and hands none to third-party code, or a plugin inside a process
 * whose allocator forbids foreign cudaMalloc calls.
 *
 * Runs solve_pressure (pressure.cpp:142-224) in FP64 on caller-owned device
 * arrays [NX][NY][NZ]: up, vp, wp (read, and their lateral boundary points
 * overwritten by the mirror or periodic copy, as the reference does) and pi
 * (written).  cols are host arrays as for ga_create; their mu, mw, rhou and
 * rhow columns are read during the call and passed to the GPU by value, so
 * the caller may free or change them as soon as the call returns.  The work
 * is queued on `stream` (a cudaStream_t, or NULL for the legacy default
 * stream) on the current CUDA device; the call returns without synchronizing.
 *
 * All scratch lives in one file-scope device array of GA_NOALLOC_SCRATCH_BYTES
 * that every GPU loading this library holds until the process exits.  The
 * first call on a device looks up that array's device address and sets the
 * kernels' shared-memory limits (once per device, with that device current).
 * Grids are rejected with GA_ERR_ARG, before anything is queued, when their
 * spectral buffer and tables exceed the array (for a non-periodic grid:
 * 16*NX*NY*NZ + 8*NX*NY + 16*(NX+NY) bytes plus small column tables, e.g.
 * 128 x 128 x 96 fits) or when a transform line is too long for the 200 KiB
 * of shared memory per block (NY above about 6400, or a long NX whose levels
 * also do not fit the unfused x transform).  Calls share the array and it
 * keeps the last call's contents (each call writes every element it reads):
 * calls that overlap on the GPU race and must be ordered by the caller.
 * The function calls no cudaMalloc, cudaFree or other allocating routine.
 */
#define GA_NOALLOC_SCRATCH_BYTES (32u << 20)
GA_API int ga_solve_pressure_noalloc(const ga_config *cfg, const ga_columns *cols, double *up,
                                     double *vp, double *wp, double *pi, double step, void *stream);

/* Optional timing of the kernel groups with CUDA events recorded on the
 * context's stream (advect, edges, div_fft_y, fft_x, thomas, ifft_y_pi,
 * post, kessler, ppm, copy).  Enabling resets the totals.  The reference
 * only prints the CPU time of whole steps (driver_serial.cpp:354-364). */
GA_API int ga_profile_enable(ga_ctx *ctx, int on);
GA_API int ga_profile_count(ga_ctx *ctx);
GA_API int ga_profile_get(ga_ctx *ctx, int idx, char *name, size_t cap, double *total_ms,
                          long long *launches);

#ifdef __cplusplus
}
#endif
#endif /* GA_ANELASTIC_H */
