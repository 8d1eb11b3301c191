// ga_api.cu - the extern "C" boundary declared in include/ga_anelastic.h.
// Argument checks, error text, context bookkeeping and the host-only column
// builders live here; everything else is forwarded to the per-precision
// engine.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <string>

#include "ga_engine.h"

namespace ga {
static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
}  // namespace ga

struct ga_ctx {
    ga::EngineBase *e;
    ga_config cfg;
};

struct ga_ens {
    ga::EnsembleBase *e;
};

using ga::set_error;

static int fail(int rc, const std::string &msg)
{
    set_error(msg);
    return rc;
}

extern "C" {

int ga_abi_version(void) { return GA_ABI_VERSION; }

const char *ga_last_error(void) { return ga::g_last_error.c_str(); }

/* setup_vertical_height_levels (initializer.cpp:840-849), stretched_grid
 * (:1340-1385), initialize_vertical_basic_state2 (:858-928) */
int ga_columns_build(int NZ, double dz, double z0, const double *tb_in, const double *qb_in,
                     ga_column_store *o)
{
    if (!tb_in || !qb_in || !o) return fail(GA_ERR_ARG, "ga_columns_build: null pointer");
    if (NZ < 6 || NZ > 512) return fail(GA_ERR_ARG, "ga_columns_build: NZ must be in [6,512]");
    if (!(dz > 0)) return fail(GA_ERR_ARG, "ga_columns_build: dz must be positive");
    const double Rd = 287.0, cp = 1004, cv = 717, p0 = 100000, grav = 9.8, pressfc = 100200;
    std::memset(o, 0, sizeof(*o));
    for (int k = 0; k < NZ; k++) {
        o->zu[k] = ((double)k - 0.5) * dz;
        o->zw[k] = ((double)k - 1) * dz;
    }
    const int lev = 1, nt = NZ - 1;
    const double dzp = dz;
    const double c2 = (1 - z0 / (dzp * lev)) / ((nt - 1) * dzp - dzp * lev);
    const double c1 = z0 / (dzp * lev) - c2 * dzp * lev;
    for (int i = 0; i <= nt; i++) {
        const double fullLev = ((double)i - 1.0) * dzp, halfLev = ((double)i - 0.5) * dzp;
        o->zsw[i] = (c1 + c2 * fullLev) * fullLev;
        o->mw[i] = 1 / (c1 + 2 * c2 * fullLev);
        o->zsu[i] = (c1 + c2 * halfLev) * halfLev;
        o->mu[i] = 1 / (c1 + 2 * c2 * halfLev);
    }
    double *tb = o->tb, *qb = o->qb, *tbw = o->tbw, *tbv = o->tbv, *pib = o->pib;
    double *rhou = o->rhou, *rhow = o->rhow, *zsu = o->zsu;
    for (int k = 0; k < NZ; k++) { tb[k] = tb_in[k]; qb[k] = qb_in[k]; }
    tb[0] = tb[1]; tb[NZ - 1] = tb[NZ - 2];
    qb[0] = qb[1]; qb[NZ - 1] = qb[NZ - 2];
    tbw[0] = 0.5 * (tb[0] + tb[1]);
    for (int k = 1; k < NZ; k++) tbw[k] = 0.5 * (tb[k] + tb[k - 1]);
    for (int k = 0; k < NZ; k++) tbv[k] = tb[k] * (1.0 + 0.61 * qb[k]);
    const double pisfc = pow((pressfc / p0), (Rd / cp));
    pib[1] = pisfc - grav * (zsu[1] - 0) / (cp * tbv[1]);
    pib[0] = pisfc + grav * (0 - zsu[0]) / (cp * tbv[0]);
    for (int k = 2; k < NZ; k++)
        pib[k] = pib[k - 1] - grav * (zsu[k] - zsu[k - 1]) / (cp * (0.5 * (tbv[k] + tbv[k - 1])));
    for (int k = 0; k < NZ; k++) rhou[k] = p0 * pow(pib[k], (cv / Rd)) / (Rd * tbv[k]);
    for (int k = 1; k < NZ; k++) rhow[k] = 0.5 * (rhou[k] + rhou[k - 1]);
    tbv[0] = tbv[1]; tbv[NZ - 1] = tbv[NZ - 2];
    tbw[0] = tbw[1]; tbw[NZ - 1] = tbw[NZ - 2];
    pib[0] = pib[1]; pib[NZ - 1] = pib[NZ - 2];
    rhow[0] = rhow[1];
    for (int k = 0; k < NZ; k++) {
        o->one_d_rhow[k] = 1. / rhow[k];
        o->one_d_rhou[k] = 1. / rhou[k];
    }
    return GA_OK;
}

/* setup_coordinates(0,-89.462997) (initializer.cpp:1948-1967) and
 * initialize_coriolis_parameter (:826-833) */
int ga_coriolis_build(int NY, double dy, double corner_lat, double *f)
{
    if (!f || NY < 1) return fail(GA_ERR_ARG, "ga_coriolis_build: bad arguments");
    const double fc = 7.292e-5, mpd = 111000, trigpi = 3.14159265358979324;
    double lat = -89.462997 + corner_lat + dy / mpd;
    for (int j = 0; j < NY; j++) {
        if (j > 0) lat = lat + dy / mpd;
        f[j] = 2 * fc * sin(lat * trigpi / 180.);
    }
    return GA_OK;
}

int ga_create(const ga_config *cfg, const ga_columns *cols, ga_ctx **out)
{
    if (!cfg || !cols || !out) return fail(GA_ERR_ARG, "ga_create: null pointer");
    *out = nullptr;
    const ga_columns &c = *cols;
    const double *req[] = {c.zu, c.zw, c.zsu, c.zsw, c.mu, c.mw, c.rhou, c.rhow, c.one_d_rhou,
                           c.one_d_rhow, c.tb, c.tbv, c.tbw, c.qb, c.pib, c.f};
    for (const double *p : req)
        if (!p) return fail(GA_ERR_ARG, "ga_create: a column array is null");
    if (cfg->nx < 12 || cfg->ny < 12) return fail(GA_ERR_CONFIG, "ga_create: NX and NY must be >= 12");
    if (cfg->nz < 6 || cfg->nz > 128) return fail(GA_ERR_CONFIG, "ga_create: NZ must be in [6,128]");
    if (!(cfg->dx > 0 && cfg->dy > 0 && cfg->dz > 0 && cfg->dt > 0))
        return fail(GA_ERR_CONFIG, "ga_create: dx, dy, dz, dt must be positive");
    if (cfg->microphysics_option < 0 || cfg->microphysics_option > 2)
        return fail(GA_ERR_CONFIG, "ga_create: microphysics_option must be 0, 1 or 2");
    if (cfg->microphysics_option >= 1 && cfg->rain_fallout != 1 && cfg->rain_fallout != 2)
        return fail(GA_ERR_CONFIG, "ga_create: rain_fallout must be 1 or 2");
    if (cfg->microphysics_option == 2 && cfg->linear_model == 1)
        return fail(GA_ERR_UNSUPPORTED, "ga_create: the linearised model has no ice scheme (linear_integrate_rk3 "
                                        "advects the vapour alone)");
    if (cfg->precision != GA_PREC_F64 && cfg->precision != GA_PREC_F32)
        return fail(GA_ERR_CONFIG, "ga_create: unknown precision");
    const int widths[] = {cfg->boundary_width_north, cfg->boundary_width_south, cfg->boundary_width_east,
                          cfg->boundary_width_west};
    for (int w : widths)
        if (w < 0 || w > 64) return fail(GA_ERR_CONFIG, "ga_create: sponge widths must be in [0,64]");
    if (cfg->periodic_ew_boundaries && cfg->nx < 13)
        return fail(GA_ERR_CONFIG, "ga_create: periodic domains need NX >= 13");
    if (cfg->use_explicit_diffusion && cfg->diffusion_order != 2 && cfg->diffusion_order != 4 &&
        cfg->diffusion_order != 6)
        return fail(GA_ERR_CONFIG, "ga_create: diffusion_order must be 2, 4 or 6");
    if (cfg->turbulence_option < 0 || cfg->turbulence_option > 1 || cfg->use_surface_heat_flux < 0 ||
        cfg->use_surface_heat_flux > 1)
        return fail(GA_ERR_CONFIG, "ga_create: turbulence_option and use_surface_heat_flux must be 0 or 1");
    if (cfg->linear_model < 0 || cfg->linear_model > 1 || cfg->hydrostatic < 0 || cfg->hydrostatic > 1)
        return fail(GA_ERR_CONFIG, "ga_create: linear_model and hydrostatic must be 0 or 1");
    if (cfg->hydrostatic && (cfg->periodic_ew_boundaries || cfg->turbulence_option || cfg->linear_model))
        return fail(GA_ERR_UNSUPPORTED, "ga_create: the hydrostatic equation set is built for non-periodic "
                                        "domains without the turbulence scheme or the linearised model");
    if (cfg->linear_model && cfg->turbulence_option)
        return fail(GA_ERR_UNSUPPORTED, "ga_create: the linearised model has no turbulence scheme "
                                        "(linear_integrate_rk3 never computes its tendencies)");
    int rc = GA_OK;
    ga::EngineBase *e = nullptr;
    try {
        e = cfg->precision == GA_PREC_F64 ? ga::make_engine_f64(cfg, cols, &rc) : ga::make_engine_f32(cfg, cols, &rc);
    } catch (const std::exception &ex) {
        return fail(GA_ERR_NOMEM, std::string("ga_create: ") + ex.what());
    }
    if (!e) return fail(rc ? rc : GA_ERR_CUDA, "ga_create: device set-up failed");
    ga_ctx *ctx = new ga_ctx;
    ctx->e = e;
    ctx->cfg = *cfg;
    *out = ctx;
    return GA_OK;
}

int ga_destroy(ga_ctx *ctx)
{
    if (!ctx) return fail(GA_ERR_ARG, "ga_destroy: null context");
    delete ctx->e;
    delete ctx;
    return GA_OK;
}

int ga_set_field(ga_ctx *ctx, int field, int slot, const double *host, size_t n)
{
    if (!ctx || !host) return fail(GA_ERR_ARG, "ga_set_field: null pointer");
    if (field < 0 || field > GA_N0S || slot < 0 || slot > 2) return fail(GA_ERR_ARG, "ga_set_field: bad field or slot");
    int rc = ctx->e->set_field(field, slot, host, n);
    if (rc == GA_ERR_ARG) set_error("ga_set_field: field not present in this context or wrong size");
    return rc;
}

int ga_get_field(ga_ctx *ctx, int field, int slot, double *host, size_t n)
{
    if (!ctx || !host) return fail(GA_ERR_ARG, "ga_get_field: null pointer");
    if (field < 0 || field > GA_N0S || slot < 0 || slot > 2) return fail(GA_ERR_ARG, "ga_get_field: bad field or slot");
    int rc = ctx->e->get_field(field, slot, host, n);
    if (rc == GA_ERR_ARG) set_error("ga_get_field: field not present in this context or wrong size");
    return rc;
}

int ga_step_async(ga_ctx *ctx, int nsteps)
{
    if (!ctx || nsteps < 0) return fail(GA_ERR_ARG, "ga_step: bad arguments");
    return ctx->e->step(nsteps);
}

int ga_synchronize(ga_ctx *ctx)
{
    if (!ctx) return fail(GA_ERR_ARG, "ga_synchronize: null context");
    cudaSetDevice(ctx->e->device);
    cudaError_t err = cudaStreamSynchronize(ctx->e->stream);
    if (err != cudaSuccess) return fail(GA_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(err));
    return GA_OK;
}

int ga_step(ga_ctx *ctx, int nsteps)
{
    int rc = ga_step_async(ctx, nsteps);
    if (rc) return rc;
    rc = ga_synchronize(ctx);
    if (rc) return rc;
    return ctx->e->op(GA_OP_SIGN_CELLS, 0.0);  /* reports a Kessler E>100 flag */
}

int ga_op(ga_ctx *ctx, int op, double step)
{
    if (!ctx) return fail(GA_ERR_ARG, "ga_op: null context");
    if (op < 0 || op >= GA_OP_COUNT) return fail(GA_ERR_ARG, "ga_op: unknown operator");
    return ctx->e->op(op, step);
}

int ga_get_counters(ga_ctx *ctx, long long *bigcounter, double *mtime)
{
    if (!ctx) return fail(GA_ERR_ARG, "ga_get_counters: null context");
    if (bigcounter) *bigcounter = ctx->e->bigcounter;
    if (mtime) *mtime = ctx->e->mtime;
    return GA_OK;
}

int ga_budget(ga_ctx *ctx, int slot, double *out, int n)
{
    if (!ctx || !out || n < GA_BUDGET_MASS + 1) return fail(GA_ERR_ARG, "ga_budget: bad arguments");
    if (slot < 0 || slot > 2) return fail(GA_ERR_ARG, "ga_budget: bad slot");
    double all[GA_NBUDGET];
    const int rc = ctx->e->budget(slot, all);
    for (int b = 0; b < n && b < GA_NBUDGET; b++) out[b] = all[b];
    return rc;
}

int ga_set_counters(ga_ctx *ctx, long long bigcounter, double mtime)
{
    if (!ctx || bigcounter < 0) return fail(GA_ERR_ARG, "ga_set_counters: bad arguments");
    ctx->e->bigcounter = bigcounter;
    ctx->e->mtime = mtime;
    return GA_OK;
}

int ga_check_finite(ga_ctx *ctx)
{
    if (!ctx) return fail(GA_ERR_ARG, "ga_check_finite: null context");
    int rc = ctx->e->check_finite();
    if (rc == GA_ERR_NONFINITE) set_error("non-finite value in a prognostic buffer");
    return rc;
}

long long ga_launch_count(ga_ctx *ctx) { return ctx ? ctx->e->launches : -1; }

int ga_ensemble_tune(ga_ens *ens)
{
    if (!ens) return fail(GA_ERR_ARG, "ga_ensemble_tune: null ensemble");
    return ens->e->tune();
}

int ga_ensemble_tuning(ga_ens *ens, char *buf, size_t n)
{
    if (!ens || !buf || n == 0) return fail(GA_ERR_ARG, "ga_ensemble_tuning: bad arguments");
    const std::string t = ens->e->tuning.empty() ? std::string("defaults (not tuned)") : ens->e->tuning;
    const size_t m = std::min(n - 1, t.size());
    std::memcpy(buf, t.data(), m);
    buf[m] = 0;
    return GA_OK;
}

int ga_tune(ga_ctx *ctx)
{
    if (!ctx) return fail(GA_ERR_ARG, "ga_tune: null context");
    return ctx->e->tune();
}

int ga_tuning(ga_ctx *ctx, char *buf, size_t n)
{
    if (!ctx || !buf || n == 0) return fail(GA_ERR_ARG, "ga_tuning: bad arguments");
    const std::string &t = ctx->e->tuning.empty() ? std::string("defaults (not tuned)") : ctx->e->tuning;
    const size_t m = std::min(n - 1, t.size());
    std::memcpy(buf, t.data(), m);
    buf[m] = 0;
    return GA_OK;
}

int ga_lin_set_field(ga_ctx *ctx, int field, int slot, const double *host, size_t n)
{
    if (!ctx || !host) return fail(GA_ERR_ARG, "ga_lin_set_field: null argument");
    if (!((field >= GA_U && field <= GA_QR) || field == GA_PI))
        return fail(GA_ERR_ARG, "ga_lin_set_field: field must be a prognostic field or GA_PI");
    int rc = ctx->e->lin_set_field(field, slot, host, n);
    if (rc == GA_ERR_ARG) set_error("ga_lin_set_field: bad slot or size");
    return rc;
}

int ga_lin_get_field(ga_ctx *ctx, int field, int slot, double *host, size_t n)
{
    if (!ctx || !host) return fail(GA_ERR_ARG, "ga_lin_get_field: null argument");
    if (!((field >= GA_U && field <= GA_QR) || field == GA_PI))
        return fail(GA_ERR_ARG, "ga_lin_get_field: field must be a prognostic field or GA_PI");
    int rc = ctx->e->lin_get_field(field, slot, host, n);
    if (rc == GA_ERR_ARG) set_error("ga_lin_get_field: bad slot or size");
    return rc;
}

int ga_tlm_step(ga_ctx *ctx, int nsteps)
{
    if (!ctx || nsteps < 0) return fail(GA_ERR_ARG, "ga_tlm_step: bad arguments");
    return ctx->e->tlm_step(nsteps);
}

int ga_adjoint(ga_ctx *ctx, int nsteps, int checkpoint_every)
{
    if (!ctx || nsteps < 0) return fail(GA_ERR_ARG, "ga_adjoint: bad arguments");
    return ctx->e->adjoint(nsteps, checkpoint_every);
}

void *ga_stream(ga_ctx *ctx) { return ctx ? (void *)ctx->e->stream : nullptr; }

void *ga_field_device_ptr(ga_ctx *ctx, int field, int slot)
{
    if (!ctx || slot < 0 || slot > 2) return nullptr;
    if ((field < 0 || field > GA_QRDIFF) && (field < GA_QS || field > GA_N0S)) return nullptr;
    return ctx->e->field_ptr(field, slot);
}

int ga_ensemble_create(const ga_config *cfgs, const ga_columns *cols, int nmembers, ga_ens **out)
{
    if (!cfgs || !cols || !out || nmembers < 1) return fail(GA_ERR_ARG, "ga_ensemble_create: bad arguments");
    *out = nullptr;
    for (int m = 0; m < nmembers; m++) {
        const ga_config &c = cfgs[m];
        if (c.precision != cfgs[0].precision || c.device != cfgs[0].device ||
            c.microphysics_option != cfgs[0].microphysics_option)
            return fail(GA_ERR_CONFIG, "ga_ensemble_create: members must share precision, device and microphysics");
        if (c.periodic_ew_boundaries)
            return fail(GA_ERR_UNSUPPORTED, "ga_ensemble_create: periodic members are not batched");
        if (c.use_explicit_diffusion)
            return fail(GA_ERR_UNSUPPORTED, "ga_ensemble_create: explicit diffusion is not batched");
        if (c.turbulence_option)
            return fail(GA_ERR_UNSUPPORTED, "ga_ensemble_create: the turbulence scheme is not batched");
        if (c.linear_model || c.hydrostatic)
            return fail(GA_ERR_UNSUPPORTED, "ga_ensemble_create: the linearised and hydrostatic sets are not batched");
        if (c.microphysics_option == 1 && c.rain_fallout != 1)
            return fail(GA_ERR_UNSUPPORTED, "ga_ensemble_create: only Eulerian rain fallout is batched");
        if (c.nx < 12 || c.ny < 12 || c.nz < 6 || c.nz > 128 || !(c.dx > 0 && c.dy > 0 && c.dz > 0 && c.dt > 0))
            return fail(GA_ERR_CONFIG, "ga_ensemble_create: member grid out of range");
        if (c.microphysics_option < 0 || c.microphysics_option > 1)
            return fail(GA_ERR_CONFIG, "ga_ensemble_create: microphysics_option must be 0 or 1");
    }
    int rc = GA_OK;
    ga::EnsembleBase *e = cfgs[0].precision == GA_PREC_F64 ? ga::make_ensemble_f64(cfgs, cols, nmembers, &rc)
                                                           : ga::make_ensemble_f32(cfgs, cols, nmembers, &rc);
    if (!e) return fail(rc ? rc : GA_ERR_CUDA, "ga_ensemble_create: set-up failed");
    *out = new ga_ens{e};
    return GA_OK;
}

int ga_ensemble_destroy(ga_ens *ens)
{
    if (!ens) return fail(GA_ERR_ARG, "ga_ensemble_destroy: null");
    delete ens->e;
    delete ens;
    return GA_OK;
}

int ga_ensemble_size(ga_ens *ens) { return ens ? ens->e->size() : -1; }

int ga_ensemble_set_field(ga_ens *ens, int member, int field, int slot, const double *host, size_t n)
{
    if (!ens || !host) return fail(GA_ERR_ARG, "ga_ensemble_set_field: null pointer");
    ga::EngineBase *m = ens->e->member(member);
    if (!m) return fail(GA_ERR_ARG, "ga_ensemble_set_field: no such member");
    if (field < 0 || field > GA_ACCRAIN || slot < 0 || slot > 2) return fail(GA_ERR_ARG, "ga_ensemble_set_field: bad field or slot");
    int rc = ens->e->synchronize();
    if (rc) return rc;
    rc = m->set_field(field, slot, host, n);
    if (rc == GA_ERR_ARG) set_error("ga_ensemble_set_field: field not present or wrong size");
    if (field >= GA_UBAR && field <= GA_PBAR) ens->e->mark_dirty();
    return rc;
}

int ga_ensemble_get_field(ga_ens *ens, int member, int field, int slot, double *host, size_t n)
{
    if (!ens || !host) return fail(GA_ERR_ARG, "ga_ensemble_get_field: null pointer");
    ga::EngineBase *m = ens->e->member(member);
    if (!m) return fail(GA_ERR_ARG, "ga_ensemble_get_field: no such member");
    if (field < 0 || field > GA_ACCRAIN || slot < 0 || slot > 2) return fail(GA_ERR_ARG, "ga_ensemble_get_field: bad field or slot");
    int rc = ens->e->synchronize();
    if (rc) return rc;
    rc = m->get_field(field, slot, host, n);
    if (rc == GA_ERR_ARG) set_error("ga_ensemble_get_field: field not present or wrong size");
    return rc;
}

int ga_ensemble_step_async(ga_ens *ens, int nsteps)
{
    if (!ens || nsteps < 0) return fail(GA_ERR_ARG, "ga_ensemble_step: bad arguments");
    return ens->e->step(nsteps);
}

int ga_ensemble_synchronize(ga_ens *ens)
{
    if (!ens) return fail(GA_ERR_ARG, "ga_ensemble_synchronize: null");
    return ens->e->synchronize();
}

int ga_ensemble_step(ga_ens *ens, int nsteps)
{
    int rc = ga_ensemble_step_async(ens, nsteps);
    if (rc) return rc;
    return ga_ensemble_synchronize(ens);
}

void *ga_ensemble_stream(ga_ens *ens) { return ens ? ens->e->stream_handle() : nullptr; }

long long ga_ensemble_launch_count(ga_ens *ens) { return ens ? ens->e->launches : -1; }

int ga_ensemble_get_counters(ga_ens *ens, int member, long long *bigcounter, double *mtime)
{
    if (!ens) return fail(GA_ERR_ARG, "ga_ensemble_get_counters: null");
    ga::EngineBase *m = ens->e->member(member);
    if (!m) return fail(GA_ERR_ARG, "ga_ensemble_get_counters: no such member");
    if (bigcounter) *bigcounter = m->bigcounter;
    if (mtime) *mtime = m->mtime;
    return GA_OK;
}

int ga_solve_pressure_noalloc(const ga_config *cfg, const ga_columns *cols, double *up, double *vp, double *wp,
                              double *pi, double step, void *stream)
{
    if (!cfg || !cols || !up || !vp || !wp || !pi)
        return fail(GA_ERR_ARG, "ga_solve_pressure_noalloc: null pointer");
    if (!cols->mu || !cols->mw || !cols->rhou || !cols->rhow)
        return fail(GA_ERR_ARG, "ga_solve_pressure_noalloc: a column array is null");
    if (cfg->nx < 12 || cfg->ny < 12 || cfg->nz < 6 || cfg->nz > 128)
        return fail(GA_ERR_CONFIG, "ga_solve_pressure_noalloc: grid out of range (NX,NY >= 12, 6 <= NZ <= 128)");
    if (cfg->periodic_ew_boundaries && cfg->nx < 13)
        return fail(GA_ERR_CONFIG, "ga_solve_pressure_noalloc: periodic domains need NX >= 13");
    if (!(cfg->dx > 0 && cfg->dy > 0 && cfg->dz > 0 && cfg->dt > 0) || !(step > 0))
        return fail(GA_ERR_CONFIG, "ga_solve_pressure_noalloc: dx, dy, dz, dt and step must be positive");
    std::string why;
    if (ga::noalloc_check(cfg, &why) != GA_OK) return fail(GA_ERR_ARG, "ga_solve_pressure_noalloc: " + why);
    return ga::solve_pressure_noalloc(cfg, cols, up, vp, wp, pi, step, (cudaStream_t)stream);
}

int ga_profile_enable(ga_ctx *ctx, int on)
{
    if (!ctx) return fail(GA_ERR_ARG, "ga_profile_enable: null context");
    ctx->e->prof_reset();
    ctx->e->prof = on != 0;
    return GA_OK;
}

int ga_profile_count(ga_ctx *ctx)
{
    (void)ctx;
    return ga::PC_COUNT;
}

int ga_profile_get(ga_ctx *ctx, int idx, char *name, size_t cap, double *total_ms, long long *launches)
{
    if (!ctx || idx < 0 || idx >= ga::PC_COUNT) return fail(GA_ERR_ARG, "ga_profile_get: bad arguments");
    ctx->e->prof_collect();
    if (name && cap) {
        std::strncpy(name, ga::kProfNames[idx], cap - 1);
        name[cap - 1] = 0;
    }
    if (total_ms) *total_ms = ctx->e->prof_ms[idx];
    if (launches) *launches = ctx->e->prof_n[idx];
    return GA_OK;
}

}  /* extern "C" */
