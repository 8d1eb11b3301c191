// ga_driver - the time loop of a run, on the C ABI of libga_anelastic.so.
//
// Replaces the reference's serial driver (s_run_model, driver_serial.cpp:
// 310-372, with initialize_serial, :44-76): it builds the vertical columns
// and the Coriolis parameter from the run's settings (ga_columns_build,
// ga_coriolis_build), creates a context, loads the basic state and the
// initial perturbation (current = start-of-step = the perturbation, forecast
// = 0, as initialize_from_output_serial leaves them), and advances the run
// in chunks of `every` steps, writing after each chunk an exact restart file
// of the whole state: all three rotation slots of every prognostic field, pi,
// the fall speed, the accumulated rain, Kessler's saturation record (with
// the turbulence scheme) and the counters, in FP64.  A run
// started from such a file continues bit for bit as if it had not stopped
// (with rain_fallout 1; under rain_fallout 2 the edge value that the PPM
// fallout carries from one rainy column to the next, microphysics.cpp:
// 616-631, also persists between steps inside the library, and the file
// does not hold it).
//
// The reference writes NetCDF output every outfilefreq steps (files.cpp:673,
// the restart protocol of files.cpp:1205-1257); NetCDF is not available
// here, so the state files use a self-describing binary bundle instead:
// "GABN", uint32 record count, then per record char name[32], int64 n,
// double data[n].
//
// usage: ga_driver INPUT OUT_PREFIX [--steps N] [--every K] [--restart FILE]
//                  [--precision f64|f32] [--device D]
//   INPUT     settings (nx ny nz dx dy dz dt microphysics_option rain_fallout
//             periodic_ew_boundaries boundary_width_{north,south,east,west}
//             rayleigh_damping_z height_lowest_level corner_lat; optional:
//             use_explicit_diffusion diffusion_order kdiffh kdiffv
//             turbulence_option use_surface_heat_flux water_temp), the base
//             columns tb_in and qb_in, the basic state (ubar vbar wbar thbar
//             qbar pbar) and the initial perturbation (u v w th [qv qc qr]
//             [accrain])
//   --restart the state file to continue from (the basic state still comes
//             from INPUT)
// Writes OUT_PREFIX_<step>.bin after every chunk; exits with the library's
// error code (negated to a positive status) on failure.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "ga_anelastic.h"

namespace {

typedef std::map<std::string, std::vector<double>> Bundle;

bool read_bundle(const char *path, Bundle *b)
{
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return false;
    char magic[4];
    uint32_t count = 0;
    bool ok = std::fread(magic, 1, 4, fp) == 4 && !std::memcmp(magic, "GABN", 4) &&
              std::fread(&count, 4, 1, fp) == 1;
    for (uint32_t r = 0; ok && r < count; r++) {
        char name[33] = {0};
        int64_t n = 0;
        ok = std::fread(name, 1, 32, fp) == 32 && std::fread(&n, 8, 1, fp) == 1 && n >= 0;
        if (!ok) break;
        std::vector<double> v((size_t)n);
        ok = n == 0 || std::fread(v.data(), 8, (size_t)n, fp) == (size_t)n;
        (*b)[name] = std::move(v);
    }
    std::fclose(fp);
    return ok;
}

bool write_bundle(const std::string &path, const Bundle &b)
{
    const std::string tmp = path + ".tmp";
    FILE *fp = std::fopen(tmp.c_str(), "wb");
    if (!fp) return false;
    const uint32_t count = (uint32_t)b.size();
    bool ok = std::fwrite("GABN", 1, 4, fp) == 4 && std::fwrite(&count, 4, 1, fp) == 1;
    for (const auto &kv : b) {
        char name[32] = {0};
        std::strncpy(name, kv.first.c_str(), 31);
        const int64_t n = (int64_t)kv.second.size();
        ok = ok && std::fwrite(name, 1, 32, fp) == 32 && std::fwrite(&n, 8, 1, fp) == 1 &&
             (n == 0 || std::fwrite(kv.second.data(), 8, (size_t)n, fp) == (size_t)n);
    }
    ok = std::fclose(fp) == 0 && ok;
    // the file appears complete or not at all (a reader never sees half a state)
    return ok && std::rename(tmp.c_str(), path.c_str()) == 0;
}

struct Run {
    Bundle in;
    ga_config cfg;
    double hll = 0, corner_lat = 0;
    size_t n3 = 0, n2 = 0;
    int nprog = 4;

    bool scalar(const char *k, double *v) const
    {
        auto it = in.find(k);
        if (it == in.end() || it->second.empty()) {
            std::fprintf(stderr, "ga_driver: input lacks %s\n", k);
            return false;
        }
        *v = it->second[0];
        return true;
    }
    bool optional(const char *k, double *v) const
    {
        auto it = in.find(k);
        if (it == in.end() || it->second.empty()) return false;
        *v = it->second[0];
        return true;
    }
    const std::vector<double> *array(const Bundle &b, const std::string &k, size_t n) const
    {
        auto it = b.find(k);
        if (it == b.end()) return nullptr;
        if (it->second.size() != n) {
            std::fprintf(stderr, "ga_driver: %s has %zu values, expected %zu\n", k.c_str(), it->second.size(), n);
            return nullptr;
        }
        return &it->second;
    }
    bool settings(int precision, int device)
    {
        std::memset(&cfg, 0, sizeof cfg);
        double v[17];
        const char *keys[17] = {"nx", "ny", "nz", "dx", "dy", "dz", "dt", "microphysics_option", "rain_fallout",
                                "periodic_ew_boundaries", "boundary_width_north", "boundary_width_south",
                                "boundary_width_east", "boundary_width_west", "rayleigh_damping_z",
                                "height_lowest_level", "corner_lat"};
        for (int i = 0; i < 17; i++)
            if (!scalar(keys[i], &v[i])) return false;
        cfg.nx = (int)v[0]; cfg.ny = (int)v[1]; cfg.nz = (int)v[2];
        cfg.dx = v[3]; cfg.dy = v[4]; cfg.dz = v[5]; cfg.dt = v[6];
        cfg.microphysics_option = (int)v[7]; cfg.rain_fallout = (int)v[8];
        cfg.periodic_ew_boundaries = (int)v[9];
        cfg.boundary_width_north = (int)v[10]; cfg.boundary_width_south = (int)v[11];
        cfg.boundary_width_east = (int)v[12]; cfg.boundary_width_west = (int)v[13];
        cfg.rayleigh_damping_z = (int)v[14];
        hll = v[15];
        corner_lat = v[16];
        // optional physics switches (input_params: use_explicit_diffusion,
        // diffusion_order, kdiffh, kdiffv, turbulence_option,
        // use_surface_heat_flux, water_temp); absent means off
        double o;
        cfg.diffusion_order = 4;
        cfg.kdiffh = cfg.kdiffv = 0.005;
        cfg.water_temp = 28.0;
        if (optional("use_explicit_diffusion", &o)) cfg.use_explicit_diffusion = (int)o;
        if (optional("diffusion_order", &o)) cfg.diffusion_order = (int)o;
        if (optional("kdiffh", &o)) cfg.kdiffh = o;
        if (optional("kdiffv", &o)) cfg.kdiffv = o;
        if (optional("turbulence_option", &o)) cfg.turbulence_option = (int)o;
        if (optional("use_surface_heat_flux", &o)) cfg.use_surface_heat_flux = (int)o;
        if (optional("water_temp", &o)) cfg.water_temp = o;
        cfg.precision = precision;
        cfg.device = device;
        n3 = (size_t)cfg.nx * cfg.ny * cfg.nz;
        n2 = (size_t)cfg.nx * cfg.ny;
        nprog = cfg.microphysics_option ? 7 : 4;
        return true;
    }
};

const char *kProg[7] = {"u", "v", "w", "th", "qv", "qc", "qr"};

// the prognostic fields of a configuration: (field id, bundle name)
std::vector<std::pair<int, std::string>> prog_fields(const Run &run)
{
    std::vector<std::pair<int, std::string>> v;
    for (int f = 0; f < run.nprog; f++) v.emplace_back(f, kProg[f]);
    if (run.cfg.microphysics_option == 2) {  // snow and cloud ice (microphysics.h:21-22)
        v.emplace_back(GA_QS, "qs");
        v.emplace_back(GA_QI, "qi");
    }
    return v;
}
const char *kBar[6] = {"ubar", "vbar", "wbar", "thbar", "qbar", "pbar"};
const char *kSlotSuffix[3] = {"", "_p", "_m"};

int fail(int rc, const char *what)
{
    std::fprintf(stderr, "ga_driver: %s failed (%d): %s\n", what, rc, ga_last_error());
    return rc < 0 ? -rc : 1;
}

// the whole state as a restart bundle
int save(ga_ctx *ctx, const Run &run, const std::string &path)
{
    Bundle out;
    std::vector<double> buf(run.n3);
    for (const auto &pf : prog_fields(run))
        for (int s = 0; s < 3; s++) {
            int rc = ga_get_field(ctx, pf.first, s, buf.data(), run.n3);
            if (rc) return fail(rc, "ga_get_field");
            out[pf.second + kSlotSuffix[s]] = buf;
        }
    int rc = ga_get_field(ctx, GA_PI, 0, buf.data(), run.n3);
    if (rc) return fail(rc, "ga_get_field(pi)");
    out["pi"] = buf;
    if (run.cfg.microphysics_option) {
        rc = ga_get_field(ctx, GA_VT, 0, buf.data(), run.n3);
        if (rc) return fail(rc, "ga_get_field(vt)");
        out["vt"] = buf;
        std::vector<double> acc(run.n2);
        rc = ga_get_field(ctx, GA_ACCRAIN, 0, acc.data(), run.n2);
        if (rc) return fail(rc, "ga_get_field(accrain)");
        out["accrain"] = acc;
        if (run.cfg.turbulence_option) {  // the saturation record feeds the next step's mixing
            rc = ga_get_field(ctx, GA_SATURATED, 0, buf.data(), run.n3);
            if (rc) return fail(rc, "ga_get_field(is_saturated)");
            out["is_saturated"] = buf;
        }
    }
    if (run.cfg.microphysics_option == 2) {  // the ice scheme's carried state
        const int f3[2] = {GA_VTS, GA_VTI};
        const char *n3[2] = {"sts", "its"};
        for (int a = 0; a < 2; a++) {
            rc = ga_get_field(ctx, f3[a], 0, buf.data(), run.n3);
            if (rc) return fail(rc, "ga_get_field(ice fall speed)");
            out[n3[a]] = buf;
        }
        std::vector<double> acc(run.n2), n0s(1);
        rc = ga_get_field(ctx, GA_ACCSNOW, 0, acc.data(), run.n2);
        if (rc) return fail(rc, "ga_get_field(accsnow)");
        out["accsnow"] = acc;
        rc = ga_get_field(ctx, GA_N0S, 0, n0s.data(), 1);
        if (rc) return fail(rc, "ga_get_field(n0s)");
        out["n0s"] = n0s;
    }
    long long bc = 0;
    double mt = 0;
    ga_get_counters(ctx, &bc, &mt);
    out["bigcounter"] = std::vector<double>(1, (double)bc);
    out["mtime"] = std::vector<double>(1, mt);
    if (!write_bundle(path, out)) {
        std::fprintf(stderr, "ga_driver: cannot write %s\n", path.c_str());
        return 2;
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: ga_driver INPUT OUT_PREFIX [--steps N] [--every K] [--restart FILE] "
                             "[--precision f64|f32] [--device D]\n");
        return 2;
    }
    long steps = -1, every = 0;
    int precision = GA_PREC_F64, device = 0;
    const char *restart = nullptr;
    for (int a = 3; a < argc; a++) {
        const std::string k = argv[a];
        const char *val = a + 1 < argc ? argv[a + 1] : nullptr;
        if (!val) { std::fprintf(stderr, "ga_driver: %s needs a value\n", k.c_str()); return 2; }
        if (k == "--steps") steps = std::atol(val);
        else if (k == "--every") every = std::atol(val);
        else if (k == "--restart") restart = val;
        else if (k == "--precision") precision = std::strcmp(val, "f32") == 0 ? GA_PREC_F32 : GA_PREC_F64;
        else if (k == "--device") device = std::atoi(val);
        else { std::fprintf(stderr, "ga_driver: unknown option %s\n", k.c_str()); return 2; }
        a++;
    }
    Run run;
    if (!read_bundle(argv[1], &run.in)) { std::fprintf(stderr, "ga_driver: cannot read %s\n", argv[1]); return 2; }
    if (!run.settings(precision, device)) return 2;
    if (steps < 0) {
        double ns = 0;
        if (!run.scalar("nsteps", &ns)) return 2;
        steps = (long)ns;
    }
    if (every <= 0) every = steps > 0 ? steps : 1;

    // columns and Coriolis parameter (initialize_serial's initializers)
    const std::vector<double> *tb = run.array(run.in, "tb_in", (size_t)run.cfg.nz);
    const std::vector<double> *qb = run.array(run.in, "qb_in", (size_t)run.cfg.nz);
    if (!tb || !qb) { std::fprintf(stderr, "ga_driver: input lacks tb_in/qb_in\n"); return 2; }
    static ga_column_store store;
    int rc = ga_columns_build(run.cfg.nz, run.cfg.dz, run.hll, tb->data(), qb->data(), &store);
    if (rc) return fail(rc, "ga_columns_build");
    std::vector<double> f((size_t)run.cfg.ny);
    rc = ga_coriolis_build(run.cfg.ny, run.cfg.dy, run.corner_lat, f.data());
    if (rc) return fail(rc, "ga_coriolis_build");
    ga_columns cols = {store.zu, store.zw, store.zsu, store.zsw, store.mu, store.mw, store.rhou, store.rhow,
                       store.one_d_rhou, store.one_d_rhow, store.tb, store.tbv, store.tbw, store.qb, store.pib,
                       f.data()};
    // every input array is present and sized before a context exists
    for (int b = 0; b < 6; b++)
        if (!run.array(run.in, kBar[b], run.n3)) {
            std::fprintf(stderr, "ga_driver: input lacks %s\n", kBar[b]);
            return 2;
        }
    if (!restart)
        for (const auto &pf : prog_fields(run))
            if (!run.array(run.in, pf.second, run.n3)) {
                std::fprintf(stderr, "ga_driver: input lacks %s\n", pf.second.c_str());
                return 2;
            }
    ga_ctx *ctx = nullptr;
    rc = ga_create(&run.cfg, &cols, &ctx);
    if (rc) return fail(rc, "ga_create");

    for (int b = 0; b < 6; b++) {
        const std::vector<double> *a = run.array(run.in, kBar[b], run.n3);
        if (!a) { std::fprintf(stderr, "ga_driver: input lacks %s\n", kBar[b]); ga_destroy(ctx); return 2; }
        rc = ga_set_field(ctx, GA_UBAR + b, 0, a->data(), run.n3);
        if (rc) { ga_destroy(ctx); return fail(rc, "ga_set_field(basic state)"); }
    }
    if (restart) {
        Bundle st;
        if (!read_bundle(restart, &st)) {
            std::fprintf(stderr, "ga_driver: cannot read %s\n", restart);
            ga_destroy(ctx);
            return 2;
        }
        for (const auto &pf : prog_fields(run))
            for (int s = 0; s < 3; s++) {
                const std::vector<double> *a = run.array(st, pf.second + kSlotSuffix[s], run.n3);
                if (!a) { ga_destroy(ctx); return 2; }
                rc = ga_set_field(ctx, pf.first, s, a->data(), run.n3);
                if (rc) { ga_destroy(ctx); return fail(rc, "ga_set_field(restart)"); }
            }
        const std::vector<double> *pi = run.array(st, "pi", run.n3);
        if (!pi) { ga_destroy(ctx); return 2; }
        ga_set_field(ctx, GA_PI, 0, pi->data(), run.n3);
        if (run.cfg.microphysics_option) {
            const std::vector<double> *vt = run.array(st, "vt", run.n3);
            const std::vector<double> *acc = run.array(st, "accrain", run.n2);
            if (!vt || !acc) { ga_destroy(ctx); return 2; }
            ga_set_field(ctx, GA_VT, 0, vt->data(), run.n3);
            ga_set_field(ctx, GA_ACCRAIN, 0, acc->data(), run.n2);
            if (run.cfg.turbulence_option) {
                const std::vector<double> *sat = run.array(st, "is_saturated", run.n3);
                if (!sat) { ga_destroy(ctx); return 2; }
                ga_set_field(ctx, GA_SATURATED, 0, sat->data(), run.n3);
            }
        }
        if (run.cfg.microphysics_option == 2) {
            const std::vector<double> *sts = run.array(st, "sts", run.n3), *its = run.array(st, "its", run.n3);
            const std::vector<double> *acc = run.array(st, "accsnow", run.n2), *n0s = run.array(st, "n0s", 1);
            if (!sts || !its || !acc || !n0s) { ga_destroy(ctx); return 2; }
            ga_set_field(ctx, GA_VTS, 0, sts->data(), run.n3);
            ga_set_field(ctx, GA_VTI, 0, its->data(), run.n3);
            ga_set_field(ctx, GA_ACCSNOW, 0, acc->data(), run.n2);
            ga_set_field(ctx, GA_N0S, 0, n0s->data(), 1);
        }
        const std::vector<double> *bc = run.array(st, "bigcounter", 1), *mt = run.array(st, "mtime", 1);
        if (!bc || !mt) { ga_destroy(ctx); return 2; }
        ga_set_counters(ctx, (long long)(*bc)[0], (*mt)[0]);
    } else {
        // initialize_from_output_serial: current = start of step = the perturbation
        const std::vector<double> zero(run.n3, 0.0);
        for (const auto &pf : prog_fields(run)) {
            const std::vector<double> *a = run.array(run.in, pf.second, run.n3);
            if (!a) {
                std::fprintf(stderr, "ga_driver: input lacks %s\n", pf.second.c_str());
                ga_destroy(ctx);
                return 2;
            }
            ga_set_field(ctx, pf.first, GA_SLOT_CUR, a->data(), run.n3);
            ga_set_field(ctx, pf.first, GA_SLOT_M, a->data(), run.n3);
            rc = ga_set_field(ctx, pf.first, GA_SLOT_P, zero.data(), run.n3);
            if (rc) { ga_destroy(ctx); return fail(rc, "ga_set_field(initial state)"); }
        }
        if (run.cfg.microphysics_option) {
            const std::vector<double> *acc = run.array(run.in, "accrain", run.n2);
            if (acc) ga_set_field(ctx, GA_ACCRAIN, 0, acc->data(), run.n2);
        }
        if (run.cfg.microphysics_option == 2) {
            const std::vector<double> *acc = run.array(run.in, "accsnow", run.n2);
            if (acc) ga_set_field(ctx, GA_ACCSNOW, 0, acc->data(), run.n2);
        }
    }

    // s_run_model: advance, write the state after every chunk
    long done = 0;
    while (done < steps) {
        const long n = every < steps - done ? every : steps - done;
        rc = ga_step(ctx, (int)n);
        if (rc) { ga_destroy(ctx); return fail(rc, "ga_step"); }
        done += n;
        long long bc = 0;
        ga_get_counters(ctx, &bc, nullptr);
        const std::string path = std::string(argv[2]) + "_" + std::to_string(bc) + ".bin";
        const int wr = save(ctx, run, path);
        if (wr) { ga_destroy(ctx); return wr; }
        std::printf("step %lld: wrote %s\n", bc, path.c_str());
    }
    ga_destroy(ctx);
    return 0;
}
