/*
 * Harness that runs the reference's own serial step (PARALLEL 0) on an
 * in-memory state and dumps every field, to pin the oracle restatement
 * (oracle/ga_oracle.c) against the reference itself.
 *
 * TEST INFRASTRUCTURE.  Built only here, from the reference's sources where
 * they lie, by oracle/build_ref.sh into oracle/_ref/.  It replaces the
 * reference's main.cpp and files.cpp; every other translation unit of the
 * serial build is compiled unmodified (include/stdafx.h is copied into the
 * build folder with PARALLEL set to 0, as the reference's serial Makefile
 * path expects).
 *
 * Initialisation mirrors initialize_basic_state_from_output_file
 * (initializer.cpp:1991-2150) and initialize_from_output_serial (:1799-1935)
 * with the file reads replaced by the arrays of the input bundle.  The time
 * loop mirrors s_run_model (driver_serial.cpp:310-372) without output.
 *
 * Usage: ref_harness IN.bin OUT.bin run NSTEPS
 *        ref_harness IN.bin OUT.bin op NAME STEP
 * Bundle format: "GABN", uint32 count, then per record char name[32],
 * int64 n, double data[n].
 */
#include "stdafx.h"
#include "advection.h"
#include "boundaries.h"
#include "damping.h"
#include "fluxes.h"
#include "initializer.h"
#include "pressure.h"
#include "turbulence.h"

#include <cstdint>
#include <map>
#include <string>
#include <vector>

void s_integrate_rk3();
void linear_integrate_rk3();
void advect_qv(double, int, int, int, int);
void advect_uv_velocity(double, int, int, int, int);
void integrate_hydro(double, int, int, int, int, int);
extern double *Kmix, *KHmix;  /* turbulence.cpp: mixing coefficients */
extern bool *isSaturated;     /* turbulence.cpp: Kessler saturation record */
void zero_moisture(int il, int ih, int jl, int jh, int size);
extern double N0S;            /* rutledge.cpp: snow intercept of the last snowy point */
void column_average_density();

/* globals normally defined by files.cpp */
char filename[len];
char inputPerturbationFileName[len];
char inputBasicStateFileName[len];
int rank = 0;

typedef std::map<std::string, std::vector<double>> bundle;

static bundle read_bundle(const char *path)
{
    bundle b;
    FILE *fp = fopen(path, "rb");
    if (!fp) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    char magic[4];
    uint32_t count = 0;
    if (fread(magic, 1, 4, fp) != 4 || memcmp(magic, "GABN", 4) || fread(&count, 4, 1, fp) != 1) {
        fprintf(stderr, "bad bundle %s\n", path);
        exit(2);
    }
    for (uint32_t r = 0; r < count; r++) {
        char name[33] = {0};
        int64_t n = 0;
        if (fread(name, 1, 32, fp) != 32 || fread(&n, 8, 1, fp) != 1) exit(2);
        std::vector<double> v((size_t)n);
        if (n && fread(v.data(), 8, (size_t)n, fp) != (size_t)n) exit(2);
        b[name] = v;
    }
    fclose(fp);
    return b;
}

static void write_bundle(const char *path, const bundle &b)
{
    FILE *fp = fopen(path, "wb");
    if (!fp) { fprintf(stderr, "cannot write %s\n", path); exit(2); }
    uint32_t count = (uint32_t)b.size();
    fwrite("GABN", 1, 4, fp);
    fwrite(&count, 4, 1, fp);
    for (auto &kv : b) {
        char name[32] = {0};
        strncpy(name, kv.first.c_str(), 31);
        int64_t n = (int64_t)kv.second.size();
        fwrite(name, 1, 32, fp);
        fwrite(&n, 8, 1, fp);
        fwrite(kv.second.data(), 8, kv.second.size(), fp);
    }
    fclose(fp);
}

static double scal(const bundle &b, const char *k)
{
    auto it = b.find(k);
    if (it == b.end() || it->second.empty()) { fprintf(stderr, "missing %s\n", k); exit(2); }
    return it->second[0];
}

static bool has(const bundle &b, const std::string &k) { return b.count(k) != 0; }

static void load(const bundle &b, const std::string &k, double *dst, size_t n)
{
    auto it = b.find(k);
    if (it == b.end()) return;
    if (it->second.size() != n) { fprintf(stderr, "size of %s\n", k.c_str()); exit(2); }
    memcpy(dst, it->second.data(), n * sizeof(double));
}

static std::vector<double> grab(const double *p, size_t n) { return std::vector<double>(p, p + n); }

int main(int argc, char **argv)
{
    if (argc < 5) { fprintf(stderr, "usage\n"); return 2; }
    bundle in = read_bundle(argv[1]);
    std::string mode = argv[3];

    memset(&inputs, 0, sizeof(inputs));
    inputs.nx = (int)scal(in, "nx");
    inputs.ny = (int)scal(in, "ny");
    inputs.nz = (int)scal(in, "nz");
    inputs.dx = scal(in, "dx");
    inputs.dy = scal(in, "dy");
    inputs.dz = scal(in, "dz");
    inputs.dt = scal(in, "dt");
    inputs.corner_lat = scal(in, "corner_lat");
    inputs.corner_lon = 0;
    inputs.time_steps = 1;
    inputs.output_frequency = 1 << 30;
    inputs.rayleigh_damping_z = (int)scal(in, "rayleigh_damping_z");
    inputs.height_lowest_level = scal(in, "height_lowest_level");
    inputs.microphysics_option = (int)scal(in, "microphysics_option");
    inputs.rain_fallout = (int)scal(in, "rain_fallout");
    inputs.periodic_ew_boundaries = (int)scal(in, "periodic_ew_boundaries");
    inputs.boundary_width_north = (int)scal(in, "boundary_width_north");
    inputs.boundary_width_south = (int)scal(in, "boundary_width_south");
    inputs.boundary_width_east = (int)scal(in, "boundary_width_east");
    inputs.boundary_width_west = (int)scal(in, "boundary_width_west");
    /* explicit diffusion (optional records; off when absent) */
    if (has(in, "use_explicit_diffusion")) {
        inputs.use_explicit_diffusion = (int)scal(in, "use_explicit_diffusion");
        inputs.diffusion_order = (int)scal(in, "diffusion_order");
        inputs.kdiffh = scal(in, "kdiffh");
        inputs.kdiffv = scal(in, "kdiffv");
    }
    if (has(in, "turbulence_option")) {  /* turbulence (optional records) */
        inputs.turbulence_option = (int)scal(in, "turbulence_option");
        inputs.use_surface_heat_flux = (int)scal(in, "use_surface_heat_flux");
        inputs.water_temp = scal(in, "water_temp");
    }
    initialize_globals();

    const size_t N = (size_t)NX * NY * NZ;
    /* initialize_basic_state_from_output_file, file reads replaced */
    setup_memory_allocation();
    setup_vertical_height_levels();
    setup_coordinates(0, -89.462997);
    initialize_coriolis_parameter(&outLats[0]);
    init_topography_to_zero();
    init_friction();
    load(in, "ubar", m_ubar, N);
    load(in, "vbar", m_vbar, N);
    load(in, "wbar", m_wbar, N);
    load(in, "thbar", m_thbar, N);
    load(in, "qbar", m_qbar, N);
    load(in, "pbar", m_pbar, N);
    load(in, "tb_in", tb, NZ);
    load(in, "qb_in", qb, NZ);
    initialize_vertical_basic_state2(tb, qb);
    column_average_density();
    /* initialize_from_output_serial, file reads replaced */
    load(in, "u", us, N);
    load(in, "v", vs, N);
    load(in, "w", ws, N);
    load(in, "th", ths, N);
    if (USE_MICROPHYSICS) {
        load(in, "qv", qvs, N);
        load(in, "qc", qcs, N);
        load(in, "qr", qrs, N);
        load(in, "accrain", accRain, (size_t)NX * NY);
    }
    if (USE_ICE) {
        load(in, "qs", qss, N);
        load(in, "qi", qis, N);
        load(in, "accsnow", accSnow, (size_t)NX * NY);
    }
    memcpy(ums, us, N * 8); memcpy(vms, vs, N * 8); memcpy(wms, ws, N * 8); memcpy(thms, ths, N * 8);
    if (USE_MICROPHYSICS) { memcpy(qvms, qvs, N * 8); memcpy(qcms, qcs, N * 8); memcpy(qrms, qrs, N * 8); }
    if (USE_ICE) { memcpy(qsms, qss, N * 8); memcpy(qims, qis, N * 8); }
    /* explicit slot overrides (per-operator tests set all three buffers) */
    load(in, "u_p", ups, N); load(in, "v_p", vps, N); load(in, "w_p", wps, N); load(in, "th_p", thps, N);
    load(in, "u_m", ums, N); load(in, "v_m", vms, N); load(in, "w_m", wms, N); load(in, "th_m", thms, N);
    load(in, "pi", pis, N);
    if (USE_MICROPHYSICS) {
        load(in, "qv_p", qvps, N); load(in, "qc_p", qcps, N); load(in, "qr_p", qrps, N);
        load(in, "qv_m", qvms, N); load(in, "qc_m", qcms, N); load(in, "qr_m", qrms, N);
        load(in, "vt", vts, N);
    }
    if (USE_ICE) {
        load(in, "qs_p", qsps, N); load(in, "qi_p", qips, N);
        load(in, "qs_m", qsms, N); load(in, "qi_m", qims, N);
        load(in, "sts", sts, N); load(in, "its", its, N);
        if (has(in, "n0s")) N0S = scal(in, "n0s");
    }
    /* rest of initialize_serial (driver_serial.cpp:44-76) */
    if (USE_TURBULENT_STRESS) {
        init_kmix(NX, NY, NZ, &ZU(0));
        if (has(in, "is_saturated")) {  /* a saturation record for operator tests */
            std::vector<double> sat(N);
            load(in, "is_saturated", sat.data(), N);
            for (size_t x = 0; x < N; x++) isSaturated[x] = sat[x] != 0;
        }
    }
    if (USE_MICROPHYSICS) init_microphysics(NX, NY);
    initialize_landsea("");
    initialize_pressure_solver();
    init_boundaries(iebuffer, iwbuffer, jnbuffer, jsbuffer, -1);
    init_damping(NX, NY, NZ);                       /* driver_serial.cpp:72-74 */
    init_diffusion_weights(DIFFUSION_ORDER, &ZU(0));

    if (has(in, "bigcounter0")) {  /* a run that starts later in the model's life (restart counters) */
        bigcounter = (int)scal(in, "bigcounter0");
        mtime = scal(in, "mtime0");
    }
    if (mode == "run") {
        int nsteps = atoi(argv[4]);
        for (int n = 0; n < nsteps; n++) {
#if ISLINEAR
            linear_integrate_rk3();  /* s_run_model, driver_serial.cpp:331 */
#else
            s_integrate_rk3();
#endif
            mtime += dt;
            bigcounter++;
        }
    } else if (mode == "op") {
        std::string name = argv[4];
        double step = argc > 5 ? atof(argv[5]) : 1.0;
        if (has(in, "step")) step = scal(in, "step");
        compute_sign_cells(0, NX, 0, NY);
        if (name == "advect_uvw") advect_uvw_velocity(step, 3, NX - 3, 3, NY - 3);
        else if (name == "solve_pressure") solve_pressure(step);
        else if (name == "integrate_non_hydro") integrate_non_hydro(step, 0, NX, 0, NY);
        else if (name == "advect_theta") advect_theta(step, 3, NX - 3, 3, NY - 3);
        else if (name == "advect_micro") advect_microphysics_cell(step, 3, NX - 3, 3, NY - 3);
        else if (name == "advect_qv") advect_qv(step, 3, NX - 3, 3, NY - 3);
        else if (name == "advect_uv") advect_uv_velocity(step, 3, NX - 3, 3, NY - 3);
        else if (name == "integrate_hydro") integrate_hydro(step, 0, 0, NX, 0, NY);
        else if (name == "zero_moisture") zero_moisture(1, NX - 1, 1, NY - 1, (int)N);
        else if (name == "bc") apply_boundary_condition(0);
        else if (name == "bc_micro") apply_boundary_condition_microphysics(0);
        else if (name == "kessler") run_microphysics(1, NX - 1, 1, NY - 1);
        else if (name == "rayleigh") rayleigh_damping(1, NX - 1, 1, NY - 1, raydampheight);
        else if (name == "explicit_diffusion") apply_explicit_diffusion(step, 3, NX - 3, 3, NY - 3);
        else if (name == "turbulence") calculate_diff_tend(1, NX - 1, 1, NY - 1);  /* driver_serial.cpp:194 */
        else if (name == "advect_ice") advect_ice_cell(step, 3, NX - 3, 3, NY - 3);  /* driver_serial.cpp:229 */
        else { fprintf(stderr, "unknown op %s\n", name.c_str()); return 2; }
    } else {
        fprintf(stderr, "unknown mode\n");
        return 2;
    }

    bundle out;
    out["u"] = grab(us, N); out["u_p"] = grab(ups, N); out["u_m"] = grab(ums, N);
    out["v"] = grab(vs, N); out["v_p"] = grab(vps, N); out["v_m"] = grab(vms, N);
    out["w"] = grab(ws, N); out["w_p"] = grab(wps, N); out["w_m"] = grab(wms, N);
    out["th"] = grab(ths, N); out["th_p"] = grab(thps, N); out["th_m"] = grab(thms, N);
    out["pi"] = grab(pis, N);
    if (USE_MICROPHYSICS) {
        out["qv"] = grab(qvs, N); out["qv_p"] = grab(qvps, N); out["qv_m"] = grab(qvms, N);
        out["qc"] = grab(qcs, N); out["qc_p"] = grab(qcps, N); out["qc_m"] = grab(qcms, N);
        out["qr"] = grab(qrs, N); out["qr_p"] = grab(qrps, N); out["qr_m"] = grab(qrms, N);
        out["vt"] = grab(vts, N);
        out["accrain"] = grab(accRain, (size_t)NX * NY);
    }
    if (USE_ICE) {
        out["qs"] = grab(qss, N); out["qs_p"] = grab(qsps, N); out["qs_m"] = grab(qsms, N);
        out["qi"] = grab(qis, N); out["qi_p"] = grab(qips, N); out["qi_m"] = grab(qims, N);
        out["sts"] = grab(sts, N); out["its"] = grab(its, N);
        out["accsnow"] = grab(accSnow, (size_t)NX * NY);
        out["n0s"] = std::vector<double>(1, N0S);
    }
    out["zu"] = grab(zu, NZ); out["zw"] = grab(zw, NZ); out["zsu"] = grab(zsu, NZ); out["zsw"] = grab(zsw, NZ);
    out["mu"] = grab(mu, NZ); out["mw"] = grab(mw, NZ);
    out["rhou"] = grab(rhou, NZ); out["rhow"] = grab(rhow, NZ);
    out["one_d_rhou"] = grab(one_d_rhou, NZ); out["one_d_rhow"] = grab(one_d_rhow, NZ);
    out["tb"] = grab(tb, NZ); out["tbv"] = grab(tbv, NZ); out["tbw"] = grab(tbw, NZ);
    out["qb"] = grab(qb, NZ); out["pib"] = grab(pib, NZ); out["f"] = grab(f, NY);
    if (USE_TURBULENT_STRESS) {  /* the turbulence tendencies of the last calculate_diff_tend */
        out["kmix"] = grab(Kmix, N); out["khmix"] = grab(KHmix, N);
        out["u_friction"] = grab(u_friction, N); out["v_friction"] = grab(v_friction, N);
        out["w_friction"] = grab(w_friction, N); out["t_diffusion"] = grab(t_diffusion, N);
        if (USE_MICROPHYSICS) {
            out["qv_diffusion"] = grab(qv_diffusion, N); out["qc_diffusion"] = grab(qc_diffusion, N);
            out["qr_diffusion"] = grab(qr_diffusion, N);
            std::vector<double> sat(N);
            for (size_t x = 0; x < N; x++) sat[x] = isSaturated[x] ? 1.0 : 0.0;
            out["is_saturated"] = sat;
        }
    }
    out["bigcounter"] = std::vector<double>(1, (double)bigcounter);
    out["mtime"] = std::vector<double>(1, mtime);
    write_bundle(argv[2], out);
    return 0;
}
