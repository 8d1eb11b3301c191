/*
 * Harness that runs the reference's own monsoon initialisers,
 * initialize_basic_state_ITCZ_shear2 (data_initializer.cpp:298-568) and
 * initialize_vortex (data_initializer.cpp:862-1064), and dumps the basic state
 * and the vortex perturbation, to pin the generator of model_gb300/configs.py
 * (monsoon_vortex) against the reference itself.
 *
 * TEST INFRASTRUCTURE.  Built only here, from the reference's sources where
 * they lie, by oracle/build_ref.sh into oracle/_ref/.
 *
 * The ITCZ initialiser is written for the parallel build: it fills the
 * full-domain arrays iubar, ivbar, ... through macros that the serial build
 * maps onto the step's own arrays instead, while the same function also
 * passes iubar and ipbar to its helpers by name.  So data_initializer.cpp is
 * compiled here with the parallel-build mapping (a build-folder copy of
 * include/stdafx.h with ENERGY set to 1, which selects it while keeping the
 * serial index arithmetic), and this harness allocates those arrays, as
 * setup_memory_allocation does in the parallel build (initializer.cpp:509-520).
 * initialize_basic_state_ITCZ_shear2 ends with
 * init_basic_state_vertical_velocity (initializer.cpp:1113), compiled with
 * the serial mapping; the harness calls it again on the step's arrays after
 * copying the winds there, which is what the parallel build computes.
 *
 * The function overflows its arrays when NZ <= 38 (create_vertical_shear_profile
 * is called with ktrop = 37), so NZ must be at least 39 here.
 *
 * Usage: itcz_harness IN.bin OUT.bin
 * The bundle holds the grid (nx, ny, nz, dx, dy, dz, dt, height_lowest_level,
 * corner_lat, corner_lon), the three shear parameters (hor_shear, vert_shear0,
 * vert_shear1) and the vortex parameters (vortex_radius,
 * vortex_height_wind_max, vortex_vertical_extent, vortex_upper_warm_anomaly,
 * vortex_lower_cold_anomaly, vortex_latitude, vortex_longitude).
 */
#include "stdafx.h"
#include "boundaries.h"
#include "initializer.h"

#include <cstdint>
#include <map>
#include <string>
#include <vector>

void initialize_basic_state_ITCZ_shear2(double hor_shear, double vert_shear0, double vert_shear1);
void initialize_vortex(double r_end, double zm, double zt, double tmax, double tmin, double zb_rh, double zt_rh,
                       double rh_prime, double r_end_rh, double rh_max, int xpos, int ypos, double *u, double *v,
                       double *th, double *q);
void init_basic_state_vertical_velocity();
int get_point_from_lat(double lat);
int get_point_from_lon(double lon);

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
    if (fread(magic, 1, 4, fp) != 4 || memcmp(magic, "GABN", 4) || fread(&count, 4, 1, fp) != 1) exit(2);
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

static std::vector<double> grab(const double *p, size_t n) { return std::vector<double>(p, p + n); }

int main(int argc, char **argv)
{
    if (argc < 3) { fprintf(stderr, "usage: itcz_harness IN.bin OUT.bin\n"); return 2; }
    bundle in = read_bundle(argv[1]);
    memset(&inputs, 0, sizeof(inputs));
    inputs.nx = (int)scal(in, "nx");
    inputs.ny = (int)scal(in, "ny");
    inputs.nz = (int)scal(in, "nz");
    inputs.dx = scal(in, "dx");
    inputs.dy = scal(in, "dy");
    inputs.dz = scal(in, "dz");
    inputs.dt = scal(in, "dt");
    inputs.height_lowest_level = scal(in, "height_lowest_level");
    inputs.corner_lat = scal(in, "corner_lat");
    inputs.corner_lon = scal(in, "corner_lon");
    inputs.rayleigh_damping_z = inputs.nz - 5;
    inputs.output_frequency = 1 << 30;
    inputs.boundary_width_north = inputs.boundary_width_south = 5;
    inputs.boundary_width_east = inputs.boundary_width_west = 5;
    initialize_globals();
    if (NZ < 39) { fprintf(stderr, "NZ must be at least 39 (ktrop = 37)\n"); return 2; }

    const size_t N = (size_t)NX * NY * NZ;
    /* the parallel build's full-domain arrays (initializer.cpp:509-520) */
    iubar = (double *)calloc(N, 8);
    ivbar = (double *)calloc(N, 8);
    iwbar = (double *)calloc(N, 8);
    ithbar = (double *)calloc(N, 8);
    ipbar = (double *)calloc(N, 8);
    iqbar = (double *)calloc(N, 8);

    initialize_basic_state_ITCZ_shear2(scal(in, "hor_shear"), scal(in, "vert_shear0"), scal(in, "vert_shear1"));

    /* basic-state vertical velocity from the parallel build's winds */
    memcpy(m_ubar, iubar, N * 8);
    memcpy(m_vbar, ivbar, N * 8);
    memset(m_wbar, 0, N * 8);
    init_basic_state_vertical_velocity();

    /* vortex perturbation (initialize_vortex_perturbation, :760-859, serial branch) */
    memset(us, 0, N * 8);
    memset(vs, 0, N * 8);
    memset(ths, 0, N * 8);
    const int lat = get_point_from_lat(scal(in, "vortex_latitude"));
    const int lon = get_point_from_lon(scal(in, "vortex_longitude"));
    initialize_vortex(scal(in, "vortex_radius"), scal(in, "vortex_height_wind_max"),
                      scal(in, "vortex_vertical_extent"), scal(in, "vortex_upper_warm_anomaly"),
                      scal(in, "vortex_lower_cold_anomaly"), 0.0, 0.0, 0.0, 1.0e6, 1.0, lon, lat, us, vs, ths,
                      (double *)nullptr);

    bundle out;
    out["ubar"] = grab(iubar, N);
    out["vbar"] = grab(ivbar, N);
    out["wbar"] = grab(m_wbar, N);
    out["thbar"] = grab(ithbar, N);
    out["qbar"] = grab(iqbar, N);
    out["pbar"] = grab(ipbar, N);
    out["u"] = grab(us, N);
    out["v"] = grab(vs, N);
    out["th"] = grab(ths, N);
    out["tb"] = grab(tb, NZ);
    out["qb"] = grab(qb, NZ);
    out["tbv"] = grab(tbv, NZ);
    out["pib"] = grab(pib, NZ);
    out["rhou"] = grab(rhou, NZ);
    out["rhow"] = grab(rhow, NZ);
    out["lats"] = grab(outLats, NY);
    out["lons"] = grab(outLons, NX);
    out["f"] = grab(f, NY);
    out["vortex_ij"] = std::vector<double>{(double)lon, (double)lat};
    write_bundle(argv[2], out);
    return 0;
}
