/*
 * Stand-ins for the NetCDF file layer of the reference (source/files.cpp),
 * which the oracle build does not compile: NetCDF-C is not installed and the
 * harness builds its state in memory.  None of these is reached on the step
 * path; each aborts loudly if it ever is.  TEST INFRASTRUCTURE.
 */
#include "stdafx.h"

static void unreachable(const char *what)
{
    fprintf(stderr, "oracle build: file layer call %s is not available\n", what);
    abort();
}

bool fileHasVar(const char *, const char *) { unreachable("fileHasVar"); return false; }
void get_data(const char *, const char *, int, double *) { unreachable("get_data"); }
double *get_data2(const char *, const char *, int) { unreachable("get_data2"); return nullptr; }
void get_data_at_time(const char *, const char *, size_t, double *) { unreachable("get_data_at_time"); }
void get_data_at_time(const char *, const char *, size_t, double *, int, int, int) { unreachable("get_data_at_time"); }
void get_dims(const char *, const char *, const char *, const char *, size_t[3]) { unreachable("get_dims"); }
size_t get_file_length(const char *, const char *) { unreachable("get_file_length"); return 0; }
int get_file_output_status() { unreachable("get_file_output_status"); return 0; }
void get_grid_spacing(const char *, const char *, const char *, const char *, float[3]) { unreachable("get_grid_spacing"); }
void get_model_data(const char *, size_t) { unreachable("get_model_data"); }
void outfile_init(char *) { unreachable("outfile_init"); }
void output_meteorological_fields_to_file(void (*)(const char *, const char *, double *, size_t),
                                          void (*)(const char *, const char *, double *, size_t), int)
{
    unreachable("output_meteorological_fields_to_file");
}
void set_outfilename(char *) { unreachable("set_outfilename"); }
void write_pvar_to_file(const char *, const char *, double *, size_t) { unreachable("write_pvar_to_file"); }
void write_pvar_to_file_2d(const char *, const char *, double *, size_t) { unreachable("write_pvar_to_file_2d"); }
void write_time_to_file(const char *, size_t) { unreachable("write_time_to_file"); }
