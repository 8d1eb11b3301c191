/* netcdf.h stand-in: the reference's headers include it, but the serial step
 * reads and writes no NetCDF file in the oracle build.  TEST INFRASTRUCTURE. */
#ifndef GA_NETCDF_SHIM_H
#define GA_NETCDF_SHIM_H
#define NC_NOERR 0
#endif
