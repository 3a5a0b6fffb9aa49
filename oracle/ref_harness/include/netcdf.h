/* netcdf.h -- stand-in for the NetCDF C header (TEST INFRASTRUCTURE ONLY).
 * The reference's netcdf_interface.h needs one constant from it; no NetCDF
 * call is compiled: the one Netcdf_handle member the hot path reaches
 * (get_variable of the initial profiles, used by Buffer::create) is defined
 * in ref_stubs.cxx and reads profiles handed over through the oracle API. */
#ifndef MHH_NETCDF_STANDIN_H
#define MHH_NETCDF_STANDIN_H
#define NC_UNLIMITED 0L
#endif
