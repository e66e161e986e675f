/* NetCDF constants needed to compile the reference Goma sources into the
 * CPU oracle (test infrastructure).  No NetCDF call is on the oracle path. */
#ifndef GB_REF_SHIM_NETCDF_H
#define GB_REF_SHIM_NETCDF_H
#define NC_NOERR 0
#define NC_NOWRITE 0
#define NC_WRITE 1
#define NC_SHARE 0x0800
#define NC_INT 4
#define NC_LONG 4
#define NC_MAX_NAME 256
#define NC_MAX_VAR_DIMS 1024
#define NC_GLOBAL (-1)
typedef int nc_type;
int nc_open();
int nc_close();
int nc_inq_dimid();
int nc_inq_dimlen();
int nc_inq_varid();
int nc_get_var();
int nc_put_var();
int nc_def_dim();
int nc_def_var();
int nc_enddef();
int nc_redef();
const char *nc_strerror();
#endif
