/* Minimal stand-in for libnetcdf's header: the declarations the reference's
 * model/nc.c uses, so that nc.c compiles into the test oracle.  The
 * functions are implemented by oracle/ref_ncstub.c, which records what
 * write_nc writes and serves read_nc from a record the test sets. */
#ifndef PHOTIC_STUB_NETCDF_H
#define PHOTIC_STUB_NETCDF_H
#include <stddef.h>

#define NC_NOWRITE 0
#define NC_CLOBBER 0
#define NC_GLOBAL (-1)
#define NC_CHAR 2
#define NC_SHORT 3
#define NC_FLOAT 5
#define NC_EBADID (-33)
#define NC_ENOTATT (-43)
#define NC_EBADDIM (-46)
#define NC_ENOTVAR (-49)

typedef int nc_type;

const char *nc_strerror(int ncerr);
int nc_create(const char *path, int cmode, int *ncidp);
int nc_open(const char *path, int mode, int *ncidp);
int nc_close(int ncid);
int nc_enddef(int ncid);
int nc_def_dim(int ncid, const char *name, size_t len, int *idp);
int nc_def_var(int ncid, const char *name, nc_type xtype, int ndims, const int *dimidsp,
               int *varidp);
int nc_put_att_text(int ncid, int varid, const char *name, size_t len, const char *op);
int nc_put_att_float(int ncid, int varid, const char *name, nc_type xtype, size_t len,
                     const float *op);
int nc_put_att_short(int ncid, int varid, const char *name, nc_type xtype, size_t len,
                     const short *op);
int nc_put_var_float(int ncid, int varid, const float *op);
int nc_put_vara_short(int ncid, int varid, const size_t *startp, const size_t *countp,
                      const short *op);
int nc_inq_varid(int ncid, const char *name, int *varidp);
int nc_inq_dimid(int ncid, const char *name, int *idp);
int nc_inq_dimlen(int ncid, int dimid, size_t *lenp);
int nc_get_att_float(int ncid, int varid, const char *name, float *ip);
int nc_get_att_short(int ncid, int varid, const char *name, short *ip);
int nc_get_var(int ncid, int varid, void *ip);

#endif
