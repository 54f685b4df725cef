/* Link stubs for building the reference inversion path without libnetcdf.
 * samodel() writes its products with write_nc (model/nc.c); the oracle only
 * reads the in-memory results, so the writer is a no-op here. */
const char *nc_strerror(int ncerr) { (void)ncerr; return "netcdf unavailable in the oracle build"; }
void write_nc(char *file, float **grid, int ncols, int nrows, float *lons, float *lats, double spval)
{ (void)file; (void)grid; (void)ncols; (void)nrows; (void)lons; (void)lats; (void)spval; }
