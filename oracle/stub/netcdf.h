/* Minimal stand-in for netcdf.h: the reference's nc.h includes it, and the
 * inversion path only needs the declaration of nc_strerror. */
const char *nc_strerror(int ncerr);
