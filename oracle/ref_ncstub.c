/*
 * ref_ncstub.c -- TEST INFRASTRUCTURE ONLY.  An in-memory stand-in for the
 * part of libnetcdf that the reference's model/nc.c calls, so that the
 * reference's own write_nc / read_nc (model/nc.c:14-246) run inside the
 * oracle build (libnetcdf is not installed here).
 *
 * write_nc's calls are recorded (dimensions, variables, attributes in call
 * order, variable data) into one record, replaced by the next nc_create.
 * read_nc is served from a second record that the test fills through
 * photic_ref_nc_read.  The harness functions at the end drive both and hand
 * the results back in flat arrays.
 */
#include <limits.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <netcdf.h>

void write_nc(char *file, float **grid, int ncols, int nrows, float *lons, float *lats,
              double spval);
void read_nc(char *file, float ***grid, int *ncols, int *nrows, float **lons, float **lats,
             double *spval);
void free_float_array_2d(float **grid, int nrows);

#define MAXD 4
#define MAXV 4
#define MAXA 32

typedef struct {
  int varid;
  char name[64];
  int type;
  size_t len;
  unsigned char val[512];
} Att;

typedef struct {
  char path[512];
  int ndims;
  char dim_name[MAXD][64];
  size_t dim_len[MAXD];
  int nvars;
  char var_name[MAXV][64];
  int var_type[MAXV];
  int var_ndims[MAXV];
  int var_dims[MAXV][2];
  void *var_data[MAXV];
  int natts;
  Att atts[MAXA];
} Rec;

static Rec W, R;

static void rec_clear(Rec *r) {
  for (int v = 0; v < MAXV; v++) free(r->var_data[v]);
  memset(r, 0, sizeof *r);
}

static size_t type_size(int t) { return t == NC_SHORT ? 2 : t == NC_FLOAT ? 4 : 1; }

static size_t var_count(const Rec *r, int v) {
  size_t n = 1;
  for (int d = 0; d < r->var_ndims[v]; d++) n *= r->dim_len[r->var_dims[v][d]];
  return n;
}

const char *nc_strerror(int ncerr) {
  (void)ncerr;
  return "netcdf call failed in the oracle's stand-in";
}

int nc_create(const char *path, int cmode, int *ncidp) {
  (void)cmode;
  rec_clear(&W);
  snprintf(W.path, sizeof W.path, "%s", path);
  *ncidp = 1;
  return 0;
}

int nc_open(const char *path, int mode, int *ncidp) {
  (void)path;
  (void)mode;
  *ncidp = 2;
  return 0;
}

int nc_close(int ncid) { return ncid == 1 || ncid == 2 ? 0 : NC_EBADID; }
int nc_enddef(int ncid) { return ncid == 1 ? 0 : NC_EBADID; }

int nc_def_dim(int ncid, const char *name, size_t len, int *idp) {
  if (ncid != 1 || W.ndims >= MAXD) return NC_EBADID;
  snprintf(W.dim_name[W.ndims], 64, "%s", name);
  W.dim_len[W.ndims] = len;
  *idp = W.ndims++;
  return 0;
}

int nc_def_var(int ncid, const char *name, nc_type xtype, int ndims, const int *dimidsp,
               int *varidp) {
  if (ncid != 1 || W.nvars >= MAXV || ndims > 2) return NC_EBADID;
  const int v = W.nvars++;
  snprintf(W.var_name[v], 64, "%s", name);
  W.var_type[v] = xtype;
  W.var_ndims[v] = ndims;
  for (int d = 0; d < ndims; d++) W.var_dims[v][d] = dimidsp[d];
  *varidp = v;
  return 0;
}

static int put_att(int ncid, int varid, const char *name, int type, size_t len, const void *op) {
  if (ncid != 1 || W.natts >= MAXA || len * type_size(type) > sizeof W.atts[0].val)
    return NC_EBADID;
  Att *a = &W.atts[W.natts++];
  a->varid = varid;
  snprintf(a->name, 64, "%s", name);
  a->type = type;
  a->len = len;
  memcpy(a->val, op, len * type_size(type));
  return 0;
}

int nc_put_att_text(int ncid, int varid, const char *name, size_t len, const char *op) {
  return put_att(ncid, varid, name, NC_CHAR, len, op);
}
int nc_put_att_float(int ncid, int varid, const char *name, nc_type xtype, size_t len,
                     const float *op) {
  return xtype == NC_FLOAT ? put_att(ncid, varid, name, NC_FLOAT, len, op) : NC_EBADID;
}
int nc_put_att_short(int ncid, int varid, const char *name, nc_type xtype, size_t len,
                     const short *op) {
  return xtype == NC_SHORT ? put_att(ncid, varid, name, NC_SHORT, len, op) : NC_EBADID;
}

static int put_data(int varid, int type, const void *op) {
  if (varid < 0 || varid >= W.nvars || W.var_type[varid] != type) return NC_ENOTVAR;
  const size_t bytes = var_count(&W, varid) * type_size(type);
  free(W.var_data[varid]);
  W.var_data[varid] = malloc(bytes);
  memcpy(W.var_data[varid], op, bytes);
  return 0;
}

int nc_put_var_float(int ncid, int varid, const float *op) {
  return ncid == 1 ? put_data(varid, NC_FLOAT, op) : NC_EBADID;
}
int nc_put_vara_short(int ncid, int varid, const size_t *startp, const size_t *countp,
                      const short *op) {
  if (ncid != 1 || startp[0] != 0 || startp[1] != 0) return NC_EBADID;
  if (countp[0] * countp[1] != var_count(&W, varid)) return NC_EBADID;
  return put_data(varid, NC_SHORT, op);
}

static const Rec *rec_of(int ncid) { return ncid == 1 ? &W : ncid == 2 ? &R : NULL; }

int nc_inq_varid(int ncid, const char *name, int *varidp) {
  const Rec *r = rec_of(ncid);
  if (!r) return NC_EBADID;
  for (int v = 0; v < r->nvars; v++)
    if (strcmp(r->var_name[v], name) == 0) {
      *varidp = v;
      return 0;
    }
  return NC_ENOTVAR;
}

int nc_inq_dimid(int ncid, const char *name, int *idp) {
  const Rec *r = rec_of(ncid);
  if (!r) return NC_EBADID;
  for (int d = 0; d < r->ndims; d++)
    if (strcmp(r->dim_name[d], name) == 0) {
      *idp = d;
      return 0;
    }
  return NC_EBADDIM;
}

int nc_inq_dimlen(int ncid, int dimid, size_t *lenp) {
  const Rec *r = rec_of(ncid);
  if (!r || dimid < 0 || dimid >= r->ndims) return NC_EBADDIM;
  *lenp = r->dim_len[dimid];
  return 0;
}

static const Att *find_att(const Rec *r, int varid, const char *name) {
  for (int i = 0; i < r->natts; i++)
    if (r->atts[i].varid == varid && strcmp(r->atts[i].name, name) == 0) return &r->atts[i];
  return NULL;
}

int nc_get_att_float(int ncid, int varid, const char *name, float *ip) {
  const Rec *r = rec_of(ncid);
  const Att *a = r ? find_att(r, varid, name) : NULL;
  if (!a || a->type != NC_FLOAT) return NC_ENOTATT;
  memcpy(ip, a->val, a->len * 4);
  return 0;
}

int nc_get_att_short(int ncid, int varid, const char *name, short *ip) {
  const Rec *r = rec_of(ncid);
  const Att *a = r ? find_att(r, varid, name) : NULL;
  if (!a || a->type != NC_SHORT) return NC_ENOTATT;
  memcpy(ip, a->val, a->len * 2);
  return 0;
}

int nc_get_var(int ncid, int varid, void *ip) {
  const Rec *r = rec_of(ncid);
  if (!r || varid < 0 || varid >= r->nvars || !r->var_data[varid]) return NC_ENOTVAR;
  memcpy(ip, r->var_data[varid], var_count(r, varid) * type_size(r->var_type[varid]));
  return 0;
}

/* ---- harness ------------------------------------------------------------ */

static float **rows_of(const float *grid, int ncols, int nrows) {
  float **g = (float **)malloc((size_t)nrows * sizeof(float *));
  for (int i = 0; i < nrows; i++) {
    g[i] = (float *)malloc((size_t)ncols * sizeof(float));
    memcpy(g[i], grid + (size_t)i * ncols, (size_t)ncols * sizeof(float));
  }
  return g;
}

/* The reference's write_nc on a row-major grid; returns the packed values
 * and the four packing attributes of the "bathy" variable it wrote. */
int photic_ref_nc_write(const float *grid, int ncols, int nrows, const float *lons,
                        const float *lats, double spval, int16_t *packed, float *add_offset,
                        float *scale_factor, int16_t *missing_value, float *spval_attr) {
  float **g = rows_of(grid, ncols, nrows);
  char file[] = "photic_ref_grid.nc";
  write_nc(file, g, ncols, nrows, (float *)lons, (float *)lats, spval);
  free_float_array_2d(g, nrows);
  int v;
  if (nc_inq_varid(1, "bathy", &v) || !W.var_data[v]) return 1;
  memcpy(packed, W.var_data[v], (size_t)ncols * nrows * 2);
  if (nc_get_att_float(1, v, "add_offset", add_offset)) return 2;
  if (nc_get_att_float(1, v, "scale_factor", scale_factor)) return 2;
  short mv;
  if (nc_get_att_short(1, v, "missing_value", &mv)) return 2;
  *missing_value = mv;
  if (nc_get_att_float(1, v, "decompressed_missing_value", spval_attr)) return 2;
  return 0;
}

/* The structure of the last write, one line per item in call order:
 *   dim <name> <len> | var <name> <type> <dim names...> | att <var|NC_GLOBAL> <name> <type> <len>
 * followed by the text value of character attributes. */
int photic_ref_nc_layout(char *buf, int len) {
  int o = 0;
  for (int d = 0; d < W.ndims && o < len; d++)
    o += snprintf(buf + o, (size_t)(len - o), "dim %s %zu\n", W.dim_name[d], W.dim_len[d]);
  for (int v = 0; v < W.nvars && o < len; v++) {
    o += snprintf(buf + o, (size_t)(len - o), "var %s %d", W.var_name[v], W.var_type[v]);
    for (int d = 0; d < W.var_ndims[v] && o < len; d++)
      o += snprintf(buf + o, (size_t)(len - o), " %s", W.dim_name[W.var_dims[v][d]]);
    if (o < len) o += snprintf(buf + o, (size_t)(len - o), "\n");
  }
  for (int i = 0; i < W.natts && o < len; i++) {
    const Att *a = &W.atts[i];
    const char *owner = a->varid == NC_GLOBAL ? "NC_GLOBAL" : W.var_name[a->varid];
    o += snprintf(buf + o, (size_t)(len - o), "att %s %s %d %zu", owner, a->name, a->type, a->len);
    if (a->type == NC_CHAR && o < len)
      o += snprintf(buf + o, (size_t)(len - o), " %.*s", (int)a->len, (const char *)a->val);
    if (o < len) o += snprintf(buf + o, (size_t)(len - o), "\n");
  }
  return o < len ? 0 : 1;
}

/* The reference's read_nc on a file holding the given packed grid and
 * attributes (has_missing / has_spval: whether missing_value and
 * decompressed_missing_value are present); returns the row-major grid and
 * the spval read_nc reports. */
int photic_ref_nc_read(const int16_t *packed, int ncols, int nrows, const float *lons,
                       const float *lats, float add_offset, float scale_factor, int has_missing,
                       int16_t missing_value, int has_spval, float spval_attr, float *grid_out,
                       double *spval_out) {
  rec_clear(&R);
  R.ndims = 2;
  snprintf(R.dim_name[0], 64, "lons");
  R.dim_len[0] = (size_t)ncols;
  snprintf(R.dim_name[1], 64, "lats");
  R.dim_len[1] = (size_t)nrows;
  const char *names[3] = {"lats", "lons", "bathy"};
  const int types[3] = {NC_FLOAT, NC_FLOAT, NC_SHORT};
  const void *data[3] = {lats, lons, packed};
  R.nvars = 3;
  for (int v = 0; v < 3; v++) {
    snprintf(R.var_name[v], 64, "%s", names[v]);
    R.var_type[v] = types[v];
  }
  R.var_ndims[0] = 1;
  R.var_dims[0][0] = 1;
  R.var_ndims[1] = 1;
  R.var_dims[1][0] = 0;
  R.var_ndims[2] = 2;
  R.var_dims[2][0] = 1;
  R.var_dims[2][1] = 0;
  for (int v = 0; v < 3; v++) {
    const size_t bytes = var_count(&R, v) * type_size(types[v]);
    R.var_data[v] = malloc(bytes);
    memcpy(R.var_data[v], data[v], bytes);
  }
  Att *a = &R.atts[R.natts++];
  a->varid = 2, snprintf(a->name, 64, "add_offset"), a->type = NC_FLOAT, a->len = 1;
  memcpy(a->val, &add_offset, 4);
  a = &R.atts[R.natts++];
  a->varid = 2, snprintf(a->name, 64, "scale_factor"), a->type = NC_FLOAT, a->len = 1;
  memcpy(a->val, &scale_factor, 4);
  if (has_missing) {
    a = &R.atts[R.natts++];
    a->varid = 2, snprintf(a->name, 64, "missing_value"), a->type = NC_SHORT, a->len = 1;
    short mv = missing_value;
    memcpy(a->val, &mv, 2);
  }
  if (has_spval) {
    a = &R.atts[R.natts++];
    a->varid = 2, snprintf(a->name, 64, "decompressed_missing_value"), a->type = NC_FLOAT;
    a->len = 1;
    memcpy(a->val, &spval_attr, 4);
  }
  float **g = NULL, *lo = NULL, *la = NULL;
  int nc = 0, nr = 0;
  char file[] = "photic_ref_grid.nc";
  read_nc(file, &g, &nc, &nr, &lo, &la, spval_out);
  if (nc != ncols || nr != nrows) return 1;
  for (int i = 0; i < nrows; i++) memcpy(grid_out + (size_t)i * ncols, g[i], (size_t)ncols * 4);
  free_float_array_2d(g, nrows);
  free(lo);
  free(la);
  return 0;
}
