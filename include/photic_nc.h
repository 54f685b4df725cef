/*
 * photic_nc.h -- the reference's netCDF grid files on both sides of the
 * inversion (model/nc.c, model/nc.h:8-12): one float grid per file, stored
 * as the short variable "bathy"[lats][lons] with the float attributes
 * add_offset and scale_factor, the short attribute missing_value and the
 * float attribute decompressed_missing_value, beside the float coordinate
 * variables "lons" and "lats".  Band grids are read straight into the
 * pixel-major layout the inversion takes; result grids are written from
 * device memory.  Packing and unpacking run on the GPU; the host reads and
 * writes the netCDF classic container (CDF-1, or CDF-2 for files past
 * 2 GiB).  netCDF-4 (HDF5) files are not read.
 *
 * Mapping to the reference (file:line inside stblake/photic):
 *   read_nc / write_nc        read_nc / write_nc, model/nc.c:138 and :14,
 *                             same signatures, results and error behaviour
 *                             (a message and exit(1)); the grid read_nc
 *                             returns is freed with the reference's
 *                             free_float_array_2d (one malloc per row).
 *   photic_nc_unpack_bands    decompress_2d, model/nc.c:251-266, for up to
 *                             PHOTIC_MAX_BANDS grids at once, interleaved.
 *   photic_nc_pack            compress_2d, model/nc.c:271-320, including
 *                             its one-pass min/max (a value that lowers the
 *                             running minimum is not compared with the
 *                             maximum; the maximum starts at FLT_MIN) and
 *                             the x86-64 result of converting out-of-range
 *                             quotients to short (truncation to a 32-bit
 *                             int, INT_MIN when out of range or NaN, then
 *                             its low 16 bits).
 *   photic_nc_read_bands      read_grid (model/io.c:14-47) for the bands of
 *                             a SCENE (model/bam.c:1310-1360), commensurate
 *                             grids required.
 *   photic_nc_write_grid      write_nc from a device grid.
 *   photic_nc_read_info / photic_nc_read_raw / photic_nc_write_raw
 *                             the container alone (host only, no GPU).
 *
 * Packed values cross the boundary as they are stored in the file:
 * big-endian 16-bit words, 2 bytes per cell, rows of lons, lats outermost.
 */
#ifndef PHOTIC_NC_H
#define PHOTIC_NC_H

#include <stdint.h>

#include "photic.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct photic_nc_grid_info {
  int32_t ncols, nrows;      /* lengths of the dimensions "lons", "lats" */
  float add_offset;          /* attribute add_offset */
  float scale_factor;        /* attribute scale_factor */
  int16_t missing_value;     /* attribute missing_value (SHRT_MIN if absent) */
  int32_t has_missing_value; /* 1 when the attribute is present */
  double spval;              /* attribute decompressed_missing_value (0 if absent) */
  int32_t has_spval;         /* 1 when the attribute is present */
  int32_t format;            /* 1: CDF-1 (classic), 2: CDF-2 (64-bit offsets) */
} photic_nc_grid_info;

/* Header of a grid file: dimensions and packing attributes. */
int photic_nc_read_info(const char *path, photic_nc_grid_info *info);

/* The packed grid (2 * nrows * ncols bytes, big-endian) and the coordinate
 * variables (ncols and nrows floats); any of the three buffers may be NULL.
 * Fills info as photic_nc_read_info does. */
int photic_nc_read_raw(const char *path, photic_nc_grid_info *info, void *h_packed_be,
                       float *h_lons, float *h_lats);

/* A grid file with the layout write_nc produces (model/nc.c:14-134):
 * dimensions lons, lats; global attributes filename (= path) and data_type;
 * variables lats, lons (float) and bathy (short) with their attributes.
 * info supplies ncols, nrows and the four packing attributes (all four are
 * written); format 0 picks CDF-1 unless the file needs 64-bit offsets. */
int photic_nc_write_raw(const char *path, const photic_nc_grid_info *info,
                        const void *h_packed_be, const float *h_lons, const float *h_lats);

/* decompress_2d of n_bands packed grids of npix cells each (device
 * pointers, big-endian) into d_rrs[npix][n_bands] (band b of pixel p at
 * d_rrs[p * n_bands + b]).  Asynchronous on stream. */
int photic_nc_unpack_bands(const void *const *d_packed_be, const photic_nc_grid_info *infos,
                           int32_t n_bands, int64_t npix, float *d_rrs, void *stream);

/* compress_2d of a device grid of n cells: the packed grid into
 * d_packed_be (2 * n bytes, big-endian), add_offset, scale_factor and
 * missing_value (SHRT_MIN) into info (spval and has_* too).  The packing
 * constants come back to the host, so the call waits for the stream. */
int photic_nc_pack(const float *d_grid, int64_t n, double spval, void *d_packed_be,
                   photic_nc_grid_info *info, void *stream);

/* The band grid files of one scene into d_rrs[nrows * ncols][n_bands]
 * (capacity_px pixels available), with band 0's header in info and its
 * coordinates in h_lons / h_lats (either may be NULL).  Every band must
 * have band 0's dimensions.  Waits for the stream. */
int photic_nc_read_bands(const char *const *paths, int32_t n_bands, float *d_rrs,
                         int64_t capacity_px, photic_nc_grid_info *info, float *h_lons,
                         float *h_lats, void *stream);

/* write_nc of a device grid (nrows * ncols floats, rows of lons); the file
 * name, and its filename attribute, with leading and trailing white space
 * removed as the reference's trim() does (read_nc / write_nc trim the
 * caller's string in place, as the reference does). */
int photic_nc_write_grid(const char *path, const float *d_grid, int32_t ncols, int32_t nrows,
                         const float *h_lons, const float *h_lats, double spval, void *stream);

/* The reference's entry points (model/nc.h:8-12). */
void write_nc(char *file, float **grid, int ncols, int nrows, float *lons, float *lats,
              double spval);
void read_nc(char *file, float ***grid, int *ncols, int *nrows, float **lons, float **lats,
             double *spval);

#ifdef __cplusplus
}
#endif
#endif
