// photic_ncgrid.cu -- the reference's netCDF grid files (model/nc.c) on
// both sides of the inversion.
//
// Host: the netCDF classic container (CDF-1 / CDF-2, big-endian; the
// published "NetCDF Classic Format Specification"), restricted to what
// write_nc produces: two fixed dimensions, no record variables.
// Device: the short packing.  decompress_2d (model/nc.c:251-266) is one
// streaming kernel that also interleaves the bands into the inversion's
// pixel-major layout.  compress_2d (model/nc.c:271-320) is sequential in
// the reference -- its minimum and maximum come from one `if / else if`
// pass -- and is restated as four kernels with the same result: per-tile
// minima, an exclusive prefix minimum over tiles, per-tile records and
// maxima (a cell lowers the running minimum exactly when it is below the
// minimum of every earlier cell), and the quantisation.
#include <cuda_runtime.h>
#include <float.h>
#include <ctype.h>
#include <limits.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/photic.h"
#include "../../include/photic_nc.h"

namespace photic {
int report_error(int code, const char *message);
}

namespace {

using photic::report_error;

int io_fail(const std::string &path, const char *what) {
  return report_error(PHOTIC_ERR_IO, (path + ": " + what).c_str());
}
int cuda_fail_nc(cudaError_t e, const char *what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return report_error(PHOTIC_ERR_CUDA, m.c_str());
}

// ---------------------------------------------------------------------------
// Container
// ---------------------------------------------------------------------------
enum : uint32_t { kAbsent = 0, kTagDim = 0x0A, kTagVar = 0x0B, kTagAtt = 0x0C };
enum : int { kByte = 1, kChar = 2, kShort = 3, kInt = 4, kFloat = 5, kDouble = 6 };

int type_bytes(int t) {
  switch (t) {
    case kByte: case kChar: return 1;
    case kShort: return 2;
    case kInt: case kFloat: return 4;
    case kDouble: return 8;
    default: return 0;
  }
}

uint32_t be32(const uint8_t *p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}
uint64_t be64(const uint8_t *p) { return ((uint64_t)be32(p) << 32) | be32(p + 4); }
float be_float(const uint8_t *p) {
  const uint32_t u = be32(p);
  float f;
  memcpy(&f, &u, 4);
  return f;
}

struct Att {
  std::string name;
  int type = 0;
  uint32_t n = 0;
  std::vector<uint8_t> raw;  // big-endian values
};

struct Var {
  std::string name;
  std::vector<uint32_t> dims;
  std::vector<Att> atts;
  int type = 0;
  uint64_t vsize = 0, begin = 0;
};

struct NcFile {
  int version = 0;
  std::vector<std::string> dim_name;
  std::vector<uint64_t> dim_len;
  std::vector<Att> gatts;
  std::vector<Var> vars;
};

// Sequential reader over the header bytes; ok() turns false when a read runs
// past the bytes held (the caller then retries with more of the file).
struct Cursor {
  const uint8_t *p;
  size_t n, o = 0;
  bool short_read = false, bad = false;
  bool take(size_t k) {
    if (o + k > n) {
      short_read = true;
      return false;
    }
    return true;
  }
  uint32_t u32() {
    if (!take(4)) return 0;
    const uint32_t v = be32(p + o);
    o += 4;
    return v;
  }
  uint64_t u64() {
    if (!take(8)) return 0;
    const uint64_t v = be64(p + o);
    o += 8;
    return v;
  }
  std::string name() {
    const uint32_t len = u32();
    if (len > (1u << 16)) {
      bad = true;
      return std::string();
    }
    const size_t padded = (len + 3u) & ~3u;
    if (!take(padded)) return std::string();
    std::string s((const char *)p + o, len);
    o += padded;
    return s;
  }
  bool ok() const { return !short_read && !bad; }
};

bool parse_atts(Cursor &c, std::vector<Att> &out) {
  const uint32_t tag = c.u32(), n = c.u32();
  if (!c.ok()) return false;
  if (tag == kAbsent && n == 0) return true;
  if (tag != kTagAtt || n > 4096) {
    c.bad = true;
    return false;
  }
  for (uint32_t i = 0; i < n; i++) {
    Att a;
    a.name = c.name();
    a.type = (int)c.u32();
    a.n = c.u32();
    const int tb = type_bytes(a.type);
    if (!c.ok()) return false;
    if (tb == 0 || a.n > (1u << 24)) {
      c.bad = true;
      return false;
    }
    const size_t bytes = (size_t)a.n * tb, padded = (bytes + 3) & ~(size_t)3;
    if (!c.take(padded)) return false;
    a.raw.assign(c.p + c.o, c.p + c.o + bytes);
    c.o += padded;
    out.push_back(std::move(a));
  }
  return true;
}

// 0: parsed; 1: more header bytes needed; 2: not a classic netCDF file.
int parse_header(const uint8_t *p, size_t n, NcFile &f, std::string &why) {
  Cursor c{p, n};
  if (!c.take(4)) return 1;
  if (p[0] == 0x89 && p[1] == 'H' && p[2] == 'D' && p[3] == 'F') {
    why = "netCDF-4 (HDF5) files are not supported; convert to netCDF classic";
    return 2;
  }
  if (p[0] != 'C' || p[1] != 'D' || p[2] != 'F' || (p[3] != 1 && p[3] != 2)) {
    why = p[0] == 'C' && p[1] == 'D' && p[2] == 'F' ? "netCDF CDF-5 files are not supported"
                                                     : "not a netCDF file";
    return 2;
  }
  f.version = p[3];
  c.o = 4;
  c.u32();  // numrecs: no record variables are read
  const uint32_t dtag = c.u32(), nd = c.u32();
  if (!c.ok()) return 1;
  if (!(dtag == kAbsent && nd == 0) && (dtag != kTagDim || nd > 1024)) {
    why = "malformed dimension list";
    return 2;
  }
  for (uint32_t i = 0; i < nd && dtag == kTagDim; i++) {
    f.dim_name.push_back(c.name());
    f.dim_len.push_back(c.u32());
    if (!c.ok()) return c.bad ? (why = "malformed dimension", 2) : 1;
  }
  if (!parse_atts(c, f.gatts)) return c.bad ? (why = "malformed global attributes", 2) : 1;
  const uint32_t vtag = c.u32(), nv = c.u32();
  if (!c.ok()) return 1;
  if (!(vtag == kAbsent && nv == 0) && (vtag != kTagVar || nv > 1024)) {
    why = "malformed variable list";
    return 2;
  }
  for (uint32_t i = 0; i < nv && vtag == kTagVar; i++) {
    Var v;
    v.name = c.name();
    const uint32_t ndims = c.u32();
    if (!c.ok()) return c.bad ? (why = "malformed variable", 2) : 1;
    if (ndims > 64) {
      why = "malformed variable";
      return 2;
    }
    for (uint32_t d = 0; d < ndims; d++) v.dims.push_back(c.u32());
    if (!parse_atts(c, v.atts)) return c.bad ? (why = "malformed variable attributes", 2) : 1;
    v.type = (int)c.u32();
    v.vsize = c.u32();
    v.begin = f.version == 2 ? c.u64() : c.u32();
    if (!c.ok()) return c.bad ? (why = "malformed variable", 2) : 1;
    for (uint32_t d : v.dims)
      if (d >= f.dim_name.size()) {
        why = "variable refers to a missing dimension";
        return 2;
      }
    f.vars.push_back(std::move(v));
  }
  return 0;
}

int read_header(FILE *fp, const std::string &path, NcFile &f) {
  std::vector<uint8_t> buf;
  size_t want = 4096;
  for (;;) {
    buf.resize(want);
    if (fseeko(fp, 0, SEEK_SET) != 0) return io_fail(path, "cannot seek");
    const size_t got = fread(buf.data(), 1, want, fp);
    std::string why;
    f = NcFile();
    const int r = parse_header(buf.data(), got, f, why);
    if (r == 0) return PHOTIC_OK;
    if (r == 2) return io_fail(path, why.c_str());
    if (got < want) return io_fail(path, "truncated netCDF header");
    if (want >= ((size_t)1 << 26)) return io_fail(path, "netCDF header too large");
    want *= 4;
  }
}

int find_var(const NcFile &f, const char *name) {
  for (size_t i = 0; i < f.vars.size(); i++)
    if (f.vars[i].name == name) return (int)i;
  return -1;
}

int find_dim(const NcFile &f, const char *name) {
  for (size_t i = 0; i < f.dim_name.size(); i++)
    if (f.dim_name[i] == name) return (int)i;
  return -1;
}

const Att *find_att(const Var &v, const char *name) {
  for (const Att &a : v.atts)
    if (a.name == name) return &a;
  return nullptr;
}

// First value of a numeric attribute, as a double.
bool att_value(const Att &a, double &out) {
  if (a.n < 1) return false;
  const uint8_t *p = a.raw.data();
  switch (a.type) {
    case kByte: out = (double)(int8_t)p[0]; return true;
    case kShort: out = (double)(int16_t)(uint16_t)((p[0] << 8) | p[1]); return true;
    case kInt: out = (double)(int32_t)be32(p); return true;
    case kFloat: out = (double)be_float(p); return true;
    case kDouble: {
      const uint64_t u = be64(p);
      memcpy(&out, &u, 8);
      return true;
    }
    default: return false;
  }
}

// Dimensions, packing attributes and variable indexes of a grid file, with
// read_nc's rules (model/nc.c:138-198): lons, lats and bathy must exist,
// add_offset and scale_factor must be present, missing_value defaults to
// SHRT_MIN and decompressed_missing_value to 0.
struct GridFile {
  NcFile f;
  int v_lons = -1, v_lats = -1, v_grid = -1;
  photic_nc_grid_info info{};
};

int open_grid(const std::string &path, FILE **fpo, GridFile &g) {
  FILE *fp = fopen(path.c_str(), "rb");
  if (!fp) return io_fail(path, "cannot open");
  int rc = read_header(fp, path, g.f);
  if (rc) {
    fclose(fp);
    return rc;
  }
  const NcFile &f = g.f;
  g.v_lons = find_var(f, "lons");
  g.v_lats = find_var(f, "lats");
  g.v_grid = find_var(f, "bathy");
  const int d_lons = find_dim(f, "lons"), d_lats = find_dim(f, "lats");
  const char *why = nullptr;
  if (g.v_lons < 0 || g.v_lats < 0 || g.v_grid < 0) why = "variables lons, lats and bathy are required";
  else if (d_lons < 0 || d_lats < 0) why = "dimensions lons and lats are required";
  else if (f.dim_len[d_lons] == 0 || f.dim_len[d_lats] == 0) why = "record dimensions are not supported";
  else if (f.dim_len[d_lons] > INT_MAX || f.dim_len[d_lats] > INT_MAX) why = "grid too large";
  else {
    const Var &vl = f.vars[g.v_lons], &va = f.vars[g.v_lats], &vg = f.vars[g.v_grid];
    if (vl.type != kFloat || vl.dims.size() != 1 || (int)vl.dims[0] != d_lons)
      why = "lons must be float[lons]";
    else if (va.type != kFloat || va.dims.size() != 1 || (int)va.dims[0] != d_lats)
      why = "lats must be float[lats]";
    else if (vg.type != kShort || vg.dims.size() != 2 || (int)vg.dims[0] != d_lats ||
             (int)vg.dims[1] != d_lons)
      why = "bathy must be short[lats][lons]";
  }
  if (why) {
    fclose(fp);
    return io_fail(path, why);
  }
  photic_nc_grid_info &in = g.info;
  in.ncols = (int32_t)f.dim_len[d_lons];
  in.nrows = (int32_t)f.dim_len[d_lats];
  in.format = f.version;
  const Var &vg = f.vars[g.v_grid];
  double v;
  const Att *a = find_att(vg, "add_offset");
  if (!a || !att_value(*a, v)) {
    fclose(fp);
    return io_fail(path, "attribute add_offset missing");
  }
  in.add_offset = (float)v;
  a = find_att(vg, "scale_factor");
  if (!a || !att_value(*a, v)) {
    fclose(fp);
    return io_fail(path, "attribute scale_factor missing");
  }
  in.scale_factor = (float)v;
  a = find_att(vg, "missing_value");
  in.has_missing_value = a && att_value(*a, v) && v >= SHRT_MIN && v <= SHRT_MAX && v == (int)v;
  in.missing_value = in.has_missing_value ? (int16_t)(int)v : (int16_t)SHRT_MIN;
  a = find_att(vg, "decompressed_missing_value");
  in.has_spval = a && att_value(*a, v);
  in.spval = in.has_spval ? (double)(float)v : 0.0;
  *fpo = fp;
  return PHOTIC_OK;
}

int read_at(FILE *fp, const std::string &path, uint64_t off, void *dst, size_t bytes) {
  if (fseeko(fp, (off_t)off, SEEK_SET) != 0) return io_fail(path, "cannot seek");
  if (fread(dst, 1, bytes, fp) != bytes) return io_fail(path, "truncated variable data");
  return PHOTIC_OK;
}

int read_floats(FILE *fp, const std::string &path, const Var &v, size_t n, float *out) {
  std::vector<uint8_t> raw(n * 4);
  int rc = read_at(fp, path, v.begin, raw.data(), raw.size());
  if (rc) return rc;
  for (size_t i = 0; i < n; i++) out[i] = be_float(raw.data() + 4 * i);
  return PHOTIC_OK;
}

// Header writer.
struct Out {
  std::vector<uint8_t> b;
  void u32(uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
  }
  void u64(uint64_t v) {
    u32((uint32_t)(v >> 32));
    u32((uint32_t)v);
  }
  void pad() {
    while (b.size() % 4) b.push_back(0);
  }
  void name(const std::string &s) {
    u32((uint32_t)s.size());
    b.insert(b.end(), s.begin(), s.end());
    pad();
  }
  void text_att(const std::string &n, const std::string &v) {
    name(n);
    u32(kChar);
    u32((uint32_t)v.size());
    b.insert(b.end(), v.begin(), v.end());
    pad();
  }
  void float_att(const std::string &n, float v) {
    name(n);
    u32(kFloat);
    u32(1);
    uint32_t u;
    memcpy(&u, &v, 4);
    u32(u);
  }
  void short_att(const std::string &n, int16_t v) {
    name(n);
    u32(kShort);
    u32(1);
    b.push_back((uint8_t)((uint16_t)v >> 8));
    b.push_back((uint8_t)(uint16_t)v);
    pad();
  }
};

// The header of write_nc's layout (model/nc.c:40-101) with the variables'
// data starting at data0, lats, lons, bathy in that order.
std::vector<uint8_t> grid_header(const std::string &file_attr, const photic_nc_grid_info &in,
                                 int version, uint64_t data0) {
  const uint64_t nr = (uint64_t)in.nrows, ncol = (uint64_t)in.ncols;
  const uint64_t b_lats = data0, b_lons = b_lats + 4 * nr, b_grid = b_lons + 4 * ncol;
  const uint64_t grid_bytes = 2 * nr * ncol;
  const uint64_t grid_vsize = grid_bytes + 3 < 0xFFFFFFFFull ? ((grid_bytes + 3) & ~3ull)
                                                              : 0xFFFFFFFFull;
  Out o;
  o.b.insert(o.b.end(), {'C', 'D', 'F', (uint8_t)version});
  o.u32(0);
  o.u32(kTagDim);
  o.u32(2);
  o.name("lons");
  o.u32((uint32_t)ncol);
  o.name("lats");
  o.u32((uint32_t)nr);
  o.u32(kTagAtt);
  o.u32(2);
  o.text_att("filename", file_attr);
  o.text_att("data_type", "regular gridded data");
  o.u32(kTagVar);
  o.u32(3);
  const char *datum = "geographical coordinates, WGS84 projection";
  auto coord = [&](const char *nm, uint32_t dim, const char *std_name, const char *units,
                   uint64_t count, uint64_t begin) {
    o.name(nm);
    o.u32(1);
    o.u32(dim);
    o.u32(kTagAtt);
    o.u32(3);
    o.text_att("standard_name", std_name);
    o.text_att("units", units);
    o.text_att("reference_datum", datum);
    o.u32(kFloat);
    o.u32((uint32_t)(4 * count));
    if (version == 2) o.u64(begin);
    else o.u32((uint32_t)begin);
  };
  coord("lats", 1, "latitude", "degrees_north", nr, b_lats);
  coord("lons", 0, "longitude", "degrees_east", ncol, b_lons);
  o.name("bathy");
  o.u32(2);
  o.u32(1);
  o.u32(0);
  o.u32(kTagAtt);
  o.u32(4);
  o.float_att("add_offset", in.add_offset);
  o.float_att("scale_factor", in.scale_factor);
  o.short_att("missing_value", in.missing_value);
  o.float_att("decompressed_missing_value", (float)in.spval);
  o.u32(kShort);
  o.u32((uint32_t)grid_vsize);
  if (version == 2) o.u64(b_grid);
  else o.u32((uint32_t)b_grid);
  return o.b;
}

int write_grid_file(const std::string &path, const std::string &file_attr,
                    const photic_nc_grid_info &in, const void *packed_be, const float *lons,
                    const float *lats) {
  if (in.ncols < 1 || in.nrows < 1) return report_error(PHOTIC_ERR_INVALID, "empty grid");
  const uint64_t nr = (uint64_t)in.nrows, ncol = (uint64_t)in.ncols;
  // the header's length does not depend on the offsets it holds
  int version = in.format == 2 ? 2 : 1;
  uint64_t h = grid_header(file_attr, in, version, 0).size();
  const uint64_t end = h + 4 * nr + 4 * ncol + 2 * nr * ncol;
  if (in.format == 0 && h + 4 * nr + 4 * ncol > 0x7FFFFFFFull - 16) version = 2;
  if (in.format == 0 && end > 0x7FFFFFFFull) version = 2;
  h = grid_header(file_attr, in, version, 0).size();
  const std::vector<uint8_t> hdr = grid_header(file_attr, in, version, h);
  FILE *fp = fopen(path.c_str(), "wb");
  if (!fp) return io_fail(path, "cannot create");
  bool ok = fwrite(hdr.data(), 1, hdr.size(), fp) == hdr.size();
  auto put_floats = [&](const float *v, uint64_t n) {
    std::vector<uint8_t> raw(4 * n);
    for (uint64_t i = 0; i < n; i++) {
      uint32_t u;
      memcpy(&u, &v[i], 4);
      raw[4 * i] = (uint8_t)(u >> 24);
      raw[4 * i + 1] = (uint8_t)(u >> 16);
      raw[4 * i + 2] = (uint8_t)(u >> 8);
      raw[4 * i + 3] = (uint8_t)u;
    }
    ok = ok && fwrite(raw.data(), 1, raw.size(), fp) == raw.size();
  };
  put_floats(lats, nr);
  put_floats(lons, ncol);
  const uint64_t gb = 2 * nr * ncol;
  ok = ok && fwrite(packed_be, 1, gb, fp) == gb;
  const uint8_t zeros[4] = {0, 0, 0, 0};
  if (gb % 4) ok = ok && fwrite(zeros, 1, 4 - gb % 4, fp) == 4 - gb % 4;
  if (fclose(fp) != 0) ok = false;
  return ok ? PHOTIC_OK : io_fail(path, "write failed");
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
struct UnpackBand {
  const uint8_t *packed;  // big-endian shorts
  float add_offset, scale_factor, spval;
  int32_t missing;
};
struct UnpackArgs {
  UnpackBand band[PHOTIC_MAX_BANDS];
  int64_t npix;
  float *out;
};

__device__ __forceinline__ int16_t load_be16(const uint8_t *p, int64_t i) {
  const uint16_t w = __ldg(reinterpret_cast<const uint16_t *>(p) + i);
  return (int16_t)(uint16_t)((w >> 8) | (w << 8));
}

// decompress_2d (model/nc.c:251-266) cell by cell, the product and the sum
// each rounded to float, bands interleaved per pixel.
template <int NB>
__global__ void __launch_bounds__(256) nc_unpack_kernel(const __grid_constant__ UnpackArgs a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.npix; p += stride) {
    float v[NB];
#pragma unroll
    for (int b = 0; b < NB; b++) {
      const UnpackBand &u = a.band[b];
      const int16_t c = load_be16(u.packed, p);
      v[b] = c == (int16_t)u.missing ? u.spval
                                     : __fadd_rn(__fmul_rn((float)c, u.scale_factor), u.add_offset);
    }
    if (NB == 4) {
      reinterpret_cast<float4 *>(a.out)[p] = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
      for (int b = 0; b < NB; b++) a.out[p * NB + b] = v[b];
    }
  }
}

constexpr int kPackThreads = 256;
constexpr int kPackPer = 16;                           // cells per thread
constexpr int kPackTile = kPackThreads * kPackPer;     // cells per tile (row-major order)

struct PackState {
  float grmin;        // running minimum over all cells (add_offset)
  float scale;        // (grmax - grmin) / SHRT_MAX
  unsigned int kmax;  // order key of grmax
  unsigned int pad;
};

__device__ __forceinline__ unsigned int order_key(float f) {
  const unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_order_key(unsigned int k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Minimum of each tile over the cells compress_2d compares (not spval;
// NaN never lowers the minimum).
__global__ void __launch_bounds__(kPackThreads) nc_tile_min_kernel(const float *g, int64_t n,
                                                                   float fspv, float *tile_min) {
  const int64_t base = (int64_t)blockIdx.x * kPackTile;
  float m = INFINITY;
#pragma unroll 4
  for (int k = 0; k < kPackPer; k++) {
    const int64_t i = base + (int64_t)k * kPackThreads + threadIdx.x;
    if (i < n) {
      const float v = __ldg(g + i);
      if (v != fspv && v < m) m = v;
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float wm[kPackThreads / 32];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = wm[0];
    for (int w = 1; w < kPackThreads / 32; w++) t = fminf(t, wm[w]);
    tile_min[blockIdx.x] = t;
  }
}

// Exclusive min-scan of one value per thread of the block (+INF for thread
// 0); *total gets the minimum over the block.  scratch holds blockDim.x
// floats; every thread of the block must call it.
__device__ float block_exclusive_min(float v, float *scratch, float *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  __shared__ float wsum[32];
  for (int o = 1; o < 32; o <<= 1) {
    const float u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v = fminf(v, u);
  }
  if (lane == 31) wsum[warp] = v;
  __syncthreads();
  if (warp == 0) {
    float w = lane < nw ? wsum[lane] : INFINITY;
    for (int o = 1; o < 32; o <<= 1) {
      const float u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w = fminf(w, u);
    }
    wsum[lane] = w;
  }
  __syncthreads();
  if (warp > 0) v = fminf(v, wsum[warp - 1]);
  scratch[threadIdx.x] = v;  // inclusive
  __syncthreads();
  const float exc = threadIdx.x > 0 ? scratch[threadIdx.x - 1] : INFINITY;
  *total = scratch[blockDim.x - 1];
  __syncthreads();
  return exc;
}

// Exclusive prefix minimum over tiles, starting from FLT_MAX (compress_2d's
// initial grmin, model/nc.c:285); one block of 1024 threads.  Also sets
// grmin and starts the maximum at FLT_MIN (model/nc.c:286).
__global__ void __launch_bounds__(1024) nc_tile_scan_kernel(const float *tile_min, int64_t ntiles,
                                                            float *tile_prefix, PackState *st) {
  __shared__ float scratch[1024];
  float carry = FLT_MAX;
  for (int64_t base = 0; base < ntiles; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    float total;
    const float exc = block_exclusive_min(i < ntiles ? tile_min[i] : INFINITY, scratch, &total);
    if (i < ntiles) tile_prefix[i] = fminf(carry, exc);
    carry = fminf(carry, total);
  }
  if (threadIdx.x == 0) {
    st->grmin = carry;
    st->kmax = order_key(FLT_MIN);
  }
}

// Shared-memory slot of cell j of a tile: one float of padding per 32, so
// that the threads' runs of kPackPer cells fall in different banks.
__device__ __forceinline__ int tile_slot(int j) { return j + (j >> 5); }

// Each tile in row-major order: the cells that lower the running minimum
// (those below the minimum of every earlier cell) are skipped; every other
// compared cell is a maximum candidate (model/nc.c:288-297).
__global__ void __launch_bounds__(kPackThreads) nc_tile_max_kernel(const float *g, int64_t n,
                                                                   float fspv,
                                                                   const float *tile_prefix,
                                                                   PackState *st) {
  __shared__ float tile[kPackTile + kPackTile / 32];
  __shared__ float scratch[kPackThreads];
  const int64_t base = (int64_t)blockIdx.x * kPackTile;
#pragma unroll 4
  for (int k = 0; k < kPackPer; k++) {
    const int j = k * kPackThreads + threadIdx.x;
    tile[tile_slot(j)] = base + j < n ? __ldg(g + base + j) : fspv;  // past the end: skipped
  }
  __syncthreads();
  // this thread's run of cells, in row-major order
  const int r0 = threadIdx.x * kPackPer;
  float m = INFINITY;
  for (int k = 0; k < kPackPer; k++) {
    const float v = tile[tile_slot(r0 + k)];
    if (v != fspv && v < m) m = v;
  }
  float total;
  const float exc = block_exclusive_min(m, scratch, &total);
  float run = fminf(tile_prefix[blockIdx.x], exc);
  float mx = FLT_MIN;
  for (int k = 0; k < kPackPer; k++) {
    const float v = tile[tile_slot(r0 + k)];
    if (v == fspv) continue;
    if (v < run) run = v;
    else if (v > mx) mx = v;
  }
  unsigned int key = order_key(mx);
  for (int o = 16; o > 0; o >>= 1) key = max(key, __shfl_xor_sync(0xffffffffu, key, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&st->kmax, key);
}

__global__ void nc_scale_kernel(PackState *st) {
  const float grmax = from_order_key(st->kmax);
  st->scale = __fdiv_rn(__fsub_rn(grmax, st->grmin), (float)SHRT_MAX);
}

// (short) rint((g - grmin) / scale) with the x86-64 conversion
// (model/nc.c:312-318), missing cells SHRT_MIN; big-endian out.
__global__ void __launch_bounds__(256) nc_quantize_kernel(const float *g, int64_t n, float fspv,
                                                          const PackState *st, uint8_t *out) {
  const float grmin = st->grmin, scale = st->scale;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float v = __ldg(g + i);
    int16_t c;
    if (v == fspv) {
      c = (int16_t)SHRT_MIN;
    } else {
      const float r = rintf(__fdiv_rn(__fsub_rn(v, grmin), scale));
      const int32_t w = (r >= -2147483648.0f && r < 2147483648.0f) ? (int32_t)r : INT_MIN;
      c = (int16_t)(uint16_t)((uint32_t)w & 0xFFFFu);
    }
    const uint16_t u = (uint16_t)c;
    reinterpret_cast<uint16_t *>(out)[i] = (uint16_t)((u >> 8) | (u << 8));
  }
}

int device_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return sms;
}

int streaming_grid(int64_t n) {
  const int sms = device_sms();
  const int64_t need = (n + 255) / 256;
  const int64_t cap = (int64_t)(sms > 0 ? sms : 1) * 8;
  return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

template <int NB>
cudaError_t launch_unpack(const UnpackArgs &a, cudaStream_t s) {
  nc_unpack_kernel<NB><<<streaming_grid(a.npix), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t unpack(const UnpackArgs &a, int nb, cudaStream_t s) {
  switch (nb) {
    case 1: return launch_unpack<1>(a, s);
    case 2: return launch_unpack<2>(a, s);
    case 3: return launch_unpack<3>(a, s);
    case 4: return launch_unpack<4>(a, s);
    case 5: return launch_unpack<5>(a, s);
    case 6: return launch_unpack<6>(a, s);
    case 7: return launch_unpack<7>(a, s);
    default: return launch_unpack<8>(a, s);
  }
}

// The file name as trim() leaves it (model/common.c:715-751): leading and
// trailing white space removed.
std::string trimmed(const char *file) {
  std::string s(file);
  size_t b = 0, e = s.size();
  while (b < e && isspace((unsigned char)s[b])) b++;
  while (e > b && isspace((unsigned char)s[e - 1])) e--;
  return s.substr(b, e - b);
}

// trim() edits the caller's string in place; the drop-ins do the same.
void trim_in_place(char *file) {
  const std::string t = trimmed(file);
  memcpy(file, t.c_str(), t.size() + 1);
}

// The reference's ERR macro (model/nc.h:6): message and exit(1).
[[noreturn]] void die(const char *what) {
  printf("Error: %s\n", what);
  exit(1);
}

}  // namespace

extern "C" {

int photic_nc_read_info(const char *path, photic_nc_grid_info *info) {
  return photic_nc_read_raw(path, info, nullptr, nullptr, nullptr);
}

int photic_nc_read_raw(const char *path, photic_nc_grid_info *info, void *h_packed_be,
                       float *h_lons, float *h_lats) {
  if (!path || !info) return report_error(PHOTIC_ERR_INVALID, "bad arguments");
  GridFile g;
  FILE *fp = nullptr;
  int rc = open_grid(path, &fp, g);
  if (rc) return rc;
  *info = g.info;
  const std::string p(path);
  const uint64_t n = (uint64_t)g.info.nrows * (uint64_t)g.info.ncols;
  if (!rc && h_packed_be) rc = read_at(fp, p, g.f.vars[g.v_grid].begin, h_packed_be, 2 * n);
  if (!rc && h_lons) rc = read_floats(fp, p, g.f.vars[g.v_lons], (size_t)g.info.ncols, h_lons);
  if (!rc && h_lats) rc = read_floats(fp, p, g.f.vars[g.v_lats], (size_t)g.info.nrows, h_lats);
  fclose(fp);
  return rc;
}

int photic_nc_write_raw(const char *path, const photic_nc_grid_info *info,
                        const void *h_packed_be, const float *h_lons, const float *h_lats) {
  if (!path || !info || !h_packed_be || !h_lons || !h_lats || info->ncols < 1 ||
      info->nrows < 1 || info->format < 0 || info->format > 2)
    return report_error(PHOTIC_ERR_INVALID, "bad arguments");
  return write_grid_file(path, path, *info, h_packed_be, h_lons, h_lats);
}

int photic_nc_unpack_bands(const void *const *d_packed_be, const photic_nc_grid_info *infos,
                           int32_t n_bands, int64_t npix, float *d_rrs, void *stream) {
  if (!d_packed_be || !infos || n_bands < 1 || n_bands > PHOTIC_MAX_BANDS || npix < 0 ||
      (npix > 0 && !d_rrs))
    return report_error(PHOTIC_ERR_INVALID, "bad arguments");
  if (npix == 0) return PHOTIC_OK;
  UnpackArgs a;
  memset(&a, 0, sizeof a);
  for (int b = 0; b < n_bands; b++) {
    if (!d_packed_be[b] || ((uintptr_t)d_packed_be[b] & 1u))
      return report_error(PHOTIC_ERR_INVALID, "packed grids must be 2-byte aligned device memory");
    a.band[b].packed = (const uint8_t *)d_packed_be[b];
    a.band[b].add_offset = infos[b].add_offset;
    a.band[b].scale_factor = infos[b].scale_factor;
    a.band[b].spval = (float)infos[b].spval;  // (float) spval, model/nc.c:258
    a.band[b].missing = infos[b].missing_value;
  }
  if (n_bands == 4 && ((uintptr_t)d_rrs & 15u))
    return report_error(PHOTIC_ERR_INVALID, "d_rrs must be 16-byte aligned for 4 bands");
  a.npix = npix;
  a.out = d_rrs;
  cudaError_t e = unpack(a, n_bands, (cudaStream_t)stream);
  return e == cudaSuccess ? PHOTIC_OK : cuda_fail_nc(e, "unpack launch");
}

int photic_nc_pack(const float *d_grid, int64_t n, double spval, void *d_packed_be,
                   photic_nc_grid_info *info, void *stream) {
  if (n < 1 || !d_grid || !d_packed_be || !info || ((uintptr_t)d_packed_be & 1u))
    return report_error(PHOTIC_ERR_INVALID, "bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t ntiles = (n + kPackTile - 1) / kPackTile;
  if (ntiles > 0x7FFFFFFFLL) return report_error(PHOTIC_ERR_INVALID, "grid too large");
  const float fspv = (float)spval;  // model/nc.c:278
  unsigned char *ws = nullptr;
  const size_t off_pref = ((size_t)ntiles * 4 + 255) / 256 * 256;
  const size_t off_st = off_pref + ((size_t)ntiles * 4 + 255) / 256 * 256;
  cudaError_t e = cudaMallocAsync((void **)&ws, off_st + sizeof(PackState), s);
  if (e != cudaSuccess) return report_error(PHOTIC_ERR_NOMEM, "pack workspace");
  float *tmin = (float *)ws, *tpre = (float *)(ws + off_pref);
  PackState *st = (PackState *)(ws + off_st);
  nc_tile_min_kernel<<<(unsigned)ntiles, kPackThreads, 0, s>>>(d_grid, n, fspv, tmin);
  nc_tile_scan_kernel<<<1, 1024, 0, s>>>(tmin, ntiles, tpre, st);
  nc_tile_max_kernel<<<(unsigned)ntiles, kPackThreads, 0, s>>>(d_grid, n, fspv, tpre, st);
  nc_scale_kernel<<<1, 1, 0, s>>>(st);
  nc_quantize_kernel<<<streaming_grid(n), 256, 0, s>>>(d_grid, n, fspv, st,
                                                       (uint8_t *)d_packed_be);
  e = cudaGetLastError();
  PackState h{};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, st, sizeof h, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(ws, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail_nc(e, "pack");
  memset(info, 0, sizeof *info);
  info->add_offset = h.grmin;
  info->scale_factor = h.scale;
  info->missing_value = (int16_t)SHRT_MIN;
  info->has_missing_value = 1;
  info->spval = spval;
  info->has_spval = 1;
  return PHOTIC_OK;
}

int photic_nc_read_bands(const char *const *paths, int32_t n_bands, float *d_rrs,
                         int64_t capacity_px, photic_nc_grid_info *info, float *h_lons,
                         float *h_lats, void *stream) {
  if (!paths || n_bands < 1 || n_bands > PHOTIC_MAX_BANDS || !d_rrs || !info)
    return report_error(PHOTIC_ERR_INVALID, "bad arguments");
  photic_nc_grid_info infos[PHOTIC_MAX_BANDS];
  for (int b = 0; b < n_bands; b++) {
    if (!paths[b]) return report_error(PHOTIC_ERR_INVALID, "bad arguments");
    int rc = photic_nc_read_info(paths[b], &infos[b]);
    if (rc) return rc;
    if (infos[b].ncols != infos[0].ncols || infos[b].nrows != infos[0].nrows)
      return io_fail(paths[b], "input grids are not commensurate");
  }
  const int64_t npix = (int64_t)infos[0].nrows * infos[0].ncols;
  if (npix > capacity_px) return report_error(PHOTIC_ERR_INVALID, "d_rrs too small for the grids");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t band_bytes = ((size_t)npix * 2 + 255) / 256 * 256;
  void *h = nullptr;
  unsigned char *d = nullptr;
  cudaError_t e = cudaMallocHost(&h, band_bytes * n_bands);
  if (e != cudaSuccess) return report_error(PHOTIC_ERR_NOMEM, "pinned staging");
  e = cudaMallocAsync((void **)&d, band_bytes * n_bands, s);
  if (e != cudaSuccess) {
    cudaFreeHost(h);
    return report_error(PHOTIC_ERR_NOMEM, "device staging");
  }
  int rc = PHOTIC_OK;
  const void *dp[PHOTIC_MAX_BANDS];
  for (int b = 0; b < n_bands && !rc; b++) {
    unsigned char *hb = (unsigned char *)h + band_bytes * b;
    rc = photic_nc_read_raw(paths[b], &infos[b], hb, b == 0 ? h_lons : nullptr,
                            b == 0 ? h_lats : nullptr);
    if (!rc) {
      e = cudaMemcpyAsync(d + band_bytes * b, hb, (size_t)npix * 2, cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) rc = cuda_fail_nc(e, "band upload");
    }
    dp[b] = d + band_bytes * b;
  }
  if (!rc) rc = photic_nc_unpack_bands(dp, infos, n_bands, npix, d_rrs, stream);
  cudaFreeAsync(d, s);
  e = cudaStreamSynchronize(s);
  cudaFreeHost(h);
  if (!rc && e != cudaSuccess) rc = cuda_fail_nc(e, "read bands");
  if (!rc) *info = infos[0];
  return rc;
}

int photic_nc_write_grid(const char *path, const float *d_grid, int32_t ncols, int32_t nrows,
                         const float *h_lons, const float *h_lats, double spval, void *stream) {
  if (!path || !d_grid || !h_lons || !h_lats || ncols < 1 || nrows < 1)
    return report_error(PHOTIC_ERR_INVALID, "bad arguments");
  const int64_t n = (int64_t)ncols * nrows;
  cudaStream_t s = (cudaStream_t)stream;
  void *dpk = nullptr, *hpk = nullptr;
  cudaError_t e = cudaMallocAsync(&dpk, (size_t)n * 2, s);
  if (e != cudaSuccess) return report_error(PHOTIC_ERR_NOMEM, "pack output");
  e = cudaMallocHost(&hpk, (size_t)n * 2);
  if (e != cudaSuccess) {
    cudaFreeAsync(dpk, s);
    return report_error(PHOTIC_ERR_NOMEM, "pinned staging");
  }
  photic_nc_grid_info info;
  int rc = photic_nc_pack(d_grid, n, spval, dpk, &info, stream);
  if (!rc) {
    e = cudaMemcpyAsync(hpk, dpk, (size_t)n * 2, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_fail_nc(e, "packed download");
  }
  if (!rc) {
    info.ncols = ncols;
    info.nrows = nrows;
    info.format = 0;
    // the filename attribute is the name trim() left in place (model/nc.c:38-44)
    const std::string name = trimmed(path);
    rc = write_grid_file(name, name, info, hpk, h_lons, h_lats);
  }
  cudaFreeAsync(dpk, s);
  cudaStreamSynchronize(s);
  cudaFreeHost(hpk);
  return rc;
}

// read_nc (model/nc.c:138-246): the grid comes back as nrows rows of ncols
// floats, one malloc per row as allocate_float_array_2d makes them
// (model/common.c:562-572); lons and lats malloc'd.
void read_nc(char *file, float ***grid, int *ncols, int *nrows, float **lons, float **lats,
             double *spval) {
  trim_in_place(file);
  const std::string path(file);
  photic_nc_grid_info info;
  if (photic_nc_read_info(path.c_str(), &info)) die(photic_last_error());
  if (!info.has_spval) printf("\nWARNING: 'decompressed_missing_value' not present. Setting to zero.\n");
  if (!info.has_missing_value)
    printf("\nWARNING: 'missing_value' not present. Setting to %d.\n", SHRT_MIN);
  const int64_t n = (int64_t)info.nrows * info.ncols;
  std::vector<uint8_t> raw((size_t)n * 2);
  *lons = (float *)malloc((size_t)info.ncols * sizeof(float));
  *lats = (float *)malloc((size_t)info.nrows * sizeof(float));
  if (!*lons || !*lats) die("out of memory");
  if (photic_nc_read_raw(path.c_str(), &info, raw.data(), *lons, *lats)) die(photic_last_error());
  void *d_raw = nullptr;
  float *d_out = nullptr;
  std::vector<float> host((size_t)n);
  cudaError_t e = cudaMalloc(&d_raw, (size_t)n * 2);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_out, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMemcpy(d_raw, raw.data(), (size_t)n * 2, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) die(cudaGetErrorString(e));
  const void *dp[1] = {d_raw};
  if (photic_nc_unpack_bands(dp, &info, 1, n, d_out, nullptr)) die(photic_last_error());
  e = cudaMemcpy(host.data(), d_out, (size_t)n * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) die(cudaGetErrorString(e));
  cudaFree(d_raw);
  cudaFree(d_out);
  float **rows = (float **)malloc((size_t)info.nrows * sizeof(float *));
  if (!rows) die("out of memory");
  for (int i = 0; i < info.nrows; i++) {
    rows[i] = (float *)malloc((size_t)info.ncols * sizeof(float));
    if (!rows[i]) die("out of memory");
    memcpy(rows[i], host.data() + (size_t)i * info.ncols, (size_t)info.ncols * sizeof(float));
  }
  *grid = rows;
  *ncols = info.ncols;
  *nrows = info.nrows;
  *spval = info.spval;
}

// write_nc (model/nc.c:14-134).
void write_nc(char *file, float **grid, int ncols, int nrows, float *lons, float *lats,
              double spval) {
  trim_in_place(file);
  if (ncols < 1 || nrows < 1) die("empty grid");
  const int64_t n = (int64_t)ncols * nrows;
  std::vector<float> host((size_t)n);
  for (int i = 0; i < nrows; i++)
    memcpy(host.data() + (size_t)i * ncols, grid[i], (size_t)ncols * sizeof(float));
  float *d = nullptr;
  cudaError_t e = cudaMalloc((void **)&d, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMemcpy(d, host.data(), (size_t)n * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) die(cudaGetErrorString(e));
  const int rc = photic_nc_write_grid(file, d, ncols, nrows, lons, lats, spval, nullptr);
  cudaFree(d);
  if (rc) die(photic_last_error());
}

}  // extern "C"
