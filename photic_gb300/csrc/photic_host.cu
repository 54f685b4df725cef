// photic_host.cu -- the extern "C" entry points of include/photic.h.
//
// Host work here is set-up only: validating the configuration, resolving
// the table interpolation at the band wavelengths (interp_1d,
// model/common.c:298) and the subsurface-angle secants once per call, and
// launching the kernels.  No pixel is ever processed on the host.
#include <cuda_runtime.h>
#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>
#include <algorithm>
#include <vector>

#include "../../include/photic.h"
#include "../../include/photic_nc.h"
#include "photic_kernels.h"
#include "photic_params.h"
#include "photic_tables.h"

using namespace photic;

namespace {

constexpr double kPiHost = 3.141592653589793;  // model/common.h:19

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(PHOTIC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Tolerant single-precision comparisons of model/common.c:392-406.
bool f_close(float a, float b, float eps) {
  double big = fabs(a) < fabs(b) ? fabs(b) : fabs(a);
  return fabs(a - b) <= big * eps;
}
bool f_le(float a, float b, float eps) { return a < b || f_close(a, b, eps); }
bool f_ge(float a, float b, float eps) { return a > b || f_close(a, b, eps); }

// Segment choice of interp_1d (model/common.c:298-330) for target x over
// abscissae X[0..n): either an exact end point, or (i0, i1, t).
InterpPlan resolve_interp(const double *X, int n, double x) {
  InterpPlan p{};
  if (f_close((float)x, (float)X[0], 1.0e-5f)) {
    p.exact = 1;
    p.i0 = p.i1 = 0;
    return p;
  }
  if (f_close((float)x, (float)X[n - 1], 1.0e-5f)) {
    p.exact = 1;
    p.i0 = p.i1 = n - 1;
    return p;
  }
  double x0 = 0.0, x1 = 1.0;
  if (X[0] < X[n - 1] && x < X[0]) {
    p.i0 = 0;
    p.i1 = 1;
  } else if (X[n - 1] > X[0] && x > X[n - 1]) {
    p.i0 = n - 2;
    p.i1 = n - 1;
  } else {
    p.i0 = 0;
    p.i1 = 0;
    for (int i = 0; i + 1 < n; i++) {
      bool up = f_le((float)X[i], (float)x, 1.0e-5f) && f_ge((float)X[i + 1], (float)x, 1.0e-5f);
      bool down = f_ge((float)X[i], (float)x, 1.0e-5f) && f_le((float)X[i + 1], (float)x, 1.0e-5f);
      if (up || down) {
        p.i0 = i;
        p.i1 = i + 1;
        break;
      }
    }
  }
  x0 = X[p.i0];
  x1 = X[p.i1];
  p.exact = 0;
  p.t = (x - x0) / (x1 - x0);
  p.one_minus_t = 1.0 - p.t;
  return p;
}

double interp_apply(const InterpPlan &p, const double *Y) {
  if (p.exact) return Y[p.i0];
  return Y[p.i0] * p.one_minus_t + Y[p.i1] * p.t;
}

double table_at(const double *tab, double x) {
  return interp_apply(resolve_interp(tables::wl, tables::kNRef, x), tab);
}

// Scene constants for a subsurface sun zenith (samodel():521-618).
void make_scene(const photic_config &cfg, double theta_sun_deg, SceneConsts &sc) {
  memset(&sc, 0, sizeof sc);
  double th = cfg.theta_view_deg;
  th *= kPiHost / 180.0;
  sc.sec_view = 1.0 / cos(th);
  th = theta_sun_deg;
  th *= kPiHost / 180.0;
  sc.sec_sun = 1.0 / cos(th);
  sc.h_tide = cfg.h_tide;
  const double S = 0.015;
  for (int b = 0; b < cfg.n_bands; b++) {
    const double l = cfg.wavelengths[b];
    sc.wl[b] = l;
    sc.a0[b] = table_at(tables::a0, l);
    sc.a1[b] = table_at(tables::a1, l);
    sc.bbw[b] = table_at(tables::bbw, l);
    sc.aw[b] = table_at(tables::aw, l);
    sc.refl[b] = table_at(tables::bottom[0], l);
    for (int k = 0; k < 3; k++) sc.refl_k[k][b] = table_at(tables::bottom[k], l);
    sc.eS[b] = exp(-S * (l - 440.0));
    sc.ratio440[b] = 440.0 / l;
  }
}

void make_fit(const photic_config &cfg, FitParams &fp) {
  memset(&fp, 0, sizeof fp);
  fp.n_bands = cfg.n_bands;
  fp.kcount = cfg.kcount;
  fp.konvge = cfg.konvge;
  fp.n_hstarts = cfg.n_hstarts;
  fp.layout = cfg.layout;
  fp.nodata = cfg.nodata_value;
  fp.reqmin = cfg.reqmin;
  fp.early_exit_per_scene = cfg.early_exit_per_scene;
  fp.seed_step_scale = cfg.seed_step_scale;
  fp.aw640 = table_at(tables::aw, 640.0);
  for (int k = 0; k < cfg.n_hstarts; k++) fp.hstarts[k] = cfg.hstarts[k];
  const double targets[kNRefTargets] = {440.0, 490.0, 550.0, 640.0, 750.0};
  for (int t = 0; t < kNRefTargets; t++)
    fp.plan[t] = resolve_interp(cfg.wavelengths, cfg.n_bands, targets[t]);
  // K penalty (model/samodel.c:2696-2732): thresholds and targets.
  const double mean_c = 0.275, min_c = 0.185;
  const double t2 = 0.5 * (1.5 * min_c + 0.5 * mean_c);
  const double t3 = 0.5 * (1.25 * min_c + 0.75 * mean_c);
  const double t5 = 0.5 * (1.75 * min_c + 0.25 * mean_c);
  const double thr[5] = {mean_c, t2, t3, t2, t5};
  const double tgt[5] = {min_c, t2, t3, t2, t5};
  for (int i = 0; i < 5; i++) {
    fp.kp.k_thr[i] = thr[i];
    fp.kp.inv_t[i] = 1.0 / (0.01 + tgt[i]);
  }
}

DfPair split(double d) {
  DfPair p;
  p.hi = (float)d;
  p.lo = (float)(d - (double)p.hi);
  return p;
}

// Double-float copies of the cost constants (PHOTIC_PREC_DF64).
void make_df(const photic_config &cfg, const FitParams &fp, const SceneConsts &sc, int n_params,
             DfScene &ds) {
  memset(&ds, 0, sizeof ds);
  for (int b = 0; b < cfg.n_bands; b++) {
    ds.a0[b] = split(sc.a0[b]);
    ds.a1[b] = split(sc.a1[b]);
    ds.aw[b] = split(sc.aw[b]);
    ds.bbw[b] = split(sc.bbw[b]);
    ds.refl[b] = split(sc.refl[b]);
    ds.eS[b] = split(sc.eS[b]);
    ds.ln_ratio440[b] = split(log(sc.ratio440[b]));
  }
  ds.sec_sun = split(sc.sec_sun);
  ds.sec_view = split(sc.sec_view);
  for (int t = 0; t < kNRefTargets; t++) {
    ds.plan_t[t] = split(fp.plan[t].t);
    ds.plan_omt[t] = split(fp.plan[t].one_minus_t);
  }
  ds.x_start_coef = split(100.0 * 30.0 * fp.aw640);
  for (int i = 0; i < 5; i++) {
    ds.k_thr[i] = split(fp.kp.k_thr[i]);
    ds.inv_t[i] = split(fp.kp.inv_t[i]);
  }
  ds.reqmin_n = split(cfg.reqmin * (double)n_params);
  for (int k = 0; k < cfg.n_hstarts; k++) ds.hstarts[k] = split(cfg.hstarts[k]);
}

// Optional device counter of exact evaluations served by the guarded
// kernel (photic_set_counter); NULL when unset.
unsigned long long *g_counter_ptr = nullptr;
unsigned long long *g_guard_stats_ptr = nullptr;

// Sticky per-device error word the kernels OR their error bits into.
std::mutex g_dev_mu;
std::vector<unsigned int *> g_dev_err;
std::vector<int> g_dev_sms;

int device_state(unsigned int **err, int *sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if ((int)g_dev_err.size() <= dev) {
    g_dev_err.resize(dev + 1, nullptr);
    g_dev_sms.resize(dev + 1, 0);
  }
  if (g_dev_err[dev] == nullptr) {
    unsigned int *p = nullptr;
    e = cudaMalloc(&p, sizeof(unsigned int));
    if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "error word: %s", cudaGetErrorString(e));
    e = cudaMemset(p, 0, sizeof(unsigned int));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemset");
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    g_dev_err[dev] = p;
    g_dev_sms[dev] = n;
  }
  *err = g_dev_err[dev];
  *sms = g_dev_sms[dev];
  return PHOTIC_OK;
}

// Per-device fork set of the joint launch (created on first use, kept for
// the life of the process); its mutex orders concurrent joint launches.
struct ForkSlot {
  JointFork f;
  bool ready = false;
  std::mutex mu;
};
std::mutex g_fork_mu;
std::vector<ForkSlot *> g_fork;

int joint_fork(ForkSlot **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_fork_mu);
  if ((int)g_fork.size() <= dev) g_fork.resize(dev + 1, nullptr);
  if (!g_fork[dev]) g_fork[dev] = new ForkSlot();
  ForkSlot *fs = g_fork[dev];
  if (!fs->ready) {
    for (int k = 0; k < 8; k++) {
      e = cudaStreamCreateWithFlags(&fs->f.side[k], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fs->f.join[k], cudaEventDisableTiming);
      if (e != cudaSuccess) return cuda_fail(e, "joint fork streams");
    }
    e = cudaEventCreateWithFlags(&fs->f.fork, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "joint fork event");
    fs->ready = true;
  }
  *out = fs;
  return PHOTIC_OK;
}

// Threads per block of the inversion when the config leaves it open.  The
// FP64 kernel runs fastest with 256 (measured on GB300 against 64 and 128,
// 3 % ahead; the fits are identical for every shape); the double-float
// kernel keeps 128.
int default_invert_block(int precision) { return precision == PHOTIC_PREC_FP64 ? 256 : 128; }

}  // namespace

namespace photic {
// Error reporting for the other translation units of the library.
int report_error(int code, const char *message) {
  g_err = message;
  return code;
}
}  // namespace photic

extern "C" {

const char *photic_version(void) { return "photic-gb300 0.1"; }

const char *photic_last_error(void) { return g_err.c_str(); }

void photic_config_default(photic_config *cfg) {
  memset(cfg, 0, sizeof *cfg);
  cfg->n_bands = 4;
  const double wl[4] = {443.0, 482.0, 561.0, 655.0};
  for (int b = 0; b < 4; b++) cfg->wavelengths[b] = wl[b];
  cfg->theta_sun_deg = 35.0;
  cfg->theta_view_deg = 0.0;
  cfg->h_tide = 0.0;
  cfg->nodata_value = -9999.0f;
  cfg->reqmin = 1.0e-10;
  cfg->konvge = 100;
  cfg->kcount = 2000;
  const double hs[8] = {40.0, 30.0, 20.0, 15.0, 10.0, 7.5, 2.5, 1.0};
  cfg->n_hstarts = 8;
  for (int k = 0; k < 8; k++) cfg->hstarts[k] = hs[k];
  cfg->early_exit_per_scene = 2.5;
  cfg->precision = PHOTIC_PREC_FP64;
  cfg->layout = PHOTIC_LAYOUT_REFERENCE;
  cfg->block_threads = 0;
  cfg->blocks_per_sm = 0;
  cfg->seed_step_scale = 1.0;
}

int photic_config_check(const photic_config *cfg) {
  if (!cfg) return fail(PHOTIC_ERR_INVALID, "config is NULL");
  if (cfg->n_bands < 2 || cfg->n_bands > PHOTIC_MAX_BANDS)
    return fail(PHOTIC_ERR_INVALID, "n_bands %d outside 2..%d", cfg->n_bands, PHOTIC_MAX_BANDS);
  for (int b = 0; b < cfg->n_bands; b++) {
    if (!(cfg->wavelengths[b] > 0.0) || !isfinite(cfg->wavelengths[b]))
      return fail(PHOTIC_ERR_INVALID, "wavelength %d is not a positive number", b);
    if (b && !(cfg->wavelengths[b] > cfg->wavelengths[b - 1]))
      return fail(PHOTIC_ERR_INVALID, "wavelengths must be ascending");
  }
  if (!(cfg->reqmin > 0.0)) return fail(PHOTIC_ERR_INVALID, "reqmin must be > 0 (nelmin ifault 1)");
  if (cfg->konvge < 1) return fail(PHOTIC_ERR_INVALID, "konvge must be >= 1 (nelmin ifault 1)");
  if (cfg->kcount < 1) return fail(PHOTIC_ERR_INVALID, "kcount must be >= 1");
  if (cfg->n_hstarts < 1 || cfg->n_hstarts > PHOTIC_MAX_HSTARTS)
    return fail(PHOTIC_ERR_INVALID, "n_hstarts %d outside 1..%d", cfg->n_hstarts, PHOTIC_MAX_HSTARTS);
  if (cfg->precision < PHOTIC_PREC_FP64 || cfg->precision > PHOTIC_PREC_GUARDED)
    return fail(PHOTIC_ERR_INVALID, "unknown precision %d", cfg->precision);
  if (cfg->layout != PHOTIC_LAYOUT_REFERENCE && cfg->layout != PHOTIC_LAYOUT_SCENE_B)
    return fail(PHOTIC_ERR_INVALID, "unknown layout %d", cfg->layout);
  if (cfg->block_threads != 0 && cfg->block_threads != 64 && cfg->block_threads != 128 &&
      cfg->block_threads != 256)
    return fail(PHOTIC_ERR_INVALID, "block_threads must be 0, 64, 128 or 256");
  if (cfg->blocks_per_sm < 0 || cfg->blocks_per_sm > 32)
    return fail(PHOTIC_ERR_INVALID, "blocks_per_sm outside 0..32");
  if (!(cfg->seed_step_scale > 0.0) || !isfinite(cfg->seed_step_scale))
    return fail(PHOTIC_ERR_INVALID, "seed_step_scale must be a positive number");
  return PHOTIC_OK;
}

double photic_interp_1d(const double *X, const double *Y, int32_t n, double x) {
  if (!X || !Y || n < 2) return NAN;
  return interp_apply(resolve_interp(X, n, x), Y);
}

int photic_band_constants(const photic_config *cfg, double *out) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  SceneConsts sc;
  make_scene(*cfg, cfg->theta_sun_deg, sc);
  const double aw640 = table_at(tables::aw, 640.0);
  for (int b = 0; b < cfg->n_bands; b++) {
    out[b * 8 + 0] = sc.a0[b];
    out[b * 8 + 1] = sc.a1[b];
    out[b * 8 + 2] = sc.aw[b];
    out[b * 8 + 3] = sc.bbw[b];
    out[b * 8 + 4] = sc.refl[b];
    out[b * 8 + 5] = sc.sec_sun;
    out[b * 8 + 6] = sc.sec_view;
    out[b * 8 + 7] = aw640;
  }
  return PHOTIC_OK;
}

int photic_bottom_reflectances(const photic_config *cfg, int32_t n_types, double *out) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (n_types < 1 || n_types > tables::kNBottom || !out)
    return fail(PHOTIC_ERR_INVALID, "n_types must be 1..%d", tables::kNBottom);
  for (int k = 0; k < n_types; k++)
    for (int b = 0; b < cfg->n_bands; b++)
      out[k * cfg->n_bands + b] = table_at(tables::bottom[k], cfg->wavelengths[b]);
  return PHOTIC_OK;
}

int photic_invert_batch(const photic_config *cfg, const float *d_rrs, int64_t npix,
                        int64_t pixel_stride, int64_t band_stride, const double *d_seeds,
                        const photic_outputs *out, void *stream) {
  return photic_invert_batch_ordered(cfg, d_rrs, npix, pixel_stride, band_stride, d_seeds,
                                     nullptr, out, stream);
}

int photic_invert_batch_ordered(const photic_config *cfg, const float *d_rrs, int64_t npix,
                                int64_t pixel_stride, int64_t band_stride,
                                const double *d_seeds, const int32_t *d_order,
                                const photic_outputs *out, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (npix < 0) return fail(PHOTIC_ERR_INVALID, "npix < 0");
  if (npix == 0) return PHOTIC_OK;
  if (!d_rrs || !out) return fail(PHOTIC_ERR_INVALID, "NULL input or output");
  if (pixel_stride < 1 || band_stride < 1)
    return fail(PHOTIC_ERR_INVALID, "strides must be >= 1");
  if (d_order && cfg->precision == PHOTIC_PREC_GUARDED)
    return fail(PHOTIC_ERR_UNSUPPORTED, "a pixel order is not supported in guarded precision");
  if (d_order && npix > 0x7fffffffLL) return fail(PHOTIC_ERR_INVALID, "npix beyond 2^31-1");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int *err = nullptr;
  int sms = 0;
  rc = device_state(&err, &sms);
  if (rc) return rc;

  InvertArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.sc);
  make_df(*cfg, a.fp, a.sc, 6, a.ds);
  a.rrs = d_rrs;
  a.npix = npix;
  a.pixel_stride = pixel_stride;
  a.band_stride = band_stride;
  a.vec4 = (cfg->n_bands == 4 && pixel_stride == 4 && band_stride == 1 &&
            ((uintptr_t)d_rrs & 15u) == 0);
  a.seeds = d_seeds;
  a.order = d_order;
  a.out = *out;
  a.error = err;
  a.early_exit = cfg->early_exit_per_scene * (double)(float)1;

  const bool guarded = cfg->precision == PHOTIC_PREC_GUARDED;
  int block = cfg->block_threads    ? cfg->block_threads
              : guarded             ? 128
                                    : default_invert_block(cfg->precision);
  if (guarded && block == 64) block = 128;
  int per_sm = cfg->blocks_per_sm;
  if (per_sm == 0) {
    per_sm = guarded ? guarded_blocks_per_sm(a, block)
                     : invert_blocks_per_sm(a, cfg->precision, block);
    if (per_sm < 1) return fail(PHOTIC_ERR_CUDA, "kernel does not fit on the device");
  }
  int64_t grid = (int64_t)sms * per_sm;
  const int64_t need = (npix + block - 1) / block;
  if (grid > need) grid = need;

  unsigned long long *queue = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&queue, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "queue head: %s", cudaGetErrorString(e));
  e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  a.queue = queue;
  a.counters = g_counter_ptr;
  a.guard_stats = g_guard_stats_ptr;
  e = guarded ? launch_guarded(a, block, (int)grid, s)
              : launch_invert(a, cfg->precision, block, (int)grid, s);
  cudaError_t e2 = cudaFreeAsync(queue, s);
  if (e != cudaSuccess) return cuda_fail(e, "invert kernel launch");
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFreeAsync");
  return PHOTIC_OK;
}

void photic_lut_config_default(photic_lut_config *lut) {
  if (!lut) return;
  memset(lut, 0, sizeof *lut);
  lut->n_lut = 16000;  // model/samodel.c:650
}

// Default chains per resident lane.  A chain is sequential (every pixel
// waits for the previous one's fit), so with one chain per lane the kernel
// lasts as long as the lane with the most work; lanes that finish take the
// next chain from the queue, and eight chains per lane bound that tail by
// one short chain.
constexpr int64_t kLutChainsPerLane = 8;

int64_t photic_lut_default_chains(const photic_config *cfg) {
  if (photic_config_check(cfg)) return 0;
  unsigned int *err = nullptr;
  int sms = 0;
  if (device_state(&err, &sms)) return 0;
  LutArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.inv.fp);
  return kLutChainsPerLane * sms * lut_blocks_per_sm(a) * lut_block();
}

int photic_lut_invert_batch(const photic_config *cfg, const photic_lut_config *lut,
                            const float *d_rrs, int64_t npix, const float *d_empirical,
                            float empirical_nodata, const photic_outputs *out,
                            int64_t *d_source, int64_t *d_order, double *d_chain_stats,
                            int64_t *n_shallow, int64_t *n_chains_used, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (n_shallow) *n_shallow = 0;
  if (n_chains_used) *n_chains_used = 0;
  if (!lut) return fail(PHOTIC_ERR_INVALID, "NULL lookup-table configuration");
  if (lut->n_lut < 1 || lut->n_chains < 0)
    return fail(PHOTIC_ERR_INVALID, "n_lut must be >= 1 and n_chains >= 0");
  if (cfg->precision != PHOTIC_PREC_FP64)
    return fail(PHOTIC_ERR_UNSUPPORTED, "the lookup-table loop runs in FP64 only");
  if (npix < 0) return fail(PHOTIC_ERR_INVALID, "npix < 0");
  if (npix == 0) return PHOTIC_OK;
  if (!d_rrs || !out) return fail(PHOTIC_ERR_INVALID, "NULL input or output");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int *err = nullptr;
  int sms = 0;
  rc = device_state(&err, &sms);
  if (rc) return rc;
  const int nb = cfg->n_bands;

  LutArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.inv.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.inv.sc);
  a.inv.rrs = d_rrs;
  a.inv.npix = npix;
  a.inv.pixel_stride = nb;
  a.inv.band_stride = 1;
  a.inv.out = *out;
  a.inv.error = err;
  a.inv.early_exit = cfg->early_exit_per_scene * (double)(float)1;
  a.source = d_source;
  a.chain_stats = d_chain_stats;
  a.emp = d_empirical;
  a.emp_nodata = empirical_nodata;

  // the order: keys, mask, stable sort (model/samodel.c:701-819)
  LutKeyArgs ka;
  memset(&ka, 0, sizeof ka);
  ka.rrs = d_rrs;
  ka.npix = npix;
  ka.n_bands = nb;
  ka.n_scenes = 1;
  ka.nodata = cfg->nodata_value;
  bool noise = lut->use_noise != 0 && nb >= 4;
  for (int b = 0; b < nb && noise; b++)
    if (lut->rrs_noise[b] < 1.0e-6) noise = false;  // :590-600
  ka.use_noise = noise ? 1 : 0;
  for (int k = 0; k < 3; k++) ka.noise[k] = noise ? lut->rrs_noise[k + 1] : 0.0;
  ka.out = *out;
  ka.source = d_source;
  ka.emp = d_empirical;
  int64_t *order = d_order;
  cudaError_t e = cudaSuccess;
  if (!order) {
    e = cudaMallocAsync((void **)&order, npix * sizeof(int64_t), s);
    if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "order: %s", cudaGetErrorString(e));
  }
  int64_t S = 0;
  e = lut_order(ka, order, &S, s);
  if (e != cudaSuccess) {
    if (!d_order) cudaFreeAsync(order, s);
    return cuda_fail(e, "lookup-table order");
  }
  if (S > 0) {
    const int per_sm = lut_blocks_per_sm(a);
    if (per_sm < 1) {
      if (!d_order) cudaFreeAsync(order, s);
      return fail(PHOTIC_ERR_CUDA, "lookup-table kernel does not fit on the device");
    }
    const int block = lut_block();
    const int64_t lanes = (int64_t)sms * per_sm * block;
    int64_t C = lut->n_chains ? lut->n_chains : kLutChainsPerLane * lanes;
    if (C > S) C = S;
    const int64_t per_chain = (S + C - 1) / C;
    const int64_t cap = per_chain < lut->n_lut ? per_chain : (int64_t)lut->n_lut;
    a.order = order;
    a.n_shallow = S;
    a.n_chains = C;
    a.cap = cap;
    unsigned long long *queue = nullptr;
    e = cudaMallocAsync((void **)&a.ring, (size_t)C * 8 * cap * sizeof(double), s);
    if (e == cudaSuccess)
      e = cudaMallocAsync((void **)&a.ring_src, (size_t)C * cap * sizeof(int64_t), s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&queue, sizeof *queue, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, sizeof *queue, s);
    if (e == cudaSuccess) {
      a.queue = queue;
      int64_t grid = (int64_t)sms * per_sm;
      const int64_t need = (C + block - 1) / block;
      if (grid > need) grid = need;
      e = launch_lut(a, (int)grid, s);
    }
    cudaFreeAsync(a.ring, s);
    cudaFreeAsync(a.ring_src, s);
    cudaFreeAsync(queue, s);
    if (e != cudaSuccess) {
      if (!d_order) cudaFreeAsync(order, s);
      return cuda_fail(e, "lookup-table kernel");
    }
    if (n_chains_used) *n_chains_used = C;
  }
  if (!d_order) cudaFreeAsync(order, s);
  if (n_shallow) *n_shallow = S;
  return PHOTIC_OK;
}

int photic_joint_invert_batch(const photic_config *cfg, const int32_t *d_offsets,
                              const double *d_theta_sun_deg, const float *d_rrs, int64_t npix,
                              int64_t n_obs, const photic_outputs *out, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (npix < 0 || n_obs < 0) return fail(PHOTIC_ERR_INVALID, "npix / n_obs < 0");
  if (npix == 0) return PHOTIC_OK;
  if (!d_offsets || !d_theta_sun_deg || !d_rrs || !out)
    return fail(PHOTIC_ERR_INVALID, "NULL input or output");
  if (npix > 0x7fffffffLL) return fail(PHOTIC_ERR_INVALID, "npix beyond 2^31-1");
  if (cfg->precision != PHOTIC_PREC_FP64 && cfg->precision != PHOTIC_PREC_GUARDED)
    return fail(PHOTIC_ERR_UNSUPPORTED, "the joint fit runs in FP64 only");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int *err = nullptr;
  int sms = 0;
  rc = device_state(&err, &sms);
  if (rc) return rc;

  JointArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.sc);
  a.offsets = d_offsets;
  a.theta_sun = d_theta_sun_deg;
  a.rrs = d_rrs;
  a.npix = npix;
  a.out = *out;
  a.error = err;

  // workspace: counts, starts, fills (8 x i32 each), queues (8 x u64), list
  const size_t head = 3 * 8 * sizeof(int32_t) + 8 * sizeof(unsigned long long);
  const size_t bytes = head + (size_t)npix * sizeof(int32_t);
  unsigned char *ws = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&ws, bytes, s);
  if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "joint workspace: %s", cudaGetErrorString(e));
  e = cudaMemsetAsync(ws, 0, head, s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  a.queues = reinterpret_cast<unsigned long long *>(ws);
  a.bin_count = reinterpret_cast<int32_t *>(ws + 8 * sizeof(unsigned long long));
  a.bin_start = a.bin_count + 8;
  int32_t *fill = a.bin_count + 16;
  a.list = reinterpret_cast<int32_t *>(ws + head);
  const int per_sm = cfg->blocks_per_sm;
  ForkSlot *fs = nullptr;
  rc = joint_fork(&fs);
  if (rc) {
    cudaFreeAsync(ws, s);
    return rc;
  }
  {
    std::lock_guard<std::mutex> lk(fs->mu);
    e = launch_joint(a, fill, sms, per_sm, s, &fs->f);
  }
  cudaError_t e2 = cudaFreeAsync(ws, s);
  if (e != cudaSuccess) return cuda_fail(e, "joint launch");
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFreeAsync");
  return PHOTIC_OK;
}

int photic_cost_batch(const photic_config *cfg, const float *d_rrs, const double *d_params,
                      int64_t n, double *d_cost, double *d_rrs_modelled, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!d_rrs || !d_params || !d_cost)))
    return fail(PHOTIC_ERR_INVALID, "bad arguments");
  if (n == 0) return PHOTIC_OK;
  CostArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.sc);
  make_df(*cfg, a.fp, a.sc, 6, a.ds);
  a.precision = cfg->precision;
  a.rrs = d_rrs;
  a.params = d_params;
  a.n = n;
  a.cost = d_cost;
  a.rrs_modelled = d_rrs_modelled;
  cudaError_t e = launch_cost(a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "cost kernel launch");
  return PHOTIC_OK;
}

int photic_generate_scene(const photic_config *cfg, uint64_t seed, int64_t pix0, int64_t npix,
                          double mask_frac, double noise_sigma, float *d_rrs, double *d_truth,
                          void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (npix < 0 || pix0 < 0 || !d_rrs) return fail(PHOTIC_ERR_INVALID, "bad arguments");
  GenArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.sc);
  a.seed = seed;
  a.pix0 = pix0;
  a.npix = npix;
  a.mask_frac = mask_frac;
  a.noise_sigma = noise_sigma;
  a.rrs = d_rrs;
  a.truth = d_truth;
  cudaError_t e = launch_generate(a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "generator launch");
  return PHOTIC_OK;
}

int photic_generate_field(const photic_config *cfg, uint64_t seed, int64_t nrows, int64_t ncols,
                          int64_t row0, int64_t n_rows, double mask_frac, double noise_sigma,
                          float *d_rrs, double *d_truth, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (nrows < 1 || ncols < 1 || row0 < 0 || n_rows < 0 || row0 + n_rows > nrows || !d_rrs)
    return fail(PHOTIC_ERR_INVALID, "bad arguments");
  GenArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.sc);
  a.seed = seed;
  a.pix0 = row0 * ncols;
  a.npix = n_rows * ncols;
  a.mask_frac = mask_frac;
  a.noise_sigma = noise_sigma;
  a.rrs = d_rrs;
  a.truth = d_truth;
  a.field_rows = nrows;
  a.field_cols = ncols;
  cudaError_t e = launch_generate(a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "generator launch");
  return PHOTIC_OK;
}

int photic_joint_counts(uint64_t seed, int64_t npix, int32_t kmin, int32_t kmax,
                        int32_t *d_counts, void *stream) {
  if (npix < 0 || !d_counts || kmin < 1 || kmax > PHOTIC_MAX_SCENES || kmin > kmax)
    return fail(PHOTIC_ERR_INVALID, "bad arguments (need 1 <= kmin <= kmax <= 8)");
  cudaError_t e = launch_joint_counts(seed, npix, kmin, kmax, d_counts, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "joint counts launch");
  return PHOTIC_OK;
}

int photic_generate_joint(const photic_config *cfg, uint64_t seed, int64_t npix,
                          const int32_t *d_offsets, double theta_sun_min, double theta_sun_max,
                          double mask_frac, double noise_sigma, double *d_theta_sun,
                          float *d_rrs, double *d_truth, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (npix < 0 || !d_offsets || !d_theta_sun || !d_rrs)
    return fail(PHOTIC_ERR_INVALID, "bad arguments");
  JointGenArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.sc);
  a.seed = seed;
  a.npix = npix;
  a.offsets = d_offsets;
  a.theta_min = theta_sun_min;
  a.theta_max = theta_sun_max;
  a.mask_frac = mask_frac;
  a.noise_sigma = noise_sigma;
  a.theta_sun = d_theta_sun;
  a.rrs = d_rrs;
  a.truth = d_truth;
  cudaError_t e = launch_generate_joint(a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "joint generator launch");
  return PHOTIC_OK;
}

int photic_gemm_bf16_strides(const void *d_A, int32_t lda, const void *d_B, int32_t ldb,
                             float *d_C, int32_t ldc, int32_t M, int32_t N, int32_t K,
                             int32_t lbo, int32_t sbo, void *stream) {
  if (!d_A || !d_B || !d_C || M < 0 || N < 0 || K < 16 || (K % 16) != 0)
    return fail(PHOTIC_ERR_INVALID, "GEMM needs K a positive multiple of 16");
  if ((lda % 8) || (ldb % 8) || lda < K || ldb < K || ldc < N ||
      ((uintptr_t)d_A & 15u) || ((uintptr_t)d_B & 15u))
    return fail(PHOTIC_ERR_INVALID, "GEMM operands need 16-byte aligned rows (ld % 8 == 0)");
  // The descriptors of one K = 16 step name 16 core matrices along M/N (sbo
  // apart) and 2 along K (lbo apart), 128 bytes each, starting up to 3 * 256
  // bytes into a 128 x 64 BF16 tile of 16 KB; every byte they name must lie
  // inside that tile.
  if (lbo <= 0 || sbo <= 0 || (lbo % 16) || (sbo % 16) ||
      (int64_t)3 * 256 + (int64_t)15 * sbo + lbo + 128 > (int64_t)128 * 64 * 2)
    return fail(PHOTIC_ERR_INVALID,
                "core-matrix strides lbo %d / sbo %d must be positive multiples of 16 that "
                "stay inside the 16 KB staged tile", lbo, sbo);
  unsigned int *err = nullptr;
  int sms = 0;
  int rc = device_state(&err, &sms);
  if (rc) return rc;
  GemmArgs g;
  memset(&g, 0, sizeof g);
  g.A = d_A;
  g.B = d_B;
  g.lda = lda;
  g.ldb = ldb;
  g.M = M;
  g.N = N;
  g.K = K;
  g.C = d_C;
  g.ldc = ldc;
  g.error = err;
  g.lbo = lbo;
  g.sbo = sbo;
  g.epi = EPI_F32;
  cudaError_t e = launch_gemm(g, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "GEMM launch");
  return PHOTIC_OK;
}

int photic_gemm_bf16(const void *d_A, int32_t lda, const void *d_B, int32_t ldb, float *d_C,
                     int32_t ldc, int32_t M, int32_t N, int32_t K, void *stream) {
  return photic_gemm_bf16_strides(d_A, lda, d_B, ldb, d_C, ldc, M, N, K, 128, 1024, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Surrogate network handle
// ---------------------------------------------------------------------------
struct photic_surrogate {
  MlpState st;
  void *block;  // one device allocation holding every buffer of st
  int step;
};

namespace {

// Workspace of a forward (inference) or forward+backward pass over Rpad rows.
struct WorkAlloc {
  void *mem = nullptr;
  MlpWork w{};
  cudaError_t alloc(int Rpad, bool train, cudaStream_t s) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
      size_t o = off;
      off += (bytes + 255) & ~(size_t)255;
      return o;
    };
    const size_t bfH = (size_t)Rpad * kMlpH * 2, fH = (size_t)Rpad * kMlpH * 4;
    size_t oX0 = take((size_t)Rpad * kMlpIn * 2), oA1 = take(bfH), oA2 = take(bfH), oA3 = take(bfH);
    size_t oY = take((size_t)Rpad * kMlpOut * 4);
    size_t oZ1 = 0, oZ2 = 0, oZ3 = 0, odY = 0, odZ = 0, odZ2 = 0, oT1 = 0, oT2 = 0, oG4 = 0, oG = 0,
           oSK = 0;
    if (train) {
      oZ1 = take(fH); oZ2 = take(fH); oZ3 = take(fH);
      odY = take((size_t)Rpad * kMlpOut * 2); odZ = take(bfH); odZ2 = take(bfH);
      oT1 = take(bfH); oT2 = take(bfH);
      oG4 = take((size_t)kMlpH * kMlpOut * 4); oG = take((size_t)kMlpParams * 4);
      oSK = take((size_t)kMlpSplitK * kMlpH * kMlpH * 4);
    }
    cudaError_t e = cudaMallocAsync(&mem, off, s);
    if (e != cudaSuccess) return e;
    unsigned char *b = (unsigned char *)mem;
    w.X0 = (__nv_bfloat16 *)(b + oX0);
    w.A1 = (__nv_bfloat16 *)(b + oA1);
    w.A2 = (__nv_bfloat16 *)(b + oA2);
    w.A3 = (__nv_bfloat16 *)(b + oA3);
    w.Y = (float *)(b + oY);
    if (train) {
      w.Z1 = (float *)(b + oZ1); w.Z2 = (float *)(b + oZ2); w.Z3 = (float *)(b + oZ3);
      w.dY = (__nv_bfloat16 *)(b + odY); w.dZ = (__nv_bfloat16 *)(b + odZ);
      w.dZ2 = (__nv_bfloat16 *)(b + odZ2); w.T1 = (__nv_bfloat16 *)(b + oT1);
      w.T2 = (__nv_bfloat16 *)(b + oT2); w.G4t = (float *)(b + oG4); w.grad = (float *)(b + oG);
      w.splitk = (float *)(b + oSK);
    }
    return cudaSuccess;
  }
  void release(cudaStream_t s) {
    if (mem) cudaFreeAsync(mem, s);
    mem = nullptr;
  }
};

int pad128(int64_t R) { return (int)((R + 127) / 128 * 128); }

}  // namespace

extern "C" {

int32_t photic_surrogate_num_params(void) { return kMlpParams; }

int photic_surrogate_create(photic_surrogate **out, uint64_t seed) {
  if (!out) return fail(PHOTIC_ERR_INVALID, "NULL handle");
  *out = nullptr;
  photic_surrogate *h = new photic_surrogate();
  const size_t nP = kMlpParams * sizeof(float);
  const size_t nW = (size_t)(kMlpH * kMlpIn + 2 * kMlpH * kMlpH + kMlpOut * kMlpH) * 2;
  const size_t total = 3 * nP + 2 * nW + 4 * 16 * sizeof(float) + 1024;
  cudaError_t e = cudaMalloc(&h->block, total);
  if (e != cudaSuccess) {
    delete h;
    return fail(PHOTIC_ERR_NOMEM, "surrogate: %s", cudaGetErrorString(e));
  }
  unsigned char *b = (unsigned char *)h->block;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char *p = b + off;
    off += (bytes + 255) & ~(size_t)255;
    return p;
  };
  MlpState &st = h->st;
  st.P = (float *)take(nP);
  st.M = (float *)take(nP);
  st.V = (float *)take(nP);
  st.W1b = (__nv_bfloat16 *)take((size_t)kMlpH * kMlpIn * 2);
  st.W2b = (__nv_bfloat16 *)take((size_t)kMlpH * kMlpH * 2);
  st.W3b = (__nv_bfloat16 *)take((size_t)kMlpH * kMlpH * 2);
  st.W4b = (__nv_bfloat16 *)take((size_t)kMlpOut * kMlpH * 2);
  st.W2t = (__nv_bfloat16 *)take((size_t)kMlpH * kMlpH * 2);
  st.W3t = (__nv_bfloat16 *)take((size_t)kMlpH * kMlpH * 2);
  st.W4t = (__nv_bfloat16 *)take((size_t)kMlpOut * kMlpH * 2);
  st.in_mean = (float *)take(64);
  st.in_std = (float *)take(64);
  st.out_mean = (float *)take(64);
  st.out_std = (float *)take(64);
  // Initial weights: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) from a
  // splitmix64 stream; biases 0; padded output rows 0.
  std::vector<float> P(kMlpParams, 0.0f);
  uint64_t z = seed ^ 0x9E3779B97F4A7C15ull;
  auto rnd = [&]() {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
  };
  auto fill = [&](int off0, int rows, int cols, int fan_in, int valid_rows, int valid_cols) {
    const double a = 1.0 / sqrt((double)fan_in);
    for (int r = 0; r < rows; r++)
      for (int c = 0; c < cols; c++)
        P[off0 + r * cols + c] =
            (r < valid_rows && c < valid_cols) ? (float)((2.0 * rnd() - 1.0) * a) : 0.0f;
  };
  fill(kOffW1, kMlpH, kMlpIn, 6, kMlpH, 6);
  fill(kOffW2, kMlpH, kMlpH, kMlpH, kMlpH, kMlpH);
  fill(kOffW3, kMlpH, kMlpH, kMlpH, kMlpH, kMlpH);
  fill(kOffW4, kMlpOut, kMlpH, kMlpH, 5, kMlpH);
  // Standardisation of inputs (Rrs of the 4 bands, sun and view zenith in
  // degrees) and outputs (ln P, ln G, ln X, B, H) from the synthetic prior.
  float in_mean[16] = {0.011f, 0.012f, 0.010f, 0.0035f, 35.0f, 0.0f};
  float in_std[16] = {0.006f, 0.007f, 0.007f, 0.004f, 10.0f, 10.0f};
  float out_mean[16] = {-3.80f, -3.45f, -4.95f, 0.275f, 12.75f};
  float out_std[16] = {0.865f, 1.065f, 1.129f, 0.130f, 7.07f};
  for (int i = 6; i < 16; i++) in_std[i] = 1.0f;
  for (int i = 5; i < 16; i++) out_std[i] = 1.0f;
  e = cudaMemcpy(st.P, P.data(), nP, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(st.M, 0, nP);
  if (e == cudaSuccess) e = cudaMemset(st.V, 0, nP);
  if (e == cudaSuccess) e = cudaMemcpy(st.in_mean, in_mean, 64, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(st.in_std, in_std, 64, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(st.out_mean, out_mean, 64, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(st.out_std, out_std, 64, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = mlp_refresh(st, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    cudaFree(h->block);
    delete h;
    return cuda_fail(e, "surrogate init");
  }
  h->step = 0;
  *out = h;
  return PHOTIC_OK;
}

int photic_surrogate_destroy(photic_surrogate *s) {
  if (!s) return PHOTIC_OK;
  cudaFree(s->block);
  delete s;
  return PHOTIC_OK;
}

int photic_surrogate_params(photic_surrogate *s, float *h_params, int32_t n, int32_t write) {
  if (!s || !h_params || n != kMlpParams) return fail(PHOTIC_ERR_INVALID, "bad arguments");
  cudaError_t e = write ? cudaMemcpy(s->st.P, h_params, n * sizeof(float), cudaMemcpyHostToDevice)
                        : cudaMemcpy(h_params, s->st.P, n * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && write) e = mlp_refresh(s->st, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "surrogate params");
  return PHOTIC_OK;
}

int photic_surrogate_grads(photic_surrogate *s, const float *d_x, const float *d_t, int32_t R,
                           float *d_grad, float *d_loss, void *stream) {
  if (!s || !d_x || !d_t || !d_grad || R <= 0) return fail(PHOTIC_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned int *err = nullptr;
  int sms = 0;
  int rc = device_state(&err, &sms);
  if (rc) return rc;
  WorkAlloc wa;
  const int Rpad = pad128(R);
  cudaError_t e = wa.alloc(Rpad, true, st);
  if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "surrogate workspace");
  e = mlp_backward(s->st, d_x, d_t, R, Rpad, wa.w, d_loss, err, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_grad, wa.w.grad, kMlpParams * sizeof(float), cudaMemcpyDeviceToDevice, st);
  wa.release(st);
  if (e != cudaSuccess) return cuda_fail(e, "surrogate gradients");
  return PHOTIC_OK;
}

int photic_surrogate_train_step(photic_surrogate *s, const float *d_x, const float *d_t,
                                int32_t R, float lr, float *d_loss, void *stream) {
  if (!s || !d_x || !d_t || R <= 0) return fail(PHOTIC_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned int *err = nullptr;
  int sms = 0;
  int rc = device_state(&err, &sms);
  if (rc) return rc;
  WorkAlloc wa;
  const int Rpad = pad128(R);
  cudaError_t e = wa.alloc(Rpad, true, st);
  if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "surrogate workspace");
  e = mlp_backward(s->st, d_x, d_t, R, Rpad, wa.w, d_loss, err, st);
  if (e == cudaSuccess) e = mlp_adam(s->st, wa.w, lr, ++s->step, st);
  wa.release(st);
  if (e != cudaSuccess) return cuda_fail(e, "surrogate train step");
  return PHOTIC_OK;
}

int photic_surrogate_infer(photic_surrogate *s, const float *d_x, int64_t R, float *d_y,
                           void *stream) {
  if (!s || !d_x || !d_y || R < 0) return fail(PHOTIC_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned int *err = nullptr;
  int sms = 0;
  int rc = device_state(&err, &sms);
  if (rc) return rc;
  const int64_t chunk = 1 << 20;
  for (int64_t r0 = 0; r0 < R; r0 += chunk) {
    const int n = (int)((R - r0) < chunk ? (R - r0) : chunk);
    WorkAlloc wa;
    const int Rpad = pad128(n);
    cudaError_t e = wa.alloc(Rpad, false, st);
    if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "surrogate workspace");
    e = mlp_forward(s->st, d_x + r0 * 6, n, Rpad, wa.w, err, st);
    if (e == cudaSuccess) e = mlp_denorm(s->st, wa.w, n, d_y + r0 * 5, st);
    wa.release(st);
    if (e != cudaSuccess) return cuda_fail(e, "surrogate inference");
  }
  return PHOTIC_OK;
}

int photic_surrogate_seed(photic_surrogate *s, const photic_config *cfg, const float *d_rrs,
                          int64_t npix, double resid_max, double *d_seeds, float *d_resid,
                          void *stream) {
  return photic_surrogate_seed_polished(s, cfg, d_rrs, npix, resid_max, 0, d_seeds, d_resid,
                                        stream);
}

}  // extern "C"

namespace {

// Polish the guesses y ([npix][5] ln P, ln G, ln X, B, H; NULL: the
// reference's cold-start guess at depth h_guess) into nelmin seeds.
cudaError_t launch_seed_polish(const photic_config &cfg, const float *d_rrs, int64_t npix,
                               const float *y, double h_guess, double resid_max,
                               int32_t polish_iters, double *d_seeds, float *d_resid,
                               cudaStream_t st) {
  SeedArgs a;
  memset(&a, 0, sizeof a);
  make_fit(cfg, a.fp);
  make_scene(cfg, cfg.theta_sun_deg, a.sc);
  a.rrs = d_rrs;
  a.y = y;
  a.h_guess = h_guess;
  a.npix = npix;
  a.resid_max = resid_max;
  a.polish_iters = polish_iters;
  for (int b = 0; b < 8; b++) {
    a.sf.refl[b] = (float)a.sc.refl[b];
    a.sf.aw[b] = (float)a.sc.aw[b];
    a.sf.a0[b] = (float)a.sc.a0[b];
    a.sf.a1[b] = (float)a.sc.a1[b];
    a.sf.eS[b] = (float)a.sc.eS[b];
    a.sf.bbw[b] = (float)a.sc.bbw[b];
  }
  a.sf.sec_sun = (float)a.sc.sec_sun;
  a.sf.sec_view = (float)a.sc.sec_view;
  a.seeds = d_seeds;
  a.resid = d_resid;
  return mlp_seeds(a, st);
}

}  // namespace

extern "C" {

int photic_seed_polished_heuristic(const photic_config *cfg, const float *d_rrs, int64_t npix,
                                   double h_guess, double resid_max, int32_t polish_iters,
                                   double *d_seeds, float *d_resid, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (npix < 0 || (npix > 0 && (!d_rrs || !d_seeds)) || polish_iters < 0 ||
      polish_iters > 100 || !(h_guess > 0.0))
    return fail(PHOTIC_ERR_INVALID, "bad arguments");
  if (npix == 0) return PHOTIC_OK;
  cudaError_t e = launch_seed_polish(*cfg, d_rrs, npix, nullptr, h_guess, resid_max,
                                     polish_iters, d_seeds, d_resid, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "heuristic seeds");
  return PHOTIC_OK;
}

int photic_surrogate_seed_polished(photic_surrogate *s, const photic_config *cfg,
                                   const float *d_rrs, int64_t npix, double resid_max,
                                   int32_t polish_iters, double *d_seeds, float *d_resid,
                                   void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (!s || npix < 0 || (npix > 0 && (!d_rrs || !d_seeds)) || polish_iters < 0 ||
      polish_iters > 100)
    return fail(PHOTIC_ERR_INVALID, "bad arguments");
  if (npix == 0) return PHOTIC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  float *x = nullptr, *y = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&x, (size_t)npix * 6 * sizeof(float), st);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&y, (size_t)npix * 5 * sizeof(float), st);
  if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "seed workspace");
  e = mlp_features(d_rrs, npix, cfg->n_bands, (float)cfg->theta_sun_deg,
                   (float)cfg->theta_view_deg, x, st);
  if (e == cudaSuccess) {
    rc = photic_surrogate_infer(s, x, npix, y, stream);
    if (rc == PHOTIC_OK)
      e = launch_seed_polish(*cfg, d_rrs, npix, y, 0.0, resid_max, polish_iters, d_seeds,
                             d_resid, st);
  }
  cudaFreeAsync(x, st);
  cudaFreeAsync(y, st);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "surrogate seeds");
  return PHOTIC_OK;
}

int photic_set_guard_stats(unsigned long long *d_stats) {
  g_guard_stats_ptr = d_stats;
  return PHOTIC_OK;
}

int photic_set_counter(unsigned long long *d_counter) {
  g_counter_ptr = d_counter;
  return PHOTIC_OK;
}

int photic_measure_peaks(double *fp64_tflops, double *fp32_tflops, double *mufu_tops) {
  if (!fp64_tflops || !fp32_tflops || !mufu_tops) return fail(PHOTIC_ERR_INVALID, "NULL output");
  cudaError_t e = measure_peaks(fp64_tflops, fp32_tflops, mufu_tops);
  if (e != cudaSuccess) return cuda_fail(e, "peak probes");
  return PHOTIC_OK;
}

int photic_sync(void *stream) {
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  unsigned int *err = nullptr;
  int sms = 0;
  int rc = device_state(&err, &sms);
  if (rc) return rc;
  unsigned int h = 0;
  e = cudaMemcpy(&h, err, sizeof h, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy error word");
  if (h) {
    cudaMemset(err, 0, sizeof h);
    if (h & PHOTIC_DEVERR_EVAL_CAP)
      return fail(PHOTIC_ERR_TIMEOUT, "a pixel exceeded the evaluation cap (device error 0x%x)", h);
    return fail(PHOTIC_ERR_INVALID, "device reported invalid input (device error 0x%x)", h);
  }
  return PHOTIC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// photic_invert_batch_noalloc: the plain-method inversion for callers that
// must not allocate device memory.
//
// Its only scratch -- the 8-byte work-queue head and a 4-byte error word --
// lives in this file-scope array instead of a per-call allocation.  The
// array is part of the library's device image: every GPU that loads the
// library holds PHOTIC_NOALLOC_SCRATCH_BYTES of it until the process exits.
// Host code cannot use the array's name as a device address, so the address
// is looked up with cudaGetSymbolAddress once per device, on the first call
// made with that device current.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned long long
    g_noalloc_scratch[PHOTIC_NOALLOC_SCRATCH_BYTES / sizeof(unsigned long long)];

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned long long *g_noalloc_ptr[kNoAllocMaxDevices];
int g_noalloc_sms[kNoAllocMaxDevices];

// Device address of the scratch array and SM count of the current device.
int noalloc_setup(unsigned long long **ptr, int *sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(PHOTIC_ERR_UNSUPPORTED, "device %d beyond the %d supported", dev, kNoAllocMaxDevices);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_ptr[dev] == nullptr) {
    unsigned long long *p = nullptr;
    e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    g_noalloc_sms[dev] = n;
    g_noalloc_ptr[dev] = p;
  }
  *ptr = g_noalloc_ptr[dev];
  *sms = g_noalloc_sms[dev];
  return PHOTIC_OK;
}

}  // namespace

extern "C" int photic_invert_batch_noalloc(const photic_config *cfg, const float *d_rrs,
                                           int64_t npix, int64_t pixel_stride,
                                           int64_t band_stride, const double *d_seeds,
                                           const photic_outputs *out, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (npix < 0) return fail(PHOTIC_ERR_INVALID, "npix < 0");
  if (npix == 0) return PHOTIC_OK;
  if (!d_rrs || !out) return fail(PHOTIC_ERR_INVALID, "NULL input or output");
  if (pixel_stride < 1 || band_stride < 1)
    return fail(PHOTIC_ERR_INVALID, "strides must be >= 1");
  if (cfg->precision == PHOTIC_PREC_FP32 || cfg->precision == PHOTIC_PREC_GUARDED)
    return fail(PHOTIC_ERR_UNSUPPORTED,
                "precision %d is not offered without allocation (fp64 and df64 are)",
                cfg->precision);
  // Kernel-detected errors (the evaluation cap) reach the caller only
  // through the per-pixel status: the error word in the static array is
  // cleared by the next call and never read back.
  if (!out->status)
    return fail(PHOTIC_ERR_INVALID, "the allocation-free inversion needs out->status");
  // queue head (8 bytes) + error word (4 bytes, padded to 8)
  const size_t needed = 2 * sizeof(unsigned long long);
  if (needed > (size_t)PHOTIC_NOALLOC_SCRATCH_BYTES)
    return fail(PHOTIC_ERR_INVALID, "needs %zu bytes of scratch, the static array holds %d",
                needed, PHOTIC_NOALLOC_SCRATCH_BYTES);
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long *scratch = nullptr;
  int sms = 0;
  rc = noalloc_setup(&scratch, &sms);
  if (rc) return rc;

  InvertArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.sc);
  make_df(*cfg, a.fp, a.sc, 6, a.ds);
  a.rrs = d_rrs;
  a.npix = npix;
  a.pixel_stride = pixel_stride;
  a.band_stride = band_stride;
  a.vec4 = (cfg->n_bands == 4 && pixel_stride == 4 && band_stride == 1 &&
            ((uintptr_t)d_rrs & 15u) == 0);
  a.seeds = d_seeds;
  a.out = *out;
  a.queue = scratch;
  a.error = reinterpret_cast<unsigned int *>(scratch + 1);
  a.early_exit = cfg->early_exit_per_scene * (double)(float)1;

  const int block =
      cfg->block_threads ? cfg->block_threads : default_invert_block(cfg->precision);
  int per_sm = cfg->blocks_per_sm;
  if (per_sm == 0) {
    per_sm = invert_blocks_per_sm(a, cfg->precision, block);
    if (per_sm < 1) return fail(PHOTIC_ERR_CUDA, "kernel does not fit on the device");
  }
  int64_t grid = (int64_t)sms * per_sm;
  const int64_t need = (npix + block - 1) / block;
  if (grid > need) grid = need;

  // The previous call left its final queue position and error bits here.
  cudaError_t e = cudaMemsetAsync(scratch, 0, needed, s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(noalloc scratch)");
  e = launch_invert(a, cfg->precision, block, (int)grid, s);
  if (e != cudaSuccess) return cuda_fail(e, "invert kernel launch");
  return PHOTIC_OK;
}

// ---------------------------------------------------------------------------
// Link-compatible samodel entry points (include/photic_samodel.h).
// ---------------------------------------------------------------------------
#include "../../include/photic_samodel.h"

namespace {

// The reference's hard-coded nelmin tolerances (model/samodel.c:2142-2144).
void reference_tolerances(photic_config &cfg) {
  cfg.reqmin = 1.0e-2;
  cfg.konvge = 100;
  cfg.kcount = 5000;
}

// Configuration and band constants of scene s of a model_data, taking the
// constants as the caller prepared them (model/samodel.c:521-618).
int from_md(const photic_model_data *md, int s, photic_config &cfg, FitParams &fp,
            SceneConsts &sc) {
  if (!md || s < 0 || s >= md->n_scenes) return fail(PHOTIC_ERR_INVALID, "bad model_data");
  photic_config_default(&cfg);
  const int nb = md->n_bands[s];
  if (nb < 2 || nb > PHOTIC_MAX_BANDS) return fail(PHOTIC_ERR_INVALID, "n_bands %d", nb);
  cfg.n_bands = nb;
  for (int b = 0; b < nb; b++) cfg.wavelengths[b] = md->wavelengths[s][b];
  cfg.theta_sun_deg = md->theta_sun ? md->theta_sun[s] * (180.0 / kPiHost) : 0.0;
  cfg.theta_view_deg = md->theta_view ? md->theta_view[s] * (180.0 / kPiHost) : 0.0;
  cfg.h_tide = md->H_tide ? md->H_tide[s] : 0.0;
  reference_tolerances(cfg);
  if (md->empirical_depth_present) {
    cfg.n_hstarts = 1;
    cfg.hstarts[0] = md->h_empirical;
  }
  int rc = photic_config_check(&cfg);
  if (rc) return rc;
  make_fit(cfg, fp);
  fp.aw640 = md->a_w640;
  memset(&sc, 0, sizeof sc);
  const int bt = md->bottom_type_indexes[0];
  for (int b = 0; b < nb; b++) {
    const double l = md->wavelengths[s][b];
    sc.wl[b] = l;
    sc.a0[b] = md->a_0[s][b];
    sc.a1[b] = md->a_1[s][b];
    sc.aw[b] = md->a_w[s][b];
    sc.bbw[b] = md->b_bw[s][b];
    sc.refl[b] = md->bottom_reflectance[bt][s][b];
    sc.eS[b] = exp(-0.015 * (l - 440.0));
    sc.ratio440[b] = 440.0 / l;
  }
  sc.sec_sun = md->sec_theta_sun[s];
  sc.sec_view = md->sec_theta_view[s];
  sc.h_tide = cfg.h_tide;
  return PHOTIC_OK;
}

// Single-scene inversion with prepared constants (same kernel and launch
// shape as photic_invert_batch).
int invert_prepared(const photic_config &cfg, const FitParams &fp, const SceneConsts &sc,
                    const float *d_rrs, int64_t npix, const double *d_seeds,
                    const photic_outputs &out, cudaStream_t s) {
  unsigned int *err = nullptr;
  int sms = 0;
  int rc = device_state(&err, &sms);
  if (rc) return rc;
  InvertArgs a;
  memset(&a, 0, sizeof a);
  a.fp = fp;
  a.sc = sc;
  make_df(cfg, a.fp, a.sc, 6, a.ds);
  a.rrs = d_rrs;
  a.npix = npix;
  a.pixel_stride = cfg.n_bands;
  a.band_stride = 1;
  a.vec4 = cfg.n_bands == 4 && ((uintptr_t)d_rrs & 15u) == 0;
  a.seeds = d_seeds;
  a.out = out;
  a.error = err;
  a.early_exit = cfg.early_exit_per_scene * (double)(float)1;
  a.no_mask = 1;  // the mask test belongs to samodel()'s pixel loop
  const int block = default_invert_block(PHOTIC_PREC_FP64);
  int per_sm = invert_blocks_per_sm(a, PHOTIC_PREC_FP64, block);
  if (per_sm < 1) return fail(PHOTIC_ERR_CUDA, "kernel does not fit on the device");
  int64_t grid = (int64_t)sms * per_sm;
  if (grid > (npix + block - 1) / block) grid = (npix + block - 1) / block;
  unsigned long long *queue = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&queue, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "queue head");
  cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  a.queue = queue;
  e = launch_invert(a, PHOTIC_PREC_FP64, block, (int)grid, s);
  cudaFreeAsync(queue, s);
  if (e != cudaSuccess) return cuda_fail(e, "invert launch");
  return PHOTIC_OK;
}

// Cost with details at n parameter vectors, prepared constants.
int cost_prepared(const photic_config &cfg, const FitParams &fp, const SceneConsts &sc,
                  const float *d_rrs, const double *d_params, int64_t n, double *d_cost,
                  double *d_rm, double *d_det, cudaStream_t s) {
  CostArgs a;
  memset(&a, 0, sizeof a);
  a.fp = fp;
  a.sc = sc;
  make_df(cfg, a.fp, a.sc, 6, a.ds);
  a.precision = PHOTIC_PREC_FP64;
  a.rrs = d_rrs;
  a.params = d_params;
  a.n = n;
  a.cost = d_cost;
  a.rrs_modelled = d_rm;
  a.details = d_det;
  cudaError_t e = launch_cost(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "cost launch");
  return PHOTIC_OK;
}

// Launch the general fit over a prepared RegionArgs (grid or list mode); allocates and frees the queue head on the stream.
int run_region(RegionArgs &a, int max_params, int per_sm, cudaStream_t s) {
  unsigned int *err = nullptr;
  int sms = 0;
  int rc = device_state(&err, &sms);
  if (rc) return rc;
  a.error = err;
  unsigned long long *queue = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&queue, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "queue head");
  cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  a.queue = queue;
  e = launch_region(a, max_params, sms, per_sm, s);
  cudaFreeAsync(queue, s);
  if (e != cudaSuccess) return cuda_fail(e, "region launch");
  return PHOTIC_OK;
}

// Device scratch of the per-pixel drop-ins: one block per host thread and
// device, allocated on the thread's first call and reused by every later one
// (a caller that drives its own nelmin over samodel_error makes about a
// thousand calls per pixel; none of them allocates).  It is released when the
// thread exits.
constexpr size_t kArenaBytes = 1 << 16;
struct DropinArena {
  unsigned char *mem = nullptr;
  int dev = -1;
  ~DropinArena() {
    if (mem) cudaFree(mem);
  }
};
thread_local DropinArena g_arena;

unsigned char *dropin_arena() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  if (g_arena.mem && g_arena.dev == dev) return g_arena.mem;
  if (g_arena.mem) {  // the thread moved to another device
    cudaSetDevice(g_arena.dev);
    cudaFree(g_arena.mem);
    cudaSetDevice(dev);
    g_arena.mem = nullptr;
  }
  if (cudaMalloc((void **)&g_arena.mem, kArenaBytes) != cudaSuccess) {
    g_arena.mem = nullptr;
    return nullptr;
  }
  g_arena.dev = dev;
  return g_arena.mem;
}

// Views into the arena for the one-region, one-bottom drop-ins.
struct PixelScratch {
  unsigned char *mem = nullptr;
  float *rrs;
  double *params, *cost, *rm, *det, *depth64;
  float *f[9];
  int32_t *evals_kept, *status;
  int alloc() {
    mem = dropin_arena();
    if (!mem) return fail(PHOTIC_ERR_NOMEM, "drop-in scratch");
    rrs = (float *)(mem);
    params = (double *)(mem + 128);
    cost = (double *)(mem + 256);
    rm = (double *)(mem + 320);
    det = (double *)(mem + 448);
    depth64 = (double *)(mem + 512);
    for (int i = 0; i < 9; i++) f[i] = (float *)(mem + 640 + 64 * i);
    evals_kept = (int32_t *)(mem + 1280);
    status = (int32_t *)(mem + 1344);
    return PHOTIC_OK;
  }
};

// A model_data problem for the general kernel (photic_region.cu): regions,
// scenes and bottom types as the caller set them, fitted (eval == nullptr)
// or its cost evaluated at eval.  The arena above 4 KB holds its inputs and
// outputs; one copy in and one copy out.
struct MixIn {
  float rrs[kRegionMaxR * PHOTIC_MAX_SCENES * PHOTIC_MAX_BANDS];
  int32_t R, origin;
  double h_emp;
  double params[96];
};
struct MixOut {
  double depth, kept[96];
  float P[PHOTIC_MAX_SCENES], G[PHOTIC_MAX_SCENES], X[PHOTIC_MAX_SCENES];
  float albedo, model_error, rrs_error, K_min, iod, pct[3], type;
  int32_t evals_kept, status;
  double cost, det[8], rm[kRegionMaxR * PHOTIC_MAX_SCENES * PHOTIC_MAX_BANDS];
};

int mix_call(photic_model_data *md, const photic_config &cfg, const FitParams &fp,
             const SceneConsts &sc, const double *eval, MixOut &res) {
  const int R = md->n_regions, S = md->n_scenes, nbt = md->n_bottoms, nb = cfg.n_bands;
  if (R < 1 || R > kRegionMaxR || S < 1 || S > PHOTIC_MAX_SCENES || nbt < 1 || nbt > 3)
    return fail(PHOTIC_ERR_UNSUPPORTED, "1..9 regions, 1..8 scenes and 1..3 bottom types");
  if (R * S * nb > 128 || R * S > 64 || region_max_params(R, nbt, S) > 96)
    return fail(PHOTIC_ERR_UNSUPPORTED, "regions x scenes x bands beyond 128");
  if (md->origin < 0 || md->origin >= R) return fail(PHOTIC_ERR_INVALID, "origin region");
  for (int s = 1; s < S; s++) {
    if (md->n_bands[s] != nb) return fail(PHOTIC_ERR_UNSUPPORTED, "scenes with other bands");
    for (int b = 0; b < nb; b++)
      if (md->wavelengths[s][b] != md->wavelengths[0][b])
        return fail(PHOTIC_ERR_UNSUPPORTED, "scenes with other wavelengths");
  }
  unsigned char *mem = dropin_arena();
  if (!mem) return fail(PHOTIC_ERR_NOMEM, "drop-in scratch");
  MixIn in;
  memset(&in, 0, sizeof in);
  for (int r = 0; r < R; r++)
    for (int s = 0; s < S; s++)
      for (int b = 0; b < nb; b++)
        in.rrs[(r * S + s) * nb + b] = (float)md->Rrs_measured[r][s][b];
  in.R = R;
  in.origin = md->origin;
  // the empirical depth picks the starts (and sand alone below 8 m) of a fit
  in.h_emp = (!eval && md->empirical_depth_present) ? md->h_empirical : NAN;
  const int n = region_max_params(R, nbt, S);
  if (eval)
    for (int i = 0; i < n; i++) in.params[i] = eval[i];
  MixIn *d_in = (MixIn *)(mem + 4096);
  MixOut *d_out = (MixOut *)(mem + 4096 + ((sizeof(MixIn) + 255) / 256) * 256);
  cudaError_t e = cudaMemcpy(d_in, &in, sizeof in, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "drop-in inputs");
  RegionArgs a;
  memset(&a, 0, sizeof a);
  a.fp = fp;
  a.sc = sc;
  for (int s = 0; s < S; s++) a.sec_sun[s] = md->sec_theta_sun[s];
  a.npix = 1;
  a.n_scenes = S;
  a.n_spatial = 1;
  a.n_bottoms = nbt;
  a.no_mask = 1;
  a.h_emp = &d_in->h_emp;
  a.list_rrs = d_in->rrs;
  a.list_R = &d_in->R;
  a.list_origin = &d_in->origin;
  a.eval_stride = 96;
  photic_outputs &o = a.out;
  if (eval) {
    a.eval_params = d_in->params;
    a.eval_cost = &d_out->cost;
    a.eval_rm = d_out->rm;
    a.eval_det = d_out->det;
  } else {
    a.list_params = d_out->kept;
    o.depth_f64 = &d_out->depth;
    o.P = d_out->P;
    o.G = d_out->G;
    o.X = d_out->X;
    o.bottom_albedo = &d_out->albedo;
    o.model_error = &d_out->model_error;
    o.rrs_error = &d_out->rrs_error;
    o.K_min = &d_out->K_min;
    o.iod = &d_out->iod;
    o.bottom_percent = d_out->pct;
    o.bottom_type = &d_out->type;
    o.evals_kept = &d_out->evals_kept;
    o.status = &d_out->status;
  }
  int rc = run_region(a, n, 0, 0);
  if (rc == PHOTIC_OK) rc = photic_sync(0);
  if (rc) return rc;
  e = cudaMemcpy(&res, d_out, sizeof res, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "drop-in outputs");
  if (!eval && (res.status & 0xFF) != PHOTIC_PX_FITTED)
    return fail(PHOTIC_ERR_CUDA, "the fit did not complete");
  return PHOTIC_OK;
}

// Band constants of all bottom types a model_data mixes.
void mix_bottoms(const photic_model_data *md, SceneConsts &sc, int nb) {
  for (int k = 0; k < md->n_bottoms && k < 3; k++)
    for (int b = 0; b < nb; b++)
      sc.refl_k[k][b] = md->bottom_reflectance[md->bottom_type_indexes[k]][0][b];
}

// Post-fit products of samodel_optimise (model/samodel.c:1994-2097) for
// one region and one bottom type, from the kept vector and its details.
void store_fit(photic_model_data *md, const double *best, const double *det, int s,
               int evals_kept, int converged) {
  md->depth = fabs(best[0]);
  md->Rrs_error = det[0];
  md->model_error = det[1];
  md->bottom_albedo = det[2];
  md->K_min = det[3];
  md->index_optical_depth = det[4];
  for (int k = 0; k < 12; k++) md->B_type_percent[k] = 0.0;
  const int bt = md->bottom_type_indexes[0];
  md->B_type_percent[bt] = 100.0 * fabs(best[2]) / fabs(best[2]);
  md->bottom_type = 1 + bt;
  md->P[s] = 0.01 * fabs(best[3]);
  md->G[s] = 0.01 * fabs(best[4]);
  md->X[s] = 0.01 * fabs(best[5]);
  if (md->prev) {
    md->prev[0] = fabs(best[3]);
    md->prev[1] = fabs(best[4]);
    md->prev[2] = fabs(best[5]);
  }
  md->n_iterations = evals_kept;
  md->converged = converged;
}

// The single-scene fit of samodel_optimise_one_bottom_combination
// (model/samodel.c:2119-2427) for md's one region and bottom type: the kept
// vector (signed, as nelmin left it), the cost details and modelled Rrs at
// it, the evaluations of the kept start and the pixel status.
int fit_single(photic_model_data *md, const photic_config &cfg, FitParams fp,
               const SceneConsts &sc, PixelScratch &ps, double best[6], double det[5],
               double *rm, int32_t *ek, int32_t *st) {
  const int nb = cfg.n_bands;
  float r[PHOTIC_MAX_BANDS];
  for (int b = 0; b < nb; b++) r[b] = (float)md->Rrs_measured[0][0][b];
  cudaMemcpy(ps.rrs, r, nb * sizeof(float), cudaMemcpyHostToDevice);
  photic_outputs o;
  memset(&o, 0, sizeof o);
  o.params = ps.params;
  o.evals_kept = ps.evals_kept;
  o.status = ps.status;
  // Hot start from the previous optimum (model/samodel.c:2234-2241,
  // 2285-2305): one start whose steps are the cold-start ratios, i.e. a
  // seed with step scale 1.
  const double *d_seed = nullptr;
  if (md->start_at_previous && md->prev) {
    const double r490 = interp_apply(resolve_interp(md->wavelengths[0], nb, 490.0),
                                     md->Rrs_measured[0][0]);
    const double seed[6] = {md->empirical_depth_present ? md->h_empirical : md->depth_prev,
                            100.0 * 4.0 * r490, 1.0, md->prev[0], md->prev[1], md->prev[2]};
    cudaMemcpy(ps.depth64, seed, sizeof seed, cudaMemcpyHostToDevice);
    d_seed = ps.depth64;
    fp.seed_step_scale = 1.0;
  }
  int rc = invert_prepared(cfg, fp, sc, ps.rrs, 1, d_seed, o, 0);
  if (rc) return rc;
  rc = cost_prepared(cfg, fp, sc, ps.rrs, ps.params, 1, ps.cost, ps.rm, ps.det, 0);
  if (rc) return rc;
  rc = photic_sync(0);
  if (rc) return rc;
  cudaMemcpy(best, ps.params, 6 * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(det, ps.det, 5 * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(rm, ps.rm, nb * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(ek, ps.evals_kept, sizeof *ek, cudaMemcpyDeviceToHost);
  cudaMemcpy(st, ps.status, sizeof *st, cudaMemcpyDeviceToHost);
  if ((*st & 0xFF) != PHOTIC_PX_FITTED)
    return fail(PHOTIC_ERR_CUDA, "the fit did not complete");
  return PHOTIC_OK;
}

bool f_close_ref(float a, float b) { return f_close(a, b, 1.0e-6f); }

}  // namespace

extern "C" {

int photic_forward_batch(const photic_config *cfg, const double *d_params,
                         const double *d_rrs440, const double *d_rrs490, int64_t n,
                         double *d_rrs, double *d_K, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!d_params || !d_rrs440 || !d_rrs490 || !d_rrs)))
    return fail(PHOTIC_ERR_INVALID, "bad arguments");
  if (n == 0) return PHOTIC_OK;
  ForwardArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.sc);
  a.params = d_params;
  a.rrs440 = d_rrs440;
  a.rrs490 = d_rrs490;
  a.n = n;
  a.rrs = d_rrs;
  a.K = d_K;
  cudaError_t e = launch_forward(a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "forward launch");
  return PHOTIC_OK;
}

}  // extern "C"

namespace {

// Rrs at 440/490/550/640/750 nm of every region and scene, stored as the
// reference does (model/samodel.c:1783-1799).
void store_reference_rrs(photic_model_data *md) {
  const double targets[5] = {440.0, 490.0, 550.0, 640.0, 750.0};
  double **dst[5] = {md->Rrs440, md->Rrs490, md->Rrs550, md->Rrs640, md->Rrs750};
  for (int r = 0; r < md->n_regions; r++)
    for (int s = 0; s < md->n_scenes; s++)
      for (int t = 0; t < 5; t++) {
        double v = interp_apply(resolve_interp(md->wavelengths[s], md->n_bands[s], targets[t]),
                                md->Rrs_measured[r][s]);
        if (t == 0 && v < 0.0) v = 0.0001;
        if (dst[t]) dst[t][r][s] = v;
      }
}

// samodel_optimise for regions, bottom mixtures and scene stacks through the
// general kernel: the fit, then the cost at the kept vector for the modelled
// spectra, then the post-fit products (model/samodel.c:1994-2104).
// params (optional) receives |kept vector| as
// samodel_optimise_one_bottom_combination returns it (:2413-2417).
void optimise_general(photic_model_data *md, double *params) {
  if (md->start_at_previous) {
    fail(PHOTIC_ERR_UNSUPPORTED,
         "samodel_optimise: the hot start is built for one region and one bottom type");
    return;
  }
  if (md->n_bottoms < 1 || md->n_bottoms > 3) {
    fail(PHOTIC_ERR_UNSUPPORTED, "samodel_optimise: 1..3 bottom types");
    return;
  }
  // ALL_BOTTOMS: every type at once, in table order (model/samodel.c:1836-1840)
  for (int k = 0; k < md->n_bottoms; k++) md->bottom_type_indexes[k] = k;
  photic_config cfg;
  FitParams fp;
  SceneConsts sc;
  if (from_md(md, 0, cfg, fp, sc)) return;
  mix_bottoms(md, sc, cfg.n_bands);
  store_reference_rrs(md);
  MixOut fit, ev;
  if (mix_call(md, cfg, fp, sc, nullptr, fit)) return;
  // a pixel deeper than 8 m was fitted with sand alone (model/samodel.c:1826-1830)
  const int nbt = (md->empirical_depth_present && md->h_empirical > 8.0) ? 1 : md->n_bottoms;
  const int saved = md->n_bottoms;
  md->n_bottoms = nbt;
  const int R = md->n_regions, S = md->n_scenes, nb = cfg.n_bands;
  const int n = region_max_params(R, nbt, S), off = R + 2 * nbt * R;
  int rc = mix_call(md, cfg, fp, sc, fit.kept, ev);
  md->n_bottoms = saved;  // restored as the reference does (:2104)
  if (rc) return;
  // the products in double precision, as the reference keeps them: from the
  // re-evaluation at the kept vector and from the vector itself
  md->depth = fit.depth;
  md->Rrs_error = ev.det[0];
  md->model_error = ev.det[1];
  md->bottom_albedo = ev.det[2];
  md->index_optical_depth = ev.det[4];
  md->K_min = ev.det[5];
  for (int k = 0; k < 12; k++) md->B_type_percent[k] = 0.0;
  double q_sum = 0.0, largest = 0.0;  // model/samodel.c:2021-2047
  const int qo = R + R * nbt + md->origin * nbt;
  for (int k = 0; k < nbt; k++) q_sum += fabs(fit.kept[qo + k]);
  for (int k = 0; k < nbt; k++) {
    md->B_type_percent[k] = 100.0 * fabs(fit.kept[qo + k]) / q_sum;
    if (md->B_type_percent[k] > largest) {
      largest = md->B_type_percent[k];
      md->bottom_type = (int)(1.0 + k);
    }
  }
  for (int s = 0; s < S; s++) {
    md->P[s] = 0.01 * fabs(fit.kept[off + 3 * s]);
    md->G[s] = 0.01 * fabs(fit.kept[off + 1 + 3 * s]);
    md->X[s] = 0.01 * fabs(fit.kept[off + 2 + 3 * s]);
    if (md->prev) {
      md->prev[3 * s] = fabs(fit.kept[off + 3 * s]);
      md->prev[3 * s + 1] = fabs(fit.kept[off + 1 + 3 * s]);
      md->prev[3 * s + 2] = fabs(fit.kept[off + 2 + 3 * s]);
    }
  }
  for (int r = 0; r < R; r++)
    for (int s = 0; s < S; s++)
      for (int b = 0; b < nb; b++)
        md->Rrs_modelled[r][s][b] = ev.rm[(r * S + s) * nb + b];
  md->n_iterations = fit.evals_kept;
  md->converged = (fit.status & PHOTIC_PX_CONVERGED) != 0;
  if (params)
    for (int i = 0; i < n; i++) params[i] = fabs(fit.kept[i]);
}

bool needs_general(const photic_model_data *md) {
  return md->n_regions != 1 || md->n_bottoms != 1;
}

}  // namespace

extern "C" {

void samodel_optimise(photic_model_data *md) {
  g_err.clear();
  if (!md) {
    fail(PHOTIC_ERR_INVALID, "NULL model_data");
    return;
  }
  if (needs_general(md)) {
    optimise_general(md, nullptr);
    return;
  }
  PixelScratch ps;
  if (ps.alloc()) return;
  const int ns = md->n_scenes;
  photic_config cfg;
  FitParams fp;
  SceneConsts sc;
  if (from_md(md, 0, cfg, fp, sc)) return;
  const int nb = cfg.n_bands;
  // Rrs at 440/490/550/640/750 nm per scene, stored as the reference does
  // (model/samodel.c:1783-1799).
  const double targets[5] = {440.0, 490.0, 550.0, 640.0, 750.0};
  double **dst[5] = {md->Rrs440, md->Rrs490, md->Rrs550, md->Rrs640, md->Rrs750};
  for (int s = 0; s < ns; s++)
    for (int t = 0; t < 5; t++) {
      double v = interp_apply(resolve_interp(md->wavelengths[s], md->n_bands[s], targets[t]),
                              md->Rrs_measured[0][s]);
      if (t == 0 && v < 0.0) v = 0.0001;
      if (dst[t]) dst[t][0][s] = v;
    }
  if (ns == 1) {
    double best[6], det[5], rm[PHOTIC_MAX_BANDS];
    int32_t ek = 0, st = 0;
    if (fit_single(md, cfg, fp, sc, ps, best, det, rm, &ek, &st)) return;
    store_fit(md, best, det, 0, ek, (st & PHOTIC_PX_CONVERGED) != 0);
    for (int b = 0; b < nb; b++) md->Rrs_modelled[0][0][b] = rm[b];
    return;
  }
  // Temporal joint fit (n_scenes = k), reference layout.
  if (ns > PHOTIC_MAX_SCENES) {
    fail(PHOTIC_ERR_UNSUPPORTED, "at most %d scenes", PHOTIC_MAX_SCENES);
    return;
  }
  std::vector<float> r((size_t)ns * nb);
  std::vector<double> th(ns);
  for (int s = 0; s < ns; s++) {
    for (int b = 0; b < nb; b++) r[(size_t)s * nb + b] = (float)md->Rrs_measured[0][s][b];
    th[s] = md->theta_sun[s] * (180.0 / kPiHost);
  }
  unsigned char *mem = nullptr;
  if (cudaMalloc((void **)&mem, 8192) != cudaSuccess) {
    fail(PHOTIC_ERR_NOMEM, "drop-in scratch");
    return;
  }
  int32_t offs[2] = {0, ns};
  int32_t *d_off = (int32_t *)mem;
  double *d_th = (double *)(mem + 64);
  float *d_r = (float *)(mem + 256);
  double *d_depth = (double *)(mem + 1024);
  float *d_P = (float *)(mem + 1088), *d_G = (float *)(mem + 1152), *d_X = (float *)(mem + 1216);
  float *d_f = (float *)(mem + 1280);  // albedo, model, rrs error, K_min, iod
  int32_t *d_i = (int32_t *)(mem + 1344);
  cudaMemcpy(d_off, offs, sizeof offs, cudaMemcpyHostToDevice);
  cudaMemcpy(d_th, th.data(), ns * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(d_r, r.data(), r.size() * sizeof(float), cudaMemcpyHostToDevice);
  photic_outputs o;
  memset(&o, 0, sizeof o);
  o.depth_f64 = d_depth;
  o.P = d_P;
  o.G = d_G;
  o.X = d_X;
  o.bottom_albedo = d_f;
  o.model_error = d_f + 1;
  o.rrs_error = d_f + 2;
  o.K_min = d_f + 3;
  o.iod = d_f + 4;
  o.evals_kept = d_i;
  o.status = d_i + 1;
  cfg.theta_sun_deg = th[0];
  int rc = photic_joint_invert_batch(&cfg, d_off, d_th, d_r, 1, ns, &o, 0);
  if (rc == PHOTIC_OK) rc = photic_sync(0);
  if (rc == PHOTIC_OK) {
    double H;
    float P[PHOTIC_MAX_SCENES], G[PHOTIC_MAX_SCENES], X[PHOTIC_MAX_SCENES], f[5];
    int32_t iv[2];
    cudaMemcpy(&H, d_depth, sizeof H, cudaMemcpyDeviceToHost);
    cudaMemcpy(P, d_P, ns * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(G, d_G, ns * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(X, d_X, ns * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(f, d_f, sizeof f, cudaMemcpyDeviceToHost);
    cudaMemcpy(iv, d_i, sizeof iv, cudaMemcpyDeviceToHost);
    md->depth = H;
    md->bottom_albedo = f[0];
    md->model_error = f[1];
    md->Rrs_error = f[2];
    md->K_min = f[3];
    md->index_optical_depth = f[4];
    for (int s = 0; s < ns; s++) {
      md->P[s] = P[s];
      md->G[s] = G[s];
      md->X[s] = X[s];
    }
    for (int k = 0; k < 12; k++) md->B_type_percent[k] = 0.0;
    md->B_type_percent[md->bottom_type_indexes[0]] = 100.0;
    md->bottom_type = 1 + md->bottom_type_indexes[0];
    md->n_iterations = iv[0];
    md->converged = (iv[1] & PHOTIC_PX_CONVERGED) != 0;
  }
  cudaFree(mem);
}

void samodel_optimise_one_bottom_combination(photic_model_data *md, double *params) {
  g_err.clear();
  if (!md || !params) {
    fail(PHOTIC_ERR_INVALID, "NULL argument");
    return;
  }
  if (needs_general(md) || md->n_scenes != 1) {
    optimise_general(md, params);
    return;
  }
  photic_config cfg;
  FitParams fp;
  SceneConsts sc;
  if (from_md(md, 0, cfg, fp, sc)) return;
  PixelScratch ps;
  if (ps.alloc()) return;
  double best[6], det[5], rm[PHOTIC_MAX_BANDS];
  int32_t ek = 0, st = 0;
  if (fit_single(md, cfg, fp, sc, ps, best, det, rm, &ek, &st)) return;
  for (int i = 0; i < 6; i++) params[i] = fabs(best[i]);  // model/samodel.c:2415-2417
  md->n_iterations = ek;
  md->converged = (st & PHOTIC_PX_CONVERGED) != 0;
  // what the final samodel_error(best) leaves in md (model/samodel.c:2413)
  for (int b = 0; b < cfg.n_bands; b++) md->Rrs_modelled[0][0][b] = rm[b];
  md->Rrs_error = det[0];
  md->model_error = det[1];
  md->bottom_albedo = det[2];
  md->depth = fabs(best[0]) + cfg.h_tide;
}

double samodel_error(double *params, photic_model_data *md) {
  g_err.clear();
  if (!md || !params) {
    fail(PHOTIC_ERR_INVALID, "NULL argument");
    return NAN;
  }
  if (needs_general(md) || md->n_scenes != 1) {
    // regions, bottom mixtures or scenes: the general kernel's cost at params
    photic_config cfg;
    FitParams fp;
    SceneConsts sc;
    if (md->n_bottoms < 1 || md->n_bottoms > 3) {
      fail(PHOTIC_ERR_UNSUPPORTED, "samodel_error: 1..3 bottom types");
      return NAN;
    }
    if (from_md(md, 0, cfg, fp, sc)) return NAN;
    mix_bottoms(md, sc, cfg.n_bands);
    MixOut ev;
    if (mix_call(md, cfg, fp, sc, params, ev)) return NAN;
    const int R = md->n_regions, S = md->n_scenes, nb = cfg.n_bands;
    for (int r = 0; r < R; r++)
      for (int s = 0; s < S; s++)
        for (int b = 0; b < nb; b++) md->Rrs_modelled[r][s][b] = ev.rm[(r * S + s) * nb + b];
    md->Rrs_error = ev.det[0];
    md->model_error = ev.det[1];
    md->bottom_albedo = ev.det[2];
    return ev.cost;
  }
  photic_config cfg;
  FitParams fp;
  SceneConsts sc;
  if (from_md(md, 0, cfg, fp, sc)) return NAN;
  PixelScratch ps;
  if (ps.alloc()) return NAN;
  const int nb = cfg.n_bands;
  float r[PHOTIC_MAX_BANDS];
  for (int b = 0; b < nb; b++) r[b] = (float)md->Rrs_measured[0][0][b];
  cudaMemcpy(ps.rrs, r, nb * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(ps.params, params, 6 * sizeof(double), cudaMemcpyHostToDevice);
  if (cost_prepared(cfg, fp, sc, ps.rrs, ps.params, 1, ps.cost, ps.rm, ps.det, 0)) return NAN;
  if (photic_sync(0)) return NAN;
  double c, det[5], rm[PHOTIC_MAX_BANDS];
  cudaMemcpy(&c, ps.cost, sizeof c, cudaMemcpyDeviceToHost);
  cudaMemcpy(det, ps.det, sizeof det, cudaMemcpyDeviceToHost);
  cudaMemcpy(rm, ps.rm, nb * sizeof(double), cudaMemcpyDeviceToHost);
  for (int b = 0; b < nb; b++) md->Rrs_modelled[0][0][b] = rm[b];
  md->Rrs_error = det[0];
  md->model_error = det[1];
  md->bottom_albedo = det[2];
  return c;
}

void samodel_Rrs(double P, double G, double X, double B[], double q[], double H, double Delta,
                 photic_model_data *md, int k_scene, int k_band, int k_region) {
  g_err.clear();
  if (!md || !B || !q || md->n_bottoms < 1 || md->n_bottoms > 3) {
    fail(PHOTIC_ERR_UNSUPPORTED, "samodel_Rrs: 1..3 bottom types");
    return;
  }
  photic_config cfg;
  FitParams fp;
  SceneConsts sc;
  if (from_md(md, k_scene, cfg, fp, sc)) return;
  if (k_band < 0 || k_band >= cfg.n_bands) {
    fail(PHOTIC_ERR_INVALID, "k_band out of range");
    return;
  }
  // reflectances of the bottom types md mixes (model/samodel.c:2880-2883)
  for (int k = 0; k < md->n_bottoms; k++)
    for (int b = 0; b < cfg.n_bands; b++)
      sc.refl_k[k][b] = md->bottom_reflectance[md->bottom_type_indexes[k]][k_scene][b];
  unsigned char *mem = dropin_arena();
  if (!mem) {
    fail(PHOTIC_ERR_NOMEM, "drop-in scratch");
    return;
  }
  // one upload: row, Rrs(440), Rrs(490), mixture; one download of the band
  struct In {
    double row[8], r440, r490, mix[6];
  } in;
  struct Out {
    double rrs[PHOTIC_MAX_BANDS], K[PHOTIC_MAX_BANDS], parts[PHOTIC_MAX_BANDS * 4];
  } out;
  memset(&in, 0, sizeof in);
  const double row[7] = {P, G, X, B[0], q[0], H, Delta};
  memcpy(in.row, row, sizeof row);
  in.r440 = md->Rrs440[k_region][k_scene];
  in.r490 = md->Rrs490[k_region][k_scene];
  for (int k = 0; k < md->n_bottoms; k++) {
    in.mix[k] = B[k];
    in.mix[3 + k] = q[k];
  }
  In *d_in = (In *)(mem + 8192);
  Out *d_out = (Out *)(mem + 8192 + 1024);
  cudaError_t e = cudaMemcpy(d_in, &in, sizeof in, cudaMemcpyHostToDevice);
  ForwardArgs a;
  memset(&a, 0, sizeof a);
  a.fp = fp;
  a.sc = sc;
  a.params = d_in->row;
  a.rrs440 = &d_in->r440;
  a.rrs490 = &d_in->r490;
  a.n = 1;
  a.rrs = d_out->rrs;
  a.K = d_out->K;
  a.parts = d_out->parts;
  if (md->n_bottoms > 1) {
    a.mix = d_in->mix;
    a.n_bottoms = md->n_bottoms;
  }
  if (e == cudaSuccess) e = launch_forward(a, 0);
  if (e == cudaSuccess) e = cudaMemcpy(&out, d_out, sizeof out, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    cuda_fail(e, "samodel_Rrs");
    return;
  }
  md->Rrs_modelled[k_region][k_scene][k_band] = out.rrs[k_band];
  md->K[k_scene][k_band] = out.K[k_band];
  const double *parts = out.parts + 4 * k_band;
  if (md->rho) md->rho[k_region][k_scene][k_band] = parts[0];
  if (md->rrs_dp) md->rrs_dp[k_region][k_scene][k_band] = parts[1];
  if (md->rrs_bottom) md->rrs_bottom[k_region][k_scene][k_band] = parts[2];
  if (md->rrs_modelled) md->rrs_modelled[k_region][k_scene][k_band] = parts[3];
  // the reference's side effects (model/samodel.c:2873-2883)
  md->depth = H + sc.h_tide;
  double albedo = 0.0;
  for (int k = 0; k < md->n_bottoms; k++) albedo += q[k] * B[k];
  md->bottom_albedo = albedo;
}

}  // extern "C"

namespace {

// The result grids samodel() writes when it ends (model/samodel.c:1492-1690),
// as netCDF files in the current directory: for each scene
// <scene>_K_coastal / _K_blue / _K_green / _K_red.nc (K of bands 0..3 at the
// fit, :1153-1156) and <scene>_P / _G / _X.nc (:1157-1159), then
// modelled_H, _H_sigma, _error, _albedo, _bottom_sand, _bottom_seagrass,
// _bottom_coral, _min_K, _bottom_type and _index_optical_depth.nc from the
// caller's grids.  Coordinates and spval come from the first band grid of
// the first scene (:1498-1510).  K is the forward model's K at the fitted
// P, G, X with the pixel's measured Rrs(440)/Rrs(490): from the fit's
// double parameters for one scene fitted pixel by pixel, from the stored
// float P, G, X for the joint and region fits.  Unfitted pixels hold 0.
int samodel_write_files(const photic_config &cfg, const photic_scene *scene_data,
                        const photic_geogrid *gridded_data, const int *scene_indexes,
                        int nscenes, int nrows, int ncols, const std::vector<float> &h_rrs,
                        const std::vector<int32_t> &st, const std::vector<float> &pgx,
                        const std::vector<double> &params6, const std::vector<int64_t> &kpix,
                        float **const *outs) {
  const int nb = cfg.n_bands;
  const int64_t npix = (int64_t)nrows * ncols, nobs = npix * nscenes;
  const photic_geogrid &g0 = gridded_data[scene_data[scene_indexes[0]].band_indexes[0]];
  std::vector<float> lons((size_t)ncols), lats((size_t)nrows);
  for (int n = 0; n < ncols; n++) lons[n] = g0.wlon + ((float)n) * g0.cellsize;
  for (int n = 0; n < nrows; n++) lats[n] = g0.slat + ((float)n) * g0.cellsize;
  const double spval = g0.nodata_value;
  float *d_grid = nullptr;
  double *d_buf = nullptr;
  const size_t nbuf = (size_t)npix * (7 + 2 + 2 * (size_t)nb);
  if (cudaMalloc((void **)&d_grid, (size_t)npix * sizeof(float)) != cudaSuccess ||
      cudaMalloc((void **)&d_buf, nbuf * sizeof(double)) != cudaSuccess) {
    cudaFree(d_grid);
    return fail(PHOTIC_ERR_NOMEM, "samodel: result-file buffers");
  }
  double *d_p7 = d_buf, *d_440 = d_p7 + 7 * npix, *d_490 = d_440 + npix;
  double *d_rm = d_490 + npix, *d_K = d_rm + (size_t)nb * npix;
  std::vector<float> host((size_t)npix);
  int rc = PHOTIC_OK;
  auto put = [&](const std::string &name) {
    if (rc != PHOTIC_OK) return;
    printf("\nWriting file %s...", name.c_str());
    cudaError_t e = cudaMemcpy(d_grid, host.data(), (size_t)npix * sizeof(float),
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "samodel: result grid upload");
      return;
    }
    rc = photic_nc_write_grid(name.c_str(), d_grid, ncols, nrows, lons.data(), lats.data(),
                              spval, nullptr);
  };
  auto fitted = [&](int64_t p) { return (st[p] & 0xFF) == PHOTIC_PX_FITTED; };
  std::vector<double> p7((size_t)npix * 7), r440((size_t)npix), r490((size_t)npix);
  std::vector<double> K((size_t)npix * nb);
  const char *kname[4] = {"K_coastal", "K_blue", "K_green", "K_red"};
  for (int k = 0; k < nscenes && rc == PHOTIC_OK; k++) {
    const photic_scene &sk = scene_data[scene_indexes[k]];
    std::string sname(sk.scene_name, strnlen(sk.scene_name, sizeof sk.scene_name));
    size_t b0 = 0, e0 = sname.size();
    while (b0 < e0 && isspace((unsigned char)sname[b0])) b0++;
    while (e0 > b0 && isspace((unsigned char)sname[e0 - 1])) e0--;
    sname = sname.substr(b0, e0 - b0);
    for (int64_t p = 0; p < npix; p++) {
      const size_t o = (size_t)(p * nscenes + k);
      double P = 0.01, G = 0.01, X = 0.01;
      if (fitted(p)) {
        if (!params6.empty()) {
          P = 0.01 * fabs(params6[(size_t)p * 6 + 3]);
          G = 0.01 * fabs(params6[(size_t)p * 6 + 4]);
          X = 0.01 * fabs(params6[(size_t)p * 6 + 5]);
        } else {
          P = pgx[o];
          G = pgx[(size_t)nobs + o];
          X = pgx[2 * (size_t)nobs + o];
        }
      }
      // md->K holds the last region's K (model/samodel.c:2911-2915): Y from
      // that region's spectrum (kpix: its pixel; empty: the pixel itself)
      const size_t ok = kpix.empty() ? o : (size_t)(kpix[p] * nscenes + k);
      double rr[PHOTIC_MAX_BANDS];
      for (int b = 0; b < nb; b++) rr[b] = h_rrs[ok * nb + b];
      double a440 = photic_interp_1d(cfg.wavelengths, rr, nb, 440.0);
      if (a440 < 0.0) a440 = 0.0001;  // model/samodel.c:1785-1799
      r440[p] = a440;
      r490[p] = photic_interp_1d(cfg.wavelengths, rr, nb, 490.0);
      const double row[7] = {P, G, X, 0.0, 1.0, 1.0, 0.0};
      memcpy(&p7[(size_t)p * 7], row, sizeof row);
    }
    photic_config ck = cfg;
    ck.theta_sun_deg = sk.theta_w;
    cudaMemcpy(d_p7, p7.data(), p7.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_440, r440.data(), r440.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_490, r490.data(), r490.size() * sizeof(double), cudaMemcpyHostToDevice);
    rc = photic_forward_batch(&ck, d_p7, d_440, d_490, npix, d_rm, d_K, nullptr);
    if (rc == PHOTIC_OK) rc = photic_sync(nullptr);
    if (rc != PHOTIC_OK) break;
    cudaMemcpy(K.data(), d_K, K.size() * sizeof(double), cudaMemcpyDeviceToHost);
    for (int kb = 0; kb < 4; kb++) {
      for (int64_t p = 0; p < npix; p++)
        host[p] = fitted(p) && kb < nb ? (float)K[(size_t)p * nb + kb] : 0.0f;
      put(sname + "_" + kname[kb] + ".nc");
    }
    const char *pname[3] = {"P", "G", "X"};
    for (int c = 0; c < 3; c++) {
      for (int64_t p = 0; p < npix; p++) {
        const size_t o = (size_t)(p * nscenes + k);
        host[p] = fitted(p) ? pgx[(size_t)c * nobs + o] : 0.0f;
      }
      put(sname + "_" + pname[c] + ".nc");
    }
  }
  const char *gname[10] = {"modelled_H.nc", "modelled_H_sigma.nc", "modelled_error.nc",
                           "modelled_albedo.nc", "modelled_bottom_sand.nc",
                           "modelled_bottom_seagrass.nc", "modelled_bottom_coral.nc",
                           "modelled_min_K.nc", "modelled_bottom_type.nc",
                           "modelled_index_optical_depth.nc"};
  for (int f = 0; f < 10 && rc == PHOTIC_OK; f++) {
    for (int i = 0; i < nrows; i++)
      for (int j = 0; j < ncols; j++) host[(size_t)i * ncols + j] = outs[f] ? outs[f][i][j] : 0.0f;
    put(gname[f]);
  }
  if (rc == PHOTIC_OK) printf("\n... finished.\n");
  cudaFree(d_grid);
  cudaFree(d_buf);
  return rc;
}

}  // namespace

extern "C" {

void samodel(photic_scene scene_data[], photic_geogrid gridded_data[], int *scene_indexes,
             int nscenes, int empirical_depth_present, photic_geogrid empirical_depths,
             int n_smoothing_radius, int n_spatial, int n_bottoms, float **depth,
             float **depth_sigma, float **model_error, float **bottom_albedo, float **bottom_sand,
             float **bottom_seagrass, float **bottom_coral, float **K_min, float **bottom_type,
             float **index_optical_depth, float pagesize, int background, int linewidth) {
  g_err.clear();
  (void)pagesize;
  (void)background;
  (void)linewidth;
  if (!scene_data || !gridded_data || !scene_indexes || nscenes < 1 ||
      nscenes > PHOTIC_MAX_SCENES) {
    fail(PHOTIC_ERR_INVALID, "samodel: bad scenes");
    return;
  }
  if (n_spatial > 2 || n_bottoms < 1 || n_bottoms > 3) {
    fail(PHOTIC_ERR_UNSUPPORTED, "samodel: n_spatial <= 2 and n_bottoms 1..3 (sand, seagrass, "
                                 "coral)");
    return;
  }
  if (n_smoothing_radius > 1) {
    fail(PHOTIC_ERR_UNSUPPORTED, "samodel: spectral smoothing (radius > 1) is not built");
    return;
  }
  const bool regions = n_spatial == 2;
  const photic_scene &s0 = scene_data[scene_indexes[0]];
  const int nrows = s0.nrows, ncols = s0.ncols, nb = s0.n_bands;
  photic_config cfg;
  photic_config_default(&cfg);
  cfg.n_bands = nb;
  for (int b = 0; b < nb && b < PHOTIC_MAX_BANDS; b++) cfg.wavelengths[b] = s0.wavelengths[b];
  cfg.theta_sun_deg = s0.theta_w;
  cfg.theta_view_deg = s0.theta_v;
  cfg.h_tide = s0.H_tide;
  reference_tolerances(cfg);
  if (photic_config_check(&cfg)) return;
  for (int k = 1; k < nscenes; k++) {
    const photic_scene &sk = scene_data[scene_indexes[k]];
    if (sk.n_bands != nb || sk.nrows != nrows || sk.ncols != ncols) {
      fail(PHOTIC_ERR_UNSUPPORTED, "samodel: scenes must share grid and bands");
      return;
    }
  }
  const int64_t npix = (int64_t)nrows * ncols;
  const int64_t nobs = npix * nscenes;
  // Gather the band grids into [pixel][scene][band] with one nodata marker.
  std::vector<float> h_rrs((size_t)nobs * nb);
  for (int k = 0; k < nscenes; k++) {
    const photic_scene &sk = scene_data[scene_indexes[k]];
    for (int b = 0; b < nb; b++) {
      const photic_geogrid &g = gridded_data[sk.band_indexes[b]];
      for (int i = 0; i < nrows; i++)
        for (int j = 0; j < ncols; j++) {
          float v = g.array[i][j];
          if (f_close_ref(v, g.nodata_value)) v = cfg.nodata_value;
          h_rrs[(((size_t)i * ncols + j) * nscenes + k) * nb + b] = v;
        }
    }
  }
  // The general loop (bottom mixtures, 3 x 3 regions, stacks of scenes)
  // takes scene-major grids; the single-scene loop takes [pixel][band].
  const bool general = n_bottoms > 1 || regions || nscenes > 1;
  std::vector<float> h_grid;
  if (general) {
    h_grid.resize(h_rrs.size());
    for (int64_t p = 0; p < npix; p++)
      for (int k = 0; k < nscenes; k++)
        for (int b = 0; b < nb; b++)
          h_grid[((size_t)k * npix + p) * nb + b] = h_rrs[((size_t)p * nscenes + k) * nb + b];
  }
  // device buffers
  float *d_rrs = nullptr;
  double *d_depth = nullptr;
  float *d_f = nullptr, *d_pgx = nullptr, *d_mix = nullptr, *d_raw = nullptr;
  double *d_params = nullptr;
  int32_t *d_status = nullptr;
  const bool one_by_one = nscenes == 1 && !general;
  bool ok = cudaMalloc((void **)&d_rrs, h_rrs.size() * sizeof(float)) == cudaSuccess &&
            cudaMalloc((void **)&d_depth, npix * sizeof(double)) == cudaSuccess &&
            cudaMalloc((void **)&d_f, 4 * npix * sizeof(float)) == cudaSuccess &&
            cudaMalloc((void **)&d_status, npix * sizeof(int32_t)) == cudaSuccess &&
            cudaMalloc((void **)&d_pgx, 3 * nobs * sizeof(float)) == cudaSuccess &&
            (!one_by_one ||
             cudaMalloc((void **)&d_params, 6 * npix * sizeof(double)) == cudaSuccess) &&
            (!general || cudaMalloc((void **)&d_mix, 4 * npix * sizeof(float)) == cudaSuccess);
  if (!ok) {
    fail(PHOTIC_ERR_NOMEM, "samodel: device buffers");
  } else {
    cudaMemcpy(d_rrs, general ? h_grid.data() : h_rrs.data(), h_rrs.size() * sizeof(float),
               cudaMemcpyHostToDevice);
    photic_outputs o;
    memset(&o, 0, sizeof o);
    o.depth_f64 = d_depth;
    o.rrs_error = d_f;
    o.bottom_albedo = d_f + npix;
    o.K_min = d_f + 2 * npix;
    o.iod = d_f + 3 * npix;
    o.status = d_status;
    o.P = d_pgx;  // per observation for the joint fit
    o.G = d_pgx + nobs;
    o.X = d_pgx + 2 * nobs;
    o.params = d_params;
    int rc = PHOTIC_OK;
    // The reference's product path is its pixel loop with the dynamic
    // lookup table (LUT 1, :649-1352) in every configuration, ordered by the
    // spectral index (times the spectral angle to the scenes' R_sigma) or by
    // the empirical depths when given (:702-767), the sorted pixels cut into
    // chains -- PHOTIC_LUT_CHAINS of them if set (1: the reference on one
    // thread), else eight per resident lane (one scene, one region, one
    // bottom type) or warp (the general fit).
    photic_lut_config lc;
    photic_lut_config_default(&lc);
    const char *ch = getenv("PHOTIC_LUT_CHAINS");
    if (ch && *ch) lc.n_chains = atoll(ch);
    if (empirical_depth_present) {
      std::vector<float> raw((size_t)npix);
      for (int i = 0; i < nrows; i++)
        for (int j = 0; j < ncols; j++) raw[(size_t)i * ncols + j] = empirical_depths.array[i][j];
      if (cudaMalloc((void **)&d_raw, npix * sizeof(float)) == cudaSuccess)
        cudaMemcpy(d_raw, raw.data(), npix * sizeof(float), cudaMemcpyHostToDevice);
      else
        rc = fail(PHOTIC_ERR_NOMEM, "samodel: empirical depth grid");
    }
    const float emp_nodata = empirical_depth_present ? empirical_depths.nodata_value : 0.0f;
    // per scene: sun zenith and R_sigma (the noise of the order and of the
    // depth uncertainty)
    double th[PHOTIC_MAX_SCENES], noise[PHOTIC_MAX_SCENES * PHOTIC_MAX_BANDS];
    for (int k = 0; k < nscenes; k++) {
      const photic_scene &sk = scene_data[scene_indexes[k]];
      th[k] = sk.theta_w;
      for (int b = 0; b < nb; b++) noise[k * nb + b] = sk.R_sigma[b];
    }
    if (rc != PHOTIC_OK) {
    } else if (general) {
      // P, G, X come out as [pixel][scene]
      o.bottom_percent = d_mix;
      o.bottom_type = d_mix + 3 * npix;
      rc = photic_region_lut_invert_batch(&cfg, &lc, d_rrs, nscenes, th, nrows, ncols,
                                          regions ? 2 : 1, n_bottoms, noise, d_raw, emp_nodata,
                                          &o, nullptr, nullptr, nullptr, nullptr, nullptr, 0);
    } else {
      lc.use_noise = 1;
      for (int b = 0; b < nb && b < PHOTIC_MAX_BANDS; b++) lc.rrs_noise[b] = s0.R_sigma[b];
      rc = photic_lut_invert_batch(&cfg, &lc, d_rrs, npix, d_raw, emp_nodata, &o, nullptr,
                                   nullptr, nullptr, nullptr, nullptr, 0);
    }
    if (rc == PHOTIC_OK) rc = photic_sync(0);
    if (rc == PHOTIC_OK) {
      std::vector<double> H((size_t)npix);
      std::vector<float> f((size_t)4 * npix);
      std::vector<int32_t> st((size_t)npix);
      std::vector<float> mix;
      if (general) {
        mix.resize((size_t)4 * npix);
        cudaMemcpy(mix.data(), d_mix, mix.size() * sizeof(float), cudaMemcpyDeviceToHost);
      }
      cudaMemcpy(H.data(), d_depth, npix * sizeof(double), cudaMemcpyDeviceToHost);
      cudaMemcpy(f.data(), d_f, 4 * npix * sizeof(float), cudaMemcpyDeviceToHost);
      cudaMemcpy(st.data(), d_status, npix * sizeof(int32_t), cudaMemcpyDeviceToHost);
      // depth uncertainty of the fitted grid (:1368-1479)
      std::vector<float> sig((size_t)npix, 0.0f);
      if (depth_sigma) {
        std::vector<float> hpos((size_t)npix);
        for (int64_t p = 0; p < npix; p++)
          hpos[p] = (st[p] & 0xFF) == PHOTIC_PX_FITTED ? (float)H[p] : 0.0f;
        float *d_hpos = nullptr, *d_sig = nullptr;
        if (cudaMalloc((void **)&d_hpos, npix * sizeof(float)) == cudaSuccess &&
            cudaMalloc((void **)&d_sig, npix * sizeof(float)) == cudaSuccess) {
          cudaMemcpy(d_hpos, hpos.data(), npix * sizeof(float), cudaMemcpyHostToDevice);
          if (general)  // the general fit's refits of each sample's regions
            rc = photic_region_depth_sigma(&cfg, d_rrs, nscenes, th, nrows, ncols,
                                           regions ? 2 : 1, n_bottoms, d_hpos, noise, 128, 1,
                                           d_sig, nullptr, nullptr, nullptr, nullptr);
          else
            rc = photic_depth_sigma(&cfg, d_rrs, npix, d_hpos, noise, 128, 1, d_sig, nullptr,
                                    nullptr, nullptr, nullptr);
          if (rc == PHOTIC_OK) rc = photic_sync(nullptr);
          if (rc == PHOTIC_OK)
            cudaMemcpy(sig.data(), d_sig, npix * sizeof(float), cudaMemcpyDeviceToHost);
        } else {
          rc = fail(PHOTIC_ERR_NOMEM, "samodel: depth-sigma buffers");
        }
        cudaFree(d_hpos);
        cudaFree(d_sig);
      }
      // outputs as the reference's pixel loop leaves them (:820-831,
      // :1120-1164), depth negative below the datum (:1486-1490)
      for (int i = 0; i < nrows && rc == PHOTIC_OK; i++)
        for (int j = 0; j < ncols; j++) {
          const size_t p = (size_t)i * ncols + j;
          const bool fit = (st[p] & 0xFF) == PHOTIC_PX_FITTED;
          depth[i][j] = fit ? (float)H[p] * -1.0f : 0.0f * -1.0f;
          if (depth_sigma) depth_sigma[i][j] = sig[p];
          model_error[i][j] = fit ? f[p] : 0.0f;
          bottom_albedo[i][j] = fit ? f[npix + p] : 0.0f;
          // shares of sand, seagrass and coral and the bottom type
          // (model/samodel.c:2021-2047, stored at :1120-1164)
          bottom_sand[i][j] = fit ? (general ? mix[3 * p] : 100.0f) : -9999.0f;
          bottom_seagrass[i][j] = fit ? (general ? mix[3 * p + 1] : 0.0f) : -9999.0f;
          bottom_coral[i][j] = fit ? (general ? mix[3 * p + 2] : 0.0f) : -9999.0f;
          K_min[i][j] = fit ? f[2 * npix + p] : 0.0f;
          bottom_type[i][j] = fit ? (general ? mix[3 * npix + p] : 1.0f) : -9999.0f;
          index_optical_depth[i][j] = fit ? f[3 * npix + p] : 0.0f;
        }
      if (rc == PHOTIC_OK) {
        std::vector<float> pgx((size_t)3 * nobs);
        std::vector<double> params6;
        cudaMemcpy(pgx.data(), d_pgx, pgx.size() * sizeof(float), cudaMemcpyDeviceToHost);
        if (one_by_one) {
          params6.resize((size_t)6 * npix);
          cudaMemcpy(params6.data(), d_params, params6.size() * sizeof(double),
                     cudaMemcpyDeviceToHost);
        }
        float **const outs[10] = {depth,     depth_sigma, model_error, bottom_albedo,
                                  bottom_sand, bottom_seagrass, bottom_coral, K_min,
                                  bottom_type, index_optical_depth};
        // the last region of each pixel's 3 x 3 neighbourhood in
        // extract_Rrs_data's order (model/samodel.c:2970-3025)
        std::vector<int64_t> kpix;
        if (regions) {
          kpix.resize((size_t)npix);
          for (int i = 0; i < nrows; i++)
            for (int j = 0; j < ncols; j++) {
              int64_t last = (int64_t)i * ncols + j;
              for (int ii = -1; ii <= 1; ii++)
                for (int jj = -1; jj <= 1; jj++) {
                  const int iii = std::min(std::max(i + ii, 0), nrows - 1);
                  const int jjj = std::min(std::max(j + jj, 0), ncols - 1);
                  const int64_t q = (int64_t)iii * ncols + jjj;
                  bool nodata = false;
                  for (int k = 0; k < nscenes && !nodata; k++)
                    for (int b = 0; b < nb; b++)
                      if (h_rrs[((size_t)q * nscenes + k) * nb + b] == cfg.nodata_value)
                        nodata = true;
                  if (!nodata) last = q;
                }
              kpix[(size_t)i * ncols + j] = last;
            }
        }
        samodel_write_files(cfg, scene_data, gridded_data, scene_indexes, nscenes, nrows, ncols,
                            h_rrs, st, pgx, params6, kpix, outs);
      }
    }
  }
  cudaFree(d_rrs);
  cudaFree(d_depth);
  cudaFree(d_f);
  cudaFree(d_pgx);
  cudaFree(d_params);
  cudaFree(d_status);
  if (d_mix) cudaFree(d_mix);
  if (d_raw) cudaFree(d_raw);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Launch-shape autotuner.
// ---------------------------------------------------------------------------
namespace {

struct TuneBuffers {
  std::vector<void *> ptrs;
  void *get(size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return p;
  }
  ~TuneBuffers() {
    for (void *p : ptrs) cudaFree(p);
  }
};

}  // namespace

extern "C" int photic_autotune(photic_config *cfg, int32_t kind, int64_t sample_npix,
                               double *results, int32_t max_results, int32_t *n_results) {
  g_err.clear();
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if ((kind != PHOTIC_TUNE_INVERT && kind != PHOTIC_TUNE_JOINT) || sample_npix < 1 ||
      sample_npix > (1LL << 26) || (max_results > 0 && !results))
    return fail(PHOTIC_ERR_INVALID, "bad autotune arguments");
  const int nb = cfg->n_bands;
  TuneBuffers buf;
  photic_outputs o;
  memset(&o, 0, sizeof o);
  float *rrs = nullptr;
  int32_t *offs = nullptr;
  double *theta = nullptr;
  int64_t n_obs = sample_npix;
  const uint64_t seed = 0x7475e5eedULL;
  if (kind == PHOTIC_TUNE_INVERT) {
    rrs = (float *)buf.get((size_t)sample_npix * nb * sizeof(float));
    if (!rrs) return fail(PHOTIC_ERR_NOMEM, "autotune sample");
    rc = photic_generate_scene(cfg, seed, 0, sample_npix, 0.15, 2.0e-4, rrs, nullptr, nullptr);
    if (rc) return rc;
  } else {
    offs = (int32_t *)buf.get((size_t)(sample_npix + 1) * sizeof(int32_t));
    if (!offs) return fail(PHOTIC_ERR_NOMEM, "autotune sample");
    rc = photic_joint_counts(seed, sample_npix, 2, PHOTIC_MAX_SCENES, offs + 1, nullptr);
    if (rc) return rc;
    std::vector<int32_t> h((size_t)sample_npix + 1, 0);
    cudaMemcpy(h.data() + 1, offs + 1, sample_npix * sizeof(int32_t), cudaMemcpyDeviceToHost);
    for (int64_t p = 1; p <= sample_npix; p++) h[p] += h[p - 1];
    n_obs = h[sample_npix];
    cudaMemcpy(offs, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    theta = (double *)buf.get((size_t)n_obs * sizeof(double));
    rrs = (float *)buf.get((size_t)n_obs * nb * sizeof(float));
    if (!theta || !rrs) return fail(PHOTIC_ERR_NOMEM, "autotune sample");
    rc = photic_generate_joint(cfg, seed, sample_npix, offs, 25.0, 50.0, 0.0, 2.0e-4, theta, rrs,
                               nullptr, nullptr);
    if (rc) return rc;
  }
  o.depth = (float *)buf.get((size_t)sample_npix * sizeof(float));
  o.status = (int32_t *)buf.get((size_t)sample_npix * sizeof(int32_t));
  if (!o.depth || !o.status) return fail(PHOTIC_ERR_NOMEM, "autotune outputs");
  if (kind == PHOTIC_TUNE_JOINT) {
    o.P = (float *)buf.get((size_t)n_obs * sizeof(float));
    if (!o.P) return fail(PHOTIC_ERR_NOMEM, "autotune outputs");
  }

  // candidates: thread-per-pixel blocks of 64/128/256 (the joint kernel's
  // block is fixed at 128) x blocks per SM (0 = occupancy limit)
  const int blocks_inv[3] = {64, 128, 256};
  const int per_sm_inv[4] = {0, 2, 3, 4};
  const int per_sm_joint[5] = {2, 3, 4, 6, 8};
  std::vector<std::pair<int, int>> cand;
  if (kind == PHOTIC_TUNE_INVERT) {
    for (int b : blocks_inv)
      for (int s : per_sm_inv) cand.push_back({b, s});
  } else {
    for (int s : per_sm_joint) cand.push_back({128, s});
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_ms = 0.0f;
  int best = -1, nres = 0;
  for (size_t c = 0; c < cand.size(); c++) {
    photic_config t = *cfg;
    t.block_threads = cand[c].first;
    t.blocks_per_sm = cand[c].second;
    float ms = 0.0f;
    for (int rep = 0; rep < 2 && rc == PHOTIC_OK; rep++) {  // first run untimed
      cudaEventRecord(e0, 0);
      rc = kind == PHOTIC_TUNE_INVERT
               ? photic_invert_batch(&t, rrs, sample_npix, nb, 1, nullptr, &o, nullptr)
               : photic_joint_invert_batch(&t, offs, theta, rrs, sample_npix, n_obs, &o, nullptr);
      cudaEventRecord(e1, 0);
      if (rc == PHOTIC_OK) rc = photic_sync(nullptr);
      cudaEventElapsedTime(&ms, e0, e1);
    }
    if (rc) break;
    if (nres < max_results) {
      results[3 * nres + 0] = cand[c].first;
      results[3 * nres + 1] = cand[c].second;
      results[3 * nres + 2] = ms;
      nres++;
    }
    if (best < 0 || ms < best_ms) {
      best = (int)c;
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (n_results) *n_results = nres;
  if (rc) return rc;
  cfg->block_threads = kind == PHOTIC_TUNE_INVERT ? cand[best].first : 0;
  cfg->blocks_per_sm = cand[best].second;
  return PHOTIC_OK;
}

// ---------------------------------------------------------------------------
// Depth uncertainty (model/samodel.c:1368-1479).
// ---------------------------------------------------------------------------
extern "C" int photic_depth_sigma(const photic_config *cfg, const float *d_rrs, int64_t npix,
                                  const float *d_depth, const double *r_sigma, int32_t n_samples,
                                  uint64_t seed, float *d_depth_sigma, double *d_table,
                                  int32_t *d_sample_pixel, double *d_sample_depth, void *stream) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (npix < 0 || (npix > 0 && (!d_rrs || !d_depth || !d_depth_sigma)) || !r_sigma ||
      n_samples < 1 || n_samples > 4096 || npix > 0xffffffffLL)
    return fail(PHOTIC_ERR_INVALID, "bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = cfg->n_bands;
  const int64_t ns = (int64_t)kDsMaxIntervals * n_samples;
  // scratch: max bits, sample pixels, sample spectra, sample depths, table
  const size_t off_pix = 256, off_rrs = off_pix + ((ns * 4 + 255) / 256) * 256;
  const size_t off_dep = off_rrs + ((ns * nb * 4 + 255) / 256) * 256;
  const size_t off_tab = off_dep + ((ns * 8 + 255) / 256) * 256;
  const size_t bytes = off_tab + kDsMaxIntervals * 8;
  unsigned char *ws = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&ws, bytes, s);
  if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "depth-sigma workspace");
  cudaMemsetAsync(ws, 0, 256, s);
  DepthSigmaArgs a;
  memset(&a, 0, sizeof a);
  a.rrs = d_rrs;
  a.depth = d_depth;
  a.npix = npix;
  a.n_bands = nb;
  a.n_samples = n_samples;
  a.n_trials = (int)sqrt((double)npix);  // (int) sqrt(nrows * ncols)
  a.interval = 0.25;
  for (int b = 0; b < nb; b++) a.r_sigma[b] = r_sigma[b];
  a.nodata = cfg->nodata_value;
  a.seed = seed;
  a.max_bits = (unsigned int *)ws;
  a.sample_pixel = d_sample_pixel ? d_sample_pixel : (int32_t *)(ws + off_pix);
  a.sample_rrs = (float *)(ws + off_rrs);
  double *sdep = d_sample_depth ? d_sample_depth : (double *)(ws + off_dep);
  a.sample_depth = sdep;
  a.table = d_table ? d_table : (double *)(ws + off_tab);
  a.depth_sigma = d_depth_sigma;
  e = launch_depth_sigma_select(a, s);
  if (e == cudaSuccess) {
    photic_outputs o;
    memset(&o, 0, sizeof o);
    o.depth_f64 = sdep;
    rc = photic_invert_batch(cfg, a.sample_rrs, ns, nb, 1, nullptr, &o, stream);
    if (rc == PHOTIC_OK) e = launch_depth_sigma_finish(a, s);
  }
  cudaFreeAsync(ws, s);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "depth-sigma kernels");
  return PHOTIC_OK;
}

// ---------------------------------------------------------------------------
// Spatial-region fit (model/samodel.c:2957-3027 with n_spatial = 2).
// ---------------------------------------------------------------------------

namespace {

// Checks shared by the general fit and its lookup-table loop; *nmax
// receives the largest parameter count.
int region_config_check(const photic_config *cfg, int32_t n_scenes, int32_t n_spatial,
                        int32_t n_bottoms, int *nmax) {
  int rc = photic_config_check(cfg);
  if (rc) return rc;
  if (n_spatial < 1 || n_spatial > 2)
    return fail(PHOTIC_ERR_UNSUPPORTED, "n_spatial must be 1 (pixels alone) or 2 (3 x 3 regions)");
  if (n_bottoms < 1 || n_bottoms > 3)
    return fail(PHOTIC_ERR_UNSUPPORTED, "n_bottoms must be 1..3 (sand, seagrass, coral)");
  if (n_scenes < 1 || n_scenes > PHOTIC_MAX_SCENES)
    return fail(PHOTIC_ERR_UNSUPPORTED, "n_scenes must be 1..%d", PHOTIC_MAX_SCENES);
  const int Rmax = n_spatial == 2 ? kRegionMaxR : 1;
  if (Rmax * n_scenes * cfg->n_bands > 128 || Rmax * n_scenes > 64)
    return fail(PHOTIC_ERR_UNSUPPORTED, "regions x scenes x bands beyond 128");
  *nmax = region_max_params(Rmax, n_bottoms, n_scenes);
  if (*nmax > 96) return fail(PHOTIC_ERR_UNSUPPORTED, "%d unknowns beyond 96", *nmax);
  return PHOTIC_OK;
}

void region_args(const photic_config *cfg, const float *d_grid, int32_t n_scenes,
                 const double *theta_sun_deg, int32_t nrows, int32_t ncols, int32_t n_spatial,
                 int32_t n_bottoms, const photic_outputs *out, RegionArgs &a) {
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  make_scene(*cfg, cfg->theta_sun_deg, a.sc);
  for (int s = 0; s < n_scenes; s++) {
    SceneConsts ss;
    make_scene(*cfg, theta_sun_deg ? theta_sun_deg[s] : cfg->theta_sun_deg, ss);
    a.sec_sun[s] = ss.sec_sun;
  }
  a.grid = d_grid;
  a.nrows = nrows;
  a.ncols = ncols;
  a.npix = (int64_t)nrows * ncols;
  a.n_scenes = n_scenes;
  a.n_spatial = n_spatial;
  a.n_bottoms = n_bottoms;
  a.out = *out;
}

// Default chains of the general loop per resident warp (one chain runs on
// a warp): as for the single-scene loop's lanes.
constexpr int64_t kRegionChainsPerWarp = 8;

}  // namespace

extern "C" int photic_region_fit_batch(const photic_config *cfg, const float *d_grid,
                                       int32_t n_scenes, const double *theta_sun_deg,
                                       int32_t nrows, int32_t ncols, int32_t n_spatial,
                                       int32_t n_bottoms, const double *d_h_empirical,
                                       const photic_outputs *out, void *stream) {
  int nmax = 0;
  int rc = region_config_check(cfg, n_scenes, n_spatial, n_bottoms, &nmax);
  if (rc) return rc;
  if (nrows < 0 || ncols < 0 || !out || ((int64_t)nrows * ncols > 0 && !d_grid))
    return fail(PHOTIC_ERR_INVALID, "bad arguments");
  if ((int64_t)nrows * ncols == 0) return PHOTIC_OK;
  RegionArgs a;
  region_args(cfg, d_grid, n_scenes, theta_sun_deg, nrows, ncols, n_spatial, n_bottoms, out, a);
  a.h_emp = d_h_empirical;
  return run_region(a, nmax, cfg->blocks_per_sm, (cudaStream_t)stream);
}


extern "C" int64_t photic_region_lut_default_chains(const photic_config *cfg, int32_t n_scenes,
                                                    int32_t n_spatial, int32_t n_bottoms) {
  int nmax = 0;
  if (region_config_check(cfg, n_scenes, n_spatial, n_bottoms, &nmax)) return 0;
  unsigned int *err = nullptr;
  int sms = 0;
  if (device_state(&err, &sms)) return 0;
  RegionArgs a;
  memset(&a, 0, sizeof a);
  make_fit(*cfg, a.fp);
  int64_t warps = 0;
  if (launch_region(a, nmax, sms, cfg->blocks_per_sm, 0, &warps) != cudaSuccess) return 0;
  return kRegionChainsPerWarp * warps;
}

extern "C" int photic_region_lut_invert_batch(
    const photic_config *cfg, const photic_lut_config *lut, const float *d_grid, int32_t n_scenes,
    const double *theta_sun_deg, int32_t nrows, int32_t ncols, int32_t n_spatial,
    int32_t n_bottoms, const double *rrs_noise, const float *d_empirical, float empirical_nodata,
    const photic_outputs *out, int64_t *d_source, int64_t *d_order, double *d_chain_stats,
    int64_t *n_shallow, int64_t *n_chains_used, void *stream) {
  int nmax = 0;
  int rc = region_config_check(cfg, n_scenes, n_spatial, n_bottoms, &nmax);
  if (rc) return rc;
  if (n_shallow) *n_shallow = 0;
  if (n_chains_used) *n_chains_used = 0;
  if (!lut) return fail(PHOTIC_ERR_INVALID, "NULL lookup-table configuration");
  if (lut->n_lut < 1 || lut->n_chains < 0)
    return fail(PHOTIC_ERR_INVALID, "n_lut must be >= 1 and n_chains >= 0");
  if (cfg->precision != PHOTIC_PREC_FP64)
    return fail(PHOTIC_ERR_UNSUPPORTED, "the lookup-table loop runs in FP64 only");
  if (nrows < 0 || ncols < 0) return fail(PHOTIC_ERR_INVALID, "nrows / ncols < 0");
  const int64_t npix = (int64_t)nrows * ncols;
  if (npix == 0) return PHOTIC_OK;
  if (!d_grid || !out) return fail(PHOTIC_ERR_INVALID, "NULL input or output");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int *err = nullptr;
  int sms = 0;
  rc = device_state(&err, &sms);
  if (rc) return rc;
  const int nb = cfg->n_bands;
  RegionArgs a;
  region_args(cfg, d_grid, n_scenes, theta_sun_deg, nrows, ncols, n_spatial, n_bottoms, out, a);
  a.error = err;
  a.source = d_source;
  a.chain_stats = d_chain_stats;
  a.emp = d_empirical;
  a.emp_nodata = empirical_nodata;

  // the order (model/samodel.c:701-819): keys summed over the scenes
  LutKeyArgs ka;
  memset(&ka, 0, sizeof ka);
  ka.rrs = d_grid;
  ka.npix = npix;
  ka.n_bands = nb;
  ka.n_scenes = n_scenes;
  ka.general = 1;
  ka.nodata = cfg->nodata_value;
  bool noise = rrs_noise != nullptr && nb >= 4;
  for (int k = 0; k < n_scenes * nb && noise; k++)
    if (rrs_noise[k] < 1.0e-6) noise = false;  // :590-600
  ka.use_noise = noise ? 1 : 0;
  for (int c = 0; c < 3 && noise; c++) {
    double t = 0.0;
    for (int k = 0; k < n_scenes; k++) t += rrs_noise[k * nb + c + 1];  // :752-756
    ka.noise[c] = t;
  }
  ka.out = *out;
  ka.source = d_source;
  ka.emp = d_empirical;
  int64_t *order = d_order;
  cudaError_t e = cudaSuccess;
  if (!order) {
    e = cudaMallocAsync((void **)&order, npix * sizeof(int64_t), s);
    if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "order: %s", cudaGetErrorString(e));
  }
  int64_t S = 0;
  e = lut_order(ka, order, &S, s);
  if (e != cudaSuccess) {
    if (!d_order) cudaFreeAsync(order, s);
    return cuda_fail(e, "lookup-table order");
  }
  if (S > 0) {
    int64_t warps = 0;
    e = launch_region(a, nmax, sms, cfg->blocks_per_sm, s, &warps);
    if (e != cudaSuccess || warps < 1) {
      if (!d_order) cudaFreeAsync(order, s);
      return fail(PHOTIC_ERR_CUDA, "region kernel does not fit on the device");
    }
    int64_t C = lut->n_chains ? lut->n_chains : kRegionChainsPerWarp * warps;
    if (C > S) C = S;
    const int64_t per_chain = (S + C - 1) / C;
    const int64_t cap = per_chain < lut->n_lut ? per_chain : (int64_t)lut->n_lut;
    a.order = order;
    a.n_shallow = S;
    a.n_chains = C;
    a.cap = cap;
    a.entry_stride = region_entry_stride(n_scenes);
    unsigned long long *queue = nullptr;
    e = cudaMallocAsync((void **)&a.ring, (size_t)C * cap * a.entry_stride * sizeof(double), s);
    if (e == cudaSuccess)
      e = cudaMallocAsync((void **)&a.ring_src, (size_t)C * cap * sizeof(int64_t), s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&queue, sizeof *queue, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, sizeof *queue, s);
    if (e == cudaSuccess && d_chain_stats)
      e = cudaMemsetAsync(d_chain_stats, 0, (size_t)C * 4 * sizeof(double), s);
    if (e == cudaSuccess) {
      a.queue = queue;
      e = launch_region(a, nmax, sms, cfg->blocks_per_sm, s);
    }
    cudaFreeAsync(a.ring, s);
    cudaFreeAsync(a.ring_src, s);
    cudaFreeAsync(queue, s);
    if (e != cudaSuccess) {
      if (!d_order) cudaFreeAsync(order, s);
      return cuda_fail(e, "lookup-table region kernel");
    }
    if (n_chains_used) *n_chains_used = C;
  }
  if (!d_order) cudaFreeAsync(order, s);
  if (n_shallow) *n_shallow = S;
  return PHOTIC_OK;
}

extern "C" int photic_region_depth_sigma(const photic_config *cfg, const float *d_grid,
                                         int32_t n_scenes, const double *theta_sun_deg,
                                         int32_t nrows, int32_t ncols, int32_t n_spatial,
                                         int32_t n_bottoms, const float *d_depth,
                                         const double *r_sigma, int32_t n_samples, uint64_t seed,
                                         float *d_depth_sigma, double *d_table,
                                         int32_t *d_sample_pixel, double *d_sample_depth,
                                         void *stream) {
  int nmax = 0;
  int rc = region_config_check(cfg, n_scenes, n_spatial, n_bottoms, &nmax);
  if (rc) return rc;
  const int64_t npix = (int64_t)nrows * ncols;
  if (nrows < 0 || ncols < 0 || (npix > 0 && (!d_grid || !d_depth || !d_depth_sigma)) ||
      !r_sigma || n_samples < 1 || n_samples > 4096 || npix > 0xffffffffLL)
    return fail(PHOTIC_ERR_INVALID, "bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = cfg->n_bands;
  const int64_t ns = (int64_t)kDsMaxIntervals * n_samples;
  // scratch: max bits, sample pixels, draws, sample depths, table, region lists
  const size_t off_pix = 256, off_n = off_pix + ((ns * 4 + 255) / 256) * 256;
  const size_t off_dep = off_n + ((ns * 4 + 255) / 256) * 256;
  const size_t off_tab = off_dep + ((ns * 8 + 255) / 256) * 256;
  const size_t off_R = off_tab + ((kDsMaxIntervals * 8 + 255) / 256) * 256;
  const size_t off_o = off_R + ((ns * 4 + 255) / 256) * 256;
  const size_t off_rrs = off_o + ((ns * 4 + 255) / 256) * 256;
  const size_t bytes = off_rrs + (size_t)ns * kRegionMaxR * n_scenes * nb * 4;
  unsigned char *ws = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&ws, bytes, s);
  if (e != cudaSuccess) return fail(PHOTIC_ERR_NOMEM, "depth-sigma workspace");
  cudaMemsetAsync(ws, 0, 256, s);
  DepthSigmaArgs a;
  memset(&a, 0, sizeof a);
  a.rrs = d_grid;
  a.depth = d_depth;
  a.npix = npix;
  a.n_bands = nb;
  a.n_samples = n_samples;
  a.n_trials = (int)sqrt((double)npix);  // (int) sqrt(nrows * ncols)
  a.interval = 0.25;
  a.nodata = cfg->nodata_value;
  a.seed = seed;
  a.max_bits = (unsigned int *)ws;
  a.sample_pixel = d_sample_pixel ? d_sample_pixel : (int32_t *)(ws + off_pix);
  a.sample_n = (float *)(ws + off_n);
  double *sdep = d_sample_depth ? d_sample_depth : (double *)(ws + off_dep);
  a.sample_depth = sdep;
  a.table = d_table ? d_table : (double *)(ws + off_tab);
  a.depth_sigma = d_depth_sigma;
  e = launch_depth_sigma_select(a, s);
  RegionSampleArgs ra;
  memset(&ra, 0, sizeof ra);
  ra.grid = d_grid;
  ra.nrows = nrows;
  ra.ncols = ncols;
  ra.n_scenes = n_scenes;
  ra.n_bands = nb;
  ra.n_spatial = n_spatial;
  ra.nodata = cfg->nodata_value;
  for (int k = 0; k < n_scenes; k++)
    for (int b = 0; b < nb; b++) ra.r_sigma[k * 8 + b] = r_sigma[k * nb + b];
  ra.sample_pixel = a.sample_pixel;
  ra.sample_n = a.sample_n;
  ra.ns = ns;
  ra.list_rrs = (float *)(ws + off_rrs);
  ra.list_R = (int32_t *)(ws + off_R);
  ra.list_origin = (int32_t *)(ws + off_o);
  if (e == cudaSuccess) e = launch_region_samples(ra, s);
  if (e == cudaSuccess) {
    // the refits: the general fit of every sample's regions, cold, with
    // the reference's h_empirical of 5 m (every bottom type; :1448)
    photic_outputs o;
    memset(&o, 0, sizeof o);
    o.depth_f64 = sdep;
    RegionArgs r;
    region_args(cfg, nullptr, n_scenes, theta_sun_deg, 0, 0, n_spatial, n_bottoms, &o, r);
    r.npix = ns;
    r.no_mask = 1;
    r.list_rrs = ra.list_rrs;
    r.list_R = ra.list_R;
    r.list_origin = ra.list_origin;
    rc = run_region(r, nmax, cfg->blocks_per_sm, s);
    if (rc == PHOTIC_OK) e = launch_depth_sigma_finish(a, s);
  }
  cudaFreeAsync(ws, s);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "depth-sigma kernels");
  return PHOTIC_OK;
}

extern "C" int photic_region_invert_batch(const photic_config *cfg, const float *d_grid,
                                          int32_t nrows, int32_t ncols, int32_t n_spatial,
                                          const photic_outputs *out, void *stream) {
  if (n_spatial != 2) return fail(PHOTIC_ERR_UNSUPPORTED, "n_spatial must be 2 (3 x 3 regions)");
  return photic_region_fit_batch(cfg, d_grid, 1, nullptr, nrows, ncols, n_spatial, 1, nullptr, out,
                                 stream);
}

