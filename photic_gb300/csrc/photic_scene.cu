// photic_scene.cu -- the reference's SCENE command (model/bam.c:1300-1543):
// the text that names a scene's band grids and gives its metadata, parsed
// into the reference's scene record, and that record mapped onto a
// photic_config.  Host code only.
//
// The grammar, the tokenizer and the defaults are the reference's:
//   SCENE NAME <name> BANDS <grid> <grid> ... WAVELENGTHS <nm> ... THETAVIEW|THETAV <deg>
//     THETASUN|THETAW <deg> [RINF <r> ...] [HTIDE <m>] [K <k> ...] [RSIGMA <s> ...]
//     [KSIGMA <s> ...] [P <grid>] [G <grid>] [X <grid>]
// tokens are split at every space or newline (two spaces make an empty
// token, model/bam.c:6610-6624), band names run up to WAVELENGTHS, values
// are read with atof and wavelengths stored as int as the record holds them
// (model/common.h:200), and an absent KSIGMA is a tenth of K (:1501-1505).
// Where the reference fills an absent RINF, K or RSIGMA from its deep-water
// estimates of earlier commands, the record keeps zeros and the `given`
// mask says so.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/photic_samodel.h"
#include "photic_kernels.h"

namespace photic {
int report_error(int code, const char *message);
}

namespace {

int scene_fail(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return photic::report_error(PHOTIC_ERR_INVALID, buf);
}

std::vector<std::string> tokenize(const char *line) {
  std::vector<std::string> t(1);
  for (const char *c = line; *c; c++) {
    if (*c == ' ' || *c == '\n') t.emplace_back();
    else t.back().push_back(*c);
  }
  return t;
}

}  // namespace

extern "C" int photic_parse_scene(const char *line, photic_scene_spec *out) {
  if (!line || !out) return scene_fail("NULL argument");
  memset(out, 0, sizeof *out);
  const std::vector<std::string> p = tokenize(line);
  auto at = [&](size_t k) -> const std::string & {
    static const std::string empty;
    return k < p.size() ? p[k] : empty;
  };
  const char *usage =
      "SCENE NAME /scene name/ BANDS /band 1/ ... WAVELENGTHS /lambda_1/ ... THETAVIEW /deg/ "
      "THETASUN /deg/ [RINF ...] [HTIDE /m/] [K ...] [RSIGMA ...] [KSIGMA ...] [P /grid/] "
      "[G /grid/] [X /grid/]";
  if (at(0) != "SCENE" || at(1) != "NAME" || at(2).empty())
    return scene_fail("expected %s", usage);
  photic_scene &s = out->scene;
  snprintf(s.scene_name, sizeof s.scene_name, "%s", at(2).c_str());
  if (at(3) != "BANDS") return scene_fail("BANDS expected: %s", usage);
  size_t k = 4;
  int nb = 0;
  while (k < p.size() && at(k) != "WAVELENGTHS") {
    if (nb >= PHOTIC_SCENE_MAX_BANDS) return scene_fail("more than %d bands", PHOTIC_SCENE_MAX_BANDS);
    snprintf(out->band_names[nb], PHOTIC_SCENE_NAME_LEN, "%s", at(k).c_str());
    s.band_indexes[nb] = nb;
    nb++;
    k++;
  }
  if (nb < 1 || at(k) != "WAVELENGTHS") return scene_fail("WAVELENGTHS expected: %s", usage);
  s.n_bands = nb;
  for (int n = 0; n < nb; n++) s.wavelengths[n] = (int)atof(at(++k).c_str());
  k++;
  if (!(at(k) == "THETAV" || at(k) == "THETAVIEW"))
    return scene_fail("THETAVIEW expected: %s", usage);
  s.theta_v = atof(at(++k).c_str());
  k++;
  if (!(at(k) == "THETAW" || at(k) == "THETASUN")) return scene_fail("THETASUN expected: %s", usage);
  s.theta_w = atof(at(++k).c_str());
  k++;
  auto per_band = [&](const char *key, double *dst, int bit) {
    if (at(k) != key) return;
    for (int n = 0; n < nb; n++) dst[n] = atof(at(++k).c_str());
    k++;
    out->given |= bit;
  };
  per_band("RINF", s.R_inf, PHOTIC_SCENE_RINF);
  if (at(k) == "HTIDE") {
    s.H_tide = atof(at(++k).c_str());
    k++;
    out->given |= PHOTIC_SCENE_HTIDE;
  }
  per_band("K", s.K, PHOTIC_SCENE_K);
  per_band("RSIGMA", s.R_sigma, PHOTIC_SCENE_RSIGMA);
  per_band("KSIGMA", s.K_sigma, PHOTIC_SCENE_KSIGMA);
  if (!(out->given & PHOTIC_SCENE_KSIGMA))
    for (int n = 0; n < PHOTIC_REF_MAX_GRIDS; n++) s.K_sigma[n] = s.K[n] / 10.0;
  const char *pgx[3] = {"P", "G", "X"};
  int present = 0;
  for (int c = 0; c < 3; c++)
    if (at(k) == pgx[c]) {
      snprintf(out->pgx_names[c], PHOTIC_SCENE_NAME_LEN, "%s", at(++k).c_str());
      k++;
      present++;
    }
  s.pgx_present = present == 3;
  return PHOTIC_OK;
}

extern "C" int photic_config_from_scene(const photic_scene *scene, photic_config *cfg) {
  if (!scene || !cfg) return scene_fail("NULL argument");
  if (scene->n_bands < 2 || scene->n_bands > PHOTIC_MAX_BANDS)
    return scene_fail("%d bands: the inversion takes 2..%d", scene->n_bands, PHOTIC_MAX_BANDS);
  photic_config_default(cfg);
  cfg->n_bands = scene->n_bands;
  for (int b = 0; b < scene->n_bands; b++) cfg->wavelengths[b] = scene->wavelengths[b];
  cfg->theta_sun_deg = scene->theta_w;   // subsurface, degrees (model/samodel.c:534-548)
  cfg->theta_view_deg = scene->theta_v;
  cfg->h_tide = scene->H_tide;
  return photic_config_check(cfg);
}
