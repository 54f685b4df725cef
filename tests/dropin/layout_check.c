/* Compile-time check that the model_data, geogrid and scene layouts of
 * include/photic_samodel.h match the reference's model/common.h field for
 * field.  Built by tests/test_dropin_layout.py with the reference headers on
 * the include path; it has no run-time part. */
#include <stddef.h>

#include "common.h"
#include "photic_samodel.h"

#define SAME(T, U, f) _Static_assert(offsetof(T, f) == offsetof(U, f), #T "." #f)

SAME(geogrid, photic_geogrid, nrows);
SAME(geogrid, photic_geogrid, cellsize);
SAME(geogrid, photic_geogrid, nodata_value);
SAME(geogrid, photic_geogrid, theta_w);
SAME(geogrid, photic_geogrid, array);
_Static_assert(sizeof(geogrid) == sizeof(photic_geogrid), "sizeof geogrid");

SAME(model_data, photic_model_data, n_bottoms);
SAME(model_data, photic_model_data, n_bands);
SAME(model_data, photic_model_data, origin);
SAME(model_data, photic_model_data, n_params);
SAME(model_data, photic_model_data, Rrs_measured);
SAME(model_data, photic_model_data, wavelengths);
SAME(model_data, photic_model_data, bottom_reflectance);
SAME(model_data, photic_model_data, a_0);
SAME(model_data, photic_model_data, b_bw);
SAME(model_data, photic_model_data, a_w640);
SAME(model_data, photic_model_data, H_tide);
SAME(model_data, photic_model_data, theta_sun);
SAME(model_data, photic_model_data, sec_theta_view);
SAME(model_data, photic_model_data, Rrs440);
SAME(model_data, photic_model_data, Rrs750);
SAME(model_data, photic_model_data, rrs_noise);
SAME(model_data, photic_model_data, h_empirical);
SAME(model_data, photic_model_data, bottom_type_indexes);
SAME(model_data, photic_model_data, B_type_name);
SAME(model_data, photic_model_data, empirical_depth_present);
SAME(model_data, photic_model_data, start_at_previous);
SAME(model_data, photic_model_data, P);
SAME(model_data, photic_model_data, prev);
SAME(model_data, photic_model_data, Rrs_modelled);
SAME(model_data, photic_model_data, rho);
SAME(model_data, photic_model_data, depth);
SAME(model_data, photic_model_data, depth_prev);
SAME(model_data, photic_model_data, Rrs_error);
SAME(model_data, photic_model_data, model_error);
SAME(model_data, photic_model_data, K_min);
SAME(model_data, photic_model_data, bottom_albedo);
SAME(model_data, photic_model_data, B_type_percent);
SAME(model_data, photic_model_data, index_optical_depth);
SAME(model_data, photic_model_data, bottom_type);
SAME(model_data, photic_model_data, converged);
SAME(model_data, photic_model_data, n_iterations);
_Static_assert(sizeof(model_data) == sizeof(photic_model_data), "sizeof model_data");

SAME(scene, photic_scene, n_bands);
SAME(scene, photic_scene, band_indexes);
SAME(scene, photic_scene, wavelengths);
SAME(scene, photic_scene, theta_w);
SAME(scene, photic_scene, H_tide);
SAME(scene, photic_scene, R_inf);
SAME(scene, photic_scene, K_sigma);
SAME(scene, photic_scene, ratio_min);
SAME(scene, photic_scene, slope_max);
SAME(scene, photic_scene, pgx_present);
SAME(scene, photic_scene, ps_x);
_Static_assert(sizeof(scene) == sizeof(photic_scene), "sizeof scene");

int photic_layout_check_unit;
