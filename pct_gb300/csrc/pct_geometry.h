/*
 * Configuration defaults, derived geometry and the numeric constants of the
 * reference formulas.  Plain C, usable from host C/C++ and CUDA device code.
 *
 * Derived sizes follow the macro arithmetic of include/pCT_data.h:215-300
 * literally (same operand order, same int truncations) so that a run-time
 * geometry reproduces the values the reference bakes in at compile time:
 *   T_BINS         int( SSD_T_SIZE / T_BIN_SIZE + 0.5 )            (:238)
 *   V_BINS         int( SSD_V_SIZE / V_BIN_SIZE + 0.5 )            (:240)
 *   ANGULAR_BINS   int( 360 / ANGULAR_BIN_SIZE + 0.5 )             (:242)
 *   GANTRY_ANGLES  int( 360 / GANTRY_ANGLE_INTERVAL )              (:224)
 *   RECON_CYL_HEIGHT (SSD_V_SIZE - 1.0)                            (:257)
 *   SLICES         int( RECON_CYL_HEIGHT / SLICE_THICKNESS )       (:266)
 *   VOXEL_WIDTH    ( (2 * RECON_CYL_RADIUS) / COLUMNS )            (:268)
 *   VOXEL_THICKNESS ( (SLICES * SLICE_THICKNESS) / SLICES )        (:270)
 *   X/Y/Z_ZERO     -R, +R, RECON_CYL_HEIGHT/2                      (:272-274)
 *   MLP_U_STEP     ( VOXEL_WIDTH / 2 )                             (:300)
 */
#ifndef PCT_GEOMETRY_H
#define PCT_GEOMETRY_H

#include "pct.h"
#include "pct_math.h"

#if defined(__CUDACC__)
#define PCT_GFN __host__ __device__ static inline
#else
#define PCT_GFN static inline
#endif

/* Angle constants as the reference spells them (pCT_data.h:441-450) with
 * atan(1.0) = pi/4 correctly rounded; products are rounded like the macros. */
#define PCT_PI_OVER_4 0.7853981633974483
#define PCT_PI_OVER_2 (2 * PCT_PI_OVER_4)
#define PCT_THREE_PI_OVER_4 (3 * PCT_PI_OVER_4)
#define PCT_FIVE_PI_OVER_4 (5 * PCT_PI_OVER_4)
#define PCT_SEVEN_PI_OVER_4 (7 * PCT_PI_OVER_4)
#define PCT_TWO_PI (8 * PCT_PI_OVER_4)
#define PCT_ANGLE_TO_RADIANS (PCT_PI / 180.0)
#define PCT_RADIANS_TO_ANGLE (180.0 / PCT_PI)
#define PCT_MM_TO_CM 0.1
#define PCT_RSP_AIR 0.00113
#define PCT_E_0 13.6
#define PCT_X_0 36.08
#define PCT_MAX_INTERSECTIONS 512

/* Scattering-power polynomial A_0..A_5 (pCT_data.h:306-311) is written as
 * "mantissa * pow((float)10, (float)-k)"; pow of two floats is the float
 * overload, so the power is the binary32 nearest 10^-k.  Inside the MLP
 * formulas the macros expand textually: "u * A_5_OVER_168" becomes
 * ((u * 2.687) * p) / 168, and a leading "A_0_OVER_3" becomes (7.457 * p) / 3.
 * The kernels spell each expansion out with these pieces. */
#define PCT_A0_M 7.457
#define PCT_A1_M 4.548
#define PCT_A2_M (-5.777)
#define PCT_A3_M 1.301
#define PCT_A4_M (-9.228)
#define PCT_A5_M 2.687
#define PCT_A0_P ((double)1e-6f)
#define PCT_A1_P ((double)1e-7f)
#define PCT_A2_P ((double)1e-8f)
#define PCT_A3_P ((double)1e-8f)
#define PCT_A4_P ((double)1e-10f)
#define PCT_A5_P ((double)1e-11f)

PCT_GFN void pct_config_fill_defaults(pct_config* c) {
    c->source_radius = 260.7;
    c->gantry_angle_interval = 4.0;
    c->ssd_t_size = 35.0;
    c->ssd_v_size = 9.0;
    c->t_bin_size = 0.1;
    c->v_bin_size = 0.25;
    c->angular_bin_size = 4.0;
    c->sigmas_to_keep = 3;
    c->sample_std_dev = 1;
    c->recon_cyl_radius = 10.0;
    c->columns = 200;
    c->rows = 200;
    c->slice_thickness = 0.25;
    c->sc_on = 0;
    c->msc_on = 1;
    c->sm_on = 0;
    c->avg_filter_hull = 1;
    c->mlp_hull = PCT_MSC_HULL;
    c->msc_diff_thresh = 50;
    c->sc_threshold = 0.0;
    c->msc_threshold = 0.0;
    c->sm_lower_threshold = 6.0;
    c->sm_scale_threshold = 1.0;
    c->hull_filter_threshold = 0.1;
    c->hull_filter_radius = 1;
    c->fbp_on = 1;
    c->fbp_filter = PCT_SHEPP_LOGAN;
    c->fbp_threshold = 0.6;
    c->x_k0 = PCT_HYBRID;
    c->iterations = 12;
    c->block_size = 3200;
    c->lambda = 0.001f;
    c->residual_tol = 0.0;
    c->chord_bf16 = 0;
    c->mlp_exact = 0;
    c->mlp_face_margin = 2e-5;
    c->drop_form = PCT_DROP_SCATTER;
    c->walk_exact = 0;
    c->voxel_order = PCT_ORDER_AUTO;
    c->drop_variant = PCT_DROP_STANDARD;
    c->eta = 2.5;
    c->psi_sign = 1;
}

/* Returns 0 on success, nonzero when a derived size is out of range. */
PCT_GFN int pct_geometry_derive(const pct_config* c, pct_geometry* g) {
    if (!(c->recon_cyl_radius > 0) || c->columns <= 0 || c->rows <= 0 || !(c->slice_thickness > 0) ||
        !(c->t_bin_size > 0) || !(c->v_bin_size > 0) || !(c->angular_bin_size > 0) ||
        !(c->gantry_angle_interval > 0))
        return 1;
    g->columns = c->columns;
    g->rows = c->rows;
    g->recon_cyl_radius = c->recon_cyl_radius;
    g->recon_cyl_height = c->ssd_v_size - 1.0;
    g->slices = pct_d2i(g->recon_cyl_height / c->slice_thickness);
    if (g->slices <= 0) return 2;
    g->num_voxels = g->columns * g->rows * g->slices;
    g->t_bins = pct_d2i(c->ssd_t_size / c->t_bin_size + 0.5);
    g->v_bins = pct_d2i(c->ssd_v_size / c->v_bin_size + 0.5);
    g->angular_bins = pct_d2i(360 / c->angular_bin_size + 0.5);
    g->gantry_angles = pct_d2i(360 / c->gantry_angle_interval);
    if (g->t_bins <= 0 || g->v_bins <= 0 || g->angular_bins <= 0 || g->gantry_angles <= 0) return 3;
    g->num_bins = g->angular_bins * g->t_bins * g->v_bins;
    g->voxel_width = (2 * c->recon_cyl_radius) / c->columns;
    g->voxel_height = (2 * c->recon_cyl_radius) / c->rows;
    g->voxel_thickness = (g->slices * c->slice_thickness) / g->slices;
    g->x_zero = -c->recon_cyl_radius;
    g->y_zero = c->recon_cyl_radius;
    g->z_zero = g->recon_cyl_height / 2;
    g->mlp_u_step = g->voxel_width / 2;
    return 0;
}

#endif /* PCT_GEOMETRY_H */
