/*
 * CPU oracle for the pCT reconstruction path — TEST INFRASTRUCTURE ONLY.
 * See pct_oracle.h.  Line references are to src/pCT_Reconstruction_Data_Segments.cu
 * of lynch829/pCT unless another file is named.
 *
 * Built with -ffp-contract=off: every expression below is evaluated in the
 * order and precision the reference writes it (binary32 where the reference
 * operands are float, binary64 otherwise).  Where the reference's behaviour
 * is undefined (out-of-range voxel writes, unbounded walks, int conversion of
 * NaN) the oracle skips the access / caps the walk and counts the event; the
 * counts are reported so a test can show they stay at zero on its inputs.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "pct_oracle.h"
#include "pct_math.h"
#include "pct_geometry.h"

int ora_version(void) { return 1; }

/* The configuration defaults of pCT_config.h / pCT_data.h (pct_geometry.h), so
 * that a caller of the oracle needs no other library. */
int ora_config_default(pct_config* cfg) {
    pct_config_fill_defaults(cfg);
    return 0;
}
int ora_geometry(const pct_config* cfg, pct_geometry* g) { return pct_geometry_derive(cfg, g); }

/* ------------------------------------------------------------------------- */
/* shared geometry helpers (.cu:8508-8867)                                    */
/* ------------------------------------------------------------------------- */
#define X_INC 1   /* X_INCREASING_DIRECTION = RIGHT (pCT_data.h:275) */
#define Y_INC (-1) /* DOWN */
#define Z_INC (-1) /* DOWN */

/* calculate_voxel_GPU (.cu:8508): int( abs(pos - zero) / size ) */
static int calculate_voxel(double zero, double pos, double size) { return pct_d2i(fabs(pos - zero) / size); }

/* edge_coordinate_GPU (.cu:8735) */
static double edge_coordinate(double zero, int voxel_entered, double size, int inc, int step) {
    int on_edge = (step == inc) ? voxel_entered : voxel_entered + 1;
    return zero + (inc * on_edge * size);
}
/* distance_remaining_GPU (.cu:8721) */
static double distance_remaining(double zero, double pos, int inc, int step, double size, int voxel) {
    int next_voxel = voxel + inc * step;
    double next_edge = edge_coordinate(zero, next_voxel, size, inc, step);
    return fabs(next_edge - pos);
}
/* corresponding_coordinate_GPU (.cu:8748) */
static double corresponding_coordinate(double m, double x, double x0, double y0) { return m * (x - x0) + y0; }

/* ------------------------------------------------------------------------- */
/* a1-a3                                                                      */
/* ------------------------------------------------------------------------- */
/* calculate_intercepts (.cu:2301-2387).  The reference leaves the outputs
 * unset when the line misses; here they are zero. */
static int calculate_intercepts(const pct_geometry* g, double u, double t, double ut_angle, double* u_int, double* t_int) {
    int cone = ((ut_angle > PCT_PI_OVER_4) && (ut_angle < PCT_THREE_PI_OVER_4)) ||
               ((ut_angle > PCT_FIVE_PI_OVER_4) && (ut_angle < PCT_SEVEN_PI_OVER_4));
    double u_temp;
    *u_int = 0.0;
    *t_int = 0.0;
    if (cone) {
        u_temp = u;
        u = -t;
        t = u_temp;
        ut_angle += PCT_PI_OVER_2;
    }
    double m = pct_tan(ut_angle);
    double b_in = t - m * u;
    double a = 1 + m * m;
    double b = 2 * m * b_in;
    double c = b_in * b_in - g->recon_cyl_radius * g->recon_cyl_radius;
    double disc = b * b - (4 * a * c);
    int intersected = disc > 0;
    if (intersected) {
        double u1 = (sqrt(disc) - b) / (2 * a);
        double u2 = (sqrt(disc) + b) / (2 * a);
        double t1 = m * u1 + b_in;
        double t2 = m * u2 - b_in;
        double d1 = (u1 - u) * (u1 - u) + (t1 - t) * (t1 - t);
        double d2 = (u2 + u) * (u2 + u) + (t2 + t) * (t2 + t);
        *u_int = u1 * (d1 <= d2) - u2 * (d1 > d2);
        *t_int = t1 * (d1 <= d2) - t2 * (d1 > d2);
    }
    if (cone) {
        u_temp = *u_int;
        *u_int = *t_int;
        *t_int = -u_temp;
    }
    return intersected;
}

static int sgn_int(float z) { return (z >= 0) - (z < 0); }

int ora_preprocess(const pct_config* cfg, int64_t n, const float* const in13[13], const float* projection_angle,
                   int32_t* gantry_angle, uint8_t* missed, int32_t* bin_num, uint8_t* bin_valid,
                   float* x_entry, float* y_entry, float* z_entry, float* x_exit, float* y_exit, float* z_exit,
                   float* xy_entry_angle, float* xz_entry_angle, float* xy_exit_angle, float* xz_exit_angle,
                   float* wepl_cm) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return 1;
    const double H = g.recon_cyl_height;
    const int T2 = g.t_bins / 2, V2 = g.v_bins / 2;
    /* cos and sin of every whole gantry angle, correctly rounded, once (the
     * same values for every history at that angle) */
    static double trig_ga[360][2];
    static int trig_ready = 0;
#pragma omp critical(ora_trig_ga)
    if (!trig_ready) {
        for (int a = 0; a < 360; ++a) pct_sincos_cr(a * PCT_ANGLE_TO_RADIANS, &trig_ga[a][1], &trig_ga[a][0]);
        trig_ready = 1;
    }
    /* and of every angle bin (this configuration's bin size) */
    double* trig_bin = (double*)malloc(sizeof(double) * 2 * (size_t)(g.angular_bins > 0 ? g.angular_bins : 1));
    if (!trig_bin) return 2;
    for (int b = 0; b < g.angular_bins; ++b)
        pct_sincos_cr(b * cfg->angular_bin_size * PCT_ANGLE_TO_RADIANS, &trig_bin[2 * b + 1], &trig_bin[2 * b]);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        /* a1: read_data_chunk_v02 unit conversion (.cu:1883-1897) and gantry angle (.cu:1921) */
        float t_in_1 = (float)((double)in13[0][i] * PCT_MM_TO_CM), t_in_2 = (float)((double)in13[1][i] * PCT_MM_TO_CM);
        float t_out_1 = (float)((double)in13[2][i] * PCT_MM_TO_CM), t_out_2 = (float)((double)in13[3][i] * PCT_MM_TO_CM);
        float v_in_1 = (float)((double)in13[4][i] * PCT_MM_TO_CM), v_in_2 = (float)((double)in13[5][i] * PCT_MM_TO_CM);
        float v_out_1 = (float)((double)in13[6][i] * PCT_MM_TO_CM), v_out_2 = (float)((double)in13[7][i] * PCT_MM_TO_CM);
        float u_in_1 = (float)((double)in13[8][i] * PCT_MM_TO_CM), u_in_2 = (float)((double)in13[9][i] * PCT_MM_TO_CM);
        float u_out_1 = (float)((double)in13[10][i] * PCT_MM_TO_CM), u_out_2 = (float)((double)in13[11][i] * PCT_MM_TO_CM);
        float w = (float)((double)in13[12][i] * PCT_MM_TO_CM);
        int ga = ((int)projection_angle[i] + 270) % 360;
        gantry_angle[i] = ga;
        wepl_cm[i] = w;

        /* a2: recon_volume_intersections_GPU (.cu:2195-2299) */
        double rot = ga * PCT_ANGLE_TO_RADIANS;
        double cr, sr; /* binary64 cos and sin, correctly rounded */
        if (ga >= 0 && ga < 360) {
            cr = trig_ga[ga][0];
            sr = trig_ga[ga][1];
        } else {
            pct_sincos_cr(rot, &sr, &cr);
        }
        double ut_entry_angle = pct_atan2f(t_in_2 - t_in_1, u_in_2 - u_in_1);
        double u_entry, t_entry, u_exit, t_exit;
        int entered = calculate_intercepts(&g, u_in_2, t_in_2, ut_entry_angle, &u_entry, &t_entry);
        float xy_in = (float)(ut_entry_angle + rot);
        float xe = (float)((cr * u_entry) - (sr * t_entry));
        float ye = (float)((sr * u_entry) + (cr * t_entry));
        double ut_exit_angle = pct_atan2f(t_out_2 - t_out_1, u_out_2 - u_out_1);
        int exited = calculate_intercepts(&g, u_out_1, t_out_1, ut_exit_angle, &u_exit, &t_exit);
        float xy_out = (float)(ut_exit_angle + rot);
        float xx = (float)((cr * u_exit) - (sr * t_exit));
        float yx = (float)((sr * u_exit) + (cr * t_exit));
        double uv_entry_slope = (double)((v_in_2 - v_in_1) / (u_in_2 - u_in_1));
        double uv_exit_slope = (double)((v_out_2 - v_out_1) / (u_out_2 - u_out_1));
        float xz_in = pct_atan2f(v_in_2 - v_in_1, u_in_2 - u_in_1);
        float xz_out = pct_atan2f(v_out_2 - v_out_1, u_out_2 - u_out_1);
        u_entry = (cr * xe) + (sr * ye);
        u_exit = (cr * xx) + (sr * yx);
        float ze = (float)(v_in_2 + uv_entry_slope * (u_entry - u_in_2));
        float zx = (float)(v_out_1 - uv_exit_slope * (u_out_1 - u_exit));
        if (entered && exited) {
            if ((fabsf(ze) < H * 0.5) && (fabsf(zx) > H * 0.5)) {
                double f = fabs((sgn_int(zx) * H * 0.5 - ze) / (zx - ze));
                xx = (float)(xe + f * (xx - xe));
                yx = (float)(ye + f * (yx - ye));
                zx = (float)(sgn_int(zx) * H * 0.5);
            } else if (fabsf(ze) > H * 0.5) {
                entered = 0;
                exited = 0;
            }
            if ((fabsf(ze) > H * 0.5) && (fabsf(zx) < H * 0.5)) {
                double f = fabs((sgn_int(zx) * H * 0.5 - zx) / (zx - ze));
                xe = (float)(xx + f * (xx - xe));
                ye = (float)(yx + f * (yx - ye));
                ze = (float)(sgn_int(ze) * H * 0.5);
            }
            if ((fabsf(t_out_1 - t_in_2) > 5) || (fabsf(v_out_1 - v_in_2) > 5)) {
                entered = 0;
                exited = 0;
            }
        }
        missed[i] = !entered || !exited;
        x_entry[i] = xe; y_entry[i] = ye; z_entry[i] = ze;
        x_exit[i] = xx; y_exit[i] = yx; z_exit[i] = zx;
        xy_entry_angle[i] = xy_in; xz_entry_angle[i] = xz_in;
        xy_exit_angle[i] = xy_out; xz_exit_angle[i] = xz_out;

        /* a3: binning_GPU bin index (.cu:2529-2550); invalid bins keep 0 (.cu:2395) */
        double x_mid = (xe + xx) / 2;
        double y_mid = (ye + yx) / 2;
        double z_mid = (ze + zx) / 2;
        double path_angle = pct_atan2f(yx - ye, xx - xe);
        if (path_angle < 0) path_angle += 2 * PCT_PI;
        int angle_bin = pct_d2i((path_angle * PCT_RADIANS_TO_ANGLE / cfg->angular_bin_size) + 0.5) % g.angular_bins;
        double s_a, c_a;
        if (angle_bin >= 0 && angle_bin < g.angular_bins) {
            c_a = trig_bin[2 * angle_bin];
            s_a = trig_bin[2 * angle_bin + 1];
        } else {
            pct_sincos_cr(angle_bin * cfg->angular_bin_size * PCT_ANGLE_TO_RADIANS, &s_a, &c_a);
        }
        double t = y_mid * c_a - x_mid * s_a;
        int t_bin = pct_d2i((t / cfg->t_bin_size) + T2);
        double v = z_mid;
        int v_bin = pct_d2i((v / cfg->v_bin_size) + V2);
        int bin = t_bin + angle_bin * g.t_bins + v_bin * g.t_bins * g.angular_bins;
        /* a negative angle bin (NaN path angle) would index outside the bins; treated as invalid */
        if ((t_bin >= 0) && (v_bin >= 0) && (t_bin < g.t_bins) && (v_bin < g.v_bins) && bin >= 0 && bin < g.num_bins) {
            bin_num[i] = bin;
            bin_valid[i] = 1;
        } else {
            bin_num[i] = 0;
            bin_valid[i] = 0;
        }
    }
    free(trig_bin);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* a4-a6: bin statistics, cuts, sinogram                                      */
/* ------------------------------------------------------------------------- */
/* relative angle with the +-2 pi wrap (.cu:2557-2566, 2681-2690, 2847-2856) */
static double rel_angle(float exit_angle, float entry_angle) {
    double r = exit_angle - entry_angle;
    if (r > PCT_PI) r -= 2 * PCT_PI;
    if (r < -PCT_PI) r += 2 * PCT_PI;
    return r;
}

int ora_bin_statistics(const pct_config* cfg, int64_t n, const int32_t* bin_num, const uint8_t* bin_valid,
                       const float* wepl, const float* xy_entry_angle, const float* xz_entry_angle,
                       const float* xy_exit_angle, const float* xz_exit_angle,
                       int32_t* counts, float* mean_wepl, float* mean_ut, float* mean_uv,
                       float* sd_wepl, float* sd_ut, float* sd_uv) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return 1;
    const int nb = g.num_bins;
    memset(counts, 0, sizeof(int32_t) * nb);
    for (int b = 0; b < nb; ++b) mean_wepl[b] = mean_ut[b] = mean_uv[b] = sd_wepl[b] = sd_ut[b] = sd_uv[b] = 0.0f;
    /* binning_GPU sums (.cu:2557-2570): only histories with a valid bin.  Every
     * sum here is binary32, added left to right in history order: the order of
     * the reference's atomicAdd calls in a sequential run of its kernels. */
    for (int64_t i = 0; i < n; ++i) {
        if (!bin_valid[i]) continue;
        int b = bin_num[i];
        float rut = (float)rel_angle(xy_exit_angle[i], xy_entry_angle[i]);
        float ruv = (float)rel_angle(xz_exit_angle[i], xz_entry_angle[i]);
        counts[b] += 1;
        mean_wepl[b] = mean_wepl[b] + wepl[i];
        mean_ut[b] = mean_ut[b] + rut;
        mean_uv[b] = mean_uv[b] + ruv;
    }
    /* calculate_means_GPU (.cu:2618-2627) */
    for (int b = 0; b < nb; ++b) {
        if (counts[b] > 0) {
            mean_wepl[b] /= counts[b];
            mean_ut[b] /= counts[b];
            mean_uv[b] /= counts[b];
        }
    }
    /* sum_squared_deviations_GPU (.cu:2678-2698): every kept history, bin 0 included */
    for (int64_t i = 0; i < n; ++i) {
        int b = bin_num[i];
        double rut = rel_angle(xy_exit_angle[i], xy_entry_angle[i]);
        double ruv = rel_angle(xz_exit_angle[i], xz_entry_angle[i]);
        double dw = wepl[i] - mean_wepl[b];
        double dut = rut - mean_ut[b];
        double duv = ruv - mean_uv[b];
        float qw = (float)(dw * dw), qut = (float)(dut * dut), quv = (float)(duv * duv);
        sd_wepl[b] = sd_wepl[b] + qw;
        sd_ut[b] = sd_ut[b] + qut;
        sd_uv[b] = sd_uv[b] + quv;
    }
    /* calculate_standard_deviations_GPU (.cu:2718-2730) */
    for (int b = 0; b < nb; ++b) {
        if (counts[b] > 1) {
            int div = counts[b] - (cfg->sample_std_dev ? 1 : 0);
            sd_wepl[b] = sqrtf(sd_wepl[b] / div);
            sd_ut[b] = sqrtf(sd_ut[b] / div);
            sd_uv[b] = sqrtf(sd_uv[b] / div);
        }
    }
    return 0;
}

int ora_statistical_cuts(const pct_config* cfg, int64_t n, const int32_t* bin_num, const float* wepl,
                         const float* xy_entry_angle, const float* xz_entry_angle, const float* xy_exit_angle,
                         const float* xz_exit_angle, const float* mean_wepl, const float* mean_ut,
                         const float* mean_uv, const float* sd_wepl, const float* sd_ut, const float* sd_uv,
                         uint8_t* failed, int32_t* counts_post, float* sinogram) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return 1;
    const int nb = g.num_bins;
    const int K = cfg->sigmas_to_keep;
    memset(counts_post, 0, sizeof(int32_t) * nb);
    for (int b = 0; b < nb; ++b) sinogram[b] = 0.0f;
    /* statistical_cuts_GPU (.cu:2844-2868) */
    for (int64_t i = 0; i < n; ++i) {
        int b = bin_num[i];
        double rut = rel_angle(xy_exit_angle[i], xy_entry_angle[i]);
        double ruv = rel_angle(xz_exit_angle[i], xz_entry_angle[i]);
        int passed_ut = fabs(rut - mean_ut[b]) < (K * sd_ut[b]);
        int passed_uv = fabs(ruv - mean_uv[b]) < (K * sd_uv[b]);
        int passed_w = fabsf(mean_wepl[b] - wepl[i]) <= (K * sd_wepl[b]);
        int f = !passed_ut || !passed_uv || !passed_w;
        failed[i] = (uint8_t)f;
        if (!f) {
            counts_post[b] += 1;
            sinogram[b] = sinogram[b] + wepl[i]; /* binary32, history order */
        }
    }
    /* construct_sinogram_GPU (.cu:2912-2917) */
    for (int b = 0; b < nb; ++b)
        if (counts_post[b] > 0) sinogram[b] /= counts_post[b];
    return 0;
}

/* ------------------------------------------------------------------------- */
/* a7: hull walks                                                             */
/* ------------------------------------------------------------------------- */
/* initialize_hull_GPU (.cu:3316-3326) */
void ora_initialize_hull(const pct_config* cfg, int32_t* image) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return;
    for (int s = 0; s < g.slices; ++s)
        for (int r = 0; r < g.rows; ++r)
            for (int c = 0; c < g.columns; ++c) {
                double x = (c - g.columns / 2 + 0.5) * g.voxel_width;
                double y = (g.rows / 2 - r - 0.5) * g.voxel_height;
                image[c + r * g.columns + s * g.columns * g.rows] =
                    (x * x + y * y < g.recon_cyl_radius * g.recon_cyl_radius) ? 1 : 0;
            }
}

typedef struct {
    double x, y, z, x_to_go, y_to_go, z_to_go;
    int vx, vy, vz, voxel;
} walk_state;

/* take_3D_step_GPU (.cu:8800-8866) */
static void take_3d_step(const pct_geometry* g, int xm, int ym, int zm, double dy_dx, double dz_dx, double dz_dy,
                         double dx_dy, double dx_dz, double dy_dz, double xs, double ys, double zs, walk_state* w) {
    double x_ext = fabs(dz_dx) * w->x_to_go;
    double y_ext = fabs(dz_dy) * w->y_to_go;
    if ((w->z_to_go <= x_ext) && (w->z_to_go <= y_ext)) {
        w->vz -= zm;
        w->z = edge_coordinate(g->z_zero, w->vz, g->voxel_thickness, Z_INC, zm);
        w->x = corresponding_coordinate(dx_dz, w->z, zs, xs);
        w->y = corresponding_coordinate(dy_dz, w->z, zs, ys);
        w->x_to_go = distance_remaining(g->x_zero, w->x, X_INC, xm, g->voxel_width, w->vx);
        w->y_to_go = distance_remaining(g->y_zero, w->y, Y_INC, ym, g->voxel_height, w->vy);
        w->z_to_go = g->voxel_thickness;
    } else if (x_ext <= y_ext) {
        w->vx += xm;
        w->x = edge_coordinate(g->x_zero, w->vx, g->voxel_width, X_INC, xm);
        w->y = corresponding_coordinate(dy_dx, w->x, xs, ys);
        w->z = corresponding_coordinate(dz_dx, w->x, xs, zs);
        w->x_to_go = g->voxel_width;
        w->y_to_go = distance_remaining(g->y_zero, w->y, Y_INC, ym, g->voxel_height, w->vy);
        w->z_to_go = distance_remaining(g->z_zero, w->z, Z_INC, zm, g->voxel_thickness, w->vz);
    } else {
        w->vy -= ym;
        w->y = edge_coordinate(g->y_zero, w->vy, g->voxel_height, Y_INC, ym);
        w->x = corresponding_coordinate(dx_dy, w->y, ys, xs);
        w->z = corresponding_coordinate(dz_dy, w->y, ys, zs);
        w->x_to_go = distance_remaining(g->x_zero, w->x, X_INC, xm, g->voxel_width, w->vx);
        w->y_to_go = g->voxel_height;
        w->z_to_go = distance_remaining(g->z_zero, w->z, Z_INC, zm, g->voxel_thickness, w->vz);
    }
    if (w->x_to_go == 0) { w->x_to_go = g->voxel_width; w->vx += xm; }
    if (w->y_to_go == 0) { w->y_to_go = g->voxel_height; w->vy -= ym; }
    if (w->z_to_go == 0) { w->z_to_go = g->voxel_thickness; w->vz -= zm; }
    if (w->vz < 0) w->vz = 0;
    w->voxel = w->vx + w->vy * g->columns + w->vz * g->columns * g->rows;
}

/* take_2D_step_GPU (.cu:8754-8799) */
static void take_2d_step(const pct_geometry* g, int xm, int ym, double dy_dx, double dx_dy, double xs, double ys,
                         walk_state* w) {
    double y_ext = fabs(dx_dy) * w->y_to_go;
    if (w->x_to_go <= y_ext) {
        w->vx += xm;
        w->x = edge_coordinate(g->x_zero, w->vx, g->voxel_width, X_INC, xm);
        w->y = corresponding_coordinate(dy_dx, w->x, xs, ys);
        w->x_to_go = g->voxel_width;
        w->y_to_go = distance_remaining(g->y_zero, w->y, Y_INC, ym, g->voxel_height, w->vy);
    } else {
        w->vy -= ym;
        w->y = edge_coordinate(g->y_zero, w->vy, g->voxel_height, Y_INC, ym);
        w->x = corresponding_coordinate(dx_dy, w->y, ys, xs);
        w->x_to_go = distance_remaining(g->x_zero, w->x, X_INC, xm, g->voxel_width, w->vx);
        w->y_to_go = g->voxel_height;
    }
    if (w->x_to_go == 0) { w->x_to_go = g->voxel_width; w->vx += xm; }
    if (w->y_to_go == 0) { w->y_to_go = g->voxel_height; w->vy -= ym; }
    if (w->vz < 0) w->vz = 0;
    w->voxel = w->vx + w->vy * g->columns + w->vz * g->columns * g->rows;
}

/* SC_GPU / MSC_GPU / SM_GPU (.cu:3338-3444, 3456-3558, 3608-3710) */
int ora_hull_walk(const pct_config* cfg, int kind, int64_t n, const uint8_t* missed, const float* wepl,
                  const float* x_entry, const float* y_entry, const float* z_entry, const float* x_exit,
                  const float* y_exit, const float* z_exit, int32_t* image, int64_t* walk_steps_capped) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return 1;
    const int cap = 4 * (g.columns + g.rows + g.slices) + 16;
    int64_t capped = 0, outside = 0;
    /* Histories walk in parallel; the image updates are integer adds (or stores
     * of 0), so the result does not depend on their order. */
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : capped, outside)
    for (int64_t i = 0; i < n; ++i) {
        int use;
        if (kind == 0) use = !missed[i] && (wepl[i] <= cfg->sc_threshold);
        else if (kind == 1) use = !missed[i] && (wepl[i] <= cfg->msc_threshold);
        else use = !missed[i] && (wepl[i] >= cfg->sm_lower_threshold);
        if (!use) continue;
        const float xe = x_entry[i], ye = y_entry[i], ze = z_entry[i];
        const float xx = x_exit[i], yx = y_exit[i], zx = z_exit[i];
        int xm = (xe <= xx) - (xe >= xx);
        int ym = (ye <= yx) - (ye >= yx);
        int zm = (ze <= zx) - (ze >= zx);
        walk_state w;
        w.x = xe; w.y = ye; w.z = ze;
        w.vx = calculate_voxel(g.x_zero, xe, g.voxel_width);
        w.vy = calculate_voxel(g.y_zero, ye, g.voxel_height);
        w.vz = calculate_voxel(g.z_zero, ze, g.voxel_thickness);
        w.voxel = w.vx + w.vy * g.columns + w.vz * g.columns * g.rows;
        w.x_to_go = distance_remaining(g.x_zero, w.x, X_INC, xm, g.voxel_width, w.vx);
        w.y_to_go = distance_remaining(g.y_zero, w.y, Y_INC, ym, g.voxel_height, w.vy);
        w.z_to_go = distance_remaining(g.z_zero, w.z, Z_INC, zm, g.voxel_thickness, w.vz);
        double dy_dx = (double)((yx - ye) / (xx - xe));
        double dz_dx = (double)((zx - ze) / (xx - xe));
        double dz_dy = (double)((zx - ze) / (yx - ye));
        double dx_dy = (double)((xx - xe) / (yx - ye));
        double dx_dz = (double)((xx - xe) / (zx - ze));
        double dy_dz = (double)((yx - ye) / (zx - ze));
        int vxo = calculate_voxel(g.x_zero, xx, g.voxel_width);
        int vyo = calculate_voxel(g.y_zero, yx, g.voxel_height);
        int vzo = calculate_voxel(g.z_zero, zx, g.voxel_thickness);
        int voxel_out = vxo + vyo * g.columns + vzo * g.columns * g.rows;
        int end = (w.voxel == voxel_out) || (w.vx >= g.columns) || (w.vy >= g.rows) || (w.vz >= g.slices);
        int steps = 0;
        for (;;) {
            if (!end) {
                if (w.voxel >= 0 && w.voxel < g.num_voxels) {
                    if (kind == 0) {
#pragma omp atomic write
                        image[w.voxel] = 0;
                    } else {
#pragma omp atomic update
                        image[w.voxel] += 1;
                    }
                } else {
                    ++outside;
                }
            }
            if (end) break;
            if (++steps > cap) { ++capped; break; }
            if (zm != 0) take_3d_step(&g, xm, ym, zm, dy_dx, dz_dx, dz_dy, dx_dy, dx_dz, dy_dz, xe, ye, ze, &w);
            else take_2d_step(&g, xm, ym, dy_dx, dx_dy, xe, ye, &w);
            end = (w.voxel == voxel_out) || (w.vx >= g.columns) || (w.vy >= g.rows) || (w.vz >= g.slices);
        }
    }
    if (walk_steps_capped) {
        walk_steps_capped[0] = capped;
        walk_steps_capped[1] = outside;
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* a8-a9: edge detection, averaging filter                                    */
/* ------------------------------------------------------------------------- */
static int outside_rim(const pct_geometry* g, int c, int r) {
    float x = (float)((c - g->columns / 2 + 0.5) * g->voxel_width);
    float y = (float)((g->rows / 2 - r - 0.5) * g->voxel_height);
    double lim = g->recon_cyl_radius - fmax(g->voxel_width, g->voxel_height) / 2;
    return (double)x * x + (double)y * y >= lim * lim;
}

/* MSC_edge_detection_GPU (.cu:3569-3596) with two buffers (the reference
 * updates in place while neighbours read; the intended result is this). */
void ora_msc_edge_detection(const pct_config* cfg, const int32_t* counts, int32_t* hull) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return;
    const int C = g.columns, R = g.rows;
    for (int s = 0; s < g.slices; ++s)
        for (int r = 0; r < R; ++r)
            for (int c = 0; c < C; ++c) {
                int v = c + r * C + s * C * R;
                int maxd = 0;
                if (r != 0 && r != R - 1 && c != 0 && c != C - 1)
                    for (int rr = r - 1; rr <= r + 1; ++rr)
                        for (int cc = c - 1; cc <= c + 1; ++cc) {
                            int d = counts[v] - counts[cc + rr * C + s * C * R];
                            if (d > maxd) maxd = d;
                        }
                hull[v] = (maxd > cfg->msc_diff_thresh) ? 0 : 1;
                if (outside_rim(&g, c, r)) hull[v] = 0;
            }
}

/* carve_differences (.cu:3274-3292), SM_edge_detection (.cu:3711-3773),
 * SM_edge_detection_GPU (.cu:3774-3789). */
void ora_sm_edge_detection(const pct_config* cfg, const int32_t* counts, int32_t* hull, int32_t* thresholds) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return;
    const int C = g.columns, R = g.rows;
    int32_t* diff = (int32_t*)calloc((size_t)g.num_voxels, sizeof(int32_t));
    if (!diff) return;
    for (int s = 0; s < g.slices; ++s)
        for (int r = 1; r < R - 1; ++r)
            for (int c = 1; c < C - 1; ++c) {
                int v = c + r * C + s * C * R;
                int maxd = 0;
                for (int rr = r - 1; rr <= r + 1; ++rr)
                    for (int cc = c - 1; cc <= c + 1; ++cc) {
                        int d = counts[v] - counts[cc + rr * C + s * C * R];
                        if (d > maxd) maxd = d;
                    }
                diff[v] = maxd;
            }
    for (int s = 0; s < g.slices; ++s) {
        int maxd = 0;
        thresholds[s] = 0;
        for (int p = 0; p < C * R; ++p) {
            int v = p + s * C * R;
            if (diff[v] > maxd) {
                maxd = diff[v];
                thresholds[s] = counts[v];
            }
        }
    }
    for (int s = 0; s < g.slices; ++s)
        for (int r = 0; r < R; ++r)
            for (int c = 0; c < C; ++c) {
                int v = c + r * C + s * C * R;
                hull[v] = (counts[v] > cfg->sm_scale_threshold * thresholds[s]) ? 1 : 0;
                if (outside_rim(&g, c, r)) hull[v] = 0;
            }
    free(diff);
}

/* averaging_filter_GPU with perform_threshold = true (.cu:4007-4029) */
void ora_averaging_filter_bool(const pct_config* cfg, const uint8_t* in, uint8_t* out, int radius, double threshold) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return;
    const int C = g.columns, R = g.rows;
    for (int s = 0; s < g.slices; ++s)
        for (int r = 0; r < R; ++r)
            for (int c = 0; c < C; ++c) {
                int left = c - radius > 0 ? c - radius : 0;
                int right = c + radius < C - 1 ? c + radius : C - 1;
                int top = r - radius > 0 ? r - radius : 0;
                int bottom = r + radius < R - 1 ? r + radius : R - 1;
                int nv = (right - left + 1) * (bottom - top + 1);
                double sum_threshold = nv * threshold;
                double sum = 0.0;
                for (int cc = left; cc <= right; ++cc)
                    for (int rr = top; rr <= bottom; ++rr) sum += in[cc + rr * C + s * C * R];
                out[c + r * C + s * C * R] = sum > sum_threshold;
            }
}

/* ------------------------------------------------------------------------- */
/* a10-a12: FBP                                                               */
/* ------------------------------------------------------------------------- */
/* filter_GPU (.cu:3036-3069).  FILTER NONE leaves the reference's filter
 * value uninitialised; here it passes the sinogram through (1/T_BIN_SIZE at
 * zero separation). */
void ora_filter(const pct_config* cfg, const float* sinogram, float* filtered) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return;
    const double TB = cfg->t_bin_size, VB = cfg->v_bin_size, SR = cfg->source_radius;
    const double tau = (double)(2 / sqrtf(2.0f)) * TB; /* RAM_LAK_TAU = 2/ROOT_TWO * T_BIN_SIZE (pCT_data.h:247) */
#pragma omp parallel for collapse(2) schedule(static)
    for (int vb = 0; vb < g.v_bins; ++vb)
        for (int ab = 0; ab < g.angular_bins; ++ab) {
            int strip = (vb * g.angular_bins * g.t_bins) + (ab * g.t_bins);
            double v = (vb - g.v_bins / 2) * VB + VB / 2.0;
            for (int tb = 0; tb < g.t_bins; ++tb) {
                float acc = 0.0f;
                for (int tr = 0; tr < g.t_bins; ++tr) {
                    double t = (tr - g.t_bins / 2) * TB + TB / 2.0;
                    int sep = tb - tr;
                    double scale = SR / sqrt(SR * SR + t * t + v * v);
                    double f;
                    if (cfg->fbp_filter == PCT_RAM_LAK) {
                        if (sep == 0) f = 1.0 / (4.0 * (tau * tau));
                        else if (sep % 2 == 0) f = 0;
                        else { double q = tau * PCT_PI * sep; f = -1.0 / (q * q); }
                    } else if (cfg->fbp_filter == PCT_SHEPP_LOGAN) {
                        f = 1 / ((TB * PCT_PI * TB * PCT_PI) * (1.0 - (2 * sep * 2 * sep)));
                    } else {
                        f = sep == 0 ? 1.0 / TB : 0.0;
                    }
                    acc = (float)(acc + TB * sinogram[strip + tr] * f * scale);
                }
                filtered[strip + tb] = acc;
            }
        }
}

/* backprojection_GPU (.cu:3155-3230).  Bins outside the sinogram read as 0
 * (the reference reads out of bounds; unreachable for in-cylinder voxels). */
void ora_backprojection(const pct_config* cfg, const float* sino, float* image) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return;
    const double delta = cfg->gantry_angle_interval * PCT_ANGLE_TO_RADIANS;
    const double SR = cfg->source_radius, R = g.recon_cyl_radius;
    const int ATB = g.angular_bins * g.t_bins;
    /* cos and sin of every projection angle, correctly rounded, once */
    double* trig = (double*)malloc(sizeof(double) * 2 * (size_t)(g.angular_bins > 0 ? g.angular_bins : 1));
    if (!trig) return;
    for (int ab = 0; ab < g.angular_bins; ++ab) pct_sincos_cr(ab * delta, &trig[2 * ab + 1], &trig[2 * ab]);
#define SINO(k) (((k) >= 0 && (k) < g.num_bins) ? sino[(k)] : 0.0f)
#pragma omp parallel for schedule(static)
    for (int voxel = 0; voxel < g.num_voxels; ++voxel) {
        int column = voxel % g.columns, row = (voxel / g.columns) % g.rows, slice = voxel / (g.columns * g.rows);
        double x = -R + (column + 0.5) * g.voxel_width;
        double y = R - (row + 0.5) * g.voxel_height;
        double z = -g.recon_cyl_height / 2.0 + (slice + 0.5) * cfg->slice_thickness;
        if ((x * x + y * y) > (R * R)) {
            image[voxel] = (float)PCT_RSP_AIR;
            continue;
        }
        float acc = 0.0f;
        for (int ab = 0; ab < g.angular_bins; ++ab) {
            const double ca = trig[2 * ab], sa = trig[2 * ab + 1];
            double u = x * ca + y * sa;
            double t = -x * sa + y * ca;
            double v = z;
            double dnt = (t - u * (t / (SR + u))) / cfg->t_bin_size + g.t_bins / 2.0;
            int t_bin = pct_d2i(dnt);
            if (t_bin > dnt) t_bin -= 1;
            double eta = dnt - t_bin;
            double dnv = (v - u * (v / (SR + u))) / cfg->v_bin_size + g.v_bins / 2.0;
            int v_bin = pct_d2i(dnv);
            if (v_bin > dnv) v_bin -= 1;
            double eps = dnv - v_bin;
            double sf = SR / (SR + u);
            double scale = sf * sf;
            int bin = t_bin + ab * g.t_bins + v_bin * ATB;
            if (v_bin == g.v_bins - 1 || (bin < 0))
                acc = (float)(acc + scale * (((1 - eta) * SINO(bin)) + (eta * SINO(bin + 1))));
            else
                acc = (float)(acc + scale * ((1 - eta) * (1 - eps) * SINO(bin) + eta * (1 - eps) * SINO(bin + 1) +
                                             (1 - eta) * eps * SINO(bin + ATB) + eta * eps * SINO(bin + ATB + 1)));
        }
        image[voxel] = (float)(acc * delta);
    }
#undef SINO
    free(trig);
}

/* FBP_image_2_hull_GPU (.cu:3250-3261) */
void ora_fbp_hull(const pct_config* cfg, const float* image, uint8_t* hull) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return;
    const double R = g.recon_cyl_radius;
    for (int voxel = 0; voxel < g.num_voxels; ++voxel) {
        int column = voxel % g.columns, row = (voxel / g.columns) % g.rows;
        double x = -R + (column + 0.5) * g.voxel_width;
        double y = R - (row + 0.5) * g.voxel_height;
        double d2 = x * x + y * y;
        hull[voxel] = (image[voxel] > cfg->fbp_threshold && d2 < R * R) ? 1 : 0;
    }
}

/* ------------------------------------------------------------------------- */
/* a13: MLP endpoints                                                         */
/* ------------------------------------------------------------------------- */
/* find_MLP_endpoints_GPU (.cu:4997-5277), with a step cap. */
static int find_endpoints(const pct_geometry* g, const uint8_t* image, double x_start, double y_start, double z_start,
                          double xy_angle, double xz_angle, double* xo, double* yo, double* zo, int* vxo, int* vyo,
                          int* vzo, int entering, int* capped) {
    const int C = g->columns, R = g->rows, S = g->slices;
    const int cap = 4 * (C + R + S) + 16;
    double x = x_start, y = y_start, z = z_start;
    int hit = 0, end, outside;
    if (!entering) xy_angle += PCT_PI;
    double cxy = pct_cos(xy_angle), sxy = pct_sin(xy_angle), sxz = pct_sin(xz_angle);
    int xm = (cxy >= 0) - (cxy <= 0);
    int ym = (sxy >= 0) - (sxy <= 0);
    int zm = (sxz >= 0) - (sxz <= 0);
    if (xm < 0) zm *= -1;
    int vx = calculate_voxel(g->x_zero, x, g->voxel_width);
    int vy = calculate_voxel(g->y_zero, y, g->voxel_height);
    int vz = calculate_voxel(g->z_zero, z, g->voxel_thickness);
    double x_to_go = distance_remaining(g->x_zero, x, X_INC, xm, g->voxel_width, vx);
    double y_to_go = distance_remaining(g->y_zero, y, Y_INC, ym, g->voxel_height, vy);
    double z_to_go = distance_remaining(g->z_zero, z, Z_INC, zm, g->voxel_thickness, vz);
    int voxel = vx + vy * C + vz * C * R;
    double txy = pct_tan(xy_angle), txz = pct_tan(xz_angle);
    double delta_yx = fabs(txy);
    double delta_zx = fabs(txz);
    double delta_zy = fabs(txz / txy);
    double dy_dx = txy;
    double dz_dx = txz;
    double dz_dy = txz / txy;
    double dx_dy = 1.0 / txy;
    double dx_dz = 1.0 / txz;
    double dy_dz = txy / txz;
    outside = (vx >= C) || (vy >= R) || (vz >= S) || (vx < 0) || (vy < 0) || (vz < 0);
    if (!outside) hit = (image[voxel] == 1);
    end = outside || hit;
    int steps = 0;
    if (zm != 0) {
        while (!end) {
            if (++steps > cap) { ++*capped; break; }
            double x_ext = delta_zx * x_to_go;
            double y_ext = delta_zy * y_to_go;
            if ((z_to_go <= x_ext) && (z_to_go <= y_ext)) {
                vz -= zm;
                z = edge_coordinate(g->z_zero, vz, g->voxel_thickness, Z_INC, zm);
                x = corresponding_coordinate(dx_dz, z, z_start, x_start);
                y = corresponding_coordinate(dy_dz, z, z_start, y_start);
                x_to_go = distance_remaining(g->x_zero, x, X_INC, xm, g->voxel_width, vx);
                y_to_go = distance_remaining(g->y_zero, y, Y_INC, ym, g->voxel_height, vy);
                z_to_go = g->voxel_thickness;
            } else if (x_ext <= y_ext) {
                vx += xm;
                x = edge_coordinate(g->x_zero, vx, g->voxel_width, X_INC, xm);
                y = corresponding_coordinate(dy_dx, x, x_start, y_start);
                z = corresponding_coordinate(dz_dx, x, x_start, z_start);
                x_to_go = g->voxel_width;
                y_to_go = distance_remaining(g->y_zero, y, Y_INC, ym, g->voxel_height, vy);
                z_to_go = distance_remaining(g->z_zero, z, Z_INC, zm, g->voxel_thickness, vz);
            } else {
                vy -= ym;
                y = edge_coordinate(g->y_zero, vy, g->voxel_height, Y_INC, ym);
                x = corresponding_coordinate(dx_dy, y, y_start, x_start);
                z = corresponding_coordinate(dz_dy, y, y_start, z_start);
                x_to_go = distance_remaining(g->x_zero, x, X_INC, xm, g->voxel_width, vx);
                y_to_go = g->voxel_height;
                z_to_go = distance_remaining(g->z_zero, z, Z_INC, zm, g->voxel_thickness, vz);
            }
            if (x_to_go == 0) { x_to_go = g->voxel_width; vx += xm; }
            if (y_to_go == 0) { y_to_go = g->voxel_height; vy -= ym; }
            if (z_to_go == 0) { z_to_go = g->voxel_thickness; vz -= zm; }
            if (vz < 0) vz = 0;
            voxel = vx + vy * C + vz * C * R;
            outside = (vx >= C) || (vy >= R) || (vz >= S) || (vx < 0) || (vy < 0) || (vz < 0);
            if (!outside) hit = (image[voxel] == 1);
            end = outside || hit;
        }
    } else {
        while (!end) {
            if (++steps > cap) { ++*capped; break; }
            double y_ext = y_to_go / delta_yx;
            if (x_to_go <= y_ext) {
                vx += xm;
                x = edge_coordinate(g->x_zero, vx, g->voxel_width, X_INC, xm);
                y = corresponding_coordinate(dy_dx, x, x_start, y_start);
                x_to_go = g->voxel_width;
                y_to_go = distance_remaining(g->y_zero, y, Y_INC, ym, g->voxel_height, vy);
            } else {
                vy -= ym;
                y = edge_coordinate(g->y_zero, vy, g->voxel_height, Z_INC, ym);
                x = corresponding_coordinate(dx_dy, y, y_start, x_start);
                x_to_go = distance_remaining(g->x_zero, x, X_INC, xm, g->voxel_width, vx);
                y_to_go = g->voxel_height;
            }
            if (x_to_go == 0) { x_to_go = g->voxel_width; vx += xm; }
            if (y_to_go == 0) { y_to_go = g->voxel_height; vy -= ym; }
            voxel = vx + vy * C + vz * C * R;
            outside = (vx >= C) || (vy >= R) || (vz >= S) || (vx < 0) || (vy < 0) || (vz < 0);
            if (!outside) hit = (image[voxel] == 1);
            end = outside || hit;
        }
    }
    if (hit) { *xo = x; *yo = y; *zo = z; }
    *vxo = vx; *vyo = vy; *vzo = vz;
    return hit;
}

/* collect_MLP_endpoints_GPU (.cu:5729-5770) */
int ora_endpoints(const pct_config* cfg, int64_t n, const uint8_t* hull, const float* x_entry, const float* y_entry,
                  const float* z_entry, const float* xy_entry_angle, const float* xz_entry_angle,
                  const float* x_exit, const float* y_exit, const float* z_exit, const float* xy_exit_angle,
                  const float* xz_exit_angle, uint8_t* intersected, uint32_t* first_voxel,
                  float* x_in, float* y_in, float* z_in, float* x_out, float* y_out, float* z_out) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return -1;
    int capped = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : capped)
    for (int64_t i = 0; i < n; ++i) {
        double xi = 0, yi = 0, zi = 0, xo = 0, yo = 0, zo = 0;
        int vx = 0, vy = 0, vz = 0, vx2 = 0, vy2 = 0, vz2 = 0;
        int entered = find_endpoints(&g, hull, x_entry[i], y_entry[i], z_entry[i], xy_entry_angle[i], xz_entry_angle[i],
                                     &xi, &yi, &zi, &vx, &vy, &vz, 1, &capped);
        int exited = find_endpoints(&g, hull, x_exit[i], y_exit[i], z_exit[i], xy_exit_angle[i], xz_exit_angle[i],
                                    &xo, &yo, &zo, &vx2, &vy2, &vz2, 0, &capped);
        intersected[i] = 0;
        first_voxel[i] = 0;
        x_in[i] = x_entry[i]; y_in[i] = y_entry[i]; z_in[i] = z_entry[i];
        x_out[i] = x_exit[i]; y_out[i] = y_exit[i]; z_out[i] = z_exit[i];
        if (entered && exited) {
            intersected[i] = 1;
            first_voxel[i] = (uint32_t)(vx + g.columns * vy + g.rows * g.columns * vz);
            x_in[i] = (float)xi; y_in[i] = (float)yi; z_in[i] = (float)zi;
            x_out[i] = (float)xo; y_out[i] = (float)yo; z_out[i] = (float)zo;
        }
    }
    return capped;
}

/* ------------------------------------------------------------------------- */
/* a14-a15: MLP rows                                                          */
/* ------------------------------------------------------------------------- */
/* EffectiveChordLength_GPU (.cu:4974-4995); sinf/cosf are the correctly
 * rounded binary32 functions. */
double ora_effective_chord_length(const pct_config* cfg, double abs_angle_t, double abs_angle_v) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return 0.0;
    const double VW = g.voxel_width, VT = g.voxel_thickness, STEP = g.mlp_u_step;
    double eff_t = abs_angle_t - ((int)(abs_angle_t / (PCT_PI / 2))) * (PCT_PI / 2);
    double eff_v = fabs(abs_angle_v);
    double sf = STEP / VW;
    float s2t = pct_sinf((float)(2 * eff_t)), ct = pct_cosf((float)eff_t), st = pct_sinf((float)eff_t);
    double c2d = (1 / 3.0) * ((sf * sf * s2t - 6) / (sf * s2t - 2 * (ct + st)) + sf * sf * s2t / (2 * (ct + st)));
    double mean_pixel_width = VW / (ct + st);
    double hf = VT / mean_pixel_width;
    sf = STEP / mean_pixel_width;
    float s2v = pct_sinf((float)(2 * eff_v)), cv = pct_cosf((float)eff_v), sv = pct_sinf((float)eff_v);
    double c3d = (1 / 3.0) * ((sf * sf * s2v - 6 * hf) / (sf * s2v - 2 * (hf * cv + sv)) + sf * sf * s2v / (2 * (hf * cv + sv)));
    return VW * c2d * c3d;
}

/* The scattering polynomial pieces as the macros expand them
 * (pCT_data.h:306-348): a leading A_k_OVER_n is (m_k * p_k) / n and an inner
 * "u * A_k_OVER_n" is ((u * m_k) * p_k) / n. */
#define AL(k, n) ((PCT_A##k##_M * PCT_A##k##_P) / (n))
#define AU(u, k, n) ((((u) * PCT_A##k##_M) * PCT_A##k##_P) / (n))
#define A0 (PCT_A0_M * PCT_A0_P)

/* find_MLP_path_GPU (.cu:5279-5501).  Voxel indices are recorded as computed;
 * the reference's 512-entry bound (.cu:5796) is not imposed. */
static int64_t mlp_path(const pct_geometry* g, double x_in, double y_in, double z_in, double x_out, double y_out,
                        double z_out, double xy_entry, double xz_entry, double xy_exit, double xz_exit,
                        uint32_t first_voxel, uint32_t* path, int64_t capacity) {
    const double STEP = g->mlp_u_step;
    int64_t n = 0;
    if (capacity < 1) return -1;
    int voxel = (int)first_voxel;
    path[n++] = (uint32_t)voxel;
    double ce = pct_cos(xy_entry), se = pct_sin(xy_entry);
    double u_in = (ce * x_in) + (se * y_in);
    double u_out = (ce * x_out) + (se * y_out);
    double t_in = (ce * y_in) - (se * x_in);
    double t_out = (ce * y_out) - (se * x_out);
    double v_in = z_in, v_out = z_out;
    if (u_in > u_out) {
        xy_entry += PCT_PI;
        xy_exit += PCT_PI;
        ce = pct_cos(xy_entry);
        se = pct_sin(xy_entry);
        u_in = (ce * x_in) + (se * y_in);
        u_out = (ce * x_out) + (se * y_out);
        t_in = (ce * y_in) - (se * x_in);
        t_out = (ce * y_out) - (se * x_out);
    }
    double T0[2] = {t_in, 0.0}, T2[2] = {t_out, xy_exit - xy_entry};
    double V0[2] = {v_in, 0.0}, V2[2] = {v_out, xz_exit - xz_entry};
    double u_0 = 0.0, u_1 = STEP, u_2 = fabs(u_out - u_in);
    double R0[4] = {1.0, 0.0, 0.0, 1.0}, R1[4] = {1.0, 0.0, 0.0, 1.0}, R1T[4] = {1.0, 0.0, 0.0, 1.0};
    double pre1 = u_2 * u_2 * u_2 * (AL(0, 3) + u_2 * (AL(1, 12) + u_2 * (AL(2, 30) + u_2 * (AL(3, 60) + u_2 * (AL(4, 105) + AU(u_2, 5, 168))))));
    double pre2 = u_2 * u_2 * (AL(0, 2) + u_2 * (AL(1, 6) + u_2 * (AL(2, 12) + u_2 * (AL(3, 20) + u_2 * (AL(4, 30) + AU(u_2, 5, 42))))));
    double pre3 = u_2 * (A0 + u_2 * (AL(1, 2) + u_2 * (AL(2, 3) + u_2 * (AL(3, 4) + u_2 * (AL(4, 5) + AU(u_2, 5, 6))))));
    const int cap = 8 * (g->columns + g->rows + g->slices) + 64;
    int steps = 0;
    while (u_1 < u_2 - STEP) {
        if (++steps > cap) break; /* non-finite endpoints only */
        R0[1] = u_1;
        R1[1] = u_2 - u_1;
        R1T[2] = u_2 - u_1;
        double k1 = PCT_E_0 * (1 + 0.038 * pct_log((u_1 - u_0) / PCT_X_0));
        double c1 = k1 * k1 / PCT_X_0;
        double st1 = c1 * (pct_cube(u_1) * (AL(0, 3) + u_1 * (AL(1, 12) + u_1 * (AL(2, 30) + u_1 * (AL(3, 60) + u_1 * (AL(4, 105) + AU(u_1, 5, 168)))))));
        double stt1 = c1 * ((u_1 * u_1) * (AL(0, 2) + u_1 * (AL(1, 6) + u_1 * (AL(2, 12) + u_1 * (AL(3, 20) + u_1 * (AL(4, 30) + AU(u_1, 5, 42)))))));
        double sth1 = c1 * (u_1 * (A0 + u_1 * (AL(1, 2) + u_1 * (AL(2, 3) + u_1 * (AL(3, 4) + u_1 * (AL(4, 5) + AU(u_1, 5, 6)))))));
        double det1 = st1 * sth1 - stt1 * stt1;
        double S1I[4] = {sth1 / det1, -stt1 / det1, -stt1 / det1, st1 / det1};
        double k2 = PCT_E_0 * (1 + 0.038 * pct_log((u_2 - u_1) / PCT_X_0));
        double c2 = k2 * k2 / PCT_X_0;
        double cst1 = u_1 * (A0 + u_1 * (AL(1, 2) + u_1 * (AL(2, 3) + u_1 * (AL(3, 4) + u_1 * (AL(4, 5) + AU(u_1, 5, 6))))));
        double cst2 = (u_1 * u_1) * (AL(0, 2) + u_1 * (AL(1, 3) + u_1 * (AL(2, 4) + u_1 * (AL(3, 5) + u_1 * (AL(4, 6) + AU(u_1, 5, 7))))));
        double cst3 = pct_cube(u_1) * (AL(0, 3) + u_1 * (AL(1, 4) + u_1 * (AL(2, 5) + u_1 * (AL(3, 6) + u_1 * (AL(4, 7) + AU(u_1, 5, 8))))));
        double st2 = c2 * (pre1 - (u_2 * u_2) * cst1 + 2 * u_2 * cst2 - cst3);
        double stt2 = c2 * (pre2 - u_2 * cst1 + cst2);
        double sth2 = c2 * (pre3 - cst1);
        double det2 = st2 * sth2 - stt2 * stt2;
        double S2I[4] = {sth2 / det2, -stt2 / det2, -stt2 / det2, st2 / det2};
        double f13_1 = S2I[0] * R1[0] + S2I[1] * R1[2];
        double f13_2 = S2I[2] * R1[0] + S2I[3] * R1[2];
        double f24_1 = S2I[0] * R1[1] + S2I[1] * R1[3];
        double f24_2 = S2I[2] * R1[1] + S2I[3] * R1[3];
        double ft[4];
        ft[0] = S1I[0] + R1T[0] * f13_1 + R1T[1] * f13_2;
        ft[1] = S1I[1] + R1T[0] * f24_1 + R1T[1] * f24_2;
        ft[2] = S1I[2] + R1T[2] * f13_1 + R1T[3] * f13_2;
        ft[3] = S1I[3] + R1T[2] * f24_1 + R1T[3] * f24_2;
        double detf = ft[0] * ft[3] - ft[1] * ft[2];
        double tmp = ft[0];
        ft[0] = ft[3] / detf;
        ft[1] = -ft[1] / detf;
        ft[2] = -ft[2] / detf;
        ft[3] = tmp / detf;
        double sc1 = R0[0] * T0[0] + R0[1] * T0[1];
        double sc2 = R0[2] * T0[0] + R0[3] * T0[1];
        double sc3 = S2I[0] * T2[0] + S2I[1] * T2[1];
        double sc4 = S2I[2] * T2[0] + S2I[3] * T2[1];
        double s0 = S1I[0] * sc1 + S1I[1] * sc2 + R1T[0] * sc3 + R1T[1] * sc4;
        double s1 = S1I[2] * sc1 + S1I[3] * sc2 + R1T[2] * sc3 + R1T[3] * sc4;
        double t_1 = ft[0] * s0 + ft[1] * s1;
        sc1 = R0[0] * V0[0] + R0[1] * V0[1];
        sc2 = R0[2] * V0[0] + R0[3] * V0[1];
        sc3 = S2I[0] * V2[0] + S2I[1] * V2[1];
        sc4 = S2I[2] * V2[0] + S2I[3] * V2[1];
        s0 = S1I[0] * sc1 + S1I[1] * sc2 + R1T[0] * sc3 + R1T[1] * sc4;
        s1 = S1I[2] * sc1 + S1I[3] * sc2 + R1T[2] * sc3 + R1T[3] * sc4;
        double v_1 = ft[0] * s0 + ft[1] * s1;
        double x_1 = (ce * (u_in + u_1)) - (se * t_1);
        double y_1 = (se * (u_in + u_1)) + (ce * t_1);
        double z_1 = v_1;
        int vx = calculate_voxel(g->x_zero, x_1, g->voxel_width);
        int vy = calculate_voxel(g->y_zero, y_1, g->voxel_height);
        int vz = calculate_voxel(g->z_zero, z_1, g->voxel_thickness);
        voxel = vx + vy * g->columns + vz * g->columns * g->rows;
        if ((uint32_t)voxel != path[n - 1]) {
            if (n >= capacity) return -1;
            path[n++] = (uint32_t)voxel;
        }
        u_1 += STEP;
    }
    return n;
}

int64_t ora_mlp_rows(const pct_config* cfg, int64_t n, const float* x_in, const float* y_in, const float* z_in,
                     const float* x_out, const float* y_out, const float* z_out, const float* xy_entry_angle,
                     const float* xz_entry_angle, const float* xy_exit_angle, const float* xz_exit_angle,
                     const uint32_t* first_voxel, int64_t* offsets, uint32_t* rows, int64_t capacity, double* chord) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return -1;
    int64_t pos = 0;
    offsets[0] = 0;
    for (int64_t i = 0; i < n; ++i) {
        double ae = xy_entry_angle[i], ax = xy_exit_angle[i], ze = xz_entry_angle[i], zx = xz_exit_angle[i];
        chord[i] = ora_effective_chord_length(cfg, (ae + ax) / 2.0, (ze + zx) / 2.0);
        int64_t k = mlp_path(&g, x_in[i], y_in[i], z_in[i], x_out[i], y_out[i], z_out[i], ae, ze, ax, zx,
                             first_voxel[i], rows + pos, capacity - pos);
        if (k < 0) return -1;
        pos += k;
        offsets[i + 1] = pos;
    }
    return pos;
}

/* Tabulated MLP (.cu:5502-5660).  Tables (.cu:4786-4911): sin/cos of
 * -2 pi + i * 0.001 deg for i <= (6 pi) / step + 0.5; per depth du = k * 5e-5 cm
 * (k <= 800000) the five moment polynomials and the scattering coefficient
 * pow(E_0 (1 + 0.038 log(du / X0)), 2) / X0. */
#define ORA_TRIG_MIN (-2 * PCT_PI)
#define ORA_TRIG_STEP (0.001 * PCT_ANGLE_TO_RADIANS)
#define ORA_TRIG_N ((int)((4 * PCT_PI - -2 * PCT_PI) / ORA_TRIG_STEP + 0.5))
#define ORA_DEPTH_STEP 0.00005
#define ORA_DEPTH_N ((int)(40.0 / ORA_DEPTH_STEP + 0.5))

static double* ora_tab_sin = NULL;
static double* ora_tab_cos = NULL;
static double* ora_tab_p12 = NULL;
static double* ora_tab_p23 = NULL;
static double* ora_tab_p34 = NULL;
static double* ora_tab_p26 = NULL;
static double* ora_tab_p312 = NULL;
static double* ora_tab_sc = NULL;

static int ora_tables(void) {
    if (ora_tab_sin) return 0;
    double* t[8];
    const int64_t sz[8] = {ORA_TRIG_N + 1, ORA_TRIG_N + 1, ORA_DEPTH_N + 1, ORA_DEPTH_N + 1,
                           ORA_DEPTH_N + 1, ORA_DEPTH_N + 1, ORA_DEPTH_N + 1, ORA_DEPTH_N + 1};
    for (int k = 0; k < 8; ++k) {
        t[k] = (double*)malloc(sizeof(double) * (size_t)sz[k]);
        if (!t[k]) {
            for (int j = 0; j < k; ++j) free(t[j]);
            return 2;
        }
    }
    for (int i = 0; i <= ORA_TRIG_N; ++i) {
        double val = ORA_TRIG_MIN + i * ORA_TRIG_STEP;
        pct_sincos_cr(val, &t[0][i], &t[1][i]);
    }
    for (int k = 0; k <= ORA_DEPTH_N; ++k) {
        double du = k * ORA_DEPTH_STEP;
        t[2][k] = du * (A0 + du * (AL(1, 2) + du * (AL(2, 3) + du * (AL(3, 4) + du * (AL(4, 5) + AU(du, 5, 6))))));
        t[3][k] = (du * du) * (AL(0, 2) + du * (AL(1, 3) + du * (AL(2, 4) + du * (AL(3, 5) + du * (AL(4, 6) + AU(du, 5, 7))))));
        t[4][k] = pct_cube(du) * (AL(0, 3) + du * (AL(1, 4) + du * (AL(2, 5) + du * (AL(3, 6) + du * (AL(4, 7) + AU(du, 5, 8))))));
        t[5][k] = (du * du) * (AL(0, 2) + du * (AL(1, 6) + du * (AL(2, 12) + du * (AL(3, 20) + du * (AL(4, 30) + AU(du, 5, 42))))));
        t[6][k] = pct_cube(du) * (AL(0, 3) + du * (AL(1, 12) + du * (AL(2, 30) + du * (AL(3, 60) + du * (AL(4, 105) + AU(du, 5, 168))))));
        double e = PCT_E_0 * (1 + 0.038 * pct_log(du / PCT_X_0));
        t[7][k] = k > 0 ? (e * e) / PCT_X_0 : 0.0;
    }
    ora_tab_sin = t[0]; ora_tab_cos = t[1]; ora_tab_p12 = t[2]; ora_tab_p23 = t[3];
    ora_tab_p34 = t[4]; ora_tab_p26 = t[5]; ora_tab_p312 = t[6]; ora_tab_sc = t[7];
    return 0;
}

static int64_t mlp_path_tab(const pct_geometry* g, double x_in, double y_in, double z_in, double x_out, double y_out,
                            double z_out, double xy_entry, double xz_entry, double xy_exit, double xz_exit,
                            uint32_t first_voxel, uint32_t* path, int64_t capacity) {
    const double STEP = g->mlp_u_step;
    int64_t n = 0;
    if (capacity < 1) return -1;
    path[n++] = first_voxel;
    unsigned idx = (unsigned)((xy_entry - ORA_TRIG_MIN) / ORA_TRIG_STEP + 0.5);
    if (idx > (unsigned)ORA_TRIG_N) return n;
    double s = ora_tab_sin[idx], c = ora_tab_cos[idx];
    double u_in = c * x_in + s * y_in;
    double u_out = c * x_out + s * y_out;
    if (u_in > u_out) {
        xy_entry += PCT_PI;
        xy_exit += PCT_PI;
        idx = (unsigned)((xy_entry - ORA_TRIG_MIN) / ORA_TRIG_STEP + 0.5);
        if (idx > (unsigned)ORA_TRIG_N) return n;
        s = ora_tab_sin[idx];
        c = ora_tab_cos[idx];
        u_in = c * x_in + s * y_in;
        u_out = c * x_out + s * y_out;
    }
    double t_in = c * y_in - s * x_in;
    double t_out = c * y_out - s * x_out;
    double T2b = xy_exit - xy_entry, V2b = xz_exit - xz_entry;
    double u_2 = fabs(u_out - u_in);
    double depth = u_2 - STEP;
    double u_sh = u_in;
    unsigned istep = (unsigned)(STEP / ORA_DEPTH_STEP + 0.5);
    unsigned i1 = istep, i2 = (unsigned)(depth / ORA_DEPTH_STEP + 0.5), ip = istep;
    unsigned iu2 = (unsigned)(u_2 / ORA_DEPTH_STEP + 0.5);
    if (!(u_2 < 40.0) || iu2 > (unsigned)ORA_DEPTH_N) return n;
    double q312 = ora_tab_p312[iu2], q26 = ora_tab_p26[iu2], q12 = ora_tab_p12[iu2];
    uint32_t last = first_voxel;
    while (depth > STEP) {
        double a12 = ora_tab_p12[ip], a23 = ora_tab_p23[ip];
        double st1 = ora_tab_p312[ip], stt1 = ora_tab_p26[ip], sth1 = a12;
        double st2 = q312 - (u_2 * u_2) * a12 + 2 * u_2 * a23 - ora_tab_p34[ip];
        double stt2 = q26 - u_2 * a12 + a23;
        double sth2 = q12 - a12;
        double d1 = ora_tab_sc[i1] * (st1 * sth1 - stt1 * stt1);
        double A1 = sth1 / d1, B1 = stt1 / d1, C1 = st1 / d1;
        double d2 = ora_tab_sc[i2] * (st2 * sth2 - stt2 * stt2);
        double A2 = sth2 / d2, B2 = stt2 / d2, C2 = st2 / d2;
        double common = A2 * depth - B2;
        double f0 = A1 + A2;
        double f1 = common - B1;
        double f2 = depth * A2 - B1 - B2;
        double f3 = C1 + C2 + depth * (common - B2);
        double det = f0 * f3 - f1 * f2;
        double k3 = A2 * t_out - B2 * T2b;
        double e0 = A1 * t_in + k3;
        double e1 = depth * k3 + C2 * T2b - B2 * t_out - B1 * t_in;
        double t_1 = (f3 * e0 - f1 * e1) / det;
        k3 = A2 * z_out - B2 * V2b;
        e0 = A1 * z_in + k3;
        e1 = depth * k3 + C2 * V2b - B2 * z_out - B1 * z_in;
        double v_1 = (f3 * e0 - f1 * e1) / det;
        u_sh += STEP;
        double x_1 = c * u_sh - s * t_1;
        double y_1 = s * u_sh + c * t_1;
        int vx = calculate_voxel(g->x_zero, x_1, g->voxel_width);
        int vy = calculate_voxel(g->y_zero, y_1, g->voxel_height);
        int vz = calculate_voxel(g->z_zero, v_1, g->voxel_thickness);
        uint32_t voxel = (uint32_t)(vx + vy * g->columns + vz * g->columns * g->rows);
        if (voxel != last) {
            if (n >= capacity) return -1;
            path[n++] = voxel;
            last = voxel;
        }
        depth -= STEP;
        i1 += istep;
        i2 -= istep;
        ip += istep;
    }
    return n;
}

int64_t ora_mlp_rows_tab(const pct_config* cfg, int64_t n, const float* x_in, const float* y_in, const float* z_in,
                         const float* x_out, const float* y_out, const float* z_out, const float* xy_entry_angle,
                         const float* xz_entry_angle, const float* xy_exit_angle, const float* xz_exit_angle,
                         const uint32_t* first_voxel, int64_t* offsets, uint32_t* rows, int64_t capacity,
                         double* chord) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g) || ora_tables()) return -1;
    int64_t pos = 0;
    offsets[0] = 0;
    for (int64_t i = 0; i < n; ++i) {
        double ae = xy_entry_angle[i], ax = xy_exit_angle[i], ze = xz_entry_angle[i], zx = xz_exit_angle[i];
        chord[i] = ora_effective_chord_length(cfg, (ae + ax) / 2.0, (ze + zx) / 2.0);
        int64_t k = mlp_path_tab(&g, x_in[i], y_in[i], z_in[i], x_out[i], y_out[i], z_out[i], ae, ze, ax, zx,
                                 first_voxel[i], rows + pos, capacity - pos);
        if (k < 0) return -1;
        pos += k;
        offsets[i + 1] = pos;
    }
    return pos;
}

/* ------------------------------------------------------------------------- */
/* a16-a19: DROP                                                              */
/* ------------------------------------------------------------------------- */
/* block_update_GPU (.cu:5774-5841) + image_update_GPU (.cu:5900-5938), the
 * same update DROP_blocks/DROP_update (.cu:8023-8055) make on the host, here
 * with the image and the update accumulator in binary64.  Row entries outside
 * the image are skipped (the reference reads and writes out of bounds). */
int ora_drop(const pct_config* cfg, int64_t n, const int64_t* offsets, const uint32_t* rows, const double* chord,
             const float* wepl, int iterations, int block_size, double lambda, double* x) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return 1;
    const int nv = g.num_voxels;
    double* upd = (double*)calloc((size_t)nv, sizeof(double));
    uint32_t* cnt = (uint32_t*)calloc((size_t)nv, sizeof(uint32_t));
    if (!upd || !cnt) { free(upd); free(cnt); return 2; }
    for (int it = 0; it < iterations; ++it) {
        for (int64_t start = 0; start < n; start += block_size) {
            int64_t end = start + block_size < n ? start + block_size : n;
            for (int64_t i = start; i < end; ++i) {
                double c = chord[i];
                int64_t a = offsets[i], b = offsets[i + 1];
                double dot = 0.0;
                for (int64_t j = a; j < b; ++j)
                    if (rows[j] < (uint32_t)nv) dot += x[rows[j]];
                dot *= c;
                double aa = (c * c) * (double)(b - a);
                double value = c * ((wepl[i] - dot) / aa) * lambda;
                for (int64_t j = a; j < b; ++j)
                    if (rows[j] < (uint32_t)nv) {
                        cnt[rows[j]] += 1;
                        upd[rows[j]] += value;
                    }
            }
            for (int v = 0; v < nv; ++v)
                if (cnt[v] > 0) {
                    x[v] += upd[v] / cnt[v];
                    upd[v] = 0.0;
                    cnt[v] = 0;
                }
        }
    }
    free(upd);
    free(cnt);
    return 0;
}

/* ora_drop over one shard: the same block update (block_update_GPU
 * .cu:5774-5841 / DROP_blocks .cu:8023-8043) on this rank's rows of block k,
 * the sums over the ranks, then DROP_update (.cu:8044-8055). */
int ora_drop_shard(const pct_config* cfg, int64_t n, const int64_t* offsets, const uint32_t* rows, const double* chord,
                   const float* wepl, int iterations, int block_size, int num_blocks, double lambda, double* x,
                   pct_allreduce_fn fn, void* user) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g) || block_size < 1 || num_blocks < 0 || !fn) return 1;
    const int nv = g.num_voxels;
    double* upd = (double*)calloc((size_t)nv, sizeof(double));
    uint32_t* cnt = (uint32_t*)calloc((size_t)nv, sizeof(uint32_t));
    if (!upd || !cnt) { free(upd); free(cnt); return 2; }
    int rc = 0;
    for (int it = 0; it < iterations && !rc; ++it) {
        for (int k = 0; k < num_blocks && !rc; ++k) {
            int64_t start = (int64_t)k * block_size;
            if (start > n) start = n;
            int64_t end = start + block_size < n ? start + block_size : n;
            for (int64_t i = start; i < end; ++i) {
                double c = chord[i];
                int64_t a = offsets[i], b = offsets[i + 1];
                double dot = 0.0;
                for (int64_t j = a; j < b; ++j)
                    if (rows[j] < (uint32_t)nv) dot += x[rows[j]];
                dot *= c;
                double aa = (c * c) * (double)(b - a);
                double value = c * ((wepl[i] - dot) / aa) * lambda;
                for (int64_t j = a; j < b; ++j)
                    if (rows[j] < (uint32_t)nv) {
                        cnt[rows[j]] += 1;
                        upd[rows[j]] += value;
                    }
            }
            if (fn(user, upd, nv, PCT_DT_F64, 0) || fn(user, cnt, nv, PCT_DT_U32, 0)) {
                rc = 3;
                break;
            }
            for (int v = 0; v < nv; ++v) {
                if (cnt[v] > 0) x[v] += upd[v] / cnt[v];
                upd[v] = 0.0;
                cnt[v] = 0;
            }
        }
    }
    free(upd);
    free(cnt);
    return rc;
}

/* DROP variants of the reference's CPU reconstruction, binary64:
 *   variant 1  DROP_blocks_red (.cu:7998-8021): each entry's update is
 *              c lambda r / (||a||^2 + psi_j), psi_j = ((1 - x_j) eta) psi_sign,
 *              relaxation DROP_update (.cu:8044-8055);
 *   variant 2  DROP_blocks_robust2 / DROP_update_robust2 (.cu:7871-7901): the
 *              standard update, and per voxel ||A||_j = sum of c^2 over every
 *              entry in voxel j of the blocks processed so far (the reference
 *              allocates norm_Ai once per reconstruction, .cu:7448, and never
 *              clears it); x_j += ||A||_j / (||A||_j + psi_j) * update_j / s_j
 *              with psi_j = psi_sign (1 - x_j) eta.
 * variant 0 is ora_drop. */
int ora_drop_variant(const pct_config* cfg, int64_t n, const int64_t* offsets, const uint32_t* rows,
                     const double* chord, const float* wepl, int iterations, int block_size, double lambda,
                     int variant, double eta, int psi_sign, double* x) {
    if (variant == 0) return ora_drop(cfg, n, offsets, rows, chord, wepl, iterations, block_size, lambda, x);
    if (variant != 1 && variant != 2) return 3;
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return 1;
    const int nv = g.num_voxels;
    double* upd = (double*)calloc((size_t)nv, sizeof(double));
    double* norm_a = (double*)calloc((size_t)nv, sizeof(double));
    uint32_t* cnt = (uint32_t*)calloc((size_t)nv, sizeof(uint32_t));
    if (!upd || !cnt || !norm_a) { free(upd); free(cnt); free(norm_a); return 2; }
    for (int it = 0; it < iterations; ++it) {
        for (int64_t start = 0; start < n; start += block_size) {
            int64_t end = start + block_size < n ? start + block_size : n;
            for (int64_t i = start; i < end; ++i) {
                double c = chord[i];
                int64_t a = offsets[i], b = offsets[i + 1];
                double dot = 0.0;
                for (int64_t j = a; j < b; ++j)
                    if (rows[j] < (uint32_t)nv) dot += x[rows[j]];
                dot *= c;
                double aa = (c * c) * (double)(b - a);
                double residual = wepl[i] - dot;
                for (int64_t j = a; j < b; ++j) {
                    uint32_t v = rows[j];
                    if (v >= (uint32_t)nv) continue;
                    cnt[v] += 1;
                    if (variant == 1) {
                        double psi = ((1.0 - x[v]) * eta) * psi_sign;
                        upd[v] += c * lambda * (residual / (aa + psi));
                    } else {
                        upd[v] += c * lambda * (residual / aa);
                        norm_a[v] += c * c;
                    }
                }
            }
            for (int v = 0; v < nv; ++v)
                if (cnt[v] > 0) {
                    if (variant == 1) {
                        x[v] += upd[v] / cnt[v];
                    } else {
                        double psi = psi_sign * (1 - x[v]) * eta;
                        x[v] += (norm_a[v] / (norm_a[v] + psi)) * upd[v] / cnt[v];
                    }
                    upd[v] = 0.0;
                    cnt[v] = 0;
                }
        }
    }
    free(upd);
    free(cnt);
    free(norm_a);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Multithreaded forms (same results) used to time the reference algorithm  */
/* on all host cores.                                                         */
/* ------------------------------------------------------------------------- */
#ifdef _OPENMP
#include <omp.h>
#endif

int64_t ora_mlp_rows_mt(const pct_config* cfg, int64_t n, const float* x_in, const float* y_in, const float* z_in,
                        const float* x_out, const float* y_out, const float* z_out, const float* xy_entry_angle,
                        const float* xz_entry_angle, const float* xy_exit_angle, const float* xz_exit_angle,
                        const uint32_t* first_voxel, int64_t* offsets, uint32_t* rows, int64_t capacity, double* chord,
                        int threads) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return -1;
    const int64_t maxlen = 8 * (g.columns + g.rows + g.slices) + 72;
    int64_t* len = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    if (!len) return -1;
    int failed = 0;
#pragma omp parallel num_threads(threads)
    {
        uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)maxlen);
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            double ae = xy_entry_angle[i], ax = xy_exit_angle[i], ze = xz_entry_angle[i], zx = xz_exit_angle[i];
            chord[i] = ora_effective_chord_length(cfg, (ae + ax) / 2.0, (ze + zx) / 2.0);
            int64_t k = tmp ? mlp_path(&g, x_in[i], y_in[i], z_in[i], x_out[i], y_out[i], z_out[i], ae, ze, ax, zx,
                                       first_voxel[i], tmp, maxlen) : -1;
            if (k < 0) failed = 1;
            len[i] = k < 0 ? 0 : k;
        }
        free(tmp);
    }
    int64_t pos = 0;
    for (int64_t i = 0; i < n; ++i) {
        offsets[i] = pos;
        pos += len[i];
    }
    offsets[n] = pos;
    free(len);
    if (failed || pos > capacity) return -1;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        double ae = xy_entry_angle[i], ax = xy_exit_angle[i], ze = xz_entry_angle[i], zx = xz_exit_angle[i];
        mlp_path(&g, x_in[i], y_in[i], z_in[i], x_out[i], y_out[i], z_out[i], ae, ze, ax, zx, first_voxel[i],
                 rows + offsets[i], offsets[i + 1] - offsets[i]);
    }
    return pos;
}

int ora_drop_mt(const pct_config* cfg, int64_t n, const int64_t* offsets, const uint32_t* rows, const double* chord,
                const float* wepl, int iterations, int block_size, double lambda, double* x, int threads) {
    pct_geometry g;
    if (pct_geometry_derive(cfg, &g)) return 1;
    const int nv = g.num_voxels;
    double* upd = (double*)calloc((size_t)nv, sizeof(double));
    uint32_t* cnt = (uint32_t*)calloc((size_t)nv, sizeof(uint32_t));
    if (!upd || !cnt) { free(upd); free(cnt); return 2; }
    for (int it = 0; it < iterations; ++it) {
        for (int64_t start = 0; start < n; start += block_size) {
            int64_t end = start + block_size < n ? start + block_size : n;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
            for (int64_t i = start; i < end; ++i) {
                double c = chord[i];
                int64_t a = offsets[i], b = offsets[i + 1];
                double dot = 0.0;
                for (int64_t j = a; j < b; ++j)
                    if (rows[j] < (uint32_t)nv) dot += x[rows[j]];
                dot *= c;
                double aa = (c * c) * (double)(b - a);
                double value = c * ((wepl[i] - dot) / aa) * lambda;
                for (int64_t j = a; j < b; ++j) {
                    uint32_t v = rows[j];
                    if (v < (uint32_t)nv) {
#pragma omp atomic update
                        cnt[v] += 1;
#pragma omp atomic update
                        upd[v] += value;
                    }
                }
            }
#pragma omp parallel for num_threads(threads) schedule(static)
            for (int v = 0; v < nv; ++v)
                if (cnt[v] > 0) {
                    x[v] += upd[v] / cnt[v];
                    upd[v] = 0.0;
                    cnt[v] = 0;
                }
        }
    }
    free(upd);
    free(cnt);
    return 0;
}
