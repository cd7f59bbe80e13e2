/*
 * Stages a13-a15: MLP hull endpoints and MLP voxel rows.
 *
 *   k_endpoints   collect_MLP_endpoints_GPU + find_MLP_endpoints_GPU
 *                 (.cu:5729-5770, 4997-5277): walk from the cylinder entry (and
 *                 backwards from the exit) to the first hull voxel; binary64 in
 *                 source order; bounded like the hull walks.
 *   k_mlp_count / k_mlp_fill
 *                 find_MLP_path_GPU (.cu:5279-5501): the Schulte most-likely path
 *                 sampled every MLP_U_STEP in depth, consecutive repeats dropped.
 *                 The rows are generated once and stay resident for every DROP
 *                 iteration (the reference recomputes them in every block of
 *                 every iteration).  Count pass, exclusive scan, fill pass.
 *   k_row_norms   EffectiveChordLength_GPU (.cu:4974-4995) per row and the DROP
 *                 row norm ||a_i||^2 = c^2 n (.cu:5825) kept as 1/||a_i||^2 in binary64.
 */
#include "pct_device.cuh"

namespace {

/* find_MLP_endpoints_GPU (.cu:4997-5277) */
__device__ int dev_find_endpoint(const DevGeom& g, const uint8_t* __restrict__ image, double x_start, double y_start,
                                 double z_start, double xy_angle, double xz_angle, double* xo, double* yo, double* zo,
                                 int* vxo, int* vyo, int* vzo, int entering, unsigned long long* flags) {
    const int C = g.columns, R = g.rows, S = g.slices;
    const int cap = 4 * (C + R + S) + 16;
    double x = x_start, y = y_start, z = z_start;
    int hit = 0, end, outside;
    if (!entering) xy_angle += PCT_PI;
    double cxy = pct_cos(xy_angle), sxy = pct_sin(xy_angle), sxz = pct_sin(xz_angle);
    int xm = (cxy >= 0) - (cxy <= 0);
    int ym = (sxy >= 0) - (sxy <= 0);
    int zm = (sxz >= 0) - (sxz <= 0);
    if (xm < 0) zm *= -1;
    int vx = dev_calculate_voxel(g.x_zero, x, g.voxel_width);
    int vy = dev_calculate_voxel(g.y_zero, y, g.voxel_height);
    int vz = dev_calculate_voxel(g.z_zero, z, g.voxel_thickness);
    double x_to_go = dev_distance_remaining(g.x_zero, x, PCT_X_INC, xm, g.voxel_width, vx);
    double y_to_go = dev_distance_remaining(g.y_zero, y, PCT_Y_INC, ym, g.voxel_height, vy);
    double z_to_go = dev_distance_remaining(g.z_zero, z, PCT_Z_INC, zm, g.voxel_thickness, vz);
    int voxel = vx + vy * C + vz * C * R;
    double txy = pct_tan(xy_angle), txz = pct_tan(xz_angle);
    double delta_yx = fabs(txy), delta_zx = fabs(txz), delta_zy = fabs(txz / txy);
    double dy_dx = txy, dz_dx = txz, dz_dy = txz / txy;
    double dx_dy = 1.0 / txy, dx_dz = 1.0 / txz, dy_dz = txy / txz;
    outside = (vx >= C) || (vy >= R) || (vz >= S) || (vx < 0) || (vy < 0) || (vz < 0);
    if (!outside) hit = (image[voxel] == 1);
    end = outside || hit;
    int steps = 0;
    if (zm != 0) {
        while (!end) {
            if (++steps > cap) {
                dev_flag(flags, ERR_WALK_CAPPED);
                break;
            }
            double x_ext = delta_zx * x_to_go;
            double y_ext = delta_zy * y_to_go;
            if ((z_to_go <= x_ext) && (z_to_go <= y_ext)) {
                vz -= zm;
                z = dev_edge_coordinate(g.z_zero, vz, g.voxel_thickness, PCT_Z_INC, zm);
                x = dev_corresponding(dx_dz, z, z_start, x_start);
                y = dev_corresponding(dy_dz, z, z_start, y_start);
                x_to_go = dev_distance_remaining(g.x_zero, x, PCT_X_INC, xm, g.voxel_width, vx);
                y_to_go = dev_distance_remaining(g.y_zero, y, PCT_Y_INC, ym, g.voxel_height, vy);
                z_to_go = g.voxel_thickness;
            } else if (x_ext <= y_ext) {
                vx += xm;
                x = dev_edge_coordinate(g.x_zero, vx, g.voxel_width, PCT_X_INC, xm);
                y = dev_corresponding(dy_dx, x, x_start, y_start);
                z = dev_corresponding(dz_dx, x, x_start, z_start);
                x_to_go = g.voxel_width;
                y_to_go = dev_distance_remaining(g.y_zero, y, PCT_Y_INC, ym, g.voxel_height, vy);
                z_to_go = dev_distance_remaining(g.z_zero, z, PCT_Z_INC, zm, g.voxel_thickness, vz);
            } else {
                vy -= ym;
                y = dev_edge_coordinate(g.y_zero, vy, g.voxel_height, PCT_Y_INC, ym);
                x = dev_corresponding(dx_dy, y, y_start, x_start);
                z = dev_corresponding(dz_dy, y, y_start, z_start);
                x_to_go = dev_distance_remaining(g.x_zero, x, PCT_X_INC, xm, g.voxel_width, vx);
                y_to_go = g.voxel_height;
                z_to_go = dev_distance_remaining(g.z_zero, z, PCT_Z_INC, zm, g.voxel_thickness, vz);
            }
            if (x_to_go == 0) { x_to_go = g.voxel_width; vx += xm; }
            if (y_to_go == 0) { y_to_go = g.voxel_height; vy -= ym; }
            if (z_to_go == 0) { z_to_go = g.voxel_thickness; vz -= zm; }
            if (vz < 0) vz = 0;
            voxel = vx + vy * C + vz * C * R;
            outside = (vx >= C) || (vy >= R) || (vz >= S) || (vx < 0) || (vy < 0) || (vz < 0);
            if (!outside) hit = (image[voxel] == 1);
            end = outside || hit;
        }
    } else {
        while (!end) {
            if (++steps > cap) {
                dev_flag(flags, ERR_WALK_CAPPED);
                break;
            }
            double y_ext = y_to_go / delta_yx;
            if (x_to_go <= y_ext) {
                vx += xm;
                x = dev_edge_coordinate(g.x_zero, vx, g.voxel_width, PCT_X_INC, xm);
                y = dev_corresponding(dy_dx, x, x_start, y_start);
                x_to_go = g.voxel_width;
                y_to_go = dev_distance_remaining(g.y_zero, y, PCT_Y_INC, ym, g.voxel_height, vy);
            } else {
                vy -= ym;
                y = dev_edge_coordinate(g.y_zero, vy, g.voxel_height, PCT_Z_INC, ym);
                x = dev_corresponding(dx_dy, y, y_start, x_start);
                x_to_go = dev_distance_remaining(g.x_zero, x, PCT_X_INC, xm, g.voxel_width, vx);
                y_to_go = g.voxel_height;
            }
            if (x_to_go == 0) { x_to_go = g.voxel_width; vx += xm; }
            if (y_to_go == 0) { y_to_go = g.voxel_height; vy -= ym; }
            voxel = vx + vy * C + vz * C * R;
            outside = (vx >= C) || (vy >= R) || (vz >= S) || (vx < 0) || (vy < 0) || (vz < 0);
            if (!outside) hit = (image[voxel] == 1);
            end = outside || hit;
        }
    }
    if (hit) {
        *xo = x;
        *yo = y;
        *zo = z;
    }
    *vxo = vx;
    *vyo = vy;
    *vzo = vz;
    return hit;
}

__global__ void __launch_bounds__(128) k_endpoints(DevGeom g, int64_t n, const uint8_t* __restrict__ hull, HistView h,
                                                   uint8_t* __restrict__ keep, unsigned long long* __restrict__ flags) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double xi = 0, yi = 0, zi = 0, xo = 0, yo = 0, zo = 0;
    int vx = 0, vy = 0, vz = 0, vx2 = 0, vy2 = 0, vz2 = 0;
    int entered = dev_find_endpoint(g, hull, h.x_entry[i], h.y_entry[i], h.z_entry[i], h.xy_entry_angle[i],
                                    h.xz_entry_angle[i], &xi, &yi, &zi, &vx, &vy, &vz, 1, flags);
    int exited = dev_find_endpoint(g, hull, h.x_exit[i], h.y_exit[i], h.z_exit[i], h.xy_exit_angle[i],
                                   h.xz_exit_angle[i], &xo, &yo, &zo, &vx2, &vy2, &vz2, 0, flags);
    int both = entered && exited;
    keep[i] = (uint8_t)both;
    h.first_voxel[i] = both ? (uint32_t)(vx + g.columns * vy + g.rows * g.columns * vz) : 0u;
    if (both) {
        h.x_entry[i] = (float)xi; h.y_entry[i] = (float)yi; h.z_entry[i] = (float)zi;
        h.x_exit[i] = (float)xo; h.y_exit[i] = (float)yo; h.z_exit[i] = (float)zo;
    }
}

/* ---- MLP path (find_MLP_path_GPU, .cu:5279-5501) --------------------------- */
/* The scattering polynomial pieces as the reference macros expand them
 * (pCT_data.h:306-348): a leading A_k_OVER_n is (m_k * p_k) / n and an inner
 * "u * A_k_OVER_n" is ((u * m_k) * p_k) / n. */
#define AL(k, n) ((PCT_A##k##_M * PCT_A##k##_P) / (n))
#define AU(u, k, n) ((((u) * PCT_A##k##_M) * PCT_A##k##_P) / (n))
#define A0 (PCT_A0_M * PCT_A0_P)

struct MlpSetup {
    double ce, se, u_in, u_2, pre1, pre2, pre3;
    double T0, T20, T21, V0, V20, V21;
};

__device__ __forceinline__ void dev_mlp_setup(const HistView& h, int64_t i, MlpSetup& m) {
    double x_in = h.x_entry[i], y_in = h.y_entry[i], z_in = h.z_entry[i];
    double x_out = h.x_exit[i], y_out = h.y_exit[i], z_out = h.z_exit[i];
    double xy_entry = h.xy_entry_angle[i], xy_exit = h.xy_exit_angle[i];
    double xz_entry = h.xz_entry_angle[i], xz_exit = h.xz_exit_angle[i];
    double ce = pct_cos(xy_entry), se = pct_sin(xy_entry);
    double u_in = (ce * x_in) + (se * y_in);
    double u_out = (ce * x_out) + (se * y_out);
    double t_in = (ce * y_in) - (se * x_in);
    double t_out = (ce * y_out) - (se * x_out);
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
    m.ce = ce;
    m.se = se;
    m.u_in = u_in;
    m.T0 = t_in;
    m.T20 = t_out;
    m.T21 = xy_exit - xy_entry;
    m.V0 = z_in;
    m.V20 = z_out;
    m.V21 = xz_exit - xz_entry;
    double u_2 = fabs(u_out - u_in);
    m.u_2 = u_2;
    m.pre1 = u_2 * u_2 * u_2 * (AL(0, 3) + u_2 * (AL(1, 12) + u_2 * (AL(2, 30) + u_2 * (AL(3, 60) + u_2 * (AL(4, 105) + AU(u_2, 5, 168))))));
    m.pre2 = u_2 * u_2 * (AL(0, 2) + u_2 * (AL(1, 6) + u_2 * (AL(2, 12) + u_2 * (AL(3, 20) + u_2 * (AL(4, 30) + AU(u_2, 5, 42))))));
    m.pre3 = u_2 * (A0 + u_2 * (AL(1, 2) + u_2 * (AL(2, 3) + u_2 * (AL(3, 4) + u_2 * (AL(4, 5) + AU(u_2, 5, 6))))));
}

/* One MLP sample at depth u_1 in binary64, the reference's operation order. */
__device__ __forceinline__ int dev_mlp_voxel(const DevGeom& g, const MlpSetup& m, double u_1) {
    const double u_0 = 0.0, u_2 = m.u_2;
    double R0_1 = u_1, R1_1 = u_2 - u_1, R1T_2 = u_2 - u_1;
    const double R0_0 = 1.0, R0_2 = 0.0, R0_3 = 1.0, R1_0 = 1.0, R1_2 = 0.0, R1_3 = 1.0;
    const double R1T_0 = 1.0, R1T_1 = 0.0, R1T_3 = 1.0;
    double k1 = PCT_E_0 * (1 + 0.038 * pct_log((u_1 - u_0) / PCT_X_0));
    double c1 = k1 * k1 / PCT_X_0;
    double st1 = c1 * (pct_cube(u_1) * (AL(0, 3) + u_1 * (AL(1, 12) + u_1 * (AL(2, 30) + u_1 * (AL(3, 60) + u_1 * (AL(4, 105) + AU(u_1, 5, 168)))))));
    double stt1 = c1 * ((u_1 * u_1) * (AL(0, 2) + u_1 * (AL(1, 6) + u_1 * (AL(2, 12) + u_1 * (AL(3, 20) + u_1 * (AL(4, 30) + AU(u_1, 5, 42)))))));
    double sth1 = c1 * (u_1 * (A0 + u_1 * (AL(1, 2) + u_1 * (AL(2, 3) + u_1 * (AL(3, 4) + u_1 * (AL(4, 5) + AU(u_1, 5, 6)))))));
    double det1 = st1 * sth1 - stt1 * stt1;
    double S1I0 = sth1 / det1, S1I1 = -stt1 / det1, S1I2 = -stt1 / det1, S1I3 = st1 / det1;
    double k2 = PCT_E_0 * (1 + 0.038 * pct_log((u_2 - u_1) / PCT_X_0));
    double c2 = k2 * k2 / PCT_X_0;
    double cst1 = u_1 * (A0 + u_1 * (AL(1, 2) + u_1 * (AL(2, 3) + u_1 * (AL(3, 4) + u_1 * (AL(4, 5) + AU(u_1, 5, 6))))));
    double cst2 = (u_1 * u_1) * (AL(0, 2) + u_1 * (AL(1, 3) + u_1 * (AL(2, 4) + u_1 * (AL(3, 5) + u_1 * (AL(4, 6) + AU(u_1, 5, 7))))));
    double cst3 = pct_cube(u_1) * (AL(0, 3) + u_1 * (AL(1, 4) + u_1 * (AL(2, 5) + u_1 * (AL(3, 6) + u_1 * (AL(4, 7) + AU(u_1, 5, 8))))));
    double st2 = c2 * (m.pre1 - (u_2 * u_2) * cst1 + 2 * u_2 * cst2 - cst3);
    double stt2 = c2 * (m.pre2 - u_2 * cst1 + cst2);
    double sth2 = c2 * (m.pre3 - cst1);
    double det2 = st2 * sth2 - stt2 * stt2;
    double S2I0 = sth2 / det2, S2I1 = -stt2 / det2, S2I2 = -stt2 / det2, S2I3 = st2 / det2;
    double f13_1 = S2I0 * R1_0 + S2I1 * R1_2;
    double f13_2 = S2I2 * R1_0 + S2I3 * R1_2;
    double f24_1 = S2I0 * R1_1 + S2I1 * R1_3;
    double f24_2 = S2I2 * R1_1 + S2I3 * R1_3;
    double ft0 = S1I0 + R1T_0 * f13_1 + R1T_1 * f13_2;
    double ft1 = S1I1 + R1T_0 * f24_1 + R1T_1 * f24_2;
    double ft2 = S1I2 + R1T_2 * f13_1 + R1T_3 * f13_2;
    double ft3 = S1I3 + R1T_2 * f24_1 + R1T_3 * f24_2;
    double detf = ft0 * ft3 - ft1 * ft2;
    double tmp = ft0;
    ft0 = ft3 / detf;
    ft1 = -ft1 / detf;
    ft2 = -ft2 / detf;
    ft3 = tmp / detf;
    (void)ft2;
    (void)ft3;
    double sc1 = R0_0 * m.T0 + R0_1 * 0.0;
    double sc2 = R0_2 * m.T0 + R0_3 * 0.0;
    double sc3 = S2I0 * m.T20 + S2I1 * m.T21;
    double sc4 = S2I2 * m.T20 + S2I3 * m.T21;
    double s0 = S1I0 * sc1 + S1I1 * sc2 + R1T_0 * sc3 + R1T_1 * sc4;
    double s1 = S1I2 * sc1 + S1I3 * sc2 + R1T_2 * sc3 + R1T_3 * sc4;
    double t_1 = ft0 * s0 + ft1 * s1;
    sc1 = R0_0 * m.V0 + R0_1 * 0.0;
    sc2 = R0_2 * m.V0 + R0_3 * 0.0;
    sc3 = S2I0 * m.V20 + S2I1 * m.V21;
    sc4 = S2I2 * m.V20 + S2I3 * m.V21;
    s0 = S1I0 * sc1 + S1I1 * sc2 + R1T_0 * sc3 + R1T_1 * sc4;
    s1 = S1I2 * sc1 + S1I3 * sc2 + R1T_2 * sc3 + R1T_3 * sc4;
    double v_1 = ft0 * s0 + ft1 * s1;
    double x_1 = (m.ce * (m.u_in + u_1)) - (m.se * t_1);
    double y_1 = (m.se * (m.u_in + u_1)) + (m.ce * t_1);
    double z_1 = v_1;
    int vx = dev_calculate_voxel(g.x_zero, x_1, g.voxel_width);
    int vy = dev_calculate_voxel(g.y_zero, y_1, g.voxel_height);
    int vz = dev_calculate_voxel(g.z_zero, z_1, g.voxel_thickness);
    return vx + vy * g.columns + vz * g.columns * g.rows;
}

/* Walks the MLP of history i; emit(voxel) is called for every row entry. */
template <class Emit>
__device__ __forceinline__ void dev_mlp_row(const DevGeom& g, const HistView& h, int64_t i, Emit emit) {
    MlpSetup m;
    dev_mlp_setup(h, i, m);
    int prev = (int)h.first_voxel[i];
    emit(prev);
    const double STEP = g.mlp_u_step;
    /* a path is never longer than the image diagonal; the cap only guards
       against non-finite endpoints */
    const int cap = 8 * (g.columns + g.rows + g.slices) + 64;
    int k = 0;
    for (double u_1 = STEP; u_1 < m.u_2 - STEP; u_1 += STEP) {
        if (++k > cap) break;
        int v = dev_mlp_voxel(g, m, u_1);
        if ((uint32_t)v != (uint32_t)prev) {
            emit(v);
            prev = v;
        }
    }
}

__global__ void __launch_bounds__(128) k_mlp_count(DevGeom g, int64_t n, HistView h, int64_t* __restrict__ len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t k = 0;
    dev_mlp_row(g, h, i, [&](int) { ++k; });
    len[i] = k;
}

__global__ void __launch_bounds__(128) k_mlp_fill(DevGeom g, int64_t n, HistView h, const int64_t* __restrict__ off,
                                                  uint32_t* __restrict__ rows, unsigned long long* __restrict__ flags) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t p = off[i], end = off[i + 1];
    int outside = 0;
    dev_mlp_row(g, h, i, [&](int v) {
        if (p < end) rows[p++] = (uint32_t)v;
        if ((uint32_t)v >= (uint32_t)g.num_voxels) ++outside;
    });
    if (outside) atomicAdd(flags + ERR_ROWS_OUTSIDE, (unsigned long long)outside);
}

/* EffectiveChordLength_GPU (.cu:4974-4995) with correctly rounded sinf/cosf */
__device__ double dev_chord(const DevGeom& g, double abs_angle_t, double abs_angle_v) {
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

__global__ void k_row_norms(DevGeom g, int64_t n, HistView h, const int64_t* __restrict__ off, float* __restrict__ chord,
                            double* __restrict__ inv_norm) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double ae = h.xy_entry_angle[i], ax = h.xy_exit_angle[i], ze = h.xz_entry_angle[i], zx = h.xz_exit_angle[i];
    double c = dev_chord(g, (ae + ax) / 2.0, (ze + zx) / 2.0);
    chord[i] = (float)c;
    double nn = (double)(off[i + 1] - off[i]);
    inv_norm[i] = 1.0 / ((c * c) * nn);
}

/* Exclusive scan of int64 lengths into offsets[0..n]: per-tile sums, a scan of
 * the tile sums in one CTA, then a local scan per tile. */
constexpr int SCAN_THREADS = 1024;

__device__ __forceinline__ int64_t block_inclusive_scan(int64_t v, int64_t* ws) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    int64_t r = x + (w > 0 ? ws[w - 1] : 0);
    __syncthreads();
    return r;
}

__global__ void k_tile_sum64(const int64_t* __restrict__ len, int64_t n, int64_t* __restrict__ tile_sum) {
    __shared__ int64_t ws[32];
    int64_t i = (int64_t)blockIdx.x * SCAN_THREADS + threadIdx.x;
    int64_t v = i < n ? len[i] : 0;
    int64_t incl = block_inclusive_scan(v, ws);
    if (threadIdx.x == SCAN_THREADS - 1) tile_sum[blockIdx.x] = incl;
}

__global__ void k_scan_tile_sums(int64_t* __restrict__ tile_sum, int64_t tiles, int64_t* __restrict__ total) {
    __shared__ int64_t ws[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < tiles; base += SCAN_THREADS) {
        int64_t i = base + threadIdx.x;
        int64_t v = i < tiles ? tile_sum[i] : 0;
        int64_t incl = block_inclusive_scan(v, ws);
        if (i < tiles) tile_sum[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == SCAN_THREADS - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_tile_scan64(const int64_t* __restrict__ len, int64_t n, const int64_t* __restrict__ tile_off,
                              const int64_t* __restrict__ total, int64_t* __restrict__ off) {
    __shared__ int64_t ws[32];
    int64_t i = (int64_t)blockIdx.x * SCAN_THREADS + threadIdx.x;
    int64_t v = i < n ? len[i] : 0;
    int64_t incl = block_inclusive_scan(v, ws);
    if (i < n) off[i] = tile_off[blockIdx.x] + incl - v;
    if (i == 0) off[n] = *total;
}

}  // namespace

pct_status pct_stage_endpoints(pct_ctx* c) {
    if (c->stage != ST_X0) return pct_fail(PCT_ERR_STATE, "collect_mlp_endpoints needs the initial iterate");
    const int64_t n = c->h.n;
    PCT_TRY(c->tmp_missed.alloc(n > 0 ? n : 1));
    uint8_t* keep = c->tmp_missed.as<uint8_t>();
    if (n > 0) {
        HistView h = c->view(c->h);
        ++c->launches;
        k_endpoints<<<pct_grid_for(n, 128), 128, 0, c->stream>>>(c->dg, n, c->x_hull_filtered.as<uint8_t>(), h, keep,
                                                                 c->err_flags.as<unsigned long long>());
        PCT_CUDA(cudaGetLastError());
    }
    int64_t kept = 0;
    PCT_TRY(pct_compact_histories(c, keep, n, &kept));
    c->counts.reconstruction_histories = kept;
    c->stage = ST_ENDPOINTS;
    return PCT_OK;
}

pct_status pct_scan_lengths(pct_ctx* c, const int64_t* len, int64_t n, int64_t* off, int64_t* total) {
    int64_t tiles = (n + SCAN_THREADS - 1) / SCAN_THREADS;
    DevBuf tmp;
    PCT_TRY(tmp.alloc(sizeof(int64_t) * (tiles + 1)));
    int64_t* tile = tmp.as<int64_t>();
    int64_t* d_total = tile + tiles;
    ++c->launches;
    k_tile_sum64<<<(unsigned)tiles, SCAN_THREADS, 0, c->stream>>>(len, n, tile);
    ++c->launches;
    k_scan_tile_sums<<<1, SCAN_THREADS, 0, c->stream>>>(tile, tiles, d_total);
    ++c->launches;
    k_tile_scan64<<<(unsigned)tiles, SCAN_THREADS, 0, c->stream>>>(len, n, tile, d_total, off);
    PCT_CUDA(cudaMemcpyAsync(total, d_total, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    cudaError_t e = cudaStreamSynchronize(c->stream);
    tmp.release();
    if (e != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "offset scan: %s", cudaGetErrorString(e));
    return PCT_OK;
}

pct_status pct_stage_mlp_rows(pct_ctx* c) {
    if (c->stage < ST_ENDPOINTS) return pct_fail(PCT_ERR_STATE, "mlp_rows needs collect_mlp_endpoints");
    const int64_t n = c->h.n;
    PCT_TRY(c->row_offsets.alloc(sizeof(int64_t) * (n + 1)));
    PCT_TRY(c->chord.alloc(sizeof(float) * (n > 0 ? n : 1)));
    PCT_TRY(c->inv_norm.alloc(sizeof(double) * (n > 0 ? n : 1)));
    int64_t total = 0;
    HistView h = c->view(c->h);
    if (n > 0) {
        DevBuf len;
        PCT_TRY(len.alloc(sizeof(int64_t) * n));
        ++c->launches;
        k_mlp_count<<<pct_grid_for(n, 128), 128, 0, c->stream>>>(c->dg, n, h, len.as<int64_t>());
        pct_status st = pct_scan_lengths(c, len.as<int64_t>(), n, c->row_offsets.as<int64_t>(), &total);
        len.release();
        PCT_TRY(st);
        PCT_TRY(c->rows.alloc(sizeof(uint32_t) * (total > 0 ? total : 1)));
        ++c->launches;
        k_mlp_fill<<<pct_grid_for(n, 128), 128, 0, c->stream>>>(c->dg, n, h, c->row_offsets.as<int64_t>(),
                                                                c->rows.as<uint32_t>(),
                                                                c->err_flags.as<unsigned long long>());
        ++c->launches;
        k_row_norms<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(c->dg, n, h, c->row_offsets.as<int64_t>(),
                                                                 c->chord.as<float>(), c->inv_norm.as<double>());
        PCT_CUDA(cudaGetLastError());
    } else {
        PCT_CUDA(cudaMemsetAsync(c->row_offsets.p, 0, sizeof(int64_t), c->stream));
    }
    c->counts.row_entries = total;
    c->diag_ready = 0;
    pct_drop_release_graph(c);
    c->stage = ST_ROWS;
    return PCT_OK;
}
