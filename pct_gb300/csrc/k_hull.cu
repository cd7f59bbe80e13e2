/*
 * Stages a7-a9: hull detection and hull selection.
 *
 *   k_init_hull      initialize_hull_GPU (.cu:3316-3326)
 *   k_hull_walk      SC_GPU / MSC_GPU / SM_GPU (.cu:3338-3710): straight-line
 *                    voxel walk from the cylinder entry to the exit voxel with
 *                    take_2D_step_GPU / take_3D_step_GPU (.cu:8754-8866), binary64
 *                    in source order, one thread per history (walk_exact).
 *   k_hull_walk_fast the same walk with certified binary32 steps (default).  The reference
 *                    walk has no bound (a walk that passes its exit voxel heading
 *                    to negative indices never ends and writes out of bounds);
 *                    here it stops after 4 (C + R + S) + 16 steps and voxels
 *                    outside the image are skipped, both counted.
 *   k_msc_edge       MSC_edge_detection_GPU (.cu:3569-3596) reading a copy of the
 *                    counts (the reference updates in place while neighbours read)
 *   k_carve, k_sm_threshold, k_sm_edge
 *                    carve_differences (.cu:3274), the host threshold scan of
 *                    SM_edge_detection (.cu:3733-3751, first maximum per slice)
 *                    and SM_edge_detection_GPU (.cu:3774)
 *   k_select, k_avg_filter
 *                    hull_selection (.cu:3954-3990) and averaging_filter_GPU with
 *                    thresholding (.cu:4007-4029)
 */
#include "pct_device.cuh"

namespace {

__global__ void k_init_hull(DevGeom g, int* __restrict__ img) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.num_voxels) return;
    int c = v % g.columns, r = (v / g.columns) % g.rows;
    double x = (c - g.columns / 2 + 0.5) * g.voxel_width;
    double y = (g.rows / 2 - r - 0.5) * g.voxel_height;
    img[v] = (x * x + y * y < g.recon_cyl_radius * g.recon_cyl_radius) ? 1 : 0;
}

struct Walk {
    double x, y, z, x_to_go, y_to_go, z_to_go;
    int vx, vy, vz, voxel;
};

__device__ __forceinline__ void step3(const DevGeom& g, int xm, int ym, int zm, double dy_dx, double dz_dx,
                                      double dz_dy, double dx_dy, double dx_dz, double dy_dz, double xs, double ys,
                                      double zs, Walk& w) {
    double x_ext = fabs(dz_dx) * w.x_to_go;
    double y_ext = fabs(dz_dy) * w.y_to_go;
    if ((w.z_to_go <= x_ext) && (w.z_to_go <= y_ext)) {
        w.vz -= zm;
        w.z = dev_edge_coordinate(g.z_zero, w.vz, g.voxel_thickness, PCT_Z_INC, zm);
        w.x = dev_corresponding(dx_dz, w.z, zs, xs);
        w.y = dev_corresponding(dy_dz, w.z, zs, ys);
        w.x_to_go = dev_distance_remaining(g.x_zero, w.x, PCT_X_INC, xm, g.voxel_width, w.vx);
        w.y_to_go = dev_distance_remaining(g.y_zero, w.y, PCT_Y_INC, ym, g.voxel_height, w.vy);
        w.z_to_go = g.voxel_thickness;
    } else if (x_ext <= y_ext) {
        w.vx += xm;
        w.x = dev_edge_coordinate(g.x_zero, w.vx, g.voxel_width, PCT_X_INC, xm);
        w.y = dev_corresponding(dy_dx, w.x, xs, ys);
        w.z = dev_corresponding(dz_dx, w.x, xs, zs);
        w.x_to_go = g.voxel_width;
        w.y_to_go = dev_distance_remaining(g.y_zero, w.y, PCT_Y_INC, ym, g.voxel_height, w.vy);
        w.z_to_go = dev_distance_remaining(g.z_zero, w.z, PCT_Z_INC, zm, g.voxel_thickness, w.vz);
    } else {
        w.vy -= ym;
        w.y = dev_edge_coordinate(g.y_zero, w.vy, g.voxel_height, PCT_Y_INC, ym);
        w.x = dev_corresponding(dx_dy, w.y, ys, xs);
        w.z = dev_corresponding(dz_dy, w.y, ys, zs);
        w.x_to_go = dev_distance_remaining(g.x_zero, w.x, PCT_X_INC, xm, g.voxel_width, w.vx);
        w.y_to_go = g.voxel_height;
        w.z_to_go = dev_distance_remaining(g.z_zero, w.z, PCT_Z_INC, zm, g.voxel_thickness, w.vz);
    }
    if (w.x_to_go == 0) { w.x_to_go = g.voxel_width; w.vx += xm; }
    if (w.y_to_go == 0) { w.y_to_go = g.voxel_height; w.vy -= ym; }
    if (w.z_to_go == 0) { w.z_to_go = g.voxel_thickness; w.vz -= zm; }
    if (w.vz < 0) w.vz = 0;
    w.voxel = w.vx + w.vy * g.columns + w.vz * g.columns * g.rows;
}

__device__ __forceinline__ void step2(const DevGeom& g, int xm, int ym, double dy_dx, double dx_dy, double xs,
                                      double ys, Walk& w) {
    double y_ext = fabs(dx_dy) * w.y_to_go;
    if (w.x_to_go <= y_ext) {
        w.vx += xm;
        w.x = dev_edge_coordinate(g.x_zero, w.vx, g.voxel_width, PCT_X_INC, xm);
        w.y = dev_corresponding(dy_dx, w.x, xs, ys);
        w.x_to_go = g.voxel_width;
        w.y_to_go = dev_distance_remaining(g.y_zero, w.y, PCT_Y_INC, ym, g.voxel_height, w.vy);
    } else {
        w.vy -= ym;
        w.y = dev_edge_coordinate(g.y_zero, w.vy, g.voxel_height, PCT_Y_INC, ym);
        w.x = dev_corresponding(dx_dy, w.y, ys, xs);
        w.x_to_go = dev_distance_remaining(g.x_zero, w.x, PCT_X_INC, xm, g.voxel_width, w.vx);
        w.y_to_go = g.voxel_height;
    }
    if (w.x_to_go == 0) { w.x_to_go = g.voxel_width; w.vx += xm; }
    if (w.y_to_go == 0) { w.y_to_go = g.voxel_height; w.vy -= ym; }
    if (w.vz < 0) w.vz = 0;
    w.voxel = w.vx + w.vy * g.columns + w.vz * g.columns * g.rows;
}

/* kind 0: SC (set 0), 1: MSC (count), 2: SM (count) */
__global__ void __launch_bounds__(256) k_hull_walk(DevGeom g, int kind, double threshold, int64_t n,
                                                   const uint8_t* __restrict__ missed, HistView h,
                                                   int* __restrict__ img, unsigned long long* __restrict__ flags) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float wepl = h.wepl[i];
    int use = kind == 2 ? (wepl >= threshold) : (wepl <= threshold);
    if (missed[i] || !use) return;
    const float xe = h.x_entry[i], ye = h.y_entry[i], ze = h.z_entry[i];
    const float xx = h.x_exit[i], yx = h.y_exit[i], zx = h.z_exit[i];
    int xm = (xe <= xx) - (xe >= xx);
    int ym = (ye <= yx) - (ye >= yx);
    int zm = (ze <= zx) - (ze >= zx);
    Walk w;
    w.x = xe; w.y = ye; w.z = ze;
    w.vx = dev_calculate_voxel(g.x_zero, xe, g.voxel_width);
    w.vy = dev_calculate_voxel(g.y_zero, ye, g.voxel_height);
    w.vz = dev_calculate_voxel(g.z_zero, ze, g.voxel_thickness);
    w.voxel = w.vx + w.vy * g.columns + w.vz * g.columns * g.rows;
    w.x_to_go = dev_distance_remaining(g.x_zero, w.x, PCT_X_INC, xm, g.voxel_width, w.vx);
    w.y_to_go = dev_distance_remaining(g.y_zero, w.y, PCT_Y_INC, ym, g.voxel_height, w.vy);
    w.z_to_go = dev_distance_remaining(g.z_zero, w.z, PCT_Z_INC, zm, g.voxel_thickness, w.vz);
    double dy_dx = (double)((yx - ye) / (xx - xe));
    double dz_dx = (double)((zx - ze) / (xx - xe));
    double dz_dy = (double)((zx - ze) / (yx - ye));
    double dx_dy = (double)((xx - xe) / (yx - ye));
    double dx_dz = (double)((xx - xe) / (zx - ze));
    double dy_dz = (double)((yx - ye) / (zx - ze));
    int vxo = dev_calculate_voxel(g.x_zero, xx, g.voxel_width);
    int vyo = dev_calculate_voxel(g.y_zero, yx, g.voxel_height);
    int vzo = dev_calculate_voxel(g.z_zero, zx, g.voxel_thickness);
    int voxel_out = vxo + vyo * g.columns + vzo * g.columns * g.rows;
    int end = (w.voxel == voxel_out) || (w.vx >= g.columns) || (w.vy >= g.rows) || (w.vz >= g.slices);
    const int cap = 4 * (g.columns + g.rows + g.slices) + 16;
    int steps = 0;
    for (;;) {
        if (!end) {
            if (w.voxel >= 0 && w.voxel < g.num_voxels) {
                if (kind == 0) img[w.voxel] = 0;
                else atomicAdd(img + w.voxel, 1);
            } else {
                dev_flag(flags, ERR_VOXEL_OUTSIDE);
            }
        }
        if (end) break;
        if (++steps > cap) {
            dev_flag(flags, ERR_WALK_CAPPED);
            break;
        }
        if (zm != 0) step3(g, xm, ym, zm, dy_dx, dz_dx, dz_dy, dx_dy, dx_dz, dy_dz, xe, ye, ze, w);
        else step2(g, xm, ym, dy_dx, dx_dy, xe, ye, w);
        end = (w.voxel == voxel_out) || (w.vx >= g.columns) || (w.vy >= g.rows) || (w.vz >= g.slices);
    }
}

/* ---- binary32 walk with certified decisions ------------------------------------
 * The state after a walk step is a function of the axis crossed and the voxel
 * indices right after that crossing: step2/step3 recompute every coordinate
 * and distance from the crossed edge (nothing accumulates).  k_hull_walk_fast
 * keeps the state in binary32 together with a bound on its distance from the
 * binary64 state, takes a step in binary32 only when every comparison that
 * decides it (and every exact-zero distance test after it) is certain under
 * those bounds, and otherwise rebuilds the binary64 state from the last
 * crossing and takes the step with step2/step3.  The voxel sequence is that
 * of the binary64 walk. */
enum { AX_NONE = 0, AX_X = 1, AX_Y = 2, AX_Z = 3 };

struct WalkLine {
    double xs, ys, zs;
    float fxs, fys, fzs; /* the same start point (binary32 inputs) */
    double dy_dx, dz_dx, dz_dy, dx_dy, dx_dz, dy_dz;
    int xm, ym, zm;
};

/* Binary64 state after crossing axis a with indices (ax, ay, az) before the
 * zero-distance adjustments (AX_NONE: the start of the walk). */
__device__ __noinline__ void walk_state64(const DevGeom& g, const WalkLine& L, int a, int ax, int ay, int az, Walk& w,
                                          double z_init, double z_to_go_init) {
    w.vx = ax;
    w.vy = ay;
    w.vz = az;
    const bool is3d = L.zm != 0;
    if (a == AX_NONE) {
        w.x = L.xs;
        w.y = L.ys;
        w.z = L.zs;
        w.x_to_go = dev_distance_remaining(g.x_zero, w.x, PCT_X_INC, L.xm, g.voxel_width, w.vx);
        w.y_to_go = dev_distance_remaining(g.y_zero, w.y, PCT_Y_INC, L.ym, g.voxel_height, w.vy);
        w.z_to_go = dev_distance_remaining(g.z_zero, w.z, PCT_Z_INC, L.zm, g.voxel_thickness, w.vz);
    } else {
        if (a == AX_X) {
            w.x = dev_edge_coordinate(g.x_zero, w.vx, g.voxel_width, PCT_X_INC, L.xm);
            w.y = dev_corresponding(L.dy_dx, w.x, L.xs, L.ys);
            w.x_to_go = g.voxel_width;
            w.y_to_go = dev_distance_remaining(g.y_zero, w.y, PCT_Y_INC, L.ym, g.voxel_height, w.vy);
            if (is3d) {
                w.z = dev_corresponding(L.dz_dx, w.x, L.xs, L.zs);
                w.z_to_go = dev_distance_remaining(g.z_zero, w.z, PCT_Z_INC, L.zm, g.voxel_thickness, w.vz);
            }
        } else if (a == AX_Y) {
            w.y = dev_edge_coordinate(g.y_zero, w.vy, g.voxel_height, PCT_Y_INC, L.ym);
            w.x = dev_corresponding(L.dx_dy, w.y, L.ys, L.xs);
            w.x_to_go = dev_distance_remaining(g.x_zero, w.x, PCT_X_INC, L.xm, g.voxel_width, w.vx);
            w.y_to_go = g.voxel_height;
            if (is3d) {
                w.z = dev_corresponding(L.dz_dy, w.y, L.ys, L.zs);
                w.z_to_go = dev_distance_remaining(g.z_zero, w.z, PCT_Z_INC, L.zm, g.voxel_thickness, w.vz);
            }
        } else {
            w.z = dev_edge_coordinate(g.z_zero, w.vz, g.voxel_thickness, PCT_Z_INC, L.zm);
            w.x = dev_corresponding(L.dx_dz, w.z, L.zs, L.xs);
            w.y = dev_corresponding(L.dy_dz, w.z, L.zs, L.ys);
            w.x_to_go = dev_distance_remaining(g.x_zero, w.x, PCT_X_INC, L.xm, g.voxel_width, w.vx);
            w.y_to_go = dev_distance_remaining(g.y_zero, w.y, PCT_Y_INC, L.ym, g.voxel_height, w.vy);
            w.z_to_go = g.voxel_thickness;
        }
        if (!is3d) {
            w.z = z_init;
            w.z_to_go = z_to_go_init;
        }
        if (w.x_to_go == 0) { w.x_to_go = g.voxel_width; w.vx += L.xm; }
        if (w.y_to_go == 0) { w.y_to_go = g.voxel_height; w.vy -= L.ym; }
        if (is3d && w.z_to_go == 0) { w.z_to_go = g.voxel_thickness; w.vz -= L.zm; }
        if (w.vz < 0) w.vz = 0;
    }
    w.voxel = w.vx + w.vy * g.columns + w.vz * g.columns * g.rows;
}

/* binary32 state with error bounds */
struct Walk32 {
    float x, y, z, xt, yt, zt;      /* coordinates and distances to the next edges */
    float ex, ey, ez, ext, eyt, ezt; /* bounds on |binary32 - binary64| */
};

__device__ __forceinline__ void walk_to32(const Walk& w, Walk32& f) {
    f.x = (float)w.x; f.y = (float)w.y; f.z = (float)w.z;
    f.xt = (float)w.x_to_go; f.yt = (float)w.y_to_go; f.zt = (float)w.z_to_go;
    f.ex = WU * fabsf(f.x); f.ey = WU * fabsf(f.y); f.ez = WU * fabsf(f.z);
    f.ext = WU * f.xt; f.eyt = WU * f.yt; f.ezt = WU * f.zt;
}

/* One walk step in binary32; returns false (state untouched) when a decision is uncertain. */
__device__ __forceinline__ bool step32(const DevGeom& g, const WalkLine& L, const float* m32, Walk32& f, int& vx,
                                       int& vy, int& vz, int& a_axis, int& ax, int& ay, int& az) {
    const float X0 = g.fx0, Y0 = g.fy0, Z0 = g.fz0;
    const float VW = g.fvw, VH = g.fvh, VT = g.fvt;
    const float xs = L.fxs, ys = L.fys, zs = L.fzs;
    /* m32: dy_dx, dz_dx, dz_dy, dx_dy, dx_dz, dy_dz */
    int axis;
    if (L.zm != 0) {
        float x_ext = fabsf(m32[1]) * f.xt, e_xext = fabsf(m32[1]) * f.ext + WU * x_ext;
        float y_ext = fabsf(m32[2]) * f.yt, e_yext = fabsf(m32[2]) * f.eyt + WU * y_ext;
        int c1 = cmp_le(f.zt, f.ezt, x_ext, e_xext);
        int c2 = cmp_le(f.zt, f.ezt, y_ext, e_yext);
        if (c1 < 0 || c2 < 0) return false;
        if (c1 && c2) {
            axis = AX_Z;
        } else {
            int c3 = cmp_le(x_ext, e_xext, y_ext, e_yext);
            if (c3 < 0) return false;
            axis = c3 ? AX_X : AX_Y;
        }
    } else {
        float y_ext = fabsf(m32[3]) * f.yt, e_yext = fabsf(m32[3]) * f.eyt + WU * y_ext;
        int c = cmp_le(f.xt, f.ext, y_ext, e_yext);
        if (c < 0) return false;
        axis = c ? AX_X : AX_Y;
    }
    int nx = vx, ny = vy, nz = vz;
    Walk32 n = f;
    float e_edge;
    if (axis == AX_X) {
        nx += L.xm;
        n.x = edge32(X0, nx, VW, PCT_X_INC, L.xm, &n.ex);
        n.y = corr32(m32[0], n.x, xs, ys, n.ex, &n.ey);
        n.xt = VW;
        n.ext = WU * VW;
        float ey_edge = 0.0f;
        float ye = edge32(Y0, ny + PCT_Y_INC * L.ym, VH, PCT_Y_INC, L.ym, &ey_edge);
        n.yt = fabsf(ye - n.y);
        n.eyt = ey_edge + n.ey + WU * n.yt;
        if (L.zm != 0) {
            n.z = corr32(m32[1], n.x, xs, zs, n.ex, &n.ez);
            float ze = edge32(Z0, nz + PCT_Z_INC * L.zm, VT, PCT_Z_INC, L.zm, &e_edge);
            n.zt = fabsf(ze - n.z);
            n.ezt = e_edge + n.ez + WU * n.zt;
        }
    } else if (axis == AX_Y) {
        ny -= L.ym;
        n.y = edge32(Y0, ny, VH, PCT_Y_INC, L.ym, &n.ey);
        n.x = corr32(m32[3], n.y, ys, xs, n.ey, &n.ex);
        float xe = edge32(X0, nx + PCT_X_INC * L.xm, VW, PCT_X_INC, L.xm, &e_edge);
        n.xt = fabsf(xe - n.x);
        n.ext = e_edge + n.ex + WU * n.xt;
        n.yt = VH;
        n.eyt = WU * VH;
        if (L.zm != 0) {
            n.z = corr32(m32[2], n.y, ys, zs, n.ey, &n.ez);
            float ze = edge32(Z0, nz + PCT_Z_INC * L.zm, VT, PCT_Z_INC, L.zm, &e_edge);
            n.zt = fabsf(ze - n.z);
            n.ezt = e_edge + n.ez + WU * n.zt;
        }
    } else {
        nz -= L.zm;
        n.z = edge32(Z0, nz, VT, PCT_Z_INC, L.zm, &n.ez);
        n.x = corr32(m32[4], n.z, zs, xs, n.ez, &n.ex);
        n.y = corr32(m32[5], n.z, zs, ys, n.ez, &n.ey);
        float xe = edge32(X0, nx + PCT_X_INC * L.xm, VW, PCT_X_INC, L.xm, &e_edge);
        n.xt = fabsf(xe - n.x);
        n.ext = e_edge + n.ex + WU * n.xt;
        float ye = edge32(Y0, ny + PCT_Y_INC * L.ym, VH, PCT_Y_INC, L.ym, &e_edge);
        n.yt = fabsf(ye - n.y);
        n.eyt = e_edge + n.ey + WU * n.yt;
        n.zt = VT;
        n.ezt = WU * VT;
    }
    /* the exact-zero distance tests must be certain too */
    if (n.xt <= n.ext || n.yt <= n.eyt || (L.zm != 0 && n.zt <= n.ezt)) return false;
    if (!(n.ext < 1e-3f && n.eyt < 1e-3f && n.ezt < 1e-3f)) return false; /* bounds out of their useful range */
    a_axis = axis;
    ax = nx;
    ay = ny;
    az = nz;
    if (nz < 0) nz = 0;
    vx = nx;
    vy = ny;
    vz = nz;
    f = n;
    return true;
}

/* Same walk and image updates as k_hull_walk. */
__global__ void __launch_bounds__(256) k_hull_walk_fast(DevGeom g, int kind, double threshold, int64_t n,
                                                        const uint32_t* __restrict__ order,
                                                        const uint8_t* __restrict__ missed, HistView h,
                                                        int* __restrict__ img, unsigned long long* __restrict__ flags) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (order) i = order[i];
    float wepl = h.wepl[i];
    int use = kind == 2 ? (wepl >= threshold) : (wepl <= threshold);
    if (missed[i] || !use) return;
    const float xe = h.x_entry[i], ye = h.y_entry[i], ze = h.z_entry[i];
    const float xx = h.x_exit[i], yx = h.y_exit[i], zx = h.z_exit[i];
    WalkLine L;
    L.xm = (xe <= xx) - (xe >= xx);
    L.ym = (ye <= yx) - (ye >= yx);
    L.zm = (ze <= zx) - (ze >= zx);
    L.xs = xe; L.ys = ye; L.zs = ze;
    L.fxs = xe; L.fys = ye; L.fzs = ze;
    float m32[6];
    m32[0] = (yx - ye) / (xx - xe);
    m32[1] = (zx - ze) / (xx - xe);
    m32[2] = (zx - ze) / (yx - ye);
    m32[3] = (xx - xe) / (yx - ye);
    m32[4] = (xx - xe) / (zx - ze);
    m32[5] = (yx - ye) / (zx - ze);
    L.dy_dx = m32[0]; L.dz_dx = m32[1]; L.dz_dy = m32[2]; L.dx_dy = m32[3]; L.dx_dz = m32[4]; L.dy_dz = m32[5];
    Walk w;
    walk_state64(g, L, AX_NONE, dev_calculate_voxel(g.x_zero, xe, g.voxel_width),
                 dev_calculate_voxel(g.y_zero, ye, g.voxel_height), dev_calculate_voxel(g.z_zero, ze, g.voxel_thickness),
                 w, 0.0, 0.0);
    const double z_init = w.z, zt_init = w.z_to_go;
    Walk32 f;
    walk_to32(w, f);
    int vx = w.vx, vy = w.vy, vz = w.vz;
    int a_axis = AX_NONE, ax = vx, ay = vy, az = vz;
    int vxo = dev_calculate_voxel(g.x_zero, xx, g.voxel_width);
    int vyo = dev_calculate_voxel(g.y_zero, yx, g.voxel_height);
    int vzo = dev_calculate_voxel(g.z_zero, zx, g.voxel_thickness);
    int voxel_out = vxo + vyo * g.columns + vzo * g.columns * g.rows;
    int voxel = vx + vy * g.columns + vz * g.columns * g.rows;
    int end = (voxel == voxel_out) || (vx >= g.columns) || (vy >= g.rows) || (vz >= g.slices);
    const int cap = 4 * (g.columns + g.rows + g.slices) + 16;
    int steps = 0;
    unsigned long long exact_steps = 0;
    for (;;) {
        if (!end) {
            if (voxel >= 0 && voxel < g.num_voxels) {
                if (kind == 0) img[voxel] = 0;
                else atomicAdd(img + voxel, 1);
            } else {
                dev_flag(flags, ERR_VOXEL_OUTSIDE);
            }
        }
        if (end) break;
        if (++steps > cap) {
            dev_flag(flags, ERR_WALK_CAPPED);
            break;
        }
        if (!step32(g, L, m32, f, vx, vy, vz, a_axis, ax, ay, az)) {
            /* binary64 step from the binary64 state of the last crossing */
            walk_state64(g, L, a_axis, ax, ay, az, w, z_init, zt_init);
            int bx = w.vx, by = w.vy, bz = w.vz;
            int axis;
            if (L.zm != 0) {
                double x_ext = fabs(L.dz_dx) * w.x_to_go, y_ext = fabs(L.dz_dy) * w.y_to_go;
                if ((w.z_to_go <= x_ext) && (w.z_to_go <= y_ext)) axis = AX_Z;
                else axis = x_ext <= y_ext ? AX_X : AX_Y;
            } else {
                axis = w.x_to_go <= fabs(L.dx_dy) * w.y_to_go ? AX_X : AX_Y;
            }
            if (axis == AX_X) bx += L.xm;
            else if (axis == AX_Y) by -= L.ym;
            else bz -= L.zm;
            a_axis = axis;
            ax = bx;
            ay = by;
            az = bz;
            walk_state64(g, L, a_axis, ax, ay, az, w, z_init, zt_init);
            walk_to32(w, f);
            vx = w.vx;
            vy = w.vy;
            vz = w.vz;
            ++exact_steps;
        }
        voxel = vx + vy * g.columns + vz * g.columns * g.rows;
        end = (voxel == voxel_out) || (vx >= g.columns) || (vy >= g.rows) || (vz >= g.slices);
    }
    if (exact_steps) atomicAdd(flags + ERR_WALK_FP64, exact_steps);
}

__device__ __forceinline__ int dev_outside_rim(const DevGeom& g, int c, int r) {
    float x = (float)((c - g.columns / 2 + 0.5) * g.voxel_width);
    float y = (float)((g.rows / 2 - r - 0.5) * g.voxel_height);
    double lim = g.recon_cyl_radius - fmax(g.voxel_width, g.voxel_height) / 2;
    return (double)x * x + (double)y * y >= lim * lim;
}

__device__ __forceinline__ int dev_max_diff(const DevGeom& g, const int* __restrict__ counts, int c, int r, int s) {
    int v = c + r * g.columns + s * g.columns * g.rows;
    int maxd = 0;
    if (r != 0 && r != g.rows - 1 && c != 0 && c != g.columns - 1) {
        int cv = counts[v];
        for (int rr = r - 1; rr <= r + 1; ++rr)
            for (int cc = c - 1; cc <= c + 1; ++cc) {
                int d = cv - counts[cc + rr * g.columns + s * g.columns * g.rows];
                if (d > maxd) maxd = d;
            }
    }
    return maxd;
}

__global__ void k_msc_edge(DevGeom g, int thresh, const int* __restrict__ counts, int* __restrict__ hull) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.num_voxels) return;
    int c = v % g.columns, r = (v / g.columns) % g.rows, s = v / (g.columns * g.rows);
    int h = dev_max_diff(g, counts, c, r, s) > thresh ? 0 : 1;
    if (dev_outside_rim(g, c, r)) h = 0;
    hull[v] = h;
}

__global__ void k_carve(DevGeom g, const int* __restrict__ counts, int* __restrict__ diff) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.num_voxels) return;
    int c = v % g.columns, r = (v / g.columns) % g.rows, s = v / (g.columns * g.rows);
    diff[v] = dev_max_diff(g, counts, c, r, s);
}

/* Per-slice threshold: counts at the first (lowest pixel index) strict
 * maximum of the difference map; 0 if every difference is 0.  One block per
 * slice: max over the slice, then the lowest pixel reaching it. */
__global__ void k_sm_threshold(DevGeom g, const int* __restrict__ counts, const int* __restrict__ diff,
                               int* __restrict__ thr) {
    int s = blockIdx.x;
    int P = g.columns * g.rows;
    const int* d = diff + (int64_t)s * P;
    __shared__ int red[32];
    __shared__ int bmax, bidx;
    int m = 0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) m = max(m, d[p]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = max(t, red[w]);
        bmax = t;
        bidx = P;
    }
    __syncthreads();
    if (bmax > 0)
        for (int p = threadIdx.x; p < P; p += blockDim.x)
            if (d[p] == bmax) atomicMin(&bidx, p);
    __syncthreads();
    if (threadIdx.x == 0) thr[s] = bmax > 0 ? counts[(int64_t)s * P + bidx] : 0;
}

__global__ void k_sm_edge(DevGeom g, double scale, const int* __restrict__ counts, const int* __restrict__ thr,
                          int* __restrict__ hull) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.num_voxels) return;
    int c = v % g.columns, r = (v / g.columns) % g.rows, s = v / (g.columns * g.rows);
    int h = (counts[v] > scale * thr[s]) ? 1 : 0;
    if (dev_outside_rim(g, c, r)) h = 0;
    hull[v] = h;
}

__global__ void k_select_int(int n, const int* __restrict__ src, uint8_t* __restrict__ dst) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) dst[v] = src[v] != 0;
}

__global__ void k_avg_filter(DevGeom g, int radius, double threshold, const uint8_t* __restrict__ in,
                             uint8_t* __restrict__ out) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.num_voxels) return;
    int c = v % g.columns, r = (v / g.columns) % g.rows, s = v / (g.columns * g.rows);
    int left = max(c - radius, 0), right = min(c + radius, g.columns - 1);
    int top = max(r - radius, 0), bottom = min(r + radius, g.rows - 1);
    int nv = (right - left + 1) * (bottom - top + 1);
    double sum_threshold = nv * threshold;
    double sum = 0.0;
    for (int cc = left; cc <= right; ++cc)
        for (int rr = top; rr <= bottom; ++rr) sum += in[cc + rr * g.columns + s * g.columns * g.rows];
    out[v] = sum > sum_threshold;
}

}  // namespace

pct_status pct_hull_images_ready(pct_ctx* c) {
    size_t V = (size_t)c->geo.num_voxels * 4;
    unsigned grid = pct_grid_for(c->geo.num_voxels, 256);
    if (c->cfg.sc_on && !c->sc_hull.p) {
        PCT_TRY(c->sc_hull.alloc(V));
        ++c->launches;
        k_init_hull<<<grid, 256, 0, c->stream>>>(c->dg, c->sc_hull.as<int>());
    }
    if (c->cfg.msc_on && !c->msc_counts.p) {
        PCT_TRY(c->msc_counts.alloc(V));
        ++c->launches;
        k_init_hull<<<grid, 256, 0, c->stream>>>(c->dg, c->msc_counts.as<int>());
    }
    if (c->cfg.sm_on && !c->sm_counts.p) {
        PCT_TRY(c->sm_counts.alloc(V));
        ++c->launches;
        k_init_hull<<<grid, 256, 0, c->stream>>>(c->dg, c->sm_counts.as<int>());
    }
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

/* Work estimate of one hull walk for the launch order: the voxel boundaries
 * between entry and exit (0 for histories the walk skips). */
__global__ void k_walk_key(DevGeom g, int kind, double threshold, int64_t n, const uint8_t* __restrict__ missed,
                           HistView h, uint32_t* __restrict__ key) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float wepl = h.wepl[i];
    const int use = kind == 2 ? (wepl >= threshold) : (wepl <= threshold);
    uint32_t k = 0;
    if (!missed[i] && use) {
        const float s = fabsf(h.x_exit[i] - h.x_entry[i]) * g.fivw + fabsf(h.y_exit[i] - h.y_entry[i]) * g.fivh +
                        fabsf(h.z_exit[i] - h.z_entry[i]) * g.fivt;
        k = s < 1.0e6f ? 1u + (uint32_t)s : 1000000u; /* NaN and huge: last bucket */
    }
    key[i] = k;
}

/* hull_detection (.cu:3265-3273) on the staged chunk c->h2[0, n). */
/* hull_detection (.cu:3265-3273) on n staged histories h (flags missed) on
 * stream st; the images exist (pct_hull_images_ready) and c->walk_order holds
 * at least 2 n entries (the launch order and its keys). */
pct_status pct_hull_walk_range(pct_ctx* c, HistView h, int64_t n, const uint8_t* missed, cudaStream_t st) {
    if (n <= 0) return PCT_OK;
    unsigned grid = pct_grid_for(n, 256);
    unsigned long long* flags = c->err_flags.as<unsigned long long>();
    const bool exact = c->cfg.walk_exact != 0;
    /* the binary32 walks run in order of walk length (warps of equal work) */
    uint32_t* order = nullptr;
    uint32_t* key = nullptr;
    if (!exact && n <= (int64_t)0xffffffffu && c->walk_order.bytes >= sizeof(uint32_t) * 2 * (size_t)n) {
        order = c->walk_order.as<uint32_t>();
        key = order + n;
    }
    auto walk = [&](const DevGeom& g, int kind, double thr, int64_t nn, const uint8_t* ms, const HistView& hv, int* img,
                    unsigned long long* fl) {
        if (exact) {
            k_hull_walk<<<grid, 256, 0, st>>>(g, kind, thr, nn, ms, hv, img, fl);
            return;
        }
        if (order) {
            c->launches += 2;
            k_walk_key<<<grid, 256, 0, st>>>(g, kind, thr, nn, ms, hv, key);
            k_chunk_order<uint32_t><<<(unsigned)((nn + ORDER_CHUNK - 1) / ORDER_CHUNK), 1024, 0, st>>>(nn, key, order);
        }
        k_hull_walk_fast<<<grid, 256, 0, st>>>(g, kind, thr, nn, order, ms, hv, img, fl);
    };
    if (c->cfg.sc_on) {
        ++c->launches;
        walk(c->dg, 0, c->cfg.sc_threshold, n, missed, h, c->sc_hull.as<int>(), flags);
    }
    if (c->cfg.msc_on) {
        ++c->launches;
        walk(c->dg, 1, c->cfg.msc_threshold, n, missed, h, c->msc_counts.as<int>(), flags);
    }
    if (c->cfg.sm_on) {
        ++c->launches;
        walk(c->dg, 2, c->cfg.sm_lower_threshold, n, missed, h, c->sm_counts.as<int>(), flags);
    }
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}


pct_status pct_stage_hull_finish(pct_ctx* c) {
    if (c->stage != ST_BINNED) return pct_fail(PCT_ERR_STATE, "hull_detection_finish needs binned histories");
    PCT_TRY(pct_hull_images_ready(c));
    const int V = c->geo.num_voxels;
    unsigned grid = pct_grid_for(V, 256);
    if (c->cfg.msc_on) {
        PCT_TRY(c->msc_hull.alloc((size_t)V * 4));
        ++c->launches;
        k_msc_edge<<<grid, 256, 0, c->stream>>>(c->dg, c->cfg.msc_diff_thresh, c->msc_counts.as<int>(),
                                                c->msc_hull.as<int>());
    }
    if (c->cfg.sm_on) {
        PCT_TRY(c->sm_hull.alloc((size_t)V * 4));
        DevBuf diff;
        PCT_TRY(diff.alloc((size_t)V * 4 + (size_t)c->geo.slices * 4));
        int* d = diff.as<int>();
        int* thr = d + V;
        ++c->launches;
        k_carve<<<grid, 256, 0, c->stream>>>(c->dg, c->sm_counts.as<int>(), d);
        ++c->launches;
        k_sm_threshold<<<c->geo.slices, 1024, 0, c->stream>>>(c->dg, c->sm_counts.as<int>(), d, thr);
        ++c->launches;
        k_sm_edge<<<grid, 256, 0, c->stream>>>(c->dg, c->cfg.sm_scale_threshold, c->sm_counts.as<int>(), thr,
                                               c->sm_hull.as<int>());
        cudaError_t e = cudaStreamSynchronize(c->stream);
        diff.release();
        if (e != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "SM edge detection: %s", cudaGetErrorString(e));
    }
    PCT_CUDA(cudaGetLastError());
    c->stage = ST_HULLS_DONE;
    return PCT_OK;
}

pct_status pct_stage_hull_selection(pct_ctx* c) {
    if (c->stage < ST_FBP && !(c->stage >= ST_CUT && !c->cfg.fbp_on))
        return pct_fail(PCT_ERR_STATE, "hull_selection before FBP");
    const int V = c->geo.num_voxels;
    unsigned grid = pct_grid_for(V, 256);
    PCT_TRY(c->x_hull.alloc(V));
    switch (c->cfg.mlp_hull) {
        case PCT_SC_HULL:
            if (!c->cfg.sc_on) return pct_fail(PCT_ERR_STATE, "MLP_HULL = SC_HULL needs sc_on");
            ++c->launches;
            k_select_int<<<grid, 256, 0, c->stream>>>(V, c->sc_hull.as<int>(), c->x_hull.as<uint8_t>());
            break;
        case PCT_MSC_HULL:
            if (!c->cfg.msc_on) return pct_fail(PCT_ERR_STATE, "MLP_HULL = MSC_HULL needs msc_on");
            ++c->launches;
            k_select_int<<<grid, 256, 0, c->stream>>>(V, c->msc_hull.as<int>(), c->x_hull.as<uint8_t>());
            break;
        case PCT_SM_HULL:
            if (!c->cfg.sm_on) return pct_fail(PCT_ERR_STATE, "MLP_HULL = SM_HULL needs sm_on");
            ++c->launches;
            k_select_int<<<grid, 256, 0, c->stream>>>(V, c->sm_hull.as<int>(), c->x_hull.as<uint8_t>());
            break;
        default:
            if (!c->fbp_hull.p) return pct_fail(PCT_ERR_STATE, "MLP_HULL = FBP_HULL needs FBP");
            PCT_CUDA(cudaMemcpyAsync(c->x_hull.p, c->fbp_hull.p, V, cudaMemcpyDeviceToDevice, c->stream));
    }
    PCT_TRY(c->x_hull_filtered.alloc(V));
    if (c->cfg.avg_filter_hull) {
        ++c->launches;
        k_avg_filter<<<grid, 256, 0, c->stream>>>(c->dg, c->cfg.hull_filter_radius, c->cfg.hull_filter_threshold,
                                                  c->x_hull.as<uint8_t>(), c->x_hull_filtered.as<uint8_t>());
    } else
        PCT_CUDA(cudaMemcpyAsync(c->x_hull_filtered.p, c->x_hull.p, V, cudaMemcpyDeviceToDevice, c->stream));
    PCT_CUDA(cudaGetLastError());
    c->stage = ST_HULL_SELECTED;
    return PCT_OK;
}
