/*
 * Stages a13-a15: MLP hull endpoints and MLP voxel rows.
 *
 *   k_endpoints   collect_MLP_endpoints_GPU + find_MLP_endpoints_GPU
 *                 (.cu:5729-5770, 4997-5277): walk from the cylinder entry (and
 *                 backwards from the exit) to the first hull voxel; binary64 in
 *                 source order; bounded like the hull walks.
 *   k_mlp_bound / k_mlp_fast
 *                 find_MLP_path_GPU (.cu:5279-5501): the Schulte most-likely path
 *                 sampled every MLP_U_STEP in depth, consecutive repeats dropped.
 *                 The rows are generated once and stay resident for every DROP
 *                 iteration (the reference recomputes them in every block of
 *                 every iteration).  The sample count of a row is known from its
 *                 depth u_2, so each row gets a slot of that size (k_mlp_bound +
 *                 scan) and one pass fills it; binary32 samples with a binary64
 *                 recomputation near voxel faces (see below).
 *   chords        EffectiveChordLength_GPU (.cu:4974-4995) per row, in binary64
 *                 inside k_mlp_fast (its FP64 work overlaps the binary32 samples),
 *                 and the DROP row scale 1 / (c n) from ||a_i||^2 = c^2 n (.cu:5825)
 *                 once the row length is final (k_mlp_fast or k_mlp_dedupe);
 *                 k_row_norms does both for rows read from a file.
 */
#include <cuda_bf16.h>
#include <utility>
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

/* ---- certified binary32 endpoint walk ---------------------------------------------
 * The walk of dev_find_endpoint, taken in binary32 with error bounds the way
 * k_hull_walk_fast takes the hull walks: the state after a step depends only on
 * the axis crossed and the voxel indices, so a step whose decision (or exact
 * zero test) the bounds cannot certify is taken in binary64 from the rebuilt
 * binary64 state.  The slopes come from binary32 sincosf/tanf of the binary32
 * angle with a bound that covers the angle's rounding and a generous 16-ulp
 * allowance for the functions; the binary64 slopes (pct_tan, as the reference
 * computes them) are formed only for a binary64 step and for the hull point,
 * which is rebuilt in binary64 from the last crossing. */
enum { EAX_NONE = 0, EAX_X = 1, EAX_Y = 2, EAX_Z = 3 };
constexpr float EU = 1.2e-7f; /* twice the binary32 unit roundoff */

struct EpLine64 {
    double xs, ys, zs;
    double dy_dx, dz_dx, dz_dy, dx_dy, dx_dz, dy_dz, delta_yx;
    int xm, ym, zm;
};

__device__ __noinline__ void ep_slopes64(double xy_angle, double xz_angle, EpLine64& L) {
    double txy = pct_tan(xy_angle), txz = pct_tan(xz_angle);
    L.delta_yx = fabs(txy);
    L.dy_dx = txy;
    L.dz_dx = txz;
    L.dz_dy = txz / txy;
    L.dx_dy = 1.0 / txy;
    L.dx_dz = 1.0 / txz;
    L.dy_dz = txy / txz;
}

/* binary64 state after crossing axis a with indices (ax, ay, az), as the
 * loops of dev_find_endpoint compute it (zero-distance adjustments applied) */
__device__ __noinline__ void ep_state64(const DevGeom& g, const EpLine64& L, int a, int ax, int ay, int az, double z0,
                                        double zt0, double* x, double* y, double* z, double* xt, double* yt,
                                        double* zt, int* vx, int* vy, int* vz) {
    const bool is3d = L.zm != 0;
    *vx = ax;
    *vy = ay;
    *vz = az;
    if (a == EAX_NONE) {
        *x = L.xs;
        *y = L.ys;
        *z = L.zs;
        *xt = dev_distance_remaining(g.x_zero, *x, PCT_X_INC, L.xm, g.voxel_width, *vx);
        *yt = dev_distance_remaining(g.y_zero, *y, PCT_Y_INC, L.ym, g.voxel_height, *vy);
        *zt = dev_distance_remaining(g.z_zero, *z, PCT_Z_INC, L.zm, g.voxel_thickness, *vz);
        return;
    }
    if (is3d) {
        if (a == EAX_Z) {
            *z = dev_edge_coordinate(g.z_zero, *vz, g.voxel_thickness, PCT_Z_INC, L.zm);
            *x = dev_corresponding(L.dx_dz, *z, L.zs, L.xs);
            *y = dev_corresponding(L.dy_dz, *z, L.zs, L.ys);
            *xt = dev_distance_remaining(g.x_zero, *x, PCT_X_INC, L.xm, g.voxel_width, *vx);
            *yt = dev_distance_remaining(g.y_zero, *y, PCT_Y_INC, L.ym, g.voxel_height, *vy);
            *zt = g.voxel_thickness;
        } else if (a == EAX_X) {
            *x = dev_edge_coordinate(g.x_zero, *vx, g.voxel_width, PCT_X_INC, L.xm);
            *y = dev_corresponding(L.dy_dx, *x, L.xs, L.ys);
            *z = dev_corresponding(L.dz_dx, *x, L.xs, L.zs);
            *xt = g.voxel_width;
            *yt = dev_distance_remaining(g.y_zero, *y, PCT_Y_INC, L.ym, g.voxel_height, *vy);
            *zt = dev_distance_remaining(g.z_zero, *z, PCT_Z_INC, L.zm, g.voxel_thickness, *vz);
        } else {
            *y = dev_edge_coordinate(g.y_zero, *vy, g.voxel_height, PCT_Y_INC, L.ym);
            *x = dev_corresponding(L.dx_dy, *y, L.ys, L.xs);
            *z = dev_corresponding(L.dz_dy, *y, L.ys, L.zs);
            *xt = dev_distance_remaining(g.x_zero, *x, PCT_X_INC, L.xm, g.voxel_width, *vx);
            *yt = g.voxel_height;
            *zt = dev_distance_remaining(g.z_zero, *z, PCT_Z_INC, L.zm, g.voxel_thickness, *vz);
        }
        if (*xt == 0) { *xt = g.voxel_width; *vx += L.xm; }
        if (*yt == 0) { *yt = g.voxel_height; *vy -= L.ym; }
        if (*zt == 0) { *zt = g.voxel_thickness; *vz -= L.zm; }
        if (*vz < 0) *vz = 0;
    } else {
        *z = z0;
        *zt = zt0;
        if (a == EAX_X) {
            *x = dev_edge_coordinate(g.x_zero, *vx, g.voxel_width, PCT_X_INC, L.xm);
            *y = dev_corresponding(L.dy_dx, *x, L.xs, L.ys);
            *xt = g.voxel_width;
            *yt = dev_distance_remaining(g.y_zero, *y, PCT_Y_INC, L.ym, g.voxel_height, *vy);
        } else {
            /* the 2-D loop places the y edge with the z increment direction (.cu:5137) */
            *y = dev_edge_coordinate(g.y_zero, *vy, g.voxel_height, PCT_Z_INC, L.ym);
            *x = dev_corresponding(L.dx_dy, *y, L.ys, L.xs);
            *xt = dev_distance_remaining(g.x_zero, *x, PCT_X_INC, L.xm, g.voxel_width, *vx);
            *yt = g.voxel_height;
        }
        if (*xt == 0) { *xt = g.voxel_width; *vx += L.xm; }
        if (*yt == 0) { *yt = g.voxel_height; *vy -= L.ym; }
    }
}

/* binary32 slope and its absolute error bound */
struct Slope32 {
    float v, e;
};

__device__ __forceinline__ Slope32 sl_quot(Slope32 a, Slope32 b) {
    Slope32 r;
    r.v = a.v / b.v;
    float rel = (a.e / fabsf(a.v)) + (b.e / fabsf(b.v)) + EU;
    r.e = fabsf(r.v) * rel * 1.01f;
    if (!(r.e < 1e30f) || !(fabsf(r.v) < 1e30f)) r.e = 3.0e38f; /* unusable: every decision goes to binary64 */
    return r;
}

__device__ int dev_find_endpoint_fast(const DevGeom& g, const uint8_t* __restrict__ image, float xs_f, float ys_f,
                                      float zs_f, float xy_angle_f, float xz_angle_f, double* xo, double* yo,
                                      double* zo, int* vxo, int* vyo, int* vzo, int entering,
                                      unsigned long long* flags, unsigned long long* exact_steps) {
    const int C = g.columns, R = g.rows, S = g.slices;
    const int cap = 4 * (C + R + S) + 16;
    double xy_angle = xy_angle_f, xz_angle = xz_angle_f;
    if (!entering) xy_angle += PCT_PI;
    /* binary32 trigonometry with bounds */
    const float axy = (float)xy_angle, axz = (float)xz_angle;
    const float dxy = (float)fabs((double)axy - xy_angle), dxz = (float)fabs((double)axz - xz_angle);
    float sxy, cxy, sxz, cxz;
    sincosf(axy, &sxy, &cxy);
    sincosf(axz, &sxz, &cxz);
    const float e_sc_xy = dxy + 16.0f * EU, e_sc_xz = dxz + 16.0f * EU;
    EpLine64 L;
    L.xs = xs_f;
    L.ys = ys_f;
    L.zs = zs_f;
    bool have64 = false;
    /* direction signs: binary64 only when binary32 cannot tell */
    if (fabsf(cxy) > e_sc_xy) L.xm = cxy > 0 ? 1 : -1;
    else { double c = pct_cos(xy_angle); L.xm = (c >= 0) - (c <= 0); }
    if (fabsf(sxy) > e_sc_xy) L.ym = sxy > 0 ? 1 : -1;
    else { double sv = pct_sin(xy_angle); L.ym = (sv >= 0) - (sv <= 0); }
    if (fabsf(sxz) > e_sc_xz) L.zm = sxz > 0 ? 1 : -1;
    else { double sv = pct_sin(xz_angle); L.zm = (sv >= 0) - (sv <= 0); }
    if (L.xm < 0) L.zm *= -1;
    Slope32 txy, txz;
    txy.v = tanf(axy);
    txy.e = (1.0f + txy.v * txy.v) * (dxy + EU) + 16.0f * EU * fabsf(txy.v);
    txz.v = tanf(axz);
    txz.e = (1.0f + txz.v * txz.v) * (dxz + EU) + 16.0f * EU * fabsf(txz.v);
    if (!(fabsf(txy.v) < 1e30f) || !(txy.e < 1e30f)) txy.e = 3.0e38f;
    if (!(fabsf(txz.v) < 1e30f) || !(txz.e < 1e30f)) txz.e = 3.0e38f;
    const Slope32 one = {1.0f, 0.0f};
    const Slope32 dy_dx = txy, dz_dx = txz, dz_dy = sl_quot(txz, txy), dx_dy = sl_quot(one, txy),
                  dx_dz = sl_quot(one, txz), dy_dz = sl_quot(txy, txz);
    /* start */
    int vx = dev_calculate_voxel(g.x_zero, L.xs, g.voxel_width);
    int vy = dev_calculate_voxel(g.y_zero, L.ys, g.voxel_height);
    int vz = dev_calculate_voxel(g.z_zero, L.zs, g.voxel_thickness);
    double x64, y64, z64, xt64, yt64, zt64;
    ep_state64(g, L, EAX_NONE, vx, vy, vz, 0.0, 0.0, &x64, &y64, &z64, &xt64, &yt64, &zt64, &vx, &vy, &vz);
    const double z_init = z64, zt_init = zt64;
    float x = (float)x64, y = (float)y64, z = (float)z64, xt = (float)xt64, yt = (float)yt64, zt = (float)zt64;
    float ex = EU * fabsf(x), ey = EU * fabsf(y), ez = EU * fabsf(z), ext = EU * xt, eyt = EU * yt, ezt = EU * zt;
    int a_axis = EAX_NONE, ax = vx, ay = vy, az = vz;
    const float X0 = g.fx0, Y0 = g.fy0, Z0 = g.fz0;
    const float VW = g.fvw, VH = g.fvh, VT = g.fvt;
    const float xs = xs_f, ys = ys_f, zs = zs_f;
    int voxel = vx + vy * C + vz * C * R;
    int outside = (vx >= C) || (vy >= R) || (vz >= S) || (vx < 0) || (vy < 0) || (vz < 0);
    int hit = outside ? 0 : (image[voxel] == 1);
    int end = outside || hit;
    int steps = 0;
    const bool is3d = L.zm != 0;
    while (!end) {
        if (++steps > cap) {
            dev_flag(flags, ERR_WALK_CAPPED);
            break;
        }
        int axis = -1;
        if (is3d) {
            float x_ext = fabsf(dz_dx.v) * xt, e_xe = fabsf(dz_dx.v) * ext + dz_dx.e * xt + EU * x_ext;
            float y_ext = fabsf(dz_dy.v) * yt, e_ye = fabsf(dz_dy.v) * eyt + dz_dy.e * yt + EU * y_ext;
            int c1 = cmp_le(zt, ezt, x_ext, e_xe), c2 = cmp_le(zt, ezt, y_ext, e_ye);
            if (c1 >= 0 && c2 >= 0) {
                if (c1 && c2) axis = EAX_Z;
                else {
                    int c3 = cmp_le(x_ext, e_xe, y_ext, e_ye);
                    if (c3 >= 0) axis = c3 ? EAX_X : EAX_Y;
                }
            }
        } else {
            float dyx = fabsf(txy.v);
            float y_ext = yt / dyx;
            float e_ye = (eyt + yt * txy.e / dyx) / dyx + EU * y_ext;
            if (!(e_ye < 1e30f)) e_ye = 3.0e38f;
            int c = cmp_le(xt, ext, y_ext, e_ye);
            if (c >= 0) axis = c ? EAX_X : EAX_Y;
        }
        bool ok = axis >= 0;
        int nx = vx, ny = vy, nz = vz;
        float n_x = x, n_y = y, n_z = z, n_xt = xt, n_yt = yt, n_zt = zt;
        float n_ex = ex, n_ey = ey, n_ez = ez, n_ext = ext, n_eyt = eyt, n_ezt = ezt;
        if (ok) {
            float ee, e_edge;
            if (axis == EAX_X) {
                nx += L.xm;
                n_x = edge32(X0, nx, VW, PCT_X_INC, L.xm, &n_ex);
                n_y = corr32(dy_dx.v, n_x, xs, ys, n_ex, &n_ey);
                n_ey += dy_dx.e * fabsf(n_x - xs);
                n_xt = VW;
                n_ext = EU * VW;
                float ye = edge32(Y0, ny + PCT_Y_INC * L.ym, VH, PCT_Y_INC, L.ym, &ee);
                n_yt = fabsf(ye - n_y);
                n_eyt = ee + n_ey + EU * n_yt;
                if (is3d) {
                    n_z = corr32(dz_dx.v, n_x, xs, zs, n_ex, &n_ez);
                    n_ez += dz_dx.e * fabsf(n_x - xs);
                    float ze = edge32(Z0, nz + PCT_Z_INC * L.zm, VT, PCT_Z_INC, L.zm, &e_edge);
                    n_zt = fabsf(ze - n_z);
                    n_ezt = e_edge + n_ez + EU * n_zt;
                }
            } else if (axis == EAX_Y) {
                ny -= L.ym;
                n_y = edge32(Y0, ny, VH, is3d ? PCT_Y_INC : PCT_Z_INC, L.ym, &n_ey);
                n_x = corr32(dx_dy.v, n_y, ys, xs, n_ey, &n_ex);
                n_ex += dx_dy.e * fabsf(n_y - ys);
                float xe = edge32(X0, nx + PCT_X_INC * L.xm, VW, PCT_X_INC, L.xm, &e_edge);
                n_xt = fabsf(xe - n_x);
                n_ext = e_edge + n_ex + EU * n_xt;
                n_yt = VH;
                n_eyt = EU * VH;
                if (is3d) {
                    n_z = corr32(dz_dy.v, n_y, ys, zs, n_ey, &n_ez);
                    n_ez += dz_dy.e * fabsf(n_y - ys);
                    float ze = edge32(Z0, nz + PCT_Z_INC * L.zm, VT, PCT_Z_INC, L.zm, &e_edge);
                    n_zt = fabsf(ze - n_z);
                    n_ezt = e_edge + n_ez + EU * n_zt;
                }
            } else {
                nz -= L.zm;
                n_z = edge32(Z0, nz, VT, PCT_Z_INC, L.zm, &n_ez);
                n_x = corr32(dx_dz.v, n_z, zs, xs, n_ez, &n_ex);
                n_ex += dx_dz.e * fabsf(n_z - zs);
                n_y = corr32(dy_dz.v, n_z, zs, ys, n_ez, &n_ey);
                n_ey += dy_dz.e * fabsf(n_z - zs);
                float xe = edge32(X0, nx + PCT_X_INC * L.xm, VW, PCT_X_INC, L.xm, &e_edge);
                n_xt = fabsf(xe - n_x);
                n_ext = e_edge + n_ex + EU * n_xt;
                float ye = edge32(Y0, ny + PCT_Y_INC * L.ym, VH, PCT_Y_INC, L.ym, &e_edge);
                n_yt = fabsf(ye - n_y);
                n_eyt = e_edge + n_ey + EU * n_yt;
                n_zt = VT;
                n_ezt = EU * VT;
            }
            /* the exact-zero distance tests and the bounds themselves must be usable */
            if (n_xt <= n_ext || n_yt <= n_eyt || (is3d && n_zt <= n_ezt)) ok = false;
            if (!(n_ext < 1e-3f && n_eyt < 1e-3f && (!is3d || n_ezt < 1e-3f))) ok = false;
        }
        if (ok) {
            a_axis = axis;
            ax = nx;
            ay = ny;
            az = nz;
            if (is3d && nz < 0) nz = 0;
            vx = nx; vy = ny; vz = nz;
            x = n_x; y = n_y; z = n_z; xt = n_xt; yt = n_yt; zt = n_zt;
            ex = n_ex; ey = n_ey; ez = n_ez; ext = n_ext; eyt = n_eyt; ezt = n_ezt;
        } else {
            /* binary64 step from the binary64 state of the last crossing */
            if (!have64) {
                ep_slopes64(xy_angle, xz_angle, L);
                have64 = true;
            }
            int bx, by, bz;
            ep_state64(g, L, a_axis, ax, ay, az, z_init, zt_init, &x64, &y64, &z64, &xt64, &yt64, &zt64, &bx, &by, &bz);
            int ax64;
            if (is3d) {
                double x_ext = fabs(L.dz_dx) * xt64, y_ext = fabs(L.dz_dy) * yt64;
                if ((zt64 <= x_ext) && (zt64 <= y_ext)) ax64 = EAX_Z;
                else ax64 = x_ext <= y_ext ? EAX_X : EAX_Y;
            } else {
                ax64 = xt64 <= yt64 / L.delta_yx ? EAX_X : EAX_Y;
            }
            if (ax64 == EAX_X) bx += L.xm;
            else if (ax64 == EAX_Y) by -= L.ym;
            else bz -= L.zm;
            a_axis = ax64;
            ax = bx;
            ay = by;
            az = bz;
            ep_state64(g, L, a_axis, ax, ay, az, z_init, zt_init, &x64, &y64, &z64, &xt64, &yt64, &zt64, &vx, &vy, &vz);
            x = (float)x64; y = (float)y64; z = (float)z64; xt = (float)xt64; yt = (float)yt64; zt = (float)zt64;
            ex = EU * fabsf(x); ey = EU * fabsf(y); ez = EU * fabsf(z);
            ext = EU * xt; eyt = EU * yt; ezt = EU * zt;
            ++*exact_steps;
        }
        voxel = vx + vy * C + vz * C * R;
        outside = (vx >= C) || (vy >= R) || (vz >= S) || (vx < 0) || (vy < 0) || (vz < 0);
        if (!outside) hit = (image[voxel] == 1);
        end = outside || hit;
    }
    if (hit) {
        /* the hull point in binary64, rebuilt from the last crossing */
        if (!have64) ep_slopes64(xy_angle, xz_angle, L);
        int bx, by, bz;
        ep_state64(g, L, a_axis, ax, ay, az, z_init, zt_init, &x64, &y64, &z64, &xt64, &yt64, &zt64, &bx, &by, &bz);
        *xo = x64;
        *yo = y64;
        *zo = z64;
    }
    *vxo = vx;
    *vyo = vy;
    *vzo = vz;
    return hit;
}

/* Launch-order key of the endpoint walks: the distance of the history's line
 * from the cylinder axis in the xy plane (walks from the cylinder to the hull
 * have about the same length at the same distance), in 1/1000 of the radius. */
__global__ void k_endpoint_key(DevGeom g, int64_t n, HistView h, uint32_t* __restrict__ key) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float xe = h.x_entry[i], ye = h.y_entry[i], xx = h.x_exit[i], yx = h.y_exit[i];
    const float dx = xx - xe, dy = yx - ye;
    const float len = sqrtf(dx * dx + dy * dy);
    const float d = len > 0.0f ? fabsf(xe * yx - xx * ye) / len : 0.0f;
    const float q = d * (1000.0f / (float)g.recon_cyl_radius);
    key[i] = q < 1.0e6f ? 1u + (uint32_t)q : 1000000u;
}

__global__ void __launch_bounds__(128) k_endpoints_fast(DevGeom g, int64_t n, const uint32_t* __restrict__ order,
                                                        const uint8_t* __restrict__ hull, HistView h,
                                                        uint8_t* __restrict__ keep,
                                                        unsigned long long* __restrict__ flags) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (order) i = order[i];
    double xi = 0, yi = 0, zi = 0, xo = 0, yo = 0, zo = 0;
    int vx = 0, vy = 0, vz = 0, vx2 = 0, vy2 = 0, vz2 = 0;
    unsigned long long exact = 0;
    int entered = dev_find_endpoint_fast(g, hull, h.x_entry[i], h.y_entry[i], h.z_entry[i], h.xy_entry_angle[i],
                                         h.xz_entry_angle[i], &xi, &yi, &zi, &vx, &vy, &vz, 1, flags, &exact);
    int exited = dev_find_endpoint_fast(g, hull, h.x_exit[i], h.y_exit[i], h.z_exit[i], h.xy_exit_angle[i],
                                        h.xz_exit_angle[i], &xo, &yo, &zo, &vx2, &vy2, &vz2, 0, flags, &exact);
    int both = entered && exited;
    keep[i] = (uint8_t)both;
    h.first_voxel[i] = both ? (uint32_t)(vx + g.columns * vy + g.rows * g.columns * vz) : 0u;
    if (both) {
        h.x_entry[i] = (float)xi; h.y_entry[i] = (float)yi; h.z_entry[i] = (float)zi;
        h.x_exit[i] = (float)xo; h.y_exit[i] = (float)yo; h.z_exit[i] = (float)zo;
    }
    if (exact) atomicAdd(flags + ERR_WALK_FP64, exact);
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
    /* The reference turns the entry direction by pi when u_in > u_out.  That
     * comparison is made in binary32 when its margin is wide (then only the
     * kept direction's binary64 sine and cosine are formed), else as the
     * reference makes it. */
    const float dxf = (float)(x_in - x_out), dyf = (float)(y_in - y_out);
    float sf, cf;
    sincosf((float)xy_entry, &sf, &cf);
    const float duf = cf * dxf + sf * dyf; /* u_in - u_out */
    const float tol = 1e-4f * (fabsf(dxf) + fabsf(dyf)) + 1e-5f;
    int flip;
    double ce, se;
    if (duf > tol || duf < -tol) {
        flip = duf > 0.0f;
        if (flip) {
            xy_entry += PCT_PI;
            xy_exit += PCT_PI;
        }
        pct_sincos(xy_entry, &se, &ce);
    } else {
        pct_sincos(xy_entry, &se, &ce);
        flip = ((ce * x_in) + (se * y_in)) > ((ce * x_out) + (se * y_out));
        if (flip) {
            xy_entry += PCT_PI;
            xy_exit += PCT_PI;
            pct_sincos(xy_entry, &se, &ce);
        }
    }
    double u_in = (ce * x_in) + (se * y_in);
    double u_out = (ce * x_out) + (se * y_out);
    double t_in = (ce * y_in) - (se * x_in);
    double t_out = (ce * y_out) - (se * x_out);
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

/* The terms of an MLP sample that depend on its depth u_1 alone (the entry
 * side Sigma_1^-1 and the exit side's polynomials in u_1), binary64. */
struct MlpDepthTerms {
    double S1I0, S1I1, S1I3, cst1, cst2, cst3;
};

__device__ __forceinline__ void dev_mlp_depth_terms(double u_1, MlpDepthTerms& t) {
    const double u_0 = 0.0;
    double k1 = PCT_E_0 * (1 + 0.038 * pct_log((u_1 - u_0) / PCT_X_0));
    double c1 = k1 * k1 / PCT_X_0;
    double st1 = c1 * (pct_cube(u_1) * (AL(0, 3) + u_1 * (AL(1, 12) + u_1 * (AL(2, 30) + u_1 * (AL(3, 60) + u_1 * (AL(4, 105) + AU(u_1, 5, 168)))))));
    double stt1 = c1 * ((u_1 * u_1) * (AL(0, 2) + u_1 * (AL(1, 6) + u_1 * (AL(2, 12) + u_1 * (AL(3, 20) + u_1 * (AL(4, 30) + AU(u_1, 5, 42)))))));
    double sth1 = c1 * (u_1 * (A0 + u_1 * (AL(1, 2) + u_1 * (AL(2, 3) + u_1 * (AL(3, 4) + u_1 * (AL(4, 5) + AU(u_1, 5, 6)))))));
    double det1 = st1 * sth1 - stt1 * stt1;
    t.S1I0 = sth1 / det1;
    t.S1I1 = -stt1 / det1; /* = S1I2 */
    t.S1I3 = st1 / det1;
    t.cst1 = u_1 * (A0 + u_1 * (AL(1, 2) + u_1 * (AL(2, 3) + u_1 * (AL(3, 4) + u_1 * (AL(4, 5) + AU(u_1, 5, 6))))));
    t.cst2 = (u_1 * u_1) * (AL(0, 2) + u_1 * (AL(1, 3) + u_1 * (AL(2, 4) + u_1 * (AL(3, 5) + u_1 * (AL(4, 6) + AU(u_1, 5, 7))))));
    t.cst3 = pct_cube(u_1) * (AL(0, 3) + u_1 * (AL(1, 4) + u_1 * (AL(2, 5) + u_1 * (AL(3, 6) + u_1 * (AL(4, 7) + AU(u_1, 5, 8))))));
}

/* One MLP sample at depth u_1 in binary64, the reference's operation order,
 * from its depth terms. */
__device__ __forceinline__ int dev_mlp_voxel_terms(const DevGeom& g, const MlpSetup& m, double u_1,
                                                   const MlpDepthTerms& t) {
    const double u_2 = m.u_2;
    double R0_1 = u_1, R1_1 = u_2 - u_1, R1T_2 = u_2 - u_1;
    const double R0_0 = 1.0, R0_2 = 0.0, R0_3 = 1.0, R1_0 = 1.0, R1_2 = 0.0, R1_3 = 1.0;
    const double R1T_0 = 1.0, R1T_1 = 0.0, R1T_3 = 1.0;
    const double S1I0 = t.S1I0, S1I1 = t.S1I1, S1I2 = t.S1I1, S1I3 = t.S1I3;
    const double cst1 = t.cst1, cst2 = t.cst2, cst3 = t.cst3;
    double k2 = PCT_E_0 * (1 + 0.038 * pct_log((u_2 - u_1) / PCT_X_0));
    double c2 = k2 * k2 / PCT_X_0;
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

__device__ __forceinline__ int dev_mlp_voxel(const DevGeom& g, const MlpSetup& m, double u_1) {
    MlpDepthTerms t;
    dev_mlp_depth_terms(u_1, t);
    return dev_mlp_voxel_terms(g, m, u_1, t);
}

/* ---- binary32 fast path ------------------------------------------------------
 * With s = u_2 - u the scattering moments of the exit side are polynomials in
 * d = u_2 - u_1 with positive weights (no cancellation):
 *   f(u_2 - s) = sum_m b_m s^m,  Q_j = sum_m b_m d^m / (m + j),
 *   Sigma_2 = c_2 [[d^3 Q_3, d^2 Q_2], [d^2 Q_2, d Q_1]],
 * and since the MLP of a straight line is the line,
 *   t_1 = t_in + beta (t_out - t_in) + gamma (theta_out - theta_in),
 * so binary32 only carries the deflection from the entry line.  The binary32
 * result is within 4e-6 cm of the binary64 reference over 6.6e7 sampled MLP
 * points; a sample whose x, y or z lies closer than mlp_face_margin to a voxel
 * face is recomputed with the reference's binary64 expression
 * (dev_mlp_voxel), so the voxel rows are those of the binary64 algorithm. */
struct MlpTableEntry {
    double u1;          /* u_1 after k steps of u_1 += MLP_U_STEP, as the reference accumulates it */
    float u1_hi, u1_lo; /* u1 as a float pair */
    float s1i0, s1i1, s1i3; /* Sigma_1^-1 at u_1 (binary64, rounded) */
    float pad;
};

__global__ void k_mlp_u1(double step, int K, MlpTableEntry* __restrict__ tab) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double u = step;
        for (int k = 0; k < K; ++k) {
            tab[k].u1 = u;
            u += step;
        }
    }
}

/* Per sample index k: the binary32 entry and the binary64 depth terms (for the
 * samples recomputed in binary64 by k_mlp_fix). */
__global__ void k_mlp_table(int K, MlpTableEntry* __restrict__ tab, MlpDepthTerms* __restrict__ terms) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    double u_1 = tab[k].u1;
    MlpDepthTerms t;
    dev_mlp_depth_terms(u_1, t);
    terms[k] = t;
    tab[k].s1i0 = (float)t.S1I0;
    tab[k].s1i1 = (float)t.S1I1;
    tab[k].s1i3 = (float)t.S1I3;
    float hi = (float)u_1;
    tab[k].u1_hi = hi;
    tab[k].u1_lo = (float)(u_1 - (double)hi);
    tab[k].pad = 0.0f;
}

/* Samples of history i: u_1 = tab[k].u1 for k < K with u_1 < u_2 - step (.cu:5376). */
__device__ __forceinline__ int dev_sample_count(const MlpTableEntry* __restrict__ tab, int kmax, double u_2, double step) {
    double lim = u_2 - step;
    int lo = 0, hi = kmax; /* first k with u1 >= lim */
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (tab[mid].u1 < lim) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* Per-history MLP constants: the binary64 setup (for the binary64 samples)
 * and the binary32 Taylor coefficients b_m of the scattering power. */
struct __align__(16) MlpRec {
    MlpSetup m;   /* 104 bytes */
    float b[6];
};
static_assert(sizeof(MlpRec) == 128, "MlpRec layout");

/* A sample whose voxel the binary32 path cannot certify: recomputed in
 * binary64 by k_mlp_fix, one thread per sample. */
struct MlpDeferred {
    int64_t pos;   /* entry of the row slot holding the sample's voxel */
    int64_t hist;
    int k;
    int pad;
};

__global__ void __launch_bounds__(256) k_mlp_bound(DevGeom g, int64_t n, HistView h,
                                                   const MlpTableEntry* __restrict__ tab, int kmax,
                                                   int64_t* __restrict__ bound, MlpRec* __restrict__ rec) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    MlpRec r;
    dev_mlp_setup(h, i, r.m);
    bound[i] = (int64_t)dev_sample_count(tab, kmax, r.m.u_2, g.mlp_u_step) + 1;
    /* Taylor coefficients of the scattering power around u_2 (binary64, then float) */
    const double A[6] = {A0, PCT_A1_M * PCT_A1_P, PCT_A2_M * PCT_A2_P, PCT_A3_M * PCT_A3_P, PCT_A4_M * PCT_A4_P,
                         PCT_A5_M * PCT_A5_P};
    /* the shift to u_2 by repeated synthetic division: afterwards
     * c[mm] = sum_k C(k, mm) A_k u_2^(k - mm) */
    double c[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) c[k] = A[k];
#pragma unroll
    for (int mm = 0; mm < 5; ++mm)
#pragma unroll
        for (int k = 4; k >= mm; --k) c[k] = fma(r.m.u_2, c[k + 1], c[k]);
#pragma unroll
    for (int mm = 0; mm < 6; ++mm) r.b[mm] = (float)((mm & 1) ? -c[mm] : c[mm]);
    rec[i] = r;
}

/* dev_mlp_voxel out of line, for the rare binary64 samples of k_mlp_fast (keeps
 * the binary32 loop's register footprint small). */
__device__ __noinline__ uint32_t dev_mlp_voxel_rec(DevGeom g, const MlpRec* __restrict__ r, double u_1) {
    MlpSetup m = r->m;
    return (uint32_t)dev_mlp_voxel(g, m, u_1);
}

/* Classification of one binary32 sample. */
enum { SAMPLE_CERTAIN = 0, SAMPLE_PAIR = 1, SAMPLE_EXACT = 2 };

struct MlpSample {
    int state;
    uint32_t v;      /* CERTAIN: the voxel; PAIR: one candidate */
    uint32_t v_alt;  /* PAIR: the candidate across the near face */
};

/* Voxel index along one axis from a binary32 coordinate; *amb is -1 / +1 when
 * the coordinate lies within the face margin of the lower / upper face of that
 * voxel (fractional position below flo / above fhi). */
__device__ __forceinline__ int axis_index(float pos, float zero, float inv_size, float flo, float fhi, int* amb) {
    float q = fabsf(pos - zero) * inv_size;
    int i0 = (int)q;
    float fr = q - (float)i0;
    *amb = fr < flo ? -1 : (fr > fhi ? 1 : 0);
    return i0;
}

/* The row entry of voxel (vx, vy, vz) in the rows' voxel order: the brick
 * index formed directly inside the grid; outside it the reference's linear
 * index vx + vy C + vz C R (which wraps into a neighbouring row or slice),
 * mapped as every other linear index is. */
__device__ __forceinline__ uint32_t row_entry(const DevGeom& g, int vx, int vy, int vz) {
    if (g.brick && (unsigned)vx < (unsigned)g.columns && (unsigned)vy < (unsigned)g.rows &&
        (unsigned)vz < (unsigned)g.slices)
        return dev_brick_xyz((uint32_t)g.columns, (uint32_t)g.rows, (uint32_t)vx, (uint32_t)vy, (uint32_t)vz);
    return dev_to_brick(g, (uint32_t)(vx + vy * g.columns + vz * g.columns * g.rows));
}

struct MlpFast {
    float b[6];
    float u2_hi, u2_lo, dT, dV, T21, V21, cef, sef, x_in, y_in, V0;
};

__device__ __forceinline__ MlpSample dev_mlp_sample(const DevGeom& g, const MlpFast& f, const MlpTableEntry te) {
    const float X0 = g.fx0, Y0 = g.fy0, Z0 = g.fz0;
    const float iVW = g.fivw, iVH = g.fivh, iVT = g.fivt;
    const float* b = f.b;
    float d = (f.u2_hi - te.u1_hi) + (f.u2_lo - te.u1_lo);
    /* k2 / sqrt(X0) = (E0 / sqrt(X0)) (1 + 0.038 ln(d / X0)) with E0 = 13.6 MeV and
     * X0 = 36.08 cm, as one FMA on log2(d): KA = (E0 / sqrt(X0)) 0.038 ln 2,
     * KB = (E0 / sqrt(X0)) (1 - 0.038 ln X0), evaluated in binary64 */
    constexpr float KA = 5.963685076e-02f;
    constexpr float KB = 1.955643309e+00f;
    const float ks = fmaf(KA, __log2f(d), KB);
    float c2 = ks * ks;
    /* the terms p_m = b_m d^m once, then each moment as a fixed-weight sum of them */
    const float d2 = d * d, d3 = d2 * d, d4 = d2 * d2, d5 = d4 * d;
    const float p0 = b[0], p1 = b[1] * d, p2 = b[2] * d2, p3 = b[3] * d3, p4 = b[4] * d4, p5 = b[5] * d5;
#define PCT_WSUM(w0, w1, w2, w3, w4, w5) \
    fmaf(p5, (w5), fmaf(p4, (w4), fmaf(p3, (w3), fmaf(p2, (w2), fmaf(p1, (w1), p0 * (w0))))))
    float Q1 = PCT_WSUM(1.0f, 1.0f / 2, 1.0f / 3, 1.0f / 4, 1.0f / 5, 1.0f / 6);
    float Q2 = PCT_WSUM(1.0f / 2, 1.0f / 3, 1.0f / 4, 1.0f / 5, 1.0f / 6, 1.0f / 7);
    float Q3 = PCT_WSUM(1.0f / 3, 1.0f / 4, 1.0f / 5, 1.0f / 6, 1.0f / 7, 1.0f / 8);
    /* E1 = Q1 - Q2 (weights 1/((m+1)(m+2))), E2 = Q1 - 2 Q2 + Q3, E3 = Q2 - Q3, each summed directly */
    float E1 = PCT_WSUM(1.0f / 2, 1.0f / 6, 1.0f / 12, 1.0f / 20, 1.0f / 30, 1.0f / 42);
    float E2 = PCT_WSUM(2.0f / 6, 2.0f / 24, 2.0f / 60, 2.0f / 120, 2.0f / 210, 2.0f / 336);
    float E3 = PCT_WSUM(1.0f / 6, 1.0f / 12, 1.0f / 20, 1.0f / 30, 1.0f / 42, 1.0f / 56);
#undef PCT_WSUM
    float D = fmaf(Q3, Q1, -Q2 * Q2);
    /* approximate reciprocals (2 ulp): far inside the face margin that certifies each voxel */
    float inv = __fdividef(1.0f, c2 * D);
    float id = __fdividef(1.0f, d);
    float i1 = inv * id, i2 = i1 * id, i3 = i2 * id; /* inv / d^k */
    float Aa = Q1 * i3;      /* (Sigma_2^-1)_00 */
    float Bm = E1 * i2;      /* (R1^T Sigma_2^-1 R1)_01 */
    float Cm = E2 * i1;      /* (R1^T Sigma_2^-1 R1)_11 */
    float bb = -Q2 * i2;     /* (Sigma_2^-1)_01 */
    float e3 = -E3 * i1;     /* d (Sigma_2^-1)_01 + (Sigma_2^-1)_11 */
    float ft0 = te.s1i0 + Aa, ft1 = te.s1i1 + Bm, ft3 = te.s1i3 + Cm;
    float idet = __fdividef(1.0f, fmaf(ft0, ft3, -ft1 * ft1));
    float beta = fmaf(ft3, Aa, -ft1 * Bm) * idet;
    float gam = fmaf(ft3, bb, -ft1 * e3) * idet;
    float ct = fmaf(beta, f.dT, gam * f.T21);
    float cv = fmaf(beta, f.dV, gam * f.V21);
    float u1f = te.u1_hi;
    float x1 = f.x_in + fmaf(f.cef, u1f, -f.sef * ct);
    float y1 = f.y_in + fmaf(f.sef, u1f, f.cef * ct);
    float z1 = f.V0 + cv;
    MlpSample s;
    s.v = s.v_alt = 0;
    if (!(fabsf(ct) < 1e3f) || !(fabsf(cv) < 1e3f)) {
        s.state = SAMPLE_EXACT;
        return s;
    }
    int ax, ay, az;
    int vx = axis_index(x1, X0, iVW, g.fmlo_x, g.fmhi_x, &ax);
    int vy = axis_index(y1, Y0, iVH, g.fmlo_y, g.fmhi_y, &ay);
    int vz = axis_index(z1, Z0, iVT, g.fmlo_z, g.fmhi_z, &az);
    s.v = row_entry(g, vx, vy, vz); /* voxels as row entries (the rows' voxel order) */
    int namb = (ax != 0) + (ay != 0) + (az != 0);
    if (namb == 0) {
        s.state = SAMPLE_CERTAIN;
    } else if (namb == 1) {
        s.state = SAMPLE_PAIR;
        s.v_alt = row_entry(g, vx + ax, vy + ay, vz + az);
    } else {
        s.state = SAMPLE_EXACT;
    }
    return s;
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

/* The row's chord length (bf16: rounded to bfloat16, nearest even); out of
 * line so that its binary64 code stays out of the callers' register budget. */
__device__ __noinline__ float dev_row_chord(const DevGeom& g, const HistView& h, int64_t i, int bf16) {
    const double ae = h.xy_entry_angle[i], ax = h.xy_exit_angle[i], ze = h.xz_entry_angle[i], zx = h.xz_exit_angle[i];
    double c = dev_chord(g, (ae + ax) / 2.0, (ze + zx) / 2.0);
    if (bf16) c = (double)__bfloat162float(__float2bfloat16_rn((float)c));
    return (float)c;
}

/* 1 / (c |a_i|) with |a_i| the row length: lambda res c / ||a_i||^2 = lambda res row_scale */
__device__ __forceinline__ float dev_row_scale(float chord, int len) { return (float)(1.0 / ((double)chord * (double)len)); }

/* Fills the row slot of each history.  A sample within `margin` of a voxel
 * face has two candidate voxels; when they are exactly the previous row entry
 * and the (certain) next sample's voxel, either choice gives the same row
 * after consecutive repeats are dropped, so the sample is skipped.  Any other
 * uncertain sample gets a placeholder entry, is queued for k_mlp_fix, and the
 * next sample is written unconditionally; k_mlp_dedupe then drops the repeats
 * around the resolved entries.  With exact != 0 every sample is binary64. */
__global__ void __launch_bounds__(128, 5) k_mlp_fast(DevGeom g, int64_t n, const uint32_t* __restrict__ order,
                                                  HistView h, int bf16, float* __restrict__ chord,
                                                  float* __restrict__ row_scale,
                                                  const MlpRec* __restrict__ rec,
                                                  const uint32_t* __restrict__ first_voxel,
                                                  const float* __restrict__ x_entry, const float* __restrict__ y_entry,
                                                  const MlpTableEntry* __restrict__ tab,
                                                  const int64_t* __restrict__ bound, int exact, const int64_t* __restrict__ row_start,
                                                  uint32_t* __restrict__ rows, int* __restrict__ row_len,
                                                  MlpDeferred* __restrict__ queue, int64_t queue_cap,
                                                  int64_t* __restrict__ fix_rows,
                                                  unsigned long long* __restrict__ flags) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (order) i = order[i];
    /* the row's chord in binary64 (EffectiveChordLength_GPU): its FP64 work
     * overlaps the other warps' binary32 samples */
    const float cf = dev_row_chord(g, h, i, bf16);
    chord[i] = cf;
    const MlpRec& R = rec[i];
    const double u_2 = R.m.u_2;
    const int K = (int)(bound[i] - 1); /* dev_sample_count, stored by k_mlp_bound */
    const uint32_t nv = (uint32_t)g.num_voxels;
    int64_t out = row_start[i];
    int len = 0;
    uint32_t prev = dev_to_brick(g, first_voxel[i]); /* row entries: the rows' voxel order */
    rows[out + len++] = prev;
    int fp64_samples = 0, deferred = 0, outside = prev >= nv;
    int first_def = 0, outside_pre = 0; /* entry of the first placeholder, outside entries before it */
    if (exact) {
        for (int k = 0; k < K; ++k) {
            uint32_t v = dev_to_brick(g, dev_mlp_voxel_rec(g, &R, tab[k].u1));
            ++fp64_samples;
            if (v != prev) {
                rows[out + len++] = v;
                prev = v;
                outside += v >= nv;
            }
        }
    } else {
        MlpFast f;
#pragma unroll
        for (int mm = 0; mm < 6; ++mm) f.b[mm] = R.b[mm];
        f.u2_hi = (float)u_2;
        f.u2_lo = (float)(u_2 - (double)f.u2_hi);
        f.dT = (float)(R.m.T20 - R.m.T0);
        f.dV = (float)(R.m.V20 - R.m.V0);
        f.T21 = (float)R.m.T21;
        f.V21 = (float)R.m.V21;
        f.cef = (float)R.m.ce;
        f.sef = (float)R.m.se;
        f.x_in = x_entry[i];
        f.y_in = y_entry[i];
        f.V0 = (float)R.m.V0;
        int force = 0; /* the last entry is a placeholder: write the next voxel whatever it is */
        MlpSample cur = K > 0 ? dev_mlp_sample(g, f, tab[0]) : MlpSample{SAMPLE_CERTAIN, 0u, 0u};
        for (int k = 0; k < K; ++k) {
            MlpSample nxt{SAMPLE_EXACT, 0u, 0u};
            if (k + 1 < K) nxt = dev_mlp_sample(g, f, tab[k + 1]);
            if (cur.state == SAMPLE_CERTAIN) {
                if (force || cur.v != prev) {
                    rows[out + len++] = cur.v;
                    prev = cur.v;
                    outside += cur.v >= nv;
                    force = 0;
                }
            } else if (cur.state == SAMPLE_PAIR && !force && nxt.state == SAMPLE_CERTAIN &&
                       ((cur.v == prev && cur.v_alt == nxt.v) || (cur.v_alt == prev && cur.v == nxt.v))) {
                /* either candidate drops out with the repeats */
            } else {
                ++fp64_samples;
                unsigned long long slot = atomicAdd(flags + ERR_MLP_QUEUED, 1ull);
                if ((int64_t)slot < queue_cap) {
                    if (!deferred) {
                        first_def = len;
                        outside_pre = outside;
                    }
                    MlpDeferred q;
                    q.pos = out + len;
                    q.hist = i;
                    q.k = k;
                    q.pad = 0;
                    queue[slot] = q;
                    rows[out + len++] = 0u;
                    ++deferred;
                    force = 1;
                } else {
                    /* queue full: binary64 here */
                    uint32_t v = dev_to_brick(g, dev_mlp_voxel_rec(g, &R, tab[k].u1));
                    if (force || v != prev) {
                        rows[out + len++] = v;
                        prev = v;
                        outside += v >= nv;
                        force = 0;
                    }
                }
            }
            cur = nxt;
        }
    }
    row_len[i] = len;
    if (!deferred) row_scale[i] = dev_row_scale(cf, len); /* rows with recomputed samples: k_mlp_dedupe */
    if (deferred) {
        unsigned long long r = atomicAdd(flags + ERR_MLP_FIXROWS, 1ull);
        fix_rows[r] = i | ((int64_t)first_def << 40); /* at most one entry per row: r < n */
        if (outside_pre) atomicAdd(flags + ERR_ROWS_OUTSIDE, (unsigned long long)outside_pre);
    } else if (outside) {
        atomicAdd(flags + ERR_ROWS_OUTSIDE, (unsigned long long)outside);
    }
    if (fp64_samples) atomicAdd(flags + ERR_MLP_FP64, (unsigned long long)fp64_samples);
}

/* The queued samples in binary64, one thread each. */
__global__ void __launch_bounds__(128) k_mlp_fix(DevGeom g, const MlpRec* __restrict__ rec,
                                                 const MlpTableEntry* __restrict__ tab,
                                                 const MlpDepthTerms* __restrict__ terms,
                                                 const MlpDeferred* __restrict__ queue, int64_t queue_cap,
                                                 const unsigned long long* __restrict__ flags,
                                                 uint32_t* __restrict__ rows) {
    int64_t count = (int64_t)flags[ERR_MLP_QUEUED];
    if (count > queue_cap) count = queue_cap;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x) {
        MlpDeferred d = queue[q];
        MlpSetup m = rec[d.hist].m;
        /* the depth terms of sample d.k come from the table: the same binary64 values */
        rows[d.pos] = dev_to_brick(g, (uint32_t)dev_mlp_voxel_terms(g, m, tab[d.k].u1, terms[d.k]));
    }
}

/* Drops consecutive repeats in the rows that had queued samples, one warp per
 * row, from the row's first placeholder on (fix_rows holds the history in its
 * low 40 bits and that entry above them; the entries before it are final and
 * their outside-the-grid count is already recorded).  An entry is kept when
 * it differs from the entry before it (the last kept value always equals that
 * entry), and kept entries are compacted in place: each 32-entry chunk is read
 * into registers before any lane writes, and writes never pass the chunk being
 * read. */
__global__ void __launch_bounds__(256) k_mlp_dedupe(int64_t rows_cap, const int64_t* __restrict__ fix_rows,
                                                    const int64_t* __restrict__ row_start, int* __restrict__ row_len,
                                                    uint32_t* __restrict__ rows, uint32_t nv,
                                                    const float* __restrict__ chord, float* __restrict__ row_scale,
                                                    unsigned long long* __restrict__ flags) {
    int64_t count = (int64_t)flags[ERR_MLP_FIXROWS];
    if (count > rows_cap) count = rows_cap;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < count; r += warps) {
        const int64_t packed = fix_rows[r];
        const int64_t i = packed & ((1ll << 40) - 1);
        const int b0 = (int)(packed >> 40); /* >= 1: entry 0 is the first voxel */
        uint32_t* row = rows + row_start[i];
        const int len = row_len[i];
        int w = b0, outside = 0;
        uint32_t last = row[b0 - 1]; /* entry base - 1 */
        for (int base = b0; base < len; base += 32) {
            const int j = base + lane;
            const uint32_t v = j < len ? row[j] : 0u;
            uint32_t before = __shfl_up_sync(0xffffffffu, v, 1);
            if (lane == 0) before = last;
            last = __shfl_sync(0xffffffffu, v, 31);
            const bool keep = j < len && (j == 0 || v != before);
            const unsigned kb = __ballot_sync(0xffffffffu, keep);
            outside += __popc(__ballot_sync(0xffffffffu, keep && v >= nv));
            __syncwarp();
            if (keep) row[w + __popc(kb & ((1u << lane) - 1u))] = v;
            w += __popc(kb);
            __syncwarp();
        }
        if (lane == 0) {
            row_len[i] = w;
            row_scale[i] = dev_row_scale(chord[i], w);
            if (outside) atomicAdd(flags + ERR_ROWS_OUTSIDE, (unsigned long long)outside);
        }
    }
}

/* Copies each row from its bounded slot to back-to-back storage, one warp per row. */
__global__ void k_copy_rows(int64_t n, const int64_t* __restrict__ src_off, const int* __restrict__ len,
                            const int64_t* __restrict__ dst_off, const uint32_t* __restrict__ src,
                            uint32_t* __restrict__ dst) {
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const uint32_t* s = src + src_off[i];
    uint32_t* d = dst + dst_off[i];
    const int m = len[i];
    for (int j = lane; j < m; j += 32) d[j] = s[j];
}

/* Dense copy of the bounded rows (for pct_get_array). */
__global__ void k_pack_rows(DevGeom g, int64_t n, const int64_t* __restrict__ start, const int* __restrict__ len,
                            const int64_t* __restrict__ dense_off, const uint32_t* __restrict__ rows,
                            uint32_t* __restrict__ dense) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t s = start[i], d = dense_off[i];
    for (int j = 0; j < len[i]; ++j) dense[d + j] = dev_from_brick(g, rows[s + j]); /* linear order */
}

__global__ void k_len64(int64_t n, const int* __restrict__ len, int64_t* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = len[i];
}


/* bf16: the chord length rounded to bfloat16 (round to nearest even), the value
 * a bf16 store holds; it then enters the row norm and the DROP updates. */
__global__ void k_row_norms(DevGeom g, int64_t n, HistView h, const int* __restrict__ len, float* __restrict__ chord,
                            float* __restrict__ row_scale, int bf16) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c = dev_row_chord(g, h, i, bf16);
    chord[i] = c;
    row_scale[i] = dev_row_scale(c, len[i]);
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

/* The binary64 chord of every row (bf16: rounded to bfloat16 first), for the
 * binary64 DROP. */
__global__ void k_row_chords64(DevGeom g, int64_t n, HistView h, int bf16, double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ae = h.xy_entry_angle[i], ax = h.xy_exit_angle[i], ze = h.xz_entry_angle[i], zx = h.xz_exit_angle[i];
    double c = dev_chord(g, (ae + ax) / 2.0, (ze + zx) / 2.0);
    if (bf16) c = (double)__bfloat162float(__float2bfloat16_rn((float)c));
    out[i] = c;
}

}  // namespace

pct_status pct_row_chords64(pct_ctx* c, double* out) {
    const int64_t n = c->h.n;
    if (n == 0) return PCT_OK;
    ++c->launches;
    k_row_chords64<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(c->dg, n, c->view(c->h), c->cfg.chord_bf16, out);
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

pct_status pct_stage_endpoints(pct_ctx* c) {
    if (c->stage != ST_X0) return pct_fail(PCT_ERR_STATE, "collect_mlp_endpoints needs the initial iterate");
    const int64_t n = c->h.n;
    PCT_TRY(c->tmp_missed.alloc(n > 0 ? n : 1));
    uint8_t* keep = c->tmp_missed.as<uint8_t>();
    if (n > 0) {
        HistView h = c->view(c->h);
        ++c->launches;
        if (c->cfg.walk_exact)
            k_endpoints<<<pct_grid_for(n, 128), 128, 0, c->stream>>>(c->dg, n, c->x_hull_filtered.as<uint8_t>(), h,
                                                                     keep, c->err_flags.as<unsigned long long>());
        else {
            uint32_t* order = nullptr;
            if (n <= (int64_t)0xffffffffu) {
                PCT_TRY(c->walk_order.alloc(sizeof(uint32_t) * 2 * (size_t)n));
                order = c->walk_order.as<uint32_t>();
                uint32_t* key = order + n;
                c->launches += 2;
                k_endpoint_key<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(c->dg, n, h, key);
                k_chunk_order<uint32_t><<<(unsigned)((n + ORDER_CHUNK - 1) / ORDER_CHUNK), 1024, 0, c->stream>>>(
                    n, key, order);
            }
            k_endpoints_fast<<<pct_grid_for(n, 128), 128, 0, c->stream>>>(c->dg, n, order,
                                                                          c->x_hull_filtered.as<uint8_t>(), h, keep,
                                                                          c->err_flags.as<unsigned long long>());
        }
        PCT_CUDA(cudaGetLastError());
    }
    int64_t kept = 0;
    PCT_TRY(pct_compact_histories(c, keep, n, &kept));
    c->counts.reconstruction_histories = kept;
    c->stage = ST_ENDPOINTS;
    return PCT_OK;
}

/* chord lengths and 1/||a_i||^2 of the rows in place (used when rows are loaded from a file) */
pct_status pct_stage_row_norms(pct_ctx* c) {
    const int64_t n = c->h.n;
    if (n == 0) return PCT_OK;
    HistView h = c->view(c->h);
    ++c->launches;
    k_row_norms<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(c->dg, n, h, c->row_len.as<int>(), c->chord.as<float>(),
                                                             c->row_scale.as<float>(), c->cfg.chord_bf16);
    PCT_CUDA(cudaGetLastError());
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

static MlpDepthTerms* mlp_depth_terms(pct_ctx* c, int K) {
    return reinterpret_cast<MlpDepthTerms*>(c->mlp_table.as<MlpTableEntry>() + K);
}

static pct_status ensure_mlp_table(pct_ctx* c, int* kmax) {
    const int K = 8 * (c->geo.columns + c->geo.rows + c->geo.slices) + 64;
    *kmax = K;
    if (c->mlp_table.p) return PCT_OK;
    /* K binary32 entries, then K binary64 depth terms (mlp_depth_terms) */
    PCT_TRY(c->mlp_table.alloc((sizeof(MlpTableEntry) + sizeof(MlpDepthTerms)) * K));
    MlpTableEntry* tab = c->mlp_table.as<MlpTableEntry>();
    ++c->launches;
    k_mlp_u1<<<1, 1, 0, c->stream>>>(c->geo.mlp_u_step, K, tab);
    ++c->launches;
    k_mlp_table<<<pct_grid_for(K, 128), 128, 0, c->stream>>>(K, tab, mlp_depth_terms(c, K));
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

pct_status pct_stage_mlp_rows(pct_ctx* c) {
    if (c->stage < ST_ENDPOINTS) return pct_fail(PCT_ERR_STATE, "mlp_rows needs collect_mlp_endpoints");
    if (c->cfg.mlp_tabulated) return pct_stage_mlp_rows_tab(c);
    const int64_t n = c->h.n;
    PCT_TRY(c->row_offsets.alloc(sizeof(int64_t) * (n + 1)));
    PCT_TRY(c->row_len.alloc(sizeof(int) * (n > 0 ? n : 1)));
    PCT_TRY(c->chord.alloc(sizeof(float) * (n > 0 ? n : 1)));
    PCT_TRY(c->row_scale.alloc(sizeof(float) * (n > 0 ? n : 1)));
    int kmax = 0;
    PCT_TRY(ensure_mlp_table(c, &kmax));
    int64_t bound_total = 0;
    HistView h = c->view(c->h);
    unsigned long long* flags = c->err_flags.as<unsigned long long>();
    /* this call's sample counters start from zero */
    PCT_CUDA(cudaMemsetAsync(flags + ERR_MLP_FP64, 0, sizeof(unsigned long long) * 4, c->stream));
    if (n > 0) {
        PCT_TRY(c->mlp_bound.alloc(sizeof(int64_t) * n));
        PCT_TRY(c->mlp_rec.alloc(sizeof(MlpRec) * n));
        /* about 0.3 samples per row need binary64 on the scan geometries; one slot per row */
        const int64_t queue_cap = n > (1 << 20) ? n : (1 << 20);
        PCT_TRY(c->mlp_queue.alloc(sizeof(MlpDeferred) * queue_cap));
        PCT_TRY(c->mlp_fix_rows.alloc(sizeof(int64_t) * n)); /* at most one entry per row */
        MlpRec* rec = c->mlp_rec.as<MlpRec>();
        ++c->launches;
        k_mlp_bound<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(c->dg, n, h, c->mlp_table.as<MlpTableEntry>(), kmax,
                                                                 c->mlp_bound.as<int64_t>(), rec);
        PCT_TRY(pct_scan_lengths(c, c->mlp_bound.as<int64_t>(), n, c->row_offsets.as<int64_t>(), &bound_total));
        PCT_TRY(c->rows.alloc(sizeof(uint32_t) * (bound_total > 0 ? bound_total : 1)));
        const int exact = c->cfg.mlp_exact != 0;
        uint32_t* order = nullptr;
        if (n <= (int64_t)0xffffffffu) {
            PCT_TRY(c->mlp_order.alloc(sizeof(uint32_t) * n));
            order = c->mlp_order.as<uint32_t>();
            ++c->launches;
            k_chunk_order<int64_t><<<(unsigned)((n + ORDER_CHUNK - 1) / ORDER_CHUNK), 1024, 0, c->stream>>>(
                n, c->mlp_bound.as<int64_t>(), order);
        }
        ++c->launches;
        k_mlp_fast<<<pct_grid_for(n, 128), 128, 0, c->stream>>>(
            c->dg, n, order, h, c->cfg.chord_bf16, c->chord.as<float>(), c->row_scale.as<float>(), rec, h.first_voxel, h.x_entry, h.y_entry, c->mlp_table.as<MlpTableEntry>(), c->mlp_bound.as<int64_t>(), exact,
            c->row_offsets.as<int64_t>(), c->rows.as<uint32_t>(), c->row_len.as<int>(), c->mlp_queue.as<MlpDeferred>(),
            queue_cap, c->mlp_fix_rows.as<int64_t>(), flags);
        c->launches += 2;
        k_mlp_fix<<<4 * 152, 128, 0, c->stream>>>(c->dg, rec, c->mlp_table.as<MlpTableEntry>(),
                                                  mlp_depth_terms(c, kmax), c->mlp_queue.as<MlpDeferred>(),
                                                  queue_cap, flags,
                                                  c->rows.as<uint32_t>());
        k_mlp_dedupe<<<8 * 152, 256, 0, c->stream>>>(n, c->mlp_fix_rows.as<int64_t>(),
                                                     c->row_offsets.as<int64_t>(), c->row_len.as<int>(),
                                                     c->rows.as<uint32_t>(), (uint32_t)c->geo.num_voxels,
                                                     c->chord.as<float>(), c->row_scale.as<float>(), flags);
        PCT_CUDA(cudaGetLastError());
    }
    c->row_capacity = bound_total;
    c->counts.row_entries = -1; /* computed on demand */
    c->diag_ready = 0;
    pct_drop_release_graph(c);
    c->stage = ST_ROWS;
    return PCT_OK;
}

/* The rows packed back to back in the rows' voxel order: the slack of the
 * bounded slots (one slot entry per MLP sample) and the MLP pass's per-history
 * scratch are returned to the device.
 * An extension of the reconstruction sequence with no reference counterpart:
 * it lets many scans' rows stay resident together (pct_drop_many). */
extern "C" pct_status pct_compact_rows(pct_ctx* c) {
    if (!c) return pct_fail(PCT_ERR_ARGUMENT, "pct_compact_rows: null context");
    PCT_TRY(c->set_device());
    if (c->stage < ST_ROWS) return pct_fail(PCT_ERR_STATE, "pct_compact_rows needs the MLP rows");
    const int64_t n = c->h.n;
    if (n == 0) return PCT_OK;
    DevBuf off, len64, dense;
    int64_t total = 0;
    PCT_TRY(off.alloc(sizeof(int64_t) * (n + 1)));
    pct_status st = len64.alloc(sizeof(int64_t) * n);
    if (st != PCT_OK) {
        off.release();
        return st;
    }
    ++c->launches;
    k_len64<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(n, c->row_len.as<int>(), len64.as<int64_t>());
    st = pct_scan_lengths(c, len64.as<int64_t>(), n, off.as<int64_t>(), &total);
    len64.release();
    if (st == PCT_OK && total < c->row_capacity) st = dense.alloc(sizeof(uint32_t) * (total > 0 ? total : 1));
    if (st != PCT_OK || total >= c->row_capacity) { /* failed, or no slack to return */
        off.release();
        return st;
    }
    ++c->launches;
    k_copy_rows<<<(unsigned)((n * 32 + 255) / 256), 256, 0, c->stream>>>(
        n, c->row_offsets.as<int64_t>(), c->row_len.as<int>(), off.as<int64_t>(), c->rows.as<uint32_t>(),
        dense.as<uint32_t>());
    PCT_CUDA(cudaGetLastError());
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    std::swap(c->rows, dense);
    std::swap(c->row_offsets, off);
    dense.release();
    off.release();
    /* the MLP pass's scratch goes too (pct_mlp_rows allocates it again) */
    c->mlp_bound.release();
    c->mlp_rec.release();
    c->mlp_queue.release();
    c->mlp_fix_rows.release();
    c->mlp_order.release();
    c->row_capacity = total;
    c->diag_ready = 0; /* the per-block structures hold row positions */
    pct_drop_release_graph(c);
    return PCT_OK;
}

/* Number of row entries, dense offsets (n+1) and, if dense != NULL, the dense rows. */
pct_status pct_rows_dense(pct_ctx* c, int64_t* total, DevBuf* dense_off, DevBuf* dense) {
    const int64_t n = c->h.n;
    PCT_TRY(dense_off->alloc(sizeof(int64_t) * (n + 1)));
    if (n == 0) {
        *total = 0;
        PCT_CUDA(cudaMemsetAsync(dense_off->p, 0, sizeof(int64_t), c->stream));
        return PCT_OK;
    }
    DevBuf len64;
    PCT_TRY(len64.alloc(sizeof(int64_t) * n));
    k_len64<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(n, c->row_len.as<int>(), len64.as<int64_t>());
    pct_status st = pct_scan_lengths(c, len64.as<int64_t>(), n, dense_off->as<int64_t>(), total);
    len64.release();
    PCT_TRY(st);
    if (dense) {
        PCT_TRY(dense->alloc(sizeof(uint32_t) * (*total > 0 ? *total : 1)));
        k_pack_rows<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(c->dg, n, c->row_offsets.as<int64_t>(), c->row_len.as<int>(),
                                                                 dense_off->as<int64_t>(), c->rows.as<uint32_t>(),
                                                                 dense->as<uint32_t>());
        PCT_CUDA(cudaGetLastError());
    }
    return PCT_OK;
}

