/*
 * Seeded synthetic phantoms and proton histories (no reference counterpart:
 * the reference only reads PCTD files, src/pCT_Reconstruction_Data_Segments.cu:1769).
 *
 * A phantom is a list of primitives (z-aligned cylinders clipped in z, and
 * ellipsoids rotated about z), each adding its RSP inside its volume.  A
 * history is a straight line through the phantom at one gantry angle, with
 * the tracker hits the reference expects: t/v on four planes u = -150, -100,
 * +100, +150 mm, written in the PCTD v0 layout (mm, projection angle such that
 * (int(angle) + 270) % 360 is the gantry angle, .cu:1921).
 *
 * Physics model (kept simple on purpose, it only has to exercise the path):
 *   entry line   t = t0 + s_t u, v = v0 + s_v u; (t0, v0) uniform over the
 *                beam field, slopes = fan divergence from the source plus a
 *                Gaussian beam spread;
 *   WEPL         line integral of RSP along the entry line, times (1 + noise N),
 *                replaced by a uniform value for the outlier fraction
 *                (nuclear events) of the histories that hit the phantom;
 *   scattering   Highland width for the traversed water-equivalent length;
 *                exit slope kick and exit offset drawn with the correlation
 *                of multiple Coulomb scattering (rho = sqrt(3)/2).
 * Randomness is a splitmix64 counter stream per history (Steele, Lea & Flood
 * 2014) and Box-Muller normals, and all arithmetic goes through pct_math.h,
 * so the same seed gives the same bits on every host.
 */
#include <cstdint>
#include <cstring>
#include <cmath>
#include "pct_internal.h"

namespace {

struct Rng {
    uint64_t state;
    uint64_t next() {
        uint64_t z = (state += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    /* uniform in (0, 1) */
    double uniform() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {
        double u1 = uniform(), u2 = uniform();
        return sqrt(-2.0 * pct_log(u1)) * pct_cos(PCT_TWO_PI * u2);
    }
};

/* Parameter interval [lo, hi] of u where the line p(u) = p0 + d u is inside
 * the primitive; returns false when it misses. */
bool chord_interval(const pct_phantom_object& o, const double p0[3], const double d[3], double* lo, double* hi) {
    if (o.kind == PCT_PRIM_CYLINDER) {
        double px = p0[0] - o.cx, py = p0[1] - o.cy;
        double a = d[0] * d[0] + d[1] * d[1];
        double b = 2.0 * (px * d[0] + py * d[1]);
        double c = px * px + py * py - o.a * o.a;
        double disc = b * b - 4.0 * a * c;
        if (!(a > 0.0) || disc <= 0.0) return false;
        double sq = sqrt(disc);
        double u0 = (-b - sq) / (2.0 * a), u1 = (-b + sq) / (2.0 * a);
        /* clip to the z slab |z - cz| <= c_half */
        double zlo = o.cz - o.c, zhi = o.cz + o.c;
        if (d[2] == 0.0) {
            if (p0[2] < zlo || p0[2] > zhi) return false;
        } else {
            double ua = (zlo - p0[2]) / d[2], ub = (zhi - p0[2]) / d[2];
            if (ua > ub) { double t = ua; ua = ub; ub = t; }
            if (ua > u0) u0 = ua;
            if (ub < u1) u1 = ub;
        }
        if (!(u1 > u0)) return false;
        *lo = u0; *hi = u1;
        return true;
    }
    /* ellipsoid: rotate into its frame (rotation -phi about z), scale to a unit sphere */
    double cp = pct_cos(o.phi), sp = pct_sin(o.phi);
    double qx = p0[0] - o.cx, qy = p0[1] - o.cy, qz = p0[2] - o.cz;
    double lx = (cp * qx + sp * qy) / o.a, ly = (-sp * qx + cp * qy) / o.b, lz = qz / o.c;
    double ex = (cp * d[0] + sp * d[1]) / o.a, ey = (-sp * d[0] + cp * d[1]) / o.b, ez = d[2] / o.c;
    double a = ex * ex + ey * ey + ez * ez;
    double b = 2.0 * (lx * ex + ly * ey + lz * ez);
    double c = lx * lx + ly * ly + lz * lz - 1.0;
    double disc = b * b - 4.0 * a * c;
    if (!(a > 0.0) || disc <= 0.0) return false;
    double sq = sqrt(disc);
    *lo = (-b - sq) / (2.0 * a);
    *hi = (-b + sq) / (2.0 * a);
    return true;
}

}  // namespace

double pct_phantom_line_integral(const pct_phantom_object* objs, int n_objs, const double p0[3], const double d[3]) {
    double len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double sum = 0.0;
    for (int k = 0; k < n_objs; ++k) {
        double lo, hi;
        if (chord_interval(objs[k], p0, d, &lo, &hi)) sum += objs[k].rsp * (hi - lo) * len;
    }
    return sum;
}

double pct_phantom_rsp_at(const pct_phantom_object* objs, int n_objs, double x, double y, double z) {
    double r = 0.0;
    for (int k = 0; k < n_objs; ++k) {
        const pct_phantom_object& o = objs[k];
        bool inside;
        if (o.kind == PCT_PRIM_CYLINDER) {
            double dx = x - o.cx, dy = y - o.cy;
            inside = dx * dx + dy * dy <= o.a * o.a && z >= o.cz - o.c && z <= o.cz + o.c;
        } else {
            double cp = pct_cos(o.phi), sp = pct_sin(o.phi);
            double qx = x - o.cx, qy = y - o.cy, qz = z - o.cz;
            double lx = (cp * qx + sp * qy) / o.a, ly = (-sp * qx + cp * qy) / o.b, lz = qz / o.c;
            inside = lx * lx + ly * ly + lz * lz <= 1.0;
        }
        if (inside) r += o.rsp;
    }
    return r;
}

extern "C" pct_status pct_generate_histories(const pct_phantom_object* objs, int n_objs, const pct_scan_params* sp,
                                             float* const out[13], float* projection_angle, int64_t n) {
    if (!sp || !out || !projection_angle || n < 0 || (n_objs > 0 && !objs)) return pct_fail(PCT_ERR_ARGUMENT, "pct_generate_histories: null argument");
    for (int k = 0; k < 13; ++k)
        if (!out[k]) return pct_fail(PCT_ERR_ARGUMENT, "pct_generate_histories: null output array");
    if (sp->num_angles <= 0) return pct_fail(PCT_ERR_ARGUMENT, "pct_generate_histories: num_angles must be positive");
    const double u_planes[4] = {-15.0, -10.0, 10.0, 15.0};
    /* 200 MeV protons: beta*c*p in MeV for the Highland width */
    const double T = sp->beam_energy_mev > 0 ? sp->beam_energy_mev : 200.0;
    const double mc2 = 938.272;
    const double pc = sqrt(T * T + 2.0 * T * mc2);
    const double betacp0 = pc * pc / (T + mc2);
    const int64_t per_angle = (n + sp->num_angles - 1) / sp->num_angles;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int ang = (int)(i / per_angle);
        int gantry = (int)(ang * sp->gantry_angle_interval);
        double g = gantry * PCT_ANGLE_TO_RADIANS;
        double cg = pct_cos(g), sg = pct_sin(g);
        Rng r;
        r.state = sp->seed * 0xD1B54A32D192ED03ULL + (uint64_t)i * 0x9E3779B97F4A7C15ULL;
        r.next();
        double t0 = (2.0 * r.uniform() - 1.0) * sp->t_extent;
        double v0 = (2.0 * r.uniform() - 1.0) * sp->v_extent;
        double st = t0 / sp->source_radius + sp->angular_spread * r.normal();
        double sv = v0 / sp->source_radius + sp->angular_spread * r.normal();
        /* world line: x = cos g u - sin g t, y = sin g u + cos g t, z = v */
        double p0[3] = {-sg * t0, cg * t0, v0};
        double dir[3] = {cg - sg * st, sg + cg * st, sv};
        double wepl_true = pct_phantom_line_integral(objs, n_objs, p0, dir);
        double wepl = wepl_true;
        double dt = 0.0, dv = 0.0, kt = 0.0, kv = 0.0;
        double n1 = r.normal(), n2 = r.normal(), n3 = r.normal(), n4 = r.normal(), n5 = r.normal();
        double uo = r.uniform(), uw = r.uniform();
        if (wepl_true > 0.0) {
            double x = wepl_true / PCT_X_0;
            double betacp = betacp0 * (1.0 - 0.5 * wepl_true / 26.0);
            if (betacp < 0.25 * betacp0) betacp = 0.25 * betacp0;
            double theta0 = sp->scatter_scale * (13.6 / betacp) * sqrt(x) * (1.0 + 0.038 * pct_log(x));
            if (theta0 < 0) theta0 = 0;
            const double rho = 0.8660254037844386;
            double L = wepl_true;
            kt = theta0 * n1;
            kv = theta0 * n2;
            dt = theta0 * L * (rho * n1 + 0.5 * n3) * 0.5773502691896258 * 0.5;
            dv = theta0 * L * (rho * n2 + 0.5 * n4) * 0.5773502691896258 * 0.5;
            wepl = wepl_true * (1.0 + sp->wepl_noise * n5);
            if (uo < sp->outlier_fraction) wepl = uw * sp->outlier_max;
        }
        for (int k = 0; k < 4; ++k) {
            double u = u_planes[k];
            double tk = t0 + st * u, vk = v0 + sv * u;
            if (k >= 2) { tk += dt + kt * u; vk += dv + kv * u; }
            out[k][i] = (float)(tk * 10.0);
            out[4 + k][i] = (float)(vk * 10.0);
            out[8 + k][i] = (float)(u * 10.0);
        }
        out[12][i] = (float)(wepl * 10.0);
        projection_angle[i] = (float)((gantry + 90) % 360);
    }
    return PCT_OK;
}

extern "C" pct_status pct_phantom_voxelize(const pct_phantom_object* objs, int n_objs, const pct_config* cfg,
                                           int supersample, float* image) {
    pct_geometry g;
    if (!cfg || !image || (n_objs > 0 && !objs)) return pct_fail(PCT_ERR_ARGUMENT, "pct_phantom_voxelize: null argument");
    if (pct_geometry_derive(cfg, &g)) return pct_fail(PCT_ERR_ARGUMENT, "pct_phantom_voxelize: bad geometry");
    int s = supersample > 0 ? supersample : 1;
    double inv = 1.0 / ((double)s * s * s);
#pragma omp parallel for schedule(static)
    for (int v = 0; v < g.num_voxels; ++v) {
        int col = v % g.columns, row = (v / g.columns) % g.rows, sl = v / (g.columns * g.rows);
        double acc = 0.0;
        for (int a = 0; a < s; ++a)
            for (int b = 0; b < s; ++b)
                for (int c = 0; c < s; ++c) {
                    /* voxel index convention of the reference walks: x from -R rightwards,
                       y from +R downwards, z from +H/2 downwards (pCT_data.h:272-277) */
                    double x = g.x_zero + (col + (a + 0.5) / s) * g.voxel_width;
                    double y = g.y_zero - (row + (b + 0.5) / s) * g.voxel_height;
                    double z = g.z_zero - (sl + (c + 0.5) / s) * g.voxel_thickness;
                    acc += pct_phantom_rsp_at(objs, n_objs, x, y, z);
                }
        image[v] = (float)(acc * inv);
    }
    return PCT_OK;
}
