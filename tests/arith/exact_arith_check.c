/*
 * Host checks of the exact-arithmetic identities the device code relies on
 * (pct_math.h), run by tests/test_exact_arith.py:
 *   1. pct_div_rn equals IEEE division on every quotient k_backproject forms
 *      (backprojection_GPU, src/pCT_Reconstruction_Data_Segments.cu:3155-3230:
 *      t / (SR + u), SR / (SR + u), v / (SR + u) and the divisions by the t
 *      and v bin sizes) for the given grids, and on random operands;
 *   2. the product error of pct_two_prod (Dekker's splitting, the host form)
 *      equals fma(a, b, -a b) (the device form);
 *   3. pct_sincos(x) equals (pct_sin(x), pct_cos(x)) bit for bit.
 * Prints one line per check and exits non-zero on any difference.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "pct_math.h"

#define ANGLE_TO_RADIANS (PCT_PI / 180.0)

static int same(double a, double b) { return memcmp(&a, &b, sizeof a) == 0; }

static uint64_t rng = 88172645463325252ull;
static uint64_t next(void) {
    rng ^= rng << 13;
    rng ^= rng >> 7;
    rng ^= rng << 17;
    return rng;
}
static double unit(void) { return ldexp((double)(next() >> 11), -53); } /* [0, 1) */

struct grid {
    const char* name;
    int columns, rows, slices, angles;
    double gantry_interval, radius, voxel_w, voxel_h, height, slice_t, source_r, t_bin, v_bin;
};

/* The quotients of k_backproject, in its order of evaluation. */
static long long check_backprojection(const struct grid* g, int angle_stride, long long* count) {
    long long bad = 0;
    const double delta = g->gantry_interval * ANGLE_TO_RADIANS, SR = g->source_r;
    const double r_t = 1.0 / g->t_bin, r_v = 1.0 / g->v_bin;
    for (int ab = 0; ab < g->angles; ab += angle_stride) {
        const double ca = pct_cos(ab * delta), sa = pct_sin(ab * delta);
        for (int row = 0; row < g->rows; ++row)
            for (int col = 0; col < g->columns; ++col) {
                const double x = -g->radius + (col + 0.5) * g->voxel_w;
                const double y = g->radius - (row + 0.5) * g->voxel_h;
                if (x * x + y * y > g->radius * g->radius) continue;
                const double u = x * ca + y * sa, t = -x * sa + y * ca, d = SR + u, rd = 1.0 / d;
                const double qt = t / d, nt = t - u * qt;
                bad += !same(pct_div_rn(t, d, rd), qt);
                bad += !same(pct_div_rn(SR, d, rd), SR / d);
                bad += !same(pct_div_rn(nt, g->t_bin, r_t), nt / g->t_bin);
                *count += 3;
                for (int s = 0; s < g->slices; ++s) {
                    const double v = -g->height / 2.0 + (s + 0.5) * g->slice_t;
                    const double qv = v / d, nv = v - u * qv;
                    bad += !same(pct_div_rn(v, d, rd), qv);
                    bad += !same(pct_div_rn(nv, g->v_bin, r_v), nv / g->v_bin);
                    *count += 2;
                }
            }
    }
    return bad;
}

int main(int argc, char** argv) {
    const long long random_n = argc > 1 ? atoll(argv[1]) : 20000000ll;
    int failed = 0;
    const struct grid grids[] = {
        {"200x200x8 (4 deg)", 200, 200, 8, 90, 4.0, 10.0, 0.1, 0.1, 2.0, 0.25, 260.7, 0.1, 0.25},
        {"256x256x32", 256, 256, 32, 180, 2.0, 12.8, 0.1, 0.1, 8.0, 0.25, 260.7, 0.1, 0.25},
        {"128x128x8", 128, 128, 8, 180, 2.0, 6.4, 0.1, 0.1, 2.0, 0.25, 260.7, 0.1, 0.25},
        {"320x320x64 (every 6th angle)", 320, 320, 64, 180, 2.0, 12.8, 0.08, 0.08, 16.0, 0.25, 260.7, 0.1, 0.25},
    };
    for (size_t k = 0; k < sizeof grids / sizeof grids[0]; ++k) {
        long long n = 0;
        const long long bad = check_backprojection(&grids[k], k == 3 ? 6 : 1, &n);
        printf("div_rn backprojection %s: %lld quotients, %lld differ\n", grids[k].name, n, bad);
        failed |= bad != 0;
    }
    long long bad = 0;
    for (long long i = 0; i < random_n; ++i) {
        const double a = ldexp(2.0 * unit() - 1.0, (int)(next() % 60) - 30);
        const double b = ldexp(1.0 + unit(), (int)(next() % 60) - 30) * ((next() & 1) ? 1.0 : -1.0);
        bad += !same(pct_div_rn(a, b, 1.0 / b), a / b);
    }
    printf("div_rn random: %lld quotients, %lld differ\n", random_n, bad);
    failed |= bad != 0;
    bad = 0;
    for (long long i = 0; i < random_n; ++i) {
        const double a = ldexp(2.0 * unit() - 1.0, (int)(next() % 80) - 40);
        const double b = ldexp(2.0 * unit() - 1.0, (int)(next() % 80) - 40);
        double p, e;
        pct_two_prod(a, b, &p, &e);
        bad += !same(p, a * b) || !same(e, fma(a, b, -(a * b)));
    }
    printf("two_prod random: %lld products, %lld differ\n", random_n, bad);
    failed |= bad != 0;
    bad = 0;
    const long long trig_n = random_n / 10;
    for (long long i = 0; i < trig_n; ++i) {
        const double x = (i & 1) ? (20.0 * unit() - 10.0) : (i / 2 % 720) * (0.5 * ANGLE_TO_RADIANS);
        double s, c;
        pct_sincos(x, &s, &c);
        bad += !same(s, pct_sin(x)) || !same(c, pct_cos(x));
    }
    printf("sincos: %lld arguments, %lld differ\n", trig_n, bad);
    failed |= bad != 0;
    return failed;
}
