/*
 * Prints x, pct_sincos_cr(x) as hexadecimal floats for the per-angle table
 * arguments of 0.5, 1, 2, 3, 4, 5 and 6 degree grids (both forms the tables
 * use: (i a) rad and i (a rad)) and for `n` random arguments in [-7, 7];
 * tests/test_exact_arith.py compares them with correctly rounded values.
 */
#include <stdio.h>
#include <stdlib.h>
#include "pct_math.h"

int main(int argc, char** argv) {
    const int n = argc > 1 ? atoi(argv[1]) : 20000;
    const double intervals[] = {0.5, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0};
    for (int t = 0; t < 7; ++t) {
        const double a = intervals[t];
        for (int i = 0; i < (int)(360.0 / a) + 2; ++i) {
            const double args[2] = {(i * a) * (PCT_PI / 180.0), i * (a * (PCT_PI / 180.0))};
            for (int k = 0; k < 2; ++k) {
                double s, c;
                pct_sincos_cr(args[k], &s, &c);
                printf("%a %a %a\n", args[k], s, c);
            }
        }
    }
    unsigned long long r = 88172645463325252ull;
    for (int i = 0; i < n; ++i) {
        r ^= r << 13;
        r ^= r >> 7;
        r ^= r << 17;
        const double x = ldexp((double)(r >> 11), -53) * 14.0 - 7.0;
        double s, c;
        pct_sincos_cr(x, &s, &c);
        printf("%a %a %a\n", x, s, c);
    }
    return 0;
}
