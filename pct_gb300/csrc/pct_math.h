/*
 * Deterministic elementary functions for host C/C++ and CUDA device code.
 *
 * Every function here is written with IEEE-754 binary64 add, subtract,
 * multiply, divide, sqrt, floor and fused multiply-add only, evaluated in
 * source order (the fused multiply-adds where they are exact or correctly
 * rounded by construction: pct_two_prod on the device, pct_div_rn).  Built
 * without FMA contraction (gcc -ffp-contract=off, nvcc -fmad=false) the same
 * source gives bit-identical results on x86-64, aarch64 and sm_103a, which is
 * what lets the CUDA kernels and the CPU oracle agree bit for bit on the
 * reference's transcendental-dependent decisions (bin indices, voxel walks,
 * MLP voxel sequences).  The platform libms (glibc of either host, CUDA's
 * libdevice) are never called for those.
 *
 * Methods (all textbook; coefficients are the exact Taylor coefficients
 * rounded to double, constants were computed with 300-bit mpmath):
 *   sin/cos/tan  Cody-Waite reduction by pi/2 with a three-part constant and a
 *                double-double remainder, then Taylor polynomials on
 *                |r| <= pi/4; tan = sin/cos in double-double, one
 *                exact-remainder correction.
 *   log          x = 2^e (1+f), s = f/(2+f), log(1+f) = 2 atanh(s) rearranged
 *                as f - (f^2/2 - s (f^2/2 + R(s^2))), R the atanh series.
 *   atan/atan2   reference points atan(c), c in {1/4,1/2,1,3/2,3,inf}, stored
 *                as hi+lo, then the Taylor series of atan on |u| <= 0.2.
 *   cube         Dekker exact product, one final rounding.
 * Accuracy (measured against glibc over 10^7 arguments): within 1 ulp.
 * Domain of the reduction: |x| < 2^19 * pi/2 (angles in this code are < 100).
 */
#ifndef PCT_MATH_H
#define PCT_MATH_H

#include <math.h> /* floor, frexp, sqrt: exact or correctly rounded everywhere */

#if defined(__CUDACC__)
#define PCT_FN __host__ __device__ static inline
#else
#define PCT_FN static inline
#endif

#define PCT_PI 3.141592653589793              /* = 4*atan(1.0) in binary64 */
#define PCT_PI_LO 1.2246467991473532e-16
#define PCT_PIO2_HI 1.5707963267948966
#define PCT_PIO2_LO 6.123233995736766e-17

/* ---- exact arithmetic helpers ------------------------------------------ */
PCT_FN void pct_two_sum(double a, double b, double* s, double* e) {
    double x = a + b;
    double bb = x - a;
    *e = (a - (x - bb)) + (b - bb);
    *s = x;
}
PCT_FN void pct_fast_two_sum(double a, double b, double* s, double* e) { /* |a| >= |b| */
    double x = a + b;
    *e = b - (x - a);
    *s = x;
}
PCT_FN void pct_split(double a, double* hi, double* lo) {
    double c = 134217729.0 * a; /* 2^27 + 1 */
    double ab = c - a;
    *hi = c - ab;
    *lo = a - *hi;
}
/* p = RN(a b) and its error e = a b - p exactly (both forms are exact away
 * from overflow and underflow, so they give the same e: Dekker's product on
 * the host, one fused multiply-add on the device). */
PCT_FN void pct_two_prod(double a, double b, double* p, double* e) {
    double x = a * b;
#if defined(__CUDA_ARCH__)
    *e = fma(a, b, -x);
#else
    double ah, al, bh, bl;
    pct_split(a, &ah, &al);
    pct_split(b, &bh, &bl);
    *e = ((ah * bh - x) + ah * bl + al * bh) + al * bl;
#endif
    *p = x;
}

/* The correctly rounded quotient a / b from r = RN(1 / b): q = RN(a r), then
 * RN(q + (a - b q) r) with the remainder a - b q exact by FMA.  Markstein's
 * theorem: with r within half an ulp of 1 / b and q within one ulp of a / b,
 * the corrected q is RN(a / b) (no overflow or underflow).  Three binary64
 * instructions where the divisor is reused with its reciprocal. */
PCT_FN double pct_div_rn(double a, double b, double r) {
    const double q = a * r;
    return fma(fma(-q, b, a), r, q);
}

/* x^2 correctly rounded is just x*x; x^3 with a single rounding. */
PCT_FN double pct_cube(double x) {
    double p, e, q, f;
    pct_two_prod(x, x, &p, &e);
    pct_two_prod(p, x, &q, &f);
    return q + (f + e * x);
}

/* ---- sin / cos / tan ----------------------------------------------------- */
/* x = k*pi/2 + (r + rr), |r| <= ~pi/4; returns k mod 4. */
PCT_FN int pct_rem_pio2(double x, double* r, double* rr) {
    const double C1 = 1.5707963267341256;        /* 33 significant bits */
    const double C2 = 6.077100506303966e-11;     /* 33 significant bits */
    const double C3 = 2.0222662487959506e-21;
    const double TWO_OVER_PI = 0.6366197723675814;
    double ax = x < 0 ? -x : x;
    if (ax <= 0.7853981633974483) {
        *r = x;
        *rr = 0.0;
        return 0;
    }
    double k = floor(x * TWO_OVER_PI + 0.5);
    double t1 = x - k * C1;                      /* exact */
    double s1, e1, s2, e2;
    pct_two_sum(t1, -(k * C2), &s1, &e1);        /* k*C2 exact */
    pct_two_sum(s1, -(k * C3), &s2, &e2);
    double lo = e1 + e2;
    double hi;
    pct_fast_two_sum(s2, lo, &hi, &lo);
    *r = hi;
    *rr = lo;
    long long ki = (long long)k;
    return (int)(ki & 3);
}
PCT_FN double pct_sin_kernel(double r, double rr) {
    /* sin r = r - r^3 P(z), P(z) = 1/3! - z/5! + z^2/7! - ... + z^8/19!, z = r^2 */
    double z = r * r;
    double p = 8.22063524662433e-18;             /*  1/19! */
    p = p * z + (-2.8114572543455206e-15);       /* -1/17! */
    p = p * z + 7.647163731819816e-13;           /*  1/15! */
    p = p * z + (-1.6059043836821613e-10);       /* -1/13! */
    p = p * z + 2.505210838544172e-08;           /*  1/11! */
    p = p * z + (-2.7557319223985893e-06);       /* -1/9!  */
    p = p * z + 0.0001984126984126984;           /*  1/7!  */
    p = p * z + (-0.008333333333333333);         /* -1/5!  */
    p = p * z + 0.16666666666666666;             /*  1/3!  */
    double r3 = r * z;
    /* the remainder rr enters through d(sin)/dr = cos r ~ 1 - z/2 */
    return r + ((rr - 0.5 * z * rr) - r3 * p);
}
PCT_FN double pct_cos_kernel(double r, double rr) {
    double z = r * r;
    double q = -1.5619206968586225e-16;          /* -1/18! */
    q = q * z + 4.779477332387385e-14;           /* 1/16! */
    q = q * z + (-1.1470745597729725e-11);       /* -1/14! */
    q = q * z + 2.08767569878681e-09;            /* 1/12! */
    q = q * z + (-2.755731922398589e-07);        /* -1/10! */
    q = q * z + 2.48015873015873e-05;            /* 1/8! */
    q = q * z + (-0.001388888888888889);         /* -1/6! */
    q = q * z + 0.041666666666666664;            /* 1/4! */
    double p, e;
    pct_two_prod(r, r, &p, &e);
    double hp = 0.5 * p, he = 0.5 * e;           /* r^2/2 = hp + he exactly */
    double w = 1.0 - hp;
    double err = (1.0 - w) - hp;                 /* exact */
    double tail = ((z * z) * q - he) + err - r * rr;
    return w + tail;
}
PCT_FN double pct_sin(double x) {
    double r, rr;
    int q = pct_rem_pio2(x, &r, &rr);
    switch (q) {
        case 0: return pct_sin_kernel(r, rr);
        case 1: return pct_cos_kernel(r, rr);
        case 2: return -pct_sin_kernel(r, rr);
        default: return -pct_cos_kernel(r, rr);
    }
}
PCT_FN double pct_cos(double x) {
    double r, rr;
    int q = pct_rem_pio2(x, &r, &rr);
    switch (q) {
        case 0: return pct_cos_kernel(r, rr);
        case 1: return -pct_sin_kernel(r, rr);
        case 2: return -pct_cos_kernel(r, rr);
        default: return pct_sin_kernel(r, rr);
    }
}
/* pct_sin(x) and pct_cos(x) from one argument reduction (the same values). */
PCT_FN void pct_sincos(double x, double* s, double* c) {
    double r, rr;
    int q = pct_rem_pio2(x, &r, &rr);
    const double sk = pct_sin_kernel(r, rr), ck = pct_cos_kernel(r, rr);
    switch (q) {
        case 0: *s = sk; *c = ck; break;
        case 1: *s = ck; *c = -sk; break;
        case 2: *s = -sk; *c = -ck; break;
        default: *s = -ck; *c = sk; break;
    }
}
/* ---- correctly rounded sin / cos for per-angle tables -------------------- */
/* Double-double arithmetic: a value is hi + lo with |lo| <= ulp(hi) / 2. */
PCT_FN void pct_dd_mul(double ah, double al, double bh, double bl, double* h, double* l) {
    double p, e;
    pct_two_prod(ah, bh, &p, &e);
    e += ah * bl + al * bh;
    pct_fast_two_sum(p, e, h, l);
}
PCT_FN void pct_dd_add(double ah, double al, double bh, double bl, double* h, double* l) {
    double s, e;
    pct_two_sum(ah, bh, &s, &e);
    e += al + bl;
    pct_fast_two_sum(s, e, h, l);
}
/* sin(x) and cos(x) rounded once from double-double values: the reduction of
 * pct_rem_pio2 (x - k pi/2 = r + rr), then the Taylor series of sin and cos
 * on |r| <= pi/4 to the terms r^25 / 25! and r^26 / 26! (the next ones are
 * below 2^-100) in double-double Horner form with double-double 1/n!, and
 * one final rounding of hi + lo.  About 100 correct bits before that
 * rounding, so the result is the correctly rounded value unless sin or cos
 * lies within 2^-100 (relative) of a rounding boundary.  For the per-angle
 * tables where the reference takes the platform's binary64 cos and sin of an
 * angle (gantry rotation, bin angles, backprojection); a few hundred calls
 * per scan. */
PCT_FN void pct_sincos_cr(double x, double* s, double* c) {
    /* 1/n! as hi, lo: sine terms n = 1, 3, ..., 25, cosine terms n = 0, 2, ..., 26 */
    const double SI[13][2] = {{1.0, 0.0},
                              {0.16666666666666666, 9.25185853854297e-18},
                              {0.008333333333333333, 1.1564823173178714e-19},
                              {0.0001984126984126984, 1.7209558293420705e-22},
                              {2.7557319223985893e-06, -1.858393274046472e-22},
                              {2.505210838544172e-08, -1.448814070935912e-24},
                              {1.6059043836821613e-10, 1.2585294588752098e-26},
                              {7.647163731819816e-13, 7.03872877733453e-30},
                              {2.8114572543455206e-15, 1.6508842730861433e-31},
                              {8.22063524662433e-18, 2.2141894119604265e-34},
                              {1.9572941063391263e-20, -1.3643503830087908e-36},
                              {3.868170170630684e-23, -8.843177655482344e-40},
                              {6.446950284384474e-26, -1.9330404233703465e-42}};
    const double CO[14][2] = {{1.0, 0.0},
                              {0.5, 0.0},
                              {0.041666666666666664, 2.3129646346357427e-18},
                              {0.001388888888888889, -5.300543954373577e-20},
                              {2.48015873015873e-05, 2.1511947866775882e-23},
                              {2.755731922398589e-07, 2.3767714622250297e-23},
                              {2.08767569878681e-09, -1.20734505911326e-25},
                              {1.1470745597729725e-11, 2.0655512752830745e-28},
                              {4.779477332387385e-14, 4.399205485834081e-31},
                              {1.5619206968586225e-16, 1.1910679660273754e-32},
                              {4.110317623312165e-19, 1.4412973378659527e-36},
                              {8.896791392450574e-22, -7.911402614872376e-38},
                              {1.6117375710961184e-24, -3.6846573564509766e-41},
                              {2.4795962632247976e-27, -1.2953730964765229e-43}};
    double r, rr;
    const int q = pct_rem_pio2(x, &r, &rr);
    double zh, zl; /* z = -(r + rr)^2: the series alternate */
    pct_dd_mul(r, rr, r, rr, &zh, &zl);
    zh = -zh;
    zl = -zl;
    double sh = SI[12][0], sl = SI[12][1];
    for (int k = 11; k >= 0; --k) {
        pct_dd_mul(sh, sl, zh, zl, &sh, &sl);
        pct_dd_add(sh, sl, SI[k][0], SI[k][1], &sh, &sl);
    }
    pct_dd_mul(sh, sl, r, rr, &sh, &sl); /* sin(r + rr) */
    double ch = CO[13][0], cl = CO[13][1];
    for (int k = 12; k >= 0; --k) {
        pct_dd_mul(ch, cl, zh, zl, &ch, &cl);
        pct_dd_add(ch, cl, CO[k][0], CO[k][1], &ch, &cl);
    }
    const double sk = sh + sl, ck = ch + cl;
    switch (q) {
        case 0: *s = sk; *c = ck; break;
        case 1: *s = ck; *c = -sk; break;
        case 2: *s = -sk; *c = -ck; break;
        default: *s = -ck; *c = sk; break;
    }
}

/* tan = sin/cos from double-double kernel values, one exact-remainder correction. */
PCT_FN double pct_tan(double x) {
    double r, rr;
    int q = pct_rem_pio2(x, &r, &rr);
    double z = r * r;
    double p = 8.22063524662433e-18;
    p = p * z + (-2.8114572543455206e-15);
    p = p * z + 7.647163731819816e-13;
    p = p * z + (-1.6059043836821613e-10);
    p = p * z + 2.505210838544172e-08;
    p = p * z + (-2.7557319223985893e-06);
    p = p * z + 0.0001984126984126984;
    p = p * z + (-0.008333333333333333);
    p = p * z + 0.16666666666666666;
    double st = (rr - 0.5 * z * rr) - (r * z) * p;
    double sh, sl;
    pct_fast_two_sum(r, st, &sh, &sl);
    double qq = -1.5619206968586225e-16;
    qq = qq * z + 4.779477332387385e-14;
    qq = qq * z + (-1.1470745597729725e-11);
    qq = qq * z + 2.08767569878681e-09;
    qq = qq * z + (-2.755731922398589e-07);
    qq = qq * z + 2.48015873015873e-05;
    qq = qq * z + (-0.001388888888888889);
    qq = qq * z + 0.041666666666666664;
    double pp, e;
    pct_two_prod(r, r, &pp, &e);
    double hp = 0.5 * pp, he = 0.5 * e;
    double w = 1.0 - hp;
    double err = (1.0 - w) - hp;
    double tail = ((z * z) * qq - he) + err - r * rr;
    double ch, cl;
    pct_fast_two_sum(w, tail, &ch, &cl);
    double nh = sh, nl = sl, dh = ch, dl = cl, sign = 1.0;
    if (q & 1) { nh = ch; nl = cl; dh = sh; dl = sl; sign = -1.0; }
    double quo = nh / dh;
    double prod, perr;
    pct_two_prod(quo, dh, &prod, &perr);
    double rem = (((nh - prod) - perr) + nl) - quo * dl;
    return sign * (quo + rem / dh);
}

/* ---- log ------------------------------------------------------------------ */
PCT_FN double pct_log(double x) {
    const double LN2_HI = 0.6931471803691238;   /* 32 significant bits */
    const double LN2_LO = 1.9082149292705877e-10;
    if (!(x > 0.0)) return x == 0.0 ? -1.0 / 0.0 : (x - x) / (x - x);
    if (x == 1.0 / 0.0) return x;
    int e;
    double m = frexp(x, &e);                     /* x = m 2^e, m in [0.5,1) */
    if (m < 0.7071067811865476) { m = m * 2.0; e -= 1; }
    double f = m - 1.0;                          /* exact */
    double s = f / (2.0 + f);
    double z = s * s;
    /* R(z) = sum_{n>=1} 2 z^n / (2n+1) */
    double R = 0.08695652173913043;              /* 2/23 */
    R = R * z + 0.09523809523809523;             /* 2/21 */
    R = R * z + 0.10526315789473684;             /* 2/19 */
    R = R * z + 0.11764705882352941;             /* 2/17 */
    R = R * z + 0.13333333333333333;             /* 2/15 */
    R = R * z + 0.15384615384615385;             /* 2/13 */
    R = R * z + 0.18181818181818182;             /* 2/11 */
    R = R * z + 0.2222222222222222;              /* 2/9 */
    R = R * z + 0.2857142857142857;              /* 2/7 */
    R = R * z + 0.4;                             /* 2/5 */
    R = R * z + 0.6666666666666666;              /* 2/3 */
    R = R * z;
    double hfsq = 0.5 * f * f;
    double dk = (double)e;
    return dk * LN2_HI + (f - (hfsq - (s * (hfsq + R) + dk * LN2_LO)));
}

/* ---- atan / atan2 ------------------------------------------------------------ */
PCT_FN double pct_atan_poly(double u) { /* |u| <= ~0.2 */
    double z = u * u;
    double p = -0.043478260869565216;            /* -1/23 */
    p = p * z + 0.047619047619047616;            /*  1/21 */
    p = p * z + (-0.05263157894736842);          /* -1/19 */
    p = p * z + 0.058823529411764705;            /*  1/17 */
    p = p * z + (-0.06666666666666667);          /* -1/15 */
    p = p * z + 0.07692307692307693;             /*  1/13 */
    p = p * z + (-0.09090909090909091);          /* -1/11 */
    p = p * z + 0.1111111111111111;              /*  1/9 */
    p = p * z + (-0.14285714285714285);          /* -1/7 */
    p = p * z + 0.2;                             /*  1/5 */
    p = p * z + (-0.3333333333333333);           /* -1/3 */
    return u + u * (z * p);
}
/* atan(t) for t >= 0 (t may be +inf): atan(t) = atan(c) + atan((t-c)/(1+tc))
 * with c in {1/4, 1/2, 1, 3/2, 3, inf}, which keeps |u| <= 0.2. */
PCT_FN double pct_atan_pos(double t) {
    double hi, lo, u;
    if (t < 0.125) return pct_atan_poly(t);
    if (t < 0.375) { hi = 0.24497866312686414; lo = 1.0698755618734451e-17; u = (4.0 * t - 1.0) / (4.0 + t); }
    else if (t < 0.6875) { hi = 0.4636476090008061; lo = 2.2698777452961687e-17; u = (2.0 * t - 1.0) / (2.0 + t); }
    else if (t < 1.1875) { hi = 0.7853981633974483; lo = 3.061616997868383e-17; u = (t - 1.0) / (t + 1.0); }
    else if (t < 2.4375) { hi = 0.982793723247329; lo = 1.3903311031230998e-17; u = (t - 1.5) / (1.0 + 1.5 * t); }
    else if (t < 5.0) { hi = 1.2490457723982544; lo = -2.196203799612311e-18; u = (t - 3.0) / (1.0 + 3.0 * t); }
    else { hi = PCT_PIO2_HI; lo = PCT_PIO2_LO; u = -1.0 / t; }
    return hi + (pct_atan_poly(u) + lo);
}
/* atan2 with the C99 special-value rules for zero arguments. */
PCT_FN double pct_atan2(double y, double x) {
    double ay = y < 0 ? -y : y, ax = x < 0 ? -x : x;
    int yneg = y < 0 || (y == 0.0 && 1.0 / y < 0);
    int xneg = x < 0 || (x == 0.0 && 1.0 / x < 0);
    double a;
    if (ay == 0.0) {
        a = xneg ? PCT_PI : 0.0;
    } else if (ax == 0.0) {
        a = PCT_PIO2_HI;
    } else if (ay <= ax) {
        double base = pct_atan_pos(ay / ax);
        a = xneg ? (PCT_PI - base) + PCT_PI_LO : base;
    } else {
        double base = pct_atan_pos(ax / ay);
        a = xneg ? (PCT_PIO2_HI + base) + PCT_PIO2_LO : (PCT_PIO2_HI - base) + PCT_PIO2_LO;
    }
    return yneg ? -a : a;
}
/* atan2f: binary32 result of the binary64 evaluation. */
PCT_FN float pct_atan2f(float y, float x) { return (float)pct_atan2((double)y, (double)x); }
PCT_FN float pct_sinf(float x) { return (float)pct_sin((double)x); }
PCT_FN float pct_cosf(float x) { return (float)pct_cos((double)x); }

/* C-style double -> int truncation with the x86-64 result (INT_MIN) for NaN
 * and out-of-range values, so oracle and device agree off the happy path. */
PCT_FN int pct_d2i(double d) {
    if (!(d > -2147483649.0 && d < 2147483648.0)) return (int)(-2147483647 - 1);
    return (int)d;
}

#endif /* PCT_MATH_H */
