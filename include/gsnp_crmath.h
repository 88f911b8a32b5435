/*
 * gsnp_crmath.h - correctly rounded exp and log10 for the per-site calling math.
 *
 * The reference evaluates three transcendental functions per site inside its
 * posterior kernel, all with the CUDA device library:
 *   - log10 of the genotype prior            (kernel/posterior_kernel.cu:763)
 *   - log10 of the rank-sum p-value          (kernel/posterior_kernel.cu:837)
 *   - exp in the normal-tail approximation   (kernel/posterior_kernel.cu:461)
 * Neither the CUDA library nor the C library rounds these correctly, so their
 * last bit depends on the implementation.  This build pins them to the
 * correctly rounded result: both the CPU oracle and the sm_103a kernels call the
 * functions below, which evaluate in double-double arithmetic (Dekker 1971
 * splitting, Knuth's TwoSum, FMA-based TwoProduct) with a relative error below
 * 2^-100 and then round once.  The result equals the correctly rounded value
 * unless the exact value lies within 2^-100 (relative) of a rounding midpoint.
 *
 * Every floating-point operation goes through GSNP_D* macros.  On the device
 * these are the _rn intrinsics, which the compiler never fuses; host code must
 * be compiled with -ffp-contract=off.  The same inputs therefore give the same
 * bits on x86-64, aarch64 and sm_103a.
 *
 * exp is evaluated for |x| <= 708 (normal results); larger magnitudes return
 * +inf or 0.  The callers only evaluate exp(-z*z/2) with |z| <= 6.
 */
#ifndef GSNP_CRMATH_H
#define GSNP_CRMATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define GSNP_HD __host__ __device__ __forceinline__
#else
#define GSNP_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define GSNP_DADD(a, b) __dadd_rn((a), (b))
#define GSNP_DSUB(a, b) __dsub_rn((a), (b))
#define GSNP_DMUL(a, b) __dmul_rn((a), (b))
#define GSNP_DDIV(a, b) __ddiv_rn((a), (b))
#define GSNP_FMA(a, b, c) __fma_rn((a), (b), (c))
#else
#define GSNP_DADD(a, b) ((a) + (b))
#define GSNP_DSUB(a, b) ((a) - (b))
#define GSNP_DMUL(a, b) ((a) * (b))
#define GSNP_DDIV(a, b) ((a) / (b))
#define GSNP_FMA(a, b, c) fma((a), (b), (c))
#endif

typedef struct { double hi, lo; } gsnp_dd;

GSNP_HD gsnp_dd gsnp_dd_make(double hi, double lo) { gsnp_dd r; r.hi = hi; r.lo = lo; return r; }

/* s + e == a + b exactly */
GSNP_HD gsnp_dd gsnp_two_sum(double a, double b) {
    double s = GSNP_DADD(a, b);
    double bb = GSNP_DSUB(s, a);
    double e = GSNP_DADD(GSNP_DSUB(a, GSNP_DSUB(s, bb)), GSNP_DSUB(b, bb));
    return gsnp_dd_make(s, e);
}

/* requires |a| >= |b| */
GSNP_HD gsnp_dd gsnp_fast_two_sum(double a, double b) {
    double s = GSNP_DADD(a, b);
    double e = GSNP_DSUB(b, GSNP_DSUB(s, a));
    return gsnp_dd_make(s, e);
}

/* p + e == a * b exactly */
GSNP_HD gsnp_dd gsnp_two_prod(double a, double b) {
    double p = GSNP_DMUL(a, b);
    double e = GSNP_FMA(a, b, -p);
    return gsnp_dd_make(p, e);
}

GSNP_HD gsnp_dd gsnp_dd_add(gsnp_dd x, gsnp_dd y) {
    gsnp_dd s = gsnp_two_sum(x.hi, y.hi);
    gsnp_dd t = gsnp_two_sum(x.lo, y.lo);
    double e = GSNP_DADD(s.lo, t.hi);
    gsnp_dd u = gsnp_fast_two_sum(s.hi, e);
    e = GSNP_DADD(u.lo, t.lo);
    return gsnp_fast_two_sum(u.hi, e);
}

GSNP_HD gsnp_dd gsnp_dd_neg(gsnp_dd x) { return gsnp_dd_make(-x.hi, -x.lo); }

GSNP_HD gsnp_dd gsnp_dd_sub(gsnp_dd x, gsnp_dd y) { return gsnp_dd_add(x, gsnp_dd_neg(y)); }

GSNP_HD gsnp_dd gsnp_dd_mul(gsnp_dd x, gsnp_dd y) {
    gsnp_dd p = gsnp_two_prod(x.hi, y.hi);
    double c = GSNP_DADD(GSNP_DMUL(x.hi, y.lo), GSNP_DMUL(x.lo, y.hi));
    double e = GSNP_DADD(p.lo, c);
    return gsnp_fast_two_sum(p.hi, e);
}

GSNP_HD gsnp_dd gsnp_dd_mul_d(gsnp_dd x, double d) {
    gsnp_dd p = gsnp_two_prod(x.hi, d);
    double e = GSNP_DADD(p.lo, GSNP_DMUL(x.lo, d));
    return gsnp_fast_two_sum(p.hi, e);
}

GSNP_HD gsnp_dd gsnp_dd_div(gsnp_dd x, gsnp_dd y) {
    double q1 = GSNP_DDIV(x.hi, y.hi);
    gsnp_dd r = gsnp_dd_sub(x, gsnp_dd_mul_d(y, q1));
    double q2 = GSNP_DDIV(r.hi, y.hi);
    r = gsnp_dd_sub(r, gsnp_dd_mul_d(y, q2));
    double q3 = GSNP_DDIV(r.hi, y.hi);
    gsnp_dd q = gsnp_fast_two_sum(q1, q2);
    return gsnp_dd_add(q, gsnp_dd_make(q3, 0.0));
}

/* ln 2 split so that k * GSNP_LN2_A is exact for |k| < 2^15 */
#define GSNP_LN2_A 0x1.62e42fefa3800p-1
#define GSNP_LN2_B 0x1.ef35793c76730p-45
#define GSNP_LN2_C 0x1.f97b57a079a19p-103
/* ln 2 and 1/ln 10 as double-double pairs (about 106 bits) */
#define GSNP_LN2_HI 0x1.62e42fefa39efp-1
#define GSNP_LN2_LO 0x1.abc9e3b39803fp-56
#define GSNP_INVLN10_HI 0x1.bcb7b1526e50ep-2
#define GSNP_INVLN10_LO 0x1.95355baaafad3p-57
#define GSNP_INVLN2 0x1.71547652b82fep+0

/* 1/(2k+1) for k = 0..21 as double-double pairs (atanh series of log) */
#define GSNP_ATANH_COEF { \
    {0x1.0000000000000p+0, 0x0.0p+0}, \
    {0x1.5555555555555p-2, 0x1.5555555555555p-56}, \
    {0x1.999999999999ap-3, -0x1.999999999999ap-57}, \
    {0x1.2492492492492p-3, 0x1.2492492492492p-57}, \
    {0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58}, \
    {0x1.745d1745d1746p-4, -0x1.745d1745d1746p-59}, \
    {0x1.3b13b13b13b14p-4, -0x1.3b13b13b13b14p-58}, \
    {0x1.1111111111111p-4, 0x1.1111111111111p-60}, \
    {0x1.e1e1e1e1e1e1ep-5, 0x1.e1e1e1e1e1e1ep-61}, \
    {0x1.af286bca1af28p-5, 0x1.af286bca1af28p-59}, \
    {0x1.8618618618618p-5, 0x1.8618618618618p-59}, \
    {0x1.642c8590b2164p-5, 0x1.642c8590b2164p-60}, \
    {0x1.47ae147ae147bp-5, -0x1.eb851eb851eb8p-61}, \
    {0x1.2f684bda12f68p-5, 0x1.2f684bda12f68p-59}, \
    {0x1.1a7b9611a7b96p-5, 0x1.1a7b9611a7b96p-61}, \
    {0x1.0842108421084p-5, 0x1.0842108421084p-60}, \
    {0x1.f07c1f07c1f08p-6, -0x1.f07c1f07c1f08p-61}, \
    {0x1.d41d41d41d41dp-6, 0x1.0750750750750p-60}, \
    {0x1.bacf914c1bad0p-6, -0x1.bacf914c1bad0p-60}, \
    {0x1.a41a41a41a41ap-6, 0x1.0690690690690p-60}, \
    {0x1.8f9c18f9c18fap-6, -0x1.f3831f3831f38p-61}, \
    {0x1.7d05f417d05f4p-6, 0x1.7d05f417d05f4p-62} \
}
/* 1/n for n = 0..9 (entries 0 and 1 unused) as double-double pairs (Taylor series of expm1) */
#define GSNP_INV_N_COEF { \
    {0.0, 0.0}, \
    {0.0, 0.0}, \
    {0x1.0000000000000p-1, 0.0}, \
    {0x1.5555555555555p-2, 0x1.5555555555555p-56}, \
    {0x1.0000000000000p-2, 0.0}, \
    {0x1.999999999999ap-3, -0x1.999999999999ap-57}, \
    {0x1.5555555555555p-3, 0x1.5555555555555p-57}, \
    {0x1.2492492492492p-3, 0x1.2492492492492p-57}, \
    {0x1.0000000000000p-3, 0.0}, \
    {0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58} \
}

GSNP_HD double gsnp_bits_to_double(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
GSNP_HD uint64_t gsnp_double_to_bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

/* 2^k for -1022 <= k <= 1023 */
GSNP_HD double gsnp_pow2(int k) { return gsnp_bits_to_double((uint64_t)(k + 1023) << 52); }

/* exp(x), correctly rounded for |x| <= 708 */
GSNP_HD double gsnp_cr_exp(double x) {
    if (x != x) return x;
    if (x > 708.0) return HUGE_VAL;
    if (x < -708.0) return 0.0;
    if (x == 0.0) return 1.0;
    /* k = nearest integer to x / ln 2 (any nearby integer works) */
    double kd = GSNP_DMUL(x, GSNP_INVLN2);
    kd = (kd >= 0.0) ? floor(GSNP_DADD(kd, 0.5)) : -floor(GSNP_DADD(-kd, 0.5));
    int k = (int)kd;
    /* r = x - k ln 2 in double-double; x - k*A is exact (Sterbenz) */
    double t1 = GSNP_DSUB(x, GSNP_DMUL(kd, GSNP_LN2_A));
    gsnp_dd r = gsnp_dd_sub(gsnp_dd_make(t1, 0.0), gsnp_two_prod(kd, GSNP_LN2_B));
    r = gsnp_dd_sub(r, gsnp_dd_make(GSNP_DMUL(kd, GSNP_LN2_C), 0.0));
    /* r' = r / 2^10, |r'| < 3.4e-4; expm1(r') by its Taylor series to degree 9 */
    gsnp_dd rp = gsnp_dd_make(GSNP_DMUL(r.hi, 0x1p-10), GSNP_DMUL(r.lo, 0x1p-10));
    const double inv_n[10][2] = GSNP_INV_N_COEF;
    gsnp_dd s = gsnp_dd_make(1.0, 0.0);
    for (int n = 9; n >= 2; --n) {
        /* s = 1 + r'/n * s */
        s = gsnp_dd_mul(s, rp);
        s = gsnp_dd_mul(s, gsnp_dd_make(inv_n[n][0], inv_n[n][1]));
        s = gsnp_dd_add(gsnp_dd_make(1.0, 0.0), s);
    }
    s = gsnp_dd_mul(s, rp); /* expm1(r') */
    /* expm1(2y) = 2 expm1(y) + expm1(y)^2, applied 10 times */
    for (int i = 0; i < 10; ++i) {
        gsnp_dd sq = gsnp_dd_mul(s, s);
        s = gsnp_dd_add(gsnp_dd_make(GSNP_DMUL(s.hi, 2.0), GSNP_DMUL(s.lo, 2.0)), sq);
    }
    gsnp_dd e = gsnp_dd_add(gsnp_dd_make(1.0, 0.0), s);
    /* e.hi is the correctly rounded value of e.hi + e.lo; scale by 2^k */
    if (k > 1000) return GSNP_DMUL(GSNP_DMUL(e.hi, gsnp_pow2(1000)), gsnp_pow2(k - 1000));
    if (k < -1000) return GSNP_DMUL(GSNP_DMUL(e.hi, gsnp_pow2(-1000)), gsnp_pow2(k + 1000));
    return GSNP_DMUL(e.hi, gsnp_pow2(k));
}

/* log10(x), correctly rounded */
GSNP_HD double gsnp_cr_log10(double x) {
    if (x != x) return x;
    if (x < 0.0) return (x - x) / (x - x);
    if (x == 0.0) return -HUGE_VAL;
    if (x == HUGE_VAL) return x;
    int e = 0;
    uint64_t u = gsnp_double_to_bits(x);
    if ((u >> 52) == 0) { /* subnormal: scale into the normal range */
        u = gsnp_double_to_bits(GSNP_DMUL(x, 0x1p54));
        e = -54;
    }
    e += (int)((u >> 52) & 0x7FF) - 1023;
    double m = gsnp_bits_to_double((u & 0x000FFFFFFFFFFFFFULL) | 0x3FF0000000000000ULL);
    if (m > 1.4142135623730951) { m = GSNP_DMUL(m, 0.5); e += 1; }
    if (m == 1.0 && e == 0) return 0.0;
    /* log m = 2 atanh(s), s = (m-1)/(m+1), |s| <= 0.1716 */
    gsnp_dd num = gsnp_dd_make(GSNP_DSUB(m, 1.0), 0.0);
    gsnp_dd den = gsnp_two_sum(m, 1.0);
    gsnp_dd s = gsnp_dd_div(num, den);
    gsnp_dd s2 = gsnp_dd_mul(s, s);
    const double coef[22][2] = GSNP_ATANH_COEF;
    gsnp_dd acc = gsnp_dd_make(coef[21][0], coef[21][1]);
    for (int k = 20; k >= 0; --k) {
        acc = gsnp_dd_mul(acc, s2);
        acc = gsnp_dd_add(acc, gsnp_dd_make(coef[k][0], coef[k][1]));
    }
    gsnp_dd lm = gsnp_dd_mul(acc, s);
    lm = gsnp_dd_make(GSNP_DMUL(lm.hi, 2.0), GSNP_DMUL(lm.lo, 2.0));
    gsnp_dd le = gsnp_dd_mul_d(gsnp_dd_make(GSNP_LN2_HI, GSNP_LN2_LO), (double)e);
    gsnp_dd l = gsnp_dd_add(le, lm);
    gsnp_dd r = gsnp_dd_mul(l, gsnp_dd_make(GSNP_INVLN10_HI, GSNP_INVLN10_LO));
    return r.hi;
}

#endif /* GSNP_CRMATH_H */
