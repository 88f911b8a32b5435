/*
 * fmt_g6.h - printf("%#.6g") of a double, exactly, on the host and the device.
 *
 * The cns text prints rank-sum p-values and copy ratios through an iostream
 * with showpoint and the default precision (cpp/call_genotype.cc:404-406),
 * which is C's %#.6g: six significant digits correctly rounded (ties to
 * even) from the double's exact binary value, fixed notation when the
 * decimal exponent X of the rounded value satisfies -4 <= X < 6, scientific
 * otherwise, trailing zeros and the decimal point kept.
 *
 * v = m * 2^e exactly; the six digits are v * 10^(5-X) rounded to an integer,
 * computed exactly as (m * 5^(5-X)) * 2^(e+5-X) in 128-bit integer arithmetic.
 * That covers every v with 5 - X in [0, 32] (1e-27 < v < 1e6, plus 0), which
 * includes every value the cns text prints (rank-sum p-values in [0, 1],
 * copy ratios below 65536); fmt_g6 returns 0 outside that range.
 */
#ifndef GSNP_FMT_G6_H
#define GSNP_FMT_G6_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define GSNP_FMT_HD __host__ __device__ __forceinline__
#else
#define GSNP_FMT_HD inline
#endif

namespace gsnp {

typedef unsigned __int128 u128;

/* floor(v * 10^k) and whether the dropped fraction is >, = or < one half
 * (cmp = 1, 0, -1); false when the exact value does not fit */
GSNP_FMT_HD bool scaled_digits(uint64_t m, int e, int k, u128* q, int* cmp) {
    if (k < 0 || k > 32) return false;
    u128 n = m;
    for (int i = 0; i < k; ++i) n *= 5u;   /* m < 2^53, 5^32 < 2^75 */
    const int s = e + k;
    if (s >= 0) {
        if (s > 20) return false;
        *q = n << s;
        *cmp = -1;
        return true;
    }
    if (-s > 127) {
        *q = 0;
        *cmp = -1;
        return true;
    }
    const int r = -s;
    *q = n >> r;
    const u128 rem = n & (((u128)1 << r) - 1);
    const u128 half = (u128)1 << (r - 1);
    *cmp = rem > half ? 1 : (rem == half ? 0 : -1);
    return true;
}

/* Writes the text of printf("%#.6g", v) to out (at least 16 bytes) and
 * returns its length, or 0 when v is outside the supported range. */
GSNP_FMT_HD int fmt_g6(double v, char* out) {
    uint64_t bits;
    memcpy(&bits, &v, 8);
    int len = 0;
    if (bits >> 63) {
        out[len++] = '-';
        bits &= ~(1ull << 63);
    }
    const int bexp = (int)(bits >> 52);
    uint64_t m = bits & ((1ull << 52) - 1);
    if (bexp == 0x7ff) return 0;
    if (bexp == 0 && m == 0) {
        const char z[] = "0.00000";
        for (int i = 0; i < 7; ++i) out[len++] = z[i];
        return len;
    }
    int e;
    if (bexp == 0) {
        e = -1074;
    } else {
        m |= 1ull << 52;
        e = bexp - 1075;
    }
    /* binary exponent of the leading bit, then a decimal estimate */
    int lead = 63;
    while (!((m >> lead) & 1)) --lead;
    const int E2 = e + lead;
    int X = (E2 >= 0) ? (E2 * 30103) / 100000 : -((-E2 * 30103 + 99999) / 100000);
    u128 q = 0;
    int cmp = -1;
    for (int it = 0; it < 4; ++it) {
        if (!scaled_digits(m, e, 5 - X, &q, &cmp)) return 0;
        if (q < (u128)100000) { --X; continue; }
        if (q >= (u128)1000000) { ++X; continue; }
        break;
    }
    if (q < (u128)100000 || q >= (u128)1000000) return 0;
    uint32_t d = (uint32_t)q;
    if (cmp > 0 || (cmp == 0 && (d & 1))) ++d;
    bool point_only = false;
    if (d == 1000000) {
        d = 100000;
        ++X;
        /* the C library keeps the fraction digits of the unrounded fixed
         * form when rounding carries into scientific form: 999999.5 prints
         * as "1.e+06" */
        point_only = X == 6;
    }
    char dig[6];
    for (int i = 5; i >= 0; --i) {
        dig[i] = (char)('0' + d % 10);
        d /= 10;
    }
    if (X >= -4 && X < 6) {
        if (X >= 0) {
            for (int i = 0; i <= X; ++i) out[len++] = dig[i];
            out[len++] = '.';
            for (int i = X + 1; i < 6; ++i) out[len++] = dig[i];
        } else {
            out[len++] = '0';
            out[len++] = '.';
            for (int i = 0; i < -X - 1; ++i) out[len++] = '0';
            for (int i = 0; i < 6; ++i) out[len++] = dig[i];
        }
    } else {
        out[len++] = dig[0];
        out[len++] = '.';
        if (!point_only)
            for (int i = 1; i < 6; ++i) out[len++] = dig[i];
        out[len++] = 'e';
        int x = X;
        out[len++] = x < 0 ? '-' : '+';
        if (x < 0) x = -x;
        if (x >= 100) {
            out[len++] = (char)('0' + x / 100);
            x %= 100;
            out[len++] = (char)('0' + x / 10);
            out[len++] = (char)('0' + x % 10);
        } else {
            out[len++] = (char)('0' + x / 10);
            out[len++] = (char)('0' + x % 10);
        }
    }
    return len;
}

}  // namespace gsnp

#endif
