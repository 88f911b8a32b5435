/*
 * site_math.cuh - per-site arithmetic of the caller shared by every calling
 * kernel: the FP64 and FP32 likelihood sums over the dependency-adjusted
 * record walk (column.cuh), the rank-sum test and the posterior.
 *
 * A site's records are 32-bit words in ascending order, `stride` words apart
 * (the tile kernels keep them in a [slot][site] column).
 *
 * Outside nvcc (the CPU checks of this arithmetic) the device intrinsics it
 * uses are the host's own IEEE operations, each rounded to nearest like the
 * _rn intrinsics; host code is built with -ffp-contract=off so that no
 * multiply and add are fused.
 */
#ifndef GSNP_SITE_MATH_CUH
#define GSNP_SITE_MATH_CUH

#include <math.h>
#include <stdint.h>

#if !defined(__CUDACC__)
#include <string.h>

#include <vector_types.h>   /* float4, double2 and the function qualifiers */
#ifndef __noinline__
#define __noinline__          /* only device code size depends on it */
#endif
static inline float __fadd_rn(float x, float y) { return x + y; }
static inline float __fsub_rn(float x, float y) { return x - y; }
static inline float __fmul_rn(float x, float y) { return x * y; }
static inline int __float2int_rz(float x) { return (int)x; }
static inline double __dsqrt_rn(double x) { return sqrt(x); }
static inline long long __double_as_longlong(double x) {
    long long v;
    memcpy(&v, &x, sizeof v);
    return v;
}
template <class T>
static inline T __ldg(const T* p) { return *p; }
#endif

#include "calling.cuh"
#include "column.cuh"

namespace gsnp {

/* SiteCall.flags */
constexpr uint8_t kCallFixup = 1;    /* the FP32 likelihood was recomputed in FP64 */
constexpr uint8_t kCallNormal = 2;   /* the rank-sum took the normal approximation */
constexpr uint8_t kCallPending = 4;  /* transient: left to the FP64 pass */
constexpr uint8_t kCallSampled = 8;  /* transient: FP32 accuracy sample */

/* Error bound factor of the FP32 likelihood sums (likelihood_fp32). */
#define GSNP_FP32_K(n) (6.0 * 0x1p-24 + (double)(n) * 0x1p-45)

__device__ __forceinline__ int64_t lower_bound_g(const int32_t* a, int64_t n, int64_t v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)__ldg(a + mid) < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

struct SitePileup {
    int cu[4], qs[4];
    uint32_t ca[4];
    uint32_t depth, repeat;
    int dep_uni, num;
};

/* The pileup counts of one site in 32 bytes: count_uni 4 x 8 bits (at most
 * 255 unique bases), q_sum and count_all 4 x 16 bits. */
struct PackedPileup {
    uint64_t qs4, ca4;
    uint32_t cu4, depth, repeat;
    uint16_t dep_uni, num;
    __host__ __device__ SitePileup unpack() const {
        SitePileup p;
        for (int i = 0; i < 4; ++i) {
            p.cu[i] = (int)((cu4 >> (8 * i)) & 0xff);
            p.qs[i] = (int)((qs4 >> (16 * i)) & 0xffff);
            p.ca[i] = (uint32_t)((ca4 >> (16 * i)) & 0xffff);
        }
        p.depth = depth;
        p.repeat = repeat;
        p.dep_uni = dep_uni;
        p.num = num;
        return p;
    }
};
static_assert(sizeof(PackedPileup) == 32, "PackedPileup is 32 bytes");

/* FP64 sums in the reference's order: the plain form and the fixup */
template <int BITS = 1>
__device__ __forceinline__ void likelihood_fp64(const CallArgs& a, const uint32_t* recs, uint32_t* seen, int stride,
                                                int num, double* tl) {
    double s[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) s[i] = 0.0;
    walk_records<false, BITS>(a, recs, seen, stride, num, [&](int, int qa, int coord, int o) {
        const double2* row = reinterpret_cast<const double2*>(a.lik64 + ((size_t)(qa * a.L + coord) * 4 + o) * 10);
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const double2 x = __ldg(row + v);
            s[2 * v] = GSNP_DADD(s[2 * v], x.x);
            s[2 * v + 1] = GSNP_DADD(s[2 * v + 1], x.y);
        }
    });
#pragma unroll
    for (int i = 0; i < 10; ++i) tl[genotype_of(i)] = s[i];
}

/* FP32 compensated sums: groups of four consecutive terms are added pairwise,
 * ((x0 + x1) + (x2 + x3)), and each group sum is Kahan-summed.  Every term is
 * <= 0 (the host checks the table), so sum|x| = |S|, and
 * |S32 - S64| <= |S32| * GSNP_FP32_K(n): the rounding of each term to FP32
 * (u), of the two levels of each group (2u), the compensated sum
 * (2u + O(n u^2)) and the FP64 sum's own rounding (n 2^-53), u = 2^-24, with
 * one u of slack. */
struct Kahan10 {
    float s[10], c[10];
    __device__ __forceinline__ void init() {
#pragma unroll
        for (int i = 0; i < 10; ++i) { s[i] = 0.f; c[i] = 0.f; }
    }
    __device__ __forceinline__ void add(const float* x) {
#pragma unroll
        for (int v = 0; v < 10; ++v) {
            const float y = __fsub_rn(x[v], c[v]);
            const float t = __fadd_rn(s[v], y);
            c[v] = __fsub_rn(__fsub_rn(t, s[v]), y);
            s[v] = t;
        }
    }
};

/* The ten FP32 terms of one table row in two loads: columns 0-7 with one
 * 256-bit load (a.lik32 rows are 32 bytes on a 32-byte boundary), columns 8-9
 * with one 64-bit load.  Table rows are read at random by the lanes of a warp,
 * and the L1 data stage takes about one wavefront per lane and load
 * instruction, so the number of loads per row, not their width, sets its
 * cost. */
__device__ __forceinline__ void lik32_row(const CallArgs& a, int qa, int coord, int o, float* x) {
    const size_t r = (size_t)(qa * a.L + coord) * 4 + o;
#ifdef __CUDA_ARCH__
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(x[0]), "=f"(x[1]), "=f"(x[2]), "=f"(x[3]), "=f"(x[4]), "=f"(x[5]), "=f"(x[6]), "=f"(x[7])
        : "l"(a.lik32 + r * 8));
#else
    for (int v = 0; v < 8; ++v) x[v] = a.lik32[r * 8 + v];
#endif
    const float2 t = __ldg(reinterpret_cast<const float2*>(a.lik32b) + r);
    x[8] = t.x;
    x[9] = t.y;
}

template <int BITS = 1>
__device__ __forceinline__ void likelihood_fp32(const CallArgs& a, const uint32_t* recs, uint32_t* seen, int stride,
                                                int num, double* tl, double* eps) {
    Kahan10 k;
    k.init();
    float g0[10], g1[10];
    int pos = 0;   /* position of the next term in its group of four */
    walk_records<false, BITS>(a, recs, seen, stride, num, [&](int, int qa, int coord, int o) {
        float x[10];
        lik32_row(a, qa, coord, o, x);
        switch (pos) {
            case 0:
#pragma unroll
                for (int v = 0; v < 10; ++v) g0[v] = x[v];
                break;
            case 1:
#pragma unroll
                for (int v = 0; v < 10; ++v) g0[v] = __fadd_rn(g0[v], x[v]);
                break;
            case 2:
#pragma unroll
                for (int v = 0; v < 10; ++v) g1[v] = x[v];
                break;
            default:
#pragma unroll
                for (int v = 0; v < 10; ++v) g0[v] = __fadd_rn(g0[v], __fadd_rn(g1[v], x[v]));
                k.add(g0);
                break;
        }
        pos = (pos + 1) & 3;
    });
    if (pos == 3) {
#pragma unroll
        for (int v = 0; v < 10; ++v) g0[v] = __fadd_rn(g0[v], g1[v]);
    }
    if (pos != 0) k.add(g0);
    const double kk = GSNP_FP32_K(num);
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        const int g = genotype_of(i);
        tl[g] = (double)k.s[i];
        eps[g] = isinf(tl[g]) ? 0.0 : fabs(tl[g]) * kk;
    }
}

/* ------------------------------------------------------------------------ */
/* rank-sum test (kernel/posterior_kernel.cu:429-572)                         */
/* ------------------------------------------------------------------------ */

__device__ __forceinline__ double table_test(const double* pr, int n1, int n2, double T1, double T2) {
    /* kernel/posterior_kernel.cu:430-443: the interpolation index shifts the
     * total by 16 bits, as the reference does */
    if (n1 <= n2) {
        const int i1 = (n1 + n2) << 17 | n1 << 11 | (int)(T1);
        const int i2 = (n1 + n2) << 16 | n1 << 11 | (int)(T1 + 1);
        const double p1 = __ldg(pr + i1), p2 = __ldg(pr + i2);
        return GSNP_DADD(p1, GSNP_DMUL(GSNP_DSUB(T1, (double)(int)T1), GSNP_DSUB(p2, p1)));
    }
    const int i3 = (n1 + n2) << 17 | n2 << 11 | (int)(T2);
    const int i4 = (n1 + n2) << 16 | n2 << 11 | (int)(T2 + 1);
    const double p3 = __ldg(pr + i3), p4 = __ldg(pr + i4);
    return GSNP_DADD(p3, GSNP_DMUL(GSNP_DSUB(T2, (double)(int)T2), GSNP_DSUB(p4, p3)));
}

__device__ __forceinline__ double normal_value(double z) {
    if (z > 6.0 || z < -6.0) return 0.0;
    const double b1 = 0.31938153, b2 = -0.356563782, b3 = 1.781477937, b4 = -1.821255978,
                 b5 = 1.330274429, p = 0.2316419, c2 = 0.39894228;
    const double aa = fabs(z);
    const double t = GSNP_DDIV(1.0, GSNP_DADD(1.0, GSNP_DMUL(aa, p)));
    /* z / 2 is computed as z * 0.5: halving is exact, so the value is the same */
    const double b = GSNP_DMUL(c2, gsnp_cr_exp(GSNP_DMUL(-z, GSNP_DMUL(z, 0.5))));
    double n = GSNP_DADD(GSNP_DMUL(b5, t), b4);
    n = GSNP_DADD(GSNP_DMUL(n, t), b3);
    n = GSNP_DADD(GSNP_DMUL(n, t), b2);
    n = GSNP_DADD(GSNP_DMUL(n, t), b1);
    n = GSNP_DMUL(n, t);
    n = GSNP_DSUB(1.0, GSNP_DMUL(b, n));
    if (z < 0.0) n = GSNP_DSUB(1.0, n);
    return n > 0.5 ? GSNP_DSUB(1.0, n) : n;
}

__device__ __forceinline__ double normal_test(int n1, int n2, double T1, double T2) {
    const double sd = __dsqrt_rn(GSNP_DDIV((double)(n1 * n2 * (n1 + n2 + 1)), 12.0));
    const double u1 = GSNP_DDIV(GSNP_DSUB(T1, (double)(n1 * (n1 + n2 + 1) / 2)), sd);
    const double u2 = GSNP_DDIV(GSNP_DSUB(T2, (double)(n2 * (n1 + n2 + 1) / 2)), sd);
    return normal_value(fabs(u1) > fabs(u2) ? u1 : u2);
}

/* Wilcoxon rank-sum p-value of a heterozygous call (kernel/posterior_kernel.cu:506-572) */
__device__ __noinline__ double rank_test(const double* p_rank, int q_max_min, const uint32_t* recs, int stride,
                                         int num, const int* cu, int bt, bool* normal_path) {
    const int ia = bt & 3, ib = (bt >> 2) & 3;
    if (ia == ib) return 1.0;
    if (cu[ia] == 0 || cu[ib] == 0) return 0.0;
    int ca[65], cb[65];
    for (int i = 0; i < 65; ++i) { ca[i] = 0; cb[i] = 0; }
    for (int i = 0; i < num; ++i) {
        const uint32_t w = recs[i * stride];
        const int o = rec_base(w);
        if (o == ia) ca[rec_q(w)] += rec_occ(w);
        else if (o == ib) cb[rec_q(w)] += rec_occ(w);
    }
    /* rank of quality q among both alleles, ties averaged; qualities above
     * q_max - q_min + 1 keep rank 0 as in the reference */
    double Ta = 0.0, Tb = 0.0;
    int rank = 0;
    const int top = q_max_min + 1 < 64 ? q_max_min + 1 : 64;
    for (int q = 0; q <= top; ++q) {
        const int c = ca[q] + cb[q];
        /* an empty bin adds +0.0 to the non-negative sums: skipping it is
         * exact; (1 + c) / 2 is computed as (1 + c) * 0.5, which is exact */
        if (c == 0) continue;
        const double ra = GSNP_DADD((double)rank, GSNP_DMUL((double)(1 + c), 0.5));
        Ta = GSNP_DADD(Ta, GSNP_DMUL(ra, (double)ca[q]));
        Tb = GSNP_DADD(Tb, GSNP_DMUL(ra, (double)cb[q]));
        rank += c;
    }
    const int n1 = cu[ia], n2 = cu[ib];
    if (n1 + n2 < 64) return table_test(p_rank, n1, n2, Ta, Tb);
    *normal_path = true;
    return normal_test(n1, n2, Ta, Tb);
}

/* ------------------------------------------------------------------------ */
/* posterior (kernel/posterior_kernel.cu:680-864)                             */
/* ------------------------------------------------------------------------ */

/* base1/base2: the two largest q_sum (count_all when no unique base passed),
 * later base winning ties; the reference base fills in for zero counts */
struct TopBases {
    int base1, base2, qual1, qual2, qual3;
};

__device__ __forceinline__ TopBases top_bases(const SitePileup& p, int ori7) {
    TopBases t;
    t.base1 = 0;
    t.base2 = 0;
    t.qual1 = -1;
    t.qual2 = -2;
    t.qual3 = -3;
    if (p.dep_uni) {
#pragma unroll
        for (int i = 0; i != 4; ++i) {
            const int v = p.qs[i];
            if (v >= t.qual1) { t.qual3 = t.qual2; t.base2 = t.base1; t.qual2 = t.qual1; t.base1 = i; t.qual1 = v; }
            else if (v >= t.qual2) { t.qual3 = t.qual2; t.base2 = i; t.qual2 = v; }
            else if (v >= t.qual3) { t.qual3 = v; }
        }
        if (t.qual1 == 0) t.base1 = ori7;
        else if (t.qual2 == 0 && t.base1 != ori7) t.base2 = ori7;
    } else {
        uint32_t c1 = 0, c2 = 0, c3 = 0;
#pragma unroll
        for (int i = 0; i != 4; ++i) {
            const uint32_t v = p.ca[i];
            if (v >= c1) { c3 = c2; t.base2 = t.base1; c2 = c1; t.base1 = i; c1 = v; }
            else if (v >= c2) { c3 = c2; t.base2 = i; c2 = v; }
            else if (v >= c3) { c3 = v; }
        }
        if (c1 == 0) t.base1 = ori7;
        else if (c2 == 0 && t.base1 != ori7) t.base2 = ori7;
    }
    return t;
}

/* consensus-quality clamps of posterior_kernel2 (kernel/posterior_kernel.cu:839-864) */
__device__ __forceinline__ int finalize_q(int q, bool hom, bool het_ok, const TopBases& tb, int type1) {
    if (hom) {
        if (tb.qual1 > 0 && tb.base1 != (type1 & 3)) q = 0;
        else if (q > tb.qual1 - tb.qual2) q = tb.qual1 - tb.qual2;
    } else {
        if (het_ok) {
            if (q > tb.qual2 - tb.qual3) q = tb.qual2 - tb.qual3;
        } else {
            q = 0;
        }
    }
    if (q > 99) q = 99;
    if (q < 0) q = 0;
    return q;
}

__device__ __forceinline__ void fill_call(SiteCall* out, const SitePileup& p, const TopBases& tb, int type1, int q,
                                          bool normal_path, double rs) {
    SiteCall c;
    c.type1 = (uint8_t)type1;
    c.base1 = (uint8_t)tb.base1;
    c.base2 = (uint8_t)tb.base2;
    c.q_cns = (uint8_t)q;
    c.avg_q1 = (tb.base1 < 4 && p.qs[tb.base1] != 0) ? (uint8_t)(p.qs[tb.base1] / p.cu[tb.base1]) : 0;
    c.avg_q2 = (tb.base2 < 4 && p.qs[tb.base2] != 0) ? (uint8_t)(p.qs[tb.base2] / p.cu[tb.base2]) : 0;
    c.flags = normal_path ? kCallNormal : 0;
    c.pad = 0;
    c.cu1 = tb.base1 < 4 ? (uint16_t)p.cu[tb.base1] : 0;
    c.ca1 = tb.base1 < 4 ? (uint16_t)p.ca[tb.base1] : 0;
    c.cu2 = tb.base2 < 4 ? (uint16_t)p.cu[tb.base2] : 0;
    c.ca2 = tb.base2 < 4 ? (uint16_t)p.ca[tb.base2] : 0;
    c.depth = p.depth;
    c.repeat_time = p.repeat;
    c.rank_sum = rs;
    *out = c;
}

__device__ __forceinline__ bool same_call(const SiteCall& x, const SiteCall& y) {
    return x.type1 == y.type1 && x.base1 == y.base1 && x.base2 == y.base2 && x.q_cns == y.q_cns &&
           x.avg_q1 == y.avg_q1 && x.avg_q2 == y.avg_q2 && x.cu1 == y.cu1 && x.ca1 == y.ca1 && x.cu2 == y.cu2 &&
           x.ca2 == y.ca2 && x.depth == y.depth && x.repeat_time == y.repeat_time &&
           __double_as_longlong(x.rank_sum) == __double_as_longlong(y.rank_sum);
}

/* log10 genotype priors of a site by genotype code: the prior table of the
 * reference base, or, for a dbSNP site in refine mode, its row's
 * (precomputed by snp_log_prior_kernel; snp_row is the row of the site) */
__device__ __forceinline__ void load_log_prior(const CallArgs& a, int64_t snp_row, uint8_t ori, double* lp) {
    const double2* src = reinterpret_cast<const double2*>(a.log_prior + ((ori & 7) << 4));
    if ((ori & 0x8) && a.refine) src = reinterpret_cast<const double2*>(a.snp_lp + snp_row * 16);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const double2 v = __ldg(src + i);
        lp[2 * i] = v.x;
        lp[2 * i + 1] = v.y;
    }
}

/* posterior_kernel + posterior_kernel2 for one site.
 *
 * tl holds type_likely and lp the log10 priors, by genotype code.  When eps
 * is given, tl is an FP32 approximation and eps[g] bounds |tl[g] - FP64
 * type_likely[g]|; the function then returns false, writing nothing, unless
 * every decision it makes (the genotype order behind type1/type2 and the
 * truncated, clamped consensus quality) is provably the one the FP64 values
 * give.  nq(b) is q_sum[b] of the next site, which the reference reads when
 * base1/base2 name an N reference base. */
template <bool FAST_LOG = false, class NQ>
__device__ bool site_posterior(const CallArgs& a, uint8_t ori, const SitePileup& p, const double* tl,
                               const double* eps, const double* lp, const uint32_t* recs, int stride, NQ&& nq,
                               SiteCall* out) {
    const TopBases tb = top_bases(p, ori & 7);
    double tp[17];
#pragma unroll
    for (int i = 0; i < 17; ++i) tp[i] = 0.0;
    int type1 = 16, type2 = 16;
#pragma unroll
    for (int a1 = 0; a1 != 4; ++a1)
#pragma unroll
        for (int a2 = a1; a2 != 4; ++a2) {
            const int g = a1 << 2 | a2;
            if (a.monoploid && a1 != a2) continue;
            tp[g] = GSNP_DADD(tl[g], lp[g]);
            if (tp[g] >= tp[type1] || type1 == 16) { type2 = type1; type1 = g; }
            else if (tp[g] >= tp[type2] || type2 == 16) { type2 = g; }
        }
    double ep[16];
    if (eps) {
        /* bound of |tp - tp_FP64|: the likelihood bound plus the rounding of the
         * prior addition; exact (0) where the likelihood is exact */
#pragma unroll
        for (int g = 0; g < 16; ++g)
            ep[g] = eps[g] == 0.0 ? 0.0 : eps[g] + 0x1p-51 * (fabs(tl[g]) + fabs(lp[g])) + 0x1p-1000;
#pragma unroll
        for (int a1 = 0; a1 != 4; ++a1)
#pragma unroll
            for (int a2 = a1; a2 != 4; ++a2) {
                const int g = a1 << 2 | a2;
                if ((a.monoploid && a1 != a2) || g == type1) continue;
                if (ep[g] + ep[type1] > 0.0 && !(tp[type1] - tp[g] > ep[g] + ep[type1])) return false;
                if (g == type2) continue;
                if (ep[g] + ep[type2] > 0.0 && !(tp[type2] - tp[g] > ep[g] + ep[type2])) return false;
            }
    }
    bool normal_path = false;
    const double rs =
        a.rank_sum ? rank_test(a.p_rank, a.q_max_min, recs, stride, p.num, p.cu, type1, &normal_path) : 1.0;
    const bool hom = (type1 & 3) == ((type1 >> 2) & 3);
    bool het_ok = false;
    if (!hom) {
        /* base1/base2 may name an N reference base (4..7): the reference then
         * reads q_sum[4*site + base], i.e. the next site's q_sum[base - 4].
         * With q_sum summing to zero that is never consulted; otherwise
         * (base2 = N code) the next site's value is used. */
        const int comb = tb.base1 < tb.base2 ? (tb.base1 << 2 | tb.base2) : (tb.base2 << 2 | tb.base1);
        het_ok = type1 == comb;
        if (het_ok) het_ok = (tb.base1 < 4 ? p.qs[tb.base1] : nq(tb.base1 - 4)) > 0;
        if (het_ok) het_ok = (tb.base2 < 4 ? p.qs[tb.base2] : nq(tb.base2 - 4)) > 0;
    }
    int q;
    if (rs == 0.0) {
        q = finalize_q(0, hom, het_ok, tb, type1);
    } else {
        const double d = GSNP_DMUL(10.0, GSNP_DSUB(tp[type1], tp[type2]));
        /* FAST_LOG: log10 of the rank-sum value from the CUDA math library,
         * whose error is far below 2^-40 relative; dl bounds the resulting
         * error of raw.  The correctly rounded log10 is evaluated only when
         * raw +- dl could change the truncated, clamped quality. */
        const bool approx = FAST_LOG && rs != 1.0;
        double lg = approx ? log10(rs) : gsnp_cr_log10(rs);
        double raw = GSNP_DADD(d, GSNP_DMUL(10.0, lg));
        const double dl = approx ? 10.0 * fabs(lg) * 0x1p-40 + 0x1p-48 * (fabs(raw) + 1.0) : 0.0;
        q = finalize_q((int)raw, hom, het_ok, tb, type1);
        if (eps && ep[type1] + ep[type2] > 0.0) {
            const double delta =
                10.0 * (ep[type1] + ep[type2]) * (1.0 + 0x1p-20) + 0x1p-48 * (fabs(raw) + 1.0) + dl;
            if (finalize_q((int)(raw - delta), hom, het_ok, tb, type1) !=
                finalize_q((int)(raw + delta), hom, het_ok, tb, type1))
                return false;
        } else if (approx && finalize_q((int)(raw - dl), hom, het_ok, tb, type1) !=
                                 finalize_q((int)(raw + dl), hom, het_ok, tb, type1)) {
            lg = gsnp_cr_log10(rs);
            raw = GSNP_DADD(d, GSNP_DMUL(10.0, lg));
            q = finalize_q((int)raw, hom, het_ok, tb, type1);
        }
    }
    fill_call(out, p, tb, type1, q, normal_path, rs);
    return true;
}

/* The FP32 posterior of the fast kernel, for sites whose best genotype is
 * homozygous (the rank-sum value is then 1 and its log10 0).  s holds the FP32
 * likelihood sums by table column, num the record count, and
 * k_units u + num 2^-45 (u = 2^-24) their relative error bound: 6 for the
 * grouping of likelihood_fp32, 9 for the warp form of the deep kernel (per-
 * lane compensated sums, then a tree of 32).  Returns false, writing
 * nothing, when the best genotype is heterozygous or when the FP32 values do
 * not prove the FP64 decisions.
 *
 * E_g bounds |tp32[g] - tp64[g]| (the likelihood bound, the FP32 rounding of
 * the prior and of the addition).  With v1 = tp32[type1], v2 the largest
 * other tp32 (genotype g2), d = v1 - v2 and B = max over the others of
 * tp32[g] - v2 + E_g:
 *   tp64[type1] - max(other tp64) lies in [d - E1 - B, d + E1 + E_g2],
 * so type1 is the FP64 best when d > E1 + B, and the truncated, clamped
 * quality is proven when it is the same at both ends of that interval.
 * Every quantity is formed as a difference first, so that each FP32 rounding
 * is relative to these small values; the bounds are then grown to cover
 * those roundings. */
__device__ __forceinline__ bool fast_posterior(const CallArgs& a, int64_t snp_row, uint8_t ori, const SitePileup& p,
                                               const float* s, int num, SiteCall* out, float k_units = 6.0f) {
    const int ori7 = ori & 7;
    const float* src = a.log_prior32 + ori7 * 12;
    if ((ori & 0x8) && a.refine) src = a.snp_lp32 + snp_row * 12;
    float lp[10];
    {
        const float4* s4 = reinterpret_cast<const float4*>(src);
        const float4 x0 = __ldg(s4), x1 = __ldg(s4 + 1), x2 = __ldg(s4 + 2);
        lp[0] = x0.x; lp[1] = x0.y; lp[2] = x0.z; lp[3] = x0.w;
        lp[4] = x1.x; lp[5] = x1.y; lp[6] = x1.z; lp[7] = x1.w;
        lp[8] = x2.x; lp[9] = x2.y;
    }
    /* |s - S64| <= |s| k; the prior's rounding <= 2^-24 |lp|; the addition's
     * <= 2^-24 |tp| <= 2^-24 (|s| + |lp|); grown by 2^-20 for the rounding of
     * the bound itself */
    const float kk1 = __fadd_rn(__fadd_rn(k_units * 0x1p-24f, __fmul_rn((float)num, 0x1p-45f)), 0x1p-23f);
    const float grow = 1.0f + 0x1p-20f;
    float tp[10], E[10];
    int t1 = -1;
    float v1 = 0.f;
#pragma unroll
    for (int t = 0; t < 10; ++t) {
        const int g = genotype_of(t);
        tp[t] = __fadd_rn(s[t], lp[t]);
        E[t] = __fmul_rn(__fadd_rn(__fmul_rn(fabsf(s[t]), kk1), __fmul_rn(fabsf(lp[t]), 0x1p-22f)), grow);
        if (a.monoploid && (g >> 2) != (g & 3)) continue;
        if (t1 < 0 || tp[t] >= v1) { t1 = t; v1 = tp[t]; }
    }
    const int g1 = genotype_of(t1);
    if ((g1 >> 2) != (g1 & 3)) return false;
    float e1 = 0.f, v2 = -INFINITY, e2 = 0.f, emax = 0.f;
#pragma unroll
    for (int t = 0; t < 10; ++t) {
        const int g = genotype_of(t);
        if (a.monoploid && (g >> 2) != (g & 3)) continue;
        if (t == t1) {
            e1 = E[t];
            continue;
        }
        if (tp[t] >= v2) { v2 = tp[t]; e2 = E[t]; }
        emax = fmaxf(emax, E[t]);
    }
    float B = 0.f;
#pragma unroll
    for (int t = 0; t < 10; ++t) {
        const int g = genotype_of(t);
        if ((a.monoploid && (g >> 2) != (g & 3)) || t == t1) continue;
        B = fmaxf(B, __fadd_rn(__fsub_rn(tp[t], v2), E[t]));
    }
    /* |fl(tp - v2 + E) - (tp - v2 + E)| <= 2^-23 (|tp - v2| + E) <= 2^-22 E at
     * the maximum, which is covered by emax 2^-21 */
    B = __fmul_rn(__fadd_rn(B, __fmul_rn(emax, 0x1p-21f)), grow);
    if (!(isfinite(v1) && isfinite(v2) && isfinite(B))) return false;
    const float d = __fsub_rn(v1, v2);                       /* error <= 2^-24 |d| */
    const float below = __fmul_rn(__fadd_rn(e1, B), grow);   /* >= E1 + B */
    const float above = __fmul_rn(__fadd_rn(e1, e2), grow);  /* >= E1 + E_g2 */
    if (!(__fsub_rn(__fmul_rn(d, 1.0f - 0x1p-22f), below) > 0.f)) return false;
    const TopBases tb = top_bases(p, ori7);
    const float raw_lo = __fmul_rn(10.f, __fsub_rn(d, below));
    const float raw_hi = __fmul_rn(10.f, __fadd_rn(d, above));
    const float slack = __fmul_rn(__fadd_rn(fabsf(raw_hi), 1.f), 0x1p-19f);
    const int q = finalize_q(__float2int_rz(__fsub_rn(raw_lo, slack)), true, false, tb, g1);
    if (q != finalize_q(__float2int_rz(__fadd_rn(raw_hi, slack)), true, false, tb, g1)) return false;
    fill_call(out, p, tb, g1, q, false, 1.0);
    return true;
}

}  // namespace gsnp

#endif
