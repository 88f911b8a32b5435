/*
 * calling.cu - fused consensus calling on sm_103a: pileup, per-site record
 * sort, dependency-adjusted likelihood, posterior, rank-sum test.
 *
 * One CTA handles a tile of kTile consecutive reference sites, one thread per
 * site.  The reference runs the same work as five kernels and a Thrust sort per
 * 262,144-site window, with every intermediate in global memory:
 *   kernel/update_kernel.cu:233-326     updateSparse_kernel (pileup)
 *   kernel/batchsort.cu:245-291         batchSortMP2 (per-site sort)
 *   kernel/likelihood_kernel.cu:168-256 likelihoodSparse_kernel
 *   kernel/posterior_kernel.cu:635-866  posterior_kernel, posterior_kernel2
 * Here the records of a site never leave shared memory: they are inserted in
 * sorted order as the pileup produces them ([slot][site] layout, so a warp's
 * accesses fall in 32 distinct banks whatever slot each lane is at), the
 * likelihood walks them in that order, and only the 32-byte SiteCall leaves the
 * SM.
 *
 * The pileup of a site is every deposited read that covers it, in (start, file)
 * order.  That equals the reference's window-resident pileup: its carried-over
 * tail holds the previous window's reads first and the 255-record cap is
 * applied in that same order (kernel/update_kernel.cu:265-268,288).
 *
 * Tiles are binned by their deepest site (kNumBins record-slot capacities) so
 * that shared memory is sized for the tile, not for the worst case.
 */
#include <cuda_runtime.h>

#include "calling.cuh"

namespace gsnp {

__device__ __forceinline__ int64_t lower_bound_g(const int32_t* a, int64_t n, int64_t v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)__ldg(a + mid) < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int lower_bound_s(const int32_t* a, int n, int64_t v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int64_t)a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* Reads with start in [s0 - L + 1, s0 + kTile); positions staged in shared
 * memory when they fit. */
struct TileRange {
    int64_t r_lo, r_hi;
    bool staged;
};

__device__ TileRange setup_tile(const CallArgs& a, int64_t s0, int32_t* spos, int64_t* sh) {
    if (threadIdx.x == 0) {
        sh[0] = lower_bound_g(a.pos, a.n_reads, s0 - a.L + 1);
        sh[1] = lower_bound_g(a.pos, a.n_reads, s0 + kTile);
    }
    __syncthreads();
    TileRange tr;
    tr.r_lo = sh[0];
    tr.r_hi = sh[1];
    tr.staged = (tr.r_hi - tr.r_lo) <= kMaxStagedReads;
    if (tr.staged)
        for (int64_t i = threadIdx.x; i < tr.r_hi - tr.r_lo; i += blockDim.x) spos[i] = __ldg(a.pos + tr.r_lo + i);
    __syncthreads();
    return tr;
}

__device__ __forceinline__ void site_read_range(const CallArgs& a, const TileRange& tr, const int32_t* spos,
                                                int64_t site, int64_t* lo, int64_t* hi) {
    if (tr.staged) {
        const int n = (int)(tr.r_hi - tr.r_lo);
        *lo = tr.r_lo + lower_bound_s(spos, n, site - a.L + 1);
        *hi = tr.r_lo + lower_bound_s(spos, n, site + 1);
    } else {
        *lo = tr.r_lo + lower_bound_g(a.pos + tr.r_lo, tr.r_hi - tr.r_lo, site - a.L + 1);
        *hi = tr.r_lo + lower_bound_g(a.pos + tr.r_lo, tr.r_hi - tr.r_lo, site + 1);
    }
}

/* ------------------------------------------------------------------------ */
/* tile classification                                                       */
/* ------------------------------------------------------------------------ */

__global__ void __launch_bounds__(kTile) classify_tiles_kernel(CallArgs a, int pass, int64_t n_tiles,
                                                               int* bin_count, int32_t* bin_tiles) {
    __shared__ int32_t spos[kMaxStagedReads];
    __shared__ int64_t sh[2];
    __shared__ int smax[kTile / 32];
    const int64_t tile = blockIdx.x;
    const int64_t s0 = tile * kTile;
    const int win = (int)(s0 / kWin);
    const bool external = (a.win_flags[win] & kWinExternalLik) != 0;
    if (external != (pass == 1)) return;
    const TileRange tr = setup_tile(a, s0, spos, sh);
    const int64_t site = s0 + threadIdx.x;
    int need = 0;
    if (site < a.chr_len) {
        int64_t lo, hi;
        site_read_range(a, tr, spos, site, &lo, &hi);
        need = (int)((hi - lo) < kMaxRecords ? (hi - lo) : kMaxRecords);
    }
    for (int off = 16; off > 0; off >>= 1) need = max(need, __shfl_xor_sync(0xffffffffu, need, off));
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = need;
    __syncthreads();
    if (threadIdx.x == 0) {
        int m = 0;
        for (int i = 0; i < kTile / 32; ++i) m = max(m, smax[i]);
        const int bin = m <= 32 ? 0 : m <= 64 ? 1 : m <= 128 ? 2 : 3;
        const int idx = atomicAdd(&bin_count[bin], 1);
        bin_tiles[(int64_t)bin * n_tiles + idx] = (int32_t)tile;
    }
}

/* ------------------------------------------------------------------------ */
/* posterior (kernel/posterior_kernel.cu:575-866)                            */
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
    const double b = GSNP_DMUL(c2, gsnp_cr_exp(GSNP_DMUL(-z, GSNP_DDIV(z, 2.0))));
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

/* Wilcoxon rank-sum p-value of a heterozygous call (kernel/posterior_kernel.cu:506-572).
 * The records are the site's shared-memory column. */
__device__ double rank_test(const CallArgs& a, const uint32_t* recs, int num, const int* cu, int bt,
                            bool* normal_path) {
    const int ia = bt & 3, ib = (bt >> 2) & 3;
    if (ia == ib) return 1.0;
    if (cu[ia] == 0 || cu[ib] == 0) return 0.0;
    int ca[65], cb[65];
    for (int i = 0; i < 65; ++i) { ca[i] = 0; cb[i] = 0; }
    for (int i = 0; i < num; ++i) {
        const uint32_t w = recs[i * kTile];
        const int o = rec_base(w);
        if (o == ia) ca[rec_q(w)] += rec_occ(w);
        else if (o == ib) cb[rec_q(w)] += rec_occ(w);
    }
    /* rank of quality q among both alleles, ties averaged; qualities above
     * q_max - q_min + 1 keep rank 0 as in the reference */
    double Ta = 0.0, Tb = 0.0;
    int rank = 0;
    const int top = min(64, a.q_max_min + 1);
    for (int q = 0; q <= top; ++q) {
        const int c = ca[q] + cb[q];
        const double ra = GSNP_DADD((double)rank, GSNP_DDIV((double)(1 + c), 2.0));
        Ta = GSNP_DADD(Ta, GSNP_DMUL(ra, (double)ca[q]));
        Tb = GSNP_DADD(Tb, GSNP_DMUL(ra, (double)cb[q]));
        rank += c;
    }
    const int n1 = cu[ia], n2 = cu[ib];
    if (n1 + n2 < 64) return table_test(a.p_rank, n1, n2, Ta, Tb);
    *normal_path = true;
    return normal_test(n1, n2, Ta, Tb);
}

__device__ int64_t find_snp(const CallArgs& a, int64_t site) {
    int64_t lo = 0, hi = a.n_snp;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)a.snp[mid].pos < site) lo = mid + 1;
        else hi = mid;
    }
    return (lo < a.n_snp && (int64_t)a.snp[lo].pos == site) ? lo : -1;
}

/* q_sum[b] of site + 1 as the reference's window array holds it when site is
 * called: every deposited read covering site + 1, except that at the last
 * site of a window the next entry is the window's tail, which holds only the
 * reads starting inside the window (kernel/update_kernel.cu:260-325). */
__device__ int neighbour_qsum(const CallArgs& a, int64_t site, int b) {
    const int64_t p = site + 1;
    const int64_t win_end = (site / kWin + 1) * (int64_t)kWin;
    const int64_t max_start = (p == win_end) ? win_end - 1 : p;
    const int64_t lo = lower_bound_g(a.pos, a.n_reads, p - a.L + 1);
    const int64_t hi = lower_bound_g(a.pos, a.n_reads, max_start + 1);
    int dep_uni = 0, qsum = 0;
    const signed char qmin = (signed char)a.qmin;
    for (int64_t r = lo; r < hi; ++r) {
        const int coord = (int)(p - __ldg(a.pos + r));
        const uint32_t lh = (uint32_t)__ldg(a.lenhit + r);
        if (coord >= (int)(lh >> 16)) continue;
        const uint16_t bq = __ldg(a.bq + r * a.L + coord);
        const signed char base = (signed char)(bq & 0xff);
        const signed char qual = (signed char)(bq >> 8);
        if (base == 'N' || qual < qmin || dep_uni >= 0xFF) continue;
        if ((lh & 0xffffu) == 1) {
            dep_uni += 1;
            if (((base >> 1) & 3) == b) qsum += qual - qmin;
        }
    }
    return qsum;
}

struct SitePileup {
    int cu[4], qs[4];
    uint32_t ca[4];
    uint32_t depth, repeat;
    int dep_uni, num;
};

/* posterior_kernel + posterior_kernel2 for one site (kernel/posterior_kernel.cu:680-864).
 *
 * tl holds type_likely by genotype code.  When eps is given, tl is an FP32
 * approximation and eps[g] bounds |tl[g] - FP64 type_likely[g]|; the function
 * then returns false, writing nothing, unless every decision it makes (the
 * genotype order behind type1/type2 and the truncated, clamped consensus
 * quality) is provably the one the FP64 values give. */
__device__ bool site_posterior(const CallArgs& a, int64_t site, uint8_t ori, const SitePileup& p,
                               const double* tl, const double* eps, const uint32_t* recs, SiteCall* out) {
    const int ori7 = ori & 7;
    int base1 = 0, base2 = 0;
    int qual1 = -1, qual2 = -2, qual3 = -3;
    if (p.dep_uni) {
        for (int i = 0; i != 4; ++i) {
            const int v = p.qs[i];
            if (v >= qual1) { qual3 = qual2; base2 = base1; qual2 = qual1; base1 = i; qual1 = v; }
            else if (v >= qual2) { qual3 = qual2; base2 = i; qual2 = v; }
            else if (v >= qual3) { qual3 = v; }
        }
        if (qual1 == 0) base1 = ori7;
        else if (qual2 == 0 && base1 != ori7) base2 = ori7;
    } else {
        uint32_t c1 = 0, c2 = 0, c3 = 0;
        for (int i = 0; i != 4; ++i) {
            const uint32_t v = p.ca[i];
            if (v >= c1) { c3 = c2; base2 = base1; c2 = c1; base1 = i; c1 = v; }
            else if (v >= c2) { c3 = c2; base2 = i; c2 = v; }
            else if (v >= c3) { c3 = v; }
        }
        if (c1 == 0) base1 = ori7;
        else if (c2 == 0 && base1 != ori7) base2 = ori7;
    }
    double lp[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) lp[i] = __ldg(a.log_prior + (ori7 << 4) + i);
    if ((ori & 0x8) && a.refine) {
        /* dbSNP prior, precomputed per dbSNP row by snp_log_prior_kernel */
        const int64_t k = find_snp(a, site);
        if (k >= 0) {
            const double2* src = reinterpret_cast<const double2*>(a.snp_lp + k * 16);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const double2 v = __ldg(src + i);
                lp[2 * i] = v.x;
                lp[2 * i + 1] = v.y;
            }
        }
    }
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
    const double rs = a.rank_sum ? rank_test(a, recs, p.num, p.cu, type1, &normal_path) : 1.0;
    /* clamps of posterior_kernel2 (kernel/posterior_kernel.cu:839-864) */
    const bool hom = (type1 & 3) == ((type1 >> 2) & 3);
    bool het_ok = false;
    if (!hom) {
        /* base1/base2 may name an N reference base (4..7): the reference then
         * reads q_sum[4*site + base], i.e. the next site's q_sum[base - 4].
         * With q_sum summing to zero that is never consulted; otherwise
         * (base2 = N code) the next site's value is recomputed. */
        const int comb = base1 < base2 ? (base1 << 2 | base2) : (base2 << 2 | base1);
        het_ok = type1 == comb;
        if (het_ok) het_ok = (base1 < 4 ? p.qs[base1] : neighbour_qsum(a, site, base1 - 4)) > 0;
        if (het_ok) het_ok = (base2 < 4 ? p.qs[base2] : neighbour_qsum(a, site, base2 - 4)) > 0;
    }
    auto finalize = [&](int q) {
        if (hom) {
            if (qual1 > 0 && base1 != (type1 & 3)) q = 0;
            else if (q > qual1 - qual2) q = qual1 - qual2;
        } else {
            if (het_ok) {
                if (q > qual2 - qual3) q = qual2 - qual3;
            } else {
                q = 0;
            }
        }
        if (q > 99) q = 99;
        if (q < 0) q = 0;
        return q;
    };
    int q;
    if (rs == 0.0) {
        q = finalize(0);
    } else {
        const double d = GSNP_DMUL(10.0, GSNP_DSUB(tp[type1], tp[type2]));
        const double raw = GSNP_DADD(d, GSNP_DMUL(10.0, gsnp_cr_log10(rs)));
        q = finalize((int)raw);
        if (eps && ep[type1] + ep[type2] > 0.0) {
            const double delta = 10.0 * (ep[type1] + ep[type2]) * (1.0 + 0x1p-20) + 0x1p-48 * (fabs(raw) + 1.0);
            if (finalize((int)(raw - delta)) != finalize((int)(raw + delta))) return false;
        }
    }
    SiteCall c;
    c.type1 = (uint8_t)type1;
    c.base1 = (uint8_t)base1;
    c.base2 = (uint8_t)base2;
    c.q_cns = (uint8_t)q;
    c.avg_q1 = (base1 < 4 && p.qs[base1] != 0) ? (uint8_t)(p.qs[base1] / p.cu[base1]) : 0;
    c.avg_q2 = (base2 < 4 && p.qs[base2] != 0) ? (uint8_t)(p.qs[base2] / p.cu[base2]) : 0;
    c.flags = normal_path ? 2 : 0;
    c.pad = 0;
    c.cu1 = base1 < 4 ? (uint16_t)p.cu[base1] : 0;
    c.ca1 = base1 < 4 ? (uint16_t)p.ca[base1] : 0;
    c.cu2 = base2 < 4 ? (uint16_t)p.cu[base2] : 0;
    c.ca2 = base2 < 4 ? (uint16_t)p.ca[base2] : 0;
    c.depth = p.depth;
    c.repeat_time = p.repeat;
    c.rank_sum = rs;
    *out = c;
    return true;
}

/* log10 genotype priors of every dbSNP row (kernel/posterior_kernel.cu:575-633,
 * the device version: no check of the number of listed alleles).  Run once per
 * reference and parameter set so that the calling kernel only loads them. */
__global__ void snp_log_prior_kernel(CallArgs a, double* out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n_snp) return;
    const DbSnpEntry e = a.snp[k];
    const int ori = a.ori[e.pos];
    const int ori7 = ori & 7;
    double lp[16];
    for (int i = 0; i < 16; ++i) lp[i] = a.log_prior[(ori7 << 4) + i];
    if (!e.indel) {
        const int t_base = ori & 3;
        for (int a1 = 0; a1 != 4; ++a1)
            for (int a2 = a1; a2 != 4; ++a2) {
                if (!(e.freq[a1] > 0 && e.freq[a2] > 0)) continue;
                double pr;
                if (!e.hapmap) {
                    if (a1 == a2 && a1 == t_base) pr = 1;
                    else if (a1 == t_base || a2 == t_base) pr = e.validated ? a.het_val : a.het_unval;
                    else if (a1 == a2) pr = e.validated ? a.althom_val : a.althom_unval;
                    else pr = e.validated ? a.het_val : a.het_unval;
                } else {
                    pr = GSNP_DMUL(GSNP_DMUL((a1 == a2 ? 1.0 : GSNP_DMUL(2.0, a.het_val)), e.freq[a1]), e.freq[a2]);
                }
                lp[(a1 << 2) | a2] = gsnp_cr_log10(pr);
            }
    }
    for (int i = 0; i < 16; ++i) out[k * 16 + i] = lp[i];
}

cudaError_t launch_snp_log_prior(const CallArgs& a, double* out, cudaStream_t stream) {
    if (a.n_snp == 0) return cudaSuccess;
    snp_log_prior_kernel<<<(unsigned)((a.n_snp + 127) / 128), 128, 0, stream>>>(a, out);
    return cudaGetLastError();
}

/* ------------------------------------------------------------------------ */
/* likelihood walk (kernel/likelihood_kernel.cu:187-255)                      */
/* ------------------------------------------------------------------------ */

/* Walk one site's sorted records: per observed-base group, count repeats of
 * each (strand, cycle) and of distinct ones, and hand each record's adjusted
 * quality, cycle and base to f.  The per-site counters are left at zero. */
template <class F>
__device__ __forceinline__ void walk_records(const CallArgs& a, const uint32_t* recs, uint8_t* cnt, int num, F&& f) {
    const int L = a.L;
    int gdc = -1, last_o = -1, gstart = 0;
    for (int i = 0; i < num; ++i) {
        const uint32_t w = recs[i * kTile];
        const int o = rec_base(w);
        const int q = rec_q(w);
        const int coord = rec_coord(w);
        const int key = rec_strand(w) * L + coord;
        if (o != last_o) {
            for (int j = gstart; j < i; ++j) {
                const uint32_t wj = recs[j * kTile];
                cnt[(rec_strand(wj) * L + rec_coord(wj)) * kTile] = 0;
            }
            gstart = i;
            gdc = -1;
            last_o = o;
        }
        int tmp = cnt[key * kTile];
        const int occ = rec_occ(w);
        for (int k = 0; k < occ; ++k) {
            if (tmp == 0) gdc += 1;
            tmp++;
            const int qa = (tmp < a.tmax && gdc < a.gmax)
                               ? (int)__ldg(a.qadj + ((size_t)tmp * a.gmax + gdc) * 65 + q)
                               : 1;
            f(qa, coord, o);
        }
        cnt[key * kTile] = (uint8_t)tmp;
    }
    for (int j = gstart; j < num; ++j) {
        const uint32_t wj = recs[j * kTile];
        cnt[(rec_strand(wj) * L + rec_coord(wj)) * kTile] = 0;
    }
}

/* FP64 sums in the reference's order: the plain form and the fixup */
__device__ __forceinline__ void likelihood_fp64(const CallArgs& a, const uint32_t* recs, uint8_t* cnt, int num,
                                                double* tl) {
    double s[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) s[i] = 0.0;
    walk_records(a, recs, cnt, num, [&](int qa, int coord, int o) {
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

/* FP32 Kahan sums with a bound on their distance to the FP64 sums.  Every
 * term is <= 0 (the host checks the table), so sum|x| = |S|; the bound covers
 * the rounding of each term to FP32, the compensated summation error
 * (2u + O(n u^2)) sum|x| and the FP64 sum's own rounding (n u64 sum|x|). */
__device__ __forceinline__ void likelihood_fp32(const CallArgs& a, const uint32_t* recs, uint8_t* cnt, int num,
                                                double* tl, double* eps) {
    float s[10], c[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) { s[i] = 0.f; c[i] = 0.f; }
    walk_records(a, recs, cnt, num, [&](int qa, int coord, int o) {
        const float4* row = reinterpret_cast<const float4*>(a.lik32 + ((size_t)(qa * a.L + coord) * 4 + o) * 12);
        const float4 x0 = __ldg(row), x1 = __ldg(row + 1), x2 = __ldg(row + 2);
        const float x[10] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w, x2.x, x2.y};
#pragma unroll
        for (int v = 0; v < 10; ++v) {
            const float y = __fsub_rn(x[v], c[v]);
            const float t = __fadd_rn(s[v], y);
            c[v] = __fsub_rn(__fsub_rn(t, s[v]), y);
            s[v] = t;
        }
    });
    const double k = 0x1p-22 + (double)num * 0x1p-45;
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        const int g = genotype_of(i);
        tl[g] = (double)s[i];
        eps[g] = fabs(tl[g]) * k;
    }
}

/* ------------------------------------------------------------------------ */
/* the fused calling kernel                                                  */
/* ------------------------------------------------------------------------ */

template <int SLOTS>
__global__ void __launch_bounds__(kTile) call_tiles_kernel(CallArgs a, const int32_t* __restrict__ tiles) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint32_t* recs_all = reinterpret_cast<uint32_t*>(smem);                       /* [SLOTS][kTile] */
    uint8_t* cnt_all = smem + (size_t)SLOTS * kTile * 4;                           /* [2L][kTile] */
    int32_t* spos = reinterpret_cast<int32_t*>(cnt_all + (((size_t)2 * a.L * kTile + 15) & ~(size_t)15));
    __shared__ int64_t sh[2];

    const int t = threadIdx.x;
    const int64_t tile = tiles[blockIdx.x];
    const int64_t s0 = tile * kTile;
    const int win = (int)(s0 / kWin);
    const uint8_t wflags = a.win_flags[win];

    /* clear the per-site pcr counters */
    {
        uint4* c4 = reinterpret_cast<uint4*>(cnt_all);
        const int n16 = (2 * a.L * kTile) / 16;
        for (int i = t; i < n16; i += kTile) c4[i] = make_uint4(0, 0, 0, 0);
    }
    const TileRange tr = setup_tile(a, s0, spos, sh);

    const int64_t site = s0 + t;
    if (site >= a.chr_len) return;
    uint32_t* recs = recs_all + t;
    uint8_t* cnt = cnt_all + t;
    const int L = a.L;

    /* ---- pileup (kernel/update_kernel.cu:260-325) ---- */
    int64_t lo, hi;
    site_read_range(a, tr, spos, site, &lo, &hi);
    SitePileup p;
#pragma unroll
    for (int i = 0; i < 4; ++i) { p.cu[i] = 0; p.qs[i] = 0; p.ca[i] = 0; }
    p.depth = 0;
    p.repeat = 0;
    p.dep_uni = 0;
    p.num = 0;
    const signed char qmin = (signed char)a.qmin;
    for (int64_t r = lo; r < hi; ++r) {
        const int32_t start = tr.staged ? spos[r - tr.r_lo] : __ldg(a.pos + r);
        const int coord = (int)(site - start);
        const uint32_t lh = (uint32_t)__ldg(a.lenhit + r);
        const int rlen = (int)(lh >> 16);
        if (coord >= rlen) continue;
        const int hit = (int)(lh & 0xffffu);
        const uint16_t bq = __ldg(a.bq + r * L + coord);
        const signed char base = (signed char)(bq & 0xff);
        const signed char qual = (signed char)(bq >> 8);
        p.depth += 1;
        p.repeat += (uint32_t)hit;
        if (base == 'N' || qual < qmin || p.dep_uni >= 0xFF) continue;
        const int b = (base >> 1) & 3;
        if (hit == 1) {
            p.dep_uni += 1;
            const bool minus = __ldg(a.strand + r) != '+';
            const uint32_t coord_val = minus ? (uint32_t)(rlen - 1 - coord) : (uint32_t)coord;
            const uint32_t w = make_record(base, qual - qmin, coord_val, minus ? 1u : 0u);
            /* insertion keeps the column sorted ascending */
            int j = p.num;
            while (j > 0) {
                const uint32_t prev = recs[(j - 1) * kTile];
                if (prev <= w) break;
                recs[j * kTile] = prev;
                --j;
            }
            recs[j * kTile] = w;
            p.num += 1;
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (i == b) { p.cu[i] += 1; p.qs[i] += qual - qmin; }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (i == b) p.ca[i] += 1;
    }
    if (p.ca[0] > 0xffff || p.ca[1] > 0xffff || p.ca[2] > 0xffff || p.ca[3] > 0xffff) atomicExch(a.error, 1);

    /* ---- likelihood over the sorted records (kernel/likelihood_kernel.cu:187-255) ---- */
    double tl[16], eps[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) { tl[i] = 0.0; eps[i] = 0.0; }
    const bool external = (wflags & kWinExternalLik) != 0;
    const bool fp32 = a.precision == 1 && !(wflags & (kWinKeepLik | kWinExternalLik));
    if (external) {
        const int src = a.win_lik_src[win];
        if (src >= 0) {
            const double* srcp = a.lik_keep + ((int64_t)src * kWin + (site - (int64_t)win * kWin)) * 10;
#pragma unroll
            for (int i = 0; i < 10; ++i) tl[genotype_of(i)] = srcp[i];
        }
    } else if (fp32) {
        likelihood_fp32(a, recs, cnt, p.num, tl, eps);
    } else {
        likelihood_fp64(a, recs, cnt, p.num, tl);
        if (wflags & kWinKeepLik) {
            double* dst = a.lik_keep + site * 10;
#pragma unroll
            for (int i = 0; i < 10; ++i) dst[i] = tl[genotype_of(i)];
        }
    }

    if (wflags & kWinKeepCounts) {
        SiteCounts c;
#pragma unroll
        for (int i = 0; i < 4; ++i) { c.cu[i] = (uint16_t)p.cu[i]; c.qs[i] = (uint16_t)p.qs[i]; c.ca[i] = p.ca[i]; }
        c.depth = p.depth;
        c.repeat_time = p.repeat;
        a.counts[site] = c;
    }

    /* ---- posterior, rank-sum, consensus quality ---- */
    const uint8_t ori = __ldg(a.ori + site);
    SiteCall call;
    if (fp32 && (site & 4095) == 0 && a.stats) {
        /* sampled accuracy of the FP32 sums against the FP64 ones */
        double t64[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) t64[i] = 0.0;
        likelihood_fp64(a, recs, cnt, p.num, t64);
        double m = 0.0;
#pragma unroll
        for (int i = 0; i < 16; ++i) m = fmax(m, fabs(t64[i] - tl[i]));
        atomicMax(a.stats + 3, (unsigned long long)__double_as_longlong(m));
        atomicAdd(a.stats + 2, 1ull);
    }
    if (!site_posterior(a, site, ori, p, tl, fp32 ? eps : nullptr, recs, &call)) {
        /* FP64 fixup: the FP32 likelihood is too close to a decision boundary */
        likelihood_fp64(a, recs, cnt, p.num, tl);
        site_posterior(a, site, ori, p, tl, nullptr, recs, &call);
        call.flags |= 1;
        atomicAdd(a.stats + 1, 1ull);
    }
    a.out[site] = call;
}

template __global__ void call_tiles_kernel<32>(CallArgs, const int32_t*);
template __global__ void call_tiles_kernel<64>(CallArgs, const int32_t*);
template __global__ void call_tiles_kernel<128>(CallArgs, const int32_t*);
template __global__ void call_tiles_kernel<256>(CallArgs, const int32_t*);

size_t call_smem_bytes(int slots, int L) {
    return (size_t)slots * kTile * 4 + (((size_t)2 * L * kTile + 15) & ~(size_t)15) + (size_t)kMaxStagedReads * 4;
}

cudaError_t launch_classify(const CallArgs& a, int pass, int64_t n_tiles, int* d_bin_count, int32_t* d_bin_tiles,
                            cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(d_bin_count, 0, sizeof(int) * kNumBins, stream);
    if (e != cudaSuccess) return e;
    classify_tiles_kernel<<<(unsigned)n_tiles, kTile, 0, stream>>>(a, pass, n_tiles, d_bin_count, d_bin_tiles);
    return cudaGetLastError();
}

/* Launch the calling kernel for the `count` tiles of one depth bin. */
cudaError_t launch_bin(const CallArgs& a, int bin, const int32_t* tiles, int count, cudaStream_t stream) {
    static const int slots[kNumBins] = {32, 64, 128, 256};
    const size_t smem = call_smem_bytes(slots[bin], a.L);
    switch (bin) {
        case 0:
            cudaFuncSetAttribute(call_tiles_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            call_tiles_kernel<32><<<count, kTile, smem, stream>>>(a, tiles);
            break;
        case 1:
            cudaFuncSetAttribute(call_tiles_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            call_tiles_kernel<64><<<count, kTile, smem, stream>>>(a, tiles);
            break;
        case 2:
            cudaFuncSetAttribute(call_tiles_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            call_tiles_kernel<128><<<count, kTile, smem, stream>>>(a, tiles);
            break;
        default:
            cudaFuncSetAttribute(call_tiles_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            call_tiles_kernel<256><<<count, kTile, smem, stream>>>(a, tiles);
            break;
    }
    return cudaGetLastError();
}

}  // namespace gsnp
