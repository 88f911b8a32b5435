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
 * applied in that same order (kernel/update_kernel.cu:265-268,288).  A warp
 * walks the reads that can cover any of its 32 sites once, in that order; each
 * read's row is read with one coalesced load per lane band.
 *
 * Two calling kernels share this structure:
 *   call_tiles_kernel  FP64 sums in the reference's order (the plain form);
 *                      also the second pass of the fast form over the sites
 *                      that form deferred;
 *   call_fast_kernel   FP32 compensated sums and an FP32 posterior for
 *                      homozygous calls that the error bound proves; every
 *                      other site is marked and its tile listed for the FP64
 *                      pass.  It runs no FP64 instruction.
 * Tiles are binned by their deepest site (kNumBins record-slot capacities) so
 * that shared memory is sized for the tile, not for the worst case.
 */
#include <cuda_runtime.h>

#include "calling.cuh"
#include "site_math.cuh"

namespace gsnp {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int lower_bound_s(const int32_t* a, int n, int64_t v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int64_t)a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* Pileup of one warp's 32 consecutive sites (kernel/update_kernel.cu:260-325).
 * Reads [r_lo, r_hi) are those starting in [w0 - L + 1, w0 + 31]; their
 * positions, lengths and strands are loaded 32 at a time and broadcast, and
 * each lane takes the reads that cover its own site.  Records are inserted so
 * that the column stays in ascending order.  Lanes with !active only keep the
 * warp's loop going. */
template <int SLOTS>
__device__ __forceinline__ void warp_pileup(const CallArgs& a, int64_t r_lo, int64_t r_hi, int64_t site, bool active,
                                            uint32_t* recs, SitePileup& p) {
#pragma unroll
    for (int i = 0; i < 4; ++i) { p.cu[i] = 0; p.qs[i] = 0; p.ca[i] = 0; }
    p.depth = 0;
    p.repeat = 0;
    p.dep_uni = 0;
    p.num = 0;
    const int lane = threadIdx.x & 31;
    const int L = a.L;
    const signed char qmin = (signed char)a.qmin;
    bool overflow = false;
    for (int64_t rb = r_lo; rb < r_hi; rb += 32) {
        const int64_t r = rb + lane;
        int32_t mpos = 0;
        uint32_t mlh = 0;
        int mminus = 0;
        if (r < r_hi) {
            mpos = __ldg(a.pos + r);
            mlh = (uint32_t)__ldg(a.lenhit + r);
            mminus = __ldg(a.strand + r) != '+';
        }
        const int cnt = (int)((r_hi - rb) < 32 ? (r_hi - rb) : 32);
        for (int k = 0; k < cnt; ++k) {
            const int32_t start = __shfl_sync(kFull, mpos, k);
            const uint32_t lh = __shfl_sync(kFull, mlh, k);
            const int minus = __shfl_sync(kFull, mminus, k);
            const int coord = (int)(site - start);
            const int rlen = (int)(lh >> 16);
            if (!active || coord < 0 || coord >= rlen) continue;
            const int hit = (int)(lh & 0xffffu);
            const uint16_t bq = __ldg(a.bq + (rb + k) * L + coord);
            const signed char base = (signed char)(bq & 0xff);
            const signed char qual = (signed char)(bq >> 8);
            p.depth += 1;
            p.repeat += (uint32_t)hit;
            if (base == 'N' || qual < qmin || p.dep_uni >= 0xFF) continue;
            const int b = (base >> 1) & 3;
            if (hit == 1) {
                p.dep_uni += 1;
                const uint32_t coord_val = minus ? (uint32_t)(rlen - 1 - coord) : (uint32_t)coord;
                const uint32_t w = make_record(base, qual - qmin, coord_val, minus ? 1u : 0u);
                if (p.num < SLOTS) {
                    int j = p.num;
                    while (j > 0) {
                        const uint32_t prev = recs[(j - 1) * kTile];
                        if (prev <= w) break;
                        recs[j * kTile] = prev;
                        --j;
                    }
                    recs[j * kTile] = w;
                    p.num += 1;
                } else {
                    overflow = true;
                }
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if (i == b) { p.cu[i] += 1; p.qs[i] += qual - qmin; }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (i == b) p.ca[i] += 1;
        }
    }
    if (overflow) atomicExch(a.error, 2);
    if (p.ca[0] > 0xffff || p.ca[1] > 0xffff || p.ca[2] > 0xffff || p.ca[3] > 0xffff) atomicExch(a.error, 1);
}

__device__ __forceinline__ void store_counts(const CallArgs& a, int64_t site, const SitePileup& p) {
    SiteCounts c;
#pragma unroll
    for (int i = 0; i < 4; ++i) { c.cu[i] = (uint16_t)p.cu[i]; c.qs[i] = (uint16_t)p.qs[i]; c.ca[i] = p.ca[i]; }
    c.depth = p.depth;
    c.repeat_time = p.repeat;
    a.counts[site] = c;
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

}  // namespace

/* ------------------------------------------------------------------------ */
/* tile classification                                                       */
/* ------------------------------------------------------------------------ */

/* Per tile: the deepest site's record need (reads starting in [site - L + 1,
 * site], capped at 255) picks the depth bin; the window's mode picks the FP64
 * kernel (bins 0..3) or the fast one (bins 4..7).  Each warp's read range is
 * stored for the calling kernels. */
__global__ void __launch_bounds__(kTile) classify_tiles_kernel(CallArgs a, int pass, int* bin_count,
                                                               int32_t* bin_tiles) {
    __shared__ int32_t spos[kMaxStagedReads];
    __shared__ int64_t sh[2];
    __shared__ int smax[kWarpsPerTile];
    const int64_t tile = blockIdx.x;
    const int64_t s0 = tile * kTile;
    const int win = (int)(s0 / kWin);
    const uint8_t wflags = a.win_flags[win];
    const bool external = (wflags & kWinExternalLik) != 0;
    if (external != (pass == 1)) return;
    if (threadIdx.x == 0) {
        sh[0] = lower_bound_g(a.pos, a.n_reads, s0 - a.L + 1);
        sh[1] = lower_bound_g(a.pos, a.n_reads, s0 + kTile);
    }
    __syncthreads();
    const int64_t r_lo = sh[0], r_hi = sh[1];
    const bool staged = (r_hi - r_lo) <= kMaxStagedReads;
    if (staged)
        for (int64_t i = threadIdx.x; i < r_hi - r_lo; i += blockDim.x) spos[i] = __ldg(a.pos + r_lo + i);
    __syncthreads();
    const int n = (int)(r_hi - r_lo);
    auto lb = [&](int64_t v) -> int64_t {
        return staged ? r_lo + lower_bound_s(spos, n, v) : r_lo + lower_bound_g(a.pos + r_lo, r_hi - r_lo, v);
    };
    const int64_t site = s0 + threadIdx.x;
    int need = 0;
    if (site < a.chr_len) {
        const int64_t c = lb(site + 1) - lb(site - a.L + 1);
        need = (int)(c < kMaxRecords ? c : kMaxRecords);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane < 2) {
        const int64_t w0 = s0 + warp * 32;
        a.warp_rng[(tile * kWarpsPerTile + warp) * 2 + lane] = lane == 0 ? lb(w0 - a.L + 1) : lb(w0 + 32);
    }
    for (int off = 16; off > 0; off >>= 1) need = max(need, __shfl_xor_sync(kFull, need, off));
    if (lane == 0) smax[warp] = need;
    __syncthreads();
    if (threadIdx.x == 0) {
        int m = 0;
        for (int i = 0; i < kWarpsPerTile; ++i) m = max(m, smax[i]);
        const bool fast = a.precision == 1 && !(wflags & (kWinKeepLik | kWinExternalLik));
        const int bin = (m <= 32 ? 0 : m <= 64 ? 1 : m <= 128 ? 2 : 3) + (fast ? kNumBins : 0);
        const int idx = atomicAdd(&bin_count[bin], 1);
        bin_tiles[(int64_t)bin * a.n_tiles + idx] = (int32_t)tile;
    }
}

/* log10 genotype priors of every dbSNP row (kernel/posterior_kernel.cu:575-633,
 * the device version: no check of the number of listed alleles).  Run once per
 * reference and parameter set so that the calling kernels only load them; the
 * FP32 copy is by table column. */
__global__ void snp_log_prior_kernel(CallArgs a, double* out, float* out32) {
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
    for (int t = 0; t < 12; ++t) out32[k * 12 + t] = t < 10 ? (float)lp[genotype_of(t)] : 0.f;
}

cudaError_t launch_snp_log_prior(const CallArgs& a, double* out, float* out32, cudaStream_t stream) {
    if (a.n_snp == 0) return cudaSuccess;
    snp_log_prior_kernel<<<(unsigned)((a.n_snp + 127) / 128), 128, 0, stream>>>(a, out, out32);
    return cudaGetLastError();
}

/* ------------------------------------------------------------------------ */
/* the FP64 calling kernel                                                   */
/* ------------------------------------------------------------------------ */

/* deferred != 0: only the sites the fast kernel marked (pending or sampled)
 * are called; their FP32 sums are tried first with the double-precision
 * bound checks, then recomputed in FP64 when those fail. */
template <int SLOTS>
__global__ void __launch_bounds__(kTile, 4) call_tiles_kernel(CallArgs a, const int32_t* __restrict__ tiles,
                                                              int deferred) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint32_t* recs = reinterpret_cast<uint32_t*>(smem) + threadIdx.x;        /* [SLOTS][kTile] */
    uint32_t* seen = reinterpret_cast<uint32_t*>(smem) + SLOTS * kTile + threadIdx.x;  /* [nw][kTile] */

    const int t = threadIdx.x, warp = t >> 5;
    const int64_t tile = tiles[blockIdx.x];
    const int64_t s0 = tile * kTile;
    const int win = (int)(s0 / kWin);
    const uint8_t wflags = a.win_flags[win];
    const int64_t site = s0 + t;
    bool active = site < a.chr_len;
    uint8_t f0 = 0;
    if (deferred) {
        if (active) f0 = a.out[site].flags;
        active = active && (f0 & (kCallPending | kCallSampled));
        if (!__any_sync(kFull, active)) return;
    }
    const int64_t r_lo = a.warp_rng[(tile * kWarpsPerTile + warp) * 2];
    const int64_t r_hi = a.warp_rng[(tile * kWarpsPerTile + warp) * 2 + 1];
    SitePileup p;
    warp_pileup<SLOTS>(a, r_lo, r_hi, site, active, recs, p);
    if (!active) return;

    double tl[16], eps[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) { tl[i] = 0.0; eps[i] = 0.0; }
    const bool external = (wflags & kWinExternalLik) != 0;
    const bool fp32 = deferred && a.precision == 1;
    if (external) {
        const int src = a.win_lik_src[win];
        if (src >= 0) {
            const double* srcp = a.lik_keep + ((int64_t)src * kWin + (site - (int64_t)win * kWin)) * 10;
#pragma unroll
            for (int i = 0; i < 10; ++i) tl[genotype_of(i)] = srcp[i];
        }
    } else if (fp32) {
        likelihood_fp32(a, recs, seen, kTile, p.num, tl, eps);
    } else {
        likelihood_fp64(a, recs, seen, kTile, p.num, tl);
        if (wflags & kWinKeepLik) {
            double* dst = a.lik_keep + site * 10;
#pragma unroll
            for (int i = 0; i < 10; ++i) dst[i] = tl[genotype_of(i)];
        }
    }
    if ((wflags & kWinKeepCounts) && !deferred) store_counts(a, site, p);

    const uint8_t ori = __ldg(a.ori + site);
    double lp[16];
    load_log_prior(a, site, ori, lp);
    auto nq = [&](int b) { return neighbour_qsum(a, site, b); };
    if (fp32 && (f0 & kCallSampled)) {
        /* sampled accuracy of the FP32 sums against the FP64 ones */
        double t64[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) t64[i] = 0.0;
        likelihood_fp64(a, recs, seen, kTile, p.num, t64);
        double m = 0.0;
#pragma unroll
        for (int i = 0; i < 16; ++i) m = fmax(m, fabs(t64[i] - tl[i]));
        atomicMax(a.stats + 3, (unsigned long long)__double_as_longlong(m));
        atomicAdd(a.stats + 2, 1ull);
    }
    SiteCall call;
    if (!site_posterior(a, ori, p, tl, fp32 ? eps : nullptr, lp, recs, kTile, nq, &call)) {
        /* FP64 fixup: the FP32 likelihood is too close to a decision boundary */
        likelihood_fp64(a, recs, seen, kTile, p.num, tl);
        site_posterior(a, ori, p, tl, nullptr, lp, recs, kTile, nq, &call);
        call.flags |= kCallFixup;
        atomicAdd(a.stats + 1, 1ull);
    }
    if (deferred) {
        if (f0 & kCallPending) {
            atomicAdd(a.stats + 4, 1ull);
        } else if (!same_call(a.out[site], call)) {
            /* a sampled site the fast kernel decided differs from the FP64 call */
            atomicAdd(a.stats + 5, 1ull);
        }
    }
    a.out[site] = call;
}

/* ------------------------------------------------------------------------ */
/* the fast calling kernel                                                   */
/* ------------------------------------------------------------------------ */

template <int SLOTS>
__global__ void __launch_bounds__(kTile, 6) call_fast_kernel(CallArgs a, const int32_t* __restrict__ tiles, int bin) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint32_t* recs = reinterpret_cast<uint32_t*>(smem) + threadIdx.x;
    uint32_t* seen = reinterpret_cast<uint32_t*>(smem) + SLOTS * kTile + threadIdx.x;

    const int t = threadIdx.x, warp = t >> 5;
    const int64_t tile = tiles[blockIdx.x];
    const int64_t s0 = tile * kTile;
    const int win = (int)(s0 / kWin);
    const uint8_t wflags = a.win_flags[win];
    const int64_t site = s0 + t;
    const bool active = site < a.chr_len;
    const int64_t r_lo = a.warp_rng[(tile * kWarpsPerTile + warp) * 2];
    const int64_t r_hi = a.warp_rng[(tile * kWarpsPerTile + warp) * 2 + 1];
    SitePileup p;
    warp_pileup<SLOTS>(a, r_lo, r_hi, site, active, recs, p);

    bool listed = false;
    if (active) {
        if (wflags & kWinKeepCounts) store_counts(a, site, p);
        /* adjusted quality of each record, written over its occurrence byte */
        walk_records<true>(a, recs, seen, kTile, p.num, [&](int i, int qa, int, int) {
            recs[i * kTile] = (recs[i * kTile] & ~0xffu) | (uint32_t)qa;
        });
        /* FP32 sums, two records per step (the pairing of likelihood_fp32) */
        Kahan10 k;
        k.init();
        for (int i = 0; i < p.num; i += 2) {
            const uint32_t w0 = recs[i * kTile];
            const bool two = i + 1 < p.num;
            const uint32_t w1 = two ? recs[(i + 1) * kTile] : w0;
            float x[10], y[10];
            lik32_row(a, (int)(w0 & 0xffu), rec_coord(w0), rec_base(w0), x);
            lik32_row(a, (int)(w1 & 0xffu), rec_coord(w1), rec_base(w1), y);
            if (two) {
#pragma unroll
                for (int v = 0; v < 10; ++v) x[v] = __fadd_rn(x[v], y[v]);
            }
            k.add(x);
        }
        const uint8_t ori = __ldg(a.ori + site);
        SiteCall call;
        const bool sampled = (site & 4095) == 0 && a.stats;
        if (fast_posterior(a, site, ori, p, k.s, p.num, &call)) {
            if (sampled) call.flags |= kCallSampled;
            listed = sampled;
        } else {
            call = SiteCall{};
            call.flags = kCallPending | (sampled ? kCallSampled : 0);
            listed = true;
        }
        a.out[site] = call;
    }
    if (__syncthreads_or(listed) && t == 0) {
        const int idx = atomicAdd(a.fix_count + bin, 1);
        a.fix_tiles[(int64_t)bin * a.n_tiles + idx] = (int32_t)tile;
    }
}

/* ------------------------------------------------------------------------ */
/* launchers                                                                 */
/* ------------------------------------------------------------------------ */

static const int kSlots[kNumBins] = {32, 64, 128, 256};

size_t call_smem_bytes(int slots, int L) {
    const int nw = (2 * L + 31) >> 5;
    return ((size_t)slots + nw) * kTile * 4;
}

cudaError_t launch_classify(const CallArgs& a, int pass, int* d_bin_count, int32_t* d_bin_tiles, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(d_bin_count, 0, sizeof(int) * 2 * kNumBins, stream);
    if (e != cudaSuccess) return e;
    classify_tiles_kernel<<<(unsigned)a.n_tiles, kTile, 0, stream>>>(a, pass, d_bin_count, d_bin_tiles);
    return cudaGetLastError();
}

template <int SLOTS>
static cudaError_t launch_one(const CallArgs& a, int kind, int bin, const int32_t* tiles, int count,
                              cudaStream_t stream) {
    const int smem = (int)call_smem_bytes(SLOTS, a.L);
    if (kind == kKindFast) {
        cudaFuncSetAttribute(call_fast_kernel<SLOTS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        call_fast_kernel<SLOTS><<<count, kTile, smem, stream>>>(a, tiles, bin);
    } else {
        cudaFuncSetAttribute(call_tiles_kernel<SLOTS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        call_tiles_kernel<SLOTS><<<count, kTile, smem, stream>>>(a, tiles, kind == kKindDeferred ? 1 : 0);
    }
    return cudaGetLastError();
}

/* Launch a calling kernel over the `count` tiles of depth bin `bin` (0..3). */
cudaError_t launch_bin(const CallArgs& a, int kind, int bin, const int32_t* tiles, int count, cudaStream_t stream) {
    switch (bin) {
        case 0: return launch_one<32>(a, kind, bin, tiles, count, stream);
        case 1: return launch_one<64>(a, kind, bin, tiles, count, stream);
        case 2: return launch_one<128>(a, kind, bin, tiles, count, stream);
        default: return launch_one<256>(a, kind, bin, tiles, count, stream);
    }
}

int bin_slots(int bin) { return kSlots[bin]; }

}  // namespace gsnp
