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
 * Here the records of a site stay on the SM: the pileup appends them to the
 * site's column ([slot][site] layout, so a warp's accesses fall in 32 distinct
 * banks whatever slot each lane is at), the column is sorted in place
 * (column.cuh), the likelihood walks it in that order, and only the 32-byte
 * SiteCall leaves the SM.  (The FP32 kernel's 256-slot bin keeps its columns
 * in a global scratch slice per CTA, read through L1.)
 *
 * The pileup of a site is every deposited read that covers it, in (start, file)
 * order.  That equals the reference's window-resident pileup: its carried-over
 * tail holds the previous window's reads first and the 255-record cap is
 * applied in that same order (kernel/update_kernel.cu:265-268,288).  A warp
 * walks the reads that can cover any of its 32 sites once, in that order; each
 * read's row is read with one coalesced load per lane band.
 *
 * Two calling kernels share this structure:
 *   call_tiles_kernel  FP64 sums in the reference's order (the plain form, and
 *                      windows whose likelihood another window reuses);
 *   call_fast_kernel   FP32 compensated sums and an FP32 posterior for
 *                      homozygous calls that the error bound proves; every
 *                      other site is deferred: its counts and sorted records
 *                      are appended to a small pool.  It runs no FP64
 *                      instruction.
 *   deferred_sites_kernel  one thread per deferred site: the FP32 sums again
 *                      with the double-precision bound checks, the FP64 sums
 *                      where those fail, the rank-sum test.
 * Tiles are binned by their deepest site (kNumBins record-slot capacities) so
 * that shared memory is sized for the tile, not for the worst case.
 */
#include <cuda_runtime.h>

#include "calling.cuh"
#include "site_math.cuh"
#include "tma.cuh"

namespace gsnp {

namespace {

constexpr unsigned kFull = 0xffffffffu;

/* bits of pcr occurrence count per (strand, cycle) key (walk_records) in the
 * bins of each record-slot capacity, for the FP32 (fast) or the FP64 kernel.
 * Two bits leave a scan back over the group only for a key seen three
 * times; at 30x one record in about fourteen repeats a key, and with one bit
 * the scans of single lanes held the whole warp (c1 at 25% scale:
 * fast<40> 2.63 -> 2.37 ms, tiles<40> 5.26 -> 4.97 ms).  The FP32 kernel's
 * 32-slot bin ran 3% slower with them and keeps one bit. */
__host__ __device__ constexpr int kPcrBits(int slots, bool fast) {
    return slots >= 96 ? 4 : (fast && slots <= 32) ? 1 : 2;
}

/* The FP32 kernel's 256-slot bin keeps its record columns in global memory
 * (CallArgs::deep_recs, one slice per CTA) instead of shared memory: 32 KB of
 * columns per one-warp CTA would allow 6 CTAs per SM, where the pcr counts
 * alone leave the SM limited by registers only (22.1 against 27.7 ms per c2
 * step).  The smaller deep bins, and the FP64 kernel's, ran slower that
 * way and keep shared memory. */
__host__ __device__ constexpr bool kGlobalRecs(int slots, bool fast) { return fast && slots >= 256; }

/* resident CTAs per SM the calling kernels are compiled for; this caps their
 * registers: 64 for the FP32 kernel (32 warps per SM, a few spilled words
 * cost less than the latency the extra warps hide), 128 for the FP64 one */
constexpr int kFastCtasPerSm = 32 * 32 / kTile;
constexpr int kFp64CtasPerSm = 16 * 32 / kTile;

__device__ __forceinline__ int lower_bound_s(const int32_t* a, int n, int64_t v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int64_t)a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* Running pileup of one site: per-base counters packed - count_uni 4 x 8
 * bits (at most 255 unique bases), q_sum and count_all 4 x 16 bits (a site
 * deeper than 65535 is a capacity error) - and its record column. */
struct PileupAcc {
    uint32_t cu4 = 0;
    uint64_t qs4 = 0, ca4 = 0;
    uint32_t depth = 0, repeat = 0;
    int dep_uni = 0, num = 0;
    bool overflow = false;

    /* one covering read's base (kernel/update_kernel.cu:278-325): bq is its
     * base | quality << 8 at the site, lh its (len << 16) | hit */
    template <int SLOTS>
    __device__ __forceinline__ void take(uint32_t bq, uint32_t lh, int coord, int minus, signed char qmin,
                                         uint32_t* recs) {
        const int rlen = (int)(lh >> 16);
        const uint32_t hit = lh & 0xffffu;
        const signed char base = (signed char)(bq & 0xff);
        const signed char qual = (signed char)(bq >> 8);
        depth += 1;
        repeat += hit;
        if (base == 'N' || qual < qmin || dep_uni >= 0xFF) return;
        const int sh = ((base >> 1) & 3) * 16;
        if (hit == 1) {
            dep_uni += 1;
            const int q = qual - qmin;
            const uint32_t coord_val = minus ? (uint32_t)(rlen - 1 - coord) : (uint32_t)coord;
            const uint32_t w = make_record(base, q, coord_val, (uint32_t)minus);
            if (num < SLOTS) {
                recs[num * kTile] = w;
                num += 1;
            } else {
                overflow = true;
            }
            cu4 += 1u << (sh >> 1);
            qs4 += (uint64_t)(uint32_t)q << sh;
        }
        ca4 += 1ull << sh;
    }

    __device__ __forceinline__ PackedPileup finish(const CallArgs& a, bool* report_overflow) const {
        if (report_overflow) *report_overflow = overflow;
        else if (overflow) atomicExch(a.error, 2);
        if (depth > 0xffff) atomicExch(a.error, 1);
        PackedPileup pk;
        pk.cu4 = cu4;
        pk.qs4 = qs4;
        pk.ca4 = ca4;
        pk.depth = depth;
        pk.repeat = repeat;
        pk.dep_uni = (uint16_t)dep_uni;
        pk.num = (uint16_t)num;
        return pk;
    }
};

/* Pileup of one warp's 32 consecutive sites (kernel/update_kernel.cu:260-325).
 * Reads [r_lo, r_hi) are those starting in [w0 - L + 1, w0 + 31]; their
 * positions, lengths and strands are loaded 32 at a time and broadcast, and
 * each lane takes the reads that cover its own site.  Records are appended to
 * the site's column in pileup order.  Lanes with !active only keep the warp's
 * loop going. */
template <int SLOTS>
__device__ __forceinline__ PackedPileup warp_pileup(const CallArgs& a, int64_t r_lo, int64_t r_hi, int64_t site,
                                                   bool active, uint32_t* recs, bool* report_overflow = nullptr) {
    /* records are appended in pileup order; sort_column puts them in
     * ascending order after the pileup */
    const int lane = threadIdx.x & 31;
    const int L = a.L;
    const signed char qmin = (signed char)a.qmin;
    PileupAcc acc;
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
        const uint16_t* rows = a.bq + rb * L;
        /* four reads at a time: their row loads are issued together, then
         * the covering ones are taken in order */
        for (int k0 = 0; k0 < cnt; k0 += 4) {
            uint32_t bqv[4], lhv[4];
            int coordv[4], minusv[4];
            bool covv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int k = k0 + u;
                const int32_t start = __shfl_sync(kFull, mpos, k & 31);
                lhv[u] = __shfl_sync(kFull, mlh, k & 31);
                minusv[u] = __shfl_sync(kFull, mminus, k & 31);
                coordv[u] = (int)(site - start);
                covv[u] = active && k < cnt && coordv[u] >= 0 && coordv[u] < (int)(lhv[u] >> 16);
                bqv[u] = covv[u] ? (uint32_t)__ldg(rows + k * L + coordv[u]) : 0u;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (covv[u]) acc.take<SLOTS>(bqv[u], lhv[u], coordv[u], minusv[u], qmin, recs);
        }
    }
    return acc.finish(a, report_overflow);
}

/* The reads of a tile staged in shared memory by the persistent kernel: per
 * read its start, (len << 16) | hit with the strand in bit 31, and the byte
 * offset in `rows` that column 0 of its row would have; the bulk copy of the
 * read holds the columns that cover the tile. */
struct StagedReads {
    const int32_t* pos;
    const uint32_t* lhs;
    const int32_t* rbase;
    const uint8_t* rows;
    int n;
};

/* warp_pileup over staged reads: the same records and counts, read from
 * shared memory (broadcast loads of the per-read values, one 16-bit load
 * per covering read and lane). */
template <int SLOTS>
__device__ __forceinline__ PackedPileup warp_pileup_staged(const CallArgs& a, const StagedReads& sr, int64_t site,
                                                          bool active, uint32_t* recs, bool* report_overflow) {
    const signed char qmin = (signed char)a.qmin;
    PileupAcc acc;
    for (int k = 0; k < sr.n; ++k) {
        const int32_t start = sr.pos[k];
        const uint32_t lhs = sr.lhs[k];
        const int coord = (int)(site - start);
        const uint32_t lh = lhs & 0x7fffffffu;
        if (active && coord >= 0 && coord < (int)(lh >> 16)) {
            const uint32_t bq = *reinterpret_cast<const uint16_t*>(sr.rows + sr.rbase[k] + 2 * coord);
            acc.take<SLOTS>(bq, lh, coord, (int)(lhs >> 31), qmin, recs);
        }
    }
    return acc.finish(a, report_overflow);
}

/* dbSNP row of each flagged site of a tile: the rows before the tile plus the
 * flagged sites before it in the tile (the rows are the flagged sites in
 * position order).  Every lane of the tile's warp calls it. */
__device__ __forceinline__ int32_t tile_snp_row(const CallArgs& a, int64_t tile, bool flagged) {
    const unsigned b = __ballot_sync(kFull, flagged);
    const int lane = threadIdx.x & 31;
    return flagged ? a.tile_snp[tile] + __popc(b & ((1u << lane) - 1u)) : -1;
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
    const int64_t t = p / kTile;
    int64_t lo, hi;
    if (p < win_end && t >= a.tile_lo && t < a.n_tiles) {
        /* p's tile's read range, [lower_bound(32 t - L + 1), lower_bound(32 t
         * + 32)): the same reads in the same order and a few more, which the
         * checks below skip, without two searches over every read.  (The
         * window's end is left to the searches: its next site can lie in a
         * tile the pass has not ranged.) */
        lo = a.tile_rng[t * 2];
        hi = a.tile_rng[t * 2 + 1];
    } else {
        lo = a.read_lo + lower_bound_g(a.pos + a.read_lo, a.n_reads - a.read_lo, p - a.L + 1);
        hi = a.read_lo + lower_bound_g(a.pos + a.read_lo, a.n_reads - a.read_lo, max_start + 1);
    }
    int dep_uni = 0, qsum = 0;
    const signed char qmin = (signed char)a.qmin;
    for (int64_t r = lo; r < hi; ++r) {
        const int64_t start = __ldg(a.pos + r);
        if (start > max_start) break;   /* the starts ascend */
        const int coord = (int)(p - start);
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

/* Read range of every tile, [lower_bound(s0 - L + 1), lower_bound(s0 + kTile)),
 * in one pass over the sorted starts: read r is the lower bound of every
 * boundary b with pos[r - 1] < b <= pos[r].  Threads r_begin .. r_end; the
 * start of read r_end is next_pos (kNoRead past the last read), so that a
 * segment of the reads can be done before the next segment is on the device:
 * consecutive segments share their boundary thread, which writes the same
 * values twice.  Only tiles [tile_lo, n_tiles) are written.  When the device
 * holds reads from read_lo > 0 on (a streamed chunk, whose first read is the
 * lower bound of its first tile's first boundary), the start before read_lo
 * is taken as tile_lo * kTile - L: it is at least that read's start and below
 * every boundary of the chunk's tiles. */
__global__ void tile_bounds_kernel(const int32_t* __restrict__ pos, int64_t r_begin, int64_t r_end, int64_t next_pos,
                                   int64_t tile_lo, int64_t n_tiles, int64_t read_lo, int L,
                                   int64_t* __restrict__ rng) {
    const int64_t r = r_begin + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r > r_end) return;
    const int64_t lo = r == 0 ? -kNoRead : r == read_lo ? tile_lo * kTile - L : (int64_t)pos[r - 1];
    const int64_t hi = r == r_end ? next_pos : (int64_t)pos[r];
    if (lo >= hi) return;
    auto fdiv = [](int64_t x) { return x >= 0 ? x / kTile : -((-x + kTile - 1) / kTile); };
    /* first boundaries t*kTile - L + 1 in (lo, hi] */
    int64_t t0 = fdiv(lo + L - 1) + 1, t1 = fdiv(hi + L - 1);
    if (t0 < tile_lo) t0 = tile_lo;
    if (t1 > n_tiles - 1) t1 = n_tiles - 1;
    for (int64_t t = t0; t <= t1; ++t) rng[t * 2] = r;
    /* second boundaries (t + 1)*kTile in (lo, hi] */
    t0 = fdiv(lo);
    t1 = fdiv(hi) - 1;
    if (t0 < tile_lo) t0 = tile_lo;
    if (t1 > n_tiles - 1) t1 = n_tiles - 1;
    for (int64_t t = t0; t <= t1; ++t) rng[t * 2 + 1] = r;
}

cudaError_t launch_tile_bounds(const CallArgs& a, int64_t r_begin, int64_t r_end, int64_t next_pos,
                               cudaStream_t stream) {
    const int64_t n = r_end - r_begin + 1;
    tile_bounds_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(a.pos, r_begin, r_end, next_pos, a.tile_lo,
                                                                         a.n_tiles, a.read_lo, a.L, a.tile_rng);
    return cudaGetLastError();
}

/* The FP64 call of a site with no record and no count for each of the 16
 * site codes (site_posterior over zero likelihoods), kept where it is
 * homozygous and does not depend on a dbSNP row. */
__global__ void empty_calls_kernel(CallArgs a, SiteCall* calls, uint8_t* valid) {
    const int code = threadIdx.x;
    if (code >= 16) return;
    SitePileup p;
#pragma unroll
    for (int i = 0; i < 4; ++i) { p.cu[i] = 0; p.qs[i] = 0; p.ca[i] = 0; }
    p.depth = 0;
    p.repeat = 0;
    p.dep_uni = 0;
    p.num = 0;
    double tl[16], lp[16];
    for (int i = 0; i < 16; ++i) {
        tl[i] = 0.0;
        lp[i] = a.log_prior[((code & 7) << 4) + i];
    }
    bool used_next = false;
    auto nq = [&](int) {
        used_next = true;
        return 0;
    };
    SiteCall c;
    site_posterior(a, (uint8_t)code, p, tl, nullptr, lp, nullptr, 1, nq, &c);
    const bool hom = (c.type1 >> 2) == (c.type1 & 3);
    valid[code] = hom && !used_next && !((code & 8) && a.refine);
    calls[code] = c;
}

cudaError_t launch_empty_calls(const CallArgs& a, SiteCall* calls, uint8_t* valid, cudaStream_t stream) {
    empty_calls_kernel<<<1, 32, 0, stream>>>(a, calls, valid);
    return cudaGetLastError();
}

/* Per tile: the deepest site's record need (reads starting in [site - L + 1,
 * site], capped at 255) picks the depth bin; the window's mode picks the FP64
 * kernel (bins 0 .. kNumBins-1) or the fast one (the next kNumBins).  Each
 * warp's read range is stored for the calling kernels.  A CTA classifies
 * kClassifyTiles tiles and adds its bin counts to the global ones with one
 * atomic per bin. */
constexpr int kClassifyThreads = 256;
constexpr int kClassifyTiles = kClassifyThreads / kTile;
constexpr int kClassifyStage = 256;   /* read starts staged in shared memory per tile */
static_assert(kClassifyThreads % kTile == 0, "a classify CTA holds whole tiles");

__global__ void __launch_bounds__(kClassifyThreads) classify_tiles_kernel(CallArgs a, int pass, int64_t t_begin,
                                                                          int64_t t_end, int* bin_count,
                                                                          int32_t* bin_tiles,
                                                                          const int32_t* __restrict__ list,
                                                                          const int* __restrict__ d_count) {
    __shared__ int32_t spos[kClassifyTiles][kClassifyStage];
    __shared__ int smax[kClassifyThreads / 32];
    __shared__ int sbin_count[2 * kNumBins], sbin_base[2 * kNumBins];
    const int lt = threadIdx.x / kTile, tt = threadIdx.x % kTile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    /* the tiles [t_begin, t_end), or with a list the tiles list[t_begin,
     * t_end); with d_count, t_end is t_begin + *d_count.  The CTAs take
     * kClassifyTiles tiles at a time, every gridDim.x-th group. */
    const int64_t end = d_count ? t_begin + *d_count : t_end;
    for (int64_t gbase = t_begin + (int64_t)blockIdx.x * kClassifyTiles; gbase < end;
         gbase += (int64_t)gridDim.x * kClassifyTiles) {
    const int64_t idx = gbase + lt;
    if (threadIdx.x < 2 * kNumBins) sbin_count[threadIdx.x] = 0;
    bool part = idx < end;
    const int64_t tile = list ? (part ? (int64_t)list[idx] : 0) : idx;
    const int64_t s0 = tile * kTile;
    uint8_t wflags = 0;
    if (part) {
        wflags = a.win_flags[(int)(s0 / kWin)];
        part = ((wflags & kWinExternalLik) != 0) == (pass == 1);
    }
    int64_t r_lo = 0, r_hi = 0;
    if (part) {
        r_lo = a.tile_rng[tile * 2];
        r_hi = a.tile_rng[tile * 2 + 1];
    }
    const int n = (int)(r_hi - r_lo);
    const bool staged = r_hi - r_lo <= kClassifyStage;
    if (part && staged)
        for (int i = tt; i < n; i += kTile) spos[lt][i] = __ldg(a.pos + r_lo + i);
    __syncthreads();
    auto lb = [&](int64_t v) -> int64_t {
        return staged ? r_lo + lower_bound_s(spos[lt], n, v) : r_lo + lower_bound_g(a.pos + r_lo, r_hi - r_lo, v);
    };
    const int64_t site = s0 + tt;
    int need = 0;
    if (part && site < a.chr_len) {
        const int64_t c = lb(site + 1) - lb(site - a.L + 1);
        need = (int)(c < kMaxRecords ? c : kMaxRecords);
    }
    if (part && lane < 2) a.warp_rng[tile * 2 + lane] = lane == 0 ? lb(s0 - a.L + 1) : lb(s0 + kTile);
    for (int off = 16; off > 0; off >>= 1) need = max(need, __shfl_xor_sync(kFull, need, off));
    if (lane == 0) smax[warp] = need;
    __syncthreads();
    int my_bin = -1, my_rank = 0;
    if (part && tt == 0) {
        const int m = smax[lt];
        const bool fast = a.precision == 1 && !(wflags & (kWinKeepLik | kWinExternalLik));
        int bin = 0;
        while (bin < kNumBins - 1 && m > a.bin_limit[bin]) ++bin;
        my_bin = bin + (fast ? kNumBins : 0);
        my_rank = atomicAdd(&sbin_count[my_bin], 1);
    }
    __syncthreads();
    if (threadIdx.x < 2 * kNumBins) {
        const int cnt = sbin_count[threadIdx.x];
        sbin_base[threadIdx.x] = cnt ? atomicAdd(&bin_count[threadIdx.x], cnt) : 0;
    }
    __syncthreads();
    if (my_bin >= 0) bin_tiles[(int64_t)my_bin * a.bin_stride + sbin_base[my_bin] + my_rank] = (int32_t)tile;
    __syncthreads();
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

/* One tile of the FP64 kernel; every lane of the warp calls it. */
template <int SLOTS>
__device__ __forceinline__ void fp64_tile(const CallArgs& a, int64_t tile, uint32_t* recs_all, uint32_t* seen_all) {
    const int t = threadIdx.x;
    const int64_t s0 = tile * kTile;
    const int win = (int)(s0 / kWin);
    const uint8_t wflags = a.win_flags[win];
    const int64_t r_lo = a.warp_rng[tile * 2];
    const int64_t r_hi = a.warp_rng[tile * 2 + 1];
    const int64_t site = s0 + t;
    const bool active = site < a.chr_len;
    const uint8_t ori = active ? __ldg(a.ori + site) : 0;
    const int32_t snp_row = tile_snp_row(a, tile, (ori & 8) != 0);
    const SitePileup p = warp_pileup<SLOTS>(a, r_lo, r_hi, site, active, recs_all + t).unpack();
    if (!active) return;
    uint32_t* recs = recs_all + t;
    uint32_t* seen = seen_all + t;
    sort_column<SLOTS>(recs, p.num);

    double tl[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) tl[i] = 0.0;
    if (wflags & kWinExternalLik) {
        const int src = a.win_lik_src[win];
        if (src >= 0) {
            const double* srcp = a.lik_keep + ((int64_t)src * kWin + (site - (int64_t)win * kWin)) * 10;
#pragma unroll
            for (int i = 0; i < 10; ++i) tl[genotype_of(i)] = srcp[i];
        }
    } else {
        likelihood_fp64<kPcrBits(SLOTS, false)>(a, recs, seen, kTile, p.num, tl);
        if (wflags & kWinKeepLik) {
            double* dst = a.lik_keep + site * 10;
#pragma unroll
            for (int i = 0; i < 10; ++i) dst[i] = tl[genotype_of(i)];
        }
    }
    if (wflags & kWinKeepCounts) store_counts(a, site, p);

    double lp[16];
    load_log_prior(a, snp_row, ori, lp);
    auto nq = [&](int b) { return neighbour_qsum(a, site, b); };
    SiteCall call;
    site_posterior(a, ori, p, tl, nullptr, lp, recs, kTile, nq, &call);
    a.out[site] = call;
}

/* The list entries [0, *count) of a grid sized to the resident CTAs (one
 * warp each): every CTA takes entry blockIdx.x first, then the next entry not
 * yet taken from the counter *next (zero before the launch), so that the
 * entries in flight stay neighbours and a CTA that drew cheap tiles takes
 * more of them. */
template <typename F>
__device__ __forceinline__ void for_each_listed(const int* __restrict__ count, int* next, F&& f) {
    const int n = *count;
    int i = blockIdx.x;
    while (i < n) {
        f(i);
        __syncwarp();
        int j = 0;
        if ((threadIdx.x & 31) == 0) j = atomicAdd(next, 1);
        i = __shfl_sync(0xffffffffu, j, 0) + (int)gridDim.x;
    }
}

/* The tiles of one depth bin: tiles[blockIdx.x] with count == nullptr (one
 * CTA per tile), else the first *count tiles of the list, handed out by
 * for_each_listed (a grid sized to the resident CTAs, whatever the count the
 * device holds). */
template <int SLOTS>
__global__ void __launch_bounds__(kTile, kFp64CtasPerSm) call_tiles_kernel(CallArgs a, const int32_t* __restrict__ tiles,
                                                                           const int* __restrict__ count, int* next) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint32_t* recs_all = reinterpret_cast<uint32_t*>(smem);                   /* [SLOTS][kTile] */
    uint32_t* seen_all = reinterpret_cast<uint32_t*>(smem) + SLOTS * kTile;    /* [nw][kTile] */
    if (!count) {
        fp64_tile<SLOTS>(a, tiles[blockIdx.x], recs_all, seen_all);
        return;
    }
    for_each_listed(count, next, [&](int i) { fp64_tile<SLOTS>(a, tiles[i], recs_all, seen_all); });
}

/* ------------------------------------------------------------------------ */
/* the fast calling kernel                                                   */
/* ------------------------------------------------------------------------ */

/* The FP32 work on one site of a tile after its pileup and sort: the
 * dependency walk, the compensated sums, the FP32 posterior, and the append
 * of the site to the deferred pool when its call is not proven.  Every lane
 * of the warp calls it (the appends are warp-aggregated). */
template <int SLOTS>
__device__ __forceinline__ void fast_site(const CallArgs& a, int64_t site, bool active, uint8_t ori, uint8_t wflags,
                                          int32_t snp_row, const SitePileup& p, uint32_t* recs, uint32_t* seen) {
    const int lane = threadIdx.x & 31;
    uint8_t dflags = 0;
    if (active) {
        if (wflags & kWinKeepCounts) store_counts(a, site, p);
        Kahan10 k;
        k.init();
        /* adjusted quality of each record, written over its occurrence byte */
        walk_records<true, kPcrBits(SLOTS, true)>(a, recs, seen, kTile, p.num, [&](int i, int qa, int, int) {
            recs[i * kTile] = (recs[i * kTile] & ~0xffu) | (uint32_t)qa;
        });
        /* FP32 sums, four records per compensated step (the grouping of
         * likelihood_fp32) */
        for (int i = 0; i < p.num; i += 4) {
            float x[10], y[10];
            uint32_t w = recs[i * kTile];
            lik32_row(a, (int)(w & 0xffu), rec_coord(w), rec_base(w), x);
            if (i + 1 < p.num) {
                w = recs[(i + 1) * kTile];
                lik32_row(a, (int)(w & 0xffu), rec_coord(w), rec_base(w), y);
#pragma unroll
                for (int v = 0; v < 10; ++v) x[v] = __fadd_rn(x[v], y[v]);
            }
            if (i + 2 < p.num) {
                float z[10];
                w = recs[(i + 2) * kTile];
                lik32_row(a, (int)(w & 0xffu), rec_coord(w), rec_base(w), y);
                if (i + 3 < p.num) {
                    w = recs[(i + 3) * kTile];
                    lik32_row(a, (int)(w & 0xffu), rec_coord(w), rec_base(w), z);
#pragma unroll
                    for (int v = 0; v < 10; ++v) y[v] = __fadd_rn(y[v], z[v]);
                }
#pragma unroll
                for (int v = 0; v < 10; ++v) x[v] = __fadd_rn(x[v], y[v]);
            }
            k.add(x);
        }
        SiteCall call;
        if ((site & 4095) == 0 && a.stats) dflags = kCallSampled;
        const bool empty = p.num == 0 && (p.ca[0] | p.ca[1] | p.ca[2] | p.ca[3]) == 0 && a.empty_valid[ori];
        if (empty) {
            /* no record and no count: the call depends on the site code only */
            call = a.empty_calls[ori];
            call.depth = p.depth;
            call.repeat_time = p.repeat;
            call.flags |= dflags;
        } else if (fast_posterior(a, snp_row, ori, p, k.s, p.num, &call)) {
            call.flags |= dflags;
        } else {
            call = SiteCall{};
            dflags |= kCallPending;
            call.flags = dflags;
        }
        a.out[site] = call;
    }
    /* append the deferred sites of the warp */
    const unsigned m = __ballot_sync(kFull, dflags != 0);
    if (m == 0) return;
    unsigned long long base = 0;
    const int leader = __ffs(m) - 1;
    if (lane == leader) base = atomicAdd(a.dcount, (unsigned long long)__popc(m));
    base = __shfl_sync(kFull, base, leader);
    if (!dflags) return;
    const unsigned long long slot = base + __popc(m & ((1u << lane) - 1u));
    const unsigned long long off = atomicAdd(a.dcount + 1, (unsigned long long)p.num);
    if ((int64_t)slot >= a.dsite_cap || (int64_t)(off + p.num) > a.dpool_cap) return;
    DeferredSite d;
    d.site = site;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        d.cu[i] = (uint16_t)p.cu[i];
        d.qs[i] = (uint16_t)p.qs[i];
        d.ca[i] = p.ca[i];
    }
    d.depth = p.depth;
    d.repeat = p.repeat;
    d.rec_off = (uint32_t)off;
    d.num = (uint16_t)p.num;
    d.dep_uni = (uint16_t)p.dep_uni;
    d.snp_row = snp_row;
    d.flags = dflags;
#pragma unroll
    for (int i = 0; i < 3; ++i) d.pad[i] = 0;
    a.dsites[slot] = d;
    uint32_t* dst = a.dpool + off;
    for (int i = 0; i < p.num; ++i) dst[i] = (recs[i * kTile] & ~0xffu) | 1u;
}

/* Sites whose call is not proven in FP32 (and every 4096th site, sampled for
 * the FP32 accuracy figure) are appended to the deferred pool: counts and the
 * sorted records with their occurrence byte restored.  The append counters
 * keep counting past the capacities so that the host can size the pool and
 * run the pass again. */
template <int SLOTS>
__device__ __forceinline__ void fast_tile(const CallArgs& a, int64_t tile, uint32_t* recs_all, uint32_t* seen_all) {
    const int t = threadIdx.x;
    const int64_t s0 = tile * kTile;
    const int win = (int)(s0 / kWin);
    const uint8_t wflags = a.win_flags[win];
    const int64_t r_lo = a.warp_rng[tile * 2];
    const int64_t r_hi = a.warp_rng[tile * 2 + 1];
    const int64_t site = s0 + t;
    const bool active = site < a.chr_len;
    const uint8_t ori = active ? __ldg(a.ori + site) : 0;
    const int32_t snp_row = tile_snp_row(a, tile, (ori & 8) != 0);
    const SitePileup p = warp_pileup<SLOTS>(a, r_lo, r_hi, site, active, recs_all + t).unpack();
    uint32_t* recs = recs_all + t;
    uint32_t* seen = seen_all + t;
    if (active) sort_column<SLOTS>(recs, p.num);

    fast_site<SLOTS>(a, site, active, ori, wflags, snp_row, p, recs, seen);
}

/* The tiles of one depth bin, as call_tiles_kernel takes them.  The deep
 * bins' record columns are the CTA's slice of a.deep_recs. */
template <int SLOTS>
__global__ void __launch_bounds__(kTile, kFastCtasPerSm) call_fast_kernel(CallArgs a, const int32_t* __restrict__ tiles,
                                                                          const int* __restrict__ count, int* next) {
    extern __shared__ __align__(16) uint8_t smem[];
    constexpr bool kGlobal = kGlobalRecs(SLOTS, true);
    uint32_t* recs_all = kGlobal ? a.deep_recs + (size_t)blockIdx.x * SLOTS * kTile : reinterpret_cast<uint32_t*>(smem);
    uint32_t* seen_all = reinterpret_cast<uint32_t*>(smem) + (kGlobal ? 0 : SLOTS * kTile);
    if (!count) {
        fast_tile<SLOTS>(a, tiles[blockIdx.x], recs_all, seen_all);
        return;
    }
    for_each_listed(count, next, [&](int i) { fast_tile<SLOTS>(a, tiles[i], recs_all, seen_all); });
}

/* ------------------------------------------------------------------------ */
/* the deep bins of the FP32 form: one warp per site                          */
/* ------------------------------------------------------------------------ */

/* Tiles with a site of more than 64 records (hotspots of hundreds of reads)
 * are called by a CTA of 32 warps, warp w calling site w of the tile, so that
 * a site's hundreds of records are spread over 32 lanes instead of walked by
 * one.  Per warp, in shared memory: the site's record column (at most 255
 * records) and a byte counter per (base, strand, cycle) key. */
constexpr int kDeepThreads = 32 * kTile;
constexpr int kDeepCap = 256;
constexpr int kDeepKeys = 4 * 2 * 256;
constexpr size_t kDeepSmem = (size_t)kTile * (kDeepCap * 4 + kDeepKeys);

/* The pileup of one site by its warp (kernel/update_kernel.cu:260-325, as
 * PileupAcc::take): the reads [r_lo, r_hi) 32 at a time, in order.  A
 * covering read counts in depth and repeat; one that is not N and reaches
 * q_min is taken while the site has fewer than 255 unique records, and a
 * unique one (hit 1) adds a record.  Whether the cap still admits a read
 * depends only on the unique valid reads before it, which a ballot gives, so
 * the 32 reads of a step are decided together with the reference's result.
 * Once the cap is reached a read can only add to depth and repeat, which
 * need no base or quality; the scan ends at the first step whose reads all
 * start past the site.
 *
 * The scan is bound by load latency (each step's base and quality load
 * depends on the read's start), so its loads run ahead of the decisions: an
 * iteration loads the starts and lengths of its kDeepAhead steps' reads in
 * the iteration before, and their bases, qualities and strands all at its
 * start (for every covering read, when the site was below the cap as the
 * iteration began; a step that finds the site capped leaves its loads
 * unused).  The steps are then decided in order, as above. */
constexpr int kDeepAhead = 2;

__device__ __forceinline__ SitePileup deep_pileup(const CallArgs& a, int64_t r_lo, int64_t r_hi, int64_t site,
                                                  uint32_t* recs) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const signed char qmin = (signed char)a.qmin;
    const int L = a.L;
    SitePileup p;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        p.cu[b] = 0;
        p.qs[b] = 0;
        p.ca[b] = 0;
    }
    p.depth = 0;
    p.repeat = 0;
    p.dep_uni = 0;
    p.num = 0;
    /* repeat and the quality sums per lane, added over the warp after the
     * scan (the same sums, modulo 2^32 as before) */
    uint32_t rep_l = 0, qs_l[4] = {0u, 0u, 0u, 0u};
    int32_t nst[kDeepAhead];
    uint32_t nlh[kDeepAhead];
#pragma unroll
    for (int u = 0; u < kDeepAhead; ++u) {
        const int64_t r = r_lo + 32 * u + lane;
        nst[u] = r < r_hi ? __ldg(a.pos + r) : 0;
        nlh[u] = r < r_hi ? (uint32_t)__ldg(a.lenhit + r) : 0u;
    }
    for (int64_t rb = r_lo; rb < r_hi; rb += 32 * kDeepAhead) {
        int coord[kDeepAhead];
        uint32_t lh[kDeepAhead], bq[kDeepAhead];
        bool cov[kDeepAhead], minus[kDeepAhead];
        const bool capped_at_start = p.dep_uni >= 0xFF;
#pragma unroll
        for (int u = 0; u < kDeepAhead; ++u) {
            const int64_t r = rb + 32 * u + lane;
            const bool in = r < r_hi;
            coord[u] = in ? (int)(site - nst[u]) : -1;
            lh[u] = nlh[u];
            cov[u] = in && coord[u] >= 0 && coord[u] < (int)(lh[u] >> 16);
            bq[u] = 0;
            minus[u] = false;
            if (cov[u] && !capped_at_start) {
                bq[u] = __ldg(a.bq + r * L + coord[u]);
                minus[u] = __ldg(a.strand + r) != '+';
            }
            const int64_t rn = r + 32 * kDeepAhead;
            nst[u] = rn < r_hi ? __ldg(a.pos + rn) : 0;
            nlh[u] = rn < r_hi ? (uint32_t)__ldg(a.lenhit + rn) : 0u;
        }
        bool past = false;
#pragma unroll
        for (int u = 0; u < kDeepAhead; ++u) {
            if (__all_sync(kFull, coord[u] < 0)) {   /* every read from here on starts past the site */
                past = true;
                break;
            }
            const unsigned mc = __ballot_sync(kFull, cov[u]);
            if (mc == 0) continue;
            const uint32_t hit = lh[u] & 0xffffu;
            p.depth += (uint32_t)__popc(mc);
            rep_l += cov[u] ? hit : 0u;
            if (p.dep_uni >= 0xFF) continue;
            const signed char base = (signed char)(bq[u] & 0xff);
            const signed char qual = (signed char)(bq[u] >> 8);
            const bool valid = cov[u] && base != 'N' && qual >= qmin;
            const bool uni = valid && hit == 1;
            const int uni_before = p.dep_uni + __popc(__ballot_sync(kFull, uni) & lt);
            const bool acc = valid && uni_before < 0xFF;
            const bool rec = acc && uni;
            const unsigned mr = __ballot_sync(kFull, rec);
            const int q = qual - qmin;
            if (rec) {
                const uint32_t cv =
                    minus[u] ? (uint32_t)((int)(lh[u] >> 16) - 1 - coord[u]) : (uint32_t)coord[u];
                recs[p.num + __popc(mr & lt)] = make_record(base, q, cv, (uint32_t)minus[u]);
            }
            p.num += __popc(mr);
            p.dep_uni += __popc(mr);
            const int bi = (base >> 1) & 3;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                p.cu[b] += __popc(__ballot_sync(kFull, rec && bi == b));
                qs_l[b] += (rec && bi == b) ? (uint32_t)q : 0u;
                p.ca[b] += (uint32_t)__popc(__ballot_sync(kFull, acc && bi == b));
            }
        }
        if (past) break;
    }
    p.repeat = __reduce_add_sync(kFull, rep_l);
#pragma unroll
    for (int b = 0; b < 4; ++b) p.qs[b] = (int)__reduce_add_sync(kFull, qs_l[b]);
    return p;
}

/* Ascending bitonic sort of v[0, n), n <= kDeepCap = 256, by the lanes of a
 * warp in registers: lane l holds elements 8l .. 8l+7 (padded with
 * 0xFFFFFFFF, which no record word equals).  The network's stages of
 * distance j < 8 are compare-exchanges within a lane; those of distance
 * j >= 8 pair lane l with lane l ^ (j / 8), which keeps the smaller or the
 * larger of each of its eight elements.  Every loop bound is a constant, so
 * the 36 stages unroll into straight code with no index arithmetic and no
 * shared-memory traffic between them. */
__device__ __forceinline__ void deep_sort(uint32_t* v, int n) {
    static_assert(kDeepCap == 256, "eight elements a lane");
    const int lane = threadIdx.x & 31;
    uint32_t x[8];
    const uint4 lo4 = reinterpret_cast<const uint4*>(v)[lane * 2];
    const uint4 hi4 = reinterpret_cast<const uint4*>(v)[lane * 2 + 1];
    x[0] = lo4.x, x[1] = lo4.y, x[2] = lo4.z, x[3] = lo4.w;
    x[4] = hi4.x, x[5] = hi4.y, x[6] = hi4.z, x[7] = hi4.w;
#pragma unroll
    for (int e = 0; e < 8; ++e)
        if (lane * 8 + e >= n) x[e] = 0xFFFFFFFFu;
#pragma unroll
    for (int k = 2; k <= 256; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 8) {
                const int d = j >> 3;
                const bool keep_min = (((lane * 8) & k) == 0) == ((lane & d) == 0);
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const uint32_t y = __shfl_xor_sync(kFull, x[e], d);
                    x[e] = keep_min ? min(x[e], y) : max(x[e], y);
                }
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    if (e & j) continue;
                    const int f = e | j;
                    const bool asc = ((lane * 8 + e) & k) == 0;
                    const uint32_t a = min(x[e], x[f]), b = max(x[e], x[f]);
                    x[e] = asc ? a : b;
                    x[f] = asc ? b : a;
                }
            }
        }
    }
    __syncwarp();
    reinterpret_cast<uint4*>(v)[lane * 2] = make_uint4(x[0], x[1], x[2], x[3]);
    reinterpret_cast<uint4*>(v)[lane * 2 + 1] = make_uint4(x[4], x[5], x[6], x[7]);
    __syncwarp();
}

/* The dependency walk and the FP32 sums of a sorted column by its warp,
 * 32 records a step, record c0 + lane on that lane.  The walk's two counts
 * (walk_records) come from the whole step at once:
 *   - tmp, the earlier records of the same (base, strand, cycle) key: the
 *     key's counter from the steps before plus the lower lanes with that key
 *     (match-any); the highest of them then stores the new count;
 *   - gdc, the first occurrences of a key (tmp = 0) so far in the record's
 *     base group, less one: a ballot prefix, from the lane where the base
 *     group starts, or carried over from the step before.
 * Each lane sums its records' rows with compensation; the 32 sums are then
 * added in a tree (the bound of fast_posterior's k_units 9). */
__device__ __forceinline__ void deep_walk_sums(const CallArgs& a, const uint32_t* recs, uint8_t* cnt, int num,
                                               float* s) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u, le = (lt << 1) | 1u;
    for (int i = lane; i < kDeepKeys / 4; i += 32) reinterpret_cast<uint32_t*>(cnt)[i] = 0u;
    __syncwarp();
    Kahan10 k;
    k.init();
    int carry_firsts = 0, carry_base = -1;
    for (int c0 = 0; c0 < num; c0 += 32) {
        const int i = c0 + lane;
        const bool valid = i < num;
        const uint32_t w = valid ? recs[i] : 0u;
        const int o = rec_base(w), coord = rec_coord(w);
        const int key = valid ? (o << 9) | (rec_strand(w) << 8) | coord : kDeepKeys + lane;
        const unsigned peers = __match_any_sync(kFull, key);
        const int seen = valid ? (int)cnt[key] : 0;
        __syncwarp();
        const int tmp = seen + __popc(peers & lt);
        if (valid && (peers >> lane) == 1u) cnt[key] = (uint8_t)(seen + __popc(peers));
        __syncwarp();
        const int prev_o = __shfl_up_sync(kFull, o, 1);
        const bool brk = valid && o != (lane == 0 ? carry_base : prev_o);
        const unsigned bm = __ballot_sync(kFull, brk) & le;
        const unsigned fm = __ballot_sync(kFull, valid && tmp == 0) & le;
        const int firsts = bm ? __popc(fm & ~((1u << (31 - __clz(bm))) - 1u)) : carry_firsts + __popc(fm);
        carry_firsts = __shfl_sync(kFull, firsts, 31);
        carry_base = __shfl_sync(kFull, o, 31);
        if (valid) {
            const int gdc = firsts - 1, t1 = tmp + 1;
            const int qa = (t1 < a.tmax && gdc < a.gmax)
                               ? (int)__ldg(a.qadj + ((size_t)t1 * a.gmax + gdc) * 65 + rec_q(w))
                               : 1;
            float x[10];
            lik32_row(a, qa, coord, o, x);
            k.add(x);
        }
    }
#pragma unroll
    for (int v = 0; v < 10; ++v) {
        float t = k.s[v];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) t = __fadd_rn(t, __shfl_xor_sync(kFull, t, d));
        s[v] = t;
    }
}

/* Site w of a deep tile, called by one warp (as fast_site: counts kept for
 * later gap windows, the FP32 posterior, or the site deferred with its
 * records). */
__device__ __forceinline__ void deep_tile(const CallArgs& a, int64_t tile, int w, uint32_t* recs, uint8_t* cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t s0 = tile * kTile, site = s0 + w;
    const int64_t sl = s0 + lane;
    const uint8_t ori_l = sl < a.chr_len ? __ldg(a.ori + sl) : 0;
    const unsigned flagged = __ballot_sync(kFull, (ori_l & 8) != 0);
    if (site >= a.chr_len) return;
    const uint8_t ori = (uint8_t)__shfl_sync(kFull, ori_l, w);
    const int32_t snp_row = (ori & 8) ? a.tile_snp[tile] + __popc(flagged & ((1u << w) - 1u)) : -1;
    const uint8_t wflags = a.win_flags[s0 / kWin];
    const SitePileup p = deep_pileup(a, a.warp_rng[tile * 2], a.warp_rng[tile * 2 + 1], site, recs);
    __syncwarp();
    deep_sort(recs, p.num);
    float s[10];
    deep_walk_sums(a, recs, cnt, p.num, s);
    uint8_t dflags = 0;
    if (lane == 0) {
        if (p.depth > 0xffff) atomicExch(a.error, 1);
        if (wflags & kWinKeepCounts) store_counts(a, site, p);
        SiteCall call;
        if ((site & 4095) == 0 && a.stats) dflags = kCallSampled;
        const bool empty = p.num == 0 && (p.ca[0] | p.ca[1] | p.ca[2] | p.ca[3]) == 0 && a.empty_valid[ori];
        if (empty) {
            call = a.empty_calls[ori];
            call.depth = p.depth;
            call.repeat_time = p.repeat;
            call.flags |= dflags;
        } else if (fast_posterior(a, snp_row, ori, p, s, p.num, &call, 9.0f)) {
            call.flags |= dflags;
        } else {
            call = SiteCall{};
            dflags |= kCallPending;
            call.flags = dflags;
        }
        a.out[site] = call;
    }
    dflags = (uint8_t)__shfl_sync(kFull, dflags, 0);
    if (!dflags) return;
    /* the site and its sorted records to the deferred pool */
    unsigned long long slot = 0, off = 0;
    if (lane == 0) {
        slot = atomicAdd(a.dcount, 1ull);
        off = atomicAdd(a.dcount + 1, (unsigned long long)p.num);
    }
    slot = __shfl_sync(kFull, slot, 0);
    off = __shfl_sync(kFull, off, 0);
    if ((int64_t)slot >= a.dsite_cap || (int64_t)(off + p.num) > a.dpool_cap) return;
    for (int i = lane; i < p.num; i += 32) a.dpool[off + i] = recs[i];
    if (lane == 0) {
        DeferredSite d;
        d.site = site;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            d.cu[b] = (uint16_t)p.cu[b];
            d.qs[b] = (uint16_t)p.qs[b];
            d.ca[b] = p.ca[b];
        }
        d.depth = p.depth;
        d.repeat = p.repeat;
        d.rec_off = (uint32_t)off;
        d.num = (uint16_t)p.num;
        d.dep_uni = (uint16_t)p.dep_uni;
        d.snp_row = snp_row;
        d.flags = dflags;
#pragma unroll
        for (int b = 0; b < 3; ++b) d.pad[b] = 0;
        a.dsites[slot] = d;
    }
}

/* The tiles of a deep FP32 bin: tiles[blockIdx.x] with count == nullptr, warp
 * w calling its site w; else the sites of the first *count tiles of the list,
 * handed out one at a time to each warp from *next (zero before the launch),
 * so that no warp waits for the deepest site of a tile. */
__global__ void __launch_bounds__(kDeepThreads, 1) call_deep_kernel(CallArgs a, const int32_t* __restrict__ tiles,
                                                                    const int* __restrict__ count, int* next) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* recs = reinterpret_cast<uint32_t*>(smem) + (size_t)w * kDeepCap;
    uint8_t* cnt = smem + (size_t)kTile * kDeepCap * 4 + (size_t)w * kDeepKeys;
    if (!count) {
        deep_tile(a, tiles[blockIdx.x], w, recs, cnt);
        return;
    }
    const unsigned items = (unsigned)*count * kTile;   /* tile-list index * kTile + site */
    unsigned item = blockIdx.x * kTile + w;
    while (item < items) {
        deep_tile(a, tiles[item / kTile], (int)(item % kTile), recs, cnt);
        unsigned nx = 0;
        if (lane == 0) nx = (unsigned)atomicAdd(next, 1) + gridDim.x * kTile;
        item = __shfl_sync(kFull, nx, 0);
    }
}

/* ------------------------------------------------------------------------ */
/* the persistent FP32 calling kernel                                        */
/* ------------------------------------------------------------------------ */

/* Reads of a tile staged in shared memory by the persistent kernel, and the
 * bytes of each read's row window (32 columns of 16-bit base|quality plus up
 * to 14 bytes before them, to start the copy on a 16-byte boundary).  A tile
 * with more reads than this (deep pileups) reads its rows from global memory
 * instead. */
constexpr int kStageReads = 56;
constexpr int kStageSlot = 80;
constexpr uint64_t kStageWaitNs = 1000000000ull;   /* bound on one wait for a tile's bulk copies */
constexpr int kStageHeader = 16 + kStageReads * 12;
/* how the persistent kernel fetches a tile's reads */
constexpr int kStreamPlain = 0;      /* loads from global memory (through L1/L2) */
constexpr int kStreamPrefetch = 1;   /* the same, after a bulk prefetch of the rows into L2 */
constexpr int kStreamStaged = 2;     /* bulk copies into shared memory, one tile ahead */
static_assert(kStageHeader % 16 == 0 && kStageSlot % 16 == 0, "staging buffers are 16-byte aligned");

/* One launch over the FP32 windows' tiles of a segment: each warp takes
 * kStreamChunk consecutive tiles at a time from a counter, so the tiles in
 * flight are neighbours and the read rows they share are fetched from DRAM
 * about once and then served by L2.  The grid is sized to the resident CTAs,
 * whatever the segment's length.  A tile whose window needs the FP64 form
 * (its likelihood is kept for, or taken from, another window), or one with a
 * site of more than SLOTS records, is appended to the leftover list for the
 * binned kernels instead.
 *
 * MODE kStreamPrefetch: as soon as a warp takes a tile, it asks the
 * bulk-copy unit to prefetch the next tile's read rows into L2
 * (cp.async.bulk.prefetch), which costs no shared memory.
 * MODE kStreamStaged: as soon as a tile's pileup is done, the warp stages the
 * next tile's reads in shared memory - their start, length and strand with plain
 * loads, and each covering read's 32-column row window with one bulk copy
 * (cp.async.bulk) completing on the warp's mbarrier - so that the copies run
 * while the current tile is sorted, walked and summed, and the next pileup
 * reads only shared memory.  A wait for the copies that does not complete
 * within kStageWaitNs sets error code 5 and ends the warp. */
template <int SLOTS, int MODE>
__global__ void __launch_bounds__(kTile, kFastCtasPerSm) call_stream_kernel(CallArgs a, StreamQueue q) {
    constexpr bool STAGED = MODE == kStreamStaged;
    extern __shared__ __align__(16) uint8_t smem[];
    uint8_t* base = smem;
    uint64_t* bar = nullptr;
    int32_t* s_pos = nullptr;
    uint32_t* s_lhs = nullptr;
    int32_t* s_rbase = nullptr;
    uint8_t* s_rows = nullptr;
    if (STAGED) {
        bar = reinterpret_cast<uint64_t*>(base);
        s_pos = reinterpret_cast<int32_t*>(base + 16);
        s_lhs = reinterpret_cast<uint32_t*>(s_pos + kStageReads);
        s_rbase = reinterpret_cast<int32_t*>(s_lhs + kStageReads);
        s_rows = base + kStageHeader;
        base = s_rows + kStageReads * kStageSlot;
    }
    uint32_t* recs_all = reinterpret_cast<uint32_t*>(base);
    uint32_t* seen_all = recs_all + SLOTS * kTile;
    const int t = threadIdx.x;
    uint32_t* recs = recs_all + t;
    uint32_t* seen = seen_all + t;
    const int64_t n = q.t_end - q.t_begin;

    /* tiles in order: kStreamChunk at a time from the counter; -1 at the end */
    int64_t chunk_next = 0, chunk_end = 0;
    auto next_tile = [&]() -> int64_t {
        if (chunk_next >= chunk_end) {
            unsigned long long first = 0;
            if (t == 0) first = atomicAdd(q.next, (unsigned long long)kStreamChunk);
            first = __shfl_sync(kFull, first, 0);
            chunk_next = (int64_t)first;
            chunk_end = min(chunk_next + (int64_t)kStreamChunk, n);
            if (chunk_next >= n) {
                chunk_end = 0;
                return -1;
            }
        }
        return q.t_begin + chunk_next++;
    };
    auto fp64_window = [&](int64_t tile) {
        return (a.win_flags[(int)(tile * kTile / kWin)] & (kWinKeepLik | kWinExternalLik)) != 0;
    };
    /* stage the reads of `tile` (see above); their count, or -1 when the
     * tile is not staged.  Every lane calls it, after its last read of the
     * buffers. */
    auto stage = [&](int64_t tile) -> int {
        if (!STAGED || tile < 0 || fp64_window(tile)) return -1;
        const int64_t r_lo = a.tile_rng[tile * 2], r_hi = a.tile_rng[tile * 2 + 1];
        const int64_t nr = r_hi - r_lo;
        if (nr > kStageReads) return -1;
        const int64_t s0 = tile * kTile;
        uint32_t bytes[2] = {0u, 0u}, total = 0;
        const uint8_t* src[2] = {nullptr, nullptr};
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int k = t + 32 * j;
            if (k >= nr) continue;
            const int64_t r = r_lo + k;
            const int32_t pos = __ldg(a.pos + r);
            const uint32_t lh = (uint32_t)__ldg(a.lenhit + r);
            const uint32_t minus = __ldg(a.strand + r) != '+';
            const int len = (int)(lh >> 16);
            const int c_lo = max(0, (int)(s0 - pos));
            const int c_hi = min(len, (int)(s0 + kTile - pos));
            const int64_t e_lo = (r * a.L + c_lo) * 2;   /* byte offset of column c_lo in the rows */
            const int m = (int)(e_lo & 15);
            if (c_hi > c_lo) {
                bytes[j] = (uint32_t)((m + 2 * (c_hi - c_lo) + 15) & ~15);
                src[j] = reinterpret_cast<const uint8_t*>(a.bq) + (e_lo - m);
            }
            s_pos[k] = pos;
            s_lhs[k] = lh | (minus << 31);
            s_rbase[k] = k * kStageSlot + m - 2 * c_lo;
            total += bytes[j];
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) total += __shfl_xor_sync(kFull, total, off);
        /* this lane's reads of the rows are done before the copies overwrite them */
        fence_proxy_async_smem();
        if (t == 0) mbar_arrive_expect_tx(bar, total);
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 2; ++j)
            if (bytes[j]) bulk_copy_g2s(s_rows + (t + 32 * j) * kStageSlot, src[j], bytes[j], bar);
        return (int)nr;
    };

    /* the read rows of `tile` into L2 (the rows of a tile's reads are one
     * contiguous block; the bulk unit wants 16-byte bounds, and the row
     * array has slack past its end for the rounding) */
    auto prefetch_l2 = [&](int64_t tile) {
        if (MODE != kStreamPrefetch || tile < 0 || t != 0) return;
        const int64_t r_lo = a.tile_rng[tile * 2], r_hi = a.tile_rng[tile * 2 + 1];
        if (r_hi <= r_lo) return;
        const uintptr_t lo = reinterpret_cast<uintptr_t>(a.bq + r_lo * a.L) & ~(uintptr_t)15;
        const uintptr_t hi = (reinterpret_cast<uintptr_t>(a.bq + r_hi * a.L) + 15) & ~(uintptr_t)15;
        bulk_prefetch_l2(reinterpret_cast<const void*>(lo), (uint32_t)(hi - lo));
    };

    uint32_t phase = 0;
    if (STAGED) {
        if (t == 0) mbar_init(bar, 1);
        __syncwarp();
    }
    int64_t tile = next_tile();
    int staged_n = stage(tile);
    while (tile >= 0) {
        const int64_t s0 = tile * kTile;
        const int win = (int)(s0 / kWin);
        const uint8_t wflags = a.win_flags[win];
        const int64_t nxt = next_tile();
        prefetch_l2(nxt);
        if (wflags & (kWinKeepLik | kWinExternalLik)) {
            if (t == 0) q.leftover[atomicAdd(q.n_leftover, 1)] = (int32_t)tile;
            tile = nxt;
            staged_n = stage(tile);
            continue;
        }
        const int64_t site = s0 + t;
        const bool active = site < a.chr_len;
        const uint8_t ori = active ? __ldg(a.ori + site) : 0;
        const int32_t snp_row = tile_snp_row(a, tile, (ori & 8) != 0);
        bool overflow = false;
        SitePileup p;
        if (STAGED && staged_n >= 0) {
            if (!mbar_wait_bounded(bar, phase, kStageWaitNs)) {
                if (t == 0) atomicExch(a.error, 5);
                (void)mbar_wait_bounded(bar, phase, kStageWaitNs);
                return;
            }
            phase ^= 1u;
            const StagedReads sr{s_pos, s_lhs, s_rbase, s_rows, staged_n};
            p = warp_pileup_staged<SLOTS>(a, sr, site, active, recs, &overflow).unpack();
        } else {
            p = warp_pileup<SLOTS>(a, a.tile_rng[tile * 2], a.tile_rng[tile * 2 + 1], site, active, recs, &overflow)
                    .unpack();
        }
        /* the staging buffers are free: stage the next tile now, so that its
         * copies run while this one is sorted, walked and summed */
        const int staged_next = stage(nxt);
        if (__any_sync(kFull, overflow)) {
            if (t == 0) q.leftover[atomicAdd(q.n_leftover, 1)] = (int32_t)tile;
        } else {
            /* one sort network for every tile: specialised networks per
             * tile depth made the kernel's code larger and it ran slower */
            if (active) sort_column<SLOTS>(recs, p.num);
            fast_site<SLOTS>(a, site, active, ori, wflags, snp_row, p, recs, seen);
        }
        tile = nxt;
        staged_n = staged_next;
        __syncwarp();
    }
}

/* The adjusted-quality table index of every record of a sorted column whose
 * records have occurrence 1 (the deferred pool's), or -1 where q_adj is 1:
 * walk_records' counts with BITS per key, without its table loads, so that
 * the loads can be issued many at a time afterwards. */
template <int BITS>
__device__ void walk_qidx(const CallArgs& a, const uint32_t* recs, uint32_t* seen, int num, int* qidx) {
    constexpr int kPer = 32 / BITS;
    constexpr uint32_t kMax = (1u << BITS) - 1u;
    const int L = a.L;
    const int nw = pcr_words(L, BITS);
    const bool sat_exact = BITS == 4 && a.tmax <= 16;
    int gdc = -1, last_o = -1, gstart = 0;
    for (int i = 0; i < num; ++i) {
        const uint32_t w = recs[i];
        const int o = rec_base(w);
        const int key = rec_strand(w) * L + rec_coord(w);
        if (o != last_o) {
            for (int k = 0; k < nw; ++k) seen[k] = 0u;
            gstart = i;
            gdc = -1;
            last_o = o;
        }
        uint32_t* cw = seen + key / kPer;
        const int sh = (key % kPer) * BITS;
        const uint32_t word = *cw;
        const uint32_t cnt = (word >> sh) & kMax;
        int tmp = (int)cnt;
        if (cnt == kMax && !sat_exact) {
            tmp = 0;
            for (int j = gstart; j < i; ++j)
                if (((recs[j] ^ w) & 0x1ff00u) == 0) tmp += 1;
        }
        if (cnt != kMax) *cw = (word & ~(kMax << sh)) | ((cnt + 1u) << sh);
        if (tmp == 0) gdc += 1;
        tmp++;
        qidx[i] = (tmp < a.tmax && gdc < a.gmax) ? (tmp * a.gmax + gdc) * 65 + rec_q(w) : -1;
    }
}

/* adjusted quality of record i from walk_qidx's index */
__device__ __forceinline__ int qa_of(const CallArgs& a, const int* qidx, int i) {
    return qidx[i] >= 0 ? (int)__ldg(a.qadj + qidx[i]) : 1;
}

/* likelihood_fp32's sums from walk_qidx's indices: four records' loads at a
 * time, added in the same grouping ((x0 + x1) + (x2 + x3)) and compensation,
 * so the values are those of likelihood_fp32 and of the fast kernels */
__device__ void deferred_fp32(const CallArgs& a, const uint32_t* recs, const int* qidx, int num, double* tl,
                              double* eps) {
    Kahan10 k;
    k.init();
    for (int i = 0; i < num; i += 4) {
        int qa[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) qa[u] = i + u < num ? qa_of(a, qidx, i + u) : 1;
        float x[10], y[10];
        lik32_row(a, qa[0], rec_coord(recs[i]), rec_base(recs[i]), x);
        if (i + 1 < num) {
            lik32_row(a, qa[1], rec_coord(recs[i + 1]), rec_base(recs[i + 1]), y);
#pragma unroll
            for (int v = 0; v < 10; ++v) x[v] = __fadd_rn(x[v], y[v]);
        }
        if (i + 2 < num) {
            float z[10];
            lik32_row(a, qa[2], rec_coord(recs[i + 2]), rec_base(recs[i + 2]), y);
            if (i + 3 < num) {
                lik32_row(a, qa[3], rec_coord(recs[i + 3]), rec_base(recs[i + 3]), z);
#pragma unroll
                for (int v = 0; v < 10; ++v) y[v] = __fadd_rn(y[v], z[v]);
            }
#pragma unroll
            for (int v = 0; v < 10; ++v) x[v] = __fadd_rn(x[v], y[v]);
        }
        k.add(x);
    }
    const double kk = GSNP_FP32_K(num);
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        const int g = genotype_of(i);
        tl[g] = (double)k.s[i];
        eps[g] = isinf(tl[g]) ? 0.0 : fabs(tl[g]) * kk;
    }
}

/* likelihood_fp64's sums from walk_qidx's indices: four records' rows loaded
 * together, their terms added record by record in the reference's order */
__device__ void deferred_fp64(const CallArgs& a, const uint32_t* recs, const int* qidx, int num, double* tl) {
    double s[10];
#pragma unroll
    for (int v = 0; v < 10; ++v) s[v] = 0.0;
    for (int i = 0; i < num; i += 4) {
        double2 r[4][5];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u < num) {
                const uint32_t w = recs[i + u];
                const double2* row = reinterpret_cast<const double2*>(
                    a.lik64 + ((size_t)(qa_of(a, qidx, i + u) * a.L + rec_coord(w)) * 4 + rec_base(w)) * 10);
#pragma unroll
                for (int v = 0; v < 5; ++v) r[u][v] = __ldg(row + v);
            }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u < num) {
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    s[2 * v] = GSNP_DADD(s[2 * v], r[u][v].x);
                    s[2 * v + 1] = GSNP_DADD(s[2 * v + 1], r[u][v].y);
                }
            }
    }
#pragma unroll
    for (int i = 0; i < 10; ++i) tl[genotype_of(i)] = s[i];
}

/* The FP64 pass over the deferred sites, one thread per site: the FP32 sums
 * again (the same pairing, hence the same values) with the double-precision
 * bound checks, then the FP64 sums where those fail.  Sampled sites also get
 * the FP64 sums for the accuracy figure, and when the fast kernel had decided
 * them its call is compared with this one. */
__device__ __forceinline__ void deferred_site(const CallArgs& a, int64_t i);

/* n sites, or with d_n the count the fast kernels requested (a.dcount[0]),
 * at most the pool's capacity, each thread taking every (grid)-th site */
__global__ void __launch_bounds__(32) deferred_sites_kernel(CallArgs a, int64_t n, const unsigned long long* d_n) {
    if (d_n) n = (int64_t)min(*d_n, (unsigned long long)a.dsite_cap);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        deferred_site(a, i);
}

__device__ __forceinline__ void deferred_site(const CallArgs& a, int64_t i) {
    const DeferredSite d = a.dsites[i];
    const int64_t site = d.site;
    const uint32_t* recs = a.dpool + d.rec_off;
    uint32_t seen[64];   /* 4-bit pcr counts of 2L <= 510 keys (walk_records) */
    SitePileup p;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        p.cu[b] = d.cu[b];
        p.qs[b] = d.qs[b];
        p.ca[b] = d.ca[b];
    }
    p.depth = d.depth;
    p.repeat = d.repeat;
    p.dep_uni = d.dep_uni;
    p.num = d.num;
    double tl[16], eps[16];
#pragma unroll
    for (int g = 0; g < 16; ++g) { tl[g] = 0.0; eps[g] = 0.0; }
    /* the walk's table indices once, then the sums with their loads batched */
    int qidx[256];
    walk_qidx<4>(a, recs, seen, p.num, qidx);
    deferred_fp32(a, recs, qidx, p.num, tl, eps);
    if (d.flags & kCallSampled) {
        double t64[16];
#pragma unroll
        for (int g = 0; g < 16; ++g) t64[g] = 0.0;
        deferred_fp64(a, recs, qidx, p.num, t64);
        double m = 0.0;
#pragma unroll
        for (int g = 0; g < 16; ++g) m = fmax(m, fabs(t64[g] - tl[g]));
        atomicMax(a.stats + 3, (unsigned long long)__double_as_longlong(m));
        atomicAdd(a.stats + 2, 1ull);
    }
    const uint8_t ori = __ldg(a.ori + site);
    double lp[16];
    load_log_prior(a, d.snp_row, ori, lp);
    auto nq = [&](int b) { return neighbour_qsum(a, site, b); };
    SiteCall call;
    if (!site_posterior<true>(a, ori, p, tl, eps, lp, recs, 1, nq, &call)) {
        /* FP64 fixup: the FP32 likelihood is too close to a decision boundary */
        deferred_fp64(a, recs, qidx, p.num, tl);
        site_posterior<true>(a, ori, p, tl, nullptr, lp, recs, 1, nq, &call);
        call.flags |= kCallFixup;
        atomicAdd(a.stats + 1, 1ull);
    }
    if (d.flags & kCallPending) {
        atomicAdd(a.stats + 4, 1ull);
    } else if (!same_call(a.out[site], call)) {
        /* a sampled site the fast kernel decided differs from the FP64 call */
        atomicAdd(a.stats + 5, 1ull);
    }
    a.out[site] = call;
}

/* ------------------------------------------------------------------------ */
/* launchers                                                                 */
/* ------------------------------------------------------------------------ */

static const int kSlots[kNumBins] = {32, 40, 48, 64, 96, 128, 256};

size_t call_smem_bytes(int slots, int L, bool fast) {
    /* records [slots][kTile] (unless in global memory), then the pcr state
     * [nw][kTile] */
    const size_t nw = (size_t)pcr_words(L, kPcrBits(slots, fast));
    return (kGlobalRecs(slots, fast) ? 0 : (size_t)slots * kTile * 4) + nw * kTile * 4;
}

/* Classify tiles [t_begin, t_end) (with a list, list[t_begin, t_end); with
 * d_count, list[0, *d_count) read on the device, by a fixed grid of `grid`
 * CTAs) into the depth bins. */
cudaError_t launch_classify(const CallArgs& a, int pass, int64_t t_begin, int64_t t_end, int* d_bin_count,
                            int32_t* d_bin_tiles, cudaStream_t stream, const int32_t* list, const int* d_count,
                            int grid) {
    cudaError_t e = cudaMemsetAsync(d_bin_count, 0, sizeof(int) * kBinCountInts, stream);
    if (e != cudaSuccess) return e;
    const unsigned blocks =
        d_count ? (unsigned)grid : (unsigned)((t_end - t_begin + kClassifyTiles - 1) / kClassifyTiles);
    if (blocks == 0) return cudaSuccess;
    classify_tiles_kernel<<<blocks, kClassifyThreads, 0, stream>>>(a, pass, t_begin, t_end, d_bin_count, d_bin_tiles,
                                                                   list, d_count);
    return cudaGetLastError();
}

/* Launchers set their kernel's shared-memory size and carveout before each
 * launch, except while this thread captures a graph: the attributes were set
 * when the grids were sized, before the capture. */
thread_local bool g_launch_attributes = true;
void set_launch_attributes(bool on) { g_launch_attributes = on; }

size_t stream_smem_bytes(int slots, int L, int mode) {
    return call_smem_bytes(slots, L, true) +
           (mode == kStreamStaged ? (size_t)kStageHeader + (size_t)kStageReads * kStageSlot : 0);
}

template <int SLOTS, int MODE>
static cudaError_t stream_attr(int L, int* ctas_per_sm, int carveout = 0) {
    const int smem = (int)stream_smem_bytes(SLOTS, L, MODE);
    cudaError_t e =
        cudaFuncSetAttribute(call_stream_kernel<SLOTS, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    /* a preferred shared-memory carveout (percent; 0 leaves the default) is a
     * hint: a refusal only costs speed, and its error is cleared */
    if (e == cudaSuccess && carveout > 0 &&
        cudaFuncSetAttribute(call_stream_kernel<SLOTS, MODE>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             carveout) != cudaSuccess)
        (void)cudaGetLastError();
    if (e == cudaSuccess && ctas_per_sm)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, call_stream_kernel<SLOTS, MODE>, kTile, smem);
    return e;
}

template <int SLOTS, int MODE>
static cudaError_t launch_stream_one(const CallArgs& a, const StreamQueue& q, int ctas, int carveout,
                                     cudaStream_t stream) {
    cudaError_t e = g_launch_attributes ? stream_attr<SLOTS, MODE>(a.L, nullptr, carveout) : cudaSuccess;
    if (e != cudaSuccess) return e;
    call_stream_kernel<SLOTS, MODE><<<ctas, kTile, stream_smem_bytes(SLOTS, a.L, MODE), stream>>>(a, q);
    return cudaGetLastError();
}

template <int SLOTS>
static cudaError_t stream_dispatch(int mode, const CallArgs* a, const StreamQueue* q, int ctas, int carveout,
                                   cudaStream_t stream, int L, int* ctas_per_sm) {
    if (!a) {
        return mode == kStreamStaged     ? stream_attr<SLOTS, kStreamStaged>(L, ctas_per_sm, carveout)
               : mode == kStreamPrefetch ? stream_attr<SLOTS, kStreamPrefetch>(L, ctas_per_sm, carveout)
                                         : stream_attr<SLOTS, kStreamPlain>(L, ctas_per_sm, carveout);
    }
    return mode == kStreamStaged     ? launch_stream_one<SLOTS, kStreamStaged>(*a, *q, ctas, carveout, stream)
           : mode == kStreamPrefetch ? launch_stream_one<SLOTS, kStreamPrefetch>(*a, *q, ctas, carveout, stream)
                                     : launch_stream_one<SLOTS, kStreamPlain>(*a, *q, ctas, carveout, stream);
}

/* resident CTAs on one SM of the persistent kernel with `slots` record
 * slots (48 or 64) and read mode `mode` (0 plain, 1 L2 prefetch, 2 staged
 * in shared memory) */
int stream_ctas_per_sm(int slots, int L, int mode, int carveout) {
    int n = 0;
    const cudaError_t e = slots <= 48 ? stream_dispatch<48>(mode, nullptr, nullptr, 0, carveout, nullptr, L, &n)
                                      : stream_dispatch<64>(mode, nullptr, nullptr, 0, carveout, nullptr, L, &n);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

/* The persistent FP32 kernel over q's tiles with `ctas` CTAs; slots is 48 or
 * 64.  q.next and q.n_leftover must be zero. */
cudaError_t launch_stream(const CallArgs& a, const StreamQueue& q, int slots, int mode, int ctas, int carveout,
                          cudaStream_t stream) {
    if (q.t_end <= q.t_begin) return cudaSuccess;
    return slots <= 48 ? stream_dispatch<48>(mode, &a, &q, ctas, carveout, stream, a.L, nullptr)
                       : stream_dispatch<64>(mode, &a, &q, ctas, carveout, stream, a.L, nullptr);
}

/* set the bin kernel's shared-memory size and carveout (percent; 0 leaves the
 * default); with ctas_per_sm, its resident CTAs on one SM */
template <int SLOTS>
static cudaError_t bin_attr(int kind, int L, int carveout, int* ctas_per_sm) {
    /* the FP32 form's deep bins run one warp per site (call_deep_kernel) */
    const bool deep = kind == kKindFast && SLOTS >= kDeepSlots;
    const int smem = deep ? (int)kDeepSmem : (int)call_smem_bytes(SLOTS, L, kind == kKindFast);
    const void* fn = deep                ? reinterpret_cast<const void*>(call_deep_kernel)
                     : kind == kKindFast ? reinterpret_cast<const void*>(call_fast_kernel<SLOTS>)
                                         : reinterpret_cast<const void*>(call_tiles_kernel<SLOTS>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    /* the carveout is a hint: a refusal only costs speed, and its error is
     * cleared so that it is not taken for the launch's */
    if (carveout > 0 && cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, carveout) != cudaSuccess)
        (void)cudaGetLastError();
    if (ctas_per_sm) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, deep ? kDeepThreads : kTile, smem);
    return cudaSuccess;
}

template <int SLOTS>
static cudaError_t launch_one(const CallArgs& a, int kind, const int32_t* tiles, const BinLaunch& bl,
                              cudaStream_t stream) {
    cudaError_t e = g_launch_attributes ? bin_attr<SLOTS>(kind, a.L, bl.carveout, nullptr) : cudaSuccess;
    if (e != cudaSuccess) return e;
    const int smem = (int)call_smem_bytes(SLOTS, a.L, kind == kKindFast);
    const unsigned grid = (unsigned)(bl.d_count ? bl.grid : bl.count);
    if (grid == 0) return cudaSuccess;
    if (kind == kKindFast && SLOTS >= kDeepSlots)
        call_deep_kernel<<<grid, kDeepThreads, kDeepSmem, stream>>>(a, tiles, bl.d_count, bl.d_next);
    else if (kind == kKindFast) call_fast_kernel<SLOTS><<<grid, kTile, smem, stream>>>(a, tiles, bl.d_count, bl.d_next);
    else call_tiles_kernel<SLOTS><<<grid, kTile, smem, stream>>>(a, tiles, bl.d_count, bl.d_next);
    return cudaGetLastError();
}

/* Launch the FP64 or the fast calling kernel over the tiles of depth bin
 * `bin` (see BinLaunch). */
cudaError_t launch_bin(const CallArgs& a, int kind, int bin, const int32_t* tiles, const BinLaunch& bl,
                       cudaStream_t stream) {
    switch (bin) {
        case 0: return launch_one<32>(a, kind, tiles, bl, stream);
        case 1: return launch_one<40>(a, kind, tiles, bl, stream);
        case 2: return launch_one<48>(a, kind, tiles, bl, stream);
        case 3: return launch_one<64>(a, kind, tiles, bl, stream);
        case 4: return launch_one<96>(a, kind, tiles, bl, stream);
        case 5: return launch_one<128>(a, kind, tiles, bl, stream);
        default: return launch_one<256>(a, kind, tiles, bl, stream);
    }
}

/* resident CTAs on one SM of bin `bin` of kernel `kind` at a carveout */
int bin_ctas_per_sm(int kind, int bin, int L, int carveout) {
    int n = 0;
    cudaError_t e;
    switch (bin) {
        case 0: e = bin_attr<32>(kind, L, carveout, &n); break;
        case 1: e = bin_attr<40>(kind, L, carveout, &n); break;
        case 2: e = bin_attr<48>(kind, L, carveout, &n); break;
        case 3: e = bin_attr<64>(kind, L, carveout, &n); break;
        case 4: e = bin_attr<96>(kind, L, carveout, &n); break;
        case 5: e = bin_attr<128>(kind, L, carveout, &n); break;
        default: e = bin_attr<256>(kind, L, carveout, &n); break;
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

/* The FP64 pass over n deferred sites, or with d_n over the count the fast
 * kernels requested (read on the device) with a fixed grid of `grid` CTAs. */
cudaError_t launch_deferred(const CallArgs& a, int64_t n, cudaStream_t stream, const unsigned long long* d_n,
                            int grid) {
    if (!d_n && n <= 0) return cudaSuccess;
    /* one warp per CTA: the deferred sites are few and each is a long serial
     * computation, so they are spread over as many SMs as possible */
    const unsigned blocks = d_n ? (unsigned)grid : (unsigned)((n + 31) / 32);
    if (blocks == 0) return cudaSuccess;
    deferred_sites_kernel<<<blocks, 32, 0, stream>>>(a, n, d_n);
    return cudaGetLastError();
}

int bin_slots(int bin) { return kSlots[bin]; }

/* 32-bit words of global record scratch a launch of `count` tiles of bin
 * `bin` of kernel `kind` needs */
int64_t bin_global_words(int kind, int bin, int64_t count) {
    return kGlobalRecs(kSlots[bin], kind == kKindFast) ? count * kSlots[bin] * kTile : 0;
}

}  // namespace gsnp
