/*
 * column.cuh - the two passes over one site's record column that every
 * calling kernel runs before its sums: the ascending sort, and the walk that
 * gives each record its dependency-adjusted quality.  Host-compilable, so
 * that the same code is checked against plain restatements on the CPU.
 *
 * A site's records are 32-bit words (gsnp_device.cuh) kTile words apart: the
 * tile kernels keep a tile's columns as [slot][site].
 */
#ifndef GSNP_COLUMN_CUH
#define GSNP_COLUMN_CUH

#include <stddef.h>
#include <stdint.h>

#include "calling.cuh"

#if defined(__CUDA_ARCH__)
#define GSNP_LDG(p) __ldg(p)
#else
#define GSNP_LDG(p) (*(p))
#endif

namespace gsnp {

/* ------------------------------------------------------------------------ */
/* column sort (the order of kernel/batchsort.cu:245-291: std::sort of the   */
/* site's words)                                                             */
/* ------------------------------------------------------------------------ */

/* Ascending in-register bitonic network over v[0, T), T a power of two; every
 * lane runs the same instruction stream. */
template <int T>
GSNP_HDI void bitonic_sort(uint32_t* v) {
#pragma unroll
    for (int k = 2; k <= T; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < T; ++i) {
                const int l = i ^ j;
                if (l > i) {
                    const uint32_t a = v[i], b = v[l];
                    const uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
                    if ((i & k) == 0) { v[i] = lo; v[l] = hi; }
                    else { v[i] = hi; v[l] = lo; }
                }
            }
}

/* Merge the ascending v[0, cnt) (cnt <= T) into the ascending column prefix
 * recs[0, P), from the back: each v[j], largest first, moves the prefix
 * records above it up by the number of v entries still to place, then takes
 * its slot.  A write at slot k = i + (entries left) never reaches a prefix
 * record not yet moved, so no scratch is needed; v is indexed by unrolled
 * constants only, so it stays in registers. */
template <int T>
GSNP_HDI void merge_back(uint32_t* recs, int P, const uint32_t* v, int cnt) {
    int i = P - 1, k = P + cnt - 1;
#pragma unroll
    for (int j = T - 1; j >= 0; --j) {
        if (j < cnt) {
            const uint32_t x = v[j];
            while (i >= 0) {
                const uint32_t h = recs[i * kTile];
                if (h <= x) break;
                recs[k * kTile] = h;
                --k;
                --i;
            }
            recs[k * kTile] = x;
            --k;
        }
    }
}

GSNP_HDI constexpr int pow2_at_least(int n) { return n <= 1 ? 1 : 2 * pow2_at_least((n + 1) / 2); }

/* Ascending sort of one site's record column of at most SLOTS records.  The
 * first 32 records are sorted by a bitonic network in registers (padded with
 * 0xFFFFFFFF, which no record word equals), so that every lane of the warp
 * runs the same instructions whatever its depth.  Deeper columns take the rest
 * in chunks of C records: each chunk is sorted the same way and merged into
 * the sorted prefix from the back.  C is the bin's excess over 32 rounded up
 * to a power of two (8 for the 40-slot bin), at most 32. */
template <int SLOTS>
GSNP_HDI void sort_column(uint32_t* recs, int num) {
    uint32_t v[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = i < num ? recs[i * kTile] : 0xFFFFFFFFu;
    bitonic_sort<32>(v);
#pragma unroll
    for (int i = 0; i < 32; ++i)
        if (i < num) recs[i * kTile] = v[i];
    if constexpr (SLOTS > 32) {
        constexpr int C = pow2_at_least(SLOTS - 32) < 32 ? pow2_at_least(SLOTS - 32) : 32;
        for (int c0 = 32; c0 < num; c0 += C) {
            const int cnt = num - c0 < C ? num - c0 : C;
#pragma unroll
            for (int i = 0; i < C; ++i) v[i] = i < cnt ? recs[(c0 + i) * kTile] : 0xFFFFFFFFu;
            bitonic_sort<C>(v);
            merge_back<C>(recs, c0, v, cnt);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* record walk (kernel/likelihood_kernel.cu:187-255)                          */
/* ------------------------------------------------------------------------ */

/* Walk one site's sorted records: per observed-base group, tmp counts the
 * earlier occurrences of the record's (strand, cycle) and gdc the distinct
 * ones; f(i, q_adj, cycle, base) is called once per occurrence.  UNIT_OCC
 * says every record's occurrence field is 1 (the tile kernels' own pileup),
 * so that f may overwrite the low byte of record i.
 *
 * The per-site state at `seen` is a BITS-wide saturating occurrence count per
 * (strand, cycle) key, pcr_words(L, BITS) words.  Below saturation the count
 * is tmp itself; a saturated count is resolved by a scan back over the group,
 * except that with 4-bit counts and tmax <= 16 every tmp of 15 or more gives
 * q_adj = 1 whatever its exact value.  One bit per key is the least state;
 * two bits make the scan rare at moderate depth (a key seen three times);
 * four bits serve deep sites, where reads starting together repeat keys
 * often. */
GSNP_HDI int pcr_words(int L, int bits) {
    const int per = 32 / bits;
    return (2 * L + per - 1) / per;
}

template <bool UNIT_OCC, int BITS = 1, class F>
GSNP_HDI void walk_records(const CallArgs& a, const uint32_t* recs, uint32_t* seen, int stride,
                                             int num, F&& f) {
    static_assert(BITS == 1 || BITS == 2 || BITS == 4, "1, 2 or 4 bits per key");
    constexpr int kPer = 32 / BITS;
    constexpr uint32_t kMax = (1u << BITS) - 1u;
    const int L = a.L;
    const int nw = pcr_words(L, BITS);
    const bool sat_exact = BITS == 4 && a.tmax <= 16;
    int gdc = -1, last_o = -1, gstart = 0;
    for (int i = 0; i < num; ++i) {
        const uint32_t w = recs[i * stride];
        const int o = rec_base(w);
        const int coord = rec_coord(w);
        const int key = rec_strand(w) * L + coord;
        if (o != last_o) {
            for (int k = 0; k < nw; ++k) seen[k * stride] = 0u;
            gstart = i;
            gdc = -1;
            last_o = o;
        }
        const int occ = UNIT_OCC ? 1 : rec_occ(w);
        uint32_t* cw = seen + (key / kPer) * stride;
        const int sh = (key % kPer) * BITS;
        const uint32_t word = *cw;
        const uint32_t cnt = (word >> sh) & kMax;
        int tmp = (int)cnt;
        if (cnt == kMax && !sat_exact) {
            tmp = 0;
            for (int j = gstart; j < i; ++j) {
                const uint32_t wj = recs[j * stride];
                if (((wj ^ w) & 0x1ff00u) == 0) tmp += UNIT_OCC ? 1 : rec_occ(wj);
            }
        }
        if (cnt != kMax) {
            const uint32_t next = cnt + (uint32_t)occ < kMax ? cnt + (uint32_t)occ : kMax;
            *cw = (word & ~(kMax << sh)) | (next << sh);
        }
        const int q = rec_q(w);
        for (int k = 0; k < occ; ++k) {
            if (tmp == 0) gdc += 1;
            tmp++;
            const int qa = (tmp < a.tmax && gdc < a.gmax)
                               ? (int)GSNP_LDG(a.qadj + ((size_t)tmp * a.gmax + gdc) * 65 + q)
                               : 1;
            f(i, qa, coord, o);
        }
    }
}

}  // namespace gsnp

#endif
