/*
 * gsnp_device.cuh - device-side layouts and helpers shared by the calling kernels.
 *
 * Record word of one unique base at one site (kernel/likelihood_kernel.cu:24-42,
 * kernel/update_kernel.cu:302-310):
 *     bits 24:23  observed base, ACTG = 0..3
 *     bits 22:17  64 - q, q = quality char - q_min
 *     bits 16:9   read cycle (coordinate on '+', read_len-1-coordinate on '-')
 *     bit  8      strand (1 = '-')
 *     bits 7:0    occurrence count (always 1)
 * The word is built with the reference's 32-bit arithmetic, so out-of-range
 * qualities spill into neighbouring fields exactly as they do there.  Ascending
 * word order is the per-site order in which the likelihood is summed.
 */
#ifndef GSNP_DEVICE_CUH
#define GSNP_DEVICE_CUH

#include <stdint.h>

#include "gsnp_crmath.h"

#if defined(__CUDACC__)
#define GSNP_HDI __host__ __device__ __forceinline__
#else
#define GSNP_HDI inline
#endif

namespace gsnp {

constexpr int kWin = 262144;            /* window size, cpp/common.h:16 */
constexpr int kMaxRecords = 255;        /* dep_uni cap, kernel/update_kernel.cu:288 */
constexpr int kMaxQ = 64;               /* MAX_QSCORE */

GSNP_HDI uint32_t make_record(int base_char, int q, uint32_t coord_val,
                                                         uint32_t strand_val) {
    const uint32_t prefix = ((uint32_t)((base_char & 0x6) >> 1) << 15) | ((uint32_t)(kMaxQ - q) << 9) |
                            (coord_val << 1) | strand_val;
    return (prefix << 8) | 1u;
}

GSNP_HDI int rec_base(uint32_t w) { return (int)((w & 0x01800000u) >> 23); }
GSNP_HDI int rec_q(uint32_t w) { return kMaxQ - (int)((w & 0x007e0000u) >> 17); }
GSNP_HDI int rec_coord(uint32_t w) { return (int)((w & 0x0001fe00u) >> 9); }
GSNP_HDI int rec_strand(uint32_t w) { return (int)((w & 0x00000100u) >> 8); }
GSNP_HDI int rec_occ(uint32_t w) { return (int)(w & 0xffu); }

/* genotype code (a1 << 2 | a2) of table column t, a1 <= a2 in ACTG order */
GSNP_HDI int genotype_of(int t) {
    const int g[10] = {0, 1, 2, 3, 5, 6, 7, 10, 11, 15};
    return g[t];
}

/* Per-site output of the caller: everything the cns row and the -C columns
 * need (32 bytes). */
struct SiteCall {
    uint8_t type1;       /* genotype code 0..15 */
    uint8_t base1;       /* 0..7 (4..7: the reference base was N) */
    uint8_t base2;
    uint8_t q_cns;       /* 0..99 */
    uint8_t avg_q1;      /* q_sum / count_uni of base1 (0 when q_sum is 0) */
    uint8_t avg_q2;
    uint8_t flags;       /* bit0: FP64 fixup taken, bit1: rank-sum normal path */
    uint8_t pad;
    uint16_t cu1, ca1;   /* count_uni / count_all of base1 */
    uint16_t cu2, ca2;
    uint32_t depth;
    uint32_t repeat_time;
    double rank_sum;
};
static_assert(sizeof(SiteCall) == 32, "SiteCall is 32 bytes");

/* Full pileup counts of one site, kept for windows whose counts a later gap
 * window shows (the reference's stale host arrays). */
struct SiteCounts {
    uint16_t cu[4];
    uint16_t qs[4];
    uint32_t ca[4];
    uint32_t depth;
    uint32_t repeat_time;
};
static_assert(sizeof(SiteCounts) == 40, "SiteCounts is 40 bytes");

struct DbSnpEntry {
    uint32_t pos;        /* 0-based */
    uint8_t validated, hapmap, indel, pad;
    double freq[4];      /* ACTG */
};

}  // namespace gsnp

#endif
