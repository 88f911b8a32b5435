/*
 * calling.cuh - argument block of the fused consensus-calling kernels.
 */
#ifndef GSNP_CALLING_CUH
#define GSNP_CALLING_CUH

#include <stdint.h>

#include "gsnp_device.cuh"

namespace gsnp {

constexpr int kNumStats = 8;

/* sites per tile (divides the window): one warp, one thread per site.  A
 * CTA's shared memory and registers are released as soon as its warp is
 * done, where with several warps per tile the shallow-site warps would hold
 * them idle until the deepest warp finished. */
constexpr int kTile = 32;
constexpr int64_t kNoRead = (int64_t)1 << 40;   /* a start beyond every read */
/* record-slot bins: 32 / 40 / 48 / 64 / 96 / 128 / 256.  At 32 sites per
 * tile a 40-slot CTA (6 KB of records and pcr bits) still fits 32 per SM. */
constexpr int kNumBins = 7;

/* calling kernels */
enum CallKind : int {
    kKindClassify = 0,
    kKindFP64 = 1,      /* FP64 likelihood, every site of the tile */
    kKindFast = 2,      /* FP32 likelihood and posterior, hard sites deferred */
    kKindDeferred = 3,  /* FP64 pass over the sites the fast kernel deferred */
    kKindStream = 4,    /* the persistent FP32 kernel over a segment's tiles */
    kKindGraph = 5,     /* a whole pass replayed as a CUDA graph */
    kKindDeep = 6,      /* FP32, one warp per site: the deep bins' tiles */
};

/* A site the fast kernel left to the FP64 pass: its pileup counts and the
 * offset of its sorted records in the deferred record pool. */
struct DeferredSite {
    int64_t site;
    uint16_t cu[4], qs[4];
    uint32_t ca[4];
    uint32_t depth, repeat;
    uint32_t rec_off;
    uint16_t num, dep_uni;
    int32_t snp_row;             /* dbSNP row of the site, -1 if none */
    uint8_t flags;               /* kCallPending and/or kCallSampled */
    uint8_t pad[3];
};
static_assert(sizeof(DeferredSite) == 64, "DeferredSite is 64 bytes");

/* per-window calling mode, decided by the host replay of the reference's
 * window loop (cpp/call_genotype.cc:422-669) */
enum WindowFlags : uint8_t {
    kWinKeepCounts = 1,   /* a later gap window shows this window's host counts */
    kWinKeepLik = 2,      /* a later window reuses this window's likelihood */
    kWinExternalLik = 4,  /* likelihood comes from another window (or zeros) */
};

/* FP32 bins of at least this many record slots are called one warp per
 * site (call_deep_kernel).  At c2 (hotspots of 300-1000x) the warp form took
 * the 256-slot bin from 26.9 to 17.9 ms, but the 96- and 128-slot bins from
 * 2.8 and 4.7 to 12.0 and 13.4 ms: below 255 records the lanes of a warp
 * sharing one scan of the tile's reads (one site each) beat a warp re-scanning
 * them per site. */
constexpr int kDeepSlots = 256;

/* tiles a warp of the persistent FP32 kernel takes per counter increment */
constexpr int kStreamChunk = 2;

/* One launch of a depth bin's kernel: `count` tiles, one CTA each; or, with
 * d_count, the count the device holds, taken by `grid` CTAs from the counter
 * d_next.  The preferred shared-memory carveout in percent (0: the default). */
struct BinLaunch {
    int count;
    const int* d_count;
    int grid;
    int carveout;
    int* d_next;
};

/* the ints of the bins' count area: the tile count of each FP64 bin, then of
 * each fast bin, then the same bins' hand-out counters (classify zeroes all) */
constexpr int kBinCountInts = 4 * kNumBins;

/* work queue of one launch of the persistent FP32 kernel (call_stream_kernel) */
struct StreamQueue {
    int64_t t_begin, t_end;       /* the segment's tiles */
    unsigned long long* next;     /* tiles handed out so far (zero before the launch) */
    int32_t* leftover;            /* tiles left to the binned kernels */
    int* n_leftover;              /* their count (zero before the launch) */
};

struct CallArgs {
    /* deposited reads, sorted by start position (file order within a start) */
    const int32_t* pos;
    const int32_t* lenhit;       /* (read_len << 16) | hit */
    const uint8_t* strand;       /* '+' or '-' */
    const uint16_t* bq;          /* [n_reads][L]: base char | quality char << 8 */
    int64_t n_reads;
    int64_t read_lo;             /* reads [read_lo, n_reads) are on the device (0 unless streamed) */
    int L;                       /* -L: read pitch and coordinate bound */
    /* reference */
    const uint8_t* ori;          /* 4-bit site code per position */
    int64_t chr_len;
    const DbSnpEntry* snp;       /* sorted by position, one row per site flagged in ori */
    int64_t n_snp;
    const int32_t* tile_snp;     /* [n_tiles]: dbSNP rows before each tile */
    const double* snp_lp;        /* [n_snp][16] log10 prior of each dbSNP site (refine mode) */
    const float* snp_lp32;       /* [n_snp][12] the same in FP32, by table column */
    /* tables */
    const double* lik64;         /* [qa_rows][L][4][10] log10 genotype terms */
    const float* lik32;          /* same, rounded to FP32: [qa_rows][L][4][8] columns 0-7 */
    const float* lik32b;         /* [qa_rows][L][4][2] columns 8-9 */
    int qa_rows;
    const uint8_t* qadj;         /* [tmax][gmax][65] adjusted quality */
    int tmax, gmax;
    const double* p_prior;       /* [8][16] */
    const double* log_prior;     /* [8][16] correctly rounded log10 of p_prior */
    const float* log_prior32;    /* [8][12] the same in FP32, by table column */
    const double* p_rank;        /* 64 x 64 x 2048 */
    /* parameters */
    int qmin;                    /* as a signed char */
    int q_max_min;
    int rank_sum, monoploid, refine;
    double het_val, het_unval, althom_val, althom_unval;
    int precision;               /* 0: FP64 sums, 1: FP32 compensated sums + FP64 fixup */
    /* windows */
    const uint8_t* win_flags;    /* per window */
    const int32_t* win_lik_src;  /* per window: window whose likelihood is used (-1: zeros) */
    /* tiles */
    int64_t n_tiles;             /* end of the tiles the tile arrays hold */
    int64_t tile_lo;             /* their first tile (0 unless streamed) */
    int64_t bin_stride;          /* entries of each depth bin's tile list */
    int64_t* tile_rng;           /* [n_tiles][2]: reads starting in [s0 - L + 1, s0 + kTile) of each tile */
    int64_t* warp_rng;           /* [n_tiles][2]: reads that can cover each tile's sites */
    int bin_limit[kNumBins];     /* deepest column each depth bin takes (at most its record slots) */
    uint32_t* deep_recs;         /* record columns of the deep bins' CTAs, [CTA][SLOTS][kTile] */
    /* the call of a site without records or counts, by site code (16 entries;
     * empty_valid[code] = 0 where it is not a fixed homozygous call) */
    const SiteCall* empty_calls;
    const uint8_t* empty_valid;
    /* sites deferred by the fast kernel */
    DeferredSite* dsites;        /* [dsite_cap] */
    uint32_t* dpool;             /* [dpool_cap] sorted records of the deferred sites */
    unsigned long long* dcount;  /* [2]: sites and record words requested (may exceed the capacities) */
    int64_t dsite_cap, dpool_cap;
    /* outputs */
    SiteCall* out;               /* [chr_len] */
    SiteCounts* counts;          /* [chr_len] or null */
    double* lik_keep;            /* [chr_len][10] or null */
    float* lik_err;              /* optional: max |FP32 - FP64| per tile (diagnostics) */
    unsigned long long* stats;   /* [kNumStats], see gsnp_get_stats */
    int* error;                  /* nonzero on a capacity overflow */
};

}  // namespace gsnp

#endif
