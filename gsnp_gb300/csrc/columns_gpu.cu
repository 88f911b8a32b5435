/*
 * columns_gpu.cu - the -C compressed output encoded on the GPU.
 *
 * The five binary files of the -C output (cpp/compress.h:86-1312; the byte
 * layouts are those of columns.cpp, which is pinned to the reference's files)
 * are encoded window by window from the calls resident on the device: one CTA
 * of 1024 threads per window, each thread owning 256 consecutive rows.  A
 * window's rows are those the host writer builds (rows.h make_row: the site's
 * call with the count columns of the window the reference's host arrays held),
 * and each file's block is written in place into a per-window slice of a
 * batch buffer:
 *   .3_4_6            2-bit reference bases, N ids, genotype and best-base
 *                     differences (ids by block-wide scans, in row order);
 *   .5_7_8_9_14_16    six columns run-length encoded (run starts counted per
 *                     thread, scanned, written in order), run values and run
 *                     lengths each dictionary coded;
 *   .10               2-bit second bases, N ids;
 *   .11_12_13         the common / extra sparse lists, three dictionaries;
 *   .15_17            sparse rank-sum values and dbSNP ids.
 * Dictionaries (cuda_dictCompression's contract: the distinct values
 * ascending, each value's index packed MSB-first) of integer columns go
 * through a presence bitmap over the value range in shared memory and a scan
 * of its word counts, which gives every value its index with no sort; those
 * of doubles through a shared-memory hash set of their bit patterns (both
 * zeros one key), sorted by a bitonic network.  The bits per index come from
 * a table the host fills with the reference's own formula.
 *
 * A window whose block would not fit its slice, or whose double column has
 * more distinct values than the hash set holds, is flagged; the host encodes
 * that window itself.  The host then writes the blocks in window order.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "columns.h"
#include "columns_gpu.h"

#include <future>
#include <memory>
#include "dict.h"
#include "rows.h"

namespace gsnp {
namespace {

constexpr int kEncThreads = 1024;
constexpr int kBitmapBits = kWin + 64;                /* value span of an integer dictionary */
constexpr int kBitmapWords = kBitmapBits / 32;
/* slots of the double hash set: 128 KB of shared memory, which costs the
 * encoder no occupancy (its 1024-thread CTAs take every register of an SM);
 * with 4096 slots, the repeat / depth column of windows of varied depth (c2's
 * copy-number segments and hotspots) overflowed and went to the host */
constexpr int kHashCap = 16384;
constexpr int kHashMax = kHashCap / 2;                /* distinct doubles a column may have */
constexpr unsigned long long kEmptyKey = ~0ull;       /* a NaN pattern, never a value */

/* per-window slice of each file's batch buffer: the worst case of every file
 * but the run-length one (15, 4.25, 40 and 16 bytes per row at most), whose
 * worst case a window of a few thousand runs is far from */
constexpr size_t kCapHost[5] = {4u << 20, 12u << 20, 1300u << 10, 11u << 20, 5u << 20};

enum : int { kF346 = 0, kFRle = 1, kF10 = 2, kF111213 = 3, kF1517 = 4 };

__constant__ char c_abbv[17] = {'A', 'M', 'W', 'R', 'M', 'C', 'Y', 'S', 'W', 'Y', 'T', 'K', 'R', 'S', 'K', 'G', 'N'};
__constant__ char c_actgn[8] = {'A', 'C', 'T', 'G', 'N', 'N', 'N', 'N'};

struct EncArgs {
    int64_t w0;                      /* first window of the batch */
    const int64_t* call_len;         /* per window */
    const int32_t* host_src;         /* per window */
    const uint8_t* codes;
    const SiteCall* calls;
    const SiteCounts* counts;
    const uint8_t* bits;             /* bits per dictionary index of a dictionary of d values */
    uint8_t* out[5];                 /* [batch][cap[f]] */
    uint64_t cap[5];
    uint64_t* len;                   /* [batch][5] bytes used */
    int* fallback;                   /* [batch][5]: the file's block did not fit */
    /* scratch, [batch][2][kWin] each: one slot for the run-length file, one
     * for .11_12_13 */
    uint64_t* s_val;                 /* run values (integer or double bits), sparse values */
    uint32_t* s_aux;                 /* run starts, then run lengths */
    uint64_t* s_dict;                /* dictionary values */
    /* per row, from rows_prep_kernel: the six run-length columns' values
     * (columns 5 7 8 9 14 as [5][batch][kWin] integers, 16 as [batch][kWin]
     * double bits), and per window whether any row is not an N row */
    uint32_t* rle32;
    uint64_t* rle64;
    int* not_n;
    int64_t stride;                  /* windows of the batch buffers */
};

__device__ __forceinline__ void put8(uint8_t* p, uint8_t v) { *p = v; }
__device__ __forceinline__ void put32(uint8_t* p, uint32_t v) {
    p[0] = (uint8_t)v;
    p[1] = (uint8_t)(v >> 8);
    p[2] = (uint8_t)(v >> 16);
    p[3] = (uint8_t)(v >> 24);
}
__device__ __forceinline__ void put64(uint8_t* p, uint64_t v) {
    put32(p, (uint32_t)v);
    put32(p + 4, (uint32_t)(v >> 32));
}

/* exclusive prefix of v over the CTA's threads in order; *total the sum */
__device__ int64_t block_scan(int64_t v, int64_t* total) {
    __shared__ int64_t ws[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t s = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    const int64_t before = (warp ? ws[warp - 1] : 0) + x - v;
    *total = ws[31];
    __syncthreads();
    return before;
}

__device__ int64_t block_min(int64_t v) {
    __shared__ int64_t ws[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) ws[warp] = v;
    __syncthreads();
    int64_t r = ws[0];
    for (int i = 1; i < 32; ++i) r = min(r, ws[i]);
    __syncthreads();
    return r;
}

__device__ int64_t block_max(int64_t v) { return -block_min(-v); }

struct Enc {
    const EncArgs& e;
    int b;            /* window in the batch */
    int64_t w;        /* window */
    int n;            /* rows */
    int hs;
    bool bad;         /* CTA-uniform: the window falls back to the host */
    int slot;         /* the file's scratch slot (two files use scratch) */

    __device__ CnsRow row(int j) const { return make_row(hs, w, j, e.codes, e.calls, e.counts); }
    __device__ uint8_t* out(int f) const { return e.out[f] + (size_t)b * e.cap[f]; }
    __device__ uint64_t* sval() const { return e.s_val + ((size_t)b * 2 + slot) * kWin; }
    __device__ uint32_t* saux() const { return e.s_aux + ((size_t)b * 2 + slot) * kWin; }
    __device__ uint64_t* sdict() const { return e.s_dict + ((size_t)b * 2 + slot) * kWin; }
    /* value of run-length column k of row j */
    __device__ uint64_t rle(int k, int64_t j) const {
        return k < 5 ? (uint64_t)e.rle32[((size_t)k * e.stride + b) * kWin + j] : e.rle64[(size_t)b * kWin + j];
    }
    __device__ bool fits(int f, uint64_t bytes) {
        if (bytes > e.cap[f]) bad = true;
        return !bad;
    }
};

/* Rows of a window in order, CTA-wide: warp k walks rows
 * [k * kWarpRows, (k + 1) * kWarpRows), 32 at a time, lane l taking row
 * base + 32 i + l, so that the lanes of a load touch consecutive rows.
 * Ordered lists are built from a count pass (ballots per warp), the
 * warps' prefix (warp_prefix) and a write pass, in which each lane's slot
 * is its warp's running offset plus the ballot's lanes below it. */
constexpr int kEncWarps = kEncThreads / 32;
constexpr int kWarpRows = kWin / kEncWarps;
static_assert(kWarpRows % 32 == 0, "a warp's rows are whole iterations");
constexpr unsigned kEncFull = 0xffffffffu;

__device__ __forceinline__ int64_t warp_base() { return (int64_t)(threadIdx.x >> 5) * kWarpRows; }
__device__ __forceinline__ unsigned lanes_below() { return (1u << (threadIdx.x & 31)) - 1u; }

/* exclusive prefix, over the CTA's warps in order, of each warp's count c
 * (the same in all its lanes); *total the sum */
__device__ int64_t warp_prefix(int64_t c, int64_t* total) {
    const int64_t off = block_scan((threadIdx.x & 31) == 0 ? c : 0, total);
    return __shfl_sync(kEncFull, off, 0);
}

/* the slot of this lane's entry in an ordered list whose next free slot
 * for the warp is *off; advances *off past the ballot's entries */
__device__ __forceinline__ int64_t list_slot(bool p, int64_t* off) {
    const unsigned m = __ballot_sync(kEncFull, p);
    const int64_t k = *off + __popc(m & lanes_below());
    *off += __popc(m);
    return k;
}

/* the 2-bit code words of rows [first, first + 16), first = the half-warp's
 * first row: the code of row j at bits 2 (last - 1 - j), last = min(n,
 * first + 16), ORed over the half-warp (every lane calls it) */
__device__ __forceinline__ uint32_t half_word(uint32_t code, int64_t j, int64_t n) {
    const int64_t first = j & ~(int64_t)15;
    const int64_t last = min(n, first + 16);
    uint32_t v = j < n ? code << (2 * (last - 1 - j)) : 0u;
#pragma unroll
    for (int d = 8; d > 0; d >>= 1) v |= __shfl_xor_sync(kEncFull, v, d);
    return v;
}

/* ---- dictionaries ---------------------------------------------------- */

/* Integer dictionary of the m values vals[0, m) (non-negative, span at most
 * kBitmapBits): the bitmap and its word prefix counts in shared memory.
 * Returns the dictionary size, or -1 when the span is too wide. */
struct IntDict {
    uint32_t* bm;     /* [kBitmapWords] */
    uint32_t* pre;    /* [kBitmapWords] */
    int64_t lo;
    int d;

    template <class V>
    __device__ int build(const V* vals, int m) {
        int64_t mn = INT64_MAX, mx = INT64_MIN;
        for (int i = threadIdx.x; i < m; i += kEncThreads) {
            mn = min(mn, (int64_t)vals[i]);
            mx = max(mx, (int64_t)vals[i]);
        }
        mn = block_min(mn);
        mx = block_max(mx);
        if (m == 0) {
            d = 0;
            return 0;
        }
        if (mx - mn >= kBitmapBits) return -1;
        lo = mn;
        for (int i = threadIdx.x; i < kBitmapWords; i += kEncThreads) bm[i] = 0u;
        __syncthreads();
        for (int i = threadIdx.x; i < m; i += kEncThreads) {
            const int64_t v = (int64_t)vals[i] - lo;
            atomicOr(&bm[v >> 5], 1u << (v & 31));
        }
        __syncthreads();
        constexpr int kChunk = (kBitmapWords + kEncThreads - 1) / kEncThreads;
        const int c0 = threadIdx.x * kChunk;
        int cnt = 0;
        for (int k = c0; k < c0 + kChunk && k < kBitmapWords; ++k) cnt += __popc(bm[k]);
        int64_t total = 0;
        int run = (int)block_scan(cnt, &total);
        for (int k = c0; k < c0 + kChunk && k < kBitmapWords; ++k) {
            pre[k] = (uint32_t)run;
            run += __popc(bm[k]);
        }
        __syncthreads();
        d = (int)total;
        return d;
    }
    __device__ uint32_t index(int64_t v) const {
        const int64_t x = v - lo;
        return pre[x >> 5] + __popc(bm[x >> 5] & ((1u << (x & 31)) - 1u));
    }
    /* the values ascending as 4-byte integers at dst.  Nothing for an empty
     * dictionary: build() leaves the bitmap as it found it then (shared
     * memory not yet written by this CTA), and no entry is written past the
     * d counted. */
    __device__ void put_values(uint8_t* dst) const {
        if (d == 0) return;
        for (int k = threadIdx.x; k < kBitmapWords; k += kEncThreads) {
            uint32_t bits = bm[k];
            uint32_t r = pre[k];
            while (bits && r < (uint32_t)d) {
                const int i = __ffs(bits) - 1;
                bits &= bits - 1;
                put32(dst + 4 * (size_t)r++, (uint32_t)(lo + (int64_t)k * 32 + i));
            }
        }
    }
};

__device__ __forceinline__ unsigned long long dkey(double v) {
    if (v == 0.0) v = 0.0;   /* -0.0 and +0.0: one key */
    return (unsigned long long)__double_as_longlong(v);
}

/* Double dictionary through a hash set in shared memory; -1 when there are
 * more than kHashMax distinct values. */
struct DblDict {
    unsigned long long* tab;   /* [kHashCap]: keys, then the sorted values' bits */
    int* counter;              /* shared */
    int* negzero;              /* shared */
    int d;

    __device__ int build(const uint64_t* vals, int m) {
        for (int i = threadIdx.x; i < kHashCap; i += kEncThreads) tab[i] = kEmptyKey;
        if (threadIdx.x == 0) {
            *counter = 0;
            *negzero = 0;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < m; i += kEncThreads) {
            const double v = __longlong_as_double((long long)vals[i]);
            if (v == 0.0 && signbit(v)) atomicOr(negzero, 1);
            const unsigned long long k = dkey(v);
            uint32_t h = (uint32_t)((k * 0x9E3779B97F4A7C15ull) >> 52) & (kHashCap - 1);
            for (int probe = 0; probe < kHashCap; ++probe) {
                const unsigned long long old = atomicCAS(&tab[h], kEmptyKey, k);
                if (old == kEmptyKey) {
                    atomicAdd(counter, 1);
                    break;
                }
                if (old == k) break;
                h = (h + 1) & (kHashCap - 1);
            }
        }
        __syncthreads();
        const int cnt = *counter;
        if (cnt > kHashMax) return -1;
        /* compact the keys to the front, then sort them by value */
        __shared__ int pos;
        if (threadIdx.x == 0) pos = 0;
        __syncthreads();
        unsigned long long mine[kHashCap / kEncThreads];
        int nm = 0;
        for (int i = threadIdx.x; i < kHashCap; i += kEncThreads)
            if (tab[i] != kEmptyKey) mine[nm++] = tab[i];
        __syncthreads();
        for (int i = 0; i < nm; ++i) tab[atomicAdd(&pos, 1)] = mine[i];
        __syncthreads();
        int p2 = 1;
        while (p2 < cnt) p2 <<= 1;
        for (int i = cnt + threadIdx.x; i < p2; i += kEncThreads)
            tab[i] = (unsigned long long)__double_as_longlong(INFINITY);
        __syncthreads();
        for (int k = 2; k <= p2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = threadIdx.x; i < p2; i += kEncThreads) {
                    const int l = i ^ j;
                    if (l > i) {
                        const double a = __longlong_as_double((long long)tab[i]);
                        const double c = __longlong_as_double((long long)tab[l]);
                        const bool up = (i & k) == 0;
                        if ((a > c) == up) {
                            const unsigned long long t = tab[i];
                            tab[i] = tab[l];
                            tab[l] = t;
                        }
                    }
                }
                __syncthreads();
            }
        d = cnt;
        return d;
    }
    /* lower_bound of the double whose bits are given, in the sorted values */
    __device__ uint32_t index(uint64_t bits) const {
        const double v = __longlong_as_double((long long)dkey(__longlong_as_double((long long)bits)));
        int lo = 0, hi = d;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__longlong_as_double((long long)tab[mid]) < v) lo = mid + 1;
            else hi = mid;
        }
        return (uint32_t)lo;
    }
    /* value bits of entry i, the zero entry -0.0 when any input was -0.0 */
    __device__ uint64_t value(int i) const {
        const double v = __longlong_as_double((long long)tab[i]);
        if (v == 0.0 && *negzero) return (uint64_t)__double_as_longlong(-0.0);
        return tab[i];
    }
};

/* the m indices of vals packed MSB-first, floor(32 / bits) per word, into
 * dst (4 bytes per word) when write; returns the word count */
template <class D, class V>
__device__ uint64_t pack(const D& dict, const uint8_t* bits_tab, const V* vals, int m, uint8_t* dst, bool write) {
    if (m == 0) return 0;
    const int bits = bits_tab[dict.d];
    const int per = 32 / bits;
    const int64_t nw = (m + per - 1) / per;
    if (write)
        for (int64_t k = threadIdx.x; k < nw; k += kEncThreads) {
            const int first = (int)(k * per), last = min(m, first + per);
            uint32_t word = 0;
            for (int i = first; i < last; ++i) word = (word << bits) | dict.index(vals[i]);
            put32(dst + 4 * k, word);
        }
    return (uint64_t)nw;
}

/* ---- files ------------------------------------------------------------- */

/* 2-bit code of A C G T (compress_kernel.cu:25-58); any other letter is an
 * A here, the callers having replaced N */
__device__ __forceinline__ uint32_t code2(char c) { return c == 'C' ? 1u : c == 'G' ? 2u : c == 'T' ? 3u : 0u; }

__device__ void file_346(Enc& x, bool all_n) {
    uint8_t* o = x.out(kF346);
    const uint64_t n = (uint64_t)x.n;
    if (all_n) {
        if (threadIdx.x == 0) {
            const uint64_t param[7] = {1, 0, n, 0, 0, 0, 0};
            for (int i = 0; i < 7; ++i) put64(o + 8 * i, param[i]);
            x.e.len[x.b * 5 + kF346] = 56;
        }
        return;
    }
    auto abc = [&](int j, char* a, char* b, char* c) {
        const CnsRow r = x.row(j);
        *a = *b = *c = 'N';
        if (r.called()) {
            *a = c_actgn[r.ori & 7];
            *b = c_abbv[r.type1];
            *c = c_actgn[r.base1 & 7];
        }
    };
    const int lane = threadIdx.x & 31;
    const int64_t wb = warp_base();
    int c4 = 0, c6 = 0, cn = 0;
    for (int64_t j0 = wb; j0 < wb + kWarpRows && j0 < x.n; j0 += 32) {
        const int64_t j = j0 + lane;
        const bool in = j < x.n;
        char a = 0, b = 0, c = 0;
        if (in) abc((int)j, &a, &b, &c);
        c4 += __popc(__ballot_sync(kEncFull, in && b != a));
        c6 += __popc(__ballot_sync(kEncFull, in && c != a));
        cn += __popc(__ballot_sync(kEncFull, in && a == 'N'));
    }
    int64_t N4, N6, NN;
    int64_t o4 = warp_prefix(c4, &N4), o6 = warp_prefix(c6, &N6), on = warp_prefix(cn, &NN);
    const uint64_t nw = (n + 15) / 16;
    const uint64_t total = 56 + 5 * N4 + 5 * N6 + 4 * NN + 4 * nw;
    if (!x.fits(kF346, total)) return;
    const uint64_t b_id4 = 56, b_v4 = b_id4 + 4 * N4, b_id6 = b_v4 + N4, b_v6 = b_id6 + 4 * N6, b_idn = b_v6 + N6,
                   b_code = b_idn + 4 * NN;
    for (int64_t j0 = wb; j0 < wb + kWarpRows && j0 < x.n; j0 += 32) {
        const int64_t j = j0 + lane;
        const bool in = j < x.n;
        char a = 0, b = 0, c = 0;
        if (in) abc((int)j, &a, &b, &c);
        const bool p4 = in && b != a, p6 = in && c != a, pn = in && a == 'N';
        const int64_t k4 = list_slot(p4, &o4), k6 = list_slot(p6, &o6), kn = list_slot(pn, &on);
        if (p4) {
            put32(o + b_id4 + 4 * k4, (uint32_t)j);
            put8(o + b_v4 + k4, (uint8_t)b);
        }
        if (p6) {
            put32(o + b_id6 + 4 * k6, (uint32_t)j);
            put8(o + b_v6 + k6, (uint8_t)c);
        }
        if (pn) put32(o + b_idn + 4 * kn, (uint32_t)j);
        /* the code words of the two half-warps' 16 rows */
        const uint32_t word = half_word(code2(a), j, x.n);
        if ((lane & 15) == 0 && in) put32(o + b_code + 4 * (uint64_t)(j / 16), word);
    }
    if (threadIdx.x == 0) {
        const uint64_t param[7] = {0, (uint64_t)(5 * N4 + 5 * N6 + 4 * NN) + 4 * nw, n, nw, (uint64_t)NN,
                                   (uint64_t)N4, (uint64_t)N6};
        for (int i = 0; i < 7; ++i) put64(o + 8 * i, param[i]);
        x.e.len[x.b * 5 + kF346] = total;
    }
}

/* value of RLE column k of a row (columns 5 7 8 9 14 as integers, 16 as the
 * bits of a double) */
__device__ __forceinline__ uint64_t rle_value(const CnsRow& r, int k) {
    const bool called = r.called();
    switch (k) {
        case 0: return (uint64_t)(called ? r.q_cns : 0);
        case 1: return (uint64_t)(called ? r.avg1 : 0);
        case 2: return (uint64_t)(called ? r.cu1 : 0);
        case 3: return (uint64_t)(called ? r.ca1 : 0);
        case 4: return (uint64_t)(called ? (int)r.depth : 0);
        default: {
            const double v = called ? (r.depth == 0 ? 255.0 : (double)r.repeat / r.depth) : 255.0;
            return (uint64_t)__double_as_longlong(v);
        }
    }
}

__device__ void file_rle(Enc& x, bool all_n, IntDict& idict, DblDict& ddict) {
    uint8_t* o = x.out(kFRle);
    __shared__ uint64_t pos;
    if (threadIdx.x == 0) {
        put32(o, all_n ? 1u : 0u);
        pos = 4;
    }
    __syncthreads();
    if (all_n) {
        if (threadIdx.x == 0) x.e.len[x.b * 5 + kFRle] = 4;
        return;
    }
    uint64_t* rv = x.sval();    /* run values */
    uint32_t* rs = x.saux();    /* run starts */
    uint64_t* rl = x.sdict();   /* run lengths */
    const int lane = threadIdx.x & 31;
    const int64_t wb = warp_base();
    for (int k = 0; k < 6; ++k) {
        /* run starts: a row whose value differs from the row before (the row
         * before a lane's is the lane below's, or for lane 0 the last row of
         * the warp's previous 32, or the row before the warp's range) */
        auto starts = [&](auto&& take) {
            uint64_t carry = wb > 0 && wb < x.n ? x.rle(k, wb - 1) : 0;
            for (int64_t j0 = wb; j0 < wb + kWarpRows && j0 < x.n; j0 += 32) {
                const int64_t j = j0 + lane;
                const bool in = j < x.n;
                const uint64_t v = in ? x.rle(k, j) : 0;
                const uint64_t up = __shfl_up_sync(kEncFull, v, 1);
                const uint64_t prev = lane == 0 ? carry : up;
                carry = __shfl_sync(kEncFull, v, 31);
                take(in && (j == 0 || v != prev), j, v);
            }
        };
        int cs = 0;
        starts([&](bool p, int64_t, uint64_t) { cs += __popc(__ballot_sync(kEncFull, p)); });
        int64_t R;
        int64_t orun = warp_prefix(cs, &R);
        starts([&](bool p, int64_t j, uint64_t v) {
            const int64_t slot = list_slot(p, &orun);
            if (p) {
                rv[slot] = v;
                rs[slot] = (uint32_t)j;
            }
        });
        __syncthreads();
        for (int64_t r = threadIdx.x; r < R; r += kEncThreads)
            rl[r] = (uint64_t)((r + 1 < R ? (int64_t)rs[r + 1] : (int64_t)x.n) - (int64_t)rs[r]);
        __syncthreads();
        const int m = (int)R;
        const bool dbl = k == 5;
        const uint64_t val_bytes = dbl ? 8 : 4;
        /* sizes: the lengths' dictionary, then the values' */
        if (idict.build(rl, m) < 0) {
            x.bad = true;
            return;
        }
        const uint64_t ndl = (uint64_t)idict.d, nwl = pack(idict, x.e.bits, rl, m, (uint8_t*)nullptr, false);
        uint64_t ndv, nwv;
        if (dbl) {
            if (ddict.build(rv, m) < 0) {
                x.bad = true;
                return;
            }
            ndv = (uint64_t)ddict.d;
            nwv = pack(ddict, x.e.bits, rv, m, (uint8_t*)nullptr, false);
        } else {
            if (idict.build(rv, m) < 0) {
                x.bad = true;
                return;
            }
            ndv = (uint64_t)idict.d;
            nwv = pack(idict, x.e.bits, rv, m, (uint8_t*)nullptr, false);
        }
        const uint64_t p0 = pos;
        const uint64_t b_cval = p0 + 48, b_clen = b_cval + 4 * nwv, b_dval = b_clen + 4 * nwl,
                       b_dlen = b_dval + val_bytes * ndv, end = b_dlen + 4 * ndl;
        if (!x.fits(kFRle, end)) return;
        /* the values' words and dictionary (the dictionary built last) */
        if (dbl) {
            pack(ddict, x.e.bits, rv, m, o + b_cval, true);
            for (int i = threadIdx.x; i < ddict.d; i += kEncThreads) put64(o + b_dval + 8 * (size_t)i, ddict.value(i));
        } else {
            pack(idict, x.e.bits, rv, m, o + b_cval, true);
            idict.put_values(o + b_dval);
        }
        __syncthreads();
        /* the lengths' dictionary again, for its words and values */
        idict.build(rl, m);
        pack(idict, x.e.bits, rl, m, o + b_clen, true);
        idict.put_values(o + b_dlen);
        if (threadIdx.x == 0) {
            const uint64_t param[6] = {(uint64_t)R, nwv, nwl, ndv, ndl, 4 * nwv + 4 * nwl + val_bytes * ndv + 4 * ndl};
            for (int i = 0; i < 6; ++i) put64(o + p0 + 8 * i, param[i]);
            pos = end;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) x.e.len[x.b * 5 + kFRle] = pos;
}

__device__ void file_10(Enc& x, bool all_n) {
    uint8_t* o = x.out(kF10);
    if (threadIdx.x == 0) put32(o, all_n ? 1u : 0u);
    if (all_n) {
        if (threadIdx.x == 0) x.e.len[x.b * 5 + kF10] = 4;
        return;
    }
    auto letter = [&](int j) {
        const CnsRow r = x.row(j);
        return (r.called() && r.base2 < 4) ? c_actgn[r.base2] : 'N';
    };
    const int lane = threadIdx.x & 31;
    const int64_t wb = warp_base();
    int cn = 0;
    for (int64_t j0 = wb; j0 < wb + kWarpRows && j0 < x.n; j0 += 32) {
        const int64_t j = j0 + lane;
        cn += __popc(__ballot_sync(kEncFull, j < x.n && letter((int)j) == 'N'));
    }
    int64_t NN;
    int64_t on = warp_prefix(cn, &NN);
    const uint64_t n = (uint64_t)x.n, nw = (n + 15) / 16;
    const uint64_t b_code = 4 + 24, b_nid = b_code + 4 * nw, total = b_nid + 4 * NN;
    if (!x.fits(kF10, total)) return;
    for (int64_t j0 = wb; j0 < wb + kWarpRows && j0 < x.n; j0 += 32) {
        const int64_t j = j0 + lane;
        const bool in = j < x.n;
        const char c = in ? letter((int)j) : 'A';
        const bool pn = in && c == 'N';
        const int64_t kn = list_slot(pn, &on);
        if (pn) put32(o + b_nid + 4 * kn, (uint32_t)j);
        const uint32_t word = half_word(code2(c == 'N' ? 'A' : c), j, x.n);
        if ((lane & 15) == 0 && in) put32(o + b_code + 4 * (uint64_t)(j / 16), word);
    }
    if (threadIdx.x == 0) {
        put64(o + 4, (uint64_t)NN);
        put64(o + 12, nw);
        put64(o + 20, n);
        x.e.len[x.b * 5 + kF10] = total;
    }
}

__device__ void file_111213(Enc& x, bool all_n, IntDict& idict) {
    uint8_t* o = x.out(kF111213);
    if (threadIdx.x == 0) put32(o, all_n ? 1u : 0u);
    if (all_n) {
        if (threadIdx.x == 0) x.e.len[x.b * 5 + kF111213] = 4;
        return;
    }
    /* 0: common, 1: extra column 12, 2: extra column 13, -1: none */
    auto cls = [&](int j, int* v11, int* v12, int* v13) {
        const CnsRow r = x.row(j);
        *v11 = *v12 = *v13 = 0;
        if (r.called() && r.base2 < 4) {
            *v11 = r.avg2;
            *v12 = r.cu2;
            *v13 = r.ca2;
        }
        if (*v11 != 0) return 0;
        if (*v11 != *v12) return 1;
        if (*v11 != *v13) return 2;
        return -1;
    };
    const int lane = threadIdx.x & 31;
    const int64_t wb = warp_base();
    int cc = 0, c12 = 0, c13 = 0;
    for (int64_t j0 = wb; j0 < wb + kWarpRows && j0 < x.n; j0 += 32) {
        const int64_t j = j0 + lane;
        int a, b, c;
        const int k = j < x.n ? cls((int)j, &a, &b, &c) : -1;
        cc += __popc(__ballot_sync(kEncFull, k == 0));
        c12 += __popc(__ballot_sync(kEncFull, k == 1));
        c13 += __popc(__ballot_sync(kEncFull, k == 2));
    }
    int64_t NC, N12, N13;
    int64_t oc = warp_prefix(cc, &NC), o12 = warp_prefix(c12, &N12), o13 = warp_prefix(c13, &N13);
    const uint64_t b_e12id = 4 + 32, b_e12 = b_e12id + 4 * N12, b_e13id = b_e12 + 4 * N12, b_e13 = b_e13id + 4 * N13,
                   b_cid = b_e13 + 4 * N13, b_dicts = b_cid + 4 * NC;
    if (!x.fits(kF111213, b_dicts)) return;
    /* the common entries' three values */
    uint64_t* v11 = x.sval();
    uint32_t* v12 = x.saux();
    uint64_t* v13 = x.sdict();
    for (int64_t j0 = wb; j0 < wb + kWarpRows && j0 < x.n; j0 += 32) {
        const int64_t j = j0 + lane;
        int a = 0, b = 0, c = 0;
        const int k = j < x.n ? cls((int)j, &a, &b, &c) : -1;
        const int64_t sc = list_slot(k == 0, &oc), s12 = list_slot(k == 1, &o12), s13 = list_slot(k == 2, &o13);
        if (k == 0) {
            put32(o + b_cid + 4 * sc, (uint32_t)j);
            v11[sc] = (uint64_t)a;
            v12[sc] = (uint32_t)b;
            v13[sc] = (uint64_t)c;
        } else if (k == 1) {
            put32(o + b_e12id + 4 * s12, (uint32_t)j);
            put32(o + b_e12 + 4 * s12, (uint32_t)b);
        } else if (k == 2) {
            put32(o + b_e13id + 4 * s13, (uint32_t)j);
            put32(o + b_e13 + 4 * s13, (uint32_t)c);
        }
    }
    __syncthreads();
    uint64_t p = b_dicts;
    for (int col = 0; col < 3; ++col) {
        const int m = (int)NC;
        int r = col == 0 ? idict.build(v11, m) : col == 1 ? idict.build(v12, m) : idict.build(v13, m);
        if (r < 0) {
            x.bad = true;
            return;
        }
        const uint64_t nd = (uint64_t)idict.d;
        const uint64_t nw = col == 0   ? pack(idict, x.e.bits, v11, m, (uint8_t*)nullptr, false)
                            : col == 1 ? pack(idict, x.e.bits, v12, m, (uint8_t*)nullptr, false)
                                       : pack(idict, x.e.bits, v13, m, (uint8_t*)nullptr, false);
        if (!x.fits(kF111213, p + 16 + 4 * nw + 4 * nd)) return;
        if (col == 0) pack(idict, x.e.bits, v11, m, o + p + 16, true);
        else if (col == 1) pack(idict, x.e.bits, v12, m, o + p + 16, true);
        else pack(idict, x.e.bits, v13, m, o + p + 16, true);
        idict.put_values(o + p + 16 + 4 * nw);
        if (threadIdx.x == 0) {
            put64(o + p, nw);
            put64(o + p + 8, nd);
        }
        p += 16 + 4 * nw + 4 * nd;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        put64(o + 4, (uint64_t)x.n);
        put64(o + 12, (uint64_t)NC);
        put64(o + 20, (uint64_t)N12);
        put64(o + 28, (uint64_t)N13);
        x.e.len[x.b * 5 + kF111213] = p;
    }
}

__device__ void file_1517(Enc& x, bool all_n) {
    uint8_t* o = x.out(kF1517);
    if (threadIdx.x == 0) put32(o, all_n ? 1u : 0u);
    if (all_n) {
        if (threadIdx.x == 0) x.e.len[x.b * 5 + kF1517] = 4;
        return;
    }
    const int lane = threadIdx.x & 31;
    const int64_t wb = warp_base();
    int cr = 0, cs = 0;
    for (int64_t j0 = wb; j0 < wb + kWarpRows && j0 < x.n; j0 += 32) {
        const int64_t j = j0 + lane;
        bool pr = false, ps = false;
        if (j < x.n) {
            const CnsRow r = x.row((int)j);
            pr = r.called() && r.rank_sum != 1.0;
            ps = r.called() && (r.ori & 8) != 0;
        }
        cr += __popc(__ballot_sync(kEncFull, pr));
        cs += __popc(__ballot_sync(kEncFull, ps));
    }
    int64_t NR, NS;
    int64_t orr = warp_prefix(cr, &NR), os = warp_prefix(cs, &NS);
    const uint64_t b_id = 8, b_val = b_id + 4 * NR, b_cnt2 = b_val + 8 * NR, b_snp = b_cnt2 + 4, total = b_snp + 4 * NS;
    if (!x.fits(kF1517, total)) return;
    for (int64_t j0 = wb; j0 < wb + kWarpRows && j0 < x.n; j0 += 32) {
        const int64_t j = j0 + lane;
        bool pr = false, ps = false;
        double rs = 1.0;
        if (j < x.n) {
            const CnsRow r = x.row((int)j);
            pr = r.called() && r.rank_sum != 1.0;
            ps = r.called() && (r.ori & 8) != 0;
            rs = r.rank_sum;
        }
        const int64_t kr = list_slot(pr, &orr), ks = list_slot(ps, &os);
        if (pr) {
            put32(o + b_id + 4 * kr, (uint32_t)j);
            put64(o + b_val + 8 * kr, (uint64_t)__double_as_longlong(rs));
        }
        if (ps) put32(o + b_snp + 4 * ks, (uint32_t)j);
    }
    if (threadIdx.x == 0) {
        put32(o + 4, (uint32_t)NR);
        put32(o + b_cnt2, (uint32_t)NS);
        x.e.len[x.b * 5 + kF1517] = total;
    }
}

/* The rows of a batch of windows in one pass over the whole GPU, for the
 * encoder's CTAs (one per window and file), which would otherwise each read
 * every row's call again on every pass: the run-length columns' values, and
 * e.not_n[b] = 1 when window b has a row that is not an N row (zeroed
 * before).  Grid: (rows / 256, windows). */
__global__ void __launch_bounds__(256) rows_prep_kernel(EncArgs e) {
    const int b = (int)blockIdx.y;
    const int64_t w = e.w0 + b;
    const int64_t j = (int64_t)blockIdx.x * 256 + threadIdx.x;
    const int64_t n = e.call_len[w];
    bool not_n = false;
    if (j < n) {
        const CnsRow r = make_row(e.host_src[w], w, j, e.codes, e.calls, e.counts);
        not_n = !r.nflag;
#pragma unroll
        for (int k = 0; k < 5; ++k) e.rle32[((size_t)k * e.stride + b) * kWin + j] = (uint32_t)rle_value(r, k);
        e.rle64[(size_t)b * kWin + j] = rle_value(r, 5);
    }
    if (__syncthreads_or(not_n) && threadIdx.x == 0) e.not_n[b] = 1;
}

__global__ void __launch_bounds__(kEncThreads) encode_windows_kernel(EncArgs e) {
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ int hash_counter, hash_negzero;
    IntDict idict;
    idict.bm = reinterpret_cast<uint32_t*>(smem);
    idict.pre = idict.bm + kBitmapWords;
    idict.d = 0;
    idict.lo = 0;
    DblDict ddict;
    ddict.tab = reinterpret_cast<unsigned long long*>(smem + 2 * kBitmapWords * 4);
    ddict.counter = &hash_counter;
    ddict.negzero = &hash_negzero;
    ddict.d = 0;

    /* one CTA per (window, file): the five files of a window are
     * independent, so a small batch of windows still fills the GPU */
    const int f = (int)blockIdx.y;
    Enc x{e, (int)blockIdx.x, e.w0 + blockIdx.x, 0, 0, false, f == kF111213 ? 1 : 0};
    x.n = (int)e.call_len[x.w];
    x.hs = e.host_src[x.w];
    const bool all_n = e.not_n[x.b] == 0;
    switch (f) {
        case kF346: file_346(x, all_n); break;
        case kFRle: file_rle(x, all_n, idict, ddict); break;
        case kF10: file_10(x, all_n); break;
        case kF111213: file_111213(x, all_n, idict); break;
        default: file_1517(x, all_n); break;
    }
    if (threadIdx.x == 0) e.fallback[x.b * 5 + f] = x.bad ? 1 : 0;
}

constexpr size_t kEncSmem = 2 * kBitmapWords * 4 + kHashCap * 8;
static_assert(kEncSmem <= 220 * 1024, "the encoder's shared memory fits one CTA per SM");

#define CKE(x, what)                                                      \
    do {                                                                  \
        cudaError_t e_ = (x);                                             \
        if (e_ != cudaSuccess) {                                          \
            *err = std::string(what) + ": " + cudaGetErrorString(e_);     \
            return 1;                                                     \
        }                                                                 \
    } while (0)

}  // namespace

ColumnsGpuWriter::~ColumnsGpuWriter() {
    if (fb_[0] || f12_) {
        std::string e;
        close(&e);
    }
    release();
    for (int set = 0; set < 2; ++set)
        for (int f = 0; f < 5; ++f)
            if (hbuf_[set][f]) cudaFreeHost(hbuf_[set][f]);
}

void ColumnsGpuWriter::release() {
    for (uint8_t*& p : d_out_) {
        cudaFree(p);
        p = nullptr;
    }
    cudaFree(d_bits_);
    cudaFree(d_len_tab_);
    cudaFree(d_len_);
    cudaFree(d_fb_);
    cudaFree(d_sval_);
    cudaFree(d_sdict_);
    cudaFree(d_saux_);
    cudaFree(d_rle32_);
    cudaFree(d_rle64_);
    cudaFree(d_not_n_);
    d_rle32_ = nullptr;
    d_rle64_ = nullptr;
    d_not_n_ = nullptr;
    d_bits_ = nullptr;
    d_len_tab_ = nullptr;
    d_len_ = nullptr;
    d_fb_ = nullptr;
    d_sval_ = d_sdict_ = nullptr;
    d_saux_ = nullptr;
    batch_cap_ = 0;
    len_tab_windows_ = 0;
}

int ColumnsGpuWriter::open(const WindowPlan& plan, const char* chr_name, const std::string& base, int64_t batch,
                           std::string* err) {
    if (fb_[0] || f12_) close(err);
    plan_ = &plan;
    next_window_ = 0;
    const char* ext[5] = {".3_4_6", ".5_7_8_9_14_16", ".10", ".11_12_13", ".15_17"};
    for (int i = 0; i < 5; ++i) {
        fb_[i] = fopen((base + ext[i]).c_str(), "wb");
        if (!fb_[i]) {
            *err = "cannot create " + base + ext[i];
            close(err);
            *err = "cannot create " + base + ext[i];
            return 1;
        }
    }
    f12_ = fopen((base + ".1_2").c_str(), "w");
    if (!f12_) {
        close(err);
        *err = "cannot create " + base + ".1_2";
        return 1;
    }
    fprintf(f12_, "%lu\n", (unsigned long)plan.n_windows);
    for (int64_t w = 0; w < plan.n_windows; ++w)
        fprintf(f12_, "%s\t%lu\t%lu\n", chr_name, (unsigned long)(w * (int64_t)kWin + 1),
                (unsigned long)plan.call_len[w]);
    /* device buffers of one batch of windows, kept from one use to the next */
    batch = std::max<int64_t>(1, batch);
    cudaError_t ce = cudaSuccess;
    if (batch > batch_cap_) {
        release();
        for (int f = 0; f < 5 && ce == cudaSuccess; ++f) ce = cudaMalloc((void**)&d_out_[f], kCapHost[f] * (size_t)batch);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&d_bits_, kWin + 2);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&d_len_, sizeof(uint64_t) * 5 * batch);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&d_fb_, sizeof(int) * 5 * batch);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&d_sval_, sizeof(uint64_t) * kWin * 2 * batch);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&d_sdict_, sizeof(uint64_t) * kWin * 2 * batch);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&d_saux_, sizeof(uint32_t) * kWin * 2 * batch);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&d_rle32_, sizeof(uint32_t) * kWin * 5 * batch);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&d_rle64_, sizeof(uint64_t) * kWin * batch);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&d_not_n_, sizeof(int) * batch);
        if (ce == cudaSuccess) {
            std::vector<uint8_t> bits(kWin + 2);
            bits[0] = 1;
            for (size_t d = 1; d < bits.size(); ++d) bits[d] = (uint8_t)dict_bits((unsigned long)d);
            ce = cudaMemcpy(d_bits_, bits.data(), bits.size(), cudaMemcpyHostToDevice);
        }
        if (ce == cudaSuccess)
            ce = cudaFuncSetAttribute(encode_windows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kEncSmem);
        if (ce != cudaSuccess) {
            release();
            close(err);
            *err = std::string("-C encoder set-up: ") + cudaGetErrorString(ce);
            return 1;
        }
        batch_cap_ = batch;
    }
    if (plan.n_windows > len_tab_windows_) {
        cudaFree(d_len_tab_);
        d_len_tab_ = nullptr;
        ce = cudaMalloc((void**)&d_len_tab_, sizeof(int64_t) * std::max<int64_t>(1, plan.n_windows));
        if (ce != cudaSuccess) {
            len_tab_windows_ = 0;
            close(err);
            *err = std::string("-C encoder set-up: ") + cudaGetErrorString(ce);
            return 1;
        }
        len_tab_windows_ = plan.n_windows;
    }
    if (plan.n_windows > 0) {
        ce = cudaMemcpy(d_len_tab_, plan.call_len.data(), sizeof(int64_t) * plan.n_windows, cudaMemcpyHostToDevice);
        if (ce != cudaSuccess) {
            close(err);
            *err = std::string("-C encoder set-up: ") + cudaGetErrorString(ce);
            return 1;
        }
    }
    return 0;
}

int ColumnsGpuWriter::write(int64_t w0, int64_t w1, const uint8_t* d_codes, const SiteCall* d_calls,
                            const SiteCounts* d_counts, const int32_t* d_host_src, const int32_t* h_host_src,
                            const uint8_t* h_codes, cudaStream_t stream, ColumnsGpuStats* st, std::string* err) {
    if (!fb_[0] || !plan_ || w0 != next_window_ || w1 < w0 || w1 > plan_->n_windows) {
        *err = "-C windows out of order";
        return 1;
    }
    const WindowPlan& plan = *plan_;
    int rc = 0;
    cudaError_t ce = cudaSuccess;
    std::vector<uint64_t> h_len((size_t)(5 * batch_cap_));
    std::vector<int> h_fb5((size_t)(5 * batch_cap_)), h_fb((size_t)batch_cap_);
    for (int64_t b0 = w0; b0 < w1 && rc == 0; b0 += batch_cap_) {
        const int64_t nb = std::min(batch_cap_, w1 - b0);
        EncArgs e;
        e.w0 = b0;
        e.call_len = d_len_tab_;
        e.host_src = d_host_src;
        e.codes = d_codes;
        e.calls = d_calls;
        e.counts = d_counts;
        e.bits = d_bits_;
        for (int f = 0; f < 5; ++f) {
            e.out[f] = d_out_[f];
            e.cap[f] = kCapHost[f];
        }
        e.len = d_len_;
        e.fallback = d_fb_;
        e.s_val = d_sval_;
        e.s_aux = d_saux_;
        e.s_dict = d_sdict_;
        e.rle32 = d_rle32_;
        e.rle64 = d_rle64_;
        e.not_n = d_not_n_;
        e.stride = batch_cap_;
        ce = cudaMemsetAsync(d_not_n_, 0, sizeof(int) * nb, stream);
        if (ce == cudaSuccess) {
            rows_prep_kernel<<<dim3((unsigned)(kWin / 256), (unsigned)nb), 256, 0, stream>>>(e);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess) {
            encode_windows_kernel<<<dim3((unsigned)nb, 5), kEncThreads, kEncSmem, stream>>>(e);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(h_len.data(), d_len_, sizeof(uint64_t) * 5 * nb, cudaMemcpyDeviceToHost, stream);
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(h_fb5.data(), d_fb_, sizeof(int) * 5 * nb, cudaMemcpyDeviceToHost, stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream);
        /* a window goes to the host encoder when any of its files did not fit */
        for (int64_t b = 0; b < nb; ++b) {
            int any = 0;
            for (int f = 0; f < 5; ++f) any |= h_fb5[(size_t)(5 * b + f)];
            h_fb[(size_t)b] = any;
        }
        if (ce != cudaSuccess) {
            *err = std::string("-C encoder: ") + cudaGetErrorString(ce);
            rc = 1;
            break;
        }
        /* the batch's blocks, window by window, into one pinned host buffer
         * per file, of the set the batch before last used (its writes are
         * waited for first) */
        const int set = set_;
        set_ ^= 1;
        if (!wait_set(set)) {
            *err = "write failed";
            rc = 1;
            break;
        }
        size_t tot[5] = {};
        for (int64_t b = 0; b < nb; ++b)
            if (!h_fb[(size_t)b])
                for (int f = 0; f < 5; ++f) tot[f] += h_len[(size_t)(5 * b + f)];
        for (int f = 0; f < 5 && ce == cudaSuccess; ++f)
            if (hcap_[set][f] < tot[f]) {
                /* pinned, so that the blocks come down at the link's speed */
                if (hbuf_[set][f]) cudaFreeHost(hbuf_[set][f]);
                hbuf_[set][f] = nullptr;
                hcap_[set][f] = 0;
                ce = cudaMallocHost((void**)&hbuf_[set][f], tot[f] + tot[f] / 4);
                if (ce == cudaSuccess) hcap_[set][f] = tot[f] + tot[f] / 4;
            }
        size_t off[5] = {};
        for (int64_t b = 0; b < nb && ce == cudaSuccess; ++b) {
            if (h_fb[(size_t)b]) continue;
            for (int f = 0; f < 5 && ce == cudaSuccess; ++f) {
                const size_t bytes = (size_t)h_len[(size_t)(5 * b + f)];
                if (bytes)
                    ce = cudaMemcpyAsync(hbuf_[set][f] + off[f], d_out_[f] + (size_t)b * kCapHost[f], bytes,
                                         cudaMemcpyDeviceToHost, stream);
                off[f] += bytes;
            }
        }
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream);
        if (ce != cudaSuccess) {
            *err = std::string("-C encoder download: ") + cudaGetErrorString(ce);
            rc = 1;
            break;
        }
        /* the windows the encoder left to the host, encoded on host threads
         * (a window each) while the pieces are assembled */
        struct HostWindow {
            std::string parts[5];
            std::string err;
            bool ok = false;
        };
        const int dev = [] {
            int d = 0;
            cudaGetDevice(&d);
            return d;
        }();
        std::vector<std::future<std::shared_ptr<HostWindow>>> host_win((size_t)nb);
        for (int64_t b = 0; b < nb; ++b) {
            if (!h_fb[(size_t)b]) continue;
            if (st) ++st->host_windows;
            const int64_t w = b0 + b;
            host_win[(size_t)b] = std::async(std::launch::async, [=, &plan]() {
                auto hw = std::make_shared<HostWindow>();
                cudaSetDevice(dev);
                const int64_t len = plan.call_len[(size_t)w];
                std::vector<SiteCall> calls((size_t)len);
                std::vector<SiteCounts> counts;
                cudaError_t e2 =
                    cudaMemcpy(calls.data(), d_calls + w * (int64_t)kWin, sizeof(SiteCall) * len, cudaMemcpyDeviceToHost);
                const int32_t src = h_host_src[w];
                if (e2 == cudaSuccess && src >= 0 && src != w && d_counts) {
                    counts.resize((size_t)len);
                    e2 = cudaMemcpy(counts.data(), d_counts + (int64_t)src * kWin, sizeof(SiteCounts) * len,
                                    cudaMemcpyDeviceToHost);
                }
                if (e2 != cudaSuccess) {
                    hw->err = std::string("-C encoder download: ") + cudaGetErrorString(e2);
                    return hw;
                }
                HostDictCodec codec;
                hw->ok = encode_window_host(len, src >= 0 && src != w ? 1 : (src == w ? 0 : -1),
                                            h_codes + w * (int64_t)kWin, calls.data(),
                                            counts.empty() ? nullptr : counts.data(), codec, hw->parts, &hw->err);
                return hw;
            });
        }
        /* each file's pieces in window order: the encoder's blocks, and the
         * host-encoded windows in their places */
        std::vector<Piece> pieces[5];
        size_t wo[5] = {};
        for (int64_t b = 0; b < nb; ++b) {
            if (!h_fb[(size_t)b]) {
                for (int f = 0; f < 5; ++f) {
                    const size_t bytes = (size_t)h_len[(size_t)(5 * b + f)];
                    if (bytes) pieces[f].push_back(Piece{hbuf_[set][f] + wo[f], bytes, nullptr});
                    wo[f] += bytes;
                }
                continue;
            }
            std::shared_ptr<HostWindow> hw = host_win[(size_t)b].get();
            if (!hw->ok) {
                if (rc == 0) *err = hw->err;
                rc = 1;
                continue;
            }
            for (int f = 0; f < 5; ++f)
                if (!hw->parts[f].empty()) {
                    auto own = std::make_shared<std::string>(std::move(hw->parts[f]));
                    pieces[f].push_back(Piece{own->data(), own->size(), own});
                }
        }
        /* the files written on their own threads, each after its previous
         * batch, while the caller goes on */
        for (int f = 0; f < 5 && rc == 0; ++f) {
            std::shared_future<bool> prev = last_[f];
            FILE* file = fb_[f];
            std::vector<Piece> ps = std::move(pieces[f]);
            last_[f] = std::async(std::launch::async, [prev, file, ps]() {
                           bool ok = prev.valid() ? prev.get() : true;
                           for (const Piece& x : ps)
                               if (fwrite(x.p, 1, x.n, file) != x.n) ok = false;
                           return ok;
                       }).share();
            pend_[set][f] = last_[f];
        }
        if (rc && err->empty()) *err = "write failed";
        if (st) st->windows += nb;
    }
    next_window_ = w1;
    return rc;
}

size_t ColumnsGpuWriter::device_bytes() const {
    size_t n = 0;
    for (int f = 0; f < 5; ++f) n += kCapHost[f] * (size_t)batch_cap_;
    return n + (size_t)batch_cap_ * (kWin * (40 + 28) + 64) + (kWin + 2) + (size_t)len_tab_windows_ * 8;
}

bool ColumnsGpuWriter::wait_set(int set) {
    bool ok = true;
    for (int f = 0; f < 5; ++f)
        if (pend_[set][f].valid()) {
            ok = pend_[set][f].get() && ok;
            pend_[set][f] = std::shared_future<bool>();
        }
    return ok;
}

int ColumnsGpuWriter::close(std::string* err) {
    int rc = 0;
    /* every write queued, in file order */
    bool ok = true;
    for (int f = 0; f < 5; ++f)
        if (last_[f].valid()) {
            ok = last_[f].get() && ok;
            last_[f] = std::shared_future<bool>();
        }
    ok = wait_set(0) && ok;
    ok = wait_set(1) && ok;
    if (!ok) {
        *err = "write failed";
        rc = 1;
    }
    for (FILE*& f : fb_)
        if (f) {
            if (fclose(f) != 0 && rc == 0) {
                *err = "write failed";
                rc = 1;
            }
            f = nullptr;
        }
    if (f12_) {
        if (fclose(f12_) != 0 && rc == 0) {
            *err = "write failed";
            rc = 1;
        }
        f12_ = nullptr;
    }
    if (rc == 0 && plan_ && next_window_ != plan_->n_windows) {
        *err = "-C files closed before their last window";
        rc = 1;
    }
    plan_ = nullptr;
    return rc;
}

}  // namespace gsnp
