/*
 * engine.cu - the C ABI of include/gsnp_gb300.h: context, tables, resident
 * chromosome state, calibration and the whole-chromosome calling pass.
 *
 * Device memory layout of one chromosome (sized for HBM, all resident):
 *   site codes      1 B/site      reference base, N and dbSNP bits
 *   reads           2*L + 9 B/read after the gather: packed base|quality
 *                   pairs [n][L] (uint16), start, len<<16|hit, strand
 *   SiteCall        32 B/site     the caller's output
 *   side buffers    40 B/site of SiteCounts and 80 B/site of likelihoods, only
 *                   for windows that a later window refers to
 * The raw alignment arrays are uploaded once per call and gathered on the
 * device into the deposited, packed layout the calling kernel reads.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <atomic>
#include <thread>
#include <future>
#include <memory>
#include <vector>

#include "calling.cuh"
#include "columns.h"
#include "columns_gpu.h"
#include "emit.h"
#include "gsnp_gb300.h"
#include "plan.h"
#include "tables.h"

namespace gsnp {

cudaError_t launch_classify(const CallArgs& a, int pass, int64_t t_begin, int64_t t_end, int* d_bin_count,
                            int32_t* d_bin_tiles, cudaStream_t stream, const int32_t* list = nullptr,
                            const int* d_count = nullptr, int grid = 0);
cudaError_t launch_stream(const CallArgs& a, const StreamQueue& q, int slots, int mode, int ctas, int carveout,
                          cudaStream_t stream);
int stream_ctas_per_sm(int slots, int L, int mode, int carveout);
cudaError_t launch_bin(const CallArgs& a, int kind, int bin, const int32_t* tiles, const BinLaunch& bl,
                       cudaStream_t stream);
int bin_ctas_per_sm(int kind, int bin, int L, int carveout);
void set_launch_attributes(bool on);
cudaError_t launch_snp_log_prior(const CallArgs& a, double* out, float* out32, cudaStream_t stream);
cudaError_t launch_deferred(const CallArgs& a, int64_t n, cudaStream_t stream,
                            const unsigned long long* d_n = nullptr, int grid = 0);
cudaError_t launch_tile_bounds(const CallArgs& a, int64_t r_begin, int64_t r_end, int64_t next_pos,
                               cudaStream_t stream);
cudaError_t launch_empty_calls(const CallArgs& a, SiteCall* calls, uint8_t* valid, cudaStream_t stream);
int bin_slots(int bin);
inline int kSlotsOf(int bin) { return bin_slots(bin); }
int64_t bin_global_words(int kind, int bin, int64_t count);

/* ---- device helpers ---- */

/* p - first as an address, for arrays that hold elements [first, ...) of an
 * array the kernels index from 0: only indices >= first are used with it */
template <class T>
T* based(T* p, int64_t first) {
    return reinterpret_cast<T*>(reinterpret_cast<uintptr_t>(p) - (uintptr_t)(first * (int64_t)sizeof(T)));
}

struct StreamRing;
void ring_free(StreamRing* g);

/* the launch record kind of a bin's kernel (the FP32 deep bins run
 * call_deep_kernel) */
inline int launch_kind(int kind, int slots) { return kind == kKindFast && slots >= kDeepSlots ? kKindDeep : kind; }

/* a site decided by the deferred pass and its call */
struct DeferredCall {
    int64_t site;
    SiteCall call;
};

/* dst[i] = (site, call) of deferred site i, i < n */
__global__ void deferred_calls_kernel(const DeferredSite* __restrict__ ds, const SiteCall* __restrict__ out, int64_t n,
                                      DeferredCall* __restrict__ dst) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t site = ds[i].site;
        dst[i].site = site;
        dst[i].call = out[site];
    }
}

/* dmax[i] = max(dmax[i], v[i]) for i < 2 (one thread each) */
__global__ void track_max_kernel(const unsigned long long* __restrict__ v, unsigned long long* __restrict__ dmax) {
    if (threadIdx.x < 2) dmax[threadIdx.x] = max(dmax[threadIdx.x], v[threadIdx.x]);
}

/* bytes between device memory and mapped host memory (small control data) */
__global__ void copy_bytes_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

/* The deposited alignments are those that pass the position filters
 * (0 <= pos, pos + len < chr_len), in file order, the first n_dep of them.
 * Their index list is built in chunks of kDepChunk alignments: a count per
 * chunk, an exclusive scan of the counts, and a pass that writes each passing
 * alignment's index at its rank. */
constexpr int kDepThreads = 256;
constexpr int kDepChunk = kDepThreads * 16;

__device__ __forceinline__ bool dep_passes(const int32_t* __restrict__ pos, const int32_t* __restrict__ len,
                                           int64_t i, int64_t chr_len) {
    const int64_t p = pos[i];
    return p >= 0 && p + len[i] < chr_len;
}

__global__ void __launch_bounds__(kDepThreads) dep_count_kernel(int64_t n, const int32_t* __restrict__ pos,
                                                                const int32_t* __restrict__ len, int64_t chr_len,
                                                                int64_t* __restrict__ counts) {
    __shared__ int warp_sum[kDepThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kDepChunk;
    int c = 0;
    for (int j = 0; j < kDepChunk / kDepThreads; ++j) {
        const int64_t i = base + j * kDepThreads + threadIdx.x;
        if (i < n && dep_passes(pos, len, i, chr_len)) ++c;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kDepThreads / 32; ++w) t += warp_sum[w];
        counts[blockIdx.x] = t;
    }
}

/* in-place exclusive scan of the chunk counts, one CTA */
__global__ void __launch_bounds__(1024) dep_scan_kernel(int64_t* __restrict__ counts, int64_t n_chunks) {
    __shared__ int64_t warp_sum[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t b = 0; b < n_chunks; b += 1024) {
        const int64_t i = b + threadIdx.x;
        const int64_t v = i < n_chunks ? counts[i] : 0;
        int64_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int64_t s = warp_sum[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            warp_sum[lane] = s;   /* inclusive over warps */
        }
        __syncthreads();
        const int64_t excl = carry + (warp > 0 ? warp_sum[warp - 1] : 0) + x - v;
        if (i < n_chunks) counts[i] = excl;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_sum[31];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kDepThreads) dep_index_kernel(int64_t n, const int32_t* __restrict__ pos,
                                                                const int32_t* __restrict__ len, int64_t chr_len,
                                                                const int64_t* __restrict__ offsets, int64_t n_dep,
                                                                int64_t* __restrict__ idx) {
    __shared__ int warp_cnt[kDepThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kDepChunk;
    int64_t run = offsets[blockIdx.x];
    for (int j = 0; j < kDepChunk / kDepThreads; ++j) {
        const int64_t i = base + j * kDepThreads + threadIdx.x;
        const bool v = i < n && dep_passes(pos, len, i, chr_len);
        const unsigned ballot = __ballot_sync(0xffffffffu, v);
        if (lane == 0) warp_cnt[warp] = __popc(ballot);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < kDepThreads / 32; ++w) {
            before += w < warp ? warp_cnt[w] : 0;
            total += warp_cnt[w];
        }
        const int64_t r = run + before + __popc(ballot & ((1u << lane) - 1u));
        if (v && r < n_dep) idx[r] = i;
        run += total;
        __syncthreads();
    }
}

constexpr int kGatherRows = 4;   /* row groups per gather block */

__device__ __forceinline__ uint8_t upper_base(uint8_t b, bool* bad) {
    switch (b) {
        case 'A': case 'a': return 'A';
        case 'C': case 'c': return 'C';
        case 'G': case 'g': return 'G';
        case 'T': case 't': return 'T';
        default: *bad = true; return 'A';
    }
}

/* The deposited reads in the packed layout of the calling kernels: start,
 * len<<16|hit, len, strand, and the base|quality row with the bases in upper
 * case ('A' past the read's end; a base other than ACGT/acgt sets *error to
 * 2).  Rows [row_begin, row_end); a block holds rows_per_block rows, each
 * thread VEC consecutive columns of one row (VEC = 4 when L and the pitch are
 * multiples of 4 and L <= pitch: 32-bit loads, 64-bit stores).  PACKED: seq
 * holds gsnp_pack_reads's bytes (qual is not read), which give the base and
 * quality - qmin, or 63 for a quality below qmin (written as qmin - 1). */
__device__ __forceinline__ uint32_t unpack_bq(uint32_t byte, int qmin) {
    const uint32_t code = byte & 63u;
    const uint32_t base = (uint32_t)(uint8_t)"ACTG"[byte >> 6];
    const uint32_t q = code == 63u ? (uint32_t)(uint8_t)(qmin - 1) : (uint32_t)(uint8_t)(qmin + (int)code);
    return base | (q << 8);
}

template <int VEC, bool PACKED = false>
__global__ void __launch_bounds__(256) gather_reads_kernel(
    int64_t row_begin, int64_t row_end, const int64_t* __restrict__ idx, int64_t n_raw, const int32_t* __restrict__ rpos,
    const int32_t* __restrict__ rlen, const int32_t* __restrict__ rhit, const uint8_t* __restrict__ rstrand,
    const uint8_t* __restrict__ seq, const uint8_t* __restrict__ qual, int pitch, int L, int rows_per_block,
    int32_t* __restrict__ pos, int32_t* __restrict__ lenhit, int32_t* __restrict__ len,
    uint8_t* __restrict__ strand, uint16_t* __restrict__ bq, int* __restrict__ error, int qmin = 0) {
    /* kGatherRows groups of rows per block, one row of each group per thread:
     * the groups' load chains (index, length, bases and qualities) are
     * independent, so they are in flight together */
    const int per_row = (L + VEC - 1) / VEC;
    const int local = threadIdx.x / per_row, cv = threadIdx.x - local * per_row;
    const int c0 = cv * VEC;
    const int64_t first = row_begin + (int64_t)blockIdx.x * rows_per_block * kGatherRows + local;
    bool bad = false, bad_idx = false;
    int64_t src[kGatherRows];
    bool ok[kGatherRows];
#pragma unroll
    for (int g = 0; g < kGatherRows; ++g) {
        const int64_t row = first + (int64_t)g * rows_per_block;
        ok[g] = local < rows_per_block && row < row_end;
        src[g] = ok[g] ? idx[row] : 0;
        if (ok[g] && (src[g] < 0 || src[g] >= n_raw)) {   /* the host and device filters disagree */
            bad_idx = true;
            ok[g] = false;
        }
    }
    int32_t rl[kGatherRows];
    uint32_t s4[kGatherRows], q4[kGatherRows];
#pragma unroll
    for (int g = 0; g < kGatherRows; ++g) {
        rl[g] = 0;
        s4[g] = q4[g] = 0;
        if (!ok[g]) continue;
        rl[g] = rlen[src[g]];
        if (VEC == 4) {
            s4[g] = *reinterpret_cast<const uint32_t*>(seq + src[g] * pitch + c0);
            if (!PACKED) q4[g] = *reinterpret_cast<const uint32_t*>(qual + src[g] * pitch + c0);
        } else if (c0 < pitch) {
            s4[g] = seq[src[g] * pitch + c0];
            if (!PACKED) q4[g] = qual[src[g] * pitch + c0];
        }
    }
#pragma unroll
    for (int g = 0; g < kGatherRows; ++g) {
        if (!ok[g]) continue;
        const int64_t row = first + (int64_t)g * rows_per_block;
        if (cv == 0) {
            pos[row] = rpos[src[g]];
            len[row] = rl[g];
            lenhit[row] = (int32_t)(((uint32_t)(rl[g] & 0xffff) << 16) | ((uint32_t)rhit[src[g]] & 0xffffu));
            strand[row] = rstrand[src[g]];
        }
        if (VEC == 4) {
            uint32_t lo = 0, hi = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                uint32_t v;
                if (PACKED) {
                    v = c0 + k < rl[g] ? unpack_bq((s4[g] >> (8 * k)) & 0xffu, qmin) : (uint32_t)'A';
                } else {
                    const uint8_t b = c0 + k < rl[g] ? upper_base((uint8_t)(s4[g] >> (8 * k)), &bad) : (uint8_t)'A';
                    v = (uint32_t)b | (((q4[g] >> (8 * k)) & 0xffu) << 8);
                }
                if (k < 2) lo |= v << (16 * k);
                else hi |= v << (16 * (k - 2));
            }
            *reinterpret_cast<uint2*>(bq + row * L + c0) = make_uint2(lo, hi);
        } else if (PACKED) {
            bq[row * L + c0] = (uint16_t)(c0 < pitch && c0 < rl[g] ? unpack_bq(s4[g] & 0xffu, qmin) : (uint32_t)'A');
        } else {
            uint8_t b = 'A';
            if (c0 < pitch && c0 < rl[g]) b = upper_base((uint8_t)s4[g], &bad);
            bq[row * L + c0] = (uint16_t)b | ((uint16_t)(c0 < pitch ? q4[g] : 0u) << 8);
        }
    }
    const unsigned any_bad = __ballot_sync(0xffffffffu, bad), any_idx = __ballot_sync(0xffffffffu, bad_idx);
    if ((threadIdx.x & 31) == 0 && (any_bad | any_idx)) atomicMax(error, any_idx ? 3 : 2);
}

/* gather_reads_kernel in the form the pitch and the read layout allow */
cudaError_t launch_gather(bool vec4, bool packed, unsigned blocks, cudaStream_t stream, int64_t row_begin,
                          int64_t row_end, const int64_t* idx, int64_t n_raw, const int32_t* rpos, const int32_t* rlen,
                          const int32_t* rhit, const uint8_t* rstrand, const uint8_t* seq, const uint8_t* qual,
                          int pitch, int L, int rows_per_block, int32_t* pos, int32_t* lenhit, int32_t* len,
                          uint8_t* strand, uint16_t* bq, int* error, int qmin) {
#define GSNP_GATHER(V, P)                                                                                      \
    gather_reads_kernel<V, P><<<blocks, 256, 0, stream>>>(row_begin, row_end, idx, n_raw, rpos, rlen, rhit,    \
                                                          rstrand, seq, qual, pitch, L, rows_per_block, pos,  \
                                                          lenhit, len, strand, bq, error, qmin)
    if (vec4) {
        if (packed) GSNP_GATHER(4, true);
        else GSNP_GATHER(4, false);
    } else {
        if (packed) GSNP_GATHER(1, true);
        else GSNP_GATHER(1, false);
    }
#undef GSNP_GATHER
    return cudaGetLastError();
}

/* gsnp_pack_reads's bytes back to base and quality chars (the calibration
 * histogram's input; seq may be packed itself); a quality below qmin becomes
 * qmin - 1 */
__global__ void unpack_reads_kernel(const uint8_t* packed, size_t n, int qmin, uint8_t* seq,
                                    uint8_t* __restrict__ qual) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t v = unpack_bq(packed[i], qmin);
        seq[i] = (uint8_t)(v & 0xffu);
        qual[i] = (uint8_t)(v >> 8);
    }
}

/* pass-1 calibration histogram (cpp/matrix.cc:58-118): unique reads, non-N
 * base, reference neither N nor dbSNP, whole read inside the chromosome.
 * Counts land in [q_char - q_min][cycle][ref][obs]; identical bins within a
 * warp are merged before the atomic. */
__global__ void calib_count_kernel(int64_t n, const int32_t* __restrict__ pos, const int32_t* __restrict__ len,
                                   const int32_t* __restrict__ hit, const uint8_t* __restrict__ strand,
                                   const uint8_t* __restrict__ seq, const uint8_t* __restrict__ qual, int pitch,
                                   const uint8_t* __restrict__ codes, int64_t chr_len, int qmin, int qmax, int L,
                                   unsigned long long* __restrict__ counts) {
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int64_t p = pos[warp];
    const int rl = len[warp];
    if (p < 0 || p + rl >= chr_len || hit[warp] != 1) return;
    const bool minus = strand[warp] != '+';
    for (int c0 = 0; c0 < rl; c0 += 32) {
        const int c = c0 + lane;
        int bin = -1;
        if (c < rl) {
            const signed char b = (signed char)seq[warp * pitch + c];
            const signed char qc = (signed char)qual[warp * pitch + c];
            const int ref = codes[p + c];
            const int cyc = minus ? rl - 1 - c : c;
            if (b != 'N' && (ref & 12) == 0 && qc >= qmin && qc <= qmax && cyc < L)
                bin = (((qc - qmin) * L + cyc) << 4) | ((ref & 3) << 2) | ((b >> 1) & 3);
        }
        const unsigned active = __ballot_sync(0xffffffffu, bin >= 0);
        if (bin >= 0) {
            const unsigned peers = __match_any_sync(active, bin);
            if ((int)(__ffs(peers) - 1) == lane) atomicAdd(counts + bin, (unsigned long long)__popc(peers));
        }
    }
}

/* The same histogram with the matching bins (observed base = reference base,
 * about 99% of the counts) in shared memory: [q - qmin][base][cycle] 32-bit
 * counters, consecutive cycles in consecutive banks, so a warp's 32 lanes
 * (32 cycles of one read) add without conflict.  Mismatches go straight to
 * the global bins.  Each CTA walks reads with a grid stride and adds its
 * shared counts to the global ones once at the end. */
__global__ void __launch_bounds__(512) calib_count_smem_kernel(
    int64_t n, const int32_t* __restrict__ pos, const int32_t* __restrict__ len, const int32_t* __restrict__ hit,
    const uint8_t* __restrict__ strand, const uint8_t* __restrict__ seq, const uint8_t* __restrict__ qual, int pitch,
    const uint8_t* __restrict__ codes, int64_t chr_len, int qmin, int qmax, int L,
    unsigned long long* __restrict__ counts) {
    extern __shared__ uint32_t diag[];
    const int nq = qmax - qmin + 1;
    const int nbins = nq * 4 * L;
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) diag[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        const int64_t p = pos[r];
        const int rl = len[r];
        if (p < 0 || p + rl >= chr_len || hit[r] != 1) continue;
        const bool minus = strand[r] != '+';
        for (int c = lane; c < rl; c += 32) {
            const signed char b = (signed char)seq[r * pitch + c];
            const signed char qc = (signed char)qual[r * pitch + c];
            const int ref = codes[p + c];
            const int cyc = minus ? rl - 1 - c : c;
            if (b == 'N' || (ref & 12) != 0 || qc < qmin || qc > qmax || cyc >= L) continue;
            const int obs = (b >> 1) & 3;
            if (obs == (ref & 3))
                atomicAdd(diag + ((qc - qmin) * 4 + obs) * L + cyc, 1u);
            else
                atomicAdd(counts + ((((qc - qmin) * L + cyc) << 4) | ((ref & 3) << 2) | obs), 1ull);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) {
        const uint32_t v = diag[i];
        if (!v) continue;
        const int cyc = i % L, qb = i / L, base = qb & 3, q = qb >> 2;
        atomicAdd(counts + (((q * L + cyc) << 4) | (base << 2) | base), (unsigned long long)v);
    }
}

}  // namespace gsnp

using namespace gsnp;

struct gsnp_context {
    int device = 0;
    std::string error;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    gsnp_params params{};
    bool have_tables = false;
    HostTables tables;
    /* device tables */
    double* d_lik64 = nullptr;
    float* d_lik32 = nullptr;
    uint8_t* d_qadj = nullptr;
    double* d_p_prior = nullptr;
    double* d_log_prior = nullptr;
    float* d_log_prior32 = nullptr;
    double* d_p_rank = nullptr;
    /* reference */
    int64_t chr_len = 0;
    std::vector<uint8_t> h_codes;
    uint8_t* d_codes = nullptr;
    DbSnpEntry* d_snp = nullptr;
    int64_t n_snp = 0;
    double* d_snp_lp = nullptr;
    float* d_snp_lp32 = nullptr;
    int32_t* d_tile_snp = nullptr;
    bool snp_lp_ready = false;
    /* raw alignments of the last call (device copies, reused across calls) */
    int32_t* d_raw_pos = nullptr;
    int32_t* d_raw_len = nullptr;
    int32_t* d_raw_hit = nullptr;
    uint8_t* d_raw_strand = nullptr;
    uint8_t* d_raw_seq = nullptr;
    uint8_t* d_raw_qual = nullptr;
    int64_t* d_idx = nullptr;
    int64_t* d_dep_off = nullptr;     /* per-chunk offsets of the deposited index list */
    int64_t dep_chunk_cap = 0;
    int64_t raw_cap = 0;
    size_t raw_bytes = 0;
    /* resident reads (deposited, packed) */
    int64_t n_dep = 0;
    int64_t cap_dep = 0;
    int32_t* d_pos = nullptr;
    int32_t* d_lenhit = nullptr;
    int32_t* d_len = nullptr;
    uint8_t* d_strand = nullptr;
    uint16_t* d_bq = nullptr;
    /* window plan */
    WindowPlan plan;
    uint8_t* d_win_flags = nullptr;
    int32_t* d_win_lik_src = nullptr;
    int32_t* d_win_host_src = nullptr;
    int64_t n_win_alloc = 0;
    /* outputs */
    SiteCall* d_out = nullptr;
    SiteCounts* d_counts = nullptr;
    double* d_lik_keep = nullptr;
    int64_t out_sites = 0;
    bool have_counts = false, have_lik_keep = false;
    /* scratch */
    int* d_error = nullptr;
    unsigned long long* d_stats = nullptr;
    int* d_bin_count = nullptr;     /* [kBinCountInts]: counts of the FP64 bins, then fast bins, then counters */
    int32_t* d_bin_tiles = nullptr; /* [2 * kNumBins][n_tiles] */
    DeferredSite* d_dsites = nullptr;        /* sites the fast kernel deferred */
    uint32_t* d_dpool = nullptr;             /* their sorted records */
    unsigned long long* d_dcount = nullptr;  /* [2] requested sites, record words */
    int64_t dsite_cap = 0, dpool_cap = 0;
    int64_t* d_warp_rng = nullptr;  /* [n_tiles][2] */
    int64_t* d_tile_rng = nullptr;  /* [n_tiles][2] */
    uint32_t* d_deep = nullptr;     /* record columns of the deep bins' CTAs */
    int64_t deep_cap = 0;           /* words */
    /* the persistent FP32 kernel: its counters (tiles handed out, leftover
     * count), the leftover tiles, its record slots and grid */
    unsigned long long* d_stream_ctl = nullptr;
    int32_t* d_leftover = nullptr;
    int stream_slots = 0, stream_ctas = 0, stream_ctas_L = -1, stream_carveout = 0;
    bool stream_path = true;
    int stream_mode = 0;            /* 0 plain loads, 1 L2 bulk prefetch, 2 staged in shared memory */
    /* Device-driven calling: the bins' kernels, the classification of the
     * persistent kernel's leftover tiles and the deferred pass read their
     * counts on the device, with grids sized to the resident CTAs, so that a
     * call queues all its work without waiting on the host; the resident
     * recall replays it as a captured CUDA graph. */
    bool device_driven = true, use_graphs = true;
    bool deferred_at_end = false;   /* the last pass ran its deferred sites after its last segment */
    DeferredCall* d_patch = nullptr;   /* their final calls, for the host copy of the calls */
    int64_t patch_cap = 0;
    /* The chunk of windows a streamed call is calling (gsnp_call_streamed):
     * when on, make_args points the kernels at the chunk's ring slot, whose
     * arrays hold reads [R0, R1), tiles [T0, T1) and sites [S0, S1), and at
     * the chunk's window tables and count / likelihood stores, which hold
     * windows [w0 - 1, w1) (entry w0 - 1 carries an earlier window). */
    struct ChunkView {
        bool on = false;
        int64_t w0 = 0, S0 = 0, T0 = 0, T1 = 0, R0 = 0, R1 = 0;
        int64_t tiles_need = 0;     /* tiles of the largest chunk */
        int32_t* pos = nullptr;
        int32_t* lenhit = nullptr;
        uint8_t* strand = nullptr;
        uint16_t* bq = nullptr;
        SiteCall* out = nullptr;
        SiteCounts* counts = nullptr;
        double* lik_keep = nullptr;
        uint8_t* win_flags = nullptr;
        int32_t* win_lik_src = nullptr;
        int32_t* win_host_src = nullptr;
    } view;
    StreamRing* ring = nullptr;
    int64_t stream_windows = 16;    /* windows per chunk of a streamed call */
    bool streamed = false;          /* the last call was streamed: no resident calls */
    /* -C files: windows encoded on the device (columns_gpu.cu), or on the
     * host threads (columns.cpp) */
    bool columns_gpu = true;
    int64_t columns_host_windows = 0;
    std::unique_ptr<ColumnsGpuWriter> colw;   /* kept, with its device buffers, from one use to the next */
    int bin_limit[kNumBins] = {32, 40, 48, 64, 96, 128, 256};
    int bin_carveout[2][kNumBins] = {{0, 0, 0, 0, 0, 0, 0}, {0, 72, 0, 0, 0, 0, 0}};
    int bin_grid[2][kNumBins] = {};
    int grid_L = -1, deferred_grid = 0, classify_grid = 0, sms = 0;
    unsigned long long* d_dmax = nullptr;   /* [2] largest deferred request of the call's segments */
    int* d_bin_hist = nullptr;              /* [2][2 * kNumBins] bin counts of each pass (launch records) */
    cudaGraphExec_t graph_exec = nullptr;
    cudaStream_t capture_stream = nullptr;
    uint64_t graph_key = 0;
    bool graph_failed = false;      /* a capture failed: graphs were turned off */
    SiteCall* d_empty_calls = nullptr;  /* [16] */
    uint8_t* d_empty_valid = nullptr;   /* [16] */
    int64_t tiles_cap = 0;
    int h_bin_count[2 * kNumBins] = {};
    unsigned long long h_dcount[2] = {0, 0};
    bool called = false;
    uint64_t stats[kNumStats] = {};
    /* CUDA events around each launch of the last calling pass */
    static const int kMaxLaunches = 128;
    cudaEvent_t ev[2 * kMaxLaunches] = {};
    gsnp_launch_info launches[kMaxLaunches];
    int launch_ref[kMaxLaunches] = {};   /* a device-driven bin launch: its count in d_bin_hist, else -1 */
    int n_launches = 0;
    uint64_t h2d_bytes = 0, d2h_bytes = 0;
    /* the call's copy streams: uploads in chunks, downloads per segment */
    static const int kUploadChunks = 16;
    static const int kMaxUpStreams = 4;
    cudaStream_t up_stream = nullptr, down_stream = nullptr, gather_stream = nullptr;
    /* the upload's pieces go round-robin over n_up copy streams (up_stream is
     * the first), so that several copy engines can share the host link */
    cudaStream_t up_extra[kMaxUpStreams - 1] = {};
    int n_up = 1;
    cudaStream_t up(int k) const { return k % n_up == 0 ? up_stream : up_extra[k % n_up - 1]; }
    std::vector<cudaEvent_t> ev_gather;   /* per segment: its reads are gathered */
    cudaEvent_t ev_index = nullptr;       /* the deposited index list is built */
    /* the depth bins of one pass run side by side, so that one bin's last
     * wave overlaps the next bin's first */
    static const int kBinStreams = 3;
    cudaStream_t bin_stream[kBinStreams] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[kBinStreams] = {};
    cudaEvent_t ev_small = nullptr, ev_seg = nullptr, ev_chunk[kUploadChunks] = {};
    int* d_gerror = nullptr;       /* gather: 2 a base other than ACGT/acgt, 3 index list mismatch */
    /* Pinned host memory mapped into the device: the small values the host
     * reads back between launches (bin counts, deferred counts, error flags,
     * statistics) and the window tables it sends.  A kernel moves them, so
     * they do not queue behind the call's bulk copies on the copy engines. */
    uint8_t* h_map = nullptr;
    uint8_t* d_map = nullptr;
    size_t map_bytes = 0;
    int64_t n_gathered = 0;        /* deposited reads in the packed layout so far */
    /* cns text emission */
    void* d_emit = nullptr;
    size_t emit_bytes = 0;
    char* d_text = nullptr;
    size_t text_bytes = 0;
    char* d_chr = nullptr;
    char* h_text = nullptr;      /* pinned staging of one chunk */
    size_t h_text_bytes = 0;
};

namespace {

/* Host wall time of the phases of one call, printed to stderr when the
 * environment variable GSNP_TIMING is set. */
struct PhaseTimer {
    const char* what;
    bool on;
    std::chrono::steady_clock::time_point t0, t;
    explicit PhaseTimer(const char* w) : what(w), on(getenv("GSNP_TIMING") != nullptr) {
        t0 = t = std::chrono::steady_clock::now();
    }
    void mark(const char* phase) {
        if (!on) return;
        const auto now = std::chrono::steady_clock::now();
        fprintf(stderr, "%s: %-26s %8.2f ms (total %8.2f ms)\n", what, phase,
                std::chrono::duration<double, std::milli>(now - t).count(),
                std::chrono::duration<double, std::milli>(now - t0).count());
        t = now;
    }
};

/* GPU timestamps of a call's stages on its streams, printed with the phase
 * times when GSNP_TIMING is set */
struct GpuTimeline {
    bool on;
    std::vector<std::pair<std::string, cudaEvent_t>> ev;
    explicit GpuTimeline(bool enabled) : on(enabled) {}
    ~GpuTimeline() {
        for (auto& e : ev) cudaEventDestroy(e.second);
    }
    void rec(const std::string& name, cudaStream_t s) {
        if (!on) return;
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        cudaEventRecord(e, s);
        ev.emplace_back(name, e);
    }
    void print(const char* what) {
        if (!on || ev.empty()) return;
        for (auto& e : ev) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ev[0].second, e.second) == cudaSuccess)
                fprintf(stderr, "%s: gpu %-24s %8.2f ms\n", what, e.first.c_str(), ms);
        }
    }
};

int fail(gsnp_context* c, int code, const std::string& msg) {
    if (c) c->error = msg;
    return code;
}

int cuda_fail(gsnp_context* c, cudaError_t e, const char* what) {
    return fail(c, GSNP_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what)                                  \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
    } while (0)

template <class T>
cudaError_t dev_alloc(T** p, size_t count) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(T));
}

/* device buffers of one call, freed when it returns, on every path */
struct CallTemps {
    std::vector<void*> ptrs;
    CallTemps() = default;
    CallTemps(const CallTemps&) = delete;
    CallTemps& operator=(const CallTemps&) = delete;
    ~CallTemps() {
        for (void* q : ptrs) cudaFree(q);
    }
    template <class T>
    cudaError_t alloc(T** q, size_t bytes) {
        const cudaError_t e = cudaMalloc((void**)q, bytes);
        if (e == cudaSuccess) ptrs.push_back(*q);
        return e;
    }
};

/* host threads for the per-alignment pass of the window replay:
 * GSNP_HOST_THREADS, else every hardware thread (at most 64) */
int host_threads() {
    static const int n = [] {
        const char* e = getenv("GSNP_HOST_THREADS");
        int v = e ? atoi(e) : 0;
        if (v <= 0) v = (int)std::thread::hardware_concurrency();
        return std::max(1, std::min(v, 64));
    }();
    return n;
}

/* layout of the mapped control area */
constexpr size_t kMapBins = 0;       /* int[2 * kNumBins] */
constexpr size_t kMapDcount = 64;    /* unsigned long long[2] */
constexpr size_t kMapError = 96;     /* int */
constexpr size_t kMapGerror = 100;   /* int */
constexpr size_t kMapLeftover = 104; /* int */
constexpr size_t kMapStats = 128;    /* unsigned long long[kNumStats] */
constexpr size_t kMapBinHist = 256;  /* int[2][2 * kNumBins]: each pass's bin counts */
constexpr size_t kMapWindows = 512;  /* the call's window tables */
static_assert(sizeof(int) * 2 * kNumBins <= kMapDcount, "bin counts overlap the deferred counts");

int ensure_map(gsnp_context* c, size_t bytes) {
    if (bytes <= c->map_bytes) return GSNP_OK;
    if (c->h_map) {
        cudaFreeHost(c->h_map);
        c->h_map = c->d_map = nullptr;
        c->map_bytes = 0;
    }
    CK(cudaHostAlloc((void**)&c->h_map, bytes, cudaHostAllocMapped), "cudaHostAlloc");
    CK(cudaHostGetDevicePointer((void**)&c->d_map, c->h_map, 0), "cudaHostGetDevicePointer");
    c->map_bytes = bytes;
    return GSNP_OK;
}

/* device bytes to the mapped area at off, and back, on the context's stream */
cudaError_t to_map(gsnp_context* c, const void* d_src, size_t off, size_t n) {
    copy_bytes_kernel<<<1, 128, 0, c->stream>>>((const uint8_t*)d_src, c->d_map + off, n);
    return cudaGetLastError();
}

cudaError_t from_map(gsnp_context* c, size_t off, void* d_dst, size_t n) {
    const unsigned blocks = (unsigned)std::max<size_t>(1, std::min<size_t>(64, (n + 255) / 256));
    copy_bytes_kernel<<<blocks, 256, 0, c->stream>>>(c->d_map + off, (uint8_t*)d_dst, n);
    return cudaGetLastError();
}

void free_all(gsnp_context* c) {
    void* ptrs[] = {c->d_lik64, c->d_lik32, c->d_qadj, c->d_p_prior, c->d_log_prior, c->d_log_prior32,
                    c->d_p_rank, c->d_codes, c->d_snp, c->d_snp_lp, c->d_snp_lp32, c->d_pos, c->d_lenhit,
                    c->d_len, c->d_strand, c->d_bq, c->d_win_flags, c->d_win_lik_src, c->d_out, c->d_counts,
                    c->d_lik_keep, c->d_error, c->d_stats, c->d_bin_count, c->d_bin_tiles, c->d_dsites,
                    c->d_dpool, c->d_dcount, c->d_warp_rng, c->d_win_host_src, c->d_emit,
                    c->d_text, c->d_chr, c->d_tile_snp, c->d_tile_rng, c->d_empty_calls, c->d_empty_valid,
                    c->d_raw_pos, c->d_raw_len, c->d_raw_hit, c->d_raw_strand, c->d_raw_seq, c->d_raw_qual,
                    c->d_idx, c->d_dep_off, c->d_gerror, c->d_deep, c->d_stream_ctl, c->d_leftover,
                    c->d_dmax, c->d_patch, c->d_bin_hist};
    for (void* p : ptrs)
        if (p) cudaFree(p);
}

CallArgs make_args(gsnp_context* c) {
    CallArgs a;
    memset(&a, 0, sizeof(a));
    a.pos = c->d_pos;
    a.lenhit = c->d_lenhit;
    a.strand = c->d_strand;
    a.bq = c->d_bq;
    a.n_reads = c->n_dep;
    a.L = c->params.read_length;
    a.ori = c->d_codes;
    a.chr_len = c->chr_len;
    a.snp = c->d_snp;
    a.n_snp = c->n_snp;
    a.tile_snp = c->d_tile_snp;
    a.snp_lp = c->d_snp_lp;
    a.snp_lp32 = c->d_snp_lp32;
    a.lik64 = c->d_lik64;
    a.lik32 = c->d_lik32;
    a.lik32b = c->d_lik32 ? c->d_lik32 + (size_t)c->tables.qa_rows * c->tables.L * 4 * 8 : nullptr;
    a.qa_rows = c->tables.qa_rows;
    a.qadj = c->d_qadj;
    a.tmax = c->tables.tmax;
    a.gmax = c->tables.gmax;
    a.p_prior = c->d_p_prior;
    a.log_prior = c->d_log_prior;
    a.log_prior32 = c->d_log_prior32;
    a.p_rank = c->d_p_rank;
    a.qmin = c->params.q_min;
    a.q_max_min = (int)(signed char)(c->params.q_max - c->params.q_min);
    a.rank_sum = c->params.rank_sum;
    a.monoploid = c->params.monoploid;
    a.refine = c->params.refine;
    a.het_val = c->params.het_val;
    a.het_unval = c->params.het_unval;
    a.althom_val = c->params.althom_val;
    a.althom_unval = c->params.althom_unval;
    /* the FP32 error bound needs every table term <= 0 */
    a.precision = c->tables.all_nonpositive ? c->params.precision : GSNP_PRECISION_FP64;
    for (int b = 0; b < kNumBins; ++b) a.bin_limit[b] = c->bin_limit[b];
    a.win_flags = c->d_win_flags;
    a.win_lik_src = c->d_win_lik_src;
    a.n_tiles = (c->chr_len + kTile - 1) / kTile;
    a.tile_lo = 0;
    a.bin_stride = c->tiles_cap;
    a.warp_rng = c->d_warp_rng;
    a.tile_rng = c->d_tile_rng;
    a.empty_calls = c->d_empty_calls;
    a.empty_valid = c->d_empty_valid;
    a.dsites = c->d_dsites;
    a.dpool = c->d_dpool;
    a.dcount = c->d_dcount;
    a.dsite_cap = c->dsite_cap;
    a.dpool_cap = c->dpool_cap;
    a.out = c->d_out;
    a.counts = c->d_counts;
    a.lik_keep = c->d_lik_keep;
    a.stats = c->d_stats;
    a.error = c->d_error;
    a.read_lo = 0;
    if (c->view.on) {
        /* a streamed chunk: every array indexed by read, tile, site or window
         * is its ring slot's, based so that the kernels' indices stay
         * absolute */
        const gsnp_context::ChunkView& v = c->view;
        const int64_t L = c->params.read_length;
        a.pos = based(v.pos, v.R0);
        a.lenhit = based(v.lenhit, v.R0);
        a.strand = based(v.strand, v.R0);
        a.bq = based(v.bq, v.R0 * L);
        a.read_lo = v.R0;
        a.n_reads = v.R1;
        a.n_tiles = v.T1;
        a.tile_lo = v.T0;
        a.warp_rng = based(c->d_warp_rng, 2 * v.T0);
        a.tile_rng = based(c->d_tile_rng, 2 * v.T0);
        a.out = based(v.out, v.S0);
        a.counts = v.counts ? based(v.counts, (v.w0 - 1) * kWin) : nullptr;
        a.lik_keep = v.lik_keep ? based(v.lik_keep, (v.w0 - 1) * kWin * 10) : nullptr;
        a.win_flags = based(v.win_flags, v.w0 - 1);
        a.win_lik_src = based(v.win_lik_src, v.w0 - 1);
    }
    return a;
}

/* A stretch of whole windows called together: its tiles, the deposited reads
 * that start in it, the alignments that hold them and the start of the next
 * deposited read. */
struct Segment {
    int64_t t0, t1;      /* tiles */
    int64_t dlo, dhi;    /* deposited reads */
    int64_t raw_hi;      /* alignments [0, raw_hi) hold deposited reads [0, dhi) */
    int64_t next_pos;    /* start of deposited read dhi, kNoRead when there is none */
};

/* The calling pass, segment by segment.  before(s) runs first for each
 * segment (the call gathers the reads there: those of segments 0 .. s must be
 * on the device), after(s) once its calls are queued. */
/* Allocations and one-time work of a calling pass, done before any of its
 * work is queued (and outside a graph capture). */
int prepare_calling(gsnp_context* c) {
    /* the tile arrays hold the chromosome's tiles, or a streamed chunk's */
    const int64_t n_tiles = c->view.on ? c->view.tiles_need : (c->chr_len + kTile - 1) / kTile;
    {
        const int rc = ensure_map(c, kMapWindows);
        if (rc != GSNP_OK) return rc;
    }
    if (!c->snp_lp_ready) {
        CK(dev_alloc(&c->d_snp_lp, (size_t)std::max<int64_t>(c->n_snp, 1) * 16), "cudaMalloc dbSNP priors");
        CK(dev_alloc(&c->d_snp_lp32, (size_t)std::max<int64_t>(c->n_snp, 1) * 12), "cudaMalloc dbSNP priors");
        if (!c->d_empty_calls) {
            CK(dev_alloc(&c->d_empty_calls, 16), "cudaMalloc");
            CK(dev_alloc(&c->d_empty_valid, 16), "cudaMalloc");
        }
        const CallArgs a0 = make_args(c);
        CK(launch_snp_log_prior(a0, c->d_snp_lp, c->d_snp_lp32, c->stream), "dbSNP prior kernel");
        CK(launch_empty_calls(a0, c->d_empty_calls, c->d_empty_valid, c->stream), "empty-site calls");
        c->snp_lp_ready = true;
    }
    if (n_tiles > c->tiles_cap) {
        CK(dev_alloc(&c->d_bin_tiles, (size_t)n_tiles * 2 * kNumBins), "cudaMalloc bins");
        CK(dev_alloc(&c->d_warp_rng, (size_t)n_tiles * 2), "cudaMalloc ranges");
        CK(dev_alloc(&c->d_tile_rng, (size_t)n_tiles * 2), "cudaMalloc ranges");
        CK(dev_alloc(&c->d_leftover, (size_t)n_tiles), "cudaMalloc leftover tiles");
        c->tiles_cap = n_tiles;
    }
    if (!c->d_stream_ctl) CK(dev_alloc(&c->d_stream_ctl, 2), "cudaMalloc stream counters");
    if (c->stream_ctas_L != c->params.read_length || c->stream_slots == 0) {
        /* the persistent kernel's grid: every resident CTA of the GPU */
        if (c->stream_slots == 0) c->stream_slots = 48;
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device), "device attribute");
        c->stream_ctas =
            sms * stream_ctas_per_sm(c->stream_slots, c->params.read_length, c->stream_mode, c->stream_carveout);
        c->stream_ctas_L = c->params.read_length;
    }
    if (c->dsite_cap == 0) {
        /* deferred sites: about 0.1% of a 30x genome; grown on demand */
        c->dsite_cap = std::max<int64_t>(1 << 16, (c->view.on ? n_tiles * kTile : c->chr_len) / 256);
        c->dpool_cap = c->dsite_cap * 48;
        CK(dev_alloc(&c->d_dsites, (size_t)c->dsite_cap), "cudaMalloc deferred");
        CK(dev_alloc(&c->d_dpool, (size_t)c->dpool_cap), "cudaMalloc deferred");
    }
    if (!c->ev[0])
        for (int i = 0; i < 2 * gsnp_context::kMaxLaunches; ++i) CK(cudaEventCreate(&c->ev[i]), "cudaEventCreate");
    if (!c->ev_fork) {
        CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "cudaEventCreate");
        for (int i = 0; i < gsnp_context::kBinStreams; ++i) {
            CK(cudaStreamCreateWithFlags(&c->bin_stream[i], cudaStreamNonBlocking), "cudaStreamCreate");
            CK(cudaEventCreateWithFlags(&c->ev_join[i], cudaEventDisableTiming), "cudaEventCreate");
        }
    }
    if (c->device_driven) {
        if (!c->d_dmax) CK(dev_alloc(&c->d_dmax, 2), "cudaMalloc");
        if (!c->d_bin_hist) {
            CK(dev_alloc(&c->d_bin_hist, 4 * kNumBins), "cudaMalloc");
            CK(cudaMemset(c->d_bin_hist, 0, sizeof(int) * 4 * kNumBins), "memset");
        }
        if (c->grid_L != c->params.read_length) {
            /* grids of the device-driven launches: the resident CTAs */
            CK(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device), "device attribute");
            for (int kind = 0; kind < 2; ++kind)
                for (int b = 0; b < kNumBins; ++b)
                    c->bin_grid[kind][b] = c->sms * bin_ctas_per_sm(kind == 0 ? kKindFP64 : kKindFast, b,
                                                                   c->params.read_length, c->bin_carveout[kind][b]);
            c->deferred_grid = c->sms * 32;
            c->classify_grid = c->sms * 4;
            c->grid_L = c->params.read_length;
        }
        /* record columns of the deepest fast bin: one slice per resident CTA */
        const int64_t words = bin_global_words(kKindFast, kNumBins - 1, c->bin_grid[1][kNumBins - 1]);
        if (words > c->deep_cap) {
            CK(dev_alloc(&c->d_deep, (size_t)words), "cudaMalloc deep scratch");
            c->deep_cap = words;
        }
    }
    return GSNP_OK;
}

/* The result checks of a device-driven pass, once its work is queued: the
 * error word, the statistics and the largest deferred-site request, through
 * the mapped control area. */
constexpr int kRedoDeferred = -100;   /* the deferred pool was too small: it was grown, call again */

int finish_device(gsnp_context* c) {
    CK(to_map(c, c->d_error, kMapError, sizeof(int)), "error flag");
    CK(to_map(c, c->d_stats, kMapStats, sizeof(c->stats)), "stats");
    CK(to_map(c, c->d_dmax, kMapDcount, sizeof(c->h_dcount)), "deferred counts");
    if (c->d_bin_hist) CK(to_map(c, c->d_bin_hist, kMapBinHist, sizeof(int) * 4 * kNumBins), "bin counts");
    CK(cudaStreamSynchronize(c->stream), "calling");
    if (c->d_bin_hist) {
        /* the tiles each recorded bin launch took, now that they are known */
        int hist[4 * kNumBins];
        memcpy(hist, c->h_map + kMapBinHist, sizeof hist);
        for (int k = 0; k < c->n_launches; ++k)
            if (c->launch_ref[k] >= 0) {
                c->launches[k].tiles = hist[c->launch_ref[k]];
                c->launches[k].sites = std::min<int64_t>((int64_t)hist[c->launch_ref[k]] * kTile, c->chr_len);
            }
    }
    int err = 0;
    memcpy(&err, c->h_map + kMapError, sizeof(int));
    memcpy(c->stats, c->h_map + kMapStats, sizeof(c->stats));
    memcpy(c->h_dcount, c->h_map + kMapDcount, sizeof(c->h_dcount));
    for (int k = 0; k < c->n_launches; ++k) cudaEventElapsedTime(&c->launches[k].ms, c->ev[2 * k], c->ev[2 * k + 1]);
    if (err == 1) return fail(c, GSNP_ERR_CAPACITY, "a site is covered by more than 65535 alignments");
    if (err == 5) return fail(c, GSNP_ERR_STATE, "a staging bulk copy of the calling kernel did not complete");
    if (err) return fail(c, GSNP_ERR_STATE, "record slots of a tile overflowed its depth bin");
    const int64_t ns = (int64_t)c->h_dcount[0], nw = (int64_t)c->h_dcount[1];
    if (ns > c->dsite_cap || nw > c->dpool_cap) {
        c->dsite_cap = std::max(c->dsite_cap, ns + ns / 8 + 1024);
        c->dpool_cap = std::max(c->dpool_cap, nw + nw / 8 + 65536);
        CK(dev_alloc(&c->d_dsites, (size_t)c->dsite_cap), "cudaMalloc deferred");
        CK(dev_alloc(&c->d_dpool, (size_t)c->dpool_cap), "cudaMalloc deferred");
        return kRedoDeferred;
    }
    c->stats[0] = (uint64_t)c->chr_len;
    c->called = true;
    return GSNP_OK;
}

/* device-driven queueing of a calling pass (defined below) */
int enqueue_device(gsnp_context* c, const std::vector<Segment>& segs, const std::function<int(size_t)>& before,
                   const std::function<int(size_t)>& after, bool record);

int run_calling(gsnp_context* c, const std::vector<Segment>& segs, const std::function<int(size_t)>& before,
                const std::function<int(size_t)>& after) {
    const int64_t n_tiles = (c->chr_len + kTile - 1) / kTile;
    c->deferred_at_end = false;
    {
        const int rc = prepare_calling(c);
        if (rc != GSNP_OK) return rc;
    }
    if (c->device_driven) {
        const int rc = enqueue_device(c, segs, before, after, true);
        if (rc != GSNP_OK) return rc;
        return finish_device(c);
    }
    CK(cudaMemsetAsync(c->d_error, 0, sizeof(int), c->stream), "memset");
    CK(cudaMemsetAsync(c->d_stats, 0, sizeof(unsigned long long) * kNumStats, c->stream), "memset");
    const CallArgs a = make_args(c);
    bool any_external = false;
    for (int64_t w = 0; w < c->plan.n_windows; ++w) any_external |= (c->plan.flags[w] & kWinExternalLik) != 0;
    c->n_launches = 0;
    auto begin = [&](int kind, int sl, int64_t tiles) -> int {
        if (c->n_launches >= gsnp_context::kMaxLaunches) return -1;
        const int k = c->n_launches++;
        c->launches[k].kind = kind;
        c->launches[k].slots = sl;
        c->launches[k].tiles = tiles;
        c->launches[k].sites = std::min<int64_t>(tiles * kTile, c->chr_len);
        c->launches[k].ms = 0.f;
        c->launch_ref[k] = -1;
        cudaEventRecord(c->ev[2 * k], c->stream);
        return k;
    };
    auto end = [&](int k) {
        if (k >= 0) cudaEventRecord(c->ev[2 * k + 1], c->stream);
    };
    /* launch records of the bins, timed on the bin's own stream */
    auto begin_on = [&](int kind, int sl, int64_t tiles, cudaStream_t st) -> int {
        const int k = begin(kind, sl, tiles);
        if (k >= 0) cudaEventRecord(c->ev[2 * k], st);
        return k;
    };
    auto end_on = [&](int k, cudaStream_t st) {
        if (k >= 0) cudaEventRecord(c->ev[2 * k + 1], st);
    };
    /* the non-empty bins of kind in decreasing tile count.  In a call of
     * several segments, whose bins are small launches, they run side by side
     * on the bin streams (the context's stream waits for all of them); a
     * single pass runs them in turn, each launch timed on its own. */
    const bool side_by_side = segs.size() > 1;
    auto launch_bins = [&](const CallArgs& args, int kind, int base) -> int {
        int order[kNumBins], m = 0;
        for (int b = 0; b < kNumBins; ++b)
            if (c->h_bin_count[base + b] > 0) order[m++] = b;
        std::sort(order, order + m, [&](int x, int y) { return c->h_bin_count[base + x] > c->h_bin_count[base + y]; });
        if (m == 0) return GSNP_OK;
        /* the deep bins' record columns: a slice of the scratch per launch */
        int64_t off[kNumBins] = {}, words = 0;
        for (int j = 0; j < m; ++j) {
            off[order[j]] = words;
            words += bin_global_words(kind, order[j], c->h_bin_count[base + order[j]]);
        }
        if (words > c->deep_cap) {
            CK(cudaStreamSynchronize(c->stream), "deep scratch");
            CK(dev_alloc(&c->d_deep, (size_t)(words + words / 4)), "cudaMalloc deep scratch");
            c->deep_cap = words + words / 4;
        }
        auto with_scratch = [&](int b) {
            CallArgs la = args;
            la.deep_recs = c->d_deep + off[b];
            return la;
        };
        if (!side_by_side) {
            for (int j = 0; j < m; ++j) {
                const int b = order[j];
                const int nb = c->h_bin_count[base + b];
                const int k = begin(launch_kind(kind, bin_slots(b)), bin_slots(b), nb);
                const BinLaunch bl{nb, nullptr, 0, c->bin_carveout[kind == kKindFast][b]};
                CK(launch_bin(with_scratch(b), kind, b, c->d_bin_tiles + (int64_t)(base + b) * c->tiles_cap, bl, c->stream),
                   "calling kernel");
                end(k);
            }
            return GSNP_OK;
        }
        CK(cudaEventRecord(c->ev_fork, c->stream), "event");
        const int ns = std::min(m, (int)gsnp_context::kBinStreams);
        for (int i = 0; i < ns; ++i) CK(cudaStreamWaitEvent(c->bin_stream[i], c->ev_fork, 0), "wait");
        for (int j = 0; j < m; ++j) {
            const int b = order[j];
            cudaStream_t st = c->bin_stream[j % ns];
            const int nb = c->h_bin_count[base + b];
            const int k = begin_on(launch_kind(kind, bin_slots(b)), bin_slots(b), nb, st);
            const BinLaunch bl{nb, nullptr, 0, c->bin_carveout[kind == kKindFast][b]};
            CK(launch_bin(with_scratch(b), kind, b, c->d_bin_tiles + (int64_t)(base + b) * c->tiles_cap, bl, st),
               "calling kernel");
            end_on(k, st);
        }
        for (int i = 0; i < ns; ++i) {
            CK(cudaEventRecord(c->ev_join[i], c->bin_stream[i]), "event");
            CK(cudaStreamWaitEvent(c->stream, c->ev_join[i], 0), "wait");
        }
        return GSNP_OK;
    };
    for (size_t si = 0; si < segs.size(); ++si) {
        const Segment& g = segs[si];
        if (before) {
            const int rc = before(si);
            if (rc != GSNP_OK) return rc;
        }
        CallArgs a = make_args(c);
        a.n_reads = c->n_gathered;
        /* In the FP32 form the persistent kernel calls the segment's tiles;
         * the binned kernels take only the tiles it leaves (the FP64 windows'
         * and those with a site deeper than its record slots). */
        const bool use_stream = c->stream_path && c->params.precision == 1 && segs.size() == 1 && !c->view.on;
        int64_t n_left = 0;
        auto run_stream = [&](const CallArgs& as) -> int {
            CK(cudaMemsetAsync(c->d_stream_ctl, 0, 2 * sizeof(unsigned long long), c->stream), "memset");
            const StreamQueue q{g.t0, g.t1, c->d_stream_ctl, c->d_leftover, reinterpret_cast<int*>(c->d_stream_ctl + 1)};
            const int ks = begin(kKindStream, c->stream_slots, g.t1 - g.t0);
            CK(launch_stream(as, q, c->stream_slots, c->stream_mode, c->stream_ctas, c->stream_carveout, c->stream),
               "persistent calling kernel");
            end(ks);
            return GSNP_OK;
        };
        CK(launch_tile_bounds(a, g.dlo, g.dhi, g.next_pos, c->stream), "tile bounds kernel");
        for (int pass = 0; pass < (any_external ? 2 : 1); ++pass) {
            const bool stream_pass = use_stream && pass == 0;
            if (stream_pass) {
                CK(cudaMemsetAsync(c->d_dcount, 0, sizeof(unsigned long long) * 2, c->stream), "memset");
                const int rc = run_stream(a);
                if (rc != GSNP_OK) return rc;
                CK(to_map(c, c->d_stream_ctl + 1, kMapLeftover, sizeof(int)), "leftover count");
                CK(cudaStreamSynchronize(c->stream), "persistent calling kernel");
                int nl = 0;
                memcpy(&nl, c->h_map + kMapLeftover, sizeof(int));
                n_left = nl;
            }
            const int k = begin(kKindClassify, 0, use_stream ? n_left : g.t1 - g.t0);
            if (use_stream)
                CK(launch_classify(a, pass, 0, n_left, c->d_bin_count, c->d_bin_tiles, c->stream, c->d_leftover),
                   "classify kernel");
            else
                CK(launch_classify(a, pass, g.t0, g.t1, c->d_bin_count, c->d_bin_tiles, c->stream), "classify kernel");
            end(k);
            CK(to_map(c, c->d_bin_count, kMapBins, sizeof(c->h_bin_count)), "bin counts");
            CK(cudaStreamSynchronize(c->stream), "classify");
            memcpy(c->h_bin_count, c->h_map + kMapBins, sizeof(c->h_bin_count));
            bool any_fast = stream_pass;
            for (int b = 0; b < kNumBins; ++b) any_fast |= c->h_bin_count[kNumBins + b] > 0;
            {
                const int rc = launch_bins(a, kKindFP64, 0);
                if (rc != GSNP_OK) return rc;
            }
            if (!any_fast) continue;
            for (int attempt = 0; attempt < 2; ++attempt) {
                CallArgs af = make_args(c);
                af.n_reads = c->n_gathered;
                const int first = c->n_launches;
                if (!(stream_pass && attempt == 0))
                    CK(cudaMemsetAsync(c->d_dcount, 0, sizeof(unsigned long long) * 2, c->stream), "memset");
                if (stream_pass && attempt > 0) {
                    /* the pool was too small: the persistent kernel's
                     * deferrals are appended again too */
                    const int rc = run_stream(af);
                    if (rc != GSNP_OK) return rc;
                }
                {
                    const int rc = launch_bins(af, kKindFast, kNumBins);
                    if (rc != GSNP_OK) return rc;
                }
                CK(to_map(c, c->d_dcount, kMapDcount, sizeof(c->h_dcount)), "deferred counts");
                CK(cudaStreamSynchronize(c->stream), "fast calling");
                memcpy(c->h_dcount, c->h_map + kMapDcount, sizeof(c->h_dcount));
                const int64_t ns = (int64_t)c->h_dcount[0], nw = (int64_t)c->h_dcount[1];
                if (ns <= c->dsite_cap && nw <= c->dpool_cap) {
                    if (ns > 0) {
                        const int kd = begin(kKindDeferred, 0, (ns + kTile - 1) / kTile);
                        if (kd >= 0) c->launches[kd].sites = ns;
                        CK(launch_deferred(af, ns, c->stream), "deferred calling kernel");
                        end(kd);
                    }
                    break;
                }
                if (attempt == 1) return fail(c, GSNP_ERR_STATE, "deferred-site pool overflow");
                /* grow the pool to what the segment asked for and run its fast
                 * kernels again (their sampled-site statistics were not yet
                 * counted: that happens in the deferred pass) */
                c->dsite_cap = std::max(c->dsite_cap, ns + ns / 8 + 1024);
                c->dpool_cap = std::max(c->dpool_cap, nw + nw / 8 + 65536);
                CK(dev_alloc(&c->d_dsites, (size_t)c->dsite_cap), "cudaMalloc deferred");
                CK(dev_alloc(&c->d_dpool, (size_t)c->dpool_cap), "cudaMalloc deferred");
                c->n_launches = first;
            }
        }
        if (after) {
            const int rc = after(si);
            if (rc != GSNP_OK) return rc;
        }
    }
    int err = 0;
    CK(to_map(c, c->d_error, kMapError, sizeof(int)), "error flag");
    CK(to_map(c, c->d_stats, kMapStats, sizeof(c->stats)), "stats");
    CK(cudaStreamSynchronize(c->stream), "calling");
    memcpy(&err, c->h_map + kMapError, sizeof(int));
    memcpy(c->stats, c->h_map + kMapStats, sizeof(c->stats));
    for (int k = 0; k < c->n_launches; ++k) cudaEventElapsedTime(&c->launches[k].ms, c->ev[2 * k], c->ev[2 * k + 1]);
    if (err == 1) return fail(c, GSNP_ERR_CAPACITY, "a site is covered by more than 65535 alignments");
    if (err == 5) return fail(c, GSNP_ERR_STATE, "a staging bulk copy of the calling kernel did not complete");
    if (err) return fail(c, GSNP_ERR_STATE, "record slots of a tile overflowed its depth bin");
    c->stats[0] = (uint64_t)c->chr_len;
    c->called = true;
    return GSNP_OK;
}


/* One pass queued with its launch sizes read on the device (see the
 * device_driven field of the context): per segment the tile ranges, in the
 * FP32 form the persistent kernel and the classification of the tiles it
 * leaves, the depth bins' kernels (each a grid of its resident CTAs taking the
 * bin's tiles in turn), the deferred pass, and, when the segment has windows
 * that take their likelihood from another window, the second pass of those.
 * Nothing here waits on the host.  record: launch records with events
 * (false while a graph is captured). */
int enqueue_device(gsnp_context* c, const std::vector<Segment>& segs, const std::function<int(size_t)>& before,
                   const std::function<int(size_t)>& after, bool record) {
    const int64_t n_tiles = (c->chr_len + kTile - 1) / kTile;
    CK(cudaMemsetAsync(c->d_error, 0, sizeof(int), c->stream), "memset");
    CK(cudaMemsetAsync(c->d_stats, 0, sizeof(unsigned long long) * kNumStats, c->stream), "memset");
    CK(cudaMemsetAsync(c->d_dmax, 0, 2 * sizeof(unsigned long long), c->stream), "memset");
    c->n_launches = 0;
    auto begin = [&](int kind, int sl, int64_t tiles) -> int {
        if (!record || c->n_launches >= gsnp_context::kMaxLaunches) return -1;
        const int k = c->n_launches++;
        c->launches[k].kind = kind;
        c->launches[k].slots = sl;
        c->launches[k].tiles = tiles;
        c->launches[k].sites = std::min<int64_t>(tiles * kTile, c->chr_len);
        c->launches[k].ms = 0.f;
        c->launch_ref[k] = -1;
        cudaEventRecord(c->ev[2 * k], c->stream);
        return k;
    };
    auto end = [&](int k) {
        if (k >= 0) cudaEventRecord(c->ev[2 * k + 1], c->stream);
    };
    const bool fast = make_args(c).precision == 1;
    /* the persistent kernel for a whole-chromosome pass: a call in segments
     * (or chunks) ends each segment's launch of it in a tail of its own, and
     * its binned kernels, handing out tiles from counters, were the faster
     * there (c1 e2e in 7 segments: 28.6-29.0 against 29.9 ms) */
    const bool use_stream = c->stream_path && fast && segs.size() == 1 && !c->view.on;
    int* d_left = reinterpret_cast<int*>(c->d_stream_ctl + 1);
    /* With several segments the deferred sites of all of them go to one pool
     * and one deferred pass runs after the last segment: the pass takes about
     * the time of its slowest site (one thread per site, serial FP64 work),
     * whatever their number, so a pass per segment would cost that time per
     * segment.  The segments' downloads then hold those sites pending, and
     * call_chromosome patches them in (patch_deferred_calls). */
    const bool defer_to_end = fast && segs.size() > 1;
    c->deferred_at_end = defer_to_end;
    if (defer_to_end) CK(cudaMemsetAsync(c->d_dcount, 0, sizeof(unsigned long long) * 2, c->stream), "memset");
    auto deferred_pass = [&]() -> int {
        CallArgs a = make_args(c);
        a.n_reads = c->n_gathered;
        a.deep_recs = c->d_deep;
        const int kd = begin(kKindDeferred, 0, 0);
        CK(launch_deferred(a, 0, c->stream, c->d_dcount, c->deferred_grid), "deferred calling kernel");
        end(kd);
        track_max_kernel<<<1, 2, 0, c->stream>>>(c->d_dcount, c->d_dmax);
        CK(cudaGetLastError(), "deferred counts");
        return GSNP_OK;
    };
    for (size_t si = 0; si < segs.size(); ++si) {
        const Segment& g = segs[si];
        if (before) {
            const int rc = before(si);
            if (rc != GSNP_OK) return rc;
        }
        /* which passes the segment's windows need (the host replay knows) */
        bool keep_lik = false, external = false;
        const int64_t w0 = g.t0 * kTile / kWin, w1 = std::min<int64_t>(c->plan.n_windows, (g.t1 * kTile + kWin - 1) / kWin);
        for (int64_t w = w0; w < w1; ++w) {
            keep_lik |= (c->plan.flags[w] & kWinKeepLik) != 0;
            external |= (c->plan.flags[w] & kWinExternalLik) != 0;
        }
        CallArgs a = make_args(c);
        a.n_reads = c->n_gathered;
        a.deep_recs = c->d_deep;
        int k = begin(kKindClassify, 0, g.t1 - g.t0);
        CK(launch_tile_bounds(a, g.dlo, g.dhi, g.next_pos, c->stream), "tile bounds kernel");
        if (!defer_to_end) CK(cudaMemsetAsync(c->d_dcount, 0, sizeof(unsigned long long) * 2, c->stream), "memset");
        auto bins = [&](int kind, int pass) -> int {
            const int ki = kind == kKindFast ? 1 : 0;
            for (int b = 0; b < kNumBins; ++b) {
                /* after the persistent kernel, the fast bins get only tiles
                 * deeper than its record slots */
                if (kind == kKindFast && use_stream && kSlotsOf(b) <= c->stream_slots) continue;
                const BinLaunch bl{0, c->d_bin_count + ki * kNumBins + b, c->bin_grid[ki][b], c->bin_carveout[ki][b],
                                   c->d_bin_count + (2 + ki) * kNumBins + b};
                const int kb = begin(launch_kind(kind, kSlotsOf(b)), kSlotsOf(b), 0);
                if (kb >= 0) c->launch_ref[kb] = pass * 2 * kNumBins + ki * kNumBins + b;
                CK(launch_bin(a, kind, b, c->d_bin_tiles + (int64_t)(ki * kNumBins + b) * c->tiles_cap, bl, c->stream),
                   "calling kernel");
                end(kb);
            }
            return GSNP_OK;
        };
        /* pass 0 */
        if (use_stream) {
            CK(cudaMemsetAsync(c->d_stream_ctl, 0, 2 * sizeof(unsigned long long), c->stream), "memset");
            end(k);
            const StreamQueue q{g.t0, g.t1, c->d_stream_ctl, c->d_leftover, d_left};
            const int ks = begin(kKindStream, c->stream_slots, g.t1 - g.t0);
            CK(launch_stream(a, q, c->stream_slots, c->stream_mode, c->stream_ctas, c->stream_carveout, c->stream),
               "persistent calling kernel");
            end(ks);
            k = begin(kKindClassify, 0, 0);
            CK(launch_classify(a, 0, 0, 0, c->d_bin_count, c->d_bin_tiles, c->stream, c->d_leftover, d_left,
                               c->classify_grid),
               "classify kernel");
        } else {
            CK(launch_classify(a, 0, g.t0, g.t1, c->d_bin_count, c->d_bin_tiles, c->stream), "classify kernel");
        }
        end(k);
        CK(cudaMemcpyAsync(c->d_bin_hist, c->d_bin_count, sizeof(int) * 2 * kNumBins, cudaMemcpyDeviceToDevice,
                           c->stream),
           "bin counts");
        if (!fast || keep_lik) {
            const int rc = bins(kKindFP64, 0);
            if (rc != GSNP_OK) return rc;
        }
        if (fast) {
            const int rc = bins(kKindFast, 0);
            if (rc != GSNP_OK) return rc;
            if (!defer_to_end) {
                const int rd = deferred_pass();
                if (rd != GSNP_OK) return rd;
            }
        }
        /* pass 1: the windows whose likelihood another window kept */
        if (external) {
            const int kc = begin(kKindClassify, 0, 0);
            if (use_stream)
                CK(launch_classify(a, 1, 0, 0, c->d_bin_count, c->d_bin_tiles, c->stream, c->d_leftover, d_left,
                                   c->classify_grid),
                   "classify kernel");
            else
                CK(launch_classify(a, 1, g.t0, g.t1, c->d_bin_count, c->d_bin_tiles, c->stream), "classify kernel");
            end(kc);
            CK(cudaMemcpyAsync(c->d_bin_hist + 2 * kNumBins, c->d_bin_count, sizeof(int) * 2 * kNumBins,
                               cudaMemcpyDeviceToDevice, c->stream),
               "bin counts");
            const int rc = bins(kKindFP64, 1);
            if (rc != GSNP_OK) return rc;
        }
        if (after) {
            const int rc = after(si);
            if (rc != GSNP_OK) return rc;
        }
    }
    if (defer_to_end) return deferred_pass();
    return GSNP_OK;
}

/* After a pass whose deferred sites ran once after its last segment: their
 * final calls into the host copy `out`, whose segments were downloaded with
 * those sites still pending.  The streams that wrote `out` are idle. */
int patch_deferred_calls(gsnp_context* c, gsnp_site_call* out) {
    const int64_t n = std::min<int64_t>((int64_t)c->h_dcount[0], c->dsite_cap);
    if (n <= 0) return GSNP_OK;
    if (n > c->patch_cap) {
        CK(dev_alloc(&c->d_patch, (size_t)n), "cudaMalloc deferred calls");
        c->patch_cap = n;
    }
    const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 1024);
    deferred_calls_kernel<<<blocks, 256, 0, c->stream>>>(c->d_dsites, c->d_out, n, c->d_patch);
    CK(cudaGetLastError(), "deferred calls");
    std::vector<DeferredCall> h((size_t)n);
    CK(cudaMemcpyAsync(h.data(), c->d_patch, (size_t)n * sizeof(DeferredCall), cudaMemcpyDeviceToHost, c->stream),
       "download");
    CK(cudaStreamSynchronize(c->stream), "download");
    SiteCall* o = reinterpret_cast<SiteCall*>(out);
    for (const DeferredCall& d : h) o[d.site] = d.call;
    c->d2h_bytes += (uint64_t)n * sizeof(DeferredCall);
    return GSNP_OK;
}

/* the whole chromosome as one segment (the deposited reads are resident) */
Segment whole_segment(const gsnp_context* c) {
    return Segment{0, (c->chr_len + kTile - 1) / kTile, 0, c->n_dep, 0, kNoRead};
}

/* Window-aligned segments with about the same number of windows each.  The
 * deposited reads of a window are the passing alignments of its run (less the
 * dropped last one), so the run list gives every segment's read ranges. */
std::vector<Segment> plan_segments(const gsnp_context* c, const ReadView& r, int n_seg) {
    const WindowPlan& P = c->plan;
    const int64_t n_tiles = (c->chr_len + kTile - 1) / kTile;
    const int64_t per = (P.n_windows + n_seg - 1) / n_seg;
    std::vector<Segment> segs;
    size_t k = 0;            /* first run at or past the segment's first window */
    int64_t dep = 0;         /* passing alignments of the runs before run k */
    int64_t raw = 0;
    for (int64_t w0 = 0; w0 < P.n_windows; w0 += per) {
        const int64_t w1 = std::min(P.n_windows, w0 + per);
        Segment g;
        g.t0 = std::min(n_tiles, w0 * (int64_t)(kWin / kTile));
        g.t1 = w1 == P.n_windows ? n_tiles : std::min(n_tiles, w1 * (int64_t)(kWin / kTile));
        g.dlo = std::min(dep, P.n_deposited);
        while (k < P.runs.size() && P.runs[k].window < w1) {
            dep += P.runs[k].count;
            ++k;
        }
        raw = k < P.runs.size() ? P.runs[k].first : r.n;
        g.dhi = std::min(dep, P.n_deposited);
        g.raw_hi = raw;
        g.next_pos = g.dhi < P.n_deposited ? (int64_t)r.pos[P.runs[k].first] : kNoRead;
        if (g.t1 > g.t0 || w1 == P.n_windows) segs.push_back(g);
    }
    return segs;
}

/* number of segments of a call: one per two million deposited reads, 1 .. 16
 * (GSNP_SEGMENTS overrides) */
int segment_count(int64_t n_dep, int64_t n_windows) {
    int n = (int)std::min<int64_t>(16, std::max<int64_t>(1, n_dep / 2000000));
    if (const char* e = getenv("GSNP_SEGMENTS")) n = std::max(1, atoi(e));
    return (int)std::max<int64_t>(1, std::min<int64_t>(n, n_windows));
}

/* gsnp_call_chromosome, and with out != NULL the download of every call.
 *   copy stream up:   start/length/hit/strand, then bases and qualities in
 *                     kUploadChunks pieces, an event after each;
 *   host:             the window replay, meanwhile;
 *   compute stream:   the deposited index list once the small arrays are
 *                     there, then per segment the gather of the next
 *                     segment's reads (after the upload pieces that hold
 *                     them) and the calling of this one;
 *   copy stream down: each segment's calls once they are final. */
/* the copy streams and events of a call, made on first use */
int ensure_call_streams(gsnp_context* c) {
    if (c->up_stream) return GSNP_OK;
    CK(cudaStreamCreateWithFlags(&c->up_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    for (int i = 0; i + 1 < c->n_up; ++i)
        CK(cudaStreamCreateWithFlags(&c->up_extra[i], cudaStreamNonBlocking), "cudaStreamCreate");
    CK(cudaStreamCreateWithFlags(&c->down_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    CK(cudaStreamCreateWithFlags(&c->gather_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    CK(cudaEventCreateWithFlags(&c->ev_index, cudaEventDisableTiming), "cudaEventCreate");
    CK(cudaEventCreateWithFlags(&c->ev_small, cudaEventDisableTiming), "cudaEventCreate");
    CK(cudaEventCreateWithFlags(&c->ev_seg, cudaEventDisableTiming), "cudaEventCreate");
    for (int i = 0; i < gsnp_context::kUploadChunks; ++i)
        CK(cudaEventCreateWithFlags(&c->ev_chunk[i], cudaEventDisableTiming), "cudaEventCreate");
    CK(dev_alloc(&c->d_gerror, 1), "cudaMalloc");
    return GSNP_OK;
}

int call_chromosome(gsnp_context* c, const gsnp_reads* r, gsnp_site_call* out) {
    if (!c || !r || r->n < 0 || r->pitch < 0 ||
        (r->n > 0 && (!r->pos || !r->len || !r->hit || !r->strand || (!r->packed && (!r->seq || !r->qual)))))
        return fail(c, GSNP_ERR_ARG, "null read arrays");
    if (r->packed && r->packed_qmin != c->params.q_min)
        return fail(c, GSNP_ERR_ARG, "reads packed with another q_min than the tables'");
    if (!c->have_tables || !c->d_codes) return fail(c, GSNP_ERR_STATE, "tables and reference must be loaded first");
    cudaSetDevice(c->device);
    PhaseTimer timer("gsnp_call_chromosome");
    const int L = c->params.read_length;
    const int64_t n = r->n;
    {
        const int rc = ensure_call_streams(c);
        if (rc != GSNP_OK) return rc;
    }
    c->streamed = false;
    if (!c->d_out || c->out_sites < c->chr_len) {
        /* the resident calls of the chromosome (a streamed call keeps none) */
        CK(dev_alloc(&c->d_out, (size_t)c->chr_len), "cudaMalloc calls");
        c->out_sites = c->chr_len;
    }
    /* the host's window replay on a thread of its own from the start: it
     * reads the caller's arrays while the uploads below are issued */
    ReadView v{r->n, r->pos, r->len, r->hit, r->seq, r->qual, r->pitch, r->packed};
    std::string err;
    const int64_t chr_len = c->chr_len;
    const int qmin = c->params.q_min;
    WindowPlan* plan_out = &c->plan;
    std::future<int> replay = std::async(std::launch::async, [v, chr_len, L, qmin, plan_out, &err]() {
        return replay_windows(v, chr_len, L, qmin, host_threads(), plan_out, &err);
    });
    /* 1. uploads, on their own stream */
    const size_t raw = (size_t)n * r->pitch;
    if (n > c->raw_cap || raw > c->raw_bytes) {
        const int64_t cap = std::max<int64_t>(n, 1);
        CK(dev_alloc(&c->d_raw_pos, (size_t)cap), "cudaMalloc raw");
        CK(dev_alloc(&c->d_raw_len, (size_t)cap), "cudaMalloc raw");
        CK(dev_alloc(&c->d_raw_hit, (size_t)cap), "cudaMalloc raw");
        CK(dev_alloc(&c->d_raw_strand, (size_t)cap), "cudaMalloc raw");
        CK(dev_alloc(&c->d_raw_seq, std::max<size_t>(raw, 1)), "cudaMalloc raw");
        CK(dev_alloc(&c->d_raw_qual, std::max<size_t>(raw, 1)), "cudaMalloc raw");
        CK(dev_alloc(&c->d_idx, (size_t)cap), "cudaMalloc raw");
        c->raw_cap = cap;
        c->raw_bytes = std::max<size_t>(raw, 1);
    }
    const int64_t chunk_rows = std::max<int64_t>(1, (n + gsnp_context::kUploadChunks - 1) / gsnp_context::kUploadChunks);
    GpuTimeline tl(timer.on);
    tl.rec("start", c->up_stream);
    if (n > 0) {
        CK(cudaMemcpyAsync(c->d_raw_pos, r->pos, n * 4, cudaMemcpyHostToDevice, c->up_stream), "upload");
        CK(cudaMemcpyAsync(c->d_raw_len, r->len, n * 4, cudaMemcpyHostToDevice, c->up_stream), "upload");
        CK(cudaMemcpyAsync(c->d_raw_hit, r->hit, n * 4, cudaMemcpyHostToDevice, c->up_stream), "upload");
        CK(cudaMemcpyAsync(c->d_raw_strand, r->strand, n, cudaMemcpyHostToDevice, c->up_stream), "upload");
    }
    CK(cudaEventRecord(c->ev_small, c->up_stream), "event");
    if (c->n_up > 1) {
        /* the other copy streams start after the small arrays' copies */
        for (int i = 0; i + 1 < c->n_up; ++i) CK(cudaStreamWaitEvent(c->up_extra[i], c->ev_small, 0), "wait");
    }
    for (int k = 0; k < gsnp_context::kUploadChunks; ++k) {
        const int64_t b = std::min(n, k * chunk_rows), e = std::min(n, (k + 1) * chunk_rows);
        cudaStream_t us = c->up(k);
        if (e > b) {
            const size_t off = (size_t)b * r->pitch, bytes = (size_t)(e - b) * r->pitch;
            if (r->packed) {
                CK(cudaMemcpyAsync(c->d_raw_seq + off, r->packed + off, bytes, cudaMemcpyHostToDevice, us),
                   "upload packed reads");
            } else {
                CK(cudaMemcpyAsync(c->d_raw_seq + off, r->seq + off, bytes, cudaMemcpyHostToDevice, us), "upload seq");
                CK(cudaMemcpyAsync(c->d_raw_qual + off, r->qual + off, bytes, cudaMemcpyHostToDevice, us),
                   "upload qual");
            }
        }
        CK(cudaEventRecord(c->ev_chunk[k], us), "event");
        if (k == 0 || k == gsnp_context::kUploadChunks / 2 - 1 || k == gsnp_context::kUploadChunks - 1)
            tl.rec("uploaded piece " + std::to_string(k), us);
    }
    timer.mark("uploads issued");
    auto sync_up = [&]() {
        cudaError_t e = cudaStreamSynchronize(c->up_stream);
        for (int i = 0; i + 1 < c->n_up; ++i) {
            const cudaError_t e2 = cudaStreamSynchronize(c->up_extra[i]);
            if (e == cudaSuccess) e = e2;
        }
        return e;
    };
    auto drain = [&]() {
        sync_up();
        if (c->gather_stream) cudaStreamSynchronize(c->gather_stream);
        for (cudaStream_t b : c->bin_stream)
            if (b) cudaStreamSynchronize(b);
        cudaStreamSynchronize(c->stream);
        cudaStreamSynchronize(c->down_stream);
    };
    /* 2. host: the length check and the window replay, started above */
    const int rc = replay.get();
    if (rc != 0) {
        drain();
        return fail(c, rc, err);
    }
    timer.mark("window replay");
    const WindowPlan& P = c->plan;
    const int64_t nd = P.n_deposited;

    /* window tables */
    if (P.n_windows > c->n_win_alloc) {
        CK(dev_alloc(&c->d_win_flags, (size_t)P.n_windows), "cudaMalloc");
        CK(dev_alloc(&c->d_win_lik_src, (size_t)P.n_windows), "cudaMalloc");
        CK(dev_alloc(&c->d_win_host_src, (size_t)P.n_windows), "cudaMalloc");
        c->n_win_alloc = P.n_windows;
    }
    {
        /* through the mapped area: a copy on the copy engine would wait for
         * the alignment uploads queued before it */
        const size_t nw = (size_t)P.n_windows, off_f = kMapWindows, off_l = off_f + ((nw + 15) & ~(size_t)15),
                     off_h = off_l + nw * 4;
        const int rcm = ensure_map(c, off_h + nw * 4);
        if (rcm != GSNP_OK) {
            drain();
            return rcm;
        }
        memcpy(c->h_map + off_f, P.flags.data(), nw);
        memcpy(c->h_map + off_l, P.lik_src.data(), nw * 4);
        memcpy(c->h_map + off_h, P.host_src.data(), nw * 4);
        CK(from_map(c, off_f, c->d_win_flags, nw), "window tables");
        CK(from_map(c, off_l, c->d_win_lik_src, nw * 4), "window tables");
        CK(from_map(c, off_h, c->d_win_host_src, nw * 4), "window tables");
    }
    bool need_counts = false, need_lik = false;
    for (int64_t w = 0; w < P.n_windows; ++w) {
        need_counts |= (P.flags[w] & kWinKeepCounts) != 0;
        need_lik |= (P.flags[w] & kWinKeepLik) != 0;
    }
    if (need_counts && !c->have_counts) {
        CK(dev_alloc(&c->d_counts, (size_t)c->chr_len), "cudaMalloc counts");
        c->have_counts = true;
    }
    if (need_lik && !c->have_lik_keep) {
        CK(dev_alloc(&c->d_lik_keep, (size_t)c->chr_len * 10), "cudaMalloc likelihood");
        c->have_lik_keep = true;
    }
    if (nd > c->cap_dep) {
        CK(dev_alloc(&c->d_pos, (size_t)nd), "cudaMalloc reads");
        CK(dev_alloc(&c->d_lenhit, (size_t)nd), "cudaMalloc reads");
        CK(dev_alloc(&c->d_len, (size_t)nd), "cudaMalloc reads");
        CK(dev_alloc(&c->d_strand, (size_t)nd), "cudaMalloc reads");
        /* 64 elements of slack: the staging bulk copies of the persistent
         * kernel round a row window up to 16 bytes past the last row */
        CK(dev_alloc(&c->d_bq, (size_t)nd * L + 64), "cudaMalloc reads");
        c->cap_dep = nd;
    }
    c->n_dep = nd;
    c->n_gathered = 0;
    c->h2d_bytes = (uint64_t)P.n_windows * 9 + (uint64_t)n * (4 + 4 + 4 + 1) +
                   (r->packed ? 1ULL : 2ULL) * (uint64_t)n * r->pitch;
    c->d2h_bytes = out ? (uint64_t)c->chr_len * sizeof(SiteCall) : 0;

    /* 3. the deposited index list, once the small arrays are on the device */
    CK(cudaMemsetAsync(c->d_gerror, 0, sizeof(int), c->stream), "memset");
    CK(cudaStreamWaitEvent(c->stream, c->ev_small, 0), "wait");
    if (nd > 0) {
        const int64_t n_chunks = (n + kDepChunk - 1) / kDepChunk;
        if (n_chunks > c->dep_chunk_cap) {
            CK(dev_alloc(&c->d_dep_off, (size_t)n_chunks), "cudaMalloc index");
            c->dep_chunk_cap = n_chunks;
        }
        dep_count_kernel<<<(unsigned)n_chunks, kDepThreads, 0, c->stream>>>(n, c->d_raw_pos, c->d_raw_len,
                                                                            c->chr_len, c->d_dep_off);
        dep_scan_kernel<<<1, 1024, 0, c->stream>>>(c->d_dep_off, n_chunks);
        dep_index_kernel<<<(unsigned)n_chunks, kDepThreads, 0, c->stream>>>(n, c->d_raw_pos, c->d_raw_len, c->chr_len,
                                                                            c->d_dep_off, nd, c->d_idx);
        CK(cudaGetLastError(), "index kernels");
    }

    /* 4. segments: gathers on their own stream one segment ahead (segment s
     *    is called once it is gathered), calls, downloads */
    CK(cudaEventRecord(c->ev_index, c->stream), "event");
    CK(cudaStreamWaitEvent(c->gather_stream, c->ev_index, 0), "wait");
    const std::vector<Segment> segs = plan_segments(c, v, segment_count(nd, P.n_windows));
    while (c->ev_gather.size() < segs.size()) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        c->ev_gather.push_back(e);
    }
    const bool vec4 = L % 4 == 0 && r->pitch % 4 == 0 && L <= r->pitch;
    const int per_row = vec4 ? L / 4 : L;
    const int rows_per_block = std::max(1, 256 / per_row);
    int64_t gathered_seg = -1, waited_chunk = -1;
    auto gather_through = [&](int64_t target) -> int {
        while (gathered_seg < target) {
            const Segment& g = segs[(size_t)++gathered_seg];
            if (g.dhi > g.dlo) {
                const int64_t chunk = std::min<int64_t>((g.raw_hi - 1) / chunk_rows, gsnp_context::kUploadChunks - 1);
                /* every piece up to the one holding the segment's last row
                 * (the pieces of several copy streams finish in any order) */
                for (; waited_chunk < chunk; ++waited_chunk)
                    CK(cudaStreamWaitEvent(c->gather_stream, c->ev_chunk[waited_chunk + 1], 0), "wait");
                const int64_t rows = g.dhi - g.dlo;
                const int64_t per_block = (int64_t)rows_per_block * kGatherRows;
                const unsigned blocks = (unsigned)((rows + per_block - 1) / per_block);
                CK(launch_gather(vec4, r->packed != nullptr, blocks, c->gather_stream, g.dlo, g.dhi, c->d_idx, n,
                                 c->d_raw_pos, c->d_raw_len, c->d_raw_hit, c->d_raw_strand, c->d_raw_seq,
                                 c->d_raw_qual, r->pitch, L, rows_per_block, c->d_pos, c->d_lenhit, c->d_len,
                                 c->d_strand, c->d_bq, c->d_gerror, c->params.q_min),
                   "gather kernel");
                CK(cudaGetLastError(), "gather kernel");
            }
            CK(cudaEventRecord(c->ev_gather[(size_t)gathered_seg], c->gather_stream), "event");
            tl.rec("gathered " + std::to_string(gathered_seg), c->gather_stream);
        }
        return GSNP_OK;
    };
    auto before = [&](size_t si) -> int {
        /* segment si's kernels read only its own reads and those before it:
         * its tile ranges end at its last read (tile_bounds_kernel takes the
         * next read's start from the host replay), and the next-site lookup
         * at a window's end takes only reads starting inside the window */
        const int64_t last = (int64_t)segs.size() - 1;
        const int64_t need = (int64_t)si;
        const int rc = gather_through(std::min<int64_t>((int64_t)si + 1, last));
        if (rc != GSNP_OK) return rc;
        CK(cudaStreamWaitEvent(c->stream, c->ev_gather[(size_t)need], 0), "wait");
        c->n_gathered = segs[(size_t)need].dhi;   /* the rows the kernels of si may read */
        tl.rec("calling " + std::to_string(si), c->stream);
        return GSNP_OK;
    };
    auto after = [&](size_t si) -> int {
        tl.rec("called " + std::to_string(si), c->stream);
        if (!out) return GSNP_OK;
        const int64_t s0 = segs[si].t0 * kTile, s1 = std::min(segs[si].t1 * kTile, c->chr_len);
        if (s1 <= s0) return GSNP_OK;
        CK(cudaEventRecord(c->ev_seg, c->stream), "event");
        CK(cudaStreamWaitEvent(c->down_stream, c->ev_seg, 0), "wait");
        CK(cudaMemcpyAsync(out + s0, c->d_out + s0, (size_t)(s1 - s0) * sizeof(SiteCall), cudaMemcpyDeviceToHost,
                           c->down_stream),
           "download");
        tl.rec("downloaded " + std::to_string(si), c->down_stream);
        return GSNP_OK;
    };
    int rc2 = run_calling(c, segs, before, after);
    if (rc2 == kRedoDeferred) {
        /* the deferred pool was too small for the device-driven pass and has
         * been grown: every read is on the device now, so the pass runs
         * again over the whole chromosome, and the calls are downloaded
         * again */
        sync_up();
        cudaStreamSynchronize(c->down_stream);
        cudaStreamSynchronize(c->gather_stream);
        rc2 = run_calling(c, {whole_segment(c)}, nullptr, nullptr);
        if (rc2 == GSNP_OK && out) {
            CK(cudaMemcpyAsync(out, c->d_out, (size_t)c->chr_len * sizeof(SiteCall), cudaMemcpyDeviceToHost,
                               c->stream),
               "download");
            CK(cudaStreamSynchronize(c->stream), "download");
        }
    }
    cudaError_t e_up = sync_up(), e_down = cudaStreamSynchronize(c->down_stream);
    const cudaError_t e_gather = cudaStreamSynchronize(c->gather_stream);
    tl.rec("end", c->down_stream);
    cudaStreamSynchronize(c->down_stream);
    tl.print("gsnp_call_chromosome");
    timer.mark("calling (pipelined)");
    if (rc2 != GSNP_OK) {
        drain();
        return rc2;
    }
    CK(e_up, "upload");
    CK(e_down, "download");
    CK(e_gather, "gather");
    int gerr = 0;
    CK(to_map(c, c->d_gerror, kMapGerror, sizeof(int)), "error flag");
    CK(cudaStreamSynchronize(c->stream), "error flag");
    memcpy(&gerr, c->h_map + kMapGerror, sizeof(int));
    if (gerr == 3) return fail(c, GSNP_ERR_STATE, "deposited alignment list does not match the window replay");
    if (gerr) return fail(c, GSNP_ERR_INPUT, "unknown base when encoding (only ACGT/acgt are accepted)");
    if (out && c->deferred_at_end) return patch_deferred_calls(c, out);
    return GSNP_OK;
}

}  // namespace

extern "C" {

int gsnp_set_option(gsnp_context* c, const char* name, int64_t value) {
    if (!c || !name) return GSNP_ERR_ARG;
    const std::string n(name);
    auto clamp = [](int64_t v, int lo, int hi) { return (int)std::max<int64_t>(lo, std::min<int64_t>(hi, v)); };
    if (n == "persistent") c->stream_path = value != 0;
    else if (n == "persistent_slots") c->stream_slots = value > 48 ? 64 : 48;
    else if (n == "persistent_mode") c->stream_mode = clamp(value, 0, 2);
    else if (n == "persistent_carveout") c->stream_carveout = clamp(value, 0, 100);
    else if (n == "device_driven") c->device_driven = value != 0;
    else if (n == "stream_windows") c->stream_windows = clamp(value, 1, 1 << 20);
    else if (n == "graphs") c->use_graphs = value != 0;
    else if (n == "columns_gpu") c->columns_gpu = value != 0;
    else if (n == "upload_streams") c->n_up = c->up_stream ? c->n_up : clamp(value, 1, gsnp_context::kMaxUpStreams);
    else if (n.rfind("fast_carveout_", 0) == 0 || n.rfind("fp64_carveout_", 0) == 0 || n.rfind("bin_limit_", 0) == 0) {
        const bool lim = n[0] == 'b';
        const int slots = atoi(n.c_str() + (lim ? 10 : 14));
        int b = 0;
        while (b < kNumBins && bin_slots(b) != slots) ++b;
        if (b == kNumBins) return fail(c, GSNP_ERR_ARG, "no depth bin of " + std::to_string(slots) + " slots");
        if (lim) {
            /* a bin takes columns up to its limit: at most its slots, above
             * the previous bin's limit (the deepest bin takes the rest) */
            if (b == kNumBins - 1) return GSNP_OK;
            c->bin_limit[b] = clamp(value, b ? c->bin_limit[b - 1] : 1, slots);
        } else {
            c->bin_carveout[n[1] == 'a' ? 1 : 0][b] = clamp(value, 0, 100);
        }
    } else {
        return fail(c, GSNP_ERR_ARG, "unknown option " + n);
    }
    /* grids and graphs follow the new settings */
    c->grid_L = -1;
    c->stream_ctas_L = -1;
    return GSNP_OK;
}

int gsnp_context_create(int device, gsnp_context** out) {
    if (!out) return GSNP_ERR_ARG;
    *out = nullptr;
    gsnp_context* c = new gsnp_context();
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_error, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_stats, sizeof(unsigned long long) * kNumStats);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_bin_count, sizeof(int) * kBinCountInts);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_dcount, sizeof(unsigned long long) * 2);
    if (e != cudaSuccess) {
        free_all(c);
        delete c;
        return GSNP_ERR_CUDA;
    }
    c->own_stream = true;
    /* options from the environment: GSNP_OPTIONS="name=value,..." (see
     * gsnp_set_option), then GSNP_TUNE_FILE if it names a file of
     * "name value" lines (written by gsnp_tune) */
    auto apply_env = [&](const char* spec) {
        std::string item;
        for (const char* p = spec;; ++p) {
            if (*p == ',' || *p == 0) {
                const size_t eq = item.find('=');
                if (eq != std::string::npos)
                    (void)gsnp_set_option(c, item.substr(0, eq).c_str(), atoll(item.c_str() + eq + 1));
                item.clear();
                if (*p == 0) break;
            } else {
                item += *p;
            }
        }
    };
    if (const char* e = getenv("GSNP_TUNE_FILE")) {
        if (FILE* f = fopen(e, "r")) {
            char name[64];
            long long v = 0;
            while (fscanf(f, "%63s %lld", name, &v) == 2) (void)gsnp_set_option(c, name, v);
            fclose(f);
        }
    }
    if (const char* e = getenv("GSNP_OPTIONS")) apply_env(e);
    *out = c;
    return GSNP_OK;
}

void gsnp_context_destroy(gsnp_context* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    /* every stream finished before any buffer it may use is freed */
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (int i = 0; i < gsnp_context::kBinStreams; ++i)
        if (c->bin_stream[i]) cudaStreamSynchronize(c->bin_stream[i]);
    if (c->gather_stream) cudaStreamSynchronize(c->gather_stream);
    if (c->up_stream) cudaStreamSynchronize(c->up_stream);
    for (cudaStream_t u : c->up_extra)
        if (u) cudaStreamSynchronize(u);
    if (c->down_stream) cudaStreamSynchronize(c->down_stream);
    free_all(c);
    ring_free(c->ring);
    c->ring = nullptr;
    c->colw.reset();
    if (c->h_text) cudaFreeHost(c->h_text);
    for (int i = 0; i < 2 * gsnp_context::kMaxLaunches; ++i)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    for (int i = 0; i < gsnp_context::kUploadChunks; ++i)
        if (c->ev_chunk[i]) cudaEventDestroy(c->ev_chunk[i]);
    if (c->ev_small) cudaEventDestroy(c->ev_small);
    if (c->h_map) cudaFreeHost(c->h_map);
    if (c->ev_seg) cudaEventDestroy(c->ev_seg);
    if (c->ev_index) cudaEventDestroy(c->ev_index);
    for (int i = 0; i < gsnp_context::kBinStreams; ++i) {
        if (c->ev_join[i]) cudaEventDestroy(c->ev_join[i]);
        if (c->bin_stream[i]) {
            cudaStreamSynchronize(c->bin_stream[i]);
            cudaStreamDestroy(c->bin_stream[i]);
        }
    }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->capture_stream) cudaStreamDestroy(c->capture_stream);
    for (cudaEvent_t e : c->ev_gather) cudaEventDestroy(e);
    if (c->gather_stream) {
        cudaStreamSynchronize(c->gather_stream);
        cudaStreamDestroy(c->gather_stream);
    }
    if (c->up_stream) {
        cudaStreamSynchronize(c->up_stream);
        cudaStreamDestroy(c->up_stream);
    }
    for (cudaStream_t u : c->up_extra)
        if (u) cudaStreamDestroy(u);
    if (c->down_stream) {
        cudaStreamSynchronize(c->down_stream);
        cudaStreamDestroy(c->down_stream);
    }
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char* gsnp_context_error(const gsnp_context* c) { return c ? c->error.c_str() : "no context"; }

int gsnp_set_stream(gsnp_context* c, void* stream) {
    if (!c) return GSNP_ERR_ARG;
    if (c->own_stream && c->stream) {
        cudaStreamSynchronize(c->stream);
        cudaStreamDestroy(c->stream);
    }
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
    return GSNP_OK;
}

int gsnp_load_tables(gsnp_context* c, const gsnp_params* p, const double* p_matrix, const double* p_prior,
                     const double* p_rank) {
    if (!c || !p || !p_matrix || !p_prior || !p_rank) return fail(c, GSNP_ERR_ARG, "null argument");
    if (p->read_length <= 0 || p->read_length > 255) return fail(c, GSNP_ERR_ARG, "read_length must be 1..255");
    cudaSetDevice(c->device);
    c->params = *p;
    std::string err;
    if (build_tables(*p, p_matrix, p_prior, &c->tables, &err) != 0) return fail(c, GSNP_ERR_ARG, err);
    const HostTables& t = c->tables;
    CK(dev_alloc(&c->d_lik64, t.lik64.size()), "cudaMalloc");
    CK(dev_alloc(&c->d_lik32, t.lik32.size()), "cudaMalloc");
    CK(dev_alloc(&c->d_qadj, t.qadj.size()), "cudaMalloc");
    CK(dev_alloc(&c->d_p_prior, 128), "cudaMalloc");
    CK(dev_alloc(&c->d_log_prior, 128), "cudaMalloc");
    CK(dev_alloc(&c->d_log_prior32, 96), "cudaMalloc");
    CK(dev_alloc(&c->d_p_rank, 64UL * 64UL * 2048UL), "cudaMalloc");
    CK(cudaMemcpy(c->d_lik64, t.lik64.data(), t.lik64.size() * 8, cudaMemcpyHostToDevice), "upload");
    CK(cudaMemcpy(c->d_lik32, t.lik32.data(), t.lik32.size() * 4, cudaMemcpyHostToDevice), "upload");
    CK(cudaMemcpy(c->d_qadj, t.qadj.data(), t.qadj.size(), cudaMemcpyHostToDevice), "upload");
    CK(cudaMemcpy(c->d_p_prior, p_prior, 128 * 8, cudaMemcpyHostToDevice), "upload");
    CK(cudaMemcpy(c->d_log_prior, t.log_prior.data(), 128 * 8, cudaMemcpyHostToDevice), "upload");
    CK(cudaMemcpy(c->d_log_prior32, t.log_prior32.data(), 96 * 4, cudaMemcpyHostToDevice), "upload");
    CK(cudaMemcpy(c->d_p_rank, p_rank, 64UL * 64UL * 2048UL * 8, cudaMemcpyHostToDevice), "upload");
    c->have_tables = true;
    c->snp_lp_ready = false;
    return GSNP_OK;
}

int gsnp_load_reference(gsnp_context* c, const uint8_t* codes, int64_t length, const gsnp_snp* snp,
                        int64_t n_snp) {
    if (!c || !codes || length <= 0 || (n_snp > 0 && !snp)) return fail(c, GSNP_ERR_ARG, "bad reference");
    if (length > 0x7fffffffLL) return fail(c, GSNP_ERR_CAPACITY, "chromosome longer than 2^31-1");
    cudaSetDevice(c->device);
    c->chr_len = length;
    c->h_codes.assign(codes, codes + length);
    CK(dev_alloc(&c->d_codes, (size_t)length), "cudaMalloc codes");
    CK(cudaMemcpy(c->d_codes, codes, (size_t)length, cudaMemcpyHostToDevice), "upload codes");
    static_assert(sizeof(gsnp_snp) == sizeof(DbSnpEntry), "dbSNP row layout");
    /* the rows are the flagged sites in position order: the kernels find a
     * site's row from the rows before its tile */
    int64_t flagged = 0;
    for (int64_t i = 0; i < length; ++i) flagged += (codes[i] & 8) != 0;
    if (flagged != n_snp) return fail(c, GSNP_ERR_ARG, "dbSNP rows and flagged site codes differ in number");
    const int64_t n_tiles = (length + kTile - 1) / kTile;
    std::vector<int32_t> tile_snp((size_t)n_tiles + 1, 0);
    for (int64_t k = 0; k < n_snp; ++k) {
        const int64_t pos = snp[k].pos;
        if (pos >= length || !(codes[pos] & 8) || (k > 0 && pos <= (int64_t)snp[k - 1].pos))
            return fail(c, GSNP_ERR_ARG, "dbSNP rows must be ascending, unique and on flagged sites");
        tile_snp[(size_t)(pos / kTile) + 1] += 1;
    }
    for (int64_t t = 0; t < n_tiles; ++t) tile_snp[(size_t)t + 1] += tile_snp[(size_t)t];
    CK(dev_alloc(&c->d_tile_snp, (size_t)n_tiles + 1), "cudaMalloc tiles");
    CK(cudaMemcpy(c->d_tile_snp, tile_snp.data(), ((size_t)n_tiles + 1) * 4, cudaMemcpyHostToDevice), "upload");
    c->n_snp = n_snp;
    CK(dev_alloc(&c->d_snp, (size_t)std::max<int64_t>(n_snp, 1)), "cudaMalloc dbsnp");
    if (n_snp > 0) CK(cudaMemcpy(c->d_snp, snp, sizeof(gsnp_snp) * n_snp, cudaMemcpyHostToDevice), "upload dbsnp");
    /* the resident calls are allocated by the first resident call */
    if (c->d_out) cudaFree(c->d_out);
    c->d_out = nullptr;
    c->out_sites = 0;
    c->snp_lp_ready = false;
    c->called = false;
    return GSNP_OK;
}

int gsnp_call_chromosome(gsnp_context* c, const gsnp_reads* r) { return call_chromosome(c, r, nullptr); }

int gsnp_call_chromosome_into(gsnp_context* c, const gsnp_reads* r, gsnp_site_call* out) {
    if (!out) return fail(c, GSNP_ERR_ARG, "null output");
    return call_chromosome(c, r, out);
}

int gsnp_calibrate(gsnp_context* c, const gsnp_params* p, const gsnp_reads* r, double* pm) {
    if (!c || !p || !r || !pm) return fail(c, GSNP_ERR_ARG, "null argument");
    if (r->n < 0 || r->pitch < 0 ||
        (r->n > 0 && (!r->pos || !r->len || !r->hit || !r->strand || (!r->packed && (!r->seq || !r->qual)))))
        return fail(c, GSNP_ERR_ARG, "null read arrays");
    if (r->packed && r->packed_qmin != p->q_min)
        return fail(c, GSNP_ERR_ARG, "reads packed with another q_min than the parameters'");
    if (!c->d_codes) return fail(c, GSNP_ERR_STATE, "reference must be loaded first");
    if (p->read_length <= 0 || p->read_length > 255) return fail(c, GSNP_ERR_ARG, "read_length must be 1..255");
    if (p->q_max < p->q_min) return fail(c, GSNP_ERR_ARG, "q_max below q_min");
    cudaSetDevice(c->device);
    const int L = p->read_length;
    const int nq = p->q_max - p->q_min + 1;
    const size_t nbins = (size_t)nq * L * 16;
    for (int64_t i = 0; i < r->n; ++i)
        if (r->len[i] < 0 || r->len[i] > L || r->len[i] > r->pitch)
            return fail(c, GSNP_ERR_INPUT, "alignment " + std::to_string(i) + " is longer than -L");
    unsigned long long* d_counts = nullptr;
    int32_t *d_pos = nullptr, *d_len = nullptr, *d_hit = nullptr;
    uint8_t *d_strand = nullptr, *d_seq = nullptr, *d_qual = nullptr;
    const size_t raw = (size_t)r->n * r->pitch;
    CallTemps tmp;
    CK(tmp.alloc(&d_counts, nbins * 8), "cudaMalloc");
    CK(tmp.alloc(&d_pos, std::max<int64_t>(r->n, 1) * 4), "cudaMalloc");
    CK(tmp.alloc(&d_len, std::max<int64_t>(r->n, 1) * 4), "cudaMalloc");
    CK(tmp.alloc(&d_hit, std::max<int64_t>(r->n, 1) * 4), "cudaMalloc");
    CK(tmp.alloc(&d_strand, std::max<int64_t>(r->n, 1)), "cudaMalloc");
    CK(tmp.alloc(&d_seq, std::max<size_t>(raw, 1)), "cudaMalloc");
    CK(tmp.alloc(&d_qual, std::max<size_t>(raw, 1)), "cudaMalloc");
    CK(cudaMemsetAsync(d_counts, 0, nbins * 8, c->stream), "memset");
    CK(cudaMemcpyAsync(d_pos, r->pos, r->n * 4, cudaMemcpyHostToDevice, c->stream), "upload");
    CK(cudaMemcpyAsync(d_len, r->len, r->n * 4, cudaMemcpyHostToDevice, c->stream), "upload");
    CK(cudaMemcpyAsync(d_hit, r->hit, r->n * 4, cudaMemcpyHostToDevice, c->stream), "upload");
    CK(cudaMemcpyAsync(d_strand, r->strand, r->n, cudaMemcpyHostToDevice, c->stream), "upload");
    if (r->packed) {
        CK(cudaMemcpyAsync(d_seq, r->packed, raw, cudaMemcpyHostToDevice, c->stream), "upload");
        if (raw > 0) {
            unpack_reads_kernel<<<(unsigned)std::min<size_t>((raw + 255) / 256, 1u << 16), 256, 0, c->stream>>>(
                d_seq, raw, (int)(signed char)p->q_min, d_seq, d_qual);
            CK(cudaGetLastError(), "unpack kernel");
        }
    } else {
        CK(cudaMemcpyAsync(d_seq, r->seq, raw, cudaMemcpyHostToDevice, c->stream), "upload");
        CK(cudaMemcpyAsync(d_qual, r->qual, raw, cudaMemcpyHostToDevice, c->stream), "upload");
    }
    if (r->n > 0) {
        /* the matching bins in shared memory when they fit (41 qualities x
         * 4 bases x 100 cycles: 64 KB), else every bin in global memory */
        const size_t smem = (size_t)nq * 4 * L * 4;
        int dev_smem = 0, n_sm = 0;
        cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
        cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, c->device);
        if (smem <= 160 * 1024 && smem <= (size_t)dev_smem) {
            CK(cudaFuncSetAttribute(calib_count_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "calibration kernel attribute");
            const int per_sm = std::max(1, (int)(200 * 1024 / std::max<size_t>(smem, 1)));
            const int64_t want = (r->n + 15) / 16;
            const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)n_sm * per_sm, want));
            calib_count_smem_kernel<<<blocks, 512, smem, c->stream>>>(
                r->n, d_pos, d_len, d_hit, d_strand, d_seq, d_qual, r->pitch, c->d_codes, c->chr_len,
                (int)(signed char)p->q_min, (int)(signed char)p->q_max, L, d_counts);
        } else {
            const int64_t threads = r->n * 32;
            calib_count_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
                r->n, d_pos, d_len, d_hit, d_strand, d_seq, d_qual, r->pitch, c->d_codes, c->chr_len,
                (int)(signed char)p->q_min, (int)(signed char)p->q_max, L, d_counts);
        }
        CK(cudaGetLastError(), "calibration kernel");
    }
    std::vector<unsigned long long> counts(nbins);
    CK(cudaMemcpyAsync(counts.data(), d_counts, nbins * 8, cudaMemcpyDeviceToHost, c->stream), "download");
    CK(cudaStreamSynchronize(c->stream), "calibration");
    for (size_t i = 0; i < 256UL * 256UL * 16UL; ++i) pm[i] = 1.0;
    calibration_fill(*p, counts.data(), pm);
    return GSNP_OK;
}

int gsnp_prior_table(const gsnp_params* p, double* out) {
    if (!p || !out) return GSNP_ERR_ARG;
    prior_table(*p, p->transition_dominant, p->het_novel, p->althom_novel, out);
    return GSNP_OK;
}

int gsnp_rank_table(double* out) {
    if (!out) return GSNP_ERR_ARG;
    rank_table(out);
    return GSNP_OK;
}

namespace gsnp {

/* everything a captured pass depends on: its arguments (pointers, sizes,
 * parameters), the segment and the launch configuration */
uint64_t graph_key_of(gsnp_context* c, const Segment& g) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t n) {
        const uint8_t* b = static_cast<const uint8_t*>(p);
        for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    };
    const CallArgs a = make_args(c);
    mix(&a, sizeof a);
    mix(&g, sizeof g);
    const int cfg[] = {c->stream_path, c->stream_slots, c->stream_mode, c->stream_carveout, c->stream_ctas,
                       c->deferred_grid, c->classify_grid};
    mix(cfg, sizeof cfg);
    mix(c->bin_grid, sizeof c->bin_grid);
    mix(c->bin_carveout, sizeof c->bin_carveout);
    mix(&c->n_gathered, sizeof c->n_gathered);
    const void* ptrs[] = {c->d_deep, c->d_leftover, c->d_stream_ctl, c->d_dmax, c->d_bin_tiles, c->d_bin_count};
    mix(ptrs, sizeof ptrs);
    return h;
}

/* The resident recall as a CUDA graph: the device-driven pass over the whole
 * chromosome is captured once and replayed while nothing it depends on
 * changes. */
int recall_graph(gsnp_context* c) {
    {
        const int rc = prepare_calling(c);
        if (rc != GSNP_OK) return rc;
    }
    const std::vector<Segment> segs{whole_segment(c)};
    const uint64_t key = graph_key_of(c, segs[0]);
    if (!c->graph_exec || key != c->graph_key) {
        if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
        c->graph_exec = nullptr;
        cudaGraph_t graph = nullptr;
        /* captured on a stream of its own: the caller's stream may be the
         * legacy default stream, which cannot be captured */
        if (!c->capture_stream)
            CK(cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        const cudaStream_t user = c->stream;
        /* the capture waits for nothing the caller queued: the pass reads
         * only what earlier calls left on the device, whose work the last
         * finish_device or call waited for */
        CK(cudaStreamSynchronize(user), "graph capture");
        c->stream = c->capture_stream;
        set_launch_attributes(false);
        const cudaError_t eb = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
        int rc = eb == cudaSuccess ? enqueue_device(c, segs, nullptr, nullptr, false) : GSNP_OK;
        const cudaError_t e = eb == cudaSuccess ? cudaStreamEndCapture(c->stream, &graph) : eb;
        set_launch_attributes(true);
        c->stream = user;
        cudaError_t ei = e;
        if (rc == GSNP_OK && e == cudaSuccess && graph) ei = cudaGraphInstantiate(&c->graph_exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (rc != GSNP_OK || ei != cudaSuccess || !c->graph_exec) {
            /* the pass cannot be captured here: it runs launch by launch,
             * now and from now on */
            (void)cudaGetLastError();
            if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
            c->graph_exec = nullptr;
            c->use_graphs = false;
            c->graph_failed = true;
            return run_calling(c, segs, nullptr, nullptr);
        }
        c->graph_key = key;
    }
    c->n_launches = 1;
    c->launches[0].kind = kKindGraph;
    c->launches[0].slots = 0;
    c->launches[0].tiles = segs[0].t1 - segs[0].t0;
    c->launches[0].sites = c->chr_len;
    c->launches[0].ms = 0.f;
    cudaEventRecord(c->ev[0], c->stream);
    CK(cudaGraphLaunch(c->graph_exec, c->stream), "graph launch");
    cudaEventRecord(c->ev[1], c->stream);
    return finish_device(c);
}

}  // namespace gsnp

namespace gsnp {

/* one tuning measurement: the calling pass over segment g, best of `reps`,
 * device time between events on the context's stream */
float time_pass(gsnp_context* c, const Segment& g, int reps, int* rc) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int r = 0; r < reps && *rc == GSNP_OK; ++r) {
        cudaEventRecord(e0, c->stream);
        *rc = run_calling(c, {g}, nullptr, nullptr);
        if (*rc == kRedoDeferred) *rc = run_calling(c, {g}, nullptr, nullptr);
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return best;
}

}  // namespace gsnp

int gsnp_tune(gsnp_context* c, int sample_windows, char* report, size_t report_cap) {
    if (!c) return GSNP_ERR_ARG;
    if (!c->called || !c->have_tables || c->n_gathered < c->n_dep)
        return fail(c, GSNP_ERR_STATE, "tuning samples the resident reads of a finished call");
    cudaSetDevice(c->device);
    const WindowPlan& P = c->plan;
    const int64_t n_tiles = (c->chr_len + kTile - 1) / kTile;
    const int64_t w0 = P.n_windows / 3, w1 = std::min<int64_t>(P.n_windows, w0 + std::max(1, sample_windows));
    /* tile ranges of every read (cheap), calling of the sample's tiles only */
    const Segment g{std::min(n_tiles, w0 * (kWin / kTile)), std::min(n_tiles, w1 * (kWin / kTile)), 0, c->n_dep, 0,
                    kNoRead};
    std::string rep;
    char line[160];
    int rc = GSNP_OK;
    const bool fast = make_args(c).precision == 1;
    const int kind = fast ? 1 : 0;
    const char* prefix = fast ? "fast_carveout_" : "fp64_carveout_";
    const bool saved_graphs = c->use_graphs;
    c->device_driven = true;
    (void)time_pass(c, g, 1, &rc);   /* warm-up: grids, scratch, tables in cache */

    /* 1. the binned kernels: each bin's carveout, measured per launch */
    c->stream_path = false;
    static const int kCarveouts[] = {0, 58, 72, 86};
    float bin_best[kNumBins];
    int bin_choice[kNumBins];
    for (int b = 0; b < kNumBins; ++b) {
        bin_best[b] = 1e30f;
        bin_choice[b] = c->bin_carveout[kind][b];
    }
    for (int cv : kCarveouts) {
        for (int b = 0; b < kNumBins; ++b) c->bin_carveout[kind][b] = cv;
        c->grid_L = -1;
        float bin_ms[kNumBins] = {};
        for (int r = 0; r < 2 && rc == GSNP_OK; ++r) {
            rc = run_calling(c, {g}, nullptr, nullptr);
            if (rc == kRedoDeferred) rc = run_calling(c, {g}, nullptr, nullptr);
            float this_ms[kNumBins] = {};
            for (int k = 0; k < c->n_launches; ++k)
                if (c->launches[k].kind == (fast ? kKindFast : kKindFP64))
                    for (int b = 0; b < kNumBins; ++b)
                        if (bin_slots(b) == c->launches[k].slots) this_ms[b] += c->launches[k].ms;
            for (int b = 0; b < kNumBins; ++b) bin_ms[b] = r == 0 ? this_ms[b] : std::min(bin_ms[b], this_ms[b]);
        }
        for (int b = 0; b < kNumBins; ++b)
            if (bin_ms[b] < bin_best[b]) {
                bin_best[b] = bin_ms[b];
                bin_choice[b] = cv;
            }
        snprintf(line, sizeof line, "binned carveout %d:", cv);
        rep += line;
        for (int b = 0; b < kNumBins; ++b) {
            snprintf(line, sizeof line, " %d:%.3f", bin_slots(b), bin_ms[b]);
            rep += line;
        }
        rep += " ms\n";
    }
    for (int b = 0; b < kNumBins; ++b) c->bin_carveout[kind][b] = bin_choice[b];
    c->grid_L = -1;

    /* 2. the depth bins' limits of the two shallowest bins */
    static const int kLimits[][2] = {{32, 40}, {30, 40}, {28, 40}, {32, 36}, {30, 38}};
    float best_binned = 1e30f;
    int best_lim = 0;
    const int saved0 = c->bin_limit[0], saved1 = c->bin_limit[1];
    for (int i = 0; i < (int)(sizeof kLimits / sizeof kLimits[0]) && rc == GSNP_OK; ++i) {
        c->bin_limit[0] = kLimits[i][0];
        c->bin_limit[1] = kLimits[i][1];
        const float ms = time_pass(c, g, 2, &rc);
        snprintf(line, sizeof line, "binned limits %d/%d: %.3f ms\n", kLimits[i][0], kLimits[i][1], ms);
        rep += line;
        if (ms < best_binned) {
            best_binned = ms;
            best_lim = i;
        }
    }
    c->bin_limit[0] = rc == GSNP_OK ? kLimits[best_lim][0] : saved0;
    c->bin_limit[1] = rc == GSNP_OK ? kLimits[best_lim][1] : saved1;

    /* 3. the persistent kernel (FP32 form): slots, carveout, read mode */
    float best_pers = 1e30f;
    int best_slots = 48, best_cv = 0, best_mode = 0;
    if (fast) {
        c->stream_path = true;
        for (int slots : {48, 64})
            for (int cv : {0, 72, 86})
                for (int mode : {0, 1}) {
                    if (rc != GSNP_OK) break;
                    c->stream_slots = slots;
                    c->stream_carveout = cv;
                    c->stream_mode = mode;
                    c->stream_ctas_L = -1;
                    const float ms = time_pass(c, g, 2, &rc);
                    snprintf(line, sizeof line, "persistent slots %d carveout %d mode %d: %.3f ms\n", slots, cv, mode,
                             ms);
                    rep += line;
                    if (ms < best_pers) {
                        best_pers = ms;
                        best_slots = slots;
                        best_cv = cv;
                        best_mode = mode;
                    }
                }
        c->stream_slots = best_slots;
        c->stream_carveout = best_cv;
        c->stream_mode = best_mode;
        c->stream_ctas_L = -1;
    }
    c->stream_path = fast && best_pers < best_binned;
    c->use_graphs = saved_graphs;
    if (rc != GSNP_OK) return rc;

    /* the choice, as option lines (gsnp_set_option names) */
    std::string opts;
    snprintf(line, sizeof line, "persistent %d\npersistent_slots %d\npersistent_carveout %d\npersistent_mode %d\n",
             c->stream_path ? 1 : 0, c->stream_slots, c->stream_carveout, c->stream_mode);
    opts += line;
    for (int b = 0; b < kNumBins; ++b) {
        snprintf(line, sizeof line, "%s%d %d\n", prefix, bin_slots(b), c->bin_carveout[kind][b]);
        opts += line;
    }
    snprintf(line, sizeof line, "bin_limit_32 %d\nbin_limit_40 %d\n", c->bin_limit[0], c->bin_limit[1]);
    opts += line;
    snprintf(line, sizeof line, "sample: windows %lld-%lld (%lld tiles); best binned %.3f ms, best persistent %.3f ms\n",
             (long long)w0, (long long)w1, (long long)(g.t1 - g.t0), best_binned, fast ? best_pers : 0.f);
    rep = opts + "# " + line + rep;
    if (const char* path = getenv("GSNP_TUNE_FILE")) {
        if (FILE* f = fopen(path, "w")) {
            fputs(opts.c_str(), f);
            fclose(f);
        }
    }
    if (report && report_cap > 0) {
        const size_t n = std::min(report_cap - 1, rep.size());
        memcpy(report, rep.data(), n);
        report[n] = 0;
    }
    return GSNP_OK;
}

int gsnp_recall_resident(gsnp_context* c) {
    if (!c || !c->have_tables || c->plan.n_windows == 0) return fail(c, GSNP_ERR_STATE, "nothing resident");
    cudaSetDevice(c->device);
    int rc = c->device_driven && c->use_graphs ? recall_graph(c) : run_calling(c, {whole_segment(c)}, nullptr, nullptr);
    /* the deferred pool was grown to what the pass asked for: run it again */
    if (rc == kRedoDeferred) rc = run_calling(c, {whole_segment(c)}, nullptr, nullptr);
    return rc;
}

int gsnp_fetch_sites(gsnp_context* c, int64_t first, int64_t count, gsnp_site_call* out) {
    if (!c || !out || first < 0 || count < 0 || first + count > c->out_sites) return fail(c, GSNP_ERR_ARG, "range");
    if (!c->called) return fail(c, GSNP_ERR_STATE, "no call results");
    cudaSetDevice(c->device);
    static_assert(sizeof(gsnp_site_call) == sizeof(SiteCall), "site call layout");
    CK(cudaMemcpyAsync(out, c->d_out + first, (size_t)count * sizeof(SiteCall), cudaMemcpyDeviceToHost, c->stream),
       "fetch");
    c->d2h_bytes += (uint64_t)count * sizeof(SiteCall);
    CK(cudaStreamSynchronize(c->stream), "fetch");
    return GSNP_OK;
}

int gsnp_last_launches(gsnp_context* c, gsnp_launch_info* out, int* n) {
    if (!c || !n) return GSNP_ERR_ARG;
    const int m = std::min(*n, c->n_launches);
    if (out) memcpy(out, c->launches, sizeof(gsnp_launch_info) * m);
    *n = c->n_launches;
    return GSNP_OK;
}

int gsnp_transfer_bytes(gsnp_context* c, uint64_t* h2d, uint64_t* d2h) {
    if (!c || !h2d || !d2h) return GSNP_ERR_ARG;
    *h2d = c->h2d_bytes;
    *d2h = c->d2h_bytes;
    return GSNP_OK;
}

int gsnp_get_stats(gsnp_context* c, uint64_t* s, int n) {
    if (!c || !s || n < 0) return GSNP_ERR_ARG;
    for (int i = 0; i < n; ++i) s[i] = i < kNumStats ? c->stats[i] : 0;
    return GSNP_OK;
}

}  // extern "C"

/* -C output (columns.cpp) and cns text (emit.cu) */
namespace gsnp {
namespace {

/* the calls (and counts) of the whole chromosome in host memory; the arrays
 * are left uninitialised, since the copies fill every entry (a zero fill of
 * 1.6 GB at 50 Mbp would cost more than the copy) */
int fetch_results(gsnp_context* c, std::unique_ptr<SiteCall[]>* calls, std::unique_ptr<SiteCounts[]>* counts) {
    calls->reset(new SiteCall[(size_t)c->chr_len]);
    CK(cudaMemcpy(calls->get(), c->d_out, (size_t)c->chr_len * sizeof(SiteCall), cudaMemcpyDeviceToHost), "fetch");
    if (c->have_counts) {
        counts->reset(new SiteCounts[(size_t)c->chr_len]);
        CK(cudaMemcpy(counts->get(), c->d_counts, (size_t)c->chr_len * sizeof(SiteCounts), cudaMemcpyDeviceToHost),
           "fetch");
    }
    return GSNP_OK;
}

}  // namespace
}  // namespace gsnp

namespace gsnp {
namespace {

constexpr int64_t kEmitChunk = 16 * (int64_t)kWin;   /* sites per emission step */

/* Emit the cns text chunk by chunk; sink(text, bytes) receives each chunk's
 * text in host memory (pinned).  With sink == nullptr only the total size is
 * computed. */
/* The chromosome name on the device and the text scratch; clears the error
 * flag that emit_finish reads. */
int emit_prepare(gsnp_context* c, const char* chr_name, int* chr_n) {
    const size_t n = strlen(chr_name);
    if (n > 255) return fail(c, GSNP_ERR_ARG, "chromosome name longer than 255 bytes");
    *chr_n = (int)n;
    if (!c->d_chr) CK(cudaMalloc((void**)&c->d_chr, 256), "cudaMalloc");
    CK(cudaMemcpyAsync(c->d_chr, chr_name, n, cudaMemcpyHostToDevice, c->stream), "upload");
    const size_t need = emit_scratch_bytes(std::min<int64_t>(kEmitChunk, c->chr_len));
    if (need > c->emit_bytes) {
        if (c->d_emit) cudaFree(c->d_emit);
        c->d_emit = nullptr;
        c->emit_bytes = 0;
        CK(cudaMalloc(&c->d_emit, need), "cudaMalloc emit");
        c->emit_bytes = need;
    }
    CK(cudaMemsetAsync(c->d_error, 0, sizeof(int), c->stream), "memset");
    return GSNP_OK;
}

/* a cns value outside the formatter's range in any row since emit_prepare */
int emit_finish(gsnp_context* c) {
    int err = 0;
    CK(cudaMemcpyAsync(&err, c->d_error, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "error flag");
    CK(cudaStreamSynchronize(c->stream), "cns text");
    if (err) return fail(c, GSNP_ERR_STATE, "a cns value is outside the text formatter's range");
    return GSNP_OK;
}

/* The cns text of sites [s_begin, s_end), from calls, counts (null: none
 * kept) and host_src indexed by absolute site and window, to sink in pieces
 * of kEmitChunk rows; *total gets the byte count (with write false only the
 * count is made). */
template <class Sink>
int emit_sites(gsnp_context* c, int chr_n, int64_t s_begin, int64_t s_end, const SiteCall* calls,
               const SiteCounts* counts, const int32_t* host_src, uint64_t* total, Sink&& sink, bool write) {
    *total = 0;
    for (int64_t s0 = s_begin; s0 < s_end; s0 += kEmitChunk) {
        EmitArgs e;
        memset(&e, 0, sizeof(e));
        e.calls = calls;
        e.counts = counts;
        e.codes = c->d_codes;
        e.host_src = host_src;
        e.chr = c->d_chr;
        e.chr_n = chr_n;
        e.site0 = s0;
        e.n = std::min<int64_t>(kEmitChunk, s_end - s0);
        e.error = c->d_error;
        uint64_t bytes = 0;
        CK(emit_lengths(e, c->d_emit, c->stream, &bytes), "cns text lengths");
        *total += bytes;
        if (!write) continue;
        if (bytes > c->text_bytes) {
            if (c->d_text) cudaFree(c->d_text);
            c->d_text = nullptr;
            c->text_bytes = 0;
            CK(cudaMalloc((void**)&c->d_text, bytes), "cudaMalloc text");
            c->text_bytes = bytes;
        }
        if (bytes > c->h_text_bytes) {
            if (c->h_text) cudaFreeHost(c->h_text);
            c->h_text = nullptr;
            c->h_text_bytes = 0;
            CK(cudaMallocHost((void**)&c->h_text, bytes), "cudaMallocHost text");
            c->h_text_bytes = bytes;
        }
        e.text = c->d_text;
        CK(emit_text(e, c->stream), "cns text");
        CK(cudaMemcpyAsync(c->h_text, c->d_text, bytes, cudaMemcpyDeviceToHost, c->stream), "download text");
        CK(cudaStreamSynchronize(c->stream), "cns text");
        c->d2h_bytes += bytes;
        if (!sink(c->h_text, bytes)) return fail(c, GSNP_ERR_INPUT, "write failed");
    }
    return GSNP_OK;
}

/* the cns text of the resident calls of the whole chromosome */
template <class Sink>
int emit_cns(gsnp_context* c, const char* chr_name, uint64_t* total, Sink&& sink, bool write) {
    int chr_n = 0;
    int rc = emit_prepare(c, chr_name, &chr_n);
    if (rc != GSNP_OK) return rc;
    rc = emit_sites(c, chr_n, 0, c->chr_len, c->d_out, c->have_counts ? c->d_counts : nullptr, c->d_win_host_src,
                    total, sink, write);
    if (rc != GSNP_OK) return rc;
    return emit_finish(c);
}

/* ------------------------------------------------------------------------ */
/* streamed calls: bounded device memory                                     */
/* ------------------------------------------------------------------------ */

/* One chunk of a streamed call: windows [w0, w1), their sites and tiles, the
 * deposited reads [R0, R1) its tiles reach (those starting in
 * [S0 - L + 1, S1)), the alignments [raw_lo, raw_hi) that hold them, and the
 * start of deposited read R1 (kNoRead past the last). */
struct Chunk {
    int64_t w0, w1, S0, S1, T0, T1, R0, R1, raw_lo, raw_hi, next_pos;
};

/* The chunks of windows_per_chunk windows each, from the window replay.  The
 * deposited reads are the passing alignments in file order (all but the last
 * when the replay dropped it); a chunk's reads start with the passing
 * alignments before its first window that still reach it. */
std::vector<Chunk> plan_chunks(const WindowPlan& P, const ReadView& v, int64_t chr_len, int L,
                               int64_t windows_per_chunk) {
    const int64_t n_tiles = (chr_len + kTile - 1) / kTile;
    const int64_t nw = P.n_windows;
    /* per window boundary w: passing alignments of the runs before it, and
     * the first alignment of the first run at or past it */
    std::vector<int64_t> dep_at((size_t)nw + 1, 0), raw_at((size_t)nw + 1, v.n), pos_at((size_t)nw + 1, kNoRead);
    {
        size_t k = 0;
        int64_t dep = 0;
        for (int64_t w = 0; w <= nw; ++w) {
            while (k < P.runs.size() && P.runs[k].window < w) dep += P.runs[k++].count;
            dep_at[(size_t)w] = dep;
            if (k < P.runs.size()) {
                raw_at[(size_t)w] = P.runs[k].first;
                pos_at[(size_t)w] = v.pos[P.runs[k].first];
            }
        }
    }
    auto passing = [&](int64_t i) { return v.pos[i] >= 0 && (int64_t)v.pos[i] + v.len[i] < chr_len; };
    std::vector<Chunk> out;
    for (int64_t w0 = 0; w0 < nw; w0 += windows_per_chunk) {
        const int64_t w1 = std::min(nw, w0 + windows_per_chunk);
        Chunk ch;
        ch.w0 = w0;
        ch.w1 = w1;
        ch.S0 = w0 * kWin;
        ch.S1 = std::min(chr_len, w1 * kWin);
        ch.T0 = ch.S0 / kTile;
        ch.T1 = w1 == nw ? n_tiles : std::min(n_tiles, w1 * (int64_t)(kWin / kTile));
        ch.R1 = std::min(dep_at[(size_t)w1], P.n_deposited);
        ch.R0 = std::min(dep_at[(size_t)w0], P.n_deposited);
        ch.raw_lo = raw_at[(size_t)w0];
        /* the passing alignments before the chunk that reach its first site */
        int64_t pidx = dep_at[(size_t)w0];
        for (int64_t i = raw_at[(size_t)w0] - 1; i >= 0; --i) {
            if (!passing(i)) continue;
            --pidx;
            if ((int64_t)v.pos[i] < ch.S0 - L + 1) break;
            if (pidx < P.n_deposited) {
                ch.R0 = pidx;
                ch.raw_lo = i;
            }
        }
        if (ch.R0 > ch.R1) ch.R0 = ch.R1;
        ch.raw_hi = std::max(ch.raw_lo, raw_at[(size_t)w1]);
        ch.next_pos = ch.R1 < P.n_deposited ? (int64_t)pos_at[(size_t)w1] : kNoRead;
        out.push_back(ch);
    }
    return out;
}

}  // namespace

/* Device buffers of a streamed call.  Two slots, each with one chunk's
 * alignments as uploaded, their deposited index, the deposited reads packed,
 * the chunk's calls and window tables; one store of counts and one of
 * likelihoods for the chunk being called (its windows and the carried
 * window), and the carried window's counts and likelihood between chunks.
 * Sized by the largest chunk, not by the chromosome. */
struct StreamRing {
    struct Slot {
        int32_t* raw_pos = nullptr;
        int32_t* raw_len = nullptr;
        int32_t* raw_hit = nullptr;
        uint8_t* raw_strand = nullptr;
        uint8_t* raw_seq = nullptr;
        uint8_t* raw_qual = nullptr;
        int64_t* idx = nullptr;
        int64_t* dep_off = nullptr;
        int32_t* pos = nullptr;
        int32_t* lenhit = nullptr;
        int32_t* len = nullptr;
        uint8_t* strand = nullptr;
        uint16_t* bq = nullptr;
        SiteCall* out = nullptr;
        uint8_t* win_flags = nullptr;
        int32_t* win_lik_src = nullptr;
        int32_t* win_host_src = nullptr;
        /* the window tables staged on the host (pinned) */
        uint8_t* h_tab = nullptr;
        cudaEvent_t uploaded = nullptr, free = nullptr;
    } slot[2];
    int64_t raw_rows = 0, raw_bytes = 0, dep_rows = 0, sites = 0, windows = 0, dep_chunks = 0;
    int L = 0;
    SiteCounts* counts = nullptr;
    SiteCounts* carry_counts = nullptr;
    double* lik = nullptr;
    double* carry_lik = nullptr;
    size_t bytes = 0;   /* device bytes held */
};

void ring_free(StreamRing* g) {
    if (!g) return;
    for (auto& s : g->slot) {
        void* p[] = {s.raw_pos, s.raw_len, s.raw_hit, s.raw_strand, s.raw_seq, s.raw_qual, s.idx, s.dep_off,
                     s.pos, s.lenhit, s.len, s.strand, s.bq, s.out, s.win_flags, s.win_lik_src, s.win_host_src};
        for (void* q : p)
            if (q) cudaFree(q);
        if (s.h_tab) cudaFreeHost(s.h_tab);
        if (s.uploaded) cudaEventDestroy(s.uploaded);
        if (s.free) cudaEventDestroy(s.free);
        s = StreamRing::Slot();
    }
    void* p[] = {g->counts, g->carry_counts, g->lik, g->carry_lik};
    for (void* q : p)
        if (q) cudaFree(q);
    delete g;
}

namespace {

/* bytes of one window-table staging area of w windows */
size_t tab_bytes(int64_t w) { return (size_t)(((w + 15) & ~(int64_t)15) + 8 * w); }

/* the ring's buffers for chunks of up to the given sizes (grown, never shrunk) */
int ring_ensure(gsnp_context* c, StreamRing* g, int64_t raw_rows, int64_t raw_bytes, int64_t dep_rows,
                int64_t sites, int64_t windows, bool counts, bool lik) {
    const int L = c->params.read_length;
    const int64_t dep_chunks = (raw_rows + kDepChunk - 1) / kDepChunk;
    if (raw_rows > g->raw_rows || raw_bytes > g->raw_bytes || dep_rows > g->dep_rows || sites > g->sites ||
        windows > g->windows || L != g->L) {
        const int64_t rr = std::max(raw_rows, g->raw_rows), rb = std::max(raw_bytes, g->raw_bytes);
        const int64_t dr = std::max(dep_rows, g->dep_rows), ns = std::max(sites, g->sites);
        const int64_t nw = std::max(windows, g->windows), dc = std::max<int64_t>(1, (rr + kDepChunk - 1) / kDepChunk);
        for (auto& s : g->slot) {
            void* p[] = {s.raw_pos, s.raw_len, s.raw_hit, s.raw_strand, s.raw_seq, s.raw_qual, s.idx, s.dep_off,
                         s.pos, s.lenhit, s.len, s.strand, s.bq, s.out, s.win_flags, s.win_lik_src, s.win_host_src};
            for (void* q : p)
                if (q) cudaFree(q);
            if (s.h_tab) cudaFreeHost(s.h_tab);
            const cudaEvent_t up = s.uploaded, fr = s.free;
            s = StreamRing::Slot();
            s.uploaded = up;
            s.free = fr;
            const int64_t r1 = std::max<int64_t>(rr, 1), d1 = std::max<int64_t>(dr, 1);
            CK(dev_alloc(&s.raw_pos, (size_t)r1), "cudaMalloc stream ring");
            CK(dev_alloc(&s.raw_len, (size_t)r1), "cudaMalloc stream ring");
            CK(dev_alloc(&s.raw_hit, (size_t)r1), "cudaMalloc stream ring");
            CK(dev_alloc(&s.raw_strand, (size_t)r1), "cudaMalloc stream ring");
            CK(dev_alloc(&s.raw_seq, (size_t)std::max<int64_t>(rb, 1)), "cudaMalloc stream ring");
            CK(dev_alloc(&s.raw_qual, (size_t)std::max<int64_t>(rb, 1)), "cudaMalloc stream ring");
            CK(dev_alloc(&s.idx, (size_t)r1), "cudaMalloc stream ring");
            CK(dev_alloc(&s.dep_off, (size_t)dc), "cudaMalloc stream ring");
            CK(dev_alloc(&s.pos, (size_t)d1), "cudaMalloc stream ring");
            CK(dev_alloc(&s.lenhit, (size_t)d1), "cudaMalloc stream ring");
            CK(dev_alloc(&s.len, (size_t)d1), "cudaMalloc stream ring");
            CK(dev_alloc(&s.strand, (size_t)d1), "cudaMalloc stream ring");
            /* slack as for the resident rows (the persistent kernel's staging copies) */
            CK(dev_alloc(&s.bq, (size_t)d1 * L + 64), "cudaMalloc stream ring");
            CK(dev_alloc(&s.out, (size_t)std::max<int64_t>(ns, 1)), "cudaMalloc stream ring");
            CK(dev_alloc(&s.win_flags, (size_t)nw), "cudaMalloc stream ring");
            CK(dev_alloc(&s.win_lik_src, (size_t)nw), "cudaMalloc stream ring");
            CK(dev_alloc(&s.win_host_src, (size_t)nw), "cudaMalloc stream ring");
            CK(cudaMallocHost((void**)&s.h_tab, tab_bytes(nw)), "cudaMallocHost stream ring");
        }
        g->raw_rows = rr;
        g->raw_bytes = rb;
        g->dep_rows = dr;
        g->sites = ns;
        g->windows = nw;
        g->dep_chunks = dc;
        g->L = L;
        if (g->counts) {
            cudaFree(g->counts);
            g->counts = nullptr;
        }
        if (g->lik) {
            cudaFree(g->lik);
            g->lik = nullptr;
        }
    }
    (void)dep_chunks;
    for (auto& s : g->slot) {
        if (!s.uploaded) CK(cudaEventCreateWithFlags(&s.uploaded, cudaEventDisableTiming), "cudaEventCreate");
        if (!s.free) CK(cudaEventCreateWithFlags(&s.free, cudaEventDisableTiming), "cudaEventCreate");
    }
    if (counts && !g->counts) {
        CK(dev_alloc(&g->counts, (size_t)g->windows * kWin), "cudaMalloc stream counts");
        if (!g->carry_counts) CK(dev_alloc(&g->carry_counts, (size_t)kWin), "cudaMalloc stream counts");
    }
    if (lik && !g->lik) {
        CK(dev_alloc(&g->lik, (size_t)g->windows * kWin * 10), "cudaMalloc stream likelihood");
        if (!g->carry_lik) CK(dev_alloc(&g->carry_lik, (size_t)kWin * 10), "cudaMalloc stream likelihood");
    }
    const int64_t rr = g->raw_rows, dr = g->dep_rows;
    g->bytes = 2 * ((size_t)rr * (4 + 4 + 4 + 1 + 8) + 2 * (size_t)g->raw_bytes + (size_t)g->dep_chunks * 8 +
                    (size_t)dr * (4 + 4 + 4 + 1 + 2 * (size_t)L) + (size_t)g->sites * sizeof(SiteCall) +
                    (size_t)g->windows * 9) +
               (g->counts ? (size_t)(g->windows + 1) * kWin * sizeof(SiteCounts) : 0) +
               (g->lik ? (size_t)(g->windows + 1) * kWin * 80 : 0);
    return GSNP_OK;
}

/* gsnp_call_streamed: the chromosome in chunks of c->stream_windows windows,
 * with device memory bounded by the largest chunk (StreamRing) instead of the
 * chromosome.
 *   copy stream up:    chunk k + 1's alignments into the other ring slot
 *                      while chunk k is called;
 *   compute stream:    per chunk its deposited index and packed reads, the
 *                      calling pass over its tiles (make_args points the
 *                      kernels at the slot through c->view), then its cns
 *                      text and -C windows;
 *   copy stream down:  the chunk's calls into out.
 * Windows that show an earlier window's counts, or use its likelihood
 * (gap windows), reach back at most to the last window before their chunk
 * that had reads; that window is carried from chunk to chunk. */
int call_streamed(gsnp_context* c, const gsnp_reads* r, const char* chr_name, gsnp_site_call* out,
                  const char* cns_path, const char* columns_base) {
    if (!c || !r || r->n < 0 || r->pitch < 0 ||
        (r->n > 0 && (!r->pos || !r->len || !r->hit || !r->strand || (!r->packed && (!r->seq || !r->qual)))))
        return fail(c, GSNP_ERR_ARG, "null read arrays");
    if (r->packed && r->packed_qmin != c->params.q_min)
        return fail(c, GSNP_ERR_ARG, "reads packed with another q_min than the tables'");
    if ((cns_path || columns_base) && !chr_name) return fail(c, GSNP_ERR_ARG, "the outputs need the chromosome name");
    if (!c->have_tables || !c->d_codes) return fail(c, GSNP_ERR_STATE, "tables and reference must be loaded first");
    cudaSetDevice(c->device);
    PhaseTimer timer("gsnp_call_streamed");
    {
        const int rc = ensure_call_streams(c);
        if (rc != GSNP_OK) return rc;
    }
    const int L = c->params.read_length;
    c->called = false;
    c->streamed = false;
    ReadView v{r->n, r->pos, r->len, r->hit, r->seq, r->qual, r->pitch, r->packed};
    std::string err;
    {
        const int rc = replay_windows(v, c->chr_len, L, c->params.q_min, host_threads(), &c->plan, &err);
        if (rc != 0) return fail(c, rc, err);
    }
    const WindowPlan& P = c->plan;
    const int64_t W = std::max<int64_t>(1, c->stream_windows);
    const std::vector<Chunk> chunks = plan_chunks(P, v, c->chr_len, L, W);
    timer.mark("window replay");

    /* the ring's sizes, and the carried window of every chunk */
    int64_t raw_rows = 0, dep_rows = 0, sites = 0, tiles = 0;
    bool need_counts = false, need_lik = false;
    for (int64_t w = 0; w < P.n_windows; ++w) {
        need_counts |= (P.flags[w] & kWinKeepCounts) != 0;
        need_lik |= (P.flags[w] & kWinKeepLik) != 0;
    }
    const size_t nk = chunks.size();
    std::vector<int64_t> carry_c(nk, -1), carry_l(nk, -1), save_c(nk, -1), save_l(nk, -1);
    for (size_t k = 0; k < nk; ++k) {
        const Chunk& ch = chunks[k];
        raw_rows = std::max(raw_rows, ch.raw_hi - ch.raw_lo);
        dep_rows = std::max(dep_rows, ch.R1 - ch.R0);
        sites = std::max(sites, ch.S1 - ch.S0);
        tiles = std::max(tiles, ch.T1 - ch.T0);
        for (int64_t w = ch.w0; w < ch.w1; ++w) {
            const int32_t hs = P.host_src[w], ls = P.lik_src[w];
            if (hs >= 0 && hs < ch.w0) {
                if (carry_c[k] >= 0 && carry_c[k] != hs) return fail(c, GSNP_ERR_STATE, "streamed call: two carried count windows");
                carry_c[k] = hs;
            }
            if ((P.flags[w] & kWinExternalLik) && ls >= 0 && ls < ch.w0) {
                if (carry_l[k] >= 0 && carry_l[k] != ls) return fail(c, GSNP_ERR_STATE, "streamed call: two carried likelihood windows");
                carry_l[k] = ls;
            }
        }
    }
    /* a chunk saves the window a later chunk carries, if it is one of its own;
     * the carried windows never decrease, so one buffer holds each until its
     * last use (checked here) */
    {
        int64_t held_c = -1, held_l = -1;
        for (size_t k = 0; k < nk; ++k) {
            if (carry_c[k] >= 0 && carry_c[k] != held_c) return fail(c, GSNP_ERR_STATE, "streamed call: carried counts lost");
            if (carry_l[k] >= 0 && carry_l[k] != held_l) return fail(c, GSNP_ERR_STATE, "streamed call: carried likelihood lost");
            for (size_t j = k + 1; j < nk; ++j) {
                if (carry_c[j] >= chunks[k].w0 && carry_c[j] < chunks[k].w1) save_c[k] = carry_c[j];
                if (carry_l[j] >= chunks[k].w0 && carry_l[j] < chunks[k].w1) save_l[k] = carry_l[j];
            }
            if (save_c[k] >= 0) held_c = save_c[k];
            if (save_l[k] >= 0) held_l = save_l[k];
        }
    }
    if (!c->ring) c->ring = new StreamRing();
    StreamRing* g = c->ring;
    {
        const int rc = ring_ensure(c, g, raw_rows, raw_rows * r->pitch, dep_rows, sites, W + 1, need_counts, need_lik);
        if (rc != GSNP_OK) return rc;
    }
    c->view = gsnp_context::ChunkView();
    c->view.tiles_need = std::max<int64_t>(tiles, 1);
    timer.mark("ring");

    /* outputs */
    FILE* cns = nullptr;
    int chr_n = 0;
    if (cns_path) {
        cns = fopen(cns_path, "wb");
        if (!cns) return fail(c, GSNP_ERR_INPUT, std::string("cannot create ") + cns_path);
        const int rc = emit_prepare(c, chr_name, &chr_n);
        if (rc != GSNP_OK) {
            fclose(cns);
            return rc;
        }
    }
    if (columns_base) {
        if (!c->colw) c->colw.reset(new ColumnsGpuWriter());
        if (!c->sms) CK(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device), "device attribute");
        if (c->colw->open(P, chr_name, columns_base, std::min<int64_t>(W, c->sms), &err) != 0) {
            if (cns) fclose(cns);
            return fail(c, GSNP_ERR_INPUT, err);
        }
    }
    int rc = GSNP_OK;
    auto close_outputs = [&]() {
        std::string e2;
        if (cns && fclose(cns) != 0 && rc == GSNP_OK) rc = fail(c, GSNP_ERR_INPUT, "write failed");
        cns = nullptr;
        if (columns_base && c->colw->close(&e2) != 0 && rc == GSNP_OK) rc = fail(c, GSNP_ERR_INPUT, e2);
    };
    auto drain = [&]() {
        cudaStreamSynchronize(c->up_stream);
        cudaStreamSynchronize(c->stream);
        cudaStreamSynchronize(c->down_stream);
        c->view.on = false;
    };

    CK(cudaMemsetAsync(c->d_gerror, 0, sizeof(int), c->stream), "memset");
    c->h2d_bytes = (uint64_t)nk * tab_bytes(W + 1);
    c->d2h_bytes = 0;
    /* chunk k's alignments into slot k & 1, once that slot's last chunk is done */
    auto upload = [&](size_t k) -> int {
        const Chunk& ch = chunks[k];
        StreamRing::Slot& s = g->slot[k & 1];
        CK(cudaStreamWaitEvent(c->up_stream, s.free, 0), "wait");
        const int64_t n = ch.raw_hi - ch.raw_lo, b = ch.raw_lo;
        if (n > 0) {
            CK(cudaMemcpyAsync(s.raw_pos, r->pos + b, n * 4, cudaMemcpyHostToDevice, c->up_stream), "upload");
            CK(cudaMemcpyAsync(s.raw_len, r->len + b, n * 4, cudaMemcpyHostToDevice, c->up_stream), "upload");
            CK(cudaMemcpyAsync(s.raw_hit, r->hit + b, n * 4, cudaMemcpyHostToDevice, c->up_stream), "upload");
            CK(cudaMemcpyAsync(s.raw_strand, r->strand + b, n, cudaMemcpyHostToDevice, c->up_stream), "upload");
            const size_t off = (size_t)b * r->pitch, bytes = (size_t)n * r->pitch;
            if (r->packed) {
                CK(cudaMemcpyAsync(s.raw_seq, r->packed + off, bytes, cudaMemcpyHostToDevice, c->up_stream),
                   "upload packed reads");
            } else {
                CK(cudaMemcpyAsync(s.raw_seq, r->seq + off, bytes, cudaMemcpyHostToDevice, c->up_stream), "upload seq");
                CK(cudaMemcpyAsync(s.raw_qual, r->qual + off, bytes, cudaMemcpyHostToDevice, c->up_stream),
                   "upload qual");
            }
            c->h2d_bytes += (uint64_t)n * (13 + (r->packed ? 1 : 2) * (uint64_t)r->pitch);
        }
        CK(cudaEventRecord(s.uploaded, c->up_stream), "event");
        return GSNP_OK;
    };
    for (auto& s : g->slot) CK(cudaEventRecord(s.free, c->stream), "event");
    if (nk > 0) rc = upload(0);
    uint64_t totals[kNumStats] = {};
    const bool vec4 = L % 4 == 0 && r->pitch % 4 == 0 && L <= r->pitch;
    const int per_row = vec4 ? L / 4 : L;
    const int rows_per_block = std::max(1, 256 / per_row);
    for (size_t k = 0; k < nk && rc == GSNP_OK; ++k) {
        if (k + 1 < nk) {
            rc = upload(k + 1);
            if (rc != GSNP_OK) break;
        }
        const Chunk& ch = chunks[k];
        StreamRing::Slot& s = g->slot[k & 1];
        const int64_t nd = ch.R1 - ch.R0, nraw = ch.raw_hi - ch.raw_lo, nwt = ch.w1 - ch.w0 + 1;
        /* window tables of windows [w0 - 1, w1): references before the chunk
         * go to the carried window, entry 0 */
        uint8_t* tf = s.h_tab;
        int32_t* tl = reinterpret_cast<int32_t*>(s.h_tab + ((nwt + 15) & ~(int64_t)15));
        int32_t* th = tl + nwt;
        tf[0] = 0;
        tl[0] = -1;
        th[0] = -1;
        for (int64_t w = ch.w0; w < ch.w1; ++w) {
            const int64_t i = w - ch.w0 + 1;
            const int32_t hs = P.host_src[w], ls = P.lik_src[w];
            tf[i] = P.flags[w];
            tl[i] = ls >= 0 && ls < ch.w0 ? (int32_t)(ch.w0 - 1) : ls;
            th[i] = hs >= 0 && hs < ch.w0 ? (int32_t)(ch.w0 - 1) : hs;
        }
        CK(cudaMemcpyAsync(s.win_flags, tf, nwt, cudaMemcpyHostToDevice, c->stream), "window tables");
        CK(cudaMemcpyAsync(s.win_lik_src, tl, nwt * 4, cudaMemcpyHostToDevice, c->stream), "window tables");
        CK(cudaMemcpyAsync(s.win_host_src, th, nwt * 4, cudaMemcpyHostToDevice, c->stream), "window tables");
        /* the chunk's deposited index and packed reads */
        CK(cudaStreamWaitEvent(c->stream, s.uploaded, 0), "wait");
        if (nd > 0) {
            const int64_t n_chunks = (nraw + kDepChunk - 1) / kDepChunk;
            dep_count_kernel<<<(unsigned)n_chunks, kDepThreads, 0, c->stream>>>(nraw, s.raw_pos, s.raw_len, c->chr_len,
                                                                                s.dep_off);
            dep_scan_kernel<<<1, 1024, 0, c->stream>>>(s.dep_off, n_chunks);
            dep_index_kernel<<<(unsigned)n_chunks, kDepThreads, 0, c->stream>>>(nraw, s.raw_pos, s.raw_len,
                                                                                c->chr_len, s.dep_off, nd, s.idx);
            CK(cudaGetLastError(), "index kernels");
            const int64_t per_block = (int64_t)rows_per_block * kGatherRows;
            const unsigned blocks = (unsigned)((nd + per_block - 1) / per_block);
            CK(launch_gather(vec4, r->packed != nullptr, blocks, c->stream, 0, nd, s.idx, nraw, s.raw_pos, s.raw_len,
                             s.raw_hit, s.raw_strand, s.raw_seq, s.raw_qual, r->pitch, L, rows_per_block, s.pos,
                             s.lenhit, s.len, s.strand, s.bq, c->d_gerror, c->params.q_min),
               "gather kernel");
        }
        if (carry_c[k] >= 0) CK(cudaMemcpyAsync(g->counts, g->carry_counts, sizeof(SiteCounts) * kWin,
                                                cudaMemcpyDeviceToDevice, c->stream), "carried counts");
        if (carry_l[k] >= 0) CK(cudaMemcpyAsync(g->lik, g->carry_lik, sizeof(double) * kWin * 10,
                                                cudaMemcpyDeviceToDevice, c->stream), "carried likelihood");
        /* the calling pass over the chunk */
        gsnp_context::ChunkView& vw = c->view;
        vw.on = true;
        vw.w0 = ch.w0;
        vw.S0 = ch.S0;
        vw.T0 = ch.T0;
        vw.T1 = ch.T1;
        vw.R0 = ch.R0;
        vw.R1 = ch.R1;
        vw.pos = s.pos;
        vw.lenhit = s.lenhit;
        vw.strand = s.strand;
        vw.bq = s.bq;
        vw.out = s.out;
        vw.counts = g->counts;
        vw.lik_keep = g->lik;
        vw.win_flags = s.win_flags;
        vw.win_lik_src = s.win_lik_src;
        vw.win_host_src = s.win_host_src;
        c->n_gathered = ch.R1;
        const std::vector<Segment> seg{Segment{ch.T0, ch.T1, ch.R0, ch.R1, ch.raw_hi, ch.next_pos}};
        rc = run_calling(c, seg, nullptr, nullptr);
        if (rc == kRedoDeferred) rc = run_calling(c, seg, nullptr, nullptr);   /* the deferred pool was grown */
        if (rc != GSNP_OK) break;
        for (int i = 1; i < kNumStats; ++i)
            totals[i] = i == 3 ? std::max(totals[i], c->stats[i]) : totals[i] + c->stats[i];
        /* windows a later chunk carries */
        if (save_c[k] >= 0)
            CK(cudaMemcpyAsync(g->carry_counts, g->counts + (save_c[k] - ch.w0 + 1) * kWin, sizeof(SiteCounts) * kWin,
                               cudaMemcpyDeviceToDevice, c->stream), "carried counts");
        if (save_l[k] >= 0)
            CK(cudaMemcpyAsync(g->carry_lik, g->lik + (save_l[k] - ch.w0 + 1) * kWin * 10, sizeof(double) * kWin * 10,
                               cudaMemcpyDeviceToDevice, c->stream), "carried likelihood");
        /* outputs */
        const SiteCall* calls = based(s.out, ch.S0);
        const SiteCounts* cnt = g->counts ? based(g->counts, (ch.w0 - 1) * kWin) : nullptr;
        if (cns) {
            uint64_t bytes = 0;
            rc = emit_sites(c, chr_n, ch.S0, ch.S1, calls, cnt, based(s.win_host_src, ch.w0 - 1), &bytes,
                            [&](const char* t, uint64_t n) { return fwrite(t, 1, n, cns) == n; }, true);
            if (rc != GSNP_OK) break;
        }
        if (columns_base) {
            ColumnsGpuStats st;
            if (c->colw->write(ch.w0, ch.w1, c->d_codes, calls, cnt, based(s.win_host_src, ch.w0 - 1),
                               based(th, ch.w0 - 1), c->h_codes.data(), c->stream, &st, &err) != 0) {
                rc = fail(c, GSNP_ERR_INPUT, err);
                break;
            }
            c->columns_host_windows += st.host_windows;
        }
        if (out) {
            CK(cudaEventRecord(c->ev_seg, c->stream), "event");
            CK(cudaStreamWaitEvent(c->down_stream, c->ev_seg, 0), "wait");
            CK(cudaMemcpyAsync(out + ch.S0, s.out, (size_t)(ch.S1 - ch.S0) * sizeof(SiteCall), cudaMemcpyDeviceToHost,
                               c->down_stream),
               "download");
            c->d2h_bytes += (uint64_t)(ch.S1 - ch.S0) * sizeof(SiteCall);
            CK(cudaEventRecord(s.free, c->down_stream), "event");
        } else {
            CK(cudaEventRecord(s.free, c->stream), "event");
        }
    }
    drain();
    if (cns && rc == GSNP_OK) rc = emit_finish(c);
    close_outputs();
    timer.mark("chunks");
    if (rc != GSNP_OK) return rc;
    int gerr = 0;
    CK(to_map(c, c->d_gerror, kMapGerror, sizeof(int)), "error flag");
    CK(cudaStreamSynchronize(c->stream), "error flag");
    memcpy(&gerr, c->h_map + kMapGerror, sizeof(int));
    if (gerr == 3) return fail(c, GSNP_ERR_STATE, "deposited alignment list does not match the window replay");
    if (gerr) return fail(c, GSNP_ERR_INPUT, "unknown base when encoding (only ACGT/acgt are accepted)");
    totals[0] = (uint64_t)c->chr_len;
    memcpy(c->stats, totals, sizeof(totals));
    c->streamed = true;
    return GSNP_OK;
}

}  // namespace
}  // namespace gsnp

extern "C" int gsnp_format_cns(gsnp_context* c, const char* chr_name, char* buf, int64_t* size) {
    if (!c || !chr_name || !size) return fail(c, GSNP_ERR_ARG, "null argument");
    if (!c->called) return fail(c, GSNP_ERR_STATE, "no call results");
    cudaSetDevice(c->device);
    uint64_t total = 0;
    if (!buf) {
        const int rc = emit_cns(c, chr_name, &total, [](const char*, uint64_t) { return true; }, false);
        if (rc == GSNP_OK) *size = (int64_t)total;
        return rc;
    }
    const int64_t cap = *size;
    int64_t at = 0;
    const int rc = emit_cns(c, chr_name, &total, [&](const char* t, uint64_t n) {
        const int64_t k = std::min<int64_t>((int64_t)n, cap - at);
        if (k > 0) memcpy(buf + at, t, (size_t)k);
        at += std::max<int64_t>(k, 0);
        return true;
    }, true);
    if (rc == GSNP_OK) *size = at;
    return rc;
}

extern "C" int gsnp_write_cns(gsnp_context* c, const char* chr_name, const char* path) {
    if (!c || !chr_name || !path) return fail(c, GSNP_ERR_ARG, "null argument");
    if (!c->called) return fail(c, GSNP_ERR_STATE, "no call results");
    cudaSetDevice(c->device);
    FILE* f = fopen(path, "wb");
    if (!f) return fail(c, GSNP_ERR_INPUT, std::string("cannot create ") + path);
    uint64_t total = 0;
    const int rc = emit_cns(c, chr_name, &total, [&](const char* t, uint64_t n) {
        return fwrite(t, 1, n, f) == n;
    }, true);
    if (fclose(f) != 0 && rc == GSNP_OK) return fail(c, GSNP_ERR_INPUT, "write failed");
    return rc;
}

extern "C" int gsnp_write_columns(gsnp_context* c, const char* chr_name, const char* base_path) {
    if (!c || !base_path) return fail(c, GSNP_ERR_ARG, "null argument");
    cudaSetDevice(c->device);
    std::unique_ptr<SiteCall[]> calls;
    std::unique_ptr<SiteCounts[]> counts;
    std::string err;
    HostDictCodec dict;
    if (!chr_name) {
        /* text-mode companion files */
        WindowPlan none;
        if (write_columns(none, nullptr, nullptr, nullptr, "", base_path, dict, 1, &err) != 0)
            return fail(c, GSNP_ERR_INPUT, err);
        return GSNP_OK;
    }
    if (!c->called) return fail(c, GSNP_ERR_STATE, "no call results");
    if (c->columns_gpu) {
        /* the windows encoded on the device, from the resident calls */
        ColumnsGpuStats st;
        if (!c->colw) c->colw.reset(new ColumnsGpuWriter());
        if (!c->sms) CK(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device), "device attribute");
        const int64_t nwin = c->plan.n_windows;
        int rc = c->colw->open(c->plan, chr_name, base_path, std::min<int64_t>(nwin, c->sms), &err);
        if (rc == 0)
            rc = c->colw->write(0, nwin, c->d_codes, c->d_out, c->have_counts ? c->d_counts : nullptr,
                                c->d_win_host_src, c->plan.host_src.data(), c->h_codes.data(), c->stream, &st, &err);
        std::string err2;
        const int rc2 = c->colw->close(&err2);
        if (rc != 0) return fail(c, GSNP_ERR_INPUT, err);
        if (rc2 != 0) return fail(c, GSNP_ERR_INPUT, err2);
        c->columns_host_windows = st.host_windows;
        return GSNP_OK;
    }
    const int rc = fetch_results(c, &calls, &counts);
    if (rc != GSNP_OK) return rc;
    if (write_columns(c->plan, c->h_codes.data(), calls.get(), c->have_counts ? counts.get() : nullptr, chr_name,
                      base_path, dict, host_threads(), &err) != 0)
        return fail(c, GSNP_ERR_INPUT, err);
    return GSNP_OK;
}

extern "C" int gsnp_call_streamed(gsnp_context* c, const gsnp_reads* r, const char* chr_name, gsnp_site_call* out,
                                  const char* cns_path, const char* columns_base) {
    if (!c) return GSNP_ERR_ARG;
    /* the chunk view stays off whatever way the call ends */
    struct ViewOff {
        gsnp_context* c;
        ~ViewOff() {
            c->view.on = false;
            c->called = false;   /* no call stays resident */
        }
    } off{c};
    c->columns_host_windows = 0;
    return gsnp::call_streamed(c, r, chr_name, out, cns_path, columns_base);
}

extern "C" int gsnp_stream_footprint(gsnp_context* c, uint64_t* ring_bytes, uint64_t* writer_bytes) {
    if (!c || !ring_bytes || !writer_bytes) return fail(c, GSNP_ERR_ARG, "null argument");
    *ring_bytes = c->ring ? (uint64_t)c->ring->bytes : 0;
    *writer_bytes = c->colw ? (uint64_t)c->colw->device_bytes() : 0;
    return GSNP_OK;
}

namespace {
/* One read of gsnp_pack_reads; nonzero for a base other than ACGT/acgt or a
 * quality above q_min + 62.  Branch-free in 8-bit lanes, so that the compiler
 * vectorizes it.  k = (b >> 1) & 3 is 0 1 2 3 for A C T G in either case, and
 * a byte is one of those letters exactly when its upper-case form (b & 0xdf)
 * is the letter of its own k: 0x41 | k << 1 gives A C E G, and k == 2 turns
 * E into T (0x45 ^ 0x11 = 0x54).  The quality tests are on signed bytes, as
 * the kernels compare them; q_min is within [-127, 127]. */
unsigned pack_row(const uint8_t* __restrict s, const uint8_t* __restrict q, uint8_t* __restrict o, int l, int q_min) {
    const int8_t lo = (int8_t)q_min;
    const int8_t hi = (int8_t)(q_min + 62 > 127 ? 127 : q_min + 62);
    const uint8_t qm = (uint8_t)q_min;
    uint8_t bad = 0;
    for (int c = 0; c < l; ++c) {
        const uint8_t b = s[c];
        const uint8_t k = (uint8_t)((b >> 1) & 3);
        const uint8_t letter = (uint8_t)((0x41 | (k << 1)) ^ (k == 2 ? 0x11 : 0));
        const int8_t qs = (int8_t)q[c];
        bad |= (uint8_t)((uint8_t)(b & 0xdf) != letter);
        bad |= (uint8_t)(qs > hi);
        const uint8_t code = qs < lo ? (uint8_t)63 : (uint8_t)(q[c] - qm);
        o[c] = (uint8_t)((uint8_t)(k << 6) | code);
    }
    return bad;
}
}  // namespace

extern "C" int gsnp_pack_reads(const uint8_t* seq, const uint8_t* qual, const int32_t* len, int64_t n, int32_t pitch,
                               int q_min, uint8_t* out, int threads) {
    if (n < 0 || pitch < 0 || (n > 0 && (!seq || !qual || !len || !out))) return GSNP_ERR_ARG;
    /* the kernels compare qualities as signed chars; the quality below
     * q_min that a skipped base is unpacked to must be one too */
    if (q_min < -127 || q_min > 127) return GSNP_ERR_ARG;
    std::atomic<int> rc{GSNP_OK};
    auto work = [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b && rc.load(std::memory_order_relaxed) == GSNP_OK; ++i) {
            const int l = len[i];
            if (l < 0 || l > pitch) {
                rc = GSNP_ERR_INPUT;
                return;
            }
            const uint8_t* s = seq + i * pitch;
            const uint8_t* q = qual + i * pitch;
            uint8_t* o = out + i * pitch;
            if (pack_row(s, q, o, l, q_min)) {
                rc = GSNP_ERR_INPUT;
                return;
            }
            memset(o + l, 0, (size_t)(pitch - l));
        }
    };
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(threads > 0 ? threads : host_threads(), n / 4096 + 1));
    std::vector<std::thread> pool;
    const int64_t per = (n + nt - 1) / nt;
    for (int t = 1; t < nt; ++t) pool.emplace_back(work, std::min(n, t * per), std::min(n, (t + 1) * per));
    work(0, std::min(n, per));
    for (std::thread& th : pool) th.join();
    return rc.load();
}
