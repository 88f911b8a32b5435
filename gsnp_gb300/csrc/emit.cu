/*
 * emit.cu - cns text rows on the device (cpp/call_genotype.cc:353-411).
 *
 * One row per site:
 *   chr pos ref type q_cns base1 avgQ1 cu1 ca1 base2 avgQ2 cu2 ca2 depth
 *   rank_sum copy_ratio dbsnp
 * tab separated, doubles as %#.6g (fmt_g6.h), and the reference's literal
 * "N ... 1.000 255.000 0" row for sites it does not call.  The row fields
 * come from make_row (rows.h), which reproduces the reference's stale host
 * count arrays in gap windows.
 *
 * The text of a range of sites is built in three steps: every thread formats
 * its row once to learn its length, an exclusive scan turns the lengths into
 * byte offsets, and every thread formats its row again into place.
 */
#include <cuda_runtime.h>

#include "emit.h"
#include "fmt_g6.h"
#include "rows.h"

namespace gsnp {

namespace {

__constant__ char c_abbv[17] = {'A', 'M', 'W', 'R', 'M', 'C', 'Y', 'S', 'W', 'Y', 'T', 'K', 'R', 'S', 'K', 'G', 'N'};
__constant__ char c_actgn[8] = {'A', 'C', 'T', 'G', 'N', 'N', 'N', 'N'};

constexpr int kRowMax = 384;          /* chromosome name (<= 255) + fields */
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;

struct Out {
    char* p;
    int n;
    __device__ void c(char x) { p[n++] = x; }
    __device__ void s(const char* x, int len) {
        for (int i = 0; i < len; ++i) p[n++] = x[i];
    }
    __device__ void u(uint64_t v) {
        char d[20];
        int k = 0;
        do {
            d[k++] = (char)('0' + v % 10);
            v /= 10;
        } while (v);
        while (k) p[n++] = d[--k];
    }
    __device__ void i(int v) {
        if (v < 0) {
            c('-');
            u((uint64_t)(-(int64_t)v));
        } else {
            u((uint64_t)v);
        }
    }
    __device__ bool g(double v) {
        const int k = fmt_g6(v, p + n);
        n += k;
        return k > 0;
    }
};

/* Format the row of site `site`; returns its length, or -1 when a double is
 * outside the exact formatter's range. */
__device__ int format_row(const EmitArgs& e, int64_t site, char* buf) {
    const int64_t w = site / kWin, j = site - w * kWin;
    const CnsRow r = make_row(e.host_src[w], w, j, e.codes, e.calls, e.counts);
    Out o{buf, 0};
    o.s(e.chr, e.chr_n);
    o.c('\t');
    o.u((uint64_t)(site + 1));
    if (!r.called()) {
        const char lit[] = "\tN\tN\t0\tN\t0\t0\t0\tN\t0\t0\t0\t0\t1.000\t255.000\t0\n";
        o.s(lit, (int)sizeof(lit) - 1);
        return o.n;
    }
    o.c('\t');
    o.c(c_actgn[r.ori & 7]);
    o.c('\t');
    o.c(c_abbv[r.type1]);
    o.c('\t');
    o.i(r.q_cns);
    o.c('\t');
    o.c(c_actgn[r.base1]);
    o.c('\t');
    o.i(r.avg1);
    o.c('\t');
    o.i(r.cu1);
    o.c('\t');
    o.i(r.ca1);
    o.c('\t');
    if (r.base2 < 4) {
        o.c(c_actgn[r.base2]);
        o.c('\t');
        o.i(r.avg2);
        o.c('\t');
        o.i(r.cu2);
        o.c('\t');
        o.i(r.ca2);
    } else {
        o.s("N\t0\t0\t0", 7);
    }
    o.c('\t');
    o.u(r.depth);
    o.c('\t');
    bool ok = o.g(r.rank_sum);
    o.c('\t');
    ok = ok && o.g(r.depth == 0 ? 255.0 : (double)r.repeat / r.depth);
    o.c('\t');
    o.c((r.ori & 8) ? '1' : '0');
    o.c('\n');
    return ok ? o.n : -1;
}

__global__ void row_len_kernel(EmitArgs e) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e.n) return;
    char buf[kRowMax];
    const int len = format_row(e, e.site0 + i, buf);
    if (len < 0) atomicExch(e.error, 1);
    e.len[i] = len < 0 ? 0u : (uint32_t)len;
}

__global__ void row_write_kernel(EmitArgs e) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e.n) return;
    char buf[kRowMax];
    const int len = format_row(e, e.site0 + i, buf);
    char* dst = e.text + e.off[i];
    for (int k = 0; k < len; ++k) dst[k] = buf[k];
}

/* exclusive scan of e.len into e.off, 64-bit */
__device__ uint64_t block_exclusive(uint64_t v, uint64_t* total) {
    __shared__ uint64_t warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t x = v;
    for (int d = 1; d < 32; d <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint64_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, s, d);
            if (lane >= d) s += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint64_t before = (warp ? warp_sums[warp - 1] : 0) + x - v;
    *total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return before;
}

__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(const uint32_t* len, int64_t n, uint64_t* bsum) {
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    uint64_t v = 0;
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) v += len[base + k];
    uint64_t total;
    block_exclusive(v, &total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(uint64_t* bsum, int64_t nb, uint64_t* grand) {
    uint64_t carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += kScanThreads) {
        const int64_t b = b0 + threadIdx.x;
        const uint64_t v = b < nb ? bsum[b] : 0;
        uint64_t total;
        const uint64_t ex = block_exclusive(v, &total);
        if (b < nb) bsum[b] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const uint32_t* len, int64_t n, const uint64_t* bsum,
                                                                uint64_t* off) {
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    uint64_t v[kScanItems], t = 0;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? len[base + k] : 0;
        t += v[k];
    }
    uint64_t total;
    uint64_t run = bsum[blockIdx.x] + block_exclusive(t, &total);
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) {
            off[base + k] = run;
            run += v[k];
        }
}

unsigned grid(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

size_t emit_scratch_bytes(int64_t n) {
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    return (size_t)n * 4 + (size_t)n * 8 + (size_t)(nb + 1) * 8 + 16;
}

cudaError_t emit_lengths(EmitArgs& e, void* scratch, cudaStream_t stream, uint64_t* h_total) {
    uint8_t* p = (uint8_t*)scratch;
    e.len = (uint32_t*)p;
    p += ((size_t)e.n * 4 + 15) & ~(size_t)15;
    e.off = (uint64_t*)p;
    p += (size_t)e.n * 8;
    uint64_t* bsum = (uint64_t*)p;
    const int64_t nb = (e.n + kScanBlock - 1) / kScanBlock;
    uint64_t* grand = bsum + nb;
    if (e.n == 0) {
        *h_total = 0;
        return cudaSuccess;
    }
    row_len_kernel<<<grid(e.n, 128), 128, 0, stream>>>(e);
    scan_sums_kernel<<<(unsigned)nb, kScanThreads, 0, stream>>>(e.len, e.n, bsum);
    scan_blocks_kernel<<<1, kScanThreads, 0, stream>>>(bsum, nb, grand);
    scan_apply_kernel<<<(unsigned)nb, kScanThreads, 0, stream>>>(e.len, e.n, bsum, e.off);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    err = cudaMemcpyAsync(h_total, grand, 8, cudaMemcpyDeviceToHost, stream);
    if (err != cudaSuccess) return err;
    return cudaStreamSynchronize(stream);
}

cudaError_t emit_text(const EmitArgs& e, cudaStream_t stream) {
    if (e.n == 0) return cudaSuccess;
    row_write_kernel<<<grid(e.n, 128), 128, 0, stream>>>(e);
    return cudaGetLastError();
}

}  // namespace gsnp
