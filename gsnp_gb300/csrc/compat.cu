/*
 * compat.cu - the reference's calling backend (include/gsnp_backend.h) on one
 * GB300, for host code written against it (cpp/call_genotype.cc and the rest
 * of the reference's driver link against these symbols unchanged).
 *
 * The contracts are the reference's, call for call, including which host
 * arrays each call refreshes and which it leaves stale:
 *   GPUInit, GSNPKernelInit   kernel/gsnp_kernel.cu:10-33
 *   cuda_init                 kernel/recycle_kernel.cu:11-32
 *   cuda_updateSparse         kernel/update_kernel.cu:233-375
 *   cuda_likelihoodSparse     kernel/likelihood_kernel.cu:258-304, kernel/batchsort.cu:194-291
 *   cuda_posterior            kernel/posterior_kernel.cu:868-991
 *   cuda_recycle              kernel/recycle_kernel.cu:91-136
 *   cuda_quickRecycle         kernel/recycle_kernel.cu:197-252
 *   gold_pos_match            kernel/update_kernel.cu:19-35
 *   encode/decode/getNumBinWord, RLECompression, cuda_dictCompression,
 *   dictComprStart/End        kernel/compress_kernel.cu:85-393
 * Errors end the process with a message, as the reference's cutilSafeCall and
 * ERROR_EXIT do; the functions are not thread-safe (one window state per
 * process, as in the reference).
 *
 * The window state lives in device memory laid out for thread-per-site
 * kernels: records [256 slots][W + L sites] (a warp's lanes touch consecutive
 * words of one slot), counts [W + L][4].  The per-site math (record walk,
 * likelihood, posterior, rank-sum) is the one the whole-chromosome kernels use
 * (site_math.cuh).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "calling.cuh"
#include "dict.h"
#include "gsnp_backend.h"
#include "gsnp_gb300.h"
#include "site_math.cuh"
#include "tables.h"

namespace gsnp {
namespace {

constexpr int kSlots = GSNP_MAX_RECORDS_PER_SITE;

void die(const char* where, const char* what) {
    fprintf(stderr, "!!!ERROR@%s: %s\n", where, what);
    exit(EXIT_FAILURE);
}

#define CC(call)                                                      \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) die(__func__, cudaGetErrorString(e_)); \
    } while (0)

template <class T>
void dalloc(T** p, size_t n) {
    if (*p) CC(cudaFree(*p));
    *p = nullptr;
    CC(cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)));
}

template <class T>
void dfree(T** p) {
    if (*p) cudaFree(*p);
    *p = nullptr;
}

/* device copy of the reference's module globals (kernel/common_kernel.h:16-61) */
struct Window {
    bool ready = false;
    int device = 0;
    cudaStream_t stream = nullptr;
    int64_t W = 0, L = 0, N = 0;    /* N = W + L sites */
    HostTables tables;
    double pcr = 0.0, glob = 0.0;
    /* tables */
    double* lik64 = nullptr;
    uint8_t* qadj = nullptr;
    double* log_prior = nullptr;
    double* p_rank = nullptr;
    /* window state */
    uint32_t* recs = nullptr;       /* [kSlots][N] */
    uint32_t* seen = nullptr;       /* [16][N] pcr-dependency bitsets */
    uint32_t* num = nullptr;        /* [N] */
    int* dep_uni = nullptr;         /* [N] */
    int* count_uni = nullptr;       /* [N][4] */
    int* q_sum = nullptr;
    int* count_all = nullptr;
    int* depth = nullptr;           /* [N] */
    int* repeat = nullptr;
    double* type_likely = nullptr;  /* [W][16]; never reset, as in the reference */
    char* base1 = nullptr;          /* [W] posterior outputs, kept across windows */
    char* base2 = nullptr;
    char* type1 = nullptr;
    int* q_cns = nullptr;
    double* rank_sum = nullptr;
    /* staging of one update / posterior call */
    char* rd = nullptr;             /* [cap][L] bases */
    char* rq = nullptr;             /* [cap][L] qualities */
    char* rs = nullptr;             /* [cap] strands */
    int* rlh = nullptr;             /* [cap] len << 16 | hit */
    int64_t read_cap = 0;
    int* site_match = nullptr;      /* [W][2] */
    unsigned int* max_num = nullptr;
    char* ori = nullptr;            /* [W] */
    bool* nflag = nullptr;
    bool* validated = nullptr;
    bool* hapmap = nullptr;
    bool* indel = nullptr;
    double* freq = nullptr;         /* [W][4] */
    /* dictionary codec scratch */
    void* dict_scratch = nullptr;
    size_t dict_bytes = 0;
};

Window g;

/* CallArgs subset that the per-site math reads */
CallArgs math_args(bool rank_sum, bool monoploid, int q_max_min) {
    CallArgs a;
    memset(&a, 0, sizeof(a));
    a.L = (int)g.L;
    a.lik64 = g.lik64;
    a.qa_rows = g.tables.qa_rows;
    a.qadj = g.qadj;
    a.tmax = g.tables.tmax;
    a.gmax = g.tables.gmax;
    a.log_prior = g.log_prior;
    a.p_rank = g.p_rank;
    a.q_max_min = q_max_min;
    a.rank_sum = rank_sum;
    a.monoploid = monoploid;
    return a;
}

struct UpdateArgs {
    const char* rd;
    const char* rq;
    const char* rs;
    const int* rlh;
    const int* site_match;
    int64_t W, L, N;
    char qmin;
    uint32_t* recs;
    uint32_t* num;
    int* dep_uni;
    int* count_uni;
    int* q_sum;
    int* count_all;
    int* depth;
    int* repeat;
    unsigned int* max_num;
};

/* updateSparse_kernel (kernel/update_kernel.cu:233-326): one thread per site
 * appends the records of every read of this call covering the site, in
 * (window offset, read index) order, after the records carried over. */
__global__ void update_kernel(UpdateArgs u) {
    const int64_t site = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (site >= u.N) return;
    const int L = (int)u.L;
    int depth = 0, repeat = 0;
    int dep_uni = site < L ? u.dep_uni[site] : 0;
    int num = site < L ? (int)u.num[site] : 0;
    int cu[4] = {0, 0, 0, 0}, qs[4] = {0, 0, 0, 0}, ca[4] = {0, 0, 0, 0};
    int64_t cov = site - L + 1;
    if (cov < 0) cov = 0;
    if (cov >= u.W) return;
    for (; cov <= site && cov < u.W; ++cov) {
        const int first = u.site_match[2 * cov];
        const int last = first + u.site_match[2 * cov + 1];
        const int coord = (int)(site - cov);
        for (int r = first; r < last; ++r) {
            const uint32_t lh = (uint32_t)u.rlh[r];
            const int rlen = (int)(lh >> 16);
            if (coord >= rlen) continue;
            const int hit = (int)(lh & 0xffffu);
            const signed char base = (signed char)u.rd[(int64_t)r * L + coord];
            const signed char qual = (signed char)u.rq[(int64_t)r * L + coord];
            depth += 1;
            repeat += hit;
            if (base == 'N' || qual < (signed char)u.qmin || dep_uni >= 0xFF) continue;
            const int b = (base >> 1) & 3;
            if (hit == 1) {
                dep_uni += 1;
                const bool plus = u.rs[r] == '+';
                const uint32_t coord_val = plus ? (uint32_t)coord : (uint32_t)(rlen - 1 - coord);
                u.recs[(int64_t)num * u.N + site] = make_record(base, qual - (signed char)u.qmin, coord_val,
                                                                plus ? 0u : 1u);
                num += 1;
                cu[b] += 1;
                qs[b] += qual - (signed char)u.qmin;
            }
            ca[b] += 1;
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        u.count_uni[site * 4 + i] += cu[i];
        u.q_sum[site * 4 + i] += qs[i];
        u.count_all[site * 4 + i] += ca[i];
    }
    u.depth[site] += depth;
    u.repeat[site] += repeat;
    u.dep_uni[site] = dep_uni;
    u.num[site] = (uint32_t)num;
    if (site < u.W) atomicMax(u.max_num, (unsigned int)num);
}

/* batchSortMP2 + likelihoodSparse_kernel: sort each site's records ascending
 * (insertion sort in the site's own column) and sum its likelihood in FP64
 * in that order. */
__global__ void likelihood_kernel(CallArgs a, uint32_t* recs, uint32_t* seen, const uint32_t* num, int64_t N,
                                  int64_t n_site, double* tl_out) {
    const int64_t site = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (site >= n_site) return;
    uint32_t* col = recs + site;
    const int n = (int)num[site];
    for (int i = 1; i < n; ++i) {
        const uint32_t w = col[(int64_t)i * N];
        int j = i;
        while (j > 0) {
            const uint32_t prev = col[(int64_t)(j - 1) * N];
            if (prev <= w) break;
            col[(int64_t)j * N] = prev;
            --j;
        }
        col[(int64_t)j * N] = w;
    }
    double tl[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) tl[i] = 0.0;
    likelihood_fp64(a, col, seen + site, (int)N, n, tl);
    double* dst = tl_out + site * 16;
#pragma unroll
    for (int i = 0; i < 16; ++i) dst[i] = tl[i];
}

struct PosteriorArgs {
    const char* ori;
    const bool* nflag;
    const bool* validated;
    const bool* hapmap;
    const bool* indel;
    const double* freq;
    double het_val, het_unval, althom_val, althom_unval;
    int refine;
    const uint32_t* recs;
    const uint32_t* num;
    const int* dep_uni;
    const int* count_uni;
    const int* q_sum;
    const int* count_all;
    const double* type_likely;
    int64_t N, call_length;
    char* base1;
    char* base2;
    char* type1;
    int* q_cns;
    double* rank_sum;
};

/* posterior_kernel + posterior_kernel2 over the window (kernel/posterior_kernel.cu:635-866),
 * with the dbSNP prior of each site generated in place (:575-633) */
__global__ void posterior_kernel(CallArgs a, PosteriorArgs pa) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= pa.call_length || pa.nflag[s]) return;
    SitePileup p;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        p.cu[i] = pa.count_uni[s * 4 + i];
        p.qs[i] = pa.q_sum[s * 4 + i];
        p.ca[i] = (uint32_t)pa.count_all[s * 4 + i];
    }
    p.depth = 0;
    p.repeat = 0;
    p.dep_uni = pa.dep_uni[s];
    p.num = (int)pa.num[s];
    const uint8_t ori = (uint8_t)pa.ori[s];
    const int ori7 = ori & 7;
    double lp[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) lp[i] = a.log_prior[(ori7 << 4) + i];
    if ((ori & 0x8) && pa.refine && !pa.indel[s]) {
        const int t_base = ori & 3;
        const double* f = pa.freq + s * 4;
        for (int a1 = 0; a1 != 4; ++a1)
            for (int a2 = a1; a2 != 4; ++a2) {
                if (!(f[a1] > 0 && f[a2] > 0)) continue;
                double pr;
                if (!pa.hapmap[s]) {
                    if (a1 == a2 && a1 == t_base) pr = 1;
                    else if (a1 == t_base || a2 == t_base) pr = pa.validated[s] ? pa.het_val : pa.het_unval;
                    else if (a1 == a2) pr = pa.validated[s] ? pa.althom_val : pa.althom_unval;
                    else pr = pa.validated[s] ? pa.het_val : pa.het_unval;
                } else {
                    pr = GSNP_DMUL(GSNP_DMUL((a1 == a2 ? 1.0 : GSNP_DMUL(2.0, pa.het_val)), f[a1]), f[a2]);
                }
                lp[(a1 << 2) | a2] = gsnp_cr_log10(pr);
            }
    }
    double tl[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) tl[i] = pa.type_likely[s * 16 + i];
    /* the reference reads q_sum[4*s + base] for an N-coded base, i.e. the
     * next site's entry */
    auto nq = [&](int b) { return pa.q_sum[(s + 1) * 4 + b]; };
    SiteCall c;
    site_posterior(a, ori, p, tl, nullptr, lp, pa.recs + s, (int)pa.N, nq, &c);
    pa.base1[s] = (char)c.base1;
    pa.base2[s] = (char)c.base2;
    pa.type1[s] = (char)c.type1;
    pa.q_cns[s] = c.q_cns;
    pa.rank_sum[s] = c.rank_sum;
}

/* window shift (kernel/recycle_kernel.cu:91-136): the L-site tail becomes the head */
__global__ void shift_copy_kernel(uint32_t* recs, uint32_t* num, int* dep_uni, int* count_uni, int* q_sum,
                                  int* count_all, int* depth, int* repeat, int64_t W, int64_t L, int64_t N) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L) return;
    const int64_t src = W + i;
    const uint32_t n = num[src];
    for (uint32_t k = 0; k < n; ++k) recs[(int64_t)k * N + i] = recs[(int64_t)k * N + src];
    num[i] = n;
    dep_uni[i] = dep_uni[src];
    depth[i] = depth[src];
    repeat[i] = repeat[src];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        count_uni[i * 4 + b] = count_uni[src * 4 + b];
        q_sum[i * 4 + b] = q_sum[src * 4 + b];
        count_all[i * 4 + b] = count_all[src * 4 + b];
    }
}

__global__ void shift_clear_kernel(uint32_t* num, int* dep_uni, int* count_uni, int* q_sum, int* count_all,
                                   int* depth, int* repeat, int64_t L, int64_t N) {
    const int64_t i = L + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    num[i] = 0;
    dep_uni[i] = 0;
    depth[i] = 0;
    repeat[i] = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        count_uni[i * 4 + b] = 0;
        q_sum[i * 4 + b] = 0;
        count_all[i * 4 + b] = 0;
    }
}

unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

void require_ready(const char* where) {
    if (!g.ready) die(where, "GSNPKernelInit has not been called");
}

void download_counts(int* count_uni, int* q_sum, int* count_all, int* depth, int* repeat) {
    const size_t n = (size_t)g.N;
    CC(cudaMemcpyAsync(count_uni, g.count_uni, n * 16, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaMemcpyAsync(q_sum, g.q_sum, n * 16, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaMemcpyAsync(count_all, g.count_all, n * 16, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaMemcpyAsync(depth, g.depth, n * 4, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaMemcpyAsync(repeat, g.repeat, n * 4, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaStreamSynchronize(g.stream));
}

void shift_window() {
    const int64_t L = g.L, W = g.W, N = g.N;
    shift_copy_kernel<<<blocks(L, 128), 128, 0, g.stream>>>(g.recs, g.num, g.dep_uni, g.count_uni, g.q_sum,
                                                              g.count_all, g.depth, g.repeat, W, L, N);
    CC(cudaGetLastError());
    shift_clear_kernel<<<blocks(N - L, 256), 256, 0, g.stream>>>(g.num, g.dep_uni, g.count_uni, g.q_sum,
                                                                   g.count_all, g.depth, g.repeat, L, N);
    CC(cudaGetLastError());
}

void shift_positions(int* posArr) {
    memmove(posArr, posArr + g.W, (size_t)g.L * sizeof(int));
    for (int64_t i = g.L; i < g.L + g.W; ++i) posArr[i] = posArr[i - 1] + 1;
}

template <class T>
void dict_compress(unsigned int* out, unsigned long* n_words, T* dict, unsigned long* n_dict, const T* in,
                   unsigned long n) {
    if (*n_dict < n) die("cuda_dictCompression", "*numElementDict < numElementInData");
    const size_t in_bytes = ((n * sizeof(T) + 255) / 256) * 256;
    const size_t need = in_bytes + dict_scratch_bytes(n);
    if (need > g.dict_bytes) {
        if (g.dict_scratch) CC(cudaFree(g.dict_scratch));
        g.dict_scratch = nullptr;
        CC(cudaMalloc(&g.dict_scratch, need));
        g.dict_bytes = need;
    }
    T* d_in = reinterpret_cast<T*>(g.dict_scratch);
    if (n) CC(cudaMemcpyAsync(d_in, in, n * sizeof(T), cudaMemcpyHostToDevice, g.stream));
    std::string err;
    const int rc = dict_compress_device<T>(d_in, n, reinterpret_cast<char*>(g.dict_scratch) + in_bytes,
                                           g.dict_bytes - in_bytes, g.stream, out, n_words, dict, n_dict, &err);
    if (rc != 0) die("cuda_dictCompression", err.c_str());
}

template <class T, class R>
unsigned int rle(T* data, unsigned long n, R* run_length) {
    if (n == 0) return 0;
    unsigned long runs = 0, start = 0;
    for (unsigned long i = 1; i <= n; ++i) {
        if (i == n || !(data[i] == data[start])) {
            data[runs] = data[start];
            run_length[runs] = (R)(i - start);
            ++runs;
            start = i;
        }
    }
    return (unsigned int)runs;
}

int base_bits(char c) {
    switch (c) {
        case 'A': case 'a': return 0;
        case 'C': case 'c': return 1;
        case 'G': case 'g': return 2;
        case 'T': case 't': return 3;
        default: return -1;
    }
}

}  // namespace
}  // namespace gsnp

using namespace gsnp;

void GPUInit() {
    const char* env = getenv("GSNP_DEVICE");
    g.device = env ? atoi(env) : 0;
    CC(cudaSetDevice(g.device));
    if (!g.stream) CC(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
}

void GSNPKernelInit(const unsigned long winSize, const int readLength, const double pcr_dependency,
                    const double global_dependency, const double* h_pmatrix, const double* p_prior,
                    const double* p_rank) {
    if (!g.stream) GPUInit();
    if (winSize == 0 || readLength <= 0 || readLength > 255) die("GSNPKernelInit", "bad window or read length");
    gsnp_params p;
    memset(&p, 0, sizeof(p));
    p.read_length = readLength;
    p.pcr_dependency = pcr_dependency;
    p.global_dependency = global_dependency;
    std::string err;
    if (build_tables(p, h_pmatrix, p_prior, &g.tables, &err) != 0) die("GSNPKernelInit", err.c_str());
    g.W = (int64_t)winSize;
    g.L = readLength;
    g.N = g.W + g.L;
    g.pcr = pcr_dependency;
    g.glob = global_dependency;
    const HostTables& t = g.tables;
    dalloc(&g.lik64, t.lik64.size());
    dalloc(&g.qadj, t.qadj.size());
    dalloc(&g.log_prior, 128);
    dalloc(&g.p_rank, GSNP_PRANK_SIZE);
    CC(cudaMemcpy(g.lik64, t.lik64.data(), t.lik64.size() * 8, cudaMemcpyHostToDevice));
    CC(cudaMemcpy(g.qadj, t.qadj.data(), t.qadj.size(), cudaMemcpyHostToDevice));
    CC(cudaMemcpy(g.log_prior, t.log_prior.data(), 128 * 8, cudaMemcpyHostToDevice));
    CC(cudaMemcpy(g.p_rank, p_rank, GSNP_PRANK_SIZE * 8, cudaMemcpyHostToDevice));
    const size_t N = (size_t)g.N, W = (size_t)g.W;
    dalloc(&g.recs, (size_t)kSlots * N);
    dalloc(&g.seen, 16 * N);
    dalloc(&g.num, N);
    dalloc(&g.dep_uni, N);
    dalloc(&g.count_uni, 4 * N);
    dalloc(&g.q_sum, 4 * N + 4);
    dalloc(&g.count_all, 4 * N);
    dalloc(&g.depth, N);
    dalloc(&g.repeat, N);
    dalloc(&g.type_likely, 16 * W);
    dalloc(&g.base1, W);
    dalloc(&g.base2, W);
    dalloc(&g.type1, W);
    dalloc(&g.q_cns, W);
    dalloc(&g.rank_sum, W);
    dalloc(&g.site_match, 2 * W);
    dalloc(&g.max_num, 1);
    dalloc(&g.ori, W);
    dalloc(&g.nflag, W);
    dalloc(&g.validated, W);
    dalloc(&g.hapmap, W);
    dalloc(&g.indel, W);
    dalloc(&g.freq, 4 * W);
    /* the reference leaves these uninitialised; zeros give them a defined value */
    CC(cudaMemset(g.type_likely, 0, 16 * W * 8));
    CC(cudaMemset(g.base1, 0, W));
    CC(cudaMemset(g.base2, 0, W));
    CC(cudaMemset(g.type1, 0, W));
    CC(cudaMemset(g.q_cns, 0, W * 4));
    CC(cudaMemset(g.rank_sum, 0, W * 8));
    CC(cudaMemset(g.num, 0, N * 4));
    CC(cudaMemset(g.dep_uni, 0, N * 4));
    CC(cudaMemset(g.count_uni, 0, N * 16));
    CC(cudaMemset(g.q_sum, 0, N * 16 + 16));
    CC(cudaMemset(g.count_all, 0, N * 16));
    CC(cudaMemset(g.depth, 0, N * 4));
    CC(cudaMemset(g.repeat, 0, N * 4));
    g.ready = true;
}

void cuda_init(unsigned long long win_size, unsigned long long read_len, unsigned long long start, int* posArr,
               const unsigned int, const unsigned int) {
    require_ready("cuda_init");
    if ((int64_t)win_size != g.W || (int64_t)read_len != g.L) die("cuda_init", "window differs from GSNPKernelInit");
    for (unsigned long long i = 0; i < win_size + read_len; ++i) posArr[i] = (int)(i + start);
    const size_t N = (size_t)g.N;
    CC(cudaMemsetAsync(g.num, 0, N * 4, g.stream));
    CC(cudaMemsetAsync(g.dep_uni, 0, N * 4, g.stream));
    CC(cudaMemsetAsync(g.count_uni, 0, N * 16, g.stream));
    CC(cudaMemsetAsync(g.q_sum, 0, N * 16, g.stream));
    CC(cudaMemsetAsync(g.count_all, 0, N * 16, g.stream));
    CC(cudaMemsetAsync(g.depth, 0, N * 4, g.stream));
    CC(cudaMemsetAsync(g.repeat, 0, N * 4, g.stream));
    CC(cudaStreamSynchronize(g.stream));
}

void gold_pos_match(int* positionArr, int* siteMatchArr, int readCount) {
    memset(siteMatchArr, 0, sizeof(int) * GSNP_WIN_SIZE * 2);
    for (int r = 0; r < readCount; ++r) {
        const int s = positionArr[r] % GSNP_WIN_SIZE;
        if (siteMatchArr[2 * s + 1] == 0) siteMatchArr[2 * s] = r;
        siteMatchArr[2 * s + 1] += 1;
    }
}

unsigned int cuda_updateSparse(struct st_update* u, unsigned int*, unsigned int*, int read_len, int* count_uniArr,
                               int* q_sumArr, int* count_allArr, int* depthArr, int* repeat_timeArr, int*,
                               int readCount, const unsigned int, const unsigned int) {
    require_ready("cuda_updateSparse");
    if (read_len != g.L) die("cuda_updateSparse", "read length differs from GSNPKernelInit");
    if (readCount < 0) die("cuda_updateSparse", "negative read count");
    const int64_t n = readCount, L = g.L;
    if (n > g.read_cap) {
        const int64_t cap = std::max<int64_t>(n, 1 << 16);
        dalloc(&g.rd, (size_t)cap * L);
        dalloc(&g.rq, (size_t)cap * L);
        dalloc(&g.rs, (size_t)cap);
        dalloc(&g.rlh, (size_t)cap);
        g.read_cap = cap;
    }
    if (n) {
        CC(cudaMemcpyAsync(g.rd, u->readArr, (size_t)n * L, cudaMemcpyHostToDevice, g.stream));
        CC(cudaMemcpyAsync(g.rq, u->qualArr, (size_t)n * L, cudaMemcpyHostToDevice, g.stream));
        CC(cudaMemcpyAsync(g.rs, u->strandArr, (size_t)n, cudaMemcpyHostToDevice, g.stream));
        CC(cudaMemcpyAsync(g.rlh, u->readLen_hitArr, (size_t)n * 4, cudaMemcpyHostToDevice, g.stream));
    }
    CC(cudaMemcpyAsync(g.site_match, u->siteMatchArr, (size_t)g.W * 8, cudaMemcpyHostToDevice, g.stream));
    CC(cudaMemsetAsync(g.max_num, 0, 4, g.stream));
    UpdateArgs a{g.rd, g.rq, g.rs, g.rlh, g.site_match, g.W, g.L, g.N, u->qmin, g.recs, g.num, g.dep_uni,
                 g.count_uni, g.q_sum, g.count_all, g.depth, g.repeat, g.max_num};
    update_kernel<<<blocks(g.N, 128), 128, 0, g.stream>>>(a);
    CC(cudaGetLastError());
    unsigned int mx = 0;
    CC(cudaMemcpyAsync(&mx, g.max_num, 4, cudaMemcpyDeviceToHost, g.stream));
    download_counts(count_uniArr, q_sumArr, count_allArr, depthArr, repeat_timeArr);
    return mx;
}

void cuda_likelihoodSparse(double* h_typeLikelihood, const unsigned int numSite, const unsigned int maxNumNonZero,
                           const unsigned int, const unsigned int, const unsigned int, const unsigned int) {
    require_ready("cuda_likelihoodSparse");
    if ((int64_t)numSite > g.W) die("cuda_likelihoodSparse", "more sites than the window");
    if (maxNumNonZero == 0) {
        /* the device likelihood keeps its previous values (kernel/likelihood_kernel.cu:269-274) */
        memset(h_typeLikelihood, 0, sizeof(double) * GSNP_LIKELY_SIZE * numSite);
        return;
    }
    const CallArgs a = math_args(false, false, 0);
    likelihood_kernel<<<blocks(numSite, 128), 128, 0, g.stream>>>(a, g.recs, g.seen, g.num, g.N, numSite,
                                                                   g.type_likely);
    CC(cudaGetLastError());
    CC(cudaStreamSynchronize(g.stream));
}

void cuda_posterior(st_likelihood* lk, char* oriArr, char* base1, char* base2, char* type1, int* q_cns,
                    double* rank_sum_test_value, bool* validatedArr, bool* hapmap_siteArr, bool* indel_siteArr,
                    double* freqArr, double het_val, double het_unval, double althom_val, double althom_unval,
                    bool rank_sum_mode, bool monoploid, bool refine, char q_max_min, unsigned long long, int win_size,
                    unsigned long call_length, unsigned int, const unsigned int, const unsigned int) {
    require_ready("cuda_posterior");
    if ((int64_t)win_size > g.W || (int64_t)call_length > g.W) die("cuda_posterior", "more sites than the window");
    const size_t W = (size_t)win_size;
    CC(cudaMemcpyAsync(g.ori, oriArr, W, cudaMemcpyHostToDevice, g.stream));
    CC(cudaMemcpyAsync(g.nflag, lk->nflag, W, cudaMemcpyHostToDevice, g.stream));
    CC(cudaMemcpyAsync(g.validated, validatedArr, W, cudaMemcpyHostToDevice, g.stream));
    CC(cudaMemcpyAsync(g.hapmap, hapmap_siteArr, W, cudaMemcpyHostToDevice, g.stream));
    CC(cudaMemcpyAsync(g.indel, indel_siteArr, W, cudaMemcpyHostToDevice, g.stream));
    CC(cudaMemcpyAsync(g.freq, freqArr, W * 32, cudaMemcpyHostToDevice, g.stream));
    const CallArgs a = math_args(rank_sum_mode, monoploid, (int)q_max_min);
    PosteriorArgs pa{g.ori, g.nflag, g.validated, g.hapmap, g.indel, g.freq, het_val, het_unval, althom_val,
                     althom_unval, refine ? 1 : 0, g.recs, g.num, g.dep_uni, g.count_uni, g.q_sum, g.count_all,
                     g.type_likely, g.N, (int64_t)call_length, g.base1, g.base2, g.type1, g.q_cns, g.rank_sum};
    if (call_length) {
        posterior_kernel<<<blocks((int64_t)call_length, 128), 128, 0, g.stream>>>(a, pa);
        CC(cudaGetLastError());
    }
    CC(cudaMemcpyAsync(base1, g.base1, W, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaMemcpyAsync(base2, g.base2, W, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaMemcpyAsync(type1, g.type1, W, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaMemcpyAsync(q_cns, g.q_cns, W * 4, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaMemcpyAsync(rank_sum_test_value, g.rank_sum, W * 8, cudaMemcpyDeviceToHost, g.stream));
    CC(cudaStreamSynchronize(g.stream));
}

void cuda_recycle(unsigned long long win_size, unsigned long long read_len, int* posArr, const unsigned int,
                  const unsigned int) {
    require_ready("cuda_recycle");
    if ((int64_t)win_size != g.W || (int64_t)read_len != g.L) die("cuda_recycle", "window differs");
    shift_positions(posArr);
    shift_window();
    CC(cudaStreamSynchronize(g.stream));
}

void cuda_quickRecycle(unsigned long long win_size, unsigned long long read_len, int* posArr, int* count_uniArr,
                       int* q_sumArr, int* count_allArr, int* depthArr, int* repeat_timeArr, const unsigned int,
                       const unsigned int) {
    require_ready("cuda_quickRecycle");
    if ((int64_t)win_size != g.W || (int64_t)read_len != g.L) die("cuda_quickRecycle", "window differs");
    shift_window();
    shift_positions(posArr);
    download_counts(count_uniArr, q_sumArr, count_allArr, depthArr, repeat_timeArr);
}

unsigned long getNumBinWord(const unsigned long numElement) { return (numElement + 15) / 16; }

unsigned long encode(unsigned int* code, const char* seq, const unsigned long numElement) {
    const unsigned long nw = getNumBinWord(numElement);
    for (unsigned long w = 0; w < nw; ++w) {
        const unsigned long nb = (w == nw - 1) ? numElement - w * 16 : 16;
        unsigned int word = 0;
        for (unsigned long i = 0; i < nb; ++i) {
            const int c = base_bits(seq[w * 16 + i]);
            if (c < 0) {
                printf("!!!ERROR@encode: unknown base when encoding.\n");
                exit(EXIT_FAILURE);
            }
            word = (word << 2) | (unsigned int)c;
        }
        code[w] = word;
    }
    return nw;
}

void decode(char* seq, const unsigned long numElement, const unsigned int* code, const unsigned long numCodeWord) {
    static const char letters[4] = {'A', 'C', 'G', 'T'};
    if (numCodeWord == 0) return;
    for (unsigned long w = 0; w + 1 < numCodeWord; ++w)
        for (unsigned int i = 0; i < 16; ++i) seq[w * 16 + i] = letters[(code[w] >> (30 - 2 * i)) & 3];
    const unsigned long left = numElement - (numCodeWord - 1) * 16;
    for (unsigned long i = 0; i < left; ++i)
        seq[(numCodeWord - 1) * 16 + i] = letters[(code[numCodeWord - 1] >> (2 * (left - i - 1))) & 3];
}

void dictComprStart(const unsigned long numElement, const unsigned long dataSize) {
    if (!g.stream) GPUInit();
    const size_t in_bytes = ((numElement * std::max<unsigned long>(dataSize, 1) + 255) / 256) * 256;
    const size_t need = in_bytes + dict_scratch_bytes(numElement);
    if (need > g.dict_bytes) {
        if (g.dict_scratch) CC(cudaFree(g.dict_scratch));
        g.dict_scratch = nullptr;
        CC(cudaMalloc(&g.dict_scratch, need));
        g.dict_bytes = need;
    }
}

void dictComprEnd() {
    if (g.dict_scratch) cudaFree(g.dict_scratch);
    g.dict_scratch = nullptr;
    g.dict_bytes = 0;
}

void cuda_dictCompression(unsigned int* out, unsigned long* nw, char* dict, unsigned long* nd, char* in,
                          const unsigned long n) {
    if (!g.stream) GPUInit();
    dict_compress(out, nw, dict, nd, in, n);
}
void cuda_dictCompression(unsigned int* out, unsigned long* nw, int* dict, unsigned long* nd, int* in,
                          const unsigned long n) {
    if (!g.stream) GPUInit();
    dict_compress(out, nw, dict, nd, in, n);
}
void cuda_dictCompression(unsigned int* out, unsigned long* nw, unsigned int* dict, unsigned long* nd,
                          unsigned int* in, const unsigned long n) {
    if (!g.stream) GPUInit();
    dict_compress(out, nw, dict, nd, in, n);
}
void cuda_dictCompression(unsigned int* out, unsigned long* nw, double* dict, unsigned long* nd, double* in,
                          const unsigned long n) {
    if (!g.stream) GPUInit();
    dict_compress(out, nw, dict, nd, in, n);
}

unsigned int RLECompression(int* data, const unsigned long n, unsigned int* runLength) {
    return rle(data, n, runLength);
}
unsigned int RLECompression(double* data, const unsigned long n, unsigned int* runLength) {
    return rle(data, n, runLength);
}
unsigned int RLECompression(char* data, const unsigned long n, int* runLength) { return rle(data, n, runLength); }
