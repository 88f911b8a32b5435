/*
 * dict.cu - dictionary codec of the -C output on sm_103a.
 *
 * Replaces cuda_dictCompression (kernel/compress_kernel.cu:224-334), which
 * runs thrust::sort, thrust::unique and thrust::lower_bound on the device and a
 * packing kernel.  The output format is unchanged:
 *   dict  = the distinct input values in ascending order
 *   words = the index of every input value in dict, packed MSB-first into
 *           32-bit words, floor(32 / bits) indices per word, the last word
 *           holding the remaining indices right-aligned;
 *   bits  = (int)ceil(log(#dict) / log(2)) with the C library's log, at least 1
 *           (cpp/dict_compression.h:47-58).
 *
 * Here the distinct values are collected in a hash set (open addressing on
 * order-preserving 64-bit keys), sorted (bitonic in shared memory up to 8192
 * keys, a global bitonic network above), then every value finds its index by
 * binary search and each output word is packed by one thread.  For doubles
 * -0.0 and +0.0 are one dictionary entry, stored as -0.0 when any -0.0 occurs,
 * as the reference's radix sort followed by unique(==) keeps it.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "dict.h"

namespace gsnp {

namespace {

constexpr uint64_t kEmpty = ~0ULL;

template <class T> struct KeyOf;
template <> struct KeyOf<char> {
    __host__ __device__ static uint64_t key(char v) { return (uint64_t)((int64_t)(signed char)v + 128); }
    static char value(uint64_t k, bool) { return (char)(signed char)((int64_t)k - 128); }
};
template <> struct KeyOf<int> {
    __host__ __device__ static uint64_t key(int v) { return (uint64_t)((int64_t)v + 2147483648LL); }
    static int value(uint64_t k, bool) { return (int)((int64_t)k - 2147483648LL); }
};
template <> struct KeyOf<unsigned int> {
    __host__ __device__ static uint64_t key(unsigned int v) { return (uint64_t)v; }
    static unsigned int value(uint64_t k, bool) { return (unsigned int)k; }
};
template <> struct KeyOf<double> {
    __host__ __device__ static uint64_t key(double v) {
        uint64_t b;
        memcpy(&b, &v, 8);
        if (b == 0x8000000000000000ULL) b = 0;   /* -0.0 and +0.0 share one key */
        return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
    }
    static double value(uint64_t k, bool negzero) {
        uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
        if (b == 0 && negzero) b = 0x8000000000000000ULL;
        double v;
        memcpy(&v, &b, 8);
        return v;
    }
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

template <class T>
__global__ void insert_kernel(const T* __restrict__ in, size_t n, uint64_t* __restrict__ table, uint64_t mask,
                              int* __restrict__ flags) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T v = in[i];
    if (sizeof(T) == 8) {
        uint64_t b;
        memcpy(&b, &v, 8);
        if (b == 0x8000000000000000ULL) atomicOr(flags, 1);
    }
    const uint64_t k = KeyOf<T>::key(v);
    uint64_t h = mix64(k) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long prev = atomicCAS((unsigned long long*)&table[h], (unsigned long long)kEmpty,
                                                  (unsigned long long)k);
        if (prev == kEmpty || prev == k) return;
        h = (h + 1) & mask;
    }
    atomicOr(flags, 2);   /* table full: cannot happen with capacity >= 2n */
}

__global__ void compact_kernel(const uint64_t* __restrict__ table, size_t cap, uint64_t* __restrict__ keys,
                               unsigned long long* __restrict__ count) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    const uint64_t k = table[i];
    if (k != kEmpty) keys[atomicAdd(count, 1ULL)] = k;
}

/* bitonic sort of m (power of two) keys in one CTA's shared memory */
__global__ void bitonic_smem_kernel(uint64_t* keys, int m) {
    extern __shared__ uint64_t sk[];
    for (int i = threadIdx.x; i < m; i += blockDim.x) sk[i] = keys[i];
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const uint64_t a = sk[i], b = sk[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) { sk[i] = b; sk[ixj] = a; }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < m; i += blockDim.x) keys[i] = sk[i];
}

/* one compare-exchange stage of a global bitonic network over m keys */
__global__ void bitonic_global_kernel(uint64_t* keys, size_t m, size_t k, size_t j) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const size_t ixj = i ^ j;
    if (ixj > i) {
        const uint64_t a = keys[i], b = keys[ixj];
        const bool up = (i & k) == 0;
        if ((a > b) == up) { keys[i] = b; keys[ixj] = a; }
    }
}

template <class T>
__global__ void index_kernel(const T* __restrict__ in, size_t n, const uint64_t* __restrict__ keys, size_t d,
                             uint32_t* __restrict__ idx) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t k = KeyOf<T>::key(in[i]);
    size_t lo = 0, hi = d;
    while (lo < hi) {
        const size_t mid = (lo + hi) >> 1;
        if (keys[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    idx[i] = (uint32_t)lo;
}

__global__ void pack_kernel(const uint32_t* __restrict__ idx, size_t n, int bits, int per_word, size_t n_words,
                            uint32_t* __restrict__ words) {
    const size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n_words) return;
    const size_t first = w * (size_t)per_word;
    const size_t cnt = (w == n_words - 1) ? n - first : (size_t)per_word;
    uint32_t out = 0;
    for (size_t i = 0; i < cnt; ++i) out = (out << bits) | idx[first + i];
    words[w] = out;
}

inline unsigned blocks(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int dict_bits(unsigned long n) {
    int bits = (int)ceil(log((double)(n)) / log((double)2.f));
    if (bits == 0) bits = 1;
    return bits;
}

size_t dict_scratch_bytes(size_t n) {
    size_t cap = 1;
    while (cap < 2 * n) cap <<= 1;
    size_t m = 1;
    while (m < n) m <<= 1;
    return cap * 8 + m * 8 + n * 4 + n * 4 + 64;
}

template <class T>
int dict_compress_device(const T* d_in, size_t n, void* d_scratch, size_t scratch_bytes, cudaStream_t stream,
                         uint32_t* h_words, unsigned long* n_words, T* h_dict, unsigned long* n_dict,
                         std::string* err) {
    if (*n_dict < n) {
        *err = "*numElementDict < numElementInData";
        return 4;
    }
    if (n == 0) {
        *n_dict = 0;
        *n_words = 0;
        return 0;
    }
    if (dict_scratch_bytes(n) > scratch_bytes) {
        *err = "dictionary scratch too small";
        return 4;
    }
    size_t cap = 1;
    while (cap < 2 * n) cap <<= 1;
    size_t m = 1;
    while (m < n) m <<= 1;
    uint8_t* p = (uint8_t*)d_scratch;
    uint64_t* table = (uint64_t*)p;
    uint64_t* keys = (uint64_t*)(p + cap * 8);
    uint32_t* idx = (uint32_t*)(p + cap * 8 + m * 8);
    uint32_t* words = (uint32_t*)(p + cap * 8 + m * 8 + n * 4);
    unsigned long long* count = (unsigned long long*)(p + cap * 8 + m * 8 + n * 8);
    int* flags = (int*)(count + 1);
    cudaMemsetAsync(table, 0xff, cap * 8, stream);
    cudaMemsetAsync(count, 0, 16, stream);
    insert_kernel<T><<<blocks(n, 256), 256, 0, stream>>>(d_in, n, table, cap - 1, flags);
    compact_kernel<<<blocks(cap, 256), 256, 0, stream>>>(table, cap, keys, count);
    unsigned long long d = 0;
    int hflags = 0;
    cudaMemcpyAsync(&d, count, 8, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(&hflags, flags, 4, cudaMemcpyDeviceToHost, stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        *err = cudaGetErrorString(e);
        return 1;
    }
    if (hflags & 2) {
        *err = "dictionary hash table overflow";
        return 4;
    }
    size_t md = 1;
    while (md < d) md <<= 1;
    if (md > d) cudaMemsetAsync(keys + d, 0xff, (md - d) * 8, stream);
    if (md <= 8192) {
        e = cudaFuncSetAttribute(bitonic_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 8192 * 8);
        if (e != cudaSuccess) {
            *err = cudaGetErrorString(e);
            return 1;
        }
        bitonic_smem_kernel<<<1, 1024, md * 8, stream>>>(keys, (int)md);
    } else {
        for (size_t k = 2; k <= md; k <<= 1)
            for (size_t j = k >> 1; j > 0; j >>= 1)
                bitonic_global_kernel<<<blocks(md, 256), 256, 0, stream>>>(keys, md, k, j);
    }
    index_kernel<T><<<blocks(n, 256), 256, 0, stream>>>(d_in, n, keys, d, idx);
    const int bits = dict_bits((unsigned long)d);
    const int per_word = (int)floor(32 / (double)bits);
    const unsigned long nw = (unsigned long)ceil(n / (double)per_word);
    if (*n_words < nw) {
        *err = "numWordOutData < numWordCompressed";
        return 4;
    }
    pack_kernel<<<blocks(nw, 256), 256, 0, stream>>>(idx, n, bits, per_word, nw, words);
    std::vector<uint64_t> hk(d);
    cudaMemcpyAsync(h_words, words, nw * 4, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(hk.data(), keys, d * 8, cudaMemcpyDeviceToHost, stream);
    /* a launch refused for its configuration is reported here, not by the
     * synchronisation */
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        *err = cudaGetErrorString(e);
        return 1;
    }
    for (size_t i = 0; i < d; ++i) h_dict[i] = KeyOf<T>::value(hk[i], (hflags & 1) != 0);
    *n_dict = (unsigned long)d;
    *n_words = nw;
    return 0;
}

/* ---- the same codec over caller-provided scratch, with no allocation ---- */

namespace {

template <class T> __device__ T dev_value(uint64_t k, bool negzero);
template <> __device__ char dev_value<char>(uint64_t k, bool) { return (char)(signed char)((int64_t)k - 128); }
template <> __device__ int dev_value<int>(uint64_t k, bool) { return (int)((int64_t)k - 2147483648LL); }
template <> __device__ unsigned int dev_value<unsigned int>(uint64_t k, bool) { return (unsigned int)k; }
template <> __device__ double dev_value<double>(uint64_t k, bool negzero) {
    uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
    if (b == 0 && negzero) b = 0x8000000000000000ULL;
    return __longlong_as_double((long long)b);
}

template <class T>
__global__ void values_kernel(const uint64_t* __restrict__ keys, size_t d, const int* __restrict__ flags,
                              T* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d) out[i] = dev_value<T>(keys[i], (*flags & 1) != 0);
}

size_t round256(size_t b) { return (b + 255) / 256 * 256; }

void static_layout(size_t n, size_t elem, size_t* cap, size_t* m, size_t offs[7]) {
    *cap = 1;
    while (*cap < 2 * n) *cap <<= 1;
    *m = 1;
    while (*m < n) *m <<= 1;
    offs[0] = 0;                                   /* input values */
    offs[1] = offs[0] + round256(n * elem);        /* hash table [cap] */
    offs[2] = offs[1] + round256(*cap * 8);        /* sorted keys [m] */
    offs[3] = offs[2] + round256(*m * 8);          /* indices [n] */
    offs[4] = offs[3] + round256(n * 4);           /* packed words [n] */
    offs[5] = offs[4] + round256(n * 4);           /* count, flags */
    offs[6] = offs[5] + 256;                       /* dictionary values [n] */
}

}  // namespace

size_t dict_static_bytes(size_t n, size_t elem) {
    size_t cap, m, offs[7];
    static_layout(n, elem, &cap, &m, offs);
    return offs[6] + round256(n * elem);
}

template <class T>
int dict_compress_prealloc(const T* h_in, size_t n, void* d_scratch, size_t scratch_bytes, cudaStream_t stream,
                           uint32_t* h_words, unsigned long* n_words, T* h_dict, unsigned long* n_dict) {
    if (*n_dict < n) return 4;
    if (n == 0) {
        *n_dict = 0;
        *n_words = 0;
        return 0;
    }
    size_t cap, m, offs[7];
    static_layout(n, sizeof(T), &cap, &m, offs);
    if (offs[6] + round256(n * sizeof(T)) > scratch_bytes) return 4;
    uint8_t* p = (uint8_t*)d_scratch;
    T* in = (T*)(p + offs[0]);
    uint64_t* table = (uint64_t*)(p + offs[1]);
    uint64_t* keys = (uint64_t*)(p + offs[2]);
    uint32_t* idx = (uint32_t*)(p + offs[3]);
    uint32_t* words = (uint32_t*)(p + offs[4]);
    unsigned long long* count = (unsigned long long*)(p + offs[5]);
    int* flags = (int*)(count + 1);
    T* vals = (T*)(p + offs[6]);
    cudaError_t e = cudaMemcpyAsync(in, h_in, n * sizeof(T), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(table, 0xff, cap * 8, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, 16, stream);
    if (e != cudaSuccess) {
        (void)cudaStreamSynchronize(stream);
        return 1;
    }
    insert_kernel<T><<<blocks(n, 256), 256, 0, stream>>>(in, n, table, cap - 1, flags);
    compact_kernel<<<blocks(cap, 256), 256, 0, stream>>>(table, cap, keys, count);
    /* every return after work was queued waits for the stream first, so
     * that no kernel of this call still uses the scratch when it returns */
    auto fail = [&](int rc) {
        (void)cudaStreamSynchronize(stream);
        return rc;
    };
    unsigned long long d = 0;
    int hflags = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&d, count, 8, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hflags, flags, 4, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(1);
    if (hflags & 2) return 4;
    /* the word count follows from the distinct count: check the caller's
     * capacity before anything more is queued */
    const int bits = dict_bits((unsigned long)d);
    const int per_word = (int)floor(32 / (double)bits);
    const unsigned long nw = (unsigned long)ceil(n / (double)per_word);
    if (*n_words < nw) return 4;
    size_t md = 1;
    while (md < d) md <<= 1;
    if (md > d && cudaMemsetAsync(keys + d, 0xff, (md - d) * 8, stream) != cudaSuccess) return fail(1);
    if (md <= 8192) {
        if (cudaFuncSetAttribute(bitonic_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 8192 * 8) !=
            cudaSuccess)
            return fail(1);
        bitonic_smem_kernel<<<1, 1024, md * 8, stream>>>(keys, (int)md);
    } else {
        for (size_t k = 2; k <= md; k <<= 1)
            for (size_t j = k >> 1; j > 0; j >>= 1)
                bitonic_global_kernel<<<blocks(md, 256), 256, 0, stream>>>(keys, md, k, j);
    }
    index_kernel<T><<<blocks(n, 256), 256, 0, stream>>>(in, n, keys, d, idx);
    pack_kernel<<<blocks(nw, 256), 256, 0, stream>>>(idx, n, bits, per_word, nw, words);
    values_kernel<T><<<blocks(d, 256), 256, 0, stream>>>(keys, d, flags, vals);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_words, words, nw * 4, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_dict, vals, d * sizeof(T), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(1);
    *n_dict = (unsigned long)d;
    *n_words = nw;
    return 0;
}

template int dict_compress_prealloc<char>(const char*, size_t, void*, size_t, cudaStream_t, uint32_t*,
                                          unsigned long*, char*, unsigned long*);
template int dict_compress_prealloc<int>(const int*, size_t, void*, size_t, cudaStream_t, uint32_t*, unsigned long*,
                                         int*, unsigned long*);
template int dict_compress_prealloc<unsigned int>(const unsigned int*, size_t, void*, size_t, cudaStream_t,
                                                  uint32_t*, unsigned long*, unsigned int*, unsigned long*);
template int dict_compress_prealloc<double>(const double*, size_t, void*, size_t, cudaStream_t, uint32_t*,
                                            unsigned long*, double*, unsigned long*);

template int dict_compress_device<char>(const char*, size_t, void*, size_t, cudaStream_t, uint32_t*, unsigned long*,
                                        char*, unsigned long*, std::string*);
template int dict_compress_device<int>(const int*, size_t, void*, size_t, cudaStream_t, uint32_t*, unsigned long*,
                                       int*, unsigned long*, std::string*);
template int dict_compress_device<unsigned int>(const unsigned int*, size_t, void*, size_t, cudaStream_t, uint32_t*,
                                                unsigned long*, unsigned int*, unsigned long*, std::string*);
template int dict_compress_device<double>(const double*, size_t, void*, size_t, cudaStream_t, uint32_t*,
                                          unsigned long*, double*, unsigned long*, std::string*);

}  // namespace gsnp
