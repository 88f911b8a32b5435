/*
 * dict_static.cu - the -C dictionary codec with statically reserved scratch.
 *
 * For callers that cannot allocate device memory on their path: a process
 * whose free device memory is held by another allocator (a caching allocator
 * that reserved it), or a streaming writer that must not call cudaMalloc or
 * cudaFree, which synchronise the whole device and stall the work of other
 * streams.  The codec's scratch is a file-scope device array, sized for the
 * reference's dictionary capacity of 32 x 8192 values; nothing is allocated per
 * call, on the device or the host.
 *
 * The array is reserved on a device when this library's device code is loaded
 * there.  With CUDA's lazy module loading (the default) that happens on the
 * first call on the device, which looks up the array's device address with
 * cudaGetSymbolAddress (that device current) and keeps it.  So make one call
 * first - a call with n = 0 does only this set-up - before another allocator
 * takes the free device memory, and before any stream capture.  The kept
 * address does not survive cudaDeviceReset: do not use this entry point on a
 * device after resetting it.  Every call clears the parts of the scratch that
 * must start cleared (the hash table and the counters) on the caller's stream,
 * so nothing needs to be zero beforehand.  All calls on one device share the
 * one scratch array: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  Every return, errors
 * included, comes after the call's device work on that stream has finished.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "dict.h"
#include "gsnp_gb300.h"

namespace gsnp {
namespace {

constexpr uint64_t kStaticDictMax = 32ull * 8192ull;
/* dict_static_bytes(kStaticDictMax, 8): input, hash table, keys, indices,
 * words, counters and dictionary values */
constexpr size_t kStaticDictBytes = 12583168;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_dict_scratch[kStaticDictBytes];

std::mutex g_mutex;
void* g_scratch[kMaxDevices] = {};

}  // namespace
}  // namespace gsnp

using namespace gsnp;

extern "C" int gsnp_dict_compress_static(int type, const void* values, uint64_t n, uint32_t* words,
                                         uint64_t* n_words, void* dict, uint64_t* n_dict, void* stream) {
    if (!words || !n_words || !dict || !n_dict || (n > 0 && !values)) return GSNP_ERR_ARG;
    if (type < GSNP_DICT_CHAR || type > GSNP_DICT_DOUBLE) return GSNP_ERR_ARG;
    if (n > kStaticDictMax) return GSNP_ERR_CAPACITY;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GSNP_ERR_CUDA;
    void* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_scratch[dev]) {
            if (cudaGetSymbolAddress(&g_scratch[dev], g_dict_scratch) != cudaSuccess) {
                g_scratch[dev] = nullptr;
                return GSNP_ERR_CUDA;
            }
        }
        scratch = g_scratch[dev];
    }
    static_assert(sizeof(unsigned long) == sizeof(uint64_t), "LP64");
    unsigned long nw = (unsigned long)*n_words, nd = (unsigned long)*n_dict;
    const cudaStream_t s = (cudaStream_t)stream;
    int rc;
    switch (type) {
        case GSNP_DICT_CHAR:
            rc = dict_compress_prealloc<char>((const char*)values, n, scratch, kStaticDictBytes, s, words, &nw,
                                              (char*)dict, &nd);
            break;
        case GSNP_DICT_INT:
            rc = dict_compress_prealloc<int>((const int*)values, n, scratch, kStaticDictBytes, s, words, &nw,
                                             (int*)dict, &nd);
            break;
        case GSNP_DICT_UINT32:
            rc = dict_compress_prealloc<unsigned int>((const unsigned int*)values, n, scratch, kStaticDictBytes, s,
                                                      words, &nw, (unsigned int*)dict, &nd);
            break;
        default:
            rc = dict_compress_prealloc<double>((const double*)values, n, scratch, kStaticDictBytes, s, words, &nw,
                                                (double*)dict, &nd);
            break;
    }
    if (rc == 4) return GSNP_ERR_CAPACITY;
    if (rc != 0) return GSNP_ERR_CUDA;
    *n_words = nw;
    *n_dict = nd;
    return GSNP_OK;
}
