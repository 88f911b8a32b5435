/*
 * dict.h - the -C dictionary codec on the device (see dict.cu).
 */
#ifndef GSNP_DICT_H
#define GSNP_DICT_H

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>

namespace gsnp {

/* bits per dictionary index for a dictionary of n values: the reference's
 * (int)ceil(log(n)/log(2)) with the C library's log, at least 1 */
int dict_bits(unsigned long n);

/* device scratch needed to compress n values */
size_t dict_scratch_bytes(size_t n);

/* Compress n device values: writes the packed index words and the ascending
 * distinct values to host memory.  *n_words and *n_dict hold capacities on
 * entry and counts on return, as cuda_dictCompression's do.  Returns 0, or a
 * GSNP_ERR_* code with *err set. */
template <class T>
int dict_compress_device(const T* d_in, size_t n, void* d_scratch, size_t scratch_bytes, cudaStream_t stream,
                         uint32_t* h_words, unsigned long* n_words, T* h_dict, unsigned long* n_dict,
                         std::string* err);

/* The same codec with host input and outputs over caller-provided device
 * scratch of at least dict_static_bytes(n, sizeof(T)) bytes; it allocates
 * nothing on the device or the host.  Returns 0, 1 (CUDA error) or 4
 * (capacity). */
size_t dict_static_bytes(size_t n, size_t elem);

template <class T>
int dict_compress_prealloc(const T* h_in, size_t n, void* d_scratch, size_t scratch_bytes, cudaStream_t stream,
                           uint32_t* h_words, unsigned long* n_words, T* h_dict, unsigned long* n_dict);

}  // namespace gsnp

#endif
