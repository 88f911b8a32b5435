/*
 * emit.h - cns text rows on the device (emit.cu).
 */
#ifndef GSNP_EMIT_H
#define GSNP_EMIT_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "gsnp_device.cuh"

namespace gsnp {

struct EmitArgs {
    const SiteCall* calls;      /* [chr_len] */
    const SiteCounts* counts;   /* [chr_len] or null */
    const uint8_t* codes;       /* [chr_len] */
    const int32_t* host_src;    /* [n_windows] window whose host counts each window shows */
    const char* chr;            /* chromosome name (device) */
    int chr_n;
    int64_t site0, n;           /* rows of sites [site0, site0 + n) */
    uint32_t* len;              /* scratch: row lengths */
    uint64_t* off;              /* scratch: byte offsets */
    char* text;                 /* output of emit_text */
    int* error;                 /* set when a value is outside the formatter's range */
};

/* device scratch of emit_lengths for n rows */
size_t emit_scratch_bytes(int64_t n);

/* Row lengths and offsets of e's rows in scratch (sets e.len, e.off);
 * *h_total receives the byte count of the rows' text.  Synchronises. */
cudaError_t emit_lengths(EmitArgs& e, void* scratch, cudaStream_t stream, uint64_t* h_total);

/* Write the rows' text to e.text (after emit_lengths). */
cudaError_t emit_text(const EmitArgs& e, cudaStream_t stream);

}  // namespace gsnp

#endif
