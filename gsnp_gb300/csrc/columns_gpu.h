/*
 * columns_gpu.h - the -C writer with its window encoding on the GPU
 * (columns_gpu.cu).
 */
#ifndef GSNP_COLUMNS_GPU_H
#define GSNP_COLUMNS_GPU_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "columns.h"
#include "gsnp_device.cuh"
#include "plan.h"

namespace gsnp {

struct ColumnsGpuStats {
    int64_t windows = 0;        /* windows encoded */
    int64_t host_windows = 0;   /* of which left to the host encoder */
};

/* Write the six -C files <base>.1_2 ... <base>.15_17 of the plan's windows,
 * byte for byte as write_columns does, encoding the windows on the current
 * device from the resident site codes, calls and (for windows that show
 * another window's counts) side counts, on `stream`.  h_codes: the site codes
 * on the host, for windows left to the host encoder.  Returns 0, or 1 with
 * *err set. */
int write_columns_gpu(const WindowPlan& plan, const uint8_t* d_codes, const SiteCall* d_calls,
                      const SiteCounts* d_counts, const uint8_t* h_codes, const char* chr_name,
                      const std::string& base, cudaStream_t stream, int threads, ColumnsGpuStats* st,
                      std::string* err);

/* One window of the -C files encoded on the host (the encoder of
 * write_columns): len rows whose site codes and calls are codes_w and
 * calls_w; mode 0: the rows show their own counts, 1: those of counts_w (the
 * window the reference's host arrays held), -1: zeros.  The five binary
 * blocks land in parts[0..5) in the order .3_4_6, .5_7_8_9_14_16, .10,
 * .11_12_13, .15_17. */
bool encode_window_host(int64_t len, int mode, const uint8_t* codes_w, const SiteCall* calls_w,
                        const SiteCounts* counts_w, const DictCodec& dict, std::string* parts, std::string* err);

}  // namespace gsnp

#endif
