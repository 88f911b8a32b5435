/*
 * columns_gpu.h - the -C writer with its window encoding on the GPU
 * (columns_gpu.cu).
 */
#ifndef GSNP_COLUMNS_GPU_H
#define GSNP_COLUMNS_GPU_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdio.h>

#include <future>
#include <memory>
#include <string>
#include <vector>

#include "columns.h"
#include "gsnp_device.cuh"
#include "plan.h"

namespace gsnp {

struct ColumnsGpuStats {
    int64_t windows = 0;        /* windows encoded */
    int64_t host_windows = 0;   /* of which left to the host encoder */
};

/* The six -C files <base>.1_2 ... <base>.15_17 of a plan's windows, byte
 * for byte as write_columns writes them, with the windows encoded on the
 * current device: open() creates the files and writes .1_2; write() appends
 * windows [w0, w1), each call continuing where the last ended, from site
 * codes, calls and counts indexed by absolute site, and each window's host
 * count source (WindowPlan::host_src, remapped as the counts are) on the
 * device and on the host; close() ends the files.  The device buffers of a
 * batch of windows stay allocated from one use to the next.  h_codes: the
 * site codes on the host, for windows left to the host encoder.  Each call
 * returns 0, or 1 with *err set. */
class ColumnsGpuWriter {
public:
    ColumnsGpuWriter() = default;
    ColumnsGpuWriter(const ColumnsGpuWriter&) = delete;
    ColumnsGpuWriter& operator=(const ColumnsGpuWriter&) = delete;
    ~ColumnsGpuWriter();
    int open(const WindowPlan& plan, const char* chr_name, const std::string& base, int64_t batch, std::string* err);
    int write(int64_t w0, int64_t w1, const uint8_t* d_codes, const SiteCall* d_calls, const SiteCounts* d_counts,
              const int32_t* d_host_src, const int32_t* h_host_src, const uint8_t* h_codes, cudaStream_t stream,
              ColumnsGpuStats* st, std::string* err);
    int close(std::string* err);
    /* device bytes held between uses */
    size_t device_bytes() const;

private:
    void release();
    const WindowPlan* plan_ = nullptr;
    int64_t next_window_ = 0;
    FILE* fb_[5] = {};
    FILE* f12_ = nullptr;
    int64_t batch_cap_ = 0, len_tab_windows_ = 0;
    uint8_t* d_out_[5] = {};
    uint8_t* d_bits_ = nullptr;
    int64_t* d_len_tab_ = nullptr;
    uint64_t* d_len_ = nullptr;
    int* d_fb_ = nullptr;
    uint64_t *d_sval_ = nullptr, *d_sdict_ = nullptr;
    uint32_t* d_saux_ = nullptr;
    uint32_t* d_rle32_ = nullptr;
    uint64_t* d_rle64_ = nullptr;
    int* d_not_n_ = nullptr;
    /* two sets of pinned buffers, a batch's blocks of each file, used in
     * turn; the file writes of a batch run on their own threads, one per
     * file, each after the same file's previous batch */
    struct Piece {
        const char* p;
        size_t n;
        std::shared_ptr<std::string> own;   /* a host-encoded block */
    };
    bool wait_set(int set);
    char* hbuf_[2][5] = {};
    size_t hcap_[2][5] = {};
    int set_ = 0;
    std::shared_future<bool> last_[5];
    std::shared_future<bool> pend_[2][5];
};

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
