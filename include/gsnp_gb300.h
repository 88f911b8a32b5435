/*
 * gsnp_gb300.h - C ABI of the GB300 consensus caller.
 *
 * Plain C types only: pointers, sizes and status codes.  Every function returns
 * GSNP_OK (0) on success or a GSNP_ERR_* code; gsnp_context_error() then holds
 * a one-line message.  Host pointers are read and written synchronously; the
 * device state lives in the context until gsnp_context_destroy().
 *
 * Two ways in:
 *   1. Whole chromosome (this library): gsnp_load_reference,
 *      gsnp_calibrate, gsnp_load_tables, gsnp_call_chromosome, then
 *      gsnp_fetch_sites, gsnp_write_cns / gsnp_format_cns or
 *      gsnp_write_columns.  One call replaces the reference's window loop
 *      Call_win::new_soap2cns (cpp/call_genotype.cc:422-669) and, per window,
 *      cuda_updateSparse / cuda_likelihoodSparse / cuda_posterior
 *      (kernel/update_kernel.cu:328, kernel/likelihood_kernel.cu:262,
 *      kernel/posterior_kernel.cu:867).  The reference's window quirks (stale
 *      host arrays in gap windows, the dropped last read, the reused
 *      likelihood) are reproduced, so the output bytes are the reference's.
 *   2. Window by window, the reference's own entry points, declared with
 *      their original C++ names in gsnp_backend.h and implemented with the
 *      window state resident on the device in a separate library,
 *      libgsnp_backend.so (gsnp_gb300/csrc/compat.cu).
 */
#ifndef GSNP_GB300_H
#define GSNP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSNP_OK 0
#define GSNP_ERR_CUDA 1        /* a CUDA call failed */
#define GSNP_ERR_ARG 2         /* bad argument */
#define GSNP_ERR_STATE 3       /* call out of order (e.g. no tables loaded) */
#define GSNP_ERR_CAPACITY 4    /* an input exceeds a stated limit */
#define GSNP_ERR_UNSORTED 5    /* alignments not sorted by position (the reference exits 255) */
#define GSNP_ERR_INPUT 6       /* invalid input (read longer than -L, bad base, unreadable file) */
#define GSNP_ERR_MISMATCH 7    /* gsnp_check_columns found a differing row */

#define GSNP_PRECISION_FP64 0        /* likelihood summed in FP64, in the reference's order */
#define GSNP_PRECISION_FP32_FIXUP 1  /* FP32 compensated sums, FP64 recomputation near ties */

typedef struct gsnp_context gsnp_context;

/* Calling parameters (cpp/common.h:123-154 Parameter). */
typedef struct gsnp_params {
    int read_length;          /* -L, at most 255 */
    int q_min;                /* quality char meaning 0 (-z), as a signed char */
    int q_max;                /* highest calibrated quality char (-Q) */
    double pcr_dependency;    /* log10 of -p */
    double global_dependency; /* log10 of -g */
    double het_val;           /* validated dbSNP HET prior (-b) */
    double het_unval;         /* unvalidated dbSNP HET prior (-k) */
    double althom_val;        /* validated dbSNP altHOM prior (-a) */
    double althom_unval;      /* unvalidated dbSNP altHOM prior (-j) */
    int rank_sum;             /* -u */
    int monoploid;            /* -m */
    int refine;               /* -2 */
    int precision;            /* GSNP_PRECISION_* */
    double het_novel;         /* novel HET prior (-e) */
    double althom_novel;      /* novel altHOM prior (-r) */
    int transition_dominant;  /* -t */
} gsnp_params;

/* One dbSNP row (cpp/soap_snp.h:714-760 Snp_info), position 0-based. */
typedef struct gsnp_snp {
    uint32_t pos;
    uint8_t validated, hapmap, indel, pad;
    double freq[4];           /* A, C, T, G */
} gsnp_snp;

/* Alignments of one chromosome in file order (cpp/soap_snp.h:119-201):
 * bases and qualities at a fixed pitch of read_length bytes per read. */
typedef struct gsnp_reads {
    int64_t n;
    const int32_t* pos;       /* 0-based start */
    const int32_t* len;       /* read length */
    const int32_t* hit;       /* number of hits */
    const uint8_t* strand;    /* '+' or '-' */
    const uint8_t* seq;       /* [n][pitch] base chars */
    const uint8_t* qual;      /* [n][pitch] quality chars */
    int32_t pitch;
    /* Optional, in place of seq and qual (NULL: not used): [n][pitch] bytes
     * of gsnp_pack_reads, base and quality in one byte, which halves the
     * bytes a call uploads; packed_qmin is the q_min they were packed with
     * and must equal the tables' (GSNP_ERR_ARG otherwise). */
    const uint8_t* packed;
    int32_t packed_qmin;
} gsnp_reads;

/* No counterpart in the reference.  Pack the bases and qualities of n reads
 * ([n][pitch] each, len[i] positions of read i used) into out ([n][pitch]
 * bytes) for gsnp_reads.packed: base A C T G (either case) as 0 1 2 3 in bits
 * 7:6, quality - q_min in bits 5:0, and 63 in bits 5:0 for a quality below
 * q_min (a base the caller skips in the pileup, the calibration and the
 * window replay alike); positions past a read's length are 0.  Runs on up to
 * `threads` host threads (0: all).  GSNP_ERR_INPUT for another base, as the
 * calls do, or for a quality above q_min + 62, which has no code (pass seq and
 * qual then). */
int gsnp_pack_reads(const uint8_t* seq, const uint8_t* qual, const int32_t* len, int64_t n, int32_t pitch, int q_min,
                    uint8_t* out, int threads);

/* Per-site call (32 bytes), the binary form of one cns row. */
typedef struct gsnp_site_call {
    uint8_t type1, base1, base2, q_cns;
    uint8_t avg_q1, avg_q2, flags, pad;
    uint16_t cu1, ca1, cu2, ca2;
    uint32_t depth, repeat_time;
    double rank_sum;
} gsnp_site_call;

/* Select device `device` and create a context (replaces GPUInit,
 * kernel/gsnp_kernel.cu:20-22). */
int gsnp_context_create(int device, gsnp_context** out);
void gsnp_context_destroy(gsnp_context* ctx);
const char* gsnp_context_error(const gsnp_context* ctx);

/* Run the context's work on this cudaStream_t (default: a stream it owns). */
int gsnp_set_stream(gsnp_context* ctx, void* stream);

/* Calibration, prior and rank-sum tables in the reference's layouts:
 * p_matrix[256*256*16] (cpp/matrix.cc:4), p_prior[8*16] (cpp/prior.cc:3),
 * p_rank[64*64*2048] (cpp/rank_sum.cc:3).  Replaces GSNPKernelInit
 * (kernel/gsnp_kernel.cu:24-33): the materialised log10 table and the
 * adjusted-quality table are built here once. */
int gsnp_load_tables(gsnp_context* ctx, const gsnp_params* params, const double* p_matrix,
                     const double* p_prior, const double* p_rank);

/* Reference of the called chromosome: one 4-bit site code per byte
 * (bit 3 dbSNP, bit 2 N, bits 1:0 base ACTG; cpp/chromosome.cc:28-64) and its
 * dbSNP rows: one row per flagged site, ascending by position, as the
 * reference's loader builds them (cpp/chromosome.cc:197-216).  Rows that do
 * not match the flags are GSNP_ERR_ARG. */
int gsnp_load_reference(gsnp_context* ctx, const uint8_t* site_codes, int64_t length, const gsnp_snp* snp,
                        int64_t n_snp);

/* Pass-1 calibration (cpp/matrix.cc:42-213): count every unique base of the
 * alignments on the device by (quality, cycle, reference base, observed base)
 * and fill the calibration matrix p_matrix[256*256*16] on the host.  The
 * reference must be loaded. */
int gsnp_calibrate(gsnp_context* ctx, const gsnp_params* params, const gsnp_reads* reads, double* p_matrix);

/* Novel genotype priors p_prior[8*16] (cpp/prior.cc:3-43). */
int gsnp_prior_table(const gsnp_params* params, double* p_prior);

/* Exact Wilcoxon rank-sum table p_rank[64*64*2048] (cpp/rank_sum.cc:3-42). */
int gsnp_rank_table(double* p_rank);

/* Call every site of the chromosome from its alignments (host buffers).
 * Reads with pos < 0 or pos + len >= length are skipped, an unsorted input is
 * GSNP_ERR_UNSORTED, and the reference's window semantics are reproduced. */
int gsnp_call_chromosome(gsnp_context* ctx, const gsnp_reads* reads);

/* gsnp_call_chromosome followed by the download of every site's call into
 * out (one gsnp_site_call per site of the chromosome).  The chromosome is
 * called in window-aligned segments, so that the upload of the alignments,
 * the calling and the download of the calls overlap; out should be pinned
 * host memory for the downloads to overlap.  The results equal those of
 * gsnp_call_chromosome + gsnp_fetch_sites, which remain available. */
int gsnp_call_chromosome_into(gsnp_context* ctx, const gsnp_reads* reads, gsnp_site_call* out);

/* The chromosome-scale form of gsnp_call_chromosome_into
 * (cpp/call_genotype.cc:422-669 streams the genome through its window the
 * same way): the chromosome is called in chunks of "stream_windows" windows
 * of 262,144 sites (gsnp_set_option, default 16), and the device holds only
 * two chunks' alignments and calls at a time, so that its memory is set by the
 * chunk size and the depth, not by the chromosome's length (the site codes,
 * one byte per site, and the tables stay resident).  While chunk k is called,
 * chunk k + 1's alignments are uploaded; each chunk's results then go to the
 * outputs that are given (any may be NULL):
 *   out           every site's call, as gsnp_call_chromosome_into;
 *   cns_path      the cns text of every site (gsnp_write_cns's bytes);
 *   columns_base  the six -C files (gsnp_write_columns's bytes).
 * chr_name is needed for the two files.  The results equal the resident
 * call's; afterwards no call stays resident (gsnp_fetch_sites, gsnp_write_cns
 * and gsnp_write_columns answer GSNP_ERR_STATE until the next resident call). */
int gsnp_call_streamed(gsnp_context* ctx, const gsnp_reads* reads, const char* chr_name, gsnp_site_call* out,
                       const char* cns_path, const char* columns_base);

/* No counterpart in the reference.  Device bytes a streamed call holds
 * besides the per-site reference codes and the tables: the chunk ring of the
 * last gsnp_call_streamed, and the -C writer's batch buffers (also used by
 * gsnp_write_columns). */
int gsnp_stream_footprint(gsnp_context* ctx, uint64_t* ring_bytes, uint64_t* writer_bytes);

/* Re-run the calling kernels on the alignments already resident on the device
 * (no host transfer); used to time the kernels alone. */
int gsnp_recall_resident(gsnp_context* ctx);

/* No counterpart in the reference (its launch configuration is fixed at
 * build time).  Set a launch option of the context; the next calling pass
 * uses it.  Names and values:
 *   persistent            FP32 form: 1 the persistent region-ordered kernel
 *                         with the binned kernels for the tiles it leaves,
 *                         0 the depth-binned kernels only
 *   persistent_slots      48 or 64 record slots of the persistent kernel
 *   persistent_mode       0 read loads, 1 after a bulk L2 prefetch of the
 *                         next tile's rows, 2 rows staged in shared memory by
 *                         bulk copies
 *   persistent_carveout   preferred shared-memory carveout, percent (0: the
 *                         default)
 *   fast_carveout_<S>, fp64_carveout_<S>   the same for the S-slot bin of the
 *                         FP32 / FP64 binned kernel (S = 32 40 48 64 96 128 256)
 *   bin_limit_<S>         deepest column the S-slot bin takes (at most S)
 *   device_driven         1: launch sizes read on the device, no host wait
 *                         inside a pass; 0: the host reads each bin's count
 *   graphs                1: gsnp_recall_resident replays a CUDA graph
 *   upload_streams        copy streams of the upload (1-4; before the first
 *                         call only)
 *   columns_gpu           1: gsnp_write_columns encodes the windows on the
 *                         GPU; 0: on the host threads (same bytes)
 *   stream_windows        windows per chunk of gsnp_call_streamed (1 and up)
 * GSNP_ERR_ARG for an unknown name or bin.  The environment variable
 * GSNP_OPTIONS="name=value,..." sets options when a context is created, after
 * the "name value" lines of the file GSNP_TUNE_FILE names (gsnp_tune). */
int gsnp_set_option(gsnp_context* ctx, const char* name, int64_t value);

/* No counterpart in the reference.  The launch autotuner: times the calling
 * pass of the resident reads of the last call over a sample of
 * `sample_windows` windows (from a third of the way along the chromosome)
 * with candidate launch settings, and keeps the fastest:
 *   - each binned kernel's shared-memory carveout (0, 58, 72, 86%), per bin;
 *   - the column-depth limits of the two shallowest bins;
 *   - for the FP32 form, the persistent kernel's record slots (48, 64),
 *     carveout (0, 72, 86%) and read mode (loads, L2 prefetch), and whether
 *     it or the binned kernels alone call the FP32 windows.
 * The chosen settings are written to `report` as "name value" lines (the
 * gsnp_set_option names), followed by the measurements as "#"-led and plain
 * lines; when GSNP_TUNE_FILE is set the option lines are written to that file,
 * which contexts created later load.  The sample's calls are recomputed with
 * the same results.  GSNP_ERR_STATE before a finished call. */
int gsnp_tune(gsnp_context* ctx, int sample_windows, char* report, size_t report_cap);

/* Copy calls for sites [first, first + count) to host memory. */
int gsnp_fetch_sites(gsnp_context* ctx, int64_t first, int64_t count, gsnp_site_call* out);

/* Format the cns text of the whole chromosome (cpp/call_genotype.cc:353-411)
 * on the device.  With buf == NULL, *size receives the number of bytes;
 * otherwise up to *size bytes are written and *size receives the count. */
int gsnp_format_cns(gsnp_context* ctx, const char* chr_name, char* buf, int64_t* size);

/* Write the cns text of the whole chromosome to the file at path, formatted
 * on the device chunk by chunk. */
int gsnp_write_cns(gsnp_context* ctx, const char* chr_name, const char* path);

/* Write the -C compressed output of the last call (cpp/compress.h:86-1312,
 * written by cpp/call_genotype.cc:440-452,616-660): the six files
 * <base_path>.1_2, .3_4_6, .5_7_8_9_14_16, .10, .11_12_13 and .15_17, byte for
 * byte as the reference writes them, the dictionary codec running on the
 * device.  With chr_name == NULL the files a text-mode run leaves are written
 * instead (.1_2 holding "0", the others empty). */
int gsnp_write_columns(gsnp_context* ctx, const char* chr_name, const char* base_path);

/* The cns rows of the -C files <base>.1_2 ... <base>.15_17, written to
 * out_path exactly as the reference's decompressor prints them
 * (cpp/decompression.cpp:130-232: its N-site literal, %#.6g doubles), decoded
 * on `threads` host threads (<= 0: all).  Needs no context or GPU.  Returns
 * GSNP_OK or GSNP_ERR_INPUT with the reason in err. */
int gsnp_decompress_columns(const char* base, const char* out_path, int threads, char* err, int err_len);

/* The reference decompressor's check (cpp/decompression.cpp:236-401): every
 * row of the cns text at cns_path against the -C files at base, characters
 * and integers exactly, the two double columns within 1e-5.  GSNP_OK when
 * every row matches, GSNP_ERR_MISMATCH with the first difference in report,
 * GSNP_ERR_INPUT when a file cannot be read. */
int gsnp_check_columns(const char* cns_path, const char* base, char* report, int report_len);

/* One kernel launch of the last calling pass, timed with CUDA events on the
 * context's stream. */
typedef struct gsnp_launch_info {
    int kind;          /* 0: tile classification; calling kernel of one depth bin: 1 FP64,
                          2 FP32 fast form, 6 FP32 fast form with one warp per site (the deep
                          bins); 3 FP64 pass over the fast form's deferred sites; 4 the
                          persistent FP32 kernel; 5 a whole pass replayed as a CUDA graph */
    int slots;         /* record slots per site of the bin (calling kernels) */
    int64_t tiles;     /* 32-site tiles processed (0 when the count is read on the device) */
    int64_t sites;
    float ms;          /* device time of the launch */
} gsnp_launch_info;

/* Launches of the last calling pass: copies up to *n entries, sets *n to the
 * number of launches. */
int gsnp_last_launches(gsnp_context* ctx, gsnp_launch_info* out, int* n);

/* Host-to-device bytes of the last gsnp_call_chromosome and device-to-host
 * bytes fetched since then. */
int gsnp_transfer_bytes(gsnp_context* ctx, uint64_t* h2d, uint64_t* d2h);

/* Diagnostics of the last call, n entries:
 *   [0] sites called
 *   [1] sites whose FP32 likelihood was recomputed in FP64 (fixups)
 *   [2] sites whose FP32 likelihood was also summed in FP64 (every 4096th)
 *   [3] the largest |FP32 - FP64| type_likely difference over those sites
 *       (raw bits of a double)
 *   [4] sites the FP32 kernel deferred to the FP64 pass (heterozygous calls,
 *       which need the FP64 rank-sum, and calls its FP32 bounds did not prove)
 *   [5] sampled sites whose FP32-kernel call differs from the FP64 call
 *       (always 0 unless the error bound is wrong)
 *   [6], [7] reserved, 0 */
int gsnp_get_stats(gsnp_context* ctx, uint64_t* stats, int n);

/* Element types of gsnp_dict_compress_static */
#define GSNP_DICT_CHAR 0
#define GSNP_DICT_INT 1
#define GSNP_DICT_UINT32 2
#define GSNP_DICT_DOUBLE 3

/* No counterpart in the reference.  The -C dictionary codec (the contract of
 * cuda_dictCompression, cpp/dict_compression.h:26-37: dict = the distinct
 * values ascending, words = their indices packed MSB-first) for callers that
 * cannot allocate device memory on their path - a process whose free device
 * memory is held by another allocator, or a streaming writer that must not
 * call cudaMalloc/cudaFree because they synchronise the device.  Its scratch
 * is a static device array of 12.6 MB, so it takes at most 262,144 values
 * (32 x 8192, the reference's dictionary capacity); larger inputs return
 * GSNP_ERR_CAPACITY without touching the device.  values: n host values of
 * the given GSNP_DICT_* type.  *n_words and *n_dict hold the capacities of
 * words and dict on entry and the counts on return; as with
 * cuda_dictCompression, dict must have room for n values (not just the
 * distinct ones), else the call returns GSNP_ERR_CAPACITY, as it does when
 * words is too small for the packed indices.  Runs on the current device and
 * the given cudaStream_t (NULL: the legacy default stream) and returns, on
 * success and on error, once its work on that stream is done.
 * The scratch is reserved on a device by the first call there (CUDA loads the
 * library's device code lazily): make one call first - n = 0 does only that
 * set-up - before another allocator takes the free memory, and before any
 * stream capture.  Do not call it on a device after cudaDeviceReset.  Every
 * call clears the scratch it needs on the stream; calls that overlap on one
 * GPU race and must be serialised. */
int gsnp_dict_compress_static(int type, const void* values, uint64_t n, uint32_t* words, uint64_t* n_words,
                              void* dict, uint64_t* n_dict, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GSNP_GB300_H */
