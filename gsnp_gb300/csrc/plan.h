/*
 * plan.h - host replay of the reference's window loop.
 *
 * The reference streams the genome through a 262,144-site window
 * (Call_win::new_soap2cns, cpp/call_genotype.cc:422-669) and its output
 * depends on that loop in three places:
 *   - gap windows (no read starts) print count columns from host arrays that
 *     cuda_recycle did not refresh (kernel/recycle_kernel.cu:91-136): they show
 *     the last refreshed window's counts at the same offset;
 *   - when a window's update found no record, the likelihood is not recomputed
 *     and the previous window's stays in device memory
 *     (kernel/likelihood_kernel.cu:269-274);
 *   - when the last alignment opens a new window it is never deposited
 *     (cpp/call_genotype.cc:525-585).
 * replay_windows() walks the alignments once and records, per window, where
 * those values come from, so the kernels can call every site in parallel.
 */
#ifndef GSNP_PLAN_H
#define GSNP_PLAN_H

#include <stdint.h>

#include <string>
#include <vector>

namespace gsnp {

/* a run of consecutive passing alignments that start in one window */
struct WindowRun {
    int64_t window;
    int64_t first;    /* index of its first alignment */
    int64_t count;    /* passing alignments in the run */
};

struct WindowPlan {
    int64_t n_windows = 0;
    std::vector<int64_t> call_len;   /* sites called in window w */
    std::vector<int32_t> host_src;   /* window whose pileup the host count arrays hold, -1: zeros */
    std::vector<int32_t> lik_src;    /* window whose likelihood is used, -1: never computed (zeros) */
    std::vector<uint8_t> flags;      /* kWin* flags for the kernels */
    std::vector<WindowRun> runs;     /* the runs of passing alignments, in order */
    int64_t n_valid = 0;             /* alignments that pass the position filters */
    int64_t n_deposited = 0;         /* the first n_deposited of those are deposited */
    int64_t skipped = 0;             /* alignments skipped by the position filters */
    bool dropped_last = false;       /* the last alignment was not deposited */
};

struct ReadView {
    int64_t n;
    const int32_t* pos;
    const int32_t* len;
    const int32_t* hit;
    const uint8_t* seq;
    const uint8_t* qual;
    int32_t pitch;
    /* gsnp_pack_reads's bytes in place of seq and qual when set (packed with
     * the replay's q_min: 63 in bits 5:0 is a quality below it) */
    const uint8_t* packed = nullptr;
};

/* An alignment passes the position filters when 0 <= pos and pos + len <
 * chr_len; those are deposited in file order, all but the last when
 * dropped_last.  Runs the per-alignment pass on up to `threads` threads.
 * Returns 0; 6 (GSNP_ERR_INPUT) when an alignment is longer than L or its
 * pitch, or when no alignment has a non-negative start; 5
 * (GSNP_ERR_UNSORTED) with the reference's message when the passing
 * alignments are not sorted by start. */
int replay_windows(const ReadView& r, int64_t chr_len, int L, int qmin, int threads, WindowPlan* plan,
                   std::string* err);

}  // namespace gsnp

#endif
