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

struct WindowPlan {
    int64_t n_windows = 0;
    std::vector<int64_t> call_len;   /* sites called in window w */
    std::vector<int32_t> host_src;   /* window whose pileup the host count arrays hold, -1: zeros */
    std::vector<int32_t> lik_src;    /* window whose likelihood is used, -1: never computed (zeros) */
    std::vector<uint8_t> flags;      /* kWin* flags for the kernels */
    std::vector<int64_t> deposited;  /* indices of the deposited alignments, in order */
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
};

/* Returns 0, or 5 (GSNP_ERR_UNSORTED) with *err set to the reference's message. */
int replay_windows(const ReadView& r, int64_t chr_len, int L, int qmin, WindowPlan* plan, std::string* err);

}  // namespace gsnp

#endif
