/*
 * rows.h - the fields of one cns row as the reference's host code prints
 * them (cpp/call_genotype.cc:353-411).
 *
 * A row combines the site's own call (type, bases, quality, rank-sum) with
 * the count columns of the window whose pileup the reference's host arrays
 * held when the site was called (WindowPlan::host_src): the site's own counts,
 * another window's counts at the same offset, or zeros.
 */
#ifndef GSNP_ROWS_H
#define GSNP_ROWS_H

#include <stdint.h>

#include "gsnp_device.cuh"
#include "plan.h"

namespace gsnp {

extern const char kAbbv[17];   /* genotype code -> IUPAC letter */
extern const char kActgN[9];   /* base code -> letter, N for 4..7 */

struct CnsRow {
    uint8_t ori;        /* 4-bit site code */
    bool nflag;         /* N reference base with no covering read */
    uint8_t type1, base1, base2;
    int q_cns;
    int avg1, cu1, ca1, avg2, cu2, ca2;
    uint32_t depth, repeat;
    double rank_sum;
    /* the row prints real values (otherwise the N literal) */
    GSNP_HDI bool called() const { return !nflag && base1 < 4; }
};

/* hs: the window whose host counts the reference shows for window w */
GSNP_HDI CnsRow make_row(int32_t hs, int64_t w, int64_t j, const uint8_t* codes, const SiteCall* calls,
                         const SiteCounts* counts) {
    const int64_t site = w * (int64_t)kWin + j;
    const SiteCall& c = calls[site];
    CnsRow r;
    r.ori = codes[site];
    r.type1 = c.type1;
    r.base1 = c.base1;
    r.base2 = c.base2;
    r.q_cns = c.q_cns;
    r.rank_sum = c.rank_sum;
    r.depth = 0;
    r.repeat = 0;
    r.avg1 = r.cu1 = r.ca1 = r.avg2 = r.cu2 = r.ca2 = 0;
    if (hs == w) {
        r.depth = c.depth;
        r.repeat = c.repeat_time;
        r.cu1 = c.cu1; r.ca1 = c.ca1; r.avg1 = c.avg_q1;
        r.cu2 = c.cu2; r.ca2 = c.ca2; r.avg2 = c.avg_q2;
    } else if (hs >= 0) {
        const SiteCounts& k = counts[(int64_t)hs * kWin + j];
        r.depth = k.depth;
        r.repeat = k.repeat_time;
        if (c.base1 < 4) {
            r.cu1 = k.cu[c.base1]; r.ca1 = (int)k.ca[c.base1];
            r.avg1 = k.qs[c.base1] == 0 ? 0 : k.qs[c.base1] / k.cu[c.base1];
        }
        if (c.base2 < 4) {
            r.cu2 = k.cu[c.base2]; r.ca2 = (int)k.ca[c.base2];
            r.avg2 = k.qs[c.base2] == 0 ? 0 : k.qs[c.base2] / k.cu[c.base2];
        }
    }
    r.nflag = (r.ori & 4) && r.depth == 0;
    return r;
}

inline CnsRow resolve_row(const WindowPlan& plan, int64_t w, int64_t j, const uint8_t* codes,
                          const SiteCall* calls, const SiteCounts* counts) {
    return make_row(plan.host_src[w], w, j, codes, calls, counts);
}

}  // namespace gsnp

#endif
