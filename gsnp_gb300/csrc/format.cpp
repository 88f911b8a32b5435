/*
 * format.cpp - cns text rows on the host (cpp/call_genotype.cc:353-411).
 *
 * The row of a site combines its own call (type, bases, quality, rank-sum)
 * with the count columns of the window the reference's host arrays held when
 * the site was called (plan.host_src): the site's own counts, another window's
 * counts at the same offset, or zeros.  Doubles are printed as the
 * reference's iostream with showpoint does: %#.6g.
 */
#include <cstdio>
#include <string>
#include <vector>

#include "gsnp_device.cuh"
#include "plan.h"

namespace gsnp {

namespace {

const char kAbbv[17] = {'A', 'M', 'W', 'R', 'M', 'C', 'Y', 'S', 'W', 'Y', 'T', 'K', 'R', 'S', 'K', 'G', 'N'};
const char* kActgN = "ACTGNNNN";

struct HostView {
    uint32_t depth = 0, repeat = 0;
    int cu1 = 0, ca1 = 0, avg1 = 0, cu2 = 0, ca2 = 0, avg2 = 0;
};

}  // namespace

int format_cns_host(const WindowPlan& plan, const std::vector<uint8_t>& codes, const SiteCall* calls,
                    const SiteCounts* counts, const char* chr_name, std::string* out) {
    std::string& s = *out;
    s.clear();
    char buf[512];
    for (int64_t w = 0; w < plan.n_windows; ++w) {
        const int64_t len = plan.call_len[w];
        const int32_t hs = plan.host_src[w];
        for (int64_t j = 0; j < len; ++j) {
            const int64_t site = w * (int64_t)kWin + j;
            const uint8_t ori = codes[site];
            const SiteCall& c = calls[site];
            HostView h;
            if (hs == w) {
                h.depth = c.depth;
                h.repeat = c.repeat_time;
                h.cu1 = c.cu1; h.ca1 = c.ca1; h.avg1 = c.avg_q1;
                h.cu2 = c.cu2; h.ca2 = c.ca2; h.avg2 = c.avg_q2;
            } else if (hs >= 0) {
                const SiteCounts& k = counts[(int64_t)hs * kWin + j];
                h.depth = k.depth;
                h.repeat = k.repeat_time;
                if (c.base1 < 4) {
                    h.cu1 = k.cu[c.base1]; h.ca1 = (int)k.ca[c.base1];
                    h.avg1 = k.qs[c.base1] == 0 ? 0 : k.qs[c.base1] / k.cu[c.base1];
                }
                if (c.base2 < 4) {
                    h.cu2 = k.cu[c.base2]; h.ca2 = (int)k.ca[c.base2];
                    h.avg2 = k.qs[c.base2] == 0 ? 0 : k.qs[c.base2] / k.cu[c.base2];
                }
            }
            const bool nflag = (ori & 4) && h.depth == 0;
            int n;
            if (nflag || c.base1 >= 4) {
                n = snprintf(buf, sizeof(buf), "%s\t%lld\tN\tN\t0\tN\t0\t0\t0\tN\t0\t0\t0\t0\t1.000\t255.000\t0\n",
                             chr_name, (long long)(site + 1));
            } else {
                char second[96];
                if (c.base2 < 4)
                    snprintf(second, sizeof(second), "%c\t%d\t%d\t%d", kActgN[c.base2], h.avg2, h.cu2, h.ca2);
                else
                    snprintf(second, sizeof(second), "N\t0\t0\t0");
                const double ratio = h.depth == 0 ? 255.0 : (double)h.repeat / h.depth;
                n = snprintf(buf, sizeof(buf), "%s\t%lld\t%c\t%c\t%d\t%c\t%d\t%d\t%d\t%s\t%u\t%#.6g\t%#.6g\t%d\n",
                             chr_name, (long long)(site + 1), kActgN[ori & 7], kAbbv[c.type1], (int)c.q_cns,
                             kActgN[c.base1], h.avg1, h.cu1, h.ca1, second, (unsigned)h.depth, c.rank_sum, ratio,
                             (ori & 8) ? 1 : 0);
            }
            s.append(buf, (size_t)n);
        }
    }
    return 0;
}

}  // namespace gsnp
