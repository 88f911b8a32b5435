/*
 * plan.cpp - host replay of the reference's window loop (see plan.h).
 *
 * Restates the control flow of Call_win::new_soap2cns
 * (cpp/call_genotype.cc:474-644) without doing any calling work: which reads
 * are deposited, which window each call covers, what the host count arrays hold
 * at that moment and which window's likelihood is in device memory.
 */
#include "plan.h"

#include <algorithm>
#include <cstdio>

#include "calling.cuh"

namespace gsnp {

namespace {

/* Does any deposited unique read leave a record at a site of window v?  That
 * is the reference's "maxNumNonZero > 0" after the update of window v
 * (kernel/update_kernel.cu:355-366). */
bool window_has_records(const ReadView& r, const std::vector<int64_t>& dep, size_t dep_end, int64_t v, int L,
                        int qmin) {
    const int64_t w0 = v * (int64_t)kWin, w1 = w0 + kWin;
    /* deposited reads are sorted by start: those covering [w0, w1) start in [w0 - L + 1, w1) */
    auto first = std::lower_bound(dep.begin(), dep.begin() + dep_end, w0 - L + 1,
                                  [&](int64_t idx, int64_t p) { return (int64_t)r.pos[idx] < p; });
    for (auto it = first; it != dep.begin() + dep_end; ++it) {
        const int64_t i = *it;
        const int64_t p = r.pos[i];
        if (p >= w1) break;
        if (r.hit[i] != 1) continue;
        const int64_t c0 = std::max<int64_t>(0, w0 - p), c1 = std::min<int64_t>(r.len[i], w1 - p);
        for (int64_t c = c0; c < c1; ++c) {
            const signed char b = (signed char)r.seq[i * r.pitch + c];
            const signed char q = (signed char)r.qual[i * r.pitch + c];
            if (b != 'N' && q >= (signed char)qmin) return true;
        }
    }
    return false;
}

}  // namespace

int replay_windows(const ReadView& r, int64_t chr_len, int L, int qmin, WindowPlan* plan, std::string* err) {
    const int64_t W = kWin;
    WindowPlan& P = *plan;
    P = WindowPlan();
    /* windows 0 .. chr_len / W; the last one is empty when W divides chr_len */
    P.n_windows = chr_len / W + 1;
    P.call_len.assign(P.n_windows, 0);
    P.host_src.assign(P.n_windows, -1);
    P.lik_src.assign(P.n_windows, -1);
    P.flags.assign(P.n_windows, 0);
    P.deposited.reserve(r.n);

    bool started = false;
    int64_t cur = 0;             /* window the device state holds */
    int64_t last_start = 0;
    std::vector<int64_t> batch;  /* indices of the open batch */
    bool mark = false;
    bool m_pos = false;          /* maxNumNonZero > 0 after the latest update */
    int32_t host_src = -1;
    int32_t lik_last = -1;

    auto call = [&](int64_t w, int64_t len) {
        if (w >= P.n_windows) return;
        P.call_len[w] = len;
        P.host_src[w] = host_src;
        if (m_pos) {
            P.lik_src[w] = (int32_t)w;
            lik_last = (int32_t)w;
        } else {
            P.lik_src[w] = lik_last;
        }
    };
    auto deposit = [&]() {
        for (int64_t i : batch) P.deposited.push_back(i);
        batch.clear();
        m_pos = window_has_records(r, P.deposited, P.deposited.size(), cur, L, qmin);
        host_src = (int32_t)cur;
    };

    for (int64_t i = 0; i < r.n; ++i) {
        const int64_t p = r.pos[i];
        if (p < 0) { ++P.skipped; continue; }
        if (!started) {
            started = true;
            cur = 0;
            last_start = 0;
        }
        if (p + r.len[i] >= chr_len) { ++P.skipped; continue; }
        if (p < last_start) {
            char buf[96];
            snprintf(buf, sizeof(buf), "Errors in sorting:%lld<%lld", (long long)p, (long long)last_start);
            *err = buf;
            return 5;
        }
        mark = false;
        if (!batch.empty() && p / W > last_start / W) {
            deposit();
            mark = true;
        }
        while (p / W > last_start / W) {
            call(cur, W);
            cur += 1;
            last_start = cur * W + W - 1;
        }
        last_start = p;
        batch.push_back(i);
    }
    if (!started) {
        *err = "no alignment with a non-negative position";
        return 6;
    }
    if (!mark) {
        deposit();
    } else {
        P.dropped_last = true;
        batch.clear();
    }
    while (chr_len > cur * W + W - 1) {
        call(cur, W);
        cur += 1;
        host_src = (int32_t)cur;   /* cuda_quickRecycle refreshes the host arrays */
    }
    call(cur, chr_len % W);

    /* kernel flags: keep counts / likelihood of windows other windows refer to */
    for (int64_t w = 0; w < P.n_windows; ++w) {
        if (P.host_src[w] >= 0 && P.host_src[w] != w) P.flags[P.host_src[w]] |= kWinKeepCounts;
        if (P.lik_src[w] != w) {
            P.flags[w] |= kWinExternalLik;
            if (P.lik_src[w] >= 0) P.flags[P.lik_src[w]] |= kWinKeepLik;
        }
    }
    return 0;
}

}  // namespace gsnp
