/*
 * plan.cpp - host replay of the reference's window loop (see plan.h).
 *
 * Restates the control flow of Call_win::new_soap2cns
 * (cpp/call_genotype.cc:474-644) without doing any calling work: which reads
 * are deposited, which window each call covers, what the host count arrays hold
 * at that moment and which window's likelihood is in device memory.
 *
 * The reference walks the alignments one by one.  Its state changes only when
 * an alignment opens a new window, so the walk splits in two:
 *   1. a per-alignment pass, run in parallel chunks: the length check, the
 *      position filters (cpp/call_genotype.cc:496-515), the sort check
 *      (cpp/call_genotype.cc:517-523) and the runs of alignments that share a
 *      window;
 *   2. the loop over those runs (a few hundred per chromosome), which makes
 *      the same deposits and calls as the reference's loop.
 * The deposited alignments are the ones that pass the filters, in file order,
 * less the last one when it opened a window of its own; the device builds
 * their index list from the same filter (engine.cu).
 */
#include "plan.h"

#include <algorithm>
#include <cstdio>
#include <thread>

#include "calling.cuh"

namespace gsnp {

namespace {

inline bool passes_filters(const ReadView& r, int64_t i, int64_t chr_len) {
    const int64_t p = r.pos[i];
    return p >= 0 && p + r.len[i] < chr_len;
}

/* what one chunk of alignments contributes (padded: the threads write their
 * own entries of one array) */
struct alignas(128) ChunkScan {
    int64_t bad_len = -1;     /* first alignment with a length outside 0..min(L, pitch) */
    int64_t unsorted = -1;    /* first passing alignment below the previous passing one of the chunk */
    int64_t n_valid = 0;
    int64_t first_valid = -1, last_valid = -1;
    bool any_nonneg = false;
    std::vector<WindowRun> runs;   /* window of each run of passing alignments, in order */
};

void scan_chunk(const ReadView& r, int64_t b, int64_t e, int64_t chr_len, int L, ChunkScan* out) {
    const int32_t* __restrict__ pos = r.pos;
    const int32_t* __restrict__ len = r.len;
    const int32_t pitch = r.pitch;
    int64_t bad_len = -1, unsorted = -1, n_valid = 0, first_valid = -1, last_valid = -1;
    bool any_nonneg = false;
    int64_t prev_p = -1;
    int64_t run_w = -1, run_first = -1, run_count = 0;
    std::vector<WindowRun> runs;
    for (int64_t i = b; i < e; ++i) {
        const int32_t l = len[i];
        if (l < 0 || l > L || l > pitch) {
            if (bad_len < 0) bad_len = i;
            continue;
        }
        const int64_t p = pos[i];
        if (p < 0) continue;
        any_nonneg = true;
        if (p + l >= chr_len) continue;
        if (prev_p > p && unsorted < 0) unsorted = i;
        prev_p = p;
        const int64_t w = p / kWin;
        if (w != run_w) {
            if (run_count > 0) runs.push_back(WindowRun{run_w, run_first, run_count});
            run_w = w;
            run_first = i;
            run_count = 0;
        }
        ++run_count;
        if (first_valid < 0) first_valid = i;
        last_valid = i;
        ++n_valid;
    }
    if (run_count > 0) runs.push_back(WindowRun{run_w, run_first, run_count});
    ChunkScan& s = *out;
    s.bad_len = bad_len;
    s.unsorted = unsorted;
    s.n_valid = n_valid;
    s.first_valid = first_valid;
    s.last_valid = last_valid;
    s.any_nonneg = any_nonneg;
    s.runs = std::move(runs);
}

/* Does any deposited unique read leave a record at a site of window v?  That
 * is the reference's "maxNumNonZero > 0" after the update of window v
 * (kernel/update_kernel.cu:355-366).  Every passing alignment that starts
 * before the end of v is deposited by the time v is updated; those covering v
 * start at v*W - L + 1 or later, in the run of v - 1 or of v. */
bool window_has_records(const ReadView& r, int64_t chr_len, int64_t start, int64_t v, int L, int qmin) {
    const int64_t w0 = v * (int64_t)kWin, w1 = w0 + kWin;
    for (int64_t i = start; i < r.n; ++i) {
        if (!passes_filters(r, i, chr_len)) continue;
        const int64_t p = r.pos[i];
        if (p >= w1) break;
        if (p < w0 - L + 1 || r.hit[i] != 1) continue;
        const int64_t c0 = std::max<int64_t>(0, w0 - p), c1 = std::min<int64_t>(r.len[i], w1 - p);
        for (int64_t c = c0; c < c1; ++c) {
            if (r.packed) {
                if ((r.packed[i * r.pitch + c] & 63) != 63) return true;
                continue;
            }
            const signed char b = (signed char)r.seq[i * r.pitch + c];
            const signed char q = (signed char)r.qual[i * r.pitch + c];
            if (b != 'N' && q >= (signed char)qmin) return true;
        }
    }
    return false;
}

}  // namespace

int replay_windows(const ReadView& r, int64_t chr_len, int L, int qmin, int threads, WindowPlan* plan,
                   std::string* err) {
    const int64_t W = kWin;
    WindowPlan& P = *plan;
    P = WindowPlan();
    /* windows 0 .. chr_len / W; the last one is empty when W divides chr_len */
    P.n_windows = chr_len / W + 1;
    P.call_len.assign(P.n_windows, 0);
    P.host_src.assign(P.n_windows, -1);
    P.lik_src.assign(P.n_windows, -1);
    P.flags.assign(P.n_windows, 0);

    /* 1. the per-alignment pass */
    const int64_t kMinChunk = 1 << 16;
    int nt = std::max(1, threads);
    nt = (int)std::min<int64_t>(nt, std::max<int64_t>(1, (r.n + kMinChunk - 1) / kMinChunk));
    std::vector<ChunkScan> cs(nt);
    const int64_t per = (r.n + nt - 1) / nt;
    if (nt == 1) {
        scan_chunk(r, 0, r.n, chr_len, L, &cs[0]);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back(scan_chunk, std::cref(r), std::min(r.n, t * per), std::min(r.n, (t + 1) * per), chr_len,
                              L, &cs[t]);
        for (auto& th : pool) th.join();
    }
    for (const ChunkScan& s : cs)
        if (s.bad_len >= 0) {
            *err = "alignment " + std::to_string(s.bad_len) + " is longer than -L";
            return 6;
        }
    /* the first alignment in file order that breaks the order: inside a
     * chunk, or the first passing one of a chunk against the chunks before */
    int64_t last_p = -1;
    bool started = false;
    for (const ChunkScan& s : cs) {
        started |= s.any_nonneg;
        int64_t bad = s.unsorted;
        if (s.first_valid >= 0 && last_p > r.pos[s.first_valid]) bad = s.first_valid;
        if (bad >= 0) {
            int64_t prev = bad - 1;
            while (!passes_filters(r, prev, chr_len)) --prev;
            char buf[96];
            snprintf(buf, sizeof(buf), "Errors in sorting:%lld<%lld", (long long)r.pos[bad], (long long)r.pos[prev]);
            *err = buf;
            return 5;
        }
        if (s.last_valid >= 0) last_p = r.pos[s.last_valid];
    }
    if (!started) {
        *err = "no alignment with a non-negative position";
        return 6;
    }
    std::vector<WindowRun>& runs = P.runs;
    for (const ChunkScan& s : cs) {
        P.n_valid += s.n_valid;
        for (const WindowRun& w : s.runs) {
            if (!runs.empty() && runs.back().window == w.window)
                runs.back().count += w.count;
            else
                runs.push_back(w);
        }
    }
    P.skipped = r.n - P.n_valid;

    /* 2. the window loop over the runs */
    int64_t cur = 0;             /* window the device state holds */
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
    /* first alignment from which the reads covering window v = runs[k].window
     * are found: back from the run's first alignment over the passing ones
     * that start at v*W - L + 1 or later (they are in the run of v - 1) */
    auto scan_start = [&](size_t k) -> int64_t {
        int64_t i = runs[k].first;
        if (k == 0 || runs[k - 1].window != runs[k].window - 1) return i;
        const int64_t lo = runs[k - 1].first, from = runs[k].window * W - L + 1;
        int64_t start = i;
        for (int64_t j = i - 1; j >= lo; --j) {
            if (!passes_filters(r, j, chr_len)) continue;
            if (r.pos[j] < from) break;
            start = j;
        }
        return start;
    };
    auto deposit = [&](size_t k) {
        m_pos = window_has_records(r, chr_len, scan_start(k), cur, L, qmin);
        host_src = (int32_t)cur;
    };
    for (size_t k = 0; k < runs.size(); ++k) {
        if (k > 0) deposit(k - 1);   /* the batch of window runs[k-1] is deposited */
        while (cur < runs[k].window) {
            call(cur, W);
            cur += 1;
        }
    }
    /* the last alignment opened a window of its own: it stays in the batch */
    if (runs.size() >= 2 && runs.back().count == 1) {
        P.dropped_last = true;
    } else if (runs.empty()) {
        m_pos = false;               /* nothing deposited */
        host_src = (int32_t)cur;
    } else {
        deposit(runs.size() - 1);
    }
    P.n_deposited = P.n_valid - (P.dropped_last ? 1 : 0);
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
