// Checks replay_windows (gsnp_gb300/csrc/plan.cpp), whose per-alignment pass
// runs in parallel chunks, against a walk over the alignments one at a time
// that follows Call_win::new_soap2cns (cpp/call_genotype.cc:474-644) step by
// step.  Random chromosomes with gap windows, windows without usable bases,
// filtered alignments, a last alignment alone in its window, and unsorted
// input inside a chunk and across chunk boundaries, at several thread counts.
// Prints the number of cases and exits 1 on the first difference.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "calling.cuh"
#include "plan.h"

using namespace gsnp;

static uint64_t state = 0x243f6a8885a308d3ull;
static uint64_t next() {
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static int64_t below(int64_t n) { return (int64_t)(next() % (uint64_t)n); }

struct Walk {
    int rc = 0;
    std::string err;
    std::vector<int64_t> call_len, deposited;
    std::vector<int32_t> host_src, lik_src;
    int64_t skipped = 0;
    bool dropped_last = false;
};

/* the reference's loop, one alignment at a time */
static Walk walk(const ReadView& r, int64_t chr_len, int L, int qmin) {
    const int64_t W = kWin;
    Walk P;
    const int64_t n_windows = chr_len / W + 1;
    P.call_len.assign(n_windows, 0);
    P.host_src.assign(n_windows, -1);
    P.lik_src.assign(n_windows, -1);
    for (int64_t i = 0; i < r.n; ++i)
        if (r.len[i] < 0 || r.len[i] > L || r.len[i] > r.pitch) {
            P.rc = 6;
            P.err = "alignment " + std::to_string(i) + " is longer than -L";
            return P;
        }
    auto has_records = [&](int64_t v) {
        const int64_t w0 = v * W, w1 = w0 + W;
        for (int64_t i : P.deposited) {
            const int64_t p = r.pos[i];
            if (p + L <= w0 || p >= w1 || r.hit[i] != 1) continue;
            for (int64_t c = std::max<int64_t>(0, w0 - p); c < std::min<int64_t>(r.len[i], w1 - p); ++c) {
                const signed char b = (signed char)r.seq[i * r.pitch + c];
                const signed char q = (signed char)r.qual[i * r.pitch + c];
                if (b != 'N' && q >= (signed char)qmin) return true;
            }
        }
        return false;
    };
    bool started = false, mark = false, m_pos = false;
    int64_t cur = 0, last_start = 0;
    int32_t host_src = -1, lik_last = -1;
    std::vector<int64_t> batch;
    auto call = [&](int64_t w, int64_t len) {
        if (w >= n_windows) return;
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
        m_pos = has_records(cur);
        host_src = (int32_t)cur;
    };
    for (int64_t i = 0; i < r.n; ++i) {
        const int64_t p = r.pos[i];
        if (p < 0) { ++P.skipped; continue; }
        if (!started) { started = true; cur = 0; last_start = 0; }
        if (p + r.len[i] >= chr_len) { ++P.skipped; continue; }
        if (p < last_start) {
            char buf[96];
            snprintf(buf, sizeof(buf), "Errors in sorting:%lld<%lld", (long long)p, (long long)last_start);
            P.rc = 5;
            P.err = buf;
            return P;
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
        P.rc = 6;
        P.err = "no alignment with a non-negative position";
        return P;
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
        host_src = (int32_t)cur;
    }
    call(cur, chr_len % W);
    return P;
}

struct Case {
    int64_t chr_len;
    int L, pitch, qmin;
    std::vector<int32_t> pos, len, hit;
    std::vector<uint8_t> seq, qual;
    ReadView view() const {
        return ReadView{(int64_t)pos.size(), pos.data(), len.data(), hit.data(), seq.data(), qual.data(), pitch};
    }
};

/* sorted alignments over a chromosome of `windows` windows, some windows
 * empty, some with only unusable bases */
static Case make_case(int windows, int64_t n, int kind) {
    Case c;
    c.L = 24;
    c.pitch = 24;
    c.qmin = 'A' + 5;
    c.chr_len = (int64_t)windows * kWin - below(kWin / 2) * (kind % 2);
    std::vector<int> wmode(windows + 1);
    for (int w = 0; w <= windows; ++w) wmode[w] = (int)below(5);   /* 0: empty, 1: no usable base */
    c.pos.reserve(n);
    int64_t p = below(kWin);
    for (int64_t i = 0; i < n; ++i) {
        p += below(3 * (int64_t)windows * kWin / n + 1);
        while (p < c.chr_len + 50 && wmode[p / kWin] == 0) p += kWin / 4;
        const int64_t q = std::min<int64_t>(p, c.chr_len + 40);
        const int l = 1 + (int)below(c.L);
        c.pos.push_back(below(50) == 0 ? -1 - (int32_t)below(100) : (int32_t)q);
        c.len.push_back(l);
        c.hit.push_back(below(6) == 0 ? 2 : 1);
        const bool dead = q < c.chr_len && wmode[q / kWin] == 1;
        for (int k = 0; k < c.pitch; ++k) {
            const uint64_t z = next();
            c.seq.push_back(dead || z % 9 == 0 ? 'N' : "ACGT"[z % 4]);
            c.qual.push_back((uint8_t)(dead ? 'A' : 'A' + (z >> 8) % 40));
        }
    }
    if (kind == 2 && n > 2) {   /* the last alignment opens a window of its own */
        c.pos[n - 1] = (int32_t)std::min<int64_t>(c.chr_len - 30, ((c.pos[n - 2] > 0 ? c.pos[n - 2] : 0) / kWin + 1) * kWin + 3);
        c.len[n - 1] = 10;
    }
    return c;
}

/* the case's reads as packed bytes (gsnp_pack_reads's layout); an N is
 * written as the skip code 63, which the replay takes as it takes an N:
 * neither base counts as a record */
static std::vector<uint8_t> pack_case(const Case& c) {
    std::vector<uint8_t> out(c.seq.size(), 0);
    for (size_t i = 0; i < c.pos.size(); ++i)
        for (int k = 0; k < c.pitch && k < c.len[i]; ++k) {
            const size_t at = i * (size_t)c.pitch + (size_t)k;
            const uint8_t b = c.seq[at];
            const int q = (int)(signed char)c.qual[at] - c.qmin;
            out[at] = (b == 'N' || q < 0) ? (uint8_t)63 : (uint8_t)((((b >> 1) & 3) << 6) | q);
        }
    return out;
}

static bool same_plan(const WindowPlan& a, const WindowPlan& b) {
    if (a.n_windows != b.n_windows || a.call_len != b.call_len || a.host_src != b.host_src ||
        a.lik_src != b.lik_src || a.flags != b.flags || a.n_valid != b.n_valid || a.n_deposited != b.n_deposited ||
        a.skipped != b.skipped || a.dropped_last != b.dropped_last || a.runs.size() != b.runs.size())
        return false;
    for (size_t k = 0; k < a.runs.size(); ++k)
        if (a.runs[k].first != b.runs[k].first || a.runs[k].count != b.runs[k].count ||
            a.runs[k].window != b.runs[k].window)
            return false;
    return true;
}

static int cases = 0;
static bool compare(const Case& c, int threads, const char* what) {
    ++cases;
    const ReadView v = c.view();
    const Walk want = walk(v, c.chr_len, c.L, c.qmin);
    WindowPlan got;
    std::string err;
    const int rc = replay_windows(v, c.chr_len, c.L, c.qmin, threads, &got, &err);
    auto fail = [&](const char* m) {
        printf("%s (threads %d, n %lld): %s; rc %d/%d err '%s'/'%s'\n", what, threads, (long long)v.n, m, rc, want.rc,
               err.c_str(), want.err.c_str());
        return false;
    };
    if (rc != want.rc || err != want.err) return fail("return code");
    /* the same reads packed: the same plan, or the same error */
    const std::vector<uint8_t> pk = pack_case(c);
    ReadView pv = v;
    pv.seq = nullptr;
    pv.qual = nullptr;
    pv.packed = pk.data();
    WindowPlan got_packed;
    std::string err_packed;
    const int rc_packed = replay_windows(pv, c.chr_len, c.L, c.qmin, threads, &got_packed, &err_packed);
    if (rc_packed != rc || err_packed != err) return fail("packed reads: return code");
    if (rc == 0 && !same_plan(got, got_packed)) return fail("packed reads: plan");
    if (rc != 0) return true;
    if (got.call_len != want.call_len) return fail("call_len");
    if (got.host_src != want.host_src) return fail("host_src");
    if (got.lik_src != want.lik_src) return fail("lik_src");
    if (got.skipped != want.skipped || got.dropped_last != want.dropped_last) return fail("skipped/dropped");
    if (got.n_deposited != (int64_t)want.deposited.size()) return fail("n_deposited");
    /* deposited = the passing alignments in order, the first n_deposited */
    int64_t k = 0;
    for (int64_t i = 0; i < v.n && k < got.n_deposited; ++i)
        if (v.pos[i] >= 0 && (int64_t)v.pos[i] + v.len[i] < c.chr_len) {
            if (want.deposited[k] != i) return fail("deposited order");
            ++k;
        }
    return true;
}

int main() {
    const int threads[] = {1, 2, 3, 7, 16};
    for (int round = 0; round < 6; ++round)
        for (int kind = 0; kind < 3; ++kind) {
            const int windows = 1 + (int)below(9);
            const int64_t n = kind == 0 ? 300000 + below(200000) : 1000 + below(140000);
            Case c = make_case(windows, n, kind);
            for (int t : threads)
                if (!compare(c, t, "sorted")) return 1;
            /* unsorted: one alignment moved back, inside a chunk or at the
             * first passing alignment of a later chunk */
            for (int u = 0; u < 3; ++u) {
                Case d = c;
                const int64_t at = u == 0 ? below(n) : (u * n) / 4;
                int64_t i = at;
                while (i < n && !(d.pos[i] > 100 && d.pos[i] + d.len[i] < d.chr_len)) ++i;
                if (i >= n) continue;
                d.pos[i] -= 50 + (int32_t)below(50);
                for (int t : threads)
                    if (!compare(d, t, "unsorted")) return 1;
            }
        }
    /* filters only, and errors */
    {
        Case c = make_case(3, 200000, 0);
        Case all_neg = c;
        for (auto& p : all_neg.pos) p = -5;
        Case past_end = c;
        for (size_t i = 0; i < past_end.pos.size(); ++i) past_end.pos[i] = (int32_t)(c.chr_len - 1);
        Case too_long = c;
        too_long.len[150000] = c.L + 1;
        for (int t : threads) {
            if (!compare(all_neg, t, "all negative")) return 1;
            if (!compare(past_end, t, "all past the end")) return 1;
            if (!compare(too_long, t, "too long")) return 1;
        }
        Case one = make_case(2, 1, 0);
        one.pos[0] = 7;
        if (!compare(one, 4, "one alignment")) return 1;
        Case two = make_case(2, 2, 0);
        two.pos[0] = 7;
        two.pos[1] = kWin + 9;
        two.len[0] = two.len[1] = 5;
        if (!compare(two, 4, "two alignments, two windows")) return 1;
    }
    printf("checked %d cases\n", cases);
    return 0;
}
