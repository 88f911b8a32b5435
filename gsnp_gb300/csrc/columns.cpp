/*
 * columns.cpp - the -C compressed output (cpp/compress.h:86-1312,
 * cpp/dict_compression.h:40-296).
 *
 * Six files per run, one block per called window, byte-compatible with the
 * reference's writers and its decompressor (cpp/decompression.cpp):
 *   <out>.1_2             window table: count, then "chr start size" lines
 *   <out>.3_4_6           reference base 2-bit packed, N ids, genotype and
 *                         best-base differences from the reference base
 *   <out>.5_7_8_9_14_16   six per-site columns, each run-length encoded and
 *                         both run values and run lengths dictionary coded
 *   <out>.10              second base 2-bit packed, N ids
 *   <out>.11_12_13        second-base quality/count columns: common entries
 *                         dictionary coded, the rest as sparse id/value lists
 *   <out>.15_17           sparse rank-sum values and dbSNP site ids
 * Windows are encoded independently, in memory, on every host thread, and
 * their blocks written in window order.  Run-length encoding, 2-bit packing,
 * the sparse lists and the dictionary codec (the contract of dict.cu, here
 * on the host so that the threads need no device) are single passes per
 * window.
 */
#include "columns.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <string>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include "dict.h"
#include "rows.h"
#include "columns_gpu.h"

namespace gsnp {

const char kAbbv[17] = {'A', 'M', 'W', 'R', 'M', 'C', 'Y', 'S', 'W', 'Y', 'T', 'K', 'R', 'S', 'K', 'G', 'N'};
const char kActgN[9] = "ACTGNNNN";

namespace {

constexpr unsigned long kDictCap = 32UL * 8192UL;   /* the reference's dictionary capacity */

/* one window's blocks of the five binary files */
struct Files {
    std::string f346, frle, f10, f111213, f1517;
    bool ok = true;
    void put(std::string& f, const void* p, size_t bytes) {
        if (bytes) f.append(static_cast<const char*>(p), bytes);
    }
    void clear() {
        for (std::string* x : {&f346, &frle, &f10, &f111213, &f1517}) x->clear();
        ok = true;
    }
};

/* dict.cu's codec on the host: dict = the distinct values ascending (-0.0
 * and +0.0 one entry, -0.0 when any -0.0 occurs), words = each value's index
 * packed MSB-first, floor(32 / bits) per word, the last word right-aligned.
 * The distinct values and each input's index come from a presence table over
 * the value range for integers of a narrow range (qualities, counts, depths,
 * run lengths: one pass each, no sort), from a hash table of the distinct
 * values otherwise; both give the indices the sorted dictionary's
 * lower_bound gives. */
template <class T>
bool pack_indices(const uint32_t* idx, size_t n, unsigned long d, uint32_t* words, unsigned long* n_words,
                  std::string* err) {
    const int bits = dict_bits(d);
    const size_t per = (size_t)floor(32 / (double)bits);
    const size_t nw = (size_t)ceil(n / (double)per);
    if (*n_words < nw) {
        *err = "numWordOutData < numWordCompressed";
        return false;
    }
    for (size_t w = 0; w < nw; ++w) {
        const size_t first = w * per, cnt = (w == nw - 1) ? n - first : per;
        uint32_t out = 0;
        for (size_t i = 0; i < cnt; ++i) out = (out << bits) | idx[first + i];
        words[w] = out;
    }
    *n_words = (unsigned long)nw;
    return true;
}

/* integer values within [lo, lo + span): indices through a dense table */
template <class T>
void dense_dict(const T* in, size_t n, int64_t lo, size_t span, std::vector<T>* d, std::vector<uint32_t>* idx) {
    thread_local std::vector<uint32_t> slot;
    if (slot.size() < span) slot.resize(span);
    std::fill(slot.begin(), slot.begin() + (ptrdiff_t)span, 0u);
    for (size_t i = 0; i < n; ++i) slot[(size_t)((int64_t)in[i] - lo)] = 1u;
    d->clear();
    for (size_t v = 0; v < span; ++v)
        if (slot[v]) {
            slot[v] = (uint32_t)d->size();
            d->push_back((T)((int64_t)v + lo));
        }
    idx->resize(n);
    for (size_t i = 0; i < n; ++i) (*idx)[i] = slot[(size_t)((int64_t)in[i] - lo)];
}

/* any values: distinct values through an open-addressing table of their
 * bit patterns (+0.0 standing for both zeros), sorted, then indexed */
template <class T>
void hashed_dict(const T* in, size_t n, std::vector<T>* d, std::vector<uint32_t>* idx) {
    static_assert(sizeof(T) <= 8, "values of at most 64 bits");
    auto key = [](T v) {
        uint64_t k = 0;
        if (v == (T)0) v = (T)0;   /* -0.0 and +0.0: one key */
        memcpy(&k, &v, sizeof(T));
        return k;
    };
    size_t cap = 64;
    while (cap < 2 * n) cap <<= 1;
    std::vector<uint64_t> keys(cap);
    std::vector<uint32_t> val(cap, 0xffffffffu);
    auto find = [&](uint64_t k) {
        size_t h = (size_t)((k * 0x9e3779b97f4a7c15ull) >> 17) & (cap - 1);
        while (val[h] != 0xffffffffu && keys[h] != k) h = (h + 1) & (cap - 1);
        return h;
    };
    d->clear();
    for (size_t i = 0; i < n; ++i) {
        const size_t h = find(key(in[i]));
        if (val[h] == 0xffffffffu) {
            keys[h] = key(in[i]);
            val[h] = 0;
            d->push_back(in[i] == (T)0 ? (T)0 : in[i]);
        }
    }
    std::sort(d->begin(), d->end());
    for (size_t r = 0; r < d->size(); ++r) val[find(key((*d)[r]))] = (uint32_t)r;
    idx->resize(n);
    for (size_t i = 0; i < n; ++i) (*idx)[i] = val[find(key(in[i]))];
}

template <class T>
bool host_dict(const T* in, size_t n, uint32_t* words, unsigned long* n_words, T* dict, unsigned long* n_dict,
               std::string* err) {
    if (*n_dict < n) {
        *err = "*numElementDict < numElementInData";
        return false;
    }
    if (n == 0) {
        *n_dict = 0;
        *n_words = 0;
        return true;
    }
    thread_local std::vector<T> d;
    thread_local std::vector<uint32_t> idx;
    bool dense = false;
    if (std::is_integral<T>::value) {
        int64_t lo = (int64_t)in[0], hi = lo;
        for (size_t i = 1; i < n; ++i) {
            lo = std::min<int64_t>(lo, (int64_t)in[i]);
            hi = std::max<int64_t>(hi, (int64_t)in[i]);
        }
        const uint64_t span = (uint64_t)(hi - lo) + 1;
        if (span <= std::max<uint64_t>(1u << 16, 4 * (uint64_t)n) && span <= (1u << 24)) {
            dense_dict(in, n, lo, (size_t)span, &d, &idx);
            dense = true;
        }
    }
    if (!dense) hashed_dict(in, n, &d, &idx);
    /* the zero entry is -0.0 when any input is -0.0 */
    for (T& v : d)
        if (v == (T)0 && std::is_floating_point<T>::value) {
            bool neg = false;
            for (size_t i = 0; i < n && !neg; ++i) neg = in[i] == (T)0 && std::signbit((double)in[i]);
            v = neg ? (T)(-0.0) : (T)0;
        }
    if (!pack_indices<T>(idx.data(), n, (unsigned long)d.size(), words, n_words, err)) return false;
    std::copy(d.begin(), d.end(), dict);
    *n_dict = (unsigned long)d.size();
    return true;
}

int base_bits(char c) {
    switch (c) {
        case 'A': return 0;
        case 'C': return 1;
        case 'G': return 2;
        case 'T': return 3;
        default: return -1;
    }
}

/* 2-bit packing, first base in the high bits, the last word right-aligned
 * (kernel/compress_kernel.cu:85-160) */
std::vector<uint32_t> pack2(const std::vector<char>& c) {
    const size_t n = c.size(), nw = (n + 15) / 16;
    std::vector<uint32_t> code(nw, 0);
    for (size_t w = 0; w < nw; ++w) {
        const size_t nb = (w == nw - 1) ? n - w * 16 : 16;
        uint32_t word = 0;
        for (size_t i = 0; i < nb; ++i) word = (word << 2) | (uint32_t)base_bits(c[w * 16 + i]);
        code[w] = word;
    }
    return code;
}

template <class T>
unsigned rle(std::vector<T>& data, std::vector<uint32_t>& runs) {
    const size_t n = data.size();
    runs.resize(n);
    if (n == 0) return 0;
    size_t r = 0, start = 0;
    for (size_t i = 1; i <= n; ++i)
        if (i == n || !(data[i] == data[start])) {
            data[r] = data[start];
            runs[r] = (uint32_t)(i - start);
            ++r;
            start = i;
        }
    return (unsigned)r;
}

class Writer {
public:
    Writer(const DictCodec& dict, Files& f) : dict_(dict), f_(f) {}

    bool window(const std::vector<CnsRow>& rows, std::string* err) {
        const size_t n = rows.size();
        bool all_n = true;
        for (const CnsRow& r : rows) all_n = all_n && r.nflag;
        col_3_4_6(rows, all_n);
        if (!col_rle(rows, all_n, err)) return false;
        col_10(rows, all_n);
        if (!col_11_12_13(rows, all_n, err)) return false;
        col_15_17(rows, all_n);
        (void)n;
        return f_.ok;
    }

private:
    const DictCodec& dict_;
    Files& f_;

    /* Column_3_4_6 (cpp/compress.h:171-409) */
    void col_3_4_6(const std::vector<CnsRow>& rows, bool all_n) {
        const unsigned long n = rows.size();
        unsigned long param[7] = {1, 0, n, 0, 0, 0, 0};
        if (all_n) {
            f_.put(f_.f346, param, sizeof(param));
            return;
        }
        std::vector<char> c3(n);
        std::vector<int> id4, id6, idn;
        std::vector<char> v4, v6;
        for (unsigned long i = 0; i < n; ++i) {
            const CnsRow& r = rows[i];
            char a = 'N', b = 'N', c = 'N';
            if (r.called()) {
                a = kActgN[r.ori & 7];
                b = kAbbv[r.type1];
                c = kActgN[r.base1];
            }
            if (b != a) { id4.push_back((int)i); v4.push_back(b); }
            if (c != a) { id6.push_back((int)i); v6.push_back(c); }
            if (a == 'N') { idn.push_back((int)i); a = 'A'; }
            c3[i] = a;
        }
        const std::vector<uint32_t> code = pack2(c3);
        param[0] = 0;
        param[3] = code.size();
        param[4] = idn.size();
        param[5] = id4.size();
        param[6] = id6.size();
        param[1] = 5 * id4.size() + 5 * id6.size() + 4 * idn.size() + 4 * code.size();
        f_.put(f_.f346, param, sizeof(param));
        f_.put(f_.f346, id4.data(), 4 * id4.size());
        f_.put(f_.f346, v4.data(), v4.size());
        f_.put(f_.f346, id6.data(), 4 * id6.size());
        f_.put(f_.f346, v6.data(), v6.size());
        f_.put(f_.f346, idn.data(), 4 * idn.size());
        f_.put(f_.f346, code.data(), 4 * code.size());
    }

    /* one column of Column_RLEDict (cpp/compress.h:495-868) */
    template <class T>
    bool rle_dict(std::vector<T>& col, std::string* err) {
        /* per-thread buffers: every entry read back is written first */
        thread_local std::vector<uint32_t> runlen, cval, clen, dlen;
        thread_local std::vector<T> dval;
        const unsigned runs = rle(col, runlen);
        for (std::vector<uint32_t>* v : {&cval, &clen, &dlen})
            if (v->size() < runs + 1) v->resize(runs + 1);
        if (dval.size() < runs + 1) dval.resize(runs + 1);
        unsigned long nwv = runs, ndv = kDictCap, nwl = runs, ndl = kDictCap;
        if (!dict_.compress(col.data(), runs, cval.data(), &nwv, dval.data(), &ndv, err)) return false;
        if (!dict_.compress(runlen.data(), runs, clen.data(), &nwl, dlen.data(), &ndl, err)) return false;
        unsigned long param[6] = {runs, nwv, nwl, ndv, ndl, 4 * nwv + 4 * nwl + sizeof(T) * ndv + 4 * ndl};
        f_.put(f_.frle, param, sizeof(param));
        f_.put(f_.frle, cval.data(), 4 * nwv);
        f_.put(f_.frle, clen.data(), 4 * nwl);
        f_.put(f_.frle, dval.data(), sizeof(T) * ndv);
        f_.put(f_.frle, dlen.data(), 4 * ndl);
        return true;
    }

    bool col_rle(const std::vector<CnsRow>& rows, bool all_n, std::string* err) {
        const int flag = all_n ? 1 : 0;
        f_.put(f_.frle, &flag, sizeof(int));
        if (flag) return true;
        /* the six columns in one pass over the rows, then each encoded */
        const size_t n = rows.size();
        thread_local std::vector<int> c5, c7, c8, c9, c14;
        thread_local std::vector<double> c16;
        for (std::vector<int>* v : {&c5, &c7, &c8, &c9, &c14}) v->resize(n);
        c16.resize(n);
        for (size_t j = 0; j < n; ++j) {
            const CnsRow& r = rows[j];
            const bool called = r.called();
            c5[j] = called ? r.q_cns : 0;
            c7[j] = called ? r.avg1 : 0;
            c8[j] = called ? r.cu1 : 0;
            c9[j] = called ? r.ca1 : 0;
            c14[j] = called ? (int)r.depth : 0;
            c16[j] = called ? (r.depth == 0 ? 255 : (double)r.repeat / r.depth) : 255.0;
        }
        for (std::vector<int>* v : {&c5, &c7, &c8, &c9, &c14})
            if (!rle_dict(*v, err)) return false;
        return rle_dict(c16, err);
    }

    /* Column_10 (cpp/compress.h:759-897) */
    void col_10(const std::vector<CnsRow>& rows, bool all_n) {
        const int flag = all_n ? 1 : 0;
        f_.put(f_.f10, &flag, sizeof(int));
        if (flag) return;
        const size_t n = rows.size();
        std::vector<char> c(n);
        std::vector<uint32_t> nid;
        for (size_t j = 0; j < n; ++j) {
            const CnsRow& r = rows[j];
            c[j] = (r.called() && r.base2 < 4) ? kActgN[r.base2] : 'N';
            if (c[j] == 'N') { nid.push_back((uint32_t)j); c[j] = 'A'; }
        }
        const std::vector<uint32_t> code = pack2(c);
        unsigned long param[3] = {nid.size(), code.size(), n};
        f_.put(f_.f10, param, sizeof(param));
        f_.put(f_.f10, code.data(), 4 * code.size());
        f_.put(f_.f10, nid.data(), 4 * nid.size());
    }

    /* Column_11_12_13 (cpp/compress.h:947-1172).  The reference writes a
     * window whose common list is empty by failing an assert in its
     * dictionary code (cpp/dict_compression.h:140-143); here such a list is
     * the pair {0, 0} with no payload. */
    bool col_11_12_13(const std::vector<CnsRow>& rows, bool all_n, std::string* err) {
        const int flag = all_n ? 1 : 0;
        f_.put(f_.f111213, &flag, sizeof(int));
        if (flag) return true;
        const size_t n = rows.size();
        std::vector<int> cid, c11, c12, c13, e12id, e12, e13id, e13;
        for (size_t j = 0; j < n; ++j) {
            const CnsRow& r = rows[j];
            int v11 = 0, v12 = 0, v13 = 0;
            if (r.called() && r.base2 < 4) {
                v11 = r.avg2;
                v12 = r.cu2;
                v13 = r.ca2;
            }
            if (v11 != 0) { cid.push_back((int)j); c11.push_back(v11); c12.push_back(v12); c13.push_back(v13); }
            else if (v11 != v12) { e12id.push_back((int)j); e12.push_back(v12); }
            else if (v11 != v13) { e13id.push_back((int)j); e13.push_back(v13); }
        }
        unsigned long param[4] = {n, cid.size(), e12id.size(), e13id.size()};
        f_.put(f_.f111213, param, sizeof(param));
        f_.put(f_.f111213, e12id.data(), 4 * e12id.size());
        f_.put(f_.f111213, e12.data(), 4 * e12.size());
        f_.put(f_.f111213, e13id.data(), 4 * e13id.size());
        f_.put(f_.f111213, e13.data(), 4 * e13.size());
        f_.put(f_.f111213, cid.data(), 4 * cid.size());
        thread_local std::vector<uint32_t> words(kWin);
        thread_local std::vector<int> dict(kWin);
        for (std::vector<int>* v : {&c11, &c12, &c13}) {
            unsigned long dp[2] = {(unsigned long)kWin, (unsigned long)kWin};
            if (!dict_.compress(v->data(), v->size(), words.data(), &dp[0], dict.data(), &dp[1], err)) return false;
            f_.put(f_.f111213, dp, sizeof(dp));
            f_.put(f_.f111213, words.data(), 4 * dp[0]);
            f_.put(f_.f111213, dict.data(), 4 * dp[1]);
        }
        return true;
    }

    /* Column_15_17 (cpp/compress.h:1175-1312) */
    void col_15_17(const std::vector<CnsRow>& rows, bool all_n) {
        const int flag = all_n ? 1 : 0;
        f_.put(f_.f1517, &flag, sizeof(int));
        if (flag) return;
        const size_t n = rows.size();
        std::vector<int> id, snp;
        std::vector<double> val;
        for (size_t j = 0; j < n; ++j) {
            const CnsRow& r = rows[j];
            if (!r.called()) continue;
            if (r.rank_sum != 1.0) { id.push_back((int)j); val.push_back(r.rank_sum); }
            if (r.ori & 8) snp.push_back((int)j);
        }
        int cnt = (int)id.size();
        f_.put(f_.f1517, &cnt, sizeof(int));
        f_.put(f_.f1517, id.data(), 4 * id.size());
        f_.put(f_.f1517, val.data(), 8 * val.size());
        cnt = (int)snp.size();
        f_.put(f_.f1517, &cnt, sizeof(int));
        f_.put(f_.f1517, snp.data(), 4 * snp.size());
    }
};

}  // namespace

bool encode_window_host(int64_t len, int mode, const uint8_t* codes_w, const SiteCall* calls_w,
                        const SiteCounts* counts_w, const DictCodec& dict, std::string* parts, std::string* err) {
    /* make_row indexes the shown window's counts at hs * kWin + j: the
     * window's counts sit after a window of padding */
    std::vector<SiteCounts> shown;
    if (mode == 1) {
        shown.resize((size_t)(kWin + len));
        std::copy(counts_w, counts_w + len, shown.begin() + kWin);
    }
    std::vector<CnsRow> rows((size_t)len);
    for (int64_t j = 0; j < len; ++j)
        rows[(size_t)j] = make_row(mode == 1 ? 1 : mode, 0, j, codes_w, calls_w, shown.empty() ? nullptr : shown.data());
    Files f;
    Writer wr(dict, f);
    if (!wr.window(rows, err)) return false;
    parts[0].swap(f.f346);
    parts[1].swap(f.frle);
    parts[2].swap(f.f10);
    parts[3].swap(f.f111213);
    parts[4].swap(f.f1517);
    return true;
}

namespace {

FILE* open_file(const std::string& path, const char* mode, std::string* err) {
    FILE* f = fopen(path.c_str(), mode);
    if (!f) *err = "cannot create " + path;
    return f;
}

}  // namespace

bool HostDictCodec::compress(const int* in, size_t n, uint32_t* words, unsigned long* n_words, int* dict,
                             unsigned long* n_dict, std::string* err) const {
    return host_dict(in, n, words, n_words, dict, n_dict, err);
}
bool HostDictCodec::compress(const uint32_t* in, size_t n, uint32_t* words, unsigned long* n_words, uint32_t* dict,
                             unsigned long* n_dict, std::string* err) const {
    return host_dict(in, n, words, n_words, dict, n_dict, err);
}
bool HostDictCodec::compress(const double* in, size_t n, uint32_t* words, unsigned long* n_words, double* dict,
                             unsigned long* n_dict, std::string* err) const {
    return host_dict(in, n, words, n_words, dict, n_dict, err);
}

int write_columns(const WindowPlan& plan, const uint8_t* codes, const SiteCall* calls, const SiteCounts* counts,
                  const char* chr_name, const std::string& base, const DictCodec& dict, int threads, std::string* err) {
    const char* ext[5] = {".3_4_6", ".5_7_8_9_14_16", ".10", ".11_12_13", ".15_17"};
    FILE* fb[5];
    for (int i = 0; i < 5; ++i) fb[i] = open_file(base + ext[i], "wb", err);
    FILE* f12 = open_file(base + ".1_2", "w", err);
    int rc = 0;
    for (FILE* x : fb)
        if (!x) rc = 1;
    if (!f12) rc = 1;
    if (rc == 0 && calls) {
        fprintf(f12, "%lu\n", (unsigned long)plan.n_windows);
        for (int64_t w = 0; w < plan.n_windows; ++w)
            fprintf(f12, "%s\t%lu\t%lu\n", chr_name, (unsigned long)(w * (int64_t)kWin + 1),
                    (unsigned long)plan.call_len[w]);
        /* windows encoded by persistent workers, taken in order from a
         * counter, at most `ahead` windows beyond the last one written; one
         * writer thread writes them in window order and frees each block */
        const int nt = std::max(1, threads);
        const int64_t nwin = plan.n_windows;
        const int64_t ahead = 4 * (int64_t)nt;
        std::vector<Files> out((size_t)nwin);
        std::vector<uint8_t> done((size_t)nwin, 0);
        std::mutex m;
        std::condition_variable cv_done, cv_written;
        int64_t written = 0;
        bool failed = false;
        std::string first_err;
        std::atomic<int64_t> next(0);
        auto fail_with = [&](const std::string& e) {
            std::lock_guard<std::mutex> g(m);
            if (!failed) first_err = e;
            failed = true;
            cv_done.notify_all();
            cv_written.notify_all();
        };
        auto work = [&]() {
            std::vector<CnsRow> rows;
            std::string e;
            for (int64_t w; (w = next.fetch_add(1)) < nwin;) {
                {
                    std::unique_lock<std::mutex> g(m);
                    cv_written.wait(g, [&] { return failed || w < written + ahead; });
                    if (failed) return;
                }
                const int64_t len = plan.call_len[w];
                rows.resize((size_t)len);
                for (int64_t j = 0; j < len; ++j) rows[(size_t)j] = resolve_row(plan, w, j, codes, calls, counts);
                Writer wr(dict, out[(size_t)w]);
                if (!wr.window(rows, &e)) {
                    fail_with(e.empty() ? std::string("write failed") : e);
                    return;
                }
                std::lock_guard<std::mutex> g(m);
                done[(size_t)w] = 1;
                cv_done.notify_all();
            }
        };
        auto write_all = [&]() {
            for (int64_t w = 0; w < nwin; ++w) {
                {
                    std::unique_lock<std::mutex> g(m);
                    cv_done.wait(g, [&] { return failed || done[(size_t)w]; });
                    if (failed) return;
                }
                Files& o = out[(size_t)w];
                std::string* parts[5] = {&o.f346, &o.frle, &o.f10, &o.f111213, &o.f1517};
                for (int f = 0; f < 5; ++f) {
                    if (!parts[f]->empty() &&
                        fwrite(parts[f]->data(), 1, parts[f]->size(), fb[f]) != parts[f]->size()) {
                        fail_with("write failed");
                        return;
                    }
                    std::string().swap(*parts[f]);
                }
                std::lock_guard<std::mutex> g(m);
                written = w + 1;
                cv_written.notify_all();
            }
        };
        std::thread writer(write_all);
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; ++t) pool.emplace_back(work);
        work();
        for (auto& th : pool) th.join();
        writer.join();
        if (failed) {
            *err = first_err;
            rc = 1;
        }
    } else if (rc == 0) {
        /* text mode: the column files exist and are empty, the table says 0 windows */
        fprintf(f12, "0\n");
    }
    for (FILE* x : {fb[0], fb[1], fb[2], fb[3], fb[4], f12})
        if (x && fclose(x) != 0 && rc == 0) {
            *err = "write failed";
            rc = 1;
        }
    return rc;
}

}  // namespace gsnp
