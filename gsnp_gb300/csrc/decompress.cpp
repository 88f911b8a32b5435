/*
 * decompress.cpp - reader of the -C compressed output: the cns rows back from
 * the six files, byte for byte as the reference's decompressor prints them
 * (cpp/decompression.cpp:130-232), and its column-by-column check against a
 * cns text (cpp/decompression.cpp:236-401).
 *
 * Per window, each file holds one block (layouts in columns.cpp, which writes
 * them; the readers restated here are cpp/compress.h:167-180,251-300,673-735,
 * 824-851,1027-1082,1214-1245):
 *   .3_4_6            all-N flag, row count, 2-bit reference bases, N ids,
 *                     the sites where the genotype / best base differ from it
 *   .5_7_8_9_14_16    six run-length + dictionary coded columns
 *   .10               2-bit second bases, N ids
 *   .11_12_13         common ids with dictionary-coded values, extra ids of
 *                     columns 12 and 13 (the writer's else-if drops a column
 *                     13 value where column 12 differs too: that loss is the
 *                     reference's)
 *   .15_17            sparse rank-sum values, dbSNP ids
 * The blocks are read in order; decoding and formatting run on several
 * threads, one window each, and the text is written in window order.
 */
#include "decompress.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "fmt_g6.h"

namespace gsnp {

namespace {

/* one window's decoded columns */
struct WindowCols {
    std::string chr;
    uint64_t start = 0, n = 0;
    std::vector<char> c3, c4, c6, c10;
    std::vector<int> c5, c7, c8, c9, c14, c11, c12, c13, c17;
    std::vector<double> c15, c16;
    void resize(size_t m) {
        for (auto* v : {&c3, &c4, &c6, &c10}) v->assign(m, 0);
        for (auto* v : {&c5, &c7, &c8, &c9, &c14, &c11, &c12, &c13, &c17}) v->assign(m, 0);
        c15.assign(m, 1.0);
        c16.assign(m, 255.0);
    }
};

/* a read position in one file's bytes; a short read is an error */
struct Cursor {
    const char* p = nullptr;
    const char* end = nullptr;
    std::string* err = nullptr;
    template <class T>
    bool get(T* out, size_t count, const char* what) {
        const size_t bytes = count * sizeof(T);
        if (count && (size_t)(end - p) < bytes) {
            if (err->empty()) *err = std::string("truncated ") + what;
            return false;
        }
        if (bytes) memcpy(out, p, bytes);
        p += bytes;
        return true;
    }
    bool skip(size_t bytes, const char* what) {
        if ((size_t)(end - p) < bytes) {
            if (err->empty()) *err = std::string("truncated ") + what;
            return false;
        }
        p += bytes;
        return true;
    }
};

/* The -C files in memory and every window's block offsets in them, found by
 * one pass over the block headers; windows then decode independently, on
 * any thread. */
class Reader {
public:
    explicit Reader(std::string* err) : err_(err) {}

    bool open(const std::string& base) {
        FILE* f12 = fopen((base + ".1_2").c_str(), "r");
        if (!f12) return fail("cannot open " + base + ".1_2");
        unsigned long nw = 0;
        bool ok = fscanf(f12, "%lu", &nw) == 1;
        char name[4096];
        for (unsigned long i = 0; ok && i < nw; ++i) {
            unsigned long s = 0, len = 0;
            ok = fscanf(f12, "%4095s %lu %lu", name, &s, &len) == 3;
            if (ok) windows_.push_back({name, s, len});
        }
        fclose(f12);
        if (!ok) return fail("malformed " + base + ".1_2");
        static const char* ext[5] = {".3_4_6", ".5_7_8_9_14_16", ".10", ".11_12_13", ".15_17"};
        for (int i = 0; i < 5; ++i) {
            FILE* f = fopen((base + ext[i]).c_str(), "rb");
            if (!f) return fail(std::string("cannot open ") + base + ext[i]);
            char buf[1 << 16];
            size_t got;
            while ((got = fread(buf, 1, sizeof(buf), f)) > 0) data_[i].insert(data_[i].end(), buf, buf + got);
            fclose(f);
        }
        return index();
    }

    size_t n_windows() const { return windows_.size(); }

    /* window w's blocks, decoded; safe to call for different windows at once */
    bool read(size_t w, WindowCols* out, std::string* err) const {
        const Win& win = windows_[w];
        out->chr = win.chr;
        out->start = win.start;
        out->n = win.len;
        out->resize((size_t)win.len);
        Cursor c[5];
        for (int i = 0; i < 5; ++i) {
            c[i].p = data_[i].data() + offs_[w][i];
            c[i].end = data_[i].data() + data_[i].size();
            c[i].err = err;
        }
        return read_346(c[0], out) && read_rle(c[1], out) && read_10(c[2], out) && read_111213(c[3], out) &&
               read_1517(c[4], out);
    }

private:
    struct Win {
        std::string chr;
        uint64_t start, len;
    };
    std::vector<Win> windows_;
    std::vector<char> data_[5];
    std::vector<std::array<size_t, 5>> offs_;
    std::string* err_;

    bool fail(const std::string& m) {
        if (err_->empty()) *err_ = m;
        return false;
    }
    static bool bad(std::string* err, const std::string& m) {
        if (err->empty()) *err = m;
        return false;
    }

    /* each window's block offsets: headers read, payloads skipped */
    bool index() {
        Cursor c[5];
        for (int i = 0; i < 5; ++i) {
            c[i].p = data_[i].data();
            c[i].end = data_[i].data() + data_[i].size();
            c[i].err = err_;
        }
        for (size_t w = 0; w < windows_.size(); ++w) {
            std::array<size_t, 5> o;
            for (int i = 0; i < 5; ++i) o[i] = (size_t)(c[i].p - data_[i].data());
            offs_.push_back(o);
            unsigned long p7[7];
            if (!c[0].get(p7, 7, ".3_4_6") || (p7[0] != 1 && !c[0].skip(p7[1], ".3_4_6"))) return false;
            int flag = 0;
            if (!c[1].get(&flag, 1, ".5_7_8_9_14_16")) return false;
            for (int k = 0; flag != 1 && k < 6; ++k) {
                unsigned long p6[6];
                if (!c[1].get(p6, 6, ".5_7_8_9_14_16") || !c[1].skip(p6[5], ".5_7_8_9_14_16")) return false;
            }
            if (!c[2].get(&flag, 1, ".10")) return false;
            if (flag != 1) {
                unsigned long p3[3];
                if (!c[2].get(p3, 3, ".10") || !c[2].skip(4 * (p3[1] + p3[0]), ".10")) return false;
            }
            if (!c[3].get(&flag, 1, ".11_12_13")) return false;
            if (flag != 1) {
                unsigned long p4[4];
                if (!c[3].get(p4, 4, ".11_12_13") || !c[3].skip(4 * (2 * p4[2] + 2 * p4[3] + p4[1]), ".11_12_13"))
                    return false;
                for (int k = 0; k < 3; ++k) {
                    unsigned long dp[2];
                    if (!c[3].get(dp, 2, ".11_12_13") || !c[3].skip(4 * (dp[0] + dp[1]), ".11_12_13")) return false;
                }
            }
            if (!c[4].get(&flag, 1, ".15_17")) return false;
            if (flag != 1) {
                int n = 0;
                if (!c[4].get(&n, 1, ".15_17") || n < 0 || !c[4].skip(12 * (size_t)n, ".15_17")) return false;
                if (!c[4].get(&n, 1, ".15_17") || n < 0 || !c[4].skip(4 * (size_t)n, ".15_17")) return false;
            }
        }
        return true;
    }

    /* 2-bit codes, first base in the high bits, the last word right-aligned
     * (kernel/compress_kernel.cu:85-160) */
    static void unpack2(const std::vector<uint32_t>& code, size_t n, char* out) {
        static const char kBase[4] = {'A', 'C', 'G', 'T'};
        const size_t nw = code.size();
        for (size_t w = 0; w < nw; ++w) {
            const size_t first = w * 16, nb = std::min<size_t>(16, n - std::min(n, first));
            for (size_t i = 0; i < nb; ++i) out[first + i] = kBase[(code[w] >> (2 * (nb - 1 - i))) & 3u];
        }
    }

    /* bits per dictionary index as the codec computes it
     * (cpp/dict_compression.h:47-58): ceil(log(n) / log(2)), at least 1 */
    static int index_bits(uint64_t n_dict) {
        int b = (int)ceil(log((double)n_dict) / log((double)2.f));
        return b == 0 ? 1 : b;
    }

    /* MSB-first packed dictionary indices, the last word right-aligned */
    template <class T>
    static bool undict(const std::vector<uint32_t>& words, const std::vector<T>& dict, size_t n, T* out,
                       std::string* err) {
        if (words.empty() || n == 0) return true;
        const int bits = index_bits(dict.size());
        const size_t per = (size_t)(32 / bits);
        const uint32_t mask = bits >= 32 ? 0xffffffffu : ((1u << bits) - 1u);
        for (size_t w = 0; w < words.size(); ++w) {
            const size_t first = w * per;
            if (first >= n) break;
            const size_t k = (w == words.size() - 1) ? n - first : std::min(per, n - first);
            for (size_t i = 0; i < k; ++i) {
                const uint32_t idx = (words[w] >> (bits * (k - 1 - i))) & mask;
                if (idx >= dict.size()) return bad(err, "dictionary index out of range");
                out[first + i] = dict[idx];
            }
        }
        return true;
    }

    static bool read_346(Cursor& f, WindowCols* o) {
        unsigned long p[7];
        if (!f.get(p, 7, ".3_4_6")) return false;
        const size_t n = p[2];
        if (n > o->n) return bad(f.err, ".3_4_6 block longer than its window");
        if (p[0] == 1) {
            std::fill(o->c3.begin(), o->c3.begin() + n, 'N');
            std::fill(o->c4.begin(), o->c4.begin() + n, 'N');
            std::fill(o->c6.begin(), o->c6.begin() + n, 'N');
            return true;
        }
        std::vector<int> id4(p[5]), id6(p[6]), idn(p[4]);
        std::vector<char> v4(p[5]), v6(p[6]);
        std::vector<uint32_t> code(p[3]);
        if (!(f.get(id4.data(), id4.size(), ".3_4_6") && f.get(v4.data(), v4.size(), ".3_4_6") &&
              f.get(id6.data(), id6.size(), ".3_4_6") && f.get(v6.data(), v6.size(), ".3_4_6") &&
              f.get(idn.data(), idn.size(), ".3_4_6") && f.get(code.data(), code.size(), ".3_4_6")))
            return false;
        unpack2(code, n, o->c3.data());
        for (int i : idn) {
            if (i < 0 || (size_t)i >= n) return bad(f.err, "N id out of range");
            o->c3[(size_t)i] = 'N';
        }
        std::copy(o->c3.begin(), o->c3.begin() + n, o->c4.begin());
        std::copy(o->c3.begin(), o->c3.begin() + n, o->c6.begin());
        for (size_t i = 0; i < id4.size(); ++i) {
            if (id4[i] < 0 || (size_t)id4[i] >= n) return bad(f.err, "column 4 id out of range");
            o->c4[(size_t)id4[i]] = v4[i];
        }
        for (size_t i = 0; i < id6.size(); ++i) {
            if (id6[i] < 0 || (size_t)id6[i] >= n) return bad(f.err, "column 6 id out of range");
            o->c6[(size_t)id6[i]] = v6[i];
        }
        return true;
    }

    template <class T>
    static bool rle_column(Cursor& f, T* out, size_t n) {
        unsigned long p[6];
        if (!f.get(p, 6, ".5_7_8_9_14_16")) return false;
        const size_t runs = p[0];
        std::vector<uint32_t> cv(p[1]), cl(p[2]), dl(p[4]);
        std::vector<T> dv(p[3]);
        if (!(f.get(cv.data(), cv.size(), ".5_7_8_9_14_16") && f.get(cl.data(), cl.size(), ".5_7_8_9_14_16") &&
              f.get(dv.data(), dv.size(), ".5_7_8_9_14_16") && f.get(dl.data(), dl.size(), ".5_7_8_9_14_16")))
            return false;
        std::vector<T> val(runs);
        std::vector<uint32_t> len(runs);
        if (!undict(cv, dv, runs, val.data(), f.err) || !undict(cl, dl, runs, len.data(), f.err)) return false;
        size_t at = 0;
        for (size_t r = 0; r < runs; ++r) {
            if (at + len[r] > n) return bad(f.err, "run lengths exceed the window");
            std::fill(out + at, out + at + len[r], val[r]);
            at += len[r];
        }
        return true;
    }

    static bool read_rle(Cursor& f, WindowCols* o) {
        int flag = 0;
        if (!f.get(&flag, 1, ".5_7_8_9_14_16")) return false;
        if (flag == 1) return true;   /* zeros and 255.0, as resize left them */
        const size_t n = o->n;
        return rle_column(f, o->c5.data(), n) && rle_column(f, o->c7.data(), n) && rle_column(f, o->c8.data(), n) &&
               rle_column(f, o->c9.data(), n) && rle_column(f, o->c14.data(), n) && rle_column(f, o->c16.data(), n);
    }

    static bool read_10(Cursor& f, WindowCols* o) {
        int flag = 0;
        if (!f.get(&flag, 1, ".10")) return false;
        if (flag == 1) {
            std::fill(o->c10.begin(), o->c10.end(), 'N');
            return true;
        }
        unsigned long p[3];
        if (!f.get(p, 3, ".10")) return false;
        if (p[2] != o->n) return bad(f.err, ".10 block length differs from its window");
        std::vector<uint32_t> code(p[1]), nid(p[0]);
        if (!f.get(code.data(), code.size(), ".10") || !f.get(nid.data(), nid.size(), ".10")) return false;
        unpack2(code, o->n, o->c10.data());
        for (uint32_t i : nid) {
            if (i >= o->n) return bad(f.err, "column 10 N id out of range");
            o->c10[i] = 'N';
        }
        return true;
    }

    static bool read_111213(Cursor& f, WindowCols* o) {
        int flag = 0;
        if (!f.get(&flag, 1, ".11_12_13")) return false;
        if (flag == 1) return true;
        unsigned long p[4];
        if (!f.get(p, 4, ".11_12_13")) return false;
        if (p[0] != o->n) return bad(f.err, ".11_12_13 block length differs from its window");
        std::vector<int> e12id(p[2]), e12(p[2]), e13id(p[3]), e13(p[3]), cid(p[1]);
        if (!(f.get(e12id.data(), e12id.size(), ".11_12_13") && f.get(e12.data(), e12.size(), ".11_12_13") &&
              f.get(e13id.data(), e13id.size(), ".11_12_13") && f.get(e13.data(), e13.size(), ".11_12_13") &&
              f.get(cid.data(), cid.size(), ".11_12_13")))
            return false;
        std::vector<int> vals[3];
        for (auto& v : vals) {
            unsigned long dp[2];
            if (!f.get(dp, 2, ".11_12_13")) return false;
            std::vector<uint32_t> words(dp[0]);
            std::vector<int> dict(dp[1]);
            if (!f.get(words.data(), words.size(), ".11_12_13") ||
                !f.get(dict.data(), dict.size(), ".11_12_13"))
                return false;
            v.assign(cid.size(), 0);
            if (!undict(words, dict, cid.size(), v.data(), f.err)) return false;
        }
        const size_t n = o->n;
        for (size_t i = 0; i < cid.size(); ++i) {
            if (cid[i] < 0 || (size_t)cid[i] >= n) return bad(f.err, "column 11 id out of range");
            o->c11[(size_t)cid[i]] = vals[0][i];
            o->c12[(size_t)cid[i]] = vals[1][i];
            o->c13[(size_t)cid[i]] = vals[2][i];
        }
        for (size_t i = 0; i < e12id.size(); ++i) {
            if (e12id[i] < 0 || (size_t)e12id[i] >= n) return bad(f.err, "column 12 id out of range");
            o->c12[(size_t)e12id[i]] = e12[i];
        }
        for (size_t i = 0; i < e13id.size(); ++i) {
            if (e13id[i] < 0 || (size_t)e13id[i] >= n) return bad(f.err, "column 13 id out of range");
            o->c13[(size_t)e13id[i]] = e13[i];
        }
        return true;
    }

    static bool read_1517(Cursor& f, WindowCols* o) {
        int flag = 0;
        if (!f.get(&flag, 1, ".15_17")) return false;
        if (flag == 1) return true;
        int cnt = 0;
        if (!f.get(&cnt, 1, ".15_17") || cnt < 0) return bad(f.err, "truncated .15_17");
        std::vector<int> id((size_t)cnt);
        std::vector<double> val((size_t)cnt);
        if (!f.get(id.data(), id.size(), ".15_17") || !f.get(val.data(), val.size(), ".15_17"))
            return false;
        for (size_t i = 0; i < id.size(); ++i) {
            if (id[i] < 0 || (uint64_t)id[i] >= o->n) return bad(f.err, "column 15 id out of range");
            o->c15[(size_t)id[i]] = val[i];
        }
        if (!f.get(&cnt, 1, ".15_17") || cnt < 0) return bad(f.err, "truncated .15_17");
        id.assign((size_t)cnt, 0);
        if (!f.get(id.data(), id.size(), ".15_17")) return false;
        for (int i : id) {
            if (i < 0 || (uint64_t)i >= o->n) return bad(f.err, "column 17 id out of range");
            o->c17[(size_t)i] = 1;
        }
        return true;
    }
};

char* put_u(char* p, uint64_t v) {
    char tmp[24];
    int k = 0;
    do {
        tmp[k++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    while (k) *p++ = tmp[--k];
    return p;
}

char* put_i(char* p, int v) {
    if (v < 0) {
        *p++ = '-';
        return put_u(p, (uint64_t)(-(int64_t)v));
    }
    return put_u(p, (uint64_t)v);
}

char* put_g6(char* p, double v) {
    const int n = fmt_g6(v, p);
    if (n > 0) return p + n;
    return p + snprintf(p, 64, "%#.6g", v);
}

/* The rows of one window as the reference's decompressor streams them:
 * chars, ints, then both doubles with showpoint at the default precision
 * (%#.6g); a site whose reference, genotype and best base are all N is a
 * fixed literal (cpp/decompression.cpp:201-217). */
void format_window(const WindowCols& w, std::string* out) {
    static const char kNRow[] = "N\tN\t0\tN\t0\t0\t0\tN\t0\t0\t0\t0\t1.000\t255.000\t0\n";
    out->clear();
    out->resize(w.n * (w.chr.size() + 160));
    char* p = &(*out)[0];
    for (uint64_t i = 0; i < w.n; ++i) {
        memcpy(p, w.chr.data(), w.chr.size());
        p += w.chr.size();
        *p++ = '\t';
        p = put_u(p, w.start + i);
        *p++ = '\t';
        if (w.c3[i] == 'N' && w.c4[i] == 'N' && w.c6[i] == 'N') {
            memcpy(p, kNRow, sizeof(kNRow) - 1);
            p += sizeof(kNRow) - 1;
            continue;
        }
        *p++ = w.c3[i];
        *p++ = '\t';
        *p++ = w.c4[i];
        *p++ = '\t';
        p = put_i(p, w.c5[i]);
        *p++ = '\t';
        *p++ = w.c6[i];
        *p++ = '\t';
        for (int v : {w.c7[i], w.c8[i], w.c9[i]}) {
            p = put_i(p, v);
            *p++ = '\t';
        }
        *p++ = w.c10[i];
        *p++ = '\t';
        for (int v : {w.c11[i], w.c12[i], w.c13[i], w.c14[i]}) {
            p = put_i(p, v);
            *p++ = '\t';
        }
        p = put_g6(p, w.c15[i]);
        *p++ = '\t';
        p = put_g6(p, w.c16[i]);
        *p++ = '\t';
        p = put_i(p, w.c17[i]);
        *p++ = '\n';
    }
    out->resize((size_t)(p - out->data()));
}

int default_threads() {
    const unsigned n = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(n, 32u));
}

}  // namespace

int decompress_columns(const std::string& base, const std::string& out_path, int threads, std::string* err) {
    Reader rd(err);
    if (!rd.open(base)) return 1;
    FILE* out = fopen(out_path.c_str(), "wb");
    if (!out) {
        *err = "cannot create " + out_path;
        return 1;
    }
    if (threads <= 0) threads = default_threads();
    std::vector<std::string> text((size_t)std::max(1, threads) * 2);
    bool ok = true;
    /* format per window, then write the batch in order */
    const size_t batch = text.size();
    const size_t nw = rd.n_windows();
    std::vector<WindowCols> cols(batch);
    std::vector<std::string> errs(batch);
    for (size_t w0 = 0; w0 < nw && ok; w0 += batch) {
        const size_t k = std::min(batch, nw - w0);
        std::atomic<size_t> next(0);
        std::atomic<bool> good(true);
        auto work = [&]() {
            for (size_t i; (i = next.fetch_add(1)) < k;) {
                if (!rd.read(w0 + i, &cols[i], &errs[i])) {
                    good = false;
                    continue;
                }
                format_window(cols[i], &text[i]);
            }
        };
        const int nt = (int)std::min<size_t>(k, (size_t)threads);
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; ++t) pool.emplace_back(work);
        work();
        for (auto& th : pool) th.join();
        if (!good) {
            for (const std::string& e : errs)
                if (!e.empty() && err->empty()) *err = e;
            ok = false;
            break;
        }
        for (size_t i = 0; i < k && ok; ++i)
            ok = fwrite(text[i].data(), 1, text[i].size(), out) == text[i].size();
    }
    if (fclose(out) != 0) ok = false;
    if (!ok && err->empty()) *err = "write failed";
    return ok ? 0 : 1;
}

namespace {

/* one cns text row split into its 17 columns */
struct TextRow {
    const char* f[17];
    size_t len[17];
};

bool split_row(const char* b, const char* e, TextRow* r) {
    int k = 0;
    const char* s = b;
    for (const char* p = b; p <= e && k < 17; ++p)
        if (p == e || *p == '\t') {
            r->f[k] = s;
            r->len[k] = (size_t)(p - s);
            ++k;
            s = p + 1;
        }
    return k == 17;
}

long parse_long(const char* s, size_t n) { return strtol(std::string(s, n).c_str(), nullptr, 10); }
double parse_double(const char* s, size_t n) { return strtod(std::string(s, n).c_str(), nullptr); }

}  // namespace

int check_columns(const std::string& cns_path, const std::string& base, std::string* report, std::string* err) {
    Reader rd(err);
    if (!rd.open(base)) return 1;
    FILE* f = fopen(cns_path.c_str(), "rb");
    if (!f) {
        *err = "cannot open " + cns_path;
        return 1;
    }
    std::string text;
    {
        char buf[1 << 16];
        size_t got;
        while ((got = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
        fclose(f);
    }
    /* row offsets of every window */
    std::vector<size_t> row_at;
    for (size_t i = 0; i < text.size();) {
        row_at.push_back(i);
        const size_t e = text.find('\n', i);
        i = e == std::string::npos ? text.size() : e + 1;
    }
    row_at.push_back(text.size());
    const size_t nrows = row_at.size() - 1;
    size_t row = 0;
    WindowCols w;
    for (size_t wi = 0; wi < rd.n_windows(); ++wi) {
        if (!rd.read(wi, &w, err)) return 1;
        for (uint64_t i = 0; i < w.n; ++i, ++row) {
            if (row >= nrows) {
                *report = "the cns text has fewer rows than the compressed files";
                return 2;
            }
            const char* b = text.data() + row_at[row];
            const char* e = text.data() + row_at[row + 1];
            if (e > b && e[-1] == '\n') --e;
            TextRow r;
            auto bad = [&](const char* col) {
                char m[160];
                snprintf(m, sizeof(m), "row %zu (window %zu, site %llu): %s differs", row, wi,
                         (unsigned long long)(w.start + i), col);
                *report = m;
                return 2;
            };
            if (!split_row(b, e, &r)) return bad("the column count");
            /* cpp/decompression.cpp:330-384: columns 1-2 exactly, chars and
             * ints exactly, columns 15 and 16 within 1e-5 */
            if (std::string(r.f[0], r.len[0]) != w.chr || (uint64_t)parse_long(r.f[1], r.len[1]) != w.start + i)
                return bad("column 1 or 2");
            const char chars[4] = {w.c3[i], w.c4[i], w.c6[i], w.c10[i]};
            const int char_col[4] = {2, 3, 5, 9};
            for (int k = 0; k < 4; ++k)
                if (r.len[char_col[k]] != 1 || r.f[char_col[k]][0] != chars[k]) {
                    char name[24];
                    snprintf(name, sizeof(name), "column %d", char_col[k] + 1);
                    return bad(name);
                }
            const int ints[9] = {w.c5[i], w.c7[i], w.c8[i], w.c9[i], w.c11[i], w.c12[i], w.c13[i], w.c14[i], w.c17[i]};
            const int int_col[9] = {4, 6, 7, 8, 10, 11, 12, 13, 16};
            for (int k = 0; k < 9; ++k)
                if (parse_long(r.f[int_col[k]], r.len[int_col[k]]) != ints[k]) {
                    char name[24];
                    snprintf(name, sizeof(name), "column %d", int_col[k] + 1);
                    return bad(name);
                }
            if (fabs(parse_double(r.f[14], r.len[14]) - w.c15[i]) > 1e-5) return bad("column 15");
            if (fabs(parse_double(r.f[15], r.len[15]) - w.c16[i]) > 1e-5) return bad("column 16");
        }
    }
    if (row != nrows) {
        *report = "the cns text has more rows than the compressed files";
        return 2;
    }
    *report = "all " + std::to_string(row) + " rows match";
    return 0;
}

}  // namespace gsnp

extern "C" int gsnp_decompress_columns(const char* base, const char* out_path, int threads, char* err, int err_len) {
    std::string e;
    const int rc = (base && out_path) ? gsnp::decompress_columns(base, out_path, threads, &e) : (e = "null path", 1);
    if (err && err_len > 0) snprintf(err, (size_t)err_len, "%s", e.c_str());
    return rc == 0 ? 0 : 6;
}

extern "C" int gsnp_check_columns(const char* cns_path, const char* base, char* report, int report_len) {
    std::string rep, e;
    const int rc = (cns_path && base) ? gsnp::check_columns(cns_path, base, &rep, &e) : (e = "null path", 1);
    if (report && report_len > 0) snprintf(report, (size_t)report_len, "%s", rc == 1 ? e.c_str() : rep.c_str());
    return rc == 0 ? 0 : (rc == 2 ? 7 : 6);
}
