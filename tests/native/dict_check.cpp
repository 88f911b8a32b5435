/*
 * dict_check.cpp - the -C writer's host dictionary codec (HostDictCodec in
 * gsnp_gb300/csrc/columns.cpp) against the codec's contract restated the
 * plain way (cpp/dict_compression.h:116-166): sort a copy, drop repeats
 * (-0.0 and +0.0 one entry, -0.0 when any -0.0 occurs), index each value by
 * lower_bound, pack floor(32 / bits) indices per word MSB-first with the last
 * word right-aligned.  Integers of narrow and wide ranges, negative values,
 * run lengths, doubles with both zeros; lengths 0 to 300,000; and the two
 * capacity errors.  Prints "checked <n> inputs" and exits 0, or names the
 * first difference and exits 1.
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <random>
#include <string>
#include <vector>

#include "columns.h"
#include "dict.h"

using namespace gsnp;

namespace {

template <class T>
bool plain_dict(const std::vector<T>& in, std::vector<uint32_t>* words, std::vector<T>* dict) {
    const size_t n = in.size();
    words->clear();
    dict->clear();
    if (n == 0) return true;
    std::vector<T> d(in);
    std::sort(d.begin(), d.end());
    d.erase(std::unique(d.begin(), d.end()), d.end());
    for (T& v : d)
        if (v == (T)0) {
            bool neg = false;
            for (size_t i = 0; i < n; ++i) neg = neg || (in[i] == (T)0 && std::signbit((double)in[i]));
            v = neg ? (T)(-0.0) : (T)0;
        }
    const int bits = dict_bits((unsigned long)d.size());
    const size_t per = (size_t)floor(32 / (double)bits);
    const size_t nw = (size_t)ceil(n / (double)per);
    for (size_t w = 0; w < nw; ++w) {
        const size_t first = w * per, cnt = (w == nw - 1) ? n - first : per;
        uint32_t out = 0;
        for (size_t i = 0; i < cnt; ++i)
            out = (out << bits) | (uint32_t)(std::lower_bound(d.begin(), d.end(), in[first + i]) - d.begin());
        words->push_back(out);
    }
    *dict = d;
    return true;
}

template <class T>
bool check(const char* what, const std::vector<T>& in) {
    std::vector<uint32_t> want_words;
    std::vector<T> want_dict;
    plain_dict(in, &want_words, &want_dict);
    const size_t n = in.size();
    std::vector<uint32_t> words(n + 1, 0xdeadbeefu);
    std::vector<T> dict(n + 1);
    unsigned long nw = n, nd = n;
    std::string err;
    const HostDictCodec codec;
    if (!codec.compress(in.data(), n, words.data(), &nw, dict.data(), &nd, &err)) {
        printf("%s (n %zu): failed: %s\n", what, n, err.c_str());
        return false;
    }
    if (nw != want_words.size() || nd != want_dict.size() ||
        memcmp(words.data(), want_words.data(), 4 * nw) != 0 ||
        memcmp(dict.data(), want_dict.data(), sizeof(T) * nd) != 0) {
        printf("%s (n %zu): words %lu/%zu dict %lu/%zu differ\n", what, n, nw, want_words.size(), nd,
               want_dict.size());
        return false;
    }
    return true;
}

}  // namespace

int main() {
    std::mt19937_64 rng(20251203);
    auto below = [&](uint64_t m) { return rng() % m; };
    long checked = 0;
    const size_t sizes[] = {0, 1, 2, 3, 31, 32, 33, 1000, 65537, 262144, 300000};
    for (size_t n : sizes) {
        for (int rep = 0; rep < 3; ++rep) {
            std::vector<int> narrow(n), wide(n), neg(n), few(n);
            std::vector<uint32_t> runs(n), sparse(n);
            std::vector<double> ratio(n), zeros(n);
            for (size_t i = 0; i < n; ++i) {
                narrow[i] = (int)below(100);
                wide[i] = (int)(uint32_t)rng();
                neg[i] = (int)below(2001) - 1000;
                few[i] = below(5) == 0 ? 7 : 99;
                runs[i] = 1 + (uint32_t)(below(8) == 0 ? below(262144) : below(4));
                sparse[i] = below(3) == 0 ? (uint32_t)rng() : (uint32_t)below(10);
                const uint64_t d = 1 + below(60);
                ratio[i] = below(50) == 0 ? 255.0 : (double)(d + below(3)) / (double)d;
                zeros[i] = below(4) == 0 ? -0.0 : below(3) == 0 ? 0.0 : (double)below(5) / 4.0;
            }
            if (rep == 1)
                for (size_t i = 0; i < n; ++i) zeros[i] = zeros[i] == 0.0 ? 0.0 : zeros[i];   /* +0.0 only */
            if (!(check("narrow int", narrow) && check("wide int", wide) && check("negative int", neg) &&
                  check("two values", few) && check("run lengths", runs) && check("sparse uint32", sparse) &&
                  check("ratios", ratio) && check("signed zeros", zeros)))
                return 1;
            checked += 8;
        }
    }
    /* the contract's two capacity errors */
    {
        const HostDictCodec codec;
        std::vector<int> in(100, 3);
        std::vector<uint32_t> words(100);
        std::vector<int> dict(100);
        std::string err;
        unsigned long nw = 100, nd = 99;
        if (codec.compress(in.data(), in.size(), words.data(), &nw, dict.data(), &nd, &err) ||
            err != "*numElementDict < numElementInData") {
            printf("dictionary capacity: %s\n", err.c_str());
            return 1;
        }
        err.clear();
        nw = 3;
        nd = 100;
        if (codec.compress(in.data(), in.size(), words.data(), &nw, dict.data(), &nd, &err) ||
            err != "numWordOutData < numWordCompressed") {
            printf("word capacity: %s\n", err.c_str());
            return 1;
        }
        checked += 2;
    }
    printf("checked %ld inputs\n", checked);
    return 0;
}
