/*
 * column_check.cpp - the calling kernels' column sort and dependency walk
 * (gsnp_gb300/csrc/column.cuh), compiled for the host, against plain
 * restatements:
 *   sort_column<SLOTS>     std::sort of the column's first num words, the
 *                          order of the reference's per-site sort
 *                          (kernel/batchsort.cu:245-291); the slots past num
 *                          untouched;
 *   walk_records<U, BITS>  the reference's walk with one integer counter per
 *                          (strand, cycle) key, cleared at each observed-base
 *                          group (kernel/likelihood_kernel.cu:200-232): the
 *                          same (record, q_adj, cycle, base) sequence for 1-,
 *                          2- and 4-bit counts, with unit and larger
 *                          occurrence fields, tables shorter and longer than
 *                          16 rows, and keys repeated past every saturation.
 * Prints "checked <n> columns" and exits 0, or names the first difference
 * and exits 1.
 */
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <random>
#include <tuple>
#include <vector>

#include "column.cuh"

using gsnp::kTile;

namespace {

std::mt19937_64 rng(20251203);

int uniform(int lo, int hi) { return std::uniform_int_distribution<int>(lo, hi)(rng); }

/* a record word as the pileup builds it, with occurrence field occ */
uint32_t record(int base, int q, int coord, int strand, int occ) {
    static const char kBases[4] = {'A', 'C', 'T', 'G'};
    const uint32_t w = gsnp::make_record(kBases[base], q, (uint32_t)coord, (uint32_t)strand);
    return (w & ~0xffu) | (uint32_t)occ;
}

template <int SLOTS>
bool check_sort(int trials, long* columns) {
    std::vector<uint32_t> tile((size_t)SLOTS * kTile);
    for (int t = 0; t < trials; ++t) {
        const int kind = t % 3;
        std::vector<std::vector<uint32_t>> want(kTile);
        std::fill(tile.begin(), tile.end(), 0xA5A5A5A5u);
        for (int lane = 0; lane < kTile; ++lane) {
            const int pick = uniform(0, 5);
            const int num = pick == 0 ? 0 : pick == 1 ? SLOTS : pick == 2 ? std::min(SLOTS, 33) : uniform(0, SLOTS);
            for (int i = 0; i < num; ++i) {
                uint32_t w;
                if (kind == 0) w = (uint32_t)rng();
                else if (kind == 1) w = (uint32_t)uniform(0, 5);   /* many equal words */
                else w = record(uniform(0, 3), uniform(0, 40), uniform(0, 99), uniform(0, 1), 1);
                tile[(size_t)i * kTile + lane] = w;
                want[lane].push_back(w);
            }
            std::sort(want[lane].begin(), want[lane].end());
            gsnp::sort_column<SLOTS>(tile.data() + lane, num);
            for (int i = 0; i < SLOTS; ++i) {
                const uint32_t got = tile[(size_t)i * kTile + lane];
                const uint32_t exp = i < num ? want[lane][i] : 0xA5A5A5A5u;
                if (got != exp) {
                    printf("sort_column<%d>: lane %d num %d slot %d: %08x, want %08x\n", SLOTS, lane, num, i, got,
                           exp);
                    return false;
                }
            }
            ++*columns;
        }
    }
    return true;
}

typedef std::tuple<int, int, int, int> Step;   /* record, q_adj, cycle, base */

/* the reference's walk: an integer counter per key, cleared per base group */
std::vector<Step> walk_reference(const gsnp::CallArgs& a, const std::vector<uint32_t>& col) {
    std::vector<Step> out;
    std::vector<int> count(2 * a.L, 0);
    int gdc = -1, last_o = -1;
    for (size_t i = 0; i < col.size(); ++i) {
        const uint32_t w = col[i];
        const int o = gsnp::rec_base(w), coord = gsnp::rec_coord(w), q = gsnp::rec_q(w);
        if (o != last_o) {
            std::fill(count.begin(), count.end(), 0);
            gdc = -1;
            last_o = o;
        }
        const int key = gsnp::rec_strand(w) * a.L + coord;
        int tmp = count[key];
        for (int k = 0; k < gsnp::rec_occ(w); ++k) {
            if (tmp == 0) gdc += 1;
            tmp++;
            const int qa = (tmp < a.tmax && gdc < a.gmax) ? a.qadj[((size_t)tmp * a.gmax + gdc) * 65 + q] : 1;
            out.emplace_back((int)i, qa, coord, o);
        }
        count[key] = tmp;
    }
    return out;
}

template <bool UNIT_OCC, int BITS>
std::vector<Step> walk_column(const gsnp::CallArgs& a, const std::vector<uint32_t>& col) {
    std::vector<Step> out;
    std::vector<uint32_t> seen((size_t)gsnp::pcr_words(a.L, BITS), 0xFFFFFFFFu);
    gsnp::walk_records<UNIT_OCC, BITS>(a, col.data(), seen.data(), 1, (int)col.size(),
                                       [&](int i, int qa, int coord, int o) { out.emplace_back(i, qa, coord, o); });
    return out;
}

bool check_walk(int trials, long* columns) {
    static const int kTmax[] = {2, 5, 16, 17, 47};
    static const int kGmax[] = {1, 3, 64};
    static const int kL[] = {35, 100, 150, 255};
    for (int t = 0; t < trials; ++t) {
        gsnp::CallArgs a{};
        a.L = kL[uniform(0, 3)];
        a.tmax = kTmax[uniform(0, 4)];
        a.gmax = kGmax[uniform(0, 2)];
        std::vector<uint8_t> qadj((size_t)a.tmax * a.gmax * 65);
        for (auto& x : qadj) x = (uint8_t)uniform(1, 255);
        a.qadj = qadj.data();
        const bool unit = t % 2 == 0;
        /* keys drawn from a pool of 1 to 300 (strand, cycle) pairs, so that
         * some keys repeat past 15 */
        const int pool_n = std::vector<int>{1, 2, 3, 8, 40, 300}[uniform(0, 5)];
        std::vector<std::pair<int, int>> pool;
        for (int k = 0; k < pool_n; ++k) pool.emplace_back(uniform(0, 1), uniform(0, a.L - 1));
        const int num = uniform(0, 255);
        std::vector<uint32_t> col;
        for (int i = 0; i < num; ++i) {
            const auto& key = pool[uniform(0, pool_n - 1)];
            col.push_back(record(uniform(0, 3) * (uniform(0, 3) != 0), uniform(0, 63), key.second, key.first,
                                 unit ? 1 : uniform(1, 3)));
        }
        std::sort(col.begin(), col.end());
        const std::vector<Step> want = walk_reference(a, col);
        const std::vector<Step> got[3] = {
            unit ? walk_column<true, 1>(a, col) : walk_column<false, 1>(a, col),
            unit ? walk_column<true, 2>(a, col) : walk_column<false, 2>(a, col),
            unit ? walk_column<true, 4>(a, col) : walk_column<false, 4>(a, col)};
        for (int b = 0; b < 3; ++b) {
            if (got[b] != want) {
                size_t k = 0;
                while (k < got[b].size() && k < want.size() && got[b][k] == want[k]) ++k;
                printf("walk_records<%d, %d>: L %d tmax %d gmax %d num %d pool %d: step %zu of %zu/%zu differs\n",
                       (int)unit, 1 << b, a.L, a.tmax, a.gmax, num, pool_n, k, got[b].size(), want.size());
                return false;
            }
        }
        ++*columns;
    }
    return true;
}

}  // namespace

int main() {
    long columns = 0;
    const bool ok = check_sort<32>(200, &columns) && check_sort<40>(200, &columns) &&
                    check_sort<48>(200, &columns) && check_sort<64>(200, &columns) &&
                    check_sort<96>(100, &columns) && check_sort<128>(100, &columns) &&
                    check_sort<256>(100, &columns) && check_walk(20000, &columns);
    if (!ok) return 1;
    printf("checked %ld columns\n", columns);
    return 0;
}
