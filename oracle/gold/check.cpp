/*
 * oracle/gold/check.cpp - the restated backend (oracle/backend.cpp,
 * oracle/calling.cpp) against the reference's own CPU twins of its calling
 * kernels (oracle/gold/twins.cpp), window by window on seeded random input.
 * TEST INFRASTRUCTURE (see oracle/oracle.h).
 *
 *     gold_check <seed> <windows>
 *
 * Each window of 262,144 sites gets reads of mixed lengths at about 30x in
 * (start, file) order over a sample with SNPs at 1 in 200 sites (two thirds
 * heterozygous, so that the rank-sum test runs often), deep clusters of reads sharing starts (pcr
 * dependency, the 255-record cap), multi-hit reads, N and low-quality bases,
 * N reference runs, and known-SNP rows (validated or not, HapMap or not, a few
 * indels).  Windows differ in read length, dependency factors, monoploid mode
 * and the Ti/Tv prior.  The same reads go through both sides, and every field
 * is compared:
 *   - pileup: records per site in deposit order and all six count arrays, for
 *     the W + L sites of the window (gold_updateSparse, update_kernel.cu:96-195);
 *   - the materialised log10 table (likelihood_kernel.cu:137-161);
 *   - the sorted records and the 16 type_likely slots of every site, bit for
 *     bit (likelihoodSparse_kernel, likelihood_kernel.cu:168-256);
 *   - base1, base2, type1, q_cns and the rank-sum value (bit for bit) of every
 *     called site (gold_posterior, posterior_kernel.cu:254-426).
 * The posterior is required to match the twin compiled with correctly
 * rounded log10/exp exactly; its differences from the twin compiled with the
 * C library's functions are counted and printed.  Exit status 0 when every
 * required comparison matches.
 *
 * With GOLD_CHECK_PLANT set, one q_cns of the restated backend is changed
 * before the comparison, to show that the check reports it.
 */
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gsnp_backend.h"
#include "oracle.h"

extern "C" {
int twin_update(int n, const int* pos, const int* len, const int* hit, const char* strand, const char* read,
                const char* qual, int L, char qmin, uint32_t* records, uint32_t* num, int* count_uni, int* q_sum,
                int* count_all, int* depth, int* repeat_time, int* dep_uni);
void twin_materialize(const double* p_matrix, double* new_pmatrix);
void twin_likelihood(int n_sites, const uint32_t* records, const uint32_t* num, int L, double pcr, double glob,
                     const double* new_pmatrix, int* pcr_scratch, double* out);
void twin_posterior(int cr, int n_sites, const bool* nflag, const double* type_likely, const double* p_prior,
                    const double* p_rank, const uint32_t* records, const uint32_t* num, const int* count_uni,
                    const int* q_sum, const int* dep_uni, const int* count_all, const char* ori,
                    const bool* validated, const bool* hapmap, const bool* indel, const double* freq,
                    double het_val, double het_unval, double althom_val, double althom_unval, int rank_sum_mode,
                    int monoploid, int refine, int q_max_min, int L, char* base1, char* base2, char* type1,
                    int* q_cns, double* rank_sum);
}

namespace {

constexpr int W = GSNP_WIN_SIZE;
constexpr int R = GSNP_MAX_RECORDS_PER_SITE;
constexpr int LK = GSNP_LIKELY_SIZE;

/* SplitMix64 */
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x1234567ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    int below(int n) { return (int)((next() >> 32) * (uint64_t)n >> 32); }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

struct WindowCase {
    int L;
    int q_max_min;        /* highest quality above q_min */
    double pcr, glob;     /* log10 dependency factors */
    bool monoploid, tidom;
};

long g_fail = 0;

void fail(const char* what, long site, long long a, long long b) {
    if (g_fail < 20) fprintf(stderr, "MISMATCH %s at site %ld: oracle %lld, twin %lld\n", what, site, a, b);
    ++g_fail;
}

long long bits(double x) {
    long long v;
    memcpy(&v, &x, sizeof v);
    return v;
}

/* a calibrated-looking p_matrix[q][coord][ref][obs] (cpp/matrix.cc:129-205
 * gives values of this shape): error rate 10^(-q/10) varied by cycle */
void make_pmatrix(Rng& rng, std::vector<double>* pm) {
    pm->assign(GSNP_PMATRIX_SIZE, 1.0);
    for (int q = 0; q < 256; ++q)
        for (int c = 0; c < 256; ++c)
            for (int a = 0; a < 4; ++a) {
                double e = pow(10.0, -(q < 64 ? q : 63) / 10.0) * (0.7 + 0.6 * rng.uniform());
                if (e > 0.74) e = 0.74;
                for (int o = 0; o < 4; ++o) {
                    const double v = o == a ? 1.0 - e : e / 3.0 * (0.8 + 0.4 * rng.uniform());
                    (*pm)[((size_t)q << 12) | ((size_t)c << 4) | ((size_t)a << 2) | (size_t)o] = v;
                }
            }
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: gold_check <seed> <windows>\n");
        return 2;
    }
    const uint64_t seed = strtoull(argv[1], nullptr, 10);
    const int windows = atoi(argv[2]);
    static const WindowCase cases[] = {
        {100, 40, log10(0.5), log10(0.9), false, true},
        {50, 40, log10(0.5), log10(0.9), false, false},
        {150, 60, log10(0.9), log10(0.95), false, true},
        {100, 60, log10(0.25), log10(0.8), true, true},
    };
    const char qmin = 64;
    Rng rng(seed);
    std::vector<double> p_matrix, p_rank(GSNP_PRANK_SIZE, 0.0), p_prior(8 * 16, 0.0);
    oracle_rank_table(p_rank.data());
    std::vector<double> newp_o(256UL * 256UL * 4UL * 10UL), newp_t(256UL * 256UL * 4UL * 10UL);
    long sites_called = 0, records_total = 0, libm_diff = 0, known_snp_sites = 0, deep_sites = 0;
    long normal_path = 0, het_calls = 0;

    for (int wi = 0; wi < windows; ++wi) {
        const WindowCase& wc = cases[wi % 4];
        const int L = wc.L;
        const int n_sites = W + L;
        make_pmatrix(rng, &p_matrix);
        oracle_prior_table(0.0010, 0.0005, wc.tidom, p_prior.data());
        oracle_materialize_pmatrix(p_matrix.data(), newp_o.data());
        twin_materialize(p_matrix.data(), newp_t.data());
        for (size_t i = 0; i < newp_o.size(); ++i)
            if (bits(newp_o[i]) != bits(newp_t[i])) {
                fail("materialised table", (long)i, bits(newp_o[i]), bits(newp_t[i]));
                break;
            }

        /* reference: ACTG codes (cpp/chromosome.cc:28-64), N runs, known SNPs */
        std::vector<char> ori(n_sites);
        std::vector<bool> is_n(n_sites, false);
        for (int s = 0; s < n_sites; ++s) ori[s] = (char)rng.below(4);
        for (int k = 0; k < 6; ++k) {
            const int a = rng.below(n_sites - 3000), len = 1 + rng.below(2500);
            for (int s = a; s < a + len; ++s) { ori[s] = 7; is_n[s] = true; }
        }
        std::vector<char> valid_b(W), hapmap_b(W), indel_b(W);
        std::vector<double> freq(4 * (size_t)W, 0.0);
        for (int s = 0; s < W; ++s) {
            if (is_n[s] || rng.below(50) != 0) continue;
            ori[s] |= 8;
            ++known_snp_sites;
            valid_b[s] = rng.below(5) != 0;
            hapmap_b[s] = rng.below(2) == 0;
            indel_b[s] = rng.below(20) == 0;
            const int r = ori[s] & 3;
            const double f = 0.01 + 0.49 * rng.uniform();
            const int alt = (r + 1 + rng.below(3)) & 3;
            freq[4 * (size_t)s + r] = 1.0 - f;
            freq[4 * (size_t)s + alt] = f;
            const int third = (alt + 1) & 3;
            if (rng.below(8) == 0 && third != r) freq[4 * (size_t)s + third] = 0.01;
        }
        /* sample: SNPs at 1e-3 (het 2/3) */
        std::vector<int> hap[2];
        hap[0].resize(n_sites);
        hap[1].resize(n_sites);
        for (int s = 0; s < n_sites; ++s) {
            const int b = is_n[s] ? rng.below(4) : (ori[s] & 3);
            hap[0][s] = hap[1][s] = b;
            if (rng.below(200) == 0) {
                const int alt = (b + 1 + rng.below(3)) & 3;
                hap[rng.below(2)][s] = alt;
                if (rng.below(3) == 0) hap[0][s] = hap[1][s] = alt;
            }
        }

        /* reads: uniform starts at about 30x, plus clusters of shared starts */
        std::vector<int> starts;
        const int lens_choice[4] = {L, L, (L * 3) / 4, L / 2};
        const long n_uniform = (long)(30.0 * W / (0.8 * L));
        for (long i = 0; i < n_uniform; ++i) starts.push_back(rng.below(W));
        for (int c = 0; c < 40; ++c) {
            const int centre = rng.below(W - 20) + 10;
            const int extra = 100 + rng.below(500);
            for (int k = 0; k < extra; ++k) starts.push_back(centre + rng.below(21) - 10);
        }
        std::sort(starts.begin(), starts.end());
        const int n = (int)starts.size();
        std::vector<int> pos(n), len(n), hit(n), lenhit(n);
        std::vector<char> strand(n), read((size_t)n * L, 'A'), qual((size_t)n * L, (char)(qmin + 10));
        for (int r = 0; r < n; ++r) {
            pos[r] = starts[r];
            len[r] = lens_choice[rng.below(4)];
            hit[r] = rng.below(20) == 0 ? 2 + rng.below(4) : 1;
            lenhit[r] = (len[r] << 16) | hit[r];
            strand[r] = rng.below(2) ? '-' : '+';
            const int h = rng.below(2);
            for (int c = 0; c < len[r]; ++c) {
                const int s = pos[r] + c < n_sites ? pos[r] + c : n_sites - 1;
                const int cycle = strand[r] == '-' ? len[r] - 1 - c : c;
                int q = wc.q_max_min - (cycle * (wc.q_max_min - 2)) / (2 * L) - rng.below(12);
                if (q < 1) q = 1;
                int b = hap[h][s];
                if (rng.uniform() < pow(10.0, -q / 10.0)) b = (b + 1 + rng.below(3)) & 3;
                char ch = "ACTG"[b];
                if (rng.below(500) == 0) ch = 'N';
                char qc = (char)(qmin + q);
                if (rng.below(100) == 0) qc = (char)(qmin - 1 - rng.below(5));   /* below -q_min */
                read[(size_t)r * L + c] = ch;
                qual[(size_t)r * L + c] = qc;
            }
        }

        /* ---- pileup ---- */
        std::vector<uint32_t> rec_t((size_t)n_sites * R, 0xFFFFFFFFu), num_t(n_sites, 0);
        std::vector<int> cu_t(4 * (size_t)n_sites), qs_t(4 * (size_t)n_sites), ca_t(4 * (size_t)n_sites);
        std::vector<int> dp_t(n_sites), rp_t(n_sites), du_t(n_sites);
        const int mx_t = twin_update(n, pos.data(), len.data(), hit.data(), strand.data(), read.data(), qual.data(),
                                     L, qmin, rec_t.data(), num_t.data(), cu_t.data(), qs_t.data(), ca_t.data(),
                                     dp_t.data(), rp_t.data(), du_t.data());

        GSNPKernelInit(W, L, wc.pcr, wc.glob, p_matrix.data(), p_prior.data(), p_rank.data());
        std::vector<int> posArr(n_sites), site_match(2 * (size_t)W);
        cuda_init(W, L, 0, posArr.data());
        gold_pos_match(pos.data(), site_match.data(), n);
        st_update u;
        memset(&u, 0, sizeof u);
        u.readArr = read.data();
        u.qualArr = qual.data();
        u.hitArr = hit.data();
        u.read_lenArr = len.data();
        u.positionArr = pos.data();
        u.siteMatchArr = site_match.data();
        u.strandArr = strand.data();
        u.readLen_hitArr = lenhit.data();
        u.qmin = qmin;
        u._read_length = (unsigned)L;
        std::vector<int> cu_o(4 * (size_t)n_sites), qs_o(4 * (size_t)n_sites), ca_o(4 * (size_t)n_sites);
        std::vector<int> dp_o(n_sites), rp_o(n_sites), du_dummy(n_sites);
        const unsigned mx_o = cuda_updateSparse(&u, nullptr, nullptr, L, cu_o.data(), qs_o.data(), ca_o.data(),
                                                dp_o.data(), rp_o.data(), du_dummy.data(), n);
        OracleBackendView v = oracle_backend_view();
        unsigned mx_tw = 0;
        for (int s = 0; s < W; ++s) mx_tw = std::max(mx_tw, num_t[s]);
        if (mx_o != mx_tw) fail("largest record count", -1, mx_o, mx_tw);
        (void)mx_t;
        for (int s = 0; s < n_sites; ++s) {
            for (int b = 0; b < 4; ++b) {
                if (cu_o[4 * s + b] != cu_t[4 * s + b]) fail("count_uni", s, cu_o[4 * s + b], cu_t[4 * s + b]);
                if (qs_o[4 * s + b] != qs_t[4 * s + b]) fail("q_sum", s, qs_o[4 * s + b], qs_t[4 * s + b]);
                if (ca_o[4 * s + b] != ca_t[4 * s + b]) fail("count_all", s, ca_o[4 * s + b], ca_t[4 * s + b]);
            }
            if (dp_o[s] != dp_t[s]) fail("depth", s, dp_o[s], dp_t[s]);
            if (rp_o[s] != rp_t[s]) fail("repeat_time", s, rp_o[s], rp_t[s]);
            if (v.dep_uni[s] != du_t[s]) fail("dep_uni", s, v.dep_uni[s], du_t[s]);
            if (v.num[s] != num_t[s]) fail("record count", s, v.num[s], num_t[s]);
            for (unsigned k = 0; k < num_t[s] && k < v.num[s]; ++k)
                if (v.records[(size_t)s * R + k] != rec_t[(size_t)s * R + k])
                    fail("record (deposit order)", s, v.records[(size_t)s * R + k], rec_t[(size_t)s * R + k]);
            if (num_t[s] >= 200) ++deep_sites;
        }

        /* ---- sort and likelihood ---- */
        std::vector<double> lik_host((size_t)W * LK, 0.0);
        cuda_likelihoodSparse(lik_host.data(), W, mx_o, W + L, R);
        for (int s = 0; s < W; ++s) std::sort(rec_t.begin() + (size_t)s * R, rec_t.begin() + (size_t)s * R + num_t[s]);
        std::vector<double> lik_t((size_t)W * LK, 0.0);
        std::vector<int> pcr_scratch((size_t)W * 2 * L, 0);
        twin_likelihood(W, rec_t.data(), num_t.data(), L, wc.pcr, wc.glob, newp_t.data(), pcr_scratch.data(),
                        lik_t.data());
        v = oracle_backend_view();
        for (int s = 0; s < W; ++s) {
            for (unsigned k = 0; k < num_t[s]; ++k)
                if (v.records[(size_t)s * R + k] != rec_t[(size_t)s * R + k])
                    fail("record (sorted)", s, v.records[(size_t)s * R + k], rec_t[(size_t)s * R + k]);
            for (int g = 0; g < 16; ++g)
                if (bits(v.type_likely[(size_t)s * LK + g]) != bits(lik_t[(size_t)s * LK + g]))
                    fail("type_likely bits", s, bits(v.type_likely[(size_t)s * LK + g]),
                         bits(lik_t[(size_t)s * LK + g]));
            records_total += num_t[s];
        }

        /* ---- posterior ---- */
        bool* nflag = new bool[W];
        bool* validated = new bool[W];
        bool* hapmap = new bool[W];
        bool* indel = new bool[W];
        for (int s = 0; s < W; ++s) {
            nflag[s] = (ori[s] & 4) != 0 && dp_t[s] == 0;
            validated[s] = valid_b[s];
            hapmap[s] = hapmap_b[s];
            indel[s] = indel_b[s];
        }
        const double het_val = 0.10, het_unval = 0.02, althom_val = 0.05, althom_unval = 0.01;
        st_likelihood lk;
        memset(&lk, 0, sizeof lk);
        lk.nflag = nflag;
        lk.typeLikelihood = lik_host.data();
        std::vector<char> b1_o(W), b2_o(W), t1_o(W), b1_t(W), b2_t(W), t1_t(W), b1_l(W), b2_l(W), t1_l(W);
        std::vector<int> q_o(W), q_t(W), q_l(W);
        std::vector<double> rs_o(W), rs_t(W), rs_l(W);
        cuda_posterior(&lk, ori.data(), b1_o.data(), b2_o.data(), t1_o.data(), q_o.data(), rs_o.data(), validated,
                       hapmap, indel, freq.data(), het_val, het_unval, althom_val, althom_unval, true, wc.monoploid,
                       true, (char)wc.q_max_min, L, W, W, mx_o);
        for (int cr = 1; cr >= 0; --cr)
            twin_posterior(cr, W, nflag, lik_t.data(), p_prior.data(), p_rank.data(), rec_t.data(), num_t.data(),
                           cu_t.data(), qs_t.data(), du_t.data(), ca_t.data(), ori.data(), validated, hapmap, indel,
                           freq.data(), het_val, het_unval, althom_val, althom_unval, 1, wc.monoploid, 1,
                           wc.q_max_min, L, cr ? b1_t.data() : b1_l.data(), cr ? b2_t.data() : b2_l.data(),
                           cr ? t1_t.data() : t1_l.data(), cr ? q_t.data() : q_l.data(),
                           cr ? rs_t.data() : rs_l.data());
        if (getenv("GOLD_CHECK_PLANT"))
            for (int s = W / 2; s < W; ++s)
                if (!nflag[s]) {
                    q_o[s] ^= 1;
                    break;
                }
        for (int s = 0; s < W; ++s) {
            if (nflag[s]) continue;
            ++sites_called;
            if (b1_o[s] != b1_t[s]) fail("base1", s, b1_o[s], b1_t[s]);
            if (b2_o[s] != b2_t[s]) fail("base2", s, b2_o[s], b2_t[s]);
            if (t1_o[s] != t1_t[s]) fail("type1", s, t1_o[s], t1_t[s]);
            if (q_o[s] != q_t[s]) fail("q_cns", s, q_o[s], q_t[s]);
            if (bits(rs_o[s]) != bits(rs_t[s])) fail("rank_sum bits", s, bits(rs_o[s]), bits(rs_t[s]));
            if (b1_o[s] != b1_l[s] || b2_o[s] != b2_l[s] || t1_o[s] != t1_l[s] || q_o[s] != q_l[s] ||
                bits(rs_o[s]) != bits(rs_l[s]))
                ++libm_diff;
            if ((t1_t[s] & 3) != ((t1_t[s] >> 2) & 3)) {
                ++het_calls;
                const int a = t1_t[s] & 3, b = (t1_t[s] >> 2) & 3;
                if (cu_t[4 * s + a] + cu_t[4 * s + b] >= 64) ++normal_path;
            }
        }
        delete[] nflag;
        delete[] validated;
        delete[] hapmap;
        delete[] indel;
        fprintf(stderr, "window %d: L=%d, %d reads, mismatches so far %ld\n", wi, L, n, g_fail);
    }
    printf("{\"windows\": %d, \"sites_called\": %ld, \"records\": %ld, \"known_snp_sites\": %ld, "
           "\"sites_200_records_or_more\": %ld, \"het_calls\": %ld, \"het_calls_normal_path\": %ld, "
           "\"mismatches\": %ld, \"differences_with_libm_twin\": %ld}\n",
           windows, sites_called, records_total, known_snp_sites, deep_sites, het_calls, normal_path, g_fail,
           libm_diff);
    return g_fail == 0 ? 0 : 1;
}
