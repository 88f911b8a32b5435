/*
 * tables.cpp - host-built lookup tables of the caller.
 *
 * Compiled with -ffp-contract=off so that every expression is evaluated as the
 * IEEE operations written.  Transcendentals that the reference evaluates on
 * the host use the C library here too (the calibration fill, the materialised
 * log10 table, the log10 quality table); the adjusted-quality table replaces
 * the reference's per-record device pow() with the C library's pow(), and the
 * prior table's log10 is the correctly rounded one of gsnp_crmath.h, as the
 * posterior kernel uses for dbSNP priors.
 */
#include "tables.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "gsnp_crmath.h"

namespace gsnp {

namespace {

/* kernel/likelihood_kernel.cu:226-231 */
int q_adjust(int q, int tmp, int gdc, double pcr, double glob, const double* log10tab) {
    int qa = (int)(pow(10.0, (log10tab[q] + (tmp - 1) * pcr + gdc * glob)) + 0.5);
    if (qa < 1) qa = 1;
    return qa;
}

}  // namespace

int build_tables(const gsnp_params& p, const double* pm, const double* p_prior, HostTables* t, std::string* err) {
    const int L = p.read_length;
    t->L = L;
    /* log10 of the record's q_score (kernel/likelihood_kernel.cu:83-87); entry
     * 64 is defined as log10(64), where the reference reads past its table */
    double log10tab[65];
    for (int i = 0; i < 65; ++i) log10tab[i] = log10((double)i);

    /* bounds of the adjusted-quality table: beyond them q_adj is 1 for every q
     * (both dependency coefficients are log10 of values in (0, 1], so q_adj
     * does not grow with tmp or gdc) */
    const double pcr = p.pcr_dependency, glob = p.global_dependency;
    if (!(pcr <= 0.0) || !(glob <= 0.0)) {
        *err = "dependency coefficients must lie in (0, 1]";
        return 1;
    }
    int tmax = 256, gmax = 256;
    if (pcr < 0.0)
        for (int tmp = 1; tmp < 256; ++tmp)
            if (q_adjust(64, tmp, 0, pcr, glob, log10tab) == 1) { tmax = tmp; break; }
    if (glob < 0.0)
        for (int g = 0; g < 256; ++g)
            if (q_adjust(64, 1, g, pcr, glob, log10tab) == 1) { gmax = g; break; }
    tmax = std::max(tmax, 2);
    gmax = std::max(gmax, 1);
    t->tmax = tmax;
    t->gmax = gmax;
    t->qadj.assign((size_t)tmax * gmax * 65, 1);
    int qa_max = 1;
    for (int tmp = 1; tmp < tmax; ++tmp)
        for (int g = 0; g < gmax; ++g)
            for (int q = 0; q < 65; ++q) {
                const int qa = q_adjust(q, tmp, g, pcr, glob, log10tab);
                if (qa > 255) {
                    *err = "adjusted quality above 255";
                    return 1;
                }
                t->qadj[((size_t)tmp * gmax + g) * 65 + q] = (uint8_t)qa;
                qa_max = std::max(qa_max, qa);
            }
    t->qa_rows = qa_max + 1;

    /* materialised genotype terms (kernel/likelihood_kernel.cu:137-161) for
     * the adjusted qualities and read cycles that can occur */
    t->lik64.assign((size_t)t->qa_rows * L * 4 * 10, 0.0);
    t->lik32.assign((size_t)t->qa_rows * L * 4 * 10, 0.0f);
    t->all_nonpositive = true;
    for (int q = 0; q < t->qa_rows; ++q)
        for (int c = 0; c < L; ++c)
            for (int o = 0; o < 4; ++o) {
                double* row = &t->lik64[(((size_t)q * L + c) * 4 + o) * 10];
                int k = 0;
                for (int a1 = 0; a1 < 4; ++a1)
                    for (int a2 = a1; a2 < 4; ++a2) {
                        const double x = pm[((unsigned long)q << 12) | ((unsigned long)c << 4) | (a1 << 2) | o];
                        const double y = pm[((unsigned long)q << 12) | ((unsigned long)c << 4) | (a2 << 2) | o];
                        row[k] = log10(0.5 * x + 0.5 * y);
                        /* the FP32 error bound is relative: every term must be
                         * <= 0 and round to 0 or to a normal FP32 number */
                        if (!(row[k] <= 0.0) || (row[k] < 0.0 && row[k] > -0x1p-126)) t->all_nonpositive = false;
                        ++k;
                    }
            }
    /* FP32 copy in two parts, so that a row takes two loads: columns 0-7 of
     * every row (32 bytes, one 256-bit load), then columns 8-9 (8 bytes) */
    const size_t rows = (size_t)t->qa_rows * L * 4;
    for (size_t r = 0; r < rows; ++r) {
        for (int k = 0; k < 8; ++k) t->lik32[r * 8 + k] = (float)t->lik64[r * 10 + k];
        for (int k = 8; k < 10; ++k) t->lik32[rows * 8 + r * 2 + (k - 8)] = (float)t->lik64[r * 10 + k];
    }

    t->log_prior.resize(128);
    for (int i = 0; i < 128; ++i) t->log_prior[i] = gsnp_cr_log10(p_prior[i]);
    static const int col_genotype[10] = {0, 1, 2, 3, 5, 6, 7, 10, 11, 15};
    t->log_prior32.assign(8 * 12, 0.0f);
    for (int r = 0; r < 8; ++r)
        for (int k = 0; k < 10; ++k) t->log_prior32[r * 12 + k] = (float)t->log_prior[r * 16 + col_genotype[k]];
    return 0;
}

void calibration_fill(const gsnp_params& p, const unsigned long long* counts, double* pm) {
    const int L = p.read_length;
    const unsigned long long sta_pow = 10;
    auto cnt = [&](int qc, int coord, int type) -> unsigned long long {
        return counts[((size_t)(qc - p.q_min) * L + coord) * 16 + type];
    };
    for (int qc = p.q_min; qc <= p.q_max; ++qc) {
        unsigned long long by_type[16] = {0}, by_t[4] = {0}, total = 0, mism = 0;
        for (int coord = 0; coord != L; ++coord)
            for (int type = 0; type != 16; ++type) {
                const unsigned long long v = cnt(qc, coord, type);
                by_type[type] += v;
                by_t[(type >> 2) & 3] += v;
                total += v;
                if (type % 5 != 0) mism += v;
            }
        const unsigned long long qrow = (unsigned long long)(qc - p.q_min) << 12;
        for (int coord = 0; coord != L; ++coord) {
            unsigned long long sum[4] = {0, 0, 0, 0};
            for (int type = 0; type != 16; ++type) sum[(type >> 2) & 3] += cnt(qc, coord, type);
            for (int tb = 0; tb != 4; ++tb)
                for (int o = 0; o != 4; ++o) {
                    double& v = pm[qrow | ((unsigned long long)coord << 4) | (tb << 2) | o];
                    const unsigned long long x = cnt(qc, coord, (tb << 2) | o);
                    if (x > sta_pow) v = ((double)x) / sum[tb];
                    else if (by_type[tb << 2 | o] > sta_pow) v = ((double)by_type[tb << 2 | o]) / by_t[tb];
                    else if (total > 0) v = (o == tb) ? ((double)(total - mism)) / total : ((double)mism) / total;
                    if (v == 0 || v == 1) {
                        if (o == tb) {
                            v = (1 - pow(10, -((qc - p.q_min) / 10.0)));
                            if (v < 0.25) v = 0.25;
                        } else {
                            v = (pow(10, -((qc - p.q_min) / 10.0)) / 3);
                            if (v > 0.25) v = 0.25;
                        }
                    }
                }
        }
    }
}

void prior_table(const gsnp_params&, int transition_dominant, double het_novel, double althom_novel, double* pr) {
    for (int i = 0; i < 128; ++i) pr[i] = 1.0;
    for (int tb = 0; tb != 4; tb++)
        for (int a1 = 0; a1 != 4; a1++)
            for (int a2 = a1; a2 != 4; a2++) {
                double& v = pr[tb << 4 | a1 << 2 | a2];
                if (a1 == tb && a2 == tb) v = 1;
                else if (a1 == tb || a2 == tb) v = het_novel;
                else if (a1 == a2) v = althom_novel;
                else v = het_novel * althom_novel;
                if (transition_dominant && ((a1 ^ tb) == 0x3 || (a2 ^ tb) == 0x3)) v *= 4;
            }
    for (int a1 = 0; a1 != 4; a1++)
        for (int a2 = a1; a2 != 4; a2++)
            for (int n = 4; n < 8; ++n) pr[n << 4 | a1 << 2 | a2] = (a1 == a2 ? 1 : (2 * het_novel)) * 0.25 * 0.25;
}

void rank_table(double* p_rank) {
    for (size_t i = 0; i < 64UL * 64UL * 2048UL; ++i) p_rank[i] = 1.0;
    double fact[64];
    fact[0] = 1.0;
    for (unsigned long long i = 1; i != 64; i++) fact[i] = fact[i - 1] * i;
    /* only the rows N-1 and N of the exact counts are needed at a time */
    std::vector<unsigned long long> prev(64UL * 2048UL, 0ULL), cur(64UL * 2048UL, 0ULL);
    prev[0] = 1;
    for (unsigned long long N = 1; N != 64; N++) {
        std::fill(cur.begin(), cur.end(), 0ULL);
        for (unsigned long long n1 = 0; n1 <= N; n1++) {
            const unsigned long long lo = (1 + n1) * n1 / 2, hi = (N + N - n1 + 1) * n1 / 2;
            for (unsigned long long T1 = lo; T1 <= hi; T1++) {
                cur[n1 << 11 | T1] = prev[(n1 << 11) | T1] + ((T1 >= N && n1 > 0) ? prev[((n1 - 1) << 11) | (T1 - N)] : 0);
                p_rank[(N << 17) | (n1 << 11) | T1] = cur[n1 << 11 | T1] / (fact[N] / (fact[n1] * fact[N - n1]));
            }
            double p_left = 0.0, p_right = 1.0;
            for (unsigned long long T1 = lo; T1 <= hi; T1++) {
                p_right = 1.0 - p_left;
                p_left += p_rank[(N << 17) | (n1 << 11) | T1];
                p_rank[N << 17 | n1 << 11 | T1] = (p_left < p_right ? p_left : p_right);
            }
        }
        std::swap(prev, cur);
    }
}

}  // namespace gsnp
