/*
 * posterior_check.cpp - the FP32 + FP64-fixup form's two claims, checked on
 * the CPU with the kernels' own per-site code (site_math.cuh, column.cuh,
 * compiled for the host) and the library's own tables (tables.cpp) on random
 * sites of realistic shape:
 *
 *  1. likelihood_fp32 stays within its bound: |S32 - S64| <= eps for every
 *     genotype, S64 being likelihood_fp64's sums in the reference's record
 *     order and eps = |S32| GSNP_FP32_K(num); and so do the sums of the deep
 *     kernel's warp form (record i on lane i mod 32, compensated per lane,
 *     the 32 lane sums then added by an xor butterfly) within
 *     |S32| (9 u + num 2^-45), the bound fast_posterior takes for them;
 *  2. every call decided from the FP32 sums equals the FP64 posterior's
 *     (site_posterior over S64):
 *       fast_posterior (the fast kernel's homozygous calls), and
 *       site_posterior with the eps bounds (the deferred kernel's first try);
 *  3. the same for adversarial sums: the FP64 sums of each site moved so
 *     that the runner-up genotype is within a few error bounds of the best,
 *     or so that 10 (tp1 - tp2) lies next to an integer, and FP32 sums
 *     anywhere inside the bound |S32 - S64| <= |S32| GSNP_FP32_K(num).
 *
 * Sites: hom-ref, hom-alt, het and low-fraction mixtures at depths 1 to 255,
 * qualities 0 to 40 with errors at their rates, repeated (strand, cycle)
 * keys, a few N reference codes, every tenth site monoploid (-m), one in
 * fifty a known-SNP site with its own prior row (-2); rank-sum on.  A
 * deterministic seed per run.
 * Prints "sites <n> fp32-decided <f> bounded-decided <b> max-relerr <r>
 * adversarial <a> decided <d>" and exits 0, or names the first failing site
 * and exits 1.
 * Usage: posterior_check <sites> <seed>
 */
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <random>
#include <string>
#include <vector>

#include "site_math.cuh"
#include "tables.h"

using namespace gsnp;

namespace {

/* a calibration matrix of the reference's layout: error 10^(-q/10) spread
 * over the three other bases, varying a little with the cycle */
void make_p_matrix(const gsnp_params& p, std::vector<double>* pm) {
    pm->assign(256UL * 256UL * 16UL, 1.0);
    for (int q = 0; q <= p.q_max - p.q_min; ++q)
        for (int coord = 0; coord < p.read_length; ++coord)
            for (int ref = 0; ref < 4; ++ref)
                for (int obs = 0; obs < 4; ++obs) {
                    const double e = std::min(0.75, pow(10.0, -q / 10.0) * (1.0 + 0.3 * coord / p.read_length));
                    (*pm)[((size_t)q << 12) | ((size_t)coord << 4) | (size_t)(ref << 2) | (size_t)obs] =
                        obs == ref ? 1.0 - e : e / 3.0;
                }
}

bool same(const SiteCall& x, const SiteCall& y) { return same_call(x, y); }

/* the prior row of one known-SNP site, as snp_log_prior_kernel forms it:
 * the novel priors of its reference base, with each listed genotype's
 * prior replaced (cpp/prior.cc:45-97, the device form) */
void snp_row(const CallArgs& a, uint8_t ori, bool validated, bool hapmap, const double* freq, double* lp,
             float* lp32) {
    for (int i = 0; i < 16; ++i) lp[i] = a.log_prior[((ori & 7) << 4) + i];
    const int t_base = ori & 3;
    for (int a1 = 0; a1 != 4; ++a1)
        for (int a2 = a1; a2 != 4; ++a2) {
            if (!(freq[a1] > 0 && freq[a2] > 0)) continue;
            double pr;
            if (!hapmap) {
                if (a1 == a2 && a1 == t_base) pr = 1;
                else if (a1 == t_base || a2 == t_base) pr = validated ? a.het_val : a.het_unval;
                else if (a1 == a2) pr = validated ? a.althom_val : a.althom_unval;
                else pr = validated ? a.het_val : a.het_unval;
            } else {
                pr = (a1 == a2 ? 1.0 : 2.0 * a.het_val) * freq[a1] * freq[a2];
            }
            lp[(a1 << 2) | a2] = gsnp_cr_log10(pr);
        }
    for (int t = 0; t < 12; ++t) lp32[t] = t < 10 ? (float)lp[genotype_of(t)] : 0.f;
}

void print_call(const char* tag, const SiteCall& c) {
    printf("  %s type1 %d base1 %d base2 %d q %d avg %d/%d cu %d/%d ca %d/%d rs %.17g flags %d\n", tag, c.type1,
           c.base1, c.base2, c.q_cns, c.avg_q1, c.avg_q2, c.cu1, c.cu2, c.ca1, c.ca2, c.rank_sum, c.flags);
}

}  // namespace

int main(int argc, char** argv) {
    const long n_sites = argc > 1 ? atol(argv[1]) : 100000;
    const unsigned long seed = argc > 2 ? strtoul(argv[2], nullptr, 10) : 1;
    gsnp_params p{};
    p.read_length = 100;
    p.q_min = 64;
    p.q_max = 64 + 40;
    p.pcr_dependency = log10(0.5);
    p.global_dependency = log10(0.9);
    p.het_val = 0.1;
    p.het_unval = 0.02;
    p.althom_val = 0.05;
    p.althom_unval = 0.01;
    p.rank_sum = 1;
    p.precision = 1;
    p.het_novel = 0.0010;
    p.althom_novel = 0.0005;
    p.transition_dominant = 1;
    std::vector<double> pm, prior(128), rank(64UL * 64UL * 2048UL);
    make_p_matrix(p, &pm);
    prior_table(p, p.transition_dominant, p.het_novel, p.althom_novel, prior.data());
    rank_table(rank.data());
    HostTables t;
    std::string err;
    if (build_tables(p, pm.data(), prior.data(), &t, &err) != 0) {
        printf("build_tables: %s\n", err.c_str());
        return 1;
    }
    CallArgs a{};
    a.L = t.L;
    a.lik64 = t.lik64.data();
    a.lik32 = t.lik32.data();
    a.lik32b = t.lik32.data() + (size_t)t.qa_rows * t.L * 4 * 8;
    a.qa_rows = t.qa_rows;
    a.qadj = t.qadj.data();
    a.tmax = t.tmax;
    a.gmax = t.gmax;
    a.p_prior = prior.data();
    a.log_prior = t.log_prior.data();
    a.log_prior32 = t.log_prior32.data();
    a.p_rank = rank.data();
    a.qmin = p.q_min;
    a.q_max_min = p.q_max - p.q_min;
    a.rank_sum = p.rank_sum;
    a.het_val = p.het_val;
    a.het_unval = p.het_unval;
    a.althom_val = p.althom_val;
    a.althom_unval = p.althom_unval;
    a.precision = 1;
    a.refine = 1;

    std::mt19937_64 rng(seed);
    auto uni = [&](double lo, double hi) { return std::uniform_real_distribution<double>(lo, hi)(rng); };
    auto below = [&](int n) { return (int)(rng() % (uint64_t)n); };
    static const char kChar[4] = {'A', 'C', 'T', 'G'};
    std::vector<uint32_t> recs, seen(64);
    long fast_decided = 0, bounded_decided = 0, adv_sites = 0, adv_decided = 0;
    double max_rel = 0.0;
    for (long site = 0; site < n_sites; ++site) {
        const int ref = below(4);
        const uint8_t ori = (uint8_t)(below(50) == 0 ? 4 + ref : ref);   /* a few N reference codes */
        const int kind = below(10);
        int alt = (ref + 1 + below(3)) & 3;
        double frac = kind < 6 ? 0.0 : kind < 7 ? 1.0 : kind < 9 ? uni(0.3, 0.7) : uni(0.02, 0.3);
        const int shape = below(20);
        const int depth = shape == 0 ? 1 + below(5) : shape < 17 ? 5 + below(60) : 60 + below(196);
        recs.clear();
        SitePileup sp{};
        for (int i = 0; i < depth && (int)recs.size() < kMaxRecords; ++i) {
            const int q = below(10) == 0 ? below(15) : 20 + below(21);
            int base = uni(0, 1) < frac ? alt : ref;
            if (uni(0, 1) < pow(10.0, -q / 10.0)) base = (base + 1 + below(3)) & 3;
            int coord = below(p.read_length), strand = below(2);
            if (!recs.empty() && below(8) == 0) {   /* a repeated (strand, cycle) key */
                const uint32_t w = recs[below((int)recs.size())];
                coord = rec_coord(w);
                strand = rec_strand(w);
            }
            recs.push_back(make_record(kChar[base], q, (uint32_t)coord, (uint32_t)strand));
            sp.cu[base] += 1;
            sp.qs[base] += q;
            sp.ca[base] += 1;
        }
        std::sort(recs.begin(), recs.end());
        sp.num = sp.dep_uni = (int)recs.size();
        for (int b = 0; b < 4; ++b) sp.ca[b] += (uint32_t)(below(4) == 0 ? below(3) : 0);
        sp.depth = sp.ca[0] + sp.ca[1] + sp.ca[2] + sp.ca[3] + (uint32_t)below(3);
        sp.repeat = sp.depth + (uint32_t)below(3);

        double tl64[16] = {0}, tl32[16] = {0}, eps[16] = {0};
        likelihood_fp64<2>(a, recs.data(), seen.data(), 1, sp.num, tl64);
        likelihood_fp32<2>(a, recs.data(), seen.data(), 1, sp.num, tl32, eps);
        for (int k = 0; k < 10; ++k) {
            const int g = genotype_of(k);
            const double d = fabs(tl32[g] - tl64[g]);
            if (tl64[g] != 0.0) max_rel = std::max(max_rel, d / fabs(tl64[g]));
            if (!(d <= eps[g])) {
                printf("site %ld: genotype %d: |S32 - S64| = %.3g above the bound %.3g (num %d)\n", site, g, d,
                       eps[g], sp.num);
                return 1;
            }
        }
        {
            /* the warp form of call_deep_kernel over the same walk */
            std::vector<Kahan10> lane(32);
            for (Kahan10& k : lane) k.init();
            walk_records<false, 2>(a, recs.data(), seen.data(), 1, sp.num, [&](int i, int qa, int coord, int o) {
                float x[10];
                lik32_row(a, qa, coord, o, x);
                lane[(size_t)(i & 31)].add(x);
            });
            float t[32][10];
            for (int l = 0; l < 32; ++l)
                for (int v = 0; v < 10; ++v) t[l][v] = lane[(size_t)l].s[v];
            for (int d = 16; d > 0; d >>= 1) {
                float u[32][10];
                for (int l = 0; l < 32; ++l)
                    for (int v = 0; v < 10; ++v) u[l][v] = __fadd_rn(t[l][v], t[l ^ d][v]);
                memcpy(t, u, sizeof t);
            }
            const double kw = 9.0 * 0x1p-24 + (double)sp.num * 0x1p-45;
            for (int k = 0; k < 10; ++k) {
                const int g = genotype_of(k);
                const double sw = (double)t[0][k], d = fabs(sw - tl64[g]);
                if (!(d <= fabs(sw) * kw) && !isinf(sw)) {
                    printf("site %ld: genotype %d: warp form |S32 - S64| = %.3g above %.3g (num %d)\n", site, g, d,
                           fabs(sw) * kw, sp.num);
                    return 1;
                }
            }
        }
        a.monoploid = site % 10 == 0;   /* -m: homozygous genotypes only */
        /* a known-SNP site (-2): its own prior row */
        static double snp_lp[16];
        static float snp_lp32[12];
        uint8_t code = ori;
        int64_t row = -1;
        if (below(50) == 0 && ori < 4) {
            double freq[4] = {0, 0, 0, 0};
            freq[ref] = uni(0.3, 1.0);
            freq[alt] = below(3) ? 1.0 - freq[ref] : 0.0;
            snp_row(a, ori, below(2) == 0, below(3) == 0, freq, snp_lp, snp_lp32);
            a.snp_lp = snp_lp;
            a.snp_lp32 = snp_lp32;
            code = (uint8_t)(ori | 8);
            row = 0;
        }
        double lp[16];
        load_log_prior(a, row, code, lp);
        auto nq = [&](int b) { return (int)((b * 7 + site) % 40); };
        SiteCall want;
        site_posterior<false>(a, code, sp, tl64, nullptr, lp, recs.data(), 1, nq, &want);
        float s[10];
        for (int k = 0; k < 10; ++k) s[k] = (float)tl32[genotype_of(k)];
        SiteCall got;
        if (fast_posterior(a, row, code, sp, s, sp.num, &got)) {
            ++fast_decided;
            if (!same(got, want)) {
                printf("site %ld: fast_posterior differs from the FP64 posterior (num %d, ori %d)\n", site, sp.num,
                       ori);
                print_call("fp32", got);
                print_call("fp64", want);
                return 1;
            }
        }
        if (site_posterior<false>(a, code, sp, tl32, eps, lp, recs.data(), 1, nq, &got)) {
            ++bounded_decided;
            if (!same(got, want)) {
                printf("site %ld: bounded posterior differs from the FP64 posterior (num %d, ori %d)\n", site,
                       sp.num, ori);
                print_call("fp32", got);
                print_call("fp64", want);
                return 1;
            }
        }

        /* adversarial sums: a runner-up within a few bounds of the best, or
         * 10 (tp1 - tp2) next to an integer; FP32 sums anywhere inside the
         * bound */
        if (sp.num == 0) continue;
        const double K = GSNP_FP32_K(sp.num);
        for (int variant = 0; variant < 4; ++variant) {
            double t64[16], t32[16], e32[16];
            for (int g = 0; g < 16; ++g) t64[g] = t32[g] = e32[g] = 0.0;
            int g1 = -1, g2 = -1;
            for (int k = 0; k < 10; ++k) {
                const int g = genotype_of(k);
                t64[g] = tl64[g];
                const double v = tl64[g] + lp[g];
                if (g1 < 0 || v >= tl64[g1] + lp[g1]) { g2 = g1; g1 = g; }
                else if (g2 < 0 || v >= tl64[g2] + lp[g2]) g2 = g;
            }
            const int other = variant < 2 ? g2 : genotype_of(below(10));
            if (other == g1) continue;
            const double scale = fabs(t64[other]) + fabs(t64[g1]) + 1.0;
            double gap;
            if (variant % 2 == 0) {
                gap = uni(-4.0, 4.0) * scale * K;            /* near a tie */
            } else {
                const double tp1 = t64[g1] + lp[g1];
                const double k10 = floor(10.0 * (tp1 - (t64[other] + lp[other])));
                gap = (std::max(k10, 1.0) + uni(-4.0, 4.0) * scale * K * 10.0) / 10.0;   /* next to an integer */
            }
            t64[other] = t64[g1] + lp[g1] - gap - lp[other];
            if (!(t64[other] <= 0.0)) continue;
            for (int k = 0; k < 10; ++k) {
                const int g = genotype_of(k);
                /* S32 first, then S64 within |S32| K of it */
                const float f = (float)t64[g];
                const double u = below(3) == 0 ? (below(2) ? 1.0 : -1.0) : uni(-1.0, 1.0);
                t32[g] = (double)f;
                t64[g] = (double)f + u * 0.999 * fabs((double)f) * K;
                if (t64[g] > 0.0) t64[g] = 0.0;
                e32[g] = fabs(t32[g]) * K;
            }
            ++adv_sites;
            SiteCall w64, w32;
            site_posterior<false>(a, code, sp, t64, nullptr, lp, recs.data(), 1, nq, &w64);
            float s32[10];
            for (int k = 0; k < 10; ++k) s32[k] = (float)t32[genotype_of(k)];
            bool decided = false;
            if (fast_posterior(a, row, code, sp, s32, sp.num, &w32)) {
                decided = true;
                if (!same(w32, w64)) {
                    printf("site %ld variant %d: fast_posterior differs on adversarial sums (num %d)\n", site,
                           variant, sp.num);
                    print_call("fp32", w32);
                    print_call("fp64", w64);
                    return 1;
                }
            }
            if (site_posterior<false>(a, code, sp, t32, e32, lp, recs.data(), 1, nq, &w32)) {
                decided = true;
                if (!same(w32, w64)) {
                    printf("site %ld variant %d: bounded posterior differs on adversarial sums (num %d)\n", site,
                           variant, sp.num);
                    print_call("fp32", w32);
                    print_call("fp64", w64);
                    return 1;
                }
            }
            adv_decided += decided;
        }
    }
    printf("sites %ld fp32-decided %ld bounded-decided %ld max-relerr %.3g adversarial %ld decided %ld\n", n_sites,
           fast_decided, bounded_decided, max_rel, adv_sites, adv_decided);
    return 0;
}
