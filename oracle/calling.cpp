/*
 * oracle/calling.cpp - per-site calling math of the CPU oracle.
 *
 * TEST INFRASTRUCTURE (see oracle/oracle.h).  Compiled with
 * -O2 -fno-fast-math -ffp-contract=off so that every floating-point operation
 * is the single IEEE operation written in the source.
 */
#include "oracle.h"

#include "gsnp_crmath.h"

void oracle_materialize_pmatrix(const double* p, double* np) {
    /* kernel/likelihood_kernel.cu:137-161 */
    for (unsigned int q = 0; q < 256; ++q)
        for (unsigned int c = 0; c < 256; ++c)
            for (unsigned int o = 0; o < 4; ++o) {
                const unsigned long base = (((unsigned long)q << 10) | (c << 2) | o) * 10UL;
                int t = 0;
                for (unsigned int a1 = 0; a1 < 4; ++a1)
                    for (unsigned int a2 = a1; a2 < 4; ++a2) {
                        const double x = p[((unsigned long)q << 12) | (c << 4) | (a1 << 2) | o];
                        const double y = p[((unsigned long)q << 12) | (c << 4) | (a2 << 2) | o];
                        np[base + t] = log10(0.5 * x + 0.5 * y);
                        ++t;
                    }
            }
}

void oracle_log10_table(double* tab) {
    for (int i = 0; i < 65; ++i) tab[i] = log10((double)i);
}

int oracle_q_adjust(int q_score, int tmp, int gdc, double pcr, double glob, const double* log10tab) {
    /* kernel/likelihood_kernel.cu:226-231 */
    int q_adj = (int)(pow(10.0, (log10tab[q_score] + (tmp - 1) * pcr + gdc * glob)) + 0.5);
    if (q_adj < 1) q_adj = 1;
    return q_adj;
}

void oracle_site_likelihood(const unsigned int* rec, unsigned int num, int L, double pcr, double glob,
                            const double* log10tab, const double* np, double* out) {
    /* kernel/likelihood_kernel.cu:187-255, one site, records already sorted */
    static thread_local std::vector<int> pcr_count;
    static thread_local std::vector<int> touched;
    if ((int)pcr_count.size() < 2 * L) pcr_count.assign(2 * L, 0);
    double s[16];
    for (int i = 0; i < 16; ++i) s[i] = 0.0;
    int gdc = -1;
    int last_o = -1;
    for (unsigned int i = 0; i < num; ++i) {
        const unsigned int w = rec[i];
        const int o = (int)((w & 0x01800000u) >> 23);
        const int q = GSNP_MAX_QSCORE_ORACLE - (int)((w & 0x007e0000u) >> 17);
        const int coord = (int)((w & 0x0001fe00u) >> 9);
        const int strand = (int)((w & 0x00000100u) >> 8);
        const int occ = (int)(w & 0xffu);
        if (o != last_o) {
            gdc = -1;
            for (int idx : touched) pcr_count[idx] = 0;
            touched.clear();
            last_o = o;
        }
        const int idx = strand * L + coord;
        int tmp = pcr_count[idx];
        for (int k = 0; k < occ; ++k) {
            if (tmp == 0) gdc += 1;
            tmp++;
            const int q_adj = oracle_q_adjust(q, tmp, gdc, pcr, glob, log10tab);
            const unsigned long row = (((unsigned long)(unsigned int)q_adj << 10) | ((unsigned long)coord << 2) | (unsigned long)o) * 10UL;
            int t = 0;
            for (int a1 = 0; a1 < 4; ++a1)
                for (int a2 = a1; a2 < 4; ++a2) {
                    s[(a1 << 2) | a2] += np[row + t];
                    ++t;
                }
        }
        pcr_count[idx] = tmp;
        touched.push_back(idx);
    }
    for (int i = 0; i < 16; ++i) out[i] = s[i];
}

void oracle_snp_prior(double* prior, char ref, bool indel, bool validated, bool hapmap,
                      const double* freq, const OraclePriorParams& pp) {
    /* kernel/posterior_kernel.cu:575-633 (the device version: no exit on a
     * single listed allele) */
    if (indel) return;
    const int t_base = ref & 0x3;
    for (int a1 = 0; a1 != 4; ++a1)
        for (int a2 = a1; a2 != 4; ++a2) {
            if (!(freq[a1] > 0 && freq[a2] > 0)) continue;
            if (!hapmap) {
                if (a1 == a2 && a1 == t_base) prior[(a1 << 2) | a2] = 1;
                else if (a1 == t_base || a2 == t_base) prior[(a1 << 2) | a2] = validated ? pp.het_val : pp.het_unval;
                else if (a1 == a2) prior[(a1 << 2) | a2] = validated ? pp.althom_val : pp.althom_unval;
                else prior[(a1 << 2) | a2] = validated ? pp.het_val : pp.het_unval;
            } else {
                prior[(a1 << 2) | a2] = (a1 == a2 ? 1 : (2 * pp.het_val)) * freq[a1] * freq[a2];
            }
        }
}

double oracle_table_test(const double* pr, int n1, int n2, double T1, double T2) {
    /* kernel/posterior_kernel.cu:430-443; the interpolation index shifts the
     * total by 16 bits, not 17, as the reference does */
    if (n1 <= n2) {
        const int i1 = (n1 + n2) << 17 | n1 << 11 | (int)(T1);
        const int i2 = (n1 + n2) << 16 | n1 << 11 | (int)(T1 + 1);
        return pr[i1] + (T1 - (int)T1) * (pr[i2] - pr[i1]);
    }
    const int i3 = (n1 + n2) << 17 | n2 << 11 | (int)(T2);
    const int i4 = (n1 + n2) << 16 | n2 << 11 | (int)(T2 + 1);
    return pr[i3] + (T2 - (int)T2) * (pr[i4] - pr[i3]);
}

double oracle_normal_value(double z) {
    /* kernel/posterior_kernel.cu:446-467, exp correctly rounded */
    if (z > 6.0 || z < -6.0) return 0.0;
    const double b1 = 0.31938153, b2 = -0.356563782, b3 = 1.781477937, b4 = -1.821255978,
                 b5 = 1.330274429, p = 0.2316419, c2 = 0.39894228;
    const double a = fabs(z);
    const double t = 1.0 / (1.0 + a * p);
    const double b = c2 * gsnp_cr_exp((-z) * (z / 2.0));
    double n = ((((b5 * t + b4) * t + b3) * t + b2) * t + b1) * t;
    n = 1.0 - b * n;
    if (z < 0.0) n = 1.0 - n;
    return n > 0.5 ? 1 - n : n;
}

double oracle_normal_test(int n1, int n2, double T1, double T2) {
    /* kernel/posterior_kernel.cu:469-474 (integer divisions as written) */
    const double u1 = (T1 - n1 * (n1 + n2 + 1) / 2) / sqrt(n1 * n2 * (n1 + n2 + 1) / (double)12);
    const double u2 = (T2 - n2 * (n1 + n2 + 1) / 2) / sqrt(n1 * n2 * (n1 + n2 + 1) / (double)12);
    return oracle_normal_value(fabs(u1) > fabs(u2) ? u1 : u2);
}

double oracle_rank_test(const unsigned int* rec, unsigned int num, const int* cu, int bt,
                        const double* pr, int q_max_min) {
    /* kernel/posterior_kernel.cu:506-572 */
    const int a = bt & 3, b = (bt >> 2) & 3;
    if (a == b) return 1.0;
    if (cu[a] == 0 || cu[b] == 0) return 0.0;
    int sqc[65];
    double ra[65];
    double T[4] = {0.0, 0.0, 0.0, 0.0};
    bool need[4] = {false, false, false, false};
    for (int i = 0; i < 65; ++i) { sqc[i] = 0; ra[i] = 0.0; }
    need[a] = true;
    need[b] = true;
    for (unsigned int i = 0; i < num; ++i) {
        const unsigned int w = rec[i];
        const int o = (int)((w & 0x01800000u) >> 23);
        const int q = GSNP_MAX_QSCORE_ORACLE - (int)((w & 0x007e0000u) >> 17);
        const int occ = (int)(w & 0xffu);
        if (cu[o] == 0 || !need[o]) continue;
        sqc[q] += occ;
    }
    int rank = 0;
    const long top = std::min<long>(64, (long)q_max_min + 1);
    for (int q = 0; q <= top; ++q) {
        ra[q] = rank + (1 + sqc[q]) / 2.0;
        rank += sqc[q];
    }
    for (unsigned int i = 0; i < num; ++i) {
        const unsigned int w = rec[i];
        const int o = (int)((w & 0x01800000u) >> 23);
        const int q = GSNP_MAX_QSCORE_ORACLE - (int)((w & 0x007e0000u) >> 17);
        const int occ = (int)(w & 0xffu);
        if (cu[o] == 0 || !need[o]) continue;
        T[o] += ra[q] * occ;
    }
    if (cu[a] + cu[b] < 64) return oracle_table_test(pr, cu[a], cu[b], T[a], T[b]);
    return oracle_normal_test(cu[a], cu[b], T[a], T[b]);
}

void oracle_site_posterior(const OracleSiteIn& in, const double* p_prior, const double* p_rank,
                           const OraclePriorParams& pp, bool rank_sum_mode, bool monoploid,
                           bool refine, int q_max_min, OracleSiteOut* out) {
    /* kernel/posterior_kernel.cu:680-782 (posterior_kernel) */
    const int ori7 = (int)((unsigned long long)(long long)in.ori & 0x7);
    char base1 = 0, base2 = 0;
    int qual1 = -1, qual2 = -2, qual3 = -3;
    if (in.dep_uni) {
        for (int i = 0; i != 4; ++i) {
            const int v = in.q_sum[i];
            if (v >= qual1) { qual3 = qual2; base2 = base1; qual2 = qual1; base1 = (char)i; qual1 = v; }
            else if (v >= qual2) { qual3 = qual2; base2 = (char)i; qual2 = v; }
            else if (v >= qual3) { qual3 = v; }
        }
        if (qual1 == 0) base1 = (char)ori7;
        else if (qual2 == 0 && base1 != ori7) base2 = (char)ori7;
    } else {
        int c1 = 0, c2 = 0, c3 = 0;
        for (int i = 0; i != 4; ++i) {
            const int v = in.count_all[i];
            if (v >= c1) { c3 = c2; base2 = base1; c2 = c1; base1 = (char)i; c1 = v; }
            else if (v >= c2) { c3 = c2; base2 = (char)i; c2 = v; }
            else if (v >= c3) { c3 = v; }
        }
        if (c1 == 0) base1 = (char)ori7;
        else if (c2 == 0 && base1 != ori7) base2 = (char)ori7;
    }
    double prior[16];
    for (int i = 0; i < 16; ++i) prior[i] = p_prior[(ori7 << 4) + i];
    if ((in.ori & 0x8) && refine)
        oracle_snp_prior(prior, in.ori, in.indel, in.validated, in.hapmap, in.freq, pp);
    double tp[17];
    for (int i = 0; i < 17; ++i) tp[i] = 0.0;
    int type1 = 16, type2 = 16;
    for (int a1 = 0; a1 != 4; ++a1)
        for (int a2 = a1; a2 != 4; ++a2) {
            const int g = a1 << 2 | a2;
            if (monoploid && a1 != a2) continue;
            tp[g] = in.type_likely[g] + gsnp_cr_log10(prior[g]);
            if (tp[g] >= tp[type1] || type1 == 16) { type2 = type1; type1 = g; }
            else if (tp[g] >= tp[type2] || type2 == 16) { type2 = g; }
        }
    /* kernel/posterior_kernel.cu:826-864 (posterior_kernel2) */
    const double rs = rank_sum_mode
                          ? oracle_rank_test(in.records, in.num_records, in.count_uni, type1, p_rank, q_max_min)
                          : 1.0;
    int q;
    if (rs == 0.0) q = 0;
    else q = (int)(10 * (tp[type1] - tp[type2]) + 10 * gsnp_cr_log10(rs));
    if ((type1 & 3) == ((type1 >> 2) & 3)) {
        if (qual1 > 0 && base1 != (type1 & 3)) q = 0;
        else if (q > qual1 - qual2) q = qual1 - qual2;
    } else {
        if (in.q_sum[(int)base1] > 0 && in.q_sum[(int)base2] > 0 &&
            type1 == (base1 < base2 ? (base1 << 2 | base2) : (base2 << 2 | base1))) {
            if (q > qual2 - qual3) q = qual2 - qual3;
        } else {
            q = 0;
        }
    }
    if (q > 99) q = 99;
    if (q < 0) q = 0;
    out->base1 = base1;
    out->base2 = base2;
    out->type1 = (char)type1;
    out->type2 = (char)type2;
    out->q_cns = q;
    out->rank_sum = rs;
    out->qual1 = qual1;
    out->qual2 = qual2;
    out->qual3 = qual3;
    for (int i = 0; i < 17; ++i) out->type_prob[i] = tp[i];
}

int oracle_base2bits(char c) {
    switch (c) {
        case 'A': case 'a': return 0;
        case 'C': case 'c': return 1;
        case 'G': case 'g': return 2;
        case 'T': case 't': return 3;
        default: return -1;
    }
}

int oracle_bits_per_index(unsigned long n) {
    int bits = (int)ceil(log((double)(n)) / log((double)2.f));
    if (bits == 0) bits = 1;
    return bits;
}
