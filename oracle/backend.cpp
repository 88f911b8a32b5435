/*
 * oracle/backend.cpp - CPU restatement of the reference's calling backend.
 *
 * TEST INFRASTRUCTURE.  This file is part of the parity oracle: it is built
 * and run only by the tests, the smoke check and the CPU-baseline leg of the
 * benchmark, never by the product.
 *
 * It implements every function of include/gsnp_backend.h on the CPU, keeping a
 * private "device" copy of the window state exactly as the reference keeps it
 * in GPU memory (kernel/common_kernel.h:16-61), so that host-visible side
 * effects - which host arrays each call refreshes and which it leaves stale -
 * match the reference call for call.  Sources restated:
 *   pileup        kernel/update_kernel.cu:233-375 (updateSparse_kernel, cuda_updateSparse)
 *   site sort     kernel/batchsort.cu:245-291, kernel/bitonic_kernel.cu:119-176
 *                 (an ascending sort of each site's records, std::sort here)
 *   likelihood    kernel/likelihood_kernel.cu:52-88,137-161,168-304
 *   posterior     kernel/posterior_kernel.cu:429-991
 *   window state  kernel/recycle_kernel.cu:11-32,91-136,197-252
 *   codecs        kernel/compress_kernel.cu:85-160,224-393, cpp/dict_compression.h:47-58
 *
 * Out-of-range reads in the reference are given a defined meaning here and in
 * the kernels alike: a Phred-0 base decodes to q_score 64, whose log10 table
 * entry is log10(64) (the reference reads past d_log10Table), and the rank-sum
 * histograms have 65 bins.
 */
#include "gsnp_backend.h"
#include "gsnp_crmath.h"
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct DeviceState {
    unsigned long W = 0;
    int L = 0;
    double pcr = 0.0, glob = 0.0;
    std::vector<double> newp;          /* materialised log10 genotype terms */
    double log10tab[65];
    std::vector<double> p_prior, p_rank;
    std::vector<unsigned int> sparse;  /* (W+L) x 256 records */
    std::vector<unsigned int> num;     /* records per site */
    std::vector<int> count_uni, q_sum, count_all, depth, repeat_time, dep_uni;
    std::vector<double> type_likely;   /* W x 17, persists across calls */
    std::vector<char> base1, base2, type1;
    std::vector<int> q_cns;
    std::vector<double> rank_sum;
    bool ready = false;
};

DeviceState g;

}  // namespace

OracleBackendView oracle_backend_view() {
    OracleBackendView v;
    v.records = g.sparse.data();
    v.num = g.num.data();
    v.dep_uni = g.dep_uni.data();
    v.type_likely = g.type_likely.data();
    return v;
}

void GPUInit() {}

void GSNPKernelInit(const unsigned long winSize, const int readLength, const double pcr_dependency,
                    const double global_dependency, const double* h_pmatrix, const double* p_prior,
                    const double* p_rank) {
    g.W = winSize;
    g.L = readLength;
    g.pcr = pcr_dependency;
    g.glob = global_dependency;
    g.newp.assign(256UL * 256UL * 4UL * 10UL, 0.0);
    oracle_materialize_pmatrix(h_pmatrix, g.newp.data());
    oracle_log10_table(g.log10tab);
    g.p_prior.assign(p_prior, p_prior + 8 * 16);
    g.p_rank.assign(p_rank, p_rank + GSNP_PRANK_SIZE);
    const unsigned long n = winSize + (unsigned long)readLength;
    g.sparse.assign(n * GSNP_MAX_RECORDS_PER_SITE, 0xFFFFFFFFu);
    g.num.assign(n, 0);
    g.count_uni.assign(n * 4, 0);
    g.q_sum.assign(n * 4, 0);
    g.count_all.assign(n * 4, 0);
    g.depth.assign(n, 0);
    g.repeat_time.assign(n, 0);
    g.dep_uni.assign(n, 0);
    /* the reference never initialises d_typeLikelihood; zeros stand in for it */
    g.type_likely.assign(winSize * GSNP_LIKELY_SIZE, 0.0);
    g.base1.assign(winSize, 0);
    g.base2.assign(winSize, 0);
    g.type1.assign(winSize, 0);
    g.q_cns.assign(winSize, 0);
    g.rank_sum.assign(winSize, 0.0);
    g.ready = true;
}

void cuda_init(unsigned long long win_size, unsigned long long read_len, unsigned long long start,
               int* posArr, const unsigned int, const unsigned int) {
    const unsigned long long n = win_size + read_len;
    for (unsigned long long i = 0; i < n; ++i) posArr[i] = (int)(i + start);
    std::fill(g.sparse.begin(), g.sparse.begin() + n * GSNP_MAX_RECORDS_PER_SITE, 0xFFFFFFFFu);
    std::fill(g.depth.begin(), g.depth.begin() + n, 0);
    std::fill(g.repeat_time.begin(), g.repeat_time.begin() + n, 0);
    std::fill(g.dep_uni.begin(), g.dep_uni.begin() + n, 0);
    std::fill(g.count_uni.begin(), g.count_uni.begin() + 4 * n, 0);
    std::fill(g.q_sum.begin(), g.q_sum.begin() + 4 * n, 0);
    std::fill(g.count_all.begin(), g.count_all.begin() + 4 * n, 0);
    std::fill(g.num.begin(), g.num.begin() + n, 0u);
}

void gold_pos_match(int* positionArr, int* siteMatchArr, int readCount) {
    memset(siteMatchArr, 0, sizeof(int) * GSNP_WIN_SIZE * 2);
    for (int r = 0; r < readCount; ++r) {
        const int s = positionArr[r] % GSNP_WIN_SIZE;
        if (siteMatchArr[2 * s + 1] == 0) {
            siteMatchArr[2 * s] = r;
            siteMatchArr[2 * s + 1] = 1;
        } else {
            siteMatchArr[2 * s + 1] += 1;
        }
    }
}

unsigned int cuda_updateSparse(struct st_update* u, unsigned int*, unsigned int*, int read_len,
                               int* count_uniArr, int* q_sumArr, int* count_allArr, int* depthArr,
                               int* repeat_timeArr, int*, int, const unsigned int,
                               const unsigned int) {
    const int W = GSNP_WIN_SIZE;
    const int L = read_len;
    const char qmin = u->qmin;
    const unsigned long n = (unsigned long)W + (unsigned long)L;
    for (int site = 0; site < W + L; ++site) {
        int depth = 0, repeat = 0, dep_uni = 0, num = 0;
        if (site < L) {
            dep_uni = g.dep_uni[site];
            num = (int)g.num[site];
        }
        int cov = site - L + 1;
        if (cov >= W) break;
        if (cov < 0) cov = 0;
        for (; cov <= site; ++cov) {
            if (cov >= W) break;
            const int first = u->siteMatchArr[cov * 2];
            const int last = first + u->siteMatchArr[cov * 2 + 1];
            for (int r = first; r < last; ++r) {
                const int coord = site - cov;
                const int lh = u->readLen_hitArr[r];
                const int rlen = (int)(((unsigned int)lh & 0xffff0000u) >> 16);
                if (coord >= rlen || coord < 0) continue;
                const int hit = lh & 0x0000ffff;
                const char base = u->readArr[(long)r * L + coord];
                const char qual = u->qualArr[(long)r * L + coord];
                depth += 1;
                repeat += hit;
                if (base == 'N' || qual < qmin || dep_uni >= 0xFF) continue;
                const int b = (base >> 1) & 3;
                if (hit == 1) {
                    dep_uni += 1;
                    const bool plus = u->strandArr[r] == '+';
                    const unsigned int strand_val = plus ? 0u : 1u;
                    const unsigned int coord_val = plus ? (unsigned int)coord : (unsigned int)(rlen - 1 - coord);
                    const unsigned int prefix = ((unsigned int)((base & 0x6) >> 1) << 15) |
                                                ((unsigned int)(GSNP_MAX_QSCORE - (qual - qmin)) << 9) |
                                                (coord_val << 1) | strand_val;
                    num += 1;
                    g.sparse[(unsigned long)site * GSNP_MAX_RECORDS_PER_SITE + num - 1] = (prefix << 8) | 1u;
                    g.count_uni[site * 4 + b] += 1;
                    g.q_sum[site * 4 + b] += qual - qmin;
                }
                g.count_all[site * 4 + b] += 1;
            }
        }
        g.depth[site] += depth;
        g.repeat_time[site] += repeat;
        g.dep_uni[site] = dep_uni;
        g.num[site] = (unsigned int)num;
    }
    unsigned int mx = 0;
    for (int s = 0; s < W; ++s) mx = std::max(mx, g.num[s]);
    memcpy(count_uniArr, g.count_uni.data(), sizeof(int) * 4 * n);
    memcpy(q_sumArr, g.q_sum.data(), sizeof(int) * 4 * n);
    memcpy(count_allArr, g.count_all.data(), sizeof(int) * 4 * n);
    memcpy(depthArr, g.depth.data(), sizeof(int) * n);
    memcpy(repeat_timeArr, g.repeat_time.data(), sizeof(int) * n);
    return mx;
}

void cuda_likelihoodSparse(double* h_typeLikelihood, const unsigned int numSite,
                           const unsigned int maxNumNonZero, const unsigned int,
                           const unsigned int, const unsigned int, const unsigned int) {
    if (maxNumNonZero == 0) {
        memset(h_typeLikelihood, 0, sizeof(double) * GSNP_LIKELY_SIZE * numSite);
        return;
    }
    for (unsigned int s = 0; s < numSite; ++s) {
        unsigned int* rec = &g.sparse[(unsigned long)s * GSNP_MAX_RECORDS_PER_SITE];
        std::sort(rec, rec + g.num[s]);
    }
    std::fill(g.type_likely.begin(), g.type_likely.begin() + (unsigned long)GSNP_LIKELY_SIZE * numSite, 0.0);
    for (unsigned int s = 0; s < numSite; ++s) {
        oracle_site_likelihood(&g.sparse[(unsigned long)s * GSNP_MAX_RECORDS_PER_SITE], g.num[s], g.L,
                               g.pcr, g.glob, g.log10tab, g.newp.data(),
                               &g.type_likely[(unsigned long)s * GSNP_LIKELY_SIZE]);
    }
}

void cuda_posterior(st_likelihood* lk, char* oriArr, char* base1, char* base2, char* type1,
                    int* q_cns, double* rank_sum_test_value, bool* validatedArr, bool* hapmap_siteArr,
                    bool* indel_siteArr, double* freqArr, double het_val, double het_unval,
                    double althom_val, double althom_unval, bool rank_sum_mode, bool monoploid,
                    bool refine, char q_max_min, unsigned long long, int win_size,
                    unsigned long call_length, unsigned int, const unsigned int, const unsigned int) {
    OraclePriorParams pp;
    pp.het_val = het_val;
    pp.het_unval = het_unval;
    pp.althom_val = althom_val;
    pp.althom_unval = althom_unval;
    for (unsigned long s = 0; s < call_length; ++s) {
        if (lk->nflag[s]) continue;
        OracleSiteIn in;
        in.ori = oriArr[s];
        in.count_uni = &g.count_uni[s * 4];
        in.q_sum = &g.q_sum[s * 4];
        in.count_all = &g.count_all[s * 4];
        in.dep_uni = g.dep_uni[s];
        in.type_likely = &g.type_likely[s * GSNP_LIKELY_SIZE];
        in.records = &g.sparse[s * GSNP_MAX_RECORDS_PER_SITE];
        in.num_records = g.num[s];
        in.validated = validatedArr[s];
        in.hapmap = hapmap_siteArr[s];
        in.indel = indel_siteArr[s];
        in.freq = &freqArr[s * 4];
        OracleSiteOut out;
        oracle_site_posterior(in, g.p_prior.data(), g.p_rank.data(), pp, rank_sum_mode, monoploid,
                              refine, (int)q_max_min, &out);
        g.base1[s] = out.base1;
        g.base2[s] = out.base2;
        g.type1[s] = out.type1;
        g.q_cns[s] = out.q_cns;
        g.rank_sum[s] = out.rank_sum;
    }
    memcpy(base1, g.base1.data(), (size_t)win_size);
    memcpy(base2, g.base2.data(), (size_t)win_size);
    memcpy(type1, g.type1.data(), (size_t)win_size);
    memcpy(q_cns, g.q_cns.data(), sizeof(int) * (size_t)win_size);
    memcpy(rank_sum_test_value, g.rank_sum.data(), sizeof(double) * (size_t)win_size);
}

namespace {

void shift_window(unsigned long long W, unsigned long long L) {
    auto shift = [&](auto& v, unsigned long long per, auto fill) {
        std::copy(v.begin() + W * per, v.begin() + (W + L) * per, v.begin());
        std::fill(v.begin() + L * per, v.begin() + (W + L) * per, fill);
    };
    shift(g.depth, 1, 0);
    shift(g.repeat_time, 1, 0);
    shift(g.dep_uni, 1, 0);
    shift(g.num, 1, 0u);
    shift(g.count_uni, 4, 0);
    shift(g.q_sum, 4, 0);
    shift(g.count_all, 4, 0);
    shift(g.sparse, GSNP_MAX_RECORDS_PER_SITE, 0xFFFFFFFFu);
}

void shift_positions(unsigned long long W, unsigned long long L, int* posArr) {
    memcpy(posArr, posArr + W, L * sizeof(int));
    for (unsigned long long i = L; i < L + W; ++i) posArr[i] = posArr[i - 1] + 1;
}

}  // namespace

void cuda_recycle(unsigned long long win_size, unsigned long long read_len, int* posArr,
                  const unsigned int, const unsigned int) {
    shift_positions(win_size, read_len, posArr);
    shift_window(win_size, read_len);
}

void cuda_quickRecycle(unsigned long long win_size, unsigned long long read_len, int* posArr,
                       int* count_uniArr, int* q_sumArr, int* count_allArr, int* depthArr,
                       int* repeat_timeArr, const unsigned int, const unsigned int) {
    shift_window(win_size, read_len);
    shift_positions(win_size, read_len, posArr);
    const unsigned long n = GSNP_WIN_SIZE + read_len;
    memcpy(count_uniArr, g.count_uni.data(), sizeof(int) * 4 * n);
    memcpy(q_sumArr, g.q_sum.data(), sizeof(int) * 4 * n);
    memcpy(count_allArr, g.count_all.data(), sizeof(int) * 4 * n);
    memcpy(depthArr, g.depth.data(), sizeof(int) * n);
    memcpy(repeat_timeArr, g.repeat_time.data(), sizeof(int) * n);
}

/* ---------------------------------------------------------------------- */
/* codecs                                                                  */
/* ---------------------------------------------------------------------- */

unsigned long getNumBinWord(const unsigned long numElement) {
    return (unsigned long)ceil(numElement / 16.0);
}

unsigned long encode(unsigned int* code, const char* seq, const unsigned long numElement) {
    const unsigned long nw = getNumBinWord(numElement);
    memset(code, 0, sizeof(unsigned int) * nw);
    for (unsigned long w = 0; w < nw; ++w) {
        const unsigned long nb = (w == nw - 1) ? numElement - w * 16 : 16;
        unsigned int word = 0;
        for (unsigned long i = 0; i < nb; ++i) {
            const int c = oracle_base2bits(seq[w * 16 + i]);
            if (c < 0) {
                printf("!!!ERROR@encode: unknown base when encoding.\n");
                exit(EXIT_FAILURE);
            }
            word = (word << 2) | (unsigned int)c;
        }
        code[w] = word;
    }
    return nw;
}

void decode(char* seq, const unsigned long numElement, const unsigned int* code,
            const unsigned long numCodeWord) {
    static const char letters[4] = {'A', 'C', 'G', 'T'};
    for (unsigned long w = 0; w + 1 < numCodeWord; ++w)
        for (unsigned int i = 0; i < 16; ++i) seq[w * 16 + i] = letters[(code[w] >> (30 - 2 * i)) & 3];
    const unsigned long left = numElement - (numCodeWord - 1) * 16;
    for (unsigned long i = 0; i < left; ++i)
        seq[(numCodeWord - 1) * 16 + i] = letters[(code[numCodeWord - 1] >> (2 * (left - i - 1))) & 3];
}

void dictComprStart(const unsigned long, const unsigned long) {}
void dictComprEnd() {}

void cuda_dictCompression(unsigned int* out, unsigned long* nw, char* dict, unsigned long* nd,
                          char* in, const unsigned long n) {
    oracle_dict_compress(out, nw, dict, nd, in, n);
}
void cuda_dictCompression(unsigned int* out, unsigned long* nw, int* dict, unsigned long* nd, int* in,
                          const unsigned long n) {
    oracle_dict_compress(out, nw, dict, nd, in, n);
}
void cuda_dictCompression(unsigned int* out, unsigned long* nw, unsigned int* dict, unsigned long* nd,
                          unsigned int* in, const unsigned long n) {
    oracle_dict_compress(out, nw, dict, nd, in, n);
}
void cuda_dictCompression(unsigned int* out, unsigned long* nw, double* dict, unsigned long* nd,
                          double* in, const unsigned long n) {
    oracle_dict_compress(out, nw, dict, nd, in, n);
}

unsigned int RLECompression(int* data, const unsigned long n, unsigned int* runLength) {
    return oracle_rle(data, n, runLength);
}
unsigned int RLECompression(double* data, const unsigned long n, unsigned int* runLength) {
    return oracle_rle(data, n, runLength);
}
unsigned int RLECompression(char* data, const unsigned long n, int* runLength) {
    return oracle_rle(data, n, runLength);
}
