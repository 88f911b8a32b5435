/*
 * oracle/oracle.h - CPU restatement of lumianph/gsnp's consensus-calling path.
 *
 * TEST INFRASTRUCTURE.  Everything under oracle/ is the parity oracle: it is
 * compiled and executed only by tests/, by __graft_entry__.smoke() as the
 * checker, and by the CPU-baseline leg of bench.py.  The product never links,
 * imports or runs it.
 *
 * Parity status: pinned.  oracle/_ref/ links the reference's own host sources
 * (cpp/main.cc, call_genotype.cc, matrix.cc, prior.cc, rank_sum.cc,
 * chromosome.cc, normal_dis.cc, compiled in place by the "ref" target of oracle/Makefile)
 * against oracle/backend.cpp; tests/test_oracle_pin.py requires the restated
 * driver (oracle/driver.cpp) to produce byte-identical cns text and -C files.
 */
#ifndef GSNP_ORACLE_H
#define GSNP_ORACLE_H

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

/* q_score offset of the record word: q_score = 64 - 6-bit field (cpp/common.h:71) */
#define GSNP_MAX_QSCORE_ORACLE 64

/* ---- calibrated-table helpers (kernel/likelihood_kernel.cu:83-87,137-161) ---- */

/* new_pmatrix[((q<<10)|(coord<<2)|o)*10 + g] = log10(0.5 p[a1] + 0.5 p[a2]) for
 * the 10 genotypes g = (a1 <= a2) in ACTG order, q and coord in [0, 256). */
void oracle_materialize_pmatrix(const double* pmatrix, double* new_pmatrix);

/* log10(i) for i in [0, 64]; entry 64 is log10(64), the defined meaning of the
 * reference's read past its 64-entry table. */
void oracle_log10_table(double* tab65);

/* 10-genotype log10 likelihood of one site from its sorted records
 * (kernel/likelihood_kernel.cu:187-255).  out[16] is left untouched. */
void oracle_site_likelihood(const unsigned int* records, unsigned int num, int read_length,
                            double pcr_dependency, double global_dependency, const double* log10tab,
                            const double* new_pmatrix, double* out);

/* q_adj of one record (kernel/likelihood_kernel.cu:226-231) */
int oracle_q_adjust(int q_score, int tmp, int gdc, double pcr_dependency,
                    double global_dependency, const double* log10tab);

struct OraclePriorParams {
    double het_val, het_unval, althom_val, althom_unval;
};

/* one site's inputs to the posterior, pointing into the window arrays */
struct OracleSiteIn {
    char ori;
    const int* count_uni;   /* [4], may be read past index 3 exactly as the reference does */
    const int* q_sum;
    const int* count_all;
    int dep_uni;
    const double* type_likely;
    const unsigned int* records;
    unsigned int num_records;
    bool validated, hapmap, indel;
    const double* freq;     /* [4] */
};

struct OracleSiteOut {
    char base1, base2, type1, type2;
    int q_cns;
    double rank_sum;
    int qual1, qual2, qual3;
    double type_prob[17];
};

/* posterior_kernel + posterior_kernel2 for one non-N site
 * (kernel/posterior_kernel.cu:575-866) */
void oracle_site_posterior(const OracleSiteIn& in, const double* p_prior, const double* p_rank,
                           const OraclePriorParams& pp, bool rank_sum_mode, bool monoploid,
                           bool refine, int q_max_min, OracleSiteOut* out);

/* rank-sum pieces (kernel/posterior_kernel.cu:429-572) */
double oracle_rank_test(const unsigned int* records, unsigned int num, const int* count_uni,
                        int best_type, const double* p_rank, int q_max_min);
double oracle_table_test(const double* p_rank, int n1, int n2, double T1, double T2);
double oracle_normal_value(double z);
double oracle_normal_test(int n1, int n2, double T1, double T2);

/* dbSNP prior override as the device does it (kernel/posterior_kernel.cu:575-633) */
void oracle_snp_prior(double* prior, char ref, bool indel, bool validated, bool hapmap,
                      const double* freq, const OraclePriorParams& pp);

/* ---- codec helpers ---- */

/* 2-bit code of a base for encode(): A/a 0, C/c 1, G/g 2, T/t 3, else -1
 * (kernel/compress_kernel.cu:25-58) */
int oracle_base2bits(char c);

/* bits per dictionary index: (int)ceil(log(n)/log(2)) with the C library's
 * log, at least 1 (cpp/dict_compression.h:47-54) */
int oracle_bits_per_index(unsigned long n);

/* dictionary codec shared by cuda_dictCompression and the host dictCompression
 * template (kernel/compress_kernel.cu:224-268, cpp/dict_compression.h:116-166) */
template <class T>
void oracle_dict_compress(unsigned int* out, unsigned long* num_word_out, T* dict,
                          unsigned long* num_dict, const T* in, unsigned long n) {
    if (*num_dict < n) {
        printf("!!!ERROR@oracle_dict_compress: *numElementDict < numElementInData\n");
        exit(EXIT_FAILURE);
    }
    std::copy(in, in + n, dict);
    std::sort(dict, dict + n);
    T* end = std::unique(dict, dict + n);
    const unsigned long nd = (unsigned long)(end - dict);
    *num_dict = nd;
    const int bits = oracle_bits_per_index(nd);
    const int per_word = (int)floor(32 / (double)bits);
    if (per_word <= 0) {
        /* the reference aborts here (empty dictionary); keep a defined result */
        *num_word_out = 0;
        return;
    }
    const unsigned long nw = (unsigned long)ceil(n / (double)per_word);
    if (*num_word_out < nw) {
        printf("!!!ERROR@oracle_dict_compress: numWordOutData < numWordCompressed\n");
        exit(EXIT_FAILURE);
    }
    *num_word_out = nw;
    for (unsigned long w = 0; w < nw; ++w) {
        const unsigned long cnt = (w == nw - 1) ? n - (unsigned long)per_word * w : (unsigned long)per_word;
        unsigned int word = 0;
        for (unsigned long i = 0; i < cnt; ++i) {
            const T v = in[w * per_word + i];
            const unsigned int idx = (unsigned int)(std::lower_bound(dict, end, v) - dict);
            word = (word << bits) | idx;
        }
        out[w] = word;
    }
}

/* run-length encoding in place (kernel/compress_kernel.cu:336-393) */
template <class T, class R>
unsigned int oracle_rle(T* data, unsigned long n, R* run_length) {
    if (n == 0) return 0;
    unsigned long runs = 0;
    unsigned long start = 0;
    for (unsigned long i = 1; i <= n; ++i) {
        if (i == n || !(data[i] == data[start])) {
            data[runs] = data[start];
            run_length[runs] = (R)(i - start);
            ++runs;
            start = i;
        }
    }
    return (unsigned int)runs;
}

/* ---- test access to the restated backend's window state ---- */

/* The private "device" arrays of oracle/backend.cpp, for the check of the
 * backend against the reference's CPU twins (oracle/gold/check.cpp). */
struct OracleBackendView {
    const unsigned int* records;   /* [site][GSNP_MAX_RECORDS_PER_SITE] */
    const unsigned int* num;       /* records per site */
    const int* dep_uni;
    const double* type_likely;     /* [site][GSNP_LIKELY_SIZE] */
};
OracleBackendView oracle_backend_view();

/* the restated driver's tables: Prob_matrix::rank_table_gen
 * (cpp/rank_sum.cc:3-42) and Prob_matrix::prior_gen (cpp/prior.cc:3-43) */
void oracle_rank_table(double* p_rank);
void oracle_prior_table(double het_novel, double althom_novel, bool transition_dominant, double* p_prior);

/* ---- restated host driver (cpp/main.cc, cpp/call_genotype.cc, ...) ---- */

/* SOAPsnp command line; returns the process exit status. */
int oracle_main(int argc, char** argv);

#endif /* GSNP_ORACLE_H */
