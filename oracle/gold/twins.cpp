/*
 * oracle/gold/twins.cpp - the reference's own CPU twins of its calling
 * kernels, compiled for the host.  TEST INFRASTRUCTURE (see oracle/oracle.h).
 *
 * The reference ships plain host code beside its kernels, written to check
 * them: gold_updateSparse (kernel/update_kernel.cu:96-195), the posterior with
 * its rank-sum test (gold_table_test .. gold_posterior,
 * kernel/posterior_kernel.cu:90-426), and a likelihood kernel whose body is
 * host-compilable once its launch qualifiers and thread indices are given a
 * meaning (likelihoodSparse_kernel, kernel/likelihood_kernel.cu:168-256, with
 * the word codec :24-42 and the table materialisation :137-161).
 *
 * This file holds none of that code.  The "ref-gold" target of oracle/Makefile
 * copies those line ranges out of the reference tree at build time into
 * oracle/_ref/twins/*.inc, and this harness includes them with:
 *   - the reference's own headers for its types and constants (cpp/common.h,
 *     cpp/gsnp.h);
 *   - empty CUDA qualifiers, __syncthreads() as a no-op, and a one-thread grid
 *     (NUM_TOTAL_THREAD 1, GLOBAL_THREAD_OFFSET 0), so that the kernel's
 *     grid-stride loop visits every site in order on the host;
 *   - d_log10Table as a host array filled as likelihoodKernelInit fills it
 *     (kernel/likelihood_kernel.cu:83-87);
 *   - the globals the twins name but the reference never defines
 *     (global_num_site, numSite): their value does not matter, since the
 *     site-major record index ignores it (cpp/common.h:89).
 * The posterior twins are compiled twice: once with the C library's log10 and
 * exp, as written, and once with the correctly rounded ones that this build
 * pins the per-site transcendentals to (include/gsnp_crmath.h), so that the
 * oracle can be required to match the second exactly and the first's
 * differences can be counted.
 *
 * The twins are reached through the extern "C" functions at the end, which
 * take plain arrays; gold/check.cpp drives them and the restated backend.
 */
#include <assert.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <iostream>
#include <vector>

#include "common.h"
#include "gsnp.h"

#include "gsnp_crmath.h"

#define __global__
#define __device__
#define __host__
#define __constant__
#define __syncthreads() ((void)0)
#define NUM_TOTAL_THREAD 1u
#define GLOBAL_THREAD_OFFSET 0u

namespace {
double d_log10Table[MAX_QSCORE];
uint64 global_num_site = 0;
uint64 numSite = 0;
}  // namespace

namespace twin {
#include "twins/words.inc"
#include "twins/update.inc"
#include "twins/materialize.inc"
#include "twins/likelihood.inc"
#include "twins/posterior.inc"
}  // namespace twin

namespace twin_cr {
/* unqualified calls in the included code find these first */
static inline double log10(double x) { return gsnp_cr_log10(x); }
static inline double exp(double x) { return gsnp_cr_exp(x); }
#include "twins/posterior.inc"
}  // namespace twin_cr

extern "C" {

/* gold_updateSparse over reads [0, n) of one window: records [site][256],
 * per-site record counts and the six count arrays ([site][4] or [site]) must
 * be zero on entry for sites [0, W + L).  Returns the largest record count. */
int twin_update(int n, const int* pos, const int* len, const int* hit, const char* strand, const char* read,
                const char* qual, int L, char qmin, uint32* records, uint32* num, int* count_uni, int* q_sum,
                int* count_all, int* depth, int* repeat_time, int* dep_uni) {
    /* the twin reads only these members; the struct's constructor (which
     * needs the whole command line) is not run */
    st_update* u = (st_update*)calloc(1, sizeof(st_update));
    u->readArr = const_cast<char*>(read);
    u->qualArr = const_cast<char*>(qual);
    u->hitArr = const_cast<int*>(hit);
    u->read_lenArr = const_cast<int*>(len);
    u->positionArr = const_cast<int*>(pos);
    u->strandArr = const_cast<char*>(strand);
    u->qmin = qmin;
    const int mx = twin::gold_updateSparse(u, &records, &num, 0, L, count_uni, q_sum, count_all, depth,
                                           repeat_time, dep_uni, n);
    free(u);
    return mx;
}

/* materializePMatrix: [q][coord][o][10] log10 genotype terms of a p_matrix */
void twin_materialize(const double* p_matrix, double* new_pmatrix) {
    twin::materializePMatrix(p_matrix, new_pmatrix);
}

/* likelihoodSparse_kernel over n_sites sites whose sorted records are
 * [site][256]; out is [site][17] and must be zero on entry, pcr_scratch
 * holds n_sites * 2 * L zero ints. */
void twin_likelihood(int n_sites, const uint32* records, const uint32* num, int L, double pcr, double glob,
                     const double* new_pmatrix, int* pcr_scratch, double* out) {
    for (int i = 0; i < MAX_QSCORE; ++i) d_log10Table[i] = log10((double)i);
    twin::likelihoodSparse_kernel(out, records, num, 256, pcr_scratch, new_pmatrix, (uint32)n_sites,
                                  (uint32)n_sites, (uint32)L, pcr, glob);
}

/* gold_posterior over sites [0, n_sites); cr selects the correctly rounded
 * log10 and exp.  Sites whose nflag is set are left untouched. */
void twin_posterior(int cr, int n_sites, const bool* nflag, const double* type_likely, const double* p_prior,
                    const double* p_rank, const uint32* records, const uint32* num, const int* count_uni,
                    const int* q_sum, const int* dep_uni, const int* count_all, const char* ori,
                    const bool* validated, const bool* hapmap, const bool* indel, const double* freq,
                    double het_val, double het_unval, double althom_val, double althom_unval, int rank_sum_mode,
                    int monoploid, int refine, int q_max_min, int L, char* base1, char* base2, char* type1,
                    int* q_cns, double* rank_sum) {
    st_likelihood* lk = (st_likelihood*)calloc(1, sizeof(st_likelihood));
    lk->nflag = const_cast<bool*>(nflag);
    lk->typeLikelihood = const_cast<double*>(type_likely);
    double type_prob[LIKELY_SIZE];
    std::vector<int> pos(n_sites, 0);
#define TWIN_POSTERIOR_ARGS                                                                                        \
    lk, const_cast<double*>(p_prior), type_prob, const_cast<double*>(p_rank), const_cast<uint32*>(records),      \
        const_cast<uint32*>(num), const_cast<int*>(count_uni), const_cast<int*>(q_sum),                          \
        const_cast<int*>(dep_uni), const_cast<int*>(count_all), const_cast<char*>(ori), pos.data(), base1, base2, \
        type1, q_cns, rank_sum, const_cast<bool*>(validated), const_cast<bool*>(hapmap),                          \
        const_cast<bool*>(indel), const_cast<double*>(freq), het_val, het_unval, althom_val, althom_unval,        \
        rank_sum_mode != 0, monoploid != 0, refine != 0, (char)q_max_min, (ubit64_t)L, (uint64_t)n_sites
    if (cr)
        twin_cr::gold_posterior(TWIN_POSTERIOR_ARGS);
    else
        twin::gold_posterior(TWIN_POSTERIOR_ARGS);
#undef TWIN_POSTERIOR_ARGS
    free(lk);
}

}  // extern "C"
