/*
 * tables.h - host-built lookup tables of the caller.
 */
#ifndef GSNP_TABLES_H
#define GSNP_TABLES_H

#include <stdint.h>

#include <string>
#include <vector>

#include "gsnp_gb300.h"

namespace gsnp {

struct HostTables {
    int L = 0;
    int qa_rows = 0;                /* adjusted qualities 0 .. qa_rows-1 */
    int tmax = 0, gmax = 0;         /* q_adj table bounds: tmp < tmax, gdc < gmax */
    std::vector<double> lik64;      /* [qa_rows][L][4][10] */
    std::vector<float> lik32;       /* FP32: [qa_rows][L][4][8] columns 0-7 of each row, then
                                       [qa_rows][L][4][2] columns 8-9 */
    std::vector<uint8_t> qadj;      /* [tmax][gmax][65] */
    std::vector<double> log_prior;  /* [128] correctly rounded log10 of p_prior */
    std::vector<float> log_prior32; /* [8][12] log_prior in FP32 by table column */
    bool all_nonpositive = true;    /* every lik64 entry <= 0, none of them an FP32 subnormal */
};

/* Tables of the likelihood and posterior kernels, built from the reference's
 * calibration matrix and prior table. */
int build_tables(const gsnp_params& p, const double* p_matrix, const double* p_prior, HostTables* t,
                 std::string* err);

/* cpp/matrix.cc:129-205: fill the calibration matrix from pass-1 counts laid
 * out [q_char - q_min][cycle][ref][obs] for q_char in [q_min, q_max]. */
void calibration_fill(const gsnp_params& p, const unsigned long long* counts, double* p_matrix);

/* cpp/prior.cc:3-43 */
void prior_table(const gsnp_params& p, int transition_dominant, double het_novel, double althom_novel,
                 double* p_prior);

/* cpp/rank_sum.cc:3-42 */
void rank_table(double* p_rank);

}  // namespace gsnp

#endif
