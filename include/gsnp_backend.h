/*
 * gsnp_backend.h - the calling backend boundary of lumianph/gsnp, declared anew.
 *
 * The reference's host code (cpp/call_genotype.cc, cpp/main.cc, cpp/soap_snp.h)
 * calls its GPU backend through plain C++ functions declared in cpp/gsnp.h and
 * cpp/dict_compression.h.  This header declares the same functions with the same
 * parameter types, so the C++ names they link by are identical, and the three
 * data structs they exchange with identical member layouts.  Any object file
 * compiled against the reference headers links against an implementation of
 * this header unchanged.  Two implementations exist:
 *   - the CPU restatement used as the test oracle (oracle/backend.cpp);
 *   - the sm_103a implementation (gsnp_gb300/csrc/compat.cu), which keeps the
 *     window state resident on one GB300.
 *
 * The structs carry data members only.  The reference defines constructors
 * for them inline in its header; declaring none here keeps the two definitions
 * from competing at link time.
 *
 * Fundamental types follow the reference's typedefs:
 *   uint64 = unsigned long (inc/gsnp_util.h:23), uint32 = unsigned int
 *   (inc/gsnp_util.h:22), ubit64_t = unsigned long long (cpp/common.h:44),
 *   rate_t = double (cpp/common.h:46), word = code_t = unsigned int
 *   (inc/gsnp_util.h:25, cpp/dict_compression.h:14).
 */
#ifndef GSNP_BACKEND_H
#define GSNP_BACKEND_H

#include <string>

/* Window geometry and record layout constants (cpp/common.h:15-16,38,71-75). */
#define GSNP_WIN_SIZE 262144                      /* global_win_size */
#define GSNP_MAX_RECORDS_PER_SITE 256             /* MAX_NUM_NON_ZERO */
#define GSNP_READS_PER_WINDOW (4 * GSNP_WIN_SIZE + 100) /* _read_num_per_window */
#define GSNP_MAX_QSCORE 64                        /* MAX_QSCORE */
#define GSNP_LIKELY_SIZE 17                       /* LIKELY_SIZE */
#define GSNP_PMATRIX_SIZE (256UL * 256UL * 4UL * 4UL) /* PMATRIX_SIZE */
#define GSNP_PRANK_SIZE (64UL * 64UL * 2048UL)

/* Per-window likelihood state owned by the driver (cpp/gsnp.h:29-124). */
struct st_likelihood {
    char qmax;
    char qmin;
    int readLength;
    double globalDependency;
    double pcrDependency;
    unsigned long maxCallLength;
    unsigned long winSize;
    unsigned long numSite;
    double* p_matrix;
    unsigned long callLength;
    bool* nflag;
    int* countuni;
    double* typeLikelihood;
};

/* Host staging buffers for one window of reads (cpp/gsnp.h:134-310).
 * readArr/qualArr hold _read_length bytes per read; readLen_hitArr packs
 * (read_len << 16) | hit; siteMatchArr holds (first read, count) per
 * window offset, filled by gold_pos_match. */
struct st_update {
    char* inputUpdateChar;
    int* inputUpdateInt;
    char* readArr;
    char* qualArr;
    std::string* char_nameArr;
    int* hitArr;
    int* read_lenArr;
    int* positionArr;
    int* siteMatchArr;
    int* mismatchArr;
    char* abArr;
    char* strandArr;
    int* readLen_hitArr;
    char qmin;
    unsigned int _read_length;
};

/* Per-window dbSNP arrays (cpp/gsnp.h:447-468). */
struct st_snp {
    bool* validatedArr;
    bool* hapmap_siteArr;
    bool* indel_siteArr;
    double* freqArr;
};

/* cpp/gsnp.h:26 - select the device (device 0). */
void GPUInit();

/* cpp/gsnp.h:127-129 - upload the calibration matrix (materialised as log10
 * genotype terms), the prior table and the rank-sum table; allocate the window
 * state.  The caller keeps ownership of the three host tables. */
void GSNPKernelInit(const unsigned long winSize, const int readLength,
                    const double pcr_dependency, const double global_dependency,
                    const double* h_pmatrix, const double* p_prior, const double* p_rank);

/* cpp/gsnp.h:492-498 - posArr[i] = start + i for i < W+L; reset the window's
 * records to 0xFFFFFFFF and its counts to 0. */
void cuda_init(unsigned long long win_size, unsigned long long read_len, unsigned long long start,
               int* posArr, const unsigned int numBlock = 1200, const unsigned int numThread = 256);

/* cpp/gsnp.h:403-417 - deposit reads [0, readCount) into the window pileup;
 * write back count_uni, q_sum, count_all, depth, repeat_time for W+L sites;
 * return the largest record count over the first W sites.  sparseBaseInfo,
 * numNonZeroPerSite and dep_uniArr are not touched. */
unsigned int cuda_updateSparse(struct st_update* updateData, unsigned int* sparseBaseInfo,
                               unsigned int* numNonZeroPerSite, int read_len, int* count_uniArr,
                               int* q_sumArr, int* count_allArr, int* depthArr, int* repeat_timeArr,
                               int* dep_uniArr, int readCount, const unsigned int numBlock = 1200,
                               const unsigned int numThread = 256);

/* cpp/gsnp.h:398-401 - sort each site's records and compute the 10-genotype
 * log10 likelihood on the device.  The host buffer is written (zeros) only
 * when maxNumNonZero == 0, in which case the device likelihood is left as it
 * was. */
void cuda_likelihoodSparse(double* h_typeLikelihood, const unsigned int numSite,
                           const unsigned int maxNumNonZero, const unsigned int sitePitch,
                           const unsigned int offsetPitch, const unsigned int numBlock = 1200,
                           const unsigned int numThread = 128);

/* cpp/gsnp.h:470-489 - posterior, consensus quality and rank-sum test; reads
 * ori, nflag and the dbSNP arrays for W sites, writes base1, base2, type1,
 * q_cns and rank_sum for W sites. */
void cuda_posterior(st_likelihood* likelihoodData, char* oriArr, char* base1, char* base2,
                    char* type1, int* q_cns, double* rank_sum_test_value, bool* validatedArr,
                    bool* hapmap_siteArr, bool* indel_siteArr, double* freqArr,
                    double para_het_val_r, double para_het_unval_r, double para_althom_val_r,
                    double para_althom_unval_r, bool para_rank_sum_mode, bool para_is_monoploid,
                    bool para_refine_mode, char para_q_max_min, unsigned long long read_len,
                    int win_size, unsigned long call_length, unsigned int maxNumNonZero,
                    const unsigned int numBlock = 1200, const unsigned int numThread = 256);

/* cpp/gsnp.h:499-504 - shift the window by W on the device (the L-site tail
 * becomes the head) and shift posArr.  Host count arrays are not refreshed. */
void cuda_recycle(unsigned long long win_size, unsigned long long read_len, int* posArr,
                  const unsigned int numBlock = 1200, const unsigned int numThread = 256);

/* cpp/gsnp.h:505-516 - the same shift, then refresh the five host count arrays. */
void cuda_quickRecycle(unsigned long long win_size, unsigned long long read_len, int* posArr,
                       int* count_uniArr, int* q_sumArr, int* count_allArr, int* depthArr,
                       int* repeat_timeArr, const unsigned int numBlock = 1200,
                       const unsigned int numThread = 256);

/* cpp/gsnp.h:385 - bucket reads by position modulo the window:
 * siteMatch[2p] = first read at offset p, siteMatch[2p+1] = count. */
void gold_pos_match(int* positionArr, int* siteMatchArr, int readCount);

/* cpp/dict_compression.h:16-18 - 2-bit base packing (A0 C1 G2 T3), 16 bases
 * per 32-bit word, first base in the high bits; the last word holds the
 * remaining bases right-aligned.  encode exits on a non-ACGT base. */
unsigned long getNumBinWord(const unsigned long numElement);
unsigned long encode(unsigned int* code, const char* seq, const unsigned long numElement);
void decode(char* seq, const unsigned long numElement, const unsigned int* code,
            const unsigned long numCodeWord);

/* cpp/dict_compression.h:23-24 - scratch reservation for the dictionary codec. */
void dictComprStart(const unsigned long numElement, const unsigned long dataSize);
void dictComprEnd();

/* cpp/dict_compression.h:26-37 - dictionary codec: dict = sorted distinct
 * values of inData, outData = their indices packed MSB-first into 32-bit
 * words (bits per index = ceil(log2(#dict)), at least 1).  *numWordOutData and
 * *numElementDict hold capacities on entry and used counts on return. */
void cuda_dictCompression(unsigned int* outData, unsigned long* numWordOutData, char* dict,
                          unsigned long* numElementDict, char* inData,
                          const unsigned long numElementInData);
void cuda_dictCompression(unsigned int* outData, unsigned long* numWordOutData, int* dict,
                          unsigned long* numElementDict, int* inData,
                          const unsigned long numElementInData);
void cuda_dictCompression(unsigned int* outData, unsigned long* numWordOutData, unsigned int* dict,
                          unsigned long* numElementDict, unsigned int* inData,
                          const unsigned long numElementInData);
void cuda_dictCompression(unsigned int* outData, unsigned long* numWordOutData, double* dict,
                          unsigned long* numElementDict, double* inData,
                          const unsigned long numElementInData);

/* cpp/dict_compression.h:95-97 - run-length encoding in place: data keeps the
 * run values, runLength the run lengths; returns the number of runs. */
unsigned int RLECompression(int* data, const unsigned long numElement, unsigned int* runLength);
unsigned int RLECompression(double* data, const unsigned long numElement, unsigned int* runLength);
unsigned int RLECompression(char* data, const unsigned long numElement, int* runLength);

#endif /* GSNP_BACKEND_H */
