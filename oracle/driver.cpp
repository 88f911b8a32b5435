/*
 * oracle/driver.cpp - restated host side of the reference's calling path.
 *
 * TEST INFRASTRUCTURE (see oracle/oracle.h).  A CPU restatement of:
 *   cpp/main.cc           command line (getopt string "i:d:o:z:g:p:r:e:ts:2a:b:j:k:unmqM:I:L:Q:S:F:E:T:h:C")
 *   cpp/chromosome.cc     FASTA 4-bit packing and dbSNP table (Genome, Chr_info)
 *   cpp/soap_snp.h        SOAP line parsing (Soap_format::operator>>), pass-1 read store
 *   cpp/matrix.cc         calibration count and fill, -M / -I matrix files
 *   cpp/prior.cc          novel genotype prior table
 *   cpp/rank_sum.cc       exact Wilcoxon rank-sum table
 *   cpp/call_genotype.cc  window driver (new_soap2cns) and per-window output (call_cns2)
 *   cpp/compress.h        the six -C column files
 * The backend is reached only through include/gsnp_backend.h, exactly as the
 * reference's call_genotype.cc reaches it, so this driver links unchanged
 * against the CPU backend (oracle/backend.cpp) or the GPU backend.
 *
 * Differences from the reference, none of which changes an output byte:
 *   - pass-1 reads are kept in memory instead of the in.* spill files;
 *   - rows end in '\n' without a flush per row;
 *   - with -I the alignment file is parsed again for pass 2 (the reference
 *     reads spill files left by an earlier run).
 */
#include "gsnp_backend.h"
#include "oracle.h"

#include <getopt.h>
#include <sys/time.h>

#include <cctype>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <string>

namespace {

const unsigned long W = GSNP_WIN_SIZE;
const char kAbbv[17] = {'A', 'M', 'W', 'R', 'M', 'C', 'Y', 'S', 'W', 'Y', 'T', 'K', 'R', 'S', 'K', 'G', 'N'};
const char* kActgN = "ACTGNNNN";

struct Params {
    signed char q_min = 64;
    signed char q_max = 64 + 40;
    unsigned char read_length = 45;
    bool monoploid = false, refine = false, rank_sum = false, transition_dominant = false;
    bool compress = false;
    double althom_novel = 0.0005, het_novel = 0.0010;
    double althom_val = 0.05, het_val = 0.10;
    double althom_unval = 0.01, het_unval = 0.02;
    double global_dep = log10(0.9), pcr_dep = log10(0.5);
};

struct SnpInfo {
    bool validated = false, hapmap = false, indel = false;
    double freq[4] = {0, 0, 0, 0};
};

struct Chromosome {
    unsigned int len = 0;
    std::vector<unsigned long long> bin;   /* 16 bases of 4 bits per word */
    std::map<unsigned long long, SnpInfo> dbsnp;
    unsigned long long base(unsigned long long pos) const { return (bin[pos / 16] >> (pos % 16 * 4)) & 0xF; }
    void binarize(const std::string& seq) {
        len = (unsigned int)seq.length();
        bin.assign(len % 16 == 0 ? len / 16 : 1 + len / 16, 0ULL);
        for (std::string::size_type i = 0; i != seq.length(); ++i)
            bin[i / 16] |= ((((unsigned long long)seq[i]) >> 1) & 7) << (i % 16 * 4);
    }
};

struct Genome {
    std::map<std::string, Chromosome> chr;
};

/* one parsed SOAP line as it reaches pass 2 */
struct ReadStore {
    unsigned L = 0;
    std::vector<char> seq, qual;     /* L bytes per read */
    std::vector<int> hit, len, pos, mismatch;
    std::vector<char> strand;
    std::string last_chr;
    size_t size() const { return pos.size(); }
};

[[noreturn]] void usage() {
    std::cerr << "GSNP" << std::endl;
    std::cerr << "Compulsory Parameters:" << std::endl;
    std::cerr << "-i <FILE> Input SORTED Soap Result" << std::endl;
    std::cerr << "-d <FILE> Reference Sequence in fasta format" << std::endl;
    std::cerr << "-o <FILE> Output consensus file" << std::endl;
    exit(1);
}

void load_genome(std::ifstream& fasta, std::ifstream* known_snp, Genome* g) {
    /* cpp/chromosome.cc:172-220 */
    std::string seq, current;
    for (std::string buff; std::getline(fasta, buff);) {
        if (!buff.empty() && buff[0] == '>') {
            auto it = g->chr.find(current);
            if (it != g->chr.end()) it->second.binarize(seq);
            std::string::size_type i;
            for (i = 1; i != buff.length() && !isspace((unsigned char)buff[i]); ++i) {}
            std::string name(buff, 1, i - 1);
            if (!g->chr.emplace(name, Chromosome()).second)
                std::cerr << "Insert Chromosome " << name << " Failed!\n";
            current = name;
            seq = "";
        } else {
            seq += buff;
        }
    }
    if (seq.length() != 0 && g->chr.find(current) != g->chr.end()) g->chr[current].binarize(seq);
    if (known_snp && *known_snp) {
        /* the name, the position and the SNP fields live across rows, as
         * there (:207-210): a field that fails to parse keeps the previous
         * row's value */
        SnpInfo form;
        std::string name;
        std::string::size_type pos = 0;
        for (std::string buff; std::getline(*known_snp, buff);) {
            std::istringstream s(buff);
            s >> name >> pos;
            s >> form.hapmap >> form.validated >> form.indel >> form.freq[0] >> form.freq[1] >> form.freq[2] >> form.freq[3];
            auto it = g->chr.find(name);
            if (it == g->chr.end()) continue;
            pos -= 1;
            if (it->second.dbsnp.emplace((unsigned long long)pos, form).second)
                it->second.bin[pos / 16] |= (1ULL << (pos % 16 * 4 + 3));
        }
    }
}

/* cpp/soap_snp.h:132-169; returns false when the stream fails */
bool parse_soap(std::istringstream& s, std::string& read, std::string& qual, int& hit, int& read_len,
                char& strand, std::string& chr, int& position, int& mismatch) {
    std::string id;
    char ab;
    s >> id >> read >> qual >> hit >> ab >> read_len >> strand >> chr >> position >> mismatch;
    if (mismatch > 200) {
        int indel_pos;
        s >> indel_pos;
        const int n = mismatch - 200;
        std::string ns(n > 0 ? n : 0, 'N');
        read = read.substr(0, indel_pos) + ns + read.substr(indel_pos, read_len - indel_pos);
        qual = qual.substr(0, indel_pos) + ns + qual.substr(indel_pos, read_len - indel_pos);
    } else if (mismatch > 100) {
        int indel_pos;
        s >> indel_pos;
        const int n = mismatch - 100;
        read = read.substr(0, indel_pos) + read.substr(indel_pos + n, read_len - indel_pos - n);
        qual = qual.substr(0, indel_pos) + qual.substr(indel_pos + n, read_len - indel_pos - n);
    }
    position -= 1;
    return !s.fail();
}

/* Store one parsed read the way the pass-1 spill returns it in pass 2:
 * bases 2-bit coded and decoded (upper case, 'A' past the read),
 * qualities raw. */
void store_read(ReadStore* rs, const std::string& read, const std::string& qual, int hit, int read_len,
                char strand, int position, int mismatch) {
    const unsigned L = rs->L;
    if (read_len < 0 || (unsigned)read_len > L || (int)read.size() < read_len || (int)qual.size() < read_len) {
        /* the reference copies read_len bytes into an L-byte slot (cpp/soap_snp.h:372) */
        printf("!!!ERROR@store_read: read longer than -L or than its sequence field.\n");
        exit(EXIT_FAILURE);
    }
    const size_t off = rs->seq.size();
    rs->seq.resize(off + L, 'A');
    rs->qual.resize(off + L, 0);
    static const char letters[4] = {'A', 'C', 'G', 'T'};
    for (int i = 0; i < read_len; ++i) {
        const int c = oracle_base2bits(read[i]);
        if (c < 0) {
            /* encode() rejects the block (kernel/compress_kernel.cu:121-123) */
            printf("!!!ERROR@encode: unknown base when encoding.\n");
            exit(EXIT_FAILURE);
        }
        rs->seq[off + i] = letters[c];
        rs->qual[off + i] = qual[i];
    }
    rs->hit.push_back(hit);
    rs->len.push_back(read_len);
    rs->pos.push_back(position);
    rs->mismatch.push_back(mismatch);
    rs->strand.push_back(strand);
}

/* pass 1 of cpp/matrix.cc:42-213 plus the read store */
void matrix_gen(std::ifstream& alignment, const Params& para, Genome* genome, double* p_matrix,
                ReadStore* rs, bool count) {
    std::vector<unsigned long long> cm;
    if (count) cm.assign(256UL * 256UL * 16UL, 0ULL);
    Chromosome* current = nullptr;
    std::string current_name;
    std::string read, qual, chr;
    int hit = 0, read_len = 0, position = 0, mismatch = 0;
    char strand = 0;
    for (std::string line; std::getline(alignment, line);) {
        std::istringstream s(line);
        if (!parse_soap(s, read, qual, hit, read_len, strand, chr, position, mismatch)) continue;
        store_read(rs, read, qual, hit, read_len, strand, position, mismatch);
        rs->last_chr = chr;
        if (!count) continue;
        if (position < 0) continue;
        if (current == nullptr || current_name != chr) {
            auto it = genome->chr.find(chr);
            if (it == genome->chr.end()) {
                std::cerr << "Assertion Failed: Chromosome: !" << chr << "! NOT found" << std::endl;
                exit(255);
            }
            current = &it->second;
            current_name = chr;
        }
        if ((long)position + read_len >= (long)current->len) continue;
        if (hit != 1) continue;
        for (int coord = 0; coord != read_len; ++coord) {
            if (read[coord] == 'N') continue;
            const unsigned long long ref = current->base((unsigned long long)position + coord);
            if ((ref & 12) != 0) continue;
            const unsigned long long cyc = (strand == '+') ? (unsigned long long)coord
                                                             : (unsigned long long)(read_len - 1 - coord);
            cm[(((unsigned long long)(long long)qual[coord]) << 12) | (cyc << 4) | ((ref & 0x3) << 2) |
               (unsigned long long)((read[coord] >> 1) & 3)] += 1;
        }
    }
    if (!count) return;
    /* fill, cpp/matrix.cc:129-205 */
    const unsigned long long sta_pow = 10;
    for (int q_char = para.q_min; q_char <= para.q_max; q_char++) {
        unsigned long long by_type[16] = {0}, by_t[4] = {0}, total = 0, mism = 0;
        const unsigned long long qc = (unsigned long long)(long long)q_char;
        for (unsigned long long coord = 0; coord != para.read_length; ++coord)
            for (unsigned long long type = 0; type != 16; ++type) {
                const unsigned long long c = cm[(qc << 12) | coord << 4 | type];
                by_type[type] += c;
                by_t[(type >> 2) & 3] += c;
                total += c;
                if (type % 5 != 0) mism += c;
            }
        const unsigned long long qrow = (unsigned long long)(q_char - para.q_min) << 12;
        for (unsigned long long coord = 0; coord != para.read_length; ++coord) {
            unsigned long long sum[4] = {0, 0, 0, 0};
            for (unsigned long long type = 0; type != 16; ++type) sum[(type >> 2) & 3] += cm[(qc << 12) | (coord << 4) | type];
            for (unsigned long long t = 0; t != 4; ++t)
                for (unsigned long long o = 0; o != 4; ++o) {
                    double& p = p_matrix[qrow | (coord << 4) | (t << 2) | o];
                    const unsigned long long c = cm[(qc << 12) | (coord << 4) | (t << 2) | o];
                    if (c > sta_pow) p = ((double)c) / sum[t];
                    else if (by_type[t << 2 | o] > sta_pow) p = ((double)by_type[t << 2 | o]) / by_t[t];
                    else if (total > 0) p = (o == t) ? ((double)(total - mism)) / total : ((double)mism) / total;
                    if (p == 0 || p == 1) {
                        if (o == t) {
                            p = (1 - pow(10, -((q_char - para.q_min) / 10.0)));
                            if (p < 0.25) p = 0.25;
                        } else {
                            p = (pow(10, -((q_char - para.q_min) / 10.0)) / 3);
                            if (p > 0.25) p = 0.25;
                        }
                    }
                }
        }
    }
}

void matrix_write(std::fstream& out, const Params& para, const double* p_matrix) {
    /* cpp/matrix.cc:230-241 */
    for (int q_char = para.q_min; q_char <= para.q_max; q_char++)
        for (std::string::size_type coord = 0; coord != para.read_length; coord++) {
            out << ((unsigned long long)(long long)q_char - (unsigned long long)(long long)para.q_min) << '\t' << coord;
            for (char type = 0; type != 16; type++)
                out << '\t' << std::scientific << std::showpoint << std::setprecision(16)
                    << p_matrix[((unsigned long long)(q_char - para.q_min) << 12) | (coord << 4) | type];
            out << std::endl;
        }
}

void matrix_read(std::fstream& in, double* p_matrix) {
    /* cpp/matrix.cc:215-228 */
    for (std::string line; std::getline(in, line);) {
        std::istringstream s(line);
        int q_char = 0;
        std::string::size_type coord = 0;
        s >> q_char >> coord;
        for (int type = 0; type != 16; type++) s >> p_matrix[((unsigned long long)q_char << 12) | (coord << 4) | type];
    }
}

void prior_gen(const Params& para, double* p_prior) {
    /* cpp/prior.cc:3-43 */
    for (int t = 0; t != 4; t++)
        for (int a1 = 0; a1 != 4; a1++)
            for (int a2 = a1; a2 != 4; a2++) {
                double& v = p_prior[t << 4 | a1 << 2 | a2];
                if (a1 == t && a2 == t) v = 1;
                else if (a1 == t || a2 == t) v = para.het_novel;
                else if (a1 == a2) v = para.althom_novel;
                else v = para.het_novel * para.althom_novel;
                if (para.transition_dominant && ((a1 ^ t) == 0x3 || (a2 ^ t) == 0x3)) v *= 4;
            }
    for (int a1 = 0; a1 != 4; a1++)
        for (int a2 = a1; a2 != 4; a2++)
            for (int n = 4; n < 8; ++n)
                p_prior[n << 4 | a1 << 2 | a2] = (a1 == a2 ? 1 : (2 * para.het_novel)) * 0.25 * 0.25;
}

void rank_table_gen(double* p_rank) {
    /* cpp/rank_sum.cc:3-42 */
    double fact[64];
    fact[0] = 1.0;
    for (unsigned long long i = 1; i != 64; i++) fact[i] = fact[i - 1] * i;
    std::vector<unsigned long long> rs(64UL * 64UL * 2048UL, 0ULL);
    rs[0] = 1;
    for (unsigned long long N = 1; N != 64; N++)
        for (unsigned long long n1 = 0; n1 <= N; n1++) {
            for (unsigned long long T1 = (1 + n1) * n1 / 2; T1 <= (N + N - n1 + 1) * n1 / 2; T1++) {
                rs[N << 17 | n1 << 11 | T1] = rs[((N - 1) << 17) | (n1 << 11) | T1] +
                                              ((T1 >= N && n1 > 0) ? rs[((N - 1) << 17) | ((n1 - 1) << 11) | (T1 - N)] : 0);
                p_rank[(N << 17) | (n1 << 11) | T1] = rs[N << 17 | n1 << 11 | T1] / (fact[N] / (fact[n1] * fact[N - n1]));
            }
            double p_left = 0.0, p_right = 1.0;
            for (unsigned long long T1 = (1 + n1) * n1 / 2; T1 <= (N + N - n1 + 1) * n1 / 2; T1++) {
                p_right = 1.0 - p_left;
                p_left += p_rank[(N << 17) | (n1 << 11) | T1];
                p_rank[N << 17 | n1 << 11 | T1] = (p_left < p_right ? p_left : p_right);
            }
        }
}

bool all_n(const bool* nflag, unsigned long n) {
    for (unsigned long i = 0; i < n; ++i)
        if (!nflag[i]) return false;
    return true;
}

/* ---- -C column writers (cpp/compress.h) ---- */

void put(FILE* f, const void* p, size_t bytes) {
    if (bytes && fwrite(p, 1, bytes, f) != bytes) {
        printf("!!!ERROR: write failed\n");
        exit(EXIT_FAILURE);
    }
}

struct Columns {
    FILE* f346 = nullptr;
    FILE* frle = nullptr;
    FILE* f10 = nullptr;
    FILE* f111213 = nullptr;
    FILE* f1517 = nullptr;
    std::vector<std::string> names;
    std::vector<unsigned long> starts, sizes;

    void open(const std::string& base) {
        f346 = fopen((base + ".3_4_6").c_str(), "wb");
        frle = fopen((base + ".5_7_8_9_14_16").c_str(), "wb");
        f10 = fopen((base + ".10").c_str(), "wb");
        f111213 = fopen((base + ".11_12_13").c_str(), "wb");
        f1517 = fopen((base + ".15_17").c_str(), "wb");
        if (!f346 || !frle || !f10 || !f111213 || !f1517) {
            printf("!!!ERROR: cannot create the column files\n");
            exit(EXIT_FAILURE);
        }
    }
    void close(const std::string& base) {
        FILE* f = fopen((base + ".1_2").c_str(), "w");
        fprintf(f, "%lu\n", (unsigned long)names.size());
        for (size_t i = 0; i < names.size(); ++i) fprintf(f, "%s\t%lu\t%lu\n", names[i].c_str(), starts[i], sizes[i]);
        fclose(f);
        fclose(f346);
        fclose(frle);
        fclose(f10);
        fclose(f111213);
        fclose(f1517);
    }

    /* Column_3_4_6::compress + write (cpp/compress.h:171-409) */
    void col_3_4_6(char* c3, const char* c4, const char* c6, const bool* nflag, unsigned long n) {
        unsigned long param[7] = {1, 0, n, 0, 0, 0, 0};
        if (all_n(nflag, n)) {
            put(f346, param, sizeof(param));
            return;
        }
        param[0] = 0;
        std::vector<int> id4, id6, idn;
        std::vector<char> v4, v6;
        for (unsigned long i = 0; i < n; ++i) {
            if (c4[i] != c3[i]) { id4.push_back((int)i); v4.push_back(c4[i]); }
            if (c6[i] != c3[i]) { id6.push_back((int)i); v6.push_back(c6[i]); }
            if (c3[i] == 'N') { idn.push_back((int)i); c3[i] = 'A'; }
        }
        const unsigned long ncode = getNumBinWord(n);
        std::vector<unsigned int> code(ncode);
        encode(code.data(), c3, n);
        param[3] = ncode;
        param[4] = idn.size();
        param[5] = id4.size();
        param[6] = id6.size();
        param[1] = 5 * id4.size() + 5 * id6.size() + 4 * idn.size() + 4 * ncode;
        put(f346, param, sizeof(param));
        put(f346, id4.data(), 4 * id4.size());
        put(f346, v4.data(), v4.size());
        put(f346, id6.data(), 4 * id6.size());
        put(f346, v6.data(), v6.size());
        put(f346, idn.data(), 4 * idn.size());
        put(f346, code.data(), 4 * ncode);
    }

    /* one column of Column_RLEDict (cpp/compress.h:495-868, dict_compression.h:235-270) */
    template <class T>
    void rle_dict(T* col, unsigned long n) {
        std::vector<unsigned int> runlen(n);
        const unsigned int runs = RLECompression(col, n, runlen.data());
        std::vector<unsigned int> cval(runs), clen(runs);
        std::vector<T> dval(runs);
        std::vector<unsigned int> dlen(runs);
        unsigned long nwv = runs, ndv = 32 * 8192, nwl = runs, ndl = 32 * 8192;
        cuda_dictCompression(cval.data(), &nwv, dval.data(), &ndv, col, runs);
        cuda_dictCompression(clen.data(), &nwl, dlen.data(), &ndl, runlen.data(), runs);
        unsigned long param[6] = {runs, nwv, nwl, ndv, ndl, 4 * nwv + 4 * nwl + sizeof(T) * ndv + 4 * ndl};
        put(frle, param, sizeof(param));
        put(frle, cval.data(), 4 * nwv);
        put(frle, clen.data(), 4 * nwl);
        put(frle, dval.data(), sizeof(T) * ndv);
        put(frle, dlen.data(), 4 * ndl);
    }

    void col_rle(const int* q_cns, const int* q_sum, const int* cu, const int* ca, const int* depth,
                 const int* repeat, const char* base1, const bool* nflag, unsigned long n) {
        int flag = all_n(nflag, n) ? 1 : 0;
        put(frle, &flag, sizeof(int));
        if (flag) return;
        std::vector<int> col(n);
        std::vector<double> dcol(n);
        auto ok = [&](unsigned long j) { return !nflag[j] && base1[j] < 4; };
        for (unsigned long j = 0; j < n; ++j) col[j] = ok(j) ? q_cns[j] : 0;
        rle_dict(col.data(), n);
        for (unsigned long j = 0; j < n; ++j)
            col[j] = ok(j) ? (q_sum[j * 4 + base1[j]] == 0 ? 0 : q_sum[j * 4 + base1[j]] / cu[j * 4 + base1[j]]) : 0;
        rle_dict(col.data(), n);
        for (unsigned long j = 0; j < n; ++j) col[j] = ok(j) ? cu[j * 4 + base1[j]] : 0;
        rle_dict(col.data(), n);
        for (unsigned long j = 0; j < n; ++j) col[j] = ok(j) ? ca[j * 4 + base1[j]] : 0;
        rle_dict(col.data(), n);
        for (unsigned long j = 0; j < n; ++j) col[j] = ok(j) ? depth[j] : 0;
        rle_dict(col.data(), n);
        for (unsigned long j = 0; j < n; ++j)
            dcol[j] = ok(j) ? (depth[j] == 0 ? 255 : (double)(repeat[j]) / depth[j]) : 255.0;
        rle_dict(dcol.data(), n);
    }

    /* Column_10 (cpp/compress.h:759-897) */
    void col_10(const char* base1, const char* base2, const bool* nflag, unsigned long n) {
        int flag = all_n(nflag, n) ? 1 : 0;
        put(f10, &flag, sizeof(int));
        if (flag) return;
        std::vector<char> c(n);
        std::vector<unsigned int> nid;
        for (unsigned long j = 0; j < n; ++j) {
            c[j] = (!nflag[j] && base1[j] < 4 && base2[j] < 4) ? kActgN[(int)base2[j]] : 'N';
            if (c[j] == 'N') { nid.push_back((unsigned int)j); c[j] = 'A'; }
        }
        const unsigned long nw = getNumBinWord(n);
        std::vector<unsigned int> code(nw);
        encode(code.data(), c.data(), n);
        unsigned long param[3] = {nid.size(), nw, n};
        put(f10, param, sizeof(param));
        put(f10, code.data(), 4 * nw);
        put(f10, nid.data(), 4 * nid.size());
    }

    /* Column_11_12_13 (cpp/compress.h:947-1172) */
    void col_11_12_13(const int* q_sum, const int* cu, const int* ca, const char* base1, const char* base2,
                      const bool* nflag, unsigned long n) {
        int flag = all_n(nflag, n) ? 1 : 0;
        put(f111213, &flag, sizeof(int));
        if (flag) return;
        std::vector<int> cid, c11, c12, c13, e12id, e12, e13id, e13;
        for (unsigned long j = 0; j < n; ++j) {
            int v11 = 0, v12 = 0, v13 = 0;
            if (!nflag[j] && base1[j] < 4 && base2[j] < 4) {
                const int b = base2[j];
                v11 = q_sum[j * 4 + b] == 0 ? 0 : q_sum[j * 4 + b] / cu[j * 4 + b];
                v12 = cu[j * 4 + b];
                v13 = ca[j * 4 + b];
            }
            if (v11 != 0) { cid.push_back((int)j); c11.push_back(v11); c12.push_back(v12); c13.push_back(v13); }
            else if (v11 != v12) { e12id.push_back((int)j); e12.push_back(v12); }
            else if (v11 != v13) { e13id.push_back((int)j); e13.push_back(v13); }
        }
        unsigned long param[4] = {n, cid.size(), e12id.size(), e13id.size()};
        put(f111213, param, sizeof(param));
        put(f111213, e12id.data(), 4 * e12id.size());
        put(f111213, e12.data(), 4 * e12.size());
        put(f111213, e13id.data(), 4 * e13id.size());
        put(f111213, e13.data(), 4 * e13.size());
        put(f111213, cid.data(), 4 * cid.size());
        /* With no common entry the reference's dictCompression fails an assert
         * (cpp/dict_compression.h:140-143) and the run aborts; this happens in
         * every gap window inside an N block of at least one window.  Here an
         * empty dictionary is written as the pair {0, 0} with no payload. */
        for (std::vector<int>* v : {&c11, &c12, &c13}) {
            std::vector<unsigned int> words(W);
            std::vector<int> dict(W);
            unsigned long dp[2] = {W, W};
            oracle_dict_compress(words.data(), &dp[0], dict.data(), &dp[1], v->data(), v->size());
            put(f111213, dp, sizeof(dp));
            put(f111213, words.data(), 4 * dp[0]);
            put(f111213, dict.data(), 4 * dp[1]);
        }
    }

    /* Column_15_17 (cpp/compress.h:1175-1312) */
    void col_15_17(const char* base1, const bool* nflag, const double* rank_sum, const char* ori, unsigned long n) {
        int flag = all_n(nflag, n) ? 1 : 0;
        put(f1517, &flag, sizeof(int));
        if (flag) return;
        std::vector<int> id;
        std::vector<double> val;
        for (unsigned long j = 0; j < n; ++j)
            if (!nflag[j] && base1[j] < 4 && rank_sum[j] != 1.0) { id.push_back((int)j); val.push_back(rank_sum[j]); }
        int cnt = (int)id.size();
        put(f1517, &cnt, sizeof(int));
        put(f1517, id.data(), 4 * id.size());
        put(f1517, val.data(), 8 * val.size());
        id.clear();
        for (unsigned long j = 0; j < n; ++j)
            if (!nflag[j] && base1[j] < 4 && (ori[j] & 8)) id.push_back((int)j);
        cnt = (int)id.size();
        put(f1517, &cnt, sizeof(int));
        put(f1517, id.data(), 4 * id.size());
    }
};

/* the window driver: cpp/call_genotype.cc:211-669 */
struct Caller {
    const Params& para;
    const std::string chr_name;
    const Chromosome& chr;
    std::ostream& cns;
    Columns& cols;
    unsigned long L;
    unsigned int maxNumNonZero = 0;
    std::vector<int> cu, qs, ca, depth, repeat, dep_uni, pos;
    std::vector<unsigned int> sparse_host, num_host;
    std::vector<char> ori, base1, base2, type1;
    std::vector<int> q_cns;
    std::vector<double> rank_sum, type_likely;
    std::vector<unsigned char> nflag_store;
    bool* nflag;
    std::vector<unsigned char> validated, hapmap, indel;
    std::vector<double> freq;
    st_likelihood lk;
    std::vector<double> pmatrix_copy;

    Caller(const Params& p, const std::string& name, const Chromosome& c, std::ostream& out, Columns& col,
           const double* p_matrix)
        : para(p), chr_name(name), chr(c), cns(out), cols(col), L(p.read_length) {
        const unsigned long n = W + L;
        cu.assign(4 * n, 0); qs.assign(4 * n, 0); ca.assign(4 * n, 0);
        depth.assign(n, 0); repeat.assign(n, 0); dep_uni.assign(n, 0);
        pos.assign(n, -1);
        ori.assign(n, (char)0xFF);
        base1.assign(W, 0); base2.assign(W, 0); type1.assign(W, 0);
        q_cns.assign(W, 0); rank_sum.assign(W, 0.0); type_likely.assign(W * GSNP_LIKELY_SIZE, 0.0);
        nflag_store.assign(W, 0);
        nflag = reinterpret_cast<bool*>(nflag_store.data());
        validated.assign(W, 0); hapmap.assign(W, 0); indel.assign(W, 0); freq.assign(4 * W, 0.0);
        pmatrix_copy.assign(p_matrix, p_matrix + GSNP_PMATRIX_SIZE);
        lk.qmax = (char)p.q_max;
        lk.qmin = (char)p.q_min;
        lk.readLength = p.read_length;
        lk.globalDependency = p.global_dep;
        lk.pcrDependency = p.pcr_dep;
        lk.maxCallLength = W;
        lk.winSize = W;
        lk.numSite = W + L;
        lk.p_matrix = pmatrix_copy.data();
        lk.callLength = 0;
        lk.nflag = nflag;
        lk.countuni = cu.data();
        lk.typeLikelihood = type_likely.data();
    }

    void call(unsigned long call_length) {
        /* 1. ref base and N flag from the host depth (cpp/call_genotype.cc:222-230) */
        for (unsigned long j = 0; j != call_length; ++j) {
            ori[j] = (char)(chr.base((unsigned long long)pos[j]) & 0xF);
            nflag[j] = ((ori[j] & 4) != 0) && depth[j] == 0;
        }
        lk.callLength = call_length;
        cuda_likelihoodSparse(type_likely.data(), (unsigned int)call_length, maxNumNonZero,
                              (unsigned int)(W + L), GSNP_MAX_RECORDS_PER_SITE);
        for (unsigned long s = 0; s < call_length; ++s) {
            if ((ori[s] & 0x8) && para.refine) {
                const SnpInfo& snp = chr.dbsnp.find((unsigned long long)pos[s])->second;
                validated[s] = snp.validated;
                hapmap[s] = snp.hapmap;
                indel[s] = snp.indel;
                for (int i = 0; i < 4; ++i) freq[s * 4 + i] = snp.freq[i];
            }
        }
        cuda_posterior(&lk, ori.data(), base1.data(), base2.data(), type1.data(), q_cns.data(),
                       rank_sum.data(), reinterpret_cast<bool*>(validated.data()),
                       reinterpret_cast<bool*>(hapmap.data()), reinterpret_cast<bool*>(indel.data()),
                       freq.data(), para.het_val, para.het_unval, para.althom_val, para.althom_unval,
                       para.rank_sum, para.monoploid, para.refine, (char)(para.q_max - para.q_min), L,
                       (int)W, call_length, maxNumNonZero);
        if (para.compress) emit_columns(call_length);
        else emit_text(call_length);
    }

    void emit_columns(unsigned long n) {
        cols.names.push_back(chr_name);
        cols.starts.push_back((unsigned long)(pos[0] + 1));
        cols.sizes.push_back(n);
        std::vector<char> c3(n), c4(n), c6(n);
        for (unsigned long j = 0; j < n; ++j) {
            if (nflag[j] || base1[j] >= 4) { c3[j] = c4[j] = c6[j] = 'N'; continue; }
            c3[j] = kActgN[ori[j] & 0x7];
            c4[j] = kAbbv[(int)type1[j]];
            c6[j] = kActgN[(int)base1[j]];
        }
        cols.col_3_4_6(c3.data(), c4.data(), c6.data(), nflag, n);
        cols.col_rle(q_cns.data(), qs.data(), cu.data(), ca.data(), depth.data(), repeat.data(), base1.data(), nflag, n);
        cols.col_10(base1.data(), base2.data(), nflag, n);
        cols.col_11_12_13(qs.data(), cu.data(), ca.data(), base1.data(), base2.data(), nflag, n);
        cols.col_15_17(base1.data(), nflag, rank_sum.data(), ori.data(), n);
    }

    void emit_text(unsigned long n) {
        /* cpp/call_genotype.cc:355-410 */
        for (unsigned long j = 0; j != n; ++j) {
            const int b1 = base1[j], b2 = base2[j];
            if (nflag[j] || b1 >= 4) {
                cns << chr_name << '\t' << (pos[j] + 1) << "\tN\tN\t0\tN\t0\t0\t0\tN\t0\t0\t0\t0\t1.000\t255.000\t0" << '\n';
                continue;
            }
            cns << chr_name << '\t' << (pos[j] + 1) << '\t' << kActgN[ori[j] & 0x7] << '\t' << kAbbv[(int)type1[j]]
                << '\t' << q_cns[j] << '\t' << kActgN[b1] << '\t'
                << (qs[j * 4 + b1] == 0 ? 0 : qs[j * 4 + b1] / cu[j * 4 + b1]) << '\t' << cu[j * 4 + b1] << '\t'
                << ca[j * 4 + b1] << '\t';
            if (b2 < 4) {
                cns << kActgN[b2] << '\t' << (qs[j * 4 + b2] == 0 ? 0 : qs[j * 4 + b2] / cu[j * 4 + b2]) << '\t'
                    << cu[j * 4 + b2] << '\t' << ca[j * 4 + b2] << '\t';
            } else {
                cns << "N\t0\t0\t0\t";
            }
            cns << depth[j] << '\t' << std::showpoint << rank_sum[j] << '\t'
                << (depth[j] == 0 ? 255 : (double)(repeat[j]) / depth[j]) << '\t' << ((ori[j] & 8) ? 1 : 0) << '\n';
        }
    }
};

int soap2cns(const Params& para, const ReadStore& rs, Genome* genome, const double* p_matrix,
             const double* p_prior, const double* p_rank, std::ostream& cns, const std::string& cns_name) {
    const unsigned long L = para.read_length;
    GSNPKernelInit(W, para.read_length, para.pcr_dep, para.global_dep, p_matrix, p_prior, p_rank);
    Columns cols;
    cols.open(cns_name);
    dictComprStart(W, sizeof(double));

    auto it = genome->chr.find(rs.last_chr);
    if (it == genome->chr.end()) {
        std::cerr << "Assertion Failed: Chromosome: !" << rs.last_chr << "! NOT found" << std::endl;
        exit(255);
    }
    Chromosome* chr = nullptr;
    std::string chr_name;

    /* st_update staging buffers (cpp/gsnp.h:152-217) */
    const unsigned long R = GSNP_READS_PER_WINDOW;
    std::vector<char> uchar(L * R * 2 + R);
    std::vector<int> uint_(R + W * 2);
    std::vector<int> positionArr(R, 0), hitArr(R, 0), lenArr(R, 0), mismatchArr(R, 0);
    std::vector<char> abArr(R, 0);
    st_update u;
    u.inputUpdateChar = uchar.data();
    u.inputUpdateInt = uint_.data();
    u.readArr = uchar.data();
    u.qualArr = uchar.data() + L * R;
    u.strandArr = uchar.data() + 2 * L * R;
    u.readLen_hitArr = uint_.data();
    u.siteMatchArr = uint_.data() + R;
    u.char_nameArr = nullptr;
    u.hitArr = hitArr.data();
    u.read_lenArr = lenArr.data();
    u.positionArr = positionArr.data();
    u.mismatchArr = mismatchArr.data();
    u.abArr = abArr.data();
    u.qmin = (char)para.q_min;
    u._read_length = (unsigned int)L;

    Caller* caller = nullptr;
    long last_start = 0;
    unsigned long readCount = 0;
    bool mark = false;
    for (size_t r = 0; r < rs.size(); ++r) {
        memcpy(u.readArr + readCount * L, &rs.seq[r * L], L);
        memcpy(u.qualArr + readCount * L, &rs.qual[r * L], L);
        hitArr[readCount] = rs.hit[r];
        lenArr[readCount] = rs.len[r];
        positionArr[readCount] = rs.pos[r];
        mismatchArr[readCount] = rs.mismatch[r];
        u.strandArr[readCount] = rs.strand[r];
        u.readLen_hitArr[readCount] = (int)(((rs.len[r]) & 0xffff) << 16 | rs.hit[r]);
        const int p = positionArr[readCount];
        if (p < 0) continue;
        if (chr == nullptr) {
            chr = &it->second;
            chr_name = it->first;
            caller = new Caller(para, chr_name, *chr, cns, cols, p_matrix);
            cuda_init(W, L, 0, caller->pos.data());
            last_start = 0;
        }
        if ((long)p + lenArr[readCount] >= (long)chr->len) continue;
        if (p < last_start) {
            std::cerr << "Errors in sorting:" << p << "<" << last_start << std::endl;
            exit(255);
        }
        mark = false;
        if (readCount != 0 && (unsigned long)p / W > (unsigned long)last_start / W) {
            gold_pos_match(positionArr.data(), u.siteMatchArr, (int)readCount);
            caller->maxNumNonZero = cuda_updateSparse(&u, nullptr, nullptr, (int)L, caller->cu.data(), caller->qs.data(),
                                                      caller->ca.data(), caller->depth.data(),
                                                      caller->repeat.data(), caller->dep_uni.data(), (int)readCount);
            mark = true;
        }
        while ((unsigned long)p / W > (unsigned long)last_start / W) {
            if (last_start > caller->pos[W - 1]) cuda_init(W, L, (last_start / W) * W, caller->pos.data());
            caller->call(W);
            cuda_recycle(W, L, caller->pos.data());
            last_start = caller->pos[W - 1];
        }
        last_start = p;
        if (mark) {
            /* st_update::updateSoap2: move the triggering read to slot 0 */
            const unsigned long t = readCount;
            memmove(u.readArr, u.readArr + t * L, L);
            memmove(u.qualArr, u.qualArr + t * L, L);
            u.readLen_hitArr[0] = (int)(((lenArr[t]) & 0xffff) << 16 | hitArr[t]);
            positionArr[0] = positionArr[t];
            mismatchArr[0] = mismatchArr[t];
            abArr[0] = abArr[t];
            u.strandArr[0] = u.strandArr[t];
            readCount = 0;
        }
        readCount += 1;
    }
    if (caller == nullptr) {
        printf("!!!ERROR: no usable alignment.\n");
        exit(EXIT_FAILURE);
    }
    if (!mark) {
        gold_pos_match(positionArr.data(), u.siteMatchArr, (int)readCount);
        caller->maxNumNonZero = cuda_updateSparse(&u, nullptr, nullptr, (int)L, caller->cu.data(), caller->qs.data(),
                                                  caller->ca.data(), caller->depth.data(), caller->repeat.data(),
                                                  caller->dep_uni.data(), (int)readCount);
    }
    while (chr->len > (unsigned int)caller->pos[W - 1]) {
        if (last_start > caller->pos[W - 1]) cuda_init(W, L, (last_start / W) * W, caller->pos.data());
        caller->call(W);
        cuda_quickRecycle(W, L, caller->pos.data(), caller->cu.data(), caller->qs.data(), caller->ca.data(),
                          caller->depth.data(), caller->repeat.data());
        last_start = caller->pos[W - 1];
    }
    if (last_start > caller->pos[W - 1]) cuda_init(W, L, (last_start / W) * W, caller->pos.data());
    caller->call(chr->len % W);
    cols.close(cns_name);
    dictComprEnd();
    delete caller;
    return 1;
}

}  // namespace

void oracle_rank_table(double* p_rank) { rank_table_gen(p_rank); }

void oracle_prior_table(double het_novel, double althom_novel, bool transition_dominant, double* p_prior) {
    Params para;
    para.het_novel = het_novel;
    para.althom_novel = althom_novel;
    para.transition_dominant = transition_dominant;
    prior_gen(para, p_prior);
}

int oracle_main(int argc, char** argv) {
    GPUInit();
    Params para;
    std::string alignment_name, consensus_name;
    std::ifstream soap, fasta, dbsnp;
    std::fstream matrix_file;
    bool matrix_in = false, have_dbsnp = false, have_matrix_file = false;
    int c;
    optind = 1;
    while ((c = getopt(argc, argv, "i:d:o:z:g:p:r:e:ts:2a:b:j:k:unmqM:I:L:Q:S:F:E:T:h:C")) != -1) {
        switch (c) {
            case 'i':
                soap.open(optarg);
                if (!soap) { std::cerr << "No such file or directory:" << optarg << std::endl; exit(1); }
                alignment_name = optarg;
                break;
            case 'd':
                fasta.open(optarg);
                if (!fasta) { std::cerr << "No such file or directory:" << optarg << std::endl; exit(1); }
                break;
            case 'o': consensus_name = optarg; break;
            case 'z': para.q_min = (signed char)optarg[0]; para.q_max = (signed char)(para.q_min + 40); break;
            case 'g': para.global_dep = log10(atof(optarg)); break;
            case 'p': para.pcr_dep = log10(atof(optarg)); break;
            case 'r': para.althom_novel = atof(optarg); break;
            case 'e': para.het_novel = atof(optarg); break;
            case 't': para.transition_dominant = true; break;
            case 's':
                dbsnp.open(optarg);
                if (!dbsnp) { std::cerr << "No such file or directory:" << optarg << std::endl; exit(1); }
                have_dbsnp = true;
                break;
            case '2': para.refine = true; break;
            /* the reference assigns -a/-b and -j/-k crosswise to its usage text (cpp/main.cc:194-213) */
            case 'a': para.althom_val = atof(optarg); break;
            case 'b': para.het_val = atof(optarg); break;
            case 'j': para.althom_unval = atof(optarg); break;
            case 'k': para.het_unval = atof(optarg); break;
            case 'u': para.rank_sum = true; break;
            case 'n': break;
            case 'm': para.monoploid = true; break;
            case 'q': printf("ERROR: The -q parameter currently is not supported.\n"); exit(0);
            case 'M':
                matrix_file.close();
                matrix_file.clear();
                matrix_file.open(optarg, std::fstream::out);
                if (!matrix_file) { std::cerr << "Cannot creat file :" << optarg << std::endl; exit(1); }
                have_matrix_file = true;
                break;
            case 'I':
                matrix_file.close();
                matrix_file.clear();
                matrix_file.open(optarg, std::fstream::in);
                if (!matrix_file) { std::cerr << "No such file or directory:" << optarg << std::endl; exit(1); }
                matrix_in = true;
                have_matrix_file = true;
                break;
            case 'S': break;
            case 'L': para.read_length = (unsigned char)atoi(optarg); break;
            case 'Q':
                para.q_max = (signed char)optarg[0];
                if (para.q_max < para.q_min) std::cerr << "FASTQ quality character error: Q_MAX > Q_MIN" << std::endl;
                break;
            case 'F': printf("ERROR: The -F parameter currently is not supported.\n"); exit(0);
            case 'E': printf("ERROR: The -E parameter currently is not supported.\n"); break;
            case 'T': printf("ERROR: the -T parameter currently is not supported.\n"); exit(0);
            case 'C': para.compress = true; break;
            default: usage();
        }
    }
    if (consensus_name.empty() || !fasta.is_open() || !soap.is_open()) usage();
    std::ofstream cns(consensus_name.c_str());
    if (!cns) { std::cerr << "Cannot creat file:" << consensus_name << std::endl; exit(1); }

    Genome genome;
    load_genome(fasta, have_dbsnp ? &dbsnp : nullptr, &genome);

    std::vector<double> p_matrix(GSNP_PMATRIX_SIZE, 1.0), p_prior(8 * 16, 1.0), p_rank(GSNP_PRANK_SIZE, 1.0);
    ReadStore rs;
    rs.L = para.read_length;
    if (!matrix_in) {
        matrix_gen(soap, para, &genome, p_matrix.data(), &rs, true);
        if (have_matrix_file) matrix_write(matrix_file, para, p_matrix.data());
    } else {
        matrix_read(matrix_file, p_matrix.data());
        matrix_gen(soap, para, &genome, p_matrix.data(), &rs, false);
    }
    matrix_file.close();
    prior_gen(para, p_prior.data());
    rank_table_gen(p_rank.data());
    struct timeval t0, t1;
    gettimeofday(&t0, nullptr);
    soap2cns(para, rs, &genome, p_matrix.data(), p_prior.data(), p_rank.data(), cns, consensus_name);
    cns.close();
    gettimeofday(&t1, nullptr);
    /* wall time of the calling pass (window loop and output), for the CPU
     * baseline of the benchmark */
    if (getenv("GSNP_ORACLE_TIMING"))
        fprintf(stderr, "pass2_seconds=%.6f\n", (t1.tv_sec - t0.tv_sec) + 1e-6 * (t1.tv_usec - t0.tv_usec));
    return 0;
}
