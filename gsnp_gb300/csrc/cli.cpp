/*
 * cli.cpp - the `gsnp` command: SOAPsnp/GSNP consensus calling on one GB300.
 *
 * Same options, inputs and outputs as the reference's command line
 * (cpp/main.cc:85-420): a sorted SOAP alignment file (-i), the reference
 * FASTA (-d), the consensus output (-o, cns text, or the -C compressed
 * files), optional dbSNP priors (-s, -2), calibration matrix output/input
 * (-M/-I) and the model parameters.  One extra option, -P fp64|fp32, picks
 * the likelihood form (default fp32: FP32 compensated sums with FP64 fixup;
 * both forms give identical output).
 *
 * The whole chromosome is resident on the device: the alignments are parsed
 * on every host core, uploaded once, calibrated and called by the kernels of
 * libgsnp_gb300.so behind include/gsnp_gb300.h.  As in the reference, the
 * called chromosome is the one named by the last alignment, and all
 * alignments must be on it.
 */
#include <fcntl.h>
#include <getopt.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gsnp_gb300.h"

namespace {

struct Options {
    std::string soap, fasta, out, dbsnp, matrix_out, matrix_in;
    gsnp_params p{};
    bool compress = false;
};

[[noreturn]] void usage() {
    std::cerr << "GSNP (GB300)\n"
                 "Compulsory Parameters:\n"
                 "-i <FILE> Input SORTED Soap Result\n"
                 "-d <FILE> Reference Sequence in fasta format\n"
                 "-o <FILE> Output consensus file\n"
                 "Optional Parameters:\n"
                 "-z <Char> ASCII chracter standing for quality==0 [@]\n"
                 "-g <Double> Global Error Dependency Coefficient, 0.0(complete dependent)~1.0(complete independent)[0.9]\n"
                 "-p <Double> PCR Error Dependency Coefficient, 0.0(complete dependent)~1.0(complete independent)[0.5]\n"
                 "-r <Double> novel altHOM prior probability [0.0005]\n"
                 "-e <Double> novel HET prior probability [0.0010]\n"
                 "-t set transition/transversion ratio to 2:1 in prior probability\n"
                 "-s <FILE> Pre-formated dbSNP information\n"
                 "-2 specify this option will REFINE SNPs using dbSNPs information [Off]\n"
                 "-a <Double> Validated HET prior, if no allele frequency known [0.1]\n"
                 "-b <Double> Validated altHOM prior, if no allele frequency known[0.05]\n"
                 "-j <Double> Unvalidated HET prior, if no allele frequency known [0.02]\n"
                 "-k <Double> Unvalidated altHOM rate, if no allele frequency known[0.01]\n"
                 "-u Enable rank sum test to give HET further penalty for better accuracy. [Off]\n"
                 "-m Enable monoploid calling mode, this will ensure all consensus as HOM and you MUST specify "
                 "this option for male chrX\n"
                 "-M <FILE> Output the quality calibration matrix\n"
                 "-I <FILE> Input previous quality calibration matrix\n"
                 "-L <short> maximum length of read [45]\n"
                 "-Q <short> maximum FASTQ quality score [40]\n"
                 "-C Output compressed consensus files\n"
                 "-P fp64|fp32 likelihood form on the GPU [fp32]\n";
    exit(1);
}

void parse_args(int argc, char** argv, Options* o) {
    gsnp_params& p = o->p;
    p.q_min = 64;
    p.q_max = 64 + 40;
    p.read_length = 45;
    p.pcr_dependency = log10(0.5);
    p.global_dependency = log10(0.9);
    p.het_novel = 0.0010;
    p.althom_novel = 0.0005;
    p.het_val = 0.10;
    p.althom_val = 0.05;
    p.het_unval = 0.02;
    p.althom_unval = 0.01;
    p.precision = GSNP_PRECISION_FP32_FIXUP;
    int c;
    while ((c = getopt(argc, argv, "i:d:o:z:g:p:r:e:ts:2a:b:j:k:unmqM:I:L:Q:S:F:E:T:h:CP:")) != -1) {
        switch (c) {
            case 'i': o->soap = optarg; break;
            case 'd': o->fasta = optarg; break;
            case 'o': o->out = optarg; break;
            case 'z': p.q_min = (signed char)optarg[0]; p.q_max = (signed char)(p.q_min + 40); break;
            case 'g': p.global_dependency = log10(atof(optarg)); break;
            case 'p': p.pcr_dependency = log10(atof(optarg)); break;
            case 'r': p.althom_novel = atof(optarg); break;
            case 'e': p.het_novel = atof(optarg); break;
            case 't': p.transition_dominant = 1; break;
            case 's': o->dbsnp = optarg; break;
            case '2': p.refine = 1; break;
            /* the reference stores -a/-b and -j/-k crosswise to its usage text
             * (cpp/main.cc:194-213); kept so that the same command line gives
             * the same output */
            case 'a': p.althom_val = atof(optarg); break;
            case 'b': p.het_val = atof(optarg); break;
            case 'j': p.althom_unval = atof(optarg); break;
            case 'k': p.het_unval = atof(optarg); break;
            case 'u': p.rank_sum = 1; break;
            case 'n': break;
            case 'm': p.monoploid = 1; break;
            case 'q': printf("ERROR: The -q parameter currently is not supported.\n"); exit(0);
            case 'M': o->matrix_out = optarg; break;
            case 'I': o->matrix_in = optarg; break;
            case 'S': break;
            case 'L': p.read_length = (unsigned char)atoi(optarg); break;
            case 'Q':
                p.q_max = (signed char)optarg[0];
                if (p.q_max < p.q_min) std::cerr << "FASTQ quality character error: Q_MAX > Q_MIN" << std::endl;
                break;
            case 'F': printf("ERROR: The -F parameter currently is not supported.\n"); exit(0);
            case 'E': printf("ERROR: The -E parameter currently is not supported.\n"); break;
            case 'T': printf("ERROR: the -T parameter currently is not supported.\n"); exit(0);
            case 'C': o->compress = true; break;
            case 'P':
                if (!strcmp(optarg, "fp64")) p.precision = GSNP_PRECISION_FP64;
                else if (!strcmp(optarg, "fp32")) p.precision = GSNP_PRECISION_FP32_FIXUP;
                else usage();
                break;
            default: usage();
        }
    }
    if (o->out.empty() || o->fasta.empty() || o->soap.empty()) usage();
}

[[noreturn]] void die(const std::string& msg, int code = EXIT_FAILURE) {
    std::cerr << msg << std::endl;
    exit(code);
}

/* ---- reference and dbSNP (cpp/chromosome.cc:28-220) ---- */

struct Chromosome {
    std::vector<uint8_t> codes;   /* (base >> 1) & 7, bit 3 = dbSNP */
    std::vector<gsnp_snp> snp;    /* by position, the first row of each position */
};

inline bool is_sep(char c) { return c == ' ' || c == '\t' || c == '\r'; }

/* The first space, tab or CR in [p, end).  Eight bytes at a time while none
 * of them is one (a byte equal to x makes (w ^ x-bytes) have a zero byte,
 * which (v - 0x01..) & ~v & 0x80.. detects exactly), then byte by byte. */
inline const char* find_sep(const char* p, const char* end) {
    auto has_zero = [](uint64_t v) { return (v - 0x0101010101010101ull) & ~v & 0x8080808080808080ull; };
    while (end - p >= 8) {
        uint64_t w;
        memcpy(&w, p, 8);
        if (has_zero(w ^ 0x2020202020202020ull) | has_zero(w ^ 0x0909090909090909ull) |
            has_zero(w ^ 0x0d0d0d0d0d0d0d0dull))
            break;
        p += 8;
    }
    while (p < end && !is_sep(*p)) ++p;
    return p;
}

bool next_token(const char*& p, const char* end, const char** tok, size_t* len) {
    while (p < end && is_sep(*p)) ++p;
    if (p >= end) return false;
    *tok = p;
    p = find_sep(p, end);
    *len = (size_t)(p - *tok);
    return true;
}

bool to_int(const char* t, size_t n, int* v) {
    char buf[32];
    if (n == 0 || n >= sizeof(buf)) return false;
    memcpy(buf, t, n);
    buf[n] = 0;
    char* e = nullptr;
    errno = 0;
    const long x = strtol(buf, &e, 10);
    if (e == buf || errno) return false;
    *v = (int)x;
    return true;
}

/* A read-only mapping of a whole file (empty: data == nullptr). */
struct MappedFile {
    const char* data = nullptr;
    size_t size = 0;
    explicit MappedFile(const std::string& path) {
        const int fd = open(path.c_str(), O_RDONLY);
        if (fd < 0) die("No such file or directory:" + path, 1);
        struct stat st;
        fstat(fd, &st);
        size = (size_t)st.st_size;
        if (size > 0) {
            void* m = mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);
            if (m == MAP_FAILED) die("cannot map " + path);
            data = (const char*)m;
        }
        close(fd);
    }
    ~MappedFile() {
        if (data) munmap((void*)data, size);
    }
    MappedFile(const MappedFile&) = delete;
    MappedFile& operator=(const MappedFile&) = delete;
};

/* Every byte of a line after a '>' line is a base of that chromosome, coded
 * (byte >> 1) & 7; the name is the header up to the first space
 * (cpp/chromosome.cc:172-205).  A sequence replaces its chromosome's codes
 * when the next header comes, or at the end of the file if it is not empty:
 * a repeated name takes the later sequence, except an empty one at the end. */
void load_fasta(const std::string& path, std::map<std::string, Chromosome>* chrs) {
    const MappedFile f(path);
    const char* p = f.data;
    const char* const end = f.data + f.size;
    Chromosome* cur = nullptr;
    std::vector<uint8_t> seq;
    while (p < end) {
        const char* eol = (const char*)memchr(p, '\n', (size_t)(end - p));
        if (!eol) eol = end;
        if (p < eol && *p == '>') {
            if (cur) cur->codes.swap(seq);
            seq.clear();
            const char* q = p + 1;
            while (q < eol && !isspace((unsigned char)*q)) ++q;
            const std::string name(p + 1, (size_t)(q - p - 1));
            auto r = chrs->emplace(name, Chromosome());
            if (!r.second) std::cerr << "Insert Chromosome " << name << " Failed!\n";
            cur = &r.first->second;
        } else if (cur && eol > p) {
            const size_t k = seq.size(), n = (size_t)(eol - p);
            seq.resize(k + n);
            uint8_t* d = seq.data() + k;
            for (size_t i = 0; i < n; ++i) d[i] = (uint8_t)((((unsigned char)p[i]) >> 1) & 7);
        }
        p = eol + 1;
    }
    if (cur && !seq.empty()) cur->codes.swap(seq);
}

/* A decimal in its plain form, [+-]digits[.digits][(e|E)[+-]digits], to the
 * nearest double; false if the form is not plain.  With at most 15
 * significant digits and a power of ten up to 1e22, the digits and the power
 * are exact doubles and one correctly rounded multiply or divide gives the
 * nearest double (Clinger's fast path, "How to read floating point numbers
 * accurately", 1990); anything else goes to strtod. */
bool plain_decimal(const char* t, size_t n, double* out) {
    size_t i = 0;
    bool neg = false;
    if (i < n && (t[i] == '+' || t[i] == '-')) neg = t[i++] == '-';
    uint64_t m = 0;
    int sig = 0, exp10 = 0;
    size_t digits = 0;
    auto take = [&](char ch, bool frac) {
        if (sig == 0 && ch == '0') {
            if (frac) --exp10;
            return;
        }
        if (sig < 19) {
            m = m * 10 + (uint64_t)(ch - '0');
            if (frac) --exp10;
        } else if (!frac) {
            ++exp10;
        }
        ++sig;
    };
    while (i < n && isdigit((unsigned char)t[i])) take(t[i++], false), ++digits;
    if (i < n && t[i] == '.') {
        ++i;
        while (i < n && isdigit((unsigned char)t[i])) take(t[i++], true), ++digits;
    }
    if (digits == 0) return false;
    if (i < n && (t[i] == 'e' || t[i] == 'E')) {
        ++i;
        bool eneg = false;
        if (i < n && (t[i] == '+' || t[i] == '-')) eneg = t[i++] == '-';
        size_t ed = 0;
        int e = 0;
        while (i < n && isdigit((unsigned char)t[i])) {
            if (e < 100000) e = e * 10 + (t[i] - '0');
            ++i, ++ed;
        }
        if (ed == 0) return false;
        exp10 += eneg ? -e : e;
    }
    if (i != n) return false;
    static const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                      1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    if (sig <= 15 && exp10 >= -22 && exp10 <= 22) {
        const double v = (double)m;
        const double x = exp10 < 0 ? v / kPow10[-exp10] : v * kPow10[exp10];
        *out = neg ? -x : x;
        return true;
    }
    char buf[64];
    if (n >= sizeof(buf)) return false;
    memcpy(buf, t, n);
    buf[n] = 0;
    /* out of range: the stream's own answer differs from strtod's */
    errno = 0;
    const double x = strtod(buf, nullptr);
    if (errno == ERANGE) return false;
    *out = x;
    return true;
}

/* A dbSNP row "chr pos hapmap validated indel fA fC fT fG ..." whose fields
 * all have their plain form (pos digits, flags 0 or 1, frequencies plain
 * decimals, no whitespace but spaces, tabs and CR) gives what the stream
 * extraction gives; false leaves the row to that extraction. */
bool parse_snp_row(const char* p, const char* e, std::string* name, size_t* pos, bool* flag, double* f) {
    for (const char* q = p; q < e; ++q)
        if (isspace((unsigned char)*q) && *q != ' ' && *q != '\t' && *q != '\r') return false;
    const char* tok;
    size_t n;
    if (!next_token(p, e, &tok, &n)) return false;
    name->assign(tok, n);
    if (!next_token(p, e, &tok, &n) || n > 18) return false;
    size_t v = 0;
    for (size_t i = 0; i < n; ++i) {
        if (!isdigit((unsigned char)tok[i])) return false;
        v = v * 10 + (size_t)(tok[i] - '0');
    }
    *pos = v;
    for (int k = 0; k < 3; ++k) {
        if (!next_token(p, e, &tok, &n) || n != 1 || (tok[0] != '0' && tok[0] != '1')) return false;
        flag[k] = tok[0] == '1';
    }
    for (int k = 0; k < 4; ++k) {
        double x;
        if (!next_token(p, e, &tok, &n) || !plain_decimal(tok, n, &x)) return false;
        f[k] = x;
    }
    return true;
}

/* The known-SNP rows (cpp/chromosome.cc:207-221).  The name, the position
 * and the SNP fields live across rows there: a field that fails to parse
 * leaves it and the fields after it as the previous row left them (a blank
 * row repeats the previous row at the position before it). */
void load_dbsnp(const std::string& path, std::map<std::string, Chromosome>* chrs) {
    const MappedFile file(path);
    const char* p = file.data;
    const char* const end = file.data + file.size;
    bool hapmap = false, validated = false, indel = false;
    double f[4] = {0, 0, 0, 0};
    std::string name;
    std::string::size_type pos = 0;
    auto last = chrs->end();
    while (p < end) {
        const char* eol = (const char*)memchr(p, '\n', (size_t)(end - p));
        if (!eol) eol = end;
        bool flag[3];
        if (parse_snp_row(p, eol, &name, &pos, flag, f)) {
            hapmap = flag[0];
            validated = flag[1];
            indel = flag[2];
        } else {
            /* the stream extraction itself */
            std::istringstream s(std::string(p, (size_t)(eol - p)));
            s >> name >> pos;
            s >> hapmap >> validated >> indel >> f[0] >> f[1] >> f[2] >> f[3];
        }
        p = eol + 1;
        if (last == chrs->end() || last->first != name) last = chrs->find(name);
        if (last == chrs->end()) continue;
        pos -= 1;
        Chromosome& c = last->second;
        if (pos >= c.codes.size()) continue;
        gsnp_snp r{};
        r.pos = (uint32_t)pos;
        r.validated = validated;
        r.hapmap = hapmap;
        r.indel = indel;
        for (int i = 0; i < 4; ++i) r.freq[i] = f[i];
        c.snp.push_back(r);
        c.codes[pos] |= 8;
    }
    /* the rows of each chromosome by position; where a position repeats, its
     * first row counts, as the first insertion into the reference's map */
    for (auto& kv : *chrs) {
        std::vector<gsnp_snp>& v = kv.second.snp;
        std::stable_sort(v.begin(), v.end(), [](const gsnp_snp& x, const gsnp_snp& y) { return x.pos < y.pos; });
        v.erase(std::unique(v.begin(), v.end(), [](const gsnp_snp& x, const gsnp_snp& y) { return x.pos == y.pos; }),
                v.end());
    }
}

/* ---- SOAP alignments (cpp/soap_snp.h:132-169) ---- */

/* An array of a trivially copyable type left uninitialised, so that the
 * threads that fill it are the first to touch its pages. */
template <class T>
struct RawArray {
    std::unique_ptr<T[]> p;
    void allocate(size_t count) { p.reset(new T[count > 0 ? count : 1]); }
    T* data() { return p.get(); }
    T& operator[](size_t i) { return p[i]; }
    const T& operator[](size_t i) const { return p[i]; }
};

struct Reads {
    size_t n = 0;                     /* alignments kept */
    RawArray<int32_t> pos, len, hit;
    RawArray<uint8_t> strand;
    RawArray<uint8_t> seq, qual;      /* L bytes per alignment */
    RawArray<uint16_t> chr_id;
    std::vector<std::string> chr;     /* distinct chromosome names, in order of first use */
    std::string bad;                  /* first error */
};

/* One thread's share of the file: whole lines [begin, end), written to the
 * output from row `first` on. */
struct Chunk {
    const char* begin = nullptr;
    const char* end = nullptr;
    size_t lines = 0;                 /* its lines: a bound on its alignments */
    size_t first = 0;                 /* output row of its first alignment */
    size_t kept = 0;                  /* alignments parsed */
    std::vector<std::string> chr;     /* its chromosome names, in order of first use */
    std::unordered_map<std::string, uint32_t> chr_id;   /* name -> index in chr */
    std::string bad;                  /* its first error */
};

size_t count_lines(const char* b, const char* e) {
    size_t n = 0;
    while (b < e) {
        const char* nl = (const char*)memchr(b, '\n', (size_t)(e - b));
        ++n;
        if (!nl) break;
        b = nl + 1;
    }
    return n;
}

/* Parse the lines of chunk c into rows c->first, c->first + 1, ... of out;
 * the reference's stream extraction skips a line whose fields do not parse.
 * Row padding past the read length is 'A' and quality 0. */
void parse_chunk(Chunk* c, int L, Reads* out) {
    std::string read, qual;
    size_t last_cid = (size_t)-1;
    const char* p = c->begin;
    while (p < c->end) {
        const char* eol = (const char*)memchr(p, '\n', (size_t)(c->end - p));
        if (!eol) eol = c->end;
        const char* q = p;
        p = eol + 1;
        const char* tok[11];
        size_t tl[11];
        int nt = 0;
        while (nt < 11 && next_token(q, eol, &tok[nt], &tl[nt])) ++nt;
        if (nt < 10) continue;
        int hit, read_len, position, mismatch;
        if (!to_int(tok[3], tl[3], &hit) || !to_int(tok[5], tl[5], &read_len) || !to_int(tok[8], tl[8], &position) ||
            !to_int(tok[9], tl[9], &mismatch))
            continue;
        const char* rs = tok[1];
        const char* qs = tok[2];
        size_t rn = tl[1], qn = tl[2];
        if (mismatch > 100) {
            int indel_pos;
            if (nt < 11 || !to_int(tok[10], tl[10], &indel_pos)) continue;
            read.assign(tok[1], tl[1]);
            qual.assign(tok[2], tl[2]);
            if (mismatch > 200) {
                const int n = mismatch - 200;
                const std::string ns(n > 0 ? n : 0, 'N');
                read = read.substr(0, indel_pos) + ns + read.substr(indel_pos, read_len - indel_pos);
                qual = qual.substr(0, indel_pos) + ns + qual.substr(indel_pos, read_len - indel_pos);
            } else {
                const int n = mismatch - 100;
                read = read.substr(0, indel_pos) + read.substr(indel_pos + n, read_len - indel_pos - n);
                qual = qual.substr(0, indel_pos) + qual.substr(indel_pos + n, read_len - indel_pos - n);
            }
            rs = read.data();
            qs = qual.data();
            rn = read.size();
            qn = qual.size();
        }
        if (read_len < 0 || read_len > L || rn < (size_t)read_len || qn < (size_t)read_len) {
            if (c->bad.empty()) c->bad = "alignment longer than -L or than its sequence field";
            continue;
        }
        /* the previous line's name first (lines of one chromosome follow
         * each other), then the chunk's table of names */
        size_t cid = last_cid;
        if (cid >= c->chr.size() || c->chr[cid].size() != tl[7] || memcmp(c->chr[cid].data(), tok[7], tl[7])) {
            std::string name(tok[7], tl[7]);
            auto it = c->chr_id.find(name);
            if (it != c->chr_id.end()) {
                cid = it->second;
            } else {
                cid = c->chr.size();
                if (cid > 0xffff) {   /* ids are 16-bit; one chromosome per run is the contract anyway */
                    if (c->bad.empty()) c->bad = "more than 65536 chromosome names";
                    continue;
                }
                c->chr_id.emplace(name, (uint32_t)cid);
                c->chr.push_back(std::move(name));
            }
            last_cid = cid;
        }
        const size_t k = c->first + c->kept++;
        out->chr_id[k] = (uint16_t)cid;
        out->pos[k] = position - 1;
        out->len[k] = read_len;
        out->hit[k] = hit;
        out->strand[k] = (uint8_t)tok[6][0];
        uint8_t* sp = out->seq.data() + k * (size_t)L;
        uint8_t* qp = out->qual.data() + k * (size_t)L;
        memcpy(sp, rs, (size_t)read_len);
        memset(sp + read_len, 'A', (size_t)(L - read_len));
        memcpy(qp, qs, (size_t)read_len);
        memset(qp + read_len, 0, (size_t)(L - read_len));
    }
}

/* Parse a SOAP file on the host threads straight into the output
 * arrays: the lines of each thread's share are counted first, so that each
 * share has its rows before it is parsed.  Only lines that do not parse
 * leave gaps, closed afterwards. */
void load_soap(const std::string& path, int L, Reads* out) {
    const int fd = open(path.c_str(), O_RDONLY);
    if (fd < 0) die("No such file or directory:" + path, 1);
    struct stat st;
    fstat(fd, &st);
    const size_t size = (size_t)st.st_size;
    if (size == 0) {
        close(fd);
        return;
    }
    const char* data = (const char*)mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);
    if (data == MAP_FAILED) die("cannot map " + path);
    /* GSNP_HOST_THREADS, else every hardware thread (at most 64), as the
     * library's host passes */
    const char* env = getenv("GSNP_HOST_THREADS");
    int want = env ? atoi(env) : 0;
    if (want <= 0) want = (int)std::thread::hardware_concurrency();
    const unsigned nt = (unsigned)std::max(1, std::min(want, 64));
    std::vector<Chunk> ch(nt);
    const char* prev = data;
    for (unsigned t = 0; t < nt; ++t) {
        ch[t].begin = prev;
        const char* c = t + 1 == nt ? data + size : data + size * (t + 1) / nt;
        if (c < prev) c = prev;
        if (t + 1 < nt) {
            const char* nl = (const char*)memchr(c, '\n', (size_t)(data + size - c));
            c = nl ? nl + 1 : data + size;
        }
        ch[t].end = prev = c;
    }
    auto on_threads = [&](auto&& f) {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t) th.emplace_back(f, t);
        for (auto& x : th) x.join();
    };
    on_threads([&](unsigned t) { ch[t].lines = count_lines(ch[t].begin, ch[t].end); });
    size_t rows = 0;
    for (Chunk& c : ch) {
        c.first = rows;
        rows += c.lines;
    }
    out->pos.allocate(rows);
    out->len.allocate(rows);
    out->hit.allocate(rows);
    out->strand.allocate(rows);
    out->chr_id.allocate(rows);
    out->seq.allocate(rows * (size_t)L);
    out->qual.allocate(rows * (size_t)L);
    on_threads([&](unsigned t) { parse_chunk(&ch[t], L, out); });
    munmap((void*)data, size);
    close(fd);
    /* chromosome ids of each share to the file's list of names */
    std::vector<std::vector<uint16_t>> remap(nt);
    std::unordered_map<std::string, size_t> file_id;
    for (unsigned t = 0; t < nt; ++t) {
        if (out->bad.empty() && !ch[t].bad.empty()) out->bad = ch[t].bad;
        for (const std::string& name : ch[t].chr) {
            auto it = file_id.find(name);
            size_t k;
            if (it != file_id.end()) {
                k = it->second;
            } else {
                k = out->chr.size();
                file_id.emplace(name, k);
                out->chr.push_back(name);
            }
            if (k > 0xffff && out->bad.empty()) out->bad = "more than 65536 chromosome names";
            remap[t].push_back((uint16_t)k);
        }
    }
    on_threads([&](unsigned t) {
        for (size_t i = ch[t].first; i < ch[t].first + ch[t].kept; ++i) out->chr_id[i] = remap[t][out->chr_id[i]];
    });
    /* close the gaps of skipped lines, share by share in file order (a
     * share's rows only move down) */
    size_t n = 0;
    for (const Chunk& c : ch) {
        if (n != c.first && c.kept > 0) {
            memmove(&out->pos[n], &out->pos[c.first], c.kept * sizeof(int32_t));
            memmove(&out->len[n], &out->len[c.first], c.kept * sizeof(int32_t));
            memmove(&out->hit[n], &out->hit[c.first], c.kept * sizeof(int32_t));
            memmove(&out->strand[n], &out->strand[c.first], c.kept);
            memmove(&out->chr_id[n], &out->chr_id[c.first], c.kept * sizeof(uint16_t));
            memmove(out->seq.data() + n * (size_t)L, out->seq.data() + c.first * (size_t)L, c.kept * (size_t)L);
            memmove(out->qual.data() + n * (size_t)L, out->qual.data() + c.first * (size_t)L, c.kept * (size_t)L);
        }
        n += c.kept;
    }
    out->n = n;
}

/* ---- calibration matrix files (cpp/matrix.cc:215-241) ---- */

void write_matrix(const std::string& path, const gsnp_params& p, const double* pm) {
    FILE* f = fopen(path.c_str(), "w");
    if (!f) die("Cannot creat file :" + path, 1);
    for (int q = p.q_min; q <= p.q_max; ++q)
        for (unsigned long coord = 0; coord != p.read_length; ++coord) {
            fprintf(f, "%llu\t%lu", (unsigned long long)(long long)q - (unsigned long long)(long long)p.q_min, coord);
            for (int t = 0; t != 16; ++t)
                fprintf(f, "\t%.16e", pm[((unsigned long long)(q - p.q_min) << 12) | (coord << 4) | (unsigned)t]);
            fprintf(f, "\n");
        }
    fclose(f);
}

void read_matrix(const std::string& path, double* pm) {
    std::ifstream in(path);
    if (!in) die("No such file or directory:" + path, 1);
    for (std::string line; std::getline(in, line);) {
        std::istringstream s(line);
        int q = 0;
        std::string::size_type coord = 0;
        s >> q >> coord;
        for (int t = 0; t != 16; ++t) s >> pm[((unsigned long long)q << 12) | (coord << 4) | (unsigned)t];
    }
}

void check(gsnp_context* ctx, int rc, const char* what) {
    if (rc == GSNP_OK) return;
    const std::string msg = gsnp_context_error(ctx);
    if (rc == GSNP_ERR_UNSORTED) die(msg, 255);
    if (rc == GSNP_ERR_INPUT && msg.find("unknown base") != std::string::npos) {
        printf("!!!ERROR@encode: unknown base when encoding.\n");
        exit(EXIT_FAILURE);
    }
    die(std::string(what) + ": " + msg);
}

}  // namespace

int main(int argc, char** argv) {
    Options o;
    parse_args(argc, argv, &o);
    gsnp_params& p = o.p;

    std::ofstream cns(o.out.c_str());
    if (!cns) die("Cannot creat file:" + o.out, 1);
    std::map<std::string, Chromosome> chrs;
    load_fasta(o.fasta, &chrs);
    if (!o.dbsnp.empty()) load_dbsnp(o.dbsnp, &chrs);

    Reads reads;
    load_soap(o.soap, p.read_length, &reads);
    if (!reads.bad.empty()) die("!!!ERROR: " + reads.bad);
    if (reads.n == 0) die("!!!ERROR: no usable alignment.");
    const uint16_t last_chr = reads.chr_id[reads.n - 1];
    const std::string chr_name = reads.chr[last_chr];
    auto it = chrs.find(chr_name);
    if (it == chrs.end()) die("Assertion Failed: Chromosome: !" + chr_name + "! NOT found", 255);
    for (size_t i = 0; i < reads.n; ++i)
        if (reads.chr_id[i] != last_chr && reads.pos[i] >= 0)
            die("!!!ERROR: alignments on more than one chromosome (" + reads.chr[reads.chr_id[i]] + ", " + chr_name +
                "); call one chromosome per run");
    Chromosome& chr = it->second;

    gsnp_context* ctx = nullptr;
    if (gsnp_context_create(0, &ctx) != GSNP_OK) die("!!!ERROR: no CUDA device");
    std::vector<gsnp_snp> snp;
    snp.assign(chr.snp.begin(), chr.snp.end());
    check(ctx, gsnp_load_reference(ctx, chr.codes.data(), (int64_t)chr.codes.size(), snp.data(), (int64_t)snp.size()),
          "reference");

    const int64_t n = (int64_t)reads.n;
    gsnp_reads r{};
    r.n = n;
    r.pos = reads.pos.data();
    r.len = reads.len.data();
    r.hit = reads.hit.data();
    r.strand = reads.strand.data();
    r.seq = reads.seq.data();
    r.qual = reads.qual.data();
    r.pitch = p.read_length;

    std::vector<double> pm(256UL * 256UL * 16UL, 1.0), prior(128), rank(64UL * 64UL * 2048UL);
    if (o.matrix_in.empty()) {
        check(ctx, gsnp_calibrate(ctx, &p, &r, pm.data()), "calibration");
        if (!o.matrix_out.empty()) write_matrix(o.matrix_out, p, pm.data());
    } else {
        read_matrix(o.matrix_in, pm.data());
    }
    gsnp_prior_table(&p, prior.data());
    gsnp_rank_table(rank.data());
    check(ctx, gsnp_load_tables(ctx, &p, pm.data(), prior.data(), rank.data()), "tables");
    check(ctx, gsnp_call_chromosome(ctx, &r), "calling");

    cns.close();
    if (o.compress) {
        check(ctx, gsnp_write_columns(ctx, chr_name.c_str(), o.out.c_str()), "-C output");
    } else {
        check(ctx, gsnp_write_cns(ctx, chr_name.c_str(), o.out.c_str()), "cns text");
        check(ctx, gsnp_write_columns(ctx, nullptr, o.out.c_str()), "column files");
    }
    gsnp_context_destroy(ctx);
    return 0;
}
