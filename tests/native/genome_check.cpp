/*
 * genome_check.cpp - the reference sequence and known-SNP file as a loader
 * leaves them, printed for comparison.  Built twice:
 *   -DGENOME_ORACLE  load_genome of the oracle's restated driver
 *                    (oracle/driver.cpp, cpp/chromosome.cc:172-221);
 *   otherwise        load_fasta and load_dbsnp of the `gsnp` command
 *                    (gsnp_gb300/csrc/cli.cpp).
 * Output, chromosomes by name:
 *   chr <name> <length>
 *   <one hex digit per base: the 4-bit site code, bit 3 = known SNP>
 *   snp <pos> <validated> <hapmap> <indel> <fA> <fC> <fT> <fG>   (by position)
 * Usage: genome_check <fasta> <dbsnp>
 */
#include <stdio.h>

#include <fstream>
#include <string>

#ifdef GENOME_ORACLE
#include "driver.cpp"

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    std::ifstream fasta(argv[1]), snp(argv[2]);
    Genome g;
    load_genome(fasta, &snp, &g);
    for (const auto& kv : g.chr) {
        const Chromosome& c = kv.second;
        printf("chr %s %u\n", kv.first.c_str(), c.len);
        for (unsigned long long i = 0; i < c.len; ++i) putchar("0123456789abcdef"[c.base(i)]);
        putchar('\n');
        for (const auto& s : c.dbsnp)
            printf("snp %llu %d %d %d %.17g %.17g %.17g %.17g\n", s.first, (int)s.second.validated,
                   (int)s.second.hapmap, (int)s.second.indel, s.second.freq[0], s.second.freq[1], s.second.freq[2],
                   s.second.freq[3]);
    }
    return 0;
}
#else
#define main gsnp_cli_main
#include "cli.cpp"
#undef main

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    std::map<std::string, Chromosome> chrs;
    load_fasta(argv[1], &chrs);
    load_dbsnp(argv[2], &chrs);
    for (const auto& kv : chrs) {
        const Chromosome& c = kv.second;
        printf("chr %s %u\n", kv.first.c_str(), (unsigned)c.codes.size());
        for (uint8_t x : c.codes) putchar("0123456789abcdef"[x & 15]);
        putchar('\n');
        for (const gsnp_snp& s : c.snp)
            printf("snp %llu %d %d %d %.17g %.17g %.17g %.17g\n", (unsigned long long)s.pos, (int)s.validated,
                   (int)s.hapmap, (int)s.indel, s.freq[0], s.freq[1], s.freq[2], s.freq[3]);
    }
    return 0;
}
#endif
