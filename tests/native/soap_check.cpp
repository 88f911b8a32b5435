/*
 * soap_check.cpp - the `gsnp` command's SOAP loader (load_soap in
 * gsnp_gb300/csrc/cli.cpp, compiled into this program) on one file: prints
 * the alignments it keeps, one per line, as
 *   pos len hit strand chr seq qual
 * (seq and qual cut to len, qual as decimal byte values), then
 *   padding ok|bad
 * for the row bytes past each read length ('A' and 0), and
 *   bad <first error, or nothing>
 * Usage: soap_check <file> <L>
 */
#define main gsnp_cli_main
#include "cli.cpp"
#undef main

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    const int L = atoi(argv[2]);
    Reads r;
    load_soap(argv[1], L, &r);
    bool pad_ok = true;
    for (size_t i = 0; i < r.n; ++i) {
        const uint8_t* s = r.seq.data() + i * (size_t)L;
        const uint8_t* q = r.qual.data() + i * (size_t)L;
        printf("%d %d %d %c %s ", r.pos[i], r.len[i], r.hit[i], (char)r.strand[i], r.chr[r.chr_id[i]].c_str());
        fwrite(s, 1, (size_t)r.len[i], stdout);
        for (int k = 0; k < r.len[i]; ++k) printf("%c%d", k ? ',' : ' ', (int)q[k]);
        printf("\n");
        for (int k = r.len[i]; k < L; ++k)
            if (s[k] != 'A' || q[k] != 0) pad_ok = false;
    }
    printf("padding %s\n", pad_ok ? "ok" : "bad");
    printf("bad %s\n", r.bad.c_str());
    return 0;
}
