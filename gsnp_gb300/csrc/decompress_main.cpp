/*
 * decompress_main.cpp - the gsnp_decompress command: the reference's -C
 * decompressor tool (cpp/decompression.cpp:130-137,404-408) over the C ABI.
 *
 *   gsnp_decompress <compressed base> <output file>
 *       the cns rows of the six -C files, as the reference's tool prints them;
 *   gsnp_decompress --check <cns text> <compressed base>
 *       its check mode: every row of the cns text against the -C files.
 */
#include <stdio.h>
#include <string.h>

#include "gsnp_gb300.h"

int main(int argc, char** argv) {
    if (argc == 4 && strcmp(argv[1], "--check") == 0) {
        char report[512];
        const int rc = gsnp_check_columns(argv[2], argv[3], report, sizeof(report));
        printf("%s\n", report);
        return rc == GSNP_OK ? 0 : 1;
    }
    if (argc != 3) {
        printf("Two parameters:\n");
        printf("1. the input compressed file.\n");
        printf("2. the output file name.\n");
        printf("(or: --check <cns text> <compressed file>)\n");
        return 1;
    }
    char err[512];
    if (gsnp_decompress_columns(argv[1], argv[2], 0, err, sizeof(err)) != GSNP_OK) {
        fprintf(stderr, "gsnp_decompress: %s\n", err);
        return 1;
    }
    return 0;
}
