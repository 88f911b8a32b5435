/*
 * decompress.h - reader of the -C compressed output (decompress.cpp).
 */
#ifndef GSNP_DECOMPRESS_H
#define GSNP_DECOMPRESS_H

#include <string>

namespace gsnp {

/* The cns rows of the six files <base>.1_2 ... <base>.15_17, written to
 * out_path as the reference's decompressor prints them, on `threads` host
 * threads (<= 0: every hardware thread, at most 32).  Returns 0, or 1 with
 * *err set. */
int decompress_columns(const std::string& base, const std::string& out_path, int threads, std::string* err);

/* The reference decompressor's check: every row of the cns text at cns_path
 * against the decompressed columns, characters and integers exactly, the two
 * doubles within 1e-5.  Returns 0 (all rows match), 2 (*report names the
 * first difference) or 1 (*err: unreadable input). */
int check_columns(const std::string& cns_path, const std::string& base, std::string* report, std::string* err);

}  // namespace gsnp

#endif
