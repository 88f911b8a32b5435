/*
 * columns.h - the -C compressed output writer (columns.cpp).
 */
#ifndef GSNP_COLUMNS_H
#define GSNP_COLUMNS_H

#include <stdint.h>

#include <string>

#include "gsnp_device.cuh"
#include "plan.h"

namespace gsnp {

/* Dictionary codec (cuda_dictCompression's contract): dict = the distinct
 * input values ascending, words = their indices packed MSB-first.  *n_words
 * and *n_dict hold capacities on entry and counts on return. */
class DictCodec {
public:
    virtual ~DictCodec() {}
    virtual bool compress(const int* in, size_t n, uint32_t* words, unsigned long* n_words, int* dict,
                          unsigned long* n_dict, std::string* err) const = 0;
    virtual bool compress(const uint32_t* in, size_t n, uint32_t* words, unsigned long* n_words, uint32_t* dict,
                          unsigned long* n_dict, std::string* err) const = 0;
    virtual bool compress(const double* in, size_t n, uint32_t* words, unsigned long* n_words, double* dict,
                          unsigned long* n_dict, std::string* err) const = 0;
};

/* The codec on the host, safe to call from several threads at once. */
class HostDictCodec : public DictCodec {
public:
    bool compress(const int* in, size_t n, uint32_t* words, unsigned long* n_words, int* dict, unsigned long* n_dict,
                  std::string* err) const override;
    bool compress(const uint32_t* in, size_t n, uint32_t* words, unsigned long* n_words, uint32_t* dict,
                  unsigned long* n_dict, std::string* err) const override;
    bool compress(const double* in, size_t n, uint32_t* words, unsigned long* n_words, double* dict,
                  unsigned long* n_dict, std::string* err) const override;
};

/* Write the six -C files <base>.1_2 ... <base>.15_17 for every called window
 * of the plan, windows encoded on `threads` host threads (dict must be safe
 * to call from that many at once).  With calls == NULL only the empty files
 * of a text-mode run are written (the reference creates them in both
 * modes).  Returns 0 or 1 with *err set. */
int write_columns(const WindowPlan& plan, const uint8_t* codes, const SiteCall* calls, const SiteCounts* counts,
                  const char* chr_name, const std::string& base, const DictCodec& dict, int threads,
                  std::string* err);

}  // namespace gsnp

#endif
