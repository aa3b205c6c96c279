// Test infrastructure only (parity checker, never shipped): a C entry point to the reference's own outputMasking
// (controlLayer4.cpp:835-1358), so the SAM and "o" text of the library's record formatter can be compared byte for
// byte with what the reference writes for the same fragments and region texts.  Built by build_ref.sh from the
// unmodified reference sources into oracle/_ref/libdcns_ref_cli.so.
#include <cstdint>
#include <string>
#include <vector>

#include <cstdio>
#include <iostream>
#include <fstream>
#include <map>

#include "impl/samFileToSeeds.h"
#include "model/PairedSimilarFragment.h"

// defined in controlLayer4.cpp (no header declares it)
void outputMasking(std::string _output, std::vector<PairedSimilarFragment> &pairedSimilarFragments0, int32_t refStrand,
                   int32_t queStrand, int32_t refStart, int32_t queStart, std::string refChr, std::string queChr,
                   std::string &seq1_string, std::string &seq2_string, std::string &seq1_0_string,
                   std::string &seq2_0_string);

static std::string without_n(const std::string &t) {
  std::string s;
  for (char c : t)
    if (c != 'n') s.push_back(c);
  return s;
}

extern "C" int ref_output_masking(const char *prefix, int64_t n_frag, const int64_t *frag, const uint32_t *cigar,
                                  const double *pvalue, const double *evalue, int ref_strand, int qry_strand,
                                  int32_t ref_start, int32_t qry_start, const char *ref_chr, const char *qry_chr,
                                  const char *ref_text, int64_t ref_len, const char *qry_text, int64_t qry_len) {
  std::vector<PairedSimilarFragment> frs;
  for (int64_t k = 0; k < n_frag; ++k) {
    const int64_t *f = frag + 7 * k;
    std::vector<uint32_t> cg(cigar + f[5], cigar + f[5] + f[6]);
    double p = pvalue[k], e = evalue[k];
    frs.emplace_back((uint32_t)f[0], (uint32_t)f[1], (uint32_t)f[2], (uint32_t)f[3], (uint32_t)f[4], cg, p, e);
  }
  std::string t1(ref_text, (size_t)ref_len), t2(qry_text, (size_t)qry_len);
  std::string s1 = without_n(t1), s2 = without_n(t2);
  outputMasking(prefix, frs, ref_strand, qry_strand, ref_start, qry_start, ref_chr, qry_chr, s1, s2, t1, t2);
  return 0;
}

// samFileToSeeds (impl/samFileToSeeds.cpp:19): reads the SAM file at sam_path; genomes by name.  Writes records of
// 7 int32 (strand 0 positive / 1 negative, reference index, query index, start1, end1, start2, end2) in the order of
// the reference's maps (strand, then reference name, then query name, then insertion); returns the count, or -1
// when cap is too small.
extern "C" int ref_sam_to_seeds(const char *sam_path, int n_ref, const char *const *ref_names,
                                const char *const *ref_texts, int n_qry, const char *const *qry_names,
                                const char *const *qry_texts, int32_t *out, int cap) {
  std::map<std::string, std::map<std::string, std::vector<Seed>>> pos, neg;
  std::map<std::string, std::string> rg, qg;
  std::map<std::string, int> ri, qi;
  for (int k = 0; k < n_ref; ++k) rg[ref_names[k]] = ref_texts[k], ri[ref_names[k]] = k;
  for (int k = 0; k < n_qry; ++k) qg[qry_names[k]] = qry_texts[k], qi[qry_names[k]] = k;
  std::string path(sam_path);
  {
    std::streambuf *old = std::cout.rdbuf(nullptr);  // the reader prints progress to stdout
    samFileToSeeds(path, pos, neg, rg, qg);
    std::cout.rdbuf(old);
  }
  int n = 0;
  for (int strand = 0; strand < 2; ++strand)
    for (auto &a : strand ? neg : pos)
      for (auto &b : a.second)
        for (Seed &sd : b.second) {
          if (n >= cap) return -1;
          int32_t *r = out + 7 * n++;
          r[0] = strand;
          r[1] = ri.count(a.first) ? ri[a.first] : -1;
          r[2] = qi.count(b.first) ? qi[b.first] : -1;
          r[3] = sd.getStart1(), r[4] = sd.getEnd1(), r[5] = sd.getStart2(), r[6] = sd.getEnd2();
        }
  return n;
}
