// Test infrastructure only (parity checker, never shipped): a C entry point to the reference's own outputMasking
// (controlLayer4.cpp:835-1358), so the SAM and "o" text of the library's record formatter can be compared byte for
// byte with what the reference writes for the same fragments and region texts.  Built by build_ref.sh from the
// unmodified reference sources into oracle/_ref/libdcns_ref_cli.so.
#include <cstdint>
#include <string>
#include <vector>

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
