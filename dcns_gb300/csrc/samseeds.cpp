// x-seeds of cut2Gaps2 from SAM records (samFileToSeeds, impl/samFileToSeeds.cpp:19-141).  Host code.
//
// A record line (not '@', at least 9 characters) is read with the same patterns: the first six whitespace-separated
// fields "query flag reference position mapq cigar" (the CIGAR field as a run of word characters), and it is used only
// when the CIGAR starts with a clip whose length is the query start.  M advances both ends, D and N the reference,
// I the query.  Then, 0-based and inclusive, each coordinate is moved onto the sequence with its lower-case 'n' runs
// removed: minus the 'n' before the start, and the end also minus the 'n' inside the seed.  Flag 0 seeds are on the
// + strand of the query; any other flag counts the query's 'n' inside and after the seed and mirrors the seed onto
// the reverse strand (the mirrored start equals the original start, as in the reference, whose second assignment
// reads the already-mirrored end).
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <regex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/dcns_gb300.h"

namespace {

int32_t n_in(const std::string *t, int64_t lo, int64_t hi) {  // 'n' in t[lo .. hi]
  if (!t) return 0;
  int32_t c = 0;
  for (int64_t i = std::max<int64_t>(lo, 0); i <= hi && i < (int64_t)t->size(); ++i) c += (*t)[i] == 'n';
  return c;
}

}  // namespace

extern "C" int dcns_sam_to_seeds(const char *sam, int64_t sam_len, int n_ref, const char *const *ref_names,
                                 const char *const *ref_texts, const int64_t *ref_lens, int n_qry,
                                 const char *const *qry_names, const char *const *qry_texts, const int64_t *qry_lens,
                                 int32_t **seeds, int64_t *n_seeds) {
  if ((sam_len > 0 && !sam) || sam_len < 0 || n_ref < 0 || n_qry < 0 || !seeds || !n_seeds) return DCNS_ERR_INVALID;
  if ((n_ref > 0 && (!ref_names || !ref_texts || !ref_lens)) || (n_qry > 0 && (!qry_names || !qry_texts || !qry_lens)))
    return DCNS_ERR_INVALID;
  *seeds = nullptr;
  *n_seeds = 0;
  try {
    std::vector<std::string> rt(n_ref), qt(n_qry);
    std::unordered_map<std::string, int> ri, qi;
    for (int k = 0; k < n_ref; ++k) {
      rt[k].assign(ref_texts[k], (size_t)ref_lens[k]);
      ri.emplace(ref_names[k], k);
    }
    for (int k = 0; k < n_qry; ++k) {
      qt[k].assign(qry_texts[k], (size_t)qry_lens[k]);
      qi.emplace(qry_names[k], k);
    }
    const std::regex rec("^(.*?)\\s+(\\d+)\\s+(\\S+)\\s+(\\d+)\\s+(\\d+)\\s+(\\w+)");
    const std::regex op("(\\d+)([MIDNSH])");
    const std::regex clip("^(\\d+)([SH])");
    std::vector<int32_t> out;
    const std::string text(sam ? sam : "", (size_t)sam_len);
    size_t pos = 0;
    while (pos < text.size()) {
      size_t eol = text.find('\n', pos);
      if (eol == std::string::npos) eol = text.size();
      const std::string line = text.substr(pos, eol - pos);
      pos = eol + 1;
      if (line.empty() || line[0] == '@' || line.size() < 9) continue;
      std::smatch m;
      if (!std::regex_search(line, m, rec)) continue;
      std::string cig = m[6];
      std::smatch c1;
      if (!std::regex_search(cig, c1, clip)) continue;
      const std::string rname = m[3], qname = m[1];
      int64_t r0 = std::stoll(m[4].str()), q0 = std::stoll(c1[1].str());
      int64_t r1 = r0, q1 = q0;
      std::smatch c;
      while (std::regex_search(cig, c, op)) {
        const char t = c[2].str()[0];
        const int64_t len = std::stoll(c[1].str());
        if (t == 'M')
          r1 += len, q1 += len;
        else if (t == 'D' || t == 'N')
          r1 += len;
        else if (t == 'I')
          q1 += len;
        cig = c.suffix().str();
      }
      const int64_t flag = std::stoll(m[2].str());
      r0 -= 1, r1 -= 2, q0 -= 1, q1 -= 2;
      const auto rit = ri.find(rname), qit = qi.find(qname);
      const std::string *R = rit == ri.end() ? nullptr : &rt[rit->second];
      const std::string *Q = qit == qi.end() ? nullptr : &qt[qit->second];
      const int32_t rn1 = n_in(R, 0, r0 - 1), rn2 = n_in(R, r0, r1);
      r0 -= rn1;
      r1 -= rn1 + rn2;
      int strand = 0;
      if (flag == 0) {
        const int32_t qn1 = n_in(Q, 0, q0 - 1), qn2 = n_in(Q, q0, q1);
        q0 -= qn1;
        q1 -= qn1 + qn2;
      } else {
        strand = 1;
        const int64_t L = Q ? (int64_t)Q->size() : 0;
        const int32_t qn1 = n_in(Q, q0, q1), qn2 = n_in(Q, q1 + 1, L - 1);
        q1 = L - 1 - q0;
        q0 = L - 1 - q1;
        q0 -= qn2;
        q1 -= qn2 + qn1;
      }
      const int32_t rec7[7] = {rit == ri.end() ? -1 : rit->second, qit == qi.end() ? -1 : qit->second, strand,
                               (int32_t)r0, (int32_t)r1, (int32_t)q0, (int32_t)q1};
      out.insert(out.end(), rec7, rec7 + 7);
    }
    int32_t *buf = static_cast<int32_t *>(std::malloc(sizeof(int32_t) * std::max<size_t>(out.size(), 1)));
    if (!buf) return DCNS_ERR_NOMEM;
    if (!out.empty()) std::memcpy(buf, out.data(), sizeof(int32_t) * out.size());
    *seeds = buf;
    *n_seeds = (int64_t)out.size() / 7;
    return DCNS_OK;
  } catch (const std::exception &) {
    return DCNS_ERR_INVALID;
  }
}

extern "C" void dcns_free_seeds(int32_t *seeds) { std::free(seeds); }
