// SAM and "o" records of one reference/query pair, as the cut1Gap driver writes them (outputMasking,
// controlLayer4.cpp:835-1358): coordinates and CIGARs are mapped back onto the region texts that still hold the
// lower-case 'n' runs the driver deleted before aligning (controlLayer4.cpp:1387,1406).  Host code; no device work.
//
// Per fragment (1-based coordinates on the n-free sequences):
//   * the c-th non-'n' character of a region text sits at index j, with k 'n' before it; the reference scans the text
//     once per coordinate and applies j and k per strand combination (below);
//   * every CIGAR unit walks both texts: an M first passes the 'n' of the reference text (emitted as op 3, printed
//     'D') and of the query text (op 6, printed 'I'), an I passes the query's, a D the reference's; consecutive units
//     of the same op code merge, so a masked run never merges with a real gap of the same letter;
//   * the CIGAR is printed forward when the reference region is on the + strand and reversed otherwise; the read
//     column is the query region text between the fragment's ends, reverse-complemented (upper-case IUPAC only)
//     when the reference region is on the - strand.
// The "o" text is a "#ref:strand:start-query:strand:start" header and one "start1 end1 start2 end2 score p" line per
// fragment (p in the default iostream format).
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/dcns_gb300.h"

namespace {

struct Hit {
  bool found = false;
  int64_t j = 0;  // index in the region text
  int64_t n = 0;  // 'n' characters in text[0 .. j]
};

// The c-th (1-based) character of `t` that is not 'n'.
Hit locate(const std::string &t, int64_t c) {
  Hit h;
  int64_t chr = 0, nn = 0;
  for (int64_t j = 0; j < (int64_t)t.size(); ++j) {
    if (t[j] == 'n')
      ++nn;
    else
      ++chr;
    if (chr == c) {
      h.found = true, h.j = j, h.n = nn;
      return h;
    }
  }
  return h;
}

char at(const std::string &t, int64_t i) { return i >= 0 && i < (int64_t)t.size() ? t[i] : '\0'; }

void push_op(std::vector<uint32_t> &cg, uint32_t op) {
  if (!cg.empty() && (cg.back() & 0xFu) == op)
    cg.back() += 1u << 4;
  else
    cg.push_back((1u << 4) | op);
}

// getSubSequence(text, start, end) with its clamping, 1-based inclusive.
std::string sub_text(const std::string &t, int64_t s, int64_t e) {
  if (s > e) std::swap(s, e);
  if (s < 1) s = 1;
  const int64_t n = (int64_t)t.size();
  if (n == 0) return std::string();
  if (s > n)
    s = e = n;
  else if (e > n)
    e = n;
  return t.substr((size_t)(s - 1), (size_t)(e - s + 1));
}

char complement(char c) {
  switch (c) {
    case 'A': return 'T';
    case 'T': return 'A';
    case 'U': return 'A';
    case 'C': return 'G';
    case 'G': return 'C';
    case 'R': return 'Y';
    case 'Y': return 'R';
    case 'K': return 'M';
    case 'M': return 'K';
    case 'B': return 'V';
    case 'V': return 'B';
    case 'D': return 'H';
    case 'H': return 'D';
    default: return c;
  }
}

char *to_c(const std::string &s, int64_t *len) {
  char *p = static_cast<char *>(std::malloc(s.size() + 1));
  if (!p) return nullptr;
  std::memcpy(p, s.data(), s.size());
  p[s.size()] = '\0';
  if (len) *len = (int64_t)s.size();
  return p;
}

int format_records(int64_t n_frag, const int64_t *frag, const uint32_t *cigar, const double *pvalue,
                   const char *ref_text, int64_t ref_len, const char *qry_text, int64_t qry_len, int ref_strand,
                   int qry_strand, int32_t ref_start, int32_t qry_start, const char *ref_chr, const char *qry_chr,
                   char **sam, int64_t *sam_len, char **o, int64_t *o_len) {
  const std::string R(ref_text ? ref_text : "", (size_t)ref_len), Q(qry_text ? qry_text : "", (size_t)qry_len);
  std::ostringstream so, oo;
  oo << "#" << ref_chr << ":" << ref_strand << ":" << ref_start << "-" << qry_chr << ":" << qry_strand << ":"
     << qry_start << "\n";
  for (int64_t f = 0; f < n_frag; ++f) {
    const int64_t *fr = frag + 7 * f;
    const uint32_t s1 = (uint32_t)fr[0], e1 = (uint32_t)fr[1], s2 = (uint32_t)fr[2], e2 = (uint32_t)fr[3];
    const uint32_t score = (uint32_t)fr[4];
    const uint32_t *cg = cigar ? cigar + fr[5] : nullptr;
    const int64_t ncg = fr[6];
    if (ncg > 0 && !cg) return DCNS_ERR_INVALID;
    const Hit qs = locate(Q, s2), qe = locate(Q, e2), rs = locate(R, s1), re = locate(R, e1);
    // positions (int32 arithmetic of the reference) and the query span in the region text
    int32_t que_pos = qry_strand == 1 ? (int32_t)(qry_start + s2 - 1) : (int32_t)(qry_start + (int64_t)Q.size() - e2);
    int32_t ref_pos = ref_strand == 1 ? (int32_t)(ref_start + s1 - 1) : (int32_t)(ref_start + (int64_t)R.size() - e1);
    if (qry_strand == 1 && qs.found) que_pos += (int32_t)qs.n;
    if (qry_strand == 0 && qe.found) que_pos -= (int32_t)qe.n;
    if (ref_strand == 1 && rs.found) ref_pos += (int32_t)rs.n;
    if (ref_strand == 0 && re.found) ref_pos -= (int32_t)re.n;
    const int64_t start = 1 + (qs.found ? qs.j : 0), end = 1 + (qe.found ? qe.j : 0);
    const int64_t ref_start_i = 1 + (rs.found ? rs.j : 0);
    const int flag = ref_strand == qry_strand ? 0 : 16;
    so << qry_chr << "\t" << flag << "\t" << ref_chr << "\t" << ref_pos << "\t" << score << "\t" << que_pos << "H";
    // CIGAR over the region texts
    std::vector<uint32_t> out;
    int64_t ri = ref_start_i - 1, qi = start - 1;
    for (int64_t k = 0; k < ncg; ++k) {
      const uint32_t op = cg[k] & 0xFu, len = cg[k] >> 4;
      for (uint32_t u = 0; u < len; ++u) {
        if (op == 0) {
          while (at(R, ri) == 'n') push_op(out, 3), ++ri;
          while (at(Q, qi) == 'n') push_op(out, 6), ++qi;
          ++ri, ++qi;
        } else if (op == 1) {
          while (at(Q, qi) == 'n') push_op(out, 6), ++qi;
          ++qi;
        } else {
          while (at(R, ri) == 'n') push_op(out, 3), ++ri;
          ++ri;
        }
        push_op(out, op);
      }
    }
    static const char kOps[] = "MIDDSHI=XB";
    if (ref_strand == 1) {
      for (uint32_t c : out) so << (c >> 4) << kOps[c & 0xFu];
    } else {
      for (size_t k = out.size(); k-- > 0;) so << (out[k] >> 4) << kOps[out[k] & 0xFu];
    }
    std::string read = sub_text(Q, start, end);
    if (ref_strand == 0) {
      std::string rc(read.rbegin(), read.rend());
      for (char &c : rc) c = complement(c);
      read.swap(rc);
    }
    so << "\t*\t0\t0\t" << read << "\t*\n";
    oo << s1 << " " << e1 << " " << s2 << " " << e2 << " " << score << " " << pvalue[f] << "\n";
  }
  *sam = to_c(so.str(), sam_len);
  *o = to_c(oo.str(), o_len);
  if (!*sam || !*o) {
    std::free(*sam);
    std::free(*o);
    *sam = *o = nullptr;
    return DCNS_ERR_NOMEM;
  }
  return DCNS_OK;
}

}  // namespace

extern "C" int dcns_format_records(int64_t n_frag, const int64_t *frag, const uint32_t *cigar, const double *pvalue,
                                   const char *ref_text, int64_t ref_len, const char *qry_text, int64_t qry_len,
                                   int ref_strand, int qry_strand, int32_t ref_start, int32_t qry_start,
                                   const char *ref_chr, const char *qry_chr, char **sam, int64_t *sam_len, char **o,
                                   int64_t *o_len) {
  if (n_frag < 0 || (n_frag > 0 && (!frag || !pvalue)) || !ref_chr || !qry_chr || !sam || !o) return DCNS_ERR_INVALID;
  if ((ref_len > 0 && !ref_text) || (qry_len > 0 && !qry_text) || ref_len < 0 || qry_len < 0) return DCNS_ERR_INVALID;
  if ((ref_strand != 0 && ref_strand != 1) || (qry_strand != 0 && qry_strand != 1)) return DCNS_ERR_INVALID;
  *sam = *o = nullptr;
  try {  // host allocation failures become a status, not an exception through the C ABI
    return format_records(n_frag, frag, cigar, pvalue, ref_text, ref_len, qry_text, qry_len, ref_strand, qry_strand,
                          ref_start, qry_start, ref_chr, qry_chr, sam, sam_len, o, o_len);
  } catch (const std::exception &) {
    std::free(*sam);
    std::free(*o);
    *sam = *o = nullptr;
    return DCNS_ERR_NOMEM;
  }
}

extern "C" void dcns_free_text(char *text) { std::free(text); }
