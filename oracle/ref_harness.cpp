// Test infrastructure only: a C-callable harness around the UNMODIFIED dCNS
// reference sources, compiled from the reference checkout by
// oracle/build_ref.sh into oracle/_ref/libdcns_ref.so.  It is the checker that
// pins the oracle restatement (oracle/dcns_oracle.cpp) and generates the golden
// fixtures under tests/golden/.  Nothing in the product links or loads it.
//
// Every entry point forwards to the reference function named in its comment;
// the only work done here is argument marshalling (building the Scorei table,
// the reverse complements, and flattening std::vector results).

#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "impl/findSimilarFragmentsForPairedSequence.h"
#include "model/Score.h"
#include "impl/sequenceAlignment.h"
#include "impl/slidingWindowAlignment.h"

// Non-static reference functions that no header declares
// (impl/sequenceAlignment3.cpp:143, impl/findSimilarFragmentsForPairedSequence4.cpp:131,288).
void SmithWaterman_non_avx(int8_t *ref, int8_t *read, const int32_t &refLen, const int32_t &readLen,
                           const int &_open_gap_penalty, const int &_extend_gap_penalty, int32_t &maxScore,
                           int32_t &endPosition1, int32_t &endPosition2, const Scorei &scorei, bool &positions);
void getSeeds(int8_t *seq1, int8_t *seq2, int8_t *seq1_rev_com, int8_t *seq2_rev_com, const int32_t &length1,
              const int32_t &length2, const int32_t &miniReferenceSize, const int32_t &_open_gap_penalty1,
              const int32_t &_extend_gap_penalty1, const int32_t &matrix_boundary_distance,
              const int32_t &startPosition2, const int32_t &mini_cns_score, const int32_t &windowsSize,
              int32_t &this_windowsSize_return, const Scorei &m, const int32_t &step_size, std::set<Seed> &seeds);
void link_seeds(std::set<Seed> &seeds);

namespace {

struct Silence {  // the reference prints progress lines to stdout; keep them out of test output
  std::streambuf *old;
  std::ostringstream sink;
  Silence() : old(std::cout.rdbuf(sink.rdbuf())) {}
  ~Silence() { std::cout.rdbuf(old); }
};

std::vector<int8_t> revcomp(const int8_t *s, int32_t n) {
  std::vector<int8_t> r(n > 0 ? n : 1);
  for (int32_t i = 0; i < n; ++i) r[i] = (int8_t)(4 - s[n - 1 - i]);
  return r;
}

std::vector<int8_t> copyseq(const int8_t *s, int32_t n) {
  std::vector<int8_t> r(n > 0 ? n : 1);
  if (n > 0) std::memcpy(r.data(), s, n);
  return r;
}

// Flat result layout shared with oracle/oracle.py:
// frag[i*8 + 0..7] = start1, end1, start2, end2, score, cigar_offset, cigar_len, 0 (all 1-based as in the reference)
// pe[i*2 + 0..1]   = p-value, e-value
int flatten(const std::vector<PairedSimilarFragment> &fr, int64_t *frag, double *pe, uint32_t *cigar, int frag_cap,
            int cigar_cap, int *n_cigar_out) {
  int nc = 0;
  for (size_t i = 0; i < fr.size(); ++i) nc += (int)fr[i].getCigar().size();
  *n_cigar_out = nc;
  if ((int)fr.size() > frag_cap || nc > cigar_cap) return -(int)fr.size() - 1;
  int off = 0;
  for (size_t i = 0; i < fr.size(); ++i) {
    const PairedSimilarFragment &f = fr[i];
    frag[i * 8 + 0] = f.getStart1();
    frag[i * 8 + 1] = f.getEnd1();
    frag[i * 8 + 2] = f.getStart2();
    frag[i * 8 + 3] = f.getEnd2();
    frag[i * 8 + 4] = f.getScore();
    frag[i * 8 + 5] = off;
    frag[i * 8 + 6] = (int64_t)f.getCigar().size();
    frag[i * 8 + 7] = 0;
    pe[i * 2 + 0] = f.getPValue();
    pe[i * 2 + 1] = f.getEValue();
    for (uint32_t c : f.getCigar()) cigar[off++] = c;
  }
  return (int)fr.size();
}

}  // namespace

extern "C" {

// SmithWaterman(..., bool&) impl/sequenceAlignment3.cpp:220 (AVX2 int8/int16 when built with -mavx2).
// out = {maxScore, endPosition1, endPosition2}; positions are only meaningful when maxScore > 0.
int ref_sw(const int8_t *ref, int32_t refLen, const int8_t *read, int32_t readLen, int open, int ext, int match,
           int mismatch, int32_t *out) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(ref, refLen), b = copyseq(read, readLen);
  int32_t mx = 0, e1 = -7, e2 = -7;
  bool pos = false;
  SmithWaterman(a.data(), b.data(), refLen, readLen, open, ext, mx, e1, e2, m, pos);
  out[0] = mx;
  out[1] = e1;
  out[2] = e2;
  return 0;
}

// SmithWaterman_non_avx impl/sequenceAlignment3.cpp:143 with positions=true.
int ref_sw_scalar(const int8_t *ref, int32_t refLen, const int8_t *read, int32_t readLen, int open, int ext,
                  int match, int mismatch, int32_t *out) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(ref, refLen), b = copyseq(read, readLen);
  int32_t mx = 0, e1 = -7, e2 = -7;
  bool pos = true;
  SmithWaterman_non_avx(a.data(), b.data(), refLen, readLen, open, ext, mx, e1, e2, m, pos);
  out[0] = mx;
  out[1] = e1;
  out[2] = e2;
  return 0;
}

// SemiGlobal_xextend without cigar, impl/sequenceAlignment3.cpp:1234. out = {maxScore, end1, end2}.
int ref_xextend(const int8_t *s1, int32_t L1, const int8_t *s2, int32_t L2, int open, int ext, int match,
                int mismatch, int xdrop, int w, int32_t *out) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(s1, L1), b = copyseq(s2, L2);
  int32_t mx, e1, e2;
  SemiGlobal_xextend(a.data(), b.data(), L1, L2, open, ext, mx, e1, e2, m, xdrop, w);
  out[0] = mx;
  out[1] = e1;
  out[2] = e2;
  return 0;
}

// SemiGlobal_xextend with cigar, impl/sequenceAlignment3.cpp:1318.
// out = {maxScore, end1, end2, iii, jjj, n_cigar}; returns -1 if cigar_cap is too small.
int ref_xextend_cigar(const int8_t *s1, int32_t L1, const int8_t *s2, int32_t L2, int open, int ext, int match,
                      int mismatch, int xdrop, int w, uint32_t *cigar, int cigar_cap, int32_t *out) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(s1, L1), b = copyseq(s2, L2);
  Matrix T(L1 + 1, L2 + 1);
  int32_t mx, e1, e2, iii = 0, jjj = 0;
  std::vector<uint32_t> c = SemiGlobal_xextend(a.data(), b.data(), L1, L2, open, ext, mx, e1, e2, m, xdrop, w, T, iii, jjj);
  out[0] = mx;
  out[1] = e1;
  out[2] = e2;
  out[3] = iii;
  out[4] = jjj;
  out[5] = (int32_t)c.size();
  if ((int)c.size() > cigar_cap) return -1;
  for (size_t i = 0; i < c.size(); ++i) cigar[i] = c[i];
  return 0;
}

// SemiGlobal (2-piece affine) impl/sequenceAlignment3.cpp:932 -> SemiGlobal_no_avx :681.
// out = {maxScore, end1, end2, n_cigar}.
int ref_semiglobal(const int8_t *s1, int32_t L1, const int8_t *s2, int32_t L2, int open1, int ext1, int open2,
                   int ext2, int match, int mismatch, int return_cigar, int zdrop, int bandwidth, uint32_t *cigar,
                   int cigar_cap, int32_t *out) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(s1, L1), b = copyseq(s2, L2);
  Matrix T(L1 + 1, L2 + 1);
  int32_t mx, e1, e2;
  std::vector<uint32_t> c = SemiGlobal(a.data(), b.data(), L1, L2, open1, ext1, open2, ext2, mx, e1, e2, m,
                                       return_cigar != 0, zdrop, bandwidth, T);
  out[0] = mx;
  out[1] = e1;
  out[2] = e2;
  out[3] = (int32_t)c.size();
  if ((int)c.size() > cigar_cap) return -1;
  for (size_t i = 0; i < c.size(); ++i) cigar[i] = c[i];
  return 0;
}

// The 1-gap window loop of findSimilarFragmentsForPairedSequence (impl/findSimilarFragmentsForPairedSequence4.cpp:462-480)
// driving the set-gated getSeeds (:131), followed by link_seeds (:288).  Dumps the raw seed set (in set order) and
// the linked set, 4 int32 per seed: start1, end1, start2, end2 (0-based).  Returns n_raw, writes n_linked.
int ref_seeds_1gap(const int8_t *s1, int32_t L1, const int8_t *s2, int32_t L2, int window, int min_score, int open,
                   int ext, int match, int mismatch, int step, int32_t *raw, int raw_cap, int32_t *linked,
                   int linked_cap, int32_t *n_linked) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(s1, L1), b = copyseq(s2, L2);
  std::vector<int8_t> ar = revcomp(s1, L1), br = revcomp(s2, L2);
  int32_t mini = min_score / match, mbd = 0, tws;
  std::set<Seed> seeds;
  int32_t sp = 0;
  while (true) {
    getSeeds(a.data(), b.data(), ar.data(), br.data(), L1, L2, mini, open, ext, mbd, sp, min_score, window, tws, m,
             step, seeds);
    sp += step;
    if (sp > L2) break;
    if (sp + window > L2) {
      getSeeds(a.data(), b.data(), ar.data(), br.data(), L1, L2, mini, open, ext, mbd, sp, min_score, window, tws, m,
               step, seeds);
      break;
    }
  }
  int n = 0;
  for (const Seed &s : seeds) {
    if (n < raw_cap) {
      raw[n * 4 + 0] = s.getStart1();
      raw[n * 4 + 1] = s.getEnd1();
      raw[n * 4 + 2] = s.getStart2();
      raw[n * 4 + 3] = s.getEnd2();
    }
    ++n;
  }
  link_seeds(seeds);
  int k = 0;
  for (const Seed &s : seeds) {
    if (k < linked_cap) {
      linked[k * 4 + 0] = s.getStart1();
      linked[k * 4 + 1] = s.getEnd1();
      linked[k * 4 + 2] = s.getStart2();
      linked[k * 4 + 3] = s.getEnd2();
    }
    ++k;
  }
  *n_linked = k;
  return n;
}

// findSimilarFragmentsForPairedSequence, 1-gap overload, impl/findSimilarFragmentsForPairedSequence4.cpp:433.
int ref_find_1gap(const int8_t *s1, int32_t L1, const int8_t *s2, int32_t L2, int window, int min_score, int open,
                  int ext, int match, int mismatch, int step, double pvalue, double lambda, double kvalue, int w,
                  int xdrop, int64_t *frag, double *pe, uint32_t *cigar, int frag_cap, int cigar_cap,
                  int *n_cigar) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(s1, L1), b = copyseq(s2, L2);
  std::vector<int8_t> ar = revcomp(s1, L1), br = revcomp(s2, L2);
  int32_t l1 = L1, l2 = L2, win = window, mbd = 0;
  std::string str1, str2;
  std::vector<PairedSimilarFragment> fr;
  {
    Silence quiet;
    fr = findSimilarFragmentsForPairedSequence(a.data(), ar.data(), b.data(), br.data(), l1, l2, win, min_score, mbd,
                                               open, ext, match, mismatch, m, step, str1, str2, pvalue, lambda, kvalue,
                                               w, xdrop);
  }
  return flatten(fr, frag, pe, cigar, frag_cap, cigar_cap, n_cigar);
}

// findSimilarFragmentsForPairedSequence, 2-gap overload, impl/findSimilarFragmentsForPairedSequence4.cpp:752.
int ref_find_2gap(const int8_t *s1, int32_t L1, const int8_t *s2, int32_t L2, int window, int min_score, int open1,
                  int ext1, int open2, int ext2, int match, int mismatch, int step, double pvalue, double lambda,
                  double kvalue, int zdrop, int bandwidth, int w, int xdrop, int64_t *frag, double *pe,
                  uint32_t *cigar, int frag_cap, int cigar_cap, int *n_cigar) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(s1, L1), b = copyseq(s2, L2);
  std::vector<int8_t> ar = revcomp(s1, L1), br = revcomp(s2, L2);
  int32_t l1 = L1, l2 = L2, win = window, mbd = 0;
  std::string str1, str2;
  std::vector<PairedSimilarFragment> fr;
  {
    Silence quiet;
    fr = findSimilarFragmentsForPairedSequence(a.data(), ar.data(), b.data(), br.data(), l1, l2, win, min_score, mbd,
                                               open1, ext1, open2, ext2, match, mismatch, m, step, str1, str2, pvalue,
                                               lambda, kvalue, zdrop, bandwidth, w, xdrop);
  }
  return flatten(fr, frag, pe, cigar, frag_cap, cigar_cap, n_cigar);
}

// findSimilarFragmentsForPairedSequence, seeded 2-gap overload (cut2Gaps2), impl/findSimilarFragmentsForPairedSequence4.cpp:624.
// seeds: n_seeds quadruples (start1, end1, start2, end2), 0-based; T is the reference's dense traceback matrix of
// (max_align + 1)^2 bytes, as cut2Gaps2 allocates it (controlLayer4.cpp:1908).
int ref_find_seeded_2gap(const int8_t *s1, int32_t L1, const int8_t *s2, int32_t L2, const int32_t *seeds,
                         int32_t n_seeds, int32_t max_align, int open1, int ext1, int open2, int ext2, int match,
                         int mismatch, double pvalue, double lambda, double kvalue, int zdrop, int bandwidth,
                         int64_t *frag, double *pe, uint32_t *cigar, int frag_cap, int cigar_cap, int *n_cigar) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(s1, L1), b = copyseq(s2, L2);
  std::vector<int8_t> ar = revcomp(s1, L1), br = revcomp(s2, L2);
  int32_t l1 = L1, l2 = L2, win = 38, mal = max_align;
  std::string str1, str2;
  std::vector<Seed> sd;
  for (int32_t k = 0; k < n_seeds; ++k) {
    int32_t a1 = seeds[4 * k], e1 = seeds[4 * k + 1], a2 = seeds[4 * k + 2], e2 = seeds[4 * k + 3];
    sd.emplace_back(a1, e1, a2, e2);
  }
  Matrix T(max_align + 1, max_align + 1);
  std::vector<PairedSimilarFragment> fr;
  {
    Silence quiet;
    fr = findSimilarFragmentsForPairedSequence(a.data(), ar.data(), b.data(), br.data(), l1, l2, win, open1, ext1,
                                               open2, ext2, match, mismatch, m, str1, str2, pvalue, lambda, kvalue,
                                               zdrop, bandwidth, sd, T, mal);
  }
  return flatten(fr, frag, pe, cigar, frag_cap, cigar_cap, n_cigar);
}

// The x-seed overload without maximumAlignLength, impl/findSimilarFragmentsForPairedSequence4.cpp:532-616, with the
// traceback matrix its caller (the 2-gap overload, :769) allocates: (L1 + 1) x (L2 + 1).
int ref_find_xseeds_2gap(const int8_t *s1, int32_t L1, const int8_t *s2, int32_t L2, const int32_t *seeds,
                         int32_t n_seeds, int open1, int ext1, int open2, int ext2, int match, int mismatch,
                         double pvalue, double lambda, double kvalue, int zdrop, int bandwidth, int64_t *frag,
                         double *pe, uint32_t *cigar, int frag_cap, int cigar_cap, int *n_cigar) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(s1, L1), b = copyseq(s2, L2);
  std::vector<int8_t> ar = revcomp(s1, L1), br = revcomp(s2, L2);
  int32_t l1 = L1, l2 = L2, win = 38;
  std::string str1, str2;
  std::vector<Seed> sd;
  for (int32_t k = 0; k < n_seeds; ++k) {
    int32_t a1 = seeds[4 * k], e1 = seeds[4 * k + 1], a2 = seeds[4 * k + 2], e2 = seeds[4 * k + 3];
    sd.emplace_back(a1, e1, a2, e2);
  }
  Matrix T(L1 + 1, L2 + 1);
  std::vector<PairedSimilarFragment> fr;
  {
    Silence quiet;
    fr = findSimilarFragmentsForPairedSequence(a.data(), ar.data(), b.data(), br.data(), l1, l2, win, open1, ext1,
                                               open2, ext2, match, mismatch, m, str1, str2, pvalue, lambda, kvalue,
                                               zdrop, bandwidth, sd, T);
  }
  return flatten(fr, frag, pe, cigar, frag_cap, cigar_cap, n_cigar);
}

// The weighted drivers, impl/findSimilarFragmentsForPairedSequence4.cpp:784 (pieces 1) and :883 (pieces 2).  The
// categories are written as a Score folder (matrixList + one 7-line file per category, model/Score.cpp:3) under
// score_dir.  The weight arrays get one extra entry on each side repeating the end categories, so the reference's
// reads one before and one past them (at the first and last row) see defined values.
int ref_find_weighted(int pieces, const int8_t *s1, int32_t L1, const int8_t *s2, int32_t L2, const int16_t *weights,
                      const int32_t *cats, int32_t n_cats, const char *score_dir, int window, int min_score, int open1,
                      int ext1, int match, int mismatch, int step, double pvalue, double lambda, double kvalue,
                      int zdrop, int bandwidth, int w, int xdrop, int64_t *frag, double *pe, uint32_t *cigar,
                      int frag_cap, int cigar_cap, int *n_cigar) {
  {
    std::ofstream list(std::string(score_dir) + "/matrixList");
    for (int32_t k = 0; k < n_cats; ++k) {
      list << k << "\n";
      std::ofstream f(std::string(score_dir) + "/" + std::to_string(k));
      for (int q = 0; q < 7; ++q) f << cats[7 * k + q] << "\n";
    }
  }
  Score score(score_dir);
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<int8_t> a = copyseq(s1, L1), b = copyseq(s2, L2);
  std::vector<int8_t> ar = revcomp(s1, L1), br = revcomp(s2, L2);
  std::vector<int16_t> wf(L1 + 2), wr(L1 + 2);
  for (int32_t i = 0; i < L1; ++i) wf[i + 1] = weights[i], wr[i + 1] = weights[L1 - 1 - i];
  if (L1 > 0) wf[0] = wf[1], wf[L1 + 1] = wf[L1], wr[0] = wr[1], wr[L1 + 1] = wr[L1];
  int32_t l1 = L1, l2 = L2, win = window, mbd = 0, ww = w;
  std::string str1, str2;
  std::vector<PairedSimilarFragment> fr;
  {
    Silence quiet;
    if (pieces == 1)
      fr = findSimilarFragmentsForPairedSequence_wighted_1gap(a.data(), ar.data(), b.data(), br.data(), l1, l2, win,
                                                              min_score, mbd, open1, ext1, match, mismatch, m, step,
                                                              str1, str2, pvalue, lambda, kvalue, zdrop, bandwidth,
                                                              ww, xdrop, score, wf.data() + 1, wr.data() + 1);
    else
      fr = findSimilarFragmentsForPairedSequence_wighted(a.data(), ar.data(), b.data(), br.data(), l1, l2, win,
                                                         min_score, mbd, open1, ext1, match, mismatch, m, step, str1,
                                                         str2, pvalue, lambda, kvalue, zdrop, bandwidth, ww, xdrop,
                                                         score, wf.data() + 1, wr.data() + 1);
  }
  return flatten(fr, frag, pe, cigar, frag_cap, cigar_cap, n_cigar);
}

// slidingWindowAlignment, impl/slidingWindowAlignment.cpp:11.  seqs[0] is the reference; the reference writes
// "j name score" lines to out_path, which the caller parses.
int ref_sliding(const int8_t *const *seqs, const int32_t *lens, int nseq, int window, int step, int open, int ext,
                int match, int mismatch, const char *out_path) {
  Scorei m((int8_t)match, (int8_t)mismatch);
  std::vector<std::vector<int8_t>> owned;
  std::vector<int8_t *> ptrs;
  std::vector<int32_t> lengths;
  std::vector<std::string> names;
  for (int i = 0; i < nseq; ++i) {
    owned.push_back(copyseq(seqs[i], lens[i]));
    lengths.push_back(lens[i]);
    names.push_back("s" + std::to_string(i));
  }
  for (auto &o : owned) ptrs.push_back(o.data());
  int32_t win = window;
  slidingWindowAlignment(ptrs.data(), lengths, names, win, open, ext, match, mismatch, std::string(out_path), step, m);
  return 0;
}

}  // extern "C"
