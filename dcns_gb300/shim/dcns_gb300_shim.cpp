// dcns_gb300_shim.cpp — dCNS's pair-alignment interface (impl/findSimilarFragmentsForPairedSequence.h:26-86) on the
// GB300 engine's C ABI (include/dcns_gb300.h).
//
// A dCNS build compiles this file in place of impl/findSimilarFragmentsForPairedSequence4.cpp and links
// libdcnsgpu.so (dcns_gb300/_lib); every caller (cut1Gap, cut2Gaps, cut2Gaps2, pairCnsXExtend, pairCns2Gaps, multCns,
// weighted1Gap, weighted2Gaps) keeps its call unchanged.  All six functions of the header are defined here with the
// reference's signatures:
//
//   1-gap overload                 (header :26-32)  -> dcns_align_pairs, DCNS_MODE_ONE_GAP
//   2-gap overload                 (header :34-42)  -> dcns_align_pairs, DCNS_MODE_TWO_GAP
//   _wighted                       (header :45-52)  -> dcns_align_weighted, pieces = 2
//   _wighted_1gap                  (header :54-61)  -> dcns_align_weighted, pieces = 1
//   x-seed overload                (header :70-77)  -> dcns_align_xseeds
//   x-seed overload with a cap     (header :79-86)  -> dcns_align_seeded (max_align_len = maximumAlignLength)
//
// The reverse-complement arrays, the Scorei and the strings are accepted and not read: the engine derives reverse
// complements on the device and scores with match / mismatch.  The caller-owned traceback matrix (Matrix& T) of the
// x-seed overloads is not touched: the engine keeps banded direction codes in device memory, so a dCNS build with this
// shim can drop the dense Matrix(maximumAlignLength + 1, maximumAlignLength + 1) allocation.  The weighted overloads
// read the categories of seq1's bases from `weight` (weight_rev, its mirror, is not needed) and turn the Score
// folder's per-category parameters into the engine's category rows.  One process-wide context on device 0 is
// created on first use; an engine error becomes a std::runtime_error (the reference has no error returns).
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "dcns_gb300.h"
#include "impl/findSimilarFragmentsForPairedSequence.h"

namespace {

dcns_ctx *engine() {
  static dcns_ctx *ctx = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    if (dcns_ctx_create(0, 0, &ctx) != DCNS_OK) throw std::runtime_error("dcns_gb300: no usable sm_103a GPU");
  });
  return ctx;
}

std::vector<PairedSimilarFragment> to_fragments(dcns_results *r) {
  std::vector<PairedSimilarFragment> out;
  out.reserve((size_t)r->n_fragments);
  for (int64_t i = 0; i < r->n_fragments; ++i) {
    const int64_t *f = r->frag + 7 * i;
    std::vector<uint32_t> cigar(r->cigar + f[5], r->cigar + f[5] + f[6]);
    double pv = r->pvalue[i], ev = r->evalue[i];
    out.emplace_back((uint32_t)f[0], (uint32_t)f[1], (uint32_t)f[2], (uint32_t)f[3], (uint32_t)f[4], cigar, pv, ev);
  }
  dcns_results_free(r);
  return out;
}

void check(int rc) {
  if (rc != DCNS_OK) throw std::runtime_error(std::string("dcns_gb300: ") + dcns_last_error(engine()));
}

dcns_params base_params(int32_t window, int32_t match, int32_t mismatch, int32_t open1, int32_t ext1, double pvalues,
                        double lambda, double kValue) {
  dcns_params p;
  dcns_params_default(&p);
  p.window = window;
  p.match = match;
  p.mismatch = mismatch;
  p.open1 = open1;
  p.ext1 = ext1;
  p.pvalue = pvalues;
  p.lambda = lambda;
  p.kvalue = kValue;
  return p;
}

std::vector<PairedSimilarFragment> align(int8_t *seq1, int32_t len1, int8_t *seq2, int32_t len2, const dcns_params &p,
                                         int mode) {
  dcns_pair pair{seq1, len1, seq2, len2};
  dcns_results *r = nullptr;
  check(dcns_align_pairs(engine(), &pair, 1, &p, mode, &r));
  return to_fragments(r);
}

// The weighted drivers: the categories of seq1's bases, renumbered 0..k-1 in order of first use, and one row of
// match, mismatch, open1, ext1, open2, ext2, zdrop per category from the Score folder (model/Score.cpp:3-60).
std::vector<PairedSimilarFragment> align_weighted(int8_t *seq1, int32_t len1, int8_t *seq2, int32_t len2,
                                                  const dcns_params &p, Score &score, const int16_t *weight,
                                                  int pieces) {
  std::map<int16_t, int16_t> id;
  std::vector<int16_t> dense((size_t)len1);
  std::vector<int32_t> cats;
  for (int32_t i = 0; i < len1; ++i) {
    auto it = id.find(weight[i]);
    if (it == id.end()) {
      const int16_t c = weight[i];
      it = id.emplace(c, (int16_t)id.size()).first;
      int32_t **m = score.getM(c);
      cats.insert(cats.end(), {m[0][0], m[0][1], score.getOpenGapPenalty1(c), score.getExtendGapPenalty1(c),
                               score.getOpenGapPenalty2(c), score.getExtendGapPenalty2(c), score.getZdrop(c)});
    }
    dense[i] = it->second;
  }
  if (cats.empty()) cats.assign(7, 0);  // an empty seq1: one unused category
  dcns_pair pair{seq1, len1, seq2, len2};
  dcns_results *r = nullptr;
  check(dcns_align_weighted(engine(), &pair, 1, dense.data(), cats.data(), (int32_t)(cats.size() / 7), pieces, &p,
                            &r));
  return to_fragments(r);
}

std::vector<PairedSimilarFragment> align_xseeds(int8_t *seq1, int32_t len1, int8_t *seq2, int32_t len2,
                                                const dcns_params &p, const std::vector<Seed> &seeds, bool capped) {
  std::vector<int32_t> flat;
  flat.reserve(4 * seeds.size());
  for (const Seed &s : seeds) flat.insert(flat.end(), {s.getStart1(), s.getEnd1(), s.getStart2(), s.getEnd2()});
  if (flat.empty()) flat.assign(4, 0);
  const int64_t off[2] = {0, (int64_t)seeds.size()};
  dcns_pair pair{seq1, len1, seq2, len2};
  dcns_results *r = nullptr;
  check((capped ? dcns_align_seeded : dcns_align_xseeds)(engine(), &pair, 1, flat.data(), off, &p, &r));
  return to_fragments(r);
}

}  // namespace

// 1-gap overload (cut1Gap, pairCnsXExtend, multCns).  matrix_boundary_distance is not used by the reference either.
std::vector<PairedSimilarFragment> findSimilarFragmentsForPairedSequence(
    int8_t *seq1, int8_t *, int8_t *seq2, int8_t *, int32_t &length1, int32_t &length2, int32_t &windowsSize,
    const int32_t &mini_cns_score, const int32_t &, const int32_t &_open_gap_penalty1,
    const int32_t &_extend_gap_penalty1, const int32_t &matchingScore, const int32_t &mismatchingPenalty,
    const Scorei &, const int32_t &step_size, std::string &, std::string &, const double &pvalues,
    const double &lambda, const double &kValue, const int32_t &w, const int32_t &xDrop) {
  dcns_params p = base_params(windowsSize, matchingScore, mismatchingPenalty, _open_gap_penalty1,
                              _extend_gap_penalty1, pvalues, lambda, kValue);
  p.min_score = mini_cns_score;
  p.step = step_size;
  p.w = w;
  p.xdrop = xDrop;
  return align(seq1, length1, seq2, length2, p, DCNS_MODE_ONE_GAP);
}

// 2-gap overload (cut2Gaps, pairCns2Gaps)
std::vector<PairedSimilarFragment> findSimilarFragmentsForPairedSequence(
    int8_t *seq1, int8_t *, int8_t *seq2, int8_t *, int32_t &length1, int32_t &length2, int32_t &windowsSize,
    const int32_t &mini_cns_score, const int32_t &, const int32_t &_open_gap_penalty1,
    const int32_t &_extend_gap_penalty1, const int32_t &_open_gap_penalty2, const int32_t &_extend_gap_penalty2,
    const int32_t &matchingScore, const int32_t &mismatchingPenalty, const Scorei &, const int32_t &step_size,
    std::string &, std::string &, const double &pvalues, const double &lambda, const double &kValue,
    const int32_t &zDrop, const int32_t &bandwidth, const int32_t &w, const int32_t &xDrop) {
  dcns_params p = base_params(windowsSize, matchingScore, mismatchingPenalty, _open_gap_penalty1,
                              _extend_gap_penalty1, pvalues, lambda, kValue);
  p.min_score = mini_cns_score;
  p.step = step_size;
  p.open2 = _open_gap_penalty2;
  p.ext2 = _extend_gap_penalty2;
  p.zdrop = zDrop;
  p.bandwidth = bandwidth;
  p.w = w;
  p.xdrop = xDrop;
  return align(seq1, length1, seq2, length2, p, DCNS_MODE_TWO_GAP);
}

// weighted2Gaps: 2-gap x-seeds, then weighted 2-piece DPs
std::vector<PairedSimilarFragment> findSimilarFragmentsForPairedSequence_wighted(
    int8_t *seq1, int8_t *, int8_t *seq2, int8_t *, int32_t &length1, int32_t &length2, int32_t &windowsSize,
    const int32_t &mini_cns_score, const int32_t &, const int32_t &_open_gap_penalty1,
    const int32_t &_extend_gap_penalty1, const int32_t &matchingScore, const int32_t &mismatchingPenalty,
    const Scorei &, const int32_t &step_size, std::string &, std::string &, const double &pvalues,
    const double &lambda, const double &kValue, const int32_t &zDrop, const int32_t &bandwidth, int32_t &w,
    const int32_t &xDrop, Score &score, int16_t *weight, int16_t *) {
  dcns_params p = base_params(windowsSize, matchingScore, mismatchingPenalty, _open_gap_penalty1,
                              _extend_gap_penalty1, pvalues, lambda, kValue);
  p.min_score = mini_cns_score;
  p.step = step_size;
  p.zdrop = zDrop;
  p.bandwidth = bandwidth;
  p.w = w;
  p.xdrop = xDrop;
  return align_weighted(seq1, length1, seq2, length2, p, score, weight, 2);
}

// weighted1Gap: 2-gap x-seeds, then weighted 1-piece DPs
std::vector<PairedSimilarFragment> findSimilarFragmentsForPairedSequence_wighted_1gap(
    int8_t *seq1, int8_t *, int8_t *seq2, int8_t *, int32_t &length1, int32_t &length2, int32_t &windowsSize,
    const int32_t &mini_cns_score, const int32_t &, const int32_t &_open_gap_penalty1,
    const int32_t &_extend_gap_penalty1, const int32_t &matchingScore, const int32_t &mismatchingPenalty,
    const Scorei &, const int32_t &step_size, std::string &, std::string &, const double &pvalues,
    const double &lambda, const double &kValue, const int32_t &zDrop, const int32_t &bandwidth, int32_t &w,
    const int32_t &xDrop, Score &score, int16_t *weight, int16_t *) {
  dcns_params p = base_params(windowsSize, matchingScore, mismatchingPenalty, _open_gap_penalty1,
                              _extend_gap_penalty1, pvalues, lambda, kValue);
  p.min_score = mini_cns_score;
  p.step = step_size;
  p.zdrop = zDrop;
  p.bandwidth = bandwidth;
  p.w = w;
  p.xdrop = xDrop;
  return align_weighted(seq1, length1, seq2, length2, p, score, weight, 1);
}

// The x-seed overload (the 2-piece stage the 2-gap overload runs on its own x-seeds)
std::vector<PairedSimilarFragment> findSimilarFragmentsForPairedSequence(
    int8_t *seq1, int8_t *, int8_t *seq2, int8_t *, int32_t &length1, int32_t &length2, int32_t &windowsSize,
    const int32_t &_open_gap_penalty1, const int32_t &_extend_gap_penalty1, const int32_t &_open_gap_penalty2,
    const int32_t &_extend_gap_penalty2, const int32_t &matchingScore, const int32_t &mismatchingPenalty,
    const Scorei &, std::string &, std::string &, const double &pvalues, const double &lambda, const double &kValue,
    const int32_t &zDrop, const int32_t &bandwidth, std::vector<Seed> &x_extend_seeds, Matrix &) {
  dcns_params p = base_params(windowsSize, matchingScore, mismatchingPenalty, _open_gap_penalty1,
                              _extend_gap_penalty1, pvalues, lambda, kValue);
  p.open2 = _open_gap_penalty2;
  p.ext2 = _extend_gap_penalty2;
  p.zdrop = zDrop;
  p.bandwidth = bandwidth;
  return align_xseeds(seq1, length1, seq2, length2, p, x_extend_seeds, false);
}

// The x-seed overload with maximumAlignLength (cut2Gaps2, controlLayer4.cpp:1928,1967)
std::vector<PairedSimilarFragment> findSimilarFragmentsForPairedSequence(
    int8_t *seq1, int8_t *, int8_t *seq2, int8_t *, int32_t &length1, int32_t &length2, int32_t &windowsSize,
    const int32_t &_open_gap_penalty1, const int32_t &_extend_gap_penalty1, const int32_t &_open_gap_penalty2,
    const int32_t &_extend_gap_penalty2, const int32_t &matchingScore, const int32_t &mismatchingPenalty,
    const Scorei &, std::string &, std::string &, const double &pvalues, const double &lambda, const double &kValue,
    const int32_t &zDrop, const int32_t &bandwidth, std::vector<Seed> &x_extend_seeds, Matrix &,
    int32_t &maximumAlignLength) {
  dcns_params p = base_params(windowsSize, matchingScore, mismatchingPenalty, _open_gap_penalty1,
                              _extend_gap_penalty1, pvalues, lambda, kValue);
  p.open2 = _open_gap_penalty2;
  p.ext2 = _extend_gap_penalty2;
  p.zdrop = zDrop;
  p.bandwidth = bandwidth;
  p.max_align_len = maximumAlignLength;
  return align_xseeds(seq1, length1, seq2, length2, p, x_extend_seeds, true);
}
