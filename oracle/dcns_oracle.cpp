// ORACLE — test infrastructure only.  A scalar CPU restatement of dCNS's pairwise CNS alignment hot path, written
// from the reference's semantics, used (1) by tests/ as the parity checker for the CUDA path, (2) by bench.py as the
// CPU baseline ("port") on hosts where the reference itself cannot be built.  Nothing in the product links it.
//
// Parity of this restatement is pinned against the unmodified reference (oracle/_ref, built by build_ref.sh from the
// reference checkout) by tests/test_oracle_pin.py, by the golden fixtures in tests/golden/, and by the reference's
// digests of the benchmark workloads (tests/test_workload_digests.py).
//
// Reference map (paths inside the dCNS project):
//   sw_striped_semantics   impl/sequenceAlignment3.cpp:220-337 (AVX2 int8) and :338-460 (AVX2 int16)
//   sw_scalar_semantics    impl/sequenceAlignment3.cpp:143-216 (SmithWaterman_non_avx)
//   sw_dispatch            impl/sequenceAlignment3.cpp:223-225, :338-339 (int8 / int16 / scalar guard)
//   xextend_pass           impl/sequenceAlignment3.cpp:1234-1314 and :1318-1451 (band restart, traceback)
//   semiglobal             impl/sequenceAlignment3.cpp:681-928 (2-piece affine, z-drop, traceback)
//   SeedLess / seed sets   model/Seed.h:29-42
//   seeds_recursive        impl/findSimilarFragmentsForPairedSequence4.cpp:61-128
//   seeds_gated            impl/findSimilarFragmentsForPairedSequence4.cpp:131-201
//   link_seeds             impl/findSimilarFragmentsForPairedSequence4.cpp:288-344
//   x_extend_seed          impl/findSimilarFragmentsForPairedSequence4.cpp:205-285
//   find_1gap              impl/findSimilarFragmentsForPairedSequence4.cpp:433-524
//   all_extend_seeds       impl/findSimilarFragmentsForPairedSequence4.cpp:348-429
//   two_piece_stage        impl/findSimilarFragmentsForPairedSequence4.cpp:532-616
//   sliding window         impl/slidingWindowAlignment.cpp:11-46

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <set>
#include <thread>
#include <utility>
#include <vector>

namespace {

constexpr int32_t OUT = -536870912;  // score of cells outside the band (impl/sequenceAlignment3.cpp:34)

struct Params {
  int32_t match, mismatch, open1, ext1, open2, ext2;
  int32_t window, min_score, step, w, xdrop, zdrop, bandwidth;
  double pvalue, lambda, kvalue;
};

// Scorei (model/Score.cpp:105-135): code 2 (N and every non-ACGTU character) scores 0 against anything.
struct Score {
  int32_t m, x;
  inline int32_t operator()(int8_t a, int8_t b) const { return (a == 2 || b == 2) ? 0 : (a == b ? m : x); }
};

struct Cells {  // algorithmic DP cells, by stage
  int64_t scan = 0, scan_rev = 0, xdrop = 0, semiglobal = 0;
};

// ---------------------------------------------------------------- Smith-Waterman (seed scan)
struct SwOut {
  int32_t score, end1, end2;  // 0-based first argmax in (ref-major, read-minor) order; untouched when score == 0
};

// Semantics of the striped SIMD kernels: the vertical-gap state E is advanced from H *before* the row's
// horizontal-gap pass merges into it; the horizontal pass then runs left to right over the read.
void sw_striped_semantics(const int8_t *ref, int32_t nref, const int8_t *read, int32_t nread, int32_t open,
                          int32_t ext, Score sc, SwOut &o) {
  o.score = 0;
  if (nread <= 0) return;
  std::vector<int32_t> H(nread, 0), Hpre(nread), E(nread, 0);
  for (int32_t i = 0; i < nref; ++i) {
    int32_t diag = 0;
    for (int32_t p = 0; p < nread; ++p) {
      int32_t h = std::max(diag + sc(ref[i], read[p]), 0);
      h = std::max(h, E[p]);
      Hpre[p] = h;
      E[p] = std::max(std::max(E[p] + ext, h + open), 0);
      diag = H[p];
    }
    int32_t del = 0, left = 0;
    for (int32_t p = 0; p < nread; ++p) {
      del = std::max(left + open, del + ext);
      int32_t h = Hpre[p] < del ? del : Hpre[p];
      del = std::max(del, 0);
      H[p] = h;
      left = h;
      if (h > o.score) {
        o.score = h;
        o.end1 = i;
        o.end2 = p;
      }
    }
  }
}

// Semantics of the scalar kernel: the vertical gap opens from the previous row's final H.
void sw_scalar_semantics(const int8_t *ref, int32_t nref, const int8_t *read, int32_t nread, int32_t open,
                         int32_t ext, Score sc, SwOut &o) {
  o.score = 0;
  o.end1 = 0;
  o.end2 = 0;
  std::vector<int32_t> prev(std::max(nread, 0) + 1, 0), cur(std::max(nread, 0) + 1, 0), F(std::max(nread, 0) + 1, 0);
  for (int32_t i = 1; i <= nref; ++i) {
    int32_t e = 0;
    for (int32_t j = 1; j <= nread; ++j) {
      e = std::max(open + cur[j - 1], ext + e);
      F[j] = std::max(open + prev[j], ext + F[j]);
      int32_t v = std::max(sc(ref[i - 1], read[j - 1]) + prev[j - 1], e);
      v = std::max(v, F[j]);
      cur[j] = std::max(v, 0);
      F[j] = std::max(F[j], 0);
      e = std::max(e, 0);
      if (v > o.score) {
        o.score = v;
        o.end1 = i;
        o.end2 = j;
      }
    }
    std::swap(prev, cur);
  }
  o.end1 -= 1;
  o.end2 -= 1;
}

// Which kernel the reference's x86 build runs for these lengths (int8 and int16 paths share the striped semantics).
bool sw_uses_striped(int32_t nref, int32_t nread, int32_t open, int32_t ext, int32_t match) {
  auto ok = [&](int32_t lim) {
    return ((-nref * ext - open) < lim || (-nread * ext - open) < lim) && (nref * match < lim || nread * match < lim);
  };
  return ok(125) || ok(32767);
}

void sw_dispatch(const int8_t *ref, int32_t nref, const int8_t *read, int32_t nread, int32_t open, int32_t ext,
                 Score sc, SwOut &o) {
  if (sw_uses_striped(nref, nread, open, ext, sc.m))
    sw_striped_semantics(ref, nref, read, nread, open, ext, sc, o);
  else
    sw_scalar_semantics(ref, nref, read, nread, open, ext, sc, o);
}

// ---------------------------------------------------------------- traceback store with reset-to-255 semantics
struct BandStore {
  // Per computed row: first column and the codes of columns [first, first+n).  Anything else reads 255,
  // which is what the reference's dense Matrix holds after reset().
  std::vector<int32_t> first;
  std::vector<std::vector<uint8_t>> codes;
  void reset() {
    first.assign(1, 0);
    codes.assign(1, {});
  }
  void begin_row(int32_t i, int32_t c0) {
    if ((int32_t)first.size() <= i) {
      first.resize(i + 1, 0);
      codes.resize(i + 1);
    }
    first[i] = c0;
    codes[i].clear();
  }
  void push(int32_t i, uint8_t c) { codes[i].push_back(c); }
  uint8_t get(int32_t i, int32_t j) const {
    if (i <= 0 || i >= (int32_t)first.size()) return 255;
    int32_t k = j - first[i];
    if (k < 0 || k >= (int32_t)codes[i].size()) return 255;
    return codes[i][k];
  }
};

inline void cigar_push(std::vector<uint32_t> &cg, uint32_t op) {
  if (cg.empty() || (cg.back() & 0xf) != op)
    cg.push_back((1u << 4) | op);
  else
    cg.back() += 1u << 4;
}

// Walk the direction codes from (ii, jj).  Codes: low 3 bits = winning state (0 diag, 1/3 vertical, 2/4 horizontal),
// bit (state+2) = "the gap state feeding this cell was extended, not opened".
void walk_codes(const BandStore &T, int32_t &ii, int32_t &jj, std::vector<uint32_t> &cg) {
  int state = 0;
  while (ii > 0 && jj > 0) {
    int t = T.get(ii, jj);
    if (state == 0)
      state = t & 7;
    else if (!((t >> (state + 2)) & 1))
      state = 0;
    if (state == 0) state = t & 7;
    if (state == 0) {
      cigar_push(cg, 0);
      --ii;
      --jj;
    } else if (state == 1 || state == 3) {
      cigar_push(cg, 2);
      --ii;
    } else {
      cigar_push(cg, 1);
      --jj;
    }
  }
}

// ---------------------------------------------------------------- x-drop banded extension
struct XOut {
  int32_t score, end1, end2, iii, jjj;
  std::vector<uint32_t> cigar;
  int64_t cells;  // band cells of the rows evaluated in the final band width
};

// One pass at half-width w.  Returns false when the row maximum touched a band edge (the caller doubles w).
bool xextend_pass(const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, int32_t open, int32_t ext, Score sc,
                  int32_t xdrop, int32_t w, BandStore *T, XOut &o) {
  std::vector<int32_t> prev(n2 + 1, OUT), cur(n2 + 1, OUT), F(n2 + 1, OUT);
  prev[0] = 0;
  o.score = 0;
  o.end1 = 0;
  o.end2 = 0;
  o.cells = 0;
  if (T) T->reset();
  for (int32_t i = 1; i <= n1; ++i) {
    int32_t best = 0, bestj = -1;
    int32_t c0 = std::max(i - w, 1), c1 = std::min(i + w, n2);
    int32_t e = OUT;
    F[c1] = OUT;
    if (T) T->begin_row(i, c0);
    for (int32_t j = c0; j <= c1; ++j) {
      int32_t v = sc(s1[i - 1], s2[j - 1]) + prev[j - 1];
      uint8_t d = v > F[j] ? 0 : 1;
      if (!(v > F[j])) v = F[j];
      if (!(v > e)) {
        d = 2;
        v = e;
      }
      cur[j] = v;
      if (v > best) {
        best = v;
        bestj = j;
      }
      int32_t h = v + open;
      int32_t f = F[j] + ext;
      if (f >= h) d |= 1 << 3;
      F[j] = f >= h ? f : h;
      e += ext;
      if (e >= h) d |= 1 << 4;
      e = e >= h ? e : h;
      if (T) T->push(i, d);
    }
    o.cells += std::max(c1 - c0 + 1, 0);
    if (bestj != n2 && bestj != 1 && (bestj == c0 || bestj == c1)) return false;
    if (best > o.score) {
      o.score = best;
      o.end1 = i;
      o.end2 = bestj;
    }
    if (o.score - best > xdrop) break;
    if (best <= 0) break;  // equivalent to "bestj <= 0": bestj is set exactly when best > 0
    std::swap(prev, cur);
    prev[0] = OUT;
    cur[0] = OUT;
  }
  return true;
}

void xextend(const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, int32_t open, int32_t ext, Score sc,
             int32_t xdrop, int32_t w, bool want_cigar, XOut &o) {
  BandStore T;
  while (!xextend_pass(s1, n1, s2, n2, open, ext, sc, xdrop, w, want_cigar ? &T : nullptr, o)) w *= 2;
  o.cigar.clear();
  if (want_cigar) {
    int32_t ii = o.end1, jj = o.end2;
    walk_codes(T, ii, jj, o.cigar);
    o.iii = ii;
    o.jjj = jj;
  }
  o.end1 -= 1;
  o.end2 -= 1;
}

// ---------------------------------------------------------------- 2-piece affine semi-global with z-drop
struct SgOut {
  int32_t score, end1, end2;
  std::vector<uint32_t> cigar;
  int64_t cells;
};

void semiglobal(const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, const Params &P, Score sc,
                bool want_cigar, SgOut &o) {
  const int32_t o1 = P.open1, x1 = P.ext1, o2 = P.open2, x2 = P.ext2, w = P.bandwidth;
  BandStore T;
  if (want_cigar) T.reset();
  std::vector<int32_t> prev(std::max(n2, 0) + 1, OUT), cur(std::max(n2, 0) + 1, OUT);
  std::vector<int32_t> F1(std::max(n2, 0) + 1, OUT), F2(std::max(n2, 0) + 1, OUT);
  prev[0] = 0;
  o.score = 0;
  o.end1 = -1;
  o.end2 = -1;
  o.cells = 0;
  for (int32_t i = 1; i <= n1; ++i) {
    int32_t best = 0, bestj = 0;
    int32_t c0 = std::max(i - w, 1), c1 = std::min(i + w, n2);
    int32_t e1 = OUT, e2 = OUT;
    F1[c1] = OUT;
    F2[c1] = OUT;
    if (want_cigar) T.begin_row(i, c0);
    // Columns [c0, c1) update the gap states and the codes; the band's last column c1 is scored but never updates
    // them, and it is scored even when the band is empty (rows more than w past the query end).
    for (int32_t j = c0; j <= c1 || j == c0; ++j) {
      const bool last = (j >= c1);
      if (last) j = c1;
      if (j < 1) break;  // n2 == 0: the reference would read before the query; unreachable from its callers
      int32_t v = sc(s1[i - 1], s2[j - 1]) + prev[j - 1];
      uint8_t d = 0;
      if (!(v > F1[j])) {
        d = 1;
        v = F1[j];
      }
      if (!(v > e1)) {
        d = 2;
        v = e1;
      }
      if (!(v > F2[j])) {
        d = 3;
        v = F2[j];
      }
      if (!(v > e2)) {
        d = 4;
        v = e2;
      }
      cur[j] = v;
      if (v > best) {
        best = v;
        bestj = j;
      }
      if (last) break;
      int32_t h = v + o1, f = F1[j] + x1;
      if (f >= h) d |= 1 << 3;
      F1[j] = f >= h ? f : h;
      e1 += x1;
      if (e1 >= h) d |= 1 << 4;
      e1 = e1 >= h ? e1 : h;
      int32_t h2 = v + o2, f2 = F2[j] + x2;
      if (f2 >= h2) d |= 1 << 5;
      F2[j] = f2 >= h2 ? f2 : h2;
      e2 += x2;
      if (e2 >= h2) d |= 1 << 6;
      e2 = e2 >= h2 ? e2 : h2;
      if (want_cigar) T.push(i, d);
    }
    o.cells += std::max(c1 - c0 + 1, 0);
    if (best > o.score) {
      o.score = best;
      o.end1 = i;
      o.end2 = bestj;
    }
    int32_t l = (i - o.end1) - (bestj - o.end2);
    l = l > 0 ? l : -l;
    if (o.score - best > P.zdrop + l * x2) break;
    if (bestj <= 0) break;
    std::swap(prev, cur);
    prev[0] = OUT;
    cur[0] = OUT;
  }
  o.cigar.clear();
  if (want_cigar) {
    int32_t ii = o.end1, jj = o.end2;
    walk_codes(T, ii, jj, o.cigar);
    while (ii > 0) {
      cigar_push(o.cigar, 2);
      --ii;
    }
    while (jj > 0) {
      cigar_push(o.cigar, 1);
      --jj;
    }
    std::reverse(o.cigar.begin(), o.cigar.end());
  }
  o.end1 -= 1;
  o.end2 -= 1;
}

// ---------------------------------------------------------------- seeds
// ---------------------------------------------------------------- weighted semi-global (per-row categories)
// One scoring category of the weighted variants (model/Score.cpp:3-60: a matrixList entry): match / mismatch (N
// scores 0), both gap models and the z-drop.
struct WCat {
  int32_t match, mismatch, open1, ext1, open2, ext2, zdrop;
};

// SemiGlobal (impl/sequenceAlignment3.cpp:1483-1709, pieces = 2) and SemiGlobal_single_gap_penalty (:1710-1890,
// pieces = 1).  Row i (1-based) scores with the category of weights[i-1]: substitution, the horizontal gap states and
// the z-drop test; the vertical gap states it leaves for the next row use the category of weights[i].  Every band
// column, the last included, updates the gap states and writes its code (F of the last column starts from OUT); an
// empty band ends the DP.  weights must hold n1 + 1 entries: the caller repeats the final category where the
// reference reads one past its array.  The bandwidth is P.bandwidth; the z-drop comes from the categories.
void weighted_semiglobal(int pieces, const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2,
                         const int16_t *weights, const WCat *cats, int32_t w, bool want_cigar, SgOut &o) {
  BandStore T;
  if (want_cigar) T.reset();
  std::vector<int32_t> prev(std::max(n2, 0) + 1, OUT), cur(std::max(n2, 0) + 1, OUT);
  std::vector<int32_t> F1(std::max(n2, 0) + 1, OUT), F2(std::max(n2, 0) + 1, OUT);
  prev[0] = 0;
  o.score = 0;
  o.end1 = -1;
  o.end2 = -1;
  o.cells = 0;
  for (int32_t i = 1; i <= n1; ++i) {
    const WCat &rc = cats[weights[i - 1]], &nc = cats[weights[i]];
    int32_t best = 0, bestj = pieces == 2 ? OUT : -1;
    const int32_t c0 = std::max(i - w, 1), c1 = std::min(i + w, n2);
    int32_t e1 = OUT, e2 = OUT;
    if (c1 >= 0) F1[c1] = OUT, F2[c1] = OUT;
    if (want_cigar) T.begin_row(i, c0);
    for (int32_t j = c0; j <= c1; ++j) {
      const int32_t sub = (s1[i - 1] == 2 || s2[j - 1] == 2) ? 0 : (s1[i - 1] == s2[j - 1] ? rc.match : rc.mismatch);
      int32_t v = sub + prev[j - 1];
      uint8_t d = 0;
      if (!(v > F1[j])) d = 1, v = F1[j];
      if (!(v > e1)) d = 2, v = e1;
      if (pieces == 2) {
        if (!(v > F2[j])) d = 3, v = F2[j];
        if (!(v > e2)) d = 4, v = e2;
      }
      cur[j] = v;
      if (v > best) best = v, bestj = j;
      int32_t h = v + nc.open1, f = F1[j] + nc.ext1;
      if (f >= h) d |= 1 << 3;
      F1[j] = f >= h ? f : h;
      h = v + rc.open1;
      e1 += rc.ext1;
      if (e1 >= h) d |= 1 << 4;
      e1 = e1 >= h ? e1 : h;
      if (pieces == 2) {
        int32_t h2 = v + nc.open2, f2 = F2[j] + nc.ext2;
        if (f2 >= h2) d |= 1 << 5;
        F2[j] = f2 >= h2 ? f2 : h2;
        h2 = v + rc.open2;
        e2 += rc.ext2;
        if (e2 >= h2) d |= 1 << 6;
        e2 = e2 >= h2 ? e2 : h2;
      }
      if (want_cigar) T.push(i, d);
    }
    o.cells += std::max(c1 - c0 + 1, 0);
    if (best > o.score) {
      o.score = best;
      o.end1 = i;
      o.end2 = bestj;
    }
    if (pieces == 2) {
      int32_t l = (i - o.end1) - (bestj - o.end2);
      l = l > 0 ? l : -l;
      if (o.score - best > rc.zdrop + l * rc.ext2) break;
    } else if (o.score - best > rc.zdrop) {
      break;
    }
    if (bestj <= 0) break;
    std::swap(prev, cur);
    prev[0] = OUT;
    cur[0] = OUT;
  }
  o.cigar.clear();
  if (want_cigar) {
    int32_t ii = o.end1, jj = o.end2;
    walk_codes(T, ii, jj, o.cigar);
    while (ii > 0) cigar_push(o.cigar, 2), --ii;
    while (jj > 0) cigar_push(o.cigar, 1), --jj;
    std::reverse(o.cigar.begin(), o.cigar.end());
  }
  o.end1 -= 1;
  o.end2 -= 1;
}

struct Seed4 {
  int32_t s1, e1, s2, e2;
};

// The reference's Seed ordering (model/Seed.h:29-42): two seeds sharing their start pair or their end pair compare
// "equal"; otherwise lexicographic on (start1, start2).  It is not a strict weak order, so a set's contents depend on
// insertion order and tree shape; every use below replays the reference's exact insertion sequence.
struct SeedLess {
  bool operator()(const Seed4 &a, const Seed4 &b) const {
    if (a.s1 == b.s1 && a.s2 == b.s2) return false;
    if (a.e1 == b.e1 && a.e2 == b.e2) return false;
    if (a.s1 < b.s1) return true;
    if (a.s1 == b.s1) return a.s2 < b.s2;
    return false;
  }
};
using SeedSet = std::set<Seed4, SeedLess>;

struct Pair {
  const int8_t *s1, *s2;
  int32_t n1, n2;
  std::vector<int8_t> rc1, rc2;
  void init() {
    rc1.resize(std::max(n1, 1));
    rc2.resize(std::max(n2, 1));
    for (int32_t i = 0; i < n1; ++i) rc1[i] = (int8_t)(4 - s1[n1 - 1 - i]);
    for (int32_t i = 0; i < n2; ++i) rc2[i] = (int8_t)(4 - s2[n2 - 1 - i]);
  }
};

// Forward scan of window [s2, s2+tw) against reference rows [lo, hi), then the reverse scan that fixes the start.
// Returns true with the seed (absolute 0-based coordinates) when the forward score reaches the minimum.
bool seed_at(const Pair &pr, const Params &P, Score sc, int32_t lo, int32_t hi, int32_t s2, int32_t tw, Seed4 &sd,
             Cells &cells) {
  SwOut f;
  int32_t nref = hi - lo;
  if (tw > 0) {
    sw_dispatch(pr.s1 + lo, nref, pr.s2 + s2, tw, P.open1, P.ext1, sc, f);
    cells.scan += (int64_t)nref * tw;
  } else {
    f.score = 0;
  }
  if (f.score < P.min_score) return false;
  int32_t lim = tw + P.window;
  int32_t r1 = std::min(1 + f.end1, lim), r2 = std::min(1 + f.end2, lim);
  int32_t end1 = lo + f.end1, end2 = s2 + f.end2;
  SwOut r;
  sw_dispatch(pr.rc1.data() + (pr.n1 - 1 - end1), r1, pr.rc2.data() + (pr.n2 - 1 - end2), r2, P.open1, P.ext1, sc, r);
  cells.scan_rev += (int64_t)r1 * r2;
  sd = Seed4{end1 - r.end1, end1, end2 - r.end2, end2};
  return true;
}

SeedSet seeds_recursive(const Pair &pr, const Params &P, Score sc, int32_t lo, int32_t hi, int32_t s2, int32_t tw,
                        Cells &cells) {
  SeedSet local;
  Seed4 sd;
  if (!seed_at(pr, P, sc, lo, hi, s2, tw, sd, cells)) return local;
  const int32_t mini = P.min_score / P.match;
  local.insert(sd);
  if (sd.s1 - lo >= mini)
    for (const Seed4 &x : seeds_recursive(pr, P, sc, lo, sd.s1, s2, tw, cells)) local.insert(x);
  if (hi - sd.e1 - 1 >= mini)
    for (const Seed4 &x : seeds_recursive(pr, P, sc, sd.e1 + 1, hi, s2, tw, cells)) local.insert(x);
  return local;
}

void seeds_gated(const Pair &pr, const Params &P, Score sc, int32_t s2, SeedSet &seeds, Cells &cells) {
  int32_t tw = (s2 + P.window) > pr.n2 ? (pr.n2 - s2) : P.window;
  Seed4 sd;
  if (!seed_at(pr, P, sc, 0, pr.n1, s2, tw, sd, cells)) return;
  if (seeds.find(sd) != seeds.end()) return;
  const int32_t mini = P.min_score / P.match;
  seeds.insert(sd);
  if (sd.s1 >= mini)
    for (const Seed4 &x : seeds_recursive(pr, P, sc, 0, sd.s1, s2, tw, cells)) seeds.insert(x);
  if (pr.n1 - sd.e1 - 1 >= mini)
    for (const Seed4 &x : seeds_recursive(pr, P, sc, sd.e1 + 1, pr.n1, s2, tw, cells)) seeds.insert(x);
}

void link_seeds(SeedSet &seeds) {
  std::vector<Seed4> cur(seeds.begin(), seeds.end());
  std::sort(cur.begin(), cur.end(), [](Seed4 a, Seed4 b) { return a.s1 < b.s1; });
  bool changed = true;
  while (changed) {
    changed = false;
    std::vector<Seed4> next;
    std::set<int> used;
    const int n = (int)cur.size();
    for (int i = 0; i < n; ++i) {
      if (used.count(i)) continue;
      const Seed4 a = cur[i];
      bool merged = false;
      for (int j = i + 1; j < n; ++j) {
        if (used.count(j)) continue;
        const Seed4 b = cur[j];
        if (a.s2 <= b.s2 && a.e1 >= b.e1 && a.e2 >= b.e2) {
          used.insert(j);  // b lies inside a
        } else if (a.s2 <= b.s2 && a.e1 <= b.e1 && a.e2 <= b.e2) {
          int32_t d = b.s1 - a.s1;
          if (d == b.s2 - a.s2 && d == b.e1 - a.e1 && d == b.e2 - a.e2) {  // same diagonal, overlapping: merge
            next.push_back(Seed4{a.s1, b.e1, a.s2, b.e2});
            used.insert(i);
            used.insert(j);
            merged = true;
            break;
          }
        } else if (b.s1 > a.e1 || b.s2 > a.e2) {
          break;
        }
      }
      if (merged)
        changed = true;
      else
        next.push_back(a);
    }
    cur.swap(next);
  }
  seeds.clear();
  for (const Seed4 &s : cur) seeds.insert(s);
}

// Window starts of the 1-gap driver (stop_past_end=true, :462-480) and of getAllExtendSeed (false, :376-390).
void window_starts(int32_t n2, const Params &P, bool stop_past_end, std::vector<int32_t> &starts) {
  starts.clear();
  int32_t s = 0;
  while (true) {
    starts.push_back(s);
    s += P.step;
    if (stop_past_end && s > n2) break;
    if (s + P.window > n2) {
      starts.push_back(s);
      break;
    }
  }
}

SeedSet scan_and_link(const Pair &pr, const Params &P, Score sc, bool one_gap, Cells &cells) {
  SeedSet seeds;
  std::vector<int32_t> starts;
  window_starts(pr.n2, P, one_gap, starts);
  for (int32_t s : starts) seeds_gated(pr, P, sc, s, seeds, cells);
  link_seeds(seeds);
  return seeds;
}

struct Frag {
  int64_t s1, e1, s2, e2, score;  // 1-based
  std::vector<uint32_t> cigar;
  double p, e;
};

inline void evalue(const Params &P, double L1, double L2, int32_t score, double &e, double &p) {
  e = P.kvalue * L1 * L2 * exp(-1.0 * P.lambda * double(score));
  p = 1.0 - exp(-1.0 * e);
}

// x_extend_seed.  Inputs are the extension start (seed start + 1).  Returns false when either pass found nothing.
bool x_extend_seed(const Pair &pr, const Params &P, Score sc, bool want_cigar, int32_t &start1, int32_t &end1,
                   int32_t &start2, int32_t &end2, int32_t &score, std::vector<uint32_t> &cigar, Cells &cells) {
  const int32_t a1 = start1, a2 = start2;
  XOut f, r;
  xextend(pr.s1 + a1, pr.n1 - a1, pr.s2 + a2, pr.n2 - a2, P.open1, P.ext1, sc, P.xdrop, P.w, false, f);
  cells.xdrop += f.cells;
  score = f.score;
  cigar.clear();
  if (f.end1 < 0 || f.end2 < 0) return false;
  const int32_t b1 = a1 + f.end1, b2 = a2 + f.end2;
  xextend(pr.rc1.data() + (pr.n1 - 1 - b1), b1 + 1, pr.rc2.data() + (pr.n2 - 1 - b2), b2 + 1, P.open1, P.ext1, sc,
          P.xdrop, P.w, want_cigar, r);
  cells.xdrop += r.cells;
  score = r.score;
  cigar = r.cigar;
  if (r.end1 < 0 || r.end2 < 0) return false;
  end1 = b1;
  end2 = b2;
  start1 = b1 - r.end1;
  start2 = b2 - r.end2;
  if (want_cigar) {
    end1 -= r.iii;
    end2 -= r.jjj;
  }
  return true;
}

std::vector<Frag> find_1gap(const Pair &pr, const Params &P, Cells &cells) {
  Score sc{P.match, P.mismatch};
  SeedSet seeds = scan_and_link(pr, P, sc, true, cells);
  std::vector<Frag> out;
  const double L1 = double(pr.n1), L2 = double(pr.n2);
  for (const Seed4 &sd : seeds) {
    int32_t s1 = sd.s1 + 1, e1 = sd.e1 + 1, s2 = sd.s2 + 1, e2 = sd.e2 + 1, score = 0;
    std::vector<uint32_t> cg;
    if (!x_extend_seed(pr, P, sc, true, s1, e1, s2, e2, score, cg, cells)) continue;  // p = 100
    double ev, pv;
    evalue(P, L1, L2, score, ev, pv);
    if (!(pv < P.pvalue)) continue;
    Frag fr{s1 + 1, e1 + 1, s2 + 1, e2 + 1, (int64_t)(uint32_t)score, cg, pv, ev};
    bool fresh = true;
    for (Frag &g : out) {
      if (g.s1 == fr.s1 && g.s2 == fr.s2) {
        fresh = false;
        if (e1 >= g.e1 && e2 >= g.e2) g = fr;  // compares the 0-based ends against stored 1-based ends, as in :506
        break;
      } else if (g.e1 == fr.e1 && g.e2 == fr.e2) {
        fresh = false;
        if (s1 <= g.s1 && s2 <= g.s2) g = fr;
        break;
      }
    }
    if (fresh) out.push_back(fr);
  }
  return out;
}

std::vector<Seed4> all_extend_seeds(const Pair &pr, const Params &P, Score sc, Cells &cells) {
  SeedSet seeds = scan_and_link(pr, P, sc, false, cells);
  std::vector<Seed4> xs;
  const double L1 = double(pr.n1), L2 = double(pr.n2);
  for (const Seed4 &sd : seeds) {
    int32_t s1 = sd.s1 + 1, e1 = sd.e1 + 1, s2 = sd.s2 + 1, e2 = sd.e2 + 1, score = 0;
    std::vector<uint32_t> cg;
    if (!x_extend_seed(pr, P, sc, false, s1, e1, s2, e2, score, cg, cells)) continue;
    double ev, pv;
    evalue(P, L1, L2, score, ev, pv);
    if (!(pv < P.pvalue)) continue;
    bool fresh = true;
    for (Seed4 &x : xs) {
      if (x.s1 == s1 && x.s2 == s2) {
        fresh = false;
        if (e1 > x.e1 && e2 > x.e2) {
          x.e1 = e1;
          x.e2 = e2;
        }
      } else if (x.e1 == e1 && x.e2 == e2) {
        if (s1 < x.s1 && s2 < x.s2) {
          x.s1 = s1;
          x.s2 = s2;
        }
        fresh = false;
      }
    }
    if (fresh) xs.push_back(Seed4{s1, e1, s2, e2});
  }
  return xs;
}

std::vector<Frag> two_piece_stage(const Pair &pr, const Params &P, const std::vector<Seed4> &xs, Cells &cells) {
  Score sc{P.match, P.mismatch};
  std::vector<Frag> out;
  std::set<std::pair<int32_t, int32_t>> starts;
  const double L1 = double(pr.n1), L2 = double(pr.n2);
  for (const Seed4 &x : xs) {
    const int32_t b1 = x.e1, b2 = x.e2;
    SgOut r;
    semiglobal(pr.rc1.data() + (pr.n1 - 1 - b1), 1 + b1, pr.rc2.data() + (pr.n2 - b2 - 1), b2 + 1, P, sc, false, r);
    cells.semiglobal += r.cells;
    const int32_t s1 = b1 - r.end1, s2 = b2 - r.end2;
    if (!starts.insert({s1, s2}).second) continue;
    SgOut f;
    semiglobal(pr.s1 + s1, pr.n1 - s1, pr.s2 + s2, pr.n2 - s2, P, sc, true, f);
    cells.semiglobal += f.cells;
    if (!(f.cigar.size() > 0 && f.end1 > 0 && f.end2 > 0)) continue;
    const int64_t e1 = f.end1 + s1, e2 = f.end2 + s2;
    int toRemove = -1;
    bool found = false;
    for (int i = 0; i < (int)out.size(); ++i) {
      if (out[i].e1 == e1 + 1 && out[i].e2 == e2 + 1) {
        found = true;
        if (s1 + 1 < out[i].s1 && s2 + 1 < out[i].s2) toRemove = i;
      }
    }
    if (found && toRemove < 0) continue;
    double ev, pv;
    evalue(P, L1, L2, f.score, ev, pv);
    Frag fr{s1 + 1, e1 + 1, s2 + 1, e2 + 1, (int64_t)(uint32_t)f.score, f.cigar, pv, ev};
    if (toRemove >= 0)
      out[toRemove] = fr;
    else
      out.push_back(fr);
  }
  return out;
}

// The seeded 2-piece overload (findSimilarFragmentsForPairedSequence4.cpp:624-745, driven by cut2Gaps2 with seeds
// read from a SAM file).  Per seed, in order:
//   * skipped when an accepted fragment covers it (:651-659: 1-based fragment coordinates compared with the 0-based
//     seed coordinates, as the reference does);
//   * reverse 2-piece z-drop from the seed end, both lengths min(1 + end, max_align) from the seed's own end; when the
//     two end bases differ the ends move back one base first (:663-667) but the lengths stay;
//   * start = end - reverse end, the StartAlignment gate, a forward 2-piece with CIGAR over
//     min(length - start, max_align), and the dedupe by end of :686-710.  No p-value filter.
// Where the moved-back end would make the reverse DP read before the start of a sequence (the reference reads outside
// its buffer there), the reverse DP is shortened to the bases that exist.
std::vector<Frag> seeded_two_piece(const Pair &pr, const Params &P, int32_t max_align, const std::vector<Seed4> &seeds,
                                   Cells &cells) {
  Score sc{P.match, P.mismatch};
  std::vector<Frag> out;
  std::set<std::pair<int32_t, int32_t>> starts;
  const double L1 = double(pr.n1), L2 = double(pr.n2);
  for (const Seed4 &x : seeds) {
    bool use = true;
    for (const Frag &f : out)
      if (f.s1 <= x.s1 && f.e1 >= x.e1 && f.s2 <= x.s2 && f.e2 >= x.e2) {
        use = false;
        break;
      }
    if (!use) continue;
    int32_t b1 = x.e1, b2 = x.e2;
    int32_t l11 = std::min(1 + b1, max_align), l12 = std::min(1 + b2, max_align);
    if (b1 >= 0 && b1 < pr.n1 && b2 >= 0 && b2 < pr.n2 && pr.rc1[pr.n1 - 1 - b1] != pr.rc2[pr.n2 - b2 - 1]) --b1, --b2;
    l11 = std::max(0, std::min(l11, b1 + 1));
    l12 = std::max(0, std::min(l12, b2 + 1));
    SgOut r;
    semiglobal(pr.rc1.data() + (pr.n1 - 1 - b1), l11, pr.rc2.data() + (pr.n2 - b2 - 1), l12, P, sc, false, r);
    cells.semiglobal += r.cells;
    const int32_t s1 = b1 - r.end1, s2 = b2 - r.end2;
    if (!starts.insert({s1, s2}).second) continue;
    const int32_t l21 = std::min(pr.n1 - s1, max_align), l22 = std::min(pr.n2 - s2, max_align);
    SgOut f;
    semiglobal(pr.s1 + s1, l21, pr.s2 + s2, l22, P, sc, true, f);
    cells.semiglobal += f.cells;
    if (!(f.cigar.size() > 0 && f.end1 > 0 && f.end2 > 0)) continue;
    const int64_t e1 = f.end1 + s1, e2 = f.end2 + s2;
    int toRemove = -1;
    bool found = false;
    for (int i = 0; i < (int)out.size(); ++i)
      if (out[i].e1 == e1 + 1 && out[i].e2 == e2 + 1) {
        found = true;
        if (s1 + 1 < out[i].s1 && s2 + 1 < out[i].s2) toRemove = i;
      }
    if (found && toRemove < 0) continue;
    double ev, pv;
    evalue(P, L1, L2, f.score, ev, pv);
    Frag fr{s1 + 1, e1 + 1, s2 + 1, e2 + 1, (int64_t)(uint32_t)f.score, f.cigar, pv, ev};
    if (toRemove >= 0)
      out[toRemove] = fr;
    else
      out.push_back(fr);
  }
  return out;
}

// The weighted drivers (findSimilarFragmentsForPairedSequence4.cpp:784-881 with pieces = 1, :883-975 with
// pieces = 2): the 2-gap x-seeds, then per x-seed a weighted reverse DP from its end (reverse-complement weights),
// the StartAlignment gate and a weighted forward DP with CIGAR; the 1-piece driver keeps a result without checking
// its CIGAR or ends, the 2-piece one requires a CIGAR and positive ends.  wf / wr: the forward and reverse weights
// of seq1, n1 + 1 entries each (the last repeating the final category).
std::vector<Frag> weighted_stage(int pieces, const Pair &pr, const Params &P, const std::vector<Seed4> &xs,
                                 const int16_t *wf, const int16_t *wr, const WCat *cats, Cells &cells) {
  std::vector<Frag> out;
  std::set<std::pair<int32_t, int32_t>> starts;
  const double L1 = double(pr.n1), L2 = double(pr.n2);
  for (const Seed4 &x : xs) {
    const int32_t b1 = x.e1, b2 = x.e2;
    SgOut r;
    weighted_semiglobal(pieces, pr.rc1.data() + (pr.n1 - 1 - b1), 1 + b1, pr.rc2.data() + (pr.n2 - b2 - 1), b2 + 1,
                        wr + (pr.n1 - 1 - b1), cats, P.bandwidth, false, r);
    cells.semiglobal += r.cells;
    const int32_t s1 = b1 - r.end1, s2 = b2 - r.end2;
    if (!starts.insert({s1, s2}).second) continue;
    SgOut f;
    weighted_semiglobal(pieces, pr.s1 + s1, pr.n1 - s1, pr.s2 + s2, pr.n2 - s2, wf + s1, cats, P.bandwidth, true, f);
    cells.semiglobal += f.cells;
    if (pieces == 2 && !(f.cigar.size() > 0 && f.end1 > 0 && f.end2 > 0)) continue;
    const int64_t e1 = (int64_t)f.end1 + s1, e2 = (int64_t)f.end2 + s2;
    int toRemove = -1;
    bool found = false;
    for (int i = 0; i < (int)out.size(); ++i)
      if (out[i].e1 == e1 + 1 && out[i].e2 == e2 + 1) {
        found = true;
        if (s1 + 1 < out[i].s1 && s2 + 1 < out[i].s2) toRemove = i;
      }
    if (found && toRemove < 0) continue;
    double ev, pv;
    evalue(P, L1, L2, f.score, ev, pv);
    Frag fr{s1 + 1, e1 + 1, s2 + 1, e2 + 1, (int64_t)(uint32_t)f.score, f.cigar, pv, ev};
    if (toRemove >= 0)
      out[toRemove] = fr;
    else
      out.push_back(fr);
  }
  return out;
}

std::vector<Frag> find_2gap(const Pair &pr, const Params &P, Cells &cells) {
  Score sc{P.match, P.mismatch};
  std::vector<Seed4> xs = all_extend_seeds(pr, P, sc, cells);
  return two_piece_stage(pr, P, xs, cells);
}

int flatten(const std::vector<Frag> &fr, int64_t *frag, double *pe, uint32_t *cigar, int frag_cap, int cigar_cap,
            int *n_cigar_out) {
  int nc = 0;
  for (const Frag &f : fr) nc += (int)f.cigar.size();
  *n_cigar_out = nc;
  if ((int)fr.size() > frag_cap || nc > cigar_cap) return -(int)fr.size() - 1;
  int off = 0;
  for (size_t i = 0; i < fr.size(); ++i) {
    const Frag &f = fr[i];
    int64_t *r = frag + i * 8;
    r[0] = f.s1;
    r[1] = f.e1;
    r[2] = f.s2;
    r[3] = f.e2;
    r[4] = f.score;
    r[5] = off;
    r[6] = (int64_t)f.cigar.size();
    r[7] = 0;
    pe[i * 2] = f.p;
    pe[i * 2 + 1] = f.e;
    for (uint32_t c : f.cigar) cigar[off++] = c;
  }
  return (int)fr.size();
}

Params params_from(const int32_t *ip, const double *dp) {
  Params P;
  P.match = ip[0];
  P.mismatch = ip[1];
  P.open1 = ip[2];
  P.ext1 = ip[3];
  P.open2 = ip[4];
  P.ext2 = ip[5];
  P.window = ip[6];
  P.min_score = ip[7];
  P.step = ip[8];
  P.w = ip[9];
  P.xdrop = ip[10];
  P.zdrop = ip[11];
  P.bandwidth = ip[12];
  P.pvalue = dp[0];
  P.lambda = dp[1];
  P.kvalue = dp[2];
  return P;
}

void cells_out(const Cells &c, int64_t *out) {
  if (!out) return;
  out[0] = c.scan;
  out[1] = c.scan_rev;
  out[2] = c.xdrop;
  out[3] = c.semiglobal;
}

}  // namespace

// ---------------------------------------------------------------- C entry points (ctypes, see oracle/oracle.py)
// Integer params ip[13] = match, mismatch, open1, ext1, open2, ext2, window, min_score, step, w, xdrop, zdrop,
// bandwidth; double params dp[3] = pvalue, lambda, kvalue.  cells[4] = scan, scan_rev, xdrop, semiglobal.
extern "C" {

int or_sw(const int8_t *ref, int32_t nref, const int8_t *read, int32_t nread, int open, int ext, int match,
          int mismatch, int mode, int32_t *out) {
  Score sc{match, mismatch};
  SwOut o{0, -7, -7};
  if (mode == 1)
    sw_striped_semantics(ref, nref, read, nread, open, ext, sc, o);
  else if (mode == 2)
    sw_scalar_semantics(ref, nref, read, nread, open, ext, sc, o);
  else
    sw_dispatch(ref, nref, read, nread, open, ext, sc, o);
  out[0] = o.score;
  out[1] = o.end1;
  out[2] = o.end2;
  return 0;
}

int or_xextend(const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, int open, int ext, int match, int mismatch,
               int xdrop, int w, int want_cigar, uint32_t *cigar, int cigar_cap, int32_t *out) {
  Score sc{match, mismatch};
  XOut o;
  xextend(s1, n1, s2, n2, open, ext, sc, xdrop, w, want_cigar != 0, o);
  out[0] = o.score;
  out[1] = o.end1;
  out[2] = o.end2;
  out[3] = want_cigar ? o.iii : 0;
  out[4] = want_cigar ? o.jjj : 0;
  out[5] = (int32_t)o.cigar.size();
  out[6] = (int32_t)o.cells;
  if ((int)o.cigar.size() > cigar_cap) return -1;
  for (size_t i = 0; i < o.cigar.size(); ++i) cigar[i] = o.cigar[i];
  return 0;
}

// x_extend_seed's two DP passes (impl/findSimilarFragmentsForPairedSequence4.cpp:245-285 calls SemiGlobal_xextend
// forward without, then again with the traceback) over n independent tasks on `threads` threads, tasks taken in
// order from a shared counter.  out[k] = score of the traceback pass; cells_o[0] = the algorithmic band cells of both
// passes; the checksum folds every task's integer outputs and CIGAR words.
int or_xextend_batch(int n, const int8_t *const *s1, const int32_t *n1, const int8_t *const *s2, const int32_t *n2,
                     int open, int ext, int match, int mismatch, int xdrop, int w, int threads, int32_t *out,
                     uint64_t *checksum_out, int64_t *cells_o) {
  Score sc{match, mismatch};
  std::atomic<int> next(0);
  const int nt = std::max(threads, 1);
  std::vector<int64_t> cells(nt, 0);
  std::vector<uint64_t> sums(nt, 0);
  auto work = [&](int t) {
    for (int k; (k = next.fetch_add(1)) < n;) {
      uint64_t h = 1469598103934665603ull;
      for (int pass = 0; pass < 2; ++pass) {
        XOut o;
        xextend(s1[k], n1[k], s2[k], n2[k], open, ext, sc, xdrop, w, pass == 1, o);
        cells[t] += o.cells;
        for (int64_t v : {(int64_t)o.score, (int64_t)o.end1, (int64_t)o.end2, (int64_t)o.iii, (int64_t)o.jjj})
          h = (h ^ (uint64_t)v) * 1099511628211ull;
        for (uint32_t c : o.cigar) h = (h ^ c) * 1099511628211ull;
        if (pass == 1) out[k] = o.score;
      }
      sums[t] += h;
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto &th : pool) th.join();
  int64_t tot = 0;
  uint64_t sum = 0;
  for (int t = 0; t < nt; ++t) tot += cells[t], sum += sums[t];
  cells_o[0] = tot;
  *checksum_out = sum;
  return 0;
}

int or_semiglobal(const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, const int32_t *ip, const double *dp,
                  int want_cigar, uint32_t *cigar, int cigar_cap, int32_t *out) {
  Params P = params_from(ip, dp);
  Score sc{P.match, P.mismatch};
  SgOut o;
  semiglobal(s1, n1, s2, n2, P, sc, want_cigar != 0, o);
  out[0] = o.score;
  out[1] = o.end1;
  out[2] = o.end2;
  out[3] = (int32_t)o.cigar.size();
  if ((int)o.cigar.size() > cigar_cap) return -1;
  for (size_t i = 0; i < o.cigar.size(); ++i) cigar[i] = o.cigar[i];
  return 0;
}

int or_seeds(const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, const int32_t *ip, const double *dp,
             int one_gap, int32_t *raw, int raw_cap, int32_t *linked, int linked_cap, int32_t *n_linked) {
  Params P = params_from(ip, dp);
  Score sc{P.match, P.mismatch};
  Pair pr{s1, s2, n1, n2, {}, {}};
  pr.init();
  Cells cells;
  SeedSet seeds;
  std::vector<int32_t> starts;
  window_starts(n2, P, one_gap != 0, starts);
  for (int32_t s : starts) seeds_gated(pr, P, sc, s, seeds, cells);
  int n = 0;
  for (const Seed4 &s : seeds) {
    if (n < raw_cap) std::memcpy(raw + n * 4, &s, 16);
    ++n;
  }
  link_seeds(seeds);
  int k = 0;
  for (const Seed4 &s : seeds) {
    if (k < linked_cap) std::memcpy(linked + k * 4, &s, 16);
    ++k;
  }
  *n_linked = k;
  return n;
}

int or_find(const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, const int32_t *ip, const double *dp,
            int two_gap, int64_t *frag, double *pe, uint32_t *cigar, int frag_cap, int cigar_cap, int *n_cigar,
            int64_t *cells_o) {
  Params P = params_from(ip, dp);
  Pair pr{s1, s2, n1, n2, {}, {}};
  pr.init();
  Cells cells;
  std::vector<Frag> fr = two_gap ? find_2gap(pr, P, cells) : find_1gap(pr, P, cells);
  cells_out(cells, cells_o);
  return flatten(fr, frag, pe, cigar, frag_cap, cigar_cap, n_cigar);
}

// seeds: n_seeds quadruples (start1, end1, start2, end2), 0-based inclusive, in the order the caller read them.
int or_find_seeded_2gap(const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, const int32_t *seeds,
                        int32_t n_seeds, int32_t max_align, const int32_t *ip, const double *dp, int64_t *frag,
                        double *pe, uint32_t *cigar, int frag_cap, int cigar_cap, int *n_cigar, int64_t *cells_o) {
  Params P = params_from(ip, dp);
  Pair pr{s1, s2, n1, n2, {}, {}};
  pr.init();
  std::vector<Seed4> sd(n_seeds);
  for (int32_t k = 0; k < n_seeds; ++k) sd[k] = Seed4{seeds[4 * k], seeds[4 * k + 1], seeds[4 * k + 2], seeds[4 * k + 3]};
  Cells cells;
  std::vector<Frag> fr = seeded_two_piece(pr, P, max_align, sd, cells);
  cells_out(cells, cells_o);
  return flatten(fr, frag, pe, cigar, frag_cap, cigar_cap, n_cigar);
}

// The x-seed overload without maximumAlignLength (two_piece_stage) on caller-given x-seeds, 0-based, in order.
int or_find_xseeds_2gap(const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, const int32_t *seeds,
                        int32_t n_seeds, const int32_t *ip, const double *dp, int64_t *frag, double *pe,
                        uint32_t *cigar, int frag_cap, int cigar_cap, int *n_cigar, int64_t *cells_o) {
  Params P = params_from(ip, dp);
  Pair pr{s1, s2, n1, n2, {}, {}};
  pr.init();
  std::vector<Seed4> sd(n_seeds);
  for (int32_t k = 0; k < n_seeds; ++k) sd[k] = Seed4{seeds[4 * k], seeds[4 * k + 1], seeds[4 * k + 2], seeds[4 * k + 3]};
  Cells cells;
  std::vector<Frag> fr = two_piece_stage(pr, P, sd, cells);
  cells_out(cells, cells_o);
  return flatten(fr, frag, pe, cigar, frag_cap, cigar_cap, n_cigar);
}

// Weighted drivers.  weights: n1 category ids of seq1 (0 .. n_cats-1); cats: 7 ints per category (match, mismatch,
// open1, ext1, open2, ext2, zdrop).  pieces 1 = the 1-gap weighted driver, 2 = the 2-gap one.
int or_find_weighted(int pieces, const int8_t *s1, int32_t n1, const int8_t *s2, int32_t n2, const int16_t *weights,
                     const int32_t *cats, int32_t n_cats, const int32_t *ip, const double *dp, int64_t *frag,
                     double *pe, uint32_t *cigar, int frag_cap, int cigar_cap, int *n_cigar, int64_t *cells_o) {
  Params P = params_from(ip, dp);
  Pair pr{s1, s2, n1, n2, {}, {}};
  pr.init();
  std::vector<WCat> cv(n_cats);
  for (int32_t k = 0; k < n_cats; ++k)
    cv[k] = WCat{cats[7 * k], cats[7 * k + 1], cats[7 * k + 2], cats[7 * k + 3], cats[7 * k + 4], cats[7 * k + 5],
                 cats[7 * k + 6]};
  std::vector<int16_t> wf(n1 + 1), wr(n1 + 1);
  for (int32_t i = 0; i < n1; ++i) wf[i] = weights[i], wr[i] = weights[n1 - 1 - i];
  if (n1 > 0) wf[n1] = wf[n1 - 1], wr[n1] = wr[n1 - 1];
  Cells cells;
  Score sc{P.match, P.mismatch};
  std::vector<Seed4> xs = all_extend_seeds(pr, P, sc, cells);
  std::vector<Frag> fr = weighted_stage(pieces, pr, P, xs, wf.data(), wr.data(), cv.data(), cells);
  cells_out(cells, cells_o);
  return flatten(fr, frag, pe, cigar, frag_cap, cigar_cap, n_cigar);
}

// CPU baseline: the pairs are independent (the reference's own scale-out is one process per pair), so each of
// `threads` workers takes the next pair index.  Per pair it returns the fragment count; fragments are discarded
// except for a checksum over (start1, end1, start2, end2, score, cigar) so the work cannot be elided.
int or_find_batch(int npairs, const int8_t *const *s1, const int32_t *n1, const int8_t *const *s2, const int32_t *n2,
                  const int32_t *ip, const double *dp, int two_gap, int threads, int32_t *nfrag_out,
                  uint64_t *checksum_out, int64_t *cells_o) {
  Params P = params_from(ip, dp);
  std::atomic<int> next(0);
  std::vector<Cells> per(std::max(threads, 1));
  std::vector<uint64_t> sums(std::max(threads, 1), 0);
  auto work = [&](int t) {
    for (int k; (k = next.fetch_add(1)) < npairs;) {
      Pair pr{s1[k], s2[k], n1[k], n2[k], {}, {}};
      pr.init();
      std::vector<Frag> fr = two_gap ? find_2gap(pr, P, per[t]) : find_1gap(pr, P, per[t]);
      nfrag_out[k] = (int32_t)fr.size();
      uint64_t h = 1469598103934665603ull;
      for (const Frag &f : fr) {
        for (int64_t v : {f.s1, f.e1, f.s2, f.e2, f.score}) h = (h ^ (uint64_t)v) * 1099511628211ull;
        for (uint32_t c : f.cigar) h = (h ^ c) * 1099511628211ull;
      }
      sums[t] += h;
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto &th : pool) th.join();
  Cells tot;
  uint64_t sum = 0;
  for (int t = 0; t < std::max(threads, 1); ++t) {
    tot.scan += per[t].scan;
    tot.scan_rev += per[t].scan_rev;
    tot.xdrop += per[t].xdrop;
    tot.semiglobal += per[t].semiglobal;
    sum += sums[t];
  }
  cells_out(tot, cells_o);
  *checksum_out = sum;
  return 0;
}

// Per-window scores of slidingWindowAlignment for one (reference, other) pair: score[k] = max / (min(tw, n_other) *
// match) for window k, with the window length shrinking (and staying shrunk) at the reference's end.
int or_sliding(const int8_t *ref, int32_t nref, const int8_t *other, int32_t nother, int window, int step, int open,
               int ext, int match, int mismatch, double *score, int32_t *maxes, int cap) {
  Score sc{match, mismatch};
  int32_t tw = window;
  int k = 0;
  for (int32_t j = 0; j < nref; j += step) {
    if (tw + j > nref) tw = nref - j;
    SwOut o;
    sw_dispatch(other, nother, ref + j, tw, open, ext, sc, o);
    if (k < cap) {
      maxes[k] = o.score;
      score[k] = double(o.score) / double(std::min(tw, nother) * match);
    }
    ++k;
  }
  return k;
}

}  // extern "C"
