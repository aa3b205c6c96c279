// Adaptive-band x-drop seed extension (SemiGlobal_xextend, impl/sequenceAlignment3.cpp:1234-1451, driven by
// x_extend_seed, impl/findSimilarFragmentsForPairedSequence4.cpp:205-285) and its traceback.
//
// Three forms of a pass, chosen by band half-width w in the chained levels:
//   w <= 20      one thread per pass, the band in registers;
//   20 < w <= 256  one warp per pass as an anti-diagonal wavefront over 32-row stripes (xdrop_level_wave_kernel);
//   w > 256      one warp per pass across the band, the band rows in global scratch (xdrop_level_warp_kernel).
// The thread form stores the band diagonal-relative: index k = j - i + w, so the diagonal predecessor of (i, j) sits
// at the same index in the previous row and the vertical predecessor at k + 1, and both arrays update in place left
// to right.  Outside the chained levels (retries, the kernel-level entry) wide bands use a per-thread global scratch.
//
// A pass ends in one of three states: done, "restart" (the row maximum touched a band edge: the reference recomputes
// from scratch with 2w, and so does the host by relaunching the seed with the doubled width), or "slot too small"
// (the reverse pass's direction codes outgrew the seed's traceback slot; the host relaunches it with a larger one).
//
// Direction codes (reverse pass) are 4-bit nibbles per band cell: bits 0-1 = winning state (0 diag, 1 vertical,
// 2 horizontal), bit 2 = vertical gap extended, bit 3 = horizontal gap extended; state 3 marks cells the reference
// never writes (its Matrix::reset value 255).  Eight nibbles per word, ceil((2w+1)/8) words per row.
#include <algorithm>

#include "device_common.cuh"

namespace dcns {

__device__ __forceinline__ int xd_words_per_row(int w) { return (2 * w + 1 + 7) / 8; }

// One pass on the register path (band capacity WC: w <= WC), advanced a row at a time.  The band arrays stay with the
// caller (locals: registers).
template <int WC>
struct XBand {
  static constexpr int NA = 2 * WC + 2, NK = 2 * WC + 1, NQ = (2 * WC + 1 + 15) / 16;
};

struct XPassScalars {
  SeqView s1, s2;
  int64_t tb_off;
  int32_t n1, n2, w, nk, wpr, tb_cap, i, score, e1, e2, rows;
  bool codes;
};

// M, F: the band of the row above, diagonal-relative; qw: query codes under the band, 4 bits per band cell k
// (column j = i - w + k).
template <int WC>
__device__ __forceinline__ void xd_begin(XPassScalars &x, int32_t (&M)[XBand<WC>::NA], int32_t (&F)[XBand<WC>::NA],
                                         uint64_t (&qw)[XBand<WC>::NQ], const XTask &T, const Arena &ar) {
  constexpr int NA = XBand<WC>::NA, NK = XBand<WC>::NK, NQ = XBand<WC>::NQ;
  x.n1 = T.n1, x.n2 = T.n2, x.w = T.w, x.nk = 2 * T.w + 1, x.wpr = xd_words_per_row(T.w);
  x.codes = T.want_codes != 0, x.tb_off = T.tb_off, x.tb_cap = T.tb_cap;
  x.s1 = SeqView{T.base1, T.a1, T.dir}, x.s2 = SeqView{T.base2, T.a2, T.dir};
  x.score = x.e1 = x.e2 = x.rows = 0;
  x.i = 1;
#pragma unroll
  for (int k = 0; k < NA; ++k) M[k] = kOut, F[k] = kOut;
#pragma unroll
  for (int u = 0; u < NQ; ++u) qw[u] = 0;
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    const int j = 1 - x.w + k;
    if (k < x.nk && j >= 1 && j <= x.n2) qw[k >> 4] |= (uint64_t)x.s2.at(ar, j - 1) << (4 * (k & 15));
  }
}

// Row x.i.  Returns -1 to go on, 0 done, 1 band-edge restart, 2 traceback slot too small.
//
// The cells are the reference's, with the row's serial chain cut to one add-max per cell: with A = max(s + diag,
// F above) (the first two comparisons), the e update e' = max(e + ext, max(A, e) + open) equals max(e + g, A + open),
// g = max(ext, open), whether A > e or not.  Every A comes from the row above, so the chain waits on nothing else; M,
// F, the codes and the row maximum then follow per cell with the reference's comparisons and tie rules.
template <int WC>
__device__ __forceinline__ int xd_row(XPassScalars &x, int32_t (&M)[XBand<WC>::NA], int32_t (&F)[XBand<WC>::NA],
                                      uint64_t (&qw)[XBand<WC>::NQ], const Arena &ar, const Params &P,
                                      uint32_t *__restrict__ tb) {
  constexpr int NK = XBand<WC>::NK, NQ = XBand<WC>::NQ;
  const int i = x.i, w = x.w, nk = x.nk, n2 = x.n2;
  if (i > x.n1) return 0;
  const int c0 = max(i - w, 1), c1 = min(i + w, n2);
  if (x.codes && (int64_t)i * x.wpr > x.tb_cap) return 2;
  const int open = P.open1, ext = P.ext1, g = ext > open ? ext : open;
  const int ci = x.s1.at(ar, i - 1);
  int best = 0, bestj = -1;
  int32_t A[NK], E[NK];
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    const int j = i - w + k;
    const int cj = (int)((qw[k >> 4] >> (4 * (k & 15))) & 15u);
    const int32_t diag = (j == 1) ? (i == 1 ? 0 : kOut) : M[k];
    const int32_t fin = (j == c1) ? kOut : F[k + 1];
    const int32_t v = score_of(ci, cj, P.match, P.mismatch) + diag;
    A[k] = v > fin ? v : fin;
  }
  int32_t ec = kOut;
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    E[k] = ec;
    const int j = i - w + k;
    if (k < nk && j >= c0 && j <= c1) ec = max(ec + g, A[k] + open);
  }
  uint32_t cw = 0;
  int kw = 0;
  uint32_t *row_codes = tb + x.tb_off + (int64_t)(i - 1) * x.wpr;
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    const int j = i - w + k;
    uint32_t nib = 0xFu;
    if (k < nk && j >= c0 && j <= c1) {
      // M[k] and F[k + 1] still hold the row above here
      const int cj = (int)((qw[k >> 4] >> (4 * (k & 15))) & 15u);
      const int32_t diag = (j == 1) ? (i == 1 ? 0 : kOut) : M[k];
      const int32_t fin = (j == c1) ? kOut : F[k + 1];
      const bool ge = !(A[k] > E[k]);  // the horizontal gap wins ties
      const int32_t v = ge ? E[k] : A[k];
      uint32_t d = ge ? 2u : (score_of(ci, cj, P.match, P.mismatch) + diag > fin ? 0u : 1u);
      M[k] = v;
      if (v > best) {
        best = v;
        bestj = j;
      }
      const int32_t h = v + open;
      const int32_t f = fin + ext;
      if (f >= h) d |= 4u;
      F[k] = f >= h ? f : h;
      if (E[k] + ext >= h) d |= 8u;
      nib = d;
    }
    if (x.codes && k < nk) {
      cw |= nib << (4 * (k & 7));
      if ((k & 7) == 7 || k == nk - 1) {
        row_codes[kw++] = cw;
        cw = 0;
      }
    }
  }
  // next row's band starts one column to the right: drop cell 0, append column (i + 1) + w
#pragma unroll
  for (int u = 0; u < NQ; ++u) qw[u] = (qw[u] >> 4) | (u + 1 < NQ ? qw[u + 1] << 60 : 0ull);
  const int jn = i + 1 + w;
  if (jn <= n2) {
    const int kl = nk - 1;
#pragma unroll
    for (int u = 0; u < NQ; ++u)
      if (u == (kl >> 4)) qw[u] |= (uint64_t)x.s2.at(ar, jn - 1) << (4 * (kl & 15));
  }
  x.rows = i;
  if (bestj != n2 && bestj != 1 && (bestj == c0 || bestj == c1)) return 1;
  if (best > x.score) {
    x.score = best;
    x.e1 = i;
    x.e2 = bestj;
  }
  if (x.score - best > P.xdrop) return 0;
  if (best <= 0) return 0;
  x.i = i + 1;
  return -1;
}

// Row x.i as one left-to-right loop: the same cells, comparisons and tie rules as xd_row, with A (the diagonal /
// vertical choice) and the incoming horizontal gap e of each cell kept in registers for that cell only, so the band
// arrays are the only per-cell state (a third of xd_row's registers: more warps per SM).  Returns as xd_row.
// CODES = false (the forward passes, which keep no direction codes) leaves out the codes and their comparisons.
template <int WC, bool CODES>
__device__ __forceinline__ int xd_row_fused(XPassScalars &x, int32_t (&M)[XBand<WC>::NA], int32_t (&F)[XBand<WC>::NA],
                                            uint64_t (&qw)[XBand<WC>::NQ], const Arena &ar, const Params &P,
                                            uint32_t *__restrict__ tb) {
  constexpr int NK = XBand<WC>::NK, NQ = XBand<WC>::NQ;
  const int i = x.i, w = x.w, nk = x.nk, n2 = x.n2;
  if (i > x.n1) return 0;
  const int c0 = max(i - w, 1), c1 = min(i + w, n2);
  const bool codes = CODES && x.codes;
  if (codes && (int64_t)i * x.wpr > x.tb_cap) return 2;
  const int open = P.open1, ext = P.ext1, g = ext > open ? ext : open;
  const int ci = x.s1.at(ar, i - 1);
  int best = 0, bestj = -1;
  int32_t ec = kOut;  // e entering the cell: the reference starts each row with e = OUT
  uint32_t cw = 0;
  int kw = 0;
  uint32_t *row_codes = tb + x.tb_off + (int64_t)(i - 1) * x.wpr;
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    const int j = i - w + k;
    uint32_t nib = 0xFu;
    // k in [0, 2w] puts j in [i - w, i + w], so the band test is 1 <= j <= n2
    if (k < nk && (unsigned)(j - 1) < (unsigned)n2) {
      // M[k] and F[k + 1] still hold the row above: F[k + 1] is rewritten at the next cell
      const int cj = (int)((qw[k >> 4] >> (4 * (k & 15))) & 15u);
      const int32_t diag = (j == 1) ? (i == 1 ? 0 : kOut) : M[k];
      const int32_t fin = (j == c1) ? kOut : F[k + 1];
      const int32_t sd = score_of(ci, cj, P.match, P.mismatch) + diag;
      const int32_t A = sd > fin ? sd : fin;
      const bool ge = !(A > ec);  // the horizontal gap wins ties
      const int32_t v = ge ? ec : A;
      M[k] = v;
      if (v > best) {
        best = v;
        bestj = j;
      }
      const int32_t h = v + open;
      const int32_t f = fin + ext;
      F[k] = f >= h ? f : h;
      if constexpr (CODES) {
        uint32_t d = ge ? 2u : (sd > fin ? 0u : 1u);
        if (f >= h) d |= 4u;
        if (ec + ext >= h) d |= 8u;
        nib = d;
      }
      ec = max(ec + g, A + open);  // = max(e + ext, max(A, e) + open), the reference's e update
    }
    if (CODES && codes && k < nk) {
      cw |= nib << (4 * (k & 7));
      if ((k & 7) == 7 || k == nk - 1) {
        row_codes[kw++] = cw;
        cw = 0;
      }
    }
  }
#pragma unroll
  for (int u = 0; u < NQ; ++u) qw[u] = (qw[u] >> 4) | (u + 1 < NQ ? qw[u + 1] << 60 : 0ull);
  const int jn = i + 1 + w;
  if (jn <= n2) {
    const int kl = nk - 1;
#pragma unroll
    for (int u = 0; u < NQ; ++u)
      if (u == (kl >> 4)) qw[u] |= (uint64_t)x.s2.at(ar, jn - 1) << (4 * (kl & 15));
  }
  x.rows = i;
  if (bestj != n2 && bestj != 1 && (bestj == c0 || bestj == c1)) return 1;
  if (best > x.score) {
    x.score = best;
    x.e1 = i;
    x.e2 = bestj;
  }
  if (x.score - best > P.xdrop) return 0;
  if (best <= 0) return 0;
  x.i = i + 1;
  return -1;
}

__device__ __forceinline__ void xd_finish(const XPassScalars &x, XTask &T, int status) {
  T.status = status;
  T.rows = x.rows;
  if (status == 0) {
    T.score = x.score;
    T.end1 = x.e1;
    T.end2 = x.e2;
  }
}

template <int WC>
__device__ void xdrop_pass(XTask &T, const Arena &ar, const Params &P, uint32_t *__restrict__ tb, int32_t *M,
                           int32_t *F) {
  if constexpr (WC > 0) {
    XPassScalars x;
    int32_t Mr[XBand<WC>::NA], Fr[XBand<WC>::NA];
    uint64_t qw[XBand<WC>::NQ];
    xd_begin<WC>(x, Mr, Fr, qw, T, ar);
    int st;
    while ((st = xd_row<WC>(x, Mr, Fr, qw, ar, P, tb)) < 0) {
    }
    xd_finish(x, T, st);
  } else {
    // wide band in per-thread global scratch (M, F: 2w + 2 ints each)
    const int w = T.w, n1 = T.n1, n2 = T.n2;
    const int open = P.open1, ext = P.ext1;
    const SeqView s1{T.base1, T.a1, T.dir}, s2{T.base2, T.a2, T.dir};
    const int nk = 2 * w + 1;
    for (int k = 0; k < nk + 1; ++k) M[k] = kOut, F[k] = kOut;
    const int wpr = xd_words_per_row(w);
    int score = 0, e1 = 0, e2 = 0, rows = 0;
    T.status = 0;
    for (int i = 1; i <= n1; ++i) {
      const int c0 = max(i - w, 1), c1 = min(i + w, n2);
      if (T.want_codes && (int64_t)i * wpr > T.tb_cap) {
        T.status = 2;
        T.rows = rows;
        return;
      }
      const int ci = s1.at(ar, i - 1);
      int best = 0, bestj = -1, e = kOut;
      uint32_t cw = 0;
      int kw = 0;
      uint32_t *row_codes = tb + T.tb_off + (int64_t)(i - 1) * wpr;
      for (int k = 0; k < nk; ++k) {
        const int j = i - w + k;
        const int cj = (j >= 1 && j <= n2) ? s2.at(ar, j - 1) : 0;
        uint32_t nib = 0xFu;
        if (j >= c0 && j <= c1) {
          const int32_t diag = (j == 1) ? (i == 1 ? 0 : kOut) : M[k];
          const int32_t fin = (j == c1) ? kOut : F[k + 1];
          int32_t v = score_of(ci, cj, P.match, P.mismatch) + diag;
          uint32_t d = v > fin ? 0u : 1u;
          if (!(v > fin)) v = fin;
          if (!(v > e)) {
            d = 2u;
            v = e;
          }
          M[k] = v;
          if (v > best) {
            best = v;
            bestj = j;
          }
          const int32_t h = v + open;
          const int32_t f = fin + ext;
          if (f >= h) d |= 4u;
          F[k] = f >= h ? f : h;
          e += ext;
          if (e >= h) d |= 8u;
          e = e >= h ? e : h;
          nib = d;
        }
        if (T.want_codes) {
          cw |= nib << (4 * (k & 7));
          if ((k & 7) == 7 || k == nk - 1) {
            row_codes[kw++] = cw;
            cw = 0;
          }
        }
      }
      rows = i;
      if (bestj != n2 && bestj != 1 && (bestj == c0 || bestj == c1)) {
        T.status = 1;
        T.rows = rows;
        return;
      }
      if (best > score) {
        score = best;
        e1 = i;
        e2 = bestj;
      }
      if (score - best > P.xdrop) break;
      if (best <= 0) break;
    }
    T.score = score;
    T.end1 = e1;
    T.end2 = e2;
    T.rows = rows;
  }
}

template <int WC>
__global__ void __launch_bounds__(128) xdrop_kernel(XTask *__restrict__ tasks, const int *__restrict__ idx, int n,
                                                    Arena ar, Params P, uint32_t *__restrict__ tb, int32_t *scratch,
                                                    int64_t per_thread) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  XTask &T = tasks[idx[k]];
  int32_t *Ms = nullptr, *Fs = nullptr;
  if (WC == 0) {  // per_thread >= 2 * (2w + 2) for every task of the launch
    Ms = scratch + per_thread * k;
    Fs = Ms + per_thread / 2;
  }
  xdrop_pass<WC>(T, ar, P, tb, Ms, Fs);
}

// ------------------------------------------------------------------ wide bands: one warp per pass
// Lanes own consecutive band cells, 4 per lane in segments of 128.  The horizontal gap chain of a row,
//   e_{j+1} = max(e_j + g, A_j + open),  g = max(ext, open),  A_j = max(s + diag, F_above)
// (the value form of e += ext; e = max(e, M + open) with M = max(A, e)), is an affine map in max-plus algebra,
// f(e) = max(e + a, b); a lane's cells compose into one map, an exclusive warp scan of the maps gives every lane its
// incoming e, and the lane then replays its cells with the reference's exact comparisons.  Cells left of the row's
// first column reset e to OUT, as the reference starts each row with e = OUT.
constexpr int kXwSeg = 4;
constexpr int32_t kNegInf = -(1 << 30);

struct AffMax {
  int32_t a, b;  // e -> max(e + a, b); a <= kNegInf means "independent of e"
};

__device__ __forceinline__ int32_t aff_apply(AffMax f, int32_t e) {
  return f.a <= kNegInf ? f.b : max(e + f.a, f.b);
}
// g after f
__device__ __forceinline__ AffMax aff_then(AffMax f, AffMax g) {
  AffMax r;
  r.a = (f.a <= kNegInf || g.a <= kNegInf) ? kNegInf : f.a + g.a;
  r.b = (g.a <= kNegInf) ? g.b : max(f.b + g.a, g.b);
  return r;
}

// One pass of task T by the calling warp; M and F are the warp's scratch (2w + 2 ints each).  Lane 0 writes the
// pass's results into T.
__device__ void xdrop_warp_pass(XTask &T, const Arena &ar, const Params &P, uint32_t *__restrict__ tb,
                                int32_t *__restrict__ M, int32_t *__restrict__ F) {
  const int lane = threadIdx.x & 31;
  const int w = T.w, n1 = T.n1, n2 = T.n2, nk = 2 * w + 1;
  const int open = P.open1, ext = P.ext1, g = max(P.ext1, P.open1);
  const SeqView s1{T.base1, T.a1, T.dir}, s2{T.base2, T.a2, T.dir};
  for (int k = lane; k <= nk; k += 32) M[k] = kOut, F[k] = kOut;
  __syncwarp();
  const int wpr = xd_words_per_row(w);
  int score = 0, e1 = 0, e2 = 0, rows = 0, status = 0;
  for (int i = 1; i <= n1; ++i) {
    const int c0 = max(i - w, 1), c1 = min(i + w, n2);
    if (T.want_codes && (int64_t)i * wpr > T.tb_cap) {
      status = 2;
      break;
    }
    const int ci = s1.at(ar, i - 1);
    uint32_t *row_codes = tb + T.tb_off + (int64_t)(i - 1) * wpr;
    int32_t ecarry = kOut;  // e entering the segment's first cell
    int lbest = 0, lbestj = -1;
    for (int seg = 0; seg < nk; seg += 32 * kXwSeg) {
      const int k0 = seg + kXwSeg * lane;
      int32_t Mk[kXwSeg], Fk[kXwSeg];
#pragma unroll
      for (int q = 0; q < kXwSeg; ++q) {
        const int k = k0 + q;
        Mk[q] = k < nk ? M[k] : kOut;
        Fk[q] = k < nk ? F[k + 1] : kOut;
      }
      __syncwarp();  // every old value is read before any cell of this segment is rewritten
      // this lane's cells as one affine map of the incoming e
      AffMax f{0, kNegInf};
      int32_t A[kXwSeg], sv[kXwSeg], fin[kXwSeg];
      bool valid[kXwSeg], before[kXwSeg];
#pragma unroll
      for (int q = 0; q < kXwSeg; ++q) {
        const int k = k0 + q, j = i - w + k;
        valid[q] = k < nk && j >= c0 && j <= c1;
        before[q] = k < nk && j < c0;
        if (valid[q]) {
          const int32_t dg = (j == 1) ? (i == 1 ? 0 : kOut) : Mk[q];
          fin[q] = (j == c1) ? kOut : Fk[q];
          sv[q] = score_of(ci, s2.at(ar, j - 1), P.match, P.mismatch) + dg;
          A[q] = sv[q] > fin[q] ? sv[q] : fin[q];
          f = aff_then(f, AffMax{g, A[q] + open});
        } else if (before[q]) {
          f = AffMax{kNegInf, kOut};
        }
      }
      // exclusive scan of the lanes' maps
      AffMax incl = f;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        AffMax o;
        o.a = __shfl_up_sync(0xFFFFFFFFu, incl.a, d);
        o.b = __shfl_up_sync(0xFFFFFFFFu, incl.b, d);
        if (lane >= d) incl = aff_then(o, incl);
      }
      AffMax excl;
      excl.a = __shfl_up_sync(0xFFFFFFFFu, incl.a, 1);
      excl.b = __shfl_up_sync(0xFFFFFFFFu, incl.b, 1);
      if (lane == 0) excl = AffMax{0, kNegInf};
      int32_t e = aff_apply(excl, ecarry);
      const AffMax all{__shfl_sync(0xFFFFFFFFu, incl.a, 31), __shfl_sync(0xFFFFFFFFu, incl.b, 31)};
      const int32_t next_carry = aff_apply(all, ecarry);
      // replay the cells with the reference's comparisons
      uint32_t nib = 0;
#pragma unroll
      for (int q = 0; q < kXwSeg; ++q) {
        const int k = k0 + q, j = i - w + k;
        uint32_t cd = 0xFu;
        if (valid[q]) {
          uint32_t d = sv[q] > fin[q] ? 0u : 1u;
          int32_t v = A[q];
          if (!(v > e)) d = 2u, v = e;
          if (v > lbest) lbest = v, lbestj = j;
          const int32_t h = v + open, fx = fin[q] + ext;
          if (fx >= h) d |= 4u;
          e += ext;
          if (e >= h) d |= 8u;
          e = e >= h ? e : h;
          M[k] = v;
          F[k] = fx >= h ? fx : h;
          cd = d;
        } else if (before[q]) {
          e = kOut;
        }
        nib |= cd << (4 * q);
      }
      ecarry = next_carry;
      if (T.want_codes) {
        // 4 nibbles per lane = half a word: even lanes write the word shared with the next lane
        const uint32_t hi = __shfl_down_sync(0xFFFFFFFFu, nib, 1);
        const int word = k0 >> 3;
        if ((lane & 1) == 0 && word < wpr) row_codes[word] = nib | (hi << 16);
      }
      __syncwarp();
    }
    rows = i;
    // the row's first maximum: largest value, then smallest column
    const int best = __reduce_max_sync(0xFFFFFFFFu, lbest);
    int bestj = __reduce_min_sync(0xFFFFFFFFu, (lbest == best && lbestj >= 0) ? lbestj : 0x7FFFFFFF);
    if (best <= 0) bestj = -1;
    if (bestj != n2 && bestj != 1 && (bestj == c0 || bestj == c1)) {
      status = 1;
      break;
    }
    if (best > score) score = best, e1 = i, e2 = bestj;
    if (score - best > P.xdrop) break;
    if (best <= 0) break;
  }
  if (lane == 0) {
    T.status = status;
    T.rows = rows;
    if (status == 0) T.score = score, T.end1 = e1, T.end2 = e2;
  }
}

__global__ void __launch_bounds__(128) xdrop_warp_kernel(XTask *__restrict__ tasks, const int *__restrict__ idx,
                                                         int n, Arena ar, Params P, uint32_t *__restrict__ tb,
                                                         int32_t *__restrict__ scratch, int64_t per_warp) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= n) return;  // whole warp
  XTask &T = tasks[idx[gw]];
  int32_t *M = scratch + per_warp * gw;
  xdrop_warp_pass(T, ar, P, tb, M, M + (2 * T.w + 2));
}

// ------------------------------------------------------------------ chained levels
// All passes of a batch start with the same band w0; level L runs the passes that reached band w0 * 2^L.  Each level
// kernel reads its work list and count from device memory, appends the passes that must restart (band edge touched;
// band doubled here, as the reference does) to the next level's list, and the passes whose traceback slot did not fit
// to the retry list; the host enqueues every level at once and synchronises once.  Traceback slots (reverse passes)
// are taken from an arena by atomic add: min(n1, slot_rows) rows of the pass's band.
struct XLevelArgs {
  XTask *tasks;
  const int *list_in;
  const int *count_in;
  int *list_out, *count_out;
  int *retry, *retry_count;
  unsigned long long *tb_cursor;
  int64_t tb_words;
  int *fetch;  // passes of the level handed out so far (the row-interleaved kernel)
  // hand-off of long register-band passes to the wavefront form (handoff_rows = 0: off): a pass still running after
  // handoff_rows rows stores its band (M then F, spill_half ints each) in spill slot s and its id in long_list[s]
  int *long_list, *long_count;
  int32_t *spill;
  int spill_cap, spill_half, handoff_rows;
  int level_w;    // the level's band half-width (every pass of a level has it)
  int slot_rows;  // rows of a traceback slot: min(n1, slot_rows)
};

__device__ __forceinline__ bool xd_take_slot(XTask &T, const XLevelArgs &L) {
  const int64_t rows = min(T.n1, L.slot_rows);
  const int64_t words = max((int64_t)1, rows * xd_words_per_row(T.w));
  if (words > INT32_MAX) return false;  // the capacity is an int: such a pass is retried with a whole-pass slot
  const unsigned long long off = atomicAdd(L.tb_cursor, (unsigned long long)words);
  if ((int64_t)off + words > L.tb_words) return false;
  T.tb_off = (int64_t)off;
  T.tb_cap = (int32_t)words;
  return true;
}

__device__ __forceinline__ void xd_route(XTask &T, int id, const XLevelArgs &L) {
  if (T.status == 1) {
    T.w *= 2;
    L.list_out[atomicAdd(L.count_out, 1)] = id;
  } else if (T.status == 2) {
    L.retry[atomicAdd(L.retry_count, 1)] = id;
  }
}

template <int WC>
__global__ void __launch_bounds__(128) xdrop_level_kernel(XLevelArgs L, Arena ar, Params P, uint32_t *__restrict__ tb) {
  const int n = *L.count_in;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int id = L.list_in[q];
    XTask &T = L.tasks[id];
    if (T.want_codes && !xd_take_slot(T, L)) {
      T.status = 2;
      L.retry[atomicAdd(L.retry_count, 1)] = id;
      continue;
    }
    xdrop_pass<WC>(T, ar, P, tb, nullptr, nullptr);
    xd_route(T, id, L);
  }
}

// The register-band level as a row-interleaved loop: every lane of a warp advances its own pass one row per
// iteration and, when that pass ends, takes the level's next pass (warp-aggregated atomic on L.fetch), so the warp
// keeps issuing full rows until the level's list runs out instead of idling until its longest pass ends.  The loop
// is warp-uniform (every lane iterates until no lane has a pass or can take one), so the lanes with a pass run each
// row together.  With L.handoff_rows > 0, a pass still running after that many rows (and more than a stripe from
// the end of seq1) leaves its band state in a spill slot for the wavefront form (xdrop_level_resume_kernel), which
// runs the rest of the pass 32 rows at a time: the level then no longer lasts as long as its longest pass on one
// thread.  A pass that finds the spill slots full stays on its thread.
template <int WC, bool CODES>
__global__ void __launch_bounds__(128) xdrop_level_flat_kernel(XLevelArgs L, Arena ar, Params P,
                                                               uint32_t *__restrict__ tb) {
  constexpr int NA = XBand<WC>::NA;
  const int n = *L.count_in;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  XPassScalars x;
  int32_t Mr[NA], Fr[NA];
  uint64_t qw[XBand<WC>::NQ];
  int id = -1;
  bool more = true;                        // the level's list may still hold a pass for this lane
  bool can_spill = L.handoff_rows > 0;
  for (;;) {
    const bool need = id < 0 && more;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, need);
    if (m != 0) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(L.fetch, __popc(m));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (need) {
        const int q = base + __popc(m & below);
        if (q >= n) {
          more = false;
        } else {
          id = L.list_in[q];
          XTask &T = L.tasks[id];
          if (T.want_codes && !xd_take_slot(T, L)) {
            T.status = 2;
            L.retry[atomicAdd(L.retry_count, 1)] = id;
            id = -1;
          } else {
            xd_begin<WC>(x, Mr, Fr, qw, T, ar);
          }
        }
      }
    }
    if (!__any_sync(0xFFFFFFFFu, id >= 0 || more)) break;
    if (id >= 0) {
      const int st = xd_row_fused<WC, CODES>(x, Mr, Fr, qw, ar, P, tb);
      if (st >= 0) {
        XTask &T = L.tasks[id];
        xd_finish(x, T, st);
        xd_route(T, id, L);
        id = -1;
      } else if (can_spill && x.rows >= L.handoff_rows && x.n1 - x.rows > 32) {
        const int s = atomicAdd(L.long_count, 1);
        if (s < L.spill_cap) {
          int32_t *sp = L.spill + (int64_t)s * 2 * L.spill_half;
#pragma unroll
          for (int k = 0; k < NA; ++k)
            if (k <= x.nk) {
              sp[k] = Mr[k];
              sp[L.spill_half + k] = Fr[k];
            }
          XTask &T = L.tasks[id];
          T.score = x.score;
          T.end1 = x.e1;
          T.end2 = x.e2;
          T.rows = x.rows;
          L.long_list[s] = id;
          id = -1;
        } else {
          can_spill = false;
        }
      }
    }
  }
}

__global__ void __launch_bounds__(128) xdrop_level_warp_kernel(XLevelArgs L, Arena ar, Params P,
                                                               uint32_t *__restrict__ tb, int32_t *__restrict__ scratch,
                                                               int64_t per_warp) {
  const int n = *L.count_in;
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  int32_t *M = scratch + per_warp * gw;
  for (int q = gw; q < n; q += nw) {
    const int id = L.list_in[q];
    XTask &T = L.tasks[id];
    int ok = 1;
    if (lane == 0 && T.want_codes) ok = xd_take_slot(T, L) ? 1 : 0;
    ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
    __syncwarp();
    if (!ok) {
      if (lane == 0) {
        T.status = 2;
        L.retry[atomicAdd(L.retry_count, 1)] = id;
      }
      continue;
    }
    xdrop_warp_pass(T, ar, P, tb, M, M + (2 * T.w + 2));
    __syncwarp();
    if (lane == 0) xd_route(T, id, L);
    __syncwarp();
  }
}

// ------------------------------------------------------------------ band levels as a wavefront (one warp per pass)
// Rows in stripes of 32, lane l owning row i = r0 + l; at step t the lane computes its band cell k = t - 2l (column
// j = i - w + k), so the cell above (column j, the previous row's band cell k + 1) was computed by lane l - 1 one step
// earlier and the diagonal cell (column j - 1, band cell k) two steps earlier: both arrive by __shfl_up_sync, as does
// the query code of column j.  Lane 0 reads the row above the stripe from the warp's boundary row in shared memory,
// which lane 31 rewrites (by band index) as it computes the stripe's last row; lane 31 writes index k at step 62 + k,
// after lane 0 has read it (steps k - 1 and k).  A cell only ever reads in-band cells of the row above (its band is
// the row above's shifted by one column, clipped to [1, n2]), so nothing else crosses rows.  The cells are exactly
// the thread pass's; each lane keeps its row's maximum and writes its row's codes, and after each stripe the rows are
// evaluated in order (slot capacity, band-edge restart, score, x-drop, non-positive maximum) with the thread pass's
// rules; rows computed past the stop row are discarded (their codes lie in the pass's own slot, after its end row).
// A row costs (2w + 63) / 32 steps of one cell per lane: a long pass runs several times faster than on one thread.
constexpr int kXwMaxW = 256;

// The pass resumes at row r_begin: bM / bF hold row r_begin - 1 by band index (row 0: every cell kOut), and the
// running maximum, its cell and the rows evaluated so far are (score, e1, e2, rows).  CODES = false (forward passes)
// leaves out the direction codes and their comparisons.
template <bool CODES>
__device__ void xdrop_wave_pass_t(XTask &T, const Arena &ar, const Params &P, uint32_t *__restrict__ tb,
                                  int32_t *__restrict__ bM, int32_t *__restrict__ bF, int64_t tb_off, int32_t tb_cap,
                                  int lane, int r_begin, int score, int e1, int e2, int rows) {
  const int w = T.w, n1 = T.n1, n2 = T.n2, nk = 2 * w + 1, wpr = xd_words_per_row(w);
  const bool codes = CODES && T.want_codes != 0;
  const SeqView s1{T.base1, T.a1, T.dir}, s2{T.base2, T.a2, T.dir};
  const int open = P.open1, ext = P.ext1;
  __syncwarp();
  int status = 0;
  bool stop = false;
  for (int r0 = r_begin; r0 <= n1 && !stop; r0 += 32) {
    const int i = r0 + lane;
    const bool live = i <= n1;
    const int c1 = min(i + w, n2);
    const int ci = live ? s1.at(ar, i - 1) : 0;
    // k in [0, 2w] puts j = i - w + k in [i - w, i + w], so the band test is 1 <= j <= n2: j - 1 unsigned below un2
    // (0 for a row past the pass: no cell)
    const unsigned un2 = live ? (unsigned)n2 : 0u;
    const bool wcode = codes && live && (int64_t)i * wpr <= tb_cap;  // rows past the slot are never kept
    uint32_t *row_codes = tb + tb_off + (int64_t)(i - 1) * wpr;
    int e = kOut, best = 0, bestj = -1, outM = kOut, outF = kOut, outC = 0, prevUp = kOut, kw = 0;
    uint32_t cw = 0;
    const int nsteps = nk + 62;
    for (int t = 0; t < nsteps; ++t) {
      const int upM = __shfl_up_sync(0xFFFFFFFFu, outM, 1);
      int upF = __shfl_up_sync(0xFFFFFFFFu, outF, 1);
      int cj = __shfl_up_sync(0xFFFFFFFFu, outC, 1);
      const int k = t - 2 * lane, j = i - w + k;
      int diagv = prevUp;
      if (lane == 0) {
        diagv = (k >= 0 && k < nk) ? bM[k] : kOut;
        upF = (k >= 0 && k + 1 <= nk) ? bF[k + 1] : kOut;
        cj = (j >= 1 && j <= n2) ? s2.at(ar, j - 1) : 0;
      }
      int nM = kOut, nF = kOut;
      if ((unsigned)k < (unsigned)nk) {
        uint32_t nib = 0xFu;
        if ((unsigned)(j - 1) < un2) {
          const int32_t diag = (j == 1) ? (i == 1 ? 0 : kOut) : diagv;
          const int32_t fin = (j == c1) ? kOut : upF;
          const int32_t sd = score_of(ci, cj, P.match, P.mismatch) + diag;
          const int32_t A = sd > fin ? sd : fin;
          const bool ge = !(A > e);  // the horizontal gap wins ties
          const int32_t v = ge ? e : A;
          if (v > best) {
            best = v;
            bestj = j;
          }
          const int32_t h = v + open;
          const int32_t f = fin + ext;
          nM = v;
          nF = f >= h ? f : h;
          const int32_t ee = e + ext;
          if constexpr (CODES) nib = (ge ? 2u : (sd > fin ? 0u : 1u)) | (f >= h ? 4u : 0u) | (ee >= h ? 8u : 0u);
          e = ee >= h ? ee : h;
          if (lane == 31) {
            bM[k] = nM;
            bF[k] = nF;
          }
        }
        if (wcode) {
          cw |= nib << (4 * (k & 7));
          if ((k & 7) == 7 || k == nk - 1) {
            row_codes[kw++] = cw;
            cw = 0;
          }
        }
      }
      prevUp = upM;
      outM = nM;
      outF = nF;
      outC = cj;
    }
    __syncwarp();
    for (int rr = 0; rr < 32; ++rr) {  // the stripe's rows in order; every lane keeps the same state
      const int tm = __shfl_sync(0xFFFFFFFFu, best, rr), tj = __shfl_sync(0xFFFFFFFFu, bestj, rr);
      if (stop) continue;
      const int ii = r0 + rr;
      if (ii > n1) {
        stop = true;
        continue;
      }
      if (codes && (int64_t)ii * wpr > tb_cap) {
        status = 2;
        stop = true;
        continue;
      }
      rows = ii;
      const int cc0 = max(ii - w, 1), cc1 = min(ii + w, n2);
      if (tj != n2 && tj != 1 && (tj == cc0 || tj == cc1)) {
        status = 1;
        stop = true;
        continue;
      }
      if (tm > score) {
        score = tm;
        e1 = ii;
        e2 = tj;
      }
      if (score - tm > P.xdrop || tm <= 0) stop = true;
    }
  }
  if (lane == 0) {
    T.status = status;
    T.rows = rows;
    if (status == 0) {
      T.score = score;
      T.end1 = e1;
      T.end2 = e2;
    }
  }
}

__device__ __forceinline__ void xdrop_wave_pass(XTask &T, const Arena &ar, const Params &P, uint32_t *__restrict__ tb,
                                                int32_t *__restrict__ bM, int32_t *__restrict__ bF, int64_t tb_off,
                                                int32_t tb_cap, int lane, int r_begin, int score, int e1, int e2,
                                                int rows) {
  if (T.want_codes)
    xdrop_wave_pass_t<true>(T, ar, P, tb, bM, bF, tb_off, tb_cap, lane, r_begin, score, e1, e2, rows);
  else
    xdrop_wave_pass_t<false>(T, ar, P, tb, bM, bF, tb_off, tb_cap, lane, r_begin, score, e1, e2, rows);
}

__global__ void __launch_bounds__(128) xdrop_level_wave_kernel(XLevelArgs L, Arena ar, Params P,
                                                               uint32_t *__restrict__ tb) {
  __shared__ int32_t sM[4][2 * kXwMaxW + 2], sF[4][2 * kXwMaxW + 2];
  const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const int n = *L.count_in;
  for (int q = gw; q < n; q += nw) {
    const int id = L.list_in[q];
    XTask &T = L.tasks[id];
    int ok = 1, cap = 0;
    long long off = 0;
    if (lane == 0) {
      if (T.want_codes) ok = xd_take_slot(T, L) ? 1 : 0;
      off = T.tb_off;
      cap = T.tb_cap;
    }
    ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
    off = __shfl_sync(0xFFFFFFFFu, off, 0);
    cap = __shfl_sync(0xFFFFFFFFu, cap, 0);
    if (!ok) {
      if (lane == 0) {
        T.status = 2;
        L.retry[atomicAdd(L.retry_count, 1)] = id;
      }
      continue;
    }
    for (int k = lane; k <= 2 * T.w + 1; k += 32) sM[wb][k] = kOut, sF[wb][k] = kOut;  // row 0
    xdrop_wave_pass(T, ar, P, tb, sM[wb], sF[wb], off, cap, lane, 1, 0, 0, 0, 0);
    __syncwarp();
    if (lane == 0) xd_route(T, id, L);
    __syncwarp();
  }
}

// The passes the register-band level handed off (L.long_list), one warp per pass, resumed from their spilled band
// and running state at the row after the last one their thread evaluated; routed like every other pass of the level.
constexpr int kXrMaxW = 20;
__global__ void __launch_bounds__(128) xdrop_level_resume_kernel(XLevelArgs L, Arena ar, Params P,
                                                                 uint32_t *__restrict__ tb) {
  __shared__ int32_t sM[4][2 * kXrMaxW + 2], sF[4][2 * kXrMaxW + 2];
  const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const int n = min(*L.long_count, L.spill_cap);
  for (int q = gw; q < n; q += nw) {
    const int id = L.long_list[q];
    XTask &T = L.tasks[id];
    const int32_t *sp = L.spill + (int64_t)q * 2 * L.spill_half;
    const int nk = 2 * T.w + 1;
    for (int k = lane; k <= nk; k += 32) sM[wb][k] = sp[k], sF[wb][k] = sp[L.spill_half + k];
    const int64_t off = T.tb_off;
    const int cap = T.tb_cap, score = T.score, e1 = T.end1, e2 = T.end2, rows = T.rows;
    __syncwarp();
    xdrop_wave_pass(T, ar, P, tb, sM[wb], sF[wb], off, cap, lane, rows + 1, score, e1, e2, rows);
    __syncwarp();
    if (lane == 0) xd_route(T, id, L);
    __syncwarp();
  }
}

// The same passes on G-lane groups (32 / G passes per warp), each group a wavefront over G-row stripes: lane g of a
// group owns row r0 + g and computes band cell k = t - 2g at step t, with the cell above and the diagonal from lane
// g - 1 (__shfl_up_sync within the group); lane 0 of the group reads the row above the stripe from the group's
// boundary row in shared memory, which lane G - 1 rewrites (index k at step k + 2(G - 1), after lane 0 read it).
// A G-row stripe is 2w + 1 + 2(G - 1) steps, so fewer lanes idle in the skew than with a 32-row stripe at bands
// 10-20 (G = 8: 75 % of lane-steps compute a cell at band 20, against 40 % for one warp per pass); every group runs
// its stripes in step with the warp (all passes of a level have the same band), evaluates its rows in order after
// each stripe, and takes its next pass (list index + the grid's group count) when its pass ends.  G = 4 idles the
// fewest lanes in the skew (78 % of lane-steps compute at band 10, 87 % at band 20) but needs eight passes per warp;
// CODES = false (forward passes) leaves out the direction codes and their comparisons.  FRESH = true runs the level's
// whole list (L.list_in) from row 1 instead of the handed-off passes: each group takes its pass's traceback slot and
// starts from the zero row, so a level of long passes (band 20: the passes that restarted) skips the one-thread form.
template <int G, bool CODES, bool FRESH>
__global__ void __launch_bounds__(128) xdrop_level_resume_group_kernel(XLevelArgs L, Arena ar, Params P,
                                                                       uint32_t *__restrict__ tb) {
  constexpr int NG = 32 / G;
  __shared__ int32_t sM[4][NG][2 * kXrMaxW + 2], sF[4][NG][2 * kXrMaxW + 2];
  const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5, g = lane / G, gl = lane % G;
  const unsigned gmask = G == 32 ? 0xFFFFFFFFu : ((1u << G) - 1u) << (lane & ~(G - 1));  // the group's lanes
  const int n = FRESH ? *L.count_in : min(*L.long_count, L.spill_cap);
  const int *const list = FRESH ? L.list_in : L.long_list;
  const int ngroups = (int)((gridDim.x * blockDim.x) / G);
  const int w = L.level_w, nk = 2 * w + 1, wpr = xd_words_per_row(w), nsteps = nk + 2 * (G - 1);
  const int open = P.open1, ext = P.ext1;
  int32_t *const bM = sM[wb][g], *const bF = sF[wb][g];
  int q = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G);  // the group's list index
  // the group's pass (the same values in every lane of the group)
  bool active = false, codes = false;
  XTask *T = nullptr;
  int id = 0, n1 = 0, n2 = 0, cap = 0, score = 0, e1 = 0, e2 = 0, rows = 0, r0 = 1;
  int64_t off = 0;
  SeqView s1{0, 0, 0}, s2{0, 0, 0};
  // List entry q into the group: its band of the row before r0 and its running state (a handed-off pass: from its
  // spill slot; a fresh pass: the zero row, after its traceback slot is taken).  Called by whole groups only.
  auto begin = [&]() {
    for (;;) {
      active = q < n;
      if (!active) return;
      id = list[q];
      T = &L.tasks[id];
      n1 = T->n1, n2 = T->n2, codes = T->want_codes != 0;
      s1 = SeqView{T->base1, T->a1, T->dir}, s2 = SeqView{T->base2, T->a2, T->dir};
      if constexpr (FRESH) {
        int ok = 1;
        long long o = 0;
        int c = 0;
        if (gl == 0) {
          if (codes) ok = xd_take_slot(*T, L) ? 1 : 0;
          if (!ok) {
            T->status = 2;
            L.retry[atomicAdd(L.retry_count, 1)] = id;
          }
          o = T->tb_off;
          c = T->tb_cap;
        }
        ok = __shfl_sync(gmask, ok, 0, G);
        if (!ok) {
          q += ngroups;
          continue;
        }
        off = __shfl_sync(gmask, o, 0, G);
        cap = __shfl_sync(gmask, c, 0, G);
        score = e1 = e2 = rows = 0, r0 = 1;
        for (int k = gl; k <= nk; k += G) bM[k] = kOut, bF[k] = kOut;
      } else {
        const int32_t *sp = L.spill + (int64_t)q * 2 * L.spill_half;
        off = T->tb_off, cap = T->tb_cap;
        score = T->score, e1 = T->end1, e2 = T->end2, rows = T->rows, r0 = rows + 1;
        for (int k = gl; k <= nk; k += G) bM[k] = sp[k], bF[k] = sp[L.spill_half + k];
      }
      return;
    }
  };
  begin();
  __syncwarp();
  while (__any_sync(0xFFFFFFFFu, active)) {
    const int i = r0 + gl;
    const bool live = active && i <= n1;
    const int c1 = min(i + w, n2);
    const int ci = live ? s1.at(ar, i - 1) : 0;
    // the row's band cells: k in [0, 2w] puts j = i - w + k in [i - w, i + w], so the band test is 1 <= j <= n2,
    // i.e. j - 1 unsigned below un2 (0 for a row past the pass: no cell)
    const unsigned un2 = live ? (unsigned)n2 : 0u;
    const bool wcode = CODES && codes && live && (int64_t)i * wpr <= cap;  // rows past the slot are never kept
    uint32_t *row_codes = tb + off + (int64_t)(i - 1) * wpr;
    int e = kOut, best = 0, bestj = -1, outM = kOut, outF = kOut, outC = 0, prevUp = kOut, kw = 0;
    uint32_t cw = 0;
    for (int t = 0; t < nsteps; ++t) {
      const int upM = __shfl_up_sync(0xFFFFFFFFu, outM, 1, G);
      int upF = __shfl_up_sync(0xFFFFFFFFu, outF, 1, G);
      int cj = __shfl_up_sync(0xFFFFFFFFu, outC, 1, G);
      const int k = t - 2 * gl, j = i - w + k;
      int diagv = prevUp;
      if (gl == 0) {
        diagv = (active && k >= 0 && k < nk) ? bM[k] : kOut;
        upF = (active && k >= 0 && k + 1 <= nk) ? bF[k + 1] : kOut;
        cj = (active && j >= 1 && j <= n2) ? s2.at(ar, j - 1) : 0;
      }
      int nM = kOut, nF = kOut;
      if ((unsigned)k < (unsigned)nk) {
        uint32_t nib = 0xFu;
        if ((unsigned)(j - 1) < un2) {
          const int32_t diag = (j == 1) ? (i == 1 ? 0 : kOut) : diagv;
          const int32_t fin = (j == c1) ? kOut : upF;
          const int32_t sd = score_of(ci, cj, P.match, P.mismatch) + diag;
          const int32_t A = sd > fin ? sd : fin;
          const bool ge = !(A > e);  // the horizontal gap wins ties
          const int32_t v = ge ? e : A;
          if (v > best) {
            best = v;
            bestj = j;
          }
          const int32_t h = v + open;
          const int32_t f = fin + ext;
          nM = v;
          nF = f >= h ? f : h;
          const int32_t ee = e + ext;
          if constexpr (CODES) nib = (ge ? 2u : (sd > fin ? 0u : 1u)) | (f >= h ? 4u : 0u) | (ee >= h ? 8u : 0u);
          e = ee >= h ? ee : h;
          if (gl == G - 1) {
            bM[k] = nM;
            bF[k] = nF;
          }
        }
        if (wcode) {
          cw |= nib << (4 * (k & 7));
          if ((k & 7) == 7 || k == nk - 1) {
            row_codes[kw++] = cw;
            cw = 0;
          }
        }
      }
      prevUp = upM;
      outM = nM;
      outF = nF;
      outC = cj;
    }
    __syncwarp();
    // the stripe's rows in order (every lane of a group keeps the same state)
    bool stop = false;
    int status = 0;
    for (int rr = 0; rr < G; ++rr) {
      const int src = (lane & ~(G - 1)) + rr;
      const int tm = __shfl_sync(0xFFFFFFFFu, best, src), tj = __shfl_sync(0xFFFFFFFFu, bestj, src);
      if (!active || stop) continue;
      const int ii = r0 + rr;
      if (ii > n1) {
        stop = true;
        continue;
      }
      if (codes && (int64_t)ii * wpr > cap) {
        status = 2;
        stop = true;
        continue;
      }
      rows = ii;
      const int cc0 = max(ii - w, 1), cc1 = min(ii + w, n2);
      if (tj != n2 && tj != 1 && (tj == cc0 || tj == cc1)) {
        status = 1;
        stop = true;
        continue;
      }
      if (tm > score) {
        score = tm;
        e1 = ii;
        e2 = tj;
      }
      if (score - tm > P.xdrop || tm <= 0) stop = true;
    }
    if (active) {
      r0 += G;
      if (stop || r0 > n1) {  // the pass ended: its result, its route, then the group's next pass
        if (gl == 0) {
          T->status = status;
          T->rows = rows;
          if (status == 0) {
            T->score = score;
            T->end1 = e1;
            T->end2 = e2;
          }
          xd_route(*T, id, L);
        }
        q += ngroups;
        begin();
      }
    }
    __syncwarp();
  }
}

__global__ void xdrop_iota_kernel(int *list, int n, int *count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) list[k] = k;
  if (k == 0) *count = n;
}

// Whole passes on the wavefront form, one warp per pass (w <= 256), with the traceback slot the host assigned
// (T.tb_off, T.tb_cap): the form for passes known to be long, such as those that outgrew their slot in the levels.
__global__ void __launch_bounds__(128) xdrop_wave_kernel(XTask *__restrict__ tasks, const int *__restrict__ idx, int n,
                                                         Arena ar, Params P, uint32_t *__restrict__ tb) {
  __shared__ int32_t sM[4][2 * kXwMaxW + 2], sF[4][2 * kXwMaxW + 2];
  const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= n) return;  // whole warp
  XTask &T = tasks[idx[gw]];
  const int64_t off = T.tb_off;
  const int cap = T.tb_cap;
  for (int k = lane; k <= 2 * T.w + 1; k += 32) sM[wb][k] = kOut, sF[wb][k] = kOut;  // row 0
  xdrop_wave_pass(T, ar, P, tb, sM[wb], sF[wb], off, cap, lane, 1, 0, 0, 0, 0);
}

void launch_xdrop(XTask *tasks, const int *idx, int n, Arena ar, Params p, uint32_t *tb, int wcap, int32_t *scratch,
                  int64_t scratch_per_thread, cudaStream_t st) {
  if (n <= 0) return;
  const int g = (n + 127) / 128;
  if (wcap < 0)  // long passes: wavefront, one warp each
    xdrop_wave_kernel<<<(n + 3) / 4, 128, 0, st>>>(tasks, idx, n, ar, p, tb);
  else if (wcap == 10)
    xdrop_kernel<10><<<g, 128, 0, st>>>(tasks, idx, n, ar, p, tb, scratch, 0);
  else if (wcap == 20)
    xdrop_kernel<20><<<g, 128, 0, st>>>(tasks, idx, n, ar, p, tb, scratch, 0);
  else  // wide band: one warp per pass, scratch_per_thread = ints per warp
    xdrop_warp_kernel<<<(n + 3) / 4, 128, 0, st>>>(tasks, idx, n, ar, p, tb, scratch, scratch_per_thread);
}

void launch_xdrop_iota(int *list, int n, int *count, cudaStream_t st) {
  xdrop_iota_kernel<<<(n + 255) / 256, 256, 0, st>>>(list, n, count);
}

template <int WC, bool CODES>
int flat_blocks_per_sm() {
  static int nb = 0;
  if (nb == 0) {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, xdrop_level_flat_kernel<WC, CODES>, 128, 0) != cudaSuccess) {
      (void)cudaGetLastError();
      v = 1;
    }
    nb = v > 0 ? v : 1;
  }
  return nb;
}

int launch_xdrop_level(XTask *tasks, const int *list_in, const int *count_in, int *list_out, int *count_out,
                       int *retry, int *retry_count, unsigned long long *tb_cursor, int64_t tb_words, int slot_rows,
                       int *fetch, const XHandoff &H, Arena ar, Params p, uint32_t *tb, int w, int n_bound, int nsm,
                       int32_t *scratch, int64_t per_warp, int warps, int warp_from, int wave_max_w, bool flat,
                       int group_from, bool codes, cudaStream_t st) {
  if (n_bound <= 0) return 0;
  const bool flat_level = flat && w <= warp_from && w <= kXrMaxW;
  // groups of G lanes: 128 / G passes per block
  auto group_grid = [&](int g, int64_t passes) {
    return (int)std::min<int64_t>((passes + 128 / g - 1) / (128 / g), (int64_t)nsm * 16);
  };
  const bool handoff = flat_level && H.rows > 0 && H.cap > 0;
  XLevelArgs L{tasks, list_in, count_in, list_out, count_out, retry, retry_count, tb_cursor, tb_words, fetch,
               H.list, H.count, H.spill, handoff ? H.cap : 0, w <= 10 ? XBand<10>::NA : XBand<20>::NA,
               handoff ? H.rows : 0, w, slot_rows};
  const int g = (int)std::min<int64_t>((n_bound + 127) / 128, (int64_t)nsm * 16);
  if (flat_level && group_from > 0 && w >= group_from) {  // every pass of the level on G-lane groups from row 1
    XLevelArgs F = L;
    F.spill_cap = 0;
    const int G = (H.lanes == 4 || H.lanes == 16) ? H.lanes : 8;
    const int gg = group_grid(G, n_bound);
    if (G == 4 && codes)
      xdrop_level_resume_group_kernel<4, true, true><<<gg, 128, 0, st>>>(F, ar, p, tb);
    else if (G == 4)
      xdrop_level_resume_group_kernel<4, false, true><<<gg, 128, 0, st>>>(F, ar, p, tb);
    else if (G == 8 && codes)
      xdrop_level_resume_group_kernel<8, true, true><<<gg, 128, 0, st>>>(F, ar, p, tb);
    else if (G == 8)
      xdrop_level_resume_group_kernel<8, false, true><<<gg, 128, 0, st>>>(F, ar, p, tb);
    else if (codes)
      xdrop_level_resume_group_kernel<16, true, true><<<gg, 128, 0, st>>>(F, ar, p, tb);
    else
      xdrop_level_resume_group_kernel<16, false, true><<<gg, 128, 0, st>>>(F, ar, p, tb);
    return 1;
  }
  if (flat_level) {  // register band, row-interleaved: one resident wave of blocks, then the handed-off passes
    auto flat_grid = [&](int per_sm) {
      return (int)std::min<int64_t>((n_bound + 127) / 128, (int64_t)nsm * per_sm);
    };
    if (w <= 10 && codes)
      xdrop_level_flat_kernel<10, true><<<flat_grid(flat_blocks_per_sm<10, true>()), 128, 0, st>>>(L, ar, p, tb);
    else if (w <= 10)
      xdrop_level_flat_kernel<10, false><<<flat_grid(flat_blocks_per_sm<10, false>()), 128, 0, st>>>(L, ar, p, tb);
    else if (codes)
      xdrop_level_flat_kernel<20, true><<<flat_grid(flat_blocks_per_sm<20, true>()), 128, 0, st>>>(L, ar, p, tb);
    else
      xdrop_level_flat_kernel<20, false><<<flat_grid(flat_blocks_per_sm<20, false>()), 128, 0, st>>>(L, ar, p, tb);
    if (!handoff) return 1;
    if (H.lanes == 4 && codes)
      xdrop_level_resume_group_kernel<4, true, false><<<group_grid(4, H.cap), 128, 0, st>>>(L, ar, p, tb);
    else if (H.lanes == 4)
      xdrop_level_resume_group_kernel<4, false, false><<<group_grid(4, H.cap), 128, 0, st>>>(L, ar, p, tb);
    else if (H.lanes == 8 && codes)
      xdrop_level_resume_group_kernel<8, true, false><<<group_grid(8, H.cap), 128, 0, st>>>(L, ar, p, tb);
    else if (H.lanes == 8)
      xdrop_level_resume_group_kernel<8, false, false><<<group_grid(8, H.cap), 128, 0, st>>>(L, ar, p, tb);
    else if (H.lanes == 16 && codes)
      xdrop_level_resume_group_kernel<16, true, false><<<group_grid(16, H.cap), 128, 0, st>>>(L, ar, p, tb);
    else if (H.lanes == 16)
      xdrop_level_resume_group_kernel<16, false, false><<<group_grid(16, H.cap), 128, 0, st>>>(L, ar, p, tb);
    else
      xdrop_level_resume_kernel<<<(int)std::min<int64_t>((H.cap + 3) / 4, (int64_t)nsm * 16), 128, 0, st>>>(L, ar, p,
                                                                                                           tb);
    return 2;
  }
  if (w > warp_from && w <= wave_max_w && w <= kXwMaxW)  // wide bands up to 256: the wavefront
    xdrop_level_wave_kernel<<<(int)std::min<int64_t>((n_bound + 3) / 4, (int64_t)nsm * 16), 128, 0, st>>>(L, ar, p,
                                                                                                         tb);
  else if (w > warp_from)
    xdrop_level_warp_kernel<<<(warps + 3) / 4, 128, 0, st>>>(L, ar, p, tb, scratch, per_warp);
  else if (w <= 10)
    xdrop_level_kernel<10><<<g, 128, 0, st>>>(L, ar, p, tb);
  else if (w <= 20)
    xdrop_level_kernel<20><<<g, 128, 0, st>>>(L, ar, p, tb);
  else
    xdrop_level_warp_kernel<<<(warps + 3) / 4, 128, 0, st>>>(L, ar, p, tb, scratch, per_warp);
  return 1;
}

// ------------------------------------------------------------------ traceback of the reverse pass
// State machine of impl/sequenceAlignment3.cpp:1413-1438: start in the state that produced the cell; a gap state
// persists while the cell's continuation bit is set; ops are appended as the walk goes (no final reverse, because
// the walk over the reverse-complement pass already runs in forward order).  Unwritten cells read 255.
//
// One warp per pass.  The band store is row-major, so every move of the walk (diagonal, up, left) goes to the same
// or a lower word: the warp stages the kXtWin words that end at the cell it needs with coalesced 16-byte loads, and
// lane 0 walks them until the path leaves the window below (one memory round trip per window instead of one per
// move).  tb_words: size of the band store (no load goes past it).
constexpr int kXtWin = 1024;

__device__ void xdrop_traceback_warp(XTask &T, const uint32_t *__restrict__ tb, int64_t tb_words,
                                     uint32_t *__restrict__ cig, uint32_t *__restrict__ win, int lane) {
  const int w = T.w, wpr = xd_words_per_row(w);
  int ii = T.end1, jj = T.end2, state = 0, nc = 0;
  uint32_t *out = cig + T.cig_off;
  uint32_t last = 0xFFFFFFFFu;
  int64_t base = -1;  // window [base, base + kXtWin) of the store; -1: none yet
  bool full = false;
  for (;;) {
    int64_t need = -1;
    if (lane == 0) {
      while (ii > 0 && jj > 0 && !full) {
        int code = 255;
        const int k = jj - ii + w;
        if (ii <= T.rows && k >= 0 && k <= 2 * w) {
          const int64_t a = T.tb_off + (int64_t)(ii - 1) * wpr + (k >> 3);
          if (base < 0 || a < base || a >= base + kXtWin) {
            need = a;
            break;
          }
          const uint32_t nib = (win[a - base] >> (4 * (k & 7))) & 0xFu;
          if ((nib & 3u) != 3u) code = (int)((nib & 3u) | (((nib >> 2) & 1u) << 3) | (((nib >> 3) & 1u) << 4));
        }
        if (state == 0)
          state = code & 7;
        else if (!((code >> (state + 2)) & 1))
          state = 0;
        if (state == 0) state = code & 7;
        uint32_t op;
        if (state == 0) {
          op = 0;
          --ii;
          --jj;
        } else if (state == 1 || state == 3) {
          op = 2;
          --ii;
        } else {
          op = 1;
          --jj;
        }
        if (nc > 0 && (last & 0xFu) == op) {
          last += 1u << 4;
          out[nc - 1] = last;
        } else if (nc >= T.cig_cap) {
          full = true;
        } else {
          last = (1u << 4) | op;
          out[nc++] = last;
        }
      }
    }
    need = __shfl_sync(0xFFFFFFFFu, need, 0);
    if (need < 0) break;
    base = ((need + 4) & ~(int64_t)3) - kXtWin;  // ends (16-byte aligned) just past the needed word
    if (base < 0) base = 0;
    __syncwarp();
    for (int c = lane; c < kXtWin / 4; c += 32) {
      const int64_t a = base + 4 * (int64_t)c;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (a + 4 <= tb_words) v = __ldg(reinterpret_cast<const uint4 *>(tb + a));
      *reinterpret_cast<uint4 *>(win + 4 * c) = v;
    }
    __syncwarp();
  }
  if (lane == 0) {
    if (full) T.status = 3;
    T.iii = ii;
    T.jjj = jj;
    T.ncig = nc;
  }
}

__global__ void __launch_bounds__(128) xdrop_traceback_kernel(XTask *__restrict__ tasks, const int *__restrict__ idx,
                                                              int n, const uint32_t *__restrict__ tb, int64_t tb_words,
                                                              uint32_t *__restrict__ cig) {
  __shared__ __align__(16) uint32_t win[4][kXtWin];
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= n) return;  // whole warp
  xdrop_traceback_warp(tasks[idx[gw]], tb, tb_words, cig, win[threadIdx.x >> 5], lane);
}

// Chained form: every task of the batch that finished with codes takes a CIGAR slot of end1 + end2 + 2 words from an
// arena sized for the bound n1 + n2 + 2 per task, then runs the walk above.
__global__ void __launch_bounds__(128) xdrop_traceback_all_kernel(XTask *__restrict__ tasks, int n,
                                                                  const uint32_t *__restrict__ tb, int64_t tb_words,
                                                                  uint32_t *__restrict__ cig,
                                                                  unsigned long long *__restrict__ cig_cursor) {
  __shared__ __align__(16) uint32_t win[4][kXtWin];
  const int lane = threadIdx.x & 31;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= n) return;  // whole warp
  XTask &T = tasks[t];
  if (T.status != 0 || !T.want_codes) return;
  if (lane == 0) {
    T.cig_cap = max(T.end1, 0) + max(T.end2, 0) + 2;
    T.cig_off = (int64_t)atomicAdd(cig_cursor, (unsigned long long)T.cig_cap);
  }
  __syncwarp();
  xdrop_traceback_warp(T, tb, tb_words, cig, win[threadIdx.x >> 5], lane);
}

void launch_xdrop_traceback_all(XTask *tasks, int n, const uint32_t *tb, int64_t tb_words, uint32_t *cig,
                                unsigned long long *cig_cursor, cudaStream_t st) {
  if (n <= 0) return;
  xdrop_traceback_all_kernel<<<(n + 3) / 4, 128, 0, st>>>(tasks, n, tb, tb_words, cig, cig_cursor);
}

// Dense offsets of the finished tasks' CIGARs in task order: one block; each thread sums a contiguous run of tasks,
// a block-wide exclusive scan of the run sums, then each thread assigns its run's offsets.
__global__ void __launch_bounds__(1024) xdrop_cigar_scan_kernel(XTask *__restrict__ tasks, int n,
                                                                unsigned long long *__restrict__ total) {
  __shared__ long long part[1024];
  const int t = threadIdx.x, per = (n + 1023) / 1024;
  const int lo = min(n, t * per), hi = min(n, lo + per);
  long long sum = 0;
  for (int k = lo; k < hi; ++k)
    if (tasks[k].status == 0 && tasks[k].want_codes) sum += tasks[k].ncig;
  part[t] = sum;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {  // inclusive Hillis-Steele scan
    const long long v = t >= d ? part[t - d] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  long long off = part[t] - sum;
  for (int k = lo; k < hi; ++k)
    if (tasks[k].status == 0 && tasks[k].want_codes) {
      tasks[k].cig_dense = off;
      off += tasks[k].ncig;
    } else {
      tasks[k].cig_dense = -1;
    }
  if (t == 1023) *total = (unsigned long long)part[1023];
}

__global__ void xdrop_cigar_copy_kernel(const XTask *__restrict__ tasks, int n, const uint32_t *__restrict__ cig,
                                        uint32_t *__restrict__ dense) {
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (k >= n) return;
  const XTask &T = tasks[k];
  if (T.cig_dense < 0) return;
  for (int q = lane; q < T.ncig; q += 32) dense[T.cig_dense + q] = cig[T.cig_off + q];
}

void launch_xdrop_cigar_pack(XTask *tasks, int n, const uint32_t *cig, uint32_t *dense, unsigned long long *total,
                             cudaStream_t st) {
  if (n <= 0) return;
  xdrop_cigar_scan_kernel<<<1, 1024, 0, st>>>(tasks, n, total);
  xdrop_cigar_copy_kernel<<<(n + 7) / 8, 256, 0, st>>>(tasks, n, cig, dense);
}

void launch_xdrop_traceback(XTask *tasks, const int *idx, int n, const uint32_t *tb, int64_t tb_words, uint32_t *cig,
                            cudaStream_t st) {
  if (n <= 0) return;
  xdrop_traceback_kernel<<<(n + 3) / 4, 128, 0, st>>>(tasks, idx, n, tb, tb_words, cig);
}

}  // namespace dcns
