// Adaptive-band x-drop seed extension (SemiGlobal_xextend, impl/sequenceAlignment3.cpp:1234-1451, driven by
// x_extend_seed, impl/findSimilarFragmentsForPairedSequence4.cpp:205-285) and its traceback.
//
// One thread runs one pass of one seed.  The band is stored diagonal-relative: index k = j - i + w, so the diagonal
// predecessor of (i, j) sits at the same index in the previous row and the vertical predecessor at k + 1, and both
// arrays update in place left to right.  For w <= the template capacity the band lives in registers; wider bands
// (after several band-edge restarts) use a per-thread global scratch.
//
// A pass ends in one of three states: done, "restart" (the row maximum touched a band edge: the reference recomputes
// from scratch with 2w, and so does the host by relaunching the seed with the doubled width), or "slot too small"
// (the reverse pass's direction codes outgrew the seed's traceback slot; the host relaunches it with a larger one).
//
// Direction codes (reverse pass) are 4-bit nibbles per band cell: bits 0-1 = winning state (0 diag, 1 vertical,
// 2 horizontal), bit 2 = vertical gap extended, bit 3 = horizontal gap extended; state 3 marks cells the reference
// never writes (its Matrix::reset value 255).  Eight nibbles per word, ceil((2w+1)/8) words per row.
#include "device_common.cuh"

namespace dcns {

__device__ __forceinline__ int xd_words_per_row(int w) { return (2 * w + 1 + 7) / 8; }

template <int WC>
__device__ void xdrop_pass(XTask &T, const Arena &ar, const Params &P, uint32_t *__restrict__ tb, int32_t *Ms,
                           int32_t *Fs) {
  const int w = T.w, n1 = T.n1, n2 = T.n2;
  const int open = P.open1, ext = P.ext1;
  const SeqView s1{T.base1, T.a1, T.dir}, s2{T.base2, T.a2, T.dir};
  constexpr int NA = WC > 0 ? 2 * WC + 2 : 1;
  int32_t Mr[NA], Fr[NA];
  int32_t *M = WC > 0 ? Mr : Ms;
  int32_t *F = WC > 0 ? Fr : Fs;
  const int nk = 2 * w + 1;
  if (WC > 0) {
#pragma unroll
    for (int k = 0; k < NA; ++k) Mr[k] = kOut, Fr[k] = kOut;
  } else {
    for (int k = 0; k < nk + 1; ++k) M[k] = kOut, F[k] = kOut;
  }
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
    auto cell = [&](int32_t *Mv, int32_t *Fv, int k) {
      const int j = i - w + k;
      uint32_t nib = 0xFu;
      if (j >= c0 && j <= c1) {
        const int32_t diag = (j == 1) ? (i == 1 ? 0 : kOut) : Mv[k];
        const int32_t fin = (j == c1) ? kOut : Fv[k + 1];
        int32_t v = score_of(ci, s2.at(ar, j - 1), P.match, P.mismatch) + diag;
        uint32_t d = v > fin ? 0u : 1u;
        if (!(v > fin)) v = fin;
        if (!(v > e)) {
          d = 2u;
          v = e;
        }
        Mv[k] = v;
        if (v > best) {
          best = v;
          bestj = j;
        }
        const int32_t h = v + open;
        const int32_t f = fin + ext;
        if (f >= h) d |= 4u;
        Fv[k] = f >= h ? f : h;
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
    };
    if constexpr (WC > 0) {
#pragma unroll
      for (int k = 0; k < 2 * WC + 1; ++k)
        if (k < nk) cell(Mr, Fr, k);
    } else {
      for (int k = 0; k < nk; ++k) cell(M, F, k);
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

void launch_xdrop(XTask *tasks, const int *idx, int n, Arena ar, Params p, uint32_t *tb, int wcap, int32_t *scratch,
                  int64_t scratch_per_thread, cudaStream_t st) {
  if (n <= 0) return;
  const int g = (n + 127) / 128;
  if (wcap == 10)
    xdrop_kernel<10><<<g, 128, 0, st>>>(tasks, idx, n, ar, p, tb, scratch, 0);
  else if (wcap == 20)
    xdrop_kernel<20><<<g, 128, 0, st>>>(tasks, idx, n, ar, p, tb, scratch, 0);
  else
    xdrop_kernel<0><<<g, 128, 0, st>>>(tasks, idx, n, ar, p, tb, scratch, scratch_per_thread);
}

// ------------------------------------------------------------------ traceback of the reverse pass
// State machine of impl/sequenceAlignment3.cpp:1413-1438: start in the state that produced the cell; a gap state
// persists while the cell's continuation bit is set; ops are appended as the walk goes (no final reverse, because
// the walk over the reverse-complement pass already runs in forward order).  Unwritten cells read 255.
__global__ void xdrop_traceback_kernel(XTask *__restrict__ tasks, const int *__restrict__ idx, int n,
                                       const uint32_t *__restrict__ tb, uint32_t *__restrict__ cig) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  XTask &T = tasks[idx[t]];
  const int w = T.w, wpr = xd_words_per_row(w);
  int ii = T.end1, jj = T.end2, state = 0, nc = 0;
  uint32_t *out = cig + T.cig_off;
  uint32_t last = 0xFFFFFFFFu;
  while (ii > 0 && jj > 0) {
    int code = 255;
    const int k = jj - ii + w;
    if (ii <= T.rows && k >= 0 && k <= 2 * w) {
      const uint32_t nib = (tb[T.tb_off + (int64_t)(ii - 1) * wpr + (k >> 3)] >> (4 * (k & 7))) & 0xFu;
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
    } else {
      if (nc >= T.cig_cap) {
        T.status = 3;
        break;
      }
      last = (1u << 4) | op;
      out[nc++] = last;
    }
  }
  T.iii = ii;
  T.jjj = jj;
  T.ncig = nc;
}

void launch_xdrop_traceback(XTask *tasks, const int *idx, int n, const uint32_t *tb, uint32_t *cig, cudaStream_t st) {
  if (n <= 0) return;
  xdrop_traceback_kernel<<<(n + 127) / 128, 128, 0, st>>>(tasks, idx, n, tb, cig);
}

}  // namespace dcns
