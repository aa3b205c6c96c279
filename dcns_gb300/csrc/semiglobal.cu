// Two-piece affine semi-global DP with z-drop and band (SemiGlobal_no_avx, impl/sequenceAlignment3.cpp:681-928)
// and its traceback.
//
// One CTA of 8 warps runs one DP.  Rows are processed in stripes of 32 (lane l owns row 32s+1+l), stripe s on warp
// s mod 8, each as an anti-diagonal wavefront: at step t lane l computes column j = jstart + t - l, receiving the cell
// above (M, both vertical-gap states, and the query code) from lane l-1 through __shfl_up_sync.  Lane 0 takes the row
// above the stripe from the previous stripe, written to global scratch at least one CTA barrier earlier and staged
// into shared memory 32-63 steps ahead of use, so consecutive stripes run concurrently on different warps.  The
// horizontal gap states stay in registers of the lane that owns the row.
//
// Direction codes are one byte per cell (state 0..4 in bits 0-2, gap-continuation flags in bits 3-6): the reference's
// traceback needs all seven bits to stay bit-exact.  Layout: stripe-major, then step, then lane, so the 32 lanes of a
// step write 32 consecutive bytes (one coalesced sector).  Cells the reference never writes (outside the band and
// the band's last column) are never read: the traceback's bounds test returns 255 for them.
//
// Row-level decisions (running maximum, z-drop, empty row) depend on all earlier rows, so each stripe is computed
// first and its 32 rows are then evaluated in order; rows after a stop are discarded.  Rows past n2 + w have an empty
// band: the reference then scores only the last column from a stale cell of column n2-1, which is replayed exactly
// from the two values the DP left there.
#include "device_common.cuh"

namespace dcns {

__host__ __device__ inline int64_t sg_stride_steps(int n2, int w) {
  return (int64_t)(n2 < 2 * w + 32 ? n2 : 2 * w + 32) + 32;
}

int64_t sg_tb_bytes(int n1, int n2, int w) {
  if (n1 <= 0 || n2 <= 0) return 0;
  return (int64_t)((n1 + 31) / 32) * sg_stride_steps(n2, w) * 32;
}

constexpr int kSgNW = 8;  // warps per CTA; one CTA runs one DP, warp w owns stripes w, w+8, ...
constexpr int kSgD = 2;   // super-steps between the starts of consecutive stripes

struct SgRec {
  int m, f1, f2;
};

// Super-step length K (wavefront steps between CTA barriers) for a DP whose stripes take at most smax steps:
//  * a warp finishes stripe s before stripe s+8 starts:   kSgD * kSgNW * K >= smax
//  * every boundary cell is written at least one barrier before the consumer stages it 32-63 steps ahead of use:
//    (kSgD - 1) * K >= 127
__host__ __device__ inline int sg_superstep(int n2, int w) {
  const int smax = (n2 < 2 * w + 32 ? n2 : 2 * w + 32) + 31;
  const int k = (smax + kSgD * kSgNW - 1) / (kSgD * kSgNW);
  return k > 128 ? k : 128;
}

// One CTA per DP, on a fixed schedule: stripe s runs steps [(g - 2s) K, (g - 2s + 1) K) in super-step g, and all
// warps meet at a barrier after every super-step, so every cross-warp dependency (the row above a stripe, the row
// evaluation order, the stop decision) crosses at least one __syncthreads.  There are no flag waits.
//   bnd   global scratch of this CTA: per stripe slot (s mod 8), the stripe's last row (M, F1, F2) by column
__global__ void __launch_bounds__(32 * kSgNW) sg_kernel(SgTask *__restrict__ tasks, const int *__restrict__ idx,
                                                         int n, Arena ar, Params P, uint8_t *__restrict__ tb,
                                                         SgRec *__restrict__ bnd_all, int64_t bnd_stride,
                                                         int *__restrict__ counter) {
  __shared__ SgRec stage[kSgNW][2][32];      // per warp: boundary cells of the next two 32-column chunks
  __shared__ int row_best[kSgNW][32], row_bestj[kSgNW][32];
  __shared__ int done_stripe[kSgNW];
  __shared__ int s_max, s_end1, s_end2, s_rows, s_next_eval, s_stop, s_stale_last, s_stale_prev, s_task;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int o1 = P.open1, x1 = P.ext1, o2 = P.open2, x2 = P.ext2, w = P.bandwidth;
  SgRec *bnd = bnd_all + (int64_t)blockIdx.x * kSgNW * bnd_stride;
  for (;;) {
    if (threadIdx.x == 0) s_task = atomicAdd(counter, 1);
    __syncthreads();
    const int q = s_task;
    if (q >= n) break;
    if (threadIdx.x < kSgNW) done_stripe[threadIdx.x] = -1;
    if (threadIdx.x == 0) {
      s_max = 0, s_end1 = -1, s_end2 = -1, s_rows = 0, s_next_eval = 0, s_stop = 0;
      s_stale_last = kOut, s_stale_prev = kOut;
    }
    __syncthreads();
    SgTask &T = tasks[idx[q]];
    const int n1 = T.n1, n2 = T.n2;
    const SeqView s1{T.base1, T.a1, T.dir}, s2{T.base2, T.a2, T.dir};
    const bool codes = T.want_codes != 0;
    const int r_last = n2 - 1 + w;
    const int n1_eff = (n1 <= 0 || n2 <= 0) ? 0 : min(n1, n2 + w);  // rows with a non-empty band
    const int nstripes = (n1_eff + 31) / 32;
    const int64_t stride = sg_stride_steps(n2, w);
    const int K = sg_superstep(n2, w);
    // per-warp stripe state (registers persist across super-steps)
    int cs = warp;  // this warp's current stripe
    int i = 0, c0 = 0, c1 = 0, jstart = 0, nsteps = 0, upB = 0, ci = 0, tdone = 0;
    bool live = false, produce = false;
    int e1 = kOut, e2 = kOut, best = 0, bestj = 0, diag = kOut;
    int outM = kOut, outF1 = kOut, outF2 = kOut, outC = 0;
    SgRec *bup = nullptr, *bdown = nullptr;
    uint8_t *trow = nullptr;
    auto stage_chunk = [&](int chunk) {  // columns jstart + 32*chunk + lane of the row above, into stage[chunk & 1]
      const int j = jstart + 32 * chunk + lane;
      SgRec r{kOut, kOut, kOut};
      if (cs > 0 && j >= 1 && j <= upB) r = bup[j];
      stage[warp][chunk & 1][lane] = r;
    };
    auto begin_stripe = [&]() {
      const int s = cs;
      i = 32 * s + 1 + lane;
      live = i <= n1_eff;
      c0 = max(i - w, 1);
      c1 = min(i + w, n2);
      const int r0 = 32 * s + 1, rl = min(32 * s + 32, n1_eff);
      jstart = max(r0 - w, 1);
      nsteps = min(rl + w, n2) - jstart + 1 + 31;
      upB = min(32 * s + w, n2);  // the row above (32s) holds columns [max(32s - w, 1), upB]
      produce = s + 1 < nstripes;
      ci = live ? s1.at(ar, i - 1) : 0;
      trow = tb + T.tb_off + (int64_t)s * stride * 32;
      bup = bnd + (int64_t)((s + kSgNW - 1) % kSgNW) * bnd_stride;
      bdown = bnd + (int64_t)(s % kSgNW) * bnd_stride;
      e1 = kOut, e2 = kOut, best = 0, bestj = 0;
      diag = (lane == 0 && s > 0 && jstart > 1) ? bup[jstart - 1].m : kOut;
      outM = kOut, outF1 = kOut, outF2 = kOut, outC = 0;
      tdone = 0;
      stage_chunk(0);
      stage_chunk(1);
      __syncwarp();
    };
    const int nsuper = nstripes > 0 ? kSgD * (nstripes - 1) + (sg_stride_steps(n2, w) + K - 1) / K + 1 : 0;
    bool started = false;
    for (int g = 0; g < nsuper; ++g) {
      // ---- compute: the warp's current stripe, if it is scheduled in this super-step
      if (cs < nstripes && g >= kSgD * cs) {
        if (!started) {
          begin_stripe();
          started = true;
        }
        const int tend = min(nsteps, (g - kSgD * cs + 1) * K);
        for (int t = tdone; t < tend; ++t) {
          int upM = __shfl_up_sync(0xFFFFFFFFu, outM, 1);
          int upF1 = __shfl_up_sync(0xFFFFFFFFu, outF1, 1);
          int upF2 = __shfl_up_sync(0xFFFFFFFFu, outF2, 1);
          int cj = __shfl_up_sync(0xFFFFFFFFu, outC, 1);
          if ((t & 31) == 0 && t > 0) {
            __syncwarp();
            stage_chunk((t >> 5) + 1);  // two chunks ahead of lane 0's reads
          }
          const int j = jstart + t - lane;
          if (lane == 0) {
            const SgRec r = stage[warp][(t >> 5) & 1][t & 31];
            upM = r.m, upF1 = r.f1, upF2 = r.f2;
            cj = j <= n2 ? s2.at(ar, j - 1) : 0;
          }
          int cM = kOut, cF1 = kOut, cF2 = kOut;
          uint8_t code = 255;
          if (live && j >= c0 && j <= c1) {
            const int dg = (j == 1) ? (i == 1 ? 0 : kOut) : diag;
            const bool last = (j == c1);
            const int fin1 = last ? kOut : upF1, fin2 = last ? kOut : upF2;
            int v = score_of(ci, cj, P.match, P.mismatch) + dg;
            int d = 0;
            if (!(v > fin1)) d = 1, v = fin1;
            if (!(v > e1)) d = 2, v = e1;
            if (!(v > fin2)) d = 3, v = fin2;
            if (!(v > e2)) d = 4, v = e2;
            cM = v;
            if (v > best) best = v, bestj = j;
            if (j == n2 - 1) {
              if (i == r_last) s_stale_last = v;
              if (i == r_last - 1) s_stale_prev = v;
            }
            if (!last) {
              const int h = v + o1, f = fin1 + x1;
              if (f >= h) d |= 8;
              cF1 = f >= h ? f : h;
              e1 += x1;
              if (e1 >= h) d |= 16;
              e1 = e1 >= h ? e1 : h;
              const int h2 = v + o2, f2 = fin2 + x2;
              if (f2 >= h2) d |= 32;
              cF2 = f2 >= h2 ? f2 : h2;
              e2 += x2;
              if (e2 >= h2) d |= 64;
              e2 = e2 >= h2 ? e2 : h2;
              code = (uint8_t)d;
            }
            if (lane == 31 && produce) bdown[j] = SgRec{cM, cF1, cF2};
          }
          if (codes && live) trow[(int64_t)t * 32 + lane] = code;
          diag = upM;
          outM = cM, outF1 = cF1, outF2 = cF2, outC = cj;
        }
        tdone = tend;
        if (tdone == nsteps) {  // stripe complete: publish its rows for the in-order evaluation
          row_best[cs % kSgNW][lane] = best;
          row_bestj[cs % kSgNW][lane] = bestj;
          __syncwarp();
          if (lane == 0) done_stripe[cs % kSgNW] = cs;
          cs += kSgNW;
          started = false;
        }
      }
      __syncthreads();
      // ---- evaluate finished stripes in row order (warp 0, lane 0)
      if (threadIdx.x == 0 && !s_stop) {
        int mx = s_max, e1r = s_end1, e2r = s_end2, rows = s_rows, ne = s_next_eval;
        bool stop = false;
        while (!stop && ne < nstripes && done_stripe[ne % kSgNW] == ne) {
          for (int r = 0; r < 32 && !stop; ++r) {
            const int ii = 32 * ne + 1 + r;
            if (ii > n1_eff) break;
            const int tm = row_best[ne % kSgNW][r], tj = row_bestj[ne % kSgNW][r];
            if (tm > mx) mx = tm, e1r = ii, e2r = tj;
            int l = (ii - e1r) - (tj - e2r);
            l = l > 0 ? l : -l;
            rows = ii;
            if (mx - tm > P.zdrop + l * x2)
              stop = true;
            else if (tj <= 0)
              stop = true;
          }
          ++ne;
        }
        s_max = mx, s_end1 = e1r, s_end2 = e2r, s_rows = rows, s_next_eval = ne;
        if (stop) s_stop = 1;
      }
      __syncthreads();
      if (s_stop || s_next_eval >= nstripes) break;  // uniform: every thread reads the same shared values
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int mx = s_max, e1r = s_end1, e2r = s_end2, rows = s_rows;
      bool stop = s_stop != 0;
      if (!stop && n1 > n1_eff && n2 >= 1 && n1_eff > 0) {
        // empty-band rows: only the last column, from the stale column n2-1 of the row with the same parity
        const int c2 = s2.at(ar, n2 - 1);
        for (int ii = n1_eff + 1; ii <= n1 && !stop; ++ii) {
          const int dg = (n2 == 1) ? (int)kOut : (((ii - 1 - r_last) % 2 == 0) ? s_stale_last : s_stale_prev);
          int v = score_of(s1.at(ar, ii - 1), c2, P.match, P.mismatch) + dg;
          if (!(v > kOut)) v = kOut;
          const int tm = v > 0 ? v : 0, tj = v > 0 ? n2 : 0;
          if (tm > mx) mx = tm, e1r = ii, e2r = tj;
          int l = (ii - e1r) - (tj - e2r);
          l = l > 0 ? l : -l;
          rows = ii;
          if (mx - tm > P.zdrop + l * x2)
            stop = true;
          else if (tj <= 0)
            stop = true;
        }
      }
      T.score = mx;
      T.end1 = e1r;
      T.end2 = e2r;
      T.rows = rows;
      T.status = 0;
    }
    __syncthreads();
  }
}

int sg_ctas_per_sm() {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, sg_kernel, 32 * kSgNW, 0) != cudaSuccess) {
    (void)cudaGetLastError();
    nb = 1;
  }
  return nb > 0 ? nb : 1;
}

int64_t sg_bnd_bytes(int grid, int max_n2) { return (int64_t)grid * kSgNW * ((int64_t)max_n2 + 2) * sizeof(SgRec); }

void launch_semiglobal(SgTask *tasks, const int *idx, int n, Arena ar, Params p, uint8_t *tb, void *bnd,
                       int max_n2, int *work_counter, int grid, cudaStream_t st) {
  if (n <= 0) return;
  sg_kernel<<<grid, 32 * kSgNW, 0, st>>>(tasks, idx, n, ar, p, tb, (SgRec *)bnd, (int64_t)max_n2 + 2, work_counter);
}

// ------------------------------------------------------------------ traceback (:869-914)
__global__ void sg_traceback_kernel(SgTask *__restrict__ tasks, const int *__restrict__ idx, int n, int w,
                                    const uint8_t *__restrict__ tb, uint32_t *__restrict__ cig) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  SgTask &T = tasks[idx[k]];
  const int n2 = T.n2;
  const int64_t stride = sg_stride_steps(n2, w);
  int ii = T.end1, jj = T.end2, state = 0, nc = 0;
  uint32_t *out = cig + T.cig_off;
  uint32_t last = 0xFFFFFFFFu;
  auto push = [&](uint32_t op) {
    if (nc > 0 && (last & 0xFu) == op) {
      last += 1u << 4;
      out[nc - 1] = last;
    } else if (nc < T.cig_cap) {
      last = (1u << 4) | op;
      out[nc++] = last;
    } else {
      T.status = 3;
    }
  };
  while (ii > 0 && jj > 0) {
    int code = 255;
    const int c0 = max(ii - w, 1), c1 = min(ii + w, n2);
    if (ii <= T.rows && jj >= c0 && jj < c1) {
      const int s = (ii - 1) >> 5, l = (ii - 1) & 31;
      const int jstart = max(32 * s + 1 - w, 1);
      const int64_t t = jj - jstart + l;
      code = tb[T.tb_off + ((int64_t)s * stride + t) * 32 + l];
    }
    if (state == 0)
      state = code & 7;
    else if (!((code >> (state + 2)) & 1))
      state = 0;
    if (state == 0) state = code & 7;
    if (state == 0) {
      push(0);
      --ii;
      --jj;
    } else if (state == 1 || state == 3) {
      push(2);
      --ii;
    } else {
      push(1);
      --jj;
    }
  }
  while (ii > 0) push(2), --ii;
  while (jj > 0) push(1), --jj;
  for (int a = 0, b = nc - 1; a < b; ++a, --b) {  // the reference reverses the walk (:915)
    const uint32_t tmp = out[a];
    out[a] = out[b];
    out[b] = tmp;
  }
  T.ncig = nc;
}

void launch_sg_traceback(SgTask *tasks, const int *idx, int n, int bandwidth, const uint8_t *tb, uint32_t *cig,
                         cudaStream_t st) {
  if (n <= 0) return;
  sg_traceback_kernel<<<(n + 127) / 128, 128, 0, st>>>(tasks, idx, n, bandwidth, tb, cig);
}

}  // namespace dcns
