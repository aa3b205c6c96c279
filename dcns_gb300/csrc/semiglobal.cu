// Two-piece affine semi-global DP with z-drop and band (SemiGlobal_no_avx, impl/sequenceAlignment3.cpp:681-928)
// and its traceback.
//
// Rows are processed in stripes of 128: lane l owns the four consecutive rows 128s+1+4l .. 128s+4+4l of stripe s as
// an anti-diagonal wavefront: at step t lane l computes column j = jstart + t - l for its four rows top to bottom,
// receiving the cell above its first row (M, both vertical-gap states, and the query code) from lane l-1 through
// __shfl_up_sync; rows inside a lane pass the cell above in registers.  Lane 0 takes the row above the stripe from
// the stripe before, through a boundary row in global memory staged into shared memory (with the query codes) 32-63
// steps ahead of use.  The horizontal gap states stay in registers of the lane that owns the row.  Each cell's
// priority chain (diag > F1 > E1 > F2 > E2) and gap updates use the DPX max-with-predicate instruction, which yields
// the maximum and the reference's comparison bit at once.
//
// Two schedules of the stripes.  The batched path runs every stripe of every DP as an independent unit of one
// persistent grid (sg_flow_kernel: a long DP spreads over as many warps as it has stripes).  The one-pair entry point
// without allocation keeps a whole DP on one CTA whose warps take its stripes in turn on a barrier schedule
// (sg_kernel), which needs only one CTA's boundary rows.
//
// Direction codes are one byte per cell (state 0..4 in bits 0-2, gap-continuation flags in bits 3-6): the reference's
// traceback needs all seven bits to stay bit-exact.  Layout: stripe-major, then step, then lane, one 32-bit word per
// lane and step holding its four rows, so the 32 lanes of a step write 128 consecutive bytes.  Cells the reference
// never writes (outside the band and the band's last column) are never read: the traceback's bounds test returns 255
// for them.
//
// Row-level decisions (running maximum, z-drop, empty row) depend on all earlier rows, so each stripe is computed
// first and its 128 rows are then evaluated in order; rows after a stop are discarded.  Rows past n2 + w have an empty
// band: the reference then scores only the last column from a stale cell of column n2-1, which is replayed exactly
// from the two values the DP left there.
#include <algorithm>
#include <climits>

#include "device_common.cuh"

namespace dcns {

constexpr int kSgD = 2;              // super-steps between the starts of consecutive stripes
constexpr int kSgR = 4;              // rows per lane
constexpr int kSgRows = 32 * kSgR;  // rows per stripe

// Wavefront steps of one stripe (columns its rows span, plus the 31-step lane skew), an upper bound for every stripe.
// Computed in 64 bits: 2w + kSgRows does not fit an int for bands near 2^30.
__host__ __device__ inline int64_t sg_stride_steps(int n2, int w) {
  const int64_t span = 2 * (int64_t)w + kSgRows;
  return (n2 < span ? (int64_t)n2 : span) + 32;
}

int64_t sg_tb_bytes(int n1, int n2, int w) {
  if (n1 <= 0 || n2 <= 0) return 0;
  return (int64_t)((n1 + kSgRows - 1) / kSgRows) * sg_stride_steps(n2, w) * 32 * kSgR;
}

// Super-step length K (wavefront steps between CTA barriers) for a DP whose stripes take at most smax steps, on a CTA
// of nw warps:
//  * a warp finishes stripe s before stripe s+nw starts:   kSgD * nw * K >= smax
//  * every boundary cell is written at least one barrier before the consumer stages it 32-63 steps ahead of use.
//    Stripe s writes column j at its step j - jstart_s + 31; stripe s+1, which starts kSgD super-steps later, stages
//    it at step j - jstart_{s+1} - 63 or later, and jstart_{s+1} - jstart_s <= kSgRows; so the producer is at most
//    kSgRows + 94 steps ahead of that read, which must be at most (kSgD - 1) * K:  K >= kSgRows + 96
__host__ __device__ inline int sg_superstep(int n2, int w, int nw) {
  const int64_t span = 2 * (int64_t)w + kSgRows;
  const int smax = (int)(n2 < span ? (int64_t)n2 : span) + 31;
  const int k = (smax + kSgD * nw - 1) / (kSgD * nw);
  static_assert(kSgD == 2, "the lower bound below assumes two super-steps between stripe starts");
  return k > kSgRows + 96 ? k : kSgRows + 96;
}

// One CTA of NW warps per DP (stripe s on warp s mod NW), on a fixed schedule: stripe s runs steps
// [(g - 2s) K, (g - 2s + 1) K) in super-step g, and all warps meet at a barrier after every super-step, so every cross-warp dependency (the row above a stripe, the row
// evaluation order, the stop decision) crosses at least one __syncthreads.  There are no flag waits.
//   bnd   global scratch of this CTA: per stripe slot (s mod 8), the stripe's last row (M, F1, F2) by column
template <int NW>
__global__ void __launch_bounds__(32 * NW) sg_kernel(SgTask *__restrict__ tasks, const int *__restrict__ idx, int n,
                                                      Arena ar, Params P, uint8_t *__restrict__ tb,
                                                      SgRec *__restrict__ bnd_all, int64_t bnd_stride,
                                                      int *__restrict__ counter) {
  __shared__ SgRec stage[NW][2][32];  // per warp: boundary cells of the next two 32-column chunks
  __shared__ int stage_c[NW][2][32];  // and the query codes of those columns
  __shared__ int row_best[NW][kSgRows], row_bestj[NW][kSgRows];
  __shared__ int done_stripe[NW];
  __shared__ int s_max, s_end1, s_end2, s_rows, s_next_eval, s_stop, s_stale_last, s_stale_prev, s_task;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int o1 = P.open1, x1 = P.ext1, o2 = P.open2, x2 = P.ext2, w = P.bandwidth;
  SgRec *bnd = bnd_all + (int64_t)blockIdx.x * NW * bnd_stride;
  for (;;) {
    if (threadIdx.x == 0) s_task = atomicAdd(counter, 1);
    __syncthreads();
    const int q = s_task;
    if (q >= n) break;
    if (threadIdx.x < NW) done_stripe[threadIdx.x] = -1;
    if (threadIdx.x == 0) {
      // ends are 1-based rows/columns and stay -1 while no cell is positive: the reference then reports -2 (0-based)
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
    const int nstripes = (n1_eff + kSgRows - 1) / kSgRows;
    const int64_t stride = sg_stride_steps(n2, w);
    const int K = sg_superstep(n2, w, NW);
    // per-warp stripe state (registers persist across super-steps)
    int cs = warp;  // this warp's current stripe
    int i0 = 0, jstart = 0, nsteps = 0, upB = 0, tdone = 0;
    bool live = false, produce = false;
    int ci[kSgR], c0[kSgR], c1[kSgR], e1[kSgR], e2[kSgR], best[kSgR], bestj[kSgR], prevM[kSgR];
    bool liver[kSgR];
    int diag = kOut, outM = kOut, outF1 = kOut, outF2 = kOut, outC = 0;
    SgRec *bup = nullptr, *bdown = nullptr;
    uint32_t *trow = nullptr;
    auto stage_chunk = [&](int chunk) {  // columns jstart + 32*chunk + lane of the row above, into stage[chunk & 1]
      const int j = jstart + 32 * chunk + lane;
      SgRec r{kOut, kOut, kOut};
      if (cs > 0 && j >= 1 && j <= upB) r = bup[j];
      stage[warp][chunk & 1][lane] = r;
      stage_c[warp][chunk & 1][lane] = (j >= 1 && j <= n2) ? s2.at(ar, j - 1) : 0;
    };
    auto begin_stripe = [&]() {
      const int s = cs;
      i0 = kSgRows * s + 1 + kSgR * lane;
      live = i0 <= n1_eff;
#pragma unroll
      for (int k = 0; k < kSgR; ++k) {
        const int i = i0 + k;
        liver[k] = i <= n1_eff;
        c0[k] = max(i - w, 1);
        c1[k] = min(i + w, n2);
        ci[k] = liver[k] ? s1.at(ar, i - 1) : 0;
        e1[k] = kOut, e2[k] = kOut, best[k] = 0, bestj[k] = 0, prevM[k] = kOut;
      }
      const int r0 = kSgRows * s + 1, rl = min(kSgRows * s + kSgRows, n1_eff);
      jstart = max(r0 - w, 1);
      nsteps = min(rl + w, n2) - jstart + 1 + 31;
      upB = min(kSgRows * s + w, n2);  // the row above (128s) holds columns [max(128s - w, 1), upB]
      produce = s + 1 < nstripes;
      trow = reinterpret_cast<uint32_t *>(tb + T.tb_off) + (int64_t)s * stride * 32;
      bup = bnd + (int64_t)((s + NW - 1) % NW) * bnd_stride;
      bdown = bnd + (int64_t)(s % NW) * bnd_stride;
      diag = (lane == 0 && s > 0 && jstart > 1) ? bup[jstart - 1].m : kOut;
      outM = kOut, outF1 = kOut, outF2 = kOut, outC = 0;
      tdone = 0;
      stage_chunk(0);
      stage_chunk(1);
      __syncwarp();
    };
    const int nsuper = nstripes > 0 ? kSgD * (nstripes - 1) + (int)((stride + K - 1) / K) + 1 : 0;
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
            cj = stage_c[warp][(t >> 5) & 1][t & 31];
          }
          // the lane's rows top to bottom; (aM, aF1, aF2) = the cell above, dg = the diagonal cell
          int aF1 = upF1, aF2 = upF2, dg = diag;
          uint32_t word = 0xFFFFFFFFu;
#pragma unroll
          for (int k = 0; k < kSgR; ++k) {
            const int i = i0 + k;
            int cM = kOut, cF1 = kOut, cF2 = kOut;
            if (liver[k] && j >= c0[k] && j <= c1[k]) {
              const int dgv = (j == 1) ? (i == 1 ? 0 : kOut) : dg;
              const bool last = (j == c1[k]);
              const int fin1 = last ? kOut : aF1, fin2 = last ? kOut : aF2;
              int v = score_of(ci[k], cj, P.match, P.mismatch) + dgv;
              int d = 0;
              bool pr;
              v = __vibmax_s32(fin1, v, &pr);  // pr: !(v > fin1)
              d = pr ? 1 : d;
              v = __vibmax_s32(e1[k], v, &pr);
              d = pr ? 2 : d;
              v = __vibmax_s32(fin2, v, &pr);
              d = pr ? 3 : d;
              v = __vibmax_s32(e2[k], v, &pr);
              d = pr ? 4 : d;
              cM = v;
              if (v > best[k]) best[k] = v, bestj[k] = j;
              if (j == n2 - 1) {
                if (i == r_last) s_stale_last = v;
                if (i == r_last - 1) s_stale_prev = v;
              }
              if (!last) {
                const int h = v + o1, h2 = v + o2;
                cF1 = __vibmax_s32(fin1 + x1, h, &pr);
                d |= pr ? 8 : 0;
                e1[k] = __vibmax_s32(e1[k] + x1, h, &pr);
                d |= pr ? 16 : 0;
                cF2 = __vibmax_s32(fin2 + x2, h2, &pr);
                d |= pr ? 32 : 0;
                e2[k] = __vibmax_s32(e2[k] + x2, h2, &pr);
                d |= pr ? 64 : 0;
                word = (word & ~(0xFFu << (8 * k))) | ((uint32_t)d << (8 * k));
              }
              if (k == kSgR - 1 && lane == 31 && produce) bdown[j] = SgRec{cM, cF1, cF2};
            }
            dg = prevM[k];  // row k at column j - 1: the diagonal of row k + 1
            prevM[k] = cM;
            aF1 = cF1, aF2 = cF2;
            if (k == kSgR - 1) outM = cM;
          }
          if (codes && live) trow[(int64_t)t * 32 + lane] = word;
          diag = upM;
          outF1 = aF1, outF2 = aF2, outC = cj;
        }
        tdone = tend;
        if (tdone == nsteps) {  // stripe complete: publish its rows for the in-order evaluation
#pragma unroll
          for (int k = 0; k < kSgR; ++k) {
            row_best[cs % NW][kSgR * lane + k] = best[k];
            row_bestj[cs % NW][kSgR * lane + k] = bestj[k];
          }
          __syncwarp();
          if (lane == 0) done_stripe[cs % NW] = cs;
          cs += NW;
          started = false;
        }
      }
      __syncthreads();
      // ---- evaluate finished stripes in row order (warp 0, lane 0)
      if (threadIdx.x == 0 && !s_stop) {
        int mx = s_max, e1r = s_end1, e2r = s_end2, rows = s_rows, ne = s_next_eval;
        bool stop = false;
        while (!stop && ne < nstripes && done_stripe[ne % NW] == ne) {
          for (int r = 0; r < kSgRows && !stop; ++r) {
            const int ii = kSgRows * ne + 1 + r;
            if (ii > n1_eff) break;
            const int tm = row_best[ne % NW][r], tj = row_bestj[ne % NW][r];
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

// Resident CTAs per SM of the NW-warp kernel.
int sg_ctas_per_sm(int nw) {
  int nb = 0;
  cudaError_t e = nw == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, sg_kernel<2>, 64, 0)
                  : nw == 4 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, sg_kernel<4>, 128, 0)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, sg_kernel<kSgNW>, 32 * kSgNW, 0);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    nb = 1;
  }
  return nb > 0 ? nb : 1;
}

int64_t sg_bnd_bytes(int grid, int max_n2, int nw) {
  return (int64_t)grid * nw * ((int64_t)max_n2 + 2) * sizeof(SgRec);
}

void launch_semiglobal(SgTask *tasks, const int *idx, int n, Arena ar, Params p, uint8_t *tb, void *bnd,
                       int max_n2, int *work_counter, int grid, int nw, cudaStream_t st) {
  if (n <= 0) return;
  const int64_t stride = (int64_t)max_n2 + 2;
  if (nw == 2)
    sg_kernel<2><<<grid, 64, 0, st>>>(tasks, idx, n, ar, p, tb, (SgRec *)bnd, stride, work_counter);
  else if (nw == 4)
    sg_kernel<4><<<grid, 128, 0, st>>>(tasks, idx, n, ar, p, tb, (SgRec *)bnd, stride, work_counter);
  else
    sg_kernel<kSgNW><<<grid, 32 * kSgNW, 0, st>>>(tasks, idx, n, ar, p, tb, (SgRec *)bnd, stride, work_counter);
}

// ------------------------------------------------------------------ stripes as a flow of independent warp units
// The DPs of a launch are cut into their 128-row stripes (units), handed out by one atomic counter in the order of
// SgFlow::order; every warp of a persistent grid takes the next unit, computes it with the per-cell code of sg_kernel
// (same wavefront, same code layout), and takes the next.  The host orders the units stripe-major within groups of
// consecutive DPs (queue order: largest DPs first): stripe 0 of every DP of the group, then stripe 1, ... so that
// when a warp takes stripe s its stripe s - 1 has been running for a while, even when a few DPs of 200,000 rows make
// up the whole launch (in DP order the late stripes of one long DP would wait for its wavefront to reach them).
// Stripe s of a DP depends only
// on stripe s - 1: the last row of s - 1 reaches s through the DP's boundary row in global memory (one row per DP:
// stripe s reads a column before it overwrites it with its own last row, and s + 1 reads it only after s published
// it), and s - 1 publishes how many columns of that row it has written (release / acquire per 32-column chunk).  So
// a long DP runs on as many warps as it has stripes, each one chunk pair behind the stripe above it, instead of on
// one CTA.  Each DP's stripes are handed out in increasing order and a stripe waits only on lower stripes of its own
// DP, which are held by running warps, so the waits always end; each still has an iteration limit, after which the
// warp flags a device error (SgFlow::err) and abandons the DP.
//
// Row-level decisions (running maximum, z-drop, non-positive row maximum) are taken in row order: after computing
// stripe s, its warp waits until s - 1 is evaluated, evaluates its 128 rows from the DP's running state and
// publishes it; the stripe whose rows stop the DP, or its last stripe, writes the DP's result.  Stripes computed past
// the stop are abandoned at their next chunk (their codes lie past the DP's last row and are never read).
// Iteration limit of every wait: each iteration is an L2 load and a ~200 ns sleep, so a wait gives up after about a
// second or more; the longest legitimate wait (a stripe of 200,000 columns while its SM is shared) is some tens of ms.
constexpr int kSgSpin = 1 << 22;

__device__ __forceinline__ int sg_ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void sg_st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int sg_ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Waits until *flag >= need, or until *stop_flag != 0; every lane polls (one broadcast load).  Returns 1 when the
// flag is reached, 0 when the DP stopped, -1 when the iteration limit ran out or another warp already flagged an
// error (*err), so that after one failed wait the whole grid winds down instead of timing out wait after wait.
__device__ __forceinline__ int sg_wait_at_least(const int *flag, int need, const int *stop_flag, const int *err) {
  for (int it = 0; it < kSgSpin; ++it) {
    const bool ok = sg_ld_acquire(flag) >= need;
    if (__all_sync(0xFFFFFFFFu, ok)) return 1;
    if (__any_sync(0xFFFFFFFFu, sg_ld_relaxed(stop_flag) != 0)) return 0;
    if ((it & 63) == 63 && __any_sync(0xFFFFFFFFu, sg_ld_relaxed(err) != 0)) return -1;
    __nanosleep(200);
  }
  return -1;
}

constexpr int kSgFlowWarps = 4;  // warps per block of the flow kernel

// One cell of a flow stripe, branch-free: (aF1, aF2) = the vertical gap states of the cell above (kOut at the row's
// last band column, which no row above has in its band or updates), dg = the diagonal cell.  Cells outside the band
// leave kOut in M and both F, and reset the row's horizontal states to kOut (the reference starts a row with them
// OUT); the band's last column takes the cell's maximum but leaves kOut in both F (its gap states are not updated,
// and the row's horizontal states are not read again).  With CODES, *d gets the cell's direction code: the winning
// state (priority order diag, F1, E1, F2, E2, a later state winning ties) and the four gap-continuation flags;
// codes of cells outside the band or on its last column are never read by the traceback.
template <bool CODES>
__device__ __forceinline__ int sg_cell(int sc, int dg, int aF1, int aF2, int &e1, int &e2, bool valid, bool last,
                                       int o1, int x1, int o2, int x2, int &cF1, int &cF2, uint32_t *d) {
  int v = sc + dg, nF1, nF2, nE1, nE2;
  if (CODES) {
    bool pr;
    uint32_t c = 0;
    v = __vibmax_s32(aF1, v, &pr);  // pr: !(v > F1)
    c = pr ? 1u : c;
    v = __vibmax_s32(e1, v, &pr);
    c = pr ? 2u : c;
    v = __vibmax_s32(aF2, v, &pr);
    c = pr ? 3u : c;
    v = __vibmax_s32(e2, v, &pr);
    c = pr ? 4u : c;
    const int h = v + o1, h2 = v + o2;
    bool p1, p2, p3, p4;
    nF1 = __vibmax_s32(aF1 + x1, h, &p1);
    nE1 = __vibmax_s32(e1 + x1, h, &p2);
    nF2 = __vibmax_s32(aF2 + x2, h2, &p3);
    nE2 = __vibmax_s32(e2 + x2, h2, &p4);
    *d = c | (p1 ? 8u : 0u) | (p2 ? 16u : 0u) | (p3 ? 32u : 0u) | (p4 ? 64u : 0u);
  } else {
    v = __vimax3_s32(__vimax3_s32(v, aF1, e1), aF2, e2);
    nF1 = __viaddmax_s32(aF1, x1, v + o1);
    nE1 = __viaddmax_s32(e1, x1, v + o1);
    nF2 = __viaddmax_s32(aF2, x2, v + o2);
    nE2 = __viaddmax_s32(e2, x2, v + o2);
  }
  const bool upd = valid && !last;
  cF1 = upd ? nF1 : kOut;
  cF2 = upd ? nF2 : kOut;
  e1 = valid ? nE1 : kOut;
  e2 = valid ? nE2 : kOut;
  return valid ? v : kOut;
}

// MINB: resident blocks per SM the register allocation must allow (5: 96 registers; 6: 80, a few spilled words)
template <bool CODES, int MINB>
__global__ void __launch_bounds__(32 * kSgFlowWarps, MINB) sg_flow_kernel(SgFlow F, Arena ar, Params P,
                                                                         uint8_t *__restrict__ tb) {
  __shared__ SgRec stage[kSgFlowWarps][2][32];
  __shared__ int stage_c[kSgFlowWarps][2][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int o1 = P.open1, x1 = P.ext1, o2 = P.open2, x2 = P.ext2, w = P.bandwidth;
  for (;;) {
    long long u = 0;
    if (lane == 0) u = (long long)atomicAdd(F.unit_counter, 1ull);
    u = __shfl_sync(0xFFFFFFFFu, u, 0);
    if (u >= F.total_units) break;
    if (__any_sync(0xFFFFFFFFu, sg_ld_relaxed(F.err) != 0)) break;  // a wait ran out: the launch fails as a whole
    const int2 qs = F.order[u];  // the u-th unit handed out: stripe qs.y of DP qs.x
    const int q = qs.x, s = qs.y;
    const int64_t ui = F.unit_begin[q] + s;  // its progress counter
    SgTask &T = F.tasks[F.idx[q]];
    SgFlowDP &D = F.dps[q];
    int *const prog_self = F.prog + ui;
    const int n1 = T.n1, n2 = T.n2;
    const int n1_eff = (n1 <= 0 || n2 <= 0) ? 0 : min(n1, n2 + w);
    const int nstripes = (n1_eff + kSgRows - 1) / kSgRows;
    if (nstripes == 0) {  // nothing to align: the reference reports score 0 and ends -2 (0-based)
      if (lane == 0) T.score = 0, T.end1 = -1, T.end2 = -1, T.rows = 0, T.status = 0;
      continue;
    }
    if (__any_sync(0xFFFFFFFFu, sg_ld_relaxed(&D.stop) != 0)) {
      if (lane == 31) sg_st_release(prog_self, INT_MAX);
      continue;
    }
    const SeqView s1{T.base1, T.a1, T.dir}, s2{T.base2, T.a2, T.dir};
    const int r_last = n2 - 1 + w;
    const int64_t stride = sg_stride_steps(n2, w);
    SgRec *const brow = F.bnd + D.bnd_off;  // the DP's boundary row, by column
    const int *const prog_up = s > 0 ? F.prog + (ui - 1) : nullptr;
    const int i0 = kSgRows * s + 1 + kSgR * lane;
    const bool live = i0 <= n1_eff;
    // per row of the lane: band [c0, c0 + span] (rows past the DP: an empty band), its base, the stale-column role,
    // running states
    int ci[kSgR], rmask[kSgR], c0[kSgR], span[kSgR], e1[kSgR], e2[kSgR], best[kSgR], bestj[kSgR], prevM[kSgR];
    int stale_rows = 0;  // bit k: row k is row r_last (bit 4 + k: row r_last - 1)
#pragma unroll
    for (int k = 0; k < kSgR; ++k) {
      const int i = i0 + k;
      const bool lv = i <= n1_eff;
      c0[k] = lv ? max(i - w, 1) : INT_MAX / 2;
      span[k] = lv ? min(i + w, n2) - c0[k] : 0;
      ci[k] = lv ? s1.at(ar, i - 1) : 0;
      rmask[k] = ci[k] == 2 ? 0 : -1;  // Scorei: an N row scores 0 against every base
      if (lv && i == r_last) stale_rows |= 1 << k;
      if (lv && i == r_last - 1) stale_rows |= 16 << k;
      e1[k] = kOut, e2[k] = kOut, best[k] = 0, bestj[k] = 0, prevM[k] = kOut;
    }
    const int r0 = kSgRows * s + 1, rl = min(kSgRows * s + kSgRows, n1_eff);
    const int jstart = max(r0 - w, 1);
    const int nsteps = min(rl + w, n2) - jstart + 1 + 31;
    const int upB = min(kSgRows * s + w, n2);  // the row above (128s) holds columns [max(128s - w, 1), upB]
    const bool produce = s + 1 < nstripes;
    uint32_t *const trow = CODES ? reinterpret_cast<uint32_t *>(tb + T.tb_off) + (int64_t)s * stride * 32 : nullptr;
    int abandon = 0;  // 0 computing, 1 the DP stopped, -1 a wait ran out
    // columns jstart + 32 * chunk + lane of the row above, into stage[warp][chunk & 1]; the producer must have
    // published them first
    auto stage_chunk = [&](int chunk) {
      if (s > 0 && abandon == 0) {
        const int need = min(jstart + 32 * chunk + 31, upB);
        const int r = sg_wait_at_least(prog_up, need, &D.stop, F.err);
        if (r <= 0) abandon = r == 0 ? 1 : -1;
      }
      const int j = jstart + 32 * chunk + lane;
      SgRec rec{kOut, kOut, kOut};
      if (s > 0 && abandon == 0 && j >= 1 && j <= upB) {
        rec.m = __ldcg(&brow[j].m);
        rec.f1 = __ldcg(&brow[j].f1);
        rec.f2 = __ldcg(&brow[j].f2);
      }
      stage[warp][chunk & 1][lane] = rec;
      stage_c[warp][chunk & 1][lane] = (j >= 1 && j <= n2) ? s2.at(ar, j - 1) : 0;
    };
    stage_chunk(0);  // waits for columns up to jstart + 31, which include the diagonal column jstart - 1
    // the diagonal of the stripe's first row at column jstart: cell (0, 0) = 0 for the DP's first row, else the
    // row above at jstart - 1 (kOut at column 0)
    int diag = kOut;
    if (lane == 0) diag = s == 0 ? 0 : (jstart > 1 && abandon == 0) ? __ldcg(&brow[jstart - 1].m) : kOut;
    stage_chunk(1);
    __syncwarp();
    int outM = kOut, outF1 = kOut, outF2 = kOut, outC = 0;
    const bool lane0 = lane == 0, write_bnd = lane == 31 && produce;
    for (int tc = 0; tc < nsteps && abandon == 0; tc += 32) {  // 32-step chunks
      if (tc > 0) {
        // chunk boundary: publish the columns of this stripe's last row written so far, stop early if the DP
        // ended, stage the chunk two ahead of lane 0's reads
        if (write_bnd) sg_st_release(prog_self, jstart + tc - 32);
        if (__any_sync(0xFFFFFFFFu, sg_ld_relaxed(&D.stop) != 0)) {
          abandon = 1;
          break;
        }
        __syncwarp();
        stage_chunk((tc >> 5) + 1);
        if (abandon != 0) break;
      }
      const SgRec *const srow = stage[warp][(tc >> 5) & 1];
      const int *const scol = stage_c[warp][(tc >> 5) & 1];
      const int tend = min(tc + 32, nsteps);
      for (int t = tc; t < tend; ++t) {
        int upM = __shfl_up_sync(0xFFFFFFFFu, outM, 1);
        int upF1 = __shfl_up_sync(0xFFFFFFFFu, outF1, 1);
        int upF2 = __shfl_up_sync(0xFFFFFFFFu, outF2, 1);
        int cj = __shfl_up_sync(0xFFFFFFFFu, outC, 1);
        const int j = jstart + t - lane;
        if (lane0) {
          const SgRec r = srow[t - tc];
          upM = r.m, upF1 = r.f1, upF2 = r.f2;
          cj = scol[t - tc];
        }
        int aF1 = upF1, aF2 = upF2, dg = diag;
        uint32_t word = 0;
        const int mt = cj == 2 ? 0 : P.match, mm = cj == 2 ? 0 : P.mismatch;  // Scorei: N scores 0
        const bool stale_col = stale_rows != 0 && j == n2 - 1;
#pragma unroll
        for (int k = 0; k < kSgR; ++k) {
          const int dj = j - c0[k];
          const bool valid = (unsigned)dj <= (unsigned)span[k];
          const bool last = dj == span[k];
          const int sc = (ci[k] == cj ? mt : mm) & rmask[k];
          int cF1, cF2;
          uint32_t d = 0;
          const int cM = sg_cell<CODES>(sc, dg, aF1, aF2, e1[k], e2[k], valid, last, o1, x1, o2, x2, cF1, cF2, &d);
          if (CODES) word |= d << (8 * k);
          bool keep;
          best[k] = __vibmax_s32(best[k], cM, &keep);  // keep: !(cM > best), the first maximum of the row stays
          bestj[k] = keep ? bestj[k] : j;
          if (stale_col && valid) {
            if ((stale_rows >> k) & 1) D.stale_last = cM;
            if ((stale_rows >> (4 + k)) & 1) D.stale_prev = cM;
          }
          if (k == kSgR - 1 && write_bnd && valid) brow[j] = SgRec{cM, cF1, cF2};
          dg = prevM[k];  // row k at column j - 1: the diagonal of row k + 1
          prevM[k] = cM;
          aF1 = cF1, aF2 = cF2;
          if (k == kSgR - 1) outM = cM;
        }
        if (CODES && live) trow[(int64_t)t * 32 + lane] = word;
        diag = upM;
        outF1 = aF1, outF2 = aF2, outC = cj;
      }
    }
    __syncwarp();
    if (lane == 31) sg_st_release(prog_self, INT_MAX);  // every column written (or abandoned): release the consumer
    if (abandon < 0 && lane == 0) {
      atomicExch(F.err, 1);
      atomicExch(&D.stop, 1);
      T.status = 4;
    }
    if (abandon != 0) continue;
    // ---- the stripe's rows in order, from the DP's running state after stripe s - 1
    if (s > 0) {
      const int r = sg_wait_at_least(&D.evaluated, s, &D.stop, F.err);
      if (r <= 0) {
        if (r < 0 && lane == 0) {
          atomicExch(F.err, 1);
          atomicExch(&D.stop, 1);
          T.status = 4;
        }
        continue;
      }
      if (__any_sync(0xFFFFFFFFu, sg_ld_relaxed(&D.stop) != 0)) continue;  // an earlier stripe ended the DP
    }
    int mx = 0, e1r = -1, e2r = -1, rows = 0;  // ends are 1-based and stay -1 while no cell is positive
    if (s > 0) mx = sg_ld_relaxed(&D.mx), e1r = sg_ld_relaxed(&D.e1r), e2r = sg_ld_relaxed(&D.e2r),
               rows = sg_ld_relaxed(&D.rows);
    bool stop = false;
    for (int ol = 0; ol < 32; ++ol) {  // row 128s + 1 + 4 ol + k is lane ol's row k
#pragma unroll
      for (int k = 0; k < kSgR; ++k) {
        const int tm = __shfl_sync(0xFFFFFFFFu, best[k], ol), tj = __shfl_sync(0xFFFFFFFFu, bestj[k], ol);
        const int ii = r0 + kSgR * ol + k;
        if (!stop && ii <= n1_eff) {
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
    }
    if (lane == 0) {
      if (!stop && s == nstripes - 1 && n1 > n1_eff && n2 >= 1) {
        // empty-band rows: only the last column, from the stale column n2-1 of the row with the same parity
        const int c2 = s2.at(ar, n2 - 1);
        const int st_last = sg_ld_relaxed(&D.stale_last), st_prev = sg_ld_relaxed(&D.stale_prev);
        for (int ii = n1_eff + 1; ii <= n1 && !stop; ++ii) {
          const int dg = (n2 == 1) ? (int)kOut : (((ii - 1 - r_last) % 2 == 0) ? st_last : st_prev);
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
      if (stop || s == nstripes - 1) {
        T.score = mx;
        T.end1 = e1r;
        T.end2 = e2r;
        T.rows = rows;
        T.status = 0;
        if (stop) atomicExch(&D.stop, 1);
      } else {
        D.mx = mx, D.e1r = e1r, D.e2r = e2r, D.rows = rows;
      }
      __threadfence();
      sg_st_release(&D.evaluated, s + 1);
    }
    __syncwarp();
  }
}

int64_t sg_flow_units(int n1, int n2, int w) {
  const int64_t n1_eff = (n1 <= 0 || n2 <= 0) ? 0 : std::min<int64_t>(n1, (int64_t)n2 + w);
  return std::max<int64_t>(1, (n1_eff + kSgRows - 1) / kSgRows);
}

int sg_flow_blocks_per_sm(int minb) {
  static int nb[2] = {0, 0};
  int &r = nb[minb == 6 ? 1 : 0];
  if (r == 0) {
    int v = 0;
    const cudaError_t e = minb == 6 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, sg_flow_kernel<true, 6>,
                                                                                     32 * kSgFlowWarps, 0)
                                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, sg_flow_kernel<true, 5>,
                                                                                     32 * kSgFlowWarps, 0);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      v = 1;
    }
    r = v > 0 ? v : 1;
  }
  return r;
}

int64_t sg_flow_grid_warps(int nsm, int minb) { return (int64_t)nsm * sg_flow_blocks_per_sm(minb) * kSgFlowWarps; }

void launch_semiglobal_flow(const SgFlow &f, Arena ar, Params p, uint8_t *tb, bool codes, int nsm, int minb,
                            cudaStream_t st) {
  if (f.total_units <= 0) return;
  const int64_t warps = std::min<int64_t>(f.total_units, sg_flow_grid_warps(nsm, minb));
  const int blocks = (int)((warps + kSgFlowWarps - 1) / kSgFlowWarps);
  if (minb == 6) {
    if (codes)
      sg_flow_kernel<true, 6><<<blocks, 32 * kSgFlowWarps, 0, st>>>(f, ar, p, tb);
    else
      sg_flow_kernel<false, 6><<<blocks, 32 * kSgFlowWarps, 0, st>>>(f, ar, p, tb);
  } else {
    if (codes)
      sg_flow_kernel<true, 5><<<blocks, 32 * kSgFlowWarps, 0, st>>>(f, ar, p, tb);
    else
      sg_flow_kernel<false, 5><<<blocks, 32 * kSgFlowWarps, 0, st>>>(f, ar, p, tb);
  }
}

// ------------------------------------------------------------------ traceback (:869-914)
// State machine of impl/sequenceAlignment3.cpp:869-914: start in the state that produced the cell; a gap state persists
// while the cell's continuation flag is set; unwritten cells (outside the band, and the unweighted DP's last band
// column) read 255; the remaining rows and columns pad the walk as D and I, and the CIGAR is reversed.  R: rows per
// lane of the layout that wrote the codes (kSgR for the unweighted kernels, 1 for the weighted kernel).
//
// One warp per DP walks through shared-memory windows of the code store.  In the stripe / step / lane
// layout every move of the walk (diagonal, up, left) goes to a lower address, at most 2 x 32 x R + R bytes lower,
// so the warp stages the kSgTbWin bytes that end at the current cell with coalesced 16-byte loads and lane 0 walks
// them until the path leaves the window below; one memory round trip then serves about kSgTbWin / (32 R) moves
// instead of one.  The CIGAR is built and reversed as in sg_traceback_kernel.  tb_bytes: size of the code store
// (no load goes past it).
constexpr int kSgTbWin = 4096;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int R>
__global__ void __launch_bounds__(128) sg_traceback_warp_kernel(SgTask *__restrict__ tasks, const int *__restrict__ idx,
                                                                int n, int w, const uint8_t *__restrict__ tb,
                                                                int64_t tb_bytes, uint32_t *__restrict__ cig) {
  constexpr int kRows = 32 * R;
  // two windows per warp: lane 0 walks one while the warp's asynchronous copies fill the other with the window just
  // below it, where the walk goes next unless it crosses into the stripe above (a jump: then a synchronous fill)
  __shared__ __align__(16) uint8_t win2[4][2][kSgTbWin];
  const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= n) return;  // whole warp
  SgTask &T = tasks[idx[gw]];
  const int n2 = T.n2;
  const int64_t span = 2 * (int64_t)w + kRows;
  const int64_t stride = (n2 < span ? (int64_t)n2 : span) + 32;
  int ii = T.end1, jj = T.end2, state = 0, nc = 0;
  uint32_t *out = cig + T.cig_off;
  uint32_t last = 0xFFFFFFFFu;
  int64_t wbase[2] = {-1, -1};  // window [wbase, wbase + kSgTbWin) of the code store in each buffer; -1: none
  int cur = 0;
  bool pending = false;  // the other buffer is being filled with the window below the current one
  int64_t base = -1;
  const uint8_t *win = win2[wb][0];
  bool full = false;
  auto push = [&](uint32_t op) {
    if (nc > 0 && (last & 0xFu) == op) {
      last += 1u << 4;
      out[nc - 1] = last;
    } else if (nc < T.cig_cap) {
      last = (1u << 4) | op;
      out[nc++] = last;
    } else {
      full = true;
    }
  };
  auto fill = [&](int b, int64_t from) {  // every lane: its share of [from, from + kSgTbWin), asynchronously
    for (int c = lane; c < kSgTbWin / 16; c += 32) {
      const int64_t a = from + 16 * (int64_t)c;
      if (a + 16 <= tb_bytes)
        cp_async16(&win2[wb][b][16 * c], tb + a);
      else
        *reinterpret_cast<uint4 *>(&win2[wb][b][16 * c]) = make_uint4(0, 0, 0, 0);
    }
    cp_async_commit();
  };
  for (;;) {
    // lane 0 walks while the next cell is outside the band (no read) or inside the window; the warp refills the
    // window when the walk needs a cell below it
    int64_t need = -1;
    if (lane == 0) {
      while (ii > 0 && jj > 0) {
        int code = 255;
        const int c0 = max(ii - w, 1), c1 = min(ii + w, n2);
        if (ii <= T.rows && jj >= c0 && (jj < c1 || (R == 1 && jj == c1))) {
          const int s = (ii - 1) / kRows, rr = (ii - 1) % kRows, l = rr / R, kk = rr % R;
          const int jstart = max(kRows * s + 1 - w, 1);
          const int64_t t = jj - jstart + l;
          const int64_t a = T.tb_off + (((int64_t)s * stride + t) * 32 + l) * R + kk;
          if (base < 0 || a < base || a >= base + kSgTbWin) {
            need = a;
            break;
          }
          code = win[a - base];
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
    }
    need = __shfl_sync(0xFFFFFFFFu, need, 0);
    if (need < 0) break;
    cp_async_wait_all();  // this lane's copies, for either buffer, have landed
    __syncwarp();
    if (pending && need >= wbase[1 - cur] && need < wbase[1 - cur] + kSgTbWin) {
      cur = 1 - cur;  // the prefetched window below
    } else {
      // the window that ends (16-byte aligned) just past the needed byte, clipped to the store
      wbase[cur] = (((need + 16) & ~(int64_t)15) - kSgTbWin);
      if (wbase[cur] < 0) wbase[cur] = 0;
      fill(cur, wbase[cur]);
      cp_async_wait_all();
      __syncwarp();
    }
    pending = false;
    base = wbase[cur];
    win = win2[wb][cur];
    if (base > 0) {  // prefetch the window below while lane 0 walks this one
      wbase[1 - cur] = base - kSgTbWin > 0 ? base - kSgTbWin : 0;
      fill(1 - cur, wbase[1 - cur]);
      pending = true;
    }
  }
  cp_async_wait_all();
  if (lane == 0) {
    while (ii > 0) push(2), --ii;
    while (jj > 0) push(1), --jj;
    for (int a = 0, b = nc - 1; a < b; ++a, --b) {  // the reference reverses the walk (:915)
      const uint32_t tmp = out[a];
      out[a] = out[b];
      out[b] = tmp;
    }
    T.ncig = nc;
    if (full) T.status = 3;
  }
}

void launch_sg_traceback(SgTask *tasks, const int *idx, int n, int bandwidth, const uint8_t *tb, int64_t tb_bytes,
                         uint32_t *cig, cudaStream_t st, bool weighted_layout) {
  if (n <= 0) return;
  const int blocks = (n + 3) / 4;
  if (weighted_layout)
    sg_traceback_warp_kernel<1><<<blocks, 128, 0, st>>>(tasks, idx, n, bandwidth, tb, tb_bytes, cig);
  else
    sg_traceback_warp_kernel<kSgR><<<blocks, 128, 0, st>>>(tasks, idx, n, bandwidth, tb, tb_bytes, cig);
}

// ------------------------------------------------------------------ weighted DPs (one warp per DP)
// SemiGlobal with weights (impl/sequenceAlignment3.cpp:1483-1709, pieces = 2) and SemiGlobal_single_gap_penalty
// (:1710-1890, pieces = 1).  Row i takes the category of its seq1 base for the substitution, the horizontal gap
// states and the z-drop, and the category of the next base for the vertical gap states it leaves (a row at the end
// of seq1 keeps its own).  Every band column, the last included, updates the gap states and writes its code; a row
// with an empty band ends the DP (no stale column, unlike the unweighted DP).
//
// One warp runs one DP: 32-row stripes one after another, lane l owning row 32s+1+l as an anti-diagonal wavefront,
// the stripe's last row kept for the next stripe in the warp's global scratch (each column is read by lane 0 at least
// 31 steps before lane 31 overwrites it).  Rows are evaluated in order after each stripe; the DP ends at the stop row.
// Codes: one byte per cell, stripe / step / lane, the traceback layout of 32-row stripes.
__host__ __device__ inline int64_t sgw_stride_steps(int n2, int w) {
  const int64_t span = 2 * (int64_t)w + 32;
  return (n2 < span ? (int64_t)n2 : span) + 32;
}

int64_t sgw_tb_bytes(int n1, int n2, int w) {
  if (n1 <= 0 || n2 <= 0) return 0;
  return (int64_t)((n1 + 31) / 32) * sgw_stride_steps(n2, w) * 32;
}

int64_t sgw_bnd_bytes(int warps, int max_n2) { return (int64_t)warps * ((int64_t)max_n2 + 2) * sizeof(SgRec); }

__device__ __forceinline__ int sgw_cat(const SgTask &T, const int16_t *__restrict__ wt, int i) {
  // category of DP row i (1-based): forward rows follow seq1 from a1, reverse rows go down from a1
  const int64_t pos = T.dir == 0 ? (int64_t)T.a1 + i - 1 : (int64_t)T.a1 - (i - 1);
  return wt[T.wbase + pos];
}

__device__ __forceinline__ int sgw_next_cat(const SgTask &T, const int16_t *__restrict__ wt, int i, int own) {
  const int64_t pos = T.dir == 0 ? (int64_t)T.a1 + i : (int64_t)T.a1 - i;
  return (pos < 0 || pos >= T.wlen) ? own : wt[T.wbase + pos];
}

__global__ void __launch_bounds__(128) sgw_kernel(SgTask *__restrict__ tasks, const int *__restrict__ idx, int n,
                                                  Arena ar, Params P, SgWeights W, uint8_t *__restrict__ tb,
                                                  SgRec *__restrict__ bnd_all, int64_t bnd_stride,
                                                  int *__restrict__ counter) {
  __shared__ int cat[kSgwMaxCats][7];
  for (int k = threadIdx.x; k < W.n_cats * 7; k += blockDim.x) cat[k / 7][k % 7] = W.cats[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  SgRec *bnd = bnd_all + (int64_t)gw * bnd_stride;
  const int w = P.bandwidth;
  const bool two = W.pieces == 2;
  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(counter, 1);
    q = __shfl_sync(0xFFFFFFFFu, q, 0);
    if (q >= n) break;
    SgTask &T = tasks[idx[q]];
    const int n1 = T.n1, n2 = T.n2;
    const SeqView s1{T.base1, T.a1, T.dir}, s2{T.base2, T.a2, T.dir};
    const bool codes = T.want_codes != 0;
    const int64_t stride = sgw_stride_steps(n2, w);
    const int nstripes = (n1 > 0 && n2 > 0) ? (n1 + 31) / 32 : 0;
    int mx = 0, e1r = -1, e2r = -1, rows = 0;  // lane 0's running evaluation
    bool stop = false;
    for (int s = 0; s < nstripes && !stop; ++s) {
      const int i = 32 * s + 1 + lane;
      const bool live = i <= n1;
      const int c0 = max(i - w, 1), c1 = min(i + w, n2);
      const int ci = live ? s1.at(ar, i - 1) : 0;
      const int rc = live ? sgw_cat(T, W.weights, i) : 0;
      const int nc = live ? sgw_next_cat(T, W.weights, i, rc) : 0;
      const int mt = cat[rc][0], mm = cat[rc][1], o1h = cat[rc][2], x1h = cat[rc][3], o2h = cat[rc][4], x2h = cat[rc][5];
      const int o1v = cat[nc][2], x1v = cat[nc][3], o2v = cat[nc][4], x2v = cat[nc][5];
      const int r0 = 32 * s + 1, rl = min(32 * s + 32, n1);
      const int jstart = max(r0 - w, 1), jend = min(rl + w, n2);
      const int nsteps = jend >= jstart ? jend - jstart + 1 + 31 : 0;
      uint8_t *trow = tb + T.tb_off + (int64_t)s * stride * 32;
      int e1 = kOut, e2 = kOut, best = 0, bestj = two ? kOut : -1;
      int diag = (lane == 0 && s > 0 && jstart > 1) ? bnd[jstart - 1].m : kOut;
      int outM = kOut, outF1 = kOut, outF2 = kOut, outC = 0;
      for (int t = 0; t < nsteps; ++t) {
        int upM = __shfl_up_sync(0xFFFFFFFFu, outM, 1);
        int upF1 = __shfl_up_sync(0xFFFFFFFFu, outF1, 1);
        int upF2 = __shfl_up_sync(0xFFFFFFFFu, outF2, 1);
        int cj = __shfl_up_sync(0xFFFFFFFFu, outC, 1);
        const int j = jstart + t - lane;
        if (lane == 0) {
          upM = kOut, upF1 = kOut, upF2 = kOut;
          if (s > 0 && j >= 1 && j <= n2) {
            const SgRec r = bnd[j];
            upM = r.m, upF1 = r.f1, upF2 = r.f2;
          }
          cj = (j >= 1 && j <= n2) ? s2.at(ar, j - 1) : 0;
        }
        int cM = kOut, cF1 = kOut, cF2 = kOut;
        uint8_t code = 255;
        if (live && j >= c0 && j <= c1) {
          const int dg = (j == 1) ? (i == 1 ? 0 : kOut) : diag;
          const bool last = (j == c1);
          const int fin1 = last ? kOut : upF1, fin2 = last ? kOut : upF2;
          int v = ((ci == 2 || cj == 2) ? 0 : (ci == cj ? mt : mm)) + dg;
          int d = 0;
          bool pr;
          v = __vibmax_s32(fin1, v, &pr);
          d = pr ? 1 : d;
          v = __vibmax_s32(e1, v, &pr);
          d = pr ? 2 : d;
          if (two) {
            v = __vibmax_s32(fin2, v, &pr);
            d = pr ? 3 : d;
            v = __vibmax_s32(e2, v, &pr);
            d = pr ? 4 : d;
          }
          cM = v;
          if (v > best) best = v, bestj = j;
          cF1 = __vibmax_s32(fin1 + x1v, v + o1v, &pr);
          d |= pr ? 8 : 0;
          e1 = __vibmax_s32(e1 + x1h, v + o1h, &pr);
          d |= pr ? 16 : 0;
          if (two) {
            cF2 = __vibmax_s32(fin2 + x2v, v + o2v, &pr);
            d |= pr ? 32 : 0;
            e2 = __vibmax_s32(e2 + x2h, v + o2h, &pr);
            d |= pr ? 64 : 0;
          }
          code = (uint8_t)d;
        }
        if (codes && live) trow[(int64_t)t * 32 + lane] = code;
        __syncwarp();
        if (lane == 31 && live && j >= c0 && j <= c1) bnd[j] = SgRec{cM, cF1, cF2};
        __syncwarp();
        diag = upM;
        outM = cM, outF1 = cF1, outF2 = cF2, outC = cj;
      }
      // the stripe's rows in order (lane 0 decides; every lane takes part in the shuffles)
      for (int r = 0; r < 32; ++r) {
        const int tm = __shfl_sync(0xFFFFFFFFu, best, r), tj = __shfl_sync(0xFFFFFFFFu, bestj, r);
        const int zd = __shfl_sync(0xFFFFFFFFu, cat[rc][6], r), xr = __shfl_sync(0xFFFFFFFFu, x2h, r);
        const int ii = 32 * s + 1 + r;
        if (stop || ii > n1) continue;
        if (tm > mx) mx = tm, e1r = ii, e2r = tj;
        rows = ii;
        if (two) {
          int l = (ii - e1r) - (tj - e2r);
          l = l > 0 ? l : -l;
          if (mx - tm > zd + l * xr) stop = true;
        } else if (mx - tm > zd) {
          stop = true;
        }
        if (!stop && tj <= 0) stop = true;
      }
      __syncwarp();
    }
    if (lane == 0) {
      T.score = mx;
      T.end1 = e1r;
      T.end2 = e2r;
      T.rows = rows;
      T.status = 0;
    }
    __syncwarp();
  }
}

void launch_semiglobal_weighted(SgTask *tasks, const int *idx, int n, Arena ar, Params p, SgWeights wt, uint8_t *tb,
                                void *bnd, int max_n2, int *work_counter, int warps, cudaStream_t st) {
  if (n <= 0) return;
  sgw_kernel<<<(warps + 3) / 4, 128, 0, st>>>(tasks, idx, n, ar, p, wt, tb, (SgRec *)bnd, (int64_t)max_n2 + 2,
                                              work_counter);
}

}  // namespace dcns
