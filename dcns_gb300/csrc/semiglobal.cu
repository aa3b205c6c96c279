// Two-piece affine semi-global DP with z-drop and band (SemiGlobal_no_avx, impl/sequenceAlignment3.cpp:681-928)
// and its traceback.
//
// One warp runs one DP.  Rows are processed in stripes of 32 (lane l owns row 32s+1+l) as an anti-diagonal
// wavefront: at step t lane l computes column j = jstart + t - l, receiving the cell above (M, both vertical-gap
// states, and the query code) from lane l-1 through __shfl_up_sync; lane 0 reads the stripe's top boundary row, which
// lane 31 of the previous stripe wrote in place (lane 0 always reads a column before lane 31 overwrites it).  The
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

constexpr int kSgWarps = 4;

__global__ void __launch_bounds__(32 * kSgWarps) sg_kernel(SgTask *__restrict__ tasks, const int *__restrict__ idx,
                                                            int n, Arena ar, Params P, uint8_t *__restrict__ tb,
                                                            int32_t *__restrict__ bnd_all, int64_t bnd_stride,
                                                            int *__restrict__ counter) {
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * kSgWarps + (threadIdx.x >> 5);
  int32_t *bM = bnd_all + (int64_t)gw * bnd_stride * 3;
  int32_t *bF1 = bM + bnd_stride, *bF2 = bF1 + bnd_stride;
  const int o1 = P.open1, x1 = P.ext1, o2 = P.open2, x2 = P.ext2, w = P.bandwidth;
  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(counter, 1);
    q = __shfl_sync(0xFFFFFFFFu, q, 0);
    if (q >= n) break;
    SgTask &T = tasks[idx[q]];
    const int n1 = T.n1, n2 = T.n2;
    const SeqView s1{T.base1, T.a1, T.dir}, s2{T.base2, T.a2, T.dir};
    const bool codes = T.want_codes != 0;
    int maxScore = 0, end1 = -1, end2 = -1, rows = 0;
    bool stop = (n1 <= 0 || n2 <= 0);
    if (!stop)
      for (int j = lane; j <= n2; j += 32) bM[j] = kOut, bF1[j] = kOut, bF2[j] = kOut;
    __syncwarp();
    // stale column n2-1 values for the empty-band tail (rows r_last and r_last-1, r_last = n2-1+w)
    const int r_last = n2 - 1 + w;
    int stale_last = kOut, stale_prev = kOut;
    const int n1_eff = min(n1, n2 + w);  // rows with a non-empty band
    const int64_t stride = sg_stride_steps(n2, w);
    for (int s = 0; !stop && 32 * s < n1_eff; ++s) {
      const int i = 32 * s + 1 + lane;
      const bool live = i <= n1_eff;
      const int c0 = max(i - w, 1), c1 = min(i + w, n2);
      const int r0 = 32 * s + 1, rl = min(32 * s + 32, n1_eff);
      const int jstart = max(r0 - w, 1), jend = min(rl + w, n2);
      const int nsteps = jend - jstart + 1 + 31;
      const int ci = live ? s1.at(ar, i - 1) : 0;
      uint8_t *trow = tb + T.tb_off + (int64_t)s * stride * 32;
      int e1 = kOut, e2 = kOut, best = 0, bestj = 0;
      // M(i-1, j-1); lane 0 starts from the boundary row's cell left of its first column
      int diag = (lane == 0 && jstart > 1) ? bM[jstart - 1] : kOut;
      int outM = kOut, outF1 = kOut, outF2 = kOut, outC = 0;  // this lane's previous-step cell, for lane+1
      // lane 0 prefetch of the boundary row and the query code for its next column
      int pj = jstart;
      int nM = kOut, nF1 = kOut, nF2 = kOut, nC = 0;
      if (lane == 0 && pj <= n2) nM = bM[pj], nF1 = bF1[pj], nF2 = bF2[pj], nC = s2.at(ar, pj - 1);
      for (int t = 0; t < nsteps; ++t) {
        int upM = __shfl_up_sync(0xFFFFFFFFu, outM, 1);
        int upF1 = __shfl_up_sync(0xFFFFFFFFu, outF1, 1);
        int upF2 = __shfl_up_sync(0xFFFFFFFFu, outF2, 1);
        int cj = __shfl_up_sync(0xFFFFFFFFu, outC, 1);
        const int j = jstart + t - lane;
        if (lane == 0) {
          upM = nM, upF1 = nF1, upF2 = nF2, cj = nC;
          ++pj;
          if (pj <= jend) nM = bM[pj], nF1 = bF1[pj], nF2 = bF2[pj], nC = s2.at(ar, pj - 1);
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
          if (i == r_last && j == n2 - 1) stale_last = v;
          if (i == r_last - 1 && j == n2 - 1) stale_prev = v;
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
        }
        if (codes && live) trow[(int64_t)t * 32 + lane] = code;
        if (lane == 31 && live && j >= c0 && j <= c1) bM[j] = cM, bF1[j] = cF1, bF2[j] = cF2;
        diag = upM;
        outM = cM, outF1 = cF1, outF2 = cF2, outC = cj;
      }
      __syncwarp();
      // the lane that owns row r_last (or r_last-1) shares its column n2-1 value with the whole warp
      if (r_last >= 1 && (r_last - 1) / 32 == s) stale_last = __shfl_sync(0xFFFFFFFFu, stale_last, (r_last - 1) & 31);
      if (r_last >= 2 && (r_last - 2) / 32 == s) stale_prev = __shfl_sync(0xFFFFFFFFu, stale_prev, (r_last - 2) & 31);
      // evaluate this stripe's rows in order (all lanes redundantly)
      for (int r = 0; r < 32; ++r) {
        const int ii = 32 * s + 1 + r;
        const int tm = __shfl_sync(0xFFFFFFFFu, best, r);
        const int tj = __shfl_sync(0xFFFFFFFFu, bestj, r);
        if (stop || ii > n1_eff) continue;
        if (tm > maxScore) maxScore = tm, end1 = ii, end2 = tj;
        int l = (ii - end1) - (tj - end2);
        l = l > 0 ? l : -l;
        rows = ii;
        if (maxScore - tm > P.zdrop + l * x2) stop = true;
        else if (tj <= 0) stop = true;
      }
    }
    if (!stop && n1 > n1_eff && n2 >= 1) {
      const int c2 = s2.at(ar, n2 - 1);
      for (int i = n1_eff + 1; i <= n1 && !stop; ++i) {
        int dg;
        if (n2 == 1)
          dg = kOut;
        else
          dg = ((i - 1 - r_last) % 2 == 0) ? stale_last : stale_prev;
        int v = score_of(s1.at(ar, i - 1), c2, P.match, P.mismatch) + dg;
        if (!(v > kOut)) v = kOut;
        int tm = 0, tj = 0;
        if (v > 0) tm = v, tj = n2;
        if (tm > maxScore) maxScore = tm, end1 = i, end2 = tj;
        int l = (i - end1) - (tj - end2);
        l = l > 0 ? l : -l;
        rows = i;
        if (maxScore - tm > P.zdrop + l * x2) stop = true;
        else if (tj <= 0) stop = true;
      }
    }
    if (lane == 0) {
      T.score = maxScore;
      T.end1 = end1;
      T.end2 = end2;
      T.rows = rows;
      T.status = 0;
    }
    __syncwarp();
  }
}

void launch_semiglobal(SgTask *tasks, const int *idx, int n, Arena ar, Params p, uint8_t *tb, int32_t *bnd,
                       int64_t bnd_stride, int *work_counter, int grid_warps, cudaStream_t st) {
  if (n <= 0) return;
  const int blocks = (grid_warps + kSgWarps - 1) / kSgWarps;
  sg_kernel<<<blocks, 32 * kSgWarps, 0, st>>>(tasks, idx, n, ar, p, tb, bnd, bnd_stride, work_counter);
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
