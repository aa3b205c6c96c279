// Seed scan: windowed local Smith-Waterman of 38-bp query windows against the reference
// (SmithWaterman(..., bool&), impl/sequenceAlignment3.cpp:220-469, driven by getSeeds,
// impl/findSimilarFragmentsForPairedSequence4.cpp:61-201).
//
// Kernels
//   pack_kernel         int8 dCNS codes -> 2-bit + N-mask arena (64-base aligned sequences)
//   scan_kernel<W, M>   the hot loop: one thread owns two window tasks of one pair as the two int16 halves of every
//                       register, scanning the same absolute reference rows; per cell pair one score word from the
//                       thread's query profile in shared memory (a 128-bit load per four columns), fused add-max DPX
//                       instructions for H, E, the merged H and the next F, and a three-way row maximum every second
//                       column.  M = 1: level-0 tiles derived from the per-pair table; M = 2: recursion rounds from
//                       the duo table
//   scan_generic_kernel int32 lanes, any window width, both reference semantics (striped / scalar); used where the
//                       fast kernel's static int16 bound or width does not hold
//   scan_generic_wave_kernel  the same semantics for one large task per warp (long reads: kernel-level calls)
//   reverse_kernel      the reverse-complement re-scan that fixes each seed's start (getSeeds :156-166)
//   l0_*_kernel         device selection of the level-0 windows that reached min_score (count, scan, emit in window
//                       order) and their reverse re-scans, one thread per selected window
//
// Semantics reproduced exactly (striped kernels of the reference): per reference row i
//   Hpre[p] = max(H[i-1][p-1] + s(ref_i, read_p), E[p], 0)
//   E[p]    = max(E[p] + ext, Hpre[p] + open)            (from Hpre, before the horizontal pass)
//   F_p     = max(H[i][p-1] + open, F_{p-1} + ext)       (left to right)
//   H[i][p] = max(Hpre[p], F_p)
// and the reported position is the first (i-major, p-minor) cell holding the maximum.
#include <climits>

#include <algorithm>
#include <type_traits>

#include "device_common.cuh"

namespace dcns {

// ------------------------------------------------------------------ packing
__global__ void pack_kernel(const int8_t *__restrict__ codes, const int64_t *__restrict__ src_off,
                            const int64_t *__restrict__ dst_base, const int32_t *__restrict__ len,
                            uint32_t *__restrict__ pk, uint32_t *__restrict__ nm) {
  const int s = blockIdx.x;
  const int64_t so = src_off[s], db = dst_base[s];
  const int32_t n = len[s];
  const int ngroups = ((n + 63) / 64) * 2;  // 32-base groups covering whole 64-base blocks
  for (int g = threadIdx.x; g < ngroups; g += blockDim.x) {
    uint32_t w0 = 0, w1 = 0, nb = 0;
    for (int t = 0; t < 32; ++t) {
      const int idx = g * 32 + t;
      if (idx >= n) break;
      const int c = codes[so + idx];
      uint32_t two = 0;
      if (c == 1)
        two = 1;
      else if (c == 3)
        two = 2;
      else if (c == 4)
        two = 3;
      else if (c != 0)
        nb |= 1u << t;
      if (t < 16)
        w0 |= two << (2 * t);
      else
        w1 |= two << (2 * (t - 16));
    }
    pk[(db >> 4) + 2 * g] = w0;
    pk[(db >> 4) + 2 * g + 1] = w1;
    nm[(db >> 5) + g] = nb;
  }
}

void launch_pack(const int8_t *codes, const int64_t *src_off, const int64_t *dst_base, const int32_t *len, int nseq,
                 uint32_t *pk, uint32_t *nm, cudaStream_t st) {
  if (nseq > 0) pack_kernel<<<nseq, 128, 0, st>>>(codes, src_off, dst_base, len, pk, nm);
}

// ------------------------------------------------------------------ fast int16x2 scan
__device__ __forceinline__ uint32_t pack2(int v) { return (uint32_t)(uint16_t)(int16_t)v * 0x00010001u; }

// prmt with sign-replicating selectors: selector nibble (k | 8) yields the sign of byte k, so (k, k|8) sign-extends
// table byte k into a 16-bit lane.
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t s) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(s));
  return d;
}

__device__ __forceinline__ int half_s16(uint32_t v, int h) { return (int)(int16_t)(h ? (v >> 16) : (v & 0xFFFF)); }

__device__ __forceinline__ int min_above(int cur, int a, int b, int c, int d, int e, int f) {
  int m = INT_MAX;
  if (a > cur && a < m) m = a;
  if (b > cur && b < m) m = b;
  if (c > cur && c < m) m = c;
  if (d > cur && d < m) m = d;
  if (e > cur && e < m) m = e;
  if (f > cur && f < m) m = f;
  return m;
}

// Level-0 tile t, derived from the per-pair table (no tile array in memory).
__device__ __forceinline__ ScanTile l0_tile(const L0Desc &D, int64_t t) {
  int lo = 0, hi = D.npairs - 1;
  while (lo < hi) {  // last pair with tile_begin <= t
    const int mid = (lo + hi + 1) >> 1;
    if (D.pairs[mid].tile_begin <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  const L0Pair P = D.pairs[lo];
  const int64_t lt = t - P.tile_begin;
  const int duo = (int)(lt / P.nch), ch = (int)(lt % P.nch);
  ScanTile tl;
  tl.ref_base = P.ref_base;
  tl.qry_base = P.qry_base;
  for (int h = 0; h < 2; ++h) {
    const int w = 2 * duo + h;
    const bool on = w < P.nfast;
    const int s2 = w * D.step;
    tl.s2[h] = on ? s2 : 0;
    tl.tw[h] = on ? min(D.window, P.n2 - s2) : 0;
    tl.lo[h] = 0;
    tl.hi[h] = P.n1;
    tl.task[h] = on ? (int32_t)(P.wstart + w) : -1;
  }
  if (P.nch == 1) {
    tl.row_begin = 0, tl.cnt_begin = 0, tl.row_end = P.n1;
  } else {
    const int c0 = ch * D.chunk;
    tl.cnt_begin = c0;
    tl.row_end = min(P.n1, c0 + D.chunk);
    tl.row_begin = c0 == 0 ? 0 : max(0, c0 - D.warm);
  }
  return tl;
}

// Tile t of a duo-described round (RecDesc).
__device__ __forceinline__ ScanTile rec_tile(const RecDesc &D, int64_t t) {
  int lo = 0, hi = D.nduo - 1;
  while (lo < hi) {  // last duo with tile_begin <= t
    const int mid = (lo + hi + 1) >> 1;
    if (D.duos[mid].tile_begin <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  const RecDuo u = D.duos[lo];
  const ScanTask A = D.tasks[u.a];
  ScanTile tl;
  tl.ref_base = D.seqbase[2 * A.pair];
  tl.qry_base = D.seqbase[2 * A.pair + 1];
  tl.s2[0] = A.s2, tl.tw[0] = A.tw, tl.lo[0] = A.lo, tl.hi[0] = A.hi, tl.task[0] = u.a;
  int r0 = A.lo, r1 = A.hi;
  if (u.b >= 0) {
    const ScanTask B = D.tasks[u.b];
    tl.s2[1] = B.s2, tl.tw[1] = B.tw, tl.lo[1] = B.lo, tl.hi[1] = B.hi, tl.task[1] = u.b;
    r0 = min(r0, B.lo);
    r1 = max(r1, B.hi);
  } else {
    tl.s2[1] = 0, tl.tw[1] = 0, tl.lo[1] = A.lo, tl.hi[1] = A.hi, tl.task[1] = -1;
  }
  const int64_t c = t - u.tile_begin;
  const int64_t c0 = (int64_t)r0 + c * D.chunk;
  tl.cnt_begin = (int32_t)c0;
  tl.row_end = (int32_t)min((int64_t)r1, c0 + D.chunk);
  tl.row_begin = c == 0 ? r0 : (int32_t)max((int64_t)r0, c0 - D.warm);
  return tl;
}

// MODE 1: level-0 tiles from the per-pair table; MODE 2: round tiles from the duo table.
constexpr int kProfGroups = (kScanW + 3) / 4;  // query columns in groups of four (one 128-bit shared load)
constexpr int kProfSyms = 4;                   // reference symbols A, C, G, T (2-bit codes 0..3); N rows below
constexpr size_t kProfBytes = sizeof(uint4) * kProfSyms * kProfGroups * kScanThreads;

template <int W, int MODE>
__global__ void __launch_bounds__(kScanThreads) scan_kernel(RecDesc rec, L0Desc l0, int64_t ntiles,
                                                   Arena ar, int open, int ext, int match, int mismatch,
                                                   unsigned long long *__restrict__ keys, int *__restrict__ counter) {
  // Score table per reference symbol (index = 2-bit code | N << 2): bytes 0..4 = s(ref, read code 0..4) - open,
  // byte 5 = 0xC0 and byte 6 = 0x00, which the padding selector (6, 5) turns into the lane value -16384.
  __shared__ uint32_t tab[16];
  // Per-thread query profile of the current tile: prof[(sym * kProfGroups + g) * kScanThreads + thread] holds the
  // int16x2 score words (s - open, both halves) of columns 4g..4g+3 against reference symbol sym (A, C, G, T).  Each
  // thread reads and writes only its own entries.  A reference N scores 0 against everything: its row takes the
  // words 0 - open (-16384 in padding columns) from registers instead, on a separate path (N rows are rare: masked
  // runs are removed before alignment), which keeps the profile at 40 KB per 64-thread block and five blocks per SM.
  extern __shared__ uint4 prof[];
  if (threadIdx.x < 8) {
    const int idx = threadIdx.x;
    const int c = (idx & 4) ? 2 : ((idx & 3) + ((idx & 3) >> 1));
    uint32_t lo = 0, hi = 0;
    for (int r = 0; r < 5; ++r) {
      const uint32_t b = (uint32_t)(uint8_t)(int8_t)(score_of(c, r, match, mismatch) - open);
      if (r < 4)
        lo |= b << (8 * r);
      else
        hi |= b;
    }
    hi |= 0xC0u << 8;
    tab[2 * idx] = lo;
    tab[2 * idx + 1] = hi;
  }
  __syncthreads();
  const uint32_t open2 = pack2(open), ext2 = pack2(ext), fext2 = pack2(max(ext, open));
  const uint32_t open_lo = open2 & 0xFFFFu, open_hi = open2 & 0xFFFF0000u;

  for (;;) {
    const int t = atomicAdd(counter, 1);
    if (t >= ntiles) break;
    const ScanTile tl = MODE == 1 ? l0_tile(l0, t) : rec_tile(rec, t);

    // Registers hold G = H + open (not H): then the diagonal term H + s is G + (s - open) from the table, the
    // horizontal candidate H + open is G itself, and H + open = max(F + open, Hpre + open) is one fused op.
    // Two banks of G alternate between rows (row r reads Ga and writes Gb, row r+1 the reverse), so the previous
    // row's values stay in place while the new row is written: no register copies in the column loop.
    const int tw0 = tl.tw[0], tw1 = tl.tw[1];
    const uint32_t nlo = (uint32_t)(uint16_t)(-open), nhi = (uint32_t)(uint16_t)(-open) << 16;  // s(N, x) - open
    uint32_t Ga[W], Gb[W], E[W];
    {
      uint32_t sel[4 * kProfGroups];
#pragma unroll
      for (int p = 0; p < 4 * kProfGroups; ++p) {
        const uint32_t ra = p < tl.tw[0] ? (uint32_t)base_code(ar, tl.qry_base + tl.s2[0] + p) : 0u;
        const uint32_t rb = p < tl.tw[1] ? (uint32_t)base_code(ar, tl.qry_base + tl.s2[1] + p) : 0u;
        const uint32_t sa = p < tl.tw[0] ? (ra | ((ra | 8u) << 4)) : 0x56u;  // padding column: -16384
        const uint32_t sb = p < tl.tw[1] ? (rb | ((rb | 8u) << 4)) : 0x56u;
        sel[p] = sa | (sb << 8);
      }
#pragma unroll
      for (int sym = 0; sym < kProfSyms; ++sym) {
        const uint32_t T0 = tab[2 * sym], T1 = tab[2 * sym + 1];  // table index sym: 2-bit code, 4 = N
#pragma unroll
        for (int g = 0; g < kProfGroups; ++g)
          prof[(sym * kProfGroups + g) * kScanThreads + threadIdx.x] =
              make_uint4(prmt(T0, T1, sel[4 * g]), prmt(T0, T1, sel[4 * g + 1]), prmt(T0, T1, sel[4 * g + 2]),
                         prmt(T0, T1, sel[4 * g + 3]));
      }
    }
#pragma unroll
    for (int p = 0; p < W; ++p) {
      Ga[p] = open2;
      E[p] = 0;
    }

    // Row events: a half whose task starts after row_begin is zeroed at its first row; each half counts maxima only
    // on its own rows within [cnt_begin, row_end).
    int zr0 = tl.lo[0] > tl.row_begin ? tl.lo[0] : INT_MAX;
    int zr1 = tl.lo[1] > tl.row_begin ? tl.lo[1] : INT_MAX;
    int cs0 = max(tl.lo[0], tl.cnt_begin), ce0 = min(tl.hi[0], tl.row_end);
    int cs1 = max(tl.lo[1], tl.cnt_begin), ce1 = min(tl.hi[1], tl.row_end);
    if (tl.task[0] < 0 || cs0 >= ce0) cs0 = ce0 = INT_MAX;
    if (tl.task[1] < 0 || cs1 >= ce1) cs1 = ce1 = INT_MAX;
    // per-half threshold in G units: best + open while counting, unreachable (0x7FFF) otherwise
    uint32_t cmpb = 0x7FFF7FFFu;
    int best0 = 0, best1 = 0, brow0 = -1, brow1 = -1, bcol0 = -1, bcol1 = -1;

    int r = tl.row_begin;
    int nev = min_above(r - 1, zr0, zr1, cs0, ce0, cs1, ce1);
    int64_t rk = tl.ref_base + r;
    uint32_t wcur = __ldg(ar.pk + (rk >> 4)) >> (2u * (uint32_t)(rk & 15));
    uint32_t ncur = __ldg(ar.nm + (rk >> 5)) >> (uint32_t)(rk & 31);

    // One reference row: Gi holds row r-1, Go receives row r.
    auto row = [&](uint32_t(&Gi)[W], uint32_t(&Go)[W]) {
      if (r == nev) {
        if (zr0 == r) {
#pragma unroll
          for (int p = 0; p < W; ++p) {
            Gi[p] = (Gi[p] & 0xFFFF0000u) | open_lo;
            E[p] &= 0xFFFF0000u;
          }
        }
        if (zr1 == r) {
#pragma unroll
          for (int p = 0; p < W; ++p) {
            Gi[p] = (Gi[p] & 0x0000FFFFu) | open_hi;
            E[p] &= 0x0000FFFFu;
          }
        }
        if (cs0 == r) cmpb = (cmpb & 0xFFFF0000u) | (uint32_t)(uint16_t)(best0 + open);
        if (ce0 == r) cmpb = (cmpb & 0xFFFF0000u) | 0x7FFFu;
        if (cs1 == r) cmpb = (cmpb & 0x0000FFFFu) | ((uint32_t)(uint16_t)(best1 + open) << 16);
        if (ce1 == r) cmpb = (cmpb & 0x0000FFFFu) | 0x7FFF0000u;
        nev = min_above(r, zr0, zr1, cs0, ce0, cs1, ce1);
      }
      const bool nrow = (ncur & 1u) != 0;
      const uint4 *pr = prof + (int)(wcur & 3u) * (kProfGroups * kScanThreads) + threadIdx.x;
      ++rk;
      wcur >>= 2;
      ncur >>= 1;
      if ((rk & 15) == 0) wcur = __ldg(ar.pk + (rk >> 4));
      if ((rk & 31) == 0) ncur = __ldg(ar.nm + (rk >> 5));

      // F of column p is max(F[p-1] + ext, H[p-1] + open) with H[p-1] = max(F[p-1], Hpre[p-1]) (H merged with F
      // before it feeds the next column), i.e. F[p] = max(F[p-1] + max(ext, open), Hpre[p-1] + open): one add-max
      // per column on the serial chain, and F[0] = max(ext, open) from the zero boundary.
      uint32_t gd = open2, F = fext2, rmax = open2, gprev = open2;
      auto columns = [&](auto is_n) {
        uint4 q4 = make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int p = 0; p < W; ++p) {
          uint32_t s;
          if constexpr (decltype(is_n)::value) {
            s = (p < tw0 ? nlo : 0xC000u) | (p < tw1 ? nhi : 0xC0000000u);
          } else {
            if ((p & 3) == 0) q4 = pr[(p >> 2) * kScanThreads];
            s = (p & 3) == 0 ? q4.x : (p & 3) == 1 ? q4.y : (p & 3) == 2 ? q4.z : q4.w;
          }
          const uint32_t hp = __viaddmax_s16x2_relu(gd, s, E[p]);  // max(H[i-1][p-1] + s, E, 0)
          gd = Gi[p];
          const uint32_t tv = __vadd2(hp, open2);
          E[p] = __viaddmax_s16x2(E[p], ext2, tv);            // max(E + ext, Hpre + open)
          const uint32_t g = __viaddmax_s16x2(F, open2, tv);  // max(F, Hpre) + open
          F = __viaddmax_s16x2(F, fext2, tv);                 // F of the next column
          Go[p] = g;
          if (p & 1)
            rmax = __vimax3_s16x2(rmax, gprev, g);
          else if (p == W - 1)
            rmax = __vmaxs2(rmax, g);
          else
            gprev = g;
        }
      };
      if (nrow)
        columns(std::true_type{});
      else
        columns(std::false_type{});
      const uint32_t gt = __vcmpgts2(rmax, cmpb);
      if (gt) {
        if (gt & 0xFFFFu) {
          const int v = half_s16(rmax, 0);
          int col = W - 1;
#pragma unroll
          for (int p = W - 1; p >= 0; --p)
            if (half_s16(Go[p], 0) == v) col = p;
          best0 = v - open;
          brow0 = r;
          bcol0 = col;
          cmpb = (cmpb & 0xFFFF0000u) | (uint32_t)(uint16_t)v;
        }
        if (gt & 0xFFFF0000u) {
          const int v = half_s16(rmax, 1);
          int col = W - 1;
#pragma unroll
          for (int p = W - 1; p >= 0; --p)
            if (half_s16(Go[p], 1) == v) col = p;
          best1 = v - open;
          brow1 = r;
          bcol1 = col;
          cmpb = (cmpb & 0x0000FFFFu) | ((uint32_t)(uint16_t)v << 16);
        }
      }
      ++r;
    };
    while (r < tl.row_end) {
      row(Ga, Gb);
      if (r >= tl.row_end) break;
      row(Gb, Ga);
    }
    if (tl.task[0] >= 0 && best0 > 0) atomicMax(keys + tl.task[0], scan_key(best0, brow0, bcol0));
    if (tl.task[1] >= 0 && best1 > 0) atomicMax(keys + tl.task[1], scan_key(best1, brow1, bcol1));
  }
}

void launch_scan(RecDesc d, int64_t ntiles, Arena ar, Params p, unsigned long long *keys, int *work_counter, int grid,
                 cudaStream_t st) {
  if (ntiles <= 0) return;
  scan_kernel<kScanW, 2><<<grid, kScanThreads, kProfBytes, st>>>(d, L0Desc{}, ntiles, ar, p.open1, p.ext1, p.match,
                                                                 p.mismatch, keys, work_counter);
}

void launch_scan_l0(L0Desc d, int64_t ntiles, Arena ar, Params p, unsigned long long *keys, int *work_counter,
                    int64_t grid, cudaStream_t st) {
  if (ntiles <= 0) return;
  scan_kernel<kScanW, 1><<<(unsigned)grid, kScanThreads, kProfBytes, st>>>(RecDesc{}, d, ntiles, ar, p.open1, p.ext1, p.match,
                                                                 p.mismatch, keys, work_counter);
}

// ------------------------------------------------------------------ generic int32 Smith-Waterman (one thread)
// Sequences are accessed through callables; H/Hp/E are per-thread arrays of nb entries.  Returns the maximum and its
// first position (0-based) exactly as the reference kernel selected by `striped` would.
template <class A, class B>
__device__ void sw_one(A sa, int na, B sb, int nb, int open, int ext, int match, int mismatch, bool striped,
                       int32_t *H, int32_t *Hp, int32_t *E, int &best, int &bi, int &bj) {
  best = 0;
  bi = -1;
  bj = -1;
  if (nb <= 0) return;
  if (striped) {
    for (int p = 0; p < nb; ++p) H[p] = 0, E[p] = 0;
    for (int i = 0; i < na; ++i) {
      const int ci = sa(i);
      int diag = 0;
      for (int p = 0; p < nb; ++p) {
        int h = max(diag + score_of(ci, sb(p), match, mismatch), 0);
        h = max(h, E[p]);
        Hp[p] = h;
        E[p] = max(max(E[p] + ext, h + open), 0);
        diag = H[p];
      }
      int del = 0, left = 0;
      for (int p = 0; p < nb; ++p) {
        del = max(left + open, del + ext);
        const int h = Hp[p] < del ? del : Hp[p];
        del = max(del, 0);
        H[p] = h;
        left = h;
        if (h > best) best = h, bi = i, bj = p;
      }
    }
  } else {
    // scalar kernel: H holds the previous row (index p+1 = column p), Hp the current row, E the vertical gap
    for (int p = 0; p <= nb; ++p) H[p] = 0, Hp[p] = 0, E[p] = 0;
    for (int i = 0; i < na; ++i) {
      const int ci = sa(i);
      int e = 0;
      for (int j = 1; j <= nb; ++j) {
        e = max(open + Hp[j - 1], ext + e);
        E[j] = max(open + H[j], ext + E[j]);
        int v = max(score_of(ci, sb(j - 1), match, mismatch) + H[j - 1], e);
        v = max(v, E[j]);
        Hp[j] = max(v, 0);
        E[j] = max(E[j], 0);
        e = max(e, 0);
        if (v > best) best = v, bi = i, bj = j - 1;
      }
      for (int j = 0; j <= nb; ++j) {
        const int tmp = H[j];
        H[j] = Hp[j];
        Hp[j] = tmp;
      }
    }
  }
}

// The reference's kernel choice for an (nref x nread) call (impl/sequenceAlignment3.cpp:223-225, :338-339).
__host__ __device__ inline bool striped_for(int nref, int nread, int open, int ext, int match) {
  auto ok = [&](int lim) {
    return ((-nref * ext - open) < lim || (-nread * ext - open) < lim) && (nref * match < lim || nread * match < lim);
  };
  return ok(125) || ok(32767);
}

__global__ void scan_generic_kernel(const ScanTask *__restrict__ tasks, const int *__restrict__ idx, int n,
                                    const int64_t *__restrict__ seq_base, Arena ar, Params P,
                                    unsigned long long *__restrict__ keys, int32_t *scratch, int64_t per_thread) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int ti = idx[k];
  const ScanTask T = tasks[ti];
  const int64_t b1 = seq_base[2 * T.pair], b2 = seq_base[2 * T.pair + 1];
  int32_t *H = scratch + per_thread * k;
  int32_t *Hp = H + (T.tw + 1);
  int32_t *E = Hp + (T.tw + 1);
  int best, bi, bj;
  sw_one([&](int i) { return base_code(ar, b1 + T.lo + i); }, T.hi - T.lo,
         [&](int p) { return base_code(ar, b2 + T.s2 + p); }, T.tw, P.open1, P.ext1, P.match, P.mismatch,
         T.striped != 0, H, Hp, E, best, bi, bj);
  keys[ti] = best > 0 ? scan_key(best, T.lo + bi, bj) : 0ull;
}

// Either semantics of sw_one for one long task per warp, as an anti-diagonal wavefront over 32-row stripes: lane l
// owns reference row r0 + l and computes read column j (1-based) at step t = j - 1 + l, with the cell above (H and
// the column's vertical gap E after the row above) and the diagonal H from lane l - 1 by __shfl_up_sync, and its own
// left H and horizontal gap state in registers.  Both semantics are local recurrences on those five values: the
// scalar kernel's (SmithWaterman_non_avx) and the striped kernels' (the vertical gap advanced from the cell's value
// before the horizontal gap is merged, and the horizontal gap merged last, as the AVX2 code's second pass does).  Lane 0 takes the row above the stripe from the task's boundary row in
// global scratch (H and E by column), staged into shared memory two 32-column chunks ahead; lane 31 rewrites it
// with the stripe's last row (column j at step j + 30, after lane 0 staged it).  Each lane keeps its row's first
// maximum; after each stripe the rows are taken in order, so the task's maximum is the first one in row-major,
// column-minor order, as the scalar kernel finds it.  scratch: 2 (read length + 2) ints per task.
__global__ void __launch_bounds__(128) scan_generic_wave_kernel(const ScanTask *__restrict__ tasks,
                                                                const int *__restrict__ idx, int n,
                                                                const int64_t *__restrict__ seq_base, Arena ar,
                                                                Params P, unsigned long long *__restrict__ keys,
                                                                int32_t *__restrict__ scratch, int64_t per_task) {
  __shared__ int stH[4][2][32], stE[4][2][32], stC[4][2][32];
  const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= n) return;  // whole warp
  const int ti = idx[gw];
  const ScanTask T = tasks[ti];
  const int64_t b1 = seq_base[2 * T.pair] + T.lo, b2 = seq_base[2 * T.pair + 1] + T.s2;
  const int na = T.hi - T.lo, nb = T.tw;
  const int open = P.open1, ext = P.ext1;
  const bool striped = T.striped != 0;
  int32_t *const bH = scratch + per_task * gw, *const bE = bH + (nb + 2);
  for (int j = lane; j <= nb + 1; j += 32) bH[j] = 0, bE[j] = 0;  // row -1: H = 0, E = 0
  __syncwarp();
  int gbest = 0, gi = -1, gj = -1;
  const int nsteps = nb + 31;
  for (int r0 = 0; r0 < na; r0 += 32) {
    const int i = r0 + lane;
    const bool live = i < na;
    const int ci = live ? base_code(ar, b1 + i) : 0;
    // columns 32 * chunk + 1 .. + 32 of the row above (and the read's codes there) into stage[chunk & 1]
    auto stage = [&](int chunk) {
      const int j = 32 * chunk + 1 + lane;
      const bool in = j <= nb;
      stH[wb][chunk & 1][lane] = in ? __ldcg(bH + j) : 0;
      stE[wb][chunk & 1][lane] = in ? __ldcg(bE + j) : 0;
      stC[wb][chunk & 1][lane] = in ? base_code(ar, b2 + j - 1) : 0;
    };
    stage(0);
    stage(1);
    __syncwarp();
    int leftH = 0, e = 0, best = 0, bestj = -1, outH = 0, outE = 0, outC = 0, prevUp = 0;
    for (int t = 0; t < nsteps; ++t) {
      int upH = __shfl_up_sync(0xFFFFFFFFu, outH, 1);
      int upE = __shfl_up_sync(0xFFFFFFFFu, outE, 1);
      int cj = __shfl_up_sync(0xFFFFFFFFu, outC, 1);
      if ((t & 31) == 0 && t > 0) {
        __syncwarp();
        stage((t >> 5) + 1);  // two chunks ahead of lane 0's reads
        __syncwarp();
      }
      const int j = t + 1 - lane;  // 1-based read column of this lane's cell
      int diagH = prevUp;
      if (lane == 0) {
        upH = stH[wb][(t >> 5) & 1][t & 31];
        upE = stE[wb][(t >> 5) & 1][t & 31];
        cj = stC[wb][(t >> 5) & 1][t & 31];
        diagH = t == 0 ? 0 : diagH;  // column 0 of the row above is 0
      }
      if (j == 1) diagH = 0;  // column 0 of the row above
      int nH = 0, nE = 0;
      if (live && j >= 1 && j <= nb) {
        const int s = score_of(ci, cj, P.match, P.mismatch);
        if (striped) {
          // first pass (H before the horizontal gap, E from it), then the horizontal gap `e` (del) merged
          const int hp = max(max(diagH + s, 0), upE);
          nE = max(max(upE + ext, hp + open), 0);
          e = max(leftH + open, e + ext);
          nH = hp < e ? e : hp;
          e = max(e, 0);
          if (nH > best) best = nH, bestj = j - 1;
        } else {
          e = max(open + leftH, ext + e);
          const int Ej = max(open + upH, ext + upE);
          int v = max(s + diagH, e);
          v = max(v, Ej);
          nH = max(v, 0);
          nE = max(Ej, 0);
          e = max(e, 0);
          if (v > best) best = v, bestj = j - 1;
        }
        leftH = nH;
        if (lane == 31) bH[j] = nH, bE[j] = nE;
      }
      prevUp = upH;
      outH = nH;
      outE = nE;
      outC = cj;
    }
    __syncwarp();
    for (int rr = 0; rr < 32; ++rr) {  // the stripe's rows in order: the first maximum in row-major order
      const int tm = __shfl_sync(0xFFFFFFFFu, best, rr), tj = __shfl_sync(0xFFFFFFFFu, bestj, rr);
      if (r0 + rr < na && tm > gbest) gbest = tm, gi = r0 + rr, gj = tj;
    }
  }
  if (lane == 0) keys[ti] = gbest > 0 ? scan_key(gbest, T.lo + gi, gj) : 0ull;
}

void launch_scan_generic_wave(const ScanTask *tasks, const int *idx, int n, const int64_t *seq_base, Arena ar,
                              Params p, unsigned long long *keys, int32_t *scratch, int64_t per_task,
                              cudaStream_t st) {
  if (n <= 0) return;
  scan_generic_wave_kernel<<<(n + 3) / 4, 128, 0, st>>>(tasks, idx, n, seq_base, ar, p, keys, scratch, per_task);
}

void launch_scan_generic(const ScanTask *tasks, const int *idx, int n, const int64_t *seq_base, Arena ar, Params p,
                         unsigned long long *keys, int32_t *scratch, int64_t scratch_per_thread, cudaStream_t st) {
  if (n <= 0) return;
  scan_generic_kernel<<<(n + 127) / 128, 128, 0, st>>>(tasks, idx, n, seq_base, ar, p, keys, scratch,
                                                       scratch_per_thread);
}

// ------------------------------------------------------------------ reverse scan -> seed start
// For every task whose maximum reaches min_score: re-scan the reverse complements ending at the maximum,
// e1 = min(end1_local + 1, tw + window) reference bases by e2 = min(end2_local + 1, tw + window) query bases
// (getSeeds :150-166); start = end - (reverse end).
constexpr int kRevMax = 128;

__global__ void reverse_kernel(ScanTask *__restrict__ tasks, int first, int n,
                               const unsigned long long *__restrict__ keys, const int64_t *__restrict__ seq_base,
                               Arena ar, Params P) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  ScanTask &T = tasks[first + k];
  int score = 0, row = -1, col = -1;
  const unsigned long long key = keys[first + k];
  if (key) scan_unkey(key, score, row, col);
  T.score = score;
  T.end1 = score > 0 ? row : -1;
  T.end2 = score > 0 ? T.s2 + col : -1;
  T.start1 = -1;
  T.start2 = -1;
  if (score < P.min_score) return;
  const int lim = T.tw + P.window;
  const int e1 = min(row - T.lo + 1, lim), e2 = min(col + 1, lim);
  const int64_t b1 = seq_base[2 * T.pair], b2 = seq_base[2 * T.pair + 1];
  const int end1 = row, end2 = T.s2 + col;
  int32_t H[kRevMax + 1], Hp[kRevMax + 1], E[kRevMax + 1];
  int best, bi, bj;
  if (e2 > kRevMax) return;  // windows wider than kRevMax are rejected by the host before launch
  sw_one([&](int i) { return 4 - base_code(ar, b1 + end1 - i); }, e1,
         [&](int p) { return 4 - base_code(ar, b2 + end2 - p); }, e2, P.open1, P.ext1, P.match, P.mismatch,
         striped_for(e1, e2, P.open1, P.ext1, P.match), H, Hp, E, best, bi, bj);
  T.start1 = end1 - bi;
  T.start2 = end2 - bj;
}

// ------------------------------------------------------------------ level-0 selection
// count -> scan -> emit: the windows whose maximum reached min_score, compacted in task order, each with its reverse
// re-scan.  Only these records travel to the host.
constexpr int kSelBlock = 256;

__global__ void l0_count_kernel(const unsigned long long *__restrict__ keys, int64_t n0, int min_score,
                                int *__restrict__ block_cnt) {
  const int64_t t = (int64_t)blockIdx.x * kSelBlock + threadIdx.x;
  int f = 0;
  if (t < n0) f = (int)(keys[t] >> 40) >= min_score;
  const int c = __syncthreads_count(f);
  if (threadIdx.x == 0) block_cnt[blockIdx.x] = c;
}

// Exclusive scan of the block counts in place (one block); the total goes to *count.
__global__ void l0_scan_kernel(int *__restrict__ block_cnt, int nb, int *__restrict__ count) {
  __shared__ int warp_sums[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? block_cnt[i] : 0;
    int x = v;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int ws = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
      for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, ws, d);
        if (lane >= d) ws += y;
      }
      warp_sums[lane] = ws;
    }
    __syncthreads();
    const int incl = x + (wid > 0 ? warp_sums[wid - 1] : 0) + carry;
    if (i < nb) block_cnt[i] = incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = carry;
}

__global__ void l0_emit_kernel(const unsigned long long *__restrict__ keys, int64_t n0,
                               const int *__restrict__ block_off, int min_score, L0Rec *__restrict__ out) {
  __shared__ int warp_cnt[kSelBlock / 32];
  const int64_t t = (int64_t)blockIdx.x * kSelBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long key = 0;
  int score = 0, row = -1, col = -1;
  if (t < n0) key = keys[t];
  if (key) scan_unkey(key, score, row, col);
  const bool f = t < n0 && score >= min_score;
  const unsigned m = __ballot_sync(0xFFFFFFFFu, f);
  if (lane == 0) warp_cnt[wid] = __popc(m);
  __syncthreads();
  if (!f) return;
  int pos = block_off[blockIdx.x] + __popc(m & ((1u << lane) - 1));
  for (int k = 0; k < wid; ++k) pos += warp_cnt[k];
  out[pos] = L0Rec{(int32_t)t, score, row, col, 0, 0};  // end2 holds the window column until the reverse scan
}

// The reverse re-scan of every compacted level-0 window (one thread each, all busy): the window's start is the
// argmax of Smith-Waterman on the reverse complements ending at the forward maximum, over at most tw + window
// cells each way (findSimilarFragmentsForPairedSequence4.cpp:131-201).
__global__ void __launch_bounds__(128) l0_reverse_kernel(L0Rec *__restrict__ recs, const int *__restrict__ count,
                                                         const int64_t *__restrict__ wstart,
                                                         const int2 *__restrict__ plen, int np,
                                                         const int64_t *__restrict__ seq_base, Arena ar, Params P) {
  const int n = *count;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    L0Rec r = recs[q];
    const int64_t t = r.task;
    int lo = 0, hi = np - 1;  // the pair owning task t: last wstart <= t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (wstart[mid] <= t)
        lo = mid;
      else
        hi = mid - 1;
    }
    const int p = lo;
    const int s2 = (int)(t - wstart[p]) * P.step;
    const int tw = min(P.window, plen[p].y - s2);
    const int lim = tw + P.window;
    const int row = r.end1, col = r.end2;
    const int e1 = min(row + 1, lim), e2 = min(col + 1, lim);
    const int64_t b1 = seq_base[2 * p], b2 = seq_base[2 * p + 1];
    const int end1 = row, end2 = s2 + col;
    int32_t H[kRevMax + 1], Hp[kRevMax + 1], E[kRevMax + 1];
    int best, bi, bj;
    sw_one([&](int i) { return 4 - base_code(ar, b1 + end1 - i); }, e1,
           [&](int k) { return 4 - base_code(ar, b2 + end2 - k); }, e2, P.open1, P.ext1, P.match, P.mismatch,
           striped_for(e1, e2, P.open1, P.ext1, P.match), H, Hp, E, best, bi, bj);
    r.end2 = end2;
    r.start1 = end1 - bi;
    r.start2 = end2 - bj;
    recs[q] = r;
  }
}

void launch_l0_select(const unsigned long long *keys, int64_t n0, const int64_t *wstart, const int2 *plen, int np,
                      const int64_t *seq_base, Arena ar, Params p, int *scratch, int *count, L0Rec *out, int nsm,
                      cudaStream_t st) {
  if (n0 <= 0) return;
  const int nb = (int)((n0 + kSelBlock - 1) / kSelBlock);
  l0_count_kernel<<<nb, kSelBlock, 0, st>>>(keys, n0, p.min_score, scratch);
  l0_scan_kernel<<<1, 1024, 0, st>>>(scratch, nb, count);
  l0_emit_kernel<<<nb, kSelBlock, 0, st>>>(keys, n0, scratch, p.min_score, out);
  const int rb = (int)std::min<int64_t>((n0 + 127) / 128, (int64_t)nsm * 16);
  l0_reverse_kernel<<<rb, 128, 0, st>>>(out, count, wstart, plen, np, seq_base, ar, p);
}

void launch_reverse(ScanTask *tasks, int first, int n, const unsigned long long *keys, const int64_t *pair_base,
                    const int32_t *pair_len, Arena ar, Params p, cudaStream_t st) {
  (void)pair_len;
  if (n <= 0) return;
  reverse_kernel<<<(n + 127) / 128, 128, 0, st>>>(tasks, first, n, keys, pair_base, ar, p);
}

}  // namespace dcns

namespace dcns {
// Resident blocks per SM of the fast scan kernel at 128 threads (sizes the persistent grid).
// Opts both scan kernels in to their dynamic shared memory (above the 48 KB default) and returns the resident blocks
// per SM.  Called once per context before any scan launch.
int scan_occupancy_impl() {
  int nb = 0;
  if (cudaFuncSetAttribute(scan_kernel<kScanW, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kProfBytes) !=
          cudaSuccess ||
      cudaFuncSetAttribute(scan_kernel<kScanW, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kProfBytes) !=
          cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, scan_kernel<kScanW, 1>, kScanThreads, kProfBytes) !=
      cudaSuccess) {
    (void)cudaGetLastError();
    nb = 1;
  }
  return nb > 0 ? nb : 1;
}
}  // namespace dcns

namespace dcns {
// ------------------------------------------------------------------ integer-issue roofline probe
// Runs the scan kernel's per-cell instruction sequence (score word from a 128-bit shared-memory profile load per four
// columns, fused add-max-relu, H + open, E and F updates, fused H merge, row maximum every second column) on 8
// independent chains per thread at full occupancy, so the only limit is instruction issue.  Each chain step is one
// int16x2 cell pair of the scan; the result is an upper bound for the scan's cells per second with exactly its
// instruction mix.
__global__ void __launch_bounds__(256) issue_probe_kernel(uint32_t *out, int iters, uint32_t seed) {
  constexpr int NC = 8;
  __shared__ uint4 pf[4 * 256];
  for (int g = 0; g < 4; ++g)
    pf[g * 256 + threadIdx.x] = make_uint4(0xFFFDFFFDu ^ seed, 0x00020002u, 0xFFFDFFFDu, 0xC000C000u ^ (g << 1));
  uint32_t d[NC], e[NC], f[NC], rm[NC];
  const uint32_t open2 = pack2(-4), ext2 = pack2(-2);
#pragma unroll
  for (int c = 0; c < NC; ++c) d[c] = seed * (c + 1), e[c] = 0, f[c] = 0, rm[c] = 0;
  for (int it = 0; it < iters; ++it) {
    uint4 q4 = make_uint4(0, 0, 0, 0);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if ((c & 3) == 0) q4 = pf[((it + (c >> 2)) & 3) * 256 + threadIdx.x];
      const uint32_t s = (c & 3) == 0 ? q4.x : (c & 3) == 1 ? q4.y : (c & 3) == 2 ? q4.z : q4.w;
      const uint32_t hp = __viaddmax_s16x2_relu(d[c], s, e[c]);
      const uint32_t tv = __vadd2(hp, open2);
      e[c] = __viaddmax_s16x2(e[c], ext2, tv);
      const uint32_t g = __viaddmax_s16x2(f[c], open2, tv);
      f[c] = __viaddmax_s16x2(f[c], ext2, tv);
      if (c & 1) rm[c] = __vimax3_s16x2(rm[c], d[c], g);
      d[c] = g;
    }
  }
  uint32_t acc = 0;
#pragma unroll
  for (int c = 0; c < NC; ++c) acc ^= d[c] ^ e[c] ^ rm[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// Returns int16x2 cell pairs per second of the probe (each = one chain step).
double measure_issue_rate(int nsm, cudaStream_t st) {
  const int threads = 256, blocks = nsm * 8, iters = 1 << 14;
  uint32_t *out = nullptr;
  if (cudaMalloc(&out, sizeof(uint32_t) * threads * blocks) != cudaSuccess) return 0;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  issue_probe_kernel<<<blocks, threads, 0, st>>>(out, 256, 1u);  // warm-up
  cudaEventRecord(a, st);
  issue_probe_kernel<<<blocks, threads, 0, st>>>(out, iters, 7u);
  cudaEventRecord(b, st);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (ms <= 0) return 0;
  return (double)threads * blocks * iters * 8 / (ms * 1e-3);
}
}  // namespace dcns
