// Shared host/device definitions of the GB300 CNS pair-alignment engine.
//
// Sequences live on the device in one packed arena: 2-bit A/C/G/T codes (16 bases per uint32 word) plus a 1-bit N
// mask (32 bases per word).  Every sequence starts on a 64-base boundary, so one 128-bit load fetches 64 bases of a
// single sequence.  Kernels decode to dCNS integer codes (A=0 C=1 N=2 G=3 T=4, impl/SequenceCharToUInt8.cpp:6-33)
// and read reverse complements by mirrored indexing (4 - code, impl/SequenceCharToUInt8.cpp:61-66), so no
// reverse-complement copy is stored.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace dcns {

constexpr int32_t kOut = -536870912;  // score of cells outside a band (impl/sequenceAlignment3.cpp:34)
constexpr int kScanW = 38;            // window width the fast seed-scan kernel is specialised for
constexpr int kScanThreads = 64;      // threads per block of the fast seed-scan kernel
constexpr int32_t kMaxSeqLen = 1 << 28;  // sequences are shorter; semi-global bands are clamped to it

struct Params {
  int32_t match, mismatch, open1, ext1, open2, ext2;
  int32_t window, min_score, step, w, xdrop, zdrop, bandwidth, max_align_len;
  double pvalue, lambda, kvalue;
};

struct Arena {
  const uint32_t *pk;  // 2-bit codes
  const uint32_t *nm;  // N mask
};

// One thread of the seed-scan kernel: up to two Smith-Waterman tasks (int16x2 halves) of the same pair that scan
// the same absolute reference rows.  Half h scores window [s2[h], s2[h]+tw[h]) of seq2 against reference rows
// [lo[h], hi[h]); the tile computes rows [row_begin, row_end) and reports maxima only for rows >= cnt_begin.
struct ScanTile {
  int64_t ref_base, qry_base;
  int32_t s2[2], tw[2];
  int32_t lo[2], hi[2];
  int32_t row_begin, cnt_begin, row_end;
  int32_t task[2];  // result slot of each half, -1 when the half is unused
};

// Level-0 scan (every window of a pair against its whole reference), described per pair instead of per tile: tile t
// belongs to the pair with tile_begin <= t < next tile_begin (pairs in longest-reference-first order), covers
// windows 2d and 2d+1 of that pair (d = (t - tile_begin) / nch) and row chunk (t - tile_begin) % nch.
struct L0Pair {
  int64_t ref_base, qry_base, tile_begin, wstart;
  int32_t n1, n2, nfast, nch;
};
struct L0Desc {
  const L0Pair *pairs;
  int32_t npairs, step, window, chunk, warm, pad;
};
// A round of tasks (recursion levels, the generic-entry batches), described per duo: two tasks of one pair that share
// a tile (b = -1 when alone).  Tile t belongs to the duo with tile_begin <= t < next tile_begin and covers row chunk
// t - tile_begin of the union of the two tasks' row ranges.  Task records are read from the device task array.
struct RecDuo {
  int64_t tile_begin;
  int32_t a, b;
};
struct ScanTask;
struct RecDesc {
  const RecDuo *duos;
  const ScanTask *tasks;
  const int64_t *seqbase;
  int32_t nduo, chunk, warm, pad;  // chunk = INT32_MAX: one tile per duo
};

// A level-0 window whose maximum reached min_score, compacted in task order.
struct L0Rec {
  int32_t task, score, end1, end2, start1, start2;
};

// Per Smith-Waterman task (window x reference range): the reduced maximum and, after the reverse scan, the seed.
struct ScanTask {
  int32_t pair, s2, tw, lo, hi;
  int32_t score, end1, end2;      // absolute 0-based first argmax (valid when score > 0)
  int32_t start1, start2;         // seed start from the reverse scan (valid when score >= min_score)
  int32_t striped;                // 1: the reference runs its striped (AVX2) kernel for this task, 0: scalar
  int32_t pad;
};

// Packed reduction key of a task maximum: larger score wins, then the earlier row, then the earlier column.
__host__ __device__ inline unsigned long long scan_key(int32_t score, int32_t row, int32_t col) {
  return ((unsigned long long)(uint32_t)score << 40) | ((unsigned long long)(0xFFFFFFu - (uint32_t)row) << 16) |
         (unsigned long long)(0xFFFFu - (uint32_t)col);
}
__host__ __device__ inline void scan_unkey(unsigned long long k, int32_t &score, int32_t &row, int32_t &col) {
  score = (int32_t)(k >> 40);
  row = (int32_t)(0xFFFFFFu - (uint32_t)((k >> 16) & 0xFFFFFF));
  col = (int32_t)(0xFFFFu - (uint32_t)(k & 0xFFFF));
}

// One banded x-drop pass (SemiGlobal_xextend, impl/sequenceAlignment3.cpp:1234/1318) of one seed.
//   dir 0: forward from (a1, a2) over seq1[a1..), seq2[a2..)
//   dir 1: backward over the reverse complements ending at (a1, a2): row i reads seq1[a1-i+1] complemented
struct XTask {
  int64_t base1, base2;
  int32_t a1, a2, n1, n2;
  int32_t dir, w, want_codes, tb_cap;  // tb_cap: traceback slot capacity in 32-bit words
  int64_t tb_off;
  // outputs
  int32_t score, end1, end2;           // 1-based best cell (0 when none)
  int32_t rows;                        // rows evaluated in this pass
  int32_t status;                      // 0 done, 1 band-edge restart needed (w doubled), 2 traceback slot too small
  int32_t iii, jjj, ncig;              // traceback results
  int64_t cig_off;                     // CIGAR slot (uint32 entries) and its capacity
  int32_t cig_cap, pad;
  int64_t cig_dense;                   // chained form: offset of the CIGAR in the batch's packed CIGAR array
};

// One 2-piece affine semi-global DP (SemiGlobal_no_avx, impl/sequenceAlignment3.cpp:681-928).
//   dir 0: seq1[a1 .. a1+n1), seq2[a2 .. a2+n2)        dir 1: reverse complements ending at (a1, a2)
struct SgTask {
  int64_t base1, base2;
  int32_t a1, a2, n1, n2;
  int32_t dir, want_codes;
  int64_t tb_off;                      // byte offset of the direction-code store (want_codes)
  int64_t tb_bytes;
  // outputs
  int32_t score, end1, end2, rows;     // end1/end2 1-based (-1 when none) ; rows evaluated
  int32_t status, ncig;
  int64_t cig_off;
  int32_t cig_cap, pad;
  // weighted variants: category ids of this DP's seq1 (the whole sequence, wlen bases) at wbase in the weight array
  int64_t wbase;
  int32_t wlen, wpad;
};

// Weighted 2-piece / 1-piece DPs (impl/sequenceAlignment3.cpp:1483-1890): per-base category ids of seq1 and, per
// category, match, mismatch, open1, ext1, open2, ext2, zdrop.
struct SgWeights {
  const int16_t *weights;
  const int32_t *cats;
  int32_t n_cats, pieces;
};
constexpr int kSgwMaxCats = 64;

// The semi-global kernel (semiglobal.cu): the largest of its CTA shapes (2, 4 or kSgNW warps; one CTA runs one DP,
// warp w owns stripes w, w+nw, ...) and the boundary record a stripe leaves for the next one in global scratch (nw
// slots of max_n2 + 2 records per CTA).
constexpr int kSgNW = 8;
struct SgRec {
  int m, f1, f2;
};

// The stripe-flow form of the unweighted semi-global kernel (semiglobal.cu, sg_flow_kernel): per DP, its boundary
// row and the state of its in-order row evaluation; per launch, the DPs in queue order and their stripes as units.
struct SgFlowDP {
  int64_t bnd_off;                  // the DP's boundary row: n2 + 2 records of SgFlow::bnd
  int evaluated, stop;              // stripes evaluated in row order; 1 once the DP ended
  int mx, e1r, e2r, rows;           // running evaluation after `evaluated` stripes (initially 0, -1, -1, 0)
  int stale_last, stale_prev;       // column n2 - 1 of rows n2 - 1 + w and n2 - 2 + w (initially kOut)
};
struct SgFlow {
  SgTask *tasks;
  const int *idx;                   // queue order: DP q is tasks[idx[q]]
  const int64_t *unit_begin;        // [n]: first unit (stripe) of DP q; DP q has max(1, stripes) units
  const int2 *order;                // [total_units]: (q, stripe) in hand-out order (each DP's stripes ascending)
  SgFlowDP *dps;                    // [n], queue order
  SgRec *bnd;
  int *prog;                        // [total_units]: columns of the unit's last row published (zero before launch)
  unsigned long long *unit_counter; // zero before launch
  int *err;                         // set to 1 when a wait ran out of iterations (zero before launch)
  int64_t total_units;
  int n, pad;
};

// ---- kernel launchers (defined in the .cu files)
void launch_pack(const int8_t *codes, const int64_t *src_off, const int64_t *dst_base, const int32_t *len, int nseq,
                 uint32_t *pk, uint32_t *nm, cudaStream_t st);
void launch_scan(RecDesc d, int64_t ntiles, Arena ar, Params p, unsigned long long *keys, int *work_counter, int grid,
                 cudaStream_t st);
void launch_scan_l0(L0Desc d, int64_t ntiles, Arena ar, Params p, unsigned long long *keys, int *work_counter,
                    int64_t grid, cudaStream_t st);
// Compacts the level-0 tasks whose maximum reached min_score (in task order) and runs their reverse scans.
// scratch: >= (n0 / 256 + 2) ints.  Returns nothing; the count is written to *count (device).
void launch_l0_select(const unsigned long long *keys, int64_t n0, const int64_t *wstart, const int2 *plen, int np,
                      const int64_t *seq_base, Arena ar, Params p, int *scratch, int *count, L0Rec *out, int nsm,
                      cudaStream_t st);
void launch_scan_generic(const ScanTask *tasks, const int *idx, int n, const int64_t *seq_base, Arena ar, Params p,
                         unsigned long long *keys, int32_t *scratch, int64_t scratch_per_thread, cudaStream_t st);
// Long tasks (either semantics), one warp each as a wavefront; scratch: per_task >= 2 (tw + 2) ints per task.
void launch_scan_generic_wave(const ScanTask *tasks, const int *idx, int n, const int64_t *seq_base, Arena ar,
                              Params p, unsigned long long *keys, int32_t *scratch, int64_t per_task,
                              cudaStream_t st);
void launch_reverse(ScanTask *tasks, int first, int n, const unsigned long long *keys, const int64_t *pair_base,
                    const int32_t *pair_len, Arena ar, Params p, cudaStream_t st);
// wcap: 10 or 20 (one thread per pass, band in registers), 0 (one warp per pass, band in scratch), -1 (one warp per
// pass as a wavefront, w <= 256: for long passes)
void launch_xdrop(XTask *tasks, const int *idx, int n, Arena ar, Params p, uint32_t *tb, int wcap, int32_t *scratch,
                  int64_t scratch_per_thread, cudaStream_t st);
// tb_words: size of the band store tb (the traceback reads nothing past it)
void launch_xdrop_traceback(XTask *tasks, const int *idx, int n, const uint32_t *tb, int64_t tb_words, uint32_t *cig,
                            cudaStream_t st);
// Chained x-drop levels (one launch per band width, work lists and counts in device memory).
void launch_xdrop_iota(int *list, int n, int *count, cudaStream_t st);
// Hand-off of long register-band passes to the wavefront form: a pass of a row-interleaved level still running after
// `rows` rows moves its band state to one of `cap` spill slots (2 x (2 x 20 + 2) ints each) and its id to list;
// *count (zero before the level) counts the slots taken; `lanes` lanes then run each such pass.  rows = 0 or
// cap = 0: off.
struct XHandoff {
  int *list, *count;
  int32_t *spill;
  int cap, rows;
  int lanes;  // lanes per handed-off pass: 4, 8 or 16 (G-lane groups, 32 / G passes per warp) or 32 (one warp)
};
constexpr int kXdropSpillInts = 2 * (2 * 20 + 2);
// fetch: the level's pass counter, zero before the launch (the row-interleaved register-band kernel, flat = true).
// Traceback slots hold min(n1, slot_rows) rows.  group_from > 0: register-band levels of band group_from and wider
// run every pass on H.lanes-lane groups from row 1 (no one-thread form).  Returns the number of kernels launched.
int launch_xdrop_level(XTask *tasks, const int *list_in, const int *count_in, int *list_out, int *count_out,
                       int *retry, int *retry_count, unsigned long long *tb_cursor, int64_t tb_words, int slot_rows,
                       int *fetch, const XHandoff &H, Arena ar, Params p, uint32_t *tb, int w, int n_bound, int nsm,
                       int32_t *scratch, int64_t per_warp, int warps, int warp_from, int wave_max_w, bool flat,
                       int group_from, bool codes, cudaStream_t st);
void launch_xdrop_traceback_all(XTask *tasks, int n, const uint32_t *tb, int64_t tb_words, uint32_t *cig,
                                unsigned long long *cig_cursor, cudaStream_t st);
// Packs the CIGARs of every finished task in task order into dense (cig_dense offsets); *total = their words.
void launch_xdrop_cigar_pack(XTask *tasks, int n, const uint32_t *cig, uint32_t *dense, unsigned long long *total,
                             cudaStream_t st);
// nw: warps per DP (2, 4 or kSgNW); bnd: sg_bnd_bytes(grid, max_n2, nw) bytes.
void launch_semiglobal(SgTask *tasks, const int *idx, int n, Arena ar, Params p, uint8_t *tb, void *bnd,
                       int max_n2, int *work_counter, int grid, int nw, cudaStream_t st);
int sg_ctas_per_sm(int nw);
// codes: the DPs keep direction codes (every DP of a launch alike)
// minb: 5 or 6 resident blocks per SM (the register budget of the kernel instantiation)
void launch_semiglobal_flow(const SgFlow &f, Arena ar, Params p, uint8_t *tb, bool codes, int nsm, int minb,
                            cudaStream_t st);
int64_t sg_flow_units(int n1, int n2, int w);  // stripe units of one DP in the flow form (at least 1)
int64_t sg_flow_grid_warps(int nsm, int minb);  // warps of the flow kernel's persistent grid
int64_t sg_bnd_bytes(int grid, int max_n2, int nw);
// tb_bytes: size of the code store tb (the traceback reads nothing past it)
void launch_sg_traceback(SgTask *tasks, const int *idx, int n, int bandwidth, const uint8_t *tb, int64_t tb_bytes,
                         uint32_t *cig, cudaStream_t st, bool weighted_layout = false);
int64_t sg_tb_bytes(int n1, int n2, int w);
int64_t sgw_tb_bytes(int n1, int n2, int w);
int64_t sgw_bnd_bytes(int warps, int max_n2);
void launch_semiglobal_weighted(SgTask *tasks, const int *idx, int n, Arena ar, Params p, SgWeights wt, uint8_t *tb,
                                void *bnd, int max_n2, int *work_counter, int warps, cudaStream_t st);

}  // namespace dcns
