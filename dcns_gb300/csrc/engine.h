// Host side of the GB300 CNS pair-alignment engine: context, device buffers and the pipeline entry points that the
// C ABI (capi.cpp) exposes.
#pragma once

#include <chrono>
#include <cstdint>
#include <condition_variable>
#include <mutex>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dcns_gb300.h"
#include "common.h"

namespace dcns {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define DCNS_CK(x)                                                                                      \
  do {                                                                                                  \
    cudaError_t e_ = (x);                                                                               \
    if (e_ != cudaSuccess) throw ::dcns::Error(DCNS_ERR_DEVICE, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct Context;

// Grow-only device buffer accounted against the context's memory budget.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  void ensure(Context &C, size_t bytes);
  void release(Context &C);
  template <class T>
  T *as() const {
    return (T *)p;
  }
};

// Grow-only pinned host buffer (staging for host<->device copies).
struct HostBuf {
  void *p = nullptr;
  size_t cap = 0;
  void ensure(size_t bytes);
  void release();
  template <class T>
  T *as() const {
    return (T *)p;
  }
};

struct PairIn {
  const int8_t *s1;
  int32_t n1;
  const int8_t *s2;
  int32_t n2;
};

struct FragOut {
  int64_t s1, e1, s2, e2, score;  // 1-based, as PairedSimilarFragment
  std::vector<uint32_t> cigar;
  double p, e;
};

struct Seed4 {
  int32_t s1, e1, s2, e2;  // 0-based inclusive
};

// The reference's Seed ordering (model/Seed.h:29-42): seeds sharing their start pair or their end pair compare equal,
// otherwise lexicographic on (start1, start2).  Not a strict weak order: set contents depend on insertion order and
// tree shape, so the replay below performs exactly the reference's insertion sequence on a libstdc++ std::set.
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

// Weighted variants: device category ids of every pair's seq1 (pair p at wbase[p]) and the category table.
struct WeightSet {
  SgWeights dev{};
  std::vector<int64_t> wbase;
};

struct Context {
  int device = 0;
  cudaStream_t st = nullptr;       // every launch and copy of the context (high priority)
  cudaStream_t st_bulk = nullptr;  // the level-0 seed scan only (low priority): other lanes' short kernels overtake it
  cudaEvent_t ev_bulk = nullptr;
  size_t budget = 0, used = 0;
  int nsm = 0, scan_blocks_per_sm = 1;
  std::string err;
  dcns_stats stats{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;

  // device buffers
  DevBuf d_codes, d_srcoff, d_dstbase, d_len, d_pk, d_nm, d_seqbase, d_flag;
  DevBuf d_tasks, d_keys, d_tiles, d_counter, d_idx, d_scratch;
  DevBuf d_x, d_tb, d_cig, d_sg, d_sgtb, d_bnd, d_wts, d_cats, d_spill, d_flow;
  const WeightSet *weights = nullptr;  // set during a weighted call
  // pinned staging
  HostBuf h_codes, h_misc, h_out, h_tasks, h_tiles;

  // arena layout of the batch being aligned (the context's own upload buffers, or a resident batch)
  std::vector<int64_t> seq_base;  // 2 per pair
  Arena arena{};
  const int64_t *seqbase_dev = nullptr;

  // Large batches are split into bins run on `lanes` (each its own stream and buffers, sharing the arena), so one
  // bin's host-side replay and linking overlap another bin's kernels.  Four lanes over four bins measured best on
  // the 10,000-pair log-normal workload (fewer leave host time exposed; more add per-bin round latency).
  std::vector<std::unique_ptr<Context>> lanes;
  // DCNS_LANES / DCNS_BINS in the environment override the defaults at context creation.
  bool is_lane = false;
  double bin_ratio = 0.6;    // bin b holds a share of the work proportional to bin_ratio^b (later bins smaller)
  bool bins_by_size = false;  // bins are consecutive runs of pairs in increasing size (else a mix of sizes each)
  int xdrop_warp_from = 20;  // x-drop bands wider than this run one warp per pass (DCNS_XDROP_WARP_FROM)
  // x-drop bands wider than xdrop_warp_from and up to this run as one-warp wavefronts (DCNS_XDROP_WAVE; 0 = off)
  int xdrop_wave_max_w = 256;
  // register-band levels (w <= 20) as the row-interleaved kernel (DCNS_XDROP_FLAT=0: one pass per thread)
  bool xdrop_flat = true;
  // a pass of a row-interleaved level still running after this many rows moves to the wavefront form
  // (DCNS_XDROP_HANDOFF; 0 = off)
  int xdrop_handoff = 96;
  // lanes that run each handed-off pass as a wavefront: 4, 8, 16 or 32 (DCNS_XDROP_RESUME_LANES)
  int xdrop_resume_lanes = 8;
  // register-band levels of this band and wider run every pass on lane groups from row 1 (DCNS_XDROP_GROUP_FROM;
  // 0 = off)
  int xdrop_group_from = 0;
  // warps per DP of the unweighted semi-global kernel: 2, 4 or 8 (DCNS_SG_WARPS; 0 = by the number of DPs)
  int sg_warps = 0;
  // unweighted semi-global DPs as a flow of stripe units over one persistent grid (DCNS_SG_FLOW=0: one CTA per DP)
  bool sg_flow = true;
  // resident blocks per SM of the stripe-flow kernel: 5 (96 registers) or 6 (80 registers) (DCNS_SG_FLOW_BLOCKS)
  int sg_flow_blocks = 5;
  // seed-scan tiling target: reference rows are split into chunks while a launch has fewer tiles than this many per
  // resident thread (DCNS_SCAN_TILES)
  int scan_tiles_per_thread = 8;
  // per-bin x-drop pass forms and seed-scan tiling target chosen by the autotuner (empty: the values above for every
  // bin)
  struct BinTune {
    int xdrop_warp_from, xdrop_wave_max_w;
    bool xdrop_flat;
    int xdrop_handoff, xdrop_resume_lanes, xdrop_group_from;
    int scan_tiles;
  };
  std::vector<BinTune> bin_tune;
  std::vector<double> last_bin_xdrop_ms;  // x-drop kernel time of each bin of the last binned call
  std::vector<double> last_bin_scan_ms;   // seed-scan kernel time of each bin of the last binned call
  // Level-0 turnstile of one binned call: the bins enqueue their level-0 scans on the parent's bulk stream in bin
  // order, so the scans run one after another and the first bins' host work overlaps the later bins' scans.
  struct Turnstile {
    std::mutex mu;
    std::condition_variable cv;
    int next = 0;
    bool abort = false;
  };
  Turnstile *l0_turn = nullptr;
  int bin = -1;
  cudaStream_t bulk_shared = nullptr;
  int trace = 0;  // DCNS_TRACE=1: per-phase host timings of each align call on stderr; 2: also a per-lane timeline
  int lane_id = -1;
  std::chrono::steady_clock::time_point call_t0;
  std::vector<std::pair<const char *, double>> phases;
  int max_lanes = 4;
  int bins = 4;

  ~Context();
};

void init_context(Context &C, int device, size_t budget);
// Frees the context's grow-only device buffers (after its stream is idle), so the next call sizes them afresh.
void release_device_buffers(Context &C);

Params to_params(const dcns_params *p);
void validate(const Params &P);

// Sequences packed and resident on the device (dcns_batch_upload).
struct Batch {
  DevBuf pk, nm, sb;
  std::vector<int64_t> seq_base;
  std::vector<PairIn> lens;  // lengths only (sequence pointers are not kept)
  Arena arena{};
};

// Whole-path entry points (engine.cpp)
void align_pairs(Context &C, const std::vector<PairIn> &pairs, const Params &P, int mode,
                 std::vector<std::vector<FragOut>> &out);
void batch_upload(Context &C, const std::vector<PairIn> &pairs, Batch &B);
void align_batch(Context &C, Batch &B, const Params &P, int mode, std::vector<std::vector<FragOut>> &out);
// The weighted drivers (pieces 1 or 2): weights[p] = category id per seq1 base of pair p; cats = 7 ints per category.
void align_weighted(Context &C, const std::vector<PairIn> &pairs, const std::vector<const int16_t *> &weights,
                    const std::vector<int32_t> &cats, int pieces, const Params &P,
                    std::vector<std::vector<FragOut>> &out);
// The seeded 2-gap overload (cut2Gaps2) over many pairs; seeds[p] in the caller's order.
void align_seeded(Context &C, const std::vector<PairIn> &pairs, const std::vector<std::vector<Seed4>> &seeds,
                  const Params &P, std::vector<std::vector<FragOut>> &out);
// The 2-piece stage over caller-given x-seeds (the x-seed overload without maximumAlignLength).
void align_xseeds(Context &C, const std::vector<PairIn> &pairs, const std::vector<std::vector<Seed4>> &seeds,
                  const Params &P, std::vector<std::vector<FragOut>> &out);
// Times the resident batch under candidate (lanes, bins, bin_ratio) shapes and keeps the fastest on C.
void autotune(Context &C, Batch &B, const Params &P, int mode);
double measure_issue_rate(int nsm, cudaStream_t st);
void smith_waterman_batch(Context &C, const std::vector<PairIn> &tasks, const Params &P, int32_t *out);
// cigar: every task's CIGAR in task order; cigar_off[k] .. cigar_off[k + 1] is task k's (n + 1 offsets)
void xextend_batch(Context &C, const std::vector<PairIn> &tasks, const Params &P, bool want_cigar, int32_t *out,
                   std::vector<uint32_t> &cigar, std::vector<int64_t> &cigar_off);
void semiglobal_batch(Context &C, const std::vector<PairIn> &tasks, const Params &P, bool want_cigar, int32_t *out,
                      std::vector<std::vector<uint32_t>> &cigars);
void sliding_window(Context &C, const int8_t *const *seqs, const int32_t *lens, int32_t n, const Params &P,
                    double *score, int32_t *max_out);

int scan_occupancy();  // resident blocks per SM of the fast scan kernel (seedscan.cu)

}  // namespace dcns
