// Host orchestration of the GB300 CNS pair-alignment path.
//
// align_pairs() runs, for a batch of independent (reference, query) pairs, what the reference runs per pair in
// findSimilarFragmentsForPairedSequence (impl/findSimilarFragmentsForPairedSequence4.cpp:433 for 1-gap, :752 for
// 2-gap):
//   1. upload + pack            all sequences into one 2-bit arena (one H2D, one pack kernel)
//   2. seed scan                every window x full reference as ScanTasks -> int16x2 tiles (seedscan.cu), then the
//                               reverse scan that fixes each seed's start
//   3. recursion + replay       the reference recurses into the reference on both sides of every new seed and
//                               gates the top-level recursion on set membership with a non-strict-weak comparator.
//                               Recursion tasks are computed level-synchronously on the device; the host replays the
//                               exact std::set insertion sequence per pair, requesting the children it needs, until
//                               no pair needs more (optimistic replay: windows later gated out may have had their
//                               children computed; such work is counted as speculative, not algorithmic).
//   4. link_seeds               per pair, host (:288-344)
//   5. x-drop                   forward pass, reverse pass with 4-bit direction codes, traceback (xdrop.cu); band
//                               restarts and traceback-slot growth are relaunches
//   6. fragments                p/e-values in FP64 on the host, dedupe in the reference's order (:497-520)
//   2-gap mode replaces 5-6 by the x-drop filter (:395-427) and the 2-piece semi-global stage (:532-616).
#include "engine.h"

#include <algorithm>
#include <cstdlib>
#include <array>
#include <map>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <deque>
#include <condition_variable>
#include <functional>
#include <thread>

namespace dcns {

// ------------------------------------------------------------------ buffers
void DevBuf::ensure(Context &C, size_t bytes) {
  if (bytes <= cap) return;
  size_t want = std::max(bytes, cap + cap / 2);
  want = (want + 255) & ~size_t(255);
  if (C.used - cap + want > C.budget) {
    want = bytes;
    if (C.used - cap + want > C.budget)
      throw Error(DCNS_ERR_NOMEM, "device memory budget exhausted (" + std::to_string(C.used - cap + want) +
                                      " > " + std::to_string(C.budget) + " bytes)");
  }
  if (p) {
    DCNS_CK(cudaFree(p));
    C.used -= cap;
    p = nullptr;
    cap = 0;
  }
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    p = nullptr;
    (void)cudaGetLastError();
    throw Error(DCNS_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  cap = want;
  C.used += want;
}

void DevBuf::release(Context &C) {
  if (p) {
    cudaFree(p);
    C.used -= cap;
  }
  p = nullptr;
  cap = 0;
}

void HostBuf::ensure(size_t bytes) {
  if (bytes <= cap) return;
  size_t want = std::max(bytes, cap + cap / 2);
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  DCNS_CK(cudaMallocHost(&p, want));
  cap = want;
}

void HostBuf::release() {
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
}

void release_device_buffers(Context &C) {
  if (C.st) cudaStreamSynchronize(C.st);  // nothing of the context still reads them
  DevBuf *bufs[] = {&C.d_codes, &C.d_srcoff, &C.d_dstbase, &C.d_len, &C.d_pk, &C.d_nm, &C.d_seqbase, &C.d_flag,
                    &C.d_tasks, &C.d_keys, &C.d_tiles, &C.d_counter, &C.d_idx, &C.d_scratch, &C.d_x, &C.d_tb,
                    &C.d_cig, &C.d_sg, &C.d_sgtb, &C.d_bnd, &C.d_wts, &C.d_cats};
  for (DevBuf *b : bufs) b->release(C);
}

Context::~Context() {
  release_device_buffers(*this);
  h_codes.release();
  h_misc.release();
  h_out.release();
  h_tasks.release();
  h_tiles.release();
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (ev2) cudaEventDestroy(ev2);
  if (ev_bulk) cudaEventDestroy(ev_bulk);
  if (st_bulk) cudaStreamDestroy(st_bulk);
  if (st) cudaStreamDestroy(st);
}

void init_context(Context &C, int device, size_t budget) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    (void)cudaGetLastError();
    throw Error(DCNS_ERR_DEVICE, "no CUDA device available (this library has no CPU fallback)");
  }
  if (device < 0 || device >= ndev) throw Error(DCNS_ERR_INVALID, "device ordinal out of range");
  DCNS_CK(cudaSetDevice(device));
  cudaDeviceProp prop;
  DCNS_CK(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10)
    throw Error(DCNS_ERR_DEVICE, "this build targets sm_103a (GB300); found sm_" + std::to_string(prop.major * 10 + prop.minor));
  C.device = device;
  C.nsm = prop.multiProcessorCount;
  C.scan_blocks_per_sm = scan_occupancy();
  if (C.scan_blocks_per_sm <= 0) throw Error(DCNS_ERR_DEVICE, "the seed-scan kernel could not be configured");
  int prio_lo = 0, prio_hi = 0;
  DCNS_CK(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
  DCNS_CK(cudaStreamCreateWithPriority(&C.st, cudaStreamNonBlocking, prio_hi));
  DCNS_CK(cudaStreamCreateWithPriority(&C.st_bulk, cudaStreamNonBlocking, prio_lo));
  DCNS_CK(cudaEventCreateWithFlags(&C.ev_bulk, cudaEventDisableTiming));
  DCNS_CK(cudaEventCreate(&C.ev0));
  DCNS_CK(cudaEventCreate(&C.ev1));
  DCNS_CK(cudaEventCreate(&C.ev2));
  if (budget == 0) {
    size_t fr = 0, tot = 0;
    DCNS_CK(cudaMemGetInfo(&fr, &tot));
    budget = fr / 10 * 8;
  }
  C.budget = budget;
  if (const char *e = std::getenv("DCNS_LANES")) C.max_lanes = std::max(1, std::min(8, std::atoi(e)));
  if (const char *e = std::getenv("DCNS_BINS")) C.bins = std::max(1, std::min(64, std::atoi(e)));
  if (const char *e = std::getenv("DCNS_TRACE")) C.trace = std::atoi(e);
  if (const char *e = std::getenv("DCNS_XDROP_WARP_FROM")) C.xdrop_warp_from = std::max(0, std::atoi(e));
  if (const char *e = std::getenv("DCNS_XDROP_WAVE")) C.xdrop_wave_max_w = std::max(0, std::atoi(e));
  if (const char *e = std::getenv("DCNS_XDROP_FLAT")) C.xdrop_flat = std::atoi(e) != 0;
  if (const char *e = std::getenv("DCNS_XDROP_HANDOFF")) C.xdrop_handoff = std::max(0, std::atoi(e));
  if (const char *e = std::getenv("DCNS_XDROP_RESUME_LANES")) {
    const int v = std::atoi(e);
    C.xdrop_resume_lanes = (v == 4 || v == 8 || v == 16 || v == 32) ? v : 8;
  }
  if (const char *e = std::getenv("DCNS_XDROP_GROUP_FROM")) C.xdrop_group_from = std::max(0, std::atoi(e));
  if (const char *e = std::getenv("DCNS_SCAN_TILES")) C.scan_tiles_per_thread = std::max(1, std::min(64, std::atoi(e)));
  if (const char *e = std::getenv("DCNS_SG_WARPS")) {
    const int v = std::atoi(e);
    C.sg_warps = (v == 2 || v == 4 || v == kSgNW) ? v : 0;
  }
  if (const char *e = std::getenv("DCNS_SG_FLOW")) {
    C.sg_flow = std::atoi(e) != 0;
  }
  if (const char *e = std::getenv("DCNS_SG_FLOW_BLOCKS")) C.sg_flow_blocks = std::atoi(e) == 6 ? 6 : 5;
  if (const char *e = std::getenv("DCNS_BIN_RATIO")) C.bin_ratio = std::max(0.1, std::min(4.0, std::atof(e)));
  if (const char *e = std::getenv("DCNS_BINS_BY_SIZE")) C.bins_by_size = std::atoi(e) != 0;
}

Params to_params(const dcns_params *p) {
  Params P;
  P.match = p->match;
  P.mismatch = p->mismatch;
  P.open1 = p->open1;
  P.ext1 = p->ext1;
  P.open2 = p->open2;
  P.ext2 = p->ext2;
  P.window = p->window;
  P.min_score = p->min_score;
  P.step = p->step;
  P.w = p->w;
  P.xdrop = p->xdrop;
  P.zdrop = p->zdrop;
  // A band wider than every sequence gives the same DP as an unbounded one, and sequences are shorter than
  // kMaxSeqLen (upload_into rejects longer ones), so wider bands are clamped: the kernels' band-edge arithmetic
  // (i + w, 2w + stripe rows) then stays inside int32.
  P.bandwidth = std::min(p->bandwidth, kMaxSeqLen);
  P.max_align_len = p->max_align_len;
  P.pvalue = p->pvalue;
  P.lambda = p->lambda;
  P.kvalue = p->kvalue;
  return P;
}

void validate(const Params &P) {
  auto bad = [](const char *m) { throw Error(DCNS_ERR_INVALID, m); };
  // Scorei stores scores as int8 (model/Score.cpp:105); the reference's striped kernels cast gap penalties to int8.
  if (P.match < 1 || P.match > 127 || P.mismatch < -127 || P.mismatch > 127) bad("match must be 1..127, mismatch -127..127");
  if (P.open1 > 0 || P.ext1 > 0 || P.open1 < -127 || P.ext1 < -127) bad("open1/ext1 must be in -127..0");
  if (P.open2 > 0 || P.ext2 > 0 || P.open2 < -100000 || P.ext2 < -100000) bad("open2/ext2 must be <= 0");
  if (P.window < 1 || P.window > 128) bad("window must be 1..128");
  if (P.step < 1) bad("step must be >= 1");
  if (P.min_score < 1) bad("min_score must be >= 1");
  if (P.w < 1 || P.w > (1 << 20)) bad("w must be 1..2^20");
  if (P.xdrop < 0 || P.zdrop < 0) bad("xdrop/zdrop must be >= 0");
  if (P.bandwidth < 1) bad("bandwidth must be >= 1");
}

namespace {

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t) { return std::chrono::duration<double, std::milli>(Clock::now() - t).count(); }

// Adds the time since t to phase `name` when tracing; returns now.
Clock::time_point phase(Context &C, const char *name, Clock::time_point t) {
  const Clock::time_point now = Clock::now();
  if (C.trace) {
    const double ms = std::chrono::duration<double, std::milli>(now - t).count();
    if (C.trace >= 2)
      std::fprintf(stderr, "[dcns tl] lane %d %s %.2f %.2f\n", C.lane_id,
                   name, std::chrono::duration<double, std::milli>(t - C.call_t0).count(),
                   std::chrono::duration<double, std::milli>(now - C.call_t0).count());
    for (auto &e : C.phases)
      if (std::strcmp(e.first, name) == 0) {
        e.second += ms;
        return now;
      }
    C.phases.push_back({name, ms});
  }
  return now;
}

void print_phases(Context &C, const char *what) {
  if (!C.trace) return;
  std::string s = std::string("[dcns trace] ") + what;
  char buf[96];
  for (auto &e : C.phases) {
    std::snprintf(buf, sizeof buf, " %s=%.2f", e.first, e.second);
    s += buf;
  }
  std::fprintf(stderr, "%s\n", s.c_str());
  C.phases.clear();
}

// Host worker pool for parallel_for: created on first use, shared by every context and lane.  Jobs are served in
// arrival order; the calling thread works on its own job too, so concurrent callers (two lanes) always progress.
class HostPool {
 public:
  struct Job {
    const std::function<void(int64_t)> *f;
    int64_t n;
    std::atomic<int64_t> next{0}, done{0};
    std::mutex m;
    std::condition_variable cv;
  };
  static HostPool &get() {
    static HostPool *pool = new HostPool();  // never destroyed: workers may outlive static destructors
    return *pool;
  }
  int size() const { return (int)th_.size() + 1; }
  void run(int64_t n, const std::function<void(int64_t)> &f) {
    auto J = std::make_shared<Job>();
    J->f = &f;
    J->n = n;
    {
      std::lock_guard<std::mutex> lk(mu_);
      q_.push_back(J);
    }
    cv_.notify_all();
    work(*J);
    {
      std::unique_lock<std::mutex> lk(J->m);
      J->cv.wait(lk, [&] { return J->done.load() >= n; });
    }
    std::lock_guard<std::mutex> lk(mu_);
    for (auto it = q_.begin(); it != q_.end(); ++it)
      if (it->get() == J.get()) {
        q_.erase(it);
        break;
      }
  }
  static thread_local bool in_worker;

 private:
  HostPool() {
    const int nt = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 32u);
    for (int t = 1; t < nt; ++t) th_.emplace_back([this] { loop(); });
    for (auto &t : th_) t.detach();
  }
  static void work(Job &J) {
    for (int64_t i; (i = J.next.fetch_add(1)) < J.n;) {
      (*J.f)(i);
      if (J.done.fetch_add(1) + 1 == J.n) {
        std::lock_guard<std::mutex> lk(J.m);
        J.cv.notify_all();
      }
    }
  }
  void loop() {
    in_worker = true;
    for (;;) {
      std::shared_ptr<Job> J;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !q_.empty(); });
        while (!q_.empty() && q_.front()->next.load() >= q_.front()->n) q_.pop_front();
        if (q_.empty()) continue;
        J = q_.front();
      }
      work(*J);
    }
  }
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::shared_ptr<Job>> q_;
  std::vector<std::thread> th_;
};
thread_local bool HostPool::in_worker = false;

void parallel_for(int64_t n, const std::function<void(int64_t)> &f, int64_t min_items = 64) {
  if (n < min_items || n < 2 || HostPool::in_worker || std::thread::hardware_concurrency() <= 1) {
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
  HostPool::get().run(n, f);
}

template <class T>
void h2d(Context &C, DevBuf &d, const T *src, size_t n, size_t off_elems = 0) {
  if (!n) return;
  DCNS_CK(cudaMemcpyAsync(d.as<T>() + off_elems, src, n * sizeof(T), cudaMemcpyHostToDevice, C.st));
}
template <class T>
void d2h(Context &C, T *dst, const DevBuf &d, size_t n, size_t off_elems = 0) {
  if (!n) return;
  DCNS_CK(cudaMemcpyAsync(dst, d.as<T>() + off_elems, n * sizeof(T), cudaMemcpyDeviceToHost, C.st));
}
void sync(Context &C) {
  DCNS_CK(cudaStreamSynchronize(C.st));
  DCNS_CK(cudaGetLastError());
}

bool striped_for_host(int nref, int nread, int open, int ext, int match) {
  auto ok = [&](int64_t lim) {
    return ((-(int64_t)nref * ext - open) < lim || (-(int64_t)nread * ext - open) < lim) &&
           ((int64_t)nref * match < lim || (int64_t)nread * match < lim);
  };
  return ok(125) || ok(32767);
}

// ------------------------------------------------------------------ 1. upload + pack
void upload_into(Context &C, const std::vector<PairIn> &pairs, DevBuf &d_pk, DevBuf &d_nm, DevBuf &d_sb,
                 std::vector<int64_t> &seq_base, Arena &arena) {
  auto tp = Clock::now();
  const int64_t np = (int64_t)pairs.size(), ns = 2 * np;
  seq_base.assign(ns, 0);
  std::vector<int64_t> src_off(ns);
  std::vector<int32_t> len(ns);
  int64_t total_src = 0, total_dst = 0;
  // A sequence passed again for the next pair on the same side (the same pointer and length: one reference against
  // many queries, as in the multi-species caller) is staged and packed once; the later pairs point at the first copy.
  const int8_t *last_src[2] = {nullptr, nullptr};
  int32_t last_n[2] = {-1, -1};
  int64_t last_base[2] = {0, 0};
  for (int64_t k = 0; k < np; ++k) {
    for (int h = 0; h < 2; ++h) {
      const int32_t n = h ? pairs[k].n2 : pairs[k].n1;
      const int8_t *src = h ? pairs[k].s2 : pairs[k].s1;
      if (n < 0) throw Error(DCNS_ERR_INVALID, "negative sequence length");
      if (n >= kMaxSeqLen) throw Error(DCNS_ERR_INVALID, "sequences must be shorter than 2^28 bases");
      if (n > 0) {
        if (src == last_src[h] && n == last_n[h]) {
          len[2 * k + h] = 0;  // nothing to stage or pack
          src_off[2 * k + h] = total_src;
          seq_base[2 * k + h] = last_base[h];
          continue;
        }
        last_src[h] = src, last_n[h] = n, last_base[h] = total_dst;
      }
      len[2 * k + h] = n;
      src_off[2 * k + h] = total_src;
      seq_base[2 * k + h] = total_dst;
      total_src += n;
      total_dst += ((int64_t)n + 63) / 64 * 64;
    }
  }
  total_dst += 128;  // lets every kernel read one 64-base block past any sequence end
  tp = phase(C, "up_index", tp);
  C.h_codes.ensure((size_t)std::max<int64_t>(total_src, 1));
  int8_t *stage = C.h_codes.as<int8_t>();
  // staged copy; the reference indexes its 5x5 score table with the codes, so anything outside 0..4 is rejected
  std::atomic<bool> badcode(false);
  // blocks of consecutive sequences of about 1 MB each (one work item per sequence would serialise a million short
  // sequences on the pool's work counter)
  std::vector<int64_t> blk{0};
  for (int64_t s = 0, acc = 0; s < ns; ++s) {
    acc += len[s] + 64;
    if (acc >= (1 << 20)) blk.push_back(s + 1), acc = 0;
  }
  if (blk.back() != ns) blk.push_back(ns);
  parallel_for((int64_t)blk.size() - 1, [&](int64_t b) {
    uint8_t bad = 0;
    for (int64_t s = blk[b]; s < blk[b + 1]; ++s) {
      if (!len[s]) continue;
      const PairIn &p = pairs[s / 2];
      const int8_t *src = (s & 1) ? p.s2 : p.s1;
      int8_t *dst = stage + src_off[s];
      std::memcpy(dst, src, (size_t)len[s]);
      for (int32_t i = 0; i < len[s]; ++i) bad |= (uint8_t)((uint8_t)dst[i] > 4);
    }
    if (bad) badcode = true;
  });
  if (badcode) throw Error(DCNS_ERR_INVALID, "sequence codes must be dCNS codes 0..4 (A C N G T)");
  tp = phase(C, "up_stage", tp);
  C.d_codes.ensure(C, (size_t)std::max<int64_t>(total_src, 1));
  C.d_srcoff.ensure(C, sizeof(int64_t) * ns + 8);
  C.d_dstbase.ensure(C, sizeof(int64_t) * ns + 8);
  C.d_len.ensure(C, sizeof(int32_t) * ns + 8);
  d_sb.ensure(C, sizeof(int64_t) * ns + 8);
  d_pk.ensure(C, sizeof(uint32_t) * (total_dst / 16));
  d_nm.ensure(C, sizeof(uint32_t) * (total_dst / 32));
  C.d_flag.ensure(C, 64);
  h2d(C, C.d_codes, stage, (size_t)total_src);
  h2d(C, C.d_srcoff, src_off.data(), ns);
  h2d(C, C.d_dstbase, seq_base.data(), ns);
  h2d(C, C.d_len, len.data(), ns);
  h2d(C, d_sb, seq_base.data(), ns);
  C.stats.bytes_h2d += total_src + (int64_t)ns * (8 + 8 + 4 + 8);
  DCNS_CK(cudaMemsetAsync(d_pk.p, 0, sizeof(uint32_t) * (total_dst / 16), C.st));
  DCNS_CK(cudaMemsetAsync(d_nm.p, 0, sizeof(uint32_t) * (total_dst / 32), C.st));
  launch_pack(C.d_codes.as<int8_t>(), C.d_srcoff.as<int64_t>(), C.d_dstbase.as<int64_t>(), C.d_len.as<int32_t>(),
              (int)ns, d_pk.as<uint32_t>(), d_nm.as<uint32_t>(), C.st);
  C.stats.kernel_launches += 1;
  arena.pk = d_pk.as<uint32_t>();
  arena.nm = d_nm.as<uint32_t>();
  phase(C, "up_enqueue", tp);
}

// Uploads into the context's own buffers and makes them the current arena.
void upload(Context &C, const std::vector<PairIn> &pairs) {
  upload_into(C, pairs, C.d_pk, C.d_nm, C.d_seqbase, C.seq_base, C.arena);
  C.seqbase_dev = C.d_seqbase.as<int64_t>();
}

// ------------------------------------------------------------------ 2./3. seed scan with recursion replay
// Smith-Waterman tasks of one batch.  tasks[0, ns) are the level-0 windows the host needs (those whose maximum
// reached min_score; every window when the generic kernel runs level 0), in pair and window order, pair p owning
// [pbeg[p], pbeg[p+1]); recursion tasks follow (ids >= ns, device slot id - ns).
struct ScanState {
  std::vector<ScanTask> tasks;
  int64_t ns = 0;
  std::vector<int64_t> pbeg;
  std::vector<int32_t> left, right;  // child task id, -1 none/not created
  int64_t first_new = 0;             // recursion tasks [first_new, size) still to be computed
  ScanTask &task(int64_t i) { return tasks[i]; }
  const ScanTask &task(int64_t i) const { return tasks[i]; }
  int64_t size() const { return (int64_t)tasks.size(); }
};

// The fast kernel's table stores s - open in int8 and pads short windows with -16384 in int16 lanes.
bool fast_scan_ok(const Params &P) { return P.window <= kScanW && P.match - P.open1 <= 127; }

int warmup_rows(const Params &P, int tw) {
  // A positive-scoring local path over tw read columns spans at most tw diagonal rows plus fewer than
  // match*tw/g vertical-gap rows (g = cheapest gap row), so a scan restarted K rows early is exact from row K on.
  const int g = std::min(-P.open1, -P.ext1);
  if (g <= 0) return INT_MAX;
  return tw + (P.match * tw + g - 1) / g + 4;
}

// Launches the scan over `tiles` plus the generic kernel over `generic` (device slots), then the reverse scans for
// recursion tasks [first, first+n) (device slots first - ns ...); downloads those tasks.
void run_scan_round(Context &C, ScanState &S, const Params &P, int64_t first, int64_t n, const RecDuo *duos,
                    int64_t nduo, int64_t ntiles, int32_t chunk, int warm, const std::vector<int32_t> &generic) {
  auto tx = Clock::now();
  const int64_t d0 = first - S.ns;  // device slot of the first task
  C.d_keys.ensure(C, sizeof(unsigned long long) * (S.size() - S.ns));
  DCNS_CK(cudaMemsetAsync(C.d_keys.as<unsigned long long>() + d0, 0, sizeof(unsigned long long) * n, C.st));
  if (ntiles > 0) {
    C.d_tiles.ensure(C, sizeof(RecDuo) * nduo);
    C.d_counter.ensure(C, 64);
    h2d(C, C.d_tiles, duos, (size_t)nduo);
    DCNS_CK(cudaMemsetAsync(C.d_counter.p, 0, sizeof(int), C.st));
    const int grid = (int)std::min<int64_t>((int64_t)C.nsm * C.scan_blocks_per_sm,
                                            (ntiles + kScanThreads - 1) / kScanThreads);
    const RecDesc D{C.d_tiles.as<RecDuo>(), C.d_tasks.as<ScanTask>(), C.seqbase_dev, (int32_t)nduo, chunk, warm, 0};
    DCNS_CK(cudaEventRecord(C.ev0, C.st));
    launch_scan(D, ntiles, C.arena, P, C.d_keys.as<unsigned long long>(), C.d_counter.as<int>(), std::max(grid, 1),
                C.st);
    DCNS_CK(cudaEventRecord(C.ev1, C.st));
    C.stats.scan_launches += 1;
    C.stats.kernel_launches += 1;
  }
  if (!generic.empty()) {
    // large tasks (long reads: only the kernel-level call has them) run one warp each as wavefronts, the rest one
    // thread each
    auto wave = [&](int32_t k) {
      const ScanTask &T = S.task(k + S.ns);
      return T.tw >= 64 && (int64_t)(T.hi - T.lo) * T.tw >= (1 << 20);
    };
    std::vector<int32_t> gl;
    gl.reserve(generic.size());
    int maxtw = 0;
    for (int32_t k : generic) {
      maxtw = std::max(maxtw, S.task(k + S.ns).tw);
      if (!wave(k)) gl.push_back(k);
    }
    const int64_t nthread = (int64_t)gl.size();
    for (int32_t k : generic)
      if (wave(k)) gl.push_back(k);
    const int64_t nwave = (int64_t)gl.size() - nthread;
    const int64_t per = 3 * ((int64_t)maxtw + 2);
    C.d_idx.ensure(C, sizeof(int32_t) * gl.size());
    C.d_scratch.ensure(C, sizeof(int32_t) * per * gl.size());
    h2d(C, C.d_idx, gl.data(), gl.size());
    launch_scan_generic(C.d_tasks.as<ScanTask>(), C.d_idx.as<int>(), (int)nthread, C.seqbase_dev, C.arena, P,
                        C.d_keys.as<unsigned long long>(), C.d_scratch.as<int32_t>(), per, C.st);
    launch_scan_generic_wave(C.d_tasks.as<ScanTask>(), C.d_idx.as<int>() + nthread, (int)nwave, C.seqbase_dev,
                             C.arena, P, C.d_keys.as<unsigned long long>(), C.d_scratch.as<int32_t>() + per * nthread,
                             per, C.st);
    C.stats.kernel_launches += (nthread > 0) + (nwave > 0);
  }
  launch_reverse(C.d_tasks.as<ScanTask>(), (int)d0, (int)n, C.d_keys.as<unsigned long long>(), C.seqbase_dev,
                 nullptr, C.arena, P, C.st);
  C.stats.kernel_launches += 1;
  d2h(C, S.tasks.data() + first, C.d_tasks, (size_t)n, (size_t)d0);
  sync(C);
  C.stats.scan_rounds += 1;
  C.stats.ms_scan_xfer += ms_since(tx);
  if (ntiles > 0) {
    float ms = 0;
    DCNS_CK(cudaEventElapsedTime(&ms, C.ev0, C.ev1));
    C.stats.ms_scan_kernel += ms;
  }
}

// Recursion rounds (and the generic level 0): tasks [S.first_new, size).  Fast tasks of one pair with similar row
// ranges are paired into int16x2 tiles; the rest go to the generic kernel.
void compute_scan_tasks(Context &C, ScanState &S, const Params &P) {
  const int64_t first = S.first_new, n = S.size() - first;
  if (n <= 0) return;
  S.first_new = S.size();
  auto t0 = Clock::now();
  auto tp = t0;
  const bool fast_ok = fast_scan_ok(P);
  std::vector<int32_t> fast, generic;  // device slots
  for (int64_t k = first; k < first + n; ++k) {
    ScanTask &T = S.task(k);
    T.striped = striped_for_host(T.hi - T.lo, T.tw, P.open1, P.ext1, P.match) ? 1 : 0;
    if (T.tw <= 0 || T.hi <= T.lo) continue;  // nothing to scan: key stays 0
    if (fast_ok && T.striped && T.tw <= kScanW)
      fast.push_back((int32_t)(k - S.ns));
    else
      generic.push_back((int32_t)(k - S.ns));
  }
  tp = phase(C, "sc_classify", tp);
  auto tk = [&](int32_t d) -> const ScanTask & { return S.task(d + S.ns); };
  // Recursion tasks arrive grouped by pair (the replay requests them pair by pair); within a pair, order by row
  // range so that the two halves of a tile cover similar rows.  Pairs' groups are sorted independently.
  std::vector<size_t> gb{0};
  for (size_t i = 1; i <= fast.size(); ++i)
    if (i == fast.size() || tk(fast[i]).pair != tk(fast[i - 1]).pair) gb.push_back(i);
  parallel_for((int64_t)gb.size() - 1, [&](int64_t g) {
    std::sort(fast.begin() + gb[g], fast.begin() + gb[g + 1], [&](int32_t a, int32_t b) {
      const ScanTask &x = tk(a), &y = tk(b);
      if (x.lo != y.lo) return x.lo < y.lo;
      if (x.hi != y.hi) return x.hi < y.hi;
      return x.s2 < y.s2;
    });
  });
  tp = phase(C, "sc_sort", tp);
  std::vector<RecDuo> duo;
  for (size_t g = 0; g + 1 < gb.size(); ++g)
    for (size_t i = gb[g]; i < gb[g + 1]; i += 2)
      duo.push_back(RecDuo{0, fast[i], i + 1 < gb[g + 1] ? fast[i + 1] : -1});
  const int64_t nd = (int64_t)duo.size();
  std::vector<int32_t> drows(nd);
  int64_t total_rows = 0;
  for (int64_t d = 0; d < nd; ++d) {
    const ScanTask &A = tk(duo[d].a);
    int lo = A.lo, hi = A.hi;
    if (duo[d].b >= 0) lo = std::min(lo, tk(duo[d].b).lo), hi = std::max(hi, tk(duo[d].b).hi);
    drows[d] = hi - lo;
    total_rows += hi - lo;
  }
  const int64_t resident = (int64_t)C.nsm * C.scan_blocks_per_sm * kScanThreads;
  const int64_t want_tiles = (int64_t)C.scan_tiles_per_thread * resident;
  const int K = warmup_rows(P, kScanW);
  int64_t chunk = INT32_MAX;
  if (nd < want_tiles && K != INT_MAX && total_rows > 0)
    chunk = std::min<int64_t>(INT32_MAX, std::max<int64_t>(4 * (int64_t)K, (total_rows + want_tiles - 1) / want_tiles));
  // longest duos first for the work queue: a counting sort by log-length (linear time); tile_begin follows that order
  std::vector<RecDuo> ord(nd);
  {
    std::vector<uint8_t> bk(nd);
    int64_t cnt[65] = {0};
    for (int64_t d = 0; d < nd; ++d) {
      const int b = std::min(63, (int)(4.0 * std::log2((double)std::max(1, drows[d]))));
      bk[d] = (uint8_t)(63 - b);
      cnt[bk[d] + 1]++;
    }
    for (int b = 0; b < 64; ++b) cnt[b + 1] += cnt[b];
    std::vector<int32_t> rows_of(nd);
    for (int64_t d = 0; d < nd; ++d) {
      const int64_t at = cnt[bk[d]]++;
      ord[at] = duo[d];
      rows_of[at] = drows[d];
    }
    int64_t tb = 0;
    for (int64_t d = 0; d < nd; ++d) {
      ord[d].tile_begin = tb;
      tb += chunk >= INT32_MAX ? 1 : std::max<int64_t>(1, (rows_of[d] + chunk - 1) / chunk);
    }
    duo.swap(ord);
    duo.push_back(RecDuo{tb, -1, -1});  // sentinel: total tile count
  }
  const int64_t ntiles = duo.back().tile_begin;
  duo.pop_back();
  tp = phase(C, "sc_tiles", tp);
  C.stats.ms_scan_prep += ms_since(t0);
  C.d_tasks.ensure(C, sizeof(ScanTask) * (S.size() - S.ns));
  h2d(C, C.d_tasks, S.tasks.data() + first, (size_t)n, (size_t)(first - S.ns));
  run_scan_round(C, S, P, first, n, duo.data(), nd, ntiles, (int32_t)chunk, K, generic);
  tp = phase(C, "sc_round", tp);
  C.stats.ms_scan += ms_since(t0);
  S.left.resize(S.size(), -1);
  S.right.resize(S.size(), -1);
}

// Number of windows of the drivers' loops (:462-480 for 1-gap, which stops once past the query end; :376-390 for
// 2-gap): start 0 always, then i*step while i*step + window <= n2, then the first i* with i*step + window > n2 unless
// the 1-gap loop already stopped at i*step > n2.
int32_t window_count(int32_t n2, const Params &P, bool one_gap) {
  const int32_t istar = (n2 - P.window < 0) ? 1 : (n2 - P.window) / P.step + 1;
  const bool pushed = !(one_gap && (int64_t)istar * P.step > n2);
  return istar + (pushed ? 1 : 0);
}

inline int32_t window_tw(int32_t n2, int32_t s2, const Params &P) { return (s2 + P.window) > n2 ? (n2 - s2) : P.window; }

// Level 0: every window of every pair against its whole reference.  On the fast path the device derives each tile
// from a per-pair table and compacts the windows whose maximum reached min_score (with their reverse re-scans);
// only those records reach the host.  Returns the level-0 algorithmic cells (every window is scanned).
int64_t scan_level0(Context &C, ScanState &S, const std::vector<PairIn> &pairs, const Params &P, bool one_gap) {
  auto t0 = Clock::now();
  const int64_t np = (int64_t)pairs.size();
  std::vector<int64_t> wstart(np + 1, 0);
  std::vector<int32_t> nwin(np), nfast(np);
  int64_t cells = 0;
  for (int64_t p = 0; p < np; ++p) {
    const int32_t n1 = pairs[p].n1, n2 = pairs[p].n2;
    nwin[p] = window_count(n2, P, one_gap);
    wstart[p + 1] = wstart[p] + nwin[p];
    // windows with tw > 0 are the prefix w * step < n2
    nfast[p] = n1 > 0 ? std::min<int32_t>(nwin[p], (n2 + P.step - 1) / P.step) : 0;
    // scan cells: n1 * sum of tw over scanned windows (full windows, then the short tail)
    const int32_t nfull = std::min<int32_t>(nfast[p], n2 >= P.window ? (n2 - P.window) / P.step + 1 : 0);
    int64_t tws = (int64_t)nfull * P.window;
    for (int32_t w = nfull; w < nfast[p]; ++w) tws += std::max(0, window_tw(n2, w * P.step, P));
    cells += (int64_t)n1 * tws;
  }
  const int64_t n0 = wstart[np];
  S.tasks.clear();
  S.pbeg.assign(np + 1, 0);
  if (!fast_scan_ok(P)) {
    if (C.l0_turn) {  // no level-0 kernel to order: let the later bins go
      std::lock_guard<std::mutex> lk(C.l0_turn->mu);
      C.l0_turn->next = std::max(C.l0_turn->next, C.bin + 1);
      C.l0_turn->cv.notify_all();
    }
    // generic level 0: every window is a task the replay walks (those below min_score are skipped there)
    S.tasks.reserve(n0);
    for (int64_t p = 0; p < np; ++p) {
      S.pbeg[p] = (int64_t)S.tasks.size();
      for (int32_t k = 0; k < nwin[p]; ++k) {
        ScanTask x{};
        x.pair = (int32_t)p;
        x.s2 = k * P.step;
        x.tw = window_tw(pairs[p].n2, x.s2, P);
        x.lo = 0;
        x.hi = pairs[p].n1;
        S.tasks.push_back(x);
      }
    }
    S.pbeg[np] = (int64_t)S.tasks.size();
    S.ns = 0;
    S.first_new = 0;
    C.stats.ms_scan_prep += ms_since(t0);
    compute_scan_tasks(C, S, P);
    S.ns = S.size();
    S.first_new = S.ns;
    S.left.assign(S.size(), -1);
    S.right.assign(S.size(), -1);
    return cells;
  }
  int64_t total_rows = 0, nduo = 0;
  for (int64_t p = 0; p < np; ++p) {
    nduo += (nfast[p] + 1) / 2;
    total_rows += (int64_t)((nfast[p] + 1) / 2) * pairs[p].n1;
  }
  const int64_t resident = (int64_t)C.nsm * C.scan_blocks_per_sm * kScanThreads;
  const int K = warmup_rows(P, kScanW);
  int64_t chunk = INT32_MAX;
  const int64_t want = (int64_t)C.scan_tiles_per_thread * resident;
  if (nduo < want && K != INT_MAX && total_rows > 0)
    chunk = std::min<int64_t>(INT32_MAX, std::max<int64_t>(4 * (int64_t)K, (total_rows + want - 1) / want));

  std::vector<int64_t> order(np);
  for (int64_t p = 0; p < np; ++p) order[p] = p;
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    return pairs[a].n1 != pairs[b].n1 ? pairs[a].n1 > pairs[b].n1 : a < b;
  });
  C.h_misc.ensure(sizeof(L0Pair) * np + sizeof(int64_t) * (np + 1) + sizeof(int2) * np + 64);
  L0Pair *tab = C.h_misc.as<L0Pair>();
  int64_t ntiles = 0;
  for (int64_t q = 0; q < np; ++q) {
    const int64_t p = order[q];
    L0Pair &e = tab[q];
    e.ref_base = C.seq_base[2 * p];
    e.qry_base = C.seq_base[2 * p + 1];
    e.tile_begin = ntiles;
    e.wstart = wstart[p];
    e.n1 = pairs[p].n1;
    e.n2 = pairs[p].n2;
    e.nfast = nfast[p];
    e.nch = chunk >= INT32_MAX ? 1 : (int32_t)std::max<int64_t>(1, (pairs[p].n1 + chunk - 1) / chunk);
    ntiles += (int64_t)((nfast[p] + 1) / 2) * e.nch;
  }
  auto tp = phase(C, "l0_table", t0);
  int64_t *wst = reinterpret_cast<int64_t *>(tab + np);
  int2 *plen = reinterpret_cast<int2 *>(wst + np + 1);
  for (int64_t p = 0; p <= np; ++p) wst[p] = wstart[p];
  for (int64_t p = 0; p < np; ++p) plen[p] = int2{pairs[p].n1, pairs[p].n2};
  C.stats.ms_scan_prep += ms_since(t0);
  auto tx = Clock::now();
  C.d_tiles.ensure(C, sizeof(L0Pair) * np + 64);
  C.d_scratch.ensure(C, sizeof(int64_t) * (np + 1) + sizeof(int2) * np + sizeof(int) * ((n0 + 255) / 256 + 8) + 64);
  C.d_keys.ensure(C, sizeof(unsigned long long) * std::max<int64_t>(n0, 1));
  C.d_counter.ensure(C, 64);
  C.d_tasks.ensure(C, sizeof(L0Rec) * std::max<int64_t>(n0, 1));
  int64_t *d_wst = C.d_scratch.as<int64_t>();
  int2 *d_plen = reinterpret_cast<int2 *>(d_wst + np + 1);
  int *d_blk = reinterpret_cast<int *>(d_plen + np);
  int *d_count = C.d_counter.as<int>() + 1;
  h2d(C, C.d_tiles, tab, (size_t)np);
  DCNS_CK(cudaMemcpyAsync(d_wst, wst, sizeof(int64_t) * (np + 1), cudaMemcpyHostToDevice, C.st));
  DCNS_CK(cudaMemcpyAsync(d_plen, plen, sizeof(int2) * np, cudaMemcpyHostToDevice, C.st));
  DCNS_CK(cudaMemsetAsync(C.d_keys.p, 0, sizeof(unsigned long long) * n0, C.st));
  DCNS_CK(cudaMemsetAsync(C.d_counter.p, 0, sizeof(int) * 2, C.st));
  L0Desc D{C.d_tiles.as<L0Pair>(), (int32_t)np, P.step, P.window, (int32_t)chunk, K, 0};
  // One thread per tile (not a persistent grid): blocks retire as they finish, so the short kernels of other lanes,
  // on higher-priority streams, are scheduled in between instead of waiting for the whole level-0 scan.
  const int64_t grid = std::max<int64_t>(1, (ntiles + kScanThreads - 1) / kScanThreads);
  cudaStream_t bulk = C.st_bulk;
  if (C.l0_turn) {  // a bin of a binned call: wait for the earlier bins' level-0 scans to be enqueued
    std::unique_lock<std::mutex> lk(C.l0_turn->mu);
    C.l0_turn->cv.wait(lk, [&] { return C.l0_turn->next >= C.bin || C.l0_turn->abort; });
    if (C.l0_turn->abort) throw Error(DCNS_ERR_DEVICE, "another bin of this call failed");
    bulk = C.bulk_shared;
  }
  DCNS_CK(cudaEventRecord(C.ev_bulk, C.st));
  DCNS_CK(cudaStreamWaitEvent(bulk, C.ev_bulk, 0));
  DCNS_CK(cudaEventRecord(C.ev0, bulk));
  launch_scan_l0(D, ntiles, C.arena, P, C.d_keys.as<unsigned long long>(), C.d_counter.as<int>(), grid, bulk);
  DCNS_CK(cudaEventRecord(C.ev1, bulk));
  DCNS_CK(cudaStreamWaitEvent(C.st, C.ev1, 0));
  if (C.l0_turn) {
    std::lock_guard<std::mutex> lk(C.l0_turn->mu);
    C.l0_turn->next = std::max(C.l0_turn->next, C.bin + 1);
    C.l0_turn->cv.notify_all();
  }
  C.stats.scan_launches += 1;
  C.stats.scan_rounds += 1;
  C.stats.kernel_launches += 1;
  launch_l0_select(C.d_keys.as<unsigned long long>(), n0, d_wst, d_plen, (int)np, C.seqbase_dev, C.arena, P, d_blk,
                   d_count, C.d_tasks.as<L0Rec>(), C.nsm, C.st);
  C.stats.kernel_launches += 4;
  int nsel = 0;
  DCNS_CK(cudaMemcpyAsync(&nsel, d_count, sizeof(int), cudaMemcpyDeviceToHost, C.st));
  tp = phase(C, "l0_launch", tp);
  sync(C);
  tp = phase(C, "l0_sync", tp);
  C.h_tasks.ensure(sizeof(L0Rec) * std::max(nsel, 1));
  L0Rec *rec = C.h_tasks.as<L0Rec>();
  d2h(C, rec, C.d_tasks, (size_t)nsel);
  sync(C);
  {
    float ms = 0;
    DCNS_CK(cudaEventElapsedTime(&ms, C.ev0, C.ev1));
    C.stats.ms_scan_kernel += ms;
  }
  C.stats.ms_scan_xfer += ms_since(tx);
  tp = phase(C, "l0_d2h", tp);
  auto tb = Clock::now();
  S.tasks.resize(nsel);
  // records are in task order: pair p's records start at the first record with task >= wstart[p]
  for (int64_t p = 0; p <= np; ++p) {
    int64_t lo = 0, hi = nsel;
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if (rec[mid].task < wstart[p])
        lo = mid + 1;
      else
        hi = mid;
    }
    S.pbeg[p] = lo;
  }
  parallel_for(np, [&](int64_t p) {
    for (int64_t k = S.pbeg[p]; k < S.pbeg[p + 1]; ++k) {
      const L0Rec &r = rec[k];
      ScanTask x{};
      x.pair = (int32_t)p;
      x.s2 = (int32_t)(r.task - wstart[p]) * P.step;
      x.tw = window_tw(pairs[p].n2, x.s2, P);
      x.lo = 0;
      x.hi = pairs[p].n1;
      x.score = r.score;
      x.end1 = r.end1;
      x.end2 = r.end2;
      x.start1 = r.start1;
      x.start2 = r.start2;
      S.tasks[k] = x;
    }
  });
  S.ns = nsel;
  S.first_new = nsel;
  S.left.assign(nsel, -1);
  S.right.assign(nsel, -1);
  phase(C, "l0_records", tp);
  C.stats.ms_scan_prep += ms_since(tb);
  C.stats.ms_scan += ms_since(t0);
  return cells;
}

inline Seed4 seed_of(const ScanTask &T) { return Seed4{T.start1, T.end1, T.start2, T.end2}; }

struct ReplayCtx {
  const ScanState &S;
  const Params &P;
  int mini;
  std::vector<std::pair<int32_t, int32_t>> req;  // (task, side) whose child must be created
  int64_t cells = 0, cells_rev = 0, visited = 0;
};

// getSeeds' recursive variant (:61-128): the local set gets the seed, then the left subtree's seeds in their set
// order, then the right subtree's.  Returns false when some child is not computed yet (requests it and continues).
bool subtree(ReplayCtx &R, int32_t t, SeedSet &out) {
  const ScanTask &T = R.S.task(t);
  R.visited++;
  R.cells += (int64_t)(T.hi - T.lo) * std::max(T.tw, 0);
  if (T.score < R.P.min_score) return true;
  const int lim = T.tw + R.P.window;
  R.cells_rev += (int64_t)std::min(T.end1 - T.lo + 1, lim) * std::min(T.end2 - T.s2 + 1, lim);
  out.insert(seed_of(T));
  bool ok = true;
  for (int side = 0; side < 2; ++side) {
    const bool cond = side == 0 ? (T.start1 - T.lo >= R.mini) : (T.hi - T.end1 - 1 >= R.mini);
    if (!cond) continue;
    const int32_t c = side == 0 ? R.S.left[t] : R.S.right[t];
    if (c < 0) {
      R.req.push_back({t, side});
      ok = false;
      continue;
    }
    SeedSet sub;
    ok &= subtree(R, c, sub);
    for (const Seed4 &s : sub) out.insert(s);
  }
  return ok;
}

// The set-gated window loop (:131-201 per window, :462-480 over windows) over the pair's level-0 windows with a seed.
bool replay_pair(ReplayCtx &R, int64_t p, SeedSet &global) {
  bool ok = true;
  for (int64_t t = R.S.pbeg[p]; t < R.S.pbeg[p + 1]; ++t) {
    const ScanTask &T = R.S.task(t);
    if (T.score < R.P.min_score) continue;
    const int lim = T.tw + R.P.window;
    R.cells_rev += (int64_t)std::min(T.end1 - T.lo + 1, lim) * std::min(T.end2 - T.s2 + 1, lim);
    const Seed4 sd = seed_of(T);
    if (global.find(sd) != global.end()) continue;
    global.insert(sd);
    for (int side = 0; side < 2; ++side) {
      const bool cond = side == 0 ? (T.start1 - T.lo >= R.mini) : (T.hi - T.end1 - 1 >= R.mini);
      if (!cond) continue;
      const int32_t c = side == 0 ? R.S.left[t] : R.S.right[t];
      if (c < 0) {
        R.req.push_back({(int32_t)t, side});
        ok = false;
        continue;
      }
      SeedSet sub;
      ok &= subtree(R, c, sub);
      for (const Seed4 &s : sub) global.insert(s);
    }
  }
  return ok;
}

void link_seeds(SeedSet &seeds) {  // :288-344
  std::vector<Seed4> cur(seeds.begin(), seeds.end());
  std::sort(cur.begin(), cur.end(), [](Seed4 a, Seed4 b) { return a.s1 < b.s1; });
  bool changed = true;
  while (changed) {
    changed = false;
    std::vector<Seed4> next;
    const int n = (int)cur.size();
    std::vector<uint8_t> used((size_t)n, 0);  // the reference's usedList
    for (int i = 0; i < n; ++i) {
      if (used[i]) continue;
      const Seed4 a = cur[i];
      bool merged = false;
      for (int j = i + 1; j < n; ++j) {
        if (used[j]) continue;
        const Seed4 b = cur[j];
        if (a.s2 <= b.s2 && a.e1 >= b.e1 && a.e2 >= b.e2) {
          used[j] = 1;
        } else if (a.s2 <= b.s2 && a.e1 <= b.e1 && a.e2 <= b.e2) {
          const int32_t d = b.s1 - a.s1;
          if (d == b.s2 - a.s2 && d == b.e1 - a.e1 && d == b.e2 - a.e2) {
            next.push_back(Seed4{a.s1, b.e1, a.s2, b.e2});
            used[i] = 1;
            used[j] = 1;
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

// Seed scan + replay + linking for every pair; returns the linked seed list of each pair in set order.
void scan_and_link(Context &C, const std::vector<PairIn> &pairs, const Params &P, bool one_gap,
                   std::vector<std::vector<Seed4>> &linked) {
  const int64_t np = (int64_t)pairs.size();
  ScanState S;
  int64_t cells = scan_level0(C, S, pairs, P, one_gap);
  int64_t level0_tasks = 0;
  for (int64_t p = 0; p < np; ++p) level0_tasks += window_count(pairs[p].n2, P, one_gap);
  const int mini = P.min_score / P.match;
  std::vector<SeedSet> sets(np);
  std::vector<uint8_t> done(np, 0);
  int64_t cells_rev = 0, visited_final = 0;
  for (int round = 0;; ++round) {
    if (round > 0) compute_scan_tasks(C, S, P);
    auto t0 = Clock::now();
    std::vector<std::vector<std::pair<int32_t, int32_t>>> reqs(np);
    std::vector<int64_t> pc(np, 0), pr(np, 0), pv(np, 0);
    std::vector<int64_t> todo;
    for (int64_t p = 0; p < np; ++p)
      if (!done[p]) todo.push_back(p);
    parallel_for((int64_t)todo.size(), [&](int64_t q) {
      const int64_t p = todo[q];
      ReplayCtx R{S, P, mini, {}, 0, 0, 0};
      SeedSet g;
      const bool ok = replay_pair(R, p, g);
      if (ok) {
        sets[p].swap(g);
        done[p] = 1;
        pc[p] = R.cells;
        pr[p] = R.cells_rev;
        pv[p] = R.visited;
      } else {
        reqs[p].swap(R.req);
      }
    });
    int64_t nreq = 0;
    for (int64_t p = 0; p < np; ++p) {
      cells += pc[p];
      cells_rev += pr[p];
      visited_final += pv[p];
      for (auto &rq : reqs[p]) {
        const int32_t t = rq.first;
        if ((rq.second == 0 ? S.left[t] : S.right[t]) >= 0) continue;
        const ScanTask P0 = S.task(t);
        ScanTask ch{};
        ch.pair = P0.pair;
        ch.s2 = P0.s2;
        ch.tw = P0.tw;
        if (rq.second == 0) {
          ch.lo = P0.lo;
          ch.hi = P0.start1;
        } else {
          ch.lo = P0.end1 + 1;
          ch.hi = P0.hi;
        }
        (rq.second == 0 ? S.left[t] : S.right[t]) = (int32_t)S.size();
        S.tasks.push_back(ch);
        ++nreq;
      }
      S.left.resize(S.size(), -1);
      S.right.resize(S.size(), -1);
    }
    C.stats.ms_replay += ms_since(t0);
    phase(C, "replay", t0);
    if (nreq == 0) break;
    if (round > 100000) throw Error(DCNS_ERR_DEVICE, "seed recursion did not converge");
  }
  C.stats.cells_scan += cells;
  C.stats.cells_scan_reverse += cells_rev;
  C.stats.tasks_scan += level0_tasks + visited_final;
  C.stats.tasks_scan_speculative += (S.size() - S.ns) - visited_final;
  auto t0 = Clock::now();
  linked.assign(np, {});
  parallel_for(
      np,
      [&](int64_t p) {
        link_seeds(sets[p]);
        linked[p].assign(sets[p].begin(), sets[p].end());
      },
      2);  // a pair of long sequences holds thousands of seeds: spread even a few pairs over the pool
  C.stats.ms_link += ms_since(t0);
}

// ------------------------------------------------------------------ 5. x-drop passes
// Sum over rows i = 1..rows of the band width max(0, min(i+w, n2) - max(i-w, 1) + 1), in closed form: the width is
// linear between the breakpoints where either clamp switches or the band empties.
int64_t band_cells(int rows, int w, int n2) {
  if (rows <= 0 || n2 <= 0) return 0;
  const int64_t W = w, N = n2, R = rows;
  auto width = [&](int64_t i) {
    return std::max<int64_t>(0, std::min(i + W, N) - std::max<int64_t>(i - W, 1) + 1);
  };
  int64_t bp[] = {1, W + 1, W + 2, N - W, N - W + 1, N + W, N + W + 1, R + 1};
  std::sort(std::begin(bp), std::end(bp));
  int64_t total = 0;
  for (int k = 0; k + 1 < 8; ++k) {
    const int64_t lo = std::max<int64_t>(bp[k], 1), hi = std::min<int64_t>(bp[k + 1], R + 1);  // [lo, hi)
    if (lo >= hi) continue;
    const int64_t cnt = hi - lo;
    total += cnt * (width(lo) + width(hi - 1)) / 2;
  }
  return total;
}

int wpr_of(int w) { return (2 * w + 1 + 7) / 8; }

// Device bytes the context's buffers hold, its lanes' included (buffers only grow, so after a call this is at least
// what the call used).
int64_t device_bytes(const Context &C) {
  int64_t b = (int64_t)C.used;
  for (const auto &L : C.lanes)
    if (L) b += (int64_t)L->used;
  return b;
}

// Runs the passes `subset` of X to completion in host-driven rounds (band restarts, traceback-slot growth), then
// their tracebacks when want_codes; X lives on the host between launches.  Traceback slots start at the whole pass
// (full_slots) or at min(n1, 1024) rows.  With want_codes, every finished pass's CIGAR is appended to *flat and
// (*hoff)[k] is its offset there (X[k].ncig words).
void run_xdrop_rounds(Context &C, std::vector<XTask> &X, const Params &P, bool want_codes, std::vector<uint32_t> *flat,
                      std::vector<int64_t> *hoff, const std::vector<int32_t> &subset, bool full_slots) {
  if (subset.empty()) return;
  const int64_t n = (int64_t)X.size();
  std::vector<int64_t> rows_cap(n, 0);
  for (int32_t k : subset) {
    X[k].want_codes = want_codes ? 1 : 0;
    X[k].status = 0;
    X[k].score = X[k].end1 = X[k].end2 = X[k].rows = 0;
    X[k].iii = X[k].jjj = X[k].ncig = 0;
    rows_cap[k] = full_slots ? (int64_t)X[k].n1 : std::min<int64_t>(X[k].n1, 1024);
  }
  std::vector<int32_t> pend(subset);
  C.d_x.ensure(C, sizeof(XTask) * n);
  while (!pend.empty()) {
    // Only the pending passes travel: gathered into a compact pinned array, indexed 0..m-1 on the device.
    const int64_t m = (int64_t)pend.size();
    int64_t words = 0;
    if (want_codes)
      for (int32_t k : pend) {
        X[k].tb_off = words;
        X[k].tb_cap = (int32_t)std::min<int64_t>(INT32_MAX, rows_cap[k] * wpr_of(X[k].w));
        words += X[k].tb_cap;
      }
    if (want_codes) C.d_tb.ensure(C, sizeof(uint32_t) * std::max<int64_t>(words, 1));
    auto tp = phase(C, "xd_prep0", Clock::now());
    C.h_misc.ensure(sizeof(XTask) * m);
    XTask *Xc = C.h_misc.as<XTask>();
    parallel_for((m + 4095) / 4096, [&](int64_t b) {
      for (int64_t q = b * 4096, e = std::min(m, q + 4096); q < e; ++q) Xc[q] = X[pend[q]];
    });
    h2d(C, C.d_x, Xc, (size_t)m);
    // passes known to be long (they outgrew their slot in the levels: full_slots) run as wavefronts up to w = 256
    std::vector<int32_t> g10, g20, gw, gwave;
    int maxw = 0;
    for (int64_t q = 0; q < m; ++q) {
      const int w = Xc[q].w;
      if (full_slots && w <= 256)
        gwave.push_back((int32_t)q);
      else if (w <= 10)
        g10.push_back((int32_t)q);
      else if (w <= 20)
        g20.push_back((int32_t)q);
      else
        gw.push_back((int32_t)q), maxw = std::max(maxw, w);
    }
    C.d_idx.ensure(C, sizeof(int32_t) * m);
    size_t off = 0;
    auto launch_group = [&](std::vector<int32_t> &g, int wcap) {
      if (g.empty()) return;
      h2d(C, C.d_idx, g.data(), g.size(), off);
      int32_t *scratch = nullptr;
      int64_t per = 0;
      if (wcap == 0) {  // warp per pass: M and F of 2w+2 cells each
        per = 2 * (2 * (int64_t)maxw + 2);
        C.d_scratch.ensure(C, sizeof(int32_t) * per * g.size());
        scratch = C.d_scratch.as<int32_t>();
      }
      launch_xdrop(C.d_x.as<XTask>(), C.d_idx.as<int>() + off, (int)g.size(), C.arena, P, C.d_tb.as<uint32_t>(),
                   wcap, scratch, per, C.st);
      C.stats.kernel_launches += 1;
      C.stats.xdrop_passes += (int64_t)g.size();
      off += g.size();
    };
    tp = phase(C, "xd_prep", tp);
    DCNS_CK(cudaEventRecord(C.ev0, C.st));
    launch_group(gwave, -1);
    launch_group(g10, 10);
    launch_group(g20, 20);
    launch_group(gw, 0);
    DCNS_CK(cudaEventRecord(C.ev1, C.st));
    d2h(C, Xc, C.d_x, (size_t)m);
    sync(C);
    {
      float ms = 0;
      DCNS_CK(cudaEventElapsedTime(&ms, C.ev0, C.ev1));
      C.stats.ms_xdrop_kernel += ms;
      C.stats.xdrop_rounds += 1;
    }
    tp = phase(C, "xd_launch_sync", tp);
    std::vector<int32_t> next, fin_c;  // fin_c: compact indices of finished passes
    parallel_for((m + 4095) / 4096, [&](int64_t b) {
      for (int64_t q = b * 4096, e = std::min(m, q + 4096); q < e; ++q) X[pend[q]] = Xc[q];
    });
    for (int64_t q = 0; q < m; ++q) {
      const int32_t k = pend[q];
      if (Xc[q].status == 1) {
        X[k].w *= 2;  // the reference restarts the whole pass with twice the band (:1272-1276)
        next.push_back(k);
      } else if (Xc[q].status == 2) {
        if (rows_cap[k] >= X[k].n1)  // a whole-pass slot did not fit its capacity field
          throw Error(DCNS_ERR_NOMEM, "x-drop traceback slot larger than 2^31 words");
        rows_cap[k] = X[k].n1;
        next.push_back(k);
      } else {
        fin_c.push_back((int32_t)q);
      }
    }
    tp = phase(C, "xd_collect", tp);
    if (want_codes && !fin_c.empty()) {
      int64_t cw = 0;
      for (int32_t q : fin_c) {
        Xc[q].cig_off = cw;
        Xc[q].cig_cap = Xc[q].end1 + Xc[q].end2 + 2;
        cw += Xc[q].cig_cap;
      }
      C.d_cig.ensure(C, sizeof(uint32_t) * std::max<int64_t>(cw, 1));
      h2d(C, C.d_x, Xc, (size_t)m);
      h2d(C, C.d_idx, fin_c.data(), fin_c.size());
      DCNS_CK(cudaEventRecord(C.ev1, C.st));
      launch_xdrop_traceback(C.d_x.as<XTask>(), C.d_idx.as<int>(), (int)fin_c.size(), C.d_tb.as<uint32_t>(), words,
                             C.d_cig.as<uint32_t>(), C.st);
      DCNS_CK(cudaEventRecord(C.ev2, C.st));
      C.stats.kernel_launches += 1;
      C.h_out.ensure(sizeof(uint32_t) * std::max<int64_t>(cw, 1));
      d2h(C, Xc, C.d_x, (size_t)m);
      d2h(C, C.h_out.as<uint32_t>(), C.d_cig, (size_t)cw);
      sync(C);
      {
        float ms = 0;
        DCNS_CK(cudaEventElapsedTime(&ms, C.ev1, C.ev2));
        C.stats.ms_xdrop_tb_kernel += ms;
      }
      tp = phase(C, "xd_tb_sync", tp);
      const uint32_t *hc = C.h_out.as<uint32_t>();
      int64_t total = (int64_t)flat->size();
      for (int32_t q : fin_c) {
        const int32_t k = pend[q];
        if (Xc[q].status == 3) throw Error(DCNS_ERR_DEVICE, "x-drop traceback exceeded its CIGAR slot");
        (*hoff)[k] = total;
        total += Xc[q].ncig;
      }
      flat->resize(total);
      uint32_t *fo = flat->data();
      const int64_t nf = (int64_t)fin_c.size();
      parallel_for((nf + 1023) / 1024, [&](int64_t b) {
        for (int64_t i = b * 1024, e = std::min(nf, i + 1024); i < e; ++i) {
          const int32_t q = fin_c[i], k = pend[q];
          X[k] = Xc[q];
          std::memcpy(fo + (*hoff)[k], hc + Xc[q].cig_off, sizeof(uint32_t) * Xc[q].ncig);
        }
      });
      tp = phase(C, "xd_tb_host", tp);
    }
    pend.swap(next);
  }
}

// Runs every pass of X to completion and, with want_codes, its traceback.  All passes start with the same band w0;
// the level kernels for bands w0, 2w0, 4w0, ... (up to a band that covers every pass, where no restart can occur)
// are enqueued at once with their work lists in device memory, then one synchronisation.  Passes whose traceback
// slot was too small (or the arena full) finish in host-driven rounds with whole-pass slots.  With want_codes,
// every pass's CIGAR is in *flat at (*hoff)[k] (X[k].ncig words), in task order.
void run_xdrop(Context &C, std::vector<XTask> &X, const Params &P, bool want_codes, std::vector<uint32_t> *flat,
               std::vector<int64_t> *hoff) {
  if (X.empty()) return;
  auto t0 = Clock::now();
  const int64_t n = (int64_t)X.size();
  if (flat) flat->clear();
  if (hoff) hoff->assign(n, -1);
  const int w0 = X[0].w;
  int64_t maxdim = 1, max_n1 = 1, tb_words = 1 << 20, cig_words = 1;
  bool uniform = w0 >= 1;
  for (int64_t k = 0; k < n; ++k) {
    XTask &T = X[k];
    uniform &= T.w == w0;
    T.want_codes = want_codes ? 1 : 0;
    T.status = 0;
    T.score = T.end1 = T.end2 = T.rows = 0;
    T.iii = T.jjj = T.ncig = 0;
    maxdim = std::max<int64_t>(maxdim, std::max(T.n1, T.n2));
    max_n1 = std::max<int64_t>(max_n1, T.n1);
    if (want_codes) cig_words += (int64_t)std::max(T.n1, 0) + std::max(T.n2, 0) + 2;
  }
  // Traceback slots of min(n1, slot_rows) rows, the arena sized for three slots per pass (a band restart takes a new
  // slot of twice the width).  A slot is reserved for the pass's bound n1, not for the rows it will use, so slot_rows
  // stays at 1,024-2,048: the longest pass up to 2,048 rows when that arena fits a quarter of the free device budget
  // (passes longer than their slot are retried with whole-pass slots).
  int slot_rows = 1024;
  if (want_codes) {
    auto words_for = [&](int64_t rows) {
      int64_t wsum = 1 << 20;
      for (int64_t k = 0; k < n; ++k) wsum += 3 * std::min<int64_t>(X[k].n1, rows) * wpr_of(w0);
      return wsum;
    };
    const int64_t room = (int64_t)((C.budget > C.used ? C.budget - C.used : 0) / 4);
    const int64_t want = std::min<int64_t>(max_n1, 2048);
    if (want > 1024 && (int64_t)sizeof(uint32_t) * words_for(want) <= room) slot_rows = (int)want;
    tb_words = words_for(slot_rows);
  }
  auto tp = phase(C, "xc_setup", t0);
  if (!uniform || n >= INT32_MAX / 4) {
    std::vector<int32_t> all(n);
    for (int64_t k = 0; k < n; ++k) all[k] = (int32_t)k;
    run_xdrop_rounds(C, X, P, want_codes, flat, hoff, all, false);
  } else {
    int nlev = 1;
    while (((int64_t)w0 << (nlev - 1)) < maxdim) ++nlev;
    // per level: warps of the wide-band kernel and their scratch (2 x (2w + 2) ints per warp, 512 MB at most)
    std::vector<int> warps(nlev, 0);
    std::vector<int64_t> per_warp(nlev, 0);
    int64_t scratch_ints = 1;
    for (int L = 0; L < nlev; ++L) {
      const int64_t w = (int64_t)w0 << L;
      if (w <= C.xdrop_warp_from || w <= std::min(C.xdrop_wave_max_w, 256)) continue;  // register band / wavefront
      per_warp[L] = 2 * (2 * w + 2);
      const int64_t cap = std::max<int64_t>(32, ((int64_t)512 << 20) / (4 * per_warp[L]));
      warps[L] = (int)(std::min<int64_t>({n, cap, (int64_t)C.nsm * 64}) + 3) / 4 * 4;  // whole blocks of 4 warps
      scratch_ints = std::max(scratch_ints, warps[L] * per_warp[L]);
    }
    // hand-off slots of the register-band levels (one level at a time: the resume kernel empties them before the
    // next level starts)
    const bool any_flat = C.xdrop_flat && C.xdrop_handoff > 0 && std::min(C.xdrop_warp_from, 20) >= w0;
    const int spill_cap = any_flat ? (int)std::min<int64_t>(n, 1 << 16) : 0;
    C.d_x.ensure(C, sizeof(XTask) * n);
    C.d_idx.ensure(C, sizeof(int32_t) * (3 * n + spill_cap + 4 + 2 * nlev + 64));
    if (spill_cap > 0) C.d_spill.ensure(C, sizeof(int32_t) * (size_t)spill_cap * kXdropSpillInts);
    C.d_counter.ensure(C, 64);
    if (want_codes) {
      C.d_tb.ensure(C, sizeof(uint32_t) * tb_words);
      C.d_cig.ensure(C, sizeof(uint32_t) * 2 * cig_words);  // slots, then the packed CIGARs
    }
    if (scratch_ints > 1) C.d_scratch.ensure(C, sizeof(int32_t) * scratch_ints);
    int *lists = C.d_idx.as<int>();
    // [0], [1]: the two work-list counts, [2]: retry count, [4 + L]: level L's fetch, [4 + nlev + L]: its hand-offs
    int *cnt = lists + 3 * n;
    int *long_list = cnt + 4 + 2 * nlev + 64;
    unsigned long long *cur = C.d_counter.as<unsigned long long>();  // [0]: traceback arena, [1]: CIGAR arena
    h2d(C, C.d_x, X.data(), (size_t)n);
    DCNS_CK(cudaMemsetAsync(cnt, 0, sizeof(int) * (4 + 2 * nlev), C.st));
    DCNS_CK(cudaMemsetAsync(cur, 0, sizeof(unsigned long long) * 2, C.st));
    launch_xdrop_iota(lists, (int)n, cnt, C.st);
    DCNS_CK(cudaEventRecord(C.ev0, C.st));
    int in = 0, launched = 0;
    for (int L = 0; L < nlev; ++L) {
      const int out = 1 - in;
      DCNS_CK(cudaMemsetAsync(cnt + out, 0, sizeof(int), C.st));
      const XHandoff H{long_list, cnt + 4 + nlev + L, C.d_spill.as<int32_t>(), spill_cap, C.xdrop_handoff,
                       C.xdrop_resume_lanes};
      launched += launch_xdrop_level(C.d_x.as<XTask>(), lists + in * n, cnt + in, lists + out * n, cnt + out,
                                     lists + 2 * n, cnt + 2, cur, want_codes ? tb_words : 0, slot_rows, cnt + 4 + L, H,
                                     C.arena, P, C.d_tb.as<uint32_t>(), w0 << L, (int)n, C.nsm,
                                     C.d_scratch.as<int32_t>(), per_warp[L], warps[L], C.xdrop_warp_from,
                                     C.xdrop_wave_max_w, C.xdrop_flat, C.xdrop_group_from, want_codes, C.st);
      in = out;
    }
    DCNS_CK(cudaEventRecord(C.ev1, C.st));
    if (want_codes) {
      launch_xdrop_traceback_all(C.d_x.as<XTask>(), (int)n, C.d_tb.as<uint32_t>(), tb_words, C.d_cig.as<uint32_t>(),
                                 cur + 1, C.st);
      launch_xdrop_cigar_pack(C.d_x.as<XTask>(), (int)n, C.d_cig.as<uint32_t>(), C.d_cig.as<uint32_t>() + cig_words,
                              cur + 1, C.st);
      DCNS_CK(cudaEventRecord(C.ev2, C.st));
    }
    C.stats.kernel_launches += launched + 1 + (want_codes ? 3 : 0);
    C.stats.xdrop_rounds += 1;
    C.h_misc.ensure(sizeof(int32_t) * (n + 8) + 64);
    int32_t *hret = C.h_misc.as<int32_t>();  // [0]: leftover count, [1]: retry count, [8..]: retry list
    unsigned long long hcur[2] = {0, 0};
    d2h(C, X.data(), C.d_x, (size_t)n);
    DCNS_CK(cudaMemcpyAsync(hret, cnt + in, sizeof(int), cudaMemcpyDeviceToHost, C.st));
    DCNS_CK(cudaMemcpyAsync(hret + 1, cnt + 2, sizeof(int), cudaMemcpyDeviceToHost, C.st));
    DCNS_CK(cudaMemcpyAsync(hret + 8, lists + 2 * n, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, C.st));
    DCNS_CK(cudaMemcpyAsync(hcur, cur, sizeof(hcur), cudaMemcpyDeviceToHost, C.st));
    tp = phase(C, "xc_enqueue", tp);
    sync(C);
    tp = phase(C, "xc_sync", tp);
    {
      float ms = 0;
      DCNS_CK(cudaEventElapsedTime(&ms, C.ev0, C.ev1));
      C.stats.ms_xdrop_kernel += ms;
      if (want_codes) {
        DCNS_CK(cudaEventElapsedTime(&ms, C.ev1, C.ev2));
        C.stats.ms_xdrop_tb_kernel += ms;
      }
    }
    if (hret[0] != 0) throw Error(DCNS_ERR_DEVICE, "x-drop band restarts did not converge");
    std::vector<int32_t> retry(hret + 8, hret + 8 + hret[1]);
    std::sort(retry.begin(), retry.end());
    if (want_codes) {
      const int64_t cw = (int64_t)hcur[1];  // words of the packed CIGARs
      flat->resize(cw);
      if (cw > 0) {
        DCNS_CK(cudaMemcpyAsync(flat->data(), C.d_cig.as<uint32_t>() + cig_words, sizeof(uint32_t) * cw,
                                cudaMemcpyDeviceToHost, C.st));
        sync(C);
      }
      for (int64_t k = 0; k < n; ++k) {
        if (X[k].status == 3) throw Error(DCNS_ERR_DEVICE, "x-drop traceback exceeded its CIGAR slot");
        if (X[k].status == 0) (*hoff)[k] = X[k].cig_dense;
      }
    }
    for (int64_t k = 0; k < n; ++k) {
      int lev = 0;
      while ((w0 << lev) < X[k].w) ++lev;
      C.stats.xdrop_passes += lev + 1;
    }
    tp = phase(C, "xc_cigars", tp);
    if (C.trace) std::fprintf(stderr, "[dcns trace] x-drop chain: %lld passes, %d levels, %zu retries\n", (long long)n, nlev, retry.size());
    run_xdrop_rounds(C, X, P, want_codes, flat, hoff, retry, true);
    tp = phase(C, "xc_retry", tp);
  }
  for (int64_t k = 0; k < n; ++k) {
    const int64_t cells = band_cells(X[k].rows, X[k].w, X[k].n2);
    C.stats.cells_xdrop += cells;
    if (want_codes) C.stats.bytes_codes_xdrop += (cells + 1) / 2;
  }
  C.stats.ms_xdrop += ms_since(t0);
}

inline void evalue(const Params &P, double L1, double L2, int32_t score, double &e, double &p) {
  e = P.kvalue * L1 * L2 * exp(-1.0 * P.lambda * double(score));
  p = 1.0 - exp(-1.0 * e);
}

struct XSeedOut {
  bool ok;
  int32_t start1, end1, start2, end2, score;
  int64_t cig_off;  // into the stage's flat CIGAR buffer
  int32_t cig_len;
};

// x_extend_seed (:205-285) for every linked seed of every pair: forward pass, reverse pass (with codes when
// want_cigar), then the coordinate bookkeeping of the reference.
void extend_seeds(Context &C, const std::vector<PairIn> &pairs, const Params &P,
                  const std::vector<std::vector<Seed4>> &linked, bool want_cigar,
                  std::vector<std::vector<XSeedOut>> &res, std::vector<uint32_t> &cig_flat) {
  const int64_t np = (int64_t)pairs.size();
  res.assign(np, {});
  std::vector<XTask> F;
  std::vector<std::pair<int32_t, int32_t>> owner;
  for (int64_t p = 0; p < np; ++p) {
    res[p].resize(linked[p].size());
    for (size_t s = 0; s < linked[p].size(); ++s) {
      const Seed4 &sd = linked[p][s];
      XTask x{};
      x.base1 = C.seq_base[2 * p];
      x.base2 = C.seq_base[2 * p + 1];
      x.a1 = sd.s1 + 1;  // the extension starts one base after the seed start (:492-495)
      x.a2 = sd.s2 + 1;
      x.n1 = pairs[p].n1 - x.a1;
      x.n2 = pairs[p].n2 - x.a2;
      x.dir = 0;
      x.w = P.w;
      F.push_back(x);
      owner.push_back({(int32_t)p, (int32_t)s});
    }
  }
  C.stats.seeds += (int64_t)F.size();
  auto tp = phase(C, "xs_build_fwd", Clock::now());
  run_xdrop(C, F, P, false, nullptr, nullptr);
  tp = phase(C, "xs_run_fwd", tp);
  const int64_t nf = (int64_t)F.size();
  std::vector<int32_t> rslot(nf + 1, 0);  // reverse task of forward pass k (exclusive prefix over kept passes)
  parallel_for((nf + 4095) / 4096, [&](int64_t b) {
    for (int64_t k = b * 4096, e = std::min(nf, k + 4096); k < e; ++k) {
      const XTask &f = F[k];
      XSeedOut &o = res[owner[k].first][owner[k].second];
      o.ok = false;
      o.score = f.score;
      o.cig_off = 0;
      o.cig_len = 0;
      rslot[k + 1] = (f.end1 - 1 < 0 || f.end2 - 1 < 0) ? 0 : 1;  // p = 100 otherwise
    }
  });
  for (int64_t k = 0; k < nf; ++k) rslot[k + 1] += rslot[k];
  std::vector<XTask> R(rslot[nf]);
  std::vector<int32_t> rmap(rslot[nf]);
  parallel_for((nf + 4095) / 4096, [&](int64_t b) {
    for (int64_t k = b * 4096, e = std::min(nf, k + 4096); k < e; ++k) {
      if (rslot[k + 1] == rslot[k]) continue;
      const XTask &f = F[k];
      const int32_t b1 = f.a1 + f.end1 - 1, b2 = f.a2 + f.end2 - 1;
      XTask r{};
      r.base1 = f.base1;
      r.base2 = f.base2;
      r.a1 = b1;
      r.a2 = b2;
      r.n1 = b1 + 1;
      r.n2 = b2 + 1;
      r.dir = 1;
      r.w = P.w;
      R[rslot[k]] = r;
      rmap[rslot[k]] = (int32_t)k;
    }
  });
  std::vector<int64_t> hoff;
  tp = phase(C, "xs_build_rev", tp);
  run_xdrop(C, R, P, want_cigar, want_cigar ? &cig_flat : nullptr, want_cigar ? &hoff : nullptr);
  tp = phase(C, "xs_run_rev", tp);
  for (size_t q = 0; q < R.size(); ++q) {
    const XTask &r = R[q];
    const XTask &f = F[rmap[q]];
    XSeedOut &o = res[owner[rmap[q]].first][owner[rmap[q]].second];
    o.score = r.score;
    if (want_cigar) o.cig_off = hoff[q], o.cig_len = r.ncig;
    if (r.end1 - 1 < 0 || r.end2 - 1 < 0) continue;
    const int32_t b1 = f.a1 + f.end1 - 1, b2 = f.a2 + f.end2 - 1;
    o.ok = true;
    o.end1 = b1;
    o.end2 = b2;
    o.start1 = b1 - (r.end1 - 1);
    o.start2 = b2 - (r.end2 - 1);
    if (want_cigar) {
      o.end1 -= r.iii;
      o.end2 -= r.jjj;
    }
  }
}

// ------------------------------------------------------------------ 2-gap stage (:532-616)
int64_t sg_band_cells(int rows, int w, int n2) { return band_cells(rows, w, n2); }


// Runs 2-piece semi-global DPs; with codes, bounded by the memory budget per launch (admission by traceback bytes).
void run_semiglobal(Context &C, std::vector<SgTask> &G, const Params &P, bool want_codes,
                    std::vector<std::vector<uint32_t>> *cigars, const SgWeights *W = nullptr) {
  if (G.empty()) return;
  auto t0 = Clock::now();
  const int64_t n = (int64_t)G.size();
  if (cigars) cigars->assign(n, {});
  // device work split into batches whose direction-code stores fit a fraction of the budget
  const size_t free_budget = C.budget > C.used ? C.budget - C.used : 0;
  const int64_t cap_bytes = std::max<int64_t>((int64_t)(free_budget / 2), (int64_t)64 << 20);
  int64_t k0 = 0;
  C.d_sg.ensure(C, sizeof(SgTask) * n);
  // the stripe-flow form (unweighted DPs): per DP also its boundary row and flow state, per stripe a progress flag
  const bool flow = W == nullptr && C.sg_flow;
  auto flow_bytes = [&](const SgTask &g) -> int64_t {
    return flow ? (int64_t)sizeof(SgRec) * (std::max(g.n2, 0) + 2) + (int64_t)sizeof(SgFlowDP) + 8 +
                      12 * sg_flow_units(g.n1, g.n2, P.bandwidth)
                : 0;
  };
  while (k0 < n) {
    int64_t bytes = 0, extra = 0, k1 = k0;
    while (k1 < n) {
      const int64_t b =
          !want_codes ? 0 : W ? sgw_tb_bytes(G[k1].n1, G[k1].n2, P.bandwidth) : sg_tb_bytes(G[k1].n1, G[k1].n2, P.bandwidth);
      const int64_t e = flow_bytes(G[k1]);
      if (k1 > k0 && bytes + extra + b + e > cap_bytes) break;
      G[k1].tb_off = bytes;
      G[k1].tb_bytes = b;
      G[k1].want_codes = want_codes ? 1 : 0;
      bytes += b;
      extra += e;
      ++k1;
    }
    const int64_t m = k1 - k0;
    if (want_codes) C.d_sgtb.ensure(C, (size_t)std::max<int64_t>(bytes, 1));
    // unweighted: the stripe flow (or, with sg_flow off, one CTA per DP); weighted: one warp per DP, 16 warps per SM.
    // CTA shape of the unweighted CTA kernel: many DPs run two warps each (short DPs stop within a few stripes, and
    // more of them run at once); few DPs keep eight warps each for the stripes of long DPs
    const int nw = C.sg_warps > 0 ? C.sg_warps : (m >= (int64_t)C.nsm * 8 ? 2 : kSgNW);
    const int grid = (int)std::min<int64_t>(m, W ? (int64_t)C.nsm * 16 : (int64_t)C.nsm * sg_ctas_per_sm(nw));
    int maxn2 = 1;
    for (int64_t q = k0; q < k1; ++q) maxn2 = std::max(maxn2, G[q].n2);
    C.d_counter.ensure(C, 64);
    DCNS_CK(cudaMemsetAsync(C.d_counter.p, 0, sizeof(int), C.st));
    // largest DPs first: the work queue then finishes with the small ones
    std::vector<int32_t> idx(m);
    for (int64_t q = 0; q < m; ++q) idx[q] = (int32_t)(k0 + q);
    std::sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) {
      const int64_t ca = (int64_t)G[a].n1 * std::min(G[a].n2, 2 * P.bandwidth + 1);
      const int64_t cb = (int64_t)G[b].n1 * std::min(G[b].n2, 2 * P.bandwidth + 1);
      return ca != cb ? ca > cb : a < b;
    });
    C.d_idx.ensure(C, sizeof(int32_t) * m);
    h2d(C, C.d_idx, idx.data(), (size_t)m);
    h2d(C, C.d_sg, G.data(), (size_t)n);
    SgFlow F{};
    if (flow) {
      // units (stripes) and boundary rows in queue order; flow state in one buffer:
      // unit_begin | dps | order | prog | counters
      std::vector<int64_t> ub((size_t)m);
      std::vector<int32_t> nst((size_t)m);
      std::vector<SgFlowDP> dps((size_t)m);
      int64_t units = 0, brows = 0;
      for (int64_t q = 0; q < m; ++q) {
        const SgTask &g = G[idx[q]];
        ub[q] = units;
        nst[q] = (int32_t)sg_flow_units(g.n1, g.n2, P.bandwidth);
        units += nst[q];
        dps[q] = SgFlowDP{brows, 0, 0, 0, -1, -1, 0, kOut, kOut};
        brows += std::max(g.n2, 0) + 2;
      }
      // hand-out order: stripe-major within groups of consecutive DPs holding at least eight grid-fulls of units;
      // inside a group the DPs go by stripe count, most first, so the DPs that have a stripe s form a prefix
      const int64_t group_units = 8 * sg_flow_grid_warps(C.nsm, C.sg_flow_blocks);
      std::vector<int2> order((size_t)units);
      {
        int64_t u = 0;
        std::vector<int32_t> perm;
        for (int64_t g0 = 0; g0 < m;) {
          int64_t g1 = g0, gu = 0;
          while (g1 < m && (g1 == g0 || gu < group_units)) gu += nst[g1++];
          perm.resize((size_t)(g1 - g0));
          for (int64_t k = g0; k < g1; ++k) perm[k - g0] = (int32_t)k;
          std::stable_sort(perm.begin(), perm.end(), [&](int32_t a, int32_t b) { return nst[a] > nst[b]; });
          for (int32_t s = 0, cnt = (int32_t)perm.size(); cnt > 0; ++s) {
            while (cnt > 0 && nst[perm[cnt - 1]] <= s) --cnt;
            for (int32_t k = 0; k < cnt; ++k) order[u++] = int2{perm[k], s};
          }
          g0 = g1;
        }
        if (u != units) throw Error(DCNS_ERR_DEVICE, "semi-global stripe order: unit count mismatch");
      }
      auto al = [](int64_t b) { return (b + 255) / 256 * 256; };
      const int64_t o_dps = al(8 * m), o_ord = o_dps + al((int64_t)sizeof(SgFlowDP) * m);
      const int64_t o_prog = o_ord + al(8 * units), o_cnt = o_prog + al(4 * units), total = o_cnt + 256;
      C.d_flow.ensure(C, (size_t)total);
      C.d_bnd.ensure(C, (size_t)(sizeof(SgRec) * brows));
      char *base = static_cast<char *>(C.d_flow.p);
      DCNS_CK(cudaMemcpyAsync(base, ub.data(), 8 * m, cudaMemcpyHostToDevice, C.st));
      DCNS_CK(cudaMemcpyAsync(base + o_dps, dps.data(), sizeof(SgFlowDP) * m, cudaMemcpyHostToDevice, C.st));
      DCNS_CK(cudaMemcpyAsync(base + o_ord, order.data(), 8 * units, cudaMemcpyHostToDevice, C.st));
      DCNS_CK(cudaMemsetAsync(base + o_prog, 0, (size_t)(total - o_prog), C.st));
      F.tasks = C.d_sg.as<SgTask>();
      F.idx = C.d_idx.as<int>();
      F.unit_begin = reinterpret_cast<const int64_t *>(base);
      F.dps = reinterpret_cast<SgFlowDP *>(base + o_dps);
      F.order = reinterpret_cast<const int2 *>(base + o_ord);
      F.bnd = C.d_bnd.as<SgRec>();
      F.prog = reinterpret_cast<int *>(base + o_prog);
      F.unit_counter = reinterpret_cast<unsigned long long *>(base + o_cnt);
      F.err = reinterpret_cast<int *>(base + o_cnt + 8);
      F.total_units = units;
      F.n = (int)m;
    } else {
      C.d_bnd.ensure(C, (size_t)(W ? sgw_bnd_bytes((grid + 3) / 4 * 4, maxn2) : sg_bnd_bytes(grid, maxn2, nw)));
    }
    DCNS_CK(cudaEventRecord(C.ev0, C.st));
    if (W)
      launch_semiglobal_weighted(C.d_sg.as<SgTask>(), C.d_idx.as<int>(), (int)m, C.arena, P, *W,
                                 C.d_sgtb.as<uint8_t>(), C.d_bnd.p, maxn2, C.d_counter.as<int>(), grid, C.st);
    else if (flow)
      launch_semiglobal_flow(F, C.arena, P, C.d_sgtb.as<uint8_t>(), want_codes, C.nsm, C.sg_flow_blocks, C.st);
    else
      launch_semiglobal(C.d_sg.as<SgTask>(), C.d_idx.as<int>(), (int)m, C.arena, P, C.d_sgtb.as<uint8_t>(),
                        C.d_bnd.p, maxn2, C.d_counter.as<int>(), grid, nw, C.st);
    DCNS_CK(cudaEventRecord(C.ev1, C.st));
    int flow_err = 0;
    if (flow) DCNS_CK(cudaMemcpyAsync(&flow_err, F.err, sizeof(int), cudaMemcpyDeviceToHost, C.st));
    C.stats.kernel_launches += 1;
    C.stats.semiglobal_dps += m;
    auto kernel_ms = [&](cudaEvent_t a, cudaEvent_t b) {
      float ms = 0;
      DCNS_CK(cudaEventElapsedTime(&ms, a, b));
      return (double)ms;
    };
    auto check_flow = [&]() {
      if (flow_err != 0) throw Error(DCNS_ERR_DEVICE, "semi-global stripe flow: a wait ran out of iterations");
    };
    if (want_codes) {
      d2h(C, G.data(), C.d_sg, (size_t)n);
      sync(C);
      check_flow();
      C.stats.ms_sg_kernel += kernel_ms(C.ev0, C.ev1);
      int64_t cw = 0;
      for (int64_t q = k0; q < k1; ++q) {
        G[q].cig_off = cw;
        G[q].cig_cap = std::max(G[q].end1, 0) + std::max(G[q].end2, 0) + 2;
        cw += G[q].cig_cap;
      }
      C.d_cig.ensure(C, sizeof(uint32_t) * std::max<int64_t>(cw, 1));
      h2d(C, C.d_sg, G.data(), (size_t)n);
      DCNS_CK(cudaEventRecord(C.ev0, C.st));
      launch_sg_traceback(C.d_sg.as<SgTask>(), C.d_idx.as<int>(), (int)m, P.bandwidth, C.d_sgtb.as<uint8_t>(), bytes,
                          C.d_cig.as<uint32_t>(), C.st, W != nullptr);
      DCNS_CK(cudaEventRecord(C.ev1, C.st));
      C.stats.kernel_launches += 1;
      C.h_out.ensure(sizeof(uint32_t) * std::max<int64_t>(cw, 1));
      d2h(C, G.data(), C.d_sg, (size_t)n);
      d2h(C, C.h_out.as<uint32_t>(), C.d_cig, (size_t)cw);
      sync(C);
      C.stats.ms_sg_tb_kernel += kernel_ms(C.ev0, C.ev1);
      const uint32_t *hc = C.h_out.as<uint32_t>();
      for (int64_t q = k0; q < k1; ++q) {
        if (G[q].status != 0) throw Error(DCNS_ERR_DEVICE, "semi-global traceback exceeded its CIGAR slot");
        (*cigars)[q].assign(hc + G[q].cig_off, hc + G[q].cig_off + G[q].ncig);
      }
    } else {
      d2h(C, G.data(), C.d_sg, (size_t)n);
      sync(C);
      check_flow();
      C.stats.ms_sg_kernel += kernel_ms(C.ev0, C.ev1);
    }
    k0 = k1;
  }
  for (auto &g : G) {
    const int64_t cells = sg_band_cells(g.rows, P.bandwidth, g.n2);
    C.stats.cells_semiglobal += cells;
    if (want_codes) C.stats.bytes_codes_sg += cells;
  }
  C.stats.ms_semiglobal += ms_since(t0);
}

void two_gap_stage(Context &C, const std::vector<PairIn> &pairs, const Params &P,
                   const std::vector<std::vector<Seed4>> &xs, std::vector<std::vector<FragOut>> &out) {
  const int64_t np = (int64_t)pairs.size();
  // reverse 2-piece from every x-seed end (no codes)
  std::vector<SgTask> Rv;
  std::vector<std::pair<int32_t, int32_t>> own;
  for (int64_t p = 0; p < np; ++p)
    for (size_t s = 0; s < xs[p].size(); ++s) {
      SgTask g{};
      g.base1 = C.seq_base[2 * p];
      g.base2 = C.seq_base[2 * p + 1];
      g.a1 = xs[p][s].e1;
      g.a2 = xs[p][s].e2;
      g.n1 = 1 + xs[p][s].e1;
      g.n2 = 1 + xs[p][s].e2;
      g.dir = 1;
      Rv.push_back(g);
      own.push_back({(int32_t)p, (int32_t)s});
    }
  run_semiglobal(C, Rv, P, false, nullptr);
  // start gate per pair in x-seed order (StartAlignment set), then forward passes with codes
  std::vector<SgTask> Fw;
  std::vector<int32_t> fw_pair;
  std::vector<std::pair<int32_t, int32_t>> fw_start;
  {
    size_t k = 0;
    for (int64_t p = 0; p < np; ++p) {
      std::set<std::pair<int32_t, int32_t>> starts;
      for (size_t s = 0; s < xs[p].size(); ++s, ++k) {
        const SgTask &r = Rv[k];
        const int32_t s1 = xs[p][s].e1 - (r.end1 - 1), s2 = xs[p][s].e2 - (r.end2 - 1);
        if (!starts.insert({s1, s2}).second) continue;
        SgTask g{};
        g.base1 = C.seq_base[2 * p];
        g.base2 = C.seq_base[2 * p + 1];
        g.a1 = s1;
        g.a2 = s2;
        g.n1 = pairs[p].n1 - s1;
        g.n2 = pairs[p].n2 - s2;
        g.dir = 0;
        Fw.push_back(g);
        fw_pair.push_back((int32_t)p);
        fw_start.push_back({s1, s2});
      }
    }
  }
  std::vector<std::vector<uint32_t>> cg;
  run_semiglobal(C, Fw, P, true, &cg);
  out.assign(np, {});
  for (size_t q = 0; q < Fw.size(); ++q) {
    const int32_t p = fw_pair[q];
    const SgTask &g = Fw[q];
    const int32_t s1 = fw_start[q].first, s2 = fw_start[q].second;
    const int32_t e1z = g.end1 - 1, e2z = g.end2 - 1;  // 0-based as returned by SemiGlobal
    if (!(cg[q].size() > 0 && e1z > 0 && e2z > 0)) continue;
    const int64_t e1 = (int64_t)e1z + s1, e2 = (int64_t)e2z + s2;
    std::vector<FragOut> &fr = out[p];
    int toRemove = -1;
    bool found = false;
    for (int i = 0; i < (int)fr.size(); ++i)
      if (fr[i].e1 == e1 + 1 && fr[i].e2 == e2 + 1) {
        found = true;
        if (s1 + 1 < fr[i].s1 && s2 + 1 < fr[i].s2) toRemove = i;
      }
    if (found && toRemove < 0) continue;
    FragOut f;
    f.s1 = s1 + 1;
    f.e1 = e1 + 1;
    f.s2 = s2 + 1;
    f.e2 = e2 + 1;
    f.score = (int64_t)(uint32_t)g.score;
    f.cigar = cg[q];
    evalue(P, double(pairs[p].n1), double(pairs[p].n2), g.score, f.e, f.p);
    if (toRemove >= 0)
      fr[toRemove] = std::move(f);
    else
      fr.push_back(std::move(f));
  }
}

// The weighted drivers (findSimilarFragmentsForPairedSequence4.cpp:784-881, pieces 1; :883-975, pieces 2): per
// x-seed a weighted reverse DP from its end, the StartAlignment gate, a weighted forward DP with CIGAR.  The 1-piece
// driver keeps every forward result; the 2-piece one needs a CIGAR and positive ends.
void weighted_stage(Context &C, const std::vector<PairIn> &pairs, const Params &P,
                    const std::vector<std::vector<Seed4>> &xs, const WeightSet &W,
                    std::vector<std::vector<FragOut>> &out) {
  const int64_t np = (int64_t)pairs.size();
  std::vector<SgTask> Rv;
  for (int64_t p = 0; p < np; ++p)
    for (const Seed4 &x : xs[p]) {
      SgTask g{};
      g.base1 = C.seq_base[2 * p];
      g.base2 = C.seq_base[2 * p + 1];
      g.a1 = x.e1;
      g.a2 = x.e2;
      g.n1 = 1 + x.e1;
      g.n2 = 1 + x.e2;
      g.dir = 1;
      g.wbase = W.wbase[p];
      g.wlen = pairs[p].n1;
      Rv.push_back(g);
    }
  run_semiglobal(C, Rv, P, false, nullptr, &W.dev);
  std::vector<SgTask> Fw;
  std::vector<int32_t> fw_pair;
  std::vector<std::pair<int32_t, int32_t>> fw_start;
  {
    size_t k = 0;
    for (int64_t p = 0; p < np; ++p) {
      std::set<std::pair<int32_t, int32_t>> starts;
      for (size_t s = 0; s < xs[p].size(); ++s, ++k) {
        const int32_t s1 = xs[p][s].e1 - (Rv[k].end1 - 1), s2 = xs[p][s].e2 - (Rv[k].end2 - 1);
        if (!starts.insert({s1, s2}).second) continue;
        SgTask g{};
        g.base1 = C.seq_base[2 * p];
        g.base2 = C.seq_base[2 * p + 1];
        g.a1 = s1;
        g.a2 = s2;
        g.n1 = pairs[p].n1 - s1;
        g.n2 = pairs[p].n2 - s2;
        g.dir = 0;
        g.wbase = W.wbase[p];
        g.wlen = pairs[p].n1;
        Fw.push_back(g);
        fw_pair.push_back((int32_t)p);
        fw_start.push_back({s1, s2});
      }
    }
  }
  std::vector<std::vector<uint32_t>> cg;
  run_semiglobal(C, Fw, P, true, &cg, &W.dev);
  out.assign(np, {});
  for (size_t q = 0; q < Fw.size(); ++q) {
    const int32_t p = fw_pair[q];
    const SgTask &g = Fw[q];
    const int32_t s1 = fw_start[q].first, s2 = fw_start[q].second;
    const int32_t e1z = g.end1 - 1, e2z = g.end2 - 1;
    if (W.dev.pieces == 2 && !(cg[q].size() > 0 && e1z > 0 && e2z > 0)) continue;
    const int64_t e1 = (int64_t)e1z + s1, e2 = (int64_t)e2z + s2;
    std::vector<FragOut> &fr = out[p];
    int toRemove = -1;
    bool found = false;
    for (int i = 0; i < (int)fr.size(); ++i)
      if (fr[i].e1 == e1 + 1 && fr[i].e2 == e2 + 1) {
        found = true;
        if (s1 + 1 < fr[i].s1 && s2 + 1 < fr[i].s2) toRemove = i;
      }
    if (found && toRemove < 0) continue;
    FragOut f;
    f.s1 = s1 + 1;
    f.e1 = e1 + 1;
    f.s2 = s2 + 1;
    f.e2 = e2 + 1;
    f.score = (int64_t)(uint32_t)g.score;
    f.cigar = cg[q];
    evalue(P, double(pairs[p].n1), double(pairs[p].n2), g.score, f.e, f.p);
    if (toRemove >= 0)
      fr[toRemove] = std::move(f);
    else
      fr.push_back(std::move(f));
  }
}

// The seeded 2-gap overload (findSimilarFragmentsForPairedSequence4.cpp:624-745; cut2Gaps2 with seeds from a SAM
// file).  The reference walks the seeds in order and skips a seed covered by a fragment it has already accepted, so
// which DPs run depends on earlier results.  Here every seed's reverse DP and the forward DP of every distinct start
// run on the device first (a superset of what the reference computes; each result depends only on its own inputs),
// then the host replays the reference's order, skip test, StartAlignment gate and dedupe over those results.
// Reverse lengths are min(1 + end, max_align) from the seed's own end; when the two end bases differ the ends move
// back one base (:663-667).  Where that would read before a sequence start (outside the reference's buffer) the DP
// is shortened to the bases that exist.  No p-value filter (the overload has none).
void seeded_two_gap(Context &C, const std::vector<PairIn> &pairs, const std::vector<std::vector<Seed4>> &seeds,
                    const Params &P, std::vector<std::vector<FragOut>> &out) {
  const int64_t np = (int64_t)pairs.size();
  const int32_t cap = P.max_align_len > 0 ? P.max_align_len : INT32_MAX;
  std::vector<SgTask> Rv;
  std::vector<std::array<int32_t, 2>> rv_end;  // the (moved) end each reverse DP starts from
  for (int64_t p = 0; p < np; ++p)
    for (const Seed4 &x : seeds[p]) {
      int32_t b1 = x.e1, b2 = x.e2;
      int32_t l11 = (int32_t)std::min<int64_t>(1 + (int64_t)b1, cap), l12 = (int32_t)std::min<int64_t>(1 + (int64_t)b2, cap);
      if (b1 >= 0 && b1 < pairs[p].n1 && b2 >= 0 && b2 < pairs[p].n2 && pairs[p].s1[b1] != pairs[p].s2[b2]) --b1, --b2;
      SgTask g{};
      g.base1 = C.seq_base[2 * p];
      g.base2 = C.seq_base[2 * p + 1];
      g.a1 = b1;
      g.a2 = b2;
      g.n1 = std::max(0, std::min(l11, b1 + 1));
      g.n2 = std::max(0, std::min(l12, b2 + 1));
      g.dir = 1;
      Rv.push_back(g);
      rv_end.push_back({b1, b2});
    }
  run_semiglobal(C, Rv, P, false, nullptr);
  // forward DP per distinct start of each pair
  std::vector<SgTask> Fw;
  std::vector<std::map<std::pair<int32_t, int32_t>, int32_t>> fw_of(np);
  {
    size_t k = 0;
    for (int64_t p = 0; p < np; ++p)
      for (size_t s = 0; s < seeds[p].size(); ++s, ++k) {
        const int32_t s1 = rv_end[k][0] - (Rv[k].end1 - 1), s2 = rv_end[k][1] - (Rv[k].end2 - 1);
        if (!fw_of[p].emplace(std::make_pair(s1, s2), (int32_t)Fw.size()).second) continue;
        SgTask g{};
        g.base1 = C.seq_base[2 * p];
        g.base2 = C.seq_base[2 * p + 1];
        g.a1 = s1;
        g.a2 = s2;
        g.n1 = (int32_t)std::max<int64_t>(0, std::min<int64_t>((int64_t)pairs[p].n1 - s1, cap));
        g.n2 = (int32_t)std::max<int64_t>(0, std::min<int64_t>((int64_t)pairs[p].n2 - s2, cap));
        if (s1 < 0 || s2 < 0 || s1 > pairs[p].n1 || s2 > pairs[p].n2) g.n1 = g.n2 = 0;
        g.dir = 0;
        Fw.push_back(g);
      }
  }
  std::vector<std::vector<uint32_t>> cg;
  run_semiglobal(C, Fw, P, true, &cg);
  // the reference's order over the computed results
  out.assign(np, {});
  size_t k = 0;
  for (int64_t p = 0; p < np; ++p) {
    std::vector<FragOut> &fr = out[p];
    std::set<std::pair<int32_t, int32_t>> starts;
    for (size_t s = 0; s < seeds[p].size(); ++s, ++k) {
      const Seed4 &x = seeds[p][s];
      bool use = true;
      for (const FragOut &f : fr)
        if (f.s1 <= (int64_t)(uint32_t)x.s1 && f.e1 >= (int64_t)(uint32_t)x.e1 && f.s2 <= (int64_t)(uint32_t)x.s2 &&
            f.e2 >= (int64_t)(uint32_t)x.e2) {
          use = false;
          break;
        }
      if (!use) continue;
      const int32_t s1 = rv_end[k][0] - (Rv[k].end1 - 1), s2 = rv_end[k][1] - (Rv[k].end2 - 1);
      if (!starts.insert({s1, s2}).second) continue;
      const int32_t q = fw_of[p].at({s1, s2});
      const SgTask &g = Fw[q];
      const int32_t e1z = g.end1 - 1, e2z = g.end2 - 1;
      if (!(cg[q].size() > 0 && e1z > 0 && e2z > 0)) continue;
      const int64_t e1 = (int64_t)e1z + s1, e2 = (int64_t)e2z + s2;
      int toRemove = -1;
      bool found = false;
      for (int i = 0; i < (int)fr.size(); ++i)
        if (fr[i].e1 == e1 + 1 && fr[i].e2 == e2 + 1) {
          found = true;
          if (s1 + 1 < fr[i].s1 && s2 + 1 < fr[i].s2) toRemove = i;
        }
      if (found && toRemove < 0) continue;
      FragOut f;
      f.s1 = s1 + 1;
      f.e1 = e1 + 1;
      f.s2 = s2 + 1;
      f.e2 = e2 + 1;
      f.score = (int64_t)(uint32_t)g.score;
      f.cigar = cg[q];
      evalue(P, double(pairs[p].n1), double(pairs[p].n2), g.score, f.e, f.p);
      if (toRemove >= 0)
        fr[toRemove] = std::move(f);
      else
        fr.push_back(std::move(f));
    }
  }
}

}  // namespace

namespace {
void check_seeded_inputs(const std::vector<PairIn> &pairs, const std::vector<std::vector<Seed4>> &seeds) {
  for (const PairIn &p : pairs) {
    if ((p.n1 > 0 && !p.s1) || (p.n2 > 0 && !p.s2)) throw Error(DCNS_ERR_INVALID, "NULL sequence");
    if (p.n1 >= (1 << 24) - 2 || p.n2 >= (1 << 24) - 2) throw Error(DCNS_ERR_INVALID, "sequences must be < 16M bases");
  }
  for (size_t p = 0; p < seeds.size(); ++p)
    for (const Seed4 &x : seeds[p])
      if (x.s1 < 0 || x.s2 < 0 || x.e1 < -1 || x.e2 < -1 || x.e1 >= pairs[p].n1 || x.e2 >= pairs[p].n2)
        throw Error(DCNS_ERR_INVALID, "seed outside its sequences");
}
}  // namespace

void align_seeded(Context &C, const std::vector<PairIn> &pairs, const std::vector<std::vector<Seed4>> &seeds,
                  const Params &P, std::vector<std::vector<FragOut>> &out) {
  validate(P);
  check_seeded_inputs(pairs, seeds);
  auto t0 = Clock::now();
  C.call_t0 = t0;
  C.stats = dcns_stats{};
  out.assign(pairs.size(), {});
  if (pairs.empty()) return;
  upload(C, pairs);
  seeded_two_gap(C, pairs, seeds, P, out);
  C.stats.ms_total = ms_since(t0);
  C.stats.bytes_device = device_bytes(C);
}

void align_xseeds(Context &C, const std::vector<PairIn> &pairs, const std::vector<std::vector<Seed4>> &seeds,
                  const Params &P, std::vector<std::vector<FragOut>> &out) {
  validate(P);
  check_seeded_inputs(pairs, seeds);
  auto t0 = Clock::now();
  C.call_t0 = t0;
  C.stats = dcns_stats{};
  out.assign(pairs.size(), {});
  if (pairs.empty()) return;
  upload(C, pairs);
  two_gap_stage(C, pairs, P, seeds, out);
  C.stats.ms_total = ms_since(t0);
  C.stats.bytes_device = device_bytes(C);
}

// getAllExtendSeed's p-value filter and x-seed merge (findSimilarFragmentsForPairedSequence4.cpp:395-427).
std::vector<std::vector<Seed4>> merge_x_seeds(const std::vector<PairIn> &pairs, const Params &P,
                                              std::vector<std::vector<XSeedOut>> &xr) {
  const int64_t np = (int64_t)pairs.size();
  std::vector<std::vector<Seed4>> xs(np);
  for (int64_t p = 0; p < np; ++p) {
    const double L1 = double(pairs[p].n1), L2 = double(pairs[p].n2);
    for (XSeedOut &x : xr[p]) {
      if (!x.ok) continue;
      double ev, pv;
      evalue(P, L1, L2, x.score, ev, pv);
      if (!(pv < P.pvalue)) continue;
      bool fresh = true;
      for (Seed4 &y : xs[p]) {
        if (y.s1 == x.start1 && y.s2 == x.start2) {
          fresh = false;
          if (x.end1 > y.e1 && x.end2 > y.e2) y.e1 = x.end1, y.e2 = x.end2;
        } else if (y.e1 == x.end1 && y.e2 == x.end2) {
          if (x.start1 < y.s1 && x.start2 < y.s2) y.s1 = x.start1, y.s2 = x.start2;
          fresh = false;
        }
      }
      if (fresh) xs[p].push_back(Seed4{x.start1, x.end1, x.start2, x.end2});
    }
  }
  return xs;
}

void align_single(Context &C, const std::vector<PairIn> &pairs, const Params &P, int mode,
                  std::vector<std::vector<FragOut>> &out);

void align_weighted(Context &C, const std::vector<PairIn> &pairs, const std::vector<const int16_t *> &weights,
                    const std::vector<int32_t> &cats, int pieces, const Params &P,
                    std::vector<std::vector<FragOut>> &out) {
  validate(P);
  if (pieces != 1 && pieces != 2) throw Error(DCNS_ERR_INVALID, "pieces must be 1 or 2");
  const int32_t ncat = (int32_t)(cats.size() / 7);
  if (ncat < 1 || ncat > kSgwMaxCats || (int64_t)cats.size() != 7 * (int64_t)ncat)
    throw Error(DCNS_ERR_INVALID, "1 to 64 categories of 7 values are needed");
  int64_t total = 0;
  for (size_t p = 0; p < pairs.size(); ++p) {
    if ((pairs[p].n1 > 0 && (!pairs[p].s1 || !weights[p])) || (pairs[p].n2 > 0 && !pairs[p].s2))
      throw Error(DCNS_ERR_INVALID, "NULL sequence or weights");
    if (pairs[p].n1 >= (1 << 24) - 2 || pairs[p].n2 >= (1 << 24) - 2)
      throw Error(DCNS_ERR_INVALID, "sequences must be < 16M bases");
    for (int32_t i = 0; i < pairs[p].n1; ++i)
      if (weights[p][i] < 0 || weights[p][i] >= ncat) throw Error(DCNS_ERR_INVALID, "weight category out of range");
    total += pairs[p].n1;
  }
  auto t0 = Clock::now();
  C.call_t0 = t0;
  C.stats = dcns_stats{};
  out.assign(pairs.size(), {});
  if (pairs.empty()) return;
  upload(C, pairs);
  WeightSet W;
  W.wbase.resize(pairs.size());
  std::vector<int16_t> flat((size_t)std::max<int64_t>(total, 1));
  int64_t off = 0;
  for (size_t p = 0; p < pairs.size(); ++p) {
    W.wbase[p] = off;
    if (pairs[p].n1 > 0) std::memcpy(flat.data() + off, weights[p], sizeof(int16_t) * pairs[p].n1);
    off += pairs[p].n1;
  }
  C.d_wts.ensure(C, sizeof(int16_t) * flat.size());
  C.d_cats.ensure(C, sizeof(int32_t) * cats.size());
  DCNS_CK(cudaMemcpyAsync(C.d_wts.p, flat.data(), sizeof(int16_t) * flat.size(), cudaMemcpyHostToDevice, C.st));
  DCNS_CK(cudaMemcpyAsync(C.d_cats.p, cats.data(), sizeof(int32_t) * cats.size(), cudaMemcpyHostToDevice, C.st));
  sync(C);
  W.dev = SgWeights{C.d_wts.as<int16_t>(), C.d_cats.as<int32_t>(), ncat, pieces};
  C.weights = &W;
  try {
    align_single(C, pairs, P, DCNS_MODE_TWO_GAP, out);
  } catch (...) {
    C.weights = nullptr;
    throw;
  }
  C.weights = nullptr;
  C.stats.ms_total = ms_since(t0);
  C.stats.bytes_device = device_bytes(C);
}

// ------------------------------------------------------------------ entry points
void align_core(Context &C, const std::vector<PairIn> &pairs, const Params &P, int mode,
                std::vector<std::vector<FragOut>> &out);
void align_single(Context &C, const std::vector<PairIn> &pairs, const Params &P, int mode,
                  std::vector<std::vector<FragOut>> &out);

void align_pairs(Context &C, const std::vector<PairIn> &pairs, const Params &P, int mode,
                 std::vector<std::vector<FragOut>> &out) {
  validate(P);
  if (mode != DCNS_MODE_ONE_GAP && mode != DCNS_MODE_TWO_GAP) throw Error(DCNS_ERR_INVALID, "mode must be 1 or 2");
  for (const PairIn &p : pairs) {
    if ((p.n1 > 0 && !p.s1) || (p.n2 > 0 && !p.s2)) throw Error(DCNS_ERR_INVALID, "NULL sequence");
    if (p.n1 >= (1 << 24) - 2 || p.n2 >= (1 << 24) - 2) throw Error(DCNS_ERR_INVALID, "sequences must be < 16M bases");
  }
  auto t0 = Clock::now();
  C.call_t0 = t0;
  C.stats = dcns_stats{};
  out.assign(pairs.size(), {});
  if (pairs.empty()) return;
  auto tu = Clock::now();
  upload(C, pairs);
  C.stats.ms_upload = ms_since(tu);
  print_phases(C, "upload");
  align_core(C, pairs, P, mode, out);
  C.stats.ms_total = ms_since(t0);
  C.stats.bytes_device = device_bytes(C);
}

void batch_upload(Context &C, const std::vector<PairIn> &pairs, Batch &B) {
  for (const PairIn &p : pairs)
    if (p.n1 >= (1 << 24) - 2 || p.n2 >= (1 << 24) - 2) throw Error(DCNS_ERR_INVALID, "sequences must be < 16M bases");
  upload_into(C, pairs, B.pk, B.nm, B.sb, B.seq_base, B.arena);
  sync(C);
  B.lens.clear();
  for (const PairIn &p : pairs) B.lens.push_back(PairIn{nullptr, p.n1, nullptr, p.n2});
}

void align_batch(Context &C, Batch &B, const Params &P, int mode, std::vector<std::vector<FragOut>> &out) {
  validate(P);
  if (mode != DCNS_MODE_ONE_GAP && mode != DCNS_MODE_TWO_GAP) throw Error(DCNS_ERR_INVALID, "mode must be 1 or 2");
  auto t0 = Clock::now();
  C.call_t0 = t0;
  C.stats = dcns_stats{};
  out.assign(B.lens.size(), {});
  if (B.lens.empty()) return;
  C.arena = B.arena;
  C.seq_base = B.seq_base;
  C.seqbase_dev = B.sb.as<int64_t>();
  align_core(C, B.lens, P, mode, out);
  C.stats.ms_total = ms_since(t0);
  C.stats.bytes_device = device_bytes(C);
}

void autotune(Context &C, Batch &B, const Params &P, int mode) {
  struct Shape {
    int lanes, bins;
    double ratio;
    bool by_size;
  };
  // Every trial call starts with a cold L2, as a call on fresh data does: a 256 MB device write (twice the L2) first,
  // untimed.  Without room for it the trials run warm.
  struct Flush {
    void *p = nullptr;
    size_t bytes = (size_t)256 << 20;
    Flush() {
      if (cudaMalloc(&p, bytes) != cudaSuccess) (void)cudaGetLastError(), p = nullptr;
    }
    ~Flush() {
      if (p) cudaFree(p);
    }
  } flush;
  auto run = [&](const Shape &sh) {
    C.max_lanes = sh.lanes, C.bins = sh.bins, C.bin_ratio = sh.ratio, C.bins_by_size = sh.by_size;
    std::vector<std::vector<FragOut>> out;
    if (flush.p) {
      DCNS_CK(cudaMemsetAsync(flush.p, 0, flush.bytes, C.st));
      sync(C);
    }
    const auto t0 = Clock::now();
    align_batch(C, B, P, mode, out);
    return ms_since(t0);
  };
  auto best_of3 = [&](const Shape &sh) { return std::min({run(sh), run(sh), run(sh)}); };
  // A candidate replaces the incumbent (the context's current setting, measured first) only when it is faster by
  // more than a margin: 2 % for kernel forms, 5 % for the pipeline shape (lanes, bins, shares), whose trial calls
  // vary most from run to run; differences within that noise keep the default.
  constexpr double kMargin = 0.02, kShapeMargin = 0.05;
  auto better = [](double ms, double incumbent) { return ms < incumbent * (1.0 - kMargin); };
  auto shape_better = [](double ms, double incumbent) { return ms < incumbent * (1.0 - kShapeMargin); };
  const Shape first[] = {{1, 1, 0.6, false}, {2, 2, 0.6, false}, {3, 3, 0.6, false},
                         {4, 4, 0.6, false}, {4, 6, 0.6, false}, {6, 6, 0.6, false}};
  Shape best{C.max_lanes, C.bins, C.bin_ratio, C.bins_by_size};
  run(best);  // warm: buffers of the current shape
  double best_ms = best_of3(best);
  for (const Shape &sh : first) {
    if (sh.lanes == best.lanes && sh.bins == best.bins && sh.ratio == best.ratio && sh.by_size == best.by_size)
      continue;
    run(sh);  // allocates this shape's lane buffers
    const double ms = best_of3(sh);
    if (shape_better(ms, best_ms)) best_ms = ms, best = sh;
  }
  // the bin shares, and bins by size (the largest pairs last) against mixed bins
  for (const Shape sh : {Shape{best.lanes, best.bins, 0.45, false}, Shape{best.lanes, best.bins, 0.75, false},
                         Shape{best.lanes, best.bins, 1.0, true}, Shape{best.lanes, best.bins, 1.6, true},
                         Shape{best.lanes, best.bins, 2.5, true}}) {
    const double ms = best_of3(sh);
    if (shape_better(ms, best_ms)) best_ms = ms, best = sh;
  }
  C.max_lanes = best.lanes, C.bins = best.bins, C.bin_ratio = best.ratio, C.bins_by_size = best.by_size;

  // Per bin: the x-drop pass forms (register-band levels row-interleaved or one pass per thread, the band where one
  // warp per pass takes over, the widest band of the wavefront form, the rows after which a register-band pass moves
  // to the wavefront form), chosen by that bin's x-drop kernel time with
  // each candidate applied to every bin; the bins differ in how many long and wide-band passes they hold.
  C.bin_tune.clear();
  if (C.max_lanes > 1 && (int64_t)B.lens.size() >= 4096) {
    const int h = C.xdrop_handoff, g = C.xdrop_resume_lanes, gf = C.xdrop_group_from, ts = C.scan_tiles_per_thread;
    // the first candidate is the context's setting (the incumbent)
    const Context::BinTune cands[] = {
        {C.xdrop_warp_from, C.xdrop_wave_max_w, C.xdrop_flat, h, g, gf, ts},
        {20, 256, false, 0, g, 0, ts},    {10, 256, true, h, g, gf, ts},   {20, 256, true, 0, g, 0, ts},
        {20, 256, true, 48, g, gf, ts},   {20, 256, true, 192, g, gf, ts}, {20, 256, true, 48, 32, 0, ts},
        {20, 256, true, 96, 32, 0, ts},   {20, 128, true, h, g, gf, ts},   {20, 256, true, h, 4, gf, ts},
        {20, 256, true, 48, 4, gf, ts},   {20, 256, true, h, g, 20, ts},   {20, 256, true, 48, g, 20, ts},
        {20, 256, true, h, 4, 20, ts},    {20, 256, true, h, g, 10, ts}};
    const int nb = std::max(C.bins, C.max_lanes);
    std::vector<double> best_ms(nb, 1e300);
    std::vector<Context::BinTune> choice(nb, cands[0]);
    for (const Context::BinTune &cd : cands) {
      C.bin_tune.assign(nb, cd);
      run(best);
      std::vector<double> ms = C.last_bin_xdrop_ms;
      run(best);
      for (int b = 0; b < nb && b < (int)ms.size() && b < (int)C.last_bin_xdrop_ms.size(); ++b) {
        const double m = std::min(ms[b], C.last_bin_xdrop_ms[b]);
        if (best_ms[b] == 1e300 || better(m, best_ms[b])) best_ms[b] = m, choice[b] = cd;
      }
    }
    C.bin_tune = choice;
  }
  // the scan's tiling target (tiles per resident thread before reference rows are split into chunks; it matters
  // for batches of few long pairs) and, on the 2-gap path, the 2-piece kernel's warps per DP: by whole-call time
  // (for the whole call, and per bin by that bin's seed-scan kernel time over the same runs)
  {
    const int t0 = C.scan_tiles_per_thread;
    const int nb = (int)C.bin_tune.size();
    std::vector<double> bin_best(nb, 1e300);
    auto timed = [&](int t) {  // best of three calls with every bin at target t; each bin's fastest scan time
      C.scan_tiles_per_thread = t;
      for (auto &bt : C.bin_tune) bt.scan_tiles = t;
      std::vector<double> bms(nb, 1e300);
      double ms = 1e300;
      for (int r = 0; r < 3; ++r) {
        ms = std::min(ms, run(best));
        for (int b = 0; b < nb && b < (int)C.last_bin_scan_ms.size(); ++b)
          bms[b] = std::min(bms[b], C.last_bin_scan_ms[b]);
      }
      return std::make_pair(ms, bms);
    };
    std::vector<int> bin_t(nb, t0);
    auto [best_t_ms, bms0] = timed(t0);
    int best_t = t0;
    bin_best = bms0;
    for (int t : {4, 8, 16}) {
      if (t == t0) continue;
      const auto [ms, bms] = timed(t);
      if (better(ms, best_t_ms)) best_t_ms = ms, best_t = t;
      for (int b = 0; b < nb; ++b)
        if (better(bms[b], bin_best[b])) bin_best[b] = bms[b], bin_t[b] = t;
    }
    C.scan_tiles_per_thread = best_t;
    for (int b = 0; b < nb; ++b) C.bin_tune[b].scan_tiles = bin_t[b];
  }
  if (mode == DCNS_MODE_TWO_GAP) {
    // the stripe flow with 5 or 6 blocks per SM (-5, -6 below), or one CTA per DP with 2, 4 or 8 warps (0: by the
    // number of DPs)
    int best_w = -5;
    double best_w_ms = 1e300;
    for (int nw : {-5, -6, 0, 2, 4, kSgNW}) {
      C.sg_flow = nw < 0;
      C.sg_flow_blocks = nw == -6 ? 6 : 5;
      C.sg_warps = std::max(nw, 0);
      const double ms = std::min(run(best), run(best));
      if (best_w_ms == 1e300 || better(ms, best_w_ms)) best_w_ms = ms, best_w = nw;
    }
    C.sg_flow = best_w < 0;
    C.sg_flow_blocks = best_w == -6 ? 6 : 5;
    C.sg_warps = std::max(best_w, 0);
  }
}

void add_stats(dcns_stats &a, const dcns_stats &b) {
  a.cells_scan += b.cells_scan, a.cells_scan_reverse += b.cells_scan_reverse, a.cells_xdrop += b.cells_xdrop;
  a.cells_semiglobal += b.cells_semiglobal, a.tasks_scan += b.tasks_scan;
  a.tasks_scan_speculative += b.tasks_scan_speculative, a.seeds += b.seeds, a.xdrop_passes += b.xdrop_passes;
  a.semiglobal_dps += b.semiglobal_dps, a.ms_upload += b.ms_upload, a.ms_scan += b.ms_scan;
  a.ms_replay += b.ms_replay, a.ms_xdrop += b.ms_xdrop, a.ms_semiglobal += b.ms_semiglobal;
  a.ms_download += b.ms_download, a.ms_scan_kernel += b.ms_scan_kernel, a.ms_scan_prep += b.ms_scan_prep;
  a.ms_scan_xfer += b.ms_scan_xfer, a.ms_link += b.ms_link, a.scan_launches += b.scan_launches;
  a.kernel_launches += b.kernel_launches, a.scan_rounds += b.scan_rounds, a.xdrop_rounds += b.xdrop_rounds;
  a.ms_xdrop_kernel += b.ms_xdrop_kernel;
  a.bytes_h2d += b.bytes_h2d;
  a.ms_xdrop_tb_kernel += b.ms_xdrop_tb_kernel, a.ms_sg_kernel += b.ms_sg_kernel;
  a.ms_sg_tb_kernel += b.ms_sg_tb_kernel;
  a.bytes_codes_xdrop += b.bytes_codes_xdrop, a.bytes_codes_sg += b.bytes_codes_sg;
}

// Batches large enough to fill the GPU several times over are split into bins of similar work (pairs dealt
// round-robin in decreasing n1*n2), and the bins are run by several lanes: while one lane's host threads replay seed
// sets and link, the other lanes' kernels run.  Results and stats are the per-pair results of the single-lane path.
void align_core(Context &C, const std::vector<PairIn> &pairs, const Params &P, int mode,
                std::vector<std::vector<FragOut>> &out) {
  const int64_t np = (int64_t)pairs.size();
  const int nl = C.is_lane ? 1 : C.max_lanes;
  if (C.trace >= 2) std::fprintf(stderr, "[dcns tl] call_start %lld pairs\n", (long long)np);
  const int kBins = std::max(C.bins, nl);
  if (nl < 2 || np < 4096) {
    align_single(C, pairs, P, mode, out);
    return;
  }
  DCNS_CK(cudaStreamSynchronize(C.st));  // the arena (packed on this context's stream) is complete
  while ((int)C.lanes.size() < nl) {
    auto L = std::make_unique<Context>();
    const size_t room = C.budget > C.used ? C.budget - C.used : 0;
    init_context(*L, C.device, std::max<size_t>(room / (2 * nl), (size_t)1 << 30));
    L->is_lane = true;
    C.lanes.push_back(std::move(L));
  }
  std::vector<int64_t> order(np);
  for (int64_t p = 0; p < np; ++p) order[p] = p;
  const bool ascending = C.bins_by_size;
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    const int64_t wa = (int64_t)pairs[a].n1 * pairs[a].n2, wb = (int64_t)pairs[b].n1 * pairs[b].n2;
    return wa != wb ? (ascending ? wa < wb : wa > wb) : a < b;
  });
  // bin b's share of the seed-scan work is proportional to bin_ratio^b.  Two ways to fill the bins:
  //  * mixed (default): pairs dealt in decreasing work to the bin furthest below its share, so every bin holds a mix
  //    of sizes and the last bins to finish their level-0 scan have the least scan work;
  //  * by size: consecutive runs of pairs in increasing work, so the last bin holds the largest pairs.  The host and
  //    x-drop work after a bin's scan grows with its number of pairs (seeds per pair do not grow with pair length),
  //    so the bin whose tail is on the critical path then has the fewest pairs; its shares grow bin to bin
  //    (bin_ratio > 1: on the 10,000-pair workload 1.6 measured 146.6 ms per step against 184.5 at 0.6).
  std::vector<double> target(kBins);
  {
    double tot = 0, wsum = 0, f = 1;
    for (int64_t p = 0; p < np; ++p) tot += (double)pairs[p].n1 * pairs[p].n2 + 1;
    for (int b = 0; b < kBins; ++b, f *= C.bin_ratio) target[b] = f, wsum += f;
    for (int b = 0; b < kBins; ++b) target[b] *= tot / wsum;
  }
  std::vector<std::vector<int64_t>> bins(kBins);
  for (int64_t q = 0, cur = 0; q < np; ++q) {
    const int64_t p = order[q];
    const double wk = (double)pairs[p].n1 * pairs[p].n2 + 1;
    int bb = 0;
    if (ascending) {
      while (cur + 1 < kBins && target[cur] <= 0) ++cur;
      bb = (int)cur;
    } else {
      for (int b = 1; b < kBins; ++b)
        if (target[b] > target[bb]) bb = b;
    }
    bins[bb].push_back(p);
    target[bb] -= wk;
  }
  for (auto &b : bins) std::sort(b.begin(), b.end());  // each bin keeps the caller's pair order
  std::atomic<int> next(0);
  Context::Turnstile turn;
  auto pass_turn = [&](int b, bool failed) {
    std::lock_guard<std::mutex> lk(turn.mu);
    turn.next = std::max(turn.next, b + 1);
    if (failed) turn.abort = true;
    turn.cv.notify_all();
  };
  std::vector<std::string> errs(nl);
  std::vector<int> codes(nl, 0);
  std::vector<dcns_stats> st(nl, dcns_stats{});
  std::vector<double> bin_xdrop_ms(kBins, 0.0), bin_scan_ms(kBins, 0.0);
  auto worker = [&](int l) {
    Context &L = *C.lanes[l];
    try {
      DCNS_CK(cudaSetDevice(C.device));
      for (int b; (b = next.fetch_add(1)) < kBins;) {
        struct Pass {  // every bin passes the turnstile, whether or not it reached its level-0 scan
          decltype(pass_turn) &fn;
          int b;
          bool failed = true;
          ~Pass() { fn(b, failed); }
        } pass{pass_turn, b};
        const std::vector<int64_t> &ids = bins[b];
        std::vector<PairIn> sub(ids.size());
        L.seq_base.resize(2 * ids.size());
        for (size_t k = 0; k < ids.size(); ++k) {
          sub[k] = pairs[ids[k]];
          L.seq_base[2 * k] = C.seq_base[2 * ids[k]];
          L.seq_base[2 * k + 1] = C.seq_base[2 * ids[k] + 1];
        }
        L.arena = C.arena;
        L.d_seqbase.ensure(L, sizeof(int64_t) * L.seq_base.size() + 8);
        DCNS_CK(cudaMemcpyAsync(L.d_seqbase.p, L.seq_base.data(), sizeof(int64_t) * L.seq_base.size(),
                                cudaMemcpyHostToDevice, L.st));
        L.seqbase_dev = L.d_seqbase.as<int64_t>();
        L.stats = dcns_stats{};
        // the bin's kernel shapes: the autotuner's per-bin choice, else the parent context's
        const Context::BinTune bt = b < (int)C.bin_tune.size()
                                        ? C.bin_tune[b]
                                        : Context::BinTune{C.xdrop_warp_from, C.xdrop_wave_max_w, C.xdrop_flat,
                                                           C.xdrop_handoff, C.xdrop_resume_lanes, C.xdrop_group_from,
                                                           C.scan_tiles_per_thread};
        L.xdrop_warp_from = bt.xdrop_warp_from, L.xdrop_wave_max_w = bt.xdrop_wave_max_w, L.xdrop_flat = bt.xdrop_flat;
        L.xdrop_handoff = bt.xdrop_handoff, L.xdrop_resume_lanes = bt.xdrop_resume_lanes;
        L.xdrop_group_from = bt.xdrop_group_from;
        L.sg_warps = C.sg_warps;
        L.sg_flow = C.sg_flow;
        L.sg_flow_blocks = C.sg_flow_blocks;
        L.scan_tiles_per_thread = bt.scan_tiles;
        L.call_t0 = C.call_t0;
        L.lane_id = l;
        L.trace = C.trace;
        L.l0_turn = &turn;
        L.bin = b;
        L.bulk_shared = C.st_bulk;
        phase(L, "bin_start", Clock::now());
        std::vector<std::vector<FragOut>> so(ids.size());
        align_single(L, sub, P, mode, so);
        pass.failed = false;
        for (size_t k = 0; k < ids.size(); ++k) out[ids[k]] = std::move(so[k]);
        bin_xdrop_ms[b] = L.stats.ms_xdrop_kernel;
        bin_scan_ms[b] = L.stats.ms_scan_kernel;
        add_stats(st[l], L.stats);
      }
    } catch (const Error &e) {
      errs[l] = e.what();
      codes[l] = e.code;
    } catch (const std::exception &e) {
      errs[l] = e.what();
      codes[l] = DCNS_ERR_DEVICE;
    }
  };
  std::vector<std::thread> th;
  for (int l = 1; l < nl; ++l) th.emplace_back(worker, l);
  worker(0);
  for (auto &t : th) t.join();
  for (int l = 0; l < nl; ++l) C.lanes[l]->l0_turn = nullptr;
  for (int l = 0; l < nl; ++l)
    if (codes[l]) throw Error(codes[l], errs[l]);
  for (int l = 0; l < nl; ++l) add_stats(C.stats, st[l]);
  C.last_bin_xdrop_ms = std::move(bin_xdrop_ms);
  C.last_bin_scan_ms = std::move(bin_scan_ms);
}

void align_single(Context &C, const std::vector<PairIn> &pairs, const Params &P, int mode,
                  std::vector<std::vector<FragOut>> &out) {
  const int64_t np = (int64_t)pairs.size();
  const bool one_gap = mode == DCNS_MODE_ONE_GAP;
  std::vector<std::vector<Seed4>> linked;
  auto tp = Clock::now();
  scan_and_link(C, pairs, P, one_gap, linked);
  tp = phase(C, "scan_and_link", tp);
  std::vector<std::vector<XSeedOut>> xr;
  std::vector<uint32_t> cig_flat;
  extend_seeds(C, pairs, P, linked, one_gap, xr, cig_flat);
  tp = phase(C, "extend_seeds", tp);
  struct Done {
    Context &C;
    Clock::time_point t;
    ~Done() {
      phase(C, "fragments", t);
      print_phases(C, C.is_lane ? "lane" : "call");
    }
  } done{C, tp};
  if (one_gap) {
    parallel_for(np, [&](int64_t p) {
      const double L1 = double(pairs[p].n1), L2 = double(pairs[p].n2);
      std::vector<FragOut> &fr = out[p];
      for (XSeedOut &x : xr[p]) {
        if (!x.ok) continue;
        double ev, pv;
        evalue(P, L1, L2, x.score, ev, pv);
        if (!(pv < P.pvalue)) continue;
        FragOut f{(int64_t)x.start1 + 1, (int64_t)x.end1 + 1, (int64_t)x.start2 + 1, (int64_t)x.end2 + 1,
                  (int64_t)(uint32_t)x.score,
                  std::vector<uint32_t>(cig_flat.begin() + x.cig_off, cig_flat.begin() + x.cig_off + x.cig_len), pv,
                  ev};
        bool fresh = true;
        for (FragOut &g : fr) {  // :503-517: compares 0-based new ends with stored 1-based ones
          if (g.s1 == f.s1 && g.s2 == f.s2) {
            fresh = false;
            if ((int64_t)x.end1 >= g.e1 && (int64_t)x.end2 >= g.e2) g = f;
            break;
          } else if (g.e1 == f.e1 && g.e2 == f.e2) {
            fresh = false;
            if ((int64_t)x.start1 <= g.s1 && (int64_t)x.start2 <= g.s2) g = f;
            break;
          }
        }
        if (fresh) fr.push_back(std::move(f));
      }
    });
  } else {
    // getAllExtendSeed's filter and x-seed merge (:395-427), then the 2-piece stage (weighted when weights are set)
    std::vector<std::vector<Seed4>> xs = merge_x_seeds(pairs, P, xr);
    if (C.weights)
      weighted_stage(C, pairs, P, xs, *C.weights, out);
    else
      two_gap_stage(C, pairs, P, xs, out);
  }
}

void smith_waterman_batch(Context &C, const std::vector<PairIn> &tasks, const Params &P, int32_t *out) {
  validate(P);
  const int64_t n = (int64_t)tasks.size();
  C.stats = dcns_stats{};
  if (n == 0) return;
  upload(C, tasks);
  ScanState S;
  for (int64_t k = 0; k < n; ++k) {
    ScanTask T{};
    T.pair = (int32_t)k;
    T.s2 = 0;
    T.tw = tasks[k].n2;
    T.lo = 0;
    T.hi = tasks[k].n1;
    S.tasks.push_back(T);
  }
  Params Q = P;
  Q.min_score = INT_MAX;  // maxima and positions only: no reverse scans
  compute_scan_tasks(C, S, Q);
  for (int64_t k = 0; k < n; ++k) {
    const ScanTask &T = S.task(k);
    out[3 * k] = T.score;
    out[3 * k + 1] = T.score > 0 ? T.end1 : -1;
    out[3 * k + 2] = T.score > 0 ? T.end2 : -1;
  }
}

void xextend_batch(Context &C, const std::vector<PairIn> &tasks, const Params &P, bool want_cigar, int32_t *out,
                   std::vector<uint32_t> &cigar, std::vector<int64_t> &cigar_off) {
  validate(P);
  const int64_t n = (int64_t)tasks.size();
  auto t0 = Clock::now();
  C.call_t0 = t0;
  C.stats = dcns_stats{};
  cigar.clear();
  cigar_off.assign(n + 1, 0);
  if (n == 0) return;
  upload(C, tasks);
  auto tp = phase(C, "upload", t0);
  std::vector<XTask> X(n);
  parallel_for((n + 4095) / 4096, [&](int64_t b) {
    for (int64_t k = b * 4096, e = std::min(n, k + 4096); k < e; ++k) {
      XTask x{};
      x.base1 = C.seq_base[2 * k];
      x.base2 = C.seq_base[2 * k + 1];
      x.n1 = tasks[k].n1;
      x.n2 = tasks[k].n2;
      x.dir = 0;
      x.w = P.w;
      X[k] = x;
    }
  });
  tp = phase(C, "tasks", tp);
  std::vector<int64_t> hoff;
  run_xdrop(C, X, P, want_cigar, want_cigar ? &cigar : nullptr, want_cigar ? &hoff : nullptr);
  tp = phase(C, "xdrop", tp);
  if (want_cigar) {
    // the CIGARs in task order, densely (the chained levels already pack them so; retried passes come after)
    bool dense = true;
    for (int64_t k = 0; k < n; ++k) {
      cigar_off[k + 1] = cigar_off[k] + X[k].ncig;
      dense &= hoff[k] == cigar_off[k] || X[k].ncig == 0;
    }
    if (!dense || (int64_t)cigar.size() != cigar_off[n]) {
      std::vector<uint32_t> packed((size_t)cigar_off[n]);
      parallel_for((n + 4095) / 4096, [&](int64_t b) {
        for (int64_t k = b * 4096, e = std::min(n, k + 4096); k < e; ++k)
          if (X[k].ncig > 0)
            std::memcpy(packed.data() + cigar_off[k], cigar.data() + hoff[k], sizeof(uint32_t) * X[k].ncig);
      });
      cigar.swap(packed);
    }
  }
  parallel_for((n + 4095) / 4096, [&](int64_t b) {
    for (int64_t k = b * 4096, e = std::min(n, k + 4096); k < e; ++k) {
      out[6 * k + 0] = X[k].score;
      out[6 * k + 1] = X[k].end1 - 1;
      out[6 * k + 2] = X[k].end2 - 1;
      out[6 * k + 3] = want_cigar ? X[k].iii : 0;
      out[6 * k + 4] = want_cigar ? X[k].jjj : 0;
      out[6 * k + 5] = want_cigar ? X[k].ncig : 0;
    }
  });
  phase(C, "results", tp);
  C.stats.ms_total = ms_since(t0);
  C.stats.bytes_device = device_bytes(C);
  print_phases(C, "xextend_batch");
}

void semiglobal_batch(Context &C, const std::vector<PairIn> &tasks, const Params &P, bool want_cigar, int32_t *out,
                      std::vector<std::vector<uint32_t>> &cigars) {
  validate(P);
  const int64_t n = (int64_t)tasks.size();
  C.stats = dcns_stats{};
  cigars.assign(n, {});
  if (n == 0) return;
  upload(C, tasks);
  std::vector<SgTask> G(n);
  for (int64_t k = 0; k < n; ++k) {
    SgTask g{};
    g.base1 = C.seq_base[2 * k];
    g.base2 = C.seq_base[2 * k + 1];
    g.n1 = tasks[k].n1;
    g.n2 = tasks[k].n2;
    g.dir = 0;
    G[k] = g;
  }
  run_semiglobal(C, G, P, want_cigar, want_cigar ? &cigars : nullptr);
  for (int64_t k = 0; k < n; ++k) {
    out[4 * k + 0] = G[k].score;
    out[4 * k + 1] = G[k].end1 - 1;
    out[4 * k + 2] = G[k].end2 - 1;
    out[4 * k + 3] = (int32_t)cigars[k].size();
  }
}

void sliding_window(Context &C, const int8_t *const *seqs, const int32_t *lens, int32_t n, const Params &P,
                    double *score, int32_t *max_out) {
  validate(P);
  C.stats = dcns_stats{};
  if (n < 2) return;
  // pair k-1 = (other sequence k as the scanned "reference", sequence 0 as the windowed "read"),
  // as slidingWindowAlignment calls SmithWaterman(seq_i, refwindow, ...) (impl/slidingWindowAlignment.cpp:36)
  std::vector<PairIn> pairs;
  for (int32_t i = 1; i < n; ++i) pairs.push_back(PairIn{seqs[i], lens[i], seqs[0], lens[0]});
  upload(C, pairs);
  ScanState S;
  const int32_t L0 = lens[0];
  int32_t nw = 0;
  std::vector<int32_t> tw_of;
  {
    int32_t tw = P.window;
    for (int32_t j = 0; j < L0; j += P.step) {
      if (tw + j > L0) tw = L0 - j;
      tw_of.push_back(tw);
      ++nw;
    }
  }
  for (int32_t i = 1; i < n; ++i)
    for (int32_t k = 0; k < nw; ++k) {
      ScanTask T{};
      T.pair = i - 1;
      T.s2 = k * P.step;
      T.tw = tw_of[k];
      T.lo = 0;
      T.hi = lens[i];
      S.tasks.push_back(T);
    }
  Params Q = P;
  Q.min_score = INT_MAX;
  compute_scan_tasks(C, S, Q);
  for (int32_t i = 1; i < n; ++i)
    for (int32_t k = 0; k < nw; ++k) {
      const ScanTask &T = S.task((int64_t)(i - 1) * nw + k);
      const int32_t md = std::min(tw_of[k], lens[i]) * P.match;
      score[(int64_t)(i - 1) * nw + k] = double(T.score) / double(md);
      max_out[(int64_t)(i - 1) * nw + k] = T.score;
    }
}

}  // namespace dcns
