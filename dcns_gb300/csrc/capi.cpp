// C ABI of the engine (include/dcns_gb300.h).  Every entry point converts C++ exceptions into status codes and keeps
// the message in the context.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>

#include "engine.h"

using namespace dcns;

struct ResultsImpl {
  dcns_results pub{};
  std::vector<int64_t> off, frag;
  std::vector<double> pv, ev;
  std::vector<uint32_t> cig;
  void finish(const std::vector<std::vector<FragOut>> &fr, const dcns_stats &st) {
    off.assign(fr.size() + 1, 0);
    int64_t nf = 0, nc = 0;
    for (size_t k = 0; k < fr.size(); ++k) {
      nf += (int64_t)fr[k].size();
      for (auto &f : fr[k]) nc += (int64_t)f.cigar.size();
      off[k + 1] = nf;
    }
    frag.resize(nf * 7);
    pv.resize(nf);
    ev.resize(nf);
    cig.resize(nc);
    int64_t i = 0, c = 0;
    for (auto &v : fr)
      for (auto &f : v) {
        int64_t *r = frag.data() + i * 7;
        r[0] = f.s1, r[1] = f.e1, r[2] = f.s2, r[3] = f.e2, r[4] = f.score, r[5] = c, r[6] = (int64_t)f.cigar.size();
        pv[i] = f.p;
        ev[i] = f.e;
        std::memcpy(cig.data() + c, f.cigar.data(), f.cigar.size() * sizeof(uint32_t));
        c += (int64_t)f.cigar.size();
        ++i;
      }
    pub.n_pairs = (int64_t)fr.size();
    pub.n_fragments = nf;
    pub.n_cigar = nc;
    pub.pair_offset = off.data();
    pub.frag = frag.data();
    pub.pvalue = pv.data();
    pub.evalue = ev.data();
    pub.cigar = cig.data();
    pub.stats = st;
  }
};

static_assert(offsetof(ResultsImpl, pub) == 0, "dcns_results must be the first member");

// ---------------------------------------------------------------- serving state
// Continuous batching.  Workers (each its own pipeline: stream and device buffers) take requests from the queue in
// arrival order into a batch until the batch's predicted device bytes would pass the worker's memory budget or its
// predicted seed-scan cells would pass the batch cap, so long requests are admitted with fewer companions and a batch
// stays short enough for the requests behind it.  While one worker replays seed sets on the host, the others' kernels
// run.  A batch the device budget rejects is halved; a batch that fails otherwise is retried one request at a time,
// so one failing request fails only itself.
struct Server {
  Params P{};
  int mode = DCNS_MODE_ONE_GAP;
  int max_inflight = 256;
  int64_t admit_bytes = 0;  // predicted device bytes a batch may hold (the worker's budget unless set)
  int64_t batch_cells = 0;
  bool running = false, stopped = false;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  struct Req {
    uint64_t ticket;
    std::vector<int8_t> s1, s2;
    int64_t bytes, cells;  // predicted device bytes and level-0 seed-scan cells
  };
  std::deque<Req> queue;
  std::unordered_map<uint64_t, ResultsImpl *> done;
  std::unordered_map<uint64_t, std::pair<int, std::string>> failed;  // status and message
  std::unordered_set<uint64_t> pending;    // queued or being aligned
  std::unordered_set<uint64_t> cancelled;  // cancelled while being aligned: the result is dropped
  uint64_t next = 1;
  dcns_serving_stats counters{};
  std::vector<std::unique_ptr<Context>> lanes;  // one pipeline (stream + buffers) per worker
  std::vector<std::thread> workers;
  ~Server() {
    for (auto &kv : done) delete kv.second;
  }
};

struct dcns_ctx {
  Context C;
  // The server is shared with the calls that use it: a stop that overlaps a wait or a poll ends the server's work,
  // and the server is freed when the last of those calls returns.
  std::mutex srv_mu;
  std::shared_ptr<Server> srv;
  int serve_workers = 3;
  int64_t serve_batch_cells = 0, serve_admit_bytes = 0;
};

struct dcns_batch {
  Batch B;
};

namespace {

int fail(dcns_ctx *ctx, const Error &e) {
  if (ctx) ctx->C.err = e.what();
  return e.code;
}

template <class F>
int guarded(dcns_ctx *ctx, F f) {
  try {
    f();
    return DCNS_OK;
  } catch (const Error &e) {
    return fail(ctx, e);
  } catch (const std::bad_alloc &) {
    if (ctx) ctx->C.err = "host allocation failed";
    return DCNS_ERR_NOMEM;
  } catch (const std::exception &e) {
    if (ctx) ctx->C.err = e.what();
    return DCNS_ERR_DEVICE;
  }
}

std::vector<PairIn> to_pairs(const dcns_pair *pairs, int64_t n) {
  if (n < 0 || (n > 0 && !pairs)) throw Error(DCNS_ERR_INVALID, "bad pair array");
  std::vector<PairIn> v((size_t)n);
  for (int64_t k = 0; k < n; ++k) v[k] = PairIn{pairs[k].seq1, pairs[k].len1, pairs[k].seq2, pairs[k].len2};
  return v;
}

// Predicted device memory of one request: sequence arena and upload staging, level-0 scan keys and window records,
// recursion tasks, and x-drop passes (one per eighth of the windows) with their traceback slots (3 x min(n1, 1024)
// rows of 4-bit band codes) and CIGAR slots (n1 + n2 + 2 words, twice); in 2-gap mode one forward 2-piece DP's
// direction codes (n1 rows of the band, bytes).  A heuristic for admission only: the engine checks the real sizes.
int64_t predict_bytes(int64_t n1, int64_t n2, const Params &P, int mode) {
  const int64_t windows = n2 / std::max(P.step, 1) + 2;
  const int64_t passes = windows / 8 + 1;
  const int64_t wpr = (2 * (int64_t)P.w + 1 + 7) / 8;
  int64_t b = 2 * (n1 + n2) + 96 * windows + passes * (3 * std::min<int64_t>(n1, 1024) * wpr * 4 + 8 * (n1 + n2 + 2));
  if (mode == DCNS_MODE_TWO_GAP) b += n1 * std::min<int64_t>(n2, 2 * (int64_t)P.bandwidth + 160);
  return b + 4096;
}

// Predicted level-0 seed-scan cells of one request (every window against the whole reference).
int64_t predict_cells(int64_t n1, int64_t n2, const Params &P) {
  return n1 * (n2 / std::max(P.step, 1) + 1) * P.window;
}

void worker_loop(std::shared_ptr<Server> Sp, Context *C) {
  Server *S = Sp.get();
  DCNS_CK(cudaSetDevice(C->device));
  for (;;) {
    std::vector<Server::Req> batch;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return !S->running || !S->queue.empty(); });
      if (!S->running && S->queue.empty()) return;
      // admission: arrival order, up to the in-flight limit, the worker's memory budget and the batch's scan cap
      int64_t bytes = 0, cells = 0;
      while (!S->queue.empty() && (int)batch.size() < S->max_inflight) {
        const Server::Req &r = S->queue.front();
        if (!batch.empty() && (bytes + r.bytes > S->admit_bytes || cells + r.cells > S->batch_cells)) break;
        bytes += r.bytes;
        cells += r.cells;
        batch.push_back(std::move(S->queue.front()));
        S->queue.pop_front();
      }
      S->counters.batches += 1;
      S->counters.max_batch = std::max<int64_t>(S->counters.max_batch, (int64_t)batch.size());
    }
    std::vector<PairIn> pairs;
    for (auto &r : batch) pairs.push_back(PairIn{r.s1.data(), (int32_t)r.s1.size(), r.s2.data(), (int32_t)r.s2.size()});
    std::vector<std::pair<size_t, size_t>> parts{{0, pairs.size()}};
    std::set<size_t> retried_alone;
    while (!parts.empty()) {
      auto [a, b] = parts.back();
      parts.pop_back();
      std::vector<PairIn> sub(pairs.begin() + a, pairs.begin() + b);
      std::vector<std::vector<FragOut>> out;
      int code = DCNS_OK;
      std::string err;
      try {
        align_pairs(*C, sub, S->P, S->mode, out);
      } catch (const Error &e) {
        code = e.code;
        err = e.what();
      } catch (const std::bad_alloc &) {
        code = DCNS_ERR_NOMEM;
        err = "host allocation failed";
      } catch (const std::exception &e) {
        code = DCNS_ERR_DEVICE;
        err = e.what();
      }
      if (code == DCNS_ERR_NOMEM) {
        // The worker's buffers only grow, so buffers sized for earlier batches may hold the budget: free them, then
        // halve the batch (a single request is retried once on the freed buffers).
        try {
          release_device_buffers(*C);
        } catch (...) {
        }
        if (b - a == 1 && !retried_alone.count(a)) {
          retried_alone.insert(a);
          parts.push_back({a, b});
          continue;
        }
      }
      if (code != DCNS_OK && b - a > 1) {
        std::lock_guard<std::mutex> lk(S->mu);
        if (code == DCNS_ERR_NOMEM) {  // too large for the device budget: halves
          S->counters.nomem_splits += 1;
          parts.push_back({a + (b - a) / 2, b});
          parts.push_back({a, a + (b - a) / 2});
        } else {  // any other failure: every request alone, so a bad one fails only itself
          S->counters.solo_retries += (int64_t)(b - a);
          for (size_t k = b; k-- > a;) parts.push_back({k, k + 1});
        }
        continue;
      }
      std::lock_guard<std::mutex> lk(S->mu);
      for (size_t k = a; k < b; ++k) {
        const uint64_t t = batch[k].ticket;
        S->pending.erase(t);
        if (S->cancelled.erase(t)) continue;
        if (code != DCNS_OK) {
          S->failed[t] = {code, err};
          S->counters.failed += 1;
        } else {
          auto *R = new ResultsImpl;
          std::vector<std::vector<FragOut>> one{std::move(out[k - a])};
          R->finish(one, C->stats);
          S->done[t] = R;
          S->counters.completed += 1;
        }
      }
      S->cv_done.notify_all();
    }
  }
}

std::shared_ptr<Server> server_of(dcns_ctx *ctx) {
  std::lock_guard<std::mutex> lk(ctx->srv_mu);
  return ctx->srv;
}

// Result of a ticket with the server's lock held.
int poll_locked(dcns_ctx *ctx, Server &S, uint64_t ticket, dcns_results **out) {
  auto it = S.done.find(ticket);
  if (it != S.done.end()) {
    *out = &it->second->pub;
    S.done.erase(it);
    return DCNS_OK;
  }
  auto f = S.failed.find(ticket);
  if (f != S.failed.end()) {
    const int code = f->second.first;
    {
      std::lock_guard<std::mutex> lk(ctx->srv_mu);
      ctx->C.err = f->second.second;
    }
    S.failed.erase(f);
    return code;
  }
  return S.pending.count(ticket) ? DCNS_ERR_BUSY : DCNS_ERR_NOTFOUND;
}

}  // namespace

namespace {
std::vector<std::vector<Seed4>> to_seeds(int64_t n_pairs, const int32_t *seeds, const int64_t *seed_offset) {
  std::vector<std::vector<Seed4>> sd(n_pairs);
  for (int64_t k = 0; k < n_pairs; ++k) {
    if (seed_offset[k + 1] < seed_offset[k] || (seed_offset[k + 1] > seed_offset[k] && !seeds))
      throw Error(DCNS_ERR_INVALID, "bad seed offsets");
    for (int64_t q = seed_offset[k]; q < seed_offset[k + 1]; ++q)
      sd[k].push_back(Seed4{seeds[4 * q], seeds[4 * q + 1], seeds[4 * q + 2], seeds[4 * q + 3]});
  }
  return sd;
}

template <class F>
int seeded_call(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, const int32_t *seeds,
                const int64_t *seed_offset, const dcns_params *params, dcns_results **out, F run) {
  if (!ctx || (n_pairs > 0 && (!pairs || !seed_offset)) || !params || !out || n_pairs < 0) return DCNS_ERR_INVALID;
  *out = nullptr;
  return guarded(ctx, [&] {
    std::vector<PairIn> pv = to_pairs(pairs, n_pairs);
    std::vector<std::vector<Seed4>> sd = to_seeds(n_pairs, seeds, seed_offset);
    std::vector<std::vector<FragOut>> fr;
    run(ctx->C, pv, sd, to_params(params), fr);
    auto *R = new ResultsImpl;
    R->finish(fr, ctx->C.stats);
    *out = &R->pub;
  });
}
}  // namespace

namespace dcns {
int scan_occupancy_impl();
int scan_occupancy() { return scan_occupancy_impl(); }
}  // namespace dcns

extern "C" {

void dcns_params_default(dcns_params *p) {
  if (!p) return;
  p->match = 2;
  p->mismatch = -3;
  p->open1 = -4;
  p->ext1 = -2;
  p->open2 = -45;
  p->ext2 = 0;
  p->window = 38;
  p->min_score = 40;
  p->step = 8;
  p->w = 10;
  p->xdrop = 20;
  p->zdrop = 50;
  p->bandwidth = 20000;
  p->max_align_len = 0;
  p->pvalue = 0.1;
  p->lambda = 0.382291;
  p->kvalue = 0.006662;
}

int dcns_ctx_create(int device, size_t mem_budget, dcns_ctx **out) {
  if (!out) return DCNS_ERR_INVALID;
  *out = nullptr;
  dcns_ctx *ctx = nullptr;
  try {  // nothing escapes the C ABI: allocation and thread failures become status codes too
    ctx = new dcns_ctx;
    init_context(ctx->C, device, mem_budget);
  } catch (const Error &e) {
    delete ctx;
    return e.code;
  } catch (const std::bad_alloc &) {
    delete ctx;
    return DCNS_ERR_NOMEM;
  } catch (const std::exception &) {
    delete ctx;
    return DCNS_ERR_DEVICE;
  }
  *out = ctx;
  return DCNS_OK;
}

void dcns_ctx_destroy(dcns_ctx *ctx) {
  if (!ctx) return;
  dcns_serve_stop(ctx);
  delete ctx;
}

const char *dcns_last_error(const dcns_ctx *ctx) { return ctx ? ctx->C.err.c_str() : "null context"; }

void *dcns_ctx_stream(dcns_ctx *ctx) { return ctx ? (void *)ctx->C.st : nullptr; }

int dcns_align_pairs(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, const dcns_params *params, int mode,
                     dcns_results **out) {
  if (!ctx || !params || !out) return DCNS_ERR_INVALID;
  *out = nullptr;
  return guarded(ctx, [&] {
    std::vector<PairIn> v = to_pairs(pairs, n_pairs);
    std::vector<std::vector<FragOut>> fr;
    align_pairs(ctx->C, v, to_params(params), mode, fr);
    auto *R = new ResultsImpl;
    R->finish(fr, ctx->C.stats);
    *out = &R->pub;
  });
}

void dcns_results_free(dcns_results *res) { delete reinterpret_cast<ResultsImpl *>(res); }

int dcns_align_weighted(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, const int16_t *weights,
                        const int32_t *cats, int32_t n_cats, int pieces, const dcns_params *params,
                        dcns_results **out) {
  if (!ctx || (n_pairs > 0 && !pairs) || !params || !out || n_pairs < 0 || n_cats < 1 || !cats)
    return DCNS_ERR_INVALID;
  *out = nullptr;
  return guarded(ctx, [&] {
    std::vector<PairIn> pv = to_pairs(pairs, n_pairs);
    std::vector<const int16_t *> wp(n_pairs);
    int64_t off = 0;
    for (int64_t k = 0; k < n_pairs; ++k) {
      if (pv[k].n1 > 0 && !weights) throw Error(DCNS_ERR_INVALID, "NULL weights");
      wp[k] = weights ? weights + off : nullptr;
      off += std::max(pv[k].n1, 0);
    }
    std::vector<int32_t> cv(cats, cats + 7 * (int64_t)n_cats);
    std::vector<std::vector<FragOut>> fr;
    align_weighted(ctx->C, pv, wp, cv, pieces, to_params(params), fr);
    auto *R = new ResultsImpl;
    R->finish(fr, ctx->C.stats);
    *out = &R->pub;
  });
}


int dcns_align_seeded(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, const int32_t *seeds,
                      const int64_t *seed_offset, const dcns_params *params, dcns_results **out) {
  return seeded_call(ctx, pairs, n_pairs, seeds, seed_offset, params, out, align_seeded);
}

int dcns_align_xseeds(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, const int32_t *seeds,
                      const int64_t *seed_offset, const dcns_params *params, dcns_results **out) {
  return seeded_call(ctx, pairs, n_pairs, seeds, seed_offset, params, out, align_xseeds);
}

int dcns_batch_upload(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, dcns_batch **out) {
  if (!ctx || !out) return DCNS_ERR_INVALID;
  *out = nullptr;
  auto *b = new dcns_batch;
  int rc = guarded(ctx, [&] { batch_upload(ctx->C, to_pairs(pairs, n_pairs), b->B); });
  if (rc != DCNS_OK) {
    dcns_batch_free(ctx, b);
    return rc;
  }
  *out = b;
  return DCNS_OK;
}

int dcns_align_batch(dcns_ctx *ctx, dcns_batch *batch, const dcns_params *params, int mode, dcns_results **out) {
  if (!ctx || !batch || !params || !out) return DCNS_ERR_INVALID;
  *out = nullptr;
  return guarded(ctx, [&] {
    std::vector<std::vector<FragOut>> fr;
    align_batch(ctx->C, batch->B, to_params(params), mode, fr);
    auto *R = new ResultsImpl;
    R->finish(fr, ctx->C.stats);
    *out = &R->pub;
  });
}

void dcns_batch_free(dcns_ctx *ctx, dcns_batch *batch) {
  if (!batch) return;
  if (ctx) {
    batch->B.pk.release(ctx->C);
    batch->B.nm.release(ctx->C);
    batch->B.sb.release(ctx->C);
  }
  delete batch;
}

int dcns_measure_scan_roofline(dcns_ctx *ctx, double *gcups) {
  if (!ctx || !gcups) return DCNS_ERR_INVALID;
  return guarded(ctx, [&] {
    const double pairs_per_s = measure_issue_rate(ctx->C.nsm, ctx->C.st);
    DCNS_CK(cudaGetLastError());
    *gcups = 2.0 * pairs_per_s / 1e9;
  });
}

int dcns_ctx_set_lanes(dcns_ctx *ctx, int lanes, int bins) {
  if (!ctx || lanes < 1 || lanes > 8 || bins < 1 || bins > 64) return DCNS_ERR_INVALID;
  ctx->C.max_lanes = lanes;
  ctx->C.bins = bins;
  return DCNS_OK;
}

int dcns_autotune(dcns_ctx *ctx, dcns_batch *batch, const dcns_params *params, int mode, int *lanes, int *bins,
                  double *bin_ratio) {
  if (!ctx || !batch || !params) return DCNS_ERR_INVALID;
  return guarded(ctx, [&] {
    autotune(ctx->C, batch->B, to_params(params), mode);
    if (lanes) *lanes = ctx->C.max_lanes;
    if (bins) *bins = ctx->C.bins;
    if (bin_ratio) *bin_ratio = ctx->C.bin_ratio;
  });
}

int dcns_get_tuning(const dcns_ctx *ctx, dcns_tuning *out) {
  if (!ctx || !out) return DCNS_ERR_INVALID;
  const Context &C = ctx->C;
  *out = dcns_tuning{};
  out->lanes = C.max_lanes;
  out->bins = C.bins;
  out->bin_ratio = C.bin_ratio;
  out->scan_tiles_per_thread = C.scan_tiles_per_thread;
  out->sg_warps = C.sg_warps;
  out->sg_flow = C.sg_flow ? 1 : 0;
  out->sg_flow_blocks = C.sg_flow_blocks;
  out->bins_by_size = C.bins_by_size ? 1 : 0;
  out->n_bins_tuned = (int32_t)std::min<size_t>(C.bin_tune.size(), 16);
  for (int b = 0; b < 16; ++b) {
    const bool own = b < (int)C.bin_tune.size();
    out->xdrop_warp_from[b] = own ? C.bin_tune[b].xdrop_warp_from : C.xdrop_warp_from;
    out->xdrop_wave_max_w[b] = own ? C.bin_tune[b].xdrop_wave_max_w : C.xdrop_wave_max_w;
    out->xdrop_flat[b] = (own ? C.bin_tune[b].xdrop_flat : C.xdrop_flat) ? 1 : 0;
    out->xdrop_handoff[b] = own ? C.bin_tune[b].xdrop_handoff : C.xdrop_handoff;
    out->xdrop_resume_lanes[b] = own ? C.bin_tune[b].xdrop_resume_lanes : C.xdrop_resume_lanes;
    out->xdrop_group_from[b] = own ? C.bin_tune[b].xdrop_group_from : C.xdrop_group_from;
    out->scan_tiles[b] = own ? C.bin_tune[b].scan_tiles : C.scan_tiles_per_thread;
  }
  return DCNS_OK;
}

int dcns_last_stats(const dcns_ctx *ctx, dcns_stats *out) {
  if (!ctx || !out) return DCNS_ERR_INVALID;
  *out = ctx->C.stats;
  return DCNS_OK;
}

int dcns_smith_waterman_batch(dcns_ctx *ctx, const dcns_pair *tasks, int64_t n, const dcns_params *params,
                              int32_t *out) {
  if (!ctx || !params || (n > 0 && !out)) return DCNS_ERR_INVALID;
  return guarded(ctx, [&] { smith_waterman_batch(ctx->C, to_pairs(tasks, n), to_params(params), out); });
}

static int copy_cigars(const std::vector<std::vector<uint32_t>> &cg, uint32_t *cigar, int64_t cap, int64_t *off) {
  int64_t tot = 0;
  for (auto &c : cg) tot += (int64_t)c.size();
  if (off) {
    off[0] = 0;
    for (size_t k = 0; k < cg.size(); ++k) off[k + 1] = off[k] + (int64_t)cg[k].size();
  }
  if (!cigar) return DCNS_OK;
  if (tot > cap) return DCNS_ERR_NOMEM;
  int64_t c = 0;
  for (auto &v : cg) {
    std::memcpy(cigar + c, v.data(), v.size() * sizeof(uint32_t));
    c += (int64_t)v.size();
  }
  return DCNS_OK;
}

int dcns_xextend_batch(dcns_ctx *ctx, const dcns_pair *tasks, int64_t n, const dcns_params *params, int want_cigar,
                       int32_t *out, uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_offset) {
  if (!ctx || !params || (n > 0 && !out)) return DCNS_ERR_INVALID;
  std::vector<uint32_t> cg;
  std::vector<int64_t> off;
  int rc = guarded(ctx, [&] {
    xextend_batch(ctx->C, to_pairs(tasks, n), to_params(params), want_cigar != 0, out, cg, off);
  });
  if (rc != DCNS_OK) return rc;
  if (cigar_offset) std::memcpy(cigar_offset, off.data(), sizeof(int64_t) * off.size());
  if (!cigar) return DCNS_OK;
  if ((int64_t)cg.size() > cigar_cap) return DCNS_ERR_NOMEM;
  if (!cg.empty()) std::memcpy(cigar, cg.data(), sizeof(uint32_t) * cg.size());
  return DCNS_OK;
}

int dcns_semiglobal_batch(dcns_ctx *ctx, const dcns_pair *tasks, int64_t n, const dcns_params *params,
                          int want_cigar, int32_t *out, uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_offset) {
  if (!ctx || !params || (n > 0 && !out)) return DCNS_ERR_INVALID;
  std::vector<std::vector<uint32_t>> cg;
  int rc =
      guarded(ctx, [&] { semiglobal_batch(ctx->C, to_pairs(tasks, n), to_params(params), want_cigar != 0, out, cg); });
  if (rc != DCNS_OK) return rc;
  return copy_cigars(cg, cigar, cigar_cap, cigar_offset);
}

int dcns_sliding_window(dcns_ctx *ctx, const int8_t *const *seqs, const int32_t *lens, int32_t n_seqs,
                        const dcns_params *params, double *score, int32_t *max_out) {
  if (!ctx || !params || !seqs || !lens || n_seqs < 1 || !score || !max_out) return DCNS_ERR_INVALID;
  return guarded(ctx, [&] { sliding_window(ctx->C, seqs, lens, n_seqs, to_params(params), score, max_out); });
}

int dcns_serve_set_shape(dcns_ctx *ctx, int workers, int64_t batch_cells, int64_t admit_bytes) {
  if (!ctx || workers < 1 || workers > 8 || batch_cells < 0 || admit_bytes < 0) return DCNS_ERR_INVALID;
  ctx->serve_workers = workers;
  ctx->serve_batch_cells = batch_cells;
  ctx->serve_admit_bytes = admit_bytes;
  return DCNS_OK;
}

int dcns_serve_start(dcns_ctx *ctx, const dcns_params *params, int mode, int max_inflight_pairs) {
  if (!ctx || !params) return DCNS_ERR_INVALID;
  if (server_of(ctx)) return DCNS_ERR_BUSY;
  return guarded(ctx, [&] {
    Params P = to_params(params);
    validate(P);
    if (mode != DCNS_MODE_ONE_GAP && mode != DCNS_MODE_TWO_GAP) throw Error(DCNS_ERR_INVALID, "bad mode");
    auto S = std::make_shared<Server>();
    S->P = P;
    S->mode = mode;
    S->max_inflight = max_inflight_pairs > 0 ? max_inflight_pairs : 256;
    // default scan cap: about 25 ms of level-0 scan at the batched rate (1e11 cells)
    S->batch_cells = ctx->serve_batch_cells > 0 ? ctx->serve_batch_cells : (int64_t)100000000000LL;
    S->running = true;
    int nlanes = ctx->serve_workers;
    if (const char *e = std::getenv("DCNS_SERVE_WORKERS")) nlanes = std::max(1, std::min(8, std::atoi(e)));
    const size_t lane_budget = ctx->C.budget / (size_t)nlanes;
    S->admit_bytes = ctx->serve_admit_bytes > 0 ? ctx->serve_admit_bytes : (int64_t)lane_budget;
    for (int k = 0; k < nlanes; ++k) {
      auto L = std::make_unique<Context>();
      init_context(*L, ctx->C.device, lane_budget);
      S->lanes.push_back(std::move(L));
    }
    for (auto &L : S->lanes) S->workers.emplace_back(worker_loop, S, L.get());
    std::lock_guard<std::mutex> lk(ctx->srv_mu);
    ctx->srv = std::move(S);
  });
}

int dcns_submit(dcns_ctx *ctx, const dcns_pair *pair, uint64_t *ticket) {
  if (!ctx || !pair || !ticket) return DCNS_ERR_INVALID;
  std::shared_ptr<Server> Sp = server_of(ctx);
  if (!Sp) return DCNS_ERR_INVALID;
  if (pair->len1 < 0 || pair->len2 < 0 || (pair->len1 && !pair->seq1) || (pair->len2 && !pair->seq2))
    return DCNS_ERR_INVALID;
  if (pair->len1 >= kMaxSeqLen || pair->len2 >= kMaxSeqLen) return DCNS_ERR_INVALID;
  for (int h = 0; h < 2; ++h) {  // a code outside 0..4 is rejected here, before it can share a batch
    const int8_t *q = h ? pair->seq2 : pair->seq1;
    const int32_t n = h ? pair->len2 : pair->len1;
    uint8_t bad = 0;
    for (int32_t i = 0; i < n; ++i) bad |= (uint8_t)((uint8_t)q[i] > 4);
    if (bad) return DCNS_ERR_INVALID;
  }
  Server &S = *Sp;
  return guarded(ctx, [&] {
    Server::Req r;
    r.s1.assign(pair->seq1, pair->seq1 + pair->len1);
    r.s2.assign(pair->seq2, pair->seq2 + pair->len2);
    r.bytes = predict_bytes(pair->len1, pair->len2, S.P, S.mode);
    r.cells = predict_cells(pair->len1, pair->len2, S.P);
    {
      std::lock_guard<std::mutex> lk(S.mu);
      if (!S.running) throw Error(DCNS_ERR_INVALID, "the serving loop is stopping");
      r.ticket = S.next++;
      *ticket = r.ticket;
      S.pending.insert(r.ticket);
      S.counters.submitted += 1;
      S.queue.push_back(std::move(r));
    }
    S.cv_work.notify_one();
  });
}

int dcns_poll(dcns_ctx *ctx, uint64_t ticket, dcns_results **out) {
  if (!ctx || !out) return DCNS_ERR_INVALID;
  *out = nullptr;
  std::shared_ptr<Server> Sp = server_of(ctx);
  if (!Sp) return DCNS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(Sp->mu);
  return poll_locked(ctx, *Sp, ticket, out);
}

int dcns_serve_wait(dcns_ctx *ctx, uint64_t ticket, int64_t timeout_ms, dcns_results **out) {
  if (!ctx || !out) return DCNS_ERR_INVALID;
  *out = nullptr;
  std::shared_ptr<Server> Sp = server_of(ctx);
  if (!Sp) return DCNS_ERR_INVALID;
  Server &S = *Sp;
  // at most about 30 days, so that the deadline cannot overflow the clock
  const int64_t ms = std::max<int64_t>(0, std::min<int64_t>(timeout_ms, (int64_t)1 << 31));
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(ms);
  std::unique_lock<std::mutex> lk(S.mu);
  if (!S.cv_done.wait_until(lk, deadline, [&] { return !S.pending.count(ticket) || S.stopped; }))
    return DCNS_ERR_TIMEOUT;
  return poll_locked(ctx, S, ticket, out);
}

int dcns_cancel(dcns_ctx *ctx, uint64_t ticket) {
  if (!ctx) return DCNS_ERR_INVALID;
  std::shared_ptr<Server> Sp = server_of(ctx);
  if (!Sp) return DCNS_ERR_INVALID;
  Server &S = *Sp;
  std::lock_guard<std::mutex> lk(S.mu);
  if (!S.pending.count(ticket)) return DCNS_ERR_NOTFOUND;
  S.pending.erase(ticket);
  S.counters.cancelled += 1;
  for (auto it = S.queue.begin(); it != S.queue.end(); ++it)
    if (it->ticket == ticket) {
      S.queue.erase(it);
      S.cv_done.notify_all();
      return DCNS_OK;
    }
  S.cancelled.insert(ticket);  // being aligned: its result is dropped when the batch ends
  S.cv_done.notify_all();
  return DCNS_OK;
}

int dcns_serve_stats(dcns_ctx *ctx, dcns_serving_stats *out) {
  if (!ctx || !out) return DCNS_ERR_INVALID;
  std::shared_ptr<Server> Sp = server_of(ctx);
  if (!Sp) return DCNS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(Sp->mu);
  *out = Sp->counters;
  out->queued = (int64_t)Sp->queue.size();
  out->pending = (int64_t)Sp->pending.size();
  out->workers = (int32_t)Sp->workers.size();
  return DCNS_OK;
}

int dcns_serve_stop(dcns_ctx *ctx) {
  if (!ctx) return DCNS_OK;
  std::shared_ptr<Server> Sp;
  {
    std::lock_guard<std::mutex> lk(ctx->srv_mu);
    Sp = std::move(ctx->srv);
    ctx->srv.reset();
  }
  if (!Sp) return DCNS_OK;
  {
    std::lock_guard<std::mutex> lk(Sp->mu);
    Sp->running = false;
  }
  Sp->cv_work.notify_all();
  for (auto &t : Sp->workers) t.join();  // the queue is drained first
  {
    std::lock_guard<std::mutex> lk(Sp->mu);
    Sp->stopped = true;
  }
  Sp->cv_done.notify_all();  // waiters return; the server is freed with the last reference
  return DCNS_OK;
}

}  // extern "C"
