/* dcns_gb300 — C ABI of the GB300 pairwise CNS alignment engine (one process, one GPU).
 *
 * Drop-in boundary for dCNS's pairwise conserved-sequence alignment path.  Each entry point replaces one reference
 * interface (paths inside the dCNS project):
 *
 *   dcns_align_pairs(..., DCNS_MODE_ONE_GAP)   findSimilarFragmentsForPairedSequence, 1-gap overload
 *                                              impl/findSimilarFragmentsForPairedSequence.h:26-32
 *                                              (impl/findSimilarFragmentsForPairedSequence4.cpp:433; called by
 *                                              cut1Gap controlLayer4.cpp:1411, pairCnsXExtend :212, multCns
 *                                              impl/getCnsForMultipleSpecies.cpp:135)
 *   dcns_align_pairs(..., DCNS_MODE_TWO_GAP)   findSimilarFragmentsForPairedSequence, 2-gap overload
 *                                              impl/findSimilarFragmentsForPairedSequence.h:34-42
 *                                              (impl/findSimilarFragmentsForPairedSequence4.cpp:752; cut2Gaps
 *                                              controlLayer4.cpp:1584, pairCns2Gaps :355)
 *   dcns_smith_waterman_batch                  SmithWaterman(..., bool &positions)  impl/sequenceAlignment.h:26-28
 *   dcns_xextend_batch                         SemiGlobal_xextend (both overloads)  impl/sequenceAlignment.h:72-81
 *   dcns_semiglobal_batch                      SemiGlobal (2-piece affine)          impl/sequenceAlignment.h:52-56
 *   dcns_sliding_window                        slidingWindowAlignment    impl/slidingWindowAlignment.h:21-24
 *   dcns_align_weighted                        findSimilarFragmentsForPairedSequence_wighted / _wighted_1gap
 *                                              impl/findSimilarFragmentsForPairedSequence.h:45-61
 *   dcns_align_xseeds                          the x-seed overload, impl/findSimilarFragmentsForPairedSequence.h:70-77
 *   dcns_align_seeded                          the x-seed overload with maximumAlignLength (cut2Gaps2)
 *                                              impl/findSimilarFragmentsForPairedSequence.h:79-86
 *
 * Sequences cross the boundary as dCNS integer codes (int8: A=0 C=1 N=2 G=3 T=4, the output of
 * SequenceCharToUInt8::seq_to_int8, with lower-case 'n' already removed as the reference's drivers do); reverse
 * complements are derived on the device.  All pointers are host pointers owned by the caller unless stated.
 * Fragment coordinates are 1-based and CIGAR words are packed (length << 4 | op), op 0=M 1=I 2=D, exactly as
 * PairedSimilarFragment (model/PairedSimilarFragment.h:14-68).
 *
 * Errors: every call returns DCNS_OK (0) or a negative status; dcns_last_error() describes the last failure of the
 * context.  There is no CPU fallback: without a usable GPU, dcns_ctx_create fails with DCNS_ERR_DEVICE.
 * Threading: a context is single-stream and thread-compatible (one host thread per context at a time).
 */
#ifndef DCNS_GB300_H
#define DCNS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DCNS_OK 0
#define DCNS_ERR_INVALID (-1)   /* bad argument (codes outside 0..4, unsupported parameter range, NULL) */
#define DCNS_ERR_NOMEM (-2)     /* device memory or memory budget exhausted */
#define DCNS_ERR_DEVICE (-3)    /* CUDA error or no device */
#define DCNS_ERR_TIMEOUT (-4)   /* a serving request did not finish in time */
#define DCNS_ERR_NOTFOUND (-5)  /* unknown request ticket */
#define DCNS_ERR_BUSY (-6)      /* serving queue full */

#define DCNS_MODE_ONE_GAP 1
#define DCNS_MODE_TWO_GAP 2

typedef struct dcns_ctx dcns_ctx;

/* Scoring and search parameters; defaults (dcns_params_default) are the reference's globals, controlLayer4.cpp:28-52. */
typedef struct {
  int32_t match, mismatch;          /* 2, -3 */
  int32_t open1, ext1;              /* -4, -2 */
  int32_t open2, ext2;              /* -45, 0  (second gap piece; 2-gap mode only) */
  int32_t window, min_score, step;  /* 38, 40, 8 */
  int32_t w, xdrop;                 /* 10, 20   x-drop band half-width and drop */
  int32_t zdrop, bandwidth;         /* 50, 20000 */
  int32_t max_align_len;            /* 0 = unlimited (cut2Gaps2's maximumAlignLength) */
  double pvalue, lambda, kvalue;    /* 0.1, 0.382291, 0.006662 */
} dcns_params;

typedef struct {
  const int8_t *seq1; /* reference codes */
  int32_t len1;
  const int8_t *seq2; /* query codes */
  int32_t len2;
} dcns_pair;

/* Algorithmic DP cells (counted identically for CPU and GPU) and stage timings of the last call. */
typedef struct {
  int64_t cells_scan, cells_scan_reverse, cells_xdrop, cells_semiglobal;
  int64_t tasks_scan, tasks_scan_speculative, seeds, xdrop_passes, semiglobal_dps;
  double ms_upload, ms_scan, ms_replay, ms_xdrop, ms_semiglobal, ms_download, ms_total;
  double ms_scan_kernel;  /* device time of the seed-scan kernel launches (CUDA events) */
  double ms_scan_prep;    /* host: task and tile generation */
  double ms_scan_xfer;    /* task/tile/result transfers and the synchronising wait of the scan rounds */
  double ms_link;         /* host: link_seeds */
  int32_t scan_launches, kernel_launches;
  int32_t scan_rounds;     /* seed-scan launches rounds (level 0 + recursion levels), summed over lanes */
  int32_t xdrop_rounds;    /* x-drop launch rounds (band restarts), summed over lanes */
  double ms_xdrop_kernel;  /* device: x-drop pass kernels, CUDA events */
  int64_t bytes_h2d;       /* host-to-device bytes of the sequence upload (codes and per-sequence offsets) */
  double ms_xdrop_tb_kernel;  /* device: x-drop traceback and CIGAR packing kernels, CUDA events */
  double ms_sg_kernel;        /* device: semi-global DP kernels, CUDA events */
  double ms_sg_tb_kernel;     /* device: semi-global traceback kernels, CUDA events */
  int64_t bytes_codes_xdrop;  /* direction codes of the final-width x-drop passes that kept them: 4 bits per band cell */
  int64_t bytes_codes_sg;     /* direction codes of the semi-global DPs that kept them: 1 byte per band cell */
  int64_t bytes_device;       /* device memory the context's buffers hold after the call (they are kept for reuse) */
} dcns_stats;

/* Results of one dcns_align_pairs call; owned by the library until dcns_results_free. */
typedef struct {
  int64_t n_pairs, n_fragments, n_cigar;
  const int64_t *pair_offset;  /* [n_pairs + 1]: fragments of pair k are [pair_offset[k], pair_offset[k+1]) */
  const int64_t *frag;         /* [n_fragments * 7]: start1, end1, start2, end2, score, cigar_offset, cigar_len */
  const double *pvalue;        /* [n_fragments] */
  const double *evalue;        /* [n_fragments] */
  const uint32_t *cigar;       /* [n_cigar] */
  dcns_stats stats;
} dcns_results;

void dcns_params_default(dcns_params *p);

/* device: CUDA ordinal.  mem_budget: bytes of device memory the context may hold (0 = 80% of free memory). */
int dcns_ctx_create(int device, size_t mem_budget, dcns_ctx **out);
void dcns_ctx_destroy(dcns_ctx *ctx);
const char *dcns_last_error(const dcns_ctx *ctx);
/* The CUDA stream (cudaStream_t) all of the context's work is issued on. */
void *dcns_ctx_stream(dcns_ctx *ctx);

/* Batched pair alignment: every pair is aligned independently, as one call of the reference overload per pair. */
int dcns_align_pairs(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, const dcns_params *params, int mode,
                     dcns_results **out);
void dcns_results_free(dcns_results *res);

/* The weighted drivers of weighted1Gap / weighted2Gaps (findSimilarFragmentsForPairedSequence_wighted_1gap,
 * impl/findSimilarFragmentsForPairedSequence4.cpp:784, pieces = 1; findSimilarFragmentsForPairedSequence_wighted, :883,
 * pieces = 2) for many pairs: the 2-gap x-seeds, then per x-seed the weighted reverse and forward DPs
 * (impl/sequenceAlignment3.cpp:1483-1890) whose rows score with the category of their seq1 base.  weights: n1 category
 * ids (0 .. n_cats-1) per pair, concatenated in pair order; cats: 7 int32 per category, as a Score folder file holds
 * them (model/Score.cpp:3-60): match, mismatch, open1, ext1, open2, ext2, zdrop.  At most 64 categories.  The DP
 * bandwidth is params->bandwidth; the z-drop of each row comes from its category. */
int dcns_align_weighted(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, const int16_t *weights,
                        const int32_t *cats, int32_t n_cats, int pieces, const dcns_params *params,
                        dcns_results **out);

/* The seeded 2-gap overload of cut2Gaps2 (impl/findSimilarFragmentsForPairedSequence4.cpp:624-745; the x-seeds come
 * from a SAM file, impl/samFileToSeeds.cpp) for many pairs: seeds are (start1, end1, start2, end2) quadruples,
 * 0-based inclusive, pair k owning seeds[4*seed_offset[k] .. 4*seed_offset[k+1]), in the caller's order.
 * params->max_align_len (maximumAlignLength; 0 = unlimited) caps every DP's lengths; no p-value filter. */
int dcns_align_seeded(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, const int32_t *seeds,
                      const int64_t *seed_offset, const dcns_params *params, dcns_results **out);

/* The x-seed overload without maximumAlignLength (impl/findSimilarFragmentsForPairedSequence.h:70-77,
 * impl/findSimilarFragmentsForPairedSequence4.cpp:532-616; the 2-gap overload runs it on its own x-seeds) for many
 * pairs: per x-seed a reverse 2-piece DP from its end, the StartAlignment gate, a forward 2-piece DP with CIGAR and
 * the dedupe by end; no p-value filter, no length cap.  Seeds and offsets as for dcns_align_seeded. */
int dcns_align_xseeds(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, const int32_t *seeds,
                      const int64_t *seed_offset, const dcns_params *params, dcns_results **out);

/* x-seeds of cut2Gaps2 from SAM text (samFileToSeeds, impl/samFileToSeeds.cpp:19-141): the reference and query
 * genomes are given by name with their texts (still holding lower-case 'n' runs).  *seeds receives a malloc'ed array
 * (free with dcns_free_seeds) of *n_seeds records of 7 int32 in line order: reference index, query index (-1 when the
 * name is not among the given ones), strand (0: flag 0, 1: any other flag), start1, end1, start2, end2 (0-based, on
 * the sequences with 'n' removed; the query coordinates of strand 1 on its reverse complement). */
int dcns_sam_to_seeds(const char *sam, int64_t sam_len, int n_ref, const char *const *ref_names,
                      const char *const *ref_texts, const int64_t *ref_lens, int n_qry, const char *const *qry_names,
                      const char *const *qry_texts, const int64_t *qry_lens, int32_t **seeds, int64_t *n_seeds);
void dcns_free_seeds(int32_t *seeds);

/* Resident batches: dcns_batch_upload packs the pairs into device memory once; dcns_align_batch then runs the
 * pipeline on the resident sequences (no sequence upload).  A batch belongs to the context that made it. */
typedef struct dcns_batch dcns_batch;
int dcns_batch_upload(dcns_ctx *ctx, const dcns_pair *pairs, int64_t n_pairs, dcns_batch **out);
int dcns_align_batch(dcns_ctx *ctx, dcns_batch *batch, const dcns_params *params, int mode, dcns_results **out);
void dcns_batch_free(dcns_ctx *ctx, dcns_batch *batch);

/* Diagnostic: the integer-issue roofline of the seed scan on this device, measured live: the scan's exact per-cell
 * instruction sequence (int16x2, two cells per instruction) run on independent chains at full occupancy.  Returns
 * the GCUPS ceiling for that instruction mix at the clock the GPU ran during the probe. */
int dcns_measure_scan_roofline(dcns_ctx *ctx, double *gcups);

/* Tuning (no counterpart in the reference): batches of at least 4096 pairs are split into `bins` bins of similar
 * work run by `lanes` concurrent lanes, each with its own stream and buffers, so host-side seed replay of one bin
 * overlaps kernels of another.  lanes = 1 runs every batch as one piece.  Defaults 4 and 4; the environment variables
 * DCNS_LANES and DCNS_BINS override them when a context is created.  Results do not depend on either value. */
int dcns_ctx_set_lanes(dcns_ctx *ctx, int lanes, int bins);

/* Autotuner (no counterpart in the reference): aligns the resident batch once per candidate pipeline shape (lanes,
 * bins, and the geometric ratio of bin sizes), times each call, and keeps the fastest on the context; then, per bin,
 * the x-drop pass forms by that bin's x-drop kernel time, and by whole-call time the seed scan's tiling target and
 * (2-gap mode) the 2-piece kernel's warps per DP (dcns_get_tuning reports them).  The pipeline shape is returned (any
 * pointer may be NULL).  Results do not depend on any of these; this only tunes throughput for batches like this. */
int dcns_autotune(dcns_ctx *ctx, dcns_batch *batch, const dcns_params *params, int mode, int *lanes, int *bins,
                  double *bin_ratio);

/* The context's kernel shapes (no counterpart in the reference): what dcns_autotune chose, or the defaults and the
 * DCNS_* environment settings.  Per bin (at most 16 reported): the x-drop band from which passes run one warp each,
 * the widest band of the one-warp wavefront form, whether the register-band levels run row-interleaved, the rows
 * after which a register-band pass moves to the wavefront form (0: never), and the lanes per such pass (8, 16, 32). */
typedef struct {
  int32_t lanes, bins;
  double bin_ratio;
  int32_t scan_tiles_per_thread;  /* seed-scan tiling target: rows split into chunks below this many tiles per thread */
  int32_t sg_warps;               /* warps per 2-piece DP when one CTA runs a DP (0: two for launches of many DPs,
                                     else eight) */
  int32_t sg_flow;                /* 1: 2-piece DPs run as a flow of 128-row stripe units over one persistent grid */
  int32_t sg_flow_blocks;         /* resident blocks per SM of that grid: 5 or 6 */
  int32_t bins_by_size;           /* 1: bins are runs of pairs in increasing size (the largest last); 0: mixed */
  int32_t n_bins_tuned;           /* bins with their own x-drop forms below (0: every bin uses bin 0's values) */
  int32_t xdrop_warp_from[16], xdrop_wave_max_w[16], xdrop_flat[16], xdrop_handoff[16], xdrop_resume_lanes[16];
  int32_t xdrop_group_from[16]; /* register-band levels of this band and wider: every pass on lane groups (0: off) */
  int32_t scan_tiles[16];       /* each bin's seed-scan tiling target */
} dcns_tuning;
int dcns_get_tuning(const dcns_ctx *ctx, dcns_tuning *out);

/* Stats of the context's last dcns_align_pairs call. */
int dcns_last_stats(const dcns_ctx *ctx, dcns_stats *out);

/* SmithWaterman(ref, read, ...) for n independent (ref, read) tasks.  out[3*k] = maxScore, out[3*k+1..2] = the
 * 0-based first argmax (endPosition1, endPosition2); positions are -1 when maxScore is 0. */
int dcns_smith_waterman_batch(dcns_ctx *ctx, const dcns_pair *tasks, int64_t n, const dcns_params *params,
                              int32_t *out);

/* SemiGlobal_xextend for n (seq1, seq2) tasks with the params' w and xdrop.  out[6*k..] = maxScore, endPosition1,
 * endPosition2 (0-based), iii, jjj, cigar_len.  With want_cigar, CIGAR words go to cigar[cigar_offset[k] ..] where
 * cigar_offset (n+1 entries) is filled by the call; cigar_cap bounds the total (DCNS_ERR_NOMEM when exceeded). */
int dcns_xextend_batch(dcns_ctx *ctx, const dcns_pair *tasks, int64_t n, const dcns_params *params, int want_cigar,
                       int32_t *out, uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_offset);

/* SemiGlobal (2-piece affine, z-drop, band) for n tasks.  out[4*k..] = maxScore, endPosition1, endPosition2,
 * cigar_len; CIGAR layout as for dcns_xextend_batch. */
int dcns_semiglobal_batch(dcns_ctx *ctx, const dcns_pair *tasks, int64_t n, const dcns_params *params,
                          int want_cigar, int32_t *out, uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_offset);

/* slidingWindowAlignment for one reference (seqs[0]) against n_seqs-1 others: for window k (start k*step) and
 * sequence i, score[(i-1) * n_windows + k] = maxScore / (min(window_len, len_i) * match) and max_out the integer
 * maxima.  n_windows = ceil(len_0 / step); both outputs are caller-allocated. */
int dcns_sliding_window(dcns_ctx *ctx, const int8_t *const *seqs, const int32_t *lens, int32_t n_seqs,
                        const dcns_params *params, double *score, int32_t *max_out);

/* No counterpart in the reference.  SemiGlobal's score and end position (the 2-piece affine DP of
 * dcns_semiglobal_batch without CIGAR) for one pair, for callers that must not allocate device memory at call time:
 * processes whose device memory belongs to another allocator or budget, and latency-bound threads that cannot afford
 * the device-wide synchronisation of cudaMalloc/cudaFree.  The caller passes device buffers: the two code sequences
 * (at most 16384 bases each; longer inputs return DCNS_ERR_INVALID) and d_out (4 int32: maxScore, endPosition1,
 * endPosition2 (0-based), status 0 ok / 1 a code outside 0..4).  Parameters are checked as dcns_semiglobal_batch
 * checks them (DCNS_ERR_INVALID for the same values).  Work is queued on `stream` (a cudaStream_t; NULL = the legacy
 * default stream); read d_out after synchronising it.  All scratch is one fixed device array of about 1.6 MB per GPU
 * that holds the library, shared by every call: calls that overlap on the GPU race, calls ordered on one stream do
 * not.  The first call on each device resolves the array's address (cudaGetSymbolAddress, with that device current);
 * make it before any stream capture.  A CUDA error still pending in the calling thread from earlier work makes the
 * call return DCNS_ERR_DEVICE without queueing anything, and leaves that error in place for its owner. */
int dcns_semiglobal_noalloc(const int8_t *d_seq1, int32_t len1, const int8_t *d_seq2, int32_t len2,
                            const dcns_params *params, int32_t *d_out, void *stream);

/* Serving loop (no counterpart in the reference, whose drivers align one pair per call): continuous batching.
 * dcns_submit checks and copies the pair and returns a ticket at once (DCNS_ERR_INVALID for codes outside 0..4).
 * Workers, each with its own stream and device buffers, admit queued requests in arrival order into a batch while
 * the batch's predicted device memory (sequence arena, scan records, x-drop traceback and CIGAR slots, 2-piece
 * direction codes) fits the worker's share of the context budget and its predicted seed-scan cells stay under the
 * batch cap (at most max_inflight_pairs requests); a worker admits new requests as soon as it finishes its batch,
 * while the other workers' batches run.  A batch the device budget rejects is halved; a batch that fails otherwise is
 * retried one request at a time, so a failing request fails only itself (its status is returned by poll / wait).
 * dcns_poll returns DCNS_OK with the result when done, DCNS_ERR_BUSY while pending, DCNS_ERR_NOTFOUND for unknown,
 * collected or cancelled tickets.  dcns_serve_wait blocks up to timeout_ms (DCNS_ERR_TIMEOUT).  dcns_cancel removes a
 * queued request, or drops the result of one being aligned.  dcns_serve_stop aligns what is queued, ends the workers
 * and wakes every waiter; it may overlap submit / poll / wait / cancel calls on other threads (those return
 * DCNS_ERR_INVALID, or what is known of their ticket, once it has run).  Serving calls are thread-safe with one
 * another; dcns_ctx_destroy must not overlap any call on the context. */
int dcns_serve_start(dcns_ctx *ctx, const dcns_params *params, int mode, int max_inflight_pairs);
int dcns_submit(dcns_ctx *ctx, const dcns_pair *pair, uint64_t *ticket);
int dcns_poll(dcns_ctx *ctx, uint64_t ticket, dcns_results **out);
int dcns_serve_wait(dcns_ctx *ctx, uint64_t ticket, int64_t timeout_ms, dcns_results **out);
int dcns_cancel(dcns_ctx *ctx, uint64_t ticket);
int dcns_serve_stop(dcns_ctx *ctx);
/* Shape of the next dcns_serve_start: workers (1..8, default 3; DCNS_SERVE_WORKERS overrides), the batch cap in
 * predicted level-0 seed-scan cells (0 = the default, 1e11, about 25 ms of scan) and in predicted device bytes
 * (0 = the worker's share of the context budget; larger values let the device budget's own check split batches).
 * Results do not depend on any of them. */
int dcns_serve_set_shape(dcns_ctx *ctx, int workers, int64_t batch_cells, int64_t admit_bytes);

/* Counters of the serving loop since dcns_serve_start. */
typedef struct {
  int64_t submitted, completed, failed, cancelled;
  int64_t batches, max_batch;
  int64_t nomem_splits;     /* batches the device budget rejected, halved */
  int64_t solo_retries;     /* requests retried alone after their batch failed for another reason */
  int64_t queued, pending;  /* now: waiting for admission; queued or being aligned */
  int32_t workers, pad;
} dcns_serving_stats;
int dcns_serve_stats(dcns_ctx *ctx, dcns_serving_stats *out);

/* SAM and "o" text of one reference/query pair, as cut1Gap writes them (outputMasking,
 * controlLayer4.cpp:835-1358; cut1Gap's per-query "#done" trailer, :1430-1432, is left to the caller).  Host only.
 *   n_frag, frag, cigar, pvalue  one pair's fragments in the dcns_results layout (frag rows of 7: start1, end1, start2,
 *                                end2, score, cigar offset into `cigar`, cigar length)
 *   ref_text, qry_text           the region texts as extracted from the genomes, still holding the lower-case 'n'
 *                                runs that were removed before aligning
 *   ref_strand, qry_strand       1 = +, 0 = -;  ref_start, qry_start: 1-based region starts;  ref_chr, qry_chr: names
 * *sam and *o receive malloc'ed NUL-terminated texts (free with dcns_free_text) of *sam_len / *o_len bytes. */
int dcns_format_records(int64_t n_frag, const int64_t *frag, const uint32_t *cigar, const double *pvalue,
                        const char *ref_text, int64_t ref_len, const char *qry_text, int64_t qry_len, int ref_strand,
                        int qry_strand, int32_t ref_start, int32_t qry_start, const char *ref_chr, const char *qry_chr,
                        char **sam, int64_t *sam_len, char **o, int64_t *o_len);
void dcns_free_text(char *text);

#ifdef __cplusplus
}
#endif

#endif /* DCNS_GB300_H */
