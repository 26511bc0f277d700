/*
 * gpm.h — C ABI of the GB300 GraphPi pattern-matching engine.
 *
 * Plain pointers and sizes only; every call returns a GPM_* status and, on
 * failure, leaves a message for gpm_last_error().  One process, one GPU
 * (device 0 unless gpm_set_device is called first).
 *
 * Each entry point names the reference interface it replaces
 * (thu-pacman/GraphPi, path:line).
 */
#ifndef GPM_H
#define GPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GPM_API __attribute__((visibility("default")))
#else
#define GPM_API
#endif

/* status codes */
#define GPM_OK 0
#define GPM_ERR_INVALID_ARG 1
#define GPM_ERR_OOM 2
#define GPM_ERR_CUDA 3
#define GPM_ERR_TIMEOUT 4
#define GPM_ERR_OVERFLOW 5
#define GPM_ERR_UNSUPPORTED 6
#define GPM_ERR_NO_DEVICE 7

/* largest pattern the engine accepts (the reference's largest built-in
 * pattern is 7 vertices, include/pattern.h:17) */
#define GPM_MAX_PATTERN 8

typedef struct gpm_graph gpm_graph; /* device-resident CSR of one data graph */
typedef struct gpm_plan gpm_plan;   /* device-resident compiled schedule */

/* exact embedding count; counts of 5-vertex motifs on scale-22 R-MAT graphs
 * exceed 2^64, so results are 128-bit */
typedef struct gpm_u128 {
    uint64_t lo;
    uint64_t hi;
} gpm_u128;

/* ------------------------------------------------------------------ */
/* errors and device                                                   */
/* ------------------------------------------------------------------ */

/* Message of the last failing call on this thread ("" if none). */
GPM_API const char* gpm_last_error(void);

/* Selects the CUDA device for later calls on this thread.  The reference
 * chose an OpenMP team size instead (src/graph.cpp:202). */
GPM_API int gpm_set_device(int32_t device);

/* ------------------------------------------------------------------ */
/* data graph                                                          */
/* ------------------------------------------------------------------ */

/* Uploads an undirected graph given as a symmetric CSR: neighbours of v are
 * col[rowptr[v] .. rowptr[v+1]), sorted ascending, no self loops, no
 * duplicates — the layout of the reference `Graph` (include/graph.h:14-15,
 * src/graph.cpp:141-145).  rowptr[v_cnt] is the directed edge count (the
 * reference's e_cnt) and must be < 2^32.
 * relabel = 1 renumbers vertices by descending degree on the device (the
 * reference's oriented_type 1, src/dataloader.cpp:96-109); counts do not
 * depend on labels.  The CSR is validated; malformed input returns
 * GPM_ERR_INVALID_ARG. */
GPM_API int gpm_graph_create(int32_t v_cnt, const uint32_t* rowptr, const int32_t* col,
                             int32_t relabel, gpm_graph** out);

/* Builds a graph on the GPU from m undirected edges (src[i], dst[i]) in host
 * memory: symmetrises, drops self loops and duplicates, sorts and builds the
 * offsets on the device — the host steps of DataLoader::general_load_data
 * (reference src/dataloader.cpp:129-160) — then validates and (relabel != 0)
 * relabels by degree like gpm_graph_create.  GPM_ERR_INVALID_ARG for an id
 * outside [0, v_cnt) or 2m >= 2^32. */
GPM_API int gpm_graph_from_edges(int32_t v_cnt, int64_t m, const int32_t* src, const int32_t* dst,
                                 int32_t relabel, gpm_graph** out);

/* Copies the graph's CSR in the caller's ids (v_cnt + 1 offsets, e_cnt
 * neighbours; sizes from gpm_graph_stats) to host arrays. */
GPM_API int gpm_graph_download(const gpm_graph* g, uint32_t* rowptr, int32_t* col);

/* Device pointers of the graph's resident CSR: the degree-relabelled copy
 * the counting kernels use (caller_ids = 0) or the caller's numbering
 * (caller_ids = 1; the same arrays when the graph was not relabelled).  They
 * stay valid until gpm_graph_destroy.  For kernels built outside the engine
 * (the per-schedule generated kernels) that count on the same numbering.
 * No reference counterpart: the reference's Graph exposes its host arrays
 * as public fields (include/graph.h:14-15). */
GPM_API int gpm_graph_device_csr(const gpm_graph* g, int32_t caller_ids, const uint32_t** rowptr,
                                 const int32_t** col);

/* Frees a graph (the reference's ~Graph, include/graph.h:24-27). *//* Frees a graph (the reference's ~Graph, include/graph.h:24-27). */
GPM_API int gpm_graph_destroy(gpm_graph* g);

/* v_cnt, directed e_cnt, max degree and the largest possible intersection
 * (second-largest degree; VertexSet::max_intersection_size,
 * src/dataloader.cpp:112-115). Any pointer may be NULL. */
GPM_API int gpm_graph_stats(const gpm_graph* g, int64_t* v_cnt, int64_t* e_cnt,
                            int64_t* max_degree, int64_t* max_intersection_size);

/* Triangle count on the GPU — Graph::triangle_counting_mt
 * (include/graph.h:36, src/graph.cpp:112-139); it feeds the schedule cost
 * model's tri_cnt (src/schedule.cpp:1496). */
GPM_API int gpm_tri_count(gpm_graph* g, uint64_t* out);

/* k-clique count (3 <= k <= GPM_MAX_PATTERN), the clique fast path: the
 * count Graph::pattern_matching gives for the complete pattern, computed the
 * way pattern_matching_func does with clique = true (src/graph.cpp:147-197,
 * the min_vertex clip of VertexSet::intersection, src/vertex_set.cpp:75-103):
 * each clique once, as its decreasing vertex sequence, with no restriction
 * or injectivity checks.  Honours the "stripes"/"stripe" options (the tasks
 * are the directed edges of the device CSR). */
GPM_API int gpm_clique_count(gpm_graph* g, int32_t k, gpm_u128* out);

/* ------------------------------------------------------------------ */
/* pattern, motifs, schedule (host)                                    */
/* ------------------------------------------------------------------ */

/* All connected k-vertex patterns up to isomorphism, in the reference's
 * generation order — MotifGenerator::generate (include/motif_generator.h:9,
 * src/motif_generator.cpp:5-43).  Writes min(count, cap) row-major k*k
 * adjacency matrices to adj_out and the total to *count. */
GPM_API int gpm_motifs(int32_t k, int32_t* adj_out, int32_t cap, int32_t* count);

/* Size of the pattern's automorphism group — Schedule::get_multiplicity
 * (src/schedule.cpp:400-403). */
GPM_API int gpm_pattern_multiplicity(int32_t n, const int32_t* adj, int64_t* out);

/* Builds a schedule — the Schedule constructor
 * Schedule(pattern, is_pattern_valid, performance_modeling_type,
 *          restricts_type, use_in_exclusion_optimize, v_cnt, e_cnt, tri_cnt)
 * (include/schedule.h:13, src/schedule.cpp:9-253) — and writes its tables
 * (the getters of include/schedule.h:23-37 plus the public restrict_pair,
 * in_exclusion_optimize_group/_val of :56-58) as int64 words:
 *   size, adj[n*n], total_prefix_num, father_prefix_id[P], last[n], next[P],
 *   loop_set_prefix_id[n], total_restrict_num, restrict_last[n],
 *   restrict_next[R], restrict_index[R], n_pairs, pairs[2*n_pairs],
 *   in_exclusion_optimize_num, n_groups,
 *     per group: val, n_blocks, per block: len, members[len],
 *   in_exclusion_optimize_redundancy, multiplicity.
 * *n_words receives the length; *valid the reference's is_pattern_valid.
 * perf_type 0..3 and restricts_type 0..2 as in include/schedule.h:14-20;
 * perf_type != 0 with tri_cnt < 0 is GPM_ERR_INVALID_ARG (the reference
 * asserts, src/schedule.cpp:11-15). */
GPM_API int gpm_schedule_build(int32_t n, const int32_t* adj, int32_t perf_type,
                               int32_t restricts_type, int32_t use_iep, int64_t v_cnt,
                               uint64_t e_cnt, int64_t tri_cnt, int64_t* tables, int32_t cap,
                               int32_t* n_words, int32_t* valid);

/* The candidates the Schedule constructor scores (src/schedule.cpp:30-139):
 * every valid loop order (for perf_type 1 only those with the longest
 * inclusion–exclusion tail) times every verified restriction set, in the
 * constructor's scan order.  For candidate i: orders[i*n .. i*n+n) (new
 * vertex j = pattern vertex orders[i*n+j]), n_pairs[i] restriction pairs in
 * pairs[i*2*GPM_MAX_PAIRS ..], and costs[i], the cost the chosen model
 * assigns (lower is preferred).  *count receives the total; at most cap are
 * written. */
#define GPM_MAX_PAIRS 28
GPM_API int gpm_schedule_candidates(int32_t n, const int32_t* adj, int32_t perf_type, int32_t restricts_type,
                                    int64_t v_cnt, uint64_t e_cnt, int64_t tri_cnt, int32_t* orders,
                                    int32_t* n_pairs, int32_t* pairs, double* costs, int32_t cap,
                                    int32_t* count);

/* The tables (layout of gpm_schedule_build) of the schedule for one
 * candidate: the pattern relabelled by `order`, restrictions `pairs` (dropped
 * when restricts_type is 0), inclusion–exclusion as requested — what the
 * Schedule constructor builds when its model picks that candidate. */
GPM_API int gpm_schedule_from_order(int32_t n, const int32_t* adj, const int32_t* order, int32_t n_pairs,
                                    const int32_t* pairs, int32_t use_iep, int32_t restricts_type,
                                    int64_t* tables, int32_t cap, int32_t* n_words, int32_t* valid);

/* Host-side analysis of schedule tables: *label_sensitive = 1 when the
 * schedule's count depends on the vertex labelling.  The reference's
 * inclusion–exclusion tail skips the restrictions of its own loops and
 * divides by a redundancy measured on K_n (src/graph.cpp:306-344,
 * src/schedule.cpp:1746-1764); when a skipped restriction ties a tail loop
 * to an earlier loop the result varies with the labels (and differs from
 * the true count).  Counting runs such schedules on the caller's vertex ids,
 * never on the degree-relabelled copy, so results equal the reference's. */
GPM_API int gpm_schedule_analyze(const int64_t* tables, int32_t n_words, int32_t* label_sensitive);

/* How the engine will evaluate a schedule: info[0] tail depth T, [1]
 * deepest loop level L, [2] inclusion–exclusion length k, [3] leaf mode of
 * level L (0 candidate by candidate, 1 batched count, 2 batched two-loop
 * inclusion–exclusion), [4] 1 when the last two loops can be summed in
 * pairs (option "pair_leaf"), [5] label-sensitive (see
 * gpm_schedule_analyze).  cap >= 6. */
GPM_API int gpm_plan_info(const int64_t* tables, int32_t n_words, int32_t* info, int32_t cap);

/* Compiles schedule tables (layout of gpm_schedule_build) into a device
 * plan: per-depth candidate lists, restriction bounds, prefix-set slots and
 * the inclusion-exclusion groups.  Replaces the table walks of
 * src/graph.cpp:217,249,306-313,353,368,383. */
GPM_API int gpm_plan_create(const int64_t* tables, int32_t n_words, gpm_plan** out);
GPM_API int gpm_plan_destroy(gpm_plan* p);

/* ------------------------------------------------------------------ */
/* counting (the hot path)                                             */
/* ------------------------------------------------------------------ */

/* Counts embeddings of the plan's pattern in g — Graph::pattern_matching
 * (include/graph.h:39, src/graph.cpp:199-398): the schedule-driven nested
 * loops, restriction pruning, injectivity checks and the
 * inclusion-exclusion tail, divided by the plan's redundancy (:244).
 * Exact in 128 bits. */
GPM_API int gpm_count(gpm_graph* g, const gpm_plan* p, gpm_u128* out);

/* Counts n_pairs (graph, plan) pairs in one persistent launch fed by
 * per-pair work queues (no reference counterpart; it replaces n_pairs
 * separate Graph::pattern_matching calls).  outs[i] belongs to pair i. */
GPM_API int gpm_batch_count(int32_t n_pairs, gpm_graph* const* graphs,
                            const gpm_plan* const* plans, gpm_u128* outs);

/* gpm_batch_count captured once into a CUDA graph and replayed: *exec is
 * created on the first call with *exec == NULL and reused afterwards for the
 * same pairs.  gpm_batch_exec_destroy frees it. */
typedef struct gpm_batch_exec gpm_batch_exec;
GPM_API int gpm_batch_exec_run(gpm_batch_exec** exec, int32_t n_pairs, gpm_graph* const* graphs,
                               const gpm_plan* const* plans, gpm_u128* outs);
GPM_API int gpm_batch_exec_destroy(gpm_batch_exec* exec);

/* One-shot host-buffer path: uploads the host CSR, relabels, counts every
 * schedule in `tables` (n_plans schedules, each n_words[i] int64 words laid
 * out as gpm_schedule_build writes them, concatenated) in one batched
 * launch, copies the counts back and frees the device copy.  This is the
 * call a host program that owns its graph in memory makes — the reference's
 * `g->pattern_matching(schedule, n)` per schedule. */
GPM_API int gpm_count_host(int32_t v_cnt, const uint32_t* rowptr, const int32_t* col,
                           int32_t n_plans, const int64_t* tables, const int32_t* n_words,
                           gpm_u128* outs);

/* ------------------------------------------------------------------ */
/* learned schedule cost model                                         */
/* ------------------------------------------------------------------ */

/* A two-layer perceptron (in_dim -> hidden ReLU -> 1, fp32) that predicts
 * the log runtime of a candidate schedule from its features; the learned
 * replacement for the scoring in Schedule::our_estimate_schedule_restrict
 * (src/schedule.cpp:1487-1574), whose analytic model stays the fallback.
 * Forward, backward and Adam are hand-written kernels on the current device.
 * Parameters are one flat float array: W1[hidden][in_dim], b1[hidden],
 * W2[hidden], b2 (hidden*in_dim + 2*hidden + 1 floats). */
typedef struct gpm_mlp gpm_mlp;
GPM_API int gpm_mlp_create(int32_t in_dim, int32_t hidden, uint64_t seed, gpm_mlp** out);
GPM_API int gpm_mlp_destroy(gpm_mlp* m);
/* copies the parameters out (set = 0) or in (set = 1; resets Adam state) */
GPM_API int gpm_mlp_params(gpm_mlp* m, float* params, int32_t n_params, int32_t set);
/* Y[i] = model(X[i*in_dim ..]) for n_rows rows (host arrays) */
GPM_API int gpm_mlp_forward(gpm_mlp* m, const float* X, int32_t n_rows, float* Y);
/* gradient of the mean squared error against targets T, and the loss */
GPM_API int gpm_mlp_gradients(gpm_mlp* m, const float* X, const float* T, int32_t n_rows, float* grads,
                              float* loss);
/* full-batch Adam for `epochs` steps; *final_loss = loss before the last step */
GPM_API int gpm_mlp_train(gpm_mlp* m, const float* X, const float* T, int32_t n_rows, int32_t epochs, float lr,
                          float weight_decay, float* final_loss);

/* Counting that allocates nothing on the device.  No counterpart in the
 * reference: it serves callers that cannot call cudaMalloc — programs whose
 * GPU memory is owned by another allocator (a framework's caching allocator
 * or a fixed arena, where a cudaMalloc fails or fragments the pool), and
 * latency-critical loops that cannot take cudaMalloc/cudaFree's implicit
 * device synchronisation.
 * The caller passes the CSR already in device memory (layout of
 * gpm_graph_create, counted on the ids as given), schedule tables (host) and
 * the result location (host).  The CSR gets the checks gpm_graph_create
 * applies (GPM_ERR_INVALID_ARG when malformed).  Work runs on the
 * per-thread default stream, which does not wait for other streams: finish
 * writing rowptr/col first (synchronize, or wait on an event recorded on
 * the writing stream).  The call waits for its own work.
 * Scratch is a 64 MiB file-scope device array that every GPU loading the
 * library holds until exit; the grid is sized to it (and to the blocks
 * resident at once), and a pattern/graph whose per-warp sets (scratch sets x
 * largest degree x 4 bytes) do not fit one block returns
 * GPM_ERR_UNSUPPORTED ("use gpm_count").  Long loops are shared with idle
 * warps as in gpm_count ("split"); the pair-sum leaf is off on this path.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the one array: it keeps the last call's contents (each
 * call clears the words that must start at zero), and calls that overlap on
 * the GPU — from several host threads — race on it. */
GPM_API int gpm_count_noalloc(int32_t v_cnt, const uint32_t* d_rowptr, const int32_t* d_col,
                              const int64_t* tables, int32_t n_words, gpm_u128* out);

/* ------------------------------------------------------------------ */
/* tuning                                                              */
/* ------------------------------------------------------------------ */

/* Engine knobs (counts never depend on them):
 *   "warps_per_block", "blocks_per_sm", "chunk" (work-queue grab size),
 *   "min_blocks" (1, or 3 / 4: the kernel variants for three / four blocks
 *   of at most 8 warps per SM),
 *   "stage_tma" (1: stage fixed leaf sets with bulk copies), "merge_vec"
 *   (1: merges read 128-bit windows), "schedule_gpu" (1: Schedule scores
 *   its candidates on the GPU when one is present), "pool" (1: graph
 *   arrays and construction temporaries from a stream-ordered pool that
 *   keeps freed memory, up to a quarter of the device, for the next upload),
 *   "split" (a loop at depth >= 2 with at least this many candidates, or
 *   fewer whose neighbour lists hold 16384 elements, is published so that
 *   idle warps take slices of it, weighted by the candidates' degrees;
 *   0 = off),
 *   "stage_max" (largest father set staged in shared memory),
 *   "leaf_batch", "pair_leaf" (batched deepest levels where the plan
 *   allows; the pair-sum leaf is on by default, the batched leaf off),
 *   "pair_log2" (entries per warp of the pair-sum table as a power of two;
 *   0 = 2^17, fewer when memory is short), "pair_max_ops" (longest pair sum one warp
 *   takes on, in list elements; longer ones run as loops; 0 = no cap),
 *   "dense_slots" (per-vertex counter arrays for pair sums too big for the
 *   table, filled and probed by idle warps together when "split" is on;
 *   default 64), "bitmap_min" (fixed leaf sets at least
 *   this large are tested through a per-warp bitmap instead of a binary
 *   search; 0 = never),
 *   "merge_alpha4_small"/"_mid"/"_large" (merge vs search per length bucket),
 *   "timeout_ms" (reserved; no engine wait reads it),
 *   "stripes"/"stripe" (a launch covers only the first-level tasks t with
 *   t mod stripes == stripe: the tasks split into `stripes` interleaved
 *   parts, e.g. one per GPU or per bounded step), "raw_sums" (1: outputs are the undivided
 *   signed 128-bit sums, to be added over stripes and then divided by the
 *   schedule's redundancy; required when stripes > 1),
 *   "count_bytes" (1: count algorithmic bytes).  Returns
 * GPM_ERR_INVALID_ARG on an unknown key or out-of-range value. */
GPM_API int gpm_set_option(const char* key, int64_t value);
GPM_API int gpm_get_option(const char* key, int64_t* value);

/* Launch statistics of the last counting call on this thread: kernel time
 * in milliseconds (CUDA events on the launch stream), number of kernels
 * launched, and the algorithmic bytes the intersections read (4 bytes per
 * element a merge would touch, plus 8 bytes per offset pair; counted only
 * when the "count_bytes" option is 1). */
GPM_API int gpm_last_launch_stats(double* kernel_ms, int64_t* launches, uint64_t* algo_bytes);

#ifdef __cplusplus
}
#endif

#endif /* GPM_H */
