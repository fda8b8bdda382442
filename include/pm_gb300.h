/*
 * pm_gb300.h — C ABI of the GB300-native PruneJuice pruning pipeline.
 *
 * The reference (tahsinreza/pattenmatching_sharedmemory) has no plugin or FFI
 * API: its hot path is reached through the `patternmatching` CLI, the TOTEM
 * file formats and the per-step C++ class contract
 *   AlgoResults <Step>::compute(const graph_t&, MultipleLabelGlobalState*)
 * driven by MultipleLabelCpu (src/patternmatching/multiple_label_cpu.h:32-53).
 * Every entry point below replaces one piece of that contract; the citation
 * in front of each names the reference interface it stands in for.  Plain
 * pointers and sizes only; no C++ or torch types cross this boundary.
 *
 * Ownership: the caller owns every host buffer it passes in.  The library
 * owns the device-resident CSR (pm_graph) and each query's device arena
 * (pm_query) until the matching *_destroy call.
 *
 * Errors follow TOTEM's error_t convention (src/totem/totem_comdef.h:31-32):
 * PM_SUCCESS = 0, PM_FAILURE = -1, plus distinct negative codes.  The last
 * error message of the calling thread is available from pm_last_error().
 *
 * Threading: calls on distinct pm_query handles may run concurrently from
 * different host threads; a single handle must not be used concurrently.
 */
#ifndef PM_GB300_H
#define PM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (src/totem/totem_comdef.h:31-32 SUCCESS/FAILURE) ---- */
typedef int32_t pm_status_t;
#define PM_SUCCESS 0
#define PM_FAILURE (-1)           /* generic failure, as TOTEM's FAILURE      */
#define PM_E_INVALID_ARG (-2)     /* null pointer, bad size, bad enum         */
#define PM_E_IO (-3)              /* file cannot be opened / read / written   */
#define PM_E_FORMAT (-4)          /* malformed or truncated TOTEM file        */
#define PM_E_PATTERN_TOO_LARGE (-5) /* template > 64 vertices or walk too long */
#define PM_E_ADMISSION_DENIED (-6)  /* server memory budget exceeded          */
#define PM_E_TIMEOUT (-7)           /* request deadline passed                */
#define PM_E_DEVICE (-8)            /* CUDA error or device-side error status */
#define PM_E_NO_DEVICE (-9)         /* no CUDA device / extension unusable    */
#define PM_E_CANCELLED (-10)        /* request cancelled before it finished   */
#define PM_E_OOM (-11)              /* host or device allocation failed       */
#define PM_E_BUSY (-12)             /* server queue full, retry later         */
#define PM_E_STATISTICS (-13)       /* dynamic order: a graph statistic its
                                       estimate reads is absent (the reference
                                       throws std::out_of_range and aborts)  */

/* Last error message of the calling host thread (never NULL). */
const char* pm_last_error(void);

/* Library version string. */
const char* pm_version(void);

/* ---- step kinds: MultipleLabelStep::Step (multiple_label_step.h:16-25) ---- */
typedef enum {
  PM_STEP_START = 0,
  PM_STEP_END = 1,
  PM_STEP_LCC0 = 2,
  PM_STEP_LCC = 3,
  PM_STEP_CC = 4,
  PM_STEP_PC = 5,
  PM_STEP_TDS = 6,
  PM_STEP_ENUMERATION = 7
} pm_step_kind;

/* AlgoResults (src/patternmatching/algorithms/algo_results.h:9-20). */
typedef struct {
  uint64_t vertex_eliminated;
  uint64_t edge_eliminated;
  uint64_t match_eliminated;
  uint64_t enumeration;
} pm_algo_results;

/* One row of the reference's results.totem
 * (MultipleLabelCpu::logResults, multiple_label_cpu.cc:187-213). */
typedef struct {
  int32_t iteration;
  int32_t step; /* pm_step_kind */
  double step_ms;
  double cumulative_ms;
  pm_algo_results results;
  uint64_t active_vertex;
  uint64_t total_vertex;
  uint64_t active_edge;
  uint64_t total_edge;
} pm_step_record;

typedef struct pm_graph pm_graph;
typedef struct pm_query pm_query;

/* ---- graph (TOTEM graph_t + I/O) ------------------------------------- */

/* graph_initialize(graph or .bin) + parseVertexFile(labels) + optional
 * graph_store_binary(bin) — the load sequence of MultipleLabelCpu::allocate
 * (multiple_label_cpu.cc:22-35), including its quirk that an existing
 * bin_path is loaded instead of graph_path and labels_path.  bin_path and
 * labels_path may be NULL or "".  The CSR is copied to device `device`. */
pm_status_t pm_graph_load(const char* graph_path, const char* bin_path,
                          const char* labels_path, int device, pm_graph** out);

/* Builds a graph from caller-owned host CSR buffers (graph_t vertices /
 * edges / values, totem_graph.h:137-180).  labels may be NULL (all 0). */
pm_status_t pm_graph_from_csr(const uint64_t* offsets, const uint32_t* adj,
                              const uint64_t* labels, uint32_t vertex_count,
                              uint64_t edge_count, int device, pm_graph** out);

/* graph_store_binary (totem_graph.cu:883-922), 32-bit edge-id layout when
 * the edge count fits, else the EID=64 layout. */
pm_status_t pm_graph_store_binary(const pm_graph* g, const char* path);

pm_status_t pm_graph_info(const pm_graph* g, uint32_t* vertex_count,
                          uint64_t* edge_count, uint64_t* device_bytes);
void pm_graph_destroy(pm_graph* g);

/* ---- query: one template over one resident graph ---------------------- */

/* MultipleLabelCpu::allocate's pattern half (multiple_label_cpu.cc:37-104):
 * loads pattern_dir/"pattern_edge[.totem]" and pattern_dir/"pattern_vertex_data",
 * generates the local, cycle, path, template and enumeration constraints,
 * allocates the per-query device state and initialises the step machine.
 * pattern_dir is concatenated exactly as the reference does (it should end
 * with '/').  load_pattern_labels mirrors the reference's rule that pattern
 * labels are read only when a graph label file was given (:44-47). */
pm_status_t pm_query_create(pm_graph* g, const char* pattern_dir,
                            int load_pattern_labels, pm_query** out);

/* Same from caller-owned template CSR buffers. */
pm_status_t pm_query_create_from_csr(pm_graph* g, const uint64_t* p_offsets,
                                     const uint32_t* p_adj,
                                     const uint64_t* p_labels,
                                     uint32_t p_vertex_count,
                                     uint64_t p_edge_count, pm_query** out);

/* The reference's article drivers (src/patternmatching/test_article,
 * CMakeLists.txt:12-33) run the same schedule with other CC / PC / TDS
 * walks: strict walks bind no graph vertex twice and keep no memo
 * (multiple_label_test, the *_strict_cpu.tpp files, optimization_none);
 * backtrack walks skip a (vertex, template vertex) pair the source's walk
 * already visited (CC, PC) or keep only the hypothesis memo (TDS) (the
 * *_backtrack_cpu.tpp files, optimization_all: work aggregation, early
 * termination, multiple validation).  Their TDS steps advance through the
 * template constraints, and their schedule ends with END where the
 * reference's would enter ENUMERATION (test_optimization_multiple_label_
 * step.cc:46-58).  pm_query_create_variant* builds such a query
 * (PM_NLCC_REFERENCE gives pm_query_create's). */
#define PM_NLCC_REFERENCE 0
#define PM_NLCC_STRICT 1
#define PM_NLCC_BACKTRACK 2
/* Flags or-ed into `variant` (with PM_NLCC_STRICT or PM_NLCC_BACKTRACK): the
 * article's constraint-order drivers (test_article/CMakeLists.txt:53-73,
 * test_order_multiple_label_cpu.cc).  Their NLCC steps run each constraint
 * once and drop it.
 *   PM_ORDER_ENUMERATE      USE_ENUMERATE: the schedule ends in ENUMERATION
 *                           (then END) instead of END.
 *   PM_ORDER_EFFECTIVENESS  ORDER_USE_DYNAMIC: after every LCC fixpoint the
 *                           graph statistics of the pruned graph are taken
 *                           on the GPU (GraphStatCpu::compute,
 *                           algorithms/graph_stat_cpu.tpp:42-80) and the
 *                           remaining constraint with the largest estimated
 *                           effectiveness (multiple_label_constraint_
 *                           effectiveness.cc) runs next; the run starts with
 *                           an empty row (step PM_STEP_START, written with
 *                           an empty step name) and no LCC0, as the
 *                           reference's driver does.  A statistic the
 *                           estimate needs but the graph lacks ends the run
 *                           with PM_E_STATISTICS.
 *   PM_ORDER_EARLY_ENUMERATION  ENUMERATE_START_EARLY (threshold 0.01):
 *                           ENUMERATION starts as soon as its estimated cost
 *                           is at most the next constraint's, or the next
 *                           constraint's effectiveness is at most 0.01. */
#define PM_ORDER_ENUMERATE 0x100
#define PM_ORDER_EFFECTIVENESS 0x200
#define PM_ORDER_EARLY_ENUMERATION 0x400
pm_status_t pm_query_create_variant(pm_graph* g, const char* pattern_dir, int load_pattern_labels,
                                    int32_t variant, pm_query** out);
/* The order drivers' OpenMP thread count (process-wide, read when a query is
 * created; default 1, the reference hard-codes 60 at
 * test_order_multiple_label_cpu.cc:15): the graph statistics split the
 * vertices into that many static-schedule blocks, each with its own
 * never-reset neighbour-label accumulation (graph_stat_cpu.tpp:46-70), and
 * the cost estimates divide by it. */
pm_status_t pm_set_order_threads(int32_t threads);
pm_status_t pm_query_create_variant_from_csr(pm_graph* g, const uint64_t* p_offsets, const uint32_t* p_adj,
                                             const uint64_t* p_labels, uint32_t p_vertex_count,
                                             uint64_t p_edge_count, int32_t variant, pm_query** out);

/* Number of cycle / path / template constraints
 * (MultipleLabelStep::initStep{Cc,Pc,Tds}, multiple_label_step.cc:12-25). */
pm_status_t pm_query_constraint_counts(const pm_query* q, int32_t* n_cycle,
                                       int32_t* n_path, int32_t* n_template);

/* The constraint dump the reference writes to log.totem (the print()
 * methods of the generators), without timestamps.  Writes up to cap bytes
 * (NUL-terminated) and the full size to *needed. */
pm_status_t pm_query_dump_constraints(const pm_query* q, char* buf, size_t cap,
                                      size_t* needed);

/* One iteration of MultipleLabelCpu::runPatternMatching
 * (multiple_label_cpu.cc:121-175): resets per-step state, runs the current
 * step's compute on the GPU and advances MultipleLabelStep::getNextStep.
 * *finished is set when the step machine reaches END. */
pm_status_t pm_query_step(pm_query* q, pm_step_record* record, int* finished);

/* The full run loop (≤1000 iterations) plus the final END row.  Writes up
 * to cap records; *n_records receives the number of rows produced. */
pm_status_t pm_query_run(pm_query* q, pm_step_record* records, int32_t cap,
                         int32_t* n_records);

/* The pruning half of the run loop: runPatternMatching
 * (multiple_label_cpu.cc:113-184) stopped where MultipleLabelStep::
 * getNextStep would enter ENUMERATION (multiple_label_step.cc:46-57), or at
 * the iteration cap.  The last row written names the step that would run
 * next (ENUMERATION), as the reference's final logResults row does.  A
 * later pm_query_run continues from there (ENUMERATION and END). */
pm_status_t pm_query_prune(pm_query* q, pm_step_record* records, int32_t cap,
                           int32_t* n_records);

/* The embeddings ENUMERATION counts, listed — the reference's
 * writeEnumeration (multiple_label_enumeration_cpu.tpp:15-35, compiled out
 * there): each match is the graph vertices bound by the enumeration walk's
 * vertex moves, in walk order (historyIndexVector), *per_match of them (the
 * template size).  Runs the pruning first when the query has not reached
 * ENUMERATION.  Writes up to cap matches to `matches` (cap x *per_match
 * uint32), in no particular order; *n_matches receives the total, which is
 * the ENUMERATION count (0 when the run ended at the iteration cap before
 * ENUMERATION). */
pm_status_t pm_query_list_matches(pm_query* q, uint32_t* matches, uint64_t cap, uint32_t* per_match,
                                  uint64_t* n_matches);

/* The same as text at `path`, the reference's format (each vertex followed
 * by ';', one match per line), at most max_matches lines. */
pm_status_t pm_query_write_matches(pm_query* q, const char* path, uint64_t max_matches, uint64_t* n_written);

/* The pruned subgraph as a CSR over the original vertex ids: the CSR
 * entries printActiveGraph prints (active entries between active vertices,
 * multiple_label_cpu.cc:270-284), in CSR order.  offsets[V + 1] (may be
 * NULL); adj receives the entries when cap is at least their number
 * (*n_entries), else PM_E_INVALID_ARG with *n_entries set. */
pm_status_t pm_query_export_subgraph(pm_query* q, uint64_t* offsets, uint32_t* adj, uint64_t cap,
                                     uint64_t* n_entries);

/* Copies the pruned state back to caller-owned host buffers (any may be
 * NULL): candidate role bitmask per vertex (bit p = pattern vertex p, the
 * FixedBitmap<64> of multiple_label_common_cpu.h:49), active flag per CSR
 * entry and per vertex. */
pm_status_t pm_query_export(const pm_query* q, uint64_t* cand_masks,
                            uint8_t* edge_active, uint8_t* vertex_active);

/* Writes results.totem, graph_NNNN.totem and vertex_NNNN.totem exactly as
 * MultipleLabelCpu::logResults / printActiveGraph / printActiveVertex do
 * (multiple_label_cpu.cc:187-296, utils/logger.cc:90-136). */
pm_status_t pm_query_write_outputs(const pm_query* q, const char* out_dir);

/* Final exact match count (the ENUMERATION row), or 0 before it ran. */
pm_status_t pm_query_match_count(const pm_query* q, uint64_t* count);

/* Device bytes held by this query's state arena. */
pm_status_t pm_query_device_bytes(const pm_query* q, uint64_t* bytes);

/* Device bytes a query over graph g with a template of p_vertex_count
 * vertices would hold (admission control). */
pm_status_t pm_query_estimate_bytes(const pm_graph* g, uint32_t p_vertex_count,
                                    uint64_t* bytes);

void pm_query_destroy(pm_query* q);

/* ---- Serving and batching ------------------------------------------------
 *
 * No counterpart in the reference, which runs one template per process
 * (MultipleLabelCpu::runPatternMatching, multiple_label_cpu.cc:113-184).
 * A server keeps one graph resident and runs submitted template queries on
 * `slots` GPU slots at once (each slot: a host thread with its own CUDA
 * stream).  Requests wait in FIFO order until a slot is free and the device
 * bytes they are charged (pm_query_estimate_bytes) fit under the memory
 * budget beside the running ones; requests that arrive while others run are
 * admitted as slots and memory free up (continuous batching).  Each request
 * runs the whole pipeline, LCC0 to ENUMERATION, with the same results as
 * pm_query_run on its own. */
typedef struct pm_server pm_server;

typedef struct pm_server_config {
  uint32_t slots;         /* queries on the GPU at once, >= 1 */
  uint64_t memory_budget; /* device bytes for admitted queries; 0 = 90% of free memory */
  uint32_t walk_share;    /* each slot's walker launches use 1/walk_share of the
                             GPU's resident walker blocks; 0 = 1/slots (requests
                             that run into their budget leave room to the
                             others), 1 = the whole GPU (requests that each fill
                             the GPU, e.g. exact counting).  Speed only. */
} pm_server_config;

/* pm_server_submit flags: keep the final state for pm_server_export;
 * run the pruning pipeline only (as pm_query_prune: no ENUMERATION, match
 * count 0). */
#define PM_SUBMIT_EXPORT_STATE 1u
#define PM_SUBMIT_PRUNE_ONLY 2u

typedef struct pm_request_result {
  int32_t status;          /* PM_SUCCESS, or the request's error code */
  int32_t n_records;       /* results.totem rows (END included) */
  uint64_t match_count;    /* ENUMERATION row */
  double queue_ms;         /* submission to admission */
  double run_ms;           /* admission to completion */
  double latency_ms;       /* submission to completion */
  double gpu_ms;           /* sum of the step times */
  uint64_t charged_bytes;  /* device bytes charged at admission */
} pm_request_result;

typedef struct pm_server_stats {
  uint64_t queued, running, done;
  uint64_t bytes_in_use, peak_bytes, memory_budget;
  uint32_t slots;
} pm_server_stats;

/* The graph must stay alive (and on its device) until pm_server_destroy. */
pm_status_t pm_server_create(pm_graph* g, const pm_server_config* config, pm_server** out);

/* Queues a template (CSR, as pm_query_create_from_csr); *ticket names it.
 * PM_E_ADMISSION_DENIED when its charge exceeds the whole budget. */
pm_status_t pm_server_submit(pm_server* s, const uint64_t* p_offsets, const uint32_t* p_adj,
                             const uint64_t* p_labels, uint32_t p_vertex_count,
                             uint64_t p_edge_count, uint32_t flags, uint64_t* ticket);

/* *done = 1 and *result filled once the request finished (result may be
 * NULL); *done = 0 while it is queued or running. */
pm_status_t pm_server_poll(pm_server* s, uint64_t ticket, int* done, pm_request_result* result);

/* Blocks until the request finished or timeout_ms passed (< 0: no limit);
 * PM_E_TIMEOUT when it has not finished in time. */
pm_status_t pm_server_wait(pm_server* s, uint64_t ticket, double timeout_ms,
                           pm_request_result* result);

/* The finished request's results.totem rows (as pm_query_run). */
pm_status_t pm_server_records(pm_server* s, uint64_t ticket, pm_step_record* records,
                              int32_t cap, int32_t* n_records);

/* The finished request's final state (as pm_query_export); the request must
 * have been submitted with PM_SUBMIT_EXPORT_STATE. */
pm_status_t pm_server_export(pm_server* s, uint64_t ticket, uint64_t* cand_masks,
                             uint8_t* edge_active, uint8_t* vertex_active);

/* Cancels a request: a queued one ends at once, a running one before its
 * next step (the step in flight finishes first); both end with
 * PM_E_CANCELLED.  A finished request is left as it is.  The ticket stays
 * valid until pm_server_release. */
pm_status_t pm_server_cancel(pm_server* s, uint64_t ticket);

/* Forgets a finished request (its rows and state). */
pm_status_t pm_server_release(pm_server* s, uint64_t ticket);

pm_status_t pm_server_stats_get(pm_server* s, pm_server_stats* stats);

/* Queued requests end with PM_E_CANCELLED; running ones finish first. */
void pm_server_destroy(pm_server* s);

/* Runs n templates over graph g on `slots` GPU slots (a server with the
 * default budget): templates[i] is template i in CSR form.  Writes each
 * template's match count and status. */
typedef struct pm_template_csr {
  const uint64_t* offsets;
  const uint32_t* adj;
  const uint64_t* labels;
  uint32_t vertex_count;
  uint64_t edge_count;
} pm_template_csr;

pm_status_t pm_batch_run(pm_graph* g, const pm_template_csr* templates, uint32_t n, uint32_t slots,
                         uint64_t* match_counts, int32_t* statuses);

/* Batched form (no counterpart in the reference, which runs one template per
 * process, multiple_label_cpu.cc:113-184): the n templates run as one batch
 * over graph g in lockstep rounds, each on the reference's schedule
 * (multiple_label_step.cc:30-83).  The LCC0 steps and the LCC fixpoints of
 * the batch's queries run as shared multi-query launches over per-query work
 * lists (blocks of different queries walk the same CSR ranges together, so
 * one HBM read of an adjacency range serves every query); their CC / PC /
 * TDS / ENUMERATION steps run on per-query streams from a pool of host
 * threads.  Each query's rows (timing columns aside), match count and state
 * equal pm_query_run's on its own (pm_query_prune's with
 * PM_SUBMIT_PRUNE_ONLY in flags).  At most 16 queries are in flight at a
 * time (one per host worker); the others enter in order as queries finish,
 * and pm_set_query_budget_ms bounds every query from when it enters.  Each
 * worker's walker launches take its share of the GPU.  Returns PM_SUCCESS
 * with per-query statuses in
 * pm_fused_batch_result; the batch keeps every query's state until
 * pm_fused_batch_destroy. */
typedef struct pm_fused_batch pm_fused_batch;

pm_status_t pm_fused_batch_run(pm_graph* g, const pm_template_csr* templates, uint32_t n, uint32_t flags,
                               pm_fused_batch** out);
/* Query i's outcome: status, rows, match count, run_ms from the start of the
 * run to its end, gpu_ms (sum of its step times), device bytes it holds. */
pm_status_t pm_fused_batch_result(const pm_fused_batch* b, uint32_t i, pm_request_result* result);
pm_status_t pm_fused_batch_records(const pm_fused_batch* b, uint32_t i, pm_step_record* records, int32_t cap,
                                   int32_t* n_records);
pm_status_t pm_fused_batch_export(const pm_fused_batch* b, uint32_t i, uint64_t* cand_masks,
                                  uint8_t* edge_active, uint8_t* vertex_active);
void pm_fused_batch_destroy(pm_fused_batch* b);

/* Allocation-free ENUMERATION.  No counterpart in the reference: it serves
 * callers that cannot allocate device memory (code running inside a host
 * framework that owns every device allocation through its own pool or arena,
 * or a latency-critical path that must not reach the driver's allocator).
 *
 * Counts the injective embeddings of the template (p_*, CSR, 1 to 56
 * vertices) in a pruned state the caller holds in device memory: the graph
 * CSR (d_offsets[vertex_count + 1], d_adj[edge_count]), the candidate role
 * mask of every vertex (d_cand_masks[vertex_count], bit p = template vertex
 * p, as pm_query_export returns it) and the active flag of every CSR entry
 * as bits (d_edge_active_bits[(edge_count + 31) / 32], bit e % 32 of word
 * e / 32).  sorted_unique != 0 promises strictly increasing adjacency lists.
 * The count is written to d_count (one device uint64_t); the call returns
 * after `stream` (a cudaStream_t, NULL = default stream) has finished it.
 *
 * It calls no cudaMalloc, cudaFree or allocating library routine: the
 * walker's tables, counters and retry bitmaps live in one file-scope 64 MiB
 * __device__ array that every GPU loading this library holds until the
 * process exits.  The first call on a device (with that device current)
 * resolves the array's address with cudaGetSymbolAddress; make that first
 * call before any stream capture begins.  The resolved address is kept for
 * the life of the process, so a process that resets the device
 * (cudaDeviceReset) must not call this entry point on it again.  Every call
 * reuses the array and clears what must start at zero; calls that overlap
 * on the GPU (other streams or host threads at the same time) race on it
 * and must be serialised by the caller.  Each call reads the walker's
 * counters back to the host after every round, to decide whether sources
 * must be re-run with larger tables, and synchronises `stream` before it
 * returns.
 *
 * Limits: vertex_count <= 67108864 (PM_E_INVALID_ARG beyond), template of
 * at most 56 vertices (PM_E_PATTERN_TOO_LARGE), PM_E_OOM when one source's
 * count memo outgrows the array, PM_E_TIMEOUT past pm_set_walk_budget_ms. */
pm_status_t pm_enumerate_noalloc(const uint64_t* d_offsets, const uint32_t* d_adj,
                                 uint32_t vertex_count, uint64_t edge_count,
                                 int sorted_unique, const uint64_t* d_cand_masks,
                                 const uint32_t* d_edge_active_bits,
                                 const uint64_t* p_offsets, const uint32_t* p_adj,
                                 const uint64_t* p_labels, uint32_t p_vertex_count,
                                 uint64_t p_edge_count, uint64_t* d_count,
                                 void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PM_GB300_H */
