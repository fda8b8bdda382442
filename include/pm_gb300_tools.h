/*
 * pm_gb300_tools.h — helpers around the pm_gb300.h boundary that the
 * reference has no counterpart for: seeded synthetic inputs (standing in for
 * the reference's external datasets), zero-copy access to the host CSR of a
 * pm_graph, and engine statistics.  Not needed by a drop-in caller.
 */
#ifndef PM_GB300_TOOLS_H
#define PM_GB300_TOOLS_H

#include "pm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Undirected RMAT graph: 2^scale vertices, edge_factor * 2^scale sampled
 * pairs with quadrant probabilities a, b, c (d = 1-a-b-c), symmetrised,
 * self-loops and duplicate edges removed, adjacency sorted; vertex ids
 * shuffled by a seeded permutation when permute != 0.  The graph is host-
 * only until pm_graph_to_device (or a query) moves it to a device. */
pm_status_t pm_graph_generate_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                                   int32_t permute, pm_graph** out);

/* Vertex labels 0..n_labels-1: kind 0 = uniform, 1 = Zipf(zipf_s),
 * 2 = correlated with degree rank.  Must precede device residency. */
pm_status_t pm_graph_assign_labels(pm_graph* g, int32_t kind, uint32_t n_labels, double zipf_s, uint64_t seed);

/* Graph ingestion tools, the TOTEM generator's ALTER commands
 * (src/generator/totem_generator.cc): host-side, on a graph not yet on a
 * device (the new graphs are host-only until pm_graph_to_device).
 * UNDIRECTED (:631-680): a new graph in which every CSR entry u -> v of g
 * gives u -> v and v -> u (duplicates kept; each list holds its entries in
 * reverse order of appearance, as the generator's edgelist_to_graph builds
 * it, :92-125).  SORT_NEIGHBOURS (:764-770): every list of g sorted
 * ascending, in place.  SORT_VERTICES (:682-748): a new graph with ids
 * renumbered by ascending degree (ties: ascending old id — the reference's
 * parallel sort leaves their order unspecified); old_to_new (V entries,
 * may be NULL) receives the renumbering.  Labels stay with their vertices. */
pm_status_t pm_graph_make_undirected(const pm_graph* g, pm_graph** out);
pm_status_t pm_graph_sort_neighbours(pm_graph* g);
pm_status_t pm_graph_sort_vertices_by_degree(const pm_graph* g, pm_graph** out, uint32_t* old_to_new);

/* Library-owned host CSR of g (valid until pm_graph_destroy). */
pm_status_t pm_graph_host_csr(const pm_graph* g, const uint64_t** offsets, const uint32_t** adj,
                              const uint64_t** labels);

/* Copies the CSR to device `device` (no-op when already there). */
pm_status_t pm_graph_to_device(pm_graph* g, int32_t device);

/* Degree classes of the LCC sweeps: vertices with more than hub_degree CSR
 * entries (at most 2^26) are hubs whose adjacency is split into segments of
 * seg_entries entries, each checked by its own warp (defaults 128 and 1024).
 * Affects speed only, never results.  The graph must be on a device and no
 * query of it may be running. */
pm_status_t pm_graph_set_hub_plan(pm_graph* g, uint32_t hub_degree, uint32_t seg_entries);

/* Writes the graph as TOTEM text and its labels as a vertex file. */
pm_status_t pm_graph_write_text(const pm_graph* g, const char* graph_path, const char* labels_path);

/* Number of visible CUDA devices (0 when none or the driver is missing). */
int32_t pm_device_count(void);

/* Kernel launches issued by this library since the process started. */
uint64_t pm_kernel_launches(void);

/* Device time of the query so far: from the start of its first step to the
 * end of its latest step, measured with CUDA events on the query's stream
 * (host gaps between steps included). */
pm_status_t pm_query_elapsed_ms(const pm_query* q, double* ms);

/* ENUMERATION overflow policy (process-wide; speed only, never results): a
 * source whose count memo overflowed with `after_levels` levels of 8x larger
 * tables is split into up to `parts` slices of its first hop, run by
 * separate warps with base-size tables (parts <= 1: never split); a slice
 * that overflows again grows its tables.  Defaults 16 and 0.  Set it while
 * no query runs. */
pm_status_t pm_set_enum_split(uint32_t parts, uint32_t after_levels);

/* ENUMERATION sources with more than slice_entries first-hop entries start
 * as slices of that many entries, queued before the other sources, so hub
 * sources are spread over many warps from the start (0: every source starts
 * whole; defaults 32 for templates whose enumeration uses a count memo, 8
 * for the others; this call sets both).  Process-wide; speed only.  Set it
 * while no query runs. */
pm_status_t pm_set_enum_presplit(uint32_t slice_entries);

/* pm_set_enum_presplit per kind: templates whose enumeration uses a count
 * memo, and the others. */
pm_status_t pm_set_enum_presplit_by_kind(uint32_t with_count_memo, uint32_t without_count_memo);

/* Autotuner over the speed-only choices (no counterpart in the reference):
 * runs up to max_per_group of the templates whose enumeration uses a count
 * memo (pairwise distinct labels) and up to max_per_group of the others
 * under candidate LCC degree classes (pm_graph_set_hub_plan), walk slice
 * and state-memo sizes, enumeration slice sizes (per kind;
 * pm_set_enum_presplit sets both) and count-memo sizes, keeps the choices
 * with the least device time in force and reports them.  Every candidate must reproduce the same match counts.  No query of
 * g may be running. */
typedef struct pm_tune_result {
  uint32_t hub_degree, seg_entries;
  uint32_t enum_presplit_memo, enum_presplit_plain, enum_table_entries;
  uint32_t walk_presplit, walk_table_entries;
  uint32_t probes_memo, probes_plain, runs;
  uint32_t enum_tail_swap, walk_tail_swap, enum_count_memo, walk_tail_state_memo;
  uint32_t enum_pair_tail, walk_pair_tail, enum_second_split;
} pm_tune_result;

pm_status_t pm_autotune(pm_graph* g, const pm_template_csr* templates, uint32_t n,
                        uint32_t max_per_group, pm_tune_result* result);

/* CC/PC/TDS walks of exact programs (no memo test can block, see the
 * walker): an item whose source has more than slice_entries first-hop
 * entries runs as slices of that many entries on separate warps, and
 * succeeds when any slice does (0: never; default 64).  Process-wide; speed
 * only.  Set it while no query runs. */
pm_status_t pm_set_walk_presplit(uint32_t slice_entries);

/* State-memo entries per warp in the first CC/PC/TDS walk round (power of
 * two, 1024 to 2^20; default 8192).  Process-wide; speed only.  Set it while
 * no query runs. */
pm_status_t pm_set_walk_table_entries(uint32_t entries);

/* Count-memo entries per warp in ENUMERATION's first round (power of two,
 * 1024 to 2^20; default 8192).  Larger tables let more sources finish in
 * the first round at the cost of device memory (warps x entries x (7 + k)
 * words per query).  Process-wide; speed only.  Set it while no query runs. */
pm_status_t pm_set_enum_table_entries(uint32_t entries);

/* Whole-run calls (pm_query_run, the server, pm_batch_run) run each LCC
 * fixpoint (LCC repeated until a pass eliminates nothing,
 * multiple_label_step.cc:30-83) as one CUDA-graph launch: a conditional
 * WHILE node over one pass, whose last kernel records the pass's row and
 * decides on the device whether another pass runs.  Rows, counts and state
 * are those of the host-driven loop; only the step_ms column is measured
 * differently (device timer per pass).  pm_query_step always runs one pass.
 * enabled = 0 turns it off (default 1).  Process-wide; speed only.  No
 * counterpart in the reference. */
pm_status_t pm_set_lcc_graph(int32_t enabled);

/* The first LCC pass after LCC0 reads one byte per CSR entry, the label of
 * the entry's target (built once with the graph's device copy when the graph
 * has at most 256 distinct labels: E bytes of device memory), instead of
 * loading the target id and gathering its role word: after LCC0 every
 * vertex holds exactly the roles of its label, so the byte determines the
 * word.  Rows, counts and state are those of the gathering pass.  enabled =
 * 0 turns it off (default 1).  Process-wide; speed only.  No counterpart in
 * the reference (lcc :26-101 reads the neighbour's state every pass). */
pm_status_t pm_set_lcc_label_stream(int32_t enabled);

/* ENUMERATION's last VERTEX step before the closing CHECKs (e.g. the fourth
 * vertex of a 4-cycle, checked against the source): on symmetric graphs,
 * when the source's list is cached (at most 256 entries) and the current
 * vertex's list has at least `ratio` times as many 32-entry chunks as the
 * source's entries holding the step's role, the step iterates over those
 * source entries and searches the current vertex's list, instead of scanning
 * the current vertex's list and searching the source's.  Both count the same
 * set (enumeration_cpu.tpp:96-104 semantics).  0 = never; default 4.
 * Process-wide; speed only.  No counterpart in the reference. */
pm_status_t pm_set_enum_tail_swap(uint32_t ratio);

/* The same choice for the last VERTEX step of exact CC/PC/TDS programs
 * (no memo test can block them): from the source's side, the step's first
 * passing candidate is still the smallest vertex id the forward scan would
 * find first, so results and alreadyMatched marks are unchanged.  0 =
 * never; default 4.  Process-wide; speed only.  No counterpart in the
 * reference. */
pm_status_t pm_set_walk_tail_swap(uint32_t ratio);

/* ENUMERATION of templates with distinct labels keeps, per source, a table of
 * subtree counts (a vertex reached again at the same step with the same
 * history adds the cached count instead of walking again).  enabled = 0
 * walks every subtree.  Counts are the same either way; default 1.
 * Process-wide; speed only.  No counterpart in the reference. */
pm_status_t pm_set_enum_count_memo(int32_t enabled);

/* Exact CC/PC/TDS programs keep a per-walk state memo (a state that failed
 * once fails again, since a success ends the walk).  enabled = 0 leaves it
 * out at the step just before the closing CHECKs, where repeating the tail
 * step can cost less than a memo probe and insert.  Results are the same
 * either way; default 1.  Process-wide; speed only.  No counterpart in the
 * reference. */
pm_status_t pm_set_walk_tail_state_memo(int32_t enabled);

/* The step just before such a tail (e.g. the third vertex of a 4-cycle):
 * instead of binding each candidate and running the tail step below it, the
 * warp tests every (candidate, cached source entry) pair, one pair per lane.
 * ENUMERATION counts the passing pairs; an exact CC/PC/TDS walk takes the
 * first passing pair in (candidate CSR order, entry ascending) order, its
 * depth-first first success.  Results are the same either way.  Separate
 * switches for ENUMERATION and for walks; default 1 / 1.  Process-wide; speed
 * only.  No counterpart in the reference. */
pm_status_t pm_set_pair_tail(int32_t enumeration, int32_t walks);

/* ENUMERATION work items below the first hop: in a source of more than
 * `entries` first-hop entries, a first-hop vertex whose own list has more
 * than 2 x `entries` entries runs as separate items, one per `entries`-entry
 * slice of its list at the second hop (for templates whose second step binds
 * a new vertex and whose tail does not start at the second step).  Counts
 * are the same; 0 = never; default 256.  Process-wide; speed only.  No
 * counterpart in the reference. */
pm_status_t pm_set_enum_second_split(uint32_t entries);

/* Time budget of one CC/PC/TDS or ENUMERATION step (default 120000 ms):
 * one absolute deadline, set when the step's first walker warp starts, bounds
 * every launch and retry round of the step (and each pm_enumerate_noalloc
 * call as a whole).  A walk still running past it stops; the step then fails
 * with PM_E_TIMEOUT and the query's state is no longer meaningful.  The
 * host-side work between launches is not interrupted, so a step can overrun
 * the budget by that much. */
pm_status_t pm_set_walk_budget_ms(double ms);

/* Count-memo entries per warp in the first round of pm_enumerate_noalloc
 * (power of two in [32, 65536], default 2048); each later round, which
 * re-runs only the sources whose tables overflowed, has 4x more.  Smaller
 * values make more sources overflow into later rounds; the count is the
 * same.  Process-wide; set it while no such call runs. */
pm_status_t pm_set_noalloc_table_entries(uint32_t entries);

/* Rounds run by the calling thread's last pm_enumerate_noalloc call: 1 when
 * every source fit its first-round tables, more when some were re-run. */
uint32_t pm_noalloc_last_rounds(void);

/* Wall-clock budget of every whole run: pm_query_run / pm_query_prune,
 * served requests (from admission) and pm_batch_run templates (0 = none,
 * the default).  Checked before every step; the remaining time also caps
 * each walker step's device budget (pm_set_walk_budget_ms), so a request
 * ends with PM_E_TIMEOUT soon after its budget runs out.  Process-wide. */
pm_status_t pm_set_query_budget_ms(double ms);

/* Host-side fault injection for tests: the n-th device buffer allocation
 * the library makes from now on (0 = the next one) fails the way an
 * out-of-memory cudaMalloc does, so the call in progress returns PM_E_OOM
 * and frees what it held; -1 turns it off.  Nothing reaches the device.
 * Process-wide. */
pm_status_t pm_debug_fail_device_alloc_after(int64_t n);

/* Statistics of a batched run: lockstep rounds, and shared LCC phases
 * (multi-query LCC0 launches and fused fixpoints) it issued. */
pm_status_t pm_fused_batch_stats(const pm_fused_batch* b, uint64_t* rounds, uint64_t* shared_lcc_phases);

/* Compiles a template (no device needed) and writes the reference-format
 * constraint dump, as pm_query_dump_constraints does. */
pm_status_t pm_template_dump_constraints(const uint64_t* p_offsets, const uint32_t* p_adj, const uint64_t* p_labels,
                                         uint32_t p_vertex_count, uint64_t p_edge_count, char* buf, size_t cap,
                                         size_t* needed);

/* Work of result row `row` (0-based, as returned by pm_query_run): for
 * CC/PC/TDS and ENUMERATION, the CSR entries tested and hops taken by the
 * walkers; for LCC, the CSR entries in the lists the sweep checked and how
 * many of them it read a neighbour word for (the others point to vertices
 * already seen without roles); 0 for LCC0. */
pm_status_t pm_query_step_walk_stats(const pm_query* q, int32_t row, uint64_t* scanned, uint64_t* descents);

/* Number of NLCC steps that needed the exact sequential emulation of the
 * reference's alreadyMatched shortcut, and of memo-table overflow retries. */
pm_status_t pm_query_stats(const pm_query* q, uint64_t* exact_resolutions, uint64_t* overflow_retries);

/* The graph statistics the dynamic constraint order ranks constraints by
 * (GraphStatCpu::compute, src/patternmatching/algorithms/graph_stat_cpu.tpp:
 * 42-80), taken on the GPU over the query's current state: active vertices
 * and the active CSR entries between them, with the vertices split into
 * `threads` static-schedule blocks whose neighbour-label accumulation is
 * never reset between a block's vertices.  Labels are the template's
 * distinct labels in order of first appearance: *n_labels of them (at most
 * 64) into labels[].  vertex_total[a], edge_total[a * n + b] and
 * at_least[(a * n + b) * 64 + i] (label-a vertices whose block's running
 * count of label-b neighbours reached i, for i up to the largest number of
 * label-b neighbours a label-a template vertex has; 0 elsewhere).  Outputs
 * may be NULL; arrays sized for 64 labels always suffice.  PM_E_STATISTICS
 * where the reference's accumulation lookup would throw (an active label
 * whose template vertices have no neighbours), or while an active vertex
 * carries no template label (before the first LCC0 or LCC step). */
pm_status_t pm_query_graph_stat(pm_query* q, int32_t threads, uint32_t* n_labels, uint64_t* labels,
                                uint64_t* vertex_total, uint64_t* edge_total, uint64_t* at_least);

/* The step that ended a run with PM_E_TIMEOUT because its walkers passed
 * their deadline (it has no result row): its kind, device time, and the CSR
 * entries its walkers tested and hops they took until then (the counters of
 * pm_query_step_walk_stats).  PM_FAILURE when no step was cut short. */
pm_status_t pm_query_aborted_step(const pm_query* q, int32_t* step, double* step_ms, uint64_t* scanned,
                                  uint64_t* hops);

#ifdef __cplusplus
}
#endif
#endif /* PM_GB300_TOOLS_H */
