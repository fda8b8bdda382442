// Host engine: resident graph, per-query device state and the step machine.
#pragma once
#include <atomic>
#include <chrono>
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include <functional>

#include "constraints.h"
#include "effectiveness.h"
#include "kernels.h"
#include "walk_compile.h"

namespace pmgb {

[[noreturn]] void throw_cuda(cudaError_t e, const char* what);
#define PM_CUDA(call)                                  \
  do {                                                 \
    cudaError_t pm_err_ = (call);                      \
    if (pm_err_ != cudaSuccess) throw_cuda(pm_err_, #call); \
  } while (0)

// Device allocation owned by RAII.  With `stream` set, allocation and
// release are stream-ordered (cudaMallocAsync / cudaFreeAsync on that
// stream), so they never wait for work on other streams.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  bool ordered = false;
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  ~DeviceBuffer() { release(); }
  void release();
  void ensure(size_t n);  // grows (contents not kept)
  template <class T>
  T* as() const {
    return static_cast<T*>(ptr);
  }
};

// The graph: host CSR (the caller-visible graph_t) plus its device copy.
struct GraphImpl {
  HostGraph host;
  std::vector<label_t> dense_values;  // sorted distinct label values
  std::vector<uint32_t> dense_ids;    // per vertex
  bool sorted_unique = false;
  bool symmetric = false;  // sorted_unique and every entry has its reverse (checked on the device)
  int device = -1;
  DeviceBuffer d_off, d_adj, d_lab;
  // Target label byte per CSR entry (DevGraph::nlab), built with the device
  // copy when the graph has at most 256 distinct labels.
  DeviceBuffer d_nlab;
  // Degree classes of the LCC sweeps (DevGraph::hub_degree and segments).
  uint32_t hub_degree = kDefaultHubDegree, seg_entries = kDefaultSegEntries;
  uint32_t n_seg = 0, n_heavy = 0, n_acc = 0;
  DeviceBuffer d_seg;
  // New process-wide unique value whenever dev() changes (hub plan,
  // symmetric flag): captured graphs that baked another DevGraph are not
  // reused.
  uint64_t plan_epoch = 0;

  static constexpr uint32_t kDefaultHubDegree = 32;
  static constexpr uint32_t kDefaultSegEntries = 1024;

  // Dense labels; sorted_unique from a scan of the lists, or from *sorted
  // when the caller already checked them.
  void finalize_host(const bool* sorted = nullptr);
  // Device copy; adj_src (default: host.adj) is where the adjacency is read
  // from, e.g. the caller's own, possibly pinned, buffer while host.adj is
  // still being filled.
  void to_device(int device, const uint32_t* adj_src = nullptr);
  // Hubs = vertices of more than hub_degree CSR entries, in segments of
  // seg_entries entries (device tables rebuilt; graph must be on a device).
  void build_hub_plan(uint32_t hub_degree, uint32_t seg_entries);
  DevGraph dev() const;
  uint64_t device_bytes() const {
    return d_off.bytes + d_adj.bytes + d_lab.bytes + d_nlab.bytes + d_seg.bytes;
  }
};

// Runs f(lo, hi) over [0, n) in contiguous chunks on up to the host's
// hardware threads (one chunk when n is small).
void parallel_ranges(uint64_t n, const std::function<void(uint64_t, uint64_t)>& f);

// One pass over a caller's CSR: offsets non-decreasing, every target below
// vertex_count, every list strictly increasing.
struct CsrScan {
  bool monotone = true, in_range = true, sorted_unique = true;
};
CsrScan scan_csr(const uint64_t* offsets, const uint32_t* adj, uint32_t vertex_count);

// Walker scratch pool (memo tables), sized on demand.
struct WalkPool {
  DeviceBuffer edge, hyp, state, epochs;
  WalkScratch sc{};
  void ensure(uint32_t n_warps, uint32_t edge_cap, uint32_t hyp_cap, uint32_t hyp_stride, uint32_t state_cap,
              uint32_t state_stride, cudaStream_t s);
  uint64_t bytes() const { return edge.bytes + hyp.bytes + state.bytes + epochs.bytes; }
};

struct StepResult {
  int kind = PM_STEP_START;
  uint64_t vertex = 0, edge = 0, match = 0, enumeration = 0;
  bool empty() const { return !vertex && !edge && !match && !enumeration; }
};

// One compiled constraint with its programs resident on the device.
struct DeviceConstraint {
  CompiledConstraint cc;
  size_t prog_offset = 0;  // index into the query's device program array
  size_t role_row = 0;     // row of the query's device role-index table
  std::vector<uint8_t> start_roles;
};

struct QueryImpl {
  GraphImpl* g = nullptr;
  PatternGraph pattern;
  QueryConstraints qc;
  std::vector<DeviceConstraint> cycles, paths, templates;
  DeviceConstraint enumeration;
  uint32_t k = 0;
  int word_kind = kWord16;
  QueryTables tables{};
  std::vector<uint8_t> dense_to_slot;

  cudaStream_t stream = nullptr;
  bool own_stream = false;
  DeviceBuffer d_vs, d_eact, d_lt, d_mod, d_sch, d_unm, d_ctr, d_tables, d_d2s, d_hub_acc, d_tile_sch;
  DeviceBuffer d_progs, d_start_roles, d_role_index;
  DeviceBuffer d_wl, d_wl_index, d_blocks, d_count, d_status, d_marker, d_marks, d_list, d_list2, d_apply_v,
      d_apply_r, d_slices;
  DeviceBuffer d_slice_tiles;  // per-tile slice counts / offsets and the total (launch_slice_count)
  DeviceBuffer d_item_scratch;  // ENUMERATION item listing (launch_enum_item_count)
  StepCounters* h_ctr = nullptr;  // pinned
  uint32_t* h_count = nullptr;    // pinned
  bool own_host = true;           // h_ctr / h_count allocated here
  WalkPool pool, big_pool;

  // step machine (MultipleLabelStep, multiple_label_step.cc:30-83)
  int step = PM_STEP_START;
  size_t next_cc = 0, next_pc = 0, next_tds = 0;
  StepResult last;
  bool finished = false;
  int iteration = 0;
  uint64_t active_vertices = 0, active_edges = 0;
  double total_ms = 0;
  uint64_t match_count = 0;
  std::vector<pm_step_record> records;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_first = nullptr;
  bool first_recorded = false;
  double elapsed_ms();
  // Set by LCC0, cleared once an LCC pass ran: the next pass may read the
  // graph's entry labels instead of gathering (DevState::first).
  bool lcc_first_pending = false;

  // Request controls, checked before every step: a deadline (its remaining
  // time also caps each walker step's device budget), a cancel flag another
  // thread may set, and a stop before ENUMERATION (pruning only).
  // CC / PC / TDS walk semantics (NlccVariant, walk_compile.h); set before
  // create().  The article drivers' variants also advance through the
  // template constraints and end with END where the reference would count.
  int nlcc_variant = 0;
  // The article's constraint-order drivers (PM_ORDER_* bits; variants 1 and
  // 2 only), set before create().  order_threads is their OpenMP thread
  // count: the static blocks of the graph statistics and the estimates'
  // cost divisor.  Their NLCC steps drop the constraint they ran; the
  // dynamic order picks `chosen` among the remaining ones (rem_*).
  int order = 0;
  int order_threads = 1;
  std::vector<size_t> rem_cc, rem_pc, rem_tds;
  size_t chosen = 0;
  AccumulationMaximum acc_max;
  DeviceBuffer d_stat, d_stat_tab;
  // Graph statistics of the active graph on the device (GraphStatCpu), with
  // the vertices in `threads` static-schedule blocks (0: order_threads).
  GraphStat graph_stat(int threads = 0);
  bool has_deadline = false;
  std::chrono::steady_clock::time_point deadline{};
  const std::atomic<bool>* cancel = nullptr;
  bool stop_before_enumeration = false;

  // statistics of the alreadyMatched emulation
  uint64_t exact_resolutions = 0, overflow_retries = 0;
  // The step that ended the run with PM_E_TIMEOUT (its walkers passed their
  // deadline): kind (-1: none), device time, walker CSR entries tested and
  // hops taken until then.  It has no result row.
  int aborted_kind = -1;
  double aborted_ms = 0;
  uint64_t aborted_scanned = 0, aborted_hops = 0;
  // per step: walker CSR entries tested and hops taken (0 for LCC steps)
  std::vector<std::pair<uint64_t, uint64_t>> walk_stats;

  ~QueryImpl();
  // s: the query's stream (null: a stream of its own).  ext_ctr / ext_count:
  // pinned host words the caller owns and keeps for the query's lifetime
  // (null: allocated here).  Device buffers are stream-ordered on s.
  void create(GraphImpl* graph, const PatternGraph& p, cudaStream_t s, StepCounters* ext_ctr = nullptr,
              uint32_t* ext_count = nullptr);
  QueryDevPtrs ptrs() const;
  uint64_t device_bytes() const;

  // Runs the current step and advances the machine; returns the row.
  pm_step_record run_step();
  void run_all(int max_iterations = 1000);
  // One unit of a whole run: the LCC fixpoint as one captured launch when
  // the schedule is at LCC (and the switch is on), otherwise one step.
  void run_unit(int max_iterations = 1000);
  // Request checks made before every step of a whole run: cancel flag
  // (PM_E_CANCELLED), deadline (PM_E_TIMEOUT); caps this host thread's
  // walker budget at the time left.
  void check_request();
  // Batched form over queries of one graph, each at a step boundary with
  // nothing in flight on its stream; `s` carries the fused launches.
  // lcc0_batch: the LCC0 step of every listed query (all at LCC0), as
  // multi-query launches.  lcc_fixpoint_batch: every listed query (all at
  // LCC with active vertices) runs LCC passes until its own fixpoint (or the
  // iteration cap); each pass of the batch is one multi-query launch
  // sequence over the queries still iterating.  Rows and state are those of
  // the queries' own steps.
  static void lcc0_batch(const std::vector<QueryImpl*>& qs, cudaStream_t s);
  static void lcc_fixpoint_batch(const std::vector<QueryImpl*>& qs, cudaStream_t s);
  pm_step_record final_record();

  void export_state(uint64_t* cand, uint8_t* eact, uint8_t* vact);
  // Every device buffer the query owns.
  std::vector<DeviceBuffer*> buffers();
  void write_outputs(const std::string& dir);
  // The embeddings ENUMERATION counts (the pruning runs first when the query
  // has not reached ENUMERATION yet): up to cap of them, n_hist vertex ids
  // each in walk order, into out; returns the total (the ENUMERATION count;
  // 0 when the run ends at the iteration cap before ENUMERATION).
  uint64_t list_matches(uint32_t* out, uint64_t cap, uint32_t* per_match);
  // The pruned subgraph in CSR form over the original ids: offsets[V + 1],
  // and up to cap entries into adj; returns the entry count.
  uint64_t export_subgraph(uint64_t* offsets, uint32_t* adj, uint64_t cap);

 private:
  void reset_modified();
  void clear_step_counters();
  void read_counters();
  StepResult step_lcc0();
  StepResult step_lcc();
  StepResult step_nlcc(const DeviceConstraint& dc);
  StepResult step_enumeration();
  uint32_t build_worklist(uint64_t mask);
  void pool_strides(uint32_t* hyp_stride, uint32_t* state_stride) const;
  void ensure_pool();
  void run_walks(const DeviceConstraint& dc, uint32_t n_wl, bool record_marks);
  void resolve_exact(const DeviceConstraint& dc, uint32_t n_wl);
  int advance(int cur);
  // The dynamic order's next step after an LCC fixpoint; sets `chosen`.
  int choose_dynamic();
  size_t cc_index() const;
  size_t pc_index() const;
  size_t tds_index() const;
  void ensure_hub_acc();
  // Runs LCC passes until the fixpoint (or max_iterations) in one graph
  // launch and appends one row per pass, as run_step would.
  void run_lcc_loop(int max_iterations);
  void append_record(const StepResult& r, int kind, double ms, uint64_t scanned, uint64_t second);
};

// Walker memo table entries per warp in the first walk round.
constexpr uint32_t kEdgeCapEntries = 1024, kHypCapEntries = 1024, kStateCapEntries = 2048;

std::string step_name(int kind);
PatternGraph load_pattern(const std::string& dir, bool load_labels);
// ENUMERATION overflow policy (process-wide): sources whose count memo
// overflowed `after_levels` times with growing tables are split into up to
// `parts` first-hop slices (parts <= 1: never split).
void set_enum_split(uint32_t parts, uint32_t after_levels);
// ENUMERATION sources with more first-hop entries than this start as slices
// of that many entries (0: every source starts whole); one value for both
// program kinds, or for programs with / without a count memo.
void set_enum_presplit(uint32_t slice_entries);
void set_enum_presplit(bool count_memo, uint32_t slice_entries);
uint32_t enum_presplit(bool count_memo);
// Exact CC/PC/TDS programs: items whose source has more first-hop entries
// than this run as slices of that many entries (0: never).
void set_walk_presplit(uint32_t slice_entries);
uint32_t walk_presplit();
// State-memo entries per warp in the first CC/PC/TDS walk round.
void set_walk_table_entries(uint32_t entries);
uint32_t walk_table_entries();
// Count-memo entries per warp in ENUMERATION's first round (power of two).
void set_enum_table_entries(uint32_t entries);
uint32_t enum_table_entries();
// Whole-run paths (run_all) run each LCC fixpoint as one captured CUDA graph
// (default on); off: one host-driven launch sequence per pass.
void set_lcc_graph(bool on);
bool lcc_graph();
// First LCC pass after LCC0 from the graph's entry labels (DevState::first).
void set_lcc_label_stream(bool on);
bool lcc_label_stream();
uint64_t next_plan_epoch();

// Fault injection on the host: the n-th device buffer allocation from now on
// (0 = the next one) fails as an out-of-memory cudaMalloc would; -1 = off.
void set_fail_alloc_after(int64_t n);

// Wall-clock budget of every whole run (run_all: pm_query_run, served and
// batched requests), from its start; 0 = none.  Process-wide.
void set_query_budget_ms(double ms);
double query_budget_ms();

// Device bytes a query of a k-vertex template holds in its first walk
// round (state, worklists, first walker pool); the admission charge.
uint64_t estimate_query_bytes(const GraphImpl& g, uint32_t k);

}  // namespace pmgb
