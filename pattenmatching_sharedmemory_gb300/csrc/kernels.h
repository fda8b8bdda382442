// Host-callable launchers for the GB300 kernels.  Plain pointers only; the
// packed vertex-word type is selected at run time by QueryDevPtrs::word_kind.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "device_common.cuh"
#include "walk_program.h"

namespace pmgb {

enum WordKind : int { kWord16 = 0, kWord32 = 1, kWord64 = 2, kWordWide = 3 };

inline int word_kind_for(uint32_t k) { return k <= 8 ? kWord16 : k <= 24 ? kWord32 : k <= 56 ? kWord64 : kWordWide; }
inline size_t word_bytes(int kind) { return kind == kWord16 ? 2 : kind == kWord32 ? 4 : kind == kWord64 ? 8 : 16; }

struct QueryDevPtrs {
  int word_kind;
  void* vs;
  uint32_t* eact;
  uint8_t* mod;
  uint8_t* sch;
  void* unm;
  StepCounters* ctr;
  const QueryTables* tables;
  HubAcc* hub_acc;  // [DevGraph::n_acc]
  uint32_t* lt;     // live-target bits (DevState::lt)
  uint8_t* tile_sch;  // DevState::tile_sch, ceil(V / 32) bytes
  uint32_t first_pass;  // DevState::first (the captured loop's tail clears it)
};

// Launch geometry shared by all kernels (SM count of the current device).
int device_sm_count();

// Process-wide count of kernel launches issued by this library.
void note_launch();
uint64_t launch_count();

// State initialisation: every vertex holds all k roles and its label slot,
// every CSR entry is active, every vertex scheduled, nothing modified
// (MultipleLabelGlobalState::allocate, multiple_label_common_cpu.tpp:30-66).
void launch_init_state(const DevGraph& g, const QueryDevPtrs& q, const uint8_t* dense_to_slot, uint64_t full_cand,
                       cudaStream_t s);

// Symmetry check of a graph whose adjacency lists are strictly increasing:
// res[3] zeroed before; afterwards the graph is symmetric (every entry
// u -> w has its reverse w -> u) iff res[0] == 0 and res[1] == res[2].
void launch_check_symmetric(const DevGraph& g, unsigned long long* res, cudaStream_t s);

// nlab[e] = lab[adj[e]] (dense label ids below 256) for every CSR entry;
// adj must be 16-byte aligned.
void launch_build_entry_labels(const DevGraph& g, uint8_t* nlab, cudaStream_t s);

// LCC0 (multiple_label_lcc0_cpu.tpp:15-87).
void launch_lcc0(const DevGraph& g, const QueryDevPtrs& q, cudaStream_t s);

// LCC sweep 1 (multiple_label_lcc_cpu.tpp:26-101).
void launch_lcc_check(const DevGraph& g, const QueryDevPtrs& q, cudaStream_t s);

// Sweep 2 shared by LCC and CC/PC/TDS (lcc :107-141, cc :134-173).
void launch_apply(const DevGraph& g, const QueryDevPtrs& q, cudaStream_t s);
// Kernels of the captured LCC fixpoint loop (rows follow ctl in memory).
void launch_lcc_loop_head(LccLoopCtl* ctl, cudaStream_t s);
void launch_lcc_loop_tail(QueryDevPtrs* a, LccLoopCtl* ctl, cudaGraphConditionalHandle h, cudaStream_t s);
// One LCC pass with the query's pointers read from the device block `a`.
void launch_lcc_pass_at(const DevGraph& g, int word_kind, const QueryDevPtrs* a, cudaStream_t s);
// Adds launches that ran inside graphs (captured launches count once).
void note_launches(int64_t n);
// Launches issued by the calling host thread.
uint64_t thread_launch_count();

// Order-preserving compaction of the vertices that hold a role of
// `start_mask`: wl[i] = i-th such vertex, wl_index[wl[i]] = i, *count = n.
// block_counts needs ceil(V / 4096) + 1 entries.
// Batched LCC (many queries of one graph in each launch): queries
// active[0, nq) of the device array qs, all of word type word_kind.  LCC0 of
// every listed query; one LCC pass (sweep 1 + sweep 2) of every listed query;
// their per-step counters cleared (clear) or copied to out[0, nq).
void launch_lcc0_multi(const DevGraph& g, int word_kind, const QueryDevPtrs* qs, const uint32_t* active, uint32_t nq,
                       cudaStream_t s);
void launch_lcc_pass_multi(const DevGraph& g, int word_kind, const QueryDevPtrs* qs, const uint32_t* active,
                           uint32_t nq, cudaStream_t s);
void launch_counters_multi(const QueryDevPtrs* qs, const uint32_t* active, uint32_t nq, StepCounters* out, bool clear,
                           cudaStream_t s);

// First-hop slices of the heavy items of an exact walk (worklist positions
// whose vertex has more than t CSR entries): ceil(deg / t) slices per
// program, {pos * R + r, lo, min(lo + t, deg), 0} in (pos, r, lo) order.
// Count: per 4096-position tile counts (ceil(n_wl / 4096) words), scanned in
// place, and the total in *total; write: the slices at the scanned offsets.
void launch_slice_count(const DevGraph& g, const uint32_t* wl, uint32_t n_wl, uint32_t R, uint32_t t,
                        unsigned long long* tile_counts, unsigned long long* total, cudaStream_t s);
void launch_slice_write(const DevGraph& g, const uint32_t* wl, uint32_t n_wl, uint32_t R, uint32_t t,
                        const unsigned long long* tile_offsets, uint4* slices, cudaStream_t s);

// ENUMERATION's up-front items over the worklist's sources: a source with
// more than t first-hop entries (heavy) takes items {i, lo, hi, 0} over runs
// of at most t entries of its list; with s2 > 0 and more than s2 entries, a
// first-hop position whose vertex has more than 2 * s2 entries closes the
// run before it and takes ceil(d1 / s2) items {i, pos, pos + 1, k + 1}.
// Heavy items first (worklist, then list order), then {i, 0, 2^32 - 1, 0}
// per light source.  Count: enum_item_scratch_words(n_wl) u64 words of
// scratch; afterwards enum_item_totals(scratch, n_wl) holds on the device
// {heavy items, light items, overflow flag}.  Write: the items, at `items`.
uint64_t enum_item_scratch_words(uint32_t n_wl);
void launch_enum_item_count(const DevGraph& g, const uint32_t* wl, uint32_t n_wl, uint32_t t, uint32_t s2,
                            unsigned long long* scratch, cudaStream_t s);
const unsigned long long* enum_item_totals(const unsigned long long* scratch, uint32_t n_wl);
void launch_enum_item_write(const DevGraph& g, const uint32_t* wl, uint32_t n_wl, uint32_t t, uint32_t s2,
                            const unsigned long long* scratch, uint4* items, cudaStream_t s);

// Graph statistics of the dynamic constraint order (GraphStatCpu::compute,
// algorithms/graph_stat_cpu.tpp:42-80) over the query's active graph, with
// the vertices split into `blocks` static-schedule blocks of q or q + 1 ids
// (the first r blocks one longer).  Outputs are zeroed by the caller:
//   vseg[t * S + a]            active vertices of slot a in block t
//   edges[a * S + b]           active CSR entries from slot a to slot b
//   at_least[(a * (S + 1) + b) * 64 + i]  label-a vertices whose block's
//                              running count of slot-b neighbours (b == S:
//                              of any neighbour) has reached i, for i up to
//                              max[a * (S + 1) + b]
//   *bad                       set when an active vertex carries no slot
// thr[b] = the largest max[. * (S + 1) + b] (0: column not needed).
struct GraphStatDev {
  uint32_t slots, blocks;
  uint64_t q, r;
  unsigned long long* vseg;
  unsigned long long* edges;
  unsigned long long* at_least;
  unsigned long long* bad;
  const uint8_t* max;
  const uint32_t* thr;
};
void launch_graph_stat(const DevGraph& g, const QueryDevPtrs& q, const GraphStatDev& p, cudaStream_t s);

void launch_worklist(const DevGraph& g, const QueryDevPtrs& q, uint64_t start_mask, uint32_t* wl,
                     uint32_t* wl_index, uint32_t* block_counts, uint32_t* count, cudaStream_t s);

// Walker item status.
enum ItemStatus : uint8_t { kItemSkip = 0, kItemFail = 1, kItemSuccess = 2, kItemOverflow = 3, kItemTimeout = 4 };

// StepCounters::error values written by kernels.
constexpr unsigned long long kDeviceErrorTimeout = 2;

// Time budget of one walker step (ns of %globaltimer): the step's first warp
// fixes the deadline in StepCounters::deadline_ns; a warp past it stops,
// marks its item kItemTimeout and sets kDeviceErrorTimeout.
void set_walk_budget_ns(uint64_t ns);
// ENUMERATION tail step from the cached source's side when the bound
// vertex's list has at least `ratio` times as many 32-entry chunks as the
// source's entries holding the tail role (0: never).
void set_enum_tail_swap(uint32_t ratio);
uint32_t enum_tail_swap();
// ENUMERATION programs that allow a count memo use it (default on).
void set_enum_count_memo(bool on);
bool enum_count_memo();
// Exact CC/PC/TDS programs use the state memo at the step before the tail
// (default on; off re-runs the tail step for a repeated state).
void set_walk_tail_state_memo(bool on);
bool walk_tail_state_memo();
// The step before a qualifying tail tests (candidate, cached source entry)
// pairs one per lane (ENUMERATION, or exact CC/PC/TDS programs; default on).
void set_pair_tail(bool enumeration, bool on);
bool pair_tail_on(bool enumeration);
// ENUMERATION items may restrict the second hop to slices of this many
// entries of the first-hop vertex's list (item.w = slice + 1; 0: never).
void set_enum_second_split(uint32_t entries);
uint32_t enum_second_split();
// The same for the tail step of exact CC/PC/TDS programs (WalkLaunch::tail_swap).
void set_walk_tail_swap(uint32_t ratio);
uint32_t walk_tail_swap();
uint64_t walk_budget_ns();
// Per host thread: caps the walker budget of the launches this thread issues
// (a request's remaining time); 0 = no cap.
void set_thread_walk_budget_cap_ns(uint64_t ns);
// The budget this thread's next walker launch gets.
uint64_t effective_walk_budget_ns();

// Per-warp scratch for the walkers' memo tables.  The edge and hypothesis
// tables reproduce the reference's memos and must hold every entry (a walk
// that fills them is re-run with larger tables); the state table is a
// best-effort cache (state memo / count memo, see walk_program.h).
struct WalkScratch {
  uint32_t* edge_tab;    // per warp 4 * edge_cap words: columns tag, a, b, step
  uint32_t* hyp_tab;     // n_warps * hyp_cap * hyp_stride words
  uint32_t* state_tab;   // n_warps * state_cap * state_stride words
  uint32_t* epochs;      // n_warps
  uint32_t n_warps;
  uint32_t edge_cap;     // power of two
  uint32_t hyp_cap;      // power of two
  uint32_t hyp_stride;   // 3 + stored vertices
  uint32_t state_cap;    // power of two
  uint32_t state_stride; // 5 + state key words (the last two hold a count)
};

struct WalkLaunch {
  const WalkProgram* progs;  // n_progs programs (device)
  const uint8_t* start_roles;  // n_progs start roles (device)
  uint32_t n_progs;
  const uint8_t* role_index;  // 64 entries (device)
  const uint32_t* wl;
  const uint32_t* wl_index;
  uint32_t n_wl;
  const uint32_t* retry_items;  // when non-null: only these items (n_retry)
  uint32_t n_retry;
  uint8_t* status;        // n_wl * n_progs
  uint32_t* min_marker;   // n_wl * n_progs, or null
  uint32_t* marks;        // n_wl * n_progs * marks_stride, or null
  uint32_t marks_stride;
  // Exact programs only: items whose source has more than skip_deg entries
  // are left out of the main launch and run as `slices` ({item, first-hop
  // lo, hi, -}) whose results meet in prio[item] (atomicMax of kPrio*).
  uint32_t skip_deg;
  const uint4* slices;
  uint32_t n_slices;
  uint32_t* prio;
  uint32_t frame_steps;  // frame stack entries per warp: longest program's n_steps + 1
  uint32_t tail_swap;    // exact programs: tail from the source's side (walk_tail_swap())
  uint32_t tail_state_memo;  // exact programs: state memo at the step before the tail
  uint32_t pair_tail;        // exact programs: pair-parallel step before the tail
};

// Walker launch geometry: resident blocks per SM the kernels are built for,
// and the dynamic shared memory of one warp's frame stack of `steps` entries.
constexpr uint32_t kWalkBlocksPerSm = 12;
__host__ __device__ constexpr uint32_t frame_bytes(uint32_t steps) {
  return (steps * (4 * 8 + 3 * 4 + 1) + 15) / 16 * 16;
}

// Result priorities of sliced items: success of any slice decides the item.
enum SlicePrio : uint32_t { kPrioSkip = 0, kPrioFail = 1, kPrioOverflow = 2, kPrioTimeout = 3, kPrioSuccess = 4 };

// status[item] of every sliced item (source degree > skip_deg) from prio.
void launch_prio_to_status(const DevGraph& g, const WalkLaunch& w, cudaStream_t s);

// Phase 1 of CC/PC/TDS: every (vertex, start role) walk, in parallel.
void launch_walk(const DevGraph& g, const QueryDevPtrs& q, const WalkLaunch& w, const WalkScratch& scratch,
                 cudaStream_t s);

// Phase 2: count failing items that an earlier success marked.
void launch_flag_rescue(const WalkLaunch& w, StepCounters* ctr, cudaStream_t s);

// Phase 3: failing items become roles to unmatch (all of them, or only
// those listed by the host's exact resolution).
void launch_apply_failures(const DevGraph& g, const QueryDevPtrs& q, const WalkLaunch& w, cudaStream_t s);
// Lists the items whose walk ran out of memo space (ctr->aux = count).
void launch_collect_overflow(const WalkLaunch& w, uint32_t* list, StepCounters* ctr, cudaStream_t s);
// Blocks of the persistent walker for a scratch pool of n_warps warps.
uint32_t walk_grid_blocks(uint32_t n_warps_available);
// Per host thread: walker launches (and walker pools sized after them) take
// 1/share of the GPU's resident walker blocks (at least one block per SM):
// a server slot among `share` slots.  1 = the whole GPU (default).
void set_thread_walk_grid_share(uint32_t share);
constexpr uint32_t kWalkWarpsPerBlock = 4;
void launch_apply_unmatch_list(const DevGraph& g, const QueryDevPtrs& q, const uint32_t* vertices, const uint64_t* roles,
                               uint32_t n, cudaStream_t s);

// ENUMERATION: sums injective embeddings from every worklist vertex, or
// over `items` {worklist position, lo, hi, -} whose first hop is limited to
// positions [lo, hi) of the source's adjacency list.  Items whose count memo
// overflowed are written to `overflow` as {position, lo, hi, source vertex}
// (count in ctr->aux) and contribute nothing.
void launch_enumerate(const DevGraph& g, const QueryDevPtrs& q, const WalkProgram* prog, uint32_t frame_steps,
                      const uint32_t* wl, uint32_t n_wl, const uint4* items, uint32_t n_items, uint4* overflow,
                      const WalkScratch& scratch, cudaStream_t s);

// Lists the embeddings of the ENUMERATION program `prog` from every
// worklist source: each completed walk takes slot counters[1]++ and, below
// cap, writes its n_hist history vertices to out[slot * n_hist ...];
// counters[0] is the work counter (both start at 0).  Stops with
// kDeviceErrorTimeout in q.ctr past the walker budget.
void launch_enum_list(const DevGraph& g, const QueryDevPtrs& q, const WalkProgram* prog, const uint32_t* wl,
                      uint32_t n_wl, uint32_t* out, uint64_t cap, unsigned long long* counters, cudaStream_t s);

// The pruned subgraph (active CSR entries between active vertices): with
// out_adj null, counts[v] = such entries of v; else writes them to
// out_adj[out_off[v] ...] in CSR order.
void launch_subgraph(const DevGraph& g, const QueryDevPtrs& q, const uint64_t* out_off, uint64_t* counts,
                     uint32_t* out_adj, cudaStream_t s);

// Export of the pruned state.
void launch_export(const DevGraph& g, const QueryDevPtrs& q, uint64_t* cand, uint8_t* vact, uint8_t* eact_bytes,
                   cudaStream_t s);

// Allocation-free ENUMERATION over a caller-held state (64-bit role masks
// per vertex, one active bit per CSR entry): the walker's tables, counters
// and retry bitmaps live in a fixed 64 MiB __device__ array instead of
// device allocations.  Writes the embedding count to d_count (device) and
// synchronises `s`.  The first call on a device resolves the array's address
// (cudaGetSymbolAddress).  Calls share the array: overlapping calls race.
// Throws PmError (PM_E_INVALID_ARG above noalloc_max_vertices(), PM_E_OOM
// when one source's count memo outgrows the array, PM_E_TIMEOUT, PM_E_DEVICE).
uint32_t noalloc_max_vertices();
// Count-memo entries per warp in the first round of enumerate_noalloc
// (power of two; each retry round has 4x more).  Default 2048.
void set_noalloc_table_entries(uint32_t entries);
// Rounds (1 + retry rounds) of the calling thread's last enumerate_noalloc.
uint32_t noalloc_last_rounds();
void enumerate_noalloc(const DevGraph& g, const uint64_t* d_cand, const uint32_t* d_edge_active,
                       const WalkProgram& prog, uint32_t state_words, uint64_t* d_count, cudaStream_t s);

}  // namespace pmgb
