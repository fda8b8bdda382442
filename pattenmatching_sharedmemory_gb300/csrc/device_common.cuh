// Device-side layout of the resident graph and of one query's pruning state.
//
// HBM layout (one graph, many queries):
//   graph   off  u64[V+1]   CSR offsets (eid_t, 64-bit)
//           adj  u32[E]     neighbour ids (vid_t)
//           lab  u32[V]     dense label id (index into the graph's sorted
//                           distinct label values)
//   query   vs   W[V]       packed vertex word: candidate role bits in the
//                           low kCandBits, the vertex's label slot in the
//                           pattern's label list above them (0xFF = a label
//                           no template vertex carries).  Active <=> cand != 0
//                           (the reference keeps a separate vertexActiveList,
//                           multiple_label_common_cpu.h:49-53, but a vertex is
//                           deactivated exactly when its role set empties).
//           eact u32[ceil(E/32)]  one active bit per CSR entry
//           mod  u8[V]      vertexModifiedList
//           sch  u8[V]      vertexScheduledList
//           unm  W[V]       vertexPatternToUnmatch (cand bits only)
// The word type W is chosen per query from the template size k:
//   k <= 8 -> u16, k <= 24 -> u32, k <= 56 -> u64, else a 16-byte pair.
// One gather of W per neighbour yields both its role set (LCC possibility
// test, NLCC role test) and its label slot (LCC label counting).
#pragma once
#include <cstdint>

#include "walk_program.h"

namespace pmgb {

struct alignas(16) Wide {
  uint64_t c;
  uint64_t s;
};

template <class W>
struct Pack;
template <>
struct Pack<uint16_t> {
  static constexpr int kMaxK = 8;
  static __host__ __device__ __forceinline__ uint64_t cand(uint16_t w) { return w & 0xFFu; }
  static __host__ __device__ __forceinline__ uint32_t slot(uint16_t w) { return w >> 8; }
  static __host__ __device__ __forceinline__ uint16_t make(uint64_t c, uint32_t s) {
    return static_cast<uint16_t>((s << 8) | (c & 0xFFu));
  }
  static __host__ __device__ __forceinline__ uint16_t zero() { return 0; }
};
template <>
struct Pack<uint32_t> {
  static constexpr int kMaxK = 24;
  static __host__ __device__ __forceinline__ uint64_t cand(uint32_t w) { return w & 0xFFFFFFu; }
  static __host__ __device__ __forceinline__ uint32_t slot(uint32_t w) { return w >> 24; }
  static __host__ __device__ __forceinline__ uint32_t make(uint64_t c, uint32_t s) {
    return (s << 24) | static_cast<uint32_t>(c & 0xFFFFFFu);
  }
  static __host__ __device__ __forceinline__ uint32_t zero() { return 0; }
};
template <>
struct Pack<uint64_t> {
  static constexpr int kMaxK = 56;
  static __host__ __device__ __forceinline__ uint64_t cand(uint64_t w) { return w & 0x00FFFFFFFFFFFFFFull; }
  static __host__ __device__ __forceinline__ uint32_t slot(uint64_t w) { return static_cast<uint32_t>(w >> 56); }
  static __host__ __device__ __forceinline__ uint64_t make(uint64_t c, uint32_t s) {
    return (static_cast<uint64_t>(s) << 56) | (c & 0x00FFFFFFFFFFFFFFull);
  }
  static __host__ __device__ __forceinline__ uint64_t zero() { return 0; }
};
template <>
struct Pack<Wide> {
  static constexpr int kMaxK = 64;
  static __host__ __device__ __forceinline__ uint64_t cand(const Wide& w) { return w.c; }
  static __host__ __device__ __forceinline__ uint32_t slot(const Wide& w) { return static_cast<uint32_t>(w.s); }
  static __host__ __device__ __forceinline__ Wide make(uint64_t c, uint32_t s) { return Wide{c, s}; }
  static __host__ __device__ __forceinline__ Wide zero() { return Wide{0, 0}; }
};

struct DevGraph {
  uint32_t V;
  uint64_t E;
  const uint64_t* __restrict__ off;
  const uint32_t* __restrict__ adj;
  const uint32_t* __restrict__ lab;
  int sorted_unique;  // every adjacency list strictly increasing
  // Degree classes of the LCC sweeps: a vertex with more than hub_degree
  // CSR entries is a hub, its list cut into segments of seg_entries entries
  // that one warp each streams; lighter vertices go in tiles of 32
  // (n_seg == 0: every vertex is light).  seg[0, n_heavy) are the segments
  // of hubs with several segments, seg[n_heavy, n_seg) the single-segment
  // hubs.
  uint32_t hub_degree;
  uint32_t seg_shift;    // seg_entries = 1 << seg_shift, 32 to 1024
  uint32_t n_seg;
  uint32_t n_heavy;
  uint32_t n_acc;                  // hubs with more than one segment
  // A vertex with more than seg_entries entries has segments i covering its
  // entries in [(off[v] / seg_entries + i) * seg_entries, + seg_entries)
  // (never crossing a multiple of seg_entries); a shorter one has a single
  // segment covering its whole list.
  const uint4* __restrict__ seg;   // [n_seg] {vertex, segment index, segments, accumulator}
  // Every CSR entry u -> w has its reverse w -> u (lists strictly increasing).
  int symmetric;
  // Label of each CSR entry's target (dense label id, lab[adj[e]]), one byte
  // per entry; null when the graph has more than 256 distinct labels.  The
  // first LCC pass after LCC0 reads it instead of gathering neighbour words.
  const uint8_t* __restrict__ nlab;
};

// Per-query accumulator of a hub with several segments.  Zero between
// launches: the last segment of the hub to finish reads and clears it.
constexpr uint32_t kHubRanks = 16;  // needed label slots the sweep counts per owner
struct HubAcc {
  uint32_t cnt[kHubRanks];  // sweep 1: surviving neighbours per needed slot (by rank)
  uint32_t elim;            // sweep 1: CSR entries eliminated
  uint32_t ticket;          // sweep 1: segments finished
  uint32_t hit;             // sweep 2: a segment saw a modified active neighbour
  uint32_t ticket2;         // sweep 2: segments finished
};

template <class W>
struct DevState {
  W* vs;
  uint32_t* eact;
  uint8_t* mod;
  uint8_t* sch;
  W* unm;
  // Live-target bits: a subset of eact without the entries whose target
  // was seen with no role left (roles never come back).  The LCC sweep
  // skips entries outside it; nothing else reads it.
  uint32_t* lt;
  // Per 32-vertex tile: 0 when sweep 2 left no vertex of the tile both
  // holding a role and scheduled (hubs under the current plan count as
  // scheduled), so LCC sweep 1 can skip the tile.  Null: no summary.
  uint8_t* tile_sch;
  // 1 for the first LCC pass after LCC0 when DevGraph::nlab exists: every
  // vertex then holds exactly the roles of its label slot, so a neighbour's
  // word follows from the entry's label byte (QueryTables::dense_slot).
  uint32_t first;
};

// Device counters.  The first kStepCounterWords words are per step
// (AlgoResults plus walker bookkeeping) and are cleared before every step;
// modified_total lives across steps and is cleared together with the
// modified flags (before CC/PC/TDS, as the reference's resetState does).
struct StepCounters {
  unsigned long long vertex_elim;
  unsigned long long edge_elim;
  unsigned long long match_elim;
  unsigned long long enumeration;
  unsigned long long overflow;   // walker items that ran out of memo space
  unsigned long long flagged;    // failing items an earlier success may rescue
  unsigned long long items;      // work counter for persistent kernels
  unsigned long long error;      // device-side error status (0 = ok)
  unsigned long long aux;        // list fill counter (overflow retry list)
  unsigned long long scanned;    // walkers: CSR entries tested; LCC: entries of the checked lists
  unsigned long long descents;   // walkers: hops taken (states entered)
  unsigned long long gathered;   // LCC: entries whose neighbour word was read
  // Walkers: absolute %globaltimer deadline of the step, 0 until the first
  // warp of the step's first walker launch sets it (now + budget).  Every
  // later warp, launch and retry round of the step uses the same value, so
  // the budget bounds the whole step, not each launch or resident wave.
  unsigned long long deadline_ns;
  unsigned long long modified_total;  // vertices with mod=1 since the last reset
  unsigned long long pad[2];
};
constexpr int kStepCounterWords = 13;

// The LCC fixpoint loop as one CUDA graph (a conditional WHILE node over one
// LCC pass): the tail of every pass appends its counters as a row, clears the
// step counters and keeps the loop going while the pass eliminated anything
// and the iteration cap allows (multiple_label_step.cc:30-83 repeats LCC
// until its AlgoResults is empty; multiple_label_cpu.cc:113-184 caps the run
// at 1000 iterations).
struct LccPassRow {
  unsigned long long vertex_elim, edge_elim, match_elim, scanned, gathered;
  unsigned long long end_ns;  // %globaltimer at the end of the pass
};
struct LccLoopCtl {
  unsigned long long start_ns;  // %globaltimer before the first pass
  unsigned long long error;     // step-counter error status seen by a tail
  uint32_t passes;              // passes run by this launch
  uint32_t max_passes;          // set by the host before each launch, >= 1
  unsigned long long pad;
};
constexpr uint32_t kLccLoopMaxPasses = 1000;

// Per-query tables derived from the local constraints
// (multiple_label_constraint_local.h:18-32), in label-slot space.
struct QueryTables {
  uint32_t k;
  uint32_t n_slots;
  uint8_t role_slot[64];         // slot of originLabel(p)
  uint64_t nbr_mask[64];         // localConstraintNeighborVertex(p)
  uint64_t req_slots[64];        // slots with a required count for p
  uint8_t req[64][64];           // required neighbour count, [role][slot]
  uint64_t slot_roles[256];      // roles whose origin label has this slot
  uint8_t dense_slot[256];       // slot of dense label ids 0..255
};

#ifdef __CUDACC__
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t warp_or32(uint32_t x) { return __reduce_or_sync(0xFFFFFFFFu, x); }

__device__ __forceinline__ uint64_t warp_or64(uint64_t x) {
  uint32_t lo = __reduce_or_sync(0xFFFFFFFFu, static_cast<uint32_t>(x));
  uint32_t hi = __reduce_or_sync(0xFFFFFFFFu, static_cast<uint32_t>(x >> 32));
  return (static_cast<uint64_t>(hi) << 32) | lo;
}

__device__ __forceinline__ bool edge_active(const uint32_t* __restrict__ eact, uint64_t e) {
  return (eact[e >> 5] >> (e & 31)) & 1u;
}

// Clears the active bits of CSR entries base + j for every set bit j of m.
__device__ __forceinline__ void clear_edge_bits(uint32_t* eact, uint64_t base, uint32_t m) {
  const uint64_t word = base >> 5;
  const uint32_t sh = static_cast<uint32_t>(base & 31);
  const uint64_t wide = static_cast<uint64_t>(m) << sh;
  const uint32_t lo = static_cast<uint32_t>(wide), hi = static_cast<uint32_t>(wide >> 32);
  if (lo) atomicAnd(eact + word, ~lo);
  if (hi) atomicAnd(eact + word + 1, ~hi);
}
#endif  // __CUDACC__

__host__ __device__ __forceinline__ uint32_t mix32(uint32_t h, uint32_t k) {
  k *= 0xcc9e2d51u;
  k = (k << 15) | (k >> 17);
  k *= 0x1b873593u;
  h ^= k;
  h = (h << 13) | (h >> 19);
  return h * 5u + 0xe6546b64u;
}
__host__ __device__ __forceinline__ uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

}  // namespace pmgb
