// Local constraint checking on GB300: state init, LCC0, LCC sweep 1, the
// shared sweep 2, worklist compaction and export.
//
// Mapping: a warp owns a tile of 32 consecutive vertices.  It loads the 32
// vertex words (and schedule flags) coalesced, ballots the ones with work,
// and then streams each selected vertex's adjacency 32 CSR entries at a time:
// lane j takes entry base+j, tests its active bit, gathers the neighbour's
// packed word (role set + label slot) and the warp reduces with ballot/popc.
// All updates a vertex makes in sweep 1 touch only its own out-entries and
// flags, so sweep 1 is race-free (the reference's Jacobi-style first loop,
// multiple_label_lcc_cpu.tpp:26-101); sweep 2 is a separate launch.
#include <cuda_runtime.h>

#include <algorithm>

#include <atomic>

#include "kernels.h"

namespace pmgb {
namespace {

constexpr int kThreads = 256;
constexpr int kWarpsPerBlock = kThreads / 32;
constexpr unsigned kFull = 0xFFFFFFFFu;

std::atomic<int> g_sm_count{0};
std::atomic<uint64_t> g_launches{0};

inline int grid_for_tiles(uint64_t V, int blocks_per_sm) {
  uint64_t tiles = (V + 31) / 32;
  uint64_t blocks = (tiles + kWarpsPerBlock - 1) / kWarpsPerBlock;
  uint64_t cap = static_cast<uint64_t>(device_sm_count()) * blocks_per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return static_cast<int>(blocks);
}

// ---- init ---------------------------------------------------------------
template <class W>
__global__ void __launch_bounds__(kThreads) k_init_state(DevGraph g, DevState<W> st, const uint8_t* __restrict__ d2s,
                                                         uint64_t full) {
  const uint64_t tid = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t v = tid; v < g.V; v += stride) {
    st.vs[v] = Pack<W>::make(full, d2s[g.lab[v]]);
    st.unm[v] = Pack<W>::zero();
    st.mod[v] = 0;
    st.sch[v] = 1;
    if ((v & 31) == 0 && st.tile_sch) st.tile_sch[v >> 5] = 1;
  }
  const uint64_t words = (g.E + 31) / 32;
  for (uint64_t i = tid; i < words; i += stride) {
    uint64_t remaining = g.E - i * 32;
    const uint32_t w = remaining >= 32 ? 0xFFFFFFFFu : ((1u << remaining) - 1u);
    st.eact[i] = w;
    st.lt[i] = w;
  }
}

// ---- graph properties -------------------------------------------------------
// Index of `target` in the strictly increasing list adj[lo, hi), or ~0:
// interpolation steps (the ids of a list spread evenly in most graphs, so a
// guess from the end values lands close) alternating with halvings (which
// bound the steps by twice the binary search's), then a scan of the last
// 16 entries.
__device__ __forceinline__ uint64_t find_sorted(const uint32_t* __restrict__ adj, uint64_t lo, uint64_t hi,
                                                uint32_t target) {
  bool interp = true;
  while (hi - lo > 16) {
    const uint32_t a = adj[lo], b = adj[hi - 1];
    if (target < a || target > b) return ~uint64_t(0);
    uint64_t mid;
    if (interp && b > a) {
      // A guess only (any position in [lo, hi) keeps the search exact), so
      // single precision replaces a 64-bit division.
      const uint64_t span = hi - 1 - lo;
      uint64_t step = static_cast<uint64_t>(static_cast<float>(target - a) / static_cast<float>(b - a) *
                                            static_cast<float>(span));
      mid = lo + (step < span ? step : span);
    } else {
      mid = lo + ((hi - lo) >> 1);
    }
    interp = !interp;
    const uint32_t x = adj[mid];
    if (x == target) return mid;
    if (x < target)
      lo = mid + 1;
    else
      hi = mid;
  }
  for (; lo < hi; ++lo) {
    const uint32_t x = adj[lo];
    if (x == target) return lo;
    if (x > target) break;
  }
  return ~uint64_t(0);
}

// Symmetry of a graph with strictly increasing lists: every entry u -> w
// with u < w finds u in w's list, and the entries with u < w and u > w are
// equally many (the reverses of the former are distinct entries of the
// latter, so equal counts leave none without a reverse; self-loops are
// their own).  res[0] = 1 when an entry has no reverse; res[1], res[2]
// count the entries with u < w and u > w.  Warp per task, lane per entry:
// the tasks are the segments of the hub plan's multi-segment hubs (so no
// warp walks a hub's whole list alone; RMAT hubs reach 10^6 entries), then
// every vertex, skipping those the segments cover.
__global__ void __launch_bounds__(kThreads) k_check_symmetric(DevGraph g, unsigned long long* res) {
  const unsigned lane = lane_id();
  const uint64_t warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t n_warps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  const uint64_t seg_entries = uint64_t(1) << g.seg_shift;
  unsigned long long up = 0, down = 0;
  uint32_t polls = 0;
  for (uint64_t task = warp; task < g.n_heavy + g.V; task += n_warps) {
    // Another warp found an entry without reverse: stop (warp-uniform read,
    // every 16th task).
    if ((polls++ & 15) == 0) {
      const unsigned found = lane == 0 ? (*reinterpret_cast<volatile unsigned long long*>(res) != 0) : 0u;
      if (__shfl_sync(kFull, found, 0)) break;
    }
    uint64_t u, b, e;
    if (task < g.n_heavy) {
      const uint4 sd = g.seg[task];
      u = sd.x;
      const uint64_t a = g.off[u], z = g.off[u + 1];
      const uint64_t blk = (a >> g.seg_shift) + sd.y;
      b = sd.y == 0 ? a : blk << g.seg_shift;
      const uint64_t lim = (blk + 1) << g.seg_shift;
      e = z < lim ? z : lim;
    } else {
      u = task - g.n_heavy;
      b = g.off[u];
      e = g.off[u + 1];
      if (g.n_heavy && e - b > g.hub_degree && e - b > seg_entries) continue;  // in the segments above
    }
    bool missing = false;
    for (uint64_t x0 = b; x0 < e && !missing; x0 += 32) {
      const uint64_t x = x0 + lane;
      bool miss = false;
      if (x < e) {
        const uint32_t w = g.adj[x];
        if (u < w) {
          ++up;
          miss = find_sorted(g.adj, g.off[w], g.off[w + 1], static_cast<uint32_t>(u)) == ~uint64_t(0);
        } else if (u > w) {
          ++down;
        }
      }
      missing = __any_sync(kFull, miss);
    }
    if (missing) {
      if (lane == 0) atomicOr(res, 1ull);
      break;
    }
  }
  for (int o = 16; o; o >>= 1) {
    up += __shfl_xor_sync(kFull, up, o);
    down += __shfl_xor_sync(kFull, down, o);
  }
  if (lane == 0) {
    if (up) atomicAdd(res + 1, up);
    if (down) atomicAdd(res + 2, down);
  }
}

// Label byte of every CSR entry's target (DevGraph::nlab): four entries per
// thread and step, the adj reads coalesced, the label reads gathered once
// per graph.
__global__ void __launch_bounds__(kThreads) k_build_entry_labels(DevGraph g, uint8_t* __restrict__ nlab) {
  const uint64_t tid = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  const uint64_t quads = g.E / 4;
  for (uint64_t i = tid; i < quads; i += stride) {
    const uint4 a = reinterpret_cast<const uint4*>(g.adj)[i];
    const uint32_t packed = (g.lab[a.x] & 0xFFu) | (g.lab[a.y] & 0xFFu) << 8 | (g.lab[a.z] & 0xFFu) << 16 |
                            (g.lab[a.w] & 0xFFu) << 24;
    reinterpret_cast<uint32_t*>(nlab)[i] = packed;
  }
  for (uint64_t e = quads * 4 + tid; e < g.E; e += stride) nlab[e] = static_cast<uint8_t>(g.lab[g.adj[e]]);
}

// ---- LCC0 ---------------------------------------------------------------
template <class W>
__global__ void __launch_bounds__(kThreads) k_lcc0(DevGraph g, DevState<W> st, const QueryTables* __restrict__ qt,
                                                   StepCounters* ctr) {
  __shared__ uint64_t slot_roles[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) slot_roles[i] = qt->slot_roles[i];
  __syncthreads();
  unsigned long long me = 0, ve = 0;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t v = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; v < g.V; v += stride) {
    W w = st.vs[v];
    uint64_t c = Pack<W>::cand(w);
    if (!c) continue;
    uint32_t s = Pack<W>::slot(w);
    uint64_t nc = c & slot_roles[s];
    if (nc != c) {
      me += __popcll(c ^ nc);
      st.vs[v] = Pack<W>::make(nc, s);
      if (!nc) ++ve;
    }
  }
  me = __reduce_add_sync(kFull, static_cast<unsigned>(me));
  ve = __reduce_add_sync(kFull, static_cast<unsigned>(ve));
  if (lane_id() == 0) {
    if (me) atomicAdd(&ctr->match_elim, me);
    if (ve) atomicAdd(&ctr->vertex_elim, ve);
  }
}

// ---- LCC sweep 1 --------------------------------------------------------
//
// A grid of resident warps over a task list; warp w takes tasks w, w + W,
// w + 2W, ...  The first tasks each cover 32 hub segments (seg_entries CSR
// entries of a vertex with more than hub_degree entries): the lanes test the
// 32 segments' vertices at once, then the warp streams each live segment,
// kUnroll x 32 entries per iteration, every lane counting the surviving
// neighbours of each needed label slot in its own shared counters.  A hub
// with one segment decides its roles at once; the others add their counts
// to the hub's HubAcc and its last segment to finish decides.  The remaining
// tasks are tiles of 32 consecutive light vertices, whose adjacency lists
// the warp streams back to back: a warp prefix sum over the lanes' degrees
// maps a stream index to its owner lane, and counts go per (owner, slot)
// with one update per group of equal keys (__match_any_sync).

constexpr int kUnroll = 4;
constexpr int kLccWarps = kThreads / 32;
constexpr uint8_t kNoRank = 0xFF;

struct LccTables {
  uint64_t nbr[64];
  uint64_t need[64];
  uint8_t role_slot[64];
  uint8_t req[64][64];
  // First pass after LCC0 (DevState::first): role set and slot of a vertex
  // by its dense label id.
  uint64_t lab_cand[256];
  uint8_t lab_slot[256];
};

struct LccWarp {
  uint32_t cnt[kHubRanks][32];  // tiles: [rank][owner lane]; segments: [rank][counting lane]
  uint32_t tot[kHubRanks];      // segments: totals per rank
  uint8_t rank_of[64];          // needed slot -> rank, kNoRank otherwise
  uint8_t code[256];            // first-pass kernel, segments: dense label -> kCode* or count rank
};

// First-pass entry codes of a segment's vertex, by the target's label: a
// count rank (< kHubRanks), or one of these.
constexpr uint8_t kCodeKeep = 0xFD;  // a possible neighbour, label not counted
constexpr uint8_t kCodeElim = 0xFE;  // target holds roles, none a neighbour role: entry eliminated
constexpr uint8_t kCodeDead = 0xFF;  // target holds no role: live-target bit cleared

// Rank table of `slots` and zeroed counters for its n_slots ranks.
__device__ __forceinline__ void set_ranks(LccWarp& lw, uint64_t slots, uint32_t n_slots) {
  const unsigned lane = lane_id();
  __syncwarp();
  for (uint32_t s = lane; s < 64; s += 32)
    lw.rank_of[s] = (slots >> s & 1) ? static_cast<uint8_t>(__popcll(slots & ((uint64_t(1) << s) - 1))) : kNoRank;
  for (uint32_t r = 0; r < n_slots; ++r) lw.cnt[r][lane] = 0;
  __syncwarp();
}

__device__ __forceinline__ void load_lcc_tables(LccTables& t, const QueryTables* __restrict__ qt, uint32_t k,
                                                bool first) {
  for (uint32_t i = threadIdx.x; i < 64; i += blockDim.x) {
    t.nbr[i] = qt->nbr_mask[i];
    t.need[i] = qt->req_slots[i];
    t.role_slot[i] = qt->role_slot[i];
  }
  const uint32_t rows = k < 64 ? k : 64;
  for (uint32_t i = threadIdx.x; i < rows * 64; i += blockDim.x) t.req[i / 64][i % 64] = qt->req[i / 64][i % 64];
  if (first) {
    for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) {
      const uint8_t sl = qt->dense_slot[i];
      t.lab_slot[i] = sl;
      t.lab_cand[i] = qt->slot_roles[sl];
    }
  }
  __syncthreads();
}

// The neighbour word of CSR entry e as LCC sweep 1 sees it.  In the first
// pass after LCC0 every vertex holds exactly the roles of its label slot
// (LCC0 intersected the full role set with them, and sweep 1 changes no
// role), so the entry's label byte gives the word without the dependent
// adj -> vs gather; later passes gather.
template <class W>
__device__ __forceinline__ W label_word(const LccTables& t, uint32_t lb) {
  return Pack<W>::make(t.lab_cand[lb], t.lab_slot[lb]);
}

__device__ __forceinline__ uint64_t shfl64(uint64_t x, int src) {
  const uint32_t lo = __shfl_sync(kFull, static_cast<uint32_t>(x), src);
  const uint32_t hi = __shfl_sync(kFull, static_cast<uint32_t>(x >> 32), src);
  return (static_cast<uint64_t>(hi) << 32) | lo;
}

// Mask of lanes [lo, hi) of a 32-lane slice, clamped to the slice.
__device__ __forceinline__ uint32_t lane_range(int64_t lo, int64_t hi) {
  lo = lo < 0 ? 0 : lo;
  hi = hi > 32 ? 32 : hi;
  if (hi <= lo) return 0;
  const uint32_t n = static_cast<uint32_t>(hi - lo);
  return (n == 32 ? kFull : ((1u << n) - 1)) << static_cast<uint32_t>(lo);
}

// CSR entry range [beg, end) of hub segment sd (DevGraph::seg).
__device__ __forceinline__ void segment_range(const DevGraph& g, const uint4 sd, uint64_t* beg, uint64_t* end) {
  const uint64_t a = g.off[sd.x], b = g.off[sd.x + 1];
  if (sd.z == 1) {
    *beg = a;
    *end = b;
    return;
  }
  const uint64_t blk = (a >> g.seg_shift) + sd.y;
  *beg = sd.y == 0 ? a : blk << g.seg_shift;
  const uint64_t lim = (blk + 1) << g.seg_shift;
  *end = b < lim ? b : lim;
}

// Union of the template neighbours of the roles in cu, and the label slots
// any of them needs counted.
__device__ __forceinline__ void role_unions(const LccTables& t, uint64_t cu, uint64_t* ncs, uint64_t* need) {
  uint64_t a = 0, b = 0;
  for (uint64_t rr = cu; rr; rr &= rr - 1) {
    const uint32_t p = __ffsll(static_cast<long long>(rr)) - 1;
    a |= t.nbr[p];
    b |= t.need[p];
  }
  *ncs = a;
  *need = b;
}

// role_unions for one vertex held by the whole warp (lane p looks at roles
// p and p + 32).
__device__ __forceinline__ void role_unions_warp(const LccTables& t, uint64_t cu, uint64_t* ncs, uint64_t* need) {
  const unsigned lane = lane_id();
  uint64_t a = 0, b = 0;
  if (cu >> lane & 1) {
    a = t.nbr[lane];
    b = t.need[lane];
  }
  if (cu >> (lane + 32) & 1) {
    a |= t.nbr[lane + 32];
    b |= t.need[lane + 32];
  }
  *ncs = warp_or64(a);
  *need = warp_or64(b);
}

// failing_roles for one vertex held by the whole warp: lane p decides roles
// p and p + 32 from the per-rank totals in lw.tot.
__device__ __forceinline__ uint64_t failing_roles_warp(const LccTables& t, const LccWarp& lw, uint64_t cu,
                                                       uint32_t su) {
  const unsigned lane = lane_id();
  bool bad[2] = {false, false};
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const uint32_t p = lane + 32 * half;
    if (cu >> p & 1) {
      bool b = t.role_slot[p] != su;
      for (uint64_t ss = t.need[p]; ss && !b; ss &= ss - 1) {
        const uint32_t sl = __ffsll(static_cast<long long>(ss)) - 1;
        if (t.req[p][sl] > lw.tot[lw.rank_of[sl]]) b = true;
      }
      bad[half] = b;
    }
  }
  return static_cast<uint64_t>(__ballot_sync(kFull, bad[0])) |
         (static_cast<uint64_t>(__ballot_sync(kFull, bad[1])) << 32);
}

// Roles of u that fail: the role's label differs from u's, or a required
// neighbour-label count is not met (lcc :79-100).  cnt(rank) is the count of
// the rank-th set slot of `slots`.
template <class F>
__device__ __forceinline__ uint64_t failing_roles(const LccTables& t, uint64_t cu, uint32_t su, uint64_t slots,
                                                  F cnt) {
  uint64_t tu = 0;
  for (uint64_t rr = cu; rr; rr &= rr - 1) {
    const uint32_t p = __ffsll(static_cast<long long>(rr)) - 1;
    bool bad = t.role_slot[p] != su;
    uint32_t rank = 0;
    for (uint64_t ss = slots; ss && !bad; ss &= ss - 1, ++rank) {
      const uint32_t s = __ffsll(static_cast<long long>(ss)) - 1;
      if (t.req[p][s] > cnt(rank)) bad = true;
    }
    if (bad) tu |= uint64_t(1) << p;
  }
  return tu;
}

// Per-lane tallies of a sweep-1 launch (one warp's share of a launch stays
// below 2^32).
struct LccTally {
  uint32_t edge_elim = 0;       // CSR entries eliminated
  uint32_t newly_modified = 0;  // vertices newly flagged modified
  uint32_t streamed = 0;        // CSR entries in the checked lists
  uint32_t gathered = 0;        // ... whose neighbour word was read
};

// Records the outcome of vertex u's check (lcc :65-100): modified when it
// lost a role or an edge, roles to unmatch in unm.
template <class W>
__device__ __forceinline__ void lcc_record(const DevState<W>& st, uint32_t u, uint64_t tu, uint32_t elim,
                                           uint32_t& newly_modified) {
  if (tu || elim) {
    if (!st.mod[u]) {
      st.mod[u] = 1;
      ++newly_modified;
    }
  }
  if (tu) st.unm[u] = Pack<W>::make(tu, 0);
}

// Whole-list check of one vertex by one warp, for owners that need more than
// kHubRanks label slots counted.
template <class W>
__device__ void lcc_vertex_warp(const DevGraph& g, const DevState<W>& st, const LccTables& t, uint32_t u,
                                LccTally& tl) {
  const unsigned lane = lane_id();
  const W wu = st.vs[u];
  const uint64_t cu = Pack<W>::cand(wu);
  const uint32_t su = Pack<W>::slot(wu);
  uint64_t ncs, need;
  role_unions(t, cu, &ncs, &need);
  uint32_t cnt_lo = 0, cnt_hi = 0;  // lane r: counts of the r-th and (r+32)-th slot of `need`
  uint32_t elim_u = 0;
  const uint64_t beg = g.off[u], end = g.off[u + 1];
  for (uint64_t e0 = beg; e0 < end; e0 += 32) {
    const uint64_t e = e0 + lane;
    const bool act = e < end && edge_active(st.eact, e);
    W ww = Pack<W>::zero();
    if (act) {
      if (st.first) {
        ww = label_word<W>(t, g.nlab[e]);
      } else {
        ww = st.vs[g.adj[e]];
        ++tl.gathered;
      }
    }
    const uint64_t cw = Pack<W>::cand(ww);
    const bool live = act && cw != 0;
    const bool poss = live && (cw & ncs) != 0;
    const unsigned em = __ballot_sync(kFull, live && !poss);
    if (em) {
      if (lane == 0) {
        clear_edge_bits(st.eact, e0, em);
        clear_edge_bits(st.lt, e0, em);
      }
      elim_u += __popc(em);
    }
    const uint32_t sw = Pack<W>::slot(ww);
    uint32_t rank = 0;
    for (uint64_t nd = need; nd; nd &= nd - 1, ++rank) {
      const uint32_t s = __ffsll(static_cast<long long>(nd)) - 1;
      const unsigned m = __ballot_sync(kFull, poss && sw == s);
      if (lane == (rank & 31)) {
        if (rank < 32)
          cnt_lo += __popc(m);
        else
          cnt_hi += __popc(m);
      }
    }
  }
  // cu and need are warp-uniform: every lane walks the same loops.
  const uint64_t tu = failing_roles(t, cu, su, need, [&](uint32_t rank) {
    return __shfl_sync(kFull, rank < 32 ? cnt_lo : cnt_hi, rank & 31);
  });
  if (lane == 0) {
    lcc_record(st, u, tu, elim_u, tl.newly_modified);
    tl.edge_elim += elim_u;
    tl.streamed += end - beg;
  }
}

// The first pass after LCC0 over hub segment [beg, end) of a vertex whose
// roles' neighbour union is ncs: every target word follows from the entry's
// label byte (label_word), so the warp streams the segment's label bytes,
// 16 per lane in one 16-byte load (512 entries per warp step), instead of
// visiting live-target words.  A per-warp table gives each label's code for
// this vertex; counts go to the lane's column of lw.cnt, and the lane pair
// of each 32-entry word merges its halves so that one lane clears the
// word's bits.  Decisions, bit updates and counts are those of the
// word-driven loop of lcc_segment.  Returns the entries eliminated
// (warp-uniform).
template <class W>
__device__ __forceinline__ uint32_t lcc_segment_first(const DevGraph& g, const DevState<W>& st,
                                                      const LccTables& t, LccWarp& lw, uint64_t ncs, uint64_t beg,
                                                      uint64_t end) {
  const unsigned lane = lane_id();
  for (uint32_t lb = lane; lb < 256; lb += 32) {
    const uint64_t cw = t.lab_cand[lb];
    uint8_t c = kCodeKeep;
    if (cw == 0) {
      c = kCodeDead;
    } else if ((cw & ncs) == 0) {
      c = kCodeElim;
    } else {
      const uint32_t sw = t.lab_slot[lb];
      if (sw < 64 && lw.rank_of[sw] != kNoRank) c = lw.rank_of[sw];
    }
    lw.code[lb] = c;
  }
  __syncwarp();
  uint32_t elim = 0;
  // Steps start on a 32-entry word: lanes 2i and 2i + 1 cover word i's low
  // and high halves.  nlab is padded to a multiple of 32 bytes, so a 16-byte
  // load that starts below `end` stays inside it.
  for (uint64_t c0 = beg & ~uint64_t(31); c0 < end; c0 += 512) {
    const uint64_t e0 = c0 + 16 * lane;
    uint32_t em = 0, dm = 0;
    if (e0 < end && e0 + 16 > beg) {
      const uint4 q = *reinterpret_cast<const uint4*>(g.nlab + e0);
      uint32_t in = (st.lt[e0 >> 5] >> static_cast<uint32_t>(e0 & 31)) & 0xFFFFu;
      if (beg > e0) in &= 0xFFFFu << static_cast<uint32_t>(beg - e0);
      if (end < e0 + 16) in &= (1u << static_cast<uint32_t>(end - e0)) - 1u;
#pragma unroll
      for (int j4 = 0; j4 < 4; ++j4) {
        const uint32_t four = j4 == 0 ? q.x : j4 == 1 ? q.y : j4 == 2 ? q.z : q.w;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int j = 4 * j4 + b;
          if (!((in >> j) & 1u)) continue;
          const uint32_t c = lw.code[(four >> (8 * b)) & 0xFFu];
          if (c < kHubRanks)
            ++lw.cnt[c][lane];
          else if (c == kCodeElim)
            em |= 1u << j;
          else if (c == kCodeDead)
            dm |= 1u << j;
        }
      }
    }
    const uint32_t sh = 16 * (lane & 1);
    uint32_t kem = em << sh, kill = (em | dm) << sh;
    kem |= __shfl_xor_sync(kFull, kem, 1);
    kill |= __shfl_xor_sync(kFull, kill, 1);
    if (!(lane & 1) && kill) {
      const uint64_t wi = e0 >> 5;
      if (kem) atomicAnd(st.eact + wi, ~kem);
      atomicAnd(st.lt + wi, ~kill);
    }
    elim += __popc(em);
  }
  return __reduce_add_sync(kFull, elim);
}

// One live hub segment, streamed by the whole warp.  Lane j holds word j of
// the segment's live-target bits; the warp then visits only the words with
// a bit set, kUnroll words per round, loading the CSR entry and gathering
// the neighbour word for set bits only.
template <class W, bool kFirst>
__device__ void lcc_segment(const DevGraph& g, const DevState<W>& st, const LccTables& t, LccWarp& lw, HubAcc* acc,
                            const uint4 sd, const W wv, const uint64_t beg, const uint64_t end, LccTally& tl) {
  const unsigned lane = lane_id();
  const uint32_t v = sd.x;
  const uint64_t cu = Pack<W>::cand(wv);
  const uint32_t su = Pack<W>::slot(wv);
  uint64_t ncs, need;
  role_unions_warp(t, cu, &ncs, &need);
  const uint32_t n_slots = __popcll(need);
  if (n_slots > kHubRanks) {
    if (sd.y == 0) lcc_vertex_warp(g, st, t, v, tl);
    return;
  }
  set_ranks(lw, need, n_slots);
  if (lane == 0) tl.streamed += end - beg;
  uint32_t elim = 0;
  if constexpr (kFirst) elim = lcc_segment_first(g, st, t, lw, ncs, beg, end);
  // Windows of 32 words (one per lane); a segment of a multi-segment hub is
  // one window, a single-segment hub's list may take two.
  for (uint64_t w0 = beg >> 5; !kFirst && end > beg && w0 <= (end - 1) >> 5; w0 += 32) {
    const uint64_t wi = w0 + lane;
    uint32_t word = 0;
    if (wi <= (end - 1) >> 5) {
      word = st.lt[wi];
      const uint64_t lo = wi << 5;
      if (beg > lo) word &= ~0u << static_cast<uint32_t>(beg - lo);
      if (end < lo + 32) word &= (1u << static_cast<uint32_t>(end - lo)) - 1u;
    }
    if (!st.first) tl.gathered += __popc(word);
    for (unsigned nz = __ballot_sync(kFull, word != 0); nz;) {
      uint32_t idx[kUnroll], bits[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        idx[u] = nz ? static_cast<uint32_t>(__ffs(nz) - 1) : 32u;
        nz &= nz - 1;
        bits[u] = __shfl_sync(kFull, word, idx[u] & 31);
        if (idx[u] == 32) bits[u] = 0;
      }
      W ww[kUnroll];
      if (st.first) {
        uint32_t lb[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
          lb[u] = ((bits[u] >> lane) & 1u) ? g.nlab[((w0 + idx[u]) << 5) + lane] : 0u;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
          ww[u] = ((bits[u] >> lane) & 1u) ? label_word<W>(t, lb[u]) : Pack<W>::zero();
      } else {
        uint32_t nb[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
          nb[u] = ((bits[u] >> lane) & 1u) ? g.adj[((w0 + idx[u]) << 5) + lane] : 0u;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) ww[u] = ((bits[u] >> lane) & 1u) ? st.vs[nb[u]] : Pack<W>::zero();
      }
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        const bool in = (bits[u] >> lane) & 1u;
        const uint64_t cw = Pack<W>::cand(ww[u]);
        const bool live = in && cw != 0;
        const bool poss = live && (cw & ncs) != 0;
        const unsigned em = __ballot_sync(kFull, live && !poss);
        const unsigned dm = __ballot_sync(kFull, in && cw == 0);
        if (lane == 0 && (em | dm)) {
          const uint64_t w = w0 + idx[u];
          if (em) atomicAnd(st.eact + w, ~em);
          atomicAnd(st.lt + w, ~(em | dm));
        }
        elim += __popc(em);
        if (poss) {
          const uint32_t sw = Pack<W>::slot(ww[u]);
          if (sw < 64) {
            const uint32_t r = lw.rank_of[sw];
            if (r != kNoRank) ++lw.cnt[r][lane];
          }
        }
      }
    }
  }
  // Segment totals: lane r ends with the count of rank r.
  uint32_t mine = 0;
  for (uint32_t r = 0; r < n_slots; ++r) {
    const uint32_t c = __reduce_add_sync(kFull, lw.cnt[r][lane]);
    if (lane == r) mine = c;
  }
  if (sd.z == 1) {
    if (lane < n_slots) lw.tot[lane] = mine;
    __syncwarp();
    const uint64_t tu = failing_roles_warp(t, lw, cu, su);
    if (lane == 0) {
      lcc_record(st, v, tu, elim, tl.newly_modified);
      tl.edge_elim += elim;
    }
    return;
  }
  HubAcc& a = acc[sd.w];
  if (lane < n_slots && mine) atomicAdd(&a.cnt[lane], mine);
  if (lane == 0 && elim) {
    atomicAdd(&a.elim, elim);
    tl.edge_elim += elim;
  }
  __threadfence();
  __syncwarp();
  uint32_t done = 0;
  if (lane == 0) done = atomicAdd(&a.ticket, 1u);
  done = __shfl_sync(kFull, done, 0);
  if (done + 1 == sd.z) {
    // Last segment of this hub: every other segment's adds are visible.
    __threadfence();
    if (lane < n_slots) lw.tot[lane] = atomicExch(&a.cnt[lane], 0u);
    uint32_t el = 0;
    if (lane == 0) {
      el = atomicExch(&a.elim, 0u);
      atomicExch(&a.ticket, 0u);
    }
    __syncwarp();
    const uint64_t tu = failing_roles_warp(t, lw, cu, su);
    if (lane == 0) lcc_record(st, v, tu, el, tl.newly_modified);
  }
}

// Segment i of a multi-segment hub.
template <class W, bool kFirst>
__device__ void lcc_heavy(const DevGraph& g, const DevState<W>& st, const LccTables& t, LccWarp& lw, HubAcc* acc,
                          uint64_t i, LccTally& tl) {
  const uint4 sd = g.seg[i];
  // Independent loads; the exits are warp-uniform (the hub is not scheduled
  // or has no role left).
  const uint8_t sch = st.sch[sd.x];
  const W wv = st.vs[sd.x];
  uint64_t beg, end;
  segment_range(g, sd, &beg, &end);
  if (!sch || !Pack<W>::cand(wv)) return;
  lcc_segment<W, kFirst>(g, st, t, lw, acc, sd, wv, beg, end, tl);
}

template <class W>
__device__ __forceinline__ W shfl_word(const W& w, int src) {
  if constexpr (sizeof(W) <= 4) {
    return static_cast<W>(__shfl_sync(kFull, static_cast<uint32_t>(w), src));
  } else if constexpr (sizeof(W) == 8) {
    return static_cast<W>(shfl64(static_cast<uint64_t>(w), src));
  } else {
    W r;
    r.c = shfl64(w.c, src);
    r.s = shfl64(w.s, src);
    return r;
  }
}

// 32 single-segment hubs: the lanes test them together (and fetch their
// ranges), the warp streams the live ones.
template <class W, bool kFirst>
__device__ void lcc_segments(const DevGraph& g, const DevState<W>& st, const LccTables& t, LccWarp& lw, HubAcc* acc,
                             uint64_t block, LccTally& tl) {
  const unsigned lane = lane_id();
  const uint64_t i = g.n_heavy + block * 32 + lane;
  uint4 sd = make_uint4(0, 0, 0, 0);
  W wv = Pack<W>::zero();
  uint64_t beg = 0, end = 0;
  bool live = false;
  if (i < g.n_seg) {
    sd = g.seg[i];
    const uint8_t sch = st.sch[sd.x];
    wv = st.vs[sd.x];
    beg = g.off[sd.x];  // single segment: the whole list
    end = g.off[sd.x + 1];
    live = sch && Pack<W>::cand(wv) != 0;
  }
  for (unsigned m = __ballot_sync(kFull, live); m; m &= m - 1) {
    const int j = __ffs(m) - 1;
    const uint4 s = make_uint4(__shfl_sync(kFull, sd.x, j), 0u, 1u, 0u);
    lcc_segment<W, kFirst>(g, st, t, lw, acc, s, shfl_word(wv, j), shfl64(beg, j), shfl64(end, j), tl);
  }
}

// One vertex per lane: each lane walks the live-target words of its own
// list [b, e), up to kUnroll set bits per round, counting into its own column
// of the warp's counters and clearing bits one atomic per word.  Returns
// false (and does nothing) when the warp's live lanes need more than
// kHubRanks label slots.
template <class W, bool kFirst>
__device__ bool lcc_lanes(const DevGraph& g, const DevState<W>& st, const LccTables& t, LccWarp& lw, uint32_t v,
                          W wv, uint64_t b, uint64_t e, bool live, LccTally& tl) {
  const unsigned lane = lane_id();
  const uint64_t cu = live ? Pack<W>::cand(wv) : 0;
  const uint32_t su = Pack<W>::slot(wv);
  uint64_t ncs, need;
  role_unions(t, cu, &ncs, &need);
  const uint64_t slots = warp_or64(need);
  const uint32_t n_slots = __popcll(slots);
  if (n_slots > kHubRanks) return false;
  set_ranks(lw, slots, n_slots);
  // Current word w of [b, e), masked to the list; done when w > wl.
  uint64_t w = b >> 5, wl = 0;
  bool more = live && e > b;
  if (more) wl = (e - 1) >> 5;
  auto load_word = [&](uint64_t x) {
    uint32_t word = st.lt[x];
    const uint64_t lo = x << 5;
    if (b > lo) word &= ~0u << static_cast<uint32_t>(b - lo);
    if (e < lo + 32) word &= (1u << static_cast<uint32_t>(e - lo)) - 1u;
    return word;
  };
  uint32_t clr = 0, elm = 0;  // bits of word w to clear in lt / eact
  uint32_t elim = 0, gathered = 0;
  if constexpr (kFirst) {
    // First pass after LCC0: the lane reads its list's label bytes 16 at a
    // time (one 16-byte load from the 16-aligned group holding entry x;
    // nlab is padded to whole 32-entry words) and decides every live entry
    // from its label as the word-driven loop below would.
    uint64_t x = b & ~uint64_t(15);
    while (__any_sync(kFull, more)) {
      if (!more) continue;
      const uint4 q = *reinterpret_cast<const uint4*>(g.nlab + x);
      const uint32_t sh = static_cast<uint32_t>(x & 31);
      uint32_t in = (st.lt[x >> 5] >> sh) & 0xFFFFu;
      if (b > x) in &= 0xFFFFu << static_cast<uint32_t>(b - x);
      if (e < x + 16) in &= (1u << static_cast<uint32_t>(e - x)) - 1u;
#pragma unroll
      for (int j4 = 0; j4 < 4; ++j4) {
        const uint32_t four = j4 == 0 ? q.x : j4 == 1 ? q.y : j4 == 2 ? q.z : q.w;
#pragma unroll
        for (int bb = 0; bb < 4; ++bb) {
          const int j = 4 * j4 + bb;
          if (!((in >> j) & 1u)) continue;
          const uint32_t lb = (four >> (8 * bb)) & 0xFFu;
          const uint64_t cw = t.lab_cand[lb];
          if ((cw & ncs) == 0) {
            clr |= 1u << (sh + j);
            if (cw) {
              elm |= 1u << (sh + j);
              ++elim;
            }
          } else {
            const uint32_t sw = t.lab_slot[lb];
            if (sw < 64) {
              const uint32_t r = lw.rank_of[sw];
              if (r != kNoRank) ++lw.cnt[r][lane];
            }
          }
        }
      }
      x += 16;
      if ((x & 31) == 0 || x >= e) {
        if (clr) atomicAnd(st.lt + ((x - 1) >> 5), ~clr);
        if (elm) atomicAnd(st.eact + ((x - 1) >> 5), ~elm);
        clr = elm = 0;
      }
      if (x >= e) more = false;
    }
  }
  uint32_t word = more ? load_word(w) : 0u;
  while (__any_sync(kFull, more)) {
    // Lanes whose word is used up flush it and move to the next one.
    while (more && word == 0) {
      if (clr) atomicAnd(st.lt + w, ~clr);
      if (elm) atomicAnd(st.eact + w, ~elm);
      clr = elm = 0;
      if (++w > wl) {
        more = false;
      } else {
        word = load_word(w);
      }
    }
    uint32_t bit[kUnroll], nb[kUnroll];
    bool in[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      in[u] = word != 0;
      bit[u] = in[u] ? static_cast<uint32_t>(__ffs(word) - 1) : 0u;
      word &= word - 1;
    }
    W ww[kUnroll];
    if (st.first) {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) nb[u] = in[u] ? g.nlab[(w << 5) + bit[u]] : 0u;
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) ww[u] = in[u] ? label_word<W>(t, nb[u]) : Pack<W>::zero();
    } else {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) nb[u] = in[u] ? g.adj[(w << 5) + bit[u]] : 0u;
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) ww[u] = in[u] ? st.vs[nb[u]] : Pack<W>::zero();
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      if (!in[u]) continue;
      gathered += !st.first;
      const uint64_t cw = Pack<W>::cand(ww[u]);
      const bool poss = (cw & ncs) != 0;
      if (!poss) {
        clr |= 1u << bit[u];
        if (cw) {
          elm |= 1u << bit[u];
          ++elim;
        }
      } else {
        const uint32_t sw = Pack<W>::slot(ww[u]);
        if (sw < 64) {
          const uint32_t r = lw.rank_of[sw];
          if (r != kNoRank) ++lw.cnt[r][lane];
        }
      }
    }
  }
  if (clr) atomicAnd(st.lt + w, ~clr);
  if (elm) atomicAnd(st.eact + w, ~elm);
  if (live) {
    const uint64_t tu = failing_roles(t, cu, su, slots, [&](uint32_t rank) { return lw.cnt[rank][lane]; });
    lcc_record(st, v, tu, elim, tl.newly_modified);
    tl.edge_elim += elim;
    tl.gathered += gathered;
    tl.streamed += static_cast<uint32_t>(e - b);
  }
  return true;
}

// 32 single-segment hubs, one per lane (lcc_lanes); lcc_segments when the
// batch needs more than kHubRanks slots.
template <class W, bool kFirst>
__device__ void lcc_batch_lanes(const DevGraph& g, const DevState<W>& st, const LccTables& t, LccWarp& lw,
                                HubAcc* acc, uint64_t block, LccTally& tl) {
  const uint64_t i = g.n_heavy + block * 32 + lane_id();
  uint32_t v = 0;
  W wv = Pack<W>::zero();
  uint64_t b = 0, e = 0;
  bool live = false;
  if (i < g.n_seg) {
    v = g.seg[i].x;
    const uint8_t sch = st.sch[v];
    wv = st.vs[v];
    b = g.off[v];
    e = g.off[v + 1];
    live = sch && Pack<W>::cand(wv) != 0;
  }
  if (!__ballot_sync(kFull, live)) return;
  if (!lcc_lanes<W, kFirst>(g, st, t, lw, v, wv, b, e, live, tl)) lcc_segments<W, kFirst>(g, st, t, lw, acc, block, tl);
}

// Lane's vertex of a light tile: scheduled, holding a role, not a hub.
template <class W>
struct TileLane {
  W wv;
  uint64_t b;
  uint32_t len;
  bool work;
};

template <class W>
__device__ __forceinline__ TileLane<W> tile_lane(const DevGraph& g, const DevState<W>& st, uint64_t vv) {
  TileLane<W> x{Pack<W>::zero(), 0, 0, false};
  if (vv < g.V) {
    const uint32_t v = static_cast<uint32_t>(vv);
    const uint8_t sch = st.sch[v];
    x.wv = st.vs[v];
    x.b = g.off[v];
    const uint64_t deg = g.off[v + 1] - x.b;
    if (sch && Pack<W>::cand(x.wv) && (g.n_seg == 0 || deg <= g.hub_degree)) {
      x.work = true;
      x.len = static_cast<uint32_t>(deg);
    }
  }
  return x;
}

// One tile of 32 consecutive vertices (light ones only), lane state loaded.
template <class W>
__device__ void lcc_tile(const DevGraph& g, const DevState<W>& st, const LccTables& t, LccWarp& lw, uint64_t v0,
                         const TileLane<W>& x, LccTally& tl) {
  const unsigned lane = lane_id();
  const uint32_t v = static_cast<uint32_t>(v0 + lane);
  const bool work = x.work;
  const W wv = x.wv;
  const uint64_t b = x.b;
  const uint32_t len = x.len;
  const unsigned wm = __ballot_sync(kFull, work);
  if (!wm) return;
  const uint64_t cu = work ? Pack<W>::cand(wv) : 0;
  const uint32_t su = Pack<W>::slot(wv);
  uint64_t ncs, need;
  role_unions(t, cu, &ncs, &need);
  const uint64_t slots = warp_or64(need);
  const uint32_t n_slots = __popcll(slots);
  if (n_slots > kHubRanks) {
    for (unsigned m = wm; m; m &= m - 1)
      lcc_vertex_warp(g, st, t, static_cast<uint32_t>(v0 + __ffs(m) - 1), tl);
    return;
  }
  set_ranks(lw, slots, n_slots);
  // Stream index i belongs to the lane j with excl_j <= i < excl_j + len_j,
  // at CSR entry base_j + i.  Totals stay below 2^31 (hub_degree <= 2^26).
  uint32_t incl = len;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, incl, d);
    if (lane >= static_cast<unsigned>(d)) incl += y;
  }
  const uint32_t excl = incl - len;
  const uint32_t total = __shfl_sync(kFull, incl, 31);
  const uint64_t base = b - excl;
  uint32_t elim_me = 0;
  for (uint32_t c = 0; c < total; c += 32 * kUnroll) {
    uint64_t e[kUnroll];
    uint32_t own[kUnroll];
    bool in[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const uint32_t i = c + 32 * u + lane;
      in[u] = i < total;
      uint32_t lo = 0;
#pragma unroll
      for (uint32_t step = 16; step; step >>= 1) {
        const uint32_t x = __shfl_sync(kFull, excl, lo + step);
        if (x <= i) lo += step;
      }
      own[u] = lo;
      e[u] = shfl64(base, lo) + i;
    }
    uint32_t aw[kUnroll], nb[kUnroll];
    const bool first = st.first;
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      aw[u] = in[u] ? st.lt[e[u] >> 5] : 0u;
      nb[u] = in[u] ? (first ? static_cast<uint32_t>(g.nlab[e[u]]) : g.adj[e[u]]) : 0u;
    }
    W ww[kUnroll];
    if (first) {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u)
        ww[u] = ((aw[u] >> (e[u] & 31)) & 1u) ? label_word<W>(t, nb[u]) : Pack<W>::zero();
    } else {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) ww[u] = ((aw[u] >> (e[u] & 31)) & 1u) ? st.vs[nb[u]] : Pack<W>::zero();
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const bool act = (aw[u] >> (e[u] & 31)) & 1u;
      tl.gathered += act && !first;
      const uint64_t cw = Pack<W>::cand(ww[u]);
      const uint64_t own_ncs = shfl64(ncs, own[u]);
      const bool live = cw != 0;  // entries outside lt gathered zero
      const bool poss = live && (cw & own_ncs) != 0;
      const bool el = live && !poss;
      if (el) atomicAnd(st.eact + (e[u] >> 5), ~(1u << (e[u] & 31)));
      if (act && !poss) atomicAnd(st.lt + (e[u] >> 5), ~(1u << (e[u] & 31)));
      const int64_t s0 = static_cast<int64_t>(c) + 32 * u;
      const uint32_t mine = lane_range(static_cast<int64_t>(excl) - s0, static_cast<int64_t>(excl) + len - s0);
      elim_me += __popc(__ballot_sync(kFull, el) & mine);
      const uint32_t sw = Pack<W>::slot(ww[u]);
      const uint32_t r = (poss && sw < 64) ? lw.rank_of[sw] : kNoRank;
      const uint32_t key = r != kNoRank ? (own[u] << 8 | r) : (0x10000u | lane);
      const uint32_t grp = __match_any_sync(kFull, key);
      if (r != kNoRank && lane == static_cast<unsigned>(__ffs(grp) - 1)) lw.cnt[r][own[u]] += __popc(grp);
      __syncwarp();
    }
  }
  if (work) {
    const uint64_t tu = failing_roles(t, cu, su, slots, [&](uint32_t rank) { return lw.cnt[rank][lane]; });
    lcc_record(st, v, tu, elim_me, tl.newly_modified);
    tl.edge_elim += elim_me;
  }
  if (lane == 0) tl.streamed += total;
}

// Sweep 1 in two launches with their own register budgets: kTiles false
// runs the hub segments (single- and multi-segment hubs), kTiles true the
// tiles of light vertices.
// Warp `warp` of `n_warps` takes tasks warp, warp + n_warps, ...: the
// launch's own warps for one query, or one query's share of the blocks of a
// multi-query launch.
__device__ __forceinline__ uint64_t grid_warp() {
  return (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
}
__device__ __forceinline__ uint64_t grid_warps() { return (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5; }

template <class W, bool kTiles, bool kFirst = false>
__device__ __forceinline__ void lcc_check_body(const DevGraph& g, const DevState<W>& st,
                                               const QueryTables* __restrict__ qt, HubAcc* hub_acc,
                                               StepCounters* ctr, const uint64_t warp, const uint64_t n_warps) {
  __shared__ LccTables t;
  __shared__ LccWarp s_lw[kLccWarps];
  load_lcc_tables(t, qt, qt->k, st.first != 0);
  LccWarp& lw = s_lw[threadIdx.x >> 5];
  const uint64_t heavy = g.n_heavy;
  const uint64_t batched = heavy + (static_cast<uint64_t>(g.n_seg - g.n_heavy) + 31) / 32;
  // Tile tasks cover 32 consecutive tiles: the lanes read the tiles'
  // summary flags (sweep 2 leaves most tiles with nothing scheduled) and the
  // warp checks the flagged ones.
  const uint64_t n_tiles = (static_cast<uint64_t>(g.V) + 31) / 32;
  const uint64_t n_tasks = kTiles ? (n_tiles + 31) / 32 : batched;
  LccTally tl;
  for (uint64_t task = warp; task < n_tasks; task += n_warps) {
    if (kTiles) {
      const uint64_t t0 = task * 32, ti = t0 + lane_id();
      const bool flagged = ti < n_tiles && (!st.tile_sch || st.tile_sch[ti]);
      for (unsigned m = __ballot_sync(kFull, flagged); m; m &= m - 1) {
        const uint64_t v0 = (t0 + __ffs(m) - 1) * 32;
        const TileLane<W> x = tile_lane(g, st, v0 + lane_id());
        if (__any_sync(kFull, x.work)) lcc_tile(g, st, t, lw, v0, x, tl);
      }
    } else if (task < heavy) {
      lcc_heavy<W, kFirst>(g, st, t, lw, hub_acc, task, tl);
    } else {
      lcc_batch_lanes<W, kFirst>(g, st, t, lw, hub_acc, task - heavy, tl);
    }
  }
  const uint32_t ee = __reduce_add_sync(kFull, tl.edge_elim);
  const uint32_t nm = __reduce_add_sync(kFull, tl.newly_modified);
  const uint32_t ga = __reduce_add_sync(kFull, tl.gathered);
  // Listed entries: lane-per-vertex batches count per lane, the other paths
  // on lane 0.
  const uint32_t ls = __reduce_add_sync(kFull, tl.streamed);
  if (lane_id() == 0) {
    if (ee) atomicAdd(&ctr->edge_elim, static_cast<unsigned long long>(ee));
    if (nm) atomicAdd(&ctr->modified_total, static_cast<unsigned long long>(nm));
    if (ga) atomicAdd(&ctr->gathered, static_cast<unsigned long long>(ga));
    if (ls) atomicAdd(&ctr->scanned, static_cast<unsigned long long>(ls));
  }
}

// The query's pointers, read from a device block (captured LCC loops: one
// instantiated graph serves every query that writes its block).
template <class W>
__device__ __forceinline__ DevState<W> state_at(const QueryDevPtrs* __restrict__ a) {
  return DevState<W>{static_cast<W*>(a->vs), a->eact, a->mod, a->sch, static_cast<W*>(a->unm), a->lt, a->tile_sch,
                     a->first_pass};
}

template <class W, bool kTiles>
__global__ void __launch_bounds__(kThreads, kTiles ? 4 : 5) k_lcc_check(DevGraph g, DevState<W> st,
                                                                        const QueryTables* __restrict__ qt,
                                                                        HubAcc* hub_acc, StepCounters* ctr) {
  lcc_check_body<W, kTiles>(g, st, qt, hub_acc, ctr, grid_warp(), grid_warps());
}

template <class W, bool kTiles>
__global__ void __launch_bounds__(kThreads, kTiles ? 4 : 5) k_lcc_check_at(DevGraph g,
                                                                           const QueryDevPtrs* __restrict__ a) {
  // The first pass after LCC0: k_lcc_first_at did the hubs.
  if (!kTiles && a->first_pass && g.nlab) return;
  if constexpr (kTiles) {
    // Staged in shared memory: read where used instead of held in
    // registers (no spills at 64 registers; the hub form spills less
    // without it).
    __shared__ DevState<W> s_st;
    if (threadIdx.x == 0) s_st = state_at<W>(a);
    __syncthreads();
    lcc_check_body<W, kTiles>(g, s_st, a->tables, a->hub_acc, a->ctr, grid_warp(), grid_warps());
  } else {
    lcc_check_body<W, kTiles>(g, state_at<W>(a), a->tables, a->hub_acc, a->ctr, grid_warp(), grid_warps());
  }
}

// The hub half of the first LCC pass after LCC0 (DevState::first, with
// entry labels), as a kernel of its own: the hub paths read each list's
// label bytes 16 at a time (lcc_segment_first, the first-pass block of
// lcc_lanes), and keeping that code out of k_lcc_check leaves the gathering
// passes' register allocation as it is (in one kernel it cost them spills
// and more time than the first pass saved).
template <class W>
__global__ void __launch_bounds__(kThreads, 5) k_lcc_first(DevGraph g, DevState<W> st,
                                                            const QueryTables* __restrict__ qt, HubAcc* hub_acc,
                                                            StepCounters* ctr) {
  lcc_check_body<W, false, true>(g, st, qt, hub_acc, ctr, grid_warp(), grid_warps());
}

// The same from a query's pointer block; returns at once unless the block
// marks the first pass (every later pass of a captured fixpoint).
template <class W>
__global__ void __launch_bounds__(kThreads, 5) k_lcc_first_at(DevGraph g, const QueryDevPtrs* __restrict__ a) {
  if (!a->first_pass || !g.nlab) return;
  lcc_check_body<W, false, true>(g, state_at<W>(a), a->tables, a->hub_acc, a->ctr, grid_warp(), grid_warps());
}

// ---- sweep 2 (LCC and NLCC) -------------------------------------------
//
// Applies the roles to unmatch and recomputes the schedule (lcc :107-141,
// cc :134-173): a vertex is scheduled when it was modified, or when an
// active CSR entry leads to a modified vertex.  Same task list as sweep 1:
// hub segments are scanned for such a neighbour (a hub with several
// segments gets its flag from the last one to finish); tiles do the rest.
// Scans hub segment sd for an active entry to a modified vertex; a hub
// with several segments gets its flag from the last segment to finish.
template <class W>
__device__ void apply_segment(const DevGraph& g, const DevState<W>& st, HubAcc* acc, const uint4 sd) {
  const unsigned lane = lane_id();
  const uint32_t v = sd.x, nseg = sd.z, ai = sd.w;
  uint64_t beg, end;
  segment_range(g, sd, &beg, &end);
  bool found = false;
  for (uint64_t e0 = beg; e0 < end && !found; e0 += 32) {
    const uint64_t e = e0 + lane;
    const bool hit = e < end && edge_active(st.eact, e) && st.mod[g.adj[e]];
    found = __any_sync(kFull, hit);
    // Another segment of this hub already found one.
    if (!found && nseg > 1 && ((e0 - beg) & 255) == 224)
      found = *reinterpret_cast<volatile uint32_t*>(&acc[ai].hit) != 0;
  }
  if (lane == 0) {
    if (nseg == 1) {
      st.sch[v] = found ? 1 : 0;
    } else {
      if (found) atomicOr(&acc[ai].hit, 1u);
      __threadfence();
      const uint32_t done = atomicAdd(&acc[ai].ticket2, 1u);
      if (done + 1 == nseg) {
        __threadfence();
        const uint32_t hit = atomicExch(&acc[ai].hit, 0u);
        atomicExch(&acc[ai].ticket2, 0u);
        st.sch[v] = hit ? 1 : 0;
      }
    }
  }
}

// The tiles own modified hubs (and nothing needs a scan when no vertex was
// modified); vs[v] is stable here because mod[v] == 0.
template <class W>
__device__ __forceinline__ bool apply_needs_scan(const DevState<W>& st, uint32_t v) {
  return !st.mod[v] && Pack<W>::cand(st.vs[v]) != 0;
}

template <class W>
__device__ void apply_segments(const DevGraph& g, const DevState<W>& st, HubAcc* acc, uint64_t block) {
  const unsigned lane = lane_id();
  const uint64_t i = g.n_heavy + block * 32 + lane;
  uint4 sd = make_uint4(0, 0, 0, 0);
  bool live = false;
  if (i < g.n_seg) {
    sd = g.seg[i];
    live = apply_needs_scan(st, sd.x);
  }
  for (unsigned m = __ballot_sync(kFull, live); m; m &= m - 1) {
    const int j = __ffs(m) - 1;
    const uint4 s = make_uint4(__shfl_sync(kFull, sd.x, j), __shfl_sync(kFull, sd.y, j), __shfl_sync(kFull, sd.z, j),
                               __shfl_sync(kFull, sd.w, j));
    apply_segment(g, st, acc, s);
  }
}

template <class W>
__device__ void apply_tile(const DevGraph& g, const DevState<W>& st, uint64_t tile, bool any_modified, unsigned& me,
                           unsigned& ve) {
  const unsigned lane = lane_id();
  const uint64_t v = tile + lane;
  bool scan = false;
  bool pending = false;  // holds a role after this sweep and is (or may be) scheduled
  if (v < g.V) {
    const W w = st.vs[v];
    const uint64_t c = Pack<W>::cand(w);
    if (c) {
      if (st.mod[v]) {
        uint64_t nc = c;
        const uint64_t tu = Pack<W>::cand(st.unm[v]);
        if (tu) {
          me += __popcll(tu);
          nc = c & ~tu;
          st.vs[v] = Pack<W>::make(nc, Pack<W>::slot(w));
          if (!nc) ++ve;
          st.unm[v] = Pack<W>::zero();
        }
        st.sch[v] = 1;
        pending = nc != 0;
      } else if (!any_modified) {
        st.sch[v] = 0;
      } else {
        const uint64_t b = g.off[v], e = g.off[v + 1];
        if (g.n_seg && e - b > g.hub_degree) {
          // A hub: its segments decide.
          pending = true;
        } else if (e - b <= 8) {
          // Short lists: the lane scans its own vertex.
          bool found = false;
          for (uint64_t x = b; x < e && !found; ++x)
            if (edge_active(st.eact, x) && st.mod[g.adj[x]]) found = true;
          st.sch[v] = found;
          pending = found;
        } else {
          scan = true;
        }
      }
    }
  }
  unsigned sm = __ballot_sync(kFull, scan);
  while (sm) {
    const unsigned j = __ffs(sm) - 1;
    sm &= sm - 1;
    const uint64_t u = tile + j;
    const uint64_t b = g.off[u], e = g.off[u + 1];
    bool found = false;
    for (uint64_t e0 = b; e0 < e && !found; e0 += 32) {
      const uint64_t x = e0 + lane;
      const bool hit = x < e && edge_active(st.eact, x) && st.mod[g.adj[x]];
      found = __any_sync(kFull, hit);
    }
    if (lane == j) {
      st.sch[u] = found;
      pending = found;
    }
  }
  const bool any = __any_sync(kFull, pending);
  if (lane == 0 && st.tile_sch) st.tile_sch[tile >> 5] = any ? 1 : 0;
}

template <class W>
__device__ __forceinline__ void apply_body(const DevGraph& g, const DevState<W>& st, HubAcc* hub_acc,
                                           StepCounters* ctr, const uint64_t warp, const uint64_t n_warps) {
  const bool any_modified = *reinterpret_cast<volatile unsigned long long*>(&ctr->modified_total) != 0;
  const uint64_t heavy = g.n_heavy;
  const uint64_t batched = heavy + (static_cast<uint64_t>(g.n_seg - g.n_heavy) + 31) / 32;
  const uint64_t n_tasks = batched + (static_cast<uint64_t>(g.V) + 31) / 32;
  unsigned me = 0, ve = 0;
  for (uint64_t task = warp; task < n_tasks; task += n_warps) {
    if (task < heavy) {
      const uint4 sd = g.seg[task];
      if (any_modified && apply_needs_scan(st, sd.x)) apply_segment(g, st, hub_acc, sd);
    } else if (task < batched) {
      if (any_modified) apply_segments(g, st, hub_acc, task - heavy);
    } else {
      apply_tile(g, st, (task - batched) * 32, any_modified, me, ve);
    }
  }
  me = __reduce_add_sync(kFull, me);
  ve = __reduce_add_sync(kFull, ve);
  if (lane_id() == 0) {
    if (me) atomicAdd(&ctr->match_elim, static_cast<unsigned long long>(me));
    if (ve) atomicAdd(&ctr->vertex_elim, static_cast<unsigned long long>(ve));
  }
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_apply(DevGraph g, DevState<W> st, HubAcc* hub_acc, StepCounters* ctr) {
  apply_body(g, st, hub_acc, ctr, grid_warp(), grid_warps());
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_apply_at(DevGraph g, const QueryDevPtrs* __restrict__ a) {
  apply_body(g, state_at<W>(a), a->hub_acc, a->ctr, grid_warp(), grid_warps());
}

// ---- sweep 2 on symmetric graphs: schedule by change -------------------
//
// A vertex's LCC outcome depends only on its own roles and the roles and
// slots of the neighbours behind its active entries.  An eliminated entry
// was not counted before either, so only role losses change anyone's
// inputs: the next pass needs to check exactly the vertices that lost roles
// in this step and their neighbours.  The reference reschedules every
// vertex next to a vertex modified since the last NLCC step
// (multiple_label_lcc_cpu.tpp:107-141); the vertices that this skips would
// find nothing to change, so every result row and the final state are the
// same.  On a symmetric CSR the changed vertices push the flag over their own
// lists (marking a neighbour behind an inactive entry only adds a check that
// finds nothing).

// Phase 1: apply the roles to unmatch.  mod[v] becomes "lost roles in this
// step", sch[v] keeps such vertices that still hold a role, tile_sch
// summarises sch per tile.
template <class W>
__device__ __forceinline__ void apply_changed_body(const DevGraph& g, const DevState<W>& st, StepCounters* ctr,
                                                   const uint64_t warp, const uint64_t n_warps) {
  const unsigned lane = lane_id();
  unsigned me = 0, ve = 0;
  for (uint64_t tile = warp * 32; tile < g.V; tile += n_warps * 32) {
    const uint64_t v = tile + lane;
    bool keep = false;
    if (v < g.V) {
      const W w = st.vs[v];
      const uint64_t c = Pack<W>::cand(w);
      const uint64_t tu = Pack<W>::cand(st.unm[v]);
      bool chg = false;
      if (c && tu) {
        me += __popcll(tu);
        const uint64_t nc = c & ~tu;
        st.vs[v] = Pack<W>::make(nc, Pack<W>::slot(w));
        if (!nc) ++ve;
        chg = true;
        keep = nc != 0;
      }
      if (tu) st.unm[v] = Pack<W>::zero();
      st.mod[v] = chg ? 1 : 0;
      st.sch[v] = keep ? 1 : 0;
    }
    const bool any = __any_sync(kFull, keep);
    if (lane == 0 && st.tile_sch) st.tile_sch[tile >> 5] = any ? 1 : 0;
  }
  me = __reduce_add_sync(kFull, me);
  ve = __reduce_add_sync(kFull, ve);
  if (lane == 0) {
    if (me) atomicAdd(&ctr->match_elim, static_cast<unsigned long long>(me));
    if (ve) atomicAdd(&ctr->vertex_elim, static_cast<unsigned long long>(ve));
  }
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_apply_changed(DevGraph g, DevState<W> st, StepCounters* ctr) {
  apply_changed_body(g, st, ctr, grid_warp(), grid_warps());
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_apply_changed_at(DevGraph g, const QueryDevPtrs* __restrict__ a) {
  apply_changed_body(g, state_at<W>(a), a->ctr, grid_warp(), grid_warps());
}

// Marks every entry target of [b, e) as scheduled (one warp).
template <class W>
__device__ __forceinline__ void push_range(const DevGraph& g, const DevState<W>& st, uint64_t b, uint64_t e) {
  for (uint64_t x = b + lane_id(); x < e; x += 32) {
    const uint32_t w = g.adj[x];
    st.sch[w] = 1;
    if (st.tile_sch) st.tile_sch[w >> 5] = 1;
  }
}

// Phase 2: the vertices that lost roles mark their neighbours, with the
// task layout of sweep 1 (hub segments, batches of 32 single-segment hubs,
// tiles of 32 light vertices).
template <class W>
__device__ __forceinline__ void push_changed_body(const DevGraph& g, const DevState<W>& st, const uint64_t warp,
                                                  const uint64_t n_warps) {
  const unsigned lane = lane_id();
  const uint64_t heavy = g.n_heavy;
  const uint64_t batched = heavy + (static_cast<uint64_t>(g.n_seg - g.n_heavy) + 31) / 32;
  const uint64_t n_tasks = batched + (static_cast<uint64_t>(g.V) + 31) / 32;
  for (uint64_t task = warp; task < n_tasks; task += n_warps) {
    if (task < heavy) {
      const uint4 sd = g.seg[task];
      if (!st.mod[sd.x]) continue;
      uint64_t b, e;
      segment_range(g, sd, &b, &e);
      push_range(g, st, b, e);
      continue;
    }
    uint32_t v = 0;
    bool chg = false;
    if (task < batched) {
      const uint64_t i = g.n_heavy + (task - heavy) * 32 + lane;
      if (i < g.n_seg) {
        v = g.seg[i].x;
        chg = st.mod[v] != 0;
      }
    } else {
      const uint64_t vv = (task - batched) * 32 + lane;
      if (vv < g.V) {
        v = static_cast<uint32_t>(vv);
        chg = st.mod[v] && (g.n_seg == 0 || g.off[v + 1] - g.off[v] <= g.hub_degree);
      }
    }
    for (unsigned m = __ballot_sync(kFull, chg); m; m &= m - 1) {
      const uint32_t u = __shfl_sync(kFull, v, __ffs(m) - 1);
      push_range(g, st, g.off[u], g.off[u + 1]);
    }
  }
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_push_changed(DevGraph g, DevState<W> st) {
  push_changed_body(g, st, grid_warp(), grid_warps());
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_push_changed_at(DevGraph g, const QueryDevPtrs* __restrict__ a) {
  push_changed_body(g, state_at<W>(a), grid_warp(), grid_warps());
}

// ---- many queries in one launch (batched LCC fixpoints) -----------------
//
// A launch of nq x bpq blocks over the queries listed in active[0, nq): block
// b works for query active[b % nq] as its virtual block b / nq of bpq, and
// runs the same sweep body over that query's state and task list.  Blocks of
// different queries with the same virtual index take the same tasks (the same
// CSR ranges) at about the same time, so an adjacency range brought from HBM
// for one query is served from L2 for the others; each query's counters,
// hub accumulators and flags are its own, so its rows are those of its own
// passes.
struct MultiSlot {
  uint32_t q;
  uint64_t warp, n_warps;
};
__device__ __forceinline__ MultiSlot multi_slot(uint32_t nq) {
  MultiSlot m;
  const uint32_t bpq = gridDim.x / nq;
  m.q = blockIdx.x % nq;
  m.warp = (static_cast<uint64_t>(blockIdx.x / nq) * blockDim.x + threadIdx.x) >> 5;
  m.n_warps = (static_cast<uint64_t>(bpq) * blockDim.x) >> 5;
  return m;
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_lcc0_multi(DevGraph g, const QueryDevPtrs* __restrict__ qs,
                                                         const uint32_t* __restrict__ active, uint32_t nq) {
  const MultiSlot m = multi_slot(nq);
  const QueryDevPtrs* a = qs + active[m.q];
  const DevState<W> st = state_at<W>(a);
  __shared__ uint64_t slot_roles[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) slot_roles[i] = a->tables->slot_roles[i];
  __syncthreads();
  unsigned long long me = 0, ve = 0;
  const uint64_t stride = m.n_warps * 32;
  for (uint64_t v = m.warp * 32 + lane_id(); v < g.V; v += stride) {
    W w = st.vs[v];
    uint64_t c = Pack<W>::cand(w);
    if (!c) continue;
    uint32_t sl = Pack<W>::slot(w);
    uint64_t nc = c & slot_roles[sl];
    if (nc != c) {
      me += __popcll(c ^ nc);
      st.vs[v] = Pack<W>::make(nc, sl);
      if (!nc) ++ve;
    }
  }
  me = __reduce_add_sync(kFull, static_cast<unsigned>(me));
  ve = __reduce_add_sync(kFull, static_cast<unsigned>(ve));
  if (lane_id() == 0) {
    if (me) atomicAdd(&a->ctr->match_elim, me);
    if (ve) atomicAdd(&a->ctr->vertex_elim, ve);
  }
}

template <class W, bool kTiles>
__global__ void __launch_bounds__(kThreads, kTiles ? 4 : 5) k_lcc_check_multi(DevGraph g,
                                                                              const QueryDevPtrs* __restrict__ qs,
                                                                              const uint32_t* __restrict__ active,
                                                                              uint32_t nq) {
  const MultiSlot m = multi_slot(nq);
  const QueryDevPtrs* a = qs + active[m.q];
  // This query's first pass after LCC0: k_lcc_first_multi did its hubs.
  if (!kTiles && a->first_pass && g.nlab) return;
  if constexpr (kTiles) {
    __shared__ DevState<W> s_st;
    if (threadIdx.x == 0) s_st = state_at<W>(a);
    __syncthreads();
    lcc_check_body<W, kTiles>(g, s_st, a->tables, a->hub_acc, a->ctr, m.warp, m.n_warps);
  } else {
    lcc_check_body<W, kTiles>(g, state_at<W>(a), a->tables, a->hub_acc, a->ctr, m.warp, m.n_warps);
  }
}

// k_lcc_first over the queries of a multi-query launch that are at their
// first pass after LCC0 (the others' blocks return at once).
template <class W>
__global__ void __launch_bounds__(kThreads, 5) k_lcc_first_multi(DevGraph g, const QueryDevPtrs* __restrict__ qs,
                                                                  const uint32_t* __restrict__ active, uint32_t nq) {
  const MultiSlot m = multi_slot(nq);
  const QueryDevPtrs* a = qs + active[m.q];
  if (!a->first_pass || !g.nlab) return;
  lcc_check_body<W, false, true>(g, state_at<W>(a), a->tables, a->hub_acc, a->ctr, m.warp, m.n_warps);
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_apply_multi(DevGraph g, const QueryDevPtrs* __restrict__ qs,
                                                          const uint32_t* __restrict__ active, uint32_t nq) {
  const MultiSlot m = multi_slot(nq);
  const QueryDevPtrs* a = qs + active[m.q];
  apply_body(g, state_at<W>(a), a->hub_acc, a->ctr, m.warp, m.n_warps);
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_apply_changed_multi(DevGraph g, const QueryDevPtrs* __restrict__ qs,
                                                                  const uint32_t* __restrict__ active, uint32_t nq) {
  const MultiSlot m = multi_slot(nq);
  const QueryDevPtrs* a = qs + active[m.q];
  apply_changed_body(g, state_at<W>(a), a->ctr, m.warp, m.n_warps);
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_push_changed_multi(DevGraph g, const QueryDevPtrs* __restrict__ qs,
                                                                 const uint32_t* __restrict__ active, uint32_t nq) {
  const MultiSlot m = multi_slot(nq);
  push_changed_body(g, state_at<W>(qs + active[m.q]), m.warp, m.n_warps);
}

// Per active query: clear the per-step counter words (clear != 0), or copy
// its counters to out[i] (clear == 0).
__global__ void k_counters_multi(const QueryDevPtrs* __restrict__ qs, const uint32_t* __restrict__ active,
                                 uint32_t nq, StepCounters* out, int clear) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nq * 16u; i += gridDim.x * blockDim.x) {
    const uint32_t q = i / 16, w = i % 16;
    unsigned long long* words = reinterpret_cast<unsigned long long*>(qs[active[q]].ctr);
    if (clear) {
      if (w < static_cast<uint32_t>(kStepCounterWords)) words[w] = 0;
    } else {
      reinterpret_cast<unsigned long long*>(out + q)[w] = words[w];
    }
  }
}

// ---- worklist compaction ----------------------------------------------
constexpr int kTileV = 4096;  // vertices per compaction block (256 threads x 16)

template <class W>
__device__ __forceinline__ bool in_worklist(const DevGraph& g, const DevState<W>& st, uint64_t v, uint64_t mask) {
  return v < g.V && (Pack<W>::cand(st.vs[v]) & mask) != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Before the first pass of a captured fixpoint loop.
__global__ void k_lcc_loop_head(LccLoopCtl* ctl) {
  if (threadIdx.x != 0) return;
  ctl->passes = 0;
  ctl->error = 0;
  ctl->start_ns = global_ns();
}

// After every pass: row `passes` gets the pass's counters; the loop goes on
// while the pass eliminated a vertex, edge or role (the reference's
// AlgoResults::isEmpty is false), no device error was raised and fewer than
// max_passes passes ran.  The step counters start the next pass at zero.
// rows holds kLccLoopMaxPasses rows and max_passes <= kLccLoopMaxPasses, so
// the row index stays in bounds.
__global__ void k_lcc_loop_tail(QueryDevPtrs* __restrict__ a, LccLoopCtl* ctl, LccPassRow* rows,
                                cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0) return;
  StepCounters* ctr = a->ctr;
  a->first_pass = 0;  // later passes gather neighbour words
  const uint32_t i = ctl->passes;
  const uint32_t cap = min(ctl->max_passes, kLccLoopMaxPasses);
  LccPassRow r;
  r.vertex_elim = ctr->vertex_elim;
  r.edge_elim = ctr->edge_elim;
  r.match_elim = ctr->match_elim;
  r.scanned = ctr->scanned;
  r.gathered = ctr->gathered;
  r.end_ns = global_ns();
  bool more = false;
  if (i < cap) {
    rows[i] = r;
    ctl->passes = i + 1;
    more = (r.vertex_elim | r.edge_elim | r.match_elim) != 0 && i + 1 < cap;
  }
  if (ctr->error) {
    ctl->error = ctr->error;
    more = false;
  }
  unsigned long long* words = reinterpret_cast<unsigned long long*>(ctr);
  for (int w = 0; w < kStepCounterWords; ++w) words[w] = 0;
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

template <class W>
__global__ void __launch_bounds__(256) k_wl_count(DevGraph g, DevState<W> st, uint64_t mask, uint32_t* block_counts) {
  __shared__ uint32_t s_cnt[8];
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTileV;
  uint32_t c = 0;
  for (int i = 0; i < kTileV / 256; ++i) c += in_worklist(g, st, base + i * 256 + threadIdx.x, mask);
  c = __reduce_add_sync(kFull, c);
  if (lane_id() == 0) s_cnt[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int i = 0; i < 8; ++i) t += s_cnt[i];
    block_counts[blockIdx.x] = t;
  }
}

// Exclusive scan of block counts in one block; writes the total to *count.
__global__ void __launch_bounds__(1024) k_wl_scan(uint32_t* block_counts, uint32_t n, uint32_t* count) {
  __shared__ uint32_t s_warp[32];
  const uint32_t per = (n + 1023) / 1024;
  const uint32_t b = threadIdx.x * per;
  uint32_t local = 0;
  for (uint32_t i = 0; i < per; ++i)
    if (b + i < n) local += block_counts[b + i];
  // block-wide exclusive scan of `local`
  uint32_t x = local;
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = s_warp[lane];
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, w, o);
      if (lane >= o) w += y;
    }
    s_warp[lane] = w;
  }
  __syncthreads();
  uint32_t excl = x - local + (wid ? s_warp[wid - 1] : 0);
  for (uint32_t i = 0; i < per; ++i)
    if (b + i < n) {
      uint32_t c = block_counts[b + i];
      block_counts[b + i] = excl;
      excl += c;
    }
  if (threadIdx.x == 1023) *count = excl;
}

template <class W>
__global__ void __launch_bounds__(256) k_wl_write(DevGraph g, DevState<W> st, uint64_t mask,
                                                  const uint32_t* __restrict__ block_offsets, uint32_t* wl,
                                                  uint32_t* wl_index) {
  __shared__ uint32_t s_warp[8];
  __shared__ uint32_t s_base;
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTileV;
  if (threadIdx.x == 0) s_base = block_offsets[blockIdx.x];
  __syncthreads();
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  // Rounds of 256 vertices; order is round-major, then warp, then lane,
  // which is ascending vertex order when each round covers 256 consecutive ids.
  for (int i = 0; i < kTileV / 256; ++i) {
    const uint64_t v = base + i * 256 + threadIdx.x;
    const bool f = in_worklist(g, st, v, mask);
    const unsigned m = __ballot_sync(kFull, f);
    if (lane == 0) s_warp[wid] = __popc(m);
    __syncthreads();
    uint32_t before = 0;
    for (unsigned w = 0; w < wid; ++w) before += s_warp[w];
    if (f) {
      const uint32_t pos = s_base + before + __popc(m & ((1u << lane) - 1));
      wl[pos] = static_cast<uint32_t>(v);
      wl_index[v] = pos;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t t = 0;
      for (int w = 0; w < 8; ++w) t += s_warp[w];
      s_base += t;
    }
    __syncthreads();
  }
}

// ---- first-hop slices of heavy walker items ---------------------------------
//
// An exact walk program's item (worklist position pos, program r) whose
// source has more than t CSR entries also runs as ceil(deg / t) slices of
// its first hop, {pos * R + r, lo, min(lo + t, deg), 0}, listed in (pos, r,
// lo) order: per-tile counts, one scan, then each tile writes its slices.
__device__ __forceinline__ uint64_t slices_of(const DevGraph& g, const uint32_t* __restrict__ wl, uint32_t n_wl,
                                              uint64_t pos, uint32_t R, uint32_t t) {
  if (pos >= n_wl) return 0;
  const uint32_t v = wl[pos];
  const uint64_t deg = g.off[v + 1] - g.off[v];
  return deg > t ? static_cast<uint64_t>(R) * ((deg + t - 1) / t) : 0;
}

__global__ void __launch_bounds__(256) k_slice_count(DevGraph g, const uint32_t* __restrict__ wl, uint32_t n_wl,
                                                     uint32_t R, uint32_t t, unsigned long long* tile_counts) {
  __shared__ unsigned long long s_cnt[8];
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTileV;
  unsigned long long c = 0;
  for (int i = 0; i < kTileV / 256; ++i) c += slices_of(g, wl, n_wl, base + i * 256 + threadIdx.x, R, t);
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
  if (lane_id() == 0) s_cnt[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long x = 0;
    for (int i = 0; i < 8; ++i) x += s_cnt[i];
    tile_counts[blockIdx.x] = x;
  }
}

// Exclusive scan of the n tile counts in one block (in place); *total gets
// the sum.
__global__ void __launch_bounds__(1024) k_slice_scan(unsigned long long* counts, uint32_t n,
                                                     unsigned long long* total) {
  __shared__ unsigned long long s_warp[32];
  const uint32_t per = (n + 1023) / 1024;
  const uint32_t b = threadIdx.x * per;
  unsigned long long local = 0;
  for (uint32_t i = 0; i < per; ++i)
    if (b + i < n) local += counts[b + i];
  unsigned long long x = local;
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(kFull, x, o);
    if (lane >= static_cast<unsigned>(o)) x += y;
  }
  if (lane == 31) s_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned long long w = s_warp[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(kFull, w, o);
      if (lane >= static_cast<unsigned>(o)) w += y;
    }
    s_warp[lane] = w;
  }
  __syncthreads();
  unsigned long long excl = x - local + (wid ? s_warp[wid - 1] : 0);
  for (uint32_t i = 0; i < per; ++i)
    if (b + i < n) {
      const unsigned long long c = counts[b + i];
      counts[b + i] = excl;
      excl += c;
    }
  if (threadIdx.x == 1023) *total = excl;
}

__global__ void __launch_bounds__(256) k_slice_write(DevGraph g, const uint32_t* __restrict__ wl, uint32_t n_wl,
                                                     uint32_t R, uint32_t t,
                                                     const unsigned long long* __restrict__ tile_offsets,
                                                     uint4* __restrict__ slices) {
  __shared__ unsigned long long s_warp[8];
  __shared__ unsigned long long s_base;
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTileV;
  if (threadIdx.x == 0) s_base = tile_offsets[blockIdx.x];
  __syncthreads();
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  for (int i = 0; i < kTileV / 256; ++i) {
    const uint64_t pos = base + i * 256 + threadIdx.x;
    const unsigned long long c = slices_of(g, wl, n_wl, pos, R, t);
    unsigned long long x = c;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(kFull, x, o);
      if (lane >= static_cast<unsigned>(o)) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    unsigned long long before = 0;
    for (unsigned w = 0; w < wid; ++w) before += s_warp[w];
    if (c) {
      const uint32_t v = wl[pos];
      const uint64_t deg = g.off[v + 1] - g.off[v];
      const uint64_t per_prog = (deg + t - 1) / t;
      uint64_t out = s_base + before + x - c;
      for (uint32_t r = 0; r < R; ++r)
        for (uint64_t k = 0; k < per_prog; ++k, ++out) {
          const uint64_t lo = k * t, hi = lo + t < deg ? lo + t : deg;
          slices[out] = make_uint4(static_cast<uint32_t>(pos * R + r), static_cast<uint32_t>(lo),
                                   static_cast<uint32_t>(hi), 0u);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long tot = 0;
      for (int w = 0; w < 8; ++w) tot += s_warp[w];
      s_base += tot;
    }
    __syncthreads();
  }
}

// ---- ENUMERATION items --------------------------------------------------------
//
// Source i of the worklist with more than t first-hop entries (heavy) takes
// items {i, lo, hi, 0} over runs of its list; with the second-hop split on
// (s2 > 0) and more than s2 entries, a first-hop position whose vertex has
// more than 2 * s2 entries ends the run before it and takes ceil(d1 / s2)
// items {i, pos, pos + 1, k + 1} of its own, and the runs between such
// positions are cut every t entries.  Heavy items come first, in worklist
// and list order; then one item {i, 0, 2^32 - 1, 0} per light source.  A
// warp per source: lane j tests position base + j, hubs are taken in order
// from the ballot.

struct EnumItemRule {
  uint32_t t, s2;  // run length, second-hop slice length (0: off)
};

__device__ __forceinline__ uint64_t ceil_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

// Count (out == nullptr) or write the heavy items of source i (degree deg,
// list at off[v]); returns the count.  Warp-uniform arguments.
__device__ uint64_t enum_heavy_items(const DevGraph& g, uint32_t i, uint32_t v, uint64_t deg, EnumItemRule r,
                                     uint4* out) {
  const unsigned lane = lane_id();
  if (r.s2 == 0 || deg <= r.s2) {
    const uint64_t n = ceil_div(deg, r.t);
    if (out)
      for (uint64_t k = lane; k < n; k += 32) {
        const uint64_t lo = k * r.t, hi = lo + r.t < deg ? lo + r.t : deg;
        out[k] = make_uint4(i, static_cast<uint32_t>(lo), static_cast<uint32_t>(hi), 0u);
      }
    return n;
  }
  const uint64_t base = g.off[v];
  uint64_t n = 0, a = 0;  // items so far, start of the current run
  auto runs = [&](uint64_t b) {  // runs of [a, b)
    if (b <= a) return;
    const uint64_t m = ceil_div(b - a, r.t);
    if (out)
      for (uint64_t k = lane; k < m; k += 32) {
        const uint64_t lo = a + k * r.t, hi = lo + r.t < b ? lo + r.t : b;
        out[n + k] = make_uint4(i, static_cast<uint32_t>(lo), static_cast<uint32_t>(hi), 0u);
      }
    n += m;
  };
  for (uint64_t p0 = 0; p0 < deg; p0 += 32) {
    const uint64_t pos = p0 + lane;
    uint64_t d1 = 0;
    if (pos < deg) {
      const uint32_t w = g.adj[base + pos];
      d1 = g.off[w + 1] - g.off[w];
    }
    const bool hub = pos < deg && d1 > 2ull * r.s2;
    for (unsigned hm = __ballot_sync(kFull, hub); hm; hm &= hm - 1) {
      const unsigned j = __ffs(hm) - 1;
      const uint64_t hp = p0 + j;
      const uint64_t hd = shfl64(d1, j);
      runs(hp);
      const uint64_t m = ceil_div(hd, r.s2);
      if (out)
        for (uint64_t k = lane; k < m; k += 32)
          out[n + k] = make_uint4(i, static_cast<uint32_t>(hp), static_cast<uint32_t>(hp + 1),
                                  static_cast<uint32_t>(k + 1));
      n += m;
      a = hp + 1;
    }
  }
  runs(deg);
  return n;
}

// Per source: heavy item count and light flag.
__global__ void __launch_bounds__(256) k_enum_item_count(DevGraph g, const uint32_t* __restrict__ wl, uint32_t n_wl,
                                                         EnumItemRule r, uint32_t* __restrict__ heavy,
                                                         uint32_t* __restrict__ light, uint32_t* overflow) {
  const uint64_t n_warps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t i = grid_warp(); i < n_wl; i += n_warps) {
    const uint32_t v = wl[i];
    const uint64_t deg = g.off[v + 1] - g.off[v];
    uint64_t h = 0;
    if (deg > r.t) h = enum_heavy_items(g, static_cast<uint32_t>(i), v, deg, r, nullptr);
    if (lane_id() == 0) {
      if (h > 0xFFFFFFFFull) atomicOr(overflow, 1u);
      heavy[i] = static_cast<uint32_t>(h);
      light[i] = deg > r.t ? 0u : 1u;
    }
  }
}

// Exclusive scan of a u32 array in tiles of 4096: per element its offset
// within the tile, per tile its sum (scanned afterwards by k_slice_scan).
__global__ void __launch_bounds__(256) k_scan_tiles(const uint32_t* __restrict__ in, uint32_t n,
                                                    unsigned long long* __restrict__ local,
                                                    unsigned long long* __restrict__ tile_sums) {
  __shared__ unsigned long long s_warp[8];
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTileV + threadIdx.x * 16ull;
  unsigned long long mine = 0;
  uint32_t v[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    v[k] = base + k < n ? in[base + k] : 0u;
    mine += v[k];
  }
  unsigned long long x = mine;
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(kFull, x, o);
    if (lane >= static_cast<unsigned>(o)) x += y;
  }
  if (lane == 31) s_warp[wid] = x;
  __syncthreads();
  unsigned long long before = 0;
  for (unsigned w = 0; w < wid; ++w) before += s_warp[w];
  unsigned long long run = before + x - mine;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    if (base + k < n) local[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 255) tile_sums[blockIdx.x] = before + x;
}

__global__ void __launch_bounds__(256) k_enum_item_write(DevGraph g, const uint32_t* __restrict__ wl, uint32_t n_wl,
                                                         EnumItemRule r, const uint32_t* __restrict__ light,
                                                         const unsigned long long* __restrict__ heavy_local,
                                                         const unsigned long long* __restrict__ heavy_tiles,
                                                         const unsigned long long* __restrict__ light_local,
                                                         const unsigned long long* __restrict__ light_tiles,
                                                         const unsigned long long* __restrict__ heavy_total,
                                                         uint4* __restrict__ items) {
  const uint64_t n_warps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t i = grid_warp(); i < n_wl; i += n_warps) {
    const uint32_t v = wl[i];
    const uint64_t deg = g.off[v + 1] - g.off[v];
    if (light[i]) {
      if (lane_id() == 0)
        items[*heavy_total + light_tiles[i / kTileV] + light_local[i]] =
            make_uint4(static_cast<uint32_t>(i), 0u, 0xFFFFFFFFu, 0u);
    } else {
      enum_heavy_items(g, static_cast<uint32_t>(i), v, deg, r, items + heavy_tiles[i / kTileV] + heavy_local[i]);
    }
  }
}

// ---- export ---------------------------------------------------------------
template <class W>
__global__ void __launch_bounds__(kThreads) k_export(DevGraph g, DevState<W> st, uint64_t* cand, uint8_t* vact,
                                                     uint8_t* eact_bytes) {
  const uint64_t tid = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t v = tid; v < g.V; v += stride) {
    uint64_t c = Pack<W>::cand(st.vs[v]);
    if (cand) cand[v] = c;
    if (vact) vact[v] = c != 0;
  }
  if (eact_bytes)
    for (uint64_t e = tid; e < g.E; e += stride) eact_bytes[e] = edge_active(st.eact, e);
}

// ---- graph statistics of the dynamic constraint order ---------------------
// GraphStatCpu::compute (src/patternmatching/algorithms/graph_stat_cpu.tpp:
// 42-80) over the active graph: active vertices per (partition block, label
// slot), active CSR entries between active vertices per (slot, slot), and
// the at-least counts of the reference's per-thread accumulation, which is
// never cleared between the vertices of one thread's block: a label-a vertex
// counts towards (a, b, i) when the running number of label-b neighbours of
// the block's active vertices up to and including it has reached i.  That
// running number only grows, so once it reaches the largest i any label
// needs (at most 63) every later vertex of the block counts fully: one warp
// per (block, b) scans from the block's start to that point and the rest of
// the block is added from the per-block vertex counts.

__device__ __forceinline__ uint32_t stat_block_of(uint64_t v, uint64_t q, uint64_t r) {
  const uint64_t big = r * (q + 1);
  return static_cast<uint32_t>(v < big ? v / (q + 1) : r + (v - big) / q);
}

template <class W>
__global__ void __launch_bounds__(kThreads) k_stat_counts(DevGraph g, const W* __restrict__ vs,
                                                           const uint32_t* __restrict__ eact, GraphStatDev p) {
  extern __shared__ uint32_t hist[];  // [S * S] entries between slots
  const uint32_t S = p.slots;
  for (uint32_t i = threadIdx.x; i < S * S; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  const uint32_t lane = lane_id();
  const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t tile = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; tile * 32 < g.V;
       tile += nwarps) {
    const uint64_t v = tile * 32 + lane;
    uint32_t a = 0;
    bool act = false;
    if (v < g.V) {
      const W w = vs[v];
      act = Pack<W>::cand(w) != 0;
      a = Pack<W>::slot(w);
    }
    if (act && a >= S) {
      atomicOr(p.bad, 1ull);
      act = false;
    }
    const unsigned am = __ballot_sync(kFull, act);
    if (act) {
      const uint32_t key = stat_block_of(v, p.q, p.r) * S + a;
      const unsigned peers = __match_any_sync(am, key);
      if (lane == static_cast<uint32_t>(__ffs(peers) - 1))
        atomicAdd(p.vseg + key, static_cast<unsigned long long>(__popc(peers)));
    }
    for (unsigned todo = am; todo; todo &= todo - 1) {
      const int src = __ffs(todo) - 1;
      const uint64_t u = tile * 32 + src;
      const uint32_t au = __shfl_sync(kFull, a, src);
      const uint64_t hi = g.off[u + 1];
      for (uint64_t e = g.off[u] + lane; e < hi; e += 32) {
        if (!edge_active(eact, e)) continue;
        const W ww = vs[g.adj[e]];
        if (Pack<W>::cand(ww) == 0) continue;
        const uint32_t b = Pack<W>::slot(ww);
        if (b >= S) {
          atomicOr(p.bad, 1ull);
          continue;
        }
        atomicAdd(&hist[au * S + b], 1u);
      }
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < S * S; i += blockDim.x)
    if (hist[i]) atomicAdd(p.edges + i, static_cast<unsigned long long>(hist[i]));
}

// One warp per (partition block t, neighbour slot b), b == S standing for
// "any label" (the accumulation holds anything); needs k_stat_counts first.
template <class W>
__global__ void __launch_bounds__(kThreads) k_stat_accum(DevGraph g, const W* __restrict__ vs,
                                                          const uint32_t* __restrict__ eact, GraphStatDev p) {
  __shared__ uint32_t scanned_all[kWarpsPerBlock][64];
  const uint32_t S = p.slots, S1 = S + 1;
  const uint32_t lane = lane_id(), wib = threadIdx.x >> 5;
  const uint64_t warp = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (warp >= static_cast<uint64_t>(p.blocks) * S1) return;
  const uint32_t t = static_cast<uint32_t>(warp / S1), b = static_cast<uint32_t>(warp % S1);
  const uint32_t thr = p.thr[b];
  if (thr == 0) return;
  uint32_t* scanned = scanned_all[wib];
  for (uint32_t a = lane; a < 64; a += 32) scanned[a] = 0;
  __syncwarp();
  const uint64_t begin = t * p.q + (t < p.r ? t : p.r), end = begin + p.q + (t < p.r ? 1 : 0);
  uint64_t run = 0, pos = begin;
  while (pos < end && run < thr) {
    const uint64_t v = pos + lane;
    uint32_t c = 0, a = S;
    if (v < end) {
      const W w = vs[v];
      if (Pack<W>::cand(w) != 0 && Pack<W>::slot(w) < S) {
        a = Pack<W>::slot(w);
        const uint64_t hi = g.off[v + 1];
        for (uint64_t e = g.off[v]; e < hi; ++e) {
          if (!edge_active(eact, e)) continue;
          const W ww = vs[g.adj[e]];
          if (Pack<W>::cand(ww) == 0) continue;
          if (b == S || Pack<W>::slot(ww) == b) ++c;
        }
      }
    }
    uint32_t incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t n = __shfl_up_sync(kFull, incl, d);
      if (lane >= static_cast<uint32_t>(d)) incl += n;
    }
    if (a < S) {
      const uint32_t most = p.max[a * S1 + b];
      const uint64_t upto = run + incl < most ? run + incl : most;
      for (uint32_t i = 1; i <= upto; ++i) atomicAdd(p.at_least + (static_cast<uint64_t>(a) * S1 + b) * 64 + i, 1ull);
      atomicAdd(&scanned[a], 1u);
    }
    run += __shfl_sync(kFull, incl, 31);
    pos += 32;
  }
  __syncwarp();
  if (pos >= end) return;
  // Every active vertex after `pos` in the block sees a running count of at
  // least thr >= every maximum of this column.
  for (uint32_t a = lane; a < S; a += 32) {
    const uint32_t most = p.max[a * S1 + b];
    if (!most) continue;
    const unsigned long long rest = p.vseg[static_cast<uint64_t>(t) * S + a] - scanned[a];
    if (!rest) continue;
    for (uint32_t i = 1; i <= most; ++i) atomicAdd(p.at_least + (static_cast<uint64_t>(a) * S1 + b) * 64 + i, rest);
  }
}

template <class W>
DevState<W> state_of(const QueryDevPtrs& q) {
  return DevState<W>{static_cast<W*>(q.vs), q.eact, q.mod, q.sch, static_cast<W*>(q.unm), q.lt, q.tile_sch,
                     q.first_pass};
}

#define PM_DISPATCH_WORD(kind, ...)            \
  note_launch();                               \
  switch (kind) {                              \
    case kWord16: {                            \
      using W = uint16_t;                      \
      __VA_ARGS__;                             \
    } break;                                   \
    case kWord32: {                            \
      using W = uint32_t;                      \
      __VA_ARGS__;                             \
    } break;                                   \
    case kWord64: {                            \
      using W = uint64_t;                      \
      __VA_ARGS__;                             \
    } break;                                   \
    default: {                                 \
      using W = Wide;                          \
      __VA_ARGS__;                             \
    } break;                                   \
  }

}  // namespace

thread_local uint64_t t_launches = 0;
void note_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  ++t_launches;
}
void note_launches(int64_t n) { g_launches.fetch_add(static_cast<uint64_t>(n), std::memory_order_relaxed); }
uint64_t thread_launch_count() { return t_launches; }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

int device_sm_count() {
  int n = g_sm_count.load(std::memory_order_relaxed);
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    g_sm_count.store(n, std::memory_order_relaxed);
  }
  return n;
}

void launch_init_state(const DevGraph& g, const QueryDevPtrs& q, const uint8_t* d2s, uint64_t full, cudaStream_t s) {
  const int grid = device_sm_count() * 8;
  PM_DISPATCH_WORD(q.word_kind, k_init_state<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), d2s, full));
}

void launch_check_symmetric(const DevGraph& g, unsigned long long* res, cudaStream_t s) {
  note_launch();
  k_check_symmetric<<<device_sm_count() * 8, kThreads, 0, s>>>(g, res);
}

void launch_build_entry_labels(const DevGraph& g, uint8_t* nlab, cudaStream_t s) {
  note_launch();
  k_build_entry_labels<<<device_sm_count() * 8, kThreads, 0, s>>>(g, nlab);
}

void launch_lcc0(const DevGraph& g, const QueryDevPtrs& q, cudaStream_t s) {
  const int grid = device_sm_count() * 8;
  PM_DISPATCH_WORD(q.word_kind, k_lcc0<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), q.tables, q.ctr));
}

// Blocks for n_tasks one-warp tasks: at most `per_sm` resident blocks per SM.
// Sweep tasks: segments of multi-segment hubs, blocks of 32 single-segment
// hubs, tiles of 32 vertices.
inline uint64_t sweep_tasks(const DevGraph& g) {
  return g.n_heavy + (static_cast<uint64_t>(g.n_seg - g.n_heavy) + 31) / 32 + (static_cast<uint64_t>(g.V) + 31) / 32;
}

inline int grid_for_tasks(uint64_t n_tasks, int per_sm) {
  uint64_t blocks = (n_tasks + kWarpsPerBlock - 1) / kWarpsPerBlock;
  const uint64_t cap = static_cast<uint64_t>(device_sm_count()) * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return static_cast<int>(blocks);
}

void launch_lcc_check(const DevGraph& g, const QueryDevPtrs& q, cudaStream_t s) {
  const uint64_t hub_tasks = g.n_heavy + (static_cast<uint64_t>(g.n_seg - g.n_heavy) + 31) / 32;
  if (hub_tasks) {
    const int grid = grid_for_tasks(hub_tasks, 5);
    if (q.first_pass && g.nlab) {
      PM_DISPATCH_WORD(q.word_kind, k_lcc_first<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), q.tables, q.hub_acc,
                                                                              q.ctr));
    } else {
      PM_DISPATCH_WORD(q.word_kind, k_lcc_check<W, false><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), q.tables,
                                                                                     q.hub_acc, q.ctr));
    }
  }
  const int grid = grid_for_tasks(((static_cast<uint64_t>(g.V) + 31) / 32 + 31) / 32, 4);
  PM_DISPATCH_WORD(q.word_kind,
                   k_lcc_check<W, true><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), q.tables, q.hub_acc, q.ctr));
}

void launch_apply(const DevGraph& g, const QueryDevPtrs& q, cudaStream_t s) {
  if (g.symmetric) {
    const int grid1 = grid_for_tiles(g.V, 8);
    PM_DISPATCH_WORD(q.word_kind, k_apply_changed<W><<<grid1, kThreads, 0, s>>>(g, state_of<W>(q), q.ctr));
    const int grid2 = grid_for_tasks(sweep_tasks(g), 8);
    PM_DISPATCH_WORD(q.word_kind, k_push_changed<W><<<grid2, kThreads, 0, s>>>(g, state_of<W>(q)));
    return;
  }
  const int grid = grid_for_tasks(sweep_tasks(g), 8);
  PM_DISPATCH_WORD(q.word_kind, k_apply<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), q.hub_acc, q.ctr));
}

void launch_lcc_loop_head(LccLoopCtl* ctl, cudaStream_t s) {
  note_launch();
  k_lcc_loop_head<<<1, 32, 0, s>>>(ctl);
}

void launch_lcc_loop_tail(QueryDevPtrs* a, LccLoopCtl* ctl, cudaGraphConditionalHandle h, cudaStream_t s) {
  note_launch();
  k_lcc_loop_tail<<<1, 32, 0, s>>>(a, ctl, reinterpret_cast<LccPassRow*>(ctl + 1), h);
}

// One LCC pass (sweep 1 + sweep 2), grids as launch_lcc_check and
// launch_apply, with the query's pointers read from the device block `a`.
void launch_lcc_pass_at(const DevGraph& g, int word_kind, const QueryDevPtrs* a, cudaStream_t s) {
  const uint64_t hub_tasks = g.n_heavy + (static_cast<uint64_t>(g.n_seg - g.n_heavy) + 31) / 32;
  if (hub_tasks) {
    const int grid = grid_for_tasks(hub_tasks, 5);
    if (g.nlab) PM_DISPATCH_WORD(word_kind, k_lcc_first_at<W><<<grid, kThreads, 0, s>>>(g, a));
    PM_DISPATCH_WORD(word_kind, k_lcc_check_at<W, false><<<grid, kThreads, 0, s>>>(g, a));
  }
  const int grid = grid_for_tasks(((static_cast<uint64_t>(g.V) + 31) / 32 + 31) / 32, 4);
  PM_DISPATCH_WORD(word_kind, k_lcc_check_at<W, true><<<grid, kThreads, 0, s>>>(g, a));
  if (g.symmetric) {
    const int grid1 = grid_for_tiles(g.V, 8);
    PM_DISPATCH_WORD(word_kind, k_apply_changed_at<W><<<grid1, kThreads, 0, s>>>(g, a));
    const int grid2 = grid_for_tasks(sweep_tasks(g), 8);
    PM_DISPATCH_WORD(word_kind, k_push_changed_at<W><<<grid2, kThreads, 0, s>>>(g, a));
    return;
  }
  const int grid2 = grid_for_tasks(sweep_tasks(g), 8);
  PM_DISPATCH_WORD(word_kind, k_apply_at<W><<<grid2, kThreads, 0, s>>>(g, a));
}

// Blocks of a multi-query launch: nq x (the single-query grid / nq, at
// least one), so the whole launch keeps the single-query residency.
inline int multi_grid(int single_grid, uint32_t nq) {
  const int per = std::max(1, single_grid / static_cast<int>(nq));
  return per * static_cast<int>(nq);
}

void launch_lcc0_multi(const DevGraph& g, int word_kind, const QueryDevPtrs* qs, const uint32_t* active, uint32_t nq,
                       cudaStream_t s) {
  if (!nq) return;
  const int grid = multi_grid(device_sm_count() * 8, nq);
  PM_DISPATCH_WORD(word_kind, k_lcc0_multi<W><<<grid, kThreads, 0, s>>>(g, qs, active, nq));
}

void launch_lcc_pass_multi(const DevGraph& g, int word_kind, const QueryDevPtrs* qs, const uint32_t* active,
                           uint32_t nq, cudaStream_t s) {
  if (!nq) return;
  const uint64_t hub_tasks = g.n_heavy + (static_cast<uint64_t>(g.n_seg - g.n_heavy) + 31) / 32;
  if (hub_tasks) {
    const int grid = multi_grid(grid_for_tasks(hub_tasks, 5), nq);
    if (g.nlab) PM_DISPATCH_WORD(word_kind, k_lcc_first_multi<W><<<grid, kThreads, 0, s>>>(g, qs, active, nq));
    PM_DISPATCH_WORD(word_kind, k_lcc_check_multi<W, false><<<grid, kThreads, 0, s>>>(g, qs, active, nq));
  }
  const int grid = multi_grid(grid_for_tasks(((static_cast<uint64_t>(g.V) + 31) / 32 + 31) / 32, 4), nq);
  PM_DISPATCH_WORD(word_kind, k_lcc_check_multi<W, true><<<grid, kThreads, 0, s>>>(g, qs, active, nq));
  if (g.symmetric) {
    const int grid1 = multi_grid(grid_for_tiles(g.V, 8), nq);
    PM_DISPATCH_WORD(word_kind, k_apply_changed_multi<W><<<grid1, kThreads, 0, s>>>(g, qs, active, nq));
    const int grid2 = multi_grid(grid_for_tasks(sweep_tasks(g), 8), nq);
    PM_DISPATCH_WORD(word_kind, k_push_changed_multi<W><<<grid2, kThreads, 0, s>>>(g, qs, active, nq));
    return;
  }
  const int grid2 = multi_grid(grid_for_tasks(sweep_tasks(g), 8), nq);
  PM_DISPATCH_WORD(word_kind, k_apply_multi<W><<<grid2, kThreads, 0, s>>>(g, qs, active, nq));
}

void launch_counters_multi(const QueryDevPtrs* qs, const uint32_t* active, uint32_t nq, StepCounters* out, bool clear,
                           cudaStream_t s) {
  if (!nq) return;
  note_launch();
  k_counters_multi<<<std::max(1u, (nq * 16 + 255) / 256), 256, 0, s>>>(qs, active, nq, out, clear ? 1 : 0);
}

void launch_worklist(const DevGraph& g, const QueryDevPtrs& q, uint64_t mask, uint32_t* wl, uint32_t* wl_index,
                     uint32_t* block_counts, uint32_t* count, cudaStream_t s) {
  const uint32_t blocks = static_cast<uint32_t>((g.V + kTileV - 1) / kTileV);
  if (blocks == 0) {
    cudaMemsetAsync(count, 0, sizeof(uint32_t), s);
    return;
  }
  PM_DISPATCH_WORD(q.word_kind, k_wl_count<W><<<blocks, 256, 0, s>>>(g, state_of<W>(q), mask, block_counts));
  note_launch();
  k_wl_scan<<<1, 1024, 0, s>>>(block_counts, blocks, count);
  PM_DISPATCH_WORD(q.word_kind,
                   k_wl_write<W><<<blocks, 256, 0, s>>>(g, state_of<W>(q), mask, block_counts, wl, wl_index));
}

void launch_slice_count(const DevGraph& g, const uint32_t* wl, uint32_t n_wl, uint32_t R, uint32_t t,
                        unsigned long long* tile_counts, unsigned long long* total, cudaStream_t s) {
  const uint32_t tiles = (n_wl + kTileV - 1) / kTileV;
  if (tiles == 0) {
    cudaMemsetAsync(total, 0, sizeof(unsigned long long), s);
    return;
  }
  note_launch();
  k_slice_count<<<tiles, 256, 0, s>>>(g, wl, n_wl, R, t, tile_counts);
  note_launch();
  k_slice_scan<<<1, 1024, 0, s>>>(tile_counts, tiles, total);
}

void launch_slice_write(const DevGraph& g, const uint32_t* wl, uint32_t n_wl, uint32_t R, uint32_t t,
                        const unsigned long long* tile_offsets, uint4* slices, cudaStream_t s) {
  const uint32_t tiles = (n_wl + kTileV - 1) / kTileV;
  if (tiles == 0) return;
  note_launch();
  k_slice_write<<<tiles, 256, 0, s>>>(g, wl, n_wl, R, t, tile_offsets, slices);
}

namespace {
// Scratch layout of the ENUMERATION item listing (u64 words).
struct EnumItemScratch {
  uint32_t* heavy;
  uint32_t* light;
  unsigned long long *heavy_local, *light_local, *heavy_tiles, *light_tiles, *totals;
  uint64_t tiles;
  EnumItemScratch(unsigned long long* scratch, uint32_t n_wl) {
    tiles = (static_cast<uint64_t>(n_wl) + kTileV - 1) / kTileV;
    heavy = reinterpret_cast<uint32_t*>(scratch);
    light = heavy + n_wl;
    heavy_local = scratch + n_wl;
    light_local = heavy_local + n_wl;
    heavy_tiles = light_local + n_wl;
    light_tiles = heavy_tiles + tiles;
    totals = light_tiles + tiles;
  }
};
}  // namespace

uint64_t enum_item_scratch_words(uint32_t n_wl) {
  const uint64_t tiles = (static_cast<uint64_t>(n_wl) + kTileV - 1) / kTileV;
  return 3ull * n_wl + 2 * tiles + 3;
}

void launch_enum_item_count(const DevGraph& g, const uint32_t* wl, uint32_t n_wl, uint32_t t, uint32_t s2,
                            unsigned long long* scratch, cudaStream_t s) {
  const EnumItemScratch x(scratch, n_wl);
  const EnumItemRule r{t, s2};
  cudaMemsetAsync(x.totals, 0, 3 * sizeof(unsigned long long), s);
  if (n_wl == 0) return;
  note_launch();
  k_enum_item_count<<<device_sm_count() * 8, 256, 0, s>>>(g, wl, n_wl, r, x.heavy, x.light,
                                                            reinterpret_cast<uint32_t*>(x.totals + 2));
  note_launch();
  k_scan_tiles<<<static_cast<unsigned>(x.tiles), 256, 0, s>>>(x.heavy, n_wl, x.heavy_local, x.heavy_tiles);
  note_launch();
  k_scan_tiles<<<static_cast<unsigned>(x.tiles), 256, 0, s>>>(x.light, n_wl, x.light_local, x.light_tiles);
  note_launch();
  k_slice_scan<<<1, 1024, 0, s>>>(x.heavy_tiles, static_cast<uint32_t>(x.tiles), x.totals);
  note_launch();
  k_slice_scan<<<1, 1024, 0, s>>>(x.light_tiles, static_cast<uint32_t>(x.tiles), x.totals + 1);
}

const unsigned long long* enum_item_totals(const unsigned long long* scratch, uint32_t n_wl) {
  return EnumItemScratch(const_cast<unsigned long long*>(scratch), n_wl).totals;
}

void launch_enum_item_write(const DevGraph& g, const uint32_t* wl, uint32_t n_wl, uint32_t t, uint32_t s2,
                            const unsigned long long* scratch, uint4* items, cudaStream_t s) {
  if (n_wl == 0) return;
  const EnumItemScratch x(const_cast<unsigned long long*>(scratch), n_wl);
  note_launch();
  k_enum_item_write<<<device_sm_count() * 8, 256, 0, s>>>(g, wl, n_wl, EnumItemRule{t, s2}, x.light, x.heavy_local,
                                                            x.heavy_tiles, x.light_local, x.light_tiles, x.totals,
                                                            items);
}

void launch_export(const DevGraph& g, const QueryDevPtrs& q, uint64_t* cand, uint8_t* vact, uint8_t* eact_bytes,
                   cudaStream_t s) {
  const int grid = device_sm_count() * 8;
  PM_DISPATCH_WORD(q.word_kind, k_export<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), cand, vact, eact_bytes));
}

void launch_graph_stat(const DevGraph& g, const QueryDevPtrs& q, const GraphStatDev& p, cudaStream_t s) {
  const int grid = grid_for_tiles(g.V, 8);
  const size_t shmem = sizeof(uint32_t) * p.slots * p.slots;
  PM_DISPATCH_WORD(q.word_kind, k_stat_counts<W><<<grid, kThreads, shmem, s>>>(g, static_cast<const W*>(q.vs), q.eact,
                                                                                p));
  const uint64_t warps = static_cast<uint64_t>(p.blocks) * (p.slots + 1);
  const int grid2 = static_cast<int>((warps + kWarpsPerBlock - 1) / kWarpsPerBlock);
  PM_DISPATCH_WORD(q.word_kind, k_stat_accum<W><<<grid2, kThreads, 0, s>>>(g, static_cast<const W*>(q.vs), q.eact, p));
}

}  // namespace pmgb
