// Non-local constraint checking (CC / PC / TDS) and ENUMERATION on GB300.
//
// One warp runs one depth-first walk (one source vertex, one start role) at
// a time, with an explicit per-step frame stack in shared memory.  The
// control flow is warp-uniform; lanes parallelise the per-step neighbour
// scan: a step loads 32 CSR entries of the current vertex at once, each
// lane tests its entry (active bit, neighbour role bit via one gather of the
// neighbour's packed word, step-specific filters) and a ballot yields the
// candidate mask.  Candidates are then taken in CSR order, exactly the order
// of the reference's recursive loops, so the memo semantics (see
// walk_program.h) and the first successful path are reproduced.
//
// The reference's per-source memos (std::unordered_map, cleared per source,
// multiple_label_cc_cpu.tpp:105-115, tds :46-63) become per-warp open-
// addressing tables in global scratch, probed 32 slots per step by the whole
// warp and invalidated per walk by an epoch number, so no clearing pass is
// needed between walks.  A walk whose reference-memo table passes half load
// stops with kItemOverflow and is re-run by the host with larger tables.  A
// third, best-effort table caches explored states (NLCC) and subtree counts
// (ENUMERATION of distinct-label templates).
//
// Work items are (worklist vertex, start role) pairs handed out through an
// atomic counter in role-major order, so consecutive items of a warp share
// the program cached in shared memory.  Item index = wl_pos * n_progs + role
// index is the reference's sequential order (ascending vertex, roles in
// constraint order), used to emulate its "alreadyMatched" shortcut.
#include <cuda_runtime.h>

#include "kernels.h"

namespace pmgb {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kWalkWarps = 4;  // warps per block
// k_walk (CC/PC/TDS) is built for two resident blocks fewer than the
// enumeration kernels: 48 registers without spills instead of 40 with.
constexpr uint32_t kStateTag = 0x80000000u;

// The frame stack of a walk, one entry per step (n_steps + 1 entries), in
// dynamic shared memory sized to the launched programs: short programs
// leave room for more resident blocks.
struct WalkFrames {
  uint64_t* next;
  uint64_t* end;
  uint64_t* chunk;
  uint64_t* leaves0;  // ENUMERATION count at descent (count memo)
  uint32_t* mask;
  uint32_t* cur;
  uint32_t* bound;
  uint8_t* child;     // a descent from this step awaits its count
};

struct WarpShared {
  WalkProgram* prog;  // the warp's program (shared memory of the warp or the block)
  WalkFrames f;
  unsigned long long scanned;   // CSR entries tested by this warp (lane 0 writes)
  unsigned long long descents;  // hops taken by this warp
  // Adjacency list of the walk's source in shared memory (src_cached): the
  // whole list when it has at most kSrcCache entries, or, for programs with
  // a tail step, only the entries whose target holds the tail step's role
  // when they fit the kernel's cache (src_n entries).
  const uint32_t* src_adj;
  uint32_t src_n;
  uint32_t src_cached;
  // ENUMERATION and exact walks: the tail step iterates over the cached
  // source entries instead of the bound vertex's list when that list has at
  // least tail_swap times as many 32-entry chunks (0: never).
  uint32_t tail_swap;
  // The step before the tail tests (candidate, cached source entry) pairs
  // one per lane instead of descending per candidate (0: never).
  uint32_t pair_tail;
  // ENUMERATION: programs that allow a count memo use it (0: never).
  uint32_t memo_on;
  // Exact CC/PC/TDS programs: the step before the tail records and tests
  // states in the state memo (0: it re-runs the tail step instead).
  uint32_t tail_state_memo;
};

// Source adjacency entries a warp caches in shared memory per walk (CC/PC/TDS
// walks; ENUMERATION, limited by registers rather than shared memory, keeps
// up to kSrcCacheEnum); a filtered cache (one role's entries) scans source
// lists of up to kSrcFilterScan entries.  The pair-parallel step before the
// tail runs on caches of at most kPairMaxSrc entries.
constexpr uint32_t kSrcCache = 256;
constexpr uint32_t kSrcCacheEnum = 768;
constexpr uint32_t kSrcFilterScan = 8192;
constexpr uint32_t kPairMaxSrc = 256;

// Points the warp's frames at its part of the kernel's dynamic shared
// memory (frame_bytes(steps) per warp).
__device__ __forceinline__ void bind_frames(WarpShared& ws, unsigned char* base, uint32_t steps) {
  if (lane_id() == 0) {
    WalkFrames& f = ws.f;
    f.next = reinterpret_cast<uint64_t*>(base);
    f.end = f.next + steps;
    f.chunk = f.end + steps;
    f.leaves0 = f.chunk + steps;
    f.mask = reinterpret_cast<uint32_t*>(f.leaves0 + steps);
    f.cur = f.mask + steps;
    f.bound = f.cur + steps;
    f.child = reinterpret_cast<uint8_t*>(f.bound + steps);
  }
  __syncwarp();
}

template <class W>
__device__ __forceinline__ bool role_of(const DevState<W>& st, uint32_t v, uint32_t role) {
  return (Pack<W>::cand(st.vs[v]) >> role) & 1;
}

// Copies the source's list into the warp's cache when it fits and the graph
// is symmetric (the only case where tail CHECKs search the source's list).
// filter_role >= 0 keeps only the entries whose target holds that role, in
// list order: a tail candidate holds the tail step's role, so it is in the
// source's list exactly when it is in the filtered one (the state does not
// change during a walk launch).
template <class W>
__device__ __forceinline__ void cache_source(const DevGraph& g, const DevState<W>& st, WarpShared& ws,
                                             uint32_t* cache, uint32_t cap, uint32_t source, int filter_role) {
  const unsigned lane = lane_id();
  uint32_t n = 0, cached = 0;
  if (g.symmetric) {
    const uint64_t b = g.off[source], e = g.off[source + 1];
    if (filter_role < 0) {
      if (e - b <= cap) {
        cached = 1;
        n = static_cast<uint32_t>(e - b);
        for (uint32_t i = lane; i < n; i += 32) cache[i] = g.adj[b + i];
      }
    } else if (e - b <= kSrcFilterScan) {
      // Cached when the role's entries fit (n stays <= cap: a chunk is
      // written only while the entries so far plus its own fit).
      const uint32_t len = static_cast<uint32_t>(e - b);
      cached = 1;
      for (uint32_t i0 = 0; i0 < len; i0 += 32) {
        const uint32_t i = i0 + lane;
        uint32_t x = 0;
        bool keep = false;
        if (i < len) {
          x = g.adj[b + i];
          keep = role_of(st, x, static_cast<uint32_t>(filter_role));
        }
        const unsigned m = __ballot_sync(kFull, keep);
        if (n + __popc(m) > cap) {
          cached = 0;
          n = 0;
          break;
        }
        if (keep) cache[n + __popc(m & ((1u << lane) - 1u))] = x;
        n += __popc(m);
      }
    }
  }
  __syncwarp();
  if (lane == 0) {
    ws.src_adj = cache;
    ws.src_n = n;
    ws.src_cached = cached;
  }
  __syncwarp();
}

enum : int { kNone = 0, kFound = 1, kOverflowHit = 2 };

// Role that the source cache keeps for program p (the tail VERTEX step's
// role; -1: keep the whole list), and whether p's tail may start from the
// source's side: symmetric graph, tail step at depth 2 or more, some closing
// CHECK against the source and none against the tail vertex itself.
__device__ __forceinline__ int tail_plan(const DevGraph& g, const WalkProgram& p, bool* swap_ok) {
  const int tail_d = static_cast<int>(p.tail_from) - 1;
  const int role =
      (tail_d >= 1 && tail_d < p.n_steps && p.steps[tail_d].kind == kStepVertex) ? static_cast<int>(p.steps[tail_d].role)
                                                                                  : -1;
  bool src_check = false, self_check = false;
  for (int j = p.tail_from; j < p.n_steps; ++j) {
    const int hs = p.hist_step[p.steps[j].hist];
    src_check |= hs == 0;
    self_check |= hs == tail_d;
  }
  *swap_ok = role >= 0 && g.symmetric && tail_d >= 2 && src_check && !self_check;
  return role;
}

uint64_t g_walk_budget_ns = 120ull * 1000000000ull;
uint32_t g_enum_tail_swap = 4;  // WarpShared::tail_swap of ENUMERATION launches
uint32_t g_walk_tail_swap = 4;  // ... of CC/PC/TDS launches (exact programs)
uint32_t g_enum_count_memo = 1;  // WarpShared::memo_on of ENUMERATION launches
uint32_t g_enum_pair_tail = 1;   // WarpShared::pair_tail of ENUMERATION launches
uint32_t g_walk_pair_tail = 1;   // WalkLaunch::pair_tail
uint32_t g_enum_second_split = 256;  // second-hop slice entries of ENUMERATION items (0: none)
uint32_t g_walk_tail_state_memo = 1;  // WalkLaunch::tail_state_memo

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// The step's deadline (StepCounters::deadline_ns), set once by the first
// warp that gets here after the host cleared it; called by lane 0 and
// broadcast to the warp.
__device__ __forceinline__ uint64_t warp_step_deadline(StepCounters* ctr, uint64_t budget_ns) {
  uint64_t d = 0;
  if (lane_id() == 0) {
    d = *reinterpret_cast<volatile unsigned long long*>(&ctr->deadline_ns);
    if (d == 0) {
      const unsigned long long want = global_timer_ns() + budget_ns;
      const unsigned long long prev = atomicCAS(&ctr->deadline_ns, 0ull, want);
      d = prev ? prev : want;
    }
  }
  return __shfl_sync(0xFFFFFFFFu, d, 0);
}

// ---- per-warp memo tables -------------------------------------------------
struct WarpMemo {
  uint32_t* edge;
  uint32_t* hyp;
  uint32_t* state;
  uint32_t edge_cap, hyp_cap, hyp_stride, state_cap, state_stride;
  uint32_t epoch;  // 1..65535
  uint32_t edge_n, hyp_n, state_n;
};

// Memo tables are open-addressing sets stored word-major (word w of slot s
// at tab[w * cap + s]) whose first word is a tag: the walk's 16-bit epoch
// in the high half and a 16-bit fingerprint of the key in the low half.
// Zeroed memory and slots of older epochs are free, so a new walk only
// bumps the epoch.  A lookup probes aligned windows of 32 slots, one lane
// per slot: the tags of a window are one 128-byte line, and the other words
// of a slot are read only where the whole tag matches (one live slot in
// 65,536 by chance), so a probe costs one line, not one line per word.
constexpr uint32_t kMaxEpoch = 0xFFFFu;

__device__ __forceinline__ uint32_t memo_tag(uint32_t epoch, uint32_t h) {
  return (epoch << 16) | (fmix32(h ^ 0x85ebca6bu) >> 16);
}

__device__ __forceinline__ uint32_t edge_hash(uint32_t a, uint32_t b, uint32_t step) {
  return fmix32(mix32(mix32(mix32(0x9747b28cu, a), b), step));
}

// Edge memo slot words: {tag, a, b, step}.  True when (a, b, step) is
// present.
__device__ bool edge_memo_find(const WarpMemo& m, uint32_t a, uint32_t b, uint32_t step) {
  const unsigned lane = lane_id();
  const uint32_t cap = m.edge_cap, mask = cap - 1;
  const uint32_t h = edge_hash(a, b, step);
  const uint32_t tag = memo_tag(m.epoch, h), base = h & mask & ~31u;
  for (uint32_t probe = 0; probe < cap; probe += 32) {
    const uint32_t* e = m.edge + ((base + probe + lane) & mask);
    const uint32_t tg = __ldcg(e);
    const bool live = (tg >> 16) == m.epoch;
    const bool match = tg == tag && __ldcg(e + cap) == a && __ldcg(e + 2 * cap) == b && __ldcg(e + 3 * cap) == step;
    if (__any_sync(kFull, match)) return true;
    if (__any_sync(kFull, !live)) return false;
  }
  return false;
}

// Inserts (a, b, step) if absent; false on overflow.
__device__ bool edge_memo_insert(WarpMemo& m, uint32_t a, uint32_t b, uint32_t step) {
  const unsigned lane = lane_id();
  const uint32_t cap = m.edge_cap, mask = cap - 1;
  const uint32_t h = edge_hash(a, b, step);
  const uint32_t tag = memo_tag(m.epoch, h), base = h & mask & ~31u;
  for (uint32_t probe = 0; probe < cap; probe += 32) {
    uint32_t* e = m.edge + ((base + probe + lane) & mask);
    const uint32_t tg = __ldcg(e);
    const bool live = (tg >> 16) == m.epoch;
    const bool match = tg == tag && __ldcg(e + cap) == a && __ldcg(e + 2 * cap) == b && __ldcg(e + 3 * cap) == step;
    if (__any_sync(kFull, match)) return true;
    const unsigned em = __ballot_sync(kFull, !live);
    if (em) {
      if (lane == static_cast<unsigned>(__ffs(em) - 1)) {
        __stcg(e + cap, a);
        __stcg(e + 2 * cap, b);
        __stcg(e + 3 * cap, step);
        __stcg(e, tag);
      }
      __syncwarp();
      return ++m.edge_n <= (m.edge_cap >> 1);
    }
  }
  return false;
}

// Key words after (nb, step) of the tuple memos: the stored vertices bound
// before step d (the reference's TDS hypothesis, tds :51-61) or the history
// entries of state_refs[d] (state / count memo).
struct KeyTuple {
  const WarpShared* ws;
  int d;
  int n;
  bool refs;
  __device__ __forceinline__ uint32_t operator[](int i) const {
    if (refs) {
      uint64_t r = ws->prog->state_refs[d];
      for (int k = 0; k < i; ++k) r &= r - 1;
      const int h = __ffsll(static_cast<long long>(r)) - 1;
      return ws->f.bound[ws->prog->hist_step[h]];
    }
    return ws->f.bound[ws->prog->store_step[i]];
  }
};

__device__ __forceinline__ KeyTuple stored_key(const WarpShared& ws, int d) {
  int n = 0;
  while (n < ws.prog->n_store && ws.prog->store_step[n] < d) ++n;
  return KeyTuple{&ws, d, n, false};
}
__device__ __forceinline__ KeyTuple state_key(const WarpShared& ws, int d) {
  return KeyTuple{&ws, d, __popcll(ws.prog->state_refs[d]), true};
}

__device__ __forceinline__ uint32_t tuple_hash(uint32_t nb, uint32_t step, const KeyTuple& t) {
  uint32_t h = mix32(mix32(0x1b873593u, nb), step);
  for (int i = 0; i < t.n; ++i) h = mix32(h, t[i]);
  return fmix32(h);
}

// Tuple table of `cap` slots, words {tag, nb, step, key words padded with
// 0xFFFFFFFF, [count lo, count hi]} (see memo_tag).  Returns the slot of a
// live match, or ~0 with *empty_slot set to the first free slot (~0 when the
// table has no free slot in reach); *tag_out is the key's tag.
__device__ uint32_t tuple_find(const uint32_t* tab, uint32_t cap, uint32_t key_words, uint32_t epoch, uint32_t nb,
                               uint32_t step, const KeyTuple& t, uint32_t* empty_slot, uint32_t* tag_out) {
  const unsigned lane = lane_id();
  const uint32_t mask = cap - 1;
  const uint32_t h = tuple_hash(nb, step, t);
  const uint32_t tag = memo_tag(epoch, h), base = h & mask & ~31u;
  *tag_out = tag;
  for (uint32_t probe = 0; probe < cap; probe += 32) {
    const uint32_t slot = (base + probe + lane) & mask;
    const uint32_t* e = tab + slot;
    const uint32_t tg = __ldcg(e);
    const bool live = (tg >> 16) == epoch;
    bool match = tg == tag && __ldcg(e + cap) == nb && __ldcg(e + 2 * cap) == step;
    for (uint32_t i = 0; match && i < key_words; ++i) {
      const uint32_t want = static_cast<int>(i) < t.n ? t[i] : 0xFFFFFFFFu;
      if (__ldcg(e + static_cast<uint64_t>(3 + i) * cap) != want) match = false;
    }
    const unsigned mm = __ballot_sync(kFull, match);
    if (mm) return (base + probe + __ffs(mm) - 1) & mask;
    const unsigned em = __ballot_sync(kFull, !live);
    if (em) {
      *empty_slot = (base + probe + __ffs(em) - 1) & mask;
      return ~0u;
    }
  }
  *empty_slot = ~0u;
  return ~0u;
}

__device__ void tuple_write(uint32_t* tab, uint32_t cap, uint32_t key_words, uint32_t slot, uint32_t tag,
                            uint32_t nb, uint32_t step, const KeyTuple& t, bool with_count, unsigned long long count) {
  if (lane_id() == 0) {
    uint32_t* w = tab + slot;
    __stcg(w + cap, nb);
    __stcg(w + 2 * cap, step);
    for (uint32_t i = 0; i < key_words; ++i)
      __stcg(w + static_cast<uint64_t>(3 + i) * cap, static_cast<int>(i) < t.n ? t[i] : 0xFFFFFFFFu);
    if (with_count) {
      __stcg(w + static_cast<uint64_t>(3 + key_words) * cap, static_cast<uint32_t>(count));
      __stcg(w + static_cast<uint64_t>(4 + key_words) * cap, static_cast<uint32_t>(count >> 32));
    }
    __stcg(w, tag);
  }
  __syncwarp();
}

// The reference's hypothesis memo (tds :51-63): kFound if (nb, step, stored)
// was bound before; otherwise inserts it (kNone, or kOverflowHit when the
// table is past half load — the host then re-runs the walk).
__device__ int hyp_memo(WarpMemo& m, uint32_t nb, uint32_t step, const WarpShared& ws, int d) {
  const KeyTuple t = stored_key(ws, d);
  uint32_t empty = ~0u;
  const uint32_t key_words = m.hyp_stride - 3;
  uint32_t tag;
  if (tuple_find(m.hyp, m.hyp_cap, key_words, m.epoch, nb, step, t, &empty, &tag) != ~0u) return kFound;
  if (empty == ~0u) return kOverflowHit;
  tuple_write(m.hyp, m.hyp_cap, key_words, empty, tag, nb, step, t, false, 0);
  return ++m.hyp_n <= (m.hyp_cap >> 1) ? kNone : kOverflowHit;
}

// State memo: kFound when (nb, step, state key) was entered before; else
// records it (kNone), or kOverflowHit once the table passes half load (the
// walk is then re-run with a larger table: a walk that forgets states can
// take exponential time).
__device__ int state_seen(WarpMemo& m, uint32_t nb, uint32_t step, const WarpShared& ws, int d) {
  const KeyTuple t = state_key(ws, d);
  uint32_t empty = ~0u;
  const uint32_t key_words = m.state_stride - 5;
  uint32_t tag;
  if (tuple_find(m.state, m.state_cap, key_words, m.epoch, nb, step | kStateTag, t, &empty, &tag) != ~0u)
    return kFound;
  if (empty == ~0u || m.state_n >= (m.state_cap >> 1)) return kOverflowHit;
  tuple_write(m.state, m.state_cap, key_words, empty, tag, nb, step | kStateTag, t, false, 0);
  ++m.state_n;
  return kNone;
}

// Count memo lookup: true and *count when the subtree count is cached.
__device__ bool count_lookup(const WarpMemo& m, uint32_t nb, uint32_t step, const WarpShared& ws, int d,
                             unsigned long long* count) {
  const KeyTuple t = state_key(ws, d);
  uint32_t empty = ~0u;
  const uint32_t key_words = m.state_stride - 5;
  uint32_t tag;
  const uint32_t slot = tuple_find(m.state, m.state_cap, key_words, m.epoch, nb, step, t, &empty, &tag);
  if (slot == ~0u) return false;
  const uint32_t* e = m.state + slot;
  *count = static_cast<unsigned long long>(__ldcg(e + static_cast<uint64_t>(3 + key_words) * m.state_cap)) |
           (static_cast<unsigned long long>(__ldcg(e + static_cast<uint64_t>(4 + key_words) * m.state_cap)) << 32);
  return true;
}

// Caches a finished subtree's count; false once the table passes half load.
__device__ bool count_store(WarpMemo& m, uint32_t nb, uint32_t step, const WarpShared& ws, int d,
                            unsigned long long count) {
  if (m.state_n >= (m.state_cap >> 1)) return false;
  const KeyTuple t = state_key(ws, d);
  uint32_t empty = ~0u;
  const uint32_t key_words = m.state_stride - 5;
  uint32_t tag;
  if (tuple_find(m.state, m.state_cap, key_words, m.epoch, nb, step, t, &empty, &tag) != ~0u) return true;
  if (empty == ~0u) return false;
  tuple_write(m.state, m.state_cap, key_words, empty, tag, nb, step, t, true, count);
  ++m.state_n;
  return true;
}

// ---- neighbour scans ------------------------------------------------------

// Index of `target` in the strictly increasing list adj[lo, hi), or ~0
// (warp-cooperative 32-way search).
__device__ uint64_t warp_find_sorted(const uint32_t* __restrict__ adj, uint64_t lo, uint64_t hi, uint32_t target) {
  const unsigned lane = lane_id();
  while (hi - lo > 32) {
    const uint64_t span = hi - lo;
    const uint64_t step = (span + 31) / 32;
    const uint64_t idx = lo + lane * step;
    const bool le = idx < hi && adj[idx] <= target;
    const unsigned m = __ballot_sync(kFull, le);
    if (!m) return ~uint64_t(0);
    const unsigned last = 31 - __clz(m);
    const uint64_t nlo = lo + last * step;
    const uint64_t nhi = nlo + step < hi ? nlo + step : hi;
    lo = nlo;
    hi = nhi;
  }
  const uint64_t idx = lo + lane;
  const bool eq = idx < hi && adj[idx] == target;
  const unsigned m = __ballot_sync(kFull, eq);
  return m ? lo + (__ffs(m) - 1) : ~uint64_t(0);
}

// Per-lane binary search of `target` in the strictly increasing adj[lo, hi).
__device__ __forceinline__ uint64_t lane_find_sorted(const uint32_t* __restrict__ adj, uint64_t lo, uint64_t hi,
                                                     uint32_t target) {
  const uint64_t end = hi;
  while (lo < hi) {
    const uint64_t mid = lo + ((hi - lo) >> 1);
    if (adj[mid] < target)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < end && adj[lo] == target) ? lo : ~uint64_t(0);
}

__device__ __forceinline__ void frame_enter(const DevGraph& g, WarpShared& ws, int d) {
  const uint32_t cur = ws.f.cur[d];
  __syncwarp();
  if (lane_id() == 0) {
    ws.f.next[d] = g.off[cur];
    ws.f.end[d] = g.off[cur + 1];
    ws.f.mask[d] = 0;
    ws.f.child[d] = 0;
  }
  __syncwarp();
}

// Loads the next chunk of up to 32 CSR entries of step d and returns the
// candidate mask (VERTEX / FINAL filters), or false when the list is done.
template <class W, bool kEnum>
__device__ bool load_chunk(const DevGraph& g, const DevState<W>& st, WarpShared& ws, int d, const WalkStep& s,
                           uint32_t source) {
  const unsigned lane = lane_id();
  const uint64_t next = ws.f.next[d], end = ws.f.end[d];
  if (next >= end) return false;
  const uint32_t cnt = end - next < 32 ? static_cast<uint32_t>(end - next) : 32u;
  const uint64_t e = next + lane;
  bool ok = lane < cnt && edge_active(st.eact, e);
  uint32_t nb = 0;
  if (ok) {
    nb = g.adj[e];
    ok = role_of(st, nb, s.role);
  }
  if (s.kind == kStepFinal) ok = ok && nb != source;
  if ((kEnum || ws.prog->injective) && ok) {
    for (int h = 0; h < ws.prog->n_hist && ws.prog->hist_step[h] < d; ++h)
      if (ws.f.bound[ws.prog->hist_step[h]] == nb) ok = false;
  }
  const unsigned mask = __ballot_sync(kFull, ok);
  __syncwarp();
  if (lane == 0) {
    ws.f.chunk[d] = next;
    ws.f.next[d] = next + cnt;
    ws.f.mask[d] = mask;
    ws.scanned += cnt;
  }
  __syncwarp();
  return true;
}

// Next candidate of VERTEX / FINAL step d, after the reference's memo tests
// and inserts and the state memo.
template <class W, bool kEnum>
__device__ int next_vertex(const DevGraph& g, const DevState<W>& st, WarpShared& ws, WarpMemo& m, int d,
                           const WalkStep& s, uint32_t cur, uint32_t source, uint32_t* out) {
  const unsigned lane = lane_id();
  while (true) {
    const uint32_t mask = ws.f.mask[d];
    if (mask == 0) {
      if (!load_chunk<W, kEnum>(g, st, ws, d, s, source)) return kNone;
      continue;
    }
    const unsigned j = __ffs(mask) - 1;
    __syncwarp();
    if (lane == 0) ws.f.mask[d] = mask & (mask - 1);
    __syncwarp();
    const uint32_t nb = g.adj[ws.f.chunk[d] + j];
    if (!kEnum && s.kind == kStepVertex) {
      if (!ws.prog->exact) {
        // The reference's memo tests and inserts, in its order (cc :105-114,
        // tds :99-119).
        const uint32_t a = cur < nb ? cur : nb, b = cur < nb ? nb : cur;
        if (s.blocker >= 0 && edge_memo_find(m, a, b, static_cast<uint32_t>(s.blocker))) continue;
        if (s.hyp) {
          const int r = hyp_memo(m, nb, static_cast<uint32_t>(d), ws, d);
          if (r == kFound) continue;
          if (r == kOverflowHit) return kOverflowHit;
        }
        if (s.record && !edge_memo_insert(m, a, b, static_cast<uint32_t>(d))) return kOverflowHit;
      }
      // Exact programs fail a state the same way every time (a success ends
      // the walk), so skipping the memo only repeats the work.
      if (ws.tail_state_memo || !ws.prog->exact || d + 1 != ws.prog->tail_from) {
        const int sr = state_seen(m, nb, static_cast<uint32_t>(d), ws, d);
        if (sr == kFound) continue;
        if (sr == kOverflowHit) return kOverflowHit;
      }
    }
    *out = nb;
    return kFound;
  }
}

// Next matching CSR entry cur -> target for CHECK step d.  The reference
// revisits duplicates in the CC/PC/TDS walks and takes only the first entry
// in ENUMERATION (enumeration_cpu.tpp:96-104).
template <class W, bool kEnum>
__device__ bool next_check(const DevGraph& g, const DevState<W>& st, WarpShared& ws, int d, uint32_t cur,
                           uint32_t target) {
  const unsigned lane = lane_id();
  if (g.sorted_unique || kEnum) {
    if (ws.f.mask[d]) return false;  // already used
    __syncwarp();
    if (lane == 0) ws.f.mask[d] = 1;
    __syncwarp();
    if (Pack<W>::cand(st.vs[target]) == 0) return false;
    if (g.sorted_unique) {
      const uint64_t idx = warp_find_sorted(g.adj, ws.f.next[d], ws.f.end[d], target);
      return idx != ~uint64_t(0) && edge_active(st.eact, idx);
    }
    for (uint64_t e0 = ws.f.next[d]; e0 < ws.f.end[d]; e0 += 32) {
      const uint64_t e = e0 + lane;
      const bool hit = e < ws.f.end[d] && edge_active(st.eact, e) && g.adj[e] == target;
      if (__any_sync(kFull, hit)) return true;
    }
    return false;
  }
  while (true) {
    uint32_t mask = ws.f.mask[d];
    if (mask == 0) {
      const uint64_t next = ws.f.next[d], end = ws.f.end[d];
      if (next >= end) return false;
      const uint32_t cnt = end - next < 32 ? static_cast<uint32_t>(end - next) : 32u;
      const uint64_t e = next + lane;
      const bool ok = lane < cnt && edge_active(st.eact, e) && g.adj[e] == target &&
                      Pack<W>::cand(st.vs[target]) != 0;
      mask = __ballot_sync(kFull, ok);
      __syncwarp();
      if (lane == 0) {
        ws.f.chunk[d] = next;
        ws.f.next[d] = next + cnt;
        ws.f.mask[d] = mask;
      }
      __syncwarp();
      continue;
    }
    __syncwarp();
    if (lane == 0) ws.f.mask[d] = mask & (mask - 1);
    __syncwarp();
    return true;
  }
}

// The last VERTEX step of a walk whose remaining steps are CHECKs only, on
// sorted adjacency: every lane binds its own candidate and evaluates all
// remaining CHECKs itself (binary search in the candidate's list), so a
// chunk of 32 candidates is finished in one pass instead of 32 descents.
// NLCC (exact programs only): kFound with the first passing candidate in
// CSR order.  ENUMERATION: adds the passing candidates to *leaves.
// Tail step from the source's side (symmetric graphs, source cached and
// filtered to the tail role): the candidates are the cached source entries
// x, kept when x is in the bound vertex's list [b2, e2) with that entry
// active, (ENUMERATION) differs from the history vertices the step compares,
// and passes the other CHECKs.  This is the set the forward scan accepts: x
// in the source's list is the source CHECK, x in [b2, e2) active and holding
// the role is the scan's entry test.  ENUMERATION adds the set's size to
// *leaves; NLCC returns its smallest vertex, which is the forward scan's
// first hit (both lists are sorted by vertex id).
template <class W, bool kEnum>
__device__ int tail_from_source(const DevGraph& g, const DevState<W>& st, WarpShared& ws, int d, uint64_t b2,
                                uint64_t e2, uint32_t* out, unsigned long long* leaves) {
  const unsigned lane = lane_id();
  const int n_steps = ws.prog->n_steps;
  unsigned long long found = 0;
  int res = kNone;
  for (uint32_t i0 = 0; i0 < ws.src_n; i0 += 32) {
    const uint32_t i = i0 + lane;
    bool ok = i < ws.src_n;
    uint32_t x = 0;
    if (ok) x = ws.src_adj[i];
    if (kEnum)
      for (int h = 0; ok && h < ws.prog->n_hist && ws.prog->hist_step[h] < d; ++h)
        if (ws.f.bound[ws.prog->hist_step[h]] == x) ok = false;
    if (ok) {
      const uint64_t idx = lane_find_sorted(g.adj, b2, e2, x);
      ok = idx != ~uint64_t(0) && edge_active(st.eact, idx);
    }
    for (int j = ws.prog->tail_from; ok && j < n_steps; ++j) {
      const int hs = ws.prog->hist_step[ws.prog->steps[j].hist];
      if (hs == 0) continue;
      const uint32_t t = ws.f.bound[hs];
      ok = lane_find_sorted(g.adj, g.off[t], g.off[t + 1], x) != ~uint64_t(0);
    }
    const unsigned mask = __ballot_sync(kFull, ok);
    if (kEnum) {
      found += __popc(mask);
    } else if (mask) {
      *out = __shfl_sync(kFull, x, __ffs(mask) - 1);
      res = kFound;
      break;
    }
  }
  __syncwarp();
  if (lane == 0) {
    ws.f.next[d] = e2;
    ws.scanned += ws.src_n;
  }
  __syncwarp();
  if (kEnum) *leaves += found;
  return res;
}

// Position of the n-th (0-based) set bit of m (n < popc(m)).
__device__ __forceinline__ int nth_set_bit(unsigned m, unsigned n) {
  for (unsigned k = 0; k < n; ++k) m &= m - 1;
  return __ffs(m) - 1;
}

// Step d just before the tail step d + 1 (whose closing CHECKs include the
// source and not the tail vertex; the source's tail-role entries cached):
// instead of binding each candidate v of step d and running the tail step
// below it, every chunk of 32 entries tests all (candidate v, cached entry
// x) pairs, one pair per lane and round, candidate-major.  A pair passes
// when x is in v's list with that entry active, (ENUMERATION) differs from
// the history vertices the tail step compares (v for step d), and passes
// the other CHECKs: exactly what the tail step below v accepts.  ENUMERATION
// adds the passing pairs to *leaves.  NLCC (exact programs): the first
// passing pair in (candidate CSR order, x ascending) order is the
// depth-first walk's first success; it binds steps d and d + 1 and returns
// kFound.  Both then leave step d exhausted.
template <class W, bool kEnum>
__device__ int pair_tail_step(const DevGraph& g, const DevState<W>& st, WarpShared& ws, int d, const WalkStep& s,
                         unsigned long long* leaves) {
  const unsigned lane = lane_id();
  const int n_steps = ws.prog->n_steps;
  const int t_step = d + 1;
  const uint32_t n_f = ws.src_n;
  unsigned long long found = 0;
  while (true) {
    const uint64_t next = ws.f.next[d], end = ws.f.end[d];
    if (next >= end) break;
    const uint32_t cnt = end - next < 32 ? static_cast<uint32_t>(end - next) : 32u;
    const uint64_t e = next + lane;
    bool ok = lane < cnt && edge_active(st.eact, e);
    uint32_t nb = 0;
    if (ok) {
      nb = g.adj[e];
      ok = role_of(st, nb, s.role);
    }
    if (kEnum && ok) {
      for (int h = 0; h < ws.prog->n_hist && ws.prog->hist_step[h] < d; ++h)
        if (ws.f.bound[ws.prog->hist_step[h]] == nb) ok = false;
    }
    __syncwarp();
    if (lane == 0) {
      ws.f.next[d] = next + cnt;
      ws.scanned += cnt;
    }
    __syncwarp();
    const unsigned cm = __ballot_sync(kFull, ok);
    if (!cm || n_f == 0) continue;
    uint64_t b2 = 0, e2 = 0;
    if (ok) {
      b2 = g.off[nb];
      e2 = g.off[nb + 1];
    }
    const uint32_t total = static_cast<uint32_t>(__popc(cm)) * n_f;
    for (uint32_t p0 = 0; p0 < total; p0 += 32) {
      const uint32_t p = p0 + lane;
      const bool act = p < total;
      const uint32_t c = act ? p / n_f : 0u, i = act ? p % n_f : 0u;
      const int from = nth_set_bit(cm, c);
      const uint32_t v = __shfl_sync(kFull, nb, from);
      const uint64_t lb = __shfl_sync(kFull, static_cast<unsigned long long>(b2), from);
      const uint64_t le = __shfl_sync(kFull, static_cast<unsigned long long>(e2), from);
      bool pass = act;
      uint32_t x = 0;
      if (pass) {
        x = ws.src_adj[i];
        if (kEnum)
          for (int h = 0; pass && h < ws.prog->n_hist && ws.prog->hist_step[h] < t_step; ++h) {
            const int hs = ws.prog->hist_step[h];
            if ((hs == d ? v : ws.f.bound[hs]) == x) pass = false;
          }
      }
      if (pass) {
        const uint64_t idx = lane_find_sorted(g.adj, lb, le, x);
        pass = idx != ~uint64_t(0) && edge_active(st.eact, idx);
      }
      for (int j = ws.prog->tail_from; pass && j < n_steps; ++j) {
        const int hs = ws.prog->hist_step[ws.prog->steps[j].hist];
        if (hs == 0) continue;
        const uint32_t t = hs == d ? v : ws.f.bound[hs];
        pass = lane_find_sorted(g.adj, g.off[t], g.off[t + 1], x) != ~uint64_t(0);
      }
      const unsigned pm = __ballot_sync(kFull, pass);
      if (kEnum) {
        found += __popc(pm);
      } else if (pm) {
        const int w = __ffs(pm) - 1;
        const uint32_t bv = __shfl_sync(kFull, v, w), bx = __shfl_sync(kFull, x, w);
        __syncwarp();
        if (lane == 0) {
          ws.f.bound[d] = bv;
          ws.f.bound[t_step] = bx;
          ws.f.next[d] = end;
        }
        __syncwarp();
        return kFound;
      }
    }
  }
  if (kEnum) *leaves += found;
  return kNone;
}

template <class W, bool kEnum>
__device__ int tail_vertex(const DevGraph& g, const DevState<W>& st, WarpShared& ws, int d, const WalkStep& s,
                           uint32_t* out, unsigned long long* leaves) {
  const unsigned lane = lane_id();
  const int n_steps = ws.prog->n_steps;
  // tail_swap is set only where the swap applies (see k_enumerate, k_walk).
  if (ws.tail_swap && ws.src_cached) {
    const uint64_t b2 = ws.f.next[d], e2 = ws.f.end[d];
    if (static_cast<uint64_t>((ws.src_n + 31) >> 5) * ws.tail_swap <= (e2 - b2 + 31) >> 5)
      return tail_from_source<W, kEnum>(g, st, ws, d, b2, e2, out, leaves);
  }
  while (true) {
    const uint64_t next = ws.f.next[d], end = ws.f.end[d];
    if (next >= end) return kNone;
    const uint32_t cnt = end - next < 32 ? static_cast<uint32_t>(end - next) : 32u;
    const uint64_t e = next + lane;
    bool ok = lane < cnt && edge_active(st.eact, e);
    uint32_t nb = 0;
    if (ok) {
      nb = g.adj[e];
      ok = role_of(st, nb, s.role);
    }
    if (kEnum && ok) {
      for (int h = 0; h < ws.prog->n_hist && ws.prog->hist_step[h] < d; ++h)
        if (ws.f.bound[ws.prog->hist_step[h]] == nb) ok = false;
    }
    for (int j = ws.prog->tail_from; ok && j < n_steps; ++j) {
      const int hs = ws.prog->hist_step[ws.prog->steps[j].hist];
      if (g.symmetric && hs != d) {
        // A CHECK is a template edge between nb's role and the bound
        // vertex's role.  LCC removes an entry only when its target holds
        // no template neighbour of the source's roles, and roles only
        // shrink, so while both hold these roles neither direction of the
        // edge was ever removed: the check is adjacency, searched in the
        // bound vertex's list, which every lane shares (for the source, in
        // its shared-memory copy when it has one).
        if (hs == 0 && ws.src_cached) {
          uint32_t lo = 0, hi = ws.src_n;
          while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (ws.src_adj[mid] < nb)
              lo = mid + 1;
            else
              hi = mid;
          }
          ok = lo < ws.src_n && ws.src_adj[lo] == nb;
        } else {
          const uint32_t t = ws.f.bound[hs];
          ok = lane_find_sorted(g.adj, g.off[t], g.off[t + 1], nb) != ~uint64_t(0);
        }
      } else {
        const uint32_t target = hs == d ? nb : ws.f.bound[hs];
        const uint64_t idx = lane_find_sorted(g.adj, g.off[nb], g.off[nb + 1], target);
        ok = idx != ~uint64_t(0) && edge_active(st.eact, idx) && Pack<W>::cand(st.vs[target]) != 0;
      }
    }
    const unsigned mask = __ballot_sync(kFull, ok);
    __syncwarp();
    if (lane == 0) {
      ws.f.next[d] = next + cnt;
      ws.scanned += cnt;
    }
    __syncwarp();
    if (kEnum) {
      *leaves += __popc(mask);
    } else if (mask) {
      *out = __shfl_sync(kFull, nb, __ffs(mask) - 1);
      return kFound;
    }
  }
}

// Runs one walk.  NLCC: returns kItemSuccess / kItemFail / kItemOverflow.
// ENUMERATION: counts completed walks into *leaves and returns kItemFail.
// Either returns kItemTimeout once %globaltimer passes `deadline`.
// [first_lo, first_hi) restricts the first hop to those positions of the
// source's adjacency list (ENUMERATION slices; the first step binds a vertex).
template <class W, bool kEnum>
__device__ uint8_t run_walk(const DevGraph& g, const DevState<W>& st, WarpShared& ws, WarpMemo& m, uint32_t source,
                            unsigned long long* leaves, uint64_t deadline, uint32_t first_lo = 0,
                            uint32_t first_hi = 0xFFFFFFFFu, uint32_t second_lo = 0,
                            uint32_t second_hi = 0xFFFFFFFFu) {
  const unsigned lane = lane_id();
  const int n_steps = ws.prog->n_steps;
  // [second_lo, second_hi) restricts the second hop the same way (ENUMERATION
  // items with one first-hop position); such items keep no count memo, so
  // they never overflow and are never re-run without the restriction.
  const bool second = second_lo != 0 || second_hi != 0xFFFFFFFFu;
  const bool count_memo = kEnum && ws.prog->count_memo && ws.memo_on && !second;
  // The deadline is read on the first iteration (so that launches of many
  // short items stop too) and every 1024 iterations after it.
  uint32_t iters = 1023;
  __syncwarp();
  if (lane == 0) {
    ws.f.bound[0] = source;
    ws.f.cur[1] = source;
  }
  __syncwarp();
  if (n_steps <= 1) {
    if (kEnum) ++*leaves;
    return kEnum ? kItemFail : kItemSuccess;
  }
  frame_enter(g, ws, 1);
  if (first_lo != 0 || first_hi != 0xFFFFFFFFu) {
    __syncwarp();
    if (lane == 0) {
      const uint64_t b = ws.f.next[1], e = ws.f.end[1];
      ws.f.next[1] = e - b > first_lo ? b + first_lo : e;
      ws.f.end[1] = e - b > first_hi ? b + first_hi : e;
    }
    __syncwarp();
  }
  int d = 1;
  while (true) {
    if ((++iters & 1023u) == 0) {
      uint64_t now = 0;
      if (lane == 0) now = global_timer_ns();
      now = __shfl_sync(kFull, now, 0);
      if (now > deadline) return kItemTimeout;
    }
    if (d == n_steps) {
      if (!kEnum) return kItemSuccess;
      ++*leaves;
      --d;
      continue;
    }
    const WalkStep s = ws.prog->steps[d];
    // Returning to a VERTEX step from a counted descent: cache the count of
    // the subtree just finished.
    if (count_memo && ws.f.child[d]) {
      if (!count_store(m, ws.f.bound[d], static_cast<uint32_t>(d), ws, d, *leaves - ws.f.leaves0[d]))
        return kItemOverflow;
      __syncwarp();
      if (lane == 0) ws.f.child[d] = 0;
      __syncwarp();
    }
    const uint32_t cur = ws.f.cur[d];
    bool adv = false;
    if (ws.pair_tail && ws.src_cached && ws.src_n <= kPairMaxSrc && s.kind == kStepVertex &&
        d + 2 == ws.prog->tail_from && (kEnum || ws.prog->exact)) {
      // pair_tail is set only for programs whose tail qualifies (k_enumerate, k_walk).
      if (pair_tail_step<W, kEnum>(g, st, ws, d, s, leaves) == kFound) return kItemSuccess;
    } else if (s.kind == kStepVertex && d + 1 == ws.prog->tail_from && g.sorted_unique &&
               (kEnum || ws.prog->exact)) {
      uint32_t nb = 0;
      if (tail_vertex<W, kEnum>(g, st, ws, d, s, &nb, leaves) == kFound) {
        __syncwarp();
        if (lane == 0) ws.f.bound[d] = nb;
        __syncwarp();
        return kItemSuccess;
      }
    } else if (s.kind == kStepVertex || s.kind == kStepFinal) {
      uint32_t nb = 0;
      int r;
      while (true) {
        r = next_vertex<W, kEnum>(g, st, ws, m, d, s, cur, source, &nb);
        // First hop on a sorted graph: each vertex comes once per item, so
        // its subtree count is never looked up again.
        if (r != kFound || !count_memo || d + 1 >= n_steps || (d == 1 && g.sorted_unique)) break;
        // Count memo: a cached subtree adds its count instead of a descent.
        unsigned long long c = 0;
        __syncwarp();
        if (lane == 0) ws.f.bound[d] = nb;
        __syncwarp();
        if (!count_lookup(m, nb, static_cast<uint32_t>(d), ws, d, &c)) break;
        *leaves += c;
      }
      if (r == kOverflowHit) return kItemOverflow;
      if (r == kFound) {
        __syncwarp();
        if (lane == 0) {
          ws.f.bound[d] = nb;
          ws.f.cur[d + 1] = nb;
          if (count_memo && d + 1 < n_steps && !(d == 1 && g.sorted_unique)) {
            ws.f.leaves0[d] = *leaves;
            ws.f.child[d] = 1;
          }
        }
        __syncwarp();
        adv = true;
      }
    } else if (s.kind == kStepCheck) {
      const uint32_t target = ws.f.bound[ws.prog->hist_step[s.hist]];
      if (next_check<W, kEnum>(g, st, ws, d, cur, target)) {
        __syncwarp();
        if (lane == 0) ws.f.cur[d + 1] = cur;
        __syncwarp();
        adv = true;
      }
    } else {  // kStepMove
      if (ws.f.mask[d] == 0) {
        const uint32_t back = ws.f.bound[ws.prog->hist_step[s.hist]];
        __syncwarp();
        if (lane == 0) {
          ws.f.mask[d] = 1;
          ws.f.cur[d + 1] = back;
        }
        __syncwarp();
        adv = true;
      }
    }
    if (adv) {
      ++d;
      if (lane == 0) ws.descents += 1;
      if (d < n_steps) {
        if (ws.prog->steps[d].kind == kStepMove) {
          __syncwarp();
          if (lane == 0) {
            ws.f.mask[d] = 0;
            ws.f.child[d] = 0;
          }
          __syncwarp();
        } else {
          frame_enter(g, ws, d);
          if (second && d == 2) {
            __syncwarp();
            if (lane == 0) {
              const uint64_t b = ws.f.next[2], e = ws.f.end[2];
              ws.f.next[2] = e - b > second_lo ? b + second_lo : e;
              ws.f.end[2] = e - b > second_hi ? b + second_hi : e;
            }
            __syncwarp();
          }
        }
      }
    } else {
      --d;
      if (d == 0) return kItemFail;
    }
  }
}

__device__ __forceinline__ void load_program(WarpShared& ws, const WalkProgram* __restrict__ src) {
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
  uint32_t* d = reinterpret_cast<uint32_t*>(ws.prog);
  __syncwarp();
  for (int i = lane_id(); i < static_cast<int>(sizeof(WalkProgram) / 4); i += 32) d[i] = s[i];
  __syncwarp();
}

__device__ __forceinline__ void next_epoch(WarpMemo& m) {
  ++m.epoch;
  if (m.epoch > kMaxEpoch || m.epoch == 0) {
    // 65,535 walks on this warp: clear the tags once and restart at 1.
    for (uint32_t i = lane_id(); i < m.edge_cap; i += 32) m.edge[i] = 0;
    for (uint32_t i = lane_id(); i < m.hyp_cap; i += 32) m.hyp[i] = 0;
    for (uint32_t i = lane_id(); i < m.state_cap; i += 32) m.state[i] = 0;
    __syncwarp();
    m.epoch = 1;
  }
  m.edge_n = 0;
  m.hyp_n = 0;
  m.state_n = 0;
}

__device__ __forceinline__ WarpMemo warp_memo(const WalkScratch& sc, uint32_t gw) {
  WarpMemo m;
  m.edge = sc.edge_tab + static_cast<uint64_t>(gw) * sc.edge_cap * 4;
  m.hyp = sc.hyp_tab + static_cast<uint64_t>(gw) * sc.hyp_cap * sc.hyp_stride;
  m.state = sc.state_tab + static_cast<uint64_t>(gw) * sc.state_cap * sc.state_stride;
  m.edge_cap = sc.edge_cap;
  m.hyp_cap = sc.hyp_cap;
  m.hyp_stride = sc.hyp_stride;
  m.state_cap = sc.state_cap;
  m.state_stride = sc.state_stride;
  m.epoch = sc.epochs[gw];
  m.edge_n = m.hyp_n = m.state_n = 0;
  return m;
}

template <class W>
__global__ void __launch_bounds__(kWalkWarps * 32, kWalkBlocksPerSm - 2) k_walk(DevGraph g, DevState<W> st, WalkLaunch w,
                                                                           WalkScratch sc,
                                                          StepCounters* ctr, uint64_t budget_ns) {
  __shared__ WarpShared s_ws[kWalkWarps];
  __shared__ WalkProgram s_prog[kWalkWarps];  // items of one launch mix programs
  __shared__ uint32_t s_src[kWalkWarps][kSrcCache];
  extern __shared__ __align__(16) unsigned char s_frames[];
  const unsigned lane = lane_id();
  const unsigned wib = threadIdx.x >> 5;
  WarpShared& ws = s_ws[wib];
  if (lane == 0) {
    ws.prog = &s_prog[wib];
    ws.scanned = 0;
    ws.descents = 0;
    ws.src_n = 0;
    ws.src_cached = 0;
    ws.tail_swap = 0;
    ws.pair_tail = 0;
    ws.memo_on = 1;
    ws.tail_state_memo = 1;
  }
  bind_frames(ws, s_frames + wib * frame_bytes(w.frame_steps), w.frame_steps);
  const uint32_t gw = blockIdx.x * kWalkWarps + wib;
  const uint64_t deadline = warp_step_deadline(ctr, budget_ns);
  WarpMemo m = warp_memo(sc, gw);
  const uint64_t n_items =
      w.slices ? w.n_slices : w.retry_items ? w.n_retry : static_cast<uint64_t>(w.n_wl) * w.n_progs;
  int cached = -1, filter_role = -1;
  unsigned long long overflow = 0;
  while (true) {
    unsigned long long gi = 0;
    if (lane == 0) gi = atomicAdd(&ctr->items, 1ull);
    gi = __shfl_sync(kFull, gi, 0);
    if (gi >= n_items) break;
    uint32_t item, r, pos, lo = 0, hi = 0xFFFFFFFFu;
    if (w.slices) {
      const uint4 sl = w.slices[gi];
      item = sl.x;
      lo = sl.y;
      hi = sl.z;
      pos = item / w.n_progs;
      r = item % w.n_progs;
      // Another slice of this item already succeeded.
      if (*reinterpret_cast<volatile uint32_t*>(w.prio + item) == kPrioSuccess) continue;
    } else if (w.retry_items) {
      item = w.retry_items[gi];
      pos = item / w.n_progs;
      r = item % w.n_progs;
    } else {
      r = static_cast<uint32_t>(gi / w.n_wl);
      pos = static_cast<uint32_t>(gi % w.n_wl);
      item = pos * w.n_progs + r;
    }
    const uint32_t v = w.wl[pos];
    // Sliced items are left to the slice launch.
    if (!w.slices && !w.retry_items && w.skip_deg && g.off[v + 1] - g.off[v] > w.skip_deg) continue;
    if (static_cast<int>(r) != cached) {
      load_program(ws, w.progs + r);
      cached = static_cast<int>(r);
      // Exact programs run the tail step on sorted lists (run_walk): cache
      // only the tail role's source entries and allow the swapped tail.
      bool swap_ok = false;
      const int role = tail_plan(g, *ws.prog, &swap_ok);
      filter_role = ws.prog->exact ? role : -1;
      __syncwarp();
      if (lane == 0) {
        ws.tail_swap = (ws.prog->exact && swap_ok) ? w.tail_swap : 0u;
        ws.pair_tail = (ws.prog->exact && swap_ok) ? w.pair_tail : 0u;
        ws.tail_state_memo = w.tail_state_memo;
      }
      __syncwarp();
    }
    if (!role_of(st, v, ws.prog->start_role)) {
      if (lane == 0 && !w.slices) w.status[item] = kItemSkip;
      continue;
    }
    next_epoch(m);
    cache_source(g, st, ws, s_src[wib], kSrcCache, v, filter_role);
    unsigned long long unused = 0;
    const uint8_t res = run_walk<W, false>(g, st, ws, m, v, &unused, deadline, lo, hi);
    if (lane == 0) {
      if (w.slices) {
        const uint32_t pr = res == kItemSuccess    ? kPrioSuccess
                            : res == kItemTimeout  ? kPrioTimeout
                            : res == kItemOverflow ? kPrioOverflow
                            : res == kItemFail     ? kPrioFail
                                                   : kPrioSkip;
        atomicMax(w.prio + item, pr);
      } else {
        w.status[item] = res;
      }
    }
    if (res == kItemOverflow) ++overflow;
    if (res == kItemTimeout) {
      if (lane == 0) atomicMax(&ctr->error, kDeviceErrorTimeout);
      break;
    }
    if (res == kItemSuccess && (w.min_marker || w.marks)) {
      // alreadyMatched marks of the successful path (cc :64, pc :42, tds :74).
      uint32_t j = 0;
      for (int d0 = 1; d0 < ws.prog->n_steps; d0 += 32) {
        const int d = d0 + static_cast<int>(lane);
        const bool mk = d < ws.prog->n_steps && ws.prog->steps[d].mark;
        const unsigned mm = __ballot_sync(kFull, mk);
        if (mk) {
          const uint32_t x = ws.f.bound[d];
          const uint32_t slot = j + __popc(mm & ((1u << lane) - 1));
          if (w.marks) w.marks[static_cast<uint64_t>(item) * w.marks_stride + slot] = x;
          if (w.min_marker) {
            const uint8_t ri = w.role_index[ws.prog->steps[d].role];
            if (ri != 0xFF) {
              const uint64_t xi = static_cast<uint64_t>(w.wl_index[x]) * w.n_progs + ri;
              atomicMin(w.min_marker + xi, item);
            }
          }
        }
        j += __popc(mm);
      }
    }
  }
  if (lane == 0) {
    sc.epochs[gw] = m.epoch;
    atomicAdd(&ctr->scanned, ws.scanned);
    atomicAdd(&ctr->descents, ws.descents);
    if (overflow) atomicAdd(&ctr->overflow, overflow);
  }
}

__global__ void k_flag_rescue(const uint8_t* __restrict__ status, const uint32_t* __restrict__ min_marker,
                              uint64_t n_items, StepCounters* ctr) {
  unsigned c = 0;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n_items; i += stride)
    if (status[i] == kItemFail && min_marker[i] < i) ++c;
  c = __reduce_add_sync(kFull, c);
  if (lane_id() == 0 && c) atomicAdd(&ctr->flagged, static_cast<unsigned long long>(c));
}

__global__ void k_prio_to_status(DevGraph g, WalkLaunch w) {
  const uint64_t n = static_cast<uint64_t>(w.n_wl) * w.n_progs;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride) {
    const uint32_t v = w.wl[i / w.n_progs];
    if (g.off[v + 1] - g.off[v] <= w.skip_deg) continue;
    const uint32_t pr = w.prio[i];
    w.status[i] = pr == kPrioSuccess    ? kItemSuccess
                  : pr == kPrioTimeout  ? kItemTimeout
                  : pr == kPrioOverflow ? kItemOverflow
                  : pr == kPrioFail     ? kItemFail
                                        : kItemSkip;
  }
}

__global__ void k_collect_overflow(const uint8_t* __restrict__ status, uint64_t n_items, uint32_t* list,
                                   StepCounters* ctr) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n_items; i += stride)
    if (status[i] == kItemOverflow) list[atomicAdd(&ctr->aux, 1ull)] = static_cast<uint32_t>(i);
}

template <class W>
__global__ void k_apply_failures(DevGraph g, DevState<W> st, const uint32_t* __restrict__ wl, uint32_t n_wl,
                                 const uint8_t* __restrict__ status, const uint8_t* __restrict__ start_roles,
                                 uint32_t n_progs, StepCounters* ctr) {
  unsigned newly = 0;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; p < n_wl; p += stride) {
    uint64_t roles = 0;
    for (uint32_t r = 0; r < n_progs; ++r)
      if (status[p * n_progs + r] == kItemFail) roles |= uint64_t(1) << start_roles[r];
    if (roles) {
      const uint32_t v = wl[p];
      st.unm[v] = Pack<W>::make(Pack<W>::cand(st.unm[v]) | roles, 0);
      if (!st.mod[v]) {
        st.mod[v] = 1;
        ++newly;
      }
    }
  }
  newly = __reduce_add_sync(kFull, newly);
  if (lane_id() == 0 && newly) atomicAdd(&ctr->modified_total, static_cast<unsigned long long>(newly));
}

template <class W>
__global__ void k_apply_list(DevGraph g, DevState<W> st, const uint32_t* __restrict__ verts,
                             const uint64_t* __restrict__ roles, uint32_t n, StepCounters* ctr) {
  unsigned newly = 0;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride) {
    const uint32_t v = verts[i];
    st.unm[v] = Pack<W>::make(Pack<W>::cand(st.unm[v]) | roles[i], 0);
    if (!st.mod[v]) {
      st.mod[v] = 1;
      ++newly;
    }
  }
  newly = __reduce_add_sync(kFull, newly);
  if (lane_id() == 0 && newly) atomicAdd(&ctr->modified_total, static_cast<unsigned long long>(newly));
}

// ENUMERATION over worklist sources, or over `items` ({worklist position,
// first-hop slice lo, hi, -}) when given.  An item whose count memo
// overflows contributes nothing and is listed in `overflow` ({position, lo,
// hi, source vertex}, ctr->aux entries) for a re-run (split, or with larger
// tables).
template <class W>
__global__ void __launch_bounds__(kWalkWarps * 32, kWalkBlocksPerSm) k_enumerate(
    DevGraph g, DevState<W> st, const WalkProgram* __restrict__ prog, uint32_t frame_steps,
    const uint32_t* __restrict__ wl, uint32_t n_wl, const uint4* __restrict__ items, uint32_t n_items,
    uint4* overflow, WalkScratch sc, StepCounters* ctr, uint64_t budget_ns, uint32_t tail_swap,
    uint32_t count_memo, uint32_t pair, uint32_t second_slice) {
  __shared__ WarpShared s_ws[kWalkWarps];
  __shared__ WalkProgram s_prog;  // every item runs the same program
  __shared__ uint32_t s_src[kWalkWarps][kSrcCacheEnum];
  extern __shared__ __align__(16) unsigned char s_frames[];
  const unsigned lane = lane_id();
  const unsigned wib = threadIdx.x >> 5;
  WarpShared& ws = s_ws[wib];
  if (lane == 0) {
    ws.prog = &s_prog;
    ws.scanned = 0;
    ws.descents = 0;
    ws.src_n = 0;
    ws.src_cached = 0;
    ws.tail_swap = 0;
    ws.pair_tail = 0;
    ws.memo_on = 1;
    ws.tail_state_memo = 1;
  }
  bind_frames(ws, s_frames + wib * frame_bytes(frame_steps), frame_steps);
  __syncwarp();
  const uint32_t gw = blockIdx.x * kWalkWarps + wib;
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(prog);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&s_prog);
    for (uint32_t i = threadIdx.x; i < sizeof(WalkProgram) / 4; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
  }
  WarpMemo m = warp_memo(sc, gw);
  const uint64_t deadline = warp_step_deadline(ctr, budget_ns);
  const uint64_t n = items ? n_items : n_wl;
  unsigned long long leaves = 0;
  // The source cache serves only the tail CHECKs, whose candidates hold the
  // tail step's role: keep just those entries.  The tail may start from the
  // source's side when the graph is symmetric, the tail step is at depth 2
  // or more, some closing CHECK is against the source and none against the
  // tail vertex itself.
  bool swap_ok = false;
  const int filter_role = tail_plan(g, s_prog, &swap_ok);
  if (lane == 0) {
    ws.tail_swap = swap_ok ? tail_swap : 0u;
    ws.pair_tail = swap_ok ? pair : 0u;
    ws.memo_on = count_memo;
  }
  __syncwarp();
  while (true) {
    unsigned long long gi = 0;
    if (lane == 0) gi = atomicAdd(&ctr->items, 1ull);
    gi = __shfl_sync(kFull, gi, 0);
    if (gi >= n) break;
    const uint4 it = items ? items[gi] : make_uint4(static_cast<uint32_t>(gi), 0u, 0xFFFFFFFFu, 0u);
    const uint32_t source = wl[it.x];
    next_epoch(m);
    cache_source(g, st, ws, s_src[wib], kSrcCacheEnum, source, filter_role);
    const unsigned long long before = leaves;
    // it.w = k + 1: entries [k * second_slice, (k + 1) * second_slice) of the
    // first-hop vertex's list at the second hop.
    uint32_t s_lo = 0, s_hi = 0xFFFFFFFFu;
    if (items && it.w && second_slice) {
      const uint64_t lo2 = static_cast<uint64_t>(it.w - 1) * second_slice;
      const uint64_t hi2 = lo2 + second_slice;
      s_lo = static_cast<uint32_t>(lo2 < 0xFFFFFFFEull ? lo2 : 0xFFFFFFFEull);
      s_hi = static_cast<uint32_t>(hi2 < 0xFFFFFFFEull ? hi2 : 0xFFFFFFFEull);
    }
    const uint8_t res = run_walk<W, true>(g, st, ws, m, source, &leaves, deadline, it.y, it.z, s_lo, s_hi);
    if (res == kItemTimeout) {
      if (lane == 0) atomicMax(&ctr->error, kDeviceErrorTimeout);
      break;
    }
    if (res == kItemOverflow) {
      leaves = before;
      if (lane == 0) {
        overflow[atomicAdd(&ctr->aux, 1ull)] = make_uint4(it.x, it.y, it.z, source);
        atomicAdd(&ctr->overflow, 1ull);
      }
    }
  }
  if (lane == 0) {
    sc.epochs[gw] = m.epoch;
    atomicAdd(&ctr->scanned, ws.scanned);
    atomicAdd(&ctr->descents, ws.descents);
    if (leaves) atomicAdd(&ctr->enumeration, leaves);
  }
}

template <class W>
DevState<W> state_of(const QueryDevPtrs& q) {
  return DevState<W>{static_cast<W*>(q.vs), q.eact, q.mod, q.sch, static_cast<W*>(q.unm), q.lt, q.tile_sch};
}

#define PM_DISPATCH_WORD(kind, ...) \
  note_launch();                    \
  switch (kind) {                   \
    case kWord16: {                 \
      using W = uint16_t;           \
      __VA_ARGS__;                  \
    } break;                        \
    case kWord32: {                 \
      using W = uint32_t;           \
      __VA_ARGS__;                  \
    } break;                        \
    case kWord64: {                 \
      using W = uint64_t;           \
      __VA_ARGS__;                  \
    } break;                        \
    default: {                      \
      using W = Wide;               \
      __VA_ARGS__;                  \
    } break;                        \
  }

}  // namespace

void set_walk_budget_ns(uint64_t ns) { g_walk_budget_ns = ns ? ns : 1; }
void set_enum_tail_swap(uint32_t ratio) { g_enum_tail_swap = ratio; }
uint32_t enum_tail_swap() { return g_enum_tail_swap; }
void set_enum_count_memo(bool on) { g_enum_count_memo = on ? 1u : 0u; }
bool enum_count_memo() { return g_enum_count_memo != 0; }
void set_walk_tail_state_memo(bool on) { g_walk_tail_state_memo = on ? 1u : 0u; }
bool walk_tail_state_memo() { return g_walk_tail_state_memo != 0; }
void set_pair_tail(bool enumeration, bool on) { (enumeration ? g_enum_pair_tail : g_walk_pair_tail) = on ? 1u : 0u; }
bool pair_tail_on(bool enumeration) { return (enumeration ? g_enum_pair_tail : g_walk_pair_tail) != 0; }
void set_enum_second_split(uint32_t entries) { g_enum_second_split = entries; }
uint32_t enum_second_split() { return g_enum_second_split; }
void set_walk_tail_swap(uint32_t ratio) { g_walk_tail_swap = ratio; }
uint32_t walk_tail_swap() { return g_walk_tail_swap; }
uint64_t walk_budget_ns() { return g_walk_budget_ns; }
namespace {
thread_local uint64_t t_walk_budget_cap_ns = 0;
}  // namespace
void set_thread_walk_budget_cap_ns(uint64_t ns) { t_walk_budget_cap_ns = ns; }
uint64_t effective_walk_budget_ns() {
  return t_walk_budget_cap_ns && t_walk_budget_cap_ns < g_walk_budget_ns ? t_walk_budget_cap_ns : g_walk_budget_ns;
}

namespace {
thread_local uint32_t t_walk_grid_share = 1;  // this thread's walker launches get 1/share of the GPU
}  // namespace
void set_thread_walk_grid_share(uint32_t share) { t_walk_grid_share = share ? share : 1; }

uint32_t walk_grid_blocks(uint32_t n_warps_available) {
  uint32_t blocks = static_cast<uint32_t>(device_sm_count()) * kWalkBlocksPerSm;
  // A share of the resident blocks (at least two per SM's worth of SMs /
  // share): persistent walker grids of concurrent requests then sit on the
  // GPU side by side instead of the first one taking every SM until it ends.
  if (t_walk_grid_share > 1) {
    const uint32_t floor_blocks = static_cast<uint32_t>(device_sm_count());
    blocks = std::max(blocks / t_walk_grid_share, floor_blocks);
  }
  if (blocks * kWalkWarps > n_warps_available) blocks = n_warps_available / kWalkWarps;
  return blocks ? blocks : 1;
}

void launch_walk(const DevGraph& g, const QueryDevPtrs& q, const WalkLaunch& w, const WalkScratch& sc,
                 cudaStream_t s) {
  const uint32_t blocks = walk_grid_blocks(sc.n_warps);
  const size_t dyn = kWalkWarps * frame_bytes(w.frame_steps);
  PM_DISPATCH_WORD(q.word_kind, k_walk<W><<<blocks, kWalkWarps * 32, dyn, s>>>(g, state_of<W>(q), w, sc, q.ctr,
                                                                               effective_walk_budget_ns()));
}

void launch_flag_rescue(const WalkLaunch& w, StepCounters* ctr, cudaStream_t s) {
  const uint64_t n = static_cast<uint64_t>(w.n_wl) * w.n_progs;
  const int grid = device_sm_count() * 4;
  note_launch();
  k_flag_rescue<<<grid, 256, 0, s>>>(w.status, w.min_marker, n, ctr);
}

void launch_prio_to_status(const DevGraph& g, const WalkLaunch& w, cudaStream_t s) {
  note_launch();
  k_prio_to_status<<<device_sm_count() * 4, 256, 0, s>>>(g, w);
}

void launch_collect_overflow(const WalkLaunch& w, uint32_t* list, StepCounters* ctr, cudaStream_t s) {
  const uint64_t n = static_cast<uint64_t>(w.n_wl) * w.n_progs;
  const int grid = device_sm_count() * 4;
  note_launch();
  k_collect_overflow<<<grid, 256, 0, s>>>(w.status, n, list, ctr);
}

void launch_apply_failures(const DevGraph& g, const QueryDevPtrs& q, const WalkLaunch& w, cudaStream_t s) {
  const int grid = device_sm_count() * 4;
  PM_DISPATCH_WORD(q.word_kind, k_apply_failures<W><<<grid, 256, 0, s>>>(g, state_of<W>(q), w.wl, w.n_wl, w.status,
                                                                         w.start_roles, w.n_progs, q.ctr));
}

void launch_apply_unmatch_list(const DevGraph& g, const QueryDevPtrs& q, const uint32_t* verts, const uint64_t* roles,
                               uint32_t n, cudaStream_t s) {
  if (!n) return;
  const int grid = device_sm_count() * 4;
  PM_DISPATCH_WORD(q.word_kind, k_apply_list<W><<<grid, 256, 0, s>>>(g, state_of<W>(q), verts, roles, n, q.ctr));
}

void launch_enumerate(const DevGraph& g, const QueryDevPtrs& q, const WalkProgram* prog, uint32_t frame_steps,
                      const uint32_t* wl, uint32_t n_wl, const uint4* items, uint32_t n_items, uint4* overflow,
                      const WalkScratch& sc, cudaStream_t s) {
  const uint32_t blocks = walk_grid_blocks(sc.n_warps);
  const size_t dyn = kWalkWarps * frame_bytes(frame_steps);
  PM_DISPATCH_WORD(q.word_kind, k_enumerate<W><<<blocks, kWalkWarps * 32, dyn, s>>>(
                                    g, state_of<W>(q), prog, frame_steps, wl, n_wl, items, n_items, overflow, sc,
                                    q.ctr, effective_walk_budget_ns(), g_enum_tail_swap, g_enum_count_memo,
                                    g_enum_pair_tail, g_enum_second_split));
}

// ---- match listing --------------------------------------------------------
//
// The embeddings ENUMERATION counts, written out: the reference's
// writeEnumeration (multiple_label_enumeration_cpu.tpp:15-35) records
// historyIndexVector, the graph vertices bound by the walk's vertex moves in
// walk order.  One warp per source of the start role, depth-first over the
// enumeration program with the reference's semantics
// (enumeration_cpu.tpp:39-118): a VERTEX step binds an active neighbour
// behind an active CSR entry that holds the step's role and is not yet in
// the history (embeddings are injective), 32 entries tested per round; a
// CHECK step needs an active entry to the history vertex it names; a MOVE
// step continues from a history vertex.  Each completed walk takes a slot
// (counters[1]); slots below `cap` are written.  No memo and no tail
// shortcut: every leaf is visited, so counters[1] ends at the ENUMERATION
// count.
namespace {
constexpr int kListWarps = 4;

template <class W>
__global__ void __launch_bounds__(kListWarps * 32) k_enum_list(DevGraph g, DevState<W> st,
                                                               const WalkProgram* __restrict__ prog_in,
                                                               const uint32_t* __restrict__ wl, uint32_t n_wl,
                                                               uint32_t* out, uint64_t cap,
                                                               unsigned long long* counters, uint64_t budget_ns,
                                                               StepCounters* ctr) {
  __shared__ WalkProgram prog;
  __shared__ uint8_t s_hidx[kMaxWalkSteps];  // VERTEX step -> history index
  __shared__ uint64_t s_pos[kListWarps][kMaxWalkSteps], s_end[kListWarps][kMaxWalkSteps],
      s_base[kListWarps][kMaxWalkSteps];
  __shared__ uint32_t s_mask[kListWarps][kMaxWalkSteps];
  __shared__ uint32_t s_hist[kListWarps][64];
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(prog_in);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&prog);
    for (uint32_t i = threadIdx.x; i < sizeof(WalkProgram) / 4; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint8_t h = 1;
    for (int d = 1; d < prog.n_steps; ++d)
      if (prog.steps[d].kind == kStepVertex || prog.steps[d].kind == kStepFinal) s_hidx[d] = h++;
  }
  __syncthreads();
  const unsigned lane = lane_id();
  const unsigned wib = threadIdx.x >> 5;
  uint64_t* pos = s_pos[wib];
  uint64_t* end = s_end[wib];
  uint64_t* base = s_base[wib];
  uint32_t* mask = s_mask[wib];
  uint32_t* hist = s_hist[wib];
  const uint64_t deadline = warp_step_deadline(ctr, budget_ns);
  const int n_steps = prog.n_steps;
  const uint32_t nh = prog.n_hist;
  uint32_t iters = 0;
  while (true) {
    unsigned long long item = 0;
    if (lane == 0) item = atomicAdd(&counters[0], 1ull);
    item = __shfl_sync(kFull, item, 0);
    if (item >= n_wl) return;
    const uint32_t v = wl[item];
    if (lane == 0) hist[0] = v;
    uint32_t cur = v;
    int d = 1;
    bool entering = true;
    __syncwarp();
    while (d > 0) {
      if ((++iters & 63u) == 0) {
        uint64_t now = 0;
        if (lane == 0) now = global_timer_ns();
        now = __shfl_sync(kFull, now, 0);
        if (now > deadline) {
          if (lane == 0) atomicMax(&ctr->error, kDeviceErrorTimeout);
          return;
        }
      }
      if (d == n_steps) {  // a completed walk
        unsigned long long slot = 0;
        if (lane == 0) slot = atomicAdd(&counters[1], 1ull);
        slot = __shfl_sync(kFull, slot, 0);
        if (slot < cap)
          for (uint32_t j = lane; j < nh; j += 32) out[slot * nh + j] = hist[j];
        --d;
        entering = false;
        __syncwarp();
        continue;
      }
      const WalkStep sp = prog.steps[d];
      if (sp.kind == kStepVertex || sp.kind == kStepFinal) {
        if (entering) {
          if (lane == 0) {
            pos[d] = g.off[cur];
            end[d] = g.off[cur + 1];
            mask[d] = 0;
          }
          __syncwarp();
        }
        const uint32_t hi = s_hidx[d];
        bool moved = false;
        while (!moved) {
          const uint32_t m = mask[d];
          if (m) {
            const uint32_t j = __ffs(m) - 1;
            const uint32_t w = g.adj[base[d] + j];
            __syncwarp();
            if (lane == 0) {
              mask[d] = m & (m - 1);
              hist[hi] = w;
            }
            __syncwarp();
            cur = w;
            ++d;
            entering = true;
            moved = true;
          } else if (pos[d] >= end[d]) {
            --d;
            entering = false;
            moved = true;
          } else {
            const uint64_t b = pos[d], e = b + lane;
            bool ok = false;
            if (e < end[d] && edge_active(st.eact, e)) {
              const uint32_t nb = g.adj[e];
              const uint64_t cw = Pack<W>::cand(st.vs[nb]);
              ok = cw != 0 && ((cw >> sp.role) & 1) && !(sp.kind == kStepFinal && nb == hist[0]);
              for (uint32_t h = 0; ok && h < hi; ++h)
                if (hist[h] == nb) ok = false;
            }
            const unsigned bm = __ballot_sync(kFull, ok);
            __syncwarp();
            if (lane == 0) {
              base[d] = b;
              pos[d] = b + 32;
              mask[d] = bm;
            }
            __syncwarp();
          }
        }
      } else if (sp.kind == kStepCheck) {
        if (!entering) {
          --d;
          continue;
        }
        const uint32_t target = hist[sp.hist];
        const uint64_t b = g.off[cur], e_end = g.off[cur + 1];
        bool found = false;
        if (Pack<W>::cand(st.vs[target]) != 0)
          for (uint64_t c = b; c < e_end && !found; c += 32) {
            const uint64_t e = c + lane;
            const bool hit = e < e_end && g.adj[e] == target && edge_active(st.eact, e);
            found = __any_sync(kFull, hit);
          }
        if (found) {
          ++d;
        } else {
          --d;
          entering = false;
        }
      } else {  // MOVE
        if (!entering) {
          --d;
          continue;
        }
        cur = hist[sp.hist];
        ++d;
      }
    }
  }
}

}  // namespace

void launch_enum_list(const DevGraph& g, const QueryDevPtrs& q, const WalkProgram* prog, const uint32_t* wl,
                      uint32_t n_wl, uint32_t* out, uint64_t cap, unsigned long long* counters, cudaStream_t s) {
  const uint32_t blocks = static_cast<uint32_t>(device_sm_count()) * 8;
  PM_DISPATCH_WORD(q.word_kind, k_enum_list<W><<<blocks, kListWarps * 32, 0, s>>>(
                                    g, state_of<W>(q), prog, wl, n_wl, out, cap, counters,
                                    effective_walk_budget_ns(), q.ctr));
}

namespace {
// ---- pruned subgraph export ---------------------------------------------------
// The reference's printActiveGraph (multiple_label_cpu.cc:270-284) prints a
// CSR entry when it is active and both its vertices are active.  Pass 1
// counts such entries per vertex (warp per vertex), the host scans, pass 2
// writes them in CSR order.
template <class W>
__global__ void __launch_bounds__(256) k_subgraph(DevGraph g, DevState<W> st, const uint64_t* __restrict__ out_off,
                                                  uint64_t* counts, uint32_t* out_adj) {
  const unsigned lane = lane_id();
  const uint64_t warps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t v = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; v < g.V; v += warps) {
    const bool va = Pack<W>::cand(st.vs[v]) != 0;
    uint64_t n = 0;
    const uint64_t b = g.off[v], e = g.off[v + 1];
    uint64_t w = out_off ? out_off[v] : 0;
    for (uint64_t c = b; va && c < e; c += 32) {
      const uint64_t x = c + lane;
      uint32_t nb = 0;
      bool keep = false;
      if (x < e && edge_active(st.eact, x)) {
        nb = g.adj[x];
        keep = Pack<W>::cand(st.vs[nb]) != 0;
      }
      const unsigned km = __ballot_sync(kFull, keep);
      if (out_adj && keep) out_adj[w + __popc(km & ((1u << lane) - 1))] = nb;
      w += __popc(km);
      n += __popc(km);
    }
    if (!out_adj && lane == 0) counts[v] = n;
  }
}
}  // namespace

void launch_subgraph(const DevGraph& g, const QueryDevPtrs& q, const uint64_t* out_off, uint64_t* counts,
                     uint32_t* out_adj, cudaStream_t s) {
  const int grid = device_sm_count() * 8;
  PM_DISPATCH_WORD(q.word_kind, k_subgraph<W><<<grid, 256, 0, s>>>(g, state_of<W>(q), out_off, counts, out_adj));
}

}  // namespace pmgb

// ===========================================================================
// Allocation-free ENUMERATION (pm_enumerate_noalloc).
//
// Some callers cannot allocate device memory at all: code that runs inside a
// host framework which owns every device allocation (a memory pool or
// arena handed out by an embedding runtime, where a stray cudaMalloc
// fragments or escapes its accounting), or code that must not reach the
// driver's allocator on a latency-critical path.  For them this entry point
// counts embeddings over a pruned state the caller already holds in device
// memory, using only the fixed scratch array below for the walker's count
// memo tables, its per-warp epochs, its work counters and the bitmaps of
// sources re-run with larger tables.
//
// The array is a file-scope __device__ variable: every GPU that loads this
// library keeps its 64 MiB until the process exits.  Host code may not take
// its address directly (the host symbol is only a stand-in); the device
// address is obtained once per device with cudaGetSymbolAddress by the first
// call made with that device current, so that first call should be made
// before any stream capture begins.  Every call reuses the array and it keeps
// the previous call's contents, so each call clears the parts that must start
// at zero; calls whose work overlaps on the GPU (different streams or host
// threads at the same time) race on the array and must be serialised by the
// caller.
// ===========================================================================
#include <algorithm>
#include <mutex>

#include "pm_types.h"

namespace pmgb {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
constexpr uint32_t kNoAllocMaxVertices = 1u << 26;         // two 8 MiB source bitmaps
constexpr size_t kNoAllocBitmapBytes = size_t(kNoAllocMaxVertices) / 8;
constexpr size_t kNoAllocHeaderBytes = 256;
constexpr size_t kNoAllocEpochBytes = 64 << 10;            // up to 16384 warps
constexpr size_t kNoAllocTableOffset = kNoAllocHeaderBytes + 2 * kNoAllocBitmapBytes + kNoAllocEpochBytes;
constexpr size_t kNoAllocTableBytes = kNoAllocScratchBytes - kNoAllocTableOffset;
constexpr uint32_t kNoAllocMaxWarps = 4096;

}  // namespace
}  // namespace pmgb

static __device__ __align__(256) unsigned char g_noalloc_scratch[pmgb::kNoAllocScratchBytes];

namespace pmgb {
namespace {

struct NoAllocLayout {
  StepCounters* ctr;
  uint32_t* bitmap_in;   // sources to run (rounds >= 1)
  uint32_t* bitmap_out;  // sources whose count memo overflowed
  uint32_t* epochs;
  uint32_t* tables;
  uint32_t cap;
  uint32_t stride;
};

// One round of ENUMERATION from every source holding the start role
// (round 0: all vertices; later rounds: the sources set in bitmap_in).
__global__ void __launch_bounds__(kWalkWarps * 32) k_enumerate_noalloc(DevGraph g, DevState<uint64_t> st,
                                                                       WalkProgram prog, NoAllocLayout L, int round,
                                                                       uint32_t n_units, uint64_t budget_ns) {
  __shared__ WarpShared s_ws[kWalkWarps];
  __shared__ WalkProgram s_prog;
  extern __shared__ __align__(16) unsigned char s_frames[];
  const unsigned lane = lane_id();
  const unsigned wib = threadIdx.x >> 5;
  WarpShared& ws = s_ws[wib];
  const uint32_t gw = blockIdx.x * kWalkWarps + wib;
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&prog);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&s_prog);
    for (uint32_t i = threadIdx.x; i < sizeof(WalkProgram) / 4; i += blockDim.x) dst[i] = src[i];
  }
  if (lane == 0) {
    ws.prog = &s_prog;
    ws.scanned = 0;
    ws.descents = 0;
    ws.src_n = 0;
    ws.src_cached = 0;
    ws.tail_swap = 0;
    ws.pair_tail = 0;
    ws.memo_on = 1;
    ws.tail_state_memo = 1;
  }
  bind_frames(ws, s_frames + wib * frame_bytes(prog.n_steps + 1u), prog.n_steps + 1u);
  __syncthreads();
  WarpMemo m{};
  m.state = L.tables + static_cast<uint64_t>(gw) * L.cap * L.stride;
  m.state_cap = L.cap;
  m.state_stride = L.stride;
  m.epoch = L.epochs[gw];
  const uint64_t deadline = warp_step_deadline(L.ctr, budget_ns);
  unsigned long long leaves = 0;
  bool stop = false;
  while (!stop) {
    unsigned long long unit = 0;
    if (lane == 0) unit = atomicAdd(&L.ctr->items, 1ull);
    unit = __shfl_sync(kFull, unit, 0);
    if (unit >= n_units) break;
    uint32_t bits = 1u, base = static_cast<uint32_t>(unit);
    if (round > 0) {
      bits = L.bitmap_in[unit];
      base = static_cast<uint32_t>(unit) * 32u;
    }
    while (bits) {
      const uint32_t b = __ffs(bits) - 1;
      bits &= bits - 1;
      const uint32_t v = base + (round > 0 ? b : 0u);
      if (!role_of(st, v, ws.prog->start_role)) continue;
      next_epoch(m);
      const unsigned long long before = leaves;
      const uint8_t res = run_walk<uint64_t, true>(g, st, ws, m, v, &leaves, deadline);
      if (res == kItemTimeout) {
        if (lane == 0) atomicMax(&L.ctr->error, kDeviceErrorTimeout);
        stop = true;
        break;
      }
      if (res == kItemOverflow) {
        leaves = before;
        if (lane == 0) {
          atomicOr(L.bitmap_out + (v >> 5), 1u << (v & 31));
          atomicAdd(&L.ctr->overflow, 1ull);
        }
      }
    }
  }
  if (lane == 0) {
    L.epochs[gw] = m.epoch;
    if (leaves) atomicAdd(&L.ctr->enumeration, leaves);
  }
}

std::mutex g_noalloc_mutex;
void* g_noalloc_base[128] = {};
uint32_t g_noalloc_first_cap = 2048;  // count-memo entries per warp, round 0
thread_local uint32_t t_noalloc_rounds = 0;  // rounds run by this thread's last call

void noalloc_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw PmError{PM_E_DEVICE, std::string(what) + ": " + cudaGetErrorString(e)};
}

// Device address of the scratch array on the current device.  Resolved once
// per device, by the first call made with that device current, with
// cudaGetSymbolAddress; later calls reuse the cached address.  The cache
// lives as long as the process: after cudaDeviceReset (or anything else that
// destroys the device's primary context) the cached address is stale, so a
// process that resets a device must not call pm_enumerate_noalloc on it
// again.
unsigned char* noalloc_scratch_current() {
  int dev = 0;
  noalloc_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= 128) throw PmError{PM_E_NO_DEVICE, "device index out of range"};
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_base[dev]) {
    void* p = nullptr;
    noalloc_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
    if (!p) throw PmError{PM_E_DEVICE, "cudaGetSymbolAddress(no-alloc scratch) returned NULL"};
    g_noalloc_base[dev] = p;
  }
  return static_cast<unsigned char*>(g_noalloc_base[dev]);
}

}  // namespace

uint32_t noalloc_max_vertices() { return kNoAllocMaxVertices; }
void set_noalloc_table_entries(uint32_t entries) { g_noalloc_first_cap = entries; }
uint32_t noalloc_last_rounds() { return t_noalloc_rounds; }

void enumerate_noalloc(const DevGraph& g, const uint64_t* d_cand, const uint32_t* d_edge_active,
                       const WalkProgram& prog, uint32_t state_words, uint64_t* d_count, cudaStream_t s) {
  if (g.V > kNoAllocMaxVertices)
    throw PmError{PM_E_INVALID_ARG, "at most 67108864 vertices (fixed 64 MiB scratch)"};
  unsigned char* base = noalloc_scratch_current();
  NoAllocLayout L{};
  L.ctr = reinterpret_cast<StepCounters*>(base);
  uint32_t* bitmap_a = reinterpret_cast<uint32_t*>(base + kNoAllocHeaderBytes);
  uint32_t* bitmap_b = reinterpret_cast<uint32_t*>(base + kNoAllocHeaderBytes + kNoAllocBitmapBytes);
  L.epochs = reinterpret_cast<uint32_t*>(base + kNoAllocHeaderBytes + 2 * kNoAllocBitmapBytes);
  L.tables = reinterpret_cast<uint32_t*>(base + kNoAllocTableOffset);
  // Count-memo entry: 5 words of epoch / step / count plus the key words.
  L.stride = 5 + std::max<uint32_t>(state_words, 1);
  const DevState<uint64_t> st{const_cast<uint64_t*>(d_cand), const_cast<uint32_t*>(d_edge_active), nullptr, nullptr,
                              nullptr, nullptr, nullptr};
  const uint32_t words = (g.V + 31) / 32;
  // The array keeps the previous call's contents: the counters (the total
  // among them) start every call at zero.
  noalloc_check(cudaMemsetAsync(L.ctr, 0, sizeof(StepCounters), s), "clear counters");
  StepCounters host_ctr{};
  t_noalloc_rounds = 0;
  for (int round = 0;; ++round) {
    t_noalloc_rounds = static_cast<uint32_t>(round) + 1;
    const uint64_t cap = uint64_t(g_noalloc_first_cap) << (2 * round);
    uint64_t warps = kNoAllocTableBytes / (cap * L.stride * 4);
    warps = std::min<uint64_t>(warps, std::min<uint64_t>(kNoAllocMaxWarps,
                                                         uint64_t(device_sm_count()) * 8 * kWalkWarps));
    warps = warps / kWalkWarps * kWalkWarps;
    if (warps == 0)
      throw PmError{PM_E_OOM, "a source's count memo needs more than the fixed 64 MiB scratch"};
    L.cap = static_cast<uint32_t>(cap);
    L.bitmap_in = (round % 2) ? bitmap_a : bitmap_b;
    L.bitmap_out = (round % 2) ? bitmap_b : bitmap_a;
    // Each round starts with empty tables (epoch 0 marks a free slot), fresh
    // epochs, no sources queued for the next round and the work counter at 0.
    noalloc_check(cudaMemsetAsync(L.tables, 0, warps * cap * L.stride * 4, s), "clear tables");
    noalloc_check(cudaMemsetAsync(L.epochs, 0, warps * 4, s), "clear epochs");
    noalloc_check(cudaMemsetAsync(L.bitmap_out, 0, size_t(words) * 4, s), "clear bitmap");
    noalloc_check(cudaMemsetAsync(&L.ctr->items, 0, sizeof(unsigned long long), s), "clear work counter");
    noalloc_check(cudaMemsetAsync(&L.ctr->overflow, 0, sizeof(unsigned long long), s), "clear overflow");
    note_launch();
    k_enumerate_noalloc<<<static_cast<unsigned>(warps / kWalkWarps), kWalkWarps * 32,
                          kWalkWarps * frame_bytes(prog.n_steps + 1u), s>>>(
        g, st, prog, L, round, round == 0 ? g.V : words, g_walk_budget_ns);
    noalloc_check(cudaGetLastError(), "k_enumerate_noalloc launch");
    noalloc_check(cudaMemcpyAsync(&host_ctr, L.ctr, sizeof(StepCounters), cudaMemcpyDeviceToHost, s),
                  "read counters");
    noalloc_check(cudaStreamSynchronize(s), "k_enumerate_noalloc");
    if (host_ctr.error == kDeviceErrorTimeout) throw PmError{PM_E_TIMEOUT, "walker time budget exceeded"};
    if (host_ctr.overflow == 0) break;
  }
  noalloc_check(cudaMemcpyAsync(d_count, &L.ctr->enumeration, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s),
                "write count");
  noalloc_check(cudaStreamSynchronize(s), "write count");
}

}  // namespace pmgb
