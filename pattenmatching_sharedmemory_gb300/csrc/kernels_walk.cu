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
// needed between walks.  A walk whose table passes half load stops with
// kItemOverflow and is re-run by the host with larger tables.
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
constexpr int kSteps = kMaxWalkSteps;

struct WalkFrames {
  uint64_t next[kSteps + 1];
  uint64_t end[kSteps + 1];
  uint64_t chunk[kSteps + 1];
  uint32_t mask[kSteps + 1];
  uint32_t cur[kSteps + 1];
  uint32_t bound[kSteps + 1];
};

struct WarpShared {
  WalkProgram prog;
  WalkFrames f;
};

enum : int { kNone = 0, kFound = 1, kOverflowHit = 2 };

// ---- per-warp memo tables -------------------------------------------------
struct WarpMemo {
  uint4* edge;
  uint32_t* hyp;
  uint32_t edge_cap, hyp_cap, hyp_stride;
  uint32_t epoch;
  uint32_t edge_n, hyp_n;
};

__device__ __forceinline__ uint32_t edge_hash(uint32_t a, uint32_t b, uint32_t step) {
  return fmix32(mix32(mix32(mix32(0x9747b28cu, a), b), step));
}

// True when (a, b, step) is present.
__device__ bool edge_memo_find(const WarpMemo& m, uint32_t a, uint32_t b, uint32_t step) {
  const unsigned lane = lane_id();
  const uint32_t mask = m.edge_cap - 1;
  const uint32_t h = edge_hash(a, b, step);
  for (uint32_t probe = 0; probe < m.edge_cap; probe += 32) {
    const uint4 ent = __ldcg(m.edge + ((h + probe + lane) & mask));
    const bool live = ent.x == m.epoch;
    const bool match = live && ent.y == a && ent.z == b && ent.w == step;
    if (__any_sync(kFull, match)) return true;
    if (__any_sync(kFull, !live)) return false;
  }
  return false;
}

// Inserts (a, b, step) if absent; false on overflow.
__device__ bool edge_memo_insert(WarpMemo& m, uint32_t a, uint32_t b, uint32_t step) {
  const unsigned lane = lane_id();
  const uint32_t mask = m.edge_cap - 1;
  const uint32_t h = edge_hash(a, b, step);
  for (uint32_t probe = 0; probe < m.edge_cap; probe += 32) {
    const uint32_t slot = (h + probe + lane) & mask;
    const uint4 ent = __ldcg(m.edge + slot);
    const bool live = ent.x == m.epoch;
    const bool match = live && ent.y == a && ent.z == b && ent.w == step;
    if (__any_sync(kFull, match)) return true;
    const unsigned em = __ballot_sync(kFull, !live);
    if (em) {
      if (lane == static_cast<unsigned>(__ffs(em) - 1)) __stcg(m.edge + slot, make_uint4(m.epoch, a, b, step));
      __syncwarp();
      return ++m.edge_n <= (m.edge_cap >> 1);
    }
  }
  return false;
}

__device__ __forceinline__ uint32_t hyp_hash(uint32_t nb, uint32_t step, const WarpShared& ws, int d) {
  uint32_t h = mix32(mix32(0x1b873593u, nb), step);
  for (int i = 0; i < ws.prog.n_store && ws.prog.store_step[i] < d; ++i) h = mix32(h, ws.f.bound[ws.prog.store_step[i]]);
  return fmix32(h);
}

// Hypothesis memo: entry = {epoch, nb, step, stored vertices..., pad 0xFFFFFFFF}.
// find_or_insert: returns kFound if present; otherwise inserts and returns
// kNone (or kOverflowHit when the table is past half load).
__device__ int hyp_memo(WarpMemo& m, uint32_t nb, uint32_t step, const WarpShared& ws, int d, bool insert) {
  const unsigned lane = lane_id();
  const uint32_t mask = m.hyp_cap - 1;
  const uint32_t h = hyp_hash(nb, step, ws, d);
  int n_h = 0;
  while (n_h < ws.prog.n_store && ws.prog.store_step[n_h] < d) ++n_h;
  const uint32_t n_words = m.hyp_stride - 3;
  for (uint32_t probe = 0; probe < m.hyp_cap; probe += 32) {
    const uint32_t slot = (h + probe + lane) & mask;
    const uint32_t* e = m.hyp + static_cast<uint64_t>(slot) * m.hyp_stride;
    const bool live = __ldcg(e) == m.epoch;
    bool match = live && __ldcg(e + 1) == nb && __ldcg(e + 2) == step;
    for (uint32_t i = 0; match && i < n_words; ++i) {
      const uint32_t want = static_cast<int>(i) < n_h ? ws.f.bound[ws.prog.store_step[i]] : 0xFFFFFFFFu;
      if (__ldcg(e + 3 + i) != want) match = false;
    }
    if (__any_sync(kFull, match)) return kFound;
    const unsigned em = __ballot_sync(kFull, !live);
    if (em) {
      if (!insert) return kNone;
      if (lane == static_cast<unsigned>(__ffs(em) - 1)) {
        uint32_t* w = m.hyp + static_cast<uint64_t>(slot) * m.hyp_stride;
        __stcg(w + 1, nb);
        __stcg(w + 2, step);
        for (uint32_t i = 0; i < n_words; ++i)
          __stcg(w + 3 + i, static_cast<int>(i) < n_h ? ws.f.bound[ws.prog.store_step[i]] : 0xFFFFFFFFu);
        __threadfence_block();
        __stcg(w, m.epoch);
      }
      __syncwarp();
      return ++m.hyp_n <= (m.hyp_cap >> 1) ? kNone : kOverflowHit;
    }
  }
  return insert ? kOverflowHit : kNone;
}

// ---- neighbour scans ------------------------------------------------------
template <class W>
__device__ __forceinline__ bool role_of(const DevState<W>& st, uint32_t v, uint32_t role) {
  return (Pack<W>::cand(st.vs[v]) >> role) & 1;
}

// Index of `target` in the strictly increasing list adj[lo, hi), or ~0.
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

template <class W, bool kEnum>
__device__ __forceinline__ void frame_enter(const DevGraph& g, WarpShared& ws, int d) {
  const uint32_t cur = ws.f.cur[d];
  if (lane_id() == 0) {
    ws.f.next[d] = g.off[cur];
    ws.f.end[d] = g.off[cur + 1];
    ws.f.mask[d] = 0;
  }
  __syncwarp();
}

// Next candidate of VERTEX / FINAL step d.
template <class W, bool kEnum>
__device__ int next_vertex(const DevGraph& g, const DevState<W>& st, WarpShared& ws, WarpMemo& m, int d,
                           const WalkStep& s, uint32_t cur, uint32_t source, uint32_t* out) {
  const unsigned lane = lane_id();
  while (true) {
    uint32_t mask = ws.f.mask[d];
    if (mask == 0) {
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
      if (s.kind == kStepFinal) ok = ok && nb != source;
      if (kEnum && ok) {
        const int n_hist = ws.prog.n_hist;
        for (int h = 0; h < n_hist && ws.prog.hist_step[h] < d; ++h)
          if (ws.f.bound[ws.prog.hist_step[h]] == nb) ok = false;
      }
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
    const unsigned j = __ffs(mask) - 1;
    __syncwarp();
    if (lane == 0) ws.f.mask[d] = mask & (mask - 1);
    __syncwarp();
    const uint32_t nb = g.adj[ws.f.chunk[d] + j];
    if (!kEnum && s.kind == kStepVertex) {
      const uint32_t a = cur < nb ? cur : nb, b = cur < nb ? nb : cur;
      if (s.blocker >= 0 && edge_memo_find(m, a, b, static_cast<uint32_t>(s.blocker))) continue;
      if (s.hyp) {
        const int r = hyp_memo(m, nb, static_cast<uint32_t>(d), ws, d, true);
        if (r == kFound) continue;
        if (r == kOverflowHit) return kOverflowHit;
      }
      if (s.record && !edge_memo_insert(m, a, b, static_cast<uint32_t>(d))) return kOverflowHit;
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

// Runs one walk.  NLCC: returns kItemSuccess / kItemFail / kItemOverflow.
// ENUMERATION: counts completed walks into *leaves and returns kItemFail.
template <class W, bool kEnum>
__device__ uint8_t run_walk(const DevGraph& g, const DevState<W>& st, WarpShared& ws, WarpMemo& m, uint32_t source,
                            unsigned long long* leaves) {
  const unsigned lane = lane_id();
  const int n_steps = ws.prog.n_steps;
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
  frame_enter<W, kEnum>(g, ws, 1);
  int d = 1;
  while (true) {
    if (d == n_steps) {
      if (!kEnum) return kItemSuccess;
      ++*leaves;
      --d;
      continue;
    }
    const WalkStep s = ws.prog.steps[d];
    const uint32_t cur = ws.f.cur[d];
    bool adv = false;
    if (s.kind == kStepVertex || s.kind == kStepFinal) {
      uint32_t nb = 0;
      const int r = next_vertex<W, kEnum>(g, st, ws, m, d, s, cur, source, &nb);
      if (r == kOverflowHit) return kItemOverflow;
      if (r == kFound) {
        __syncwarp();
        if (lane == 0) {
          ws.f.bound[d] = nb;
          ws.f.cur[d + 1] = nb;
        }
        __syncwarp();
        adv = true;
      }
    } else if (s.kind == kStepCheck) {
      const uint32_t target = ws.f.bound[ws.prog.hist_step[s.hist]];
      if (next_check<W, kEnum>(g, st, ws, d, cur, target)) {
        __syncwarp();
        if (lane == 0) ws.f.cur[d + 1] = cur;
        __syncwarp();
        adv = true;
      }
    } else {  // kStepMove
      if (ws.f.mask[d] == 0) {
        const uint32_t back = ws.f.bound[ws.prog.hist_step[s.hist]];
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
      if (d < n_steps) {
        if (ws.prog.steps[d].kind == kStepMove) {
          __syncwarp();
          if (lane == 0) ws.f.mask[d] = 0;
          __syncwarp();
        } else {
          frame_enter<W, kEnum>(g, ws, d);
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
  uint32_t* d = reinterpret_cast<uint32_t*>(&ws.prog);
  __syncwarp();
  for (int i = lane_id(); i < static_cast<int>(sizeof(WalkProgram) / 4); i += 32) d[i] = s[i];
  __syncwarp();
}

__device__ __forceinline__ uint32_t next_epoch(WarpMemo& m) {
  ++m.epoch;
  if (m.epoch == 0) {
    // 2^32 walks on this warp: wipe the tables once and restart at 1.
    for (uint32_t i = lane_id(); i < m.edge_cap; i += 32) m.edge[i] = make_uint4(0, 0, 0, 0);
    for (uint64_t i = lane_id(); i < static_cast<uint64_t>(m.hyp_cap) * m.hyp_stride; i += 32) m.hyp[i] = 0;
    __syncwarp();
    m.epoch = 1;
  }
  m.edge_n = 0;
  m.hyp_n = 0;
  return m.epoch;
}

template <class W>
__global__ void __launch_bounds__(kWalkWarps * 32) k_walk(DevGraph g, DevState<W> st, WalkLaunch w, WalkScratch sc,
                                                          StepCounters* ctr) {
  __shared__ WarpShared s_ws[kWalkWarps];
  const unsigned lane = lane_id();
  const unsigned wib = threadIdx.x >> 5;
  WarpShared& ws = s_ws[wib];
  const uint32_t gw = blockIdx.x * kWalkWarps + wib;
  WarpMemo m;
  m.edge = sc.edge_tab + static_cast<uint64_t>(gw) * sc.edge_cap;
  m.hyp = sc.hyp_tab + static_cast<uint64_t>(gw) * sc.hyp_cap * sc.hyp_stride;
  m.edge_cap = sc.edge_cap;
  m.hyp_cap = sc.hyp_cap;
  m.hyp_stride = sc.hyp_stride;
  m.epoch = sc.epochs[gw];
  m.edge_n = m.hyp_n = 0;
  const uint64_t n_items = w.retry_items ? w.n_retry : static_cast<uint64_t>(w.n_wl) * w.n_progs;
  int cached = -1;
  unsigned long long overflow = 0;
  while (true) {
    unsigned long long gi = 0;
    if (lane == 0) gi = atomicAdd(&ctr->items, 1ull);
    gi = __shfl_sync(kFull, gi, 0);
    if (gi >= n_items) break;
    uint32_t item, r, pos;
    if (w.retry_items) {
      item = w.retry_items[gi];
      pos = item / w.n_progs;
      r = item % w.n_progs;
    } else {
      r = static_cast<uint32_t>(gi / w.n_wl);
      pos = static_cast<uint32_t>(gi % w.n_wl);
      item = pos * w.n_progs + r;
    }
    if (static_cast<int>(r) != cached) {
      load_program(ws, w.progs + r);
      cached = static_cast<int>(r);
    }
    const uint32_t v = w.wl[pos];
    if (!role_of(st, v, ws.prog.start_role)) {
      if (lane == 0) w.status[item] = kItemSkip;
      continue;
    }
    next_epoch(m);
    unsigned long long unused = 0;
    const uint8_t res = run_walk<W, false>(g, st, ws, m, v, &unused);
    if (lane == 0) w.status[item] = res;
    if (res == kItemOverflow) ++overflow;
    if (res == kItemSuccess && (w.min_marker || w.marks)) {
      // alreadyMatched marks of the successful path (cc :64, pc :42, tds :74).
      uint32_t j = 0;
      for (int d0 = 1; d0 < ws.prog.n_steps; d0 += 32) {
        const int d = d0 + static_cast<int>(lane);
        const bool mk = d < ws.prog.n_steps && ws.prog.steps[d].mark;
        const unsigned mm = __ballot_sync(kFull, mk);
        if (mk) {
          const uint32_t x = ws.f.bound[d];
          const uint32_t slot = j + __popc(mm & ((1u << lane) - 1));
          if (w.marks) w.marks[static_cast<uint64_t>(item) * w.marks_stride + slot] = x;
          if (w.min_marker) {
            const uint8_t ri = w.role_index[ws.prog.steps[d].role];
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

template <class W>
__global__ void __launch_bounds__(kWalkWarps * 32) k_enumerate(DevGraph g, DevState<W> st,
                                                               const WalkProgram* __restrict__ prog,
                                                               const uint32_t* __restrict__ wl, uint32_t n_wl,
                                                               StepCounters* ctr) {
  __shared__ WarpShared s_ws[kWalkWarps];
  const unsigned lane = lane_id();
  WarpShared& ws = s_ws[threadIdx.x >> 5];
  load_program(ws, prog);
  WarpMemo m{};
  unsigned long long leaves = 0;
  while (true) {
    unsigned long long gi = 0;
    if (lane == 0) gi = atomicAdd(&ctr->items, 1ull);
    gi = __shfl_sync(kFull, gi, 0);
    if (gi >= n_wl) break;
    run_walk<W, true>(g, st, ws, m, wl[gi], &leaves);
  }
  if (lane == 0 && leaves) atomicAdd(&ctr->enumeration, leaves);
}

template <class W>
DevState<W> state_of(const QueryDevPtrs& q) {
  return DevState<W>{static_cast<W*>(q.vs), q.eact, q.mod, q.sch, static_cast<W*>(q.unm)};
}

#define PM_DISPATCH_WORD(kind, ...) \
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

uint32_t walk_grid_blocks(uint32_t n_warps_available) {
  uint32_t blocks = static_cast<uint32_t>(device_sm_count()) * 12;
  if (blocks * kWalkWarps > n_warps_available) blocks = n_warps_available / kWalkWarps;
  return blocks ? blocks : 1;
}

void launch_walk(const DevGraph& g, const QueryDevPtrs& q, const WalkLaunch& w, const WalkScratch& sc,
                 cudaStream_t s) {
  const uint32_t blocks = walk_grid_blocks(sc.n_warps);
  PM_DISPATCH_WORD(q.word_kind, k_walk<W><<<blocks, kWalkWarps * 32, 0, s>>>(g, state_of<W>(q), w, sc, q.ctr));
}

void launch_flag_rescue(const WalkLaunch& w, StepCounters* ctr, cudaStream_t s) {
  const uint64_t n = static_cast<uint64_t>(w.n_wl) * w.n_progs;
  const int grid = device_sm_count() * 4;
  k_flag_rescue<<<grid, 256, 0, s>>>(w.status, w.min_marker, n, ctr);
}

void launch_collect_overflow(const WalkLaunch& w, uint32_t* list, StepCounters* ctr, cudaStream_t s) {
  const uint64_t n = static_cast<uint64_t>(w.n_wl) * w.n_progs;
  const int grid = device_sm_count() * 4;
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

void launch_enumerate(const DevGraph& g, const QueryDevPtrs& q, const WalkProgram* prog, const uint32_t* wl,
                      uint32_t n_wl, cudaStream_t s) {
  const int blocks = device_sm_count() * 12;
  PM_DISPATCH_WORD(q.word_kind,
                   k_enumerate<W><<<blocks, kWalkWarps * 32, 0, s>>>(g, state_of<W>(q), prog, wl, n_wl, q.ctr));
}

}  // namespace pmgb
