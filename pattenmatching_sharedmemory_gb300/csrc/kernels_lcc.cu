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

#include <atomic>

#include "kernels.h"

namespace pmgb {
namespace {

constexpr int kThreads = 256;
constexpr int kWarpsPerBlock = kThreads / 32;
constexpr unsigned kFull = 0xFFFFFFFFu;

int g_sm_count = 0;
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
  }
  const uint64_t words = (g.E + 31) / 32;
  for (uint64_t i = tid; i < words; i += stride) {
    uint64_t remaining = g.E - i * 32;
    st.eact[i] = remaining >= 32 ? 0xFFFFFFFFu : ((1u << remaining) - 1u);
  }
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
template <class W>
__global__ void __launch_bounds__(kThreads) k_lcc_check(DevGraph g, DevState<W> st, const QueryTables* __restrict__ qt,
                                                        StepCounters* ctr) {
  __shared__ uint64_t s_nbr[64];
  __shared__ uint64_t s_need[64];
  __shared__ uint8_t s_role_slot[64];
  __shared__ uint8_t s_req[64][64];
  const uint32_t k = qt->k;
  for (int i = threadIdx.x; i < 64; i += blockDim.x) {
    s_nbr[i] = qt->nbr_mask[i];
    s_need[i] = qt->req_slots[i];
    s_role_slot[i] = qt->role_slot[i];
  }
  for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x) s_req[i / 64][i % 64] = qt->req[i / 64][i % 64];
  __syncthreads();

  const unsigned lane = lane_id();
  const uint64_t warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t n_warps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  unsigned long long edge_elim = 0, newly_modified = 0;

  for (uint64_t tile = warp * 32; tile < g.V; tile += n_warps * 32) {
    const uint64_t v = tile + lane;
    bool work = false;
    if (v < g.V) work = st.sch[v] && Pack<W>::cand(st.vs[v]) != 0;
    unsigned wm = __ballot_sync(kFull, work);
    while (wm) {
      const unsigned j = __ffs(wm) - 1;
      wm &= wm - 1;
      const uint32_t u = static_cast<uint32_t>(tile + j);
      const W wu = st.vs[u];
      const uint64_t cu = Pack<W>::cand(wu);
      const uint32_t su = Pack<W>::slot(wu);
      // Union of the template neighbours of u's roles, and the label slots
      // any of u's roles needs counted.
      uint64_t ncs = 0, need = 0;
      for (uint32_t p = lane; p < k; p += 32)
        if (cu >> p & 1) {
          ncs |= s_nbr[p];
          need |= s_need[p];
        }
      ncs = warp_or64(ncs);
      need = warp_or64(need);

      uint32_t cnt_lo = 0, cnt_hi = 0;  // counts of slot `lane` and `lane+32`
      uint32_t elim_u = 0;
      const uint64_t beg = g.off[u], end = g.off[u + 1];
      for (uint64_t e0 = beg; e0 < end; e0 += 32) {
        const uint64_t e = e0 + lane;
        const bool act = e < end && edge_active(st.eact, e);
        W ww = Pack<W>::zero();
        if (act) ww = st.vs[g.adj[e]];
        const uint64_t cw = Pack<W>::cand(ww);
        const bool live = act && cw != 0;
        const bool poss = live && (cw & ncs) != 0;
        const unsigned em = __ballot_sync(kFull, live && !poss);
        if (em) {
          if (lane == 0) clear_edge_bits(st.eact, e0, em);
          elim_u += __popc(em);
        }
        const uint32_t sw = Pack<W>::slot(ww);
        uint64_t nd = need;
        while (nd) {
          const unsigned s = __ffsll(static_cast<long long>(nd)) - 1;
          nd &= nd - 1;
          const unsigned m = __ballot_sync(kFull, poss && sw == s);
          if (lane == (s & 31)) {
            if (s < 32)
              cnt_lo += __popc(m);
            else
              cnt_hi += __popc(m);
          }
        }
      }
      // Role p fails if its label differs from u's or a required
      // neighbour-label count is not met (lcc :79-100).
      const bool has_lo = lane < k && (cu >> lane & 1);
      const bool has_hi = lane + 32 < k && (cu >> (lane + 32) & 1);
      bool bad_lo = has_lo && s_role_slot[lane] != su;
      bool bad_hi = has_hi && s_role_slot[lane + 32] != su;
      uint64_t nd = need;
      while (nd) {
        const unsigned s = __ffsll(static_cast<long long>(nd)) - 1;
        nd &= nd - 1;
        const uint32_t c = __shfl_sync(kFull, s < 32 ? cnt_lo : cnt_hi, s & 31);
        if (has_lo && s_req[lane][s] > c) bad_lo = true;
        if (has_hi && s_req[lane + 32][s] > c) bad_hi = true;
      }
      const uint64_t tu = static_cast<uint64_t>(__ballot_sync(kFull, bad_lo)) |
                          (static_cast<uint64_t>(__ballot_sync(kFull, bad_hi)) << 32);
      if (lane == 0) {
        if (tu || elim_u) {
          if (!st.mod[u]) {
            st.mod[u] = 1;
            ++newly_modified;
          }
        }
        if (tu) st.unm[u] = Pack<W>::make(tu, 0);
        edge_elim += elim_u;
      }
    }
  }
  if (lane == 0) {
    if (edge_elim) atomicAdd(&ctr->edge_elim, edge_elim);
    if (newly_modified) atomicAdd(&ctr->modified_total, newly_modified);
  }
}

// ---- sweep 2 (LCC and NLCC) -------------------------------------------
template <class W>
__global__ void __launch_bounds__(kThreads) k_apply(DevGraph g, DevState<W> st, StepCounters* ctr) {
  const unsigned lane = lane_id();
  const uint64_t warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t n_warps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  const bool any_modified = *reinterpret_cast<volatile unsigned long long*>(&ctr->modified_total) != 0;
  unsigned me = 0, ve = 0;
  for (uint64_t tile = warp * 32; tile < g.V; tile += n_warps * 32) {
    const uint64_t v = tile + lane;
    bool scan = false;
    if (v < g.V) {
      const W w = st.vs[v];
      const uint64_t c = Pack<W>::cand(w);
      if (c) {
        if (st.mod[v]) {
          const uint64_t tu = Pack<W>::cand(st.unm[v]);
          if (tu) {
            me += __popcll(tu);
            const uint64_t nc = c & ~tu;
            st.vs[v] = Pack<W>::make(nc, Pack<W>::slot(w));
            if (!nc) ++ve;
            st.unm[v] = Pack<W>::zero();
          }
          st.sch[v] = 1;
        } else if (!any_modified) {
          st.sch[v] = 0;
        } else {
          const uint64_t b = g.off[v], e = g.off[v + 1];
          if (e - b <= 8) {
            // Short lists: the lane scans its own vertex.
            bool found = false;
            for (uint64_t x = b; x < e && !found; ++x)
              if (edge_active(st.eact, x) && st.mod[g.adj[x]]) found = true;
            st.sch[v] = found;
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
      const uint32_t u = static_cast<uint32_t>(tile + j);
      const uint64_t b = g.off[u], e = g.off[u + 1];
      bool found = false;
      for (uint64_t e0 = b; e0 < e && !found; e0 += 32) {
        const uint64_t x = e0 + lane;
        const bool hit = x < e && edge_active(st.eact, x) && st.mod[g.adj[x]];
        found = __any_sync(kFull, hit);
      }
      if (lane == j) st.sch[u] = found;
    }
  }
  me = __reduce_add_sync(kFull, me);
  ve = __reduce_add_sync(kFull, ve);
  if (lane == 0) {
    if (me) atomicAdd(&ctr->match_elim, static_cast<unsigned long long>(me));
    if (ve) atomicAdd(&ctr->vertex_elim, static_cast<unsigned long long>(ve));
  }
}

// ---- worklist compaction ----------------------------------------------
constexpr int kTileV = 4096;  // vertices per compaction block (256 threads x 16)

template <class W>
__device__ __forceinline__ bool in_worklist(const DevGraph& g, const DevState<W>& st, uint64_t v, uint64_t mask) {
  return v < g.V && (Pack<W>::cand(st.vs[v]) & mask) != 0;
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

template <class W>
DevState<W> state_of(const QueryDevPtrs& q) {
  return DevState<W>{static_cast<W*>(q.vs), q.eact, q.mod, q.sch, static_cast<W*>(q.unm)};
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

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

int device_sm_count() {
  if (g_sm_count == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (g_sm_count <= 0) g_sm_count = 1;
  }
  return g_sm_count;
}

void launch_init_state(const DevGraph& g, const QueryDevPtrs& q, const uint8_t* d2s, uint64_t full, cudaStream_t s) {
  const int grid = device_sm_count() * 8;
  PM_DISPATCH_WORD(q.word_kind, k_init_state<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), d2s, full));
}

void launch_lcc0(const DevGraph& g, const QueryDevPtrs& q, cudaStream_t s) {
  const int grid = device_sm_count() * 8;
  PM_DISPATCH_WORD(q.word_kind, k_lcc0<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), q.tables, q.ctr));
}

void launch_lcc_check(const DevGraph& g, const QueryDevPtrs& q, cudaStream_t s) {
  const int grid = grid_for_tiles(g.V, 8);
  PM_DISPATCH_WORD(q.word_kind, k_lcc_check<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), q.tables, q.ctr));
}

void launch_apply(const DevGraph& g, const QueryDevPtrs& q, cudaStream_t s) {
  const int grid = grid_for_tiles(g.V, 8);
  PM_DISPATCH_WORD(q.word_kind, k_apply<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), q.ctr));
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

void launch_export(const DevGraph& g, const QueryDevPtrs& q, uint64_t* cand, uint8_t* vact, uint8_t* eact_bytes,
                   cudaStream_t s) {
  const int grid = device_sm_count() * 8;
  PM_DISPATCH_WORD(q.word_kind, k_export<W><<<grid, kThreads, 0, s>>>(g, state_of<W>(q), cand, vact, eact_bytes));
}

}  // namespace pmgb
