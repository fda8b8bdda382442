// Host engine: device residency, step orchestration, output writers.
#include <nvtx3/nvToolsExt.h>

#include "engine.h"

#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <exception>
#include <mutex>
#include <thread>

#include "totem_io.h"

namespace pmgb {

void throw_cuda(cudaError_t e, const char* what) {
  const int code = (e == cudaErrorMemoryAllocation) ? PM_E_OOM
                   : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? PM_E_NO_DEVICE
                                                                                 : PM_E_DEVICE;
  throw PmError{code, std::string(what) + ": " + cudaGetErrorString(e)};
}

void DeviceBuffer::release() {
  if (ptr) {
    if (ordered)
      cudaFreeAsync(ptr, stream);
    else
      cudaFree(ptr);
  }
  ptr = nullptr;
  bytes = 0;
}

namespace {
// Host-side fault injection (pm_debug_fail_device_alloc_after): counts down
// the library's device allocations; the one that reaches zero fails as an
// out-of-memory cudaMalloc would.  -1 = off.
std::atomic<int64_t> g_fail_alloc_countdown{-1};
}  // namespace
void set_fail_alloc_after(int64_t n) { g_fail_alloc_countdown.store(n < 0 ? -1 : n); }

void DeviceBuffer::ensure(size_t n) {
  if (n <= bytes && ptr) return;
  release();
  if (n == 0) n = 16;
  int64_t left = g_fail_alloc_countdown.load();
  while (left >= 0 && !g_fail_alloc_countdown.compare_exchange_weak(left, left - 1)) {
  }
  if (left == 0) throw_cuda(cudaErrorMemoryAllocation, "injected device allocation failure");
  if (ordered)
    PM_CUDA(cudaMallocAsync(&ptr, n, stream));
  else
    PM_CUDA(cudaMalloc(&ptr, n));
  bytes = n;
}

// ---- graph ------------------------------------------------------------------
void parallel_ranges(uint64_t n, const std::function<void(uint64_t, uint64_t)>& f) {
  const unsigned hw = std::thread::hardware_concurrency();
  const uint64_t T = std::min<uint64_t>(std::max(1u, hw), 32);
  if (T == 1 || n < (uint64_t(1) << 16)) {
    f(0, n);
    return;
  }
  std::vector<std::thread> ts;
  std::exception_ptr err;
  std::mutex mu;
  for (uint64_t t = 0; t < T; ++t) {
    const uint64_t lo = n * t / T, hi = n * (t + 1) / T;
    ts.emplace_back([&, lo, hi] {
      try {
        f(lo, hi);
      } catch (...) {
        std::lock_guard<std::mutex> lock(mu);
        if (!err) err = std::current_exception();
      }
    });
  }
  for (auto& t : ts) t.join();
  if (err) std::rethrow_exception(err);
}

CsrScan scan_csr(const uint64_t* offsets, const uint32_t* adj, uint32_t vertex_count) {
  std::atomic<bool> mono{true}, range{true}, sorted{true};
  parallel_ranges(vertex_count, [&](uint64_t lo, uint64_t hi) {
    bool m = true, r = true, so = true;
    for (uint64_t v = lo; v < hi; ++v) {
      const uint64_t b = offsets[v], e = offsets[v + 1];
      if (b > e) {
        m = false;
        continue;
      }
      for (uint64_t x = b; x < e; ++x) {
        if (adj[x] >= vertex_count) r = false;
        if (x > b && adj[x - 1] >= adj[x]) so = false;
      }
    }
    if (!m) mono = false;
    if (!r) range = false;
    if (!so) sorted = false;
  });
  CsrScan c;
  c.monotone = mono;
  c.in_range = range;
  c.sorted_unique = sorted;
  return c;
}

void GraphImpl::finalize_host(const bool* sorted) {
  const uint32_t V = host.vertex_count;
  if (host.labels.size() != V) host.labels.assign(V, 0);
  // Dense ids: the rank of each label among the distinct values.  Labels
  // below 2^22 (the common case) go through a presence table, larger ones
  // through a sorted copy.
  label_t top = 0;
  for (uint32_t v = 0; v < V; ++v) top = std::max(top, host.labels[v]);
  dense_ids.resize(V);
  if (top < (label_t(1) << 22)) {
    std::vector<uint32_t> id(static_cast<size_t>(top) + 1, 0);
    for (uint32_t v = 0; v < V; ++v) id[host.labels[v]] = 1;
    dense_values.clear();
    for (size_t x = 0; x < id.size(); ++x)
      if (id[x]) {
        id[x] = static_cast<uint32_t>(dense_values.size());
        dense_values.push_back(static_cast<label_t>(x));
      }
    parallel_ranges(V, [&](uint64_t lo, uint64_t hi) {
      for (uint64_t v = lo; v < hi; ++v) dense_ids[v] = id[host.labels[v]];
    });
  } else {
    dense_values.assign(host.labels.begin(), host.labels.end());
    std::sort(dense_values.begin(), dense_values.end());
    dense_values.erase(std::unique(dense_values.begin(), dense_values.end()), dense_values.end());
    parallel_ranges(V, [&](uint64_t lo, uint64_t hi) {
      for (uint64_t v = lo; v < hi; ++v)
        dense_ids[v] = static_cast<uint32_t>(
            std::lower_bound(dense_values.begin(), dense_values.end(), host.labels[v]) - dense_values.begin());
    });
  }
  if (sorted) {
    sorted_unique = *sorted;
  } else {
    std::atomic<bool> ok{true};
    parallel_ranges(V, [&](uint64_t lo, uint64_t hi) {
      for (uint64_t v = lo; v < hi && ok.load(std::memory_order_relaxed); ++v)
        for (uint64_t e = host.offsets[v] + 1; e < host.offsets[v + 1]; ++e)
          if (host.adj[e - 1] >= host.adj[e]) {
            ok = false;
            break;
          }
    });
    sorted_unique = ok;
  }
}

void GraphImpl::to_device(int dev, const uint32_t* adj_src) {
  if (device == dev && d_off.ptr) return;
  if (!adj_src) adj_src = host.adj.data();
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    throw PmError{PM_E_NO_DEVICE, "no CUDA device available for the GB300 pruning kernels"};
  PM_CUDA(cudaSetDevice(dev));
  // Queries allocate stream-ordered from the device's default pool; keep
  // freed blocks in the pool for the next query instead of returning them.
  cudaMemPool_t mempool;
  if (cudaDeviceGetDefaultMemPool(&mempool, dev) == cudaSuccess) {
    uint64_t keep = ~uint64_t(0);
    cudaMemPoolSetAttribute(mempool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  const uint32_t V = host.vertex_count;
  d_off.ensure(sizeof(uint64_t) * (static_cast<size_t>(V) + 1));
  d_adj.ensure(sizeof(uint32_t) * std::max<uint64_t>(host.edge_count, 1));
  d_lab.ensure(sizeof(uint32_t) * std::max<uint32_t>(V, 1));
  PM_CUDA(cudaMemcpy(d_off.ptr, host.offsets.data(), sizeof(uint64_t) * (V + 1), cudaMemcpyHostToDevice));
  if (host.edge_count)
    PM_CUDA(cudaMemcpy(d_adj.ptr, adj_src, sizeof(uint32_t) * host.edge_count, cudaMemcpyHostToDevice));
  if (V) PM_CUDA(cudaMemcpy(d_lab.ptr, dense_ids.data(), sizeof(uint32_t) * V, cudaMemcpyHostToDevice));
  device = dev;
  if (host.edge_count && dense_values.size() <= 256) {
    // Padded to whole 32-entry words plus one: LCC's first pass reads it in
    // 16-byte loads that start below the edge count.
    d_nlab.ensure((host.edge_count + 31) / 32 * 32 + 32);
    launch_build_entry_labels(this->dev(), d_nlab.as<uint8_t>(), nullptr);
    PM_CUDA(cudaGetLastError());
    PM_CUDA(cudaDeviceSynchronize());
  }
  build_hub_plan(hub_degree, seg_entries);
  symmetric = false;
  if (sorted_unique && V) {
    unsigned long long* d_res = nullptr;
    unsigned long long res[3] = {0, 0, 0};
    PM_CUDA(cudaMalloc(&d_res, sizeof(res)));
    PM_CUDA(cudaMemset(d_res, 0, sizeof(res)));
    launch_check_symmetric(this->dev(), d_res, nullptr);
    const cudaError_t e = cudaMemcpy(res, d_res, sizeof(res), cudaMemcpyDeviceToHost);
    cudaFree(d_res);
    PM_CUDA(e);
    symmetric = res[0] == 0 && res[1] == res[2];
  }
  plan_epoch = next_plan_epoch();
}

void GraphImpl::build_hub_plan(uint32_t degree, uint32_t entries) {
  if (entries < 32 || entries > 1024 || (entries & (entries - 1)))
    throw PmError{PM_E_INVALID_ARG, "seg_entries must be a power of two in [32, 1024]"};
  // Light tiles stream at most 32 * hub_degree entries (32-bit stream index).
  if (degree > (1u << 26)) throw PmError{PM_E_INVALID_ARG, "hub_degree above 2^26"};
  // Segments of multi-segment hubs first (one sweep task each, in vertex
  // order; the accumulator index is the hub's rank), then the single-segment
  // hubs (batched 32 to a task) by degree, ties by vertex id, so the 32
  // lanes of a batch get lists of similar length.  Chunks of vertex ids are
  // scanned in parallel and concatenated in order; the single-segment hubs
  // (at most `entries` entries each) are ordered by a stable counting sort
  // on their degree.
  struct Part {
    uint64_t lo = 0;
    std::vector<uint4> seg;
    std::vector<uint32_t> single;
    uint32_t multi = 0;
  };
  std::vector<Part> parts;
  std::mutex parts_mu;
  const uint32_t V = host.vertex_count;
  const uint64_t* off = host.offsets.data();
  parallel_ranges(V, [&](uint64_t lo, uint64_t hi) {
    Part pt;
    pt.lo = lo;
    for (uint64_t v = lo; v < hi; ++v) {
      const uint64_t deg = off[v + 1] - off[v];
      if (deg <= degree) continue;
      if (deg <= entries) {
        pt.single.push_back(static_cast<uint32_t>(v));
        continue;
      }
      // Lists longer than `entries` are cut at multiples of it (see
      // DevGraph::seg).
      const uint64_t n = (off[v + 1] - 1) / entries - off[v] / entries + 1;
      for (uint64_t i = 0; i < n; ++i)
        pt.seg.push_back(make_uint4(static_cast<uint32_t>(v), static_cast<uint32_t>(i), static_cast<uint32_t>(n),
                                    pt.multi));
      ++pt.multi;
    }
    std::lock_guard<std::mutex> lk(parts_mu);
    parts.push_back(std::move(pt));
  });
  std::sort(parts.begin(), parts.end(), [](const Part& x, const Part& y) { return x.lo < y.lo; });
  size_t n_heavy_seg = 0, n_single = 0;
  for (const Part& pt : parts) {
    n_heavy_seg += pt.seg.size();
    n_single += pt.single.size();
  }
  if (n_heavy_seg + n_single > 0x7fffffffull) throw PmError{PM_E_INVALID_ARG, "too many hub segments"};
  std::vector<uint4> seg;
  seg.reserve(n_heavy_seg + n_single);
  uint32_t n_multi = 0;
  for (const Part& pt : parts) {
    for (uint4 sd : pt.seg) {
      sd.w += n_multi;
      seg.push_back(sd);
    }
    n_multi += pt.multi;
  }
  const uint32_t heavy = static_cast<uint32_t>(seg.size());
  std::vector<uint64_t> pos(static_cast<size_t>(entries) + 2, 0);
  for (const Part& pt : parts)
    for (uint32_t v : pt.single) ++pos[off[v + 1] - off[v] + 1];
  for (size_t d = 1; d < pos.size(); ++d) pos[d] += pos[d - 1];
  seg.resize(heavy + n_single);
  for (const Part& pt : parts)
    for (uint32_t v : pt.single) seg[heavy + pos[off[v + 1] - off[v]]++] = make_uint4(v, 0, 1, 0xFFFFFFFFu);
  d_seg.ensure(sizeof(uint4) * std::max<size_t>(seg.size(), 1));
  if (!seg.empty())
    PM_CUDA(cudaMemcpy(d_seg.ptr, seg.data(), sizeof(uint4) * seg.size(), cudaMemcpyHostToDevice));
  hub_degree = degree;
  seg_entries = entries;
  n_seg = static_cast<uint32_t>(seg.size());
  n_heavy = heavy;
  n_acc = n_multi;
  plan_epoch = next_plan_epoch();
}

DevGraph GraphImpl::dev() const {
  DevGraph g{host.vertex_count, host.edge_count, d_off.as<uint64_t>(), d_adj.as<uint32_t>(), d_lab.as<uint32_t>(),
             sorted_unique ? 1 : 0};
  g.hub_degree = hub_degree;
  g.seg_shift = static_cast<uint32_t>(__builtin_ctz(seg_entries));
  g.n_seg = n_seg;
  g.n_heavy = n_heavy;
  g.n_acc = n_acc;
  g.seg = d_seg.as<uint4>();
  g.symmetric = symmetric ? 1 : 0;
  g.nlab = d_nlab.as<uint8_t>();
  return g;
}

// ---- walker scratch --------------------------------------------------------
void WalkPool::ensure(uint32_t n_warps, uint32_t edge_cap, uint32_t hyp_cap, uint32_t hyp_stride, uint32_t state_cap,
                      uint32_t state_stride, cudaStream_t s) {
  if (edge.ptr && sc.n_warps == n_warps && sc.edge_cap == edge_cap && sc.hyp_cap == hyp_cap &&
      sc.hyp_stride == hyp_stride && sc.state_cap == state_cap && sc.state_stride == state_stride)
    return;
  edge.ensure(sizeof(uint4) * static_cast<size_t>(n_warps) * edge_cap);
  hyp.ensure(sizeof(uint32_t) * static_cast<size_t>(n_warps) * hyp_cap * hyp_stride);
  state.ensure(sizeof(uint32_t) * static_cast<size_t>(n_warps) * state_cap * state_stride);
  epochs.ensure(sizeof(uint32_t) * n_warps);
  // Epoch 0 marks every slot free; per-warp epochs start at 0 and walks use 1+.
  PM_CUDA(cudaMemsetAsync(edge.ptr, 0, edge.bytes, s));
  PM_CUDA(cudaMemsetAsync(hyp.ptr, 0, hyp.bytes, s));
  PM_CUDA(cudaMemsetAsync(state.ptr, 0, state.bytes, s));
  PM_CUDA(cudaMemsetAsync(epochs.ptr, 0, epochs.bytes, s));
  sc.edge_tab = edge.as<uint32_t>();
  sc.hyp_tab = hyp.as<uint32_t>();
  sc.state_tab = state.as<uint32_t>();
  sc.epochs = epochs.as<uint32_t>();
  sc.n_warps = n_warps;
  sc.edge_cap = edge_cap;
  sc.hyp_cap = hyp_cap;
  sc.hyp_stride = hyp_stride;
  sc.state_cap = state_cap;
  sc.state_stride = state_stride;
}

// ---- query ------------------------------------------------------------------
namespace {
// NVTX range around a step or a captured LCC fixpoint, so that a profiler's
// timeline shows the reference's schedule (no-ops when no tool is attached).
struct StepRange {
  explicit StepRange(const char* name) { nvtxRangePushA(name); }
  ~StepRange() { nvtxRangePop(); }
  StepRange(const StepRange&) = delete;
  StepRange& operator=(const StepRange&) = delete;
};

const char* step_label(int kind) {
  static const char* const kNames[] = {"START", "END", "LCC0", "LCC", "CC", "PC", "TDS", "ENUMERATION"};
  return kind >= 0 && kind <= PM_STEP_ENUMERATION ? kNames[kind] : "?";
}
}  // namespace

std::string step_name(int kind) {
  switch (kind) {
    case PM_STEP_START: return "START";
    case PM_STEP_END: return "END";
    case PM_STEP_LCC0: return "LCC0";
    case PM_STEP_LCC: return "LCC";
    case PM_STEP_CC: return "CC";
    case PM_STEP_PC: return "PC";
    case PM_STEP_TDS: return "TDS";
    case PM_STEP_ENUMERATION: return "ENUMERATION";
  }
  return "?";
}

PatternGraph load_pattern(const std::string& dir, bool load_labels) {
  // multiple_label_cpu.cc:37-47: pattern_edge.totem if present, else
  // pattern_edge; labels from pattern_vertex_data.
  std::string edge_path = dir + "pattern_edge.totem";
  if (!is_regular_file(edge_path)) edge_path = dir + "pattern_edge";
  HostGraph pg = read_totem_graph(edge_path);
  if (load_labels && is_regular_file(dir + "pattern_vertex_data")) read_vertex_labels(dir + "pattern_vertex_data", pg);
  PatternGraph p;
  p.n = pg.vertex_count;
  p.offsets.assign(pg.offsets.begin(), pg.offsets.end());
  p.adj.assign(pg.adj.begin(), pg.adj.end());
  if (pg.labels.empty())
    p.labels.assign(p.n, 0);
  else
    p.labels.assign(pg.labels.begin(), pg.labels.end());
  return p;
}

namespace {
DeviceConstraint make_device_constraint(CompiledConstraint cc) {
  DeviceConstraint dc;
  dc.cc = std::move(cc);
  for (const auto& p : dc.cc.programs) dc.start_roles.push_back(p.start_role);
  return dc;
}

uint32_t max_state_words(const std::vector<DeviceConstraint>& v) {
  uint32_t m = 0;
  for (const auto& dc : v) m = std::max<uint32_t>(m, dc.cc.max_state_words);
  return m;
}
}  // namespace

uint64_t estimate_query_bytes(const GraphImpl& g, uint32_t k) {
  const uint64_t V = g.host.vertex_count, E = g.host.edge_count;
  const uint64_t wb = word_bytes(word_kind_for(k));
  const uint64_t kk = std::min<uint64_t>(k, 64);
  // Walker pool of the first walk round: per warp the edge memo, a
  // hypothesis memo of (3 + stored vertices) words and a state memo of
  // (5 + key words) words per entry, both bounded through k.
  const uint64_t warps = static_cast<uint64_t>(walk_grid_blocks(1u << 30)) * kWalkWarpsPerBlock;
  const uint64_t state_entries = std::max<uint64_t>(walk_table_entries(), enum_table_entries());
  const uint64_t pool = warps * (16ull * kEdgeCapEntries + 4ull * kHypCapEntries * (3 + kk) +
                                 4ull * state_entries * (7 + kk));
  // state + per-step worklist/status/markers (items bounded by V * roles)
  return V * (2 * wb + 2) + ((E + 31) / 32) * 8 + V * 8 + V * kk * 5 +
         sizeof(HubAcc) * static_cast<uint64_t>(g.n_acc) + pool + (1 << 20);
}

QueryImpl::~QueryImpl() {
  // Stream-ordered frees go before the stream is destroyed.
  for (DeviceBuffer* b : buffers()) b->release();
  if (own_host) {
    if (h_ctr) cudaFreeHost(h_ctr);
    if (h_count) cudaFreeHost(h_count);
  }
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (ev_first) cudaEventDestroy(ev_first);
  if (own_stream && stream) cudaStreamDestroy(stream);
}

QueryDevPtrs QueryImpl::ptrs() const {
  const uint32_t first = lcc_first_pending && g->d_nlab.ptr && lcc_label_stream() ? 1u : 0u;
  return QueryDevPtrs{word_kind, d_vs.ptr, d_eact.as<uint32_t>(), d_mod.as<uint8_t>(), d_sch.as<uint8_t>(),
                      d_unm.ptr, d_ctr.as<StepCounters>(), d_tables.as<QueryTables>(), d_hub_acc.as<HubAcc>(),
                      d_lt.as<uint32_t>(), d_tile_sch.as<uint8_t>(), first};
}

uint64_t QueryImpl::device_bytes() const {
  return d_vs.bytes + d_eact.bytes + d_lt.bytes + d_tile_sch.bytes + d_mod.bytes + d_sch.bytes + d_unm.bytes + d_ctr.bytes + d_tables.bytes +
         d_d2s.bytes + d_hub_acc.bytes + d_progs.bytes + d_start_roles.bytes + d_role_index.bytes + d_wl.bytes + d_wl_index.bytes +
         d_blocks.bytes + d_count.bytes + d_status.bytes + d_marker.bytes + d_marks.bytes + d_list.bytes + d_slices.bytes +
         d_slice_tiles.bytes + d_item_scratch.bytes +
         pool.bytes() + big_pool.bytes();
}

std::vector<DeviceBuffer*> QueryImpl::buffers() {
  return {&d_vs,          &d_eact,      &d_lt,        &d_mod,       &d_sch,        &d_unm,         &d_ctr,
          &d_tile_sch,
          &d_tables,      &d_d2s,       &d_hub_acc,   &d_progs,     &d_start_roles, &d_role_index,  &d_wl,
          &d_wl_index,    &d_blocks,    &d_count,     &d_status,    &d_marker,     &d_marks,       &d_list,
          &d_list2,       &d_apply_v,   &d_apply_r,   &d_slices,    &d_slice_tiles, &d_item_scratch, &pool.edge,
          &pool.hyp,      &pool.state,
          &pool.epochs,
          &big_pool.edge, &big_pool.hyp, &big_pool.state, &big_pool.epochs, &d_stat, &d_stat_tab};
}

void QueryImpl::create(GraphImpl* graph, const PatternGraph& p, cudaStream_t s, StepCounters* ext_ctr,
                       uint32_t* ext_count) {
  g = graph;
  pattern = p;
  k = p.n;
  qc = compile_constraints(p);
  for (const auto& c : qc.cycles)
    cycles.push_back(make_device_constraint(compile_cycle(c, p.labels, nlcc_variant)));
  for (const auto& pc : qc.paths) paths.push_back(make_device_constraint(compile_path(pc, p.labels, nlcc_variant)));
  for (const auto& t : qc.templates)
    templates.push_back(make_device_constraint(compile_template(t, p.labels, nlcc_variant)));
  enumeration = make_device_constraint(compile_enumeration(qc.enumeration, p.labels));
  word_kind = word_kind_for(k);

  // Label slots: the pattern's distinct labels in order of first use.
  std::vector<label_t> slot_labels;
  for (uint32_t v = 0; v < k; ++v)
    if (std::find(slot_labels.begin(), slot_labels.end(), p.labels[v]) == slot_labels.end())
      slot_labels.push_back(p.labels[v]);
  auto slot_of = [&](label_t l) -> int {
    auto it = std::find(slot_labels.begin(), slot_labels.end(), l);
    return it == slot_labels.end() ? 0xFF : static_cast<int>(it - slot_labels.begin());
  };
  memset(&tables, 0, sizeof(tables));
  tables.k = k;
  tables.n_slots = static_cast<uint32_t>(slot_labels.size());
  for (uint32_t r = 0; r < k; ++r) {
    const LocalConstraint& lc = qc.local[r];
    tables.role_slot[r] = static_cast<uint8_t>(slot_of(lc.origin_label));
    tables.nbr_mask[r] = lc.neighbor_mask;
    for (const auto& kv : lc.required) {
      int sl = slot_of(kv.first);
      tables.req[r][sl] = static_cast<uint8_t>(std::min<size_t>(kv.second, 255));
      tables.req_slots[r] |= uint64_t(1) << sl;
    }
    tables.slot_roles[tables.role_slot[r]] |= uint64_t(1) << r;
  }
  dense_to_slot.resize(std::max<size_t>(g->dense_values.size(), 1), 0xFF);
  for (size_t i = 0; i < g->dense_values.size(); ++i) dense_to_slot[i] = static_cast<uint8_t>(slot_of(g->dense_values[i]));
  for (size_t i = 0; i < 256; ++i) tables.dense_slot[i] = i < dense_to_slot.size() ? dense_to_slot[i] : 0xFF;

  if (s) {
    stream = s;
  } else {
    PM_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    own_stream = true;
  }
  for (DeviceBuffer* b : buffers()) {
    b->stream = stream;
    b->ordered = true;
  }
  PM_CUDA(cudaEventCreate(&ev0));
  PM_CUDA(cudaEventCreate(&ev1));
  PM_CUDA(cudaEventCreate(&ev_first));
  if (ext_ctr && ext_count) {
    h_ctr = ext_ctr;
    h_count = ext_count;
    own_host = false;
  } else {
    PM_CUDA(cudaMallocHost(&h_ctr, sizeof(StepCounters)));
    PM_CUDA(cudaMallocHost(&h_count, sizeof(uint32_t)));
  }

  const uint64_t V = g->host.vertex_count, E = g->host.edge_count;
  const size_t wb = word_bytes(word_kind);
  d_vs.ensure(wb * std::max<uint64_t>(V, 1));
  d_unm.ensure(wb * std::max<uint64_t>(V, 1));
  d_eact.ensure(4 * std::max<uint64_t>((E + 31) / 32, 1));
  d_lt.ensure(4 * std::max<uint64_t>((E + 31) / 32, 1));
  d_mod.ensure(std::max<uint64_t>(V, 1));
  d_sch.ensure(std::max<uint64_t>(V, 1));
  d_tile_sch.ensure(std::max<uint64_t>((V + 31) / 32, 1));
  d_ctr.ensure(sizeof(StepCounters));
  d_tables.ensure(sizeof(QueryTables));
  d_d2s.ensure(dense_to_slot.size());
  d_wl.ensure(4 * std::max<uint64_t>(V, 1));
  d_wl_index.ensure(4 * std::max<uint64_t>(V, 1));
  d_blocks.ensure(4 * ((V + 4095) / 4096 + 2));
  d_count.ensure(4);
  d_hub_acc.ensure(sizeof(HubAcc) * std::max<uint32_t>(g->n_acc, 1));
  PM_CUDA(cudaMemsetAsync(d_hub_acc.ptr, 0, d_hub_acc.bytes, stream));
  PM_CUDA(cudaMemsetAsync(d_ctr.ptr, 0, sizeof(StepCounters), stream));
  PM_CUDA(cudaMemcpyAsync(d_tables.ptr, &tables, sizeof(tables), cudaMemcpyHostToDevice, stream));
  PM_CUDA(cudaMemcpyAsync(d_d2s.ptr, dense_to_slot.data(), dense_to_slot.size(), cudaMemcpyHostToDevice, stream));

  // Every walk program of the query in one device array.
  std::vector<WalkProgram> progs;
  std::vector<uint8_t> start_roles, role_index;
  size_t row = 0;
  auto add = [&](DeviceConstraint& dc) {
    dc.prog_offset = progs.size();
    dc.role_row = row++;
    progs.insert(progs.end(), dc.cc.programs.begin(), dc.cc.programs.end());
    start_roles.insert(start_roles.end(), dc.start_roles.begin(), dc.start_roles.end());
    role_index.insert(role_index.end(), dc.cc.role_index, dc.cc.role_index + 64);
  };
  for (auto& dc : cycles) add(dc);
  for (auto& dc : paths) add(dc);
  for (auto& dc : templates) add(dc);
  add(enumeration);
  d_progs.ensure(sizeof(WalkProgram) * progs.size());
  d_start_roles.ensure(start_roles.size());
  d_role_index.ensure(role_index.size());
  PM_CUDA(cudaMemcpyAsync(d_progs.ptr, progs.data(), sizeof(WalkProgram) * progs.size(), cudaMemcpyHostToDevice,
                          stream));
  PM_CUDA(cudaMemcpyAsync(d_start_roles.ptr, start_roles.data(), start_roles.size(), cudaMemcpyHostToDevice, stream));
  PM_CUDA(cudaMemcpyAsync(d_role_index.ptr, role_index.data(), role_index.size(), cudaMemcpyHostToDevice, stream));

  const uint64_t full = k >= 64 ? ~uint64_t(0) : ((uint64_t(1) << k) - 1);
  launch_init_state(g->dev(), ptrs(), d_d2s.as<uint8_t>(), full, stream);
  PM_CUDA(cudaGetLastError());
  PM_CUDA(cudaStreamSynchronize(stream));
  active_vertices = V;
  active_edges = E;
  for (size_t i = 0; i < cycles.size(); ++i) rem_cc.push_back(i);
  for (size_t i = 0; i < paths.size(); ++i) rem_pc.push_back(i);
  for (size_t i = 0; i < templates.size(); ++i) rem_tds.push_back(i);
  if (order & PM_ORDER_EFFECTIVENESS) acc_max = accumulation_maximum(p);
  // The dynamic order's driver never sets its first step
  // (test_order_multiple_label_cpu.cc:128-130 call getNextStep only without
  // ORDER_USE_DYNAMIC): its first iteration runs nothing and logs a row with
  // an empty step name (START here), and LCC0 never runs.
  step = (order & PM_ORDER_EFFECTIVENESS) ? PM_STEP_START : advance(PM_STEP_START);
}

size_t QueryImpl::cc_index() const { return (order & PM_ORDER_EFFECTIVENESS) ? rem_cc[chosen] : next_cc; }
size_t QueryImpl::pc_index() const { return (order & PM_ORDER_EFFECTIVENESS) ? rem_pc[chosen] : next_pc; }
size_t QueryImpl::tds_index() const { return (order & PM_ORDER_EFFECTIVENESS) ? rem_tds[chosen] : next_tds; }

GraphStat QueryImpl::graph_stat(int threads) {
  if (acc_max.slots == 0) acc_max = accumulation_maximum(pattern);
  const uint32_t S = acc_max.slots, S1 = S + 1;
  const uint32_t T = static_cast<uint32_t>(std::max(threads > 0 ? threads : order_threads, 1));
  const uint64_t V = g->host.vertex_count;
  // Host tables: accumulation maxima (column S: 1 for labels without
  // template neighbours, whose accumulation the reference cannot look up)
  // and the largest maximum of each column.
  std::vector<uint8_t> max(static_cast<size_t>(S) * S1, 0);
  std::vector<uint32_t> thr(S1, 0);
  for (uint32_t a = 0; a < S; ++a) {
    for (uint32_t b = 0; b < S; ++b)
      max[a * S1 + b] = static_cast<uint8_t>(std::min<uint32_t>(acc_max.max[a * S + b], GraphStat::kMaxAtLeast - 1));
    max[a * S1 + S] = acc_max.has_a[a] ? 0 : 1;
    for (uint32_t b = 0; b < S1; ++b) thr[b] = std::max<uint32_t>(thr[b], max[a * S1 + b]);
  }
  const size_t n_vseg = static_cast<size_t>(T) * S, n_edges = static_cast<size_t>(S) * S,
               n_at = static_cast<size_t>(S) * S1 * 64;
  const size_t words = n_vseg + n_edges + n_at + 1;
  d_stat.ensure(8 * words);
  d_stat_tab.ensure(max.size() + 4 * thr.size() + 16);
  uint8_t* tab = d_stat_tab.as<uint8_t>();
  const size_t thr_off = (max.size() + 15) / 16 * 16;
  PM_CUDA(cudaMemsetAsync(d_stat.ptr, 0, 8 * words, stream));
  PM_CUDA(cudaMemcpyAsync(tab, max.data(), max.size(), cudaMemcpyHostToDevice, stream));
  PM_CUDA(cudaMemcpyAsync(tab + thr_off, thr.data(), 4 * thr.size(), cudaMemcpyHostToDevice, stream));
  unsigned long long* base = d_stat.as<unsigned long long>();
  GraphStatDev p{};
  p.slots = S;
  p.blocks = T;
  p.q = V / T;
  p.r = V % T;
  p.vseg = base;
  p.edges = base + n_vseg;
  p.at_least = base + n_vseg + n_edges;
  p.bad = base + n_vseg + n_edges + n_at;
  p.max = tab;
  p.thr = reinterpret_cast<const uint32_t*>(tab + thr_off);
  if (S) launch_graph_stat(g->dev(), ptrs(), p, stream);
  PM_CUDA(cudaGetLastError());
  std::vector<unsigned long long> h(words);
  PM_CUDA(cudaMemcpyAsync(h.data(), d_stat.ptr, 8 * words, cudaMemcpyDeviceToHost, stream));
  PM_CUDA(cudaStreamSynchronize(stream));
  if (h[words - 1]) throw_stat_missing("an active vertex carries no template label");
  GraphStat gs;
  gs.slots = S;
  gs.label_of_slot = acc_max.label_of_slot;
  gs.vertex_total.assign(S, 0);
  gs.edge_total.assign(h.begin() + n_vseg, h.begin() + n_vseg + n_edges);
  gs.edge_outbound.assign(S, 0);
  gs.at_least.assign(static_cast<size_t>(S) * S * GraphStat::kMaxAtLeast, 0);
  for (uint32_t t = 0; t < T; ++t)
    for (uint32_t a = 0; a < S; ++a) gs.vertex_total[a] += h[t * S + a];
  for (uint32_t a = 0; a < S; ++a) {
    for (uint32_t b = 0; b < S; ++b) gs.edge_outbound[a] += gs.edge_total[a * S + b];
    for (uint32_t b = 0; b < S; ++b)
      for (uint32_t i = 1; i < GraphStat::kMaxAtLeast; ++i)
        gs.at_least[(a * S + b) * GraphStat::kMaxAtLeast + i] = h[n_vseg + n_edges + (a * S1 + b) * 64 + i];
    // GraphStat::addAccumulation reads accumulationMaximumMap.at(a) as soon
    // as a label-a vertex's accumulation holds anything.
    if (!acc_max.has_a[a] && h[n_vseg + n_edges + (a * S1 + S) * 64 + 1])
      throw_stat_missing("accumulationMaximumMap has no entry for an active label");
  }
  return gs;
}

int QueryImpl::choose_dynamic() {
  const GraphStat gs = graph_stat();
  std::vector<const CycleConstraint*> cs;
  std::vector<const PathConstraint*> ps;
  std::vector<const TemplateConstraint*> ts;
  for (size_t i : rem_cc) cs.push_back(&qc.cycles[i]);
  for (size_t i : rem_pc) ps.push_back(&qc.paths[i]);
  for (size_t i : rem_tds) ts.push_back(&qc.templates[i]);
  const OrderChoice c = choose_next_constraint(gs, cs, ps, ts, qc.enumeration, order & PM_ORDER_ENUMERATE,
                                               order & PM_ORDER_EARLY_ENUMERATION, 0.01, std::max(order_threads, 1));
  chosen = c.index;
  return c.kind;
}

void QueryImpl::reset_modified() {
  PM_CUDA(cudaMemsetAsync(d_mod.ptr, 0, g->host.vertex_count ? g->host.vertex_count : 1, stream));
  PM_CUDA(cudaMemsetAsync(reinterpret_cast<char*>(d_ctr.ptr) + offsetof(StepCounters, modified_total), 0,
                          sizeof(unsigned long long), stream));
}

void QueryImpl::clear_step_counters() {
  PM_CUDA(cudaMemsetAsync(d_ctr.ptr, 0, sizeof(unsigned long long) * kStepCounterWords, stream));
}

void QueryImpl::read_counters() {
  PM_CUDA(cudaMemcpyAsync(h_ctr, d_ctr.ptr, sizeof(StepCounters), cudaMemcpyDeviceToHost, stream));
  PM_CUDA(cudaStreamSynchronize(stream));
  if (h_ctr->error == kDeviceErrorTimeout)
    throw PmError{PM_E_TIMEOUT, "the step's walkers exceeded their time budget of " +
                                    std::to_string(effective_walk_budget_ns() / 1000000) + " ms"};
  if (h_ctr->error) throw PmError{PM_E_DEVICE, "device-side error status " + std::to_string(h_ctr->error)};
}

StepResult QueryImpl::step_lcc0() {
  launch_lcc0(g->dev(), ptrs(), stream);
  PM_CUDA(cudaGetLastError());
  read_counters();
  lcc_first_pending = true;
  StepResult r;
  r.vertex = h_ctr->vertex_elim;
  r.match = h_ctr->match_elim;
  return r;
}

StepResult QueryImpl::step_lcc() {
  launch_lcc_check(g->dev(), ptrs(), stream);
  launch_apply(g->dev(), ptrs(), stream);
  lcc_first_pending = false;
  PM_CUDA(cudaGetLastError());
  read_counters();
  StepResult r;
  r.vertex = h_ctr->vertex_elim;
  r.edge = h_ctr->edge_elim;
  r.match = h_ctr->match_elim;
  return r;
}

uint32_t QueryImpl::build_worklist(uint64_t mask) {
  launch_worklist(g->dev(), ptrs(), mask, d_wl.as<uint32_t>(), d_wl_index.as<uint32_t>(), d_blocks.as<uint32_t>(),
                  d_count.as<uint32_t>(), stream);
  PM_CUDA(cudaGetLastError());
  PM_CUDA(cudaMemcpyAsync(h_count, d_count.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
  PM_CUDA(cudaStreamSynchronize(stream));
  return *h_count;
}

namespace {
constexpr uint32_t kEdgeCap = kEdgeCapEntries, kHypCap = kHypCapEntries, kStateCap = kStateCapEntries;
uint32_t g_walk_state_cap = 8192;  // CC/PC/TDS state-memo entries per warp, first round
uint32_t g_walk_presplit = 64;     // exact programs: first-hop entries per slice of a heavy item (0: off)
void zero_field(void* base, size_t offset, cudaStream_t s) {
  PM_CUDA(cudaMemsetAsync(static_cast<char*>(base) + offset, 0, sizeof(unsigned long long), s));
}
// Warps of retry round r (tables 8^r times larger): as many as fit a 6 GB
// scratch budget, at most half of the previous round's.
uint32_t retry_warps(uint32_t base_warps, int round, uint32_t hyp_stride, uint32_t state_stride) {
  const uint64_t per_warp = (uint64_t(16) * (1024ull << (3 * round))) + 4ull * hyp_stride * (1024ull << (3 * round)) +
                            4ull * state_stride * (2048ull << (3 * round));
  const uint64_t budget = 6ull << 30;
  uint64_t w = std::min<uint64_t>(base_warps >> round, budget / per_warp);
  w = std::max<uint64_t>(w, 32);
  return static_cast<uint32_t>(w / kWalkWarpsPerBlock * kWalkWarpsPerBlock);
}

uint32_t max_hyp_words(const std::vector<DeviceConstraint>& v) {
  uint32_t m = 0;
  for (const auto& dc : v) m = std::max<uint32_t>(m, dc.cc.max_hyp_words);
  return m;
}
}  // namespace

void set_walk_table_entries(uint32_t entries) { g_walk_state_cap = entries; }
void set_walk_presplit(uint32_t slice_entries) { g_walk_presplit = slice_entries; }
uint32_t walk_presplit() { return g_walk_presplit; }
uint32_t walk_table_entries() { return g_walk_state_cap; }

void QueryImpl::pool_strides(uint32_t* hyp_stride, uint32_t* state_stride) const {
  *hyp_stride = 3 + std::max<uint32_t>({max_hyp_words(cycles), max_hyp_words(paths), max_hyp_words(templates), 1u});
  *state_stride = 5 + std::max<uint32_t>({max_state_words(cycles), max_state_words(paths), max_state_words(templates),
                                          enumeration.cc.max_state_words, 1u});
}

void QueryImpl::ensure_pool() {
  uint32_t hs, ss;
  pool_strides(&hs, &ss);
  const uint32_t base_warps = walk_grid_blocks(1u << 30) * kWalkWarpsPerBlock;
  pool.ensure(base_warps, kEdgeCap, kHypCap, hs, g_walk_state_cap, ss, stream);
}

void QueryImpl::run_walks(const DeviceConstraint& dc, uint32_t n_wl, bool record_marks) {
  const uint32_t R = static_cast<uint32_t>(dc.cc.programs.size());
  const uint64_t n_items = static_cast<uint64_t>(n_wl) * R;
  if (n_items >= 0xFFFFFFFFull) throw PmError{PM_E_DEVICE, "too many walker items for 32-bit item ids"};
  d_status.ensure(std::max<uint64_t>(n_items, 1));
  d_marker.ensure(4 * std::max<uint64_t>(n_items, 1));
  const uint32_t M = std::max(1, dc.cc.marks_per_success);
  // Exact constraints cannot be rescued by alreadyMatched marks (see
  // walk_program.h), so they skip the mark bookkeeping entirely.
  const bool track_markers = !record_marks && !dc.cc.exact;
  if (record_marks) d_marks.ensure(4ull * std::max<uint64_t>(n_items, 1) * M);
  if (track_markers) PM_CUDA(cudaMemsetAsync(d_marker.ptr, 0xFF, 4 * n_items, stream));

  uint32_t hyp_stride, state_stride;
  pool_strides(&hyp_stride, &state_stride);
  const uint32_t base_warps = walk_grid_blocks(1u << 30) * kWalkWarpsPerBlock;
  ensure_pool();

  WalkLaunch w{};
  w.progs = d_progs.as<WalkProgram>() + dc.prog_offset;
  w.start_roles = d_start_roles.as<uint8_t>() + dc.prog_offset;
  w.n_progs = R;
  w.role_index = d_role_index.as<uint8_t>() + 64 * dc.role_row;
  w.wl = d_wl.as<uint32_t>();
  w.wl_index = d_wl_index.as<uint32_t>();
  w.n_wl = n_wl;
  w.status = d_status.as<uint8_t>();
  w.min_marker = track_markers ? d_marker.as<uint32_t>() : nullptr;
  w.marks = record_marks ? d_marks.as<uint32_t>() : nullptr;
  w.marks_stride = M;
  w.frame_steps = 1;
  for (const WalkProgram& pr : dc.cc.programs) w.frame_steps = std::max<uint32_t>(w.frame_steps, pr.n_steps + 1u);
  w.tail_swap = walk_tail_swap();
  w.tail_state_memo = walk_tail_state_memo() ? 1u : 0u;
  w.pair_tail = pair_tail_on(false) ? 1u : 0u;

  // Exact programs may split heavy items into first-hop slices: an item
  // succeeds when any slice does (no alreadyMatched marks to keep).
  bool sliced = dc.cc.exact && !record_marks && g_walk_presplit > 0 && g->sorted_unique;
  for (const WalkProgram& pr : dc.cc.programs)
    if (pr.n_steps < 2 || (pr.steps[1].kind != kStepVertex && pr.steps[1].kind != kStepFinal)) sliced = false;
  // The slices are listed on the device; only their number comes back.
  uint64_t n_slices = 0;
  if (sliced) {
    d_slice_tiles.ensure(8 * (static_cast<uint64_t>(n_wl) / 4096 + 2));
    unsigned long long* tiles = d_slice_tiles.as<unsigned long long>();
    unsigned long long* total = tiles + static_cast<uint64_t>(n_wl) / 4096 + 1;
    launch_slice_count(g->dev(), d_wl.as<uint32_t>(), n_wl, R, g_walk_presplit, tiles, total, stream);
    PM_CUDA(cudaGetLastError());
    unsigned long long total_h = 0;
    PM_CUDA(cudaMemcpyAsync(&total_h, total, sizeof(total_h), cudaMemcpyDeviceToHost, stream));
    PM_CUDA(cudaStreamSynchronize(stream));
    n_slices = total_h;
    if (n_slices >= 0xFFFFFFFFull) throw PmError{PM_E_DEVICE, "too many walker slices for 32-bit slice ids"};
    sliced = n_slices != 0;
  }
  zero_field(d_ctr.ptr, offsetof(StepCounters, items), stream);
  zero_field(d_ctr.ptr, offsetof(StepCounters, overflow), stream);
  if (sliced) {
    w.skip_deg = g_walk_presplit;
    w.prio = d_marker.as<uint32_t>();
    PM_CUDA(cudaMemsetAsync(d_marker.ptr, 0, 4 * n_items, stream));
  }
  launch_walk(g->dev(), ptrs(), w, pool.sc, stream);
  PM_CUDA(cudaGetLastError());
  if (sliced) {
    d_slices.ensure(sizeof(uint4) * n_slices);
    launch_slice_write(g->dev(), d_wl.as<uint32_t>(), n_wl, R, g_walk_presplit,
                       d_slice_tiles.as<unsigned long long>(), d_slices.as<uint4>(), stream);
    PM_CUDA(cudaGetLastError());
    WalkLaunch ws = w;
    ws.slices = d_slices.as<uint4>();
    ws.n_slices = static_cast<uint32_t>(n_slices);
    zero_field(d_ctr.ptr, offsetof(StepCounters, items), stream);
    launch_walk(g->dev(), ptrs(), ws, pool.sc, stream);
    PM_CUDA(cudaGetLastError());
    launch_prio_to_status(g->dev(), w, stream);
    PM_CUDA(cudaGetLastError());
    // Overflowed items (sliced ones included) are counted from the statuses.
    d_list.ensure(4 * std::max<uint64_t>(n_items, 1));
    zero_field(d_ctr.ptr, offsetof(StepCounters, aux), stream);
    launch_collect_overflow(w, d_list.as<uint32_t>(), d_ctr.as<StepCounters>(), stream);
  }
  read_counters();
  uint64_t overflow = sliced ? h_ctr->aux : h_ctr->overflow;
  w.skip_deg = 0;
  w.prio = nullptr;
  int round = 0;
  while (overflow) {
    ++round;
    ++overflow_retries;
    if (round > 6) throw PmError{PM_E_DEVICE, "walk memo tables exceed the retry limit"};
    d_list.ensure(4 * std::max<uint64_t>(n_items, 1));
    zero_field(d_ctr.ptr, offsetof(StepCounters, aux), stream);
    launch_collect_overflow(w, d_list.as<uint32_t>(), d_ctr.as<StepCounters>(), stream);
    read_counters();
    const uint32_t n_retry = static_cast<uint32_t>(h_ctr->aux);
    const uint32_t warps = retry_warps(base_warps, round, hyp_stride, state_stride * (g_walk_state_cap / kStateCap));
    big_pool.ensure(warps, kEdgeCap << (3 * round), kHypCap << (3 * round), hyp_stride, g_walk_state_cap << (3 * round),
                    state_stride, stream);
    WalkLaunch r = w;
    r.retry_items = d_list.as<uint32_t>();
    r.n_retry = n_retry;
    zero_field(d_ctr.ptr, offsetof(StepCounters, items), stream);
    zero_field(d_ctr.ptr, offsetof(StepCounters, overflow), stream);
    launch_walk(g->dev(), ptrs(), r, big_pool.sc, stream);
    PM_CUDA(cudaGetLastError());
    read_counters();
    overflow = h_ctr->overflow;
  }
}

// Exact emulation of the reference's sequential alreadyMatched shortcut
// (cc :105-108, pc :104-128, tds :163-166 run with one thread): items in
// order; an item marked by an earlier successful walk is skipped; a
// successful walk marks every (vertex, role) it bound; a failed one unmatches.
void QueryImpl::resolve_exact(const DeviceConstraint& dc, uint32_t n_wl) {
  ++exact_resolutions;
  run_walks(dc, n_wl, true);
  const uint32_t R = static_cast<uint32_t>(dc.cc.programs.size());
  const uint64_t n_items = static_cast<uint64_t>(n_wl) * R;
  const uint32_t M = std::max(1, dc.cc.marks_per_success);
  std::vector<uint8_t> status(n_items);
  std::vector<uint32_t> marks(n_items * M), wl(n_wl);
  PM_CUDA(cudaMemcpyAsync(status.data(), d_status.ptr, n_items, cudaMemcpyDeviceToHost, stream));
  PM_CUDA(cudaMemcpyAsync(marks.data(), d_marks.ptr, 4 * n_items * M, cudaMemcpyDeviceToHost, stream));
  PM_CUDA(cudaMemcpyAsync(wl.data(), d_wl.ptr, 4ull * n_wl, cudaMemcpyDeviceToHost, stream));
  PM_CUDA(cudaStreamSynchronize(stream));
  std::vector<uint8_t> marked(n_items, 0);
  std::vector<uint64_t> unmatch(n_wl, 0);
  for (uint64_t item = 0; item < n_items; ++item) {
    const uint8_t st = status[item];
    if (st == kItemSkip || marked[item]) continue;
    const uint32_t r = static_cast<uint32_t>(item % R);
    const WalkProgram& p = dc.cc.programs[r];
    if (st == kItemSuccess) {
      uint32_t j = 0;
      for (int d = 1; d < p.n_steps; ++d) {
        if (!p.steps[d].mark) continue;
        const uint32_t x = marks[item * M + j++];
        const uint8_t ri = dc.cc.role_index[p.steps[d].role];
        if (ri == 0xFF) continue;
        auto it = std::lower_bound(wl.begin(), wl.end(), x);
        if (it == wl.end() || *it != x) continue;
        marked[static_cast<uint64_t>(it - wl.begin()) * R + ri] = 1;
      }
    } else {
      unmatch[item / R] |= uint64_t(1) << p.start_role;
    }
  }
  std::vector<uint32_t> lv;
  std::vector<uint64_t> lr;
  for (uint32_t i = 0; i < n_wl; ++i)
    if (unmatch[i]) {
      lv.push_back(wl[i]);
      lr.push_back(unmatch[i]);
    }
  if (!lv.empty()) {
    d_apply_v.ensure(4 * lv.size());
    d_apply_r.ensure(8 * lr.size());
    PM_CUDA(cudaMemcpyAsync(d_apply_v.ptr, lv.data(), 4 * lv.size(), cudaMemcpyHostToDevice, stream));
    PM_CUDA(cudaMemcpyAsync(d_apply_r.ptr, lr.data(), 8 * lr.size(), cudaMemcpyHostToDevice, stream));
    launch_apply_unmatch_list(g->dev(), ptrs(), d_apply_v.as<uint32_t>(), d_apply_r.as<uint64_t>(),
                              static_cast<uint32_t>(lv.size()), stream);
    PM_CUDA(cudaGetLastError());
  }
}

StepResult QueryImpl::step_nlcc(const DeviceConstraint& dc) {
  const uint32_t n_wl = build_worklist(dc.cc.start_mask);
  if (n_wl) {
    run_walks(dc, n_wl, false);
    const uint32_t R = static_cast<uint32_t>(dc.cc.programs.size());
    WalkLaunch w{};
    w.status = d_status.as<uint8_t>();
    w.min_marker = d_marker.as<uint32_t>();
    w.n_wl = n_wl;
    w.n_progs = R;
    w.wl = d_wl.as<uint32_t>();
    w.start_roles = d_start_roles.as<uint8_t>() + dc.prog_offset;
    zero_field(d_ctr.ptr, offsetof(StepCounters, flagged), stream);
    if (!dc.cc.exact) {
      launch_flag_rescue(w, d_ctr.as<StepCounters>(), stream);
      read_counters();
    }
    if (dc.cc.exact || h_ctr->flagged == 0)
      launch_apply_failures(g->dev(), ptrs(), w, stream);
    else
      resolve_exact(dc, n_wl);
  }
  launch_apply(g->dev(), ptrs(), stream);
  PM_CUDA(cudaGetLastError());
  read_counters();
  StepResult r;
  r.vertex = h_ctr->vertex_elim;
  r.match = h_ctr->match_elim;
  return r;
}

namespace {
uint32_t g_enum_split_parts = 16;  // slices per split source (<= 1: never split)
uint32_t g_enum_split_after = 0;   // table growth levels before sources are split
uint32_t g_enum_state_cap = 8192;  // count-memo entries per warp, first round
// First-hop entries per slice of a heavy source (0: no up-front slicing),
// for programs with and without a count memo.
uint32_t g_enum_presplit_memo = 32;
uint32_t g_enum_presplit_plain = 8;
}  // namespace

void set_enum_presplit(uint32_t slice_entries) { g_enum_presplit_memo = g_enum_presplit_plain = slice_entries; }
void set_enum_presplit(bool count_memo, uint32_t slice_entries) {
  (count_memo ? g_enum_presplit_memo : g_enum_presplit_plain) = slice_entries;
}
uint32_t enum_presplit(bool count_memo) { return count_memo ? g_enum_presplit_memo : g_enum_presplit_plain; }

void set_enum_split(uint32_t parts, uint32_t after_levels) {
  g_enum_split_parts = parts;
  g_enum_split_after = after_levels;
}

void set_enum_table_entries(uint32_t entries) { g_enum_state_cap = entries; }
uint32_t enum_table_entries() { return g_enum_state_cap; }

// ENUMERATION (multiple_label_enumeration_cpu.tpp:39-118): every source of
// the first walk's start role, one warp each.  A source whose count memo
// overflows is re-run, either with tables 8x larger per growth level (the
// memo keeps reusing subtree counts across the source's first hops), or,
// once `after` growth levels were needed, split into slices of its first
// hop that separate warps take with base-size tables (parallel, but the
// slices do not share counts).  A slice is split once; after that it grows.
StepResult QueryImpl::step_enumeration() {
  const uint64_t kEnumSplit = g_enum_split_parts;
  const WalkProgram& p = enumeration.cc.programs[0];
  const uint32_t n_wl = build_worklist(uint64_t(1) << p.start_role);
  zero_field(d_ctr.ptr, offsetof(StepCounters, items), stream);
  if (n_wl) {
    {
      uint32_t hs0, ss0;
      pool_strides(&hs0, &ss0);
      pool.ensure(walk_grid_blocks(1u << 30) * kWalkWarpsPerBlock, kEdgeCap, kHypCap, hs0, g_enum_state_cap, ss0,
                  stream);
    }
    const WalkProgram* prog = d_progs.as<WalkProgram>() + enumeration.prog_offset;
    // Slicing the first hop is exact when that step binds a new vertex.
    const bool splittable =
        p.n_steps > 1 && (p.steps[1].kind == kStepVertex || p.steps[1].kind == kStepFinal);
    const auto& off = g->host.offsets;
    std::vector<uint4> over, items;
    zero_field(d_ctr.ptr, offsetof(StepCounters, aux), stream);
    const uint32_t presplit = enum_presplit(p.count_memo != 0);
    if (splittable && presplit) {
      // Sources with more first-hop entries than `presplit` start as slices
      // of that many entries, queued first (the longest work).  In sources
      // of more than s2 entries, a first-hop vertex whose list has more than
      // twice s2 entries takes its own items, one per s2-entry slice of its
      // list at the second hop (exact when the second step also binds a new
      // vertex; not when the tail starts at step 2, whose pair step at step
      // 1 would read whole lists).  The items are listed on the device
      // (launch_enum_item_count / _write); only their number comes back.
      const uint64_t s2 = enum_second_split();
      const bool second_ok = s2 && p.n_steps > 2 &&
                             (p.steps[2].kind == kStepVertex || p.steps[2].kind == kStepFinal) && p.tail_from != 3;
      const uint32_t s2_used = second_ok ? static_cast<uint32_t>(s2) : 0u;
      d_item_scratch.ensure(8 * enum_item_scratch_words(n_wl));
      unsigned long long* scratch = d_item_scratch.as<unsigned long long>();
      launch_enum_item_count(g->dev(), d_wl.as<uint32_t>(), n_wl, presplit, s2_used, scratch, stream);
      PM_CUDA(cudaGetLastError());
      unsigned long long totals[3] = {0, 0, 0};
      PM_CUDA(cudaMemcpyAsync(totals, enum_item_totals(scratch, n_wl), sizeof(totals), cudaMemcpyDeviceToHost,
                              stream));
      PM_CUDA(cudaStreamSynchronize(stream));
      const uint64_t n_items = totals[0] + totals[1];
      if (totals[2] || n_items >= 0xFFFFFFFFull)
        throw PmError{PM_E_DEVICE, "too many enumeration items for 32-bit item ids"};
      d_list.ensure(sizeof(uint4) * std::max<uint64_t>(n_items, 1));
      d_list2.ensure(sizeof(uint4) * std::max<uint64_t>(n_items, 1));
      launch_enum_item_write(g->dev(), d_wl.as<uint32_t>(), n_wl, presplit, s2_used, scratch, d_list.as<uint4>(),
                             stream);
      PM_CUDA(cudaGetLastError());
      launch_enumerate(g->dev(), ptrs(), prog, p.n_steps + 1u, d_wl.as<uint32_t>(), n_wl, d_list.as<uint4>(),
                       static_cast<uint32_t>(n_items), d_list2.as<uint4>(), pool.sc, stream);
    } else {
      d_list2.ensure(sizeof(uint4) * n_wl);
      launch_enumerate(g->dev(), ptrs(), prog, p.n_steps + 1u, d_wl.as<uint32_t>(), n_wl, nullptr, 0, d_list2.as<uint4>(), pool.sc,
                       stream);
    }
    PM_CUDA(cudaGetLastError());
    read_counters();
    uint32_t n_over = static_cast<uint32_t>(h_ctr->aux);
    uint32_t hs, ss;
    pool_strides(&hs, &ss);
    const uint32_t base_warps = walk_grid_blocks(1u << 30) * kWalkWarpsPerBlock;
    int grow_level = 0;
    for (int round = 1; n_over; ++round) {
      ++overflow_retries;
      if (round > 32) throw PmError{PM_E_DEVICE, "enumeration count memo exceeds the retry limit"};
      over.resize(n_over);
      PM_CUDA(cudaMemcpyAsync(over.data(), d_list2.ptr, sizeof(uint4) * n_over, cudaMemcpyDeviceToHost, stream));
      PM_CUDA(cudaStreamSynchronize(stream));
      // An overflow record is {position, lo, hi, source}; an item that was
      // split carries lo/hi inside the list, an unsplit one [0, 2^32).
      items.clear();
      size_t n_split = 0;
      auto split_now = [&](const uint4& it, uint64_t* lo, uint64_t* len) {
        const uint64_t deg = off[it.w + 1] - off[it.w];
        *lo = it.y;
        const uint64_t hi = std::min<uint64_t>(it.z, deg);
        *len = hi > *lo ? hi - *lo : 0;
        const bool unsplit = it.y == 0 && it.z == 0xFFFFFFFFu;
        return splittable && unsplit && kEnumSplit > 1 && *len > 1 &&
               static_cast<uint32_t>(grow_level) >= g_enum_split_after;
      };
      for (const uint4& it : over) {
        uint64_t lo, len;
        if (!split_now(it, &lo, &len)) continue;
        const uint64_t parts = std::min<uint64_t>(len, kEnumSplit);
        for (uint64_t k = 0; k < parts; ++k)
          items.push_back(make_uint4(it.x, static_cast<uint32_t>(lo + len * k / parts),
                                     static_cast<uint32_t>(lo + len * (k + 1) / parts), 0));
      }
      n_split = items.size();
      for (const uint4& it : over) {
        uint64_t lo, len;
        if (!split_now(it, &lo, &len)) items.push_back(make_uint4(it.x, it.y, it.z, 0));
      }
      const size_t n_grow = items.size() - n_split;
      d_list.ensure(sizeof(uint4) * items.size());
      d_list2.ensure(sizeof(uint4) * items.size());
      PM_CUDA(cudaMemcpyAsync(d_list.ptr, items.data(), sizeof(uint4) * items.size(), cudaMemcpyHostToDevice,
                              stream));
      zero_field(d_ctr.ptr, offsetof(StepCounters, aux), stream);
      if (n_split) {
        zero_field(d_ctr.ptr, offsetof(StepCounters, items), stream);
        launch_enumerate(g->dev(), ptrs(), prog, p.n_steps + 1u, d_wl.as<uint32_t>(), n_wl, d_list.as<uint4>(),
                         static_cast<uint32_t>(n_split), d_list2.as<uint4>(), pool.sc, stream);
        PM_CUDA(cudaGetLastError());
      }
      if (n_grow) {
        if (++grow_level > 6) throw PmError{PM_E_DEVICE, "enumeration count memo exceeds the retry limit"};
        const uint32_t warps = retry_warps(base_warps, grow_level, hs, ss * (g_enum_state_cap / kStateCap));
        big_pool.ensure(warps, kEdgeCap, kHypCap, hs, g_enum_state_cap << (3 * grow_level), ss, stream);
        zero_field(d_ctr.ptr, offsetof(StepCounters, items), stream);
        launch_enumerate(g->dev(), ptrs(), prog, p.n_steps + 1u, d_wl.as<uint32_t>(), n_wl, d_list.as<uint4>() + n_split,
                         static_cast<uint32_t>(n_grow), d_list2.as<uint4>(), big_pool.sc, stream);
        PM_CUDA(cudaGetLastError());
      }
      read_counters();
      n_over = static_cast<uint32_t>(h_ctr->aux);
    }
  }
  read_counters();
  StepResult r;
  r.enumeration = h_ctr->enumeration;
  return r;
}

int QueryImpl::advance(int cur) {
  if (order & PM_ORDER_EFFECTIVENESS) {
    // test_order_multiple_label_cpu.cc:177-300 (ORDER_USE_DYNAMIC).
    switch (cur) {
      case PM_STEP_START: return PM_STEP_LCC;
      case PM_STEP_LCC: return last.empty() ? choose_dynamic() : PM_STEP_LCC;
      case PM_STEP_CC: rem_cc.erase(rem_cc.begin() + chosen); return PM_STEP_LCC;
      case PM_STEP_PC: rem_pc.erase(rem_pc.begin() + chosen); return PM_STEP_LCC;
      case PM_STEP_TDS: rem_tds.erase(rem_tds.begin() + chosen); return PM_STEP_LCC;
      default: return PM_STEP_END;
    }
  }
  switch (cur) {
    case PM_STEP_START: return PM_STEP_LCC0;
    case PM_STEP_LCC0: return PM_STEP_LCC;
    case PM_STEP_LCC:
      if (!last.empty()) return PM_STEP_LCC;
      if (next_cc < cycles.size()) return PM_STEP_CC;
      if (next_pc < paths.size()) return PM_STEP_PC;
      if (next_tds < templates.size()) return PM_STEP_TDS;
      // The article drivers end their schedule here
      // (test_optimization_multiple_label_step.cc:46-58), the order drivers
      // built with USE_ENUMERATE count first (test_order_multiple_label_
      // step.cc:52-61).
      return nlcc_variant && !(order & PM_ORDER_ENUMERATE) ? PM_STEP_END : PM_STEP_ENUMERATION;
    case PM_STEP_CC: ++next_cc; return PM_STEP_LCC;
    case PM_STEP_PC: ++next_pc; return PM_STEP_LCC;
    case PM_STEP_TDS: ++next_tds; return PM_STEP_LCC;
    default: return PM_STEP_END;
  }
}

pm_step_record QueryImpl::run_step() {
  if (finished) return final_record();
  const int kind = step;
  const StepRange range(step_label(kind));
  // The dynamic order's first iteration runs no step.
  if (kind == PM_STEP_START) {
    append_record(StepResult{}, kind, 0.0, 0, 0);
    return records.back();
  }
  // No vertex holds a role: every step of the reference's schedule finds
  // nothing (its loops visit active vertices only, and ENUMERATION counts
  // 0), so the remaining rows are produced without touching the device.
  if (active_vertices == 0) {
    append_record(StepResult{}, kind, 0.0, 0, 0);
    return records.back();
  }
  if (kind == PM_STEP_CC || kind == PM_STEP_PC || kind == PM_STEP_TDS) reset_modified();
  ensure_hub_acc();
  clear_step_counters();
  PM_CUDA(cudaEventRecord(ev0, stream));
  if (!first_recorded) {
    PM_CUDA(cudaEventRecord(ev_first, stream));
    first_recorded = true;
  }
  StepResult r;
  try {
    switch (kind) {
      case PM_STEP_LCC0: r = step_lcc0(); break;
      case PM_STEP_LCC: r = step_lcc(); break;
      case PM_STEP_CC: r = step_nlcc(cycles[cc_index()]); break;
      case PM_STEP_PC: r = step_nlcc(paths[pc_index()]); break;
      // The reference's TDS step never advances its constraint iterator
      // (multiple_label_tds_cpu.tpp:136-244, unlike cc :180 and pc :186):
      // each of the n_template TDS steps checks template constraint 0.
      // The article drivers' TDS steps do advance (tds_strict_cpu.tpp:192).
      case PM_STEP_TDS: r = step_nlcc(templates[nlcc_variant ? tds_index() : 0]); break;
      case PM_STEP_ENUMERATION: r = step_enumeration(); break;
      default: break;
    }
  } catch (const PmError& e) {
    if (e.code == PM_E_TIMEOUT) {
      // The walkers' counters were read when the deadline was seen.
      float ms = 0;
      if (cudaEventRecord(ev1, stream) == cudaSuccess && cudaEventSynchronize(ev1) == cudaSuccess)
        cudaEventElapsedTime(&ms, ev0, ev1);
      aborted_kind = kind;
      aborted_ms = ms;
      aborted_scanned = h_ctr->scanned;
      aborted_hops = h_ctr->descents;
    }
    throw;
  }
  PM_CUDA(cudaEventRecord(ev1, stream));
  PM_CUDA(cudaEventSynchronize(ev1));
  float ms = 0;
  PM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
  append_record(r, kind, ms, h_ctr->scanned, kind == PM_STEP_LCC ? h_ctr->gathered : h_ctr->descents);
  return records.back();
}

void QueryImpl::ensure_hub_acc() {
  // The graph's hub plan may have changed since the last step.
  if (d_hub_acc.bytes < sizeof(HubAcc) * static_cast<size_t>(g->n_acc)) {
    d_hub_acc.ensure(sizeof(HubAcc) * static_cast<size_t>(g->n_acc));
    PM_CUDA(cudaMemsetAsync(d_hub_acc.ptr, 0, d_hub_acc.bytes, stream));
  }
}

void QueryImpl::append_record(const StepResult& r_in, int kind, double ms, uint64_t scanned, uint64_t second) {
  pm_step_record rec{};
  StepResult r = r_in;
  r.kind = kind;
  last = r;
  active_vertices -= r.vertex;
  active_edges -= r.edge;
  if (kind == PM_STEP_ENUMERATION) match_count = r.enumeration;
  total_ms += ms;
  rec.iteration = iteration;
  rec.step = kind;
  rec.step_ms = ms;
  rec.cumulative_ms = total_ms;
  rec.results.vertex_eliminated = r.vertex;
  rec.results.edge_eliminated = r.edge;
  rec.results.match_eliminated = r.match;
  rec.results.enumeration = r.enumeration;
  rec.active_vertex = active_vertices;
  rec.total_vertex = g->host.vertex_count;
  rec.active_edge = active_edges;
  rec.total_edge = g->host.edge_count;
  records.push_back(rec);
  walk_stats.emplace_back(scanned, second);
  step = advance(kind);
  if (kind == PM_STEP_ENUMERATION || step == PM_STEP_END) finished = true;
  ++iteration;
  if (iteration >= 1000) finished = true;
}

// ---- the LCC fixpoint as one CUDA graph ----------------------------------
//
// Graph: head kernel -> WHILE(cond) { LCC sweep 1, sweep 2, tail kernel }.
// Its kernels read the query's pointers from a device block, so one
// instantiated graph per (graph plan, word type) serves every query a host
// thread runs: a query writes its block and launches.  Each host thread keeps
// its own graphs (a server slot is one thread), so no two queries share a
// block at the same time; instantiating and destroying graphs (which may wait
// for the whole device) stays out of the per-query path.
namespace {
bool g_lcc_graph = true;
std::atomic<uint64_t> g_plan_epochs{0};

constexpr size_t kArgsBytes = 256;  // QueryDevPtrs, padded
constexpr size_t kLoopBytes = kArgsBytes + sizeof(LccLoopCtl) + sizeof(LccPassRow) * kLccLoopMaxPasses;
static_assert(sizeof(QueryDevPtrs) <= kArgsBytes, "argument block");

struct LccLoop {
  const GraphImpl* g = nullptr;
  uint64_t epoch = 0;
  int device = -1, word_kind = -1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned char* d_block = nullptr;  // arguments | control | rows
  unsigned char* h_block = nullptr;  // pinned mirror
  int64_t pass_launches = 0;         // kernels per pass
  uint64_t used = 0;
  LccLoop() = default;
  LccLoop(const LccLoop&) = delete;
  LccLoop& operator=(const LccLoop&) = delete;
  ~LccLoop() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (d_block) cudaFree(d_block);
    if (h_block) cudaFreeHost(h_block);
  }
  QueryDevPtrs* d_args() const { return reinterpret_cast<QueryDevPtrs*>(d_block); }
  LccLoopCtl* d_ctl() const { return reinterpret_cast<LccLoopCtl*>(d_block + kArgsBytes); }

  void build(const GraphImpl& graph_impl, int kind) {
    PM_CUDA(cudaMalloc(&d_block, kLoopBytes));
    PM_CUDA(cudaMallocHost(&h_block, kLoopBytes));
    cudaStream_t cs = nullptr;
    PM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    try {
      PM_CUDA(cudaGraphCreate(&graph, 0));
      cudaGraphConditionalHandle handle;
      PM_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
      // Relaxed capture: other host threads may allocate meanwhile.
      PM_CUDA(cudaStreamBeginCaptureToGraph(cs, graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
      launch_lcc_loop_head(d_ctl(), cs);
      PM_CUDA(cudaStreamEndCapture(cs, &graph));
      cudaGraphNode_t head = nullptr;
      size_t n_nodes = 1;
      PM_CUDA(cudaGraphGetNodes(graph, &head, &n_nodes));
      if (n_nodes != 1 || !head) throw PmError{PM_FAILURE, "LCC loop graph: unexpected head nodes"};
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t loop = nullptr;
      PM_CUDA(cudaGraphAddNode(&loop, graph, &head, nullptr, 1, &cp));
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      const uint64_t before = thread_launch_count();
      PM_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
      const DevGraph dg = graph_impl.dev();
      launch_lcc_pass_at(dg, kind, d_args(), cs);
      launch_lcc_loop_tail(d_args(), d_ctl(), handle, cs);
      PM_CUDA(cudaStreamEndCapture(cs, &body));
      pass_launches = static_cast<int64_t>(thread_launch_count() - before);
      // Captured launches ran nothing; each run adds what it executes.
      note_launches(-pass_launches - 1);
      PM_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    } catch (...) {
      cudaStreamDestroy(cs);
      throw;
    }
    PM_CUDA(cudaStreamDestroy(cs));
    g = &graph_impl;
    epoch = graph_impl.plan_epoch;
    device = graph_impl.device;
    word_kind = kind;
  }
};

// Per host thread: the loops it built, least recently used dropped first.
struct LccLoopCache {
  static constexpr size_t kMax = 8;
  std::vector<std::unique_ptr<LccLoop>> loops;
  uint64_t tick = 0;
  LccLoop& get(const GraphImpl& g, int kind) {
    for (auto& l : loops)
      if (l->g == &g && l->epoch == g.plan_epoch && l->device == g.device && l->word_kind == kind) {
        l->used = ++tick;
        return *l;
      }
    if (loops.size() >= kMax) {
      auto lru = std::min_element(loops.begin(), loops.end(),
                                  [](const auto& a, const auto& b) { return a->used < b->used; });
      loops.erase(lru);
    }
    auto l = std::make_unique<LccLoop>();
    l->build(g, kind);
    l->used = ++tick;
    loops.push_back(std::move(l));
    return *loops.back();
  }
};
thread_local LccLoopCache t_lcc_loops;
}  // namespace

uint64_t next_plan_epoch() { return g_plan_epochs.fetch_add(1, std::memory_order_relaxed) + 1; }
void set_lcc_graph(bool on) { g_lcc_graph = on; }
bool lcc_graph() { return g_lcc_graph; }
namespace {
std::atomic<bool> g_lcc_label_stream{true};
}  // namespace
void set_lcc_label_stream(bool on) { g_lcc_label_stream.store(on, std::memory_order_relaxed); }
bool lcc_label_stream() { return g_lcc_label_stream.load(std::memory_order_relaxed); }

void QueryImpl::run_lcc_loop(int max_iterations) {
  const int cap = std::min(max_iterations, 1000) - iteration;
  if (cap <= 0) return;
  const StepRange range("LCC fixpoint");
  ensure_hub_acc();
  LccLoop& loop = t_lcc_loops.get(*g, word_kind);
  // Arguments and the pass cap in one copy; the head kernel resets the rest.
  const QueryDevPtrs args = ptrs();
  std::memcpy(loop.h_block, &args, sizeof(args));
  LccLoopCtl ctl{};
  ctl.max_passes = static_cast<uint32_t>(cap);
  std::memcpy(loop.h_block + kArgsBytes, &ctl, sizeof(ctl));
  clear_step_counters();
  PM_CUDA(cudaMemcpyAsync(loop.d_block, loop.h_block, kArgsBytes + sizeof(LccLoopCtl), cudaMemcpyHostToDevice,
                          stream));
  PM_CUDA(cudaEventRecord(ev0, stream));
  if (!first_recorded) {
    PM_CUDA(cudaEventRecord(ev_first, stream));
    first_recorded = true;
  }
  PM_CUDA(cudaGraphLaunch(loop.exec, stream));
  lcc_first_pending = false;  // the loop's first tail cleared the block's flag
  PM_CUDA(cudaEventRecord(ev1, stream));
  // Control block and the first rows in one read; the rest only if needed.
  constexpr size_t kFirstRows = 64;
  const size_t first = sizeof(LccLoopCtl) + sizeof(LccPassRow) * kFirstRows;
  unsigned char* h_ctl = loop.h_block + kArgsBytes;
  PM_CUDA(cudaMemcpyAsync(h_ctl, loop.d_ctl(), first, cudaMemcpyDeviceToHost, stream));
  PM_CUDA(cudaStreamSynchronize(stream));
  LccLoopCtl hc;
  std::memcpy(&hc, h_ctl, sizeof(hc));
  if (hc.passes > kFirstRows && hc.passes <= kLccLoopMaxPasses) {
    PM_CUDA(cudaMemcpyAsync(h_ctl + first, reinterpret_cast<unsigned char*>(loop.d_ctl()) + first,
                            sizeof(LccPassRow) * (hc.passes - kFirstRows), cudaMemcpyDeviceToHost, stream));
    PM_CUDA(cudaStreamSynchronize(stream));
  }
  note_launches(1 + loop.pass_launches * static_cast<int64_t>(std::min(hc.passes, kLccLoopMaxPasses)));
  if (hc.error) throw PmError{PM_E_DEVICE, "device-side error status " + std::to_string(hc.error)};
  if (hc.passes == 0 || hc.passes > static_cast<uint32_t>(cap))
    throw PmError{PM_FAILURE, "LCC loop graph ran " + std::to_string(hc.passes) + " passes"};
  LccPassRow row;
  unsigned long long prev = hc.start_ns;
  for (uint32_t i = 0; i < hc.passes; ++i) {
    std::memcpy(&row, h_ctl + sizeof(LccLoopCtl) + sizeof(LccPassRow) * i, sizeof(row));
    StepResult r;
    r.vertex = row.vertex_elim;
    r.edge = row.edge_elim;
    r.match = row.match_elim;
    const double ms = row.end_ns >= prev ? (row.end_ns - prev) * 1e-6 : 0.0;
    prev = row.end_ns;
    append_record(r, PM_STEP_LCC, ms, row.scanned, row.gathered);
  }
}

// ---- batched form: many queries per launch ---------------------------------
namespace {
// Device copies of the listed queries' pointer blocks and an index list.
struct BatchPtrs {
  DeviceBuffer d_qs, d_active, d_out;
  std::vector<QueryDevPtrs> h_qs;
  std::vector<uint32_t> h_active;
  StepCounters* h_out = nullptr;
  explicit BatchPtrs(cudaStream_t s) {
    for (DeviceBuffer* b : {&d_qs, &d_active, &d_out}) {
      b->stream = s;
      b->ordered = true;
    }
  }
  ~BatchPtrs() {
    if (h_out) cudaFreeHost(h_out);
  }
  void upload(const std::vector<QueryImpl*>& qs, cudaStream_t s) {
    h_qs.clear();
    for (QueryImpl* q : qs) h_qs.push_back(q->ptrs());
    d_qs.ensure(sizeof(QueryDevPtrs) * h_qs.size());
    d_active.ensure(4 * h_qs.size());
    d_out.ensure(sizeof(StepCounters) * h_qs.size());
    if (!h_out) PM_CUDA(cudaMallocHost(&h_out, sizeof(StepCounters) * h_qs.size()));
    PM_CUDA(cudaMemcpyAsync(d_qs.ptr, h_qs.data(), sizeof(QueryDevPtrs) * h_qs.size(), cudaMemcpyHostToDevice, s));
  }
  // The same queries' pointer blocks again (their flags changed).
  void refresh(const std::vector<QueryImpl*>& qs, cudaStream_t s) {
    for (size_t i = 0; i < qs.size(); ++i) h_qs[i] = qs[i]->ptrs();
    PM_CUDA(cudaMemcpyAsync(d_qs.ptr, h_qs.data(), sizeof(QueryDevPtrs) * h_qs.size(), cudaMemcpyHostToDevice, s));
  }
  void set_active(const std::vector<uint32_t>& a, cudaStream_t s) {
    h_active = a;
    PM_CUDA(cudaMemcpyAsync(d_active.ptr, h_active.data(), 4 * h_active.size(), cudaMemcpyHostToDevice, s));
  }
};

// Queries grouped by word type (the multi-query kernels are per type).
std::vector<std::vector<QueryImpl*>> by_word_kind(const std::vector<QueryImpl*>& qs) {
  std::vector<std::vector<QueryImpl*>> out;
  for (QueryImpl* q : qs) {
    auto it = std::find_if(out.begin(), out.end(), [&](const auto& v) { return v[0]->word_kind == q->word_kind; });
    if (it == out.end())
      out.push_back({q});
    else
      it->push_back(q);
  }
  return out;
}

void check_batch_counters(const StepCounters& c) {
  if (c.error) throw PmError{PM_E_DEVICE, "device-side error status " + std::to_string(c.error)};
}
}  // namespace

void QueryImpl::lcc0_batch(const std::vector<QueryImpl*>& all, cudaStream_t s) {
  for (auto& qs : by_word_kind(all)) {
    const GraphImpl* g = qs[0]->g;
    for (QueryImpl* q : qs) {
      if (q->g != g || q->step != PM_STEP_LCC0 || q->finished) throw PmError{PM_FAILURE, "lcc0_batch: bad query"};
      q->ensure_hub_acc();
      PM_CUDA(cudaStreamSynchronize(q->stream));
    }
    BatchPtrs b(s);
    b.upload(qs, s);
    std::vector<uint32_t> active(qs.size());
    for (uint32_t i = 0; i < active.size(); ++i) active[i] = i;
    b.set_active(active, s);
    cudaEvent_t e0, e1;
    PM_CUDA(cudaEventCreate(&e0));
    PM_CUDA(cudaEventCreate(&e1));
    const uint32_t n = static_cast<uint32_t>(qs.size());
    launch_counters_multi(b.d_qs.as<QueryDevPtrs>(), b.d_active.as<uint32_t>(), n, nullptr, true, s);
    PM_CUDA(cudaEventRecord(e0, s));
    launch_lcc0_multi(g->dev(), qs[0]->word_kind, b.d_qs.as<QueryDevPtrs>(), b.d_active.as<uint32_t>(), n, s);
    PM_CUDA(cudaEventRecord(e1, s));
    launch_counters_multi(b.d_qs.as<QueryDevPtrs>(), b.d_active.as<uint32_t>(), n, b.d_out.as<StepCounters>(), false,
                          s);
    PM_CUDA(cudaGetLastError());
    PM_CUDA(cudaMemcpyAsync(b.h_out, b.d_out.ptr, sizeof(StepCounters) * n, cudaMemcpyDeviceToHost, s));
    PM_CUDA(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (uint32_t i = 0; i < n; ++i) {
      check_batch_counters(b.h_out[i]);
      StepResult r;
      r.vertex = b.h_out[i].vertex_elim;
      r.match = b.h_out[i].match_elim;
      qs[i]->append_record(r, PM_STEP_LCC0, ms, 0, 0);
      qs[i]->lcc_first_pending = true;
    }
  }
}

void QueryImpl::lcc_fixpoint_batch(const std::vector<QueryImpl*>& all, cudaStream_t s) {
  for (auto& qs : by_word_kind(all)) {
    const GraphImpl* g = qs[0]->g;
    for (QueryImpl* q : qs) {
      if (q->g != g || q->step != PM_STEP_LCC || q->finished || q->active_vertices == 0)
        throw PmError{PM_FAILURE, "lcc_fixpoint_batch: bad query"};
      q->ensure_hub_acc();
      PM_CUDA(cudaStreamSynchronize(q->stream));
    }
    BatchPtrs b(s);
    b.upload(qs, s);
    std::vector<uint32_t> active(qs.size());
    for (uint32_t i = 0; i < active.size(); ++i) active[i] = i;
    cudaEvent_t e0, e1;
    PM_CUDA(cudaEventCreate(&e0));
    PM_CUDA(cudaEventCreate(&e1));
    try {
      while (!active.empty()) {
        const uint32_t n = static_cast<uint32_t>(active.size());
        b.set_active(active, s);
        const QueryDevPtrs* dq = b.d_qs.as<QueryDevPtrs>();
        const uint32_t* da = b.d_active.as<uint32_t>();
        launch_counters_multi(dq, da, n, nullptr, true, s);
        PM_CUDA(cudaEventRecord(e0, s));
        launch_lcc_pass_multi(g->dev(), qs[0]->word_kind, dq, da, n, s);
        PM_CUDA(cudaEventRecord(e1, s));
        // Passes after the first gather neighbour words: clear the flags in
        // the device copies (stream-ordered after this pass's kernels).
        bool any_first = false;
        for (QueryImpl* q : qs) any_first |= q->lcc_first_pending;
        if (any_first) {
          for (QueryImpl* q : qs) q->lcc_first_pending = false;
          b.refresh(qs, s);
        }
        launch_counters_multi(dq, da, n, b.d_out.as<StepCounters>(), false, s);
        PM_CUDA(cudaGetLastError());
        PM_CUDA(cudaMemcpyAsync(b.h_out, b.d_out.ptr, sizeof(StepCounters) * n, cudaMemcpyDeviceToHost, s));
        PM_CUDA(cudaStreamSynchronize(s));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        std::vector<uint32_t> next;
        for (uint32_t j = 0; j < n; ++j) {
          const StepCounters& c = b.h_out[j];
          check_batch_counters(c);
          QueryImpl* q = qs[active[j]];
          StepResult r;
          r.vertex = c.vertex_elim;
          r.edge = c.edge_elim;
          r.match = c.match_elim;
          q->append_record(r, PM_STEP_LCC, ms, c.scanned, c.gathered);
          if (!q->finished && q->step == PM_STEP_LCC && q->active_vertices != 0) next.push_back(active[j]);
        }
        active.swap(next);
      }
    } catch (...) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
}

double QueryImpl::elapsed_ms() {
  if (!first_recorded) return 0.0;
  PM_CUDA(cudaEventSynchronize(ev1));
  float ms = 0;
  PM_CUDA(cudaEventElapsedTime(&ms, ev_first, ev1));
  return ms;
}

pm_step_record QueryImpl::final_record() {
  pm_step_record rec{};
  rec.iteration = iteration;
  rec.step = step;
  rec.step_ms = 0;
  rec.cumulative_ms = total_ms;
  rec.active_vertex = active_vertices;
  rec.total_vertex = g->host.vertex_count;
  rec.active_edge = active_edges;
  rec.total_edge = g->host.edge_count;
  return rec;
}

namespace {
double g_query_budget_ms = 0;
}  // namespace
void set_query_budget_ms(double ms) { g_query_budget_ms = ms > 0 ? ms : 0; }
double query_budget_ms() { return g_query_budget_ms; }

void QueryImpl::check_request() {
  if (cancel && cancel->load(std::memory_order_relaxed))
    throw PmError{PM_E_CANCELLED, "request cancelled while running"};
  if (has_deadline) {
    const auto left = deadline - std::chrono::steady_clock::now();
    const int64_t left_ns = std::chrono::duration_cast<std::chrono::nanoseconds>(left).count();
    if (left_ns <= 0) throw PmError{PM_E_TIMEOUT, "the request's time budget ran out"};
    set_thread_walk_budget_cap_ns(static_cast<uint64_t>(left_ns));
  }
}

void QueryImpl::run_all(int max_iterations) {
  if (!has_deadline && g_query_budget_ms > 0) {
    has_deadline = true;
    deadline = std::chrono::steady_clock::now() +
               std::chrono::microseconds(static_cast<int64_t>(g_query_budget_ms * 1000.0));
  }
  struct CapReset {
    ~CapReset() { set_thread_walk_budget_cap_ns(0); }
  } cap_reset;
  while (!finished && iteration < max_iterations) {
    if (stop_before_enumeration && step == PM_STEP_ENUMERATION) break;
    check_request();
    run_unit(max_iterations);
  }
}

void QueryImpl::run_unit(int max_iterations) {
  if (step == PM_STEP_LCC && g_lcc_graph && active_vertices != 0)
    run_lcc_loop(max_iterations);
  else
    run_step();
}

void QueryImpl::export_state(uint64_t* cand, uint8_t* eact, uint8_t* vact) {
  const uint64_t V = g->host.vertex_count, E = g->host.edge_count;
  DeviceBuffer dc, de, dv;
  for (DeviceBuffer* b : {&dc, &de, &dv}) {
    b->stream = stream;
    b->ordered = true;
  }
  if (cand) dc.ensure(8 * std::max<uint64_t>(V, 1));
  if (eact) de.ensure(std::max<uint64_t>(E, 1));
  if (vact) dv.ensure(std::max<uint64_t>(V, 1));
  launch_export(g->dev(), ptrs(), cand ? dc.as<uint64_t>() : nullptr, vact ? dv.as<uint8_t>() : nullptr,
                eact ? de.as<uint8_t>() : nullptr, stream);
  PM_CUDA(cudaGetLastError());
  if (cand && V) PM_CUDA(cudaMemcpyAsync(cand, dc.ptr, 8 * V, cudaMemcpyDeviceToHost, stream));
  if (eact && E) PM_CUDA(cudaMemcpyAsync(eact, de.ptr, E, cudaMemcpyDeviceToHost, stream));
  if (vact && V) PM_CUDA(cudaMemcpyAsync(vact, dv.ptr, V, cudaMemcpyDeviceToHost, stream));
  PM_CUDA(cudaStreamSynchronize(stream));
}

uint64_t QueryImpl::list_matches(uint32_t* out, uint64_t cap, uint32_t* per_match) {
  if (!finished && step != PM_STEP_ENUMERATION) {
    struct Restore {
      QueryImpl& q;
      ~Restore() { q.stop_before_enumeration = false; }
    } restore{*this};
    stop_before_enumeration = true;
    run_all();
  }
  const WalkProgram& p = enumeration.cc.programs[0];
  if (per_match) *per_match = p.n_hist;
  // The run ended at the iteration cap before ENUMERATION: nothing counted.
  const bool counted = step == PM_STEP_ENUMERATION ||
                       std::any_of(records.begin(), records.end(),
                                   [](const pm_step_record& r) { return r.step == PM_STEP_ENUMERATION; });
  if (!counted || active_vertices == 0) return 0;
  const uint32_t n_wl = build_worklist(uint64_t(1) << p.start_role);
  if (!n_wl) return 0;
  DeviceBuffer d_out, d_cnt;
  for (DeviceBuffer* b : {&d_out, &d_cnt}) {
    b->stream = stream;
    b->ordered = true;
  }
  d_out.ensure(4ull * p.n_hist * std::max<uint64_t>(cap, 1));
  d_cnt.ensure(2 * sizeof(unsigned long long));
  PM_CUDA(cudaMemsetAsync(d_cnt.ptr, 0, 2 * sizeof(unsigned long long), stream));
  clear_step_counters();
  launch_enum_list(g->dev(), ptrs(), d_progs.as<WalkProgram>() + enumeration.prog_offset, d_wl.as<uint32_t>(), n_wl,
                   d_out.as<uint32_t>(), cap, d_cnt.as<unsigned long long>(), stream);
  PM_CUDA(cudaGetLastError());
  unsigned long long cnt[2] = {0, 0};
  PM_CUDA(cudaMemcpyAsync(cnt, d_cnt.ptr, sizeof(cnt), cudaMemcpyDeviceToHost, stream));
  read_counters();  // synchronises; a timeout or device error throws
  const uint64_t rows = std::min<uint64_t>(cnt[1], cap);
  if (out && rows) {
    PM_CUDA(cudaMemcpyAsync(out, d_out.ptr, 4ull * p.n_hist * rows, cudaMemcpyDeviceToHost, stream));
    PM_CUDA(cudaStreamSynchronize(stream));
  }
  return cnt[1];
}

uint64_t QueryImpl::export_subgraph(uint64_t* offsets, uint32_t* adj, uint64_t cap) {
  const uint64_t V = g->host.vertex_count;
  DeviceBuffer d_counts, d_off, d_adj;
  for (DeviceBuffer* b : {&d_counts, &d_off, &d_adj}) {
    b->stream = stream;
    b->ordered = true;
  }
  d_counts.ensure(8 * std::max<uint64_t>(V, 1));
  launch_subgraph(g->dev(), ptrs(), nullptr, d_counts.as<uint64_t>(), nullptr, stream);
  PM_CUDA(cudaGetLastError());
  std::vector<uint64_t> off(V + 1, 0);
  if (V) PM_CUDA(cudaMemcpyAsync(off.data() + 1, d_counts.ptr, 8 * V, cudaMemcpyDeviceToHost, stream));
  PM_CUDA(cudaStreamSynchronize(stream));
  for (uint64_t v = 0; v < V; ++v) off[v + 1] += off[v];
  const uint64_t total = off[V];
  if (offsets) std::memcpy(offsets, off.data(), 8 * (V + 1));
  if (adj && total && cap >= total) {
    d_off.ensure(8 * (V + 1));
    d_adj.ensure(4 * total);
    PM_CUDA(cudaMemcpyAsync(d_off.ptr, off.data(), 8 * (V + 1), cudaMemcpyHostToDevice, stream));
    launch_subgraph(g->dev(), ptrs(), d_off.as<uint64_t>(), nullptr, d_adj.as<uint32_t>(), stream);
    PM_CUDA(cudaGetLastError());
    PM_CUDA(cudaMemcpyAsync(adj, d_adj.ptr, 4 * total, cudaMemcpyDeviceToHost, stream));
    PM_CUDA(cudaStreamSynchronize(stream));
  }
  return total;
}

namespace {
void make_dirs(const std::string& path) {
  std::string cur;
  std::stringstream ss(path);
  std::string item;
  bool first = true;
  while (std::getline(ss, item, '/')) {
    if (!item.empty() || first) {
      cur += item + "/";
      mkdir(cur.c_str(), 0777);
      first = false;
    }
  }
}
}  // namespace

void QueryImpl::write_outputs(const std::string& dir_in) {
  std::string dir = dir_in;
  if (dir.empty() || dir.back() != '/') dir += "/";
  make_dirs(dir);
  const uint32_t V = g->host.vertex_count;
  const uint64_t E = g->host.edge_count;
  std::vector<uint64_t> cand(V);
  std::vector<uint8_t> eact(E), vact(V);
  export_state(cand.data(), eact.data(), vact.data());
  const pm_step_record fin = final_record();
  {
    std::ofstream f(dir + "results.totem", std::ofstream::trunc);
    if (!f) throw PmError{PM_E_IO, "cannot write " + dir + "results.totem"};
    f << "Iteration; Step; Step time; Cumulative time; Eliminated vertex; Active vertex; Total vertex; "
         "Eliminated edge; Active edge; Total edge; Eliminated match; Enumeration number\n";
    char line[512];
    auto row = [&](const pm_step_record& r) {
      snprintf(line, sizeof(line), "%04d; %s; %.4f ; %.4f ; %llu; %llu; %llu; %llu; %llu; %llu; %llu; %llu\n",
               // The only START row is the dynamic order's first one, which
               // the reference logs with an empty step name.
               r.iteration, r.step == PM_STEP_START ? "" : step_name(r.step).c_str(), r.step_ms, r.cumulative_ms,
               (unsigned long long)r.results.vertex_eliminated, (unsigned long long)r.active_vertex,
               (unsigned long long)r.total_vertex, (unsigned long long)r.results.edge_eliminated,
               (unsigned long long)r.active_edge, (unsigned long long)r.total_edge,
               (unsigned long long)r.results.match_eliminated, (unsigned long long)r.results.enumeration);
      f << line;
    };
    for (const auto& r : records) row(r);
    row(fin);
  }
  char name[64];
  snprintf(name, sizeof(name), "graph_%04d.totem", fin.iteration);
  {
    FILE* f = fopen((dir + name).c_str(), "wb");
    if (!f) throw PmError{PM_E_IO, "cannot write " + dir + name};
    const auto& lab = g->host.labels;
    for (uint32_t v = 0; v < V; ++v) {
      if (!vact[v]) continue;
      for (uint64_t e = g->host.offsets[v]; e < g->host.offsets[v + 1]; ++e) {
        if (!eact[e]) continue;
        const uint32_t w = g->host.adj[e];
        if (!vact[w]) continue;
        fprintf(f, "%u %u %llu %llu\n", v, w, (unsigned long long)lab[v], (unsigned long long)lab[w]);
      }
    }
    fputc('\n', f);
    fclose(f);
  }
  snprintf(name, sizeof(name), "vertex_%04d.totem", fin.iteration);
  {
    FILE* f = fopen((dir + name).c_str(), "wb");
    if (!f) throw PmError{PM_E_IO, "cannot write " + dir + name};
    for (uint32_t v = 0; v < V; ++v) {
      if (!vact[v]) continue;
      fprintf(f, "%u ", v);
      for (uint32_t p = 0; p < 64; ++p)
        if (cand[v] >> p & 1) fprintf(f, "%u ", p);
      fputc('\n', f);
    }
    fputc('\n', f);
    fclose(f);
  }
  {
    std::ofstream f(dir + "log.totem", std::ofstream::trunc);
    f << dump_constraints(qc);
  }
  { std::ofstream f(dir + "effectiveness.totem", std::ofstream::trunc); }
  { std::ofstream f(dir + "enumeration_0000.totem", std::ofstream::trunc); }
}

}  // namespace pmgb
