// The C ABI of include/pm_gb300.h and include/pm_gb300_tools.h.
#include <cstring>
#include <new>
#include <string>
#include <exception>
#include <thread>

#include "../../include/pm_gb300_tools.h"
#include "engine.h"
#include "generators.h"
#include "autotune.h"
#include "fused_batch.h"
#include "server.h"
#include "totem_io.h"

using namespace pmgb;

struct pm_graph {
  GraphImpl impl;
};
struct pm_query {
  QueryImpl impl;
};
struct pm_fused_batch {
  std::unique_ptr<pmgb::FusedBatch> impl;
};

struct pm_server {
  std::unique_ptr<Server> impl;
};

namespace {
thread_local std::string g_last_error;

pm_status_t fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

template <class F>
pm_status_t guarded(F&& f) {
  try {
    g_last_error.clear();
    return f();
  } catch (const PmError& e) {
    return fail(e.code, e.message);
  } catch (const std::bad_alloc&) {
    return fail(PM_E_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(PM_FAILURE, e.what());
  }
}

#define PM_REQUIRE(cond, msg) \
  if (!(cond)) return fail(PM_E_INVALID_ARG, msg)
}  // namespace

extern "C" {

const char* pm_last_error(void) { return g_last_error.c_str(); }
const char* pm_version(void) { return "pm_gb300 1.0 (sm_103a)"; }

pm_status_t pm_graph_load(const char* graph_path, const char* bin_path, const char* labels_path, int device,
                          pm_graph** out) {
  PM_REQUIRE(out, "out is NULL");
  return guarded([&]() -> pm_status_t {
    auto* g = new pm_graph();
    try {
      const std::string bin = bin_path ? bin_path : "";
      // MultipleLabelCpu::allocate (multiple_label_cpu.cc:22-35): an existing
      // binary replaces the text graph and its labels; otherwise the text is
      // parsed, labels applied and the binary cache written.
      if (!bin.empty() && is_regular_file(bin)) {
        g->impl.host = read_totem_graph(bin);
      } else {
        PM_REQUIRE(graph_path && *graph_path, "graph_path is empty");
        g->impl.host = read_totem_graph(graph_path);
        if (labels_path && *labels_path && is_regular_file(labels_path)) read_vertex_labels(labels_path, g->impl.host);
        if (!bin.empty()) write_totem_binary(g->impl.host, bin, g->impl.host.edge_count > 0xFFFFFFFFull ? 8 : 4);
      }
      g->impl.finalize_host();
      if (device >= 0) g->impl.to_device(device);
    } catch (...) {
      delete g;
      throw;
    }
    *out = g;
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_from_csr(const uint64_t* offsets, const uint32_t* adj, const uint64_t* labels,
                              uint32_t vertex_count, uint64_t edge_count, int device, pm_graph** out) {
  PM_REQUIRE(out && offsets && (adj || edge_count == 0), "null CSR buffer");
  PM_REQUIRE(offsets[vertex_count] == edge_count, "offsets[vertex_count] != edge_count");
  // One parallel pass checks the offsets, the targets and the list order.
  const CsrScan scan = scan_csr(offsets, adj, vertex_count);
  PM_REQUIRE(scan.monotone, "offsets not monotone");
  PM_REQUIRE(scan.in_range, "edge target out of range");
  return guarded([&]() -> pm_status_t {
    auto* g = new pm_graph();
    try {
      HostGraph& h = g->impl.host;
      h.vertex_count = vertex_count;
      h.edge_count = edge_count;
      auto fill = [](auto& dst, const auto* src, uint64_t n) {
        dst.resize(n);  // unwritten: the parallel copy touches each page first
        auto* d = dst.data();
        parallel_ranges(n, [&](uint64_t lo, uint64_t hi) { std::memcpy(d + lo, src + lo, sizeof(*d) * (hi - lo)); });
      };
      fill(h.offsets, offsets, uint64_t(vertex_count) + 1);
      h.valued = labels != nullptr;
      if (labels) fill(h.labels, labels, vertex_count);
      g->impl.finalize_host(&scan.sorted_unique);
      // The host copy of the adjacency is filled while the device copy is
      // made from the caller's buffer.
      std::exception_ptr copy_err;
      std::thread copier([&] {
        try {
          fill(h.adj, adj, edge_count);
        } catch (...) {
          copy_err = std::current_exception();
        }
      });
      try {
        if (device >= 0) g->impl.to_device(device, adj);
      } catch (...) {
        copier.join();
        throw;
      }
      copier.join();
      if (copy_err) std::rethrow_exception(copy_err);
    } catch (...) {
      delete g;
      throw;
    }
    *out = g;
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_store_binary(const pm_graph* g, const char* path) {
  PM_REQUIRE(g && path, "null argument");
  return guarded([&]() -> pm_status_t {
    write_totem_binary(g->impl.host, path, g->impl.host.edge_count > 0xFFFFFFFFull ? 8 : 4);
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_info(const pm_graph* g, uint32_t* vertex_count, uint64_t* edge_count, uint64_t* device_bytes) {
  PM_REQUIRE(g, "graph is NULL");
  if (vertex_count) *vertex_count = g->impl.host.vertex_count;
  if (edge_count) *edge_count = g->impl.host.edge_count;
  if (device_bytes) *device_bytes = g->impl.device_bytes();
  return PM_SUCCESS;
}

void pm_graph_destroy(pm_graph* g) { delete g; }

pm_status_t pm_graph_generate_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                                   int32_t permute, pm_graph** out) {
  PM_REQUIRE(out, "out is NULL");
  return guarded([&]() -> pm_status_t {
    auto* g = new pm_graph();
    try {
      g->impl.host = generate_rmat(scale, edge_factor, a, b, c, seed, permute != 0);
      g->impl.finalize_host();
    } catch (...) {
      delete g;
      throw;
    }
    *out = g;
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_assign_labels(pm_graph* g, int32_t kind, uint32_t n_labels, double zipf_s, uint64_t seed) {
  PM_REQUIRE(g, "graph is NULL");
  PM_REQUIRE(kind >= 0 && kind <= 2, "label kind must be 0, 1 or 2");
  PM_REQUIRE(g->impl.device < 0, "labels must be assigned before the graph moves to a device");
  return guarded([&]() -> pm_status_t {
    assign_labels(g->impl.host, kind, n_labels, zipf_s, seed);
    g->impl.finalize_host();
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_make_undirected(const pm_graph* g, pm_graph** out) {
  PM_REQUIRE(g && out, "null argument");
  return guarded([&]() -> pm_status_t {
    auto* n = new pm_graph();
    try {
      n->impl.host = make_undirected(g->impl.host);
      n->impl.finalize_host();
    } catch (...) {
      delete n;
      throw;
    }
    *out = n;
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_sort_neighbours(pm_graph* g) {
  PM_REQUIRE(g, "graph is NULL");
  PM_REQUIRE(g->impl.device < 0, "sort the graph before it moves to a device");
  return guarded([&]() -> pm_status_t {
    sort_neighbours(g->impl.host);
    g->impl.finalize_host();
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_sort_vertices_by_degree(const pm_graph* g, pm_graph** out, uint32_t* old_to_new) {
  PM_REQUIRE(g && out, "null argument");
  return guarded([&]() -> pm_status_t {
    auto* n = new pm_graph();
    try {
      std::vector<uint32_t> map;
      n->impl.host = sort_vertices_by_degree(g->impl.host, &map);
      n->impl.finalize_host();
      if (old_to_new && !map.empty()) std::memcpy(old_to_new, map.data(), 4 * map.size());
    } catch (...) {
      delete n;
      throw;
    }
    *out = n;
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_host_csr(const pm_graph* g, const uint64_t** offsets, const uint32_t** adj,
                              const uint64_t** labels) {
  PM_REQUIRE(g, "graph is NULL");
  if (offsets) *offsets = g->impl.host.offsets.data();
  if (adj) *adj = g->impl.host.adj.data();
  if (labels) *labels = g->impl.host.labels.data();
  return PM_SUCCESS;
}

pm_status_t pm_graph_to_device(pm_graph* g, int32_t device) {
  PM_REQUIRE(g && device >= 0, "bad argument");
  return guarded([&]() -> pm_status_t {
    g->impl.to_device(device);
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_write_text(const pm_graph* g, const char* graph_path, const char* labels_path) {
  PM_REQUIRE(g, "graph is NULL");
  return guarded([&]() -> pm_status_t {
    if (graph_path && *graph_path) write_totem_text(g->impl.host, graph_path);
    if (labels_path && *labels_path) write_vertex_labels(g->impl.host, labels_path);
    return PM_SUCCESS;
  });
}

std::atomic<int> g_order_threads{1};

static pm_status_t create_query(pm_graph* g, const PatternGraph& p, pm_query** out, int variant = 0) {
  auto* q = new pm_query();
  try {
    g->impl.to_device(g->impl.device >= 0 ? g->impl.device : 0);
    q->impl.nlcc_variant = variant & 0xFF;
    q->impl.order = variant & ~0xFF;
    q->impl.order_threads = g_order_threads.load();
    q->impl.create(&g->impl, p, nullptr);
  } catch (...) {
    delete q;
    throw;
  }
  *out = q;
  return PM_SUCCESS;
}

pm_status_t pm_query_create(pm_graph* g, const char* pattern_dir, int load_pattern_labels, pm_query** out) {
  PM_REQUIRE(g && pattern_dir && out, "null argument");
  return guarded([&]() -> pm_status_t { return create_query(g, load_pattern(pattern_dir, load_pattern_labels != 0), out); });
}

pm_status_t pm_query_create_from_csr(pm_graph* g, const uint64_t* p_offsets, const uint32_t* p_adj,
                                     const uint64_t* p_labels, uint32_t p_vertex_count, uint64_t p_edge_count,
                                     pm_query** out) {
  PM_REQUIRE(g && p_offsets && out, "null argument");
  PM_REQUIRE(p_offsets[0] == 0, "pattern offsets must start at 0");
  for (uint32_t i = 0; i < p_vertex_count; ++i)
    PM_REQUIRE(p_offsets[i] <= p_offsets[i + 1], "pattern offsets must not decrease");
  PM_REQUIRE(p_offsets[p_vertex_count] == p_edge_count, "pattern offsets do not end at the edge count");
  for (uint64_t e = 0; e < p_edge_count; ++e) PM_REQUIRE(p_adj[e] < p_vertex_count, "pattern edge out of range");
  return guarded([&]() -> pm_status_t {
    PatternGraph p;
    p.n = p_vertex_count;
    p.offsets.assign(p_offsets, p_offsets + p_vertex_count + 1);
    p.adj.assign(p_adj, p_adj + p_edge_count);
    p.labels = p_labels ? std::vector<uint64_t>(p_labels, p_labels + p_vertex_count)
                        : std::vector<uint64_t>(p_vertex_count, 0);
    return create_query(g, p, out);
  });
}

// Walk variant in the low byte, PM_ORDER_* flags above it; the order
// drivers run the article's walks only.
static bool valid_variant(int32_t variant) {
  const int32_t walk = variant & 0xFF, order = variant & ~0xFF;
  if (walk < PM_NLCC_REFERENCE || walk > PM_NLCC_BACKTRACK) return false;
  if (order & ~(PM_ORDER_ENUMERATE | PM_ORDER_EFFECTIVENESS | PM_ORDER_EARLY_ENUMERATION)) return false;
  if (order && walk == PM_NLCC_REFERENCE) return false;
  if ((order & PM_ORDER_EARLY_ENUMERATION) && !(order & PM_ORDER_EFFECTIVENESS)) return false;
  return true;
}

pm_status_t pm_set_order_threads(int32_t threads) {
  PM_REQUIRE(threads >= 1, "thread count must be at least 1");
  g_order_threads.store(threads);
  return PM_SUCCESS;
}

pm_status_t pm_query_create_variant(pm_graph* g, const char* pattern_dir, int load_pattern_labels, int32_t variant,
                                    pm_query** out) {
  PM_REQUIRE(g && pattern_dir && out, "null argument");
  PM_REQUIRE(valid_variant(variant), "unknown walk variant or order flags");
  return guarded([&]() -> pm_status_t {
    return create_query(g, load_pattern(pattern_dir, load_pattern_labels != 0), out, variant);
  });
}

pm_status_t pm_query_constraint_counts(const pm_query* q, int32_t* n_cycle, int32_t* n_path, int32_t* n_template) {
  PM_REQUIRE(q, "query is NULL");
  if (n_cycle) *n_cycle = static_cast<int32_t>(q->impl.cycles.size());
  if (n_path) *n_path = static_cast<int32_t>(q->impl.paths.size());
  if (n_template) *n_template = static_cast<int32_t>(q->impl.templates.size());
  return PM_SUCCESS;
}

pm_status_t pm_query_dump_constraints(const pm_query* q, char* buf, size_t cap, size_t* needed) {
  PM_REQUIRE(q, "query is NULL");
  return guarded([&]() -> pm_status_t {
    const std::string d = dump_constraints(q->impl.qc);
    if (needed) *needed = d.size() + 1;
    if (buf && cap) {
      const size_t n = d.size() < cap - 1 ? d.size() : cap - 1;
      memcpy(buf, d.data(), n);
      buf[n] = 0;
    }
    return PM_SUCCESS;
  });
}

pm_status_t pm_query_step(pm_query* q, pm_step_record* record, int* finished) {
  PM_REQUIRE(q, "query is NULL");
  return guarded([&]() -> pm_status_t {
    pm_step_record r = q->impl.finished ? q->impl.final_record() : q->impl.run_step();
    if (record) *record = r;
    if (finished) *finished = q->impl.finished ? 1 : 0;
    return PM_SUCCESS;
  });
}

pm_status_t pm_query_run(pm_query* q, pm_step_record* records, int32_t cap, int32_t* n_records) {
  PM_REQUIRE(q, "query is NULL");
  return guarded([&]() -> pm_status_t {
    q->impl.run_all();
    int32_t n = 0;
    for (const auto& r : q->impl.records) {
      if (records && n < cap) records[n] = r;
      ++n;
    }
    if (records && n < cap) records[n] = q->impl.final_record();
    ++n;
    if (n_records) *n_records = n;
    return PM_SUCCESS;
  });
}

pm_status_t pm_query_prune(pm_query* q, pm_step_record* records, int32_t cap, int32_t* n_records) {
  PM_REQUIRE(q, "query is NULL");
  return guarded([&]() -> pm_status_t {
    struct Restore {
      QueryImpl& q;
      ~Restore() { q.stop_before_enumeration = false; }
    } restore{q->impl};
    q->impl.stop_before_enumeration = true;
    q->impl.run_all();
    int32_t n = 0;
    for (const auto& r : q->impl.records) {
      if (records && n < cap) records[n] = r;
      ++n;
    }
    if (records && n < cap) records[n] = q->impl.final_record();
    ++n;
    if (n_records) *n_records = n;
    return PM_SUCCESS;
  });
}

pm_status_t pm_debug_fail_device_alloc_after(int64_t n) {
  set_fail_alloc_after(n);
  return PM_SUCCESS;
}

pm_status_t pm_query_list_matches(pm_query* q, uint32_t* matches, uint64_t cap, uint32_t* per_match,
                                  uint64_t* n_matches) {
  PM_REQUIRE(q, "query is NULL");
  PM_REQUIRE(matches || cap == 0, "null match buffer");
  return guarded([&]() -> pm_status_t {
    const uint64_t n = q->impl.list_matches(matches, cap, per_match);
    if (n_matches) *n_matches = n;
    return PM_SUCCESS;
  });
}

pm_status_t pm_query_write_matches(pm_query* q, const char* path, uint64_t max_matches, uint64_t* n_written) {
  PM_REQUIRE(q && path, "null argument");
  return guarded([&]() -> pm_status_t {
    uint32_t k = 0;
    std::vector<uint32_t> buf(static_cast<size_t>(std::min<uint64_t>(max_matches, 1ull << 28)) *
                              std::max<uint32_t>(q->impl.k, 1));
    const uint64_t total = q->impl.list_matches(buf.data(), max_matches, &k);
    const uint64_t rows = std::min(total, max_matches);
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(PM_E_IO, std::string("cannot open ") + path);
    // The reference's text form: each bound vertex followed by ';', one
    // match per line (multiple_label_enumeration_cpu.tpp:27-33).
    for (uint64_t r = 0; r < rows; ++r) {
      for (uint32_t j = 0; j < k; ++j) std::fprintf(f, "%u;", buf[r * k + j]);
      std::fputc('\n', f);
    }
    const bool ok = std::fclose(f) == 0;
    if (!ok) return fail(PM_E_IO, std::string("cannot write ") + path);
    if (n_written) *n_written = rows;
    return PM_SUCCESS;
  });
}

pm_status_t pm_query_export_subgraph(pm_query* q, uint64_t* offsets, uint32_t* adj, uint64_t cap,
                                     uint64_t* n_entries) {
  PM_REQUIRE(q, "query is NULL");
  return guarded([&]() -> pm_status_t {
    const uint64_t n = q->impl.export_subgraph(offsets, adj, cap);
    if (n_entries) *n_entries = n;
    if (adj && cap < n) return fail(PM_E_INVALID_ARG, "adjacency buffer holds fewer entries than the subgraph");
    return PM_SUCCESS;
  });
}

pm_status_t pm_set_query_budget_ms(double ms) {
  PM_REQUIRE(ms >= 0, "budget must not be negative");
  set_query_budget_ms(ms);
  return PM_SUCCESS;
}

pm_status_t pm_query_export(const pm_query* q, uint64_t* cand_masks, uint8_t* edge_active, uint8_t* vertex_active) {
  PM_REQUIRE(q, "query is NULL");
  return guarded([&]() -> pm_status_t {
    const_cast<QueryImpl&>(q->impl).export_state(cand_masks, edge_active, vertex_active);
    return PM_SUCCESS;
  });
}

pm_status_t pm_query_write_outputs(const pm_query* q, const char* out_dir) {
  PM_REQUIRE(q && out_dir, "null argument");
  return guarded([&]() -> pm_status_t {
    const_cast<QueryImpl&>(q->impl).write_outputs(out_dir);
    return PM_SUCCESS;
  });
}

pm_status_t pm_query_match_count(const pm_query* q, uint64_t* count) {
  PM_REQUIRE(q && count, "null argument");
  *count = q->impl.match_count;
  return PM_SUCCESS;
}

pm_status_t pm_query_device_bytes(const pm_query* q, uint64_t* bytes) {
  PM_REQUIRE(q && bytes, "null argument");
  *bytes = q->impl.device_bytes();
  return PM_SUCCESS;
}

pm_status_t pm_query_estimate_bytes(const pm_graph* g, uint32_t p_vertex_count, uint64_t* bytes) {
  PM_REQUIRE(g && bytes, "null argument");
  *bytes = estimate_query_bytes(g->impl, p_vertex_count);
  return PM_SUCCESS;
}

uint64_t pm_kernel_launches(void) { return launch_count(); }

pm_status_t pm_query_elapsed_ms(const pm_query* q, double* ms) {
  PM_REQUIRE(q && ms, "null argument");
  return guarded([&]() -> pm_status_t {
    *ms = const_cast<QueryImpl&>(q->impl).elapsed_ms();
    return PM_SUCCESS;
  });
}

pm_status_t pm_graph_set_hub_plan(pm_graph* g, uint32_t hub_degree, uint32_t seg_entries) {
  PM_REQUIRE(g, "graph is NULL");
  PM_REQUIRE(seg_entries > 0, "seg_entries must be positive");
  PM_REQUIRE(g->impl.device >= 0, "graph is not on a device");
  return guarded([&]() -> pm_status_t {
    PM_CUDA(cudaSetDevice(g->impl.device));
    g->impl.build_hub_plan(hub_degree, seg_entries);
    return PM_SUCCESS;
  });
}

pm_status_t pm_set_enum_split(uint32_t parts, uint32_t after_levels) {
  set_enum_split(parts, after_levels);
  return PM_SUCCESS;
}

pm_status_t pm_set_enum_presplit(uint32_t slice_entries) {
  set_enum_presplit(slice_entries);
  return PM_SUCCESS;
}


pm_status_t pm_set_walk_presplit(uint32_t slice_entries) {
  set_walk_presplit(slice_entries);
  return PM_SUCCESS;
}

pm_status_t pm_set_walk_table_entries(uint32_t entries) {
  PM_REQUIRE(entries >= 1024 && entries <= (1u << 20) && !(entries & (entries - 1)),
             "entries must be a power of two in [1024, 2^20]");
  set_walk_table_entries(entries);
  return PM_SUCCESS;
}

pm_status_t pm_set_enum_table_entries(uint32_t entries) {
  PM_REQUIRE(entries >= 1024 && entries <= (1u << 20) && !(entries & (entries - 1)),
             "entries must be a power of two in [1024, 2^20]");
  set_enum_table_entries(entries);
  return PM_SUCCESS;
}

pm_status_t pm_set_noalloc_table_entries(uint32_t entries) {
  PM_REQUIRE(entries >= 32 && entries <= (1u << 16) && !(entries & (entries - 1)),
             "entries must be a power of two in [32, 65536]");
  set_noalloc_table_entries(entries);
  return PM_SUCCESS;
}

uint32_t pm_noalloc_last_rounds(void) { return noalloc_last_rounds(); }

pm_status_t pm_set_enum_tail_swap(uint32_t ratio) {
  set_enum_tail_swap(ratio);
  return PM_SUCCESS;
}

pm_status_t pm_set_walk_tail_swap(uint32_t ratio) {
  set_walk_tail_swap(ratio);
  return PM_SUCCESS;
}

pm_status_t pm_set_enum_count_memo(int32_t enabled) {
  set_enum_count_memo(enabled != 0);
  return PM_SUCCESS;
}

pm_status_t pm_set_walk_tail_state_memo(int32_t enabled) {
  set_walk_tail_state_memo(enabled != 0);
  return PM_SUCCESS;
}

pm_status_t pm_set_pair_tail(int32_t enumeration, int32_t walks) {
  set_pair_tail(true, enumeration != 0);
  set_pair_tail(false, walks != 0);
  return PM_SUCCESS;
}

pm_status_t pm_set_enum_second_split(uint32_t entries) {
  set_enum_second_split(entries);
  return PM_SUCCESS;
}

pm_status_t pm_set_lcc_graph(int32_t enabled) {
  set_lcc_graph(enabled != 0);
  return PM_SUCCESS;
}

pm_status_t pm_set_lcc_label_stream(int32_t enabled) {
  set_lcc_label_stream(enabled != 0);
  return PM_SUCCESS;
}

pm_status_t pm_set_walk_budget_ms(double ms) {
  PM_REQUIRE(ms > 0, "budget must be positive");
  set_walk_budget_ns(static_cast<uint64_t>(ms * 1e6));
  return PM_SUCCESS;
}

int32_t pm_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

pm_status_t pm_template_dump_constraints(const uint64_t* p_offsets, const uint32_t* p_adj, const uint64_t* p_labels,
                                         uint32_t p_vertex_count, uint64_t p_edge_count, char* buf, size_t cap,
                                         size_t* needed) {
  PM_REQUIRE(p_offsets && (p_adj || p_edge_count == 0), "null argument");
  PM_REQUIRE(p_offsets[0] == 0, "pattern offsets must start at 0");
  for (uint32_t i = 0; i < p_vertex_count; ++i)
    PM_REQUIRE(p_offsets[i] <= p_offsets[i + 1], "pattern offsets must not decrease");
  PM_REQUIRE(p_offsets[p_vertex_count] == p_edge_count, "pattern offsets do not end at the edge count");
  for (uint64_t e = 0; e < p_edge_count; ++e) PM_REQUIRE(p_adj[e] < p_vertex_count, "pattern edge out of range");
  return guarded([&]() -> pm_status_t {
    PatternGraph p;
    p.n = p_vertex_count;
    p.offsets.assign(p_offsets, p_offsets + p_vertex_count + 1);
    p.adj.assign(p_adj, p_adj + p_edge_count);
    p.labels = p_labels ? std::vector<uint64_t>(p_labels, p_labels + p_vertex_count)
                        : std::vector<uint64_t>(p_vertex_count, 0);
    const std::string d = dump_constraints(compile_constraints(p));
    if (needed) *needed = d.size() + 1;
    if (buf && cap) {
      const size_t n = d.size() < cap - 1 ? d.size() : cap - 1;
      memcpy(buf, d.data(), n);
      buf[n] = 0;
    }
    return PM_SUCCESS;
  });
}

pm_status_t pm_query_step_walk_stats(const pm_query* q, int32_t row, uint64_t* scanned, uint64_t* descents) {
  PM_REQUIRE(q, "query is NULL");
  PM_REQUIRE(row >= 0 && static_cast<size_t>(row) < q->impl.walk_stats.size(), "row out of range");
  if (scanned) *scanned = q->impl.walk_stats[row].first;
  if (descents) *descents = q->impl.walk_stats[row].second;
  return PM_SUCCESS;
}

pm_status_t pm_query_stats(const pm_query* q, uint64_t* exact_resolutions, uint64_t* overflow_retries) {
  PM_REQUIRE(q, "query is NULL");
  if (exact_resolutions) *exact_resolutions = q->impl.exact_resolutions;
  if (overflow_retries) *overflow_retries = q->impl.overflow_retries;
  return PM_SUCCESS;
}

pm_status_t pm_query_graph_stat(pm_query* q, int32_t threads, uint32_t* n_labels, uint64_t* labels,
                                uint64_t* vertex_total, uint64_t* edge_total, uint64_t* at_least) {
  PM_REQUIRE(q, "null argument");
  PM_REQUIRE(threads >= 1, "thread count must be at least 1");
  return guarded([&]() -> pm_status_t {
    const GraphStat gs = q->impl.graph_stat(threads);
    const uint32_t n = gs.slots;
    if (n_labels) *n_labels = n;
    for (uint32_t a = 0; a < n; ++a) {
      if (labels) labels[a] = gs.label_of_slot[a];
      if (vertex_total) vertex_total[a] = gs.vertex_total[a];
      for (uint32_t b = 0; b < n; ++b) {
        if (edge_total) edge_total[a * n + b] = gs.edge_total[a * n + b];
        if (at_least)
          for (uint32_t i = 0; i < GraphStat::kMaxAtLeast; ++i)
            at_least[(static_cast<size_t>(a) * n + b) * 64 + i] =
                gs.at_least[(static_cast<size_t>(a) * n + b) * GraphStat::kMaxAtLeast + i];
      }
    }
    return PM_SUCCESS;
  });
}

pm_status_t pm_query_aborted_step(const pm_query* q, int32_t* step, double* step_ms, uint64_t* scanned,
                                  uint64_t* hops) {
  PM_REQUIRE(q, "null argument");
  if (q->impl.aborted_kind < 0) return fail(PM_FAILURE, "no step of this query was cut short");
  if (step) *step = q->impl.aborted_kind;
  if (step_ms) *step_ms = q->impl.aborted_ms;
  if (scanned) *scanned = q->impl.aborted_scanned;
  if (hops) *hops = q->impl.aborted_hops;
  return PM_SUCCESS;
}

void pm_query_destroy(pm_query* q) { delete q; }

namespace {
PatternGraph pattern_from_csr(const uint64_t* p_offsets, const uint32_t* p_adj, const uint64_t* p_labels,
                              uint32_t p_vertex_count, uint64_t p_edge_count) {
  if (!p_offsets || (!p_adj && p_edge_count)) throw PmError{PM_E_INVALID_ARG, "null template buffer"};
  if (p_offsets[0] != 0) throw PmError{PM_E_INVALID_ARG, "pattern offsets must start at 0"};
  for (uint32_t i = 0; i < p_vertex_count; ++i)
    if (p_offsets[i] > p_offsets[i + 1]) throw PmError{PM_E_INVALID_ARG, "pattern offsets must not decrease"};
  if (p_offsets[p_vertex_count] != p_edge_count)
    throw PmError{PM_E_INVALID_ARG, "pattern offsets do not end at the edge count"};
  for (uint64_t e = 0; e < p_edge_count; ++e)
    if (p_adj[e] >= p_vertex_count) throw PmError{PM_E_INVALID_ARG, "pattern edge out of range"};
  if (p_vertex_count > 64) throw PmError{PM_E_PATTERN_TOO_LARGE, "templates of more than 64 vertices"};
  PatternGraph p;
  p.n = p_vertex_count;
  p.offsets.assign(p_offsets, p_offsets + p_vertex_count + 1);
  p.adj.assign(p_adj, p_adj + p_edge_count);
  p.labels = p_labels ? std::vector<uint64_t>(p_labels, p_labels + p_vertex_count)
                      : std::vector<uint64_t>(p_vertex_count, 0);
  return p;
}

double ms_between(ServeRequest::Clock::time_point a, ServeRequest::Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

void fill_result(const ServeRequest& r, pm_request_result* out) {
  if (!out) return;
  out->status = r.status;
  out->n_records = static_cast<int32_t>(r.records.size());
  out->match_count = r.match_count;
  const bool admitted = r.t_admit.time_since_epoch().count() != 0;
  out->queue_ms = admitted ? ms_between(r.t_submit, r.t_admit) : ms_between(r.t_submit, r.t_done);
  out->run_ms = admitted ? ms_between(r.t_admit, r.t_done) : 0.0;
  out->latency_ms = ms_between(r.t_submit, r.t_done);
  out->gpu_ms = r.gpu_ms;
  out->charged_bytes = r.bytes;
}

std::shared_ptr<ServeRequest> finished_request(pm_server* s, uint64_t ticket) {
  bool done = false;
  auto r = s->impl->find(ticket, &done);
  if (!r) throw PmError{PM_E_INVALID_ARG, "unknown ticket"};
  if (!done) throw PmError{PM_E_BUSY, "request still queued or running"};
  return r;
}
}  // namespace

pm_status_t pm_server_create(pm_graph* g, const pm_server_config* config, pm_server** out) {
  PM_REQUIRE(g && config && out, "null argument");
  PM_REQUIRE(config->slots >= 1, "slots must be at least 1");
  return guarded([&]() -> pm_status_t {
    g->impl.to_device(g->impl.device >= 0 ? g->impl.device : 0);
    auto* s = new pm_server();
    try {
      s->impl = std::make_unique<Server>(&g->impl, config->slots, config->memory_budget, config->walk_share);
    } catch (...) {
      delete s;
      throw;
    }
    *out = s;
    return PM_SUCCESS;
  });
}

pm_status_t pm_server_submit(pm_server* s, const uint64_t* p_offsets, const uint32_t* p_adj,
                             const uint64_t* p_labels, uint32_t p_vertex_count, uint64_t p_edge_count,
                             uint32_t flags, uint64_t* ticket) {
  PM_REQUIRE(s && ticket, "null argument");
  return guarded([&]() -> pm_status_t {
    *ticket = s->impl->submit(pattern_from_csr(p_offsets, p_adj, p_labels, p_vertex_count, p_edge_count), flags);
    return PM_SUCCESS;
  });
}

pm_status_t pm_server_poll(pm_server* s, uint64_t ticket, int* done, pm_request_result* result) {
  PM_REQUIRE(s && done, "null argument");
  return guarded([&]() -> pm_status_t {
    bool d = false;
    auto r = s->impl->find(ticket, &d);
    if (!r) throw PmError{PM_E_INVALID_ARG, "unknown ticket"};
    *done = d ? 1 : 0;
    if (d) fill_result(*r, result);
    return PM_SUCCESS;
  });
}

pm_status_t pm_server_wait(pm_server* s, uint64_t ticket, double timeout_ms, pm_request_result* result) {
  PM_REQUIRE(s, "server is NULL");
  return guarded([&]() -> pm_status_t {
    if (!s->impl->wait(ticket, timeout_ms)) return fail(PM_E_TIMEOUT, "request not finished within the timeout");
    fill_result(*finished_request(s, ticket), result);
    return PM_SUCCESS;
  });
}

pm_status_t pm_server_records(pm_server* s, uint64_t ticket, pm_step_record* records, int32_t cap,
                              int32_t* n_records) {
  PM_REQUIRE(s, "server is NULL");
  return guarded([&]() -> pm_status_t {
    auto r = finished_request(s, ticket);
    const int32_t n = static_cast<int32_t>(r->records.size());
    for (int32_t i = 0; records && i < n && i < cap; ++i) records[i] = r->records[i];
    if (n_records) *n_records = n;
    return PM_SUCCESS;
  });
}

pm_status_t pm_server_export(pm_server* s, uint64_t ticket, uint64_t* cand_masks, uint8_t* edge_active,
                             uint8_t* vertex_active) {
  PM_REQUIRE(s, "server is NULL");
  return guarded([&]() -> pm_status_t {
    auto r = finished_request(s, ticket);
    if (!(r->flags & kSubmitExportState)) return fail(PM_E_INVALID_ARG, "request was not submitted with PM_SUBMIT_EXPORT_STATE");
    if (r->status != PM_SUCCESS) return fail(r->status, "request failed: " + r->error);
    if (cand_masks && !r->cand.empty()) memcpy(cand_masks, r->cand.data(), r->cand.size() * 8);
    if (edge_active && !r->eact.empty()) memcpy(edge_active, r->eact.data(), r->eact.size());
    if (vertex_active && !r->vact.empty()) memcpy(vertex_active, r->vact.data(), r->vact.size());
    return PM_SUCCESS;
  });
}

pm_status_t pm_server_cancel(pm_server* s, uint64_t ticket) {
  PM_REQUIRE(s, "server is NULL");
  return guarded([&]() -> pm_status_t {
    s->impl->cancel(ticket);
    return PM_SUCCESS;
  });
}

pm_status_t pm_server_release(pm_server* s, uint64_t ticket) {
  PM_REQUIRE(s, "server is NULL");
  return guarded([&]() -> pm_status_t {
    s->impl->release(ticket);
    return PM_SUCCESS;
  });
}

pm_status_t pm_server_stats_get(pm_server* s, pm_server_stats* stats) {
  PM_REQUIRE(s && stats, "null argument");
  return guarded([&]() -> pm_status_t {
    const ServerStats st = s->impl->stats();
    stats->queued = st.queued;
    stats->running = st.running;
    stats->done = st.done;
    stats->bytes_in_use = st.bytes_in_use;
    stats->peak_bytes = st.peak_bytes;
    stats->memory_budget = st.budget;
    stats->slots = st.slots;
    return PM_SUCCESS;
  });
}

void pm_server_destroy(pm_server* s) { delete s; }

pm_status_t pm_batch_run(pm_graph* g, const pm_template_csr* templates, uint32_t n, uint32_t slots,
                         uint64_t* match_counts, int32_t* statuses) {
  PM_REQUIRE(g && (templates || n == 0) && slots >= 1, "bad argument");
  return guarded([&]() -> pm_status_t {
    g->impl.to_device(g->impl.device >= 0 ? g->impl.device : 0);
    Server server(&g->impl, slots, 0);
    std::vector<uint64_t> tickets(n, 0);
    std::vector<int32_t> submit_status(n, PM_SUCCESS);
    for (uint32_t i = 0; i < n; ++i) {
      const pm_template_csr& t = templates[i];
      try {
        tickets[i] = server.submit(pattern_from_csr(t.offsets, t.adj, t.labels, t.vertex_count, t.edge_count), 0);
      } catch (const PmError& e) {
        submit_status[i] = e.code;
      }
    }
    for (uint32_t i = 0; i < n; ++i) {
      int32_t st = submit_status[i];
      uint64_t count = 0;
      if (st == PM_SUCCESS) {
        server.wait(tickets[i], -1.0);
        auto r = server.find(tickets[i]);
        st = r->status;
        count = r->match_count;
      }
      if (match_counts) match_counts[i] = count;
      if (statuses) statuses[i] = st;
    }
    return PM_SUCCESS;
  });
}

pm_status_t pm_autotune(pm_graph* g, const pm_template_csr* templates, uint32_t n, uint32_t max_per_group,
                        pm_tune_result* result) {
  PM_REQUIRE(g && templates && n > 0, "bad argument");
  return guarded([&]() -> pm_status_t {
    g->impl.to_device(g->impl.device >= 0 ? g->impl.device : 0);
    std::vector<PatternGraph> ps;
    for (uint32_t i = 0; i < n; ++i) {
      const pm_template_csr& t = templates[i];
      ps.push_back(pattern_from_csr(t.offsets, t.adj, t.labels, t.vertex_count, t.edge_count));
    }
    const TuneResult r = autotune(&g->impl, ps, max_per_group);
    if (result) {
      result->hub_degree = r.hub_degree;
      result->seg_entries = r.seg_entries;
      result->enum_presplit_memo = r.enum_presplit_memo;
      result->enum_presplit_plain = r.enum_presplit_plain;
      result->enum_table_entries = r.enum_table_entries;
      result->enum_tail_swap = r.enum_tail_swap;
      result->walk_tail_swap = r.walk_tail_swap;
      result->enum_count_memo = r.enum_count_memo;
      result->walk_tail_state_memo = r.walk_tail_state_memo;
      result->enum_pair_tail = r.enum_pair_tail;
      result->walk_pair_tail = r.walk_pair_tail;
      result->enum_second_split = r.enum_second_split;
      result->walk_presplit = r.walk_presplit;
      result->walk_table_entries = r.walk_table_entries;
      result->probes_memo = r.probes_memo;
      result->probes_plain = r.probes_plain;
      result->runs = r.runs;
    }
    return PM_SUCCESS;
  });
}

pm_status_t pm_set_enum_presplit_by_kind(uint32_t with_count_memo, uint32_t without_count_memo) {
  set_enum_presplit(true, with_count_memo);
  set_enum_presplit(false, without_count_memo);
  return PM_SUCCESS;
}

pm_status_t pm_enumerate_noalloc(const uint64_t* d_offsets, const uint32_t* d_adj, uint32_t vertex_count,
                                 uint64_t edge_count, int sorted_unique, const uint64_t* d_cand_masks,
                                 const uint32_t* d_edge_active_bits, const uint64_t* p_offsets,
                                 const uint32_t* p_adj, const uint64_t* p_labels, uint32_t p_vertex_count,
                                 uint64_t p_edge_count, uint64_t* d_count, void* stream) {
  PM_REQUIRE(d_offsets && d_cand_masks && d_count && p_offsets, "null argument");
  PM_REQUIRE((d_adj && d_edge_active_bits) || edge_count == 0, "null adjacency or edge-active buffer");
  PM_REQUIRE(p_adj || p_edge_count == 0, "null pattern adjacency");
  if (vertex_count > noalloc_max_vertices())
    return fail(PM_E_INVALID_ARG,
                "pm_enumerate_noalloc: graph of " + std::to_string(vertex_count) +
                    " vertices exceeds the maximum of 67108864 (fixed 64 MiB scratch); use pm_query_run");
  if (p_vertex_count == 0 || p_vertex_count > 56)
    return fail(PM_E_PATTERN_TOO_LARGE, "pm_enumerate_noalloc: template of " + std::to_string(p_vertex_count) +
                                            " vertices; 1 to 56 supported (56-bit role masks)");
  PM_REQUIRE(p_offsets[0] == 0, "pattern offsets must start at 0");
  for (uint32_t i = 0; i < p_vertex_count; ++i)
    PM_REQUIRE(p_offsets[i] <= p_offsets[i + 1], "pattern offsets must not decrease");
  PM_REQUIRE(p_offsets[p_vertex_count] == p_edge_count, "pattern offsets do not end at the edge count");
  for (uint64_t e = 0; e < p_edge_count; ++e) PM_REQUIRE(p_adj[e] < p_vertex_count, "pattern edge out of range");
  return guarded([&]() -> pm_status_t {
    PatternGraph p;
    p.n = p_vertex_count;
    p.offsets.assign(p_offsets, p_offsets + p_vertex_count + 1);
    p.adj.assign(p_adj, p_adj + p_edge_count);
    p.labels = p_labels ? std::vector<uint64_t>(p_labels, p_labels + p_vertex_count)
                        : std::vector<uint64_t>(p_vertex_count, 0);
    const QueryConstraints qc = compile_constraints(p);
    const CompiledConstraint cc = compile_enumeration(qc.enumeration, p.labels);
    PM_REQUIRE(!cc.programs.empty(), "template has no enumeration walk");
    const DevGraph g{vertex_count, edge_count, d_offsets, d_adj, nullptr, sorted_unique ? 1 : 0};
    enumerate_noalloc(g, d_cand_masks, d_edge_active_bits, cc.programs[0], cc.max_state_words, d_count,
                      static_cast<cudaStream_t>(stream));
    return PM_SUCCESS;
  });
}


// ---- batched form ---------------------------------------------------------
pm_status_t pm_fused_batch_run(pm_graph* g, const pm_template_csr* templates, uint32_t n, uint32_t flags,
                               pm_fused_batch** out) {
  PM_REQUIRE(g && out && (templates || n == 0), "null argument");
  return guarded([&]() -> pm_status_t {
    std::vector<PatternGraph> ps;
    ps.reserve(n);
    for (uint32_t i = 0; i < n; ++i)
      ps.push_back(pattern_from_csr(templates[i].offsets, templates[i].adj, templates[i].labels,
                                    templates[i].vertex_count, templates[i].edge_count));
    g->impl.to_device(g->impl.device >= 0 ? g->impl.device : 0);
    auto* b = new pm_fused_batch();
    try {
      b->impl = std::make_unique<FusedBatch>(&g->impl, ps, (flags & PM_SUBMIT_PRUNE_ONLY) != 0);
      b->impl->run();
    } catch (...) {
      delete b;
      throw;
    }
    *out = b;
    return PM_SUCCESS;
  });
}

pm_status_t pm_fused_batch_result(const pm_fused_batch* b, uint32_t i, pm_request_result* result) {
  PM_REQUIRE(b && result, "null argument");
  PM_REQUIRE(i < b->impl->size(), "query index out of range");
  return guarded([&]() -> pm_status_t {
    FusedBatchItem& it = b->impl->item(i);
    *result = pm_request_result{};
    result->status = it.status;
    result->n_records = static_cast<int32_t>(it.q->records.size() + 1);
    result->match_count = it.q->match_count;
    result->run_ms = it.run_ms;
    result->latency_ms = it.run_ms;
    result->gpu_ms = it.q->total_ms;
    result->charged_bytes = it.q->device_bytes();
    return PM_SUCCESS;
  });
}

pm_status_t pm_fused_batch_records(const pm_fused_batch* b, uint32_t i, pm_step_record* records, int32_t cap,
                                   int32_t* n_records) {
  PM_REQUIRE(b, "null argument");
  PM_REQUIRE(i < b->impl->size(), "query index out of range");
  return guarded([&]() -> pm_status_t {
    QueryImpl& q = *b->impl->item(i).q;
    int32_t n = 0;
    for (const auto& r : q.records) {
      if (records && n < cap) records[n] = r;
      ++n;
    }
    if (records && n < cap) records[n] = q.final_record();
    ++n;
    if (n_records) *n_records = n;
    return PM_SUCCESS;
  });
}

pm_status_t pm_fused_batch_export(const pm_fused_batch* b, uint32_t i, uint64_t* cand_masks, uint8_t* edge_active,
                                  uint8_t* vertex_active) {
  PM_REQUIRE(b, "null argument");
  PM_REQUIRE(i < b->impl->size(), "query index out of range");
  return guarded([&]() -> pm_status_t {
    FusedBatchItem& it = b->impl->item(i);
    if (it.status != PM_SUCCESS) return fail(it.status, "query failed: " + it.error);
    it.q->export_state(cand_masks, edge_active, vertex_active);
    return PM_SUCCESS;
  });
}

pm_status_t pm_fused_batch_stats(const pm_fused_batch* b, uint64_t* rounds, uint64_t* shared_lcc_phases) {
  PM_REQUIRE(b, "null argument");
  if (rounds) *rounds = b->impl->rounds;
  if (shared_lcc_phases) *shared_lcc_phases = b->impl->fused_lcc_passes;
  return PM_SUCCESS;
}

void pm_fused_batch_destroy(pm_fused_batch* b) { delete b; }

pm_status_t pm_query_create_variant_from_csr(pm_graph* g, const uint64_t* p_offsets, const uint32_t* p_adj,
                                             const uint64_t* p_labels, uint32_t p_vertex_count,
                                             uint64_t p_edge_count, int32_t variant, pm_query** out) {
  PM_REQUIRE(g && out, "null argument");
  PM_REQUIRE(valid_variant(variant), "unknown walk variant or order flags");
  return guarded([&]() -> pm_status_t {
    return create_query(g, pattern_from_csr(p_offsets, p_adj, p_labels, p_vertex_count, p_edge_count), out,
                        variant);
  });
}

}  // extern "C"
