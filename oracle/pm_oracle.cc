// ORACLE — test infrastructure only.  A CPU restatement of the reference's
// PruneJuice pipeline (tahsinreza/pattenmatching_sharedmemory,
// src/patternmatching/multiple_label/), used by tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg as the checker.  The product never calls
// it.  Pinned against the reference's own compiled CPU path (oracle/Makefile)
// through the golden fixtures under tests/golden/.
//
// Semantics follow the reference file:line cited on each function.  With
// threads == 1 the per-vertex loops run in ascending vertex order, which is
// the canonical order of the reference's timing-dependent "alreadyMatched"
// shortcut (multiple_label_cc_cpu.tpp:107, pc :107/:127, tds :165); with
// threads > 1 the loops are OpenMP-parallel like the reference's, for timing.
// Template constraints come from the product's template compiler
// (constraints.cc), itself pinned against the reference's log.totem dumps.
#include <omp.h>

#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../pattenmatching_sharedmemory_gb300/csrc/constraints.h"
#include "../pattenmatching_sharedmemory_gb300/csrc/effectiveness.h"
#include "../pattenmatching_sharedmemory_gb300/csrc/generators.h"

using namespace pmgb;

namespace {

// Wall-clock limit of one run (bounded CPU-baseline samples): the loops and
// walks poll it and unwind once it passed; the run then reports a timeout.
std::atomic<bool> g_expired{false};
std::chrono::steady_clock::time_point g_deadline;
bool g_has_deadline = false;
thread_local uint32_t t_poll = 0;
inline bool expired() {
  if (!g_has_deadline) return false;
  if ((++t_poll & 1023u) == 0 && std::chrono::steady_clock::now() > g_deadline)
    g_expired.store(true, std::memory_order_relaxed);
  return g_expired.load(std::memory_order_relaxed);
}

struct PairHashO {
  size_t operator()(const std::pair<uint32_t, uint32_t>& x) const {
    return std::hash<uint32_t>()(x.first) ^ std::hash<uint32_t>()(x.second);
  }
};
using EdgeMemo = std::unordered_map<std::pair<uint32_t, uint32_t>, uint64_t, PairHashO>;

inline std::pair<uint32_t, uint32_t> undirected(uint32_t a, uint32_t b) {
  return a > b ? std::make_pair(a, b) : std::make_pair(b, a);
}

struct Results {
  uint64_t vertex = 0, edge = 0, match = 0, enumeration = 0;
  bool empty() const { return !vertex && !edge && !match && !enumeration; }
};

// MultipleLabelGlobalState<uint32_t> (multiple_label_common_cpu.h:24-59),
// one flag byte per vertex / CSR entry, one 64-bit role set per vertex.
struct State {
  const uint64_t* off;
  const uint32_t* adj;
  const uint64_t* lab;
  uint32_t V;
  uint64_t E;
  uint32_t k;
  std::vector<uint8_t> active, modified, scheduled, edge_active;
  std::vector<uint64_t> cand, matched, unmatch;
  uint64_t active_vertices, active_edges;
  bool parallel;       // LCC0 / LCC sweeps (deterministic in any order)
  bool nlcc_parallel;  // CC / PC / TDS / ENUMERATION source loops
  int64_t sample_stride = 1;  // timing samples: NLCC / ENUMERATION sources v % stride == 0
  int64_t enum_stride = 1;    // ENUMERATION only: sources v % enum_stride == 0
  bool sampled(int64_t v) const { return sample_stride <= 1 || v % sample_stride == 0; }
  bool enum_sampled(int64_t v) const { return sampled(v) && (enum_stride <= 1 || v % enum_stride == 0); }
  void mark_matched(uint32_t v, uint32_t p) {
    if (nlcc_parallel)
      __atomic_fetch_or(&matched[v], uint64_t(1) << p, __ATOMIC_RELAXED);
    else
      matched[v] |= uint64_t(1) << p;
  }
  bool is_matched(uint32_t v, uint32_t p) const {
    uint64_t w = nlcc_parallel ? __atomic_load_n(&matched[v], __ATOMIC_RELAXED) : matched[v];
    return w >> p & 1;
  }
  bool has(uint32_t v, uint32_t p) const { return cand[v] >> p & 1; }
};

// Second sweep shared by the CC, PC and TDS steps (multiple_label_cc_cpu.tpp:134-173,
// pc :150-186, tds :203-241): apply the roles to unmatch, deactivate empty
// vertices, and reschedule modified vertices and their neighbours.
// keep_schedule: the article drivers' CC/PC/TDS variants
// (multiple_label_test/*_{strict,backtrack}_cpu.tpp) leave a vertex's
// schedule flag as it was when no active entry leads to a modified vertex,
// instead of clearing it.
void apply_unmatch(State& s, Results& r, bool keep_schedule = false) {
  uint64_t ve = 0, me = 0;
#pragma omp parallel for reduction(+ : ve, me) if (s.parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v]) continue;
    s.matched[v] = 0;
    if (s.modified[v]) {
      me += __builtin_popcountll(s.unmatch[v]);
      s.cand[v] &= ~s.unmatch[v];
      if (s.cand[v] == 0) {
        s.active[v] = 0;
        ++ve;
      }
      s.scheduled[v] = 1;
      s.unmatch[v] = 0;
    } else {
      bool sched = false;
      for (uint64_t e = s.off[v]; e < s.off[v + 1]; ++e) {
        if (!s.edge_active[e]) continue;
        if (!s.modified[s.adj[e]]) continue;
        sched = true;
        break;
      }
      if (sched || !keep_schedule) s.scheduled[v] = sched;
    }
  }
  s.active_vertices -= ve;
  r.vertex = ve;
  r.match = me;
}

// LCC0 (multiple_label_lcc0_cpu.tpp:15-87).
Results step_lcc0(State& s, const QueryConstraints& qc) {
  Results r;
  uint64_t ve = 0, me = 0;
#pragma omp parallel for reduction(+ : ve, me) if (s.parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v]) continue;
    for (uint32_t p = 0; p < s.k; ++p) {
      if (!s.has(v, p)) continue;
      if (s.lab[v] != qc.local[p].origin_label) {
        ++me;
        s.cand[v] &= ~(uint64_t(1) << p);
      }
    }
    if (s.cand[v] == 0) {
      s.active[v] = 0;
      ++ve;
    }
  }
  s.active_vertices -= ve;
  r.vertex = ve;
  r.match = me;
  return r;
}

// LCC (multiple_label_lcc_cpu.tpp:20-151).
Results step_lcc(State& s, const QueryConstraints& qc) {
  Results r;
  uint64_t ee = 0;
#pragma omp parallel for reduction(+ : ee) if (s.parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v] || !s.scheduled[v] || expired()) continue;
    uint64_t nbr_set = 0;
    for (uint32_t p = 0; p < s.k; ++p)
      if (s.has(v, p)) nbr_set |= qc.local[p].neighbor_mask;
    std::unordered_map<uint64_t, size_t> counts;
    for (uint64_t e = s.off[v]; e < s.off[v + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t w = s.adj[e];
      if (!s.active[w]) continue;
      if ((s.cand[w] & nbr_set) == 0) {
        ++ee;
        s.edge_active[e] = 0;
        s.modified[v] = 1;
        continue;
      }
      ++counts[s.lab[w]];
    }
    bool changed = false;
    for (uint32_t p = 0; p < s.k; ++p) {
      if (!s.has(v, p)) continue;
      const LocalConstraint& lc = qc.local[p];
      if (s.lab[v] != lc.origin_label) {
        s.unmatch[v] |= uint64_t(1) << p;
        changed = true;
        continue;
      }
      for (const auto& req : lc.required) {
        auto it = counts.find(req.first);
        size_t have = it == counts.end() ? 0 : it->second;
        if (have < req.second) {
          s.unmatch[v] |= uint64_t(1) << p;
          changed = true;
          break;
        }
      }
    }
    if (changed) s.modified[v] = 1;
  }
  uint64_t ve = 0, me = 0;
#pragma omp parallel for reduction(+ : ve, me) if (s.parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v]) continue;
    if (s.modified[v]) {
      me += __builtin_popcountll(s.unmatch[v]);
      s.cand[v] &= ~s.unmatch[v];
      if (s.cand[v] == 0) {
        s.active[v] = 0;
        ++ve;
      }
      s.scheduled[v] = 1;
      s.unmatch[v] = 0;
    } else {
      bool sched = false;
      for (uint64_t e = s.off[v]; e < s.off[v + 1]; ++e) {
        if (!s.edge_active[e]) continue;
        if (!s.modified[s.adj[e]]) continue;
        sched = true;
        break;
      }
      s.scheduled[v] = sched;
    }
  }
  s.active_vertices -= ve;
  s.active_edges -= ee;
  r.vertex = ve;
  r.edge = ee;
  r.match = me;
  return r;
}

// CC walk (multiple_label_cc_cpu.tpp:13-70).  The memo is keyed by the
// undirected edge; it is tested with the current cycle position and filled
// with the next template vertex id, and never rolled back within one source.
bool cc_walk(State& s, const CycleConstraint& c, EdgeMemo& memo, uint32_t source, uint32_t cur, size_t start,
             size_t remaining) {
  if (expired()) return false;
  const size_t L = c.length();
  if (remaining == 1) {
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t w = s.adj[e];
      if (!s.active[w]) continue;
      if (w == source) return true;
    }
    return false;
  }
  const size_t cur_pos = (start + L - remaining) % L;
  const size_t next_pos = (start + L - (remaining - 1)) % L;
  const uint32_t next_role = c.ids[next_pos];
  for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
    if (!s.edge_active[e]) continue;
    uint32_t w = s.adj[e];
    if (!s.active[w]) continue;
    if (!s.has(w, next_role)) continue;
    auto key = undirected(cur, w);
    auto it = memo.find(key);
    if (it != memo.end() && (it->second >> cur_pos & 1)) continue;
    memo[key] |= uint64_t(1) << next_role;
    if (cc_walk(s, c, memo, source, w, start, remaining - 1)) {
      s.mark_matched(w, next_role);
      return true;
    }
  }
  return false;
}

// CC step (multiple_label_cc_cpu.tpp:79-183).
Results step_cc(State& s, const CycleConstraint& c) {
  Results r;
  EdgeMemo memo;
#pragma omp parallel for private(memo) if (s.nlcc_parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v] || !s.sampled(vi) || expired()) continue;
    bool changed = false;
    for (size_t pos = 0; pos < c.length(); ++pos) {
      uint32_t role = c.ids[pos];
      if (!s.has(v, role)) continue;
      if (s.is_matched(v, role)) continue;
      memo.clear();
      if (!cc_walk(s, c, memo, v, v, pos, c.length())) {
        s.unmatch[v] |= uint64_t(1) << role;
        changed = true;
      }
    }
    if (changed) s.modified[v] = 1;
  }
  apply_unmatch(s, r);
  return r;
}

// PC walk (multiple_label_pc_cpu.tpp:12-81).
bool pc_walk(State& s, const PathConstraint& pc, bool reverse, EdgeMemo& memo, uint32_t source, uint32_t cur,
             size_t remaining) {
  if (expired()) return false;
  const size_t L = pc.length();
  const size_t cur_pos = reverse ? remaining : (L - remaining - 1);
  const size_t next_pos = reverse ? remaining - 1 : (L - remaining);
  const uint32_t next_role = pc.ids[next_pos];
  if (remaining == 1) {
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t w = s.adj[e];
      if (!s.active[w]) continue;
      if (!s.has(w, next_role)) continue;
      if (source != w) {
        s.mark_matched(w, next_role);
        return true;
      }
    }
    return false;
  }
  for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
    if (!s.edge_active[e]) continue;
    uint32_t w = s.adj[e];
    if (!s.active[w]) continue;
    if (!s.has(w, next_role)) continue;
    auto key = undirected(cur, w);
    auto it = memo.find(key);
    if (it != memo.end() && (it->second >> cur_pos & 1)) continue;
    memo[key] |= uint64_t(1) << next_role;
    if (pc_walk(s, pc, reverse, memo, source, w, remaining - 1)) return true;
  }
  return false;
}

// PC step (multiple_label_pc_cpu.tpp:84-197).
Results step_pc(State& s, const PathConstraint& pc) {
  Results r;
  EdgeMemo memo;
  const size_t L = pc.length();
#pragma omp parallel for private(memo) if (s.nlcc_parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v] || !s.sampled(vi) || expired()) continue;
    if (s.lab[v] != pc.initial_label) continue;
    bool changed = false;
    for (int end = 0; end < 2; ++end) {
      uint32_t role = end == 0 ? pc.ids[0] : pc.ids[L - 1];
      if (!s.has(v, role)) continue;
      if (s.is_matched(v, role)) continue;
      memo.clear();
      if (!pc_walk(s, pc, end == 1, memo, v, v, L - 1)) {
        s.unmatch[v] |= uint64_t(1) << role;
        changed = true;
      }
    }
    if (changed) s.modified[v] = 1;
  }
  apply_unmatch(s, r);
  return r;
}

// TDS walk (multiple_label_tds_cpu.tpp:14-127).
struct TdsMemo {
  std::unordered_map<uint32_t, std::unordered_map<uint32_t, std::vector<std::vector<uint32_t>>>> hyp;
  EdgeMemo edges;
  std::vector<uint32_t> history;
  std::vector<uint32_t> stored;
};

bool tds_walk(State& s, const Walk& w, TdsMemo& m, uint32_t source, uint32_t cur, size_t pos) {
  if (pos == w.length()) return true;
  if (expired()) return false;
  const int move = w.moves[pos];
  if (move == kVertexNoStore || move == kVertexStore) {
    const uint32_t cur_role = w.ids[pos - 1];
    const uint32_t next_role = w.ids[pos];
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t nb = s.adj[e];
      if (!s.active[nb]) continue;
      if (!s.has(nb, next_role)) continue;
      auto key = undirected(cur, nb);
      auto it = m.edges.find(key);
      if (it != m.edges.end() && (it->second >> cur_role & 1)) continue;
      auto hv = m.hyp.find(nb);
      if (hv != m.hyp.end()) {
        auto hr = hv->second.find(next_role);
        if (hr != hv->second.end()) {
          bool seen = false;
          for (const auto& h : hr->second)
            if (h == m.stored) {
              seen = true;
              break;
            }
          if (seen) continue;
        }
      }
      if (move == kVertexStore) m.stored.push_back(nb);
      m.hyp[nb][next_role].push_back(m.stored);
      m.history.push_back(nb);
      m.edges[key] |= uint64_t(1) << next_role;
      if (tds_walk(s, w, m, source, nb, pos + 1)) {
        s.mark_matched(nb, next_role);
        return true;
      }
      m.history.pop_back();
      if (move == kVertexStore) m.stored.pop_back();
    }
  } else if (move == kCheck) {
    const uint32_t target = m.history[w.back[pos]];
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t nb = s.adj[e];
      if (!s.active[nb]) continue;
      if (nb != target) continue;
      if (tds_walk(s, w, m, source, cur, pos + 1)) return true;
    }
  } else {  // kMoveBack
    const uint32_t back_to = m.history[w.back[pos]];
    if (tds_walk(s, w, m, source, back_to, pos + 1)) return true;
  }
  return false;
}

// TDS step (multiple_label_tds_cpu.tpp:136-244).
Results step_tds(State& s, const TemplateConstraint& t) {
  Results r;
  TdsMemo m;
#pragma omp parallel for private(m) if (s.nlcc_parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v] || !s.sampled(vi) || expired()) continue;
    bool changed = false;
    for (const auto& kv : t.walks) {
      uint32_t role = kv.first;
      if (!s.has(v, role)) continue;
      if (s.is_matched(v, role)) continue;
      m.hyp.clear();
      m.edges.clear();
      m.history.clear();
      m.history.push_back(v);
      m.stored.clear();
      if (!tds_walk(s, kv.second, m, v, v, 1)) {
        s.unmatch[v] |= uint64_t(1) << role;
        changed = true;
      }
    }
    if (changed) s.modified[v] = 1;
  }
  apply_unmatch(s, r);
  return r;
}

// ---- the article drivers' NLCC variants (test_article/CMakeLists.txt:12-33)
// Strict (multiple_label_test/*_strict_cpu.tpp): walks bind no vertex twice
// (isInVector over the history, source included) and keep no memo.
// Backtrack (*_backtrack_cpu.tpp, built with work aggregation, early
// termination and multiple validation): CC and PC skip a (vertex, template
// vertex) pair already visited by the source's walk; TDS keeps only the
// hypothesis memo.  Every success marks alreadyMatched as the regular walks do.
bool in_history(const std::vector<uint32_t>& h, uint32_t v) {
  for (uint32_t x : h)
    if (x == v) return true;
  return false;
}

// cc_strict_cpu.tpp:13-64
bool cc_strict_walk(State& s, const CycleConstraint& c, std::vector<uint32_t>& hist, uint32_t source, uint32_t cur,
                    size_t start, size_t remaining) {
  if (expired()) return false;
  const size_t L = c.length();
  if (remaining == 1) {
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t w = s.adj[e];
      if (!s.active[w]) continue;
      if (w == source) return true;
    }
    return false;
  }
  const uint32_t next_role = c.ids[(start + L - (remaining - 1)) % L];
  for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
    if (!s.edge_active[e]) continue;
    uint32_t w = s.adj[e];
    if (!s.active[w] || !s.has(w, next_role) || in_history(hist, w)) continue;
    hist.push_back(w);
    if (cc_strict_walk(s, c, hist, source, w, start, remaining - 1)) {
      s.mark_matched(w, next_role);
      return true;
    }
    hist.pop_back();
  }
  return false;
}

// cc_backtrack_cpu.tpp:13-78 (early termination, multiple validation)
bool cc_backtrack_walk(State& s, const CycleConstraint& c, std::unordered_map<uint32_t, uint64_t>& seen,
                       uint32_t source, uint32_t cur, size_t start, size_t remaining) {
  if (expired()) return false;
  const size_t L = c.length();
  if (remaining == 1) {
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t w = s.adj[e];
      if (!s.active[w]) continue;
      if (w == source) return true;
    }
    return false;
  }
  const uint32_t next_role = c.ids[(start + L - (remaining - 1)) % L];
  for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
    if (!s.edge_active[e]) continue;
    uint32_t w = s.adj[e];
    if (!s.active[w] || !s.has(w, next_role)) continue;
    auto it = seen.find(w);
    if (it != seen.end() && (it->second >> next_role & 1)) continue;
    seen[w] |= uint64_t(1) << next_role;
    if (cc_backtrack_walk(s, c, seen, source, w, start, remaining - 1)) {
      s.mark_matched(w, next_role);
      return true;
    }
  }
  return false;
}

// CC step of either variant (cc_strict_cpu.tpp:72-178, cc_backtrack_cpu.tpp:86-190).
Results step_cc_variant(State& s, const CycleConstraint& c, int variant) {
  Results r;
  std::vector<uint32_t> hist;
  std::unordered_map<uint32_t, uint64_t> seen;
#pragma omp parallel for private(hist, seen) if (s.nlcc_parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v] || !s.sampled(vi) || expired()) continue;
    bool changed = false;
    for (size_t pos = 0; pos < c.length(); ++pos) {
      uint32_t role = c.ids[pos];
      if (!s.has(v, role) || s.is_matched(v, role)) continue;
      bool ok;
      if (variant == 1) {
        hist.assign(1, v);
        ok = cc_strict_walk(s, c, hist, v, v, pos, c.length());
      } else {
        seen.clear();
        ok = cc_backtrack_walk(s, c, seen, v, v, pos, c.length());
      }
      if (!ok) {
        s.unmatch[v] |= uint64_t(1) << role;
        changed = true;
      }
    }
    if (changed) s.modified[v] = 1;
  }
  apply_unmatch(s, r, true);
  return r;
}

// pc_strict_cpu.tpp:12-76 / pc_backtrack_cpu.tpp:12-78
bool pc_variant_walk(State& s, const PathConstraint& pc, bool reverse, int variant, std::vector<uint32_t>& hist,
                     std::unordered_map<uint32_t, uint64_t>& seen, uint32_t source, uint32_t cur, size_t remaining) {
  if (expired()) return false;
  const size_t L = pc.length();
  const uint32_t next_role = pc.ids[reverse ? remaining - 1 : (L - remaining)];
  auto blocked = [&](uint32_t w) {
    if (variant == 1) return in_history(hist, w);
    auto it = seen.find(w);
    return it != seen.end() && (it->second >> next_role & 1) != 0;
  };
  if (remaining == 1) {
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t w = s.adj[e];
      if (!s.active[w] || !s.has(w, next_role) || blocked(w)) continue;
      if (source != w) {
        s.mark_matched(w, next_role);
        return true;
      }
    }
    return false;
  }
  for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
    if (!s.edge_active[e]) continue;
    uint32_t w = s.adj[e];
    if (!s.active[w] || !s.has(w, next_role) || blocked(w)) continue;
    if (variant == 1)
      hist.push_back(w);
    else
      seen[w] |= uint64_t(1) << next_role;
    if (pc_variant_walk(s, pc, reverse, variant, hist, seen, source, w, remaining - 1)) return true;
    if (variant == 1) hist.pop_back();
  }
  return false;
}

// PC step of either variant (pc_strict_cpu.tpp:78-189).
Results step_pc_variant(State& s, const PathConstraint& pc, int variant) {
  Results r;
  std::vector<uint32_t> hist;
  std::unordered_map<uint32_t, uint64_t> seen;
  const size_t L = pc.length();
#pragma omp parallel for private(hist, seen) if (s.nlcc_parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v] || !s.sampled(vi) || expired()) continue;
    if (s.lab[v] != pc.initial_label) continue;
    bool changed = false;
    for (int end = 0; end < 2; ++end) {
      uint32_t role = end == 0 ? pc.ids[0] : pc.ids[L - 1];
      if (!s.has(v, role) || s.is_matched(v, role)) continue;
      hist.assign(1, v);
      seen.clear();
      if (!pc_variant_walk(s, pc, end == 1, variant, hist, seen, v, v, L - 1)) {
        s.unmatch[v] |= uint64_t(1) << role;
        changed = true;
      }
    }
    if (changed) s.modified[v] = 1;
  }
  apply_unmatch(s, r, true);
  return r;
}

// tds_strict_cpu.tpp:12-98 (history injective, no memo) and
// tds_backtrack_cpu.tpp:12-116 (hypothesis memo only).
bool tds_variant_walk(State& s, const Walk& w, int variant, TdsMemo& m, uint32_t source, uint32_t cur, size_t pos) {
  if (pos == w.length()) return true;
  if (expired()) return false;
  const int move = w.moves[pos];
  if (move == kVertexNoStore || move == kVertexStore) {
    const uint32_t next_role = w.ids[pos];
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t nb = s.adj[e];
      if (!s.active[nb] || !s.has(nb, next_role)) continue;
      if (variant == 1) {
        if (in_history(m.history, nb)) continue;
      } else {
        auto hv = m.hyp.find(nb);
        if (hv != m.hyp.end()) {
          auto hr = hv->second.find(next_role);
          if (hr != hv->second.end()) {
            bool seen = false;
            for (const auto& h : hr->second)
              if (h == m.stored) seen = true;
            if (seen) continue;
          }
        }
        if (move == kVertexStore) m.stored.push_back(nb);
        m.hyp[nb][next_role].push_back(m.stored);
      }
      m.history.push_back(nb);
      if (tds_variant_walk(s, w, variant, m, source, nb, pos + 1)) {
        s.mark_matched(nb, next_role);
        return true;
      }
      m.history.pop_back();
      if (variant != 1 && move == kVertexStore) m.stored.pop_back();
    }
  } else if (move == kCheck) {
    const uint32_t target = m.history[w.back[pos]];
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t nb = s.adj[e];
      if (!s.active[nb] || nb != target) continue;
      if (tds_variant_walk(s, w, variant, m, source, cur, pos + 1)) return true;
    }
  } else {
    if (tds_variant_walk(s, w, variant, m, source, m.history[w.back[pos]], pos + 1)) return true;
  }
  return false;
}

// TDS step of either variant (tds_strict_cpu.tpp:100-195); unlike the
// regular TDS step the drivers advance to the next template constraint.
Results step_tds_variant(State& s, const TemplateConstraint& t, int variant) {
  Results r;
  TdsMemo m;
#pragma omp parallel for private(m) if (s.nlcc_parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v] || !s.sampled(vi) || expired()) continue;
    bool changed = false;
    for (const auto& kv : t.walks) {
      uint32_t role = kv.first;
      if (!s.has(v, role) || s.is_matched(v, role)) continue;
      m.hyp.clear();
      m.edges.clear();
      m.history.assign(1, v);
      m.stored.clear();
      if (!tds_variant_walk(s, kv.second, variant, m, v, v, 1)) {
        s.unmatch[v] |= uint64_t(1) << role;
        changed = true;
      }
    }
    if (changed) s.modified[v] = 1;
  }
  apply_unmatch(s, r, true);
  return r;
}

// ENUMERATION walk (multiple_label_enumeration_cpu.tpp:39-118): injective
// embeddings following the walk; CHECK follows only the first matching entry.
uint64_t enum_walk(const State& s, const Walk& w, std::vector<uint32_t>& history, uint32_t cur, size_t pos) {
  if (pos == w.length()) return 1;
  if (expired()) return 0;
  const int move = w.moves[pos];
  uint64_t count = 0;
  if (move == kVertexNoStore || move == kVertexStore) {
    const uint32_t next_role = w.ids[pos];
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t nb = s.adj[e];
      if (!s.active[nb]) continue;
      if (!s.has(nb, next_role)) continue;
      bool seen = false;
      for (uint32_t h : history)
        if (h == nb) {
          seen = true;
          break;
        }
      if (seen) continue;
      history.push_back(nb);
      count += enum_walk(s, w, history, nb, pos + 1);
      history.pop_back();
    }
  } else if (move == kCheck) {
    const uint32_t target = history[w.back[pos]];
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t nb = s.adj[e];
      if (!s.active[nb]) continue;
      if (nb != target) continue;
      return enum_walk(s, w, history, cur, pos + 1);
    }
  } else {
    return enum_walk(s, w, history, history[w.back[pos]], pos + 1);
  }
  return count;
}

// ENUMERATION step (multiple_label_enumeration_cpu.tpp:126-174).
Results step_enumeration(State& s, const TemplateConstraint& t) {
  Results r;
  auto first = t.walks.cbegin();
  const uint32_t start_role = first->first;
  const Walk& w = first->second;
  uint64_t total = 0;
  std::vector<uint32_t> history;
#pragma omp parallel for reduction(+ : total) private(history) schedule(dynamic, 1000) if (s.nlcc_parallel)
  for (int64_t vi = 0; vi < s.V; ++vi) {
    uint32_t v = static_cast<uint32_t>(vi);
    if (!s.active[v] || !s.enum_sampled(vi) || expired()) continue;
    if (!s.has(v, start_role)) continue;
    history.clear();
    history.push_back(v);
    total += enum_walk(s, w, history, v, 1);
  }
  r.enumeration = total;
  return r;
}

}  // namespace

namespace {

// GraphStatCpu::compute (src/patternmatching/algorithms/graph_stat_cpu.tpp:
// 42-80) with `threads` OpenMP threads under the static schedule, run here
// one thread block after the other: each block keeps one label -> count
// accumulation that is never cleared between its vertices (the reference
// declares it outside the vertex loop), and GraphStat::addAccumulation
// (graph_stat.cc:103-114) counts a label-a vertex towards (a, b, i) when the
// accumulated b count has reached i, for i up to the template's maximum.
// The reference reads accumulationMaximumMap.at(a) once the accumulation
// holds anything; a label a without template neighbours then throws
// (PM_E_STATISTICS here).
GraphStat oracle_graph_stat(const State& s, const AccumulationMaximum& am, uint32_t threads) {
  const uint32_t S = am.slots;
  GraphStat gs;
  gs.slots = S;
  gs.label_of_slot = am.label_of_slot;
  gs.vertex_total.assign(S, 0);
  gs.edge_total.assign(static_cast<size_t>(S) * S, 0);
  gs.edge_outbound.assign(S, 0);
  gs.at_least.assign(static_cast<size_t>(S) * S * GraphStat::kMaxAtLeast, 0);
  auto slot = [&](uint64_t label) -> uint32_t {
    for (uint32_t a = 0; a < S; ++a)
      if (am.label_of_slot[a] == label) return a;
    throw_stat_missing("active vertex without a template label");
  };
  const StaticPartition part(s.V, threads);
  for (uint32_t t = 0; t < threads; ++t) {
    std::vector<uint64_t> acc(S, 0);
    bool any = false;
    for (uint64_t v = part.begin(t); v < part.end(t); ++v) {
      if (!s.active[v]) continue;
      const uint32_t a = slot(s.lab[v]);
      ++gs.vertex_total[a];
      for (uint64_t e = s.off[v]; e < s.off[v + 1]; ++e) {
        if (!s.edge_active[e]) continue;
        const uint32_t w = s.adj[e];
        if (!s.active[w]) continue;
        const uint32_t b = slot(s.lab[w]);
        ++gs.edge_total[a * S + b];
        ++gs.edge_outbound[a];
        ++acc[b];
        any = true;
      }
      if (!any) continue;
      if (!am.has_a[a]) throw_stat_missing("accumulationMaximumMap has no entry for an active label");
      for (uint32_t b = 0; b < S; ++b) {
        const uint32_t most = am.max[a * S + b];
        for (uint32_t i = 1; i <= most; ++i)
          if (acc[b] >= i) ++gs.at_least[(static_cast<size_t>(a) * S + b) * GraphStat::kMaxAtLeast + i];
      }
    }
  }
  return gs;
}

}  // namespace

extern "C" {

// Runs the reference pipeline (MultipleLabelCpu::runPatternMatching,
// multiple_label_cpu.cc:113-184, with MultipleLabelStep::getNextStep,
// multiple_label_step.cc:30-83) over a host CSR graph and template.
//   threads      1 = canonical sequential order; >1 OpenMP like the reference.
//   stop_before_enumeration  1 = end the run when the schedule reaches
//                ENUMERATION (pruning-only timing).
//   sample_stride  >1 = timing sample: CC/PC/TDS/ENUMERATION visit only
//                sources with id % sample_stride == 0 (results then differ
//                from the full run; used to bound CPU-baseline timing)
//                (bounded CPU-baseline samples); 0 = all.
// Outputs (any may be NULL): step records (as pm_step_record), final role
// sets, per-CSR-entry and per-vertex active flags, the matched count.
// Returns 0, or a negative status on bad input.
// Options of pmo_run_ex beyond pmo_run's.
struct pmo_options {
  int32_t threads;                  // LCC0 / LCC threads (deterministic in any order)
  int32_t nlcc_threads;             // CC / PC / TDS / ENUMERATION threads; 1 = canonical order
  int32_t stop_before_enumeration;  // 1 = end when the schedule reaches ENUMERATION
  int32_t variant;                  // 0 = the reference's walks; 1 = strict, 2 = backtrack
                                    // (the article drivers: TDS steps advance through
                                    // the template constraints, END instead of ENUMERATION)
  int64_t sample_stride;            // >1: CC/PC/TDS/ENUMERATION sources v % stride == 0 only
  int64_t enum_sample_stride;       // >1: ENUMERATION sources v % stride == 0 only (a
                                    // per-source sampled count; pruning unchanged)
  double deadline_ms;               // >0: wall-clock limit; the run returns -7 past it
  int64_t max_steps;                // >0: stop after that many steps (the last row names the next)
  int32_t order;                    // the article's order drivers (variants 1 / 2 only):
                                    // PM_ORDER_* bits of pm_gb300.h
  int32_t order_threads;            // their OpenMP thread count (statistics partition and
                                    // cost divisor); 0 = 1
};

int pmo_run_ex(const uint64_t* off, const uint32_t* adj, const uint64_t* lab, uint32_t V, uint64_t E,
               const uint64_t* p_off, const uint32_t* p_adj, const uint64_t* p_lab, uint32_t k,
               const pmo_options* opt, pm_step_record* records, int32_t cap, int32_t* n_records, uint64_t* cand_out,
               uint8_t* edge_active_out, uint8_t* vertex_active_out);

int pmo_run(const uint64_t* off, const uint32_t* adj, const uint64_t* lab, uint32_t V, uint64_t E,
            const uint64_t* p_off, const uint32_t* p_adj, const uint64_t* p_lab, uint32_t k, int threads,
            int stop_before_enumeration, int64_t sample_stride, pm_step_record* records, int32_t cap,
            int32_t* n_records, uint64_t* cand_out, uint8_t* edge_active_out, uint8_t* vertex_active_out) {
  pmo_options o{};
  o.threads = threads;
  o.nlcc_threads = threads;
  o.stop_before_enumeration = stop_before_enumeration;
  o.sample_stride = sample_stride;
  return pmo_run_ex(off, adj, lab, V, E, p_off, p_adj, p_lab, k, &o, records, cap, n_records, cand_out,
                    edge_active_out, vertex_active_out);
}

int pmo_run_ex(const uint64_t* off, const uint32_t* adj, const uint64_t* lab, uint32_t V, uint64_t E,
               const uint64_t* p_off, const uint32_t* p_adj, const uint64_t* p_lab, uint32_t k,
               const pmo_options* opt, pm_step_record* records, int32_t cap, int32_t* n_records, uint64_t* cand_out,
               uint8_t* edge_active_out, uint8_t* vertex_active_out) {
  const int threads = opt->threads;
  const int stop_before_enumeration = opt->stop_before_enumeration;
  const int64_t sample_stride = opt->sample_stride;
  g_expired.store(false);
  g_has_deadline = opt->deadline_ms > 0;
  if (g_has_deadline)
    g_deadline = std::chrono::steady_clock::now() +
                 std::chrono::microseconds(static_cast<int64_t>(opt->deadline_ms * 1000.0));
  try {
    PatternGraph pg;
    pg.n = k;
    pg.offsets.assign(p_off, p_off + k + 1);
    pg.adj.assign(p_adj, p_adj + p_off[k]);
    pg.labels.assign(p_lab, p_lab + k);
    QueryConstraints qc = compile_constraints(pg);
    State s;
    s.off = off;
    s.adj = adj;
    s.lab = lab;
    s.V = V;
    s.E = E;
    s.k = k;
    s.parallel = threads > 1;
    s.nlcc_parallel = opt->nlcc_threads > 1;
    s.sample_stride = sample_stride;
    s.enum_stride = opt->enum_sample_stride;
    const int max_threads = threads > opt->nlcc_threads ? threads : opt->nlcc_threads;
    if (max_threads >= 1) omp_set_num_threads(max_threads);
    s.active.assign(V, 1);
    s.modified.assign(V, 0);
    s.scheduled.assign(V, 1);
    s.edge_active.assign(E, 1);
    const uint64_t full = k == 64 ? ~uint64_t(0) : ((uint64_t(1) << k) - 1);
    s.cand.assign(V, full);
    s.matched.assign(V, 0);
    s.unmatch.assign(V, 0);
    s.active_vertices = V;
    s.active_edges = E;

    enum { START, END, LCC0, LCC, CC, PC, TDS, ENUM };
    int step = START;
    size_t next_cc = 0, next_pc = 0, next_tds = 0;
    Results res;
    const int order = opt->variant ? opt->order : 0;
    const bool dynamic = order & PM_ORDER_EFFECTIVENESS;
    const bool use_enumerate = order & PM_ORDER_ENUMERATE;
    const int order_threads = opt->order_threads > 0 ? opt->order_threads : 1;
    const AccumulationMaximum am = accumulation_maximum(pg);
    // The order drivers' NLCC steps erase the constraint they ran
    // (multiple_label_test/*_cpu.tpp, e.g. cc_backtrack :192); the dynamic
    // order picks by index among the remaining ones.
    std::vector<size_t> rem_cc, rem_pc, rem_tds;
    for (size_t i = 0; i < qc.cycles.size(); ++i) rem_cc.push_back(i);
    for (size_t i = 0; i < qc.paths.size(); ++i) rem_pc.push_back(i);
    for (size_t i = 0; i < qc.templates.size(); ++i) rem_tds.push_back(i);
    size_t chosen = 0;
    auto choose = [&]() -> int {
      const GraphStat gs = oracle_graph_stat(s, am, static_cast<uint32_t>(order_threads));
      std::vector<const CycleConstraint*> cs;
      std::vector<const PathConstraint*> ps;
      std::vector<const TemplateConstraint*> ts;
      for (size_t i : rem_cc) cs.push_back(&qc.cycles[i]);
      for (size_t i : rem_pc) ps.push_back(&qc.paths[i]);
      for (size_t i : rem_tds) ts.push_back(&qc.templates[i]);
      const OrderChoice c = choose_next_constraint(gs, cs, ps, ts, qc.enumeration, use_enumerate,
                                                   order & PM_ORDER_EARLY_ENUMERATION, 0.01, order_threads);
      chosen = c.index;
      return c.kind - PM_STEP_START;
    };
    auto advance = [&](int cur) -> int {
      if (dynamic) {
        switch (cur) {
          case START: return LCC;
          case LCC: return res.empty() ? choose() : LCC;
          case CC: rem_cc.erase(rem_cc.begin() + chosen); return LCC;
          case PC: rem_pc.erase(rem_pc.begin() + chosen); return LCC;
          case TDS: rem_tds.erase(rem_tds.begin() + chosen); return LCC;
          default: return END;
        }
      }
      switch (cur) {
        case START: return LCC0;
        case LCC0: return LCC;
        case LCC:
          if (!res.empty()) return LCC;
          if (next_cc < qc.cycles.size()) return CC;
          if (next_pc < qc.paths.size()) return PC;
          if (next_tds < qc.templates.size()) return TDS;
          return opt->variant && !use_enumerate ? END : ENUM;
        case CC: ++next_cc; return LCC;
        case PC: ++next_pc; return LCC;
        case TDS: ++next_tds; return LCC;
        default: return END;
      }
    };
    auto cc_index = [&]() { return dynamic ? rem_cc[chosen] : next_cc; };
    auto pc_index = [&]() { return dynamic ? rem_pc[chosen] : next_pc; };
    auto tds_index = [&]() { return dynamic ? rem_tds[chosen] : next_tds; };
    int32_t n = 0;
    double total_ms = 0;
    auto emit = [&](int kind, double ms, const Results& r) {
      total_ms += ms;
      if (records && n < cap) {
        pm_step_record& rec = records[n];
        rec.iteration = n;
        rec.step = kind;
        rec.step_ms = ms;
        rec.cumulative_ms = total_ms;
        rec.results.vertex_eliminated = r.vertex;
        rec.results.edge_eliminated = r.edge;
        rec.results.match_eliminated = r.match;
        rec.results.enumeration = r.enumeration;
        rec.active_vertex = s.active_vertices;
        rec.total_vertex = V;
        rec.active_edge = s.active_edges;
        rec.total_edge = E;
      }
      ++n;
    };
    // The dynamic order's driver never sets its first step
    // (test_order_multiple_label_cpu.cc:128-130 skip getNextStep under
    // ORDER_USE_DYNAMIC): its first iteration runs no step and logs a row
    // with an empty step name (START here), then goes to LCC; LCC0 never
    // runs.
    step = dynamic ? START : advance(START);
    int iteration = 0;
    bool finished = false;
    while (!finished && iteration < 1000) {
      if (step == CC || step == PC || step == TDS) std::fill(s.modified.begin(), s.modified.end(), 0);
      if (step == ENUM && stop_before_enumeration) break;
      if (opt->max_steps > 0 && n >= opt->max_steps) break;
      auto t0 = std::chrono::steady_clock::now();
      switch (step) {
        case LCC0: res = step_lcc0(s, qc); break;
        case LCC: res = step_lcc(s, qc); break;
        case CC: res = opt->variant ? step_cc_variant(s, qc.cycles[cc_index()], opt->variant)
                                    : step_cc(s, qc.cycles[next_cc]); break;
        case PC: res = opt->variant ? step_pc_variant(s, qc.paths[pc_index()], opt->variant)
                                    : step_pc(s, qc.paths[next_pc]); break;
        // MultipleLabelTdsCpu::compute never advances its constraint
        // iterator (multiple_label_tds_cpu.tpp:136-244, unlike cc :180 and
        // pc :186), so every TDS step checks template constraint 0.
        case TDS: res = opt->variant ? step_tds_variant(s, qc.templates[tds_index()], opt->variant)
                                     : step_tds(s, qc.templates[0]); break;
        case ENUM: res = step_enumeration(s, qc.enumeration); break;
        default: res = Results(); break;
      }
      double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      if (g_expired.load()) {
        g_has_deadline = false;
        return PM_E_TIMEOUT;
      }
      emit(step + PM_STEP_START, ms, res);
      int next = advance(step);
      finished = (step == ENUM) || next == END;
      step = next;
      ++iteration;
    }
    // Final row: logResults(iteration, true) with cleared results and the
    // name of the step the machine would run next (END after ENUMERATION,
    // multiple_label_cpu.cc:177-181; ENUMERATION when the run stopped before
    // it).
    emit(finished ? PM_STEP_END : step + PM_STEP_START, 0.0, Results());
    if (n_records) *n_records = n;
    if (cand_out) memcpy(cand_out, s.cand.data(), sizeof(uint64_t) * V);
    if (edge_active_out) memcpy(edge_active_out, s.edge_active.data(), E);
    if (vertex_active_out) memcpy(vertex_active_out, s.active.data(), V);
    g_has_deadline = false;
    return 0;
  } catch (const PmError& e) {
    g_has_deadline = false;
    return e.code;
  }
}

// GraphStatCpu::compute over a given pruned state (role masks per vertex,
// one active flag per CSR entry; a vertex is active when it holds a role),
// `threads` static-schedule blocks, in pm_query_graph_stat's layout.
int pmo_graph_stat(const uint64_t* off, const uint32_t* adj, const uint64_t* lab, uint32_t V, uint64_t E,
                   const uint64_t* p_off, const uint32_t* p_adj, const uint64_t* p_lab, uint32_t k,
                   const uint64_t* cand, const uint8_t* edge_active, int32_t threads, uint32_t* n_labels,
                   uint64_t* labels, uint64_t* vertex_total, uint64_t* edge_total, uint64_t* at_least) {
  try {
    PatternGraph pg;
    pg.n = k;
    pg.offsets.assign(p_off, p_off + k + 1);
    pg.adj.assign(p_adj, p_adj + p_off[k]);
    pg.labels.assign(p_lab, p_lab + k);
    State s;
    s.off = off;
    s.adj = adj;
    s.lab = lab;
    s.V = V;
    s.E = E;
    s.k = k;
    s.active.resize(V);
    for (uint32_t v = 0; v < V; ++v) s.active[v] = cand[v] != 0;
    s.edge_active.assign(edge_active, edge_active + E);
    const AccumulationMaximum am = accumulation_maximum(pg);
    const GraphStat gs = oracle_graph_stat(s, am, static_cast<uint32_t>(threads > 0 ? threads : 1));
    const uint32_t n = gs.slots;
    if (n_labels) *n_labels = n;
    for (uint32_t a = 0; a < n; ++a) {
      if (labels) labels[a] = gs.label_of_slot[a];
      if (vertex_total) vertex_total[a] = gs.vertex_total[a];
      for (uint32_t b = 0; b < n; ++b) {
        if (edge_total) edge_total[a * n + b] = gs.edge_total[a * n + b];
        if (at_least)
          for (uint32_t i = 0; i < 64; ++i)
            at_least[(static_cast<size_t>(a) * n + b) * 64 + i] =
                gs.at_least[(static_cast<size_t>(a) * n + b) * GraphStat::kMaxAtLeast + i];
      }
    }
    return 0;
  } catch (const PmError& e) {
    return e.code;
  }
}

// The embeddings ENUMERATION counts, listed: the reference's
// writeEnumeration (multiple_label_enumeration_cpu.tpp:15-35, compiled out
// there) writes historyIndexVector, the graph vertices bound by the walk's
// vertex moves in walk order.  Runs the pipeline to the ENUMERATION step
// (one thread, the canonical order), then lists up to cap matches of k
// vertices each into out; *n_matches receives the total.
namespace {
void enum_list(const State& s, const Walk& w, std::vector<uint32_t>& history, uint32_t cur, size_t pos,
               std::vector<uint32_t>& out, uint64_t cap, uint64_t& n) {
  if (pos == w.length()) {
    if (n < cap) out.insert(out.end(), history.begin(), history.end());
    ++n;
    return;
  }
  const int move = w.moves[pos];
  if (move == kVertexNoStore || move == kVertexStore) {
    const uint32_t next_role = w.ids[pos];
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t nb = s.adj[e];
      if (!s.active[nb] || !s.has(nb, next_role)) continue;
      bool seen = false;
      for (uint32_t h : history)
        if (h == nb) seen = true;
      if (seen) continue;
      history.push_back(nb);
      enum_list(s, w, history, nb, pos + 1, out, cap, n);
      history.pop_back();
    }
  } else if (move == kCheck) {
    const uint32_t target = history[w.back[pos]];
    for (uint64_t e = s.off[cur]; e < s.off[cur + 1]; ++e) {
      if (!s.edge_active[e]) continue;
      uint32_t nb = s.adj[e];
      if (!s.active[nb] || nb != target) continue;
      enum_list(s, w, history, cur, pos + 1, out, cap, n);
      return;
    }
  } else {
    enum_list(s, w, history, history[w.back[pos]], pos + 1, out, cap, n);
  }
}
}  // namespace

int pmo_list_matches(const uint64_t* off, const uint32_t* adj, const uint64_t* lab, uint32_t V, uint64_t E,
                     const uint64_t* p_off, const uint32_t* p_adj, const uint64_t* p_lab, uint32_t k,
                     uint32_t* out, uint64_t cap, uint64_t* n_matches) {
  try {
    // Pruned state: run the pipeline up to ENUMERATION.
    std::vector<uint64_t> cand(V);
    std::vector<uint8_t> eact(E), vact(V);
    int32_t n_rec = 0;
    const int st = pmo_run(off, adj, lab, V, E, p_off, p_adj, p_lab, k, 1, 1, 1, nullptr, 0, &n_rec, cand.data(),
                           eact.data(), vact.data());
    if (st != 0) return st;
    PatternGraph pg;
    pg.n = k;
    pg.offsets.assign(p_off, p_off + k + 1);
    pg.adj.assign(p_adj, p_adj + p_off[k]);
    pg.labels.assign(p_lab, p_lab + k);
    const QueryConstraints qc = compile_constraints(pg);
    State s;
    s.off = off;
    s.adj = adj;
    s.lab = lab;
    s.V = V;
    s.E = E;
    s.k = k;
    s.parallel = s.nlcc_parallel = false;
    s.active = vact;
    s.edge_active = eact;
    s.cand = cand;
    auto first = qc.enumeration.walks.cbegin();
    const uint32_t start_role = first->first;
    std::vector<uint32_t> list, history;
    uint64_t n = 0;
    for (uint32_t v = 0; v < V; ++v) {
      if (!s.active[v] || !s.has(v, start_role)) continue;
      history.assign(1, v);
      enum_list(s, first->second, history, v, 1, list, cap, n);
    }
    if (out && !list.empty()) memcpy(out, list.data(), 4 * list.size());
    if (n_matches) *n_matches = n;
    return 0;
  } catch (const PmError& e) {
    return e.code;
  }
}

// ENUMERATION (multiple_label_enumeration_cpu.tpp:126-174) over a given
// pruned state (role masks, CSR-entry flags; active = any role), counting
// only sources v % stride == 0: a per-source sampled count.
int pmo_enumerate_state(const uint64_t* off, const uint32_t* adj, const uint64_t* lab, uint32_t V, uint64_t E,
                        const uint64_t* p_off, const uint32_t* p_adj, const uint64_t* p_lab, uint32_t k,
                        const uint64_t* cand, const uint8_t* eact, int64_t stride, int threads, uint64_t* count) {
  try {
    PatternGraph pg;
    pg.n = k;
    pg.offsets.assign(p_off, p_off + k + 1);
    pg.adj.assign(p_adj, p_adj + p_off[k]);
    pg.labels.assign(p_lab, p_lab + k);
    const QueryConstraints qc = compile_constraints(pg);
    State s;
    s.off = off;
    s.adj = adj;
    s.lab = lab;
    s.V = V;
    s.E = E;
    s.k = k;
    s.parallel = false;
    s.nlcc_parallel = threads > 1;
    if (threads >= 1) omp_set_num_threads(threads);
    s.cand.assign(cand, cand + V);
    s.edge_active.assign(eact, eact + E);
    s.active.resize(V);
    for (uint32_t v = 0; v < V; ++v) s.active[v] = cand[v] != 0;
    s.enum_stride = stride;
    *count = step_enumeration(s, qc.enumeration).enumeration;
    return 0;
  } catch (const PmError& e) {
    return e.code;
  }
}

// The start role of the enumeration walk (walkMap.cbegin()->first,
// multiple_label_enumeration_cpu.tpp:126-174): ENUMERATION's sources are the
// active vertices holding it.
int pmo_enumeration_start_role(const uint64_t* p_off, const uint32_t* p_adj, const uint64_t* p_lab, uint32_t k) {
  try {
    PatternGraph pg;
    pg.n = k;
    pg.offsets.assign(p_off, p_off + k + 1);
    pg.adj.assign(p_adj, p_adj + p_off[k]);
    pg.labels.assign(p_lab, p_lab + k);
    const QueryConstraints qc = compile_constraints(pg);
    if (qc.enumeration.walks.empty()) return -1;
    return static_cast<int>(qc.enumeration.walks.cbegin()->first);
  } catch (const PmError& e) {
    return e.code;
  }
}

// Seeded synthetic graph for callers that must not load the product library
// (the CPU baseline's graph): the same generator source, compiled into this
// library.  Returns an owning handle; pmo_graph_csr exposes its CSR.
int pmo_generate_graph(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                       int32_t permute, int32_t label_kind, uint32_t n_labels, double zipf_s, uint64_t label_seed,
                       void** out) {
  try {
    auto* g = new HostGraph(generate_rmat(scale, edge_factor, a, b, c, seed, permute != 0));
    if (n_labels) assign_labels(*g, label_kind, n_labels, zipf_s, label_seed);
    else g->labels.assign(g->vertex_count, 0);
    *out = g;
    return 0;
  } catch (const PmError& e) {
    return e.code;
  }
}

int pmo_graph_csr(void* h, uint32_t* V, uint64_t* E, const uint64_t** off, const uint32_t** adj,
                  const uint64_t** lab) {
  auto* g = static_cast<HostGraph*>(h);
  *V = g->vertex_count;
  *E = g->edge_count;
  *off = g->offsets.data();
  *adj = g->adj.data();
  *lab = g->labels.data();
  return 0;
}

void pmo_graph_free(void* h) { delete static_cast<HostGraph*>(h); }

// Compiles a template and returns the reference-format constraint dump
// (for pinning the template compiler against log.totem).
int pmo_dump_constraints(const uint64_t* p_off, const uint32_t* p_adj, const uint64_t* p_lab, uint32_t k, char* buf,
                         size_t cap, size_t* needed) {
  try {
    PatternGraph pg;
    pg.n = k;
    pg.offsets.assign(p_off, p_off + k + 1);
    pg.adj.assign(p_adj, p_adj + p_off[k]);
    pg.labels.assign(p_lab, p_lab + k);
    std::string d = dump_constraints(compile_constraints(pg));
    if (needed) *needed = d.size() + 1;
    if (buf && cap) {
      size_t c = d.size() < cap - 1 ? d.size() : cap - 1;
      memcpy(buf, d.data(), c);
      buf[c] = 0;
    }
    return 0;
  } catch (const PmError& e) {
    return e.code;
  }
}

}  // extern "C"
