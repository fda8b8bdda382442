// Template compilation.  Each generator follows the algorithm of the
// reference file cited beside it; see constraints.h for why the container
// types are kept.
#include "constraints.h"

#include <deque>
#include <sstream>
#include <unordered_set>

namespace pmgb {
namespace {

template <class T>
bool contains(const std::vector<T>& v, const T& x) {
  for (const auto& y : v)
    if (y == x) return true;
  return false;
}

// Membership of generated constraints by their identifying ids, so that
// deduplication stays linear in the number found (dense templates yield
// thousands of cycles, each found once per rotation and direction); `out`
// keeps the order of first discovery, as the reference's list does.
struct IdsHash {
  size_t operator()(const std::vector<uint32_t>& v) const {
    uint64_t h = 0x9E3779B97F4A7C15ull ^ v.size();
    for (uint32_t x : v) h = (h ^ x) * 0x100000001B3ull;
    return static_cast<size_t>(h ^ (h >> 29));
  }
};

// --- local constraints: generate_constraint_local.cc:12-33 --------------
std::vector<LocalConstraint> gen_local(const PatternGraph& p) {
  std::vector<LocalConstraint> out(p.n);
  for (uint32_t v = 0; v < p.n; ++v) {
    LocalConstraint& lc = out[v];
    lc.origin = v;
    lc.origin_label = p.labels[v];
    for (uint64_t e = p.offsets[v]; e < p.offsets[v + 1]; ++e) {
      uint32_t w = p.adj[e];
      lc.neighbor_mask |= uint64_t(1) << w;
      auto it = lc.required.find(p.labels[w]);
      if (it != lc.required.end())
        ++it->second;
      else
        lc.required[p.labels[w]] = 1;
    }
  }
  return out;
}

// --- cycles: generate_constraint_circular.cc:13-86, constraint_circular.cc:12-58
CycleConstraint make_cycle(const std::vector<uint32_t>& hist, const std::vector<label_t>& hist_labels) {
  // The walk ends on its start vertex; drop that repeat, then rotate so the
  // smallest id comes first and orient towards the smaller neighbour.
  std::vector<uint32_t> ids(hist.begin(), hist.end() - 1);
  std::vector<label_t> lab(hist_labels.begin(), hist_labels.end() - 1);
  const size_t len = ids.size();
  size_t min_index = 0;
  for (size_t i = 1; i < len; ++i)
    if (ids[i] < ids[min_index]) min_index = i;
  bool reverse;
  if (min_index > 0 && min_index < len - 1)
    reverse = ids[min_index - 1] < ids[min_index + 1];
  else if (min_index == 0)
    reverse = ids[len - 1] < ids[1];
  else
    reverse = ids[len - 2] < ids[0];
  CycleConstraint c;
  c.ids.resize(len);
  c.labels.resize(len);
  long pos = static_cast<long>(min_index);
  for (size_t k = 0; k < len; ++k) {
    c.ids[k] = ids[pos];
    c.labels[k] = lab[pos];
    pos += reverse ? -1 : 1;
    if (pos == static_cast<long>(len)) pos = 0;
    if (pos == -1) pos = static_cast<long>(len) - 1;
  }
  return c;
}

// The reference runs one DFS per (start vertex, cycle length) and records
// the walks that come back to the start after exactly that many steps
// (generate_constraint_circular.cc:13-56).  A walk that meets the start
// earlier marks it visited and can no longer close, so the recorded walks of
// length L are the simple cycles through the start, in the DFS order of
// their choices.  One DFS per start vertex visits every simple path once and
// files each closing walk under its length; emitting the lengths in
// increasing order gives the reference's sequence.
struct CycleSearch {
  const PatternGraph& p;
  std::vector<CycleConstraint>& out;
  std::vector<uint32_t> hist;
  std::vector<label_t> hist_labels;
  uint64_t visited = 0;
  std::vector<std::vector<CycleConstraint>> by_length;      // closing walks of the current start
  std::unordered_set<std::vector<uint32_t>, IdsHash> seen;  // ids of out's entries
  void dfs(uint32_t source, uint32_t cur, size_t depth) {
    for (uint64_t e = p.offsets[cur]; e < p.offsets[cur + 1]; ++e) {
      uint32_t w = p.adj[e];
      if (w == source) {
        if (depth + 1 >= 3) {
          hist.push_back(w);
          hist_labels.push_back(p.labels[w]);
          by_length[depth + 1].push_back(make_cycle(hist, hist_labels));
          hist.pop_back();
          hist_labels.pop_back();
        }
        continue;
      }
      if ((visited >> w & 1) || depth + 1 >= p.n) continue;
      hist.push_back(w);
      hist_labels.push_back(p.labels[w]);
      visited |= uint64_t(1) << w;
      dfs(source, w, depth + 1);
      visited &= ~(uint64_t(1) << w);
      hist.pop_back();
      hist_labels.pop_back();
    }
  }
};

std::vector<CycleConstraint> gen_cycles(const PatternGraph& p) {
  std::vector<CycleConstraint> out;
  CycleSearch s{p, out, {}, {}, 0, {}, {}};
  for (uint32_t v = 0; v < p.n; ++v) {
    s.by_length.assign(p.n + 1, {});
    s.hist.push_back(v);
    s.hist_labels.push_back(p.labels[v]);
    s.visited = 0;
    s.dfs(v, v, 0);
    s.hist.pop_back();
    s.hist_labels.pop_back();
    for (size_t len = 3; len <= p.n; ++len)
      for (auto& c : s.by_length[len])
        if (s.seen.insert(c.ids).second) out.push_back(std::move(c));
  }
  return out;
}

// --- paths: generate_constraint_path.cc:11-74, constraint_path.cc:9-29 ---
PathConstraint make_path(const std::vector<uint32_t>& hist, const std::vector<label_t>& hist_labels) {
  PathConstraint pc;
  pc.initial_label = hist_labels[0];
  const size_t len = hist.size();
  if (hist[len - 1] > hist[0]) {
    pc.ids.assign(hist.rbegin(), hist.rend());
    pc.labels.assign(hist_labels.rbegin(), hist_labels.rend());
  } else {
    pc.ids = hist;
    pc.labels = hist_labels;
  }
  return pc;
}

struct PathSearch {
  const PatternGraph& p;
  std::vector<PathConstraint>& out;
  std::vector<uint32_t> hist;
  std::vector<label_t> hist_labels;
  uint64_t visited = 0;
  // ids of out's entries (a path's initial label is its first vertex's
  // label, so the ids identify it)
  std::unordered_set<std::vector<uint32_t>, IdsHash> seen;
  void dfs(uint32_t source, uint32_t cur, size_t depth) {
    if (depth >= 2 && p.labels[source] == p.labels[cur] && source != cur) {
      PathConstraint pc = make_path(hist, hist_labels);
      if (seen.insert(pc.ids).second) out.push_back(std::move(pc));
      return;
    }
    for (uint64_t e = p.offsets[cur]; e < p.offsets[cur + 1]; ++e) {
      uint32_t w = p.adj[e];
      if (visited >> w & 1) continue;
      hist.push_back(w);
      hist_labels.push_back(p.labels[w]);
      visited |= uint64_t(1) << w;
      dfs(source, w, depth + 1);
      visited &= ~(uint64_t(1) << w);
      hist.pop_back();
      hist_labels.pop_back();
    }
  }
};

std::vector<PathConstraint> gen_paths(const PatternGraph& p) {
  std::vector<PathConstraint> out;
  PathSearch s{p, out, {}, {}, 0, {}};
  for (uint32_t v = 0; v < p.n; ++v) {
    // A path ends at another vertex with the start's label: without one the
    // search from v records nothing.
    bool other = false;
    for (uint32_t u = 0; u < p.n && !other; ++u) other = u != v && p.labels[u] == p.labels[v];
    if (!other) continue;
    s.hist.push_back(v);
    s.hist_labels.push_back(p.labels[v]);
    s.visited = uint64_t(1) << v;
    s.dfs(v, v, 0);
    s.hist.pop_back();
    s.hist_labels.pop_back();
  }
  return out;
}

// --- template construction: constraint_template.cc:9-77 ------------------
TemplateConstraint template_from_cycle(const CycleConstraint& c) {
  TemplateConstraint t;
  t.origin = kCC;
  t.length = c.length();
  for (size_t i = 0; i + 1 < c.ids.size(); ++i) {
    t.graph[c.ids[i]].insert(c.ids[i + 1]);
    t.graph[c.ids[i + 1]].insert(c.ids[i]);
  }
  t.graph[c.ids.back()].insert(c.ids.front());
  t.graph[c.ids.front()].insert(c.ids.back());
  return t;
}

TemplateConstraint template_from_path(const PathConstraint& pc) {
  TemplateConstraint t;
  t.origin = kPC;
  t.length = pc.length();
  for (size_t i = 0; i + 1 < pc.ids.size(); ++i) {
    t.graph[pc.ids[i]].insert(pc.ids[i + 1]);
    t.graph[pc.ids[i + 1]].insert(pc.ids[i]);
  }
  return t;
}

TemplateConstraint template_merge(const TemplateConstraint& a, const TemplateConstraint& b) {
  TemplateConstraint t;
  const bool a_cc = a.origin == kCC || a.origin == kTdsCC;
  const bool b_cc = b.origin == kCC || b.origin == kTdsCC;
  const bool a_pc = a.origin == kPC || a.origin == kTdsPC;
  const bool b_pc = b.origin == kPC || b.origin == kTdsPC;
  t.origin = (a_cc && b_cc) ? kTdsCC : (a_pc && b_pc) ? kTdsPC : kTdsSub;
  t.length = a.length;
  t.graph = a.graph;  // copy-assignment, as the reference does
  for (const auto& kv : b.graph) {
    if (t.graph.count(kv.first) == 0) ++t.length;
    for (uint32_t s : kv.second) t.graph[kv.first].insert(s);
  }
  return t;
}

TemplateConstraint template_full(const PatternGraph& p) {
  TemplateConstraint t;
  t.origin = kTdsFull;
  t.length = p.n;
  for (uint32_t v = 0; v < p.n; ++v)
    for (uint64_t e = p.offsets[v]; e < p.offsets[v + 1]; ++e) {
      uint32_t w = p.adj[e];
      t.graph[v].insert(w);
      t.graph[w].insert(v);
    }
  return t;
}

bool share_vertex(const TemplateConstraint& a, const TemplateConstraint& b) {
  for (const auto& kv : a.graph)
    if (b.graph.count(kv.first) > 0) return true;
  return false;
}

bool share_edge(const TemplateConstraint& a, const TemplateConstraint& b) {
  for (const auto& kv : a.graph) {
    if (b.graph.count(kv.first) == 0) continue;
    const auto& other = b.graph.at(kv.first);
    for (uint32_t s : kv.second)
      for (uint32_t t : other)
        if (t == s) return true;
  }
  return false;
}

// The reference merges two list entries with
//     list.erase(it1); list.erase(it2);
// (generate_constraint_template.cc:33-34, 73-74): it2 is used after the
// first erase invalidated it.  Under libstdc++ (the GNU C++ standard
// library), deque::erase shifts the shorter side: when it1 lies in the front half
// the elements before it move back one slot and it2 still designates the
// same element; otherwise the elements after it1 move forward one slot, so
// it2 designates the element that followed it (or end(), in which case the
// library pops the last element).  This function reproduces that outcome
// with well-defined operations.
void erase_pair_as_reference(std::deque<TemplateConstraint>& list, size_t i1, size_t i2) {
  const size_t n = list.size();
  const bool front_half = i1 < (n >> 1);
  list.erase(list.begin() + static_cast<long>(i1));
  if (front_half)
    list.erase(list.begin() + static_cast<long>(i2 - 1));
  else if (i2 < n - 1)
    list.erase(list.begin() + static_cast<long>(i2));
  else
    list.pop_back();
}

// Pairwise merge loop of preprocessCircularConstraint / preprocessPathConstraint
// (generate_constraint_template.cc:20-38, 60-78).
template <class Pred>
void merge_pairs(std::deque<TemplateConstraint>& list, Pred overlap) {
  size_t i1 = 0;
  while (i1 < list.size()) {
    size_t i2 = i1 + 1;
    bool merged = false;
    while (i2 < list.size()) {
      if (overlap(list[i1], list[i2])) {
        TemplateConstraint m = template_merge(list[i1], list[i2]);
        merged = true;
        erase_pair_as_reference(list, i1, i2);
        list.push_back(std::move(m));
        i1 = 0;
        break;
      }
      ++i2;
    }
    if (!merged) ++i1;
  }
}

// --- walks: constraint_template.cc:121-169, utils/walk.cc:16-60 ----------
struct WalkBuilder {
  const PatternGraph& p;
  const TemplateConstraint& t;
  Walk walk;
  std::vector<uint32_t> hist;                          // visited template vertices
  std::vector<std::pair<uint32_t, uint32_t>> hist_edges;  // undirected (min, max)

  void add_vertex(uint32_t v) {
    walk.moves.push_back(kVertexNoStore);
    walk.ids.push_back(v);
    walk.labels.push_back(p.labels[v]);
    walk.back.push_back(0);
    ++walk.vertex_length;
  }
  void add_ref(int kind, uint32_t v, size_t back) {
    walk.moves.push_back(kind);
    walk.ids.push_back(v);
    walk.labels.push_back(p.labels[v]);
    walk.back.push_back(back);
  }
  size_t hist_index(uint32_t v) const {
    size_t i = 0;
    for (; i < hist.size(); ++i)
      if (hist[i] == v) return i;
    return i;
  }
  void dfs(uint32_t cur) {
    bool on_path = true;  // false right after returning from a subtree
    const size_t cur_walk_index = walk.vertex_length - 1;
    for (uint32_t nb : t.graph.at(cur)) {
      std::pair<uint32_t, uint32_t> e(cur < nb ? cur : nb, cur < nb ? nb : cur);
      if (!contains(hist, nb)) {
        if (!on_path) add_ref(kMoveBack, cur, cur_walk_index);
        hist_edges.push_back(e);
        hist.push_back(nb);
        add_vertex(nb);
        dfs(nb);
        on_path = false;
      } else {
        if (contains(hist_edges, e)) continue;
        if (!on_path) {
          add_ref(kMoveBack, cur, cur_walk_index);
          on_path = true;
        }
        size_t prev = hist_index(nb);
        hist_edges.push_back(e);
        add_ref(kCheck, nb, prev);
      }
    }
  }
  // Walk::computeStoredVertex: a vertex move whose template vertex is
  // checked again later must keep its graph vertex.
  void mark_stored() {
    std::vector<uint32_t> stored;
    for (size_t i = 0; i < walk.length(); ++i) {
      if (walk.moves[i] != kVertexNoStore) continue;
      bool checked_later = false;
      for (size_t j = i + 1; j < walk.length(); ++j)
        if (walk.ids[j] == walk.ids[i] && walk.moves[j] == kCheck) {
          checked_later = true;
          break;
        }
      if (checked_later && !contains(stored, walk.ids[i])) {
        walk.moves[i] = kVertexStore;
        stored.push_back(walk.ids[i]);
      }
    }
  }
};

void build_walks(const PatternGraph& p, TemplateConstraint& t) {
  for (const auto& kv : t.graph) {
    WalkBuilder b{p, t, {}, {}, {}};
    b.hist.push_back(kv.first);
    b.add_vertex(kv.first);
    b.dfs(kv.first);
    b.mark_stored();
    t.walks[kv.first] = b.walk;
  }
}

// --- merged templates: generate_constraint_template.cc:13-145 ------------
std::vector<TemplateConstraint> gen_templates(const PatternGraph& p, const std::vector<CycleConstraint>& cycles,
                                              const std::vector<PathConstraint>& paths) {
  std::vector<TemplateConstraint> out;
  {
    std::deque<TemplateConstraint> list;
    for (const auto& c : cycles) list.push_back(template_from_cycle(c));
    merge_pairs(list, share_edge);
    for (const auto& t : list)
      if (t.origin != kCC) out.push_back(t);
  }
  {
    std::unordered_map<label_t, std::deque<TemplateConstraint>> by_label;
    for (const auto& pc : paths) by_label[pc.initial_label].push_back(template_from_path(pc));
    for (auto& kv : by_label) merge_pairs(kv.second, share_vertex);
    for (const auto& kv : by_label)
      for (const auto& t : kv.second)
        if (t.origin != kPC) out.push_back(t);
  }
  {
    // preprocessSubtemplateConstraint (:94-130): grow one template by every
    // later list entry sharing a vertex with it, restarting the scan from the
    // front after each merge; keep each new merged template once.
    std::deque<TemplateConstraint> list(out.begin(), out.end());
    size_t offset = 0;
    while (!list.empty() && offset < list.size() - 1) {
      int merged = 0;
      size_t i = offset;
      TemplateConstraint current = list[i];
      ++i;
      while (i < list.size()) {
        if (share_vertex(current, list[i])) {
          current = template_merge(current, list[i]);
          list.erase(list.begin() + static_cast<long>(i));
          i = 0;
          ++merged;
        } else {
          ++i;
        }
      }
      if (merged > 0) {
        offset = 0;
        if (!contains(out, current)) out.push_back(current);
      } else {
        ++offset;
      }
    }
  }
  for (auto& t : out) build_walks(p, t);
  return out;
}

// --- log.totem printers (the generators' print methods) -----------------
void print_walk(std::ostream& os, const Walk& w) {
  os << "Walk : ";
  for (size_t i = 0; i < w.length(); ++i) {
    if (i) os << " -> ";
    const char* m = w.moves[i] == kCheck ? "CK" : w.moves[i] == kMoveBack ? "MB" : w.moves[i] == kVertexStore ? "VS" : "VN";
    os << "[" << m << "," << w.ids[i] << "," << w.labels[i] << "," << w.back[i] << "]";
  }
  os << "\n";
}

void print_template(std::ostream& os, const TemplateConstraint& t) {
  os << "Vertex Index Graph [length : " << t.length << "] : ";
  for (const auto& kv : t.graph)
    for (uint32_t s : kv.second) os << " (" << kv.first << "," << s << ")";
  os << "\n";
  os << "Vertex Index Walk : ";
  for (const auto& kv : t.walks) print_walk(os, kv.second);
  os << "\n";
}

}  // namespace

QueryConstraints compile_constraints(const PatternGraph& p) {
  if (p.n > kMaxPatternSize)
    throw PmError{PM_E_PATTERN_TOO_LARGE, "template has " + std::to_string(p.n) + " vertices; at most 64 are supported"};
  if (p.n == 0) throw PmError{PM_E_INVALID_ARG, "template has no vertices"};
  QueryConstraints qc;
  qc.local = gen_local(p);
  qc.cycles = gen_cycles(p);
  qc.paths = gen_paths(p);
  qc.templates = gen_templates(p, qc.cycles, qc.paths);
  qc.enumeration = template_full(p);
  build_walks(p, qc.enumeration);
  return qc;
}

std::string dump_constraints(const QueryConstraints& qc) {
  std::ostringstream os;
  os << "Generate Local constraint\n";
  for (const auto& lc : qc.local) {
    os << "Vertex " << lc.origin << " : Label " << lc.origin_label << "\n";
    for (const auto& kv : lc.required) os << "\t Sublabel " << kv.first << " : " << kv.second << "\n";
    for (uint32_t b = 0; b < 64; ++b)
      if (lc.neighbor_mask >> b & 1) os << "\t Neighbor " << b << "\n";
  }
  os << "Generate Circular constraint\n";
  os << "Constraint number =  " << qc.cycles.size() << ". \n";
  for (size_t i = 0; i < qc.cycles.size(); ++i) {
    os << "=== Current constraint = " << i << " ===\n";
    os << "Vertex Index : ";
    for (uint32_t v : qc.cycles[i].ids) os << v << " -> ";
    os << qc.cycles[i].ids[0] << "\n";
    os << "Vertex Label : ";
    for (label_t l : qc.cycles[i].labels) os << l << " -> ";
    os << qc.cycles[i].labels[0] << "\n";
  }
  os << "Generate Path constraint\n";
  os << "Constraint number =  " << qc.paths.size() << ". \n";
  for (size_t i = 0; i < qc.paths.size(); ++i) {
    os << "=== Current constraint = " << i << " ===\n";
    os << "Vertex Index : ";
    for (size_t j = 0; j < qc.paths[i].ids.size(); ++j) os << (j ? " -> " : "") << qc.paths[i].ids[j];
    os << "\n";
    os << "Vertex Label : ";
    for (size_t j = 0; j < qc.paths[i].labels.size(); ++j) os << (j ? " -> " : "") << qc.paths[i].labels[j];
    os << "\n";
  }
  os << "Generate Template constraint\n";
  os << "Constraint number =  " << qc.templates.size() << ". \n";
  for (size_t i = 0; i < qc.templates.size(); ++i) {
    os << "=== Current constraint = " << i << " ===\n";
    print_template(os, qc.templates[i]);
  }
  os << "Generate Enumeration constraint\n";
  os << "=== enumeration constraint ===\n";
  print_template(os, qc.enumeration);
  return os.str();
}

}  // namespace pmgb
