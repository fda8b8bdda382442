// Effectiveness estimates of the reference's dynamic constraint order
// (src/patternmatching/multiple_label/multiple_label_constraint_effectiveness.cc).
// Every formula keeps the reference's operands and evaluation order; the
// arguments the reference passes as constants (knowingEdgeNumber and
// knowingVertexNumber are 0 at every call site it makes) are folded in.
#include "effectiveness.h"

#include "pm_gb300.h"

#include <cmath>
#include <string>

namespace pmgb {

int GraphStat::slot(uint64_t label) const {
  for (uint32_t s = 0; s < slots; ++s)
    if (label_of_slot[s] == label) return static_cast<int>(s);
  return -1;
}

void throw_stat_missing(const std::string& what) { throw PmError{PM_E_STATISTICS, what}; }

[[noreturn]] static void missing(const char* what, uint64_t a, uint64_t b = 0) {
  throw_stat_missing(std::string("graph statistic absent: ") + what + " (" + std::to_string(a) + ", " +
                     std::to_string(b) + ")");
}

double GraphStat::vertices(uint64_t label) const {
  const int a = slot(label);
  if (a < 0 || vertex_total[a] == 0) missing("vertexLabelTotalNumber", label);
  return static_cast<double>(vertex_total[a]);
}

double GraphStat::edges(uint64_t from, uint64_t to) const {
  const int a = slot(from), b = slot(to);
  if (a < 0 || b < 0 || edge_total[a * slots + b] == 0) missing("edgeLabelTotalNumber", from, to);
  return static_cast<double>(edge_total[a * slots + b]);
}

double GraphStat::outbound(uint64_t from) const {
  const int a = slot(from);
  if (a < 0 || edge_outbound[a] == 0) missing("edgeOutboundLabelTotalNumber", from);
  return static_cast<double>(edge_outbound[a]);
}

double GraphStat::at_least_count(uint64_t from, uint64_t to, size_t i) const {
  const int a = slot(from), b = slot(to);
  if (a < 0 || b < 0 || i >= kMaxAtLeast || at_least[(a * slots + b) * kMaxAtLeast + i] == 0)
    missing("vertexLabelWithAtLeastNeighborLabel", from, to);
  return static_cast<double>(at_least[(a * slots + b) * kMaxAtLeast + i]);
}

AccumulationMaximum accumulation_maximum(const PatternGraph& p) {
  AccumulationMaximum m;
  for (uint32_t v = 0; v < p.n; ++v) {
    bool seen = false;
    for (uint64_t l : m.label_of_slot) seen |= l == p.labels[v];
    if (!seen) m.label_of_slot.push_back(p.labels[v]);
  }
  m.slots = static_cast<uint32_t>(m.label_of_slot.size());
  m.max.assign(static_cast<size_t>(m.slots) * m.slots, 0);
  m.has_a.assign(m.slots, 0);
  auto slot = [&](uint64_t l) {
    uint32_t s = 0;
    while (m.label_of_slot[s] != l) ++s;
    return s;
  };
  for (uint32_t v = 0; v < p.n; ++v) {
    const uint32_t a = slot(p.labels[v]);
    std::vector<uint32_t> count(m.slots, 0);
    for (uint64_t e = p.offsets[v]; e < p.offsets[v + 1]; ++e) ++count[slot(p.labels[p.adj[e]])];
    for (uint32_t b = 0; b < m.slots; ++b) {
      if (!count[b]) continue;
      m.has_a[a] = 1;
      if (m.max[a * m.slots + b] < count[b]) m.max[a * m.slots + b] = count[b];
    }
  }
  return m;
}

namespace {

// probaFindVertex (effectiveness.cc:1120-1134) with knowingEdgeNumber = 0.
double proba_find_vertex(const GraphStat& gs, uint64_t from, uint64_t to) {
  const double full = gs.vertices(from);
  const double set = full;
  const double different = std::pow((full - 0.0 - 0.0) / (full - 0.0), 1);
  return gs.at_least_count(from, to, 1) / set * different;
}

// probaFindOnePathKnowing (:1141-1149).
double one_path(const GraphStat& gs, double n, uint64_t from, uint64_t to) {
  return 1 - std::pow(1 - proba_find_vertex(gs, from, to), n);
}

// probaFindSameVertex (:1151-1156).
double same_vertex(const GraphStat& gs, double n, uint64_t label) {
  const double size = gs.vertices(label);
  return 1 - std::pow((size - 1) / size, n);
}

// probaFindDifferentVertex (:1158-1163).
double different_vertex(const GraphStat& gs, double n, uint64_t label) {
  const double size = gs.vertices(label);
  return 1 - std::pow((1.) / size, n);
}

// averageNumberOfVertex(labelFrom) (:1165-1171).
double avg_vertex(const GraphStat& gs, double n, uint64_t from) {
  const double out = gs.outbound(from);
  return n * out / gs.vertices(from);
}

// averageNumberOfVertexKnowing (:1180-1200): tries times an integer 1.
double avg_vertex_to(const GraphStat& gs, double n, uint64_t from, uint64_t to) {
  gs.vertices(from);
  const double e = gs.edges(from, to);
  return n * e / gs.vertices(from);
}

// averageNumberOfUniqueVertexKnowing (:1209-1230) with the strong
// approximation min(tries, label-to vertices) (.tpp:9-12).
double avg_unique(const GraphStat& gs, double n, uint64_t from, uint64_t to) {
  gs.vertices(from);
  const double e = gs.edges(from, to);
  const double tries = n * e / gs.vertices(from);
  const double most = gs.vertices(to);
  return (tries <= most) ? tries : most;
}

// 1 - E(from, to) / V(from) + unique: the known-edge branch of the cycle and
// path estimates.
double known_edge(const GraphStat& gs, double n, uint64_t from, uint64_t to) {
  const double e = gs.edges(from, to);
  const double v = gs.vertices(from);
  return 1 - e / v + avg_unique(gs, n, from, to);
}

double cost_share(double possible, double cost, double fp, int threads, size_t length) {
  double c = possible * cost * (1 - fp);
  c /= threads;
  c /= 1 + static_cast<double>(length - 1) / 2 * fp;
  return c;
}

std::vector<uint64_t> history_labels(const Walk& w) {
  std::vector<uint64_t> h;
  for (size_t i = 0; i < w.length(); ++i)
    if (w.moves[i] == kVertexStore || w.moves[i] == kVertexNoStore) h.push_back(w.labels[i]);
  return h;
}

// Finding probability of one walk of a template (effectiveness.cc:704-761 /
// 980-1047): moves 1 .. last_move.
double walk_probability(const GraphStat& gs, const Walk& w, size_t moves) {
  const std::vector<uint64_t> hist = history_labels(w);
  double fp = 1.;
  double u = 1;
  uint64_t from = w.labels[0];
  std::vector<double> uv{u};
  for (size_t j = 0; j + 1 <= moves; ++j) {
    const int type = w.moves[j + 1];
    if (type == kVertexStore || type == kVertexNoStore) {
      const uint64_t to = w.labels[j + 1];
      fp *= one_path(gs, u, from, to);
      u = avg_unique(gs, u, from, to);
      from = to;
      uv.push_back(u);
    } else if (type == kMoveBack) {
      const size_t back = w.back[j + 1];
      u = uv[back];
      from = hist[back];
    } else if (type == kCheck) {
      const uint64_t to = w.labels[j + 1];
      fp *= one_path(gs, u, from, to) * same_vertex(gs, u, to);
    }
  }
  return fp;
}

// Cost of one walk (effectiveness.cc:779-829 / 1059-1114): moves 1 .. len-2.
double walk_cost(const GraphStat& gs, const Walk& w) {
  const std::vector<uint64_t> hist = history_labels(w);
  double t = 1;
  double cost = t;
  uint64_t from = w.labels[0];
  std::vector<double> tv{t};
  const size_t len = w.length();
  for (size_t j = 0; j + 2 < len; ++j) {
    const int type = w.moves[j + 1];
    if (type == kVertexStore || type == kVertexNoStore) {
      const uint64_t to = w.labels[j + 1];
      cost += avg_vertex(gs, t, from);
      t = j == 0 ? avg_vertex_to(gs, t, from, to) : avg_unique(gs, t, from, to);
      tv.push_back(t);
      from = to;
    } else if (type == kMoveBack) {
      const size_t back = w.back[j + 1];
      t = tv[back];
      from = hist[back];
    } else if (type == kCheck) {
      cost += avg_vertex(gs, t, from);
    }
  }
  return cost + t;
}

}  // namespace

Effectiveness effectiveness_backtrack(const GraphStat& gs, const CycleConstraint& c, int threads) {
  Effectiveness r;
  const size_t L = c.length();
  const std::vector<uint64_t>& lab = c.labels;
  std::vector<double> fpa;
  for (size_t i = 0; i < L; ++i) {
    double fp = 1.;
    double u = 1;
    for (size_t j = 0; j < L; ++j) {
      const uint64_t from = lab[(i + j) % L], to = lab[(i + j + 1) % L];
      if (j == 0 || lab[(i + j - 1) % L] != to) {
        fp *= one_path(gs, u, from, to);
        u = avg_unique(gs, u, from, to);
      } else {
        u = known_edge(gs, u, from, to);
      }
    }
    fp *= same_vertex(gs, u, lab[(i + L) % L]);
    fpa.push_back(fp);
  }
  for (size_t i = 0; i < L; ++i) r.match_eliminated += gs.vertices(lab[i]) * (1 - fpa[i]);
  for (size_t i = 0; i < L; ++i) {
    double t = 1;
    double cost = t;
    for (size_t j = 0; j + 1 < L; ++j) {
      const uint64_t from = lab[(i + j) % L], to = lab[(i + j + 1) % L];
      cost += avg_vertex(gs, t, from);
      if (j == 0)
        t = avg_vertex_to(gs, t, from, to);
      else if (lab[(i + j - 1) % L] != to)
        t = avg_unique(gs, t, from, to);
      else
        t = known_edge(gs, t, from, to);
    }
    cost += avg_vertex(gs, t, lab[(i + L - 1) % L]);
    cost += t;
    r.cost_eliminated += cost_share(gs.vertices(lab[i]), cost, fpa[i], threads, L);
  }
  r.effectiveness = r.match_eliminated / r.cost_eliminated;
  return r;
}

Effectiveness effectiveness_backtrack(const GraphStat& gs, const PathConstraint& c, int threads) {
  Effectiveness r;
  const size_t L = c.length();
  const std::vector<uint64_t>& lab = c.labels;
  std::vector<double> fpa;
  for (int i = 0; i <= 1; ++i) {
    const bool reverse = i == 1;
    double fp = 1.;
    double u = 1;
    for (size_t j = 0; j + 2 < L; ++j) {
      const size_t cur = reverse ? L - j - 1 : j, next = reverse ? L - j - 2 : j + 1;
      const uint64_t from = lab[cur], to = lab[next];
      if (j == 0 || lab[reverse ? L - j : j - 1] != to) {
        fp *= one_path(gs, u, from, to);
        u = avg_unique(gs, u, from, to);
      } else {
        u = known_edge(gs, u, from, to);
      }
    }
    // The closing label is position i (0 or 1) in both directions.
    fp *= different_vertex(gs, u, lab[(i + L) % L]);
    fpa.push_back(fp);
  }
  for (int i = 0; i <= 1; ++i) r.match_eliminated += gs.vertices(lab[i]) * (1 - fpa[i]);
  for (int i = 0; i <= 1; ++i) {
    const bool reverse = i == 1;
    double t = 1;
    double cost = t;
    for (size_t j = 0; j + 2 < L; ++j) {
      const size_t cur = reverse ? L - j - 1 : j, next = reverse ? L - j - 2 : j + 1;
      const uint64_t from = lab[cur], to = lab[next];
      cost += avg_vertex(gs, t, from);
      if (j == 0)
        t = avg_vertex_to(gs, t, from, to);
      else if (lab[reverse ? L - j : j - 1] != to)
        t = avg_unique(gs, t, from, to);
      else
        t = known_edge(gs, t, from, to);
    }
    cost += avg_vertex(gs, t, lab[(i + L - 1) % L]);
    cost += t;
    r.cost_eliminated += cost_share(gs.vertices(lab[i]), cost, fpa[i], threads, L);
  }
  r.effectiveness = r.match_eliminated / r.cost_eliminated;
  return r;
}

Effectiveness effectiveness_backtrack(const GraphStat& gs, const TemplateConstraint& t, int threads) {
  Effectiveness r;
  std::vector<double> fpa;
  for (const auto& kv : t.walks) fpa.push_back(walk_probability(gs, kv.second, kv.second.length() - 2));
  size_t index = 0;
  for (const auto& kv : t.walks) r.match_eliminated += gs.vertices(kv.second.labels[0]) * (1 - fpa[index++]);
  index = 0;
  for (const auto& kv : t.walks) {
    const Walk& w = kv.second;
    const double cost = walk_cost(gs, w);
    r.cost_eliminated += cost_share(gs.vertices(w.labels[0]), cost, fpa[index], threads, w.vertex_length);
    ++index;
  }
  r.effectiveness = r.match_eliminated / r.cost_eliminated;
  return r;
}

Effectiveness effectiveness_enumeration(const GraphStat& gs, const TemplateConstraint& t, int threads) {
  Effectiveness r;
  std::vector<double> fpa;
  // compute() walks every move after the first (j < length - 1) ...
  for (const auto& kv : t.walks) fpa.push_back(walk_probability(gs, kv.second, kv.second.length() - 1));
  size_t index = 0;
  for (const auto& kv : t.walks) r.match_eliminated += gs.vertices(kv.second.labels[0]) * (1 - fpa[index++]);
  // ... and its cost loop never advances its index: every walk's cost uses
  // the first walk's finding probability (effectiveness.cc:775-829).
  for (const auto& kv : t.walks) {
    const Walk& w = kv.second;
    const double cost = walk_cost(gs, w);
    r.cost_eliminated += cost_share(gs.vertices(w.labels[0]), cost, fpa[0], threads, w.vertex_length);
  }
  r.effectiveness = r.match_eliminated / r.cost_eliminated;
  return r;
}

OrderChoice choose_next_constraint(const GraphStat& gs, const std::vector<const CycleConstraint*>& cycles,
                                   const std::vector<const PathConstraint*>& paths,
                                   const std::vector<const TemplateConstraint*>& templates,
                                   const TemplateConstraint& enumeration, bool use_enumerate, bool early_start,
                                   double threshold, int threads) {
  double max_c = 0, max_p = 0, max_t = 0, time_c = 0, time_p = 0, time_t = 0;
  size_t id_c = 0, id_p = 0, id_t = 0;
  for (size_t i = 0; i < cycles.size(); ++i) {
    const Effectiveness e = effectiveness_backtrack(gs, *cycles[i], threads);
    if (e.effectiveness > max_c) {
      id_c = i;
      max_c = e.effectiveness;
      time_c = e.cost_eliminated;
    }
  }
  for (size_t i = 0; i < paths.size(); ++i) {
    const Effectiveness e = effectiveness_backtrack(gs, *paths[i], threads);
    if (e.effectiveness > max_p) {
      id_p = i;
      max_p = e.effectiveness;
      time_p = e.cost_eliminated;
    }
  }
  for (size_t i = 0; i < templates.size(); ++i) {
    const Effectiveness e = effectiveness_backtrack(gs, *templates[i], threads);
    if (e.effectiveness > max_t) {
      id_t = i;
      max_t = e.effectiveness;
      time_t = e.cost_eliminated;
    }
  }
  const double time_enumeration = early_start ? effectiveness_enumeration(gs, enumeration, threads).cost_eliminated : 0;
  OrderChoice c;
  double next_time = 0, next_effectiveness = 0;
  bool enumerate = false;
  if (max_c >= max_p && max_c >= max_t && !cycles.empty()) {
    c = {PM_STEP_CC, id_c};
    next_time = time_c;
    next_effectiveness = max_c;
  } else if (max_p >= max_c && max_p >= max_t && !paths.empty()) {
    c = {PM_STEP_PC, id_p};
    next_time = time_p;
    next_effectiveness = max_p;
  } else if (max_t >= max_c && max_t >= max_p && !templates.empty()) {
    c = {PM_STEP_TDS, id_t};
    next_time = time_t;
    next_effectiveness = max_t;
  } else {
    c = {use_enumerate ? PM_STEP_ENUMERATION : PM_STEP_END, 0};
    enumerate = true;
  }
  if (early_start && !enumerate && (time_enumeration <= next_time || next_effectiveness <= threshold))
    c = {use_enumerate ? PM_STEP_ENUMERATION : PM_STEP_END, 0};
  return c;
}

}  // namespace pmgb
