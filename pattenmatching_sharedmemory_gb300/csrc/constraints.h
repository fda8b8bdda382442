// Template compilation: the local, cycle, path, merged-template and
// enumeration constraints the reference derives from a pattern, in the
// reference's order.
//
// Order matters for bit-exactness: the step machine runs the constraints in
// generation order, the template walks are keyed by an std::unordered_map
// whose iteration order picks the TDS start roles and the enumeration start
// role (src/patternmatching/multiple_label/multiple_label_constraint_template.h:58-59,
// multiple_label_enumeration_cpu.tpp:133).  The containers below are the
// same standard-library types, filled by the same sequence of insertions, so
// iteration order is identical under the same C++ standard library.
#pragma once
#include <cstdint>
#include <set>
#include <string>
#include <unordered_map>
#include <vector>

#include "pm_types.h"

namespace pmgb {

// The template graph as loaded from pattern_edge (+ pattern_vertex_data).
struct PatternGraph {
  uint32_t n = 0;
  std::vector<uint64_t> offsets;
  std::vector<uint32_t> adj;
  std::vector<uint64_t> labels;
};

// MultipleLabelConstraintLocal (multiple_label_constraint_local.h:18-32).
struct LocalConstraint {
  uint32_t origin = 0;
  label_t origin_label = 0;
  std::unordered_map<label_t, size_t> required;  // neighbour label -> count
  uint64_t neighbor_mask = 0;                    // localConstraintNeighborVertex
};

// MultipleLabelConstraintCircular (multiple_label_constraint_circular.cc:12-58):
// canonical rotation (minimum id first) and direction.
struct CycleConstraint {
  std::vector<uint32_t> ids;
  std::vector<label_t> labels;
  size_t length() const { return ids.size(); }
  bool operator==(const CycleConstraint& o) const { return ids == o.ids; }
};

// MultipleLabelConstraintPath (multiple_label_constraint_path.cc:9-29).
struct PathConstraint {
  label_t initial_label = 0;
  std::vector<uint32_t> ids;
  std::vector<label_t> labels;
  size_t length() const { return ids.size(); }
  bool operator==(const PathConstraint& o) const {
    return initial_label == o.initial_label && ids == o.ids;
  }
};

// Walk (src/patternmatching/utils/walk.h:12-34).
enum WalkMove : int { kMoveBack = 0, kCheck = 1, kVertexStore = 2, kVertexNoStore = 3 };
struct Walk {
  std::vector<int> moves;
  std::vector<uint32_t> ids;
  std::vector<label_t> labels;
  std::vector<size_t> back;  // moveBackIndexVector
  size_t vertex_length = 0;
  size_t length() const { return moves.size(); }
};

// MultipleLabelConstraintTemplate (multiple_label_constraint_template.h:20-60).
enum TemplateOrigin : int { kEmpty = 0, kCC, kPC, kTdsCC, kTdsPC, kTdsSub, kTdsFull };
struct TemplateConstraint {
  int origin = kEmpty;
  size_t length = 0;
  std::unordered_map<uint32_t, std::set<uint32_t>> graph;  // vertexIndexGraph
  std::unordered_map<uint32_t, Walk> walks;                // walkMap
  bool operator==(const TemplateConstraint& o) const { return length == o.length && graph == o.graph; }
};

struct QueryConstraints {
  std::vector<LocalConstraint> local;
  std::vector<CycleConstraint> cycles;
  std::vector<PathConstraint> paths;
  std::vector<TemplateConstraint> templates;
  TemplateConstraint enumeration;
};

// Throws PmError(PM_E_PATTERN_TOO_LARGE) above 64 pattern vertices.
QueryConstraints compile_constraints(const PatternGraph& pattern);

// The text the reference's generators print into log.totem
// (generate_constraint_*::print), concatenated in generation order.
std::string dump_constraints(const QueryConstraints& qc);

}  // namespace pmgb
