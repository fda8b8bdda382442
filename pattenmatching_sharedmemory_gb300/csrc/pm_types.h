// Shared host-side types of the GB300 PruneJuice pipeline.
//
// Vertex ids are 32-bit and CSR offsets 64-bit (the reference's vid_t /
// eid_t with FEATURE_64BIT_EDGE_ID, src/totem/totem_graph.h:64-72); vertex
// labels are the reference's 64-bit weight_t values
// (src/totem/totem_graph.h:89-95).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pm_gb300.h"

namespace pmgb {

using vid_t = uint32_t;
using eid_t = uint64_t;
using label_t = uint64_t;

// Maximum template size (reference: C_MAXIMUM_PATTERN_SIZE = 64,
// src/patternmatching/multiple_label/multiple_label_common.h:14).
constexpr uint32_t kMaxPatternSize = 64;

// A host CSR graph in the TOTEM layout (src/totem/totem_graph.h:137-180):
// offsets has V+1 entries, adj has E entries, labels has V entries
// (the reference's graph->values; 0 when no label file was given).
struct HostGraph {
  uint32_t vertex_count = 0;
  uint64_t edge_count = 0;
  bool directed = false;
  bool valued = false;
  std::vector<uint64_t> offsets;
  std::vector<uint32_t> adj;
  std::vector<uint64_t> labels;
};

// Error with a TOTEM-style status code (SUCCESS=0 / FAILURE=-1 plus the
// distinct negative codes declared in pm_gb300.h).
struct PmError {
  int code;
  std::string message;
};

}  // namespace pmgb
