// Autotuner over the speed-only choices: LCC degree classes of a graph and
// the ENUMERATION slicing / count-memo size (see autotune.cc).
#pragma once
#include <vector>

#include "engine.h"

namespace pmgb {

struct TuneResult {
  uint32_t hub_degree = 0, seg_entries = 0;
  uint32_t enum_presplit_memo = 0, enum_presplit_plain = 0, enum_table_entries = 0;
  uint32_t walk_presplit = 0, walk_table_entries = 0;
  uint32_t probes_memo = 0, probes_plain = 0;  // probe templates per program kind
  uint32_t runs = 0;                            // candidate runs over the probes
  uint32_t enum_tail_swap = 0, walk_tail_swap = 0, enum_count_memo = 1, walk_tail_state_memo = 1;
  uint32_t enum_pair_tail = 1, walk_pair_tail = 1, enum_second_split = 0;
};

// Times up to max_per_group templates with and without a count memo under
// each candidate and leaves the fastest choices in force (the graph's plan,
// the process-wide enumeration settings).  No query of g may be running.
TuneResult autotune(GraphImpl* g, const std::vector<PatternGraph>& templates, uint32_t max_per_group);

}  // namespace pmgb
