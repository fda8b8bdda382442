// Dynamic constraint order: graph statistics of the pruned graph and the
// effectiveness estimates the reference's order drivers rank the remaining
// CC / PC / TDS constraints by after every LCC fixpoint
// (src/patternmatching/test_article/test_order_multiple_label_cpu.cc:177-300,
// src/patternmatching/multiple_label/multiple_label_constraint_effectiveness.cc,
// src/patternmatching/algorithms/graph_stat.{h,cc}, graph_stat_cpu.tpp).
//
// The statistics are counts over the active graph (vertices holding a role,
// active CSR entries between them), keyed by template label.  The reference
// keeps them in maps whose entries exist exactly when the count is at least
// one, and reads them with .at(): a read of an absent entry throws
// std::out_of_range and ends the reference's process.  Here every lookup of
// a zero count throws PmError{PM_E_STATISTICS} instead.
//
// The estimates are double-precision formulas restated operation for
// operation (same operands, same order, no contraction), so the ranking they
// give matches the reference's.
#pragma once
#include <cstdint>
#include <vector>

#include "constraints.h"

namespace pmgb {

// PmError{PM_E_STATISTICS, what}.
[[noreturn]] void throw_stat_missing(const std::string& what);

// GraphStat over the template's label slots (slot s = the s-th distinct
// template label in order of first appearance, as in the packed vertex
// word).
struct GraphStat {
  uint32_t slots = 0;
  std::vector<uint64_t> label_of_slot;  // slot -> label value
  std::vector<uint64_t> vertex_total;   // [a]: active vertices of label a
  std::vector<uint64_t> edge_total;     // [a * slots + b]: active entries a -> b
  std::vector<uint64_t> edge_outbound;  // [a]: active entries leaving label a
  // [(a * slots + b) * kMaxAtLeast + i]: vertexLabelWithAtLeastNeighborLabelMap
  // (i = 1 .. accumulation maximum of (a, b); index 0 unused)
  std::vector<uint64_t> at_least;
  static constexpr uint32_t kMaxAtLeast = 64;

  int slot(uint64_t label) const;  // -1 when the label is no template label
  double vertices(uint64_t label) const;
  double edges(uint64_t from, uint64_t to) const;
  double outbound(uint64_t from) const;
  double at_least_count(uint64_t from, uint64_t to, size_t i) const;
};

// GraphStatCpu::preprocessPatern (graph_stat_cpu.tpp:12-38): for each pair of
// template labels (a, b) the largest number of label-b neighbours a label-a
// template vertex has ([a * slots + b], 0 = no such pair), and for each
// label a whether any label-a template vertex has a neighbour at all.
struct AccumulationMaximum {
  uint32_t slots = 0;
  std::vector<uint64_t> label_of_slot;
  std::vector<uint32_t> max;   // [a * slots + b]
  std::vector<uint8_t> has_a;  // accumulationMaximumMap has key a
};
AccumulationMaximum accumulation_maximum(const PatternGraph& p);

struct Effectiveness {
  double match_eliminated = 0, cost_eliminated = 0, effectiveness = 0;
};

// MultipleLabelConstraintEffectiveness::computeBacktrack for a cycle, a path
// and a template constraint (effectiveness.cc:226-340, 570-695, 972-1118);
// threads is the reference's omp_get_max_threads() (the cost divisor).
Effectiveness effectiveness_backtrack(const GraphStat& gs, const CycleConstraint& c, int threads);
Effectiveness effectiveness_backtrack(const GraphStat& gs, const PathConstraint& c, int threads);
Effectiveness effectiveness_backtrack(const GraphStat& gs, const TemplateConstraint& t, int threads);
// MultipleLabelConstraintEffectiveness::compute for the enumeration template
// (effectiveness.cc:697-833), used to decide an early start of ENUMERATION.
Effectiveness effectiveness_enumeration(const GraphStat& gs, const TemplateConstraint& t, int threads);

// The choice the order driver makes after an LCC fixpoint
// (test_order_multiple_label_cpu.cc:177-300): the most effective remaining
// constraint of each kind (first of the largest; none above 0 gives index
// 0), then cycle over path over template on ties, ENUMERATION (use_enumerate)
// or END when no constraint remains, and with early_start ENUMERATION also
// when its estimated cost is at most the chosen constraint's or the chosen
// effectiveness is at most `threshold`.  kind is a pm_step_kind; index
// points into the remaining constraints of that kind.
struct OrderChoice {
  int kind = 0;
  size_t index = 0;
};
OrderChoice choose_next_constraint(const GraphStat& gs, const std::vector<const CycleConstraint*>& cycles,
                                   const std::vector<const PathConstraint*>& paths,
                                   const std::vector<const TemplateConstraint*>& templates,
                                   const TemplateConstraint& enumeration, bool use_enumerate, bool early_start,
                                   double threshold, int threads);

// The static OpenMP schedule the reference's graph-statistics loop runs
// under (graph_stat_cpu.tpp:46-70, `omp for` without a schedule clause):
// `threads` contiguous blocks of vertex ids, the first V % threads of them
// one vertex longer.  Its per-thread accumulation is never reset between
// vertices, so the at-least counts depend on this partition.
struct StaticPartition {
  uint64_t q = 0, r = 0;
  StaticPartition(uint64_t vertices, uint32_t threads) : q(vertices / threads), r(vertices % threads) {}
  uint64_t begin(uint32_t t) const { return t * q + (t < r ? t : r); }
  uint64_t end(uint32_t t) const { return begin(t) + q + (t < r ? 1 : 0); }
};

}  // namespace pmgb
