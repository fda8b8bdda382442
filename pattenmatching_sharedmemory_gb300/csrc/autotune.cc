// Autotuner for the speed-only choices of the pipeline: the LCC degree
// classes of a graph (hub_degree, seg_entries), the CC/PC/TDS slicing and
// state-memo size, and the ENUMERATION slicing and count-memo size.  It runs
// the caller's probe templates under each candidate, keeps the candidate
// with the least device time for the steps it affects, and leaves it in
// force.  Every candidate must reproduce the
// same match counts (the choices change speed only); a difference is an
// internal error.
#include "autotune.h"

#include <algorithm>
#include <limits>

namespace pmgb {
namespace {

struct ProbeRun {
  double lcc_ms = 0, walk_ms = 0, enum_ms = 0;
  std::vector<uint64_t> counts;
};

ProbeRun run_probes(GraphImpl* g, const std::vector<const PatternGraph*>& probes) {
  ProbeRun r;
  for (const PatternGraph* p : probes) {
    QueryImpl q;
    q.create(g, *p, nullptr);
    q.run_all();
    for (const pm_step_record& rec : q.records) {
      if (rec.step == PM_STEP_LCC) r.lcc_ms += rec.step_ms;
      if (rec.step == PM_STEP_CC || rec.step == PM_STEP_PC || rec.step == PM_STEP_TDS) r.walk_ms += rec.step_ms;
      if (rec.step == PM_STEP_ENUMERATION) r.enum_ms += rec.step_ms;
    }
    r.counts.push_back(q.match_count);
  }
  return r;
}

bool has_count_memo(const PatternGraph& p) {
  const QueryConstraints qc = compile_constraints(p);
  const CompiledConstraint cc = compile_enumeration(qc.enumeration, p.labels);
  return !cc.programs.empty() && cc.programs[0].count_memo;
}

}  // namespace

TuneResult autotune(GraphImpl* g, const std::vector<PatternGraph>& templates, uint32_t max_per_group) {
  if (templates.empty()) throw PmError{PM_E_INVALID_ARG, "autotune needs at least one template"};
  if (max_per_group == 0) max_per_group = 1;
  std::vector<const PatternGraph*> memo, plain;
  for (const PatternGraph& p : templates) {
    auto& grp = has_count_memo(p) ? memo : plain;
    if (grp.size() < max_per_group) grp.push_back(&p);
  }
  std::vector<const PatternGraph*> all(memo);
  all.insert(all.end(), plain.begin(), plain.end());

  TuneResult out;
  const std::vector<uint64_t> reference = run_probes(g, all).counts;
  auto check = [&](const ProbeRun& r, const std::vector<const PatternGraph*>& set) {
    ++out.runs;
    // Counts of `set`, which is a prefix (memo) or suffix (plain) of `all`.
    const size_t off = (&set == &plain) ? memo.size() : 0;
    for (size_t i = 0; i < r.counts.size(); ++i)
      if (r.counts[i] != reference[off + i])
        throw PmError{PM_FAILURE, "autotune: a candidate changed a match count"};
  };

  // 1. LCC degree classes, timed on the LCC steps of every probe.
  const std::pair<uint32_t, uint32_t> plans[] = {{32, 1024}, {16, 1024}, {64, 1024}, {32, 512}, {128, 1024}};
  double best = std::numeric_limits<double>::infinity();
  std::pair<uint32_t, uint32_t> best_plan = {g->hub_degree, g->seg_entries};
  for (const auto& pl : plans) {
    g->build_hub_plan(pl.first, pl.second);
    const ProbeRun r = run_probes(g, all);
    check(r, all);
    if (r.lcc_ms < best) {
      best = r.lcc_ms;
      best_plan = pl;
    }
  }
  g->build_hub_plan(best_plan.first, best_plan.second);
  out.hub_degree = best_plan.first;
  out.seg_entries = best_plan.second;

  // 2. CC/PC/TDS slices and state-memo size, timed on those steps.
  {
    const uint32_t walk_slices[] = {0, 16, 64, 256};
    double b = std::numeric_limits<double>::infinity();
    uint32_t pick = walk_presplit();
    for (uint32_t sl : walk_slices) {
      set_walk_presplit(sl);
      const ProbeRun r = run_probes(g, all);
      check(r, all);
      if (r.walk_ms < b) {
        b = r.walk_ms;
        pick = sl;
      }
    }
    set_walk_presplit(pick);
    const uint32_t walk_tables[] = {2048, 8192, 32768};
    b = std::numeric_limits<double>::infinity();
    uint32_t pick_t = walk_table_entries();
    for (uint32_t t : walk_tables) {
      set_walk_table_entries(t);
      const ProbeRun r = run_probes(g, all);
      check(r, all);
      if (r.walk_ms < b) {
        b = r.walk_ms;
        pick_t = t;
      }
    }
    set_walk_table_entries(pick_t);
    out.walk_presplit = pick;
    out.walk_table_entries = pick_t;
    const uint32_t ratios[] = {0, 2, 4, 8};
    b = std::numeric_limits<double>::infinity();
    uint32_t pick_r = walk_tail_swap();
    for (uint32_t rt : ratios) {
      set_walk_tail_swap(rt);
      const ProbeRun r = run_probes(g, all);
      check(r, all);
      if (r.walk_ms < b) {
        b = r.walk_ms;
        pick_r = rt;
      }
    }
    set_walk_tail_swap(pick_r);
    out.walk_tail_swap = pick_r;
    b = std::numeric_limits<double>::infinity();
    bool pick_m = walk_tail_state_memo();
    for (bool on : {true, false}) {
      set_walk_tail_state_memo(on);
      const ProbeRun r = run_probes(g, all);
      check(r, all);
      if (r.walk_ms < b) {
        b = r.walk_ms;
        pick_m = on;
      }
    }
    set_walk_tail_state_memo(pick_m);
    out.walk_tail_state_memo = pick_m ? 1 : 0;
    b = std::numeric_limits<double>::infinity();
    bool pick_p = pair_tail_on(false);
    for (bool on : {true, false}) {
      set_pair_tail(false, on);
      const ProbeRun r = run_probes(g, all);
      check(r, all);
      if (r.walk_ms < b) {
        b = r.walk_ms;
        pick_p = on;
      }
    }
    set_pair_tail(false, pick_p);
    out.walk_pair_tail = pick_p ? 1 : 0;
  }

  // 3. ENUMERATION slices, per program kind, timed on the ENUMERATION steps.
  const uint32_t slices[] = {4, 8, 16, 32, 64};
  for (int kind = 0; kind < 2; ++kind) {
    const bool with_memo = kind == 0;
    const auto& set = with_memo ? memo : plain;
    if (set.empty()) continue;
    double b = std::numeric_limits<double>::infinity();
    uint32_t pick = enum_presplit(with_memo);
    for (uint32_t sl : slices) {
      set_enum_presplit(with_memo, sl);
      const ProbeRun r = run_probes(g, set);
      check(r, set);
      if (r.enum_ms < b) {
        b = r.enum_ms;
        pick = sl;
      }
    }
    set_enum_presplit(with_memo, pick);
  }
  out.enum_presplit_memo = enum_presplit(true);
  out.enum_presplit_plain = enum_presplit(false);

  // 4. ENUMERATION tail from the source's side: chunk ratio, on every probe.
  {
    const uint32_t ratios[] = {0, 2, 4, 8};
    double b = std::numeric_limits<double>::infinity();
    uint32_t pick = enum_tail_swap();
    for (uint32_t rt : ratios) {
      set_enum_tail_swap(rt);
      const ProbeRun r = run_probes(g, all);
      check(r, all);
      if (r.enum_ms < b) {
        b = r.enum_ms;
        pick = rt;
      }
    }
    set_enum_tail_swap(pick);
    out.enum_tail_swap = pick;
  }

  // 5. Count memo on or off, on the probes that can use it.
  if (!memo.empty()) {
    double b = std::numeric_limits<double>::infinity();
    bool pick = enum_count_memo();
    for (bool on : {true, false}) {
      set_enum_count_memo(on);
      const ProbeRun r = run_probes(g, memo);
      check(r, memo);
      if (r.enum_ms < b) {
        b = r.enum_ms;
        pick = on;
      }
    }
    set_enum_count_memo(pick);
  }
  out.enum_count_memo = enum_count_memo() ? 1 : 0;

  // ENUMERATION's pair-parallel step before the tail, on every probe.
  {
    double b = std::numeric_limits<double>::infinity();
    bool pick = pair_tail_on(true);
    for (bool on : {true, false}) {
      set_pair_tail(true, on);
      const ProbeRun r = run_probes(g, all);
      check(r, all);
      if (r.enum_ms < b) {
        b = r.enum_ms;
        pick = on;
      }
    }
    set_pair_tail(true, pick);
    out.enum_pair_tail = pick ? 1 : 0;
  }

  // ENUMERATION second-hop slices, on every probe.
  {
    const uint32_t sizes[] = {0, 64, 256, 1024};
    double b = std::numeric_limits<double>::infinity();
    uint32_t pick = enum_second_split();
    for (uint32_t sz : sizes) {
      set_enum_second_split(sz);
      const ProbeRun r = run_probes(g, all);
      check(r, all);
      if (r.enum_ms < b) {
        b = r.enum_ms;
        pick = sz;
      }
    }
    set_enum_second_split(pick);
    out.enum_second_split = pick;
  }

  // 6. Count-memo entries per warp, on every probe.
  const uint32_t tables[] = {4096, 8192, 16384};
  double bt = std::numeric_limits<double>::infinity();
  uint32_t pick_t = enum_table_entries();
  for (uint32_t t : tables) {
    set_enum_table_entries(t);
    const ProbeRun r = run_probes(g, all);
    check(r, all);
    if (r.enum_ms < bt) {
      bt = r.enum_ms;
      pick_t = t;
    }
  }
  set_enum_table_entries(pick_t);
  out.enum_table_entries = pick_t;
  out.probes_memo = static_cast<uint32_t>(memo.size());
  out.probes_plain = static_cast<uint32_t>(plain.size());
  return out;
}

}  // namespace pmgb
