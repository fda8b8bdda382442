#include "walk_compile.h"

#include <cstring>

namespace pmgb {
namespace {

WalkProgram empty_program(uint8_t family, uint8_t start_role) {
  WalkProgram p;
  memset(&p, 0, sizeof(p));
  p.family = family;
  p.start_role = start_role;
  p.n_hist = 1;
  p.hist_step[0] = 0;
  for (int i = 0; i < kMaxWalkSteps; ++i) p.steps[i].blocker = -1;
  return p;
}

void check_length(size_t n_steps) {
  if (n_steps + 1 > static_cast<size_t>(kMaxWalkSteps))
    throw PmError{PM_E_PATTERN_TOO_LARGE,
                  "constraint walk has " + std::to_string(n_steps) + " steps; the device walker supports " +
                      std::to_string(kMaxWalkSteps - 1)};
}

WalkStep vertex_step(uint8_t role) {
  WalkStep s;
  memset(&s, 0, sizeof(s));
  s.kind = kStepVertex;
  s.role = role;
  s.blocker = -1;
  return s;
}

// Resolves blockers: a VERTEX step testing value X is blocked by the VERTEX
// step (index >= 1) whose role is X.
void finish(WalkProgram& p, const std::vector<int>& test_value) {
  for (int d = 1; d < p.n_steps; ++d) {
    WalkStep& s = p.steps[d];
    if (s.kind != kStepVertex || test_value[d] < 0) continue;
    for (int t = 1; t < p.n_steps; ++t) {
      const WalkStep& o = p.steps[t];
      if (o.kind == kStepVertex && o.role == static_cast<uint8_t>(test_value[d])) {
        s.blocker = static_cast<int8_t>(t);
        p.steps[t].record = 1;
        break;
      }
    }
  }
  p.any_memo = 0;
  for (int d = 1; d < p.n_steps; ++d)
    if (p.steps[d].blocker >= 0 || p.steps[d].hyp) p.any_memo = 1;
}

void add_history(WalkProgram& p, int step) { p.hist_step[p.n_hist++] = static_cast<uint8_t>(step); }

void finalize(CompiledConstraint& cc) {
  memset(cc.role_index, 0xFF, sizeof(cc.role_index));
  cc.start_mask = 0;
  cc.marks_per_success = 0;
  cc.any_memo = false;
  for (size_t i = 0; i < cc.programs.size(); ++i) {
    const WalkProgram& p = cc.programs[i];
    cc.role_index[p.start_role] = static_cast<uint8_t>(i);
    cc.start_mask |= uint64_t(1) << p.start_role;
    int marks = 0;
    for (int d = 1; d < p.n_steps; ++d) marks += p.steps[d].mark;
    if (marks > cc.marks_per_success) cc.marks_per_success = marks;
    cc.any_memo = cc.any_memo || p.any_memo;
  }
}

}  // namespace

CompiledConstraint compile_cycle(const CycleConstraint& c) {
  CompiledConstraint cc;
  cc.family = kFamilyCC;
  const int L = static_cast<int>(c.length());
  check_length(L);
  for (int s = 0; s < L; ++s) {
    WalkProgram p = empty_program(kFamilyCC, static_cast<uint8_t>(c.ids[s]));
    p.n_steps = static_cast<uint16_t>(L + 1);
    std::vector<int> test(p.n_steps, -1);
    for (int t = 1; t < L; ++t) {
      p.steps[t] = vertex_step(static_cast<uint8_t>(c.ids[(s + t) % L]));
      p.steps[t].mark = 1;
      test[t] = (s + t - 1) % L;  // current cycle position
      add_history(p, t);
    }
    WalkStep close;
    memset(&close, 0, sizeof(close));
    close.kind = kStepCheck;
    close.hist = 0;
    close.blocker = -1;
    p.steps[L] = close;
    finish(p, test);
    cc.programs.push_back(p);
  }
  finalize(cc);
  return cc;
}

CompiledConstraint compile_path(const PathConstraint& pc) {
  CompiledConstraint cc;
  cc.family = kFamilyPC;
  const int L = static_cast<int>(pc.length());
  check_length(L);
  for (int dir = 0; dir < 2; ++dir) {
    const bool reverse = dir == 1;
    auto role_at = [&](int t) { return static_cast<uint8_t>(reverse ? pc.ids[L - 1 - t] : pc.ids[t]); };
    WalkProgram p = empty_program(kFamilyPC, role_at(0));
    p.n_steps = static_cast<uint16_t>(L);
    std::vector<int> test(p.n_steps, -1);
    for (int t = 1; t <= L - 2; ++t) {
      p.steps[t] = vertex_step(role_at(t));
      test[t] = reverse ? (L - t) : (t - 1);  // current path position
      add_history(p, t);
    }
    WalkStep fin = vertex_step(role_at(L - 1));
    fin.kind = kStepFinal;
    fin.mark = 1;
    p.steps[L - 1] = fin;
    add_history(p, L - 1);
    finish(p, test);
    cc.programs.push_back(p);
  }
  finalize(cc);
  return cc;
}

namespace {
WalkProgram program_from_walk(const Walk& w, uint32_t start_role, uint8_t family) {
  WalkProgram p = empty_program(family, static_cast<uint8_t>(start_role));
  const int n = static_cast<int>(w.length());
  check_length(n);
  p.n_steps = static_cast<uint16_t>(n);
  std::vector<int> test(n, -1);
  for (int d = 1; d < n; ++d) {
    const int m = w.moves[d];
    if (m == kVertexStore || m == kVertexNoStore) {
      WalkStep s = vertex_step(static_cast<uint8_t>(w.ids[d]));
      if (family == kFamilyTDS) {
        s.mark = 1;
        s.store = m == kVertexStore;
        s.hyp = m == kVertexNoStore;
        test[d] = static_cast<int>(w.ids[d - 1]);
      }
      p.steps[d] = s;
      add_history(p, d);
      if (s.store) p.store_step[p.n_store++] = static_cast<uint8_t>(d);
    } else {
      WalkStep s;
      memset(&s, 0, sizeof(s));
      s.kind = m == kCheck ? kStepCheck : kStepMove;
      s.hist = static_cast<uint8_t>(w.back[d]);
      s.blocker = -1;
      p.steps[d] = s;
    }
  }
  if (family == kFamilyTDS) finish(p, test);
  return p;
}
}  // namespace

CompiledConstraint compile_template(const TemplateConstraint& t) {
  CompiledConstraint cc;
  cc.family = kFamilyTDS;
  for (const auto& kv : t.walks) cc.programs.push_back(program_from_walk(kv.second, kv.first, kFamilyTDS));
  finalize(cc);
  return cc;
}

CompiledConstraint compile_enumeration(const TemplateConstraint& t) {
  CompiledConstraint cc;
  cc.family = kFamilyEnum;
  auto first = t.walks.cbegin();
  cc.programs.push_back(program_from_walk(first->second, first->first, kFamilyEnum));
  finalize(cc);
  return cc;
}

}  // namespace pmgb
