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

// A VERTEX step testing value X is blocked by the VERTEX step (index >= 1)
// whose role is X (see walk_program.h).
void resolve_blockers(WalkProgram& p, const std::vector<int>& test_value) {
  for (int d = 1; d < p.n_steps; ++d) {
    WalkStep& s = p.steps[d];
    if (s.kind != kStepVertex || test_value[d] < 0) continue;
    for (int t = 1; t < p.n_steps; ++t) {
      const WalkStep& o = p.steps[t];
      if (o.kind == kStepVertex && o.role == static_cast<uint8_t>(test_value[d])) {
        s.blocker = static_cast<int8_t>(t);
        break;
      }
    }
  }
}

// Static analysis (see walk_program.h): drops memo tests that can never
// block, decides exactness, computes state keys and the CHECK-only tail.
void analyze(WalkProgram& p, const std::vector<label_t>& role_label) {
  const int n = p.n_steps;
  auto hist_role = [&](int h) -> int { return h == 0 ? p.start_role : p.steps[p.hist_step[h]].role; };
  std::vector<int> cur_role(n + 1, -1);
  cur_role[1] = p.start_role;
  for (int d = 1; d < n; ++d) {
    const WalkStep& s = p.steps[d];
    cur_role[d + 1] = (s.kind == kStepVertex || s.kind == kStepFinal) ? s.role
                      : s.kind == kStepCheck                          ? cur_role[d]
                                                                      : hist_role(s.hist);
  }
  auto compat = [&](int a, int b) { return a == b || role_label[a] == role_label[b]; };
  for (int d = 1; d < n; ++d) {
    WalkStep& s = p.steps[d];
    if (s.kind != kStepVertex || s.blocker < 0) continue;
    // The test at d (current role A -> candidate role B) is blocked only by
    // a traversal at step t (current role X -> bound role Y) of the same
    // undirected edge: {A-vertex, B-vertex} = {X-vertex, Y-vertex}.
    const int t = s.blocker;
    const int A = cur_role[d], B = s.role, X = cur_role[t], Y = p.steps[t].role;
    const bool possible = (compat(A, X) && compat(B, Y)) || (compat(A, Y) && compat(B, X));
    if (!possible) s.blocker = -1;
  }
  for (int t = 1; t < n; ++t) p.steps[t].record = 0;
  p.any_memo = 0;
  for (int d = 1; d < n; ++d) {
    if (p.steps[d].blocker >= 0) p.steps[p.steps[d].blocker].record = 1;
    if (p.steps[d].blocker >= 0 || p.steps[d].hyp) p.any_memo = 1;
  }
  // History entries read after step d that were bound before it.
  std::vector<uint64_t> refs(n + 1, 0);
  for (int d = 1; d < n; ++d)
    for (int j = d + 1; j < n; ++j) {
      const WalkStep& s = p.steps[j];
      if (s.kind != kStepCheck && s.kind != kStepMove) continue;
      const int h = s.hist;
      if (h > 0 && p.hist_step[h] < d) refs[d] |= uint64_t(1) << h;
    }
  // Injective (strict) walks: the subtree below a hop depends on every
  // vertex bound so far, and the tail shortcuts of exact programs do not
  // test injectivity, so such programs are walked as non-exact ones with
  // the whole history in their state key.
  bool exact = p.family != kFamilyEnum && !p.injective;
  for (int d = 1; d < n && exact; ++d) {
    const WalkStep& s = p.steps[d];
    if (s.kind == kStepVertex && s.blocker >= 0) exact = false;
    if (s.kind == kStepVertex && s.hyp) {
      for (int h = 1; h < p.n_hist; ++h)
        if ((refs[d] >> h & 1) && !p.steps[p.hist_step[h]].store) exact = false;
    }
  }
  p.exact = exact ? 1 : 0;
  // State key: the history entries the subtree reads, plus (for programs
  // that keep the reference's hypothesis memo) every stored vertex so far.
  p.max_refs = 0;
  for (int d = 1; d < n; ++d) {
    uint64_t key = 0;
    if (p.steps[d].kind == kStepVertex || (p.injective && p.steps[d].kind == kStepFinal)) {
      key = refs[d];
      if (p.injective)
        for (int h = 1; h < p.n_hist; ++h)
          if (p.hist_step[h] < d) key |= uint64_t(1) << h;
      if (!exact)
        for (int h = 1; h < p.n_hist; ++h)
          if (p.hist_step[h] < d && p.steps[p.hist_step[h]].store) key |= uint64_t(1) << h;
    }
    p.state_refs[d] = key;
    const int c = __builtin_popcountll(key);
    if (c > p.max_refs) p.max_refs = static_cast<uint8_t>(c);
  }
  bool distinct = true;
  for (size_t a = 0; a < role_label.size() && distinct; ++a)
    for (size_t b = a + 1; b < role_label.size(); ++b)
      if (role_label[a] == role_label[b]) {
        distinct = false;
        break;
      }
  p.count_memo = (p.family == kFamilyEnum && distinct) ? 1 : 0;
  int tail = n;
  while (tail - 1 >= 1 && p.steps[tail - 1].kind == kStepCheck) --tail;
  p.tail_from = static_cast<uint8_t>(tail);
}

void add_history(WalkProgram& p, int step) { p.hist_step[p.n_hist++] = static_cast<uint8_t>(step); }

void finalize(CompiledConstraint& cc) {
  memset(cc.role_index, 0xFF, sizeof(cc.role_index));
  cc.start_mask = 0;
  cc.marks_per_success = 0;
  cc.any_memo = false;
  cc.exact = true;
  cc.max_state_words = 0;
  cc.max_hyp_words = 0;
  for (size_t i = 0; i < cc.programs.size(); ++i) {
    const WalkProgram& p = cc.programs[i];
    cc.role_index[p.start_role] = static_cast<uint8_t>(i);
    cc.start_mask |= uint64_t(1) << p.start_role;
    int marks = 0;
    for (int d = 1; d < p.n_steps; ++d) marks += p.steps[d].mark;
    if (marks > cc.marks_per_success) cc.marks_per_success = marks;
    cc.any_memo = cc.any_memo || p.any_memo;
    cc.exact = cc.exact && p.exact;
    if (p.max_refs > cc.max_state_words) cc.max_state_words = p.max_refs;
    if (!p.exact && p.n_store > cc.max_hyp_words) cc.max_hyp_words = p.n_store;
  }
}

}  // namespace

CompiledConstraint compile_cycle(const CycleConstraint& c, const std::vector<label_t>& role_label, int variant) {
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
    p.injective = variant == kNlccStrict;
    // The reference's edge memo; the backtrack walks' (vertex, template
    // vertex) memo never blocks a walk that could still succeed, so it is
    // the state memo of exact programs.
    if (variant == kNlccReference) resolve_blockers(p, test);
    analyze(p, role_label);
    cc.programs.push_back(p);
  }
  finalize(cc);
  return cc;
}

CompiledConstraint compile_path(const PathConstraint& pc, const std::vector<label_t>& role_label, int variant) {
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
    p.injective = variant == kNlccStrict;
    if (variant == kNlccReference) resolve_blockers(p, test);
    analyze(p, role_label);
    cc.programs.push_back(p);
  }
  finalize(cc);
  return cc;
}

namespace {
WalkProgram program_from_walk(const Walk& w, uint32_t start_role, uint8_t family,
                              const std::vector<label_t>& role_label, int variant = kNlccReference) {
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
        // Strict walks keep no hypothesis memo (and so no stored vertices).
        s.store = variant != kNlccStrict && m == kVertexStore;
        s.hyp = variant != kNlccStrict && m == kVertexNoStore;
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
  p.injective = family == kFamilyTDS && variant == kNlccStrict;
  if (family == kFamilyTDS && variant == kNlccReference) resolve_blockers(p, test);
  analyze(p, role_label);
  return p;
}
}  // namespace

CompiledConstraint compile_template(const TemplateConstraint& t, const std::vector<label_t>& role_label,
                                    int variant) {
  CompiledConstraint cc;
  cc.family = kFamilyTDS;
  for (const auto& kv : t.walks)
    cc.programs.push_back(program_from_walk(kv.second, kv.first, kFamilyTDS, role_label, variant));
  finalize(cc);
  return cc;
}

CompiledConstraint compile_enumeration(const TemplateConstraint& t, const std::vector<label_t>& role_label) {
  CompiledConstraint cc;
  cc.family = kFamilyEnum;
  auto first = t.walks.cbegin();
  cc.programs.push_back(program_from_walk(first->second, first->first, kFamilyEnum, role_label));
  finalize(cc);
  cc.exact = false;
  return cc;
}

}  // namespace pmgb
