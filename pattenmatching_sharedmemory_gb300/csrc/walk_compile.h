// Compiles CC / PC / TDS / enumeration constraints into WalkPrograms.
// role_label[p] is the label of template vertex p (for the memo analysis).
#pragma once
#include <vector>

#include "constraints.h"
#include "walk_program.h"

namespace pmgb {

struct CompiledConstraint {
  uint8_t family = 0;
  std::vector<WalkProgram> programs;  // one per start role, in the reference's order
  uint64_t start_mask = 0;            // union of start roles
  uint8_t role_index[64];             // role -> program index (0xFF: not a start role)
  int marks_per_success = 0;          // marking steps of the longest program
  bool any_memo = false;
  bool exact = false;                 // every program exact (see walk_program.h)
  uint32_t max_state_words = 0;       // key words of the state / count memo
  uint32_t max_hyp_words = 0;         // key words of the reference's hypothesis memo
};

// Walk semantics of the CC / PC / TDS steps: the reference's walks with their
// edge memo (and TDS hypothesis memo), or the article drivers' variants
// (test_article/CMakeLists.txt:12-33): strict walks bind no vertex twice and
// keep no memo (multiple_label_test/*_strict_cpu.tpp); backtrack walks skip
// a (vertex, template vertex) pair the source's walk already visited (CC,
// PC) or keep only the hypothesis memo (TDS) (*_backtrack_cpu.tpp).
enum NlccVariant : int { kNlccReference = 0, kNlccStrict = 1, kNlccBacktrack = 2 };

// CC: one program per cycle position (multiple_label_cc_cpu.tpp:94-129).
CompiledConstraint compile_cycle(const CycleConstraint& c, const std::vector<label_t>& role_label,
                                 int variant = kNlccReference);
// PC: forward from ids[0], then backward from ids[L-1] (pc :104-142).
CompiledConstraint compile_path(const PathConstraint& p, const std::vector<label_t>& role_label,
                                int variant = kNlccReference);
// TDS: one program per walkMap entry, in walkMap order (tds :153-195).
CompiledConstraint compile_template(const TemplateConstraint& t, const std::vector<label_t>& role_label,
                                    int variant = kNlccReference);
// ENUMERATION: the first walkMap entry (enumeration :133-135).
CompiledConstraint compile_enumeration(const TemplateConstraint& t, const std::vector<label_t>& role_label);

}  // namespace pmgb
