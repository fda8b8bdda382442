// Compiles CC / PC / TDS / enumeration constraints into WalkPrograms.
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
};

// CC: one program per cycle position (multiple_label_cc_cpu.tpp:94-129).
CompiledConstraint compile_cycle(const CycleConstraint& c);
// PC: forward from ids[0], then backward from ids[L-1] (pc :104-142).
CompiledConstraint compile_path(const PathConstraint& p);
// TDS: one program per walkMap entry, in walkMap order (tds :153-195).
CompiledConstraint compile_template(const TemplateConstraint& t);
// ENUMERATION: the first walkMap entry (enumeration :133-135).
CompiledConstraint compile_enumeration(const TemplateConstraint& t);

}  // namespace pmgb
