// Flat "walk programs": the device form of the non-local constraints.
//
// Every CC, PC and TDS check of the reference is a depth-first token walk
// from one source vertex holding one start role:
//   CC   multiple_label_cc_cpu.tpp:13-70   (closed walk along a cycle)
//   PC   multiple_label_pc_cpu.tpp:12-81   (walk along a path, end != source)
//   TDS  multiple_label_tds_cpu.tpp:14-127 (template walk: vertex / check /
//        move-back moves, utils/walk.cc)
// A WalkProgram lists the steps after the source.  Step kinds:
//   VERTEX  bind an active neighbour (active CSR entry) holding `role`
//   FINAL   PC's last hop: like VERTEX, neighbour must differ from the source
//   CHECK   an active CSR entry from the current vertex to history[hist]
//           must exist (CC's closing hop is CHECK of history[0])
//   MOVE    continue from history[hist] (TDS move-back)
// and reaching step n_steps is success.
//
// Memo semantics made explicit.  The reference keeps, per source, a map
// undirected edge -> 64-bit set that a VERTEX hop tests with one value and
// fills with another (CC/PC: test the current cycle/path position, insert
// the next template vertex id; TDS: test the previous walk entry's template
// vertex, insert the next).  Inserted values are the roles of VERTEX steps,
// and those are distinct, so "value X is in memo[edge]" means "edge was
// traversed by the VERTEX step whose role is X".  Each VERTEX step therefore
// carries `blocker` — the step whose traversals block it, or -1 — and each
// step that some other step tests against carries `record`.  TDS adds, for
// no-store vertex moves, a memo of (vertex, step, stored-vertex tuple): a
// hop is skipped when the same neighbour was already bound at this step with
// the same stored vertices (store moves never match, their entries are one
// element longer).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define PM_HD __host__ __device__
#else
#define PM_HD
#endif

namespace pmgb {

constexpr int kMaxWalkSteps = 96;  // steps per program, source included

enum WalkStepKind : uint8_t { kStepVertex = 0, kStepCheck = 1, kStepMove = 2, kStepFinal = 3 };
enum WalkFamily : uint8_t { kFamilyCC = 0, kFamilyPC = 1, kFamilyTDS = 2, kFamilyEnum = 3 };

struct WalkStep {
  uint8_t kind;
  uint8_t role;     // VERTEX / FINAL
  uint8_t hist;     // CHECK / MOVE: history index (0 = source)
  int8_t blocker;   // VERTEX: blocking step, -1 none
  uint8_t record;   // VERTEX: traversals recorded in the edge memo
  uint8_t hyp;      // VERTEX: no-store TDS move (hypothesis memo)
  uint8_t store;    // VERTEX: store TDS move
  uint8_t mark;     // success marks (bound vertex, role) — alreadyMatched
};

// Exact programs.  When no memo test of a program can ever block a hop (the
// two roles involved in every possible block carry different labels, so no
// vertex can hold both) and every TDS hypothesis memo keys on all history
// entries its subtree reads, the reference's walk returns exactly whether a
// valid walk exists: its memos only skip subtrees that already failed.  For
// such programs the walker may prune any revisited state (neighbour, step,
// values of the earlier history entries read later — `state_refs`), which
// turns the exponential walk into a search over distinct states with the
// same outcome, and no alreadyMatched rescue can occur (a vertex on a
// successful walk has a valid walk itself).
//
// State memo (every CC/PC/TDS program).  The subtree below a hop depends only
// on the bound neighbour, the step, the earlier history entries it reads
// and — for the reference's hypothesis memo — the stored vertices bound so
// far; the memos only ever block, so a second visit of the same state can
// neither succeed where the first failed nor insert memo entries the first
// did not.  The walker therefore skips revisits of a state keyed by
// (neighbour, step, values of the history entries in state_refs[d]) after
// doing the reference's own memo tests and inserts: same outcome, same memo
// contents, polynomial instead of exponential work.  The table is
// best-effort: when it fills up the walker stops inserting.
//
// Count memo (ENUMERATION of templates whose labels are pairwise distinct):
// no vertex can hold two roles, so the embeddings are injective by
// construction and the number of completions below a hop depends only on the
// same state; it is memoized per source.
struct WalkProgram {
  uint16_t n_steps;      // steps[1 .. n_steps-1]; step n_steps = success
  uint8_t start_role;
  uint8_t family;
  uint8_t n_hist;        // history entries (source + VERTEX/FINAL steps)
  uint8_t n_store;       // store steps
  uint8_t any_memo;      // some step has blocker >= 0 or hyp
  uint8_t exact;         // see above
  uint8_t max_refs;      // largest popcount of state_refs
  uint8_t tail_from;     // first step of the trailing CHECK-only suffix
  uint8_t count_memo;    // ENUMERATION: subtree counts may be memoized
  uint8_t injective;     // CC/PC/TDS: no vertex bound twice (the article
                         // drivers' strict walks); ENUMERATION always is
  uint8_t pad[4];
  uint8_t hist_step[kMaxWalkSteps];   // history index -> step index
  uint8_t store_step[kMaxWalkSteps];  // i-th store step
  uint64_t state_refs[kMaxWalkSteps]; // history indices (>0) keyed by the
                                      // state / count memo at step d
  WalkStep steps[kMaxWalkSteps];
};

}  // namespace pmgb
