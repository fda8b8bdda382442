// Batched form: many template queries over one resident graph advanced in
// lockstep rounds, with the LCC work of all of them in shared launches.
//
// The reference runs one template per process (MultipleLabelCpu::
// runPatternMatching, multiple_label_cpu.cc:113-184); each query here keeps
// that schedule (multiple_label_step.cc:30-83) on its own state.  A round
// advances every unfinished query by at least one step:
//   1. the queries at LCC0 run it together (one multi-query launch);
//   2. the queries at LCC run their fixpoints together: each pass is one
//      multi-query launch sequence over the queries still iterating, whose
//      blocks of different queries walk the same CSR ranges at the same time
//      (one HBM read of an adjacency range serves every query in the batch);
//   3. every other query runs its next step (CC / PC / TDS / ENUMERATION, or
//      any step of a query whose graph state is empty) on its own stream,
//      from a pool of host threads, so their walker launches overlap.
// Results are those of each query run alone: the same rows (timing columns
// aside), state and match count.
#pragma once
#include <condition_variable>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

namespace pmgb {

struct FusedBatchItem {
  std::unique_ptr<QueryImpl> q;
  int status = PM_SUCCESS;
  std::string error;
  bool done = false;
  double run_ms = 0;
};

class FusedBatch {
 public:
  // Compiles every template and allocates its state (stream of its own).
  // prune_only: stop each query where its schedule reaches ENUMERATION.
  FusedBatch(GraphImpl* g, const std::vector<PatternGraph>& patterns, bool prune_only);
  ~FusedBatch();
  FusedBatch(const FusedBatch&) = delete;
  FusedBatch& operator=(const FusedBatch&) = delete;

  // Runs every query to its end (or failure).  A per-query budget
  // (query_budget_ms) runs from the start of this call.
  void run();
  size_t size() const { return items_.size(); }
  FusedBatchItem& item(size_t i) { return items_.at(i); }
  // Rounds run and shared LCC launches issued (statistics).
  uint64_t rounds = 0, fused_lcc_passes = 0;

 private:
  void parallel_steps(const std::vector<size_t>& idx);

  GraphImpl* g_;
  bool prune_only_;
  std::vector<FusedBatchItem> items_;
  cudaStream_t stream_ = nullptr;
  // host thread pool for step 3
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::vector<std::function<void()>> tasks_;
  size_t next_task_ = 0, finished_tasks_ = 0;
  uint64_t generation_ = 0;
  bool stop_ = false;
};

}  // namespace pmgb
