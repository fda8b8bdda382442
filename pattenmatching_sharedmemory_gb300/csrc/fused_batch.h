// Batched form: many template queries over one resident graph, with the LCC
// work of all of them in shared launches.
//
// The reference runs one template per process (MultipleLabelCpu::
// runPatternMatching, multiple_label_cpu.cc:113-184); each query here keeps
// that schedule (multiple_label_step.cc:30-83) on its own state.  A
// coordinator thread repeatedly takes the queries that are between steps:
//   - those whose next step is LCC0, or the LCC fixpoint right after LCC0
//     (every vertex scheduled), run it together: one multi-query launch
//     (LCC0), or one multi-query launch sequence per pass over the queries
//     still iterating (LCC), whose blocks of different queries walk the same
//     CSR ranges at the same time, so one HBM read of an adjacency range
//     serves every query in the group;
//   - every other query goes to a pool of host threads, where a worker runs
//     its units (later LCC fixpoints as one captured launch each, CC / PC /
//     TDS / ENUMERATION, any step of a query whose graph state is empty) on
//     the query's own stream up to its end, overlapping the walker launches
//     of other queries and the shared LCC launches.
// No query waits for another's walker step.  Results are those of each query
// run alone: the same rows (timing columns aside), state and match count.
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

  // Runs every query to its end (or failure).  At most one query per host
  // worker (16 at most) is in flight at a time, the others enter in order as
  // queries finish; a per-query budget (query_budget_ms) runs from when the
  // query enters.
  void run();
  size_t size() const { return items_.size(); }
  FusedBatchItem& item(size_t i) { return items_.at(i); }
  // Coordinator passes and shared LCC phases issued (statistics).
  uint64_t rounds = 0, fused_lcc_passes = 0;

 private:
  void worker();

  GraphImpl* g_;
  bool prune_only_;
  std::vector<FusedBatchItem> items_;
  std::vector<uint8_t> running_;  // a step of the query is on a worker
  cudaStream_t stream_ = nullptr;
  // host thread pool for the per-query steps
  std::vector<std::thread> workers_;
  uint32_t n_workers_ = 1;  // the walker grid share of each worker
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::vector<size_t> queue_;     // queries whose next step a worker should run
  size_t finished_steps_ = 0;     // steps finished since the coordinator last looked
  bool stop_ = false;
};

}  // namespace pmgb
