// Query server over one resident graph: continuous batching of template
// queries onto a fixed number of GPU slots with admission by device memory.
//
// Each slot is a worker thread with its own CUDA stream and pinned counter
// words.  A request waits in a FIFO queue until a slot is free and the
// device bytes it is charged (estimate_query_bytes) fit under the memory
// budget beside the requests already running; it then runs the full
// pipeline (LCC0 ... ENUMERATION) on its slot's stream while the other
// slots' queries run on theirs, so their kernels overlap on the GPU.  A
// request that could never fit (charged bytes above the budget) is refused
// at submission.  Query buffers are stream-ordered allocations, so a query
// starting or finishing never waits for another slot's work.
#pragma once
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"

namespace pmgb {

constexpr uint32_t kSubmitExportState = 1;  // keep the final state for export
constexpr uint32_t kSubmitPruneOnly = 2;    // stop when the schedule reaches ENUMERATION

struct ServeRequest {
  using Clock = std::chrono::steady_clock;
  enum State { kQueued, kRunning, kDone };

  uint64_t ticket = 0;
  PatternGraph pattern;
  uint32_t flags = 0;
  uint64_t bytes = 0;  // device bytes charged at admission
  State state = kQueued;
  Clock::time_point t_submit, t_admit, t_done;
  std::atomic<bool> cancel{false};  // set by Server::cancel while running

  int status = PM_SUCCESS;
  std::string error;
  uint64_t match_count = 0;
  double gpu_ms = 0;  // sum of the step times
  std::vector<pm_step_record> records;  // results.totem rows, END included
  std::vector<uint64_t> cand;           // with kSubmitExportState
  std::vector<uint8_t> eact, vact;
};

struct ServerStats {
  uint64_t queued = 0, running = 0, done = 0;
  uint64_t bytes_in_use = 0, peak_bytes = 0, budget = 0;
  uint32_t slots = 0;
};

class Server {
 public:
  // slots >= 1; budget 0 = 90 % of the device's free memory now.
  Server(GraphImpl* graph, uint32_t slots, uint64_t budget, uint32_t walk_share = 0);
  ~Server();  // queued requests end with PM_E_CANCELLED; running ones finish
  Server(const Server&) = delete;
  Server& operator=(const Server&) = delete;

  uint64_t submit(const PatternGraph& pattern, uint32_t flags);
  // The request, or null for an unknown (or released) ticket; *done tells
  // (read under the server's lock) whether its results may be read.
  std::shared_ptr<ServeRequest> find(uint64_t ticket, bool* done = nullptr);
  // Waits until the request is done or timeout_ms (< 0: forever) passed;
  // true when done.
  bool wait(uint64_t ticket, double timeout_ms);
  void release(uint64_t ticket);
  // A queued request is dropped (PM_E_CANCELLED); a running one stops before
  // its next step (PM_E_CANCELLED); a finished one is left as it is.
  // Returns the request's state when the call was made.
  int cancel(uint64_t ticket);
  ServerStats stats();

 private:
  void worker(uint32_t slot);
  bool admissible() const;

  GraphImpl* g_;
  uint32_t slots_;
  uint64_t budget_;
  uint32_t walk_share_ = 0;  // walker grid share of a slot (0: one per slot)
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::deque<std::shared_ptr<ServeRequest>> queue_;
  std::unordered_map<uint64_t, std::shared_ptr<ServeRequest>> requests_;
  uint64_t next_ticket_ = 1;
  uint64_t used_ = 0, peak_ = 0, running_ = 0, done_ = 0;
  bool stop_ = false;
  std::string start_error_;
  std::vector<std::thread> workers_;
};

}  // namespace pmgb
