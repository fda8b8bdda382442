// Batched form: shared LCC launches, per-query walker steps on a host pool
// (see fused_batch.h).
#include "fused_batch.h"

#include <algorithm>
#include <chrono>

namespace pmgb {

FusedBatch::FusedBatch(GraphImpl* g, const std::vector<PatternGraph>& patterns, bool prune_only)
    : g_(g), prune_only_(prune_only) {
  if (!g_ || g_->device < 0) throw PmError{PM_E_INVALID_ARG, "the graph is not on a device"};
  PM_CUDA(cudaSetDevice(g_->device));
  PM_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  items_.resize(patterns.size());
  running_.assign(patterns.size(), 0);
  try {
    for (size_t i = 0; i < patterns.size(); ++i) {
      items_[i].q = std::make_unique<QueryImpl>();
      items_[i].q->create(g_, patterns[i], nullptr);
      items_[i].q->stop_before_enumeration = prune_only_;
    }
  } catch (...) {
    items_.clear();
    cudaStreamDestroy(stream_);
    throw;
  }
  const size_t n_threads = std::min<size_t>(std::max<size_t>(patterns.size(), 1), 16);
  n_workers_ = static_cast<uint32_t>(n_threads);
  for (size_t t = 0; t < n_threads; ++t) workers_.emplace_back(&FusedBatch::worker, this);
}

FusedBatch::~FusedBatch() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_work_.notify_all();
  for (auto& t : workers_) t.join();
  items_.clear();  // queries free their stream-ordered buffers first
  if (stream_) {
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
}

// Runs the next step of the queries the coordinator queues, one at a time.
void FusedBatch::worker() {
  if (cudaSetDevice(g_->device) != cudaSuccess) return;
  set_thread_walk_grid_share(n_workers_);
  while (true) {
    size_t i = 0;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_work_.wait(lk, [&] { return stop_ || !queue_.empty(); });
      if (stop_) return;
      i = queue_.back();
      queue_.pop_back();
    }
    FusedBatchItem& it = items_[i];
    try {
      // The query's units up to its end or its next shared phase (only
      // LCC0 and the fixpoint right after it are shared, so once a query
      // is past them its worker runs it to the end, as a server slot does).
      QueryImpl& q = *it.q;
      while (true) {
        q.check_request();
        q.run_unit();
        if (q.finished || q.iteration >= 1000 || (prune_only_ && q.step == PM_STEP_ENUMERATION)) break;
        if (q.active_vertices != 0 && (q.step == PM_STEP_LCC0 || (q.step == PM_STEP_LCC && q.lcc_first_pending)))
          break;
      }
    } catch (const PmError& e) {
      it.status = e.code;
      it.error = e.message;
    } catch (const std::bad_alloc&) {
      it.status = PM_E_OOM;
      it.error = "host allocation failed";
    } catch (const std::exception& e) {
      it.status = PM_FAILURE;
      it.error = e.what();
    }
    set_thread_walk_budget_cap_ns(0);
    {
      std::lock_guard<std::mutex> lk(mu_);
      running_[i] = 0;
      ++finished_steps_;
    }
    cv_done_.notify_all();
  }
}

void FusedBatch::run() {
  using Clock = std::chrono::steady_clock;
  const auto t0 = Clock::now();
  // At most one query per worker is in flight; the others wait their turn,
  // and a query's budget (query_budget_ms) starts when it enters.
  const size_t window = std::max<size_t>(n_workers_, 1);
  size_t entered = 0;
  auto enter = [&]() {
    while (entered < items_.size()) {
      size_t in_flight = 0;
      for (size_t i = 0; i < entered; ++i) in_flight += items_[i].done ? 0 : 1;
      if (in_flight >= window) break;
      FusedBatchItem& it = items_[entered++];
      if (query_budget_ms() > 0) {
        it.q->has_deadline = true;
        it.q->deadline = Clock::now() + std::chrono::microseconds(static_cast<int64_t>(query_budget_ms() * 1000.0));
      }
    }
  };
  auto mark_done = [&](FusedBatchItem& it) {
    it.done = true;
    it.run_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
  };
  // A shared LCC phase on this thread; a failure ends every query it covered.
  auto shared_phase = [&](const std::vector<size_t>& idx, bool lcc0) {
    std::vector<size_t> ok;
    for (size_t i : idx) {
      try {
        items_[i].q->check_request();
        ok.push_back(i);
      } catch (const PmError& e) {
        items_[i].status = e.code;
        items_[i].error = e.message;
        mark_done(items_[i]);
      }
    }
    set_thread_walk_budget_cap_ns(0);
    if (ok.empty()) return;
    std::vector<QueryImpl*> qs;
    for (size_t i : ok) qs.push_back(items_[i].q.get());
    try {
      if (lcc0)
        QueryImpl::lcc0_batch(qs, stream_);
      else
        QueryImpl::lcc_fixpoint_batch(qs, stream_);
      ++fused_lcc_passes;
    } catch (const PmError& e) {
      for (size_t i : ok) {
        items_[i].status = e.code;
        items_[i].error = e.message;
        mark_done(items_[i]);
      }
    }
  };
  std::unique_lock<std::mutex> lk(mu_);
  while (true) {
    enter();
    // Queries between steps (not on a worker) and what they need next.
    std::vector<size_t> at_lcc0, at_lcc, others;
    size_t busy = 0;
    for (size_t i = 0; i < entered; ++i) {
      FusedBatchItem& it = items_[i];
      if (it.done) continue;
      if (running_[i]) {
        ++busy;
        continue;
      }
      QueryImpl& q = *it.q;
      if (it.status != PM_SUCCESS || q.finished || q.iteration >= 1000 ||
          (prune_only_ && q.step == PM_STEP_ENUMERATION)) {
        mark_done(it);
        continue;
      }
      // Shared launches for LCC0 and the fixpoint right after it (every
      // vertex scheduled: the passes that read most of the adjacency, which
      // the queries of one launch share through L2).  Later fixpoints are
      // short (only vertices next to a change are rescheduled) and run on a
      // worker as one captured launch, so that no query waits for a group.
      if (q.active_vertices != 0 && q.step == PM_STEP_LCC0)
        at_lcc0.push_back(i);
      else if (q.active_vertices != 0 && q.step == PM_STEP_LCC && q.lcc_first_pending)
        at_lcc.push_back(i);
      else
        others.push_back(i);
    }
    if (!busy && at_lcc0.empty() && at_lcc.empty() && others.empty()) {
      if (entered < items_.size()) continue;  // the next queries enter
      break;
    }
    ++rounds;
    for (size_t i : others) {
      running_[i] = 1;
      queue_.push_back(i);
    }
    if (!others.empty()) cv_work_.notify_all();
    if (!at_lcc0.empty() || !at_lcc.empty()) {
      // The shared phases run while workers keep stepping other queries.
      lk.unlock();
      shared_phase(at_lcc0, true);
      shared_phase(at_lcc, false);
      lk.lock();
      continue;
    }
    // Nothing for this thread: wait for a worker to finish a step.
    finished_steps_ = 0;
    cv_done_.wait(lk, [&] { return finished_steps_ != 0; });
  }
}

}  // namespace pmgb
