// Query server: FIFO admission by device memory onto worker slots.
#include "server.h"

#include <algorithm>

namespace pmgb {

Server::Server(GraphImpl* graph, uint32_t slots, uint64_t budget, uint32_t walk_share)
    : g_(graph), slots_(slots), budget_(budget), walk_share_(walk_share) {
  if (!g_ || g_->device < 0) throw PmError{PM_E_INVALID_ARG, "the graph is not on a device"};
  if (slots_ == 0) throw PmError{PM_E_INVALID_ARG, "a server needs at least one slot"};
  PM_CUDA(cudaSetDevice(g_->device));
  if (budget_ == 0) {
    size_t free_b = 0, total_b = 0;
    PM_CUDA(cudaMemGetInfo(&free_b, &total_b));
    budget_ = free_b / 10 * 9;
  }
  workers_.reserve(slots_);
  for (uint32_t i = 0; i < slots_; ++i) workers_.emplace_back(&Server::worker, this, i);
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    for (auto& r : queue_) {
      r->status = PM_E_CANCELLED;
      r->error = "server shut down before the request was admitted";
      r->state = ServeRequest::kDone;
      r->t_done = ServeRequest::Clock::now();
    }
    queue_.clear();
    stop_ = true;
  }
  cv_work_.notify_all();
  for (auto& t : workers_) t.join();
  cv_done_.notify_all();
}

uint64_t Server::submit(const PatternGraph& pattern, uint32_t flags) {
  auto r = std::make_shared<ServeRequest>();
  r->pattern = pattern;
  r->flags = flags;
  r->bytes = estimate_query_bytes(*g_, pattern.n);
  r->t_submit = ServeRequest::Clock::now();
  std::lock_guard<std::mutex> lk(mu_);
  if (stop_) throw PmError{PM_E_CANCELLED, "server is shutting down"};
  if (r->bytes > budget_)
    throw PmError{PM_E_ADMISSION_DENIED, "request needs " + std::to_string(r->bytes) +
                                             " device bytes, above the server's budget of " +
                                             std::to_string(budget_)};
  r->ticket = next_ticket_++;
  requests_[r->ticket] = r;
  queue_.push_back(r);
  cv_work_.notify_one();
  return r->ticket;
}

std::shared_ptr<ServeRequest> Server::find(uint64_t ticket, bool* done) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = requests_.find(ticket);
  if (it == requests_.end()) return nullptr;
  if (done) *done = it->second->state == ServeRequest::kDone;
  return it->second;
}

bool Server::wait(uint64_t ticket, double timeout_ms) {
  std::unique_lock<std::mutex> lk(mu_);
  auto it = requests_.find(ticket);
  if (it == requests_.end()) throw PmError{PM_E_INVALID_ARG, "unknown ticket"};
  std::shared_ptr<ServeRequest> r = it->second;
  auto done = [&] { return r->state == ServeRequest::kDone; };
  if (timeout_ms < 0) {
    cv_done_.wait(lk, done);
    return true;
  }
  return cv_done_.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), done);
}

void Server::release(uint64_t ticket) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = requests_.find(ticket);
  if (it == requests_.end()) throw PmError{PM_E_INVALID_ARG, "unknown ticket"};
  if (it->second->state != ServeRequest::kDone) throw PmError{PM_E_BUSY, "request still queued or running"};
  requests_.erase(it);
}

int Server::cancel(uint64_t ticket) {
  std::shared_ptr<ServeRequest> r;
  int was = ServeRequest::kDone;
  {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = requests_.find(ticket);
    if (it == requests_.end()) throw PmError{PM_E_INVALID_ARG, "unknown ticket"};
    r = it->second;
    was = r->state;
    if (r->state == ServeRequest::kQueued) {
      queue_.erase(std::find(queue_.begin(), queue_.end(), r));
      r->status = PM_E_CANCELLED;
      r->error = "request cancelled before it was admitted";
      r->state = ServeRequest::kDone;
      r->t_admit = r->t_done = ServeRequest::Clock::now();
      ++done_;
    } else if (r->state == ServeRequest::kRunning) {
      r->cancel.store(true);
    }
  }
  if (was == ServeRequest::kQueued) {
    cv_done_.notify_all();
    cv_work_.notify_all();
  }
  return was;
}

ServerStats Server::stats() {
  std::lock_guard<std::mutex> lk(mu_);
  ServerStats s;
  s.queued = queue_.size();
  s.running = running_;
  s.done = done_;
  s.bytes_in_use = used_;
  s.peak_bytes = peak_;
  s.budget = budget_;
  s.slots = slots_;
  return s;
}

// Head of the queue fits beside the running requests (FIFO: a large request
// at the head holds back smaller ones behind it).
bool Server::admissible() const {
  if (queue_.empty()) return false;
  return used_ + queue_.front()->bytes <= budget_;
}

void Server::worker(uint32_t) {
  cudaStream_t stream = nullptr;
  StepCounters* h_ctr = nullptr;
  uint32_t* h_count = nullptr;
  std::string err;
  // Each slot's walker launches take its share of the GPU, so that requests
  // running side by side overlap instead of queueing behind the first
  // persistent walker grid (speed only).
  set_thread_walk_grid_share(walk_share_ ? walk_share_ : slots_);
  if (cudaSetDevice(g_->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMallocHost(&h_ctr, sizeof(StepCounters)) != cudaSuccess ||
      cudaMallocHost(&h_count, sizeof(uint32_t)) != cudaSuccess)
    err = "slot set-up failed: " + std::string(cudaGetErrorString(cudaGetLastError()));
  while (true) {
    std::shared_ptr<ServeRequest> r;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_work_.wait(lk, [&] { return stop_ || admissible(); });
      if (stop_) break;
      r = queue_.front();
      queue_.pop_front();
      used_ += r->bytes;
      peak_ = std::max(peak_, used_);
      ++running_;
      r->state = ServeRequest::kRunning;
      r->t_admit = ServeRequest::Clock::now();
    }
    // Another slot may admit the next request while this one runs.
    cv_work_.notify_one();
    if (!err.empty()) {
      r->status = PM_E_DEVICE;
      r->error = err;
    } else {
      try {
        QueryImpl q;
        // The request's budget (pm_set_query_budget_ms) runs from admission,
        // so template compilation and allocation count against it too.
        if (query_budget_ms() > 0) {
          q.has_deadline = true;
          q.deadline = r->t_admit + std::chrono::microseconds(static_cast<int64_t>(query_budget_ms() * 1000.0));
        }
        q.create(g_, r->pattern, stream, h_ctr, h_count);
        q.cancel = &r->cancel;
        q.stop_before_enumeration = (r->flags & kSubmitPruneOnly) != 0;
        q.run_all();
        r->records = q.records;
        r->records.push_back(q.final_record());
        r->match_count = q.match_count;
        r->gpu_ms = q.total_ms;
        if (r->flags & kSubmitExportState) {
          r->cand.resize(g_->host.vertex_count);
          r->eact.resize(g_->host.edge_count);
          r->vact.resize(g_->host.vertex_count);
          q.export_state(r->cand.data(), r->eact.data(), r->vact.data());
        }
      } catch (const PmError& e) {
        r->status = e.code;
        r->error = e.message;
      } catch (const std::bad_alloc&) {
        r->status = PM_E_OOM;
        r->error = "host allocation failed";
      } catch (const std::exception& e) {
        r->status = PM_FAILURE;
        r->error = e.what();
      }
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      used_ -= r->bytes;
      --running_;
      ++done_;
      r->state = ServeRequest::kDone;
      r->t_done = ServeRequest::Clock::now();
    }
    cv_done_.notify_all();
    cv_work_.notify_all();
  }
  if (stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
  if (h_ctr) cudaFreeHost(h_ctr);
  if (h_count) cudaFreeHost(h_count);
}

}  // namespace pmgb
