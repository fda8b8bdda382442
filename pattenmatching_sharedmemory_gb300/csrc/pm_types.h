// Shared host-side types of the GB300 PruneJuice pipeline.
//
// Vertex ids are 32-bit and CSR offsets 64-bit (the reference's vid_t /
// eid_t with FEATURE_64BIT_EDGE_ID, src/totem/totem_graph.h:64-72); vertex
// labels are the reference's 64-bit weight_t values
// (src/totem/totem_graph.h:89-95).
#pragma once
#include <sys/mman.h>

#include <cstdint>
#include <cstdlib>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/pm_gb300.h"

namespace pmgb {

using vid_t = uint32_t;
using eid_t = uint64_t;
using label_t = uint64_t;

// Maximum template size (reference: C_MAXIMUM_PATTERN_SIZE = 64,
// src/patternmatching/multiple_label/multiple_label_common.h:14).
constexpr uint32_t kMaxPatternSize = 64;

// Allocator of the host CSR's adjacency: elements are default-initialised
// (a resize leaves them unwritten, so the copy that fills them is the first
// touch and can run on many threads), and blocks of 2 MiB or more are
// 2 MiB-aligned and offered to transparent huge pages, so a multi-GB list
// takes few page faults.
template <class T>
struct HostArrayAlloc {
  using value_type = T;
  static constexpr size_t kHuge = size_t(2) << 20;
  HostArrayAlloc() = default;
  template <class U>
  HostArrayAlloc(const HostArrayAlloc<U>&) {}
  T* allocate(size_t n) {
    const size_t bytes = n * sizeof(T);
    if (bytes < kHuge) return static_cast<T*>(::operator new(bytes));
    void* p = nullptr;
    if (posix_memalign(&p, kHuge, bytes) != 0) throw std::bad_alloc();
#ifdef MADV_HUGEPAGE
    madvise(p, bytes, MADV_HUGEPAGE);
#endif
    return static_cast<T*>(p);
  }
  void deallocate(T* p, size_t n) noexcept {
    if (n * sizeof(T) < kHuge)
      ::operator delete(p);
    else
      std::free(p);
  }
  template <class U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
  template <class U>
  bool operator==(const HostArrayAlloc<U>&) const { return true; }
  template <class U>
  bool operator!=(const HostArrayAlloc<U>&) const { return false; }
};

// A host CSR graph in the TOTEM layout (src/totem/totem_graph.h:137-180):
// offsets has V+1 entries, adj has E entries, labels has V entries
// (the reference's graph->values; 0 when no label file was given).
struct HostGraph {
  uint32_t vertex_count = 0;
  uint64_t edge_count = 0;
  bool directed = false;
  bool valued = false;
  std::vector<uint64_t, HostArrayAlloc<uint64_t>> offsets;
  std::vector<uint32_t, HostArrayAlloc<uint32_t>> adj;
  std::vector<uint64_t, HostArrayAlloc<uint64_t>> labels;
};

// Error with a TOTEM-style status code (SUCCESS=0 / FAILURE=-1 plus the
// distinct negative codes declared in pm_gb300.h).
struct PmError {
  int code;
  std::string message;
};

}  // namespace pmgb
