// Minimal stand-in for the one TBB header the reference's TOTEM core includes
// (src/totem/totem_comdef.h:28).  The pattern-matching path never sorts in
// parallel; TOTEM's partitioner only needs the symbol to exist.  Test
// infrastructure only: used when building the reference CPU path into
// oracle/_ref for validation.
#ifndef PM_REF_SHIM_TBB_PARALLEL_SORT_H
#define PM_REF_SHIM_TBB_PARALLEL_SORT_H
#include <algorithm>
namespace tbb {
template <typename It, typename Cmp>
inline void parallel_sort(It first, It last, const Cmp& cmp) { std::sort(first, last, cmp); }
template <typename It>
inline void parallel_sort(It first, It last) { std::sort(first, last); }
}  // namespace tbb
#endif
