// Force-included into the reference's src/patternmatching/multiple_label_cpu.cc
// when it is compiled into oracle/_ref.  The reference hard-codes
// omp_set_num_threads(60) (multiple_label_cpu.cc:15); this lets the test
// harness pick the thread count through PM_REF_THREADS (1 = the canonical
// single-thread order used for golden vectors).  Test infrastructure only.
#ifndef PM_REF_SHIM_OMP_THREADS_OVERRIDE_H
#define PM_REF_SHIM_OMP_THREADS_OVERRIDE_H
#include <omp.h>
#include <stdlib.h>
static inline void pm_ref_set_num_threads(int requested) {
  const char* env = getenv("PM_REF_THREADS");
  int n = (env && atoi(env) > 0) ? atoi(env) : requested;
  omp_set_num_threads(n);
}
#define omp_set_num_threads(n) pm_ref_set_num_threads(n)
#endif
