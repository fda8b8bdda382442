// Stand-in for src/totem/totem_grooves_internal.cc, which needs
// tbb/concurrent_unordered_set.h (not installed).  The pattern-matching path
// never builds TOTEM partitions, so the function is never called; it only has
// to link.  Compiled against the reference's own totem_partition.h so the
// signature matches.  Test infrastructure only.
#include <cstdio>
#include <cstdlib>
#include "totem_partition.h"
void init_get_rmt_nbrs(partition_set_t*, int, vid_t**, vid_t*) {
  fprintf(stderr, "init_get_rmt_nbrs: not available in the oracle build\n");
  abort();
}
