// patternmatching_gb300 — drop-in for the reference's `patternmatching` CLI
// (src/patternmatching/patternmatching_binary.cc:13-42,
// utils/cmd_line_option.cc:22-78):
//   -i <graph>  -b <binary cache>  -v <vertex labels>  -e <unused>
//   -p <pattern directory/>  -o <output directory>  -h
// Without -b the binary cache is <graph>.bin.  Outputs the reference's
// results.totem, graph_NNNN.totem, vertex_NNNN.totem and log.totem.
// Additional option: -d <device> (default 0).
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <string>

#include "../../include/pm_gb300.h"

static void usage() {
  fprintf(stderr,
          "Usage: -i <string> -p <string> -o <string>\n"
          " -i <string>   - input graph base filename (required)\n"
          " -b <string>   - input binary graph base filename (optional)\n"
          " -v <string>   - vertex metadata base filename (optional, Default is degree based metadata)\n"
          " -e <string>   - edge metadata base filename (optional)\n"
          " -p <string>   - pattern base directory (required)\n"
          " -o <string>   - output base directory (required)\n"
          " -d <int>      - CUDA device (optional, default 0)\n"
          " -h            - print help and exit\n\n");
}

static int check(pm_status_t s, const char* what) {
  if (s != PM_SUCCESS) {
    fprintf(stderr, "%s failed (%d): %s\n", what, s, pm_last_error());
    return 1;
  }
  return 0;
}

int main(int argc, char** argv) {
  std::string graph, bin, labels, pattern, out;
  int device = 0;
  bool help = false;
  int c;
  while ((c = getopt(argc, argv, "i:b:v:e:p:o:x:d:h")) != -1) {
    switch (c) {
      case 'i': graph = optarg; break;
      case 'b': bin = optarg; break;
      case 'v': labels = optarg; break;
      case 'e': break;
      case 'p': pattern = optarg; break;
      case 'o': out = optarg; break;
      case 'd': device = atoi(optarg); break;
      case 'x': break;
      default: help = true; break;
    }
  }
  if (help || graph.empty() || pattern.empty() || out.empty()) {
    usage();
    return 255;
  }
  if (bin.empty()) bin = graph + ".bin";
  pm_graph* g = nullptr;
  if (check(pm_graph_load(graph.c_str(), bin.c_str(), labels.c_str(), device, &g), "pm_graph_load")) return 1;
  pm_query* q = nullptr;
  if (check(pm_query_create(g, pattern.c_str(), labels.empty() ? 0 : 1, &q), "pm_query_create")) return 1;
  int finished = 0;
  while (!finished) {
    pm_step_record r;
    if (check(pm_query_step(q, &r, &finished), "pm_query_step")) return 1;
    printf("Start %s\n", r.step == PM_STEP_LCC0 ? "LCC0" : r.step == PM_STEP_LCC ? "LCC" : r.step == PM_STEP_CC ? "CC"
                                : r.step == PM_STEP_PC ? "PC" : r.step == PM_STEP_TDS ? "TDS" : "ENUMERATION");
  }
  if (check(pm_query_write_outputs(q, out.c_str()), "pm_query_write_outputs")) return 1;
  pm_query_destroy(q);
  pm_graph_destroy(g);
  return 0;
}
