// TOTEM graph file formats, bit-compatible with the reference's reader and
// writer (src/totem/totem_graph.cu:20-409, 883-922) and its vertex-label
// parser (src/patternmatching/utils/common_utils.cc:9-56).
#pragma once
#include <string>

#include "pm_types.h"

namespace pmgb {

// graph_initialize (totem_graph.cu:388-409): binary when the file starts
// with the magic word 0x10102048, else the text format.  Throws PmError.
HostGraph read_totem_graph(const std::string& path);

// parseVertexFile (common_utils.cc:9-56): "vid value" lines in increasing
// vid order, '#' comments skipped, missing vids get 0, values parsed with
// atoll.  Sets graph.valued and graph.labels.  Throws PmError.
void read_vertex_labels(const std::string& path, HostGraph& graph);

// graph_store_binary (totem_graph.cu:883-922).  eid_bytes = 4 writes the
// default EID=32 layout, 8 the FEATURE_64BIT_EDGE_ID layout.
void write_totem_binary(const HostGraph& graph, const std::string& path, int eid_bytes);

// Text writer in the format the reader accepts (used by the input
// generators and tests).
void write_totem_text(const HostGraph& graph, const std::string& path);
void write_vertex_labels(const HostGraph& graph, const std::string& path);

bool is_regular_file(const std::string& path);

}  // namespace pmgb
