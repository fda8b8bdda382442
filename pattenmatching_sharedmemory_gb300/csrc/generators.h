// Seeded synthetic graph and label generators (see generators.cc).
#pragma once
#include "pm_types.h"

namespace pmgb {

enum LabelKind : int { kLabelUniform = 0, kLabelZipf = 1, kLabelDegree = 2 };

// Undirected RMAT graph with 2^scale vertices and edge_factor * 2^scale
// sampled pairs; vertex ids optionally shuffled by a seeded permutation.
HostGraph generate_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, bool permute);

// Assigns labels 0..n_labels-1 to every vertex.
void assign_labels(HostGraph& g, int kind, uint32_t n_labels, double s, uint64_t seed);

// Graph ingestion tools: the TOTEM generator's UNDIRECTED, SORT_NEIGHBOURS
// and SORT_VERTICES commands (see generators.cc).
HostGraph make_undirected(const HostGraph& in);
void sort_neighbours(HostGraph& g);
HostGraph sort_vertices_by_degree(const HostGraph& in, std::vector<uint32_t>* old_to_new);

}  // namespace pmgb
