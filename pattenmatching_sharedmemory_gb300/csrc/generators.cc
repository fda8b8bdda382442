// Seeded synthetic inputs standing in for the reference's external datasets:
// undirected RMAT graphs (recursive quadrant choice with probabilities
// a/b/c/d, symmetrised, self-loops and duplicate edges removed, adjacency
// sorted) and vertex label assignments (uniform, Zipf(s), degree-correlated).
//
// Determinism across machines: every random draw comes from splitmix64 on a
// per-item counter, quadrant choice compares 64-bit integers, and the only
// floating point (Zipf weights) uses +,-,*,/ in a fixed order (this file is
// compiled with -ffp-contract=off), so x86 and aarch64 produce identical
// graphs for the same seed.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "generators.h"

namespace pmgb {
namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Uniform integer in [0, n) from a 64-bit draw (multiply-shift).
inline uint64_t bounded(uint64_t r, uint64_t n) {
  return static_cast<uint64_t>((static_cast<unsigned __int128>(r) * n) >> 64);
}

inline uint64_t prob_threshold(double p) {
  if (p <= 0) return 0;
  if (p >= 1) return ~uint64_t(0);
  return static_cast<uint64_t>(p * 18446744073709551616.0);
}

// x^(1/10) by Newton's method on y^10 = x (x >= 1); only +,*,/ are used.
double root10(double x) {
  double y = 1.0 + (x - 1.0) / 10.0;
  if (y > x) y = x;
  for (int it = 0; it < 200; ++it) {
    double y2 = y * y, y4 = y2 * y2, y8 = y4 * y4, y9 = y8 * y;
    double next = y - (y9 * y - x) / (10.0 * y9);
    if (next == y) break;
    y = next;
  }
  return y;
}

// x^s for s a multiple of 0.1 (s rounded to one decimal).
double pow_tenths(double x, double s) {
  long tenths = std::lround(s * 10.0);
  double r = root10(x);
  double out = 1.0;
  for (long i = 0; i < tenths; ++i) out *= r;
  return out;
}

}  // namespace

HostGraph generate_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, bool permute) {
  if (scale < 1 || scale > 31) throw PmError{PM_E_INVALID_ARG, "rmat scale must be in [1, 31]"};
  if (edge_factor < 1) throw PmError{PM_E_INVALID_ARG, "edge factor must be positive"};
  const uint64_t V = uint64_t(1) << scale;
  const uint64_t M = V * static_cast<uint64_t>(edge_factor);
  const uint64_t ta = prob_threshold(a), tab = prob_threshold(a + b), tabc = prob_threshold(a + b + c);

  std::vector<uint32_t> perm(V);
  std::iota(perm.begin(), perm.end(), 0u);
  if (permute) {
    uint64_t st = splitmix64(seed ^ 0x5EED5EED5EEDull);
    for (uint64_t i = V - 1; i > 0; --i) {
      st = splitmix64(st);
      uint64_t j = bounded(st, i + 1);
      std::swap(perm[i], perm[j]);
    }
  }
  // Sample M directed pairs; each contributes both directions unless it is a
  // self-loop.
  std::vector<uint32_t> src(M), dst(M);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < static_cast<int64_t>(M); ++i) {
    uint64_t st = splitmix64(seed * 0x100000001B3ull + static_cast<uint64_t>(i));
    uint64_t u = 0, v = 0;
    for (int l = 0; l < scale; ++l) {
      st = splitmix64(st);
      uint64_t bit = uint64_t(1) << (scale - 1 - l);
      if (st < ta) {
      } else if (st < tab) {
        v |= bit;
      } else if (st < tabc) {
        u |= bit;
      } else {
        u |= bit;
        v |= bit;
      }
    }
    src[i] = perm[u];
    dst[i] = perm[v];
  }
  // Bucket by source (both directions), then sort + dedup each adjacency.
  std::vector<uint64_t> deg(V + 1, 0);
  for (uint64_t i = 0; i < M; ++i) {
    if (src[i] == dst[i]) continue;
    ++deg[src[i]];
    ++deg[dst[i]];
  }
  std::vector<uint64_t> start(V + 1, 0);
  for (uint64_t v = 0; v < V; ++v) start[v + 1] = start[v] + deg[v];
  std::vector<uint32_t> buf(start[V]);
  std::vector<uint64_t> fill(start.begin(), start.end() - 1);
  for (uint64_t i = 0; i < M; ++i) {
    if (src[i] == dst[i]) continue;
    buf[fill[src[i]]++] = dst[i];
    buf[fill[dst[i]]++] = src[i];
  }
  std::vector<uint64_t>().swap(fill);
  std::vector<uint32_t>().swap(src);
  std::vector<uint32_t>().swap(dst);
  std::vector<uint64_t> uniq(V, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < static_cast<int64_t>(V); ++v) {
    uint32_t* b0 = buf.data() + start[v];
    uint32_t* b1 = buf.data() + start[v + 1];
    std::sort(b0, b1);
    uniq[v] = static_cast<uint64_t>(std::unique(b0, b1) - b0);
  }
  HostGraph g;
  g.vertex_count = static_cast<uint32_t>(V);
  g.directed = false;
  g.offsets.assign(V + 1, 0);
  for (uint64_t v = 0; v < V; ++v) g.offsets[v + 1] = g.offsets[v] + uniq[v];
  g.edge_count = g.offsets[V];
  g.adj.resize(g.edge_count);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < static_cast<int64_t>(V); ++v)
    memcpy(g.adj.data() + g.offsets[v], buf.data() + start[v], sizeof(uint32_t) * uniq[v]);
  return g;
}

void assign_labels(HostGraph& g, int kind, uint32_t n_labels, double s, uint64_t seed) {
  if (n_labels == 0) throw PmError{PM_E_INVALID_ARG, "need at least one label"};
  const uint32_t V = g.vertex_count;
  g.labels.assign(V, 0);
  g.valued = true;
  if (kind == kLabelUniform) {
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < V; ++v) g.labels[v] = bounded(splitmix64(seed ^ (0xA5A5ull << 40) ^ v), n_labels);
    return;
  }
  // Zipf(s) weights 1/(i+1)^s, cumulative thresholds over 2^64.
  std::vector<double> w(n_labels);
  double total = 0;
  for (uint32_t i = 0; i < n_labels; ++i) {
    w[i] = 1.0 / pow_tenths(static_cast<double>(i + 1), s);
    total += w[i];
  }
  std::vector<uint64_t> cdf(n_labels);
  double acc = 0;
  for (uint32_t i = 0; i < n_labels; ++i) {
    acc += w[i];
    cdf[i] = i + 1 == n_labels ? ~uint64_t(0) : prob_threshold(acc / total);
  }
  auto draw = [&](uint64_t r) -> uint64_t {
    size_t i = static_cast<size_t>(std::upper_bound(cdf.begin(), cdf.end(), r) - cdf.begin());
    return i >= n_labels ? n_labels - 1 : i;
  };
  if (kind == kLabelZipf) {
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < V; ++v) g.labels[v] = draw(splitmix64(seed ^ (0x5A5Aull << 40) ^ v));
    return;
  }
  // Degree-correlated: vertices sorted by degree (descending, ties by id);
  // a vertex of degree rank r draws its label from the Zipf distribution
  // with probability 1/2, else takes label floor(n * r / V), so frequent
  // (low) labels concentrate on high-degree vertices.
  std::vector<uint32_t> order(V);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
    uint64_t dx = g.offsets[x + 1] - g.offsets[x], dy = g.offsets[y + 1] - g.offsets[y];
    return dx > dy;
  });
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < V; ++r) {
    uint32_t v = order[r];
    uint64_t rnd = splitmix64(seed ^ (0x3C3Cull << 40) ^ v);
    if (rnd >> 63)
      g.labels[v] = draw(splitmix64(rnd));
    else
      g.labels[v] = static_cast<uint64_t>(r) * n_labels / V;
  }
}

// ---- graph ingestion tools (the TOTEM generator's ALTER commands,
// src/generator/totem_generator.cc) ------------------------------------------

namespace {
// CSR from an edge list the way the generator's edgelist_to_graph does it
// (totem_generator.cc:92-125): per-vertex degree counts, then each entry is
// placed at the last free position of its source's list, so a list holds
// its entries in reverse order of appearance.
HostGraph csr_from_edgelist(const std::vector<uint32_t>& src, const std::vector<uint32_t>& dst, uint32_t V,
                            bool directed) {
  HostGraph g;
  g.vertex_count = V;
  g.directed = directed;
  g.offsets.assign(static_cast<size_t>(V) + 1, 0);
  std::vector<uint64_t> fill(V, 0);
  for (uint32_t u : src) ++fill[u];
  for (uint32_t v = 0; v < V; ++v) g.offsets[v + 1] = g.offsets[v] + fill[v];
  g.edge_count = g.offsets[V];
  g.adj.resize(g.edge_count);
  for (size_t i = 0; i < src.size(); ++i) g.adj[g.offsets[src[i]] + --fill[src[i]]] = dst[i];
  return g;
}
}  // namespace

// UNDIRECTED (alter_undirected_handler, totem_generator.cc:631-680): every
// CSR entry u -> v contributes u -> v and v -> u, in CSR order; duplicates
// are kept.  Labels are carried over.
HostGraph make_undirected(const HostGraph& in) {
  std::vector<uint32_t> src, dst;
  src.reserve(2 * in.edge_count);
  dst.reserve(2 * in.edge_count);
  for (uint32_t v = 0; v < in.vertex_count; ++v)
    for (uint64_t e = in.offsets[v]; e < in.offsets[v + 1]; ++e) {
      src.push_back(v);
      dst.push_back(in.adj[e]);
      src.push_back(in.adj[e]);
      dst.push_back(v);
    }
  HostGraph g = csr_from_edgelist(src, dst, in.vertex_count, false);
  g.labels = in.labels;
  g.valued = in.valued;
  return g;
}

// SORT_NEIGHBOURS (alter_sort_neighbours_handler, totem_generator.cc:764-770,
// graph_sort_nbrs ascending): every adjacency list sorted by id, in place.
void sort_neighbours(HostGraph& g) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < static_cast<int64_t>(g.vertex_count); ++v)
    std::sort(g.adj.begin() + static_cast<int64_t>(g.offsets[v]), g.adj.begin() + static_cast<int64_t>(g.offsets[v + 1]));
}

// SORT_VERTICES (alter_sort_vertices_handler, totem_generator.cc:682-748):
// vertex ids renumbered in ascending order of degree, then the edge list
// (old CSR order, both ends renamed) rebuilt as edgelist_to_graph does.  The
// reference sorts with a parallel sort, which leaves the order of equal
// degrees unspecified; here ties keep ascending old ids (a stable sort).
// Labels move with their vertices; old_to_new receives the renumbering.
HostGraph sort_vertices_by_degree(const HostGraph& in, std::vector<uint32_t>* old_to_new) {
  const uint32_t V = in.vertex_count;
  std::vector<uint32_t> order(V);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
    return in.offsets[a + 1] - in.offsets[a] < in.offsets[b + 1] - in.offsets[b];
  });
  std::vector<uint32_t> map(V);
  for (uint32_t i = 0; i < V; ++i) map[order[i]] = i;
  std::vector<uint32_t> src, dst;
  src.reserve(in.edge_count);
  dst.reserve(in.edge_count);
  for (uint32_t v = 0; v < V; ++v)
    for (uint64_t e = in.offsets[v]; e < in.offsets[v + 1]; ++e) {
      src.push_back(map[v]);
      dst.push_back(map[in.adj[e]]);
    }
  HostGraph g = csr_from_edgelist(src, dst, V, in.directed);
  if (!in.labels.empty()) {
    g.labels.assign(V, 0);
    for (uint32_t v = 0; v < V; ++v) g.labels[map[v]] = in.labels[v];
  }
  g.valued = in.valued;
  if (old_to_new) *old_to_new = std::move(map);
  return g;
}

}  // namespace pmgb
