// TOTEM graph reader / writer.  Behaviour follows the reference
// (src/totem/totem_graph.cu, src/patternmatching/utils/common_utils.cc):
//   * text header: three '#' lines holding NODES <n> [Y], EDGES <m> and
//     DIRECTED | UNDIRECTED, keywords case-insensitive, tokens split on
//     " \t\n:" (totem_graph.cu:30-118); counts parsed with atoi (:88, :97);
//   * optional vertex list when the NODES line carries 'y' (values via atof,
//     :129-172);
//   * edge list "src dst [w]" sorted by src, '#' lines skipped, every CSR
//     slot of a vertex without edges points at the next edge (:180-251);
//   * binary: magic, vid/eid sizes, counts, three bool flags, vertices,
//     values, edges, weights (:253-312, :883-922).
// The reader is a whole-file tokenizer rather than fgets into a 100-byte
// buffer; for well-formed files (every line shorter than 100 bytes, as the
// reference requires) the result is identical.
#include "totem_io.h"

#include <sys/stat.h>

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>

namespace pmgb {
namespace {

constexpr uint32_t kBinaryMagic = 0x10102048u;

[[noreturn]] void fail(int code, const std::string& msg) { throw PmError{code, msg}; }

struct FileCloser {
  void operator()(FILE* f) const {
    if (f) fclose(f);
  }
};
using FilePtr = std::unique_ptr<FILE, FileCloser>;

std::string slurp(FILE* f, const std::string& path) {
  std::string data;
  if (fseek(f, 0, SEEK_END) != 0) fail(PM_E_IO, "cannot seek " + path);
  long size = ftell(f);
  if (size < 0) fail(PM_E_IO, "cannot size " + path);
  rewind(f);
  data.resize(static_cast<size_t>(size));
  if (size > 0 && fread(&data[0], 1, data.size(), f) != data.size())
    fail(PM_E_IO, "short read on " + path);
  return data;
}

// Line cursor over an in-memory file.
struct Lines {
  const char* p;
  const char* end;
  uint64_t line_number = 0;
  bool next(const char*& b, const char*& e) {
    if (p >= end) return false;
    b = p;
    const char* nl = static_cast<const char*>(memchr(p, '\n', end - p));
    e = nl ? nl : end;
    p = nl ? nl + 1 : end;
    ++line_number;
    return true;
  }
};

inline bool is_delim(char c) { return c == ' ' || c == '\t' || c == '\n' || c == ':' || c == '\r'; }

// strtok_r over [b, e) with the reference's delimiter set " \t\n:".
struct Tokens {
  const char* p;
  const char* e;
  bool next(std::string& tok) {
    while (p < e && is_delim(*p)) ++p;
    if (p >= e) return false;
    const char* s = p;
    while (p < e && !is_delim(*p)) ++p;
    tok.assign(s, p - s);
    return true;
  }
};

// is_numeric (totem_comdef.h:115-124): every character a decimal digit.
bool is_numeric(const std::string& s) {
  for (char c : s)
    if (!isdigit(static_cast<unsigned char>(c))) return false;
  return true;
}

HostGraph parse_text(const std::string& data, const std::string& path) {
  HostGraph g;
  Lines lines{data.data(), data.data() + data.size()};
  const char* b;
  const char* e;
  bool found_nodes = false, found_edges = false;
  bool directed = true, valued = false;
  int64_t vcount = 0, ecount = 0;
  std::string tok;
  for (int i = 0; i < 3; ++i) {
    if (!lines.next(b, e) || b == e || *b != '#')
      fail(PM_E_FORMAT, path + ": error in metadata format (first three lines)");
    Tokens t{b + 1, e};
    if (!t.next(tok)) fail(PM_E_FORMAT, path + ": empty metadata line");
    for (auto& c : tok) c = static_cast<char>(toupper(static_cast<unsigned char>(c)));
    if (tok == "NODES") {
      if (!t.next(tok) || !is_numeric(tok)) fail(PM_E_FORMAT, path + ": bad NODES line");
      vcount = atoi(tok.c_str());
      if (t.next(tok) && tolower(static_cast<unsigned char>(tok[0])) == 'y') valued = true;
      found_nodes = true;
    } else if (tok == "EDGES") {
      if (!t.next(tok) || !is_numeric(tok)) fail(PM_E_FORMAT, path + ": bad EDGES line");
      ecount = atoi(tok.c_str());
      found_edges = true;
    } else if (tok == "DIRECTED") {
      directed = true;
    } else if (tok == "UNDIRECTED") {
      directed = false;
    } else {
      fail(PM_E_FORMAT, path + ": unknown metadata keyword " + tok);
    }
  }
  if (!found_nodes || !found_edges) fail(PM_E_FORMAT, path + ": missing NODES or EDGES");
  if (vcount < 0 || ecount < 0) fail(PM_E_FORMAT, path + ": negative counts");
  g.vertex_count = static_cast<uint32_t>(vcount);
  g.edge_count = static_cast<uint64_t>(ecount);
  g.directed = directed;
  g.valued = valued;
  g.offsets.assign(static_cast<size_t>(g.vertex_count) + 1, 0);
  g.adj.resize(g.edge_count);
  if (valued) {
    g.labels.assign(g.vertex_count, 0);
    uint32_t vi = 0;
    while (vi < g.vertex_count) {
      if (!lines.next(b, e)) break;
      if (b < e && *b == '#') continue;
      Tokens t{b, e};
      if (!t.next(tok) || !is_numeric(tok)) fail(PM_E_FORMAT, path + ": bad vertex list line");
      unsigned long long id = strtoull(tok.c_str(), nullptr, 10);
      if (id >= UINT32_MAX) fail(PM_E_FORMAT, path + ": vertex id overflow");
      if (!t.next(tok)) fail(PM_E_FORMAT, path + ": missing vertex value");
      uint64_t value = static_cast<uint64_t>(atof(tok.c_str()));
      if (id != vi) {
        if (!(id > vi && id < g.vertex_count)) fail(PM_E_FORMAT, path + ": vertex list out of order");
        while (vi < id) g.labels[vi++] = 0;
      }
      g.labels[vi++] = value;
    }
  }
  uint64_t vindex = 0, eindex = 0;
  while (lines.next(b, e)) {
    if (b < e && *b == '#') continue;
    Tokens t{b, e};
    if (!t.next(tok)) fail(PM_E_FORMAT, path + ": empty edge line " + std::to_string(lines.line_number));
    if (!is_numeric(tok)) fail(PM_E_FORMAT, path + ": bad edge source at line " + std::to_string(lines.line_number));
    unsigned long long src = strtoull(tok.c_str(), nullptr, 10);
    if (src >= UINT32_MAX) fail(PM_E_FORMAT, path + ": vertex id overflow");
    if (!t.next(tok) || !is_numeric(tok))
      fail(PM_E_FORMAT, path + ": bad edge destination at line " + std::to_string(lines.line_number));
    unsigned long long dst = strtoull(tok.c_str(), nullptr, 10);
    if (dst >= UINT32_MAX) fail(PM_E_FORMAT, path + ": vertex id overflow");
    if (src != vindex - 1) {
      if (!(src >= vindex && src < g.vertex_count))
        fail(PM_E_FORMAT, path + ": edge list not sorted by source at line " + std::to_string(lines.line_number));
      while (vindex <= src) g.offsets[vindex++] = eindex;
    }
    if (eindex >= g.edge_count) fail(PM_E_FORMAT, path + ": more edges than declared");
    g.adj[eindex++] = static_cast<uint32_t>(dst);
  }
  if (!(vindex <= g.vertex_count)) fail(PM_E_FORMAT, path + ": vertex index overflow");
  if (eindex != g.edge_count) fail(PM_E_FORMAT, path + ": fewer edges than declared (truncated file?)");
  while (vindex <= g.vertex_count) g.offsets[vindex++] = eindex;
  return g;
}

template <typename T>
void read_exact(FILE* f, T* dst, size_t n, const std::string& path) {
  if (n && fread(dst, sizeof(T), n, f) != n) fail(PM_E_FORMAT, path + ": invalid binary file format (truncated)");
}

HostGraph parse_binary(FILE* f, const std::string& path) {
  HostGraph g;
  uint32_t vid_size = 0, eid_size = 0;
  read_exact(f, &vid_size, 1, path);
  read_exact(f, &eid_size, 1, path);
  if (vid_size != 4 || (eid_size != 4 && eid_size != 8))
    fail(PM_E_FORMAT, path + ": unsupported vid/eid sizes in binary header");
  uint32_t vcount = 0;
  read_exact(f, &vcount, 1, path);
  uint64_t ecount = 0;
  if (eid_size == 4) {
    uint32_t e32 = 0;
    read_exact(f, &e32, 1, path);
    ecount = e32;
  } else {
    read_exact(f, &ecount, 1, path);
  }
  uint8_t flags[3];
  read_exact(f, flags, 3, path);
  g.vertex_count = vcount;
  g.edge_count = ecount;
  g.valued = flags[0] != 0;
  bool weighted = flags[1] != 0;
  g.directed = flags[2] != 0;
  g.offsets.resize(static_cast<size_t>(vcount) + 1);
  if (eid_size == 4) {
    std::vector<uint32_t> off32(static_cast<size_t>(vcount) + 1);
    read_exact(f, off32.data(), off32.size(), path);
    for (size_t i = 0; i < off32.size(); ++i) g.offsets[i] = off32[i];
  } else {
    read_exact(f, g.offsets.data(), g.offsets.size(), path);
  }
  if (g.valued) {
    g.labels.resize(vcount);
    read_exact(f, g.labels.data(), g.labels.size(), path);
  }
  g.adj.resize(ecount);
  read_exact(f, g.adj.data(), g.adj.size(), path);
  (void)weighted;  // weights are not loaded (graph_initialize(path, false, ...))
  if (g.offsets[vcount] != ecount) fail(PM_E_FORMAT, path + ": CSR offsets do not end at edge count");
  for (uint32_t v = 0; v < vcount; ++v)
    if (g.offsets[v] > g.offsets[v + 1]) fail(PM_E_FORMAT, path + ": CSR offsets not monotone");
  for (uint64_t i = 0; i < ecount; ++i)
    if (g.adj[i] >= vcount) fail(PM_E_FORMAT, path + ": edge target out of range");
  return g;
}

}  // namespace

bool is_regular_file(const std::string& path) {
  struct stat st;
  return stat(path.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

HostGraph read_totem_graph(const std::string& path) {
  FilePtr f(fopen(path.c_str(), "rb"));
  if (!f) fail(PM_E_IO, "can't open file " + path);
  uint32_t magic = 0;
  if (fread(&magic, sizeof(magic), 1, f.get()) != 1) fail(PM_E_IO, "can't open file " + path);
  if (magic == kBinaryMagic) return parse_binary(f.get(), path);
  std::string data = slurp(f.get(), path);
  HostGraph g = parse_text(data, path);
  for (uint64_t i = 0; i < g.edge_count; ++i)
    if (g.adj[i] >= g.vertex_count) fail(PM_E_FORMAT, path + ": edge target out of range");
  return g;
}

void read_vertex_labels(const std::string& path, HostGraph& g) {
  FilePtr f(fopen(path.c_str(), "rb"));
  if (!f) fail(PM_E_IO, "can't open vertex label file " + path);
  std::string data = slurp(f.get(), path);
  g.valued = true;
  g.labels.assign(g.vertex_count, 0);
  Lines lines{data.data(), data.data() + data.size()};
  const char* b;
  const char* e;
  std::string tok;
  uint32_t vi = 0;
  while (vi < g.vertex_count) {
    if (!lines.next(b, e)) break;
    if (b < e && *b == '#') continue;
    Tokens t{b, e};
    if (!t.next(tok) || !is_numeric(tok)) fail(PM_E_FORMAT, path + ": parse_vertex_list");
    unsigned long long id = strtoull(tok.c_str(), nullptr, 10);
    if (id >= UINT32_MAX) fail(PM_E_FORMAT, path + ": vertex id overflow");
    if (!t.next(tok)) fail(PM_E_FORMAT, path + ": parse_vertex_list");
    uint64_t value = static_cast<uint64_t>(atoll(tok.c_str()));
    if (id != vi) {
      if (!(id > vi && id < g.vertex_count)) fail(PM_E_FORMAT, path + ": parse_vertex_list");
      while (vi < id) g.labels[vi++] = 0;
    }
    g.labels[vi++] = value;
  }
}

void write_totem_binary(const HostGraph& g, const std::string& path, int eid_bytes) {
  if (eid_bytes != 4 && eid_bytes != 8) fail(PM_E_INVALID_ARG, "eid_bytes must be 4 or 8");
  if (eid_bytes == 4 && g.edge_count > UINT32_MAX) fail(PM_E_INVALID_ARG, "edge count needs 64-bit edge ids");
  FilePtr f(fopen(path.c_str(), "wb"));
  if (!f) fail(PM_E_IO, "can't create " + path);
  auto put = [&](const void* p, size_t sz, size_t n) {
    if (n && fwrite(p, sz, n, f.get()) != n) fail(PM_E_IO, "write failed on " + path);
  };
  uint32_t w = kBinaryMagic;
  put(&w, 4, 1);
  w = 4;
  put(&w, 4, 1);
  w = static_cast<uint32_t>(eid_bytes);
  put(&w, 4, 1);
  put(&g.vertex_count, 4, 1);
  if (eid_bytes == 4) {
    uint32_t e32 = static_cast<uint32_t>(g.edge_count);
    put(&e32, 4, 1);
  } else {
    put(&g.edge_count, 8, 1);
  }
  uint8_t flags[3] = {static_cast<uint8_t>(g.valued), 0, static_cast<uint8_t>(g.directed)};
  put(flags, 1, 3);
  if (eid_bytes == 4) {
    std::vector<uint32_t> off32(g.offsets.begin(), g.offsets.end());
    put(off32.data(), 4, off32.size());
  } else {
    put(g.offsets.data(), 8, g.offsets.size());
  }
  if (g.valued) put(g.labels.data(), 8, g.labels.size());
  put(g.adj.data(), 4, g.adj.size());
}

void write_totem_text(const HostGraph& g, const std::string& path) {
  FilePtr f(fopen(path.c_str(), "wb"));
  if (!f) fail(PM_E_IO, "can't create " + path);
  fprintf(f.get(), "#Nodes:%u\n#Edges:%llu\n#%s\n", g.vertex_count,
          static_cast<unsigned long long>(g.edge_count), g.directed ? "Directed" : "Undirected");
  for (uint32_t v = 0; v < g.vertex_count; ++v)
    for (uint64_t i = g.offsets[v]; i < g.offsets[v + 1]; ++i) fprintf(f.get(), "%u %u\n", v, g.adj[i]);
}

void write_vertex_labels(const HostGraph& g, const std::string& path) {
  FilePtr f(fopen(path.c_str(), "wb"));
  if (!f) fail(PM_E_IO, "can't create " + path);
  for (uint32_t v = 0; v < g.vertex_count; ++v)
    fprintf(f.get(), "%u %llu\n", v, static_cast<unsigned long long>(g.labels.empty() ? 0 : g.labels[v]));
}

}  // namespace pmgb
