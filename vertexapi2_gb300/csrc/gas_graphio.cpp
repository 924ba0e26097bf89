// Graph files (gas_load_graph / gas_write_graph_* / gas_write_vertex_values
// in gas_gb300.h): the formats the reference's drivers read and write
// (graphio.cpp), with the same edge lists.
//
//   .mtx  MatrixMarket coordinate (graphio.cpp:190-262): header
//         "%%MatrixMarket matrix coordinate <field> <symmetry>", '%'
//         comments, the size line skipped, 1-based ids, self-loops dropped,
//         symmetric / skew-symmetric / hermitian add the reverse edge
//         (skew negates its value), values read as float and truncated to
//         int; "pattern" has no values, "complex" is refused.
//   .edge SNAP / GraphLab edge list (graphio.cpp:178-188): '#' comments,
//         0-based "src dst" lines, self-loops dropped, no values.
//   .gr   Lonestar binary CSR (graphio.cpp:265-362): u64 version, u64 edge
//         value width (4), u64 vertices, u64 edges, u64 end offsets per
//         vertex, u32 destinations padded to 8 bytes, u32 values.
//   .gz   any of the text formats gzip-compressed (when built with zlib).
//
// Lines are read in 1023-byte pieces as the reference reads them; the
// vertex count is the largest id seen + 1, where a dropped self-loop still
// counts when the file has no values (graphio.cpp:126-160).
#include <cctype>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#ifdef GAS_HAVE_ZLIB
#include <zlib.h>
#endif

#include "gas_gb300.h"
#include "gas_internal.h"

using gas::internal::fail;

namespace {

// A text source read in pieces of at most 1023 bytes (a line, or the part
// of a longer line that fits), plain or gzip.
class LineReader {
 public:
  ~LineReader() { close(); }
  bool open(const char *path, bool gz) {
    gz_ = gz;
#ifdef GAS_HAVE_ZLIB
    if (gz) {
      zf_ = gzopen(path, "rb");
      return zf_ != nullptr;
    }
#else
    if (gz) return false;
#endif
    f_ = fopen(path, "rb");
    return f_ != nullptr;
  }
  // false at end of input
  bool next(char *buf, int size) {
    buf[0] = 0;
#ifdef GAS_HAVE_ZLIB
    if (gz_) return gzgets(zf_, buf, size) != nullptr;
#endif
    return fgets(buf, size, f_) != nullptr;
  }
  void close() {
#ifdef GAS_HAVE_ZLIB
    if (zf_) gzclose(zf_);
    zf_ = nullptr;
#endif
    if (f_) fclose(f_);
    f_ = nullptr;
  }

 private:
  bool gz_ = false;
  FILE *f_ = nullptr;
#ifdef GAS_HAVE_ZLIB
  gzFile zf_ = nullptr;
#endif
};

enum Symmetry { kGeneral, kSymmetric, kSkew, kHermitian };

bool blank(const char *s) {
  for (; *s; ++s)
    if (!isspace((unsigned char)*s)) return false;
  return true;
}

int to_int(float v) {  // float -> int as a C conversion, kept inside int range
  if (std::isnan(v)) return 0;
  if (v >= 2147483647.0f) return INT_MAX;
  if (v <= -2147483648.0f) return INT_MIN;
  return (int)v;
}

struct EdgeLists {
  std::vector<int32_t> s, d, w;
  int32_t nV = 0;
  bool hasValues = false;  // the file carries edge values and they were asked for
};

// The line loop shared by the text formats.
gas_status read_edges(LineReader &in, char comment, bool skipSizeLine, bool oneBased,
                      Symmetry sym, bool values, EdgeLists &g, const char *path) {
  char buf[1024];
  long long line = 0, maxId = 0;
  bool sizeLine = skipSizeLine;
  while (in.next(buf, sizeof(buf))) {
    ++line;
    if (buf[0] == 0 || buf[0] == comment || blank(buf)) continue;
    if (sizeLine) {
      sizeLine = false;
      continue;
    }
    int a = 0, b = 0, used = 0;
    if (sscanf(buf, "%d%d%n", &a, &b, &used) != 2)
      return fail(GAS_ERR_INVALID, "%s: no src/dst at line %lld", path, line);
    if (oneBased) {
      --a;
      --b;
    }
    float val = 0.0f;
    if (values && sscanf(buf + used, "%f", &val) != 1) val = 0.0f;
    if (a < 0 || b < 0) return fail(GAS_ERR_INVALID, "%s: negative id at line %lld", path, line);
    if (a == b) {                 // self-loop: dropped
      if (values) continue;       // (and, with values, not counted)
    } else {
      g.s.push_back(a);
      g.d.push_back(b);
      if (sym != kGeneral) {
        g.s.push_back(b);
        g.d.push_back(a);
      }
      if (values) {
        g.w.push_back(to_int(val));
        if (sym == kSymmetric) g.w.push_back(to_int(val));
        if (sym == kSkew) g.w.push_back(to_int(-val));
      }
    }
    maxId = std::max<long long>(maxId, std::max(a, b));
  }
  if (maxId >= INT_MAX) return fail(GAS_ERR_UNSUPPORTED, "%s: vertex id above int32", path);
  g.nV = (int32_t)(maxId + 1);
  return GAS_OK;
}

gas_status load_mtx(const char *path, bool gz, bool wantValues, EdgeLists &g) {
  LineReader in;
  if (!in.open(path, gz)) return fail(GAS_ERR_INVALID, "cannot open %s", path);
  char head[1024];
  if (!in.next(head, sizeof(head)) || head[0] == 0)
    return fail(GAS_ERR_INVALID, "%s: no MatrixMarket header", path);
  // "%%MatrixMarket matrix coordinate <field> <symmetry>", split on ' ' and '\n'
  std::vector<std::string> tok;
  {
    std::string cur;
    for (const char *p = head; *p; ++p) {
      if (*p == ' ' || *p == '\n') {
        if (!cur.empty()) tok.push_back(cur);
        cur.clear();
      } else {
        cur += *p;
      }
    }
    if (!cur.empty()) tok.push_back(cur);
  }
  if (tok.size() < 5) return fail(GAS_ERR_INVALID, "%s: short MatrixMarket header", path);
  if (tok[1] != "matrix") return fail(GAS_ERR_INVALID, "%s: header token '%s'", path, tok[1].c_str());
  if (tok[2] != "coordinate")
    return fail(GAS_ERR_UNSUPPORTED, "%s: only coordinate MatrixMarket files", path);
  bool values = wantValues;
  if (tok[3] == "pattern") values = false;
  if (tok[3] == "complex") return fail(GAS_ERR_UNSUPPORTED, "%s: complex values", path);
  Symmetry sym;
  if (tok[4] == "general") sym = kGeneral;
  else if (tok[4] == "symmetric") sym = kSymmetric;
  else if (tok[4] == "skew-symmetric") sym = kSkew;
  else if (tok[4] == "hermitian") sym = kHermitian;
  else return fail(GAS_ERR_INVALID, "%s: symmetry '%s'", path, tok[4].c_str());
  if (sym == kHermitian && values)
    return fail(GAS_ERR_UNSUPPORTED, "%s: hermitian files with values", path);
  g.hasValues = values;
  return read_edges(in, '%', true, true, sym, values, g, path);
}

gas_status load_snap(const char *path, bool gz, EdgeLists &g) {
  LineReader in;
  if (!in.open(path, gz)) return fail(GAS_ERR_INVALID, "cannot open %s", path);
  return read_edges(in, '#', false, false, kGeneral, false, g, path);
}

gas_status load_gr(const char *path, bool wantValues, EdgeLists &g) {
  FILE *f = fopen(path, "rb");
  if (!f) return fail(GAS_ERR_INVALID, "cannot open %s", path);
  struct Closer {
    FILE *f;
    ~Closer() { fclose(f); }
  } closer{f};
  uint64_t h[4];
  if (fread(h, 8, 4, f) != 4) return fail(GAS_ERR_INVALID, "%s: short .gr header", path);
  const uint64_t width = h[1], nV = h[2], nE = h[3];
  if (width != 4 && !(width == 0 && !wantValues))
    return fail(GAS_ERR_UNSUPPORTED, "%s: edge values of %llu bytes", path,
                (unsigned long long)width);
  if (width == 0 && wantValues) return fail(GAS_ERR_INVALID, "%s: no edge values", path);
  if (nV >= (uint64_t)INT_MAX || nE >= (uint64_t)INT_MAX)
    return fail(GAS_ERR_UNSUPPORTED, "%s: graph above int32 sizes", path);
  std::vector<uint64_t> ends(nV);
  if (nV && fread(ends.data(), 8, nV, f) != nV) return fail(GAS_ERR_INVALID, "%s: short offsets", path);
  g.d.resize(nE);
  if (nE && fread(g.d.data(), 4, nE, f) != nE) return fail(GAS_ERR_INVALID, "%s: short edges", path);
  if (nE % 2) {
    uint32_t pad;
    if (fread(&pad, 4, 1, f) != 1) return fail(GAS_ERR_INVALID, "%s: missing padding", path);
  }
  g.s.resize(nE);
  uint64_t j = 0;
  for (uint64_t v = 0; v < nV; ++v) {
    if (ends[v] > nE || ends[v] < j) return fail(GAS_ERR_INVALID, "%s: bad offsets", path);
    for (; j < ends[v]; ++j) g.s[j] = (int32_t)v;
  }
  if (j != nE) return fail(GAS_ERR_INVALID, "%s: offsets end at %llu of %llu edges", path,
                           (unsigned long long)j, (unsigned long long)nE);
  if (wantValues) {
    g.w.resize(nE);
    if (nE && fread(g.w.data(), 4, nE, f) != nE) return fail(GAS_ERR_INVALID, "%s: short values", path);
    g.hasValues = true;
  }
  g.nV = (int32_t)nV;
  return GAS_OK;
}

// Extension dispatch of graphio.cpp:441-473: the last '.' (before a ".gz").
const char *extension(const char *path, bool &gz) {
  const char *p = path + strlen(path);
  while (p >= path && *p != '.') --p;
  gz = false;
  if (p >= path && strcmp(p, ".gz") == 0) {
    gz = true;
    --p;
    while (p >= path && *p != '.') --p;
  }
  return p >= path ? p : path;
}

template <typename T>
T *copy_out(const std::vector<T> &v) {
  T *p = static_cast<T *>(malloc(sizeof(T) * (v.size() + 1)));
  if (p && !v.empty()) memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}

}  // namespace

extern "C" {

gas_status gas_load_graph(const char *path, int32_t wantValues, gas_edge_list *out) {
  if (!path || !out) return fail(GAS_ERR_INVALID, "gas_load_graph: null argument");
  memset(out, 0, sizeof(*out));
  bool gz = false;
  const char *ext = extension(path, gz);
  EdgeLists g;
  gas_status st;
  if (strncmp(ext, ".edge", 5) == 0) {
    st = load_snap(path, gz, g);
  } else if (strncmp(ext, ".mtx", 4) == 0) {
    st = load_mtx(path, gz, wantValues != 0, g);
  } else if (strncmp(ext, ".gr", 3) == 0) {
    st = gz ? fail(GAS_ERR_UNSUPPORTED, "%s: compressed .gr files", path)
            : load_gr(path, wantValues != 0, g);
  } else {
    st = fail(GAS_ERR_UNSUPPORTED, "%s: unknown graph file extension '%s'", path, ext);
  }
#ifndef GAS_HAVE_ZLIB
  if (gz && st == GAS_ERR_INVALID) st = fail(GAS_ERR_UNSUPPORTED, "%s: built without zlib", path);
#endif
  if (st) return st;
  out->nVertices = g.nV;
  out->nEdges = (int64_t)g.s.size();
  out->srcs = copy_out(g.s);
  out->dsts = copy_out(g.d);
  out->weights = g.hasValues ? copy_out(g.w) : nullptr;
  if (!out->srcs || !out->dsts || (g.hasValues && !out->weights)) {
    gas_edge_list_free(out);
    return fail(GAS_ERR_OOM, "host allocation");
  }
  return GAS_OK;
}

gas_status gas_write_graph_mtx(const char *path, int32_t nVertices, int64_t nEdges,
                               const int32_t *srcs, const int32_t *dsts, const int32_t *values) {
  if (!path || nVertices < 0 || nEdges < 0 || (nEdges > 0 && (!srcs || !dsts)))
    return fail(GAS_ERR_INVALID, "gas_write_graph_mtx: bad argument");
  FILE *f = fopen(path, "w");
  if (!f) return fail(GAS_ERR_INVALID, "cannot write %s", path);
  fprintf(f, "%%%%MatrixMarket matrix coordinate Integer general\n");
  fprintf(f, "%d %d %lld\n", nVertices, nVertices, (long long)nEdges);
  for (int64_t i = 0; i < nEdges; ++i) {
    if (values)
      fprintf(f, "%d %d %d\n", srcs[i] + 1, dsts[i] + 1, values[i]);
    else
      fprintf(f, "%d %d\n", srcs[i] + 1, dsts[i] + 1);
  }
  return fclose(f) == 0 ? GAS_OK : fail(GAS_ERR_INVALID, "write error on %s", path);
}

gas_status gas_write_graph_gr(const char *path, int32_t nVertices, int64_t nEdges,
                              const int32_t *offsets, const int32_t *dsts, const int32_t *values) {
  if (!path || nVertices < 0 || nEdges < 0 || !offsets || (nEdges > 0 && !dsts))
    return fail(GAS_ERR_INVALID, "gas_write_graph_gr: bad argument");
  FILE *f = fopen(path, "wb");
  if (!f) return fail(GAS_ERR_INVALID, "cannot write %s", path);
  const uint64_t h[4] = {1u, values ? 4u : 0u, (uint64_t)nVertices, (uint64_t)nEdges};
  bool ok = fwrite(h, 8, 4, f) == 4;
  for (int32_t v = 0; v < nVertices && ok; ++v) {
    const uint64_t end = (uint64_t)offsets[v + 1];
    ok = fwrite(&end, 8, 1, f) == 1;
  }
  if (ok && nEdges) ok = fwrite(dsts, 4, (size_t)nEdges, f) == (size_t)nEdges;
  if (ok && nEdges % 2) {
    const uint32_t pad = 0;
    ok = fwrite(&pad, 4, 1, f) == 1;
  }
  if (ok && values && nEdges) ok = fwrite(values, 4, (size_t)nEdges, f) == (size_t)nEdges;
  ok = (fclose(f) == 0) && ok;
  return ok ? GAS_OK : fail(GAS_ERR_INVALID, "write error on %s", path);
}

gas_status gas_write_vertex_values(const char *path, int32_t nVertices, const void *values,
                                   int32_t isFloat, int32_t strideBytes) {
  if (!path || nVertices < 0 || (nVertices > 0 && !values))
    return fail(GAS_ERR_INVALID, "gas_write_vertex_values: bad argument");
  if (strideBytes == 0) strideBytes = 4;
  if (strideBytes < 4) return fail(GAS_ERR_INVALID, "stride below 4 bytes");
  FILE *f = fopen(path, "w");
  if (!f) return fail(GAS_ERR_INVALID, "cannot write %s", path);
  const char *p = static_cast<const char *>(values);
  for (int32_t i = 0; i < nVertices; ++i, p += strideBytes) {
    if (isFloat) {
      float x;
      memcpy(&x, p, 4);
      fprintf(f, "%d %f\n", i, x);
    } else {
      int32_t x;
      memcpy(&x, p, 4);
      fprintf(f, "%d %d\n", i, x);
    }
  }
  return fclose(f) == 0 ? GAS_OK : fail(GAS_ERR_INVALID, "write error on %s", path);
}

}  // extern "C"
