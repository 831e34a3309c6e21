// cm_graph.cpp -- host graphs: allocation, validation, synthetic generators,
// METIS .graph IO, partition file output, edge cut and imbalance.
//
// Reference behaviour mirrored here (paths inside the cuMetis project):
//   cuMetis.cu:3712-3851  cuMetis_readgraph   (format digits, 1-based ids,
//                                              error cases; nedges *= 2)
//   cuMetis.cu:3856-3870  cuMetis_writetofile (<graph>.part.<k>, one id per line)
//   cuMetis.cu:356-366    cuMetis_computecut  (sum of cut entries / 2)
//   mtx_to_graph.c        MatrixMarket -> graph: the pattern of A + A^T
//                         without the diagonal, unit weights
// The generators have no reference counterpart: they produce the synthetic
// workloads (meshes, R-MAT, random geometric graphs) with counter-based
// randomness, so the same (sizes, seed) give the same graph on any host and
// for any thread count.
#include "cm_internal.h"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local char g_errbuf[1024] = "";

inline uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Builds a sorted, symmetric CSR from a list of unique undirected keys
// (lo << 32 | hi, lo < hi) that is already sorted ascending.
int csr_from_sorted_keys(int64_t n, const std::vector<uint64_t> &keys, cm_graph *out,
                         uint64_t wseed, int32_t wmin, int32_t wmax) {
  const int64_t m = 2 * (int64_t)keys.size();
  if (n > INT32_MAX - 1 || m > INT32_MAX) return cm_fail(CM_ERR_UNSUPPORTED, "graph exceeds int32 CSR limits (n=%lld m=%lld)", (long long)n, (long long)m);
  int rc = cm_graph_alloc((int32_t)n, (int32_t)m, out);
  if (rc) return rc;
  int32_t *xadj = out->xadj;
  std::fill(xadj, xadj + n + 1, 0);
  for (uint64_t k : keys) {
    xadj[(k >> 32) + 1]++;
    xadj[(k & 0xffffffffu) + 1]++;
  }
  for (int64_t i = 0; i < n; ++i) xadj[i + 1] += xadj[i];
  std::vector<int32_t> pos(xadj, xadj + n);
  const uint64_t span = (uint64_t)(wmax - wmin) + 1;
  // Keys sorted by (lo, hi): row r receives its smaller neighbours (as hi of
  // earlier keys) before its larger ones (as lo of its own block), so every
  // row comes out sorted by neighbour id.
  for (uint64_t k : keys) {
    int32_t lo = (int32_t)(k >> 32), hi = (int32_t)(k & 0xffffffffu);
    int32_t w = wmin + (int32_t)(mix64(wseed ^ k) % span);
    int32_t p = pos[lo]++;
    out->adjncy[p] = hi; out->adjwgt[p] = w;
    p = pos[hi]++;
    out->adjncy[p] = lo; out->adjwgt[p] = w;
  }
  for (int64_t i = 0; i < n; ++i) out->vwgt[i] = 1;
  return CM_OK;
}

// LSD radix sort of 64-bit keys on their low `bits` bits (16-bit digits).
void radix_sort_u64(std::vector<uint64_t> &a, int bits) {
  std::vector<uint64_t> tmp(a.size());
  const int digit = 16;
  std::vector<size_t> cnt(1u << digit);
  for (int shift = 0; shift < bits; shift += digit) {
    std::fill(cnt.begin(), cnt.end(), 0);
    for (uint64_t k : a) cnt[(k >> shift) & 0xffff]++;
    size_t s = 0;
    for (auto &c : cnt) { size_t t = c; c = s; s += t; }
    for (uint64_t k : a) tmp[cnt[(k >> shift) & 0xffff]++] = k;
    a.swap(tmp);
  }
}

}  // namespace

int cm_fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errbuf, sizeof g_errbuf, fmt, ap);
  va_end(ap);
  return code;
}

extern "C" const char *cm_last_error(void) { return g_errbuf; }

extern "C" int cm_graph_alloc(int32_t nvtxs, int32_t nedges, cm_graph *out) {
  if (!out || nvtxs < 0 || nedges < 0) return cm_fail(CM_ERR_INVALID, "cm_graph_alloc: bad arguments");
  memset(out, 0, sizeof *out);
  out->nvtxs = nvtxs;
  out->nedges = nedges;
  out->xadj = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nvtxs + 1));
  out->vwgt = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nvtxs + 1));
  out->adjncy = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nedges + 1));
  out->adjwgt = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nedges + 1));
  if (!out->xadj || !out->vwgt || !out->adjncy || !out->adjwgt) {
    cm_graph_free(out);
    return cm_fail(CM_ERR_NOMEM, "cm_graph_alloc: out of host memory (n=%d m=%d)", nvtxs, nedges);
  }
  out->xadj[0] = 0;
  return CM_OK;
}

extern "C" void cm_graph_free(cm_graph *g) {
  if (!g) return;
  free(g->xadj); free(g->vwgt); free(g->adjncy); free(g->adjwgt);
  memset(g, 0, sizeof *g);
}

extern "C" int cm_graph_validate(const cm_graph *g, int check_symmetry, int allow_self_loops) {
  if (!g || g->nvtxs < 0 || g->nedges < 0 || !g->xadj) return cm_fail(CM_ERR_INVALID, "validate: null graph");
  const int32_t n = g->nvtxs;
  if (g->xadj[0] != 0) return cm_fail(CM_ERR_INVALID, "validate: xadj[0] != 0");
  for (int32_t v = 0; v < n; ++v)
    if (g->xadj[v + 1] < g->xadj[v]) return cm_fail(CM_ERR_INVALID, "validate: xadj decreases at %d", v);
  if (g->xadj[n] != g->nedges) return cm_fail(CM_ERR_INVALID, "validate: xadj[n]=%d != nedges=%d", g->xadj[n], g->nedges);
  for (int32_t v = 0; v < n; ++v) {
    if (g->vwgt && g->vwgt[v] < 0) return cm_fail(CM_ERR_INVALID, "validate: negative vwgt at %d", v);
    for (int32_t j = g->xadj[v]; j < g->xadj[v + 1]; ++j) {
      int32_t u = g->adjncy[j];
      if (u < 0 || u >= n) return cm_fail(CM_ERR_INVALID, "validate: neighbour %d of %d out of range", u, v);
      if (u == v && !allow_self_loops) return cm_fail(CM_ERR_INVALID, "validate: self loop at %d", v);
      if (g->adjwgt && g->adjwgt[j] <= 0) return cm_fail(CM_ERR_INVALID, "validate: non-positive weight at entry %d", j);
    }
  }
  if (check_symmetry) {
    // Transpose by counting sort; compare sorted (nbr, w) multisets per row.
    std::vector<int64_t> tx(n + 1, 0);
    for (int32_t j = 0; j < g->nedges; ++j) tx[g->adjncy[j] + 1]++;
    for (int32_t v = 0; v < n; ++v) tx[v + 1] += tx[v];
    std::vector<std::pair<int32_t, int32_t>> t(g->nedges);
    std::vector<int64_t> p(tx.begin(), tx.end() - 1);
    for (int32_t v = 0; v < n; ++v)
      for (int32_t j = g->xadj[v]; j < g->xadj[v + 1]; ++j)
        t[p[g->adjncy[j]]++] = {v, g->adjwgt ? g->adjwgt[j] : 1};
    std::vector<std::pair<int32_t, int32_t>> row;
    for (int32_t v = 0; v < n; ++v) {
      row.clear();
      for (int32_t j = g->xadj[v]; j < g->xadj[v + 1]; ++j) row.push_back({g->adjncy[j], g->adjwgt ? g->adjwgt[j] : 1});
      std::sort(row.begin(), row.end());
      std::sort(t.begin() + tx[v], t.begin() + tx[v + 1]);
      if ((int64_t)row.size() != tx[v + 1] - tx[v] || !std::equal(row.begin(), row.end(), t.begin() + tx[v]))
        return cm_fail(CM_ERR_INVALID, "validate: adjacency of %d is not symmetric", v);
    }
  }
  return CM_OK;
}

// ---------------------------------------------------------------------------
// Generators
// ---------------------------------------------------------------------------
namespace {
int mesh_from_offsets(int32_t nx, int32_t ny, int32_t nz, const int (*off)[3], int noff, cm_graph *out) {
  // Vertex (i,j,k) -> id (i*ny + j)*nz + k.  Undirected edges are listed by
  // positive offsets; both directions are emitted and rows sorted.
  const int64_t n = (int64_t)nx * ny * nz;
  if (n <= 0 || n > INT32_MAX - 1) return cm_fail(CM_ERR_INVALID, "mesh: bad size");
  std::vector<int64_t> deg(n + 1, 0);
  auto id = [&](int64_t i, int64_t j, int64_t k) { return (i * ny + j) * nz + k; };
  auto inside = [&](int64_t i, int64_t j, int64_t k) { return i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k < nz; };
  for (int pass = 0; pass < 2; ++pass) {
    for (int64_t i = 0; i < nx; ++i)
      for (int64_t j = 0; j < ny; ++j)
        for (int64_t k = 0; k < nz; ++k) {
          int64_t v = id(i, j, k);
          for (int s = -1; s <= 1; s += 2)
            for (int o = 0; o < noff; ++o) {
              int64_t a = i + s * off[o][0], b = j + s * off[o][1], c = k + s * off[o][2];
              if (!inside(a, b, c)) continue;
              if (pass == 0) deg[v + 1]++;
              else { int32_t p = (int32_t)deg[v]++; out->adjncy[p] = (int32_t)id(a, b, c); out->adjwgt[p] = 1; }
            }
        }
    if (pass == 0) {
      for (int64_t v = 0; v < n; ++v) deg[v + 1] += deg[v];
      if (deg[n] > INT32_MAX) return cm_fail(CM_ERR_UNSUPPORTED, "mesh: too many edges");
      int rc = cm_graph_alloc((int32_t)n, (int32_t)deg[n], out);
      if (rc) return rc;
      for (int64_t v = 0; v <= n; ++v) out->xadj[v] = (int32_t)deg[v];
    }
  }
  for (int64_t v = 0; v < n; ++v) {
    std::sort(out->adjncy + out->xadj[v], out->adjncy + out->xadj[v + 1]);
    out->vwgt[v] = 1;
  }
  return CM_OK;
}
}  // namespace

extern "C" int cm_gen_tri_grid(int32_t nx, int32_t ny, cm_graph *out) {
  static const int off[3][3] = {{0, 1, 0}, {1, 0, 0}, {1, 1, 0}};
  if (nx <= 0 || ny <= 0 || !out) return cm_fail(CM_ERR_INVALID, "tri_grid: bad size");
  return mesh_from_offsets(nx, ny, 1, off, 3, out);
}

extern "C" int cm_gen_grid2d(int32_t nx, int32_t ny, cm_graph *out) {
  static const int off[2][3] = {{0, 1, 0}, {1, 0, 0}};
  if (nx <= 0 || ny <= 0 || !out) return cm_fail(CM_ERR_INVALID, "grid2d: bad size");
  return mesh_from_offsets(nx, ny, 1, off, 2, out);
}

extern "C" int cm_gen_grid3d(int32_t nx, int32_t ny, int32_t nz, cm_graph *out) {
  static const int off[3][3] = {{0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
  if (nx <= 0 || ny <= 0 || nz <= 0 || !out) return cm_fail(CM_ERR_INVALID, "grid3d: bad size");
  return mesh_from_offsets(nx, ny, nz, off, 3, out);
}

extern "C" int cm_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c,
                           uint64_t seed, int32_t wmin, int32_t wmax, cm_graph *out) {
  if (!out || scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0 ||
      wmin < 1 || wmax < wmin)
    return cm_fail(CM_ERR_INVALID, "rmat: bad parameters");
  const int64_t n = (int64_t)1 << scale;
  const int64_t ne = (int64_t)edge_factor << scale;
  const uint64_t ta = (uint64_t)(a * 4294967296.0), tb = (uint64_t)((a + b) * 4294967296.0),
                 tc = (uint64_t)((a + b + c) * 4294967296.0);
  const uint64_t s0 = mix64(seed ^ 0x52414D4147454E31ull);  // "RAMAGEN1"
  std::vector<uint64_t> keys(ne);
  // Pair e draws one 32-bit uniform per level from a counter hash; bit pairs
  // are chosen most-significant first.
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    uint64_t u = 0, v = 0;
    for (int l = 0; l < scale; l += 2) {
      uint64_t r = mix64(s0 + (uint64_t)e * 32 + (uint64_t)(l >> 1));
      for (int h = 0; h < 2 && l + h < scale; ++h) {
        uint64_t x = h ? (r >> 32) : (r & 0xffffffffu);
        uint64_t bu = x >= tb, bv = (x >= ta && x < tb) || x >= tc;
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
    }
    uint64_t lo = u < v ? u : v, hi = u < v ? v : u;
    keys[e] = (lo == hi) ? ~0ull : ((lo << 32) | hi);  // self loops sort last
  }
  radix_sort_u64(keys, 2 * 32);
  size_t w = 0;
  for (size_t i = 0; i < keys.size(); ++i) {
    if (keys[i] == ~0ull) break;
    if (w == 0 || keys[i] != keys[w - 1]) keys[w++] = keys[i];
  }
  keys.resize(w);
  keys.shrink_to_fit();
  return csr_from_sorted_keys(n, keys, out, mix64(seed ^ 0x5745494748543031ull), wmin, wmax);
}

extern "C" int cm_gen_rgg(int32_t n, double mean_degree, uint64_t seed, cm_graph *out) {
  if (!out || n < 2 || mean_degree <= 0) return cm_fail(CM_ERR_INVALID, "rgg: bad parameters");
  const double r = std::sqrt(mean_degree / (M_PI * (double)n));
  const int64_t G = std::max<int64_t>(1, (int64_t)std::floor(1.0 / r));  // cells per side, cell >= r
  const uint64_t s0 = mix64(seed ^ 0x52474747454E3031ull);
  std::vector<double> px(n), py(n);
  std::vector<int64_t> cell(n);
  for (int32_t i = 0; i < n; ++i) {
    uint64_t h = mix64(s0 + (uint64_t)i);
    px[i] = (double)(h >> 32) / 4294967296.0;
    py[i] = (double)(h & 0xffffffffu) / 4294967296.0;
    int64_t cx = std::min<int64_t>(G - 1, (int64_t)(px[i] * G)), cy = std::min<int64_t>(G - 1, (int64_t)(py[i] * G));
    cell[i] = cx * G + cy;
  }
  // Renumber points in cell order (stable), so ids follow space.
  std::vector<int64_t> cstart(G * G + 1, 0);
  for (int32_t i = 0; i < n; ++i) cstart[cell[i] + 1]++;
  for (int64_t k = 0; k < G * G; ++k) cstart[k + 1] += cstart[k];
  std::vector<int32_t> order(n);
  {
    std::vector<int64_t> p(cstart.begin(), cstart.end() - 1);
    for (int32_t i = 0; i < n; ++i) order[p[cell[i]]++] = i;
  }
  std::vector<double> X(n), Y(n);
  for (int32_t k = 0; k < n; ++k) { X[k] = px[order[k]]; Y[k] = py[order[k]]; }
  const double r2 = r * r;
  std::vector<int64_t> deg(n + 1, 0);
  auto scan_row = [&](int32_t v, int32_t *dst) -> int32_t {
    int64_t cx = std::min<int64_t>(G - 1, (int64_t)(X[v] * G)), cy = std::min<int64_t>(G - 1, (int64_t)(Y[v] * G));
    int32_t cnt = 0;
    for (int64_t a = cx - 1; a <= cx + 1; ++a)
      for (int64_t b = cy - 1; b <= cy + 1; ++b) {
        if (a < 0 || b < 0 || a >= G || b >= G) continue;
        for (int64_t k = cstart[a * G + b]; k < cstart[a * G + b + 1]; ++k) {
          if (k == v) continue;
          double dx = X[k] - X[v], dy = Y[k] - Y[v];
          if (dx * dx + dy * dy < r2) { if (dst) dst[cnt] = (int32_t)k; ++cnt; }
        }
      }
    return cnt;
  };
#pragma omp parallel for schedule(dynamic, 4096)
  for (int32_t v = 0; v < n; ++v) deg[v + 1] = scan_row(v, nullptr);
  for (int32_t v = 0; v < n; ++v) deg[v + 1] += deg[v];
  if (deg[n] > INT32_MAX) return cm_fail(CM_ERR_UNSUPPORTED, "rgg: too many edges");
  int rc = cm_graph_alloc(n, (int32_t)deg[n], out);
  if (rc) return rc;
  for (int32_t v = 0; v <= n; ++v) out->xadj[v] = (int32_t)deg[v];
#pragma omp parallel for schedule(dynamic, 4096)
  for (int32_t v = 0; v < n; ++v) {
    scan_row(v, out->adjncy + out->xadj[v]);
    std::sort(out->adjncy + out->xadj[v], out->adjncy + out->xadj[v + 1]);
  }
  for (int32_t j = 0; j < out->nedges; ++j) out->adjwgt[j] = 1;
  for (int32_t v = 0; v < n; ++v) out->vwgt[v] = 1;
  return CM_OK;
}

// ---------------------------------------------------------------------------
// METIS .graph IO
// ---------------------------------------------------------------------------
extern "C" int cm_read_graph(const char *path, cm_graph *out) {
  if (!path || !out) return cm_fail(CM_ERR_INVALID, "read_graph: null argument");
  memset(out, 0, sizeof *out);
  FILE *fp = fopen(path, "r");
  if (!fp) return cm_fail(CM_ERR_IO, "file: %s, mode: r: %s", path, strerror(errno));
  char *line = nullptr;
  size_t cap = 0;
  int rc = CM_OK;
  auto next_line = [&]() -> bool {  // skips '%' comment lines (cu:3731-3735)
    do {
      if (getline(&line, &cap, fp) == -1) return false;
    } while (line[0] == '%');
    return true;
  };
  long long n = 0, nedges = 0;
  int fmt = 0;
  do {
    if (!next_line()) { rc = cm_fail(CM_ERR_IO, "Premature end of input file: file: %s", path); break; }
    int nf = sscanf(line, "%lld %lld %d", &n, &nedges, &fmt);
    if (nf < 2) { rc = cm_fail(CM_ERR_IO, "The input file does not specify the number of vertices and edges."); break; }
    if (n <= 0 || nedges <= 0) { rc = cm_fail(CM_ERR_IO, "The supplied nvtxs:%lld and nedges:%lld must be positive.", n, nedges); break; }
    if (fmt > 111) { rc = cm_fail(CM_ERR_IO, "Cannot read this type of file format [fmt=%d]!", fmt); break; }
    if (n > INT32_MAX - 1 || 2 * nedges > INT32_MAX) { rc = cm_fail(CM_ERR_UNSUPPORTED, "graph exceeds int32 CSR limits"); break; }
    char fs[8];
    snprintf(fs, sizeof fs, "%03d", fmt % 1000);
    // The hundreds digit (vertex sizes) is recognised but, as in the
    // reference reader, no size field is parsed.
    const bool readvw = fs[1] == '1', readew = fs[2] == '1';
    const int32_t m = (int32_t)(2 * nedges);
    if ((rc = cm_graph_alloc((int32_t)n, m, out))) break;
    for (long long i = 0; i < n; ++i) out->vwgt[i] = 1;
    int32_t k = 0;
    out->xadj[0] = 0;
    for (long long i = 0; i < n && rc == CM_OK; ++i) {
      if (!next_line()) { rc = cm_fail(CM_ERR_IO, "Premature end of input file while reading vertex %lld.", i + 1); break; }
      char *cur = line, *nxt = nullptr;
      if (readvw) {
        long vw = strtol(cur, &nxt, 10);
        if (nxt == cur) { rc = cm_fail(CM_ERR_IO, "The line for vertex %lld does not have enough weights for the 1 constraints.", i + 1); break; }
        if (vw < 0) { rc = cm_fail(CM_ERR_IO, "The weight vertex %lld and constraint 0 must be >= 0", i + 1); break; }
        out->vwgt[i] = (int32_t)vw;
        cur = nxt;
      }
      while (true) {
        long e = strtol(cur, &nxt, 10);
        if (nxt == cur) break;
        cur = nxt;
        if (e < 1 || e > n) { rc = cm_fail(CM_ERR_IO, "Edge %ld for vertex %lld is out of bounds", e, i + 1); break; }
        long ew = 1;
        if (readew) {
          ew = strtol(cur, &nxt, 10);
          if (nxt == cur) { rc = cm_fail(CM_ERR_IO, "Premature end of line for vertex %lld", i + 1); break; }
          if (ew <= 0) { rc = cm_fail(CM_ERR_IO, "The weight (%ld) for edge (%lld, %ld) must be positive.", ew, i + 1, e); break; }
          cur = nxt;
        }
        if (k == m) { rc = cm_fail(CM_ERR_IO, "There are more edges in the file than the %lld specified.", nedges); break; }
        out->adjncy[k] = (int32_t)(e - 1);
        out->adjwgt[k] = (int32_t)ew;
        ++k;
      }
      out->xadj[i + 1] = k;
    }
    if (rc == CM_OK && k != m)
      rc = cm_fail(CM_ERR_IO, "In the first line of the file, you specified that the graph contained %lld edges. However, I only found %d edges in the file.", nedges, k / 2);
  } while (0);
  free(line);
  fclose(fp);
  if (rc) cm_graph_free(out);
  return rc;
}

extern "C" int cm_write_graph(const char *path, const cm_graph *g) {
  if (!path || !g || !g->xadj) return cm_fail(CM_ERR_INVALID, "write_graph: null argument");
  bool vw = false, ew = false;
  for (int32_t v = 0; v < g->nvtxs && g->vwgt; ++v) vw |= g->vwgt[v] != 1;
  for (int32_t j = 0; j < g->nedges && g->adjwgt; ++j) ew |= g->adjwgt[j] != 1;
  FILE *fp = fopen(path, "w");
  if (!fp) return cm_fail(CM_ERR_IO, "file: %s, mode: w: %s", path, strerror(errno));
  if (vw || ew) fprintf(fp, "%d %d %d%d\n", g->nvtxs, g->nedges / 2, vw ? 1 : 0, ew ? 1 : 0);
  else fprintf(fp, "%d %d\n", g->nvtxs, g->nedges / 2);
  for (int32_t v = 0; v < g->nvtxs; ++v) {
    bool first = true;
    if (vw) { fprintf(fp, "%d", g->vwgt[v]); first = false; }
    for (int32_t j = g->xadj[v]; j < g->xadj[v + 1]; ++j) {
      fprintf(fp, first ? "%d" : " %d", g->adjncy[j] + 1);
      first = false;
      if (ew) fprintf(fp, " %d", g->adjwgt[j]);
    }
    fputc('\n', fp);
  }
  int bad = ferror(fp);
  fclose(fp);
  return bad ? cm_fail(CM_ERR_IO, "write_graph: write error on %s", path) : CM_OK;
}

// MatrixMarket coordinate file -> graph with the pattern of A + A^T minus the
// diagonal, rows sorted, unit weights (what mtx_to_graph.c writes: it merges
// each row of A with the same row of A^T and drops i == j).  Symmetric,
// skew-symmetric and Hermitian files list one triangle; both directions are
// added either way.  Values are ignored.  The matrix must be square.
extern "C" int cm_read_mtx(const char *path, cm_graph *out) {
  if (!path || !out) return cm_fail(CM_ERR_INVALID, "read_mtx: null argument");
  *out = cm_graph{};
  FILE *fp = fopen(path, "r");
  if (!fp) return cm_fail(CM_ERR_IO, "file: %s, mode: r: %s", path, strerror(errno));
  char line[4096];
  if (!fgets(line, sizeof line, fp) || strncmp(line, "%%MatrixMarket", 14) != 0) {
    fclose(fp);
    return cm_fail(CM_ERR_IO, "read_mtx: %s: missing %%%%MatrixMarket header", path);
  }
  if (!strstr(line, "coordinate")) {
    fclose(fp);
    return cm_fail(CM_ERR_IO, "read_mtx: %s: only coordinate matrices are graphs", path);
  }
  long long nr = 0, nc = 0, nnz = 0;
  while (fgets(line, sizeof line, fp)) {
    if (line[0] == '%') continue;
    if (sscanf(line, "%lld %lld %lld", &nr, &nc, &nnz) == 3) break;
    nr = -1;
    break;
  }
  if (nr <= 0 || nr != nc || nnz < 0 || nr >= INT32_MAX) {
    fclose(fp);
    return cm_fail(CM_ERR_IO, "read_mtx: %s: bad or non-square size line", path);
  }
  std::vector<std::pair<int32_t, int32_t>> e;
  e.reserve((size_t)nnz * 2);
  for (long long k = 0; k < nnz; ++k) {
    long long i, j;
    if (!fgets(line, sizeof line, fp) || sscanf(line, "%lld %lld", &i, &j) != 2 || i < 1 || j < 1 || i > nr ||
        j > nr) {
      fclose(fp);
      return cm_fail(CM_ERR_IO, "read_mtx: %s: bad entry %lld", path, k + 1);
    }
    if (i == j) continue;
    e.emplace_back((int32_t)(i - 1), (int32_t)(j - 1));
    e.emplace_back((int32_t)(j - 1), (int32_t)(i - 1));
  }
  fclose(fp);
  std::sort(e.begin(), e.end());
  e.erase(std::unique(e.begin(), e.end()), e.end());
  if (e.size() >= (size_t)INT32_MAX) return cm_fail(CM_ERR_UNSUPPORTED, "read_mtx: %s: too many entries", path);
  int rc = cm_graph_alloc((int32_t)nr, (int32_t)e.size(), out);
  if (rc) return rc;
  std::fill(out->xadj, out->xadj + nr + 1, 0);
  for (size_t k = 0; k < e.size(); ++k) {
    out->xadj[e[k].first + 1]++;
    out->adjncy[k] = e[k].second;
    out->adjwgt[k] = 1;
  }
  for (long long v = 0; v < nr; ++v) {
    out->xadj[v + 1] += out->xadj[v];
    out->vwgt[v] = 1;
  }
  return CM_OK;
}

extern "C" int cm_write_partition(const char *graph_path, int32_t nparts, int32_t nvtxs, const int32_t *part) {
  if (!graph_path || !part || nvtxs < 0) return cm_fail(CM_ERR_INVALID, "write_partition: bad arguments");
  std::string fn = std::string(graph_path) + ".part." + std::to_string(nparts);
  FILE *fp = fopen(fn.c_str(), "w");
  if (!fp) return cm_fail(CM_ERR_IO, "file: %s, mode: w: %s", fn.c_str(), strerror(errno));
  for (int32_t i = 0; i < nvtxs; ++i) fprintf(fp, "%d\n", part[i]);
  int bad = ferror(fp);
  fclose(fp);
  return bad ? cm_fail(CM_ERR_IO, "write_partition: write error on %s", fn.c_str()) : CM_OK;
}

extern "C" int64_t cm_edge_cut(const cm_graph *g, const int32_t *part) {
  if (!g || !part) return -1;
  int64_t cut = 0;
  for (int32_t v = 0; v < g->nvtxs; ++v)
    for (int32_t j = g->xadj[v]; j < g->xadj[v + 1]; ++j)
      if (part[v] != part[g->adjncy[j]]) cut += g->adjwgt ? g->adjwgt[j] : 1;
  return cut / 2;
}

extern "C" double cm_imbalance(const cm_graph *g, int32_t nparts, const int32_t *part) {
  if (!g || !part || nparts <= 0) return -1.0;
  std::vector<int64_t> pw(nparts, 0);
  int64_t tot = 0;
  for (int32_t v = 0; v < g->nvtxs; ++v) {
    int64_t w = g->vwgt ? g->vwgt[v] : 1;
    if (part[v] >= 0 && part[v] < nparts) pw[part[v]] += w;
    tot += w;
  }
  int64_t mx = *std::max_element(pw.begin(), pw.end());
  return tot > 0 ? (double)mx * nparts / (double)tot : 0.0;
}
