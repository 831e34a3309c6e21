// cm_initpart.cpp -- initial partition of the coarsest graph on the host:
// multilevel recursive bisection, restating cuMetis_initialpartition
// (cuMetis.cu:3091-3108) and everything under it:
//   cuMetis_rbbisection / cuMetis_mlevel_rbbisection   cu:3046-3061, 2964-3028
//   cuMetis_cpu_mlevelbisect                            cu:2806-2828
//   cuMetis_cpu_coarsen, cuMetis_cpu_match,
//   cuMetis_cpu_create_cgraph                           cu:1854-1874, 830-887, 737-825
//   cuMetis_cpu_growbisection                           cu:2536-2660
//   cuMetis_compute_cpu_2wayparam, _2way_bal,
//   cuMetis_bndvertex_2way_bal, cuMetis_cpu_2way_refine cu:1895-1945, 2328-2338, 2241-2325, 2343-2530
//   cuMetis_2way_project, cuMetis_cpu_refinement        cu:2690-2763, 2769-2800
//   cuMetis_splitgraph                                  cu:2858-2957
//   the max-priority queue                              cu:1968-2237
//
// The steps, their order, the float/double arithmetic of every threshold and
// the random stream are kept exactly, so that the same coarsest graph gives
// the same partition as the reference.  The reference draws from the C
// library's rand() without seeding it (glibc's default seed 1); the library
// keeps no global state, so the stream is regenerated here from glibc's
// published additive-feedback generator (random(3), TYPE_3: degree 31,
// separation 3, seeded through the Park-Miller minimal standard generator).
// Memory is owned by std::vector; the reference's arena allocator is not
// needed.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <memory>
#include <vector>

#include "cm.h"
#include "cm_internal.h"

namespace cm {
namespace {

// glibc random(): r[0] = seed; r[i] = 16807 r[i-1] mod (2^31 - 1) for
// i < 31; r[i] = r[i-31] for i in 31..33; then r[i] = r[i-31] + r[i-3]
// (mod 2^32); the k-th output is r[k + 344] >> 1.
class LibcRand {
 public:
  explicit LibcRand(uint32_t seed) {
    int32_t s = (int32_t)seed;
    if (s == 0) s = 1;
    r_[0] = (uint32_t)s;
    int32_t prev = s;
    for (int i = 1; i < 31; ++i) {
      const int32_t hi = prev / 127773, lo = prev % 127773;
      int32_t w = 16807 * lo - 2836 * hi;
      if (w < 0) w += 2147483647;
      r_[i] = (uint32_t)w;
      prev = w;
    }
    for (int i = 31; i < 34; ++i) r_[i] = r_[i - 31];
    pos_ = 34;
    for (int i = 34; i < 344; ++i) step();
  }
  int next() { return (int)(step() >> 1); }

 private:
  uint32_t step() {
    const uint32_t v = r_[(pos_ - 31) % 34] + r_[(pos_ - 3) % 34];
    r_[pos_ % 34] = v;
    ++pos_;
    return v;
  }
  uint32_t r_[34];
  uint64_t pos_;
};

struct Admin {
  int threshold = 200;      // cuMetis_set_graph_admin, cu:380-381
  int iteration_num = 10;
  int maxvwgt = 0;
  float ubfactor = 1.03f;   // the ubvec argument is ignored (cu:370-394)
  float part_balance[2] = {0.f, 0.f};
  LibcRand rng;
  explicit Admin(uint32_t seed) : rng(seed) {}
  int randinrange(int max) { return rng.next() % max; }
};

struct HGraph {
  int n = 0, m = 0;
  std::vector<int> xadj, adjncy, adjwgt, vwgt, label, cmap;
  std::vector<int> where, id, ed, bndptr, bndlist;
  int pwgts[2] = {0, 0};
  int tvwgt = 0;
  float tvwgt_rev = 0.f;
  int mincut = -1, nbnd = -1;
  std::unique_ptr<HGraph> coarser;
  HGraph *finer = nullptr;

  void set_tvwgt() {  // cuMetis_set_graph_tvwgt, cu:440-452
    int s = 0;
    for (int i = 0; i < n; ++i) s += vwgt[i];
    tvwgt = s;
    tvwgt_rev = 1.0f / (float)(tvwgt > 0 ? tvwgt : 1);
  }
  void alloc_2way() {  // cuMetis_allocate_cpu_2waymem, cu:1880-1890
    where.assign(n, 0);
    id.assign(n, 0);
    ed.assign(n, 0);
    bndptr.assign(n, 0);
    bndlist.assign(n, 0);
  }
};

inline void listinsert(int &nb, int *list, int *lptr, int i) {
  list[nb] = i;
  lptr[i] = nb++;
}
inline void listdelete(int &nb, int *list, int *lptr, int i) {
  list[lptr[i]] = list[--nb];
  lptr[list[nb]] = lptr[i];
  lptr[i] = -1;
}

// cuMetis_int_randarrayofp, cu:639-668.
void randarrayofp(Admin &a, int n, int *p, int nshuffles, bool init) {
  if (init)
    for (int i = 0; i < n; ++i) p[i] = i;
  if (n < 10) {
    for (int i = 0; i < n; ++i) {
      const int v = a.randinrange(n), u = a.randinrange(n);
      std::swap(p[v], p[u]);
    }
  } else {
    for (int i = 0; i < nshuffles; ++i) {
      const int v = a.randinrange(n - 3), u = a.randinrange(n - 3);
      std::swap(p[v + 0], p[u + 2]);
      std::swap(p[v + 1], p[u + 3]);
      std::swap(p[v + 2], p[u + 0]);
      std::swap(p[v + 3], p[u + 1]);
    }
  }
}

// Max-priority queue with float keys and a locator per node (cu:1968-2237).
class Queue {
 public:
  // Heap slots at or beyond the current size are never read, so only the
  // locators are initialised.
  explicit Queue(int maxnodes)
      : heap_(new KV[maxnodes > 0 ? maxnodes : 1]), loc_(new int[maxnodes > 0 ? maxnodes : 1]) {
    std::fill(loc_.get(), loc_.get() + maxnodes, -1);
  }
  void insert(int node, int key) {
    const float k = (float)key;
    long i = nn_++;
    while (i > 0) {
      const long j = (i - 1) >> 1;
      if (k > heap_[j].key) {
        heap_[i] = heap_[j];
        loc_[heap_[i].val] = i;
        i = j;
      } else {
        break;
      }
    }
    heap_[i] = {k, node};
    loc_[node] = i;
  }
  int top() {
    if (nn_ == 0) return -1;
    nn_--;
    const int vtx = heap_[0].val;
    loc_[vtx] = -1;
    long i = nn_;
    if (i > 0) {
      const float key = heap_[i].key;
      const int node = heap_[i].val;
      i = 0;
      long j;
      while ((j = 2 * i + 1) < nn_) {
        if (heap_[j].key > key) {
          if (j + 1 < nn_ && heap_[j + 1].key > heap_[j].key) j = j + 1;
          heap_[i] = heap_[j];
          loc_[heap_[i].val] = i;
          i = j;
        } else if (j + 1 < nn_ && heap_[j + 1].key > key) {
          j = j + 1;
          heap_[i] = heap_[j];
          loc_[heap_[i].val] = i;
          i = j;
        } else {
          break;
        }
      }
      heap_[i] = {key, node};
      loc_[node] = i;
    }
    return vtx;
  }
  void remove(int node) {
    long i = loc_[node];
    loc_[node] = -1;
    if (--nn_ > 0 && heap_[nn_].val != node) {
      node = heap_[nn_].val;
      const float newkey = heap_[nn_].key, oldkey = heap_[i].key;
      sift(i, node, newkey, oldkey);
    }
  }
  void update(int node, int newkey_i) {
    const float newkey = (float)newkey_i;
    const long i = loc_[node];
    sift(i, node, newkey, heap_[i].key);
  }
  void reset() {
    for (long i = nn_ - 1; i >= 0; --i) loc_[heap_[i].val] = -1;
    nn_ = 0;
  }

 private:
  struct KV {
    float key;
    int val;
  };
  // Moves node (new key) from slot i up or down (cu:2125-2170, 2177-2227).
  void sift(long i, int node, float newkey, float oldkey) {
    if (newkey > oldkey) {
      while (i > 0) {
        const long j = (i - 1) >> 1;
        if (newkey > heap_[j].key) {
          heap_[i] = heap_[j];
          loc_[heap_[i].val] = i;
          i = j;
        } else {
          break;
        }
      }
    } else {
      long j;
      while ((j = (i << 1) + 1) < nn_) {
        if (heap_[j].key > newkey) {
          if (j + 1 < nn_ && heap_[j + 1].key > heap_[j].key) j++;
          heap_[i] = heap_[j];
          loc_[heap_[i].val] = i;
          i = j;
        } else if (j + 1 < nn_ && heap_[j + 1].key > newkey) {
          j++;
          heap_[i] = heap_[j];
          loc_[heap_[i].val] = i;
          i = j;
        } else {
          break;
        }
      }
    }
    heap_[i] = {newkey, node};
    loc_[node] = i;
  }
  std::unique_ptr<KV[]> heap_;
  std::unique_ptr<int[]> loc_;  // heap slot of each node, -1 when absent
  long nn_ = 0;
};

// cuMetis_cpu_match + cuMetis_cpu_create_cgraph (cu:830-887, 737-825).
void cpu_match(Admin &a, HGraph &g) {
  const int n = g.n;
  std::vector<int> match(n, -1), perm(n), tperm(n), d(n);
  randarrayofp(a, n, tperm.data(), n / 8, true);
  const int aved = (int)(0.7 * (g.xadj[n] / n));
  for (int i = 0; i < n; ++i) {
    const int dg = g.xadj[i + 1] - g.xadj[i];
    d[i] = dg > aved ? aved : dg;
  }
  {  // cuMetis_matching_sort: counting sort by d, in tperm order
    std::vector<int> counts(aved + 2, 0);
    for (int i = 0; i < n; ++i) counts[d[i]]++;
    for (int i = 1; i < aved + 1; ++i) counts[i] += counts[i - 1];
    for (int i = aved + 1; i > 0; --i) counts[i] = counts[i - 1];
    counts[0] = 0;
    for (int ii = 0; ii < n; ++ii) {
      const int i = tperm[ii];
      perm[counts[d[i]]++] = i;
    }
  }
  int cn = 0;
  for (int pi = 0; pi < n; ++pi) {
    const int i = perm[pi];
    if (match[i] != -1) continue;
    int maxidx = i, maxwgt = -1;
    for (int j = g.xadj[i]; j < g.xadj[i + 1]; ++j) {
      const int k = g.adjncy[j];
      if (match[k] == -1 && maxwgt < g.adjwgt[j] && g.vwgt[i] + g.vwgt[k] <= a.maxvwgt) {
        maxidx = k;
        maxwgt = g.adjwgt[j];
      }
      if (maxidx == i && 3 * g.vwgt[i] < a.maxvwgt) maxidx = -1;
    }
    if (maxidx != -1) {
      g.cmap[i] = g.cmap[maxidx] = cn++;
      match[i] = maxidx;
      match[maxidx] = i;
    }
  }
  cn = 0;
  for (int i = 0; i < n; ++i) {
    if (match[i] == -1) {
      match[i] = i;
      g.cmap[i] = cn++;
    } else if (i <= match[i]) {
      g.cmap[i] = g.cmap[match[i]] = cn++;
    }
  }
  // contraction: rows in first-seen order via a hash table over coarse ids
  auto cg = std::make_unique<HGraph>();
  cg->n = cn;
  cg->xadj.assign(cn + 1, 0);
  cg->vwgt.assign(cn, 0);
  cg->adjncy.assign(g.m, 0);
  cg->adjwgt.assign(g.m, 0);
  std::vector<int> htable(cn, -1);
  int c = 0, cne = 0;
  for (int v = 0; v < n; ++v) {
    const int u = match[v];
    if (u < v) continue;
    int *rk = cg->adjncy.data() + cne, *rw = cg->adjwgt.data() + cne;
    int ne = 0;
    cg->vwgt[c] = g.vwgt[v];
    for (int j = g.xadj[v]; j < g.xadj[v + 1]; ++j) {
      const int k = g.cmap[g.adjncy[j]];
      const int mm = htable[k];
      if (mm == -1) {
        rk[ne] = k;
        rw[ne] = g.adjwgt[j];
        htable[k] = ne++;
      } else {
        rw[mm] += g.adjwgt[j];
      }
    }
    if (v != u) {
      cg->vwgt[c] += g.vwgt[u];
      for (int j = g.xadj[u]; j < g.xadj[u + 1]; ++j) {
        const int k = g.cmap[g.adjncy[j]];
        const int mm = htable[k];
        if (mm == -1) {
          rk[ne] = k;
          rw[ne] = g.adjwgt[j];
          htable[k] = ne++;
        } else {
          rw[mm] += g.adjwgt[j];
        }
      }
      const int j = htable[c];
      if (j != -1) {
        rk[j] = rk[--ne];
        rw[j] = rw[ne];
        htable[c] = -1;
      }
    }
    for (int j = 0; j < ne; ++j) htable[rk[j]] = -1;
    cne += ne;
    cg->xadj[++c] = cne;
  }
  cg->m = cne;
  cg->adjncy.resize(cne);
  cg->adjwgt.resize(cne);
  cg->set_tvwgt();
  cg->finer = &g;
  g.coarser = std::move(cg);
}

// cuMetis_cpu_coarsen, cu:1854-1874.
HGraph *cpu_coarsen(Admin &a, HGraph *g) {
  a.maxvwgt = (int)(1.5 * g->tvwgt / a.threshold);
  do {
    if (g->cmap.empty()) g->cmap.assign(g->n, 0);
    cpu_match(a, *g);
    g = g->coarser.get();
  } while (g->n > a.threshold && g->n < 0.75 * g->finer->n && g->m > g->n / 2);
  return g;
}

// cuMetis_compute_cpu_2wayparam, cu:1895-1945.
void compute_2wayparam(HGraph &g) {
  g.pwgts[0] = g.pwgts[1] = 0;
  for (int i = 0; i < g.n; ++i) g.bndptr[i] = -1;
  for (int i = 0; i < g.n; ++i) g.pwgts[g.where[i]] += g.vwgt[i];
  int nbnd = 0, mincut = 0;
  for (int i = 0; i < g.n; ++i) {
    const int istart = g.xadj[i], iend = g.xadj[i + 1], me = g.where[i];
    int tid = 0, ted = 0;
    for (int j = istart; j < iend; ++j) {
      if (me == g.where[g.adjncy[j]]) tid += g.adjwgt[j];
      else ted += g.adjwgt[j];
    }
    g.id[i] = tid;
    g.ed[i] = ted;
    if (ted > 0 || istart == iend) {
      listinsert(nbnd, g.bndlist.data(), g.bndptr.data(), i);
      mincut += ted;
    }
  }
  g.mincut = mincut / 2;
  g.nbnd = nbnd;
}

// cuMetis_compute_cpu_imbal with nparts = 2, cu:1950-1965.
float compute_imbal(const Admin &a, const HGraph &g) {
  float mx = -1.0f;
  for (int j = 0; j < 2; ++j) {
    const float cur = g.pwgts[j] * a.part_balance[j] - a.ubfactor;
    if (cur > mx) mx = cur;
  }
  return mx;
}

// Moves boundary vertices from the heavy side until the target is met
// (cuMetis_bndvertex_2way_bal, cu:2241-2325).
void bndvertex_2way_bal(Admin &a, HGraph &g, const float *ntpwgts) {
  const int n = g.n;
  int *where = g.where.data(), *id = g.id.data(), *ed = g.ed.data(), *bndptr = g.bndptr.data(),
      *bndlist = g.bndlist.data(), *pwgts = g.pwgts;
  std::vector<int> moved(n, -1), perm(n);
  int tpwgts[2];
  tpwgts[0] = g.tvwgt * ntpwgts[0];
  tpwgts[1] = g.tvwgt - tpwgts[0];
  const int mindiff = std::abs(tpwgts[0] - pwgts[0]);
  const int from = pwgts[0] < tpwgts[0] ? 1 : 0;
  const int to = (from + 1) % 2;
  Queue q(n);
  int nbnd = g.nbnd;
  randarrayofp(a, nbnd, perm.data(), nbnd / 5, true);
  for (int ii = 0; ii < nbnd; ++ii) {
    const int i = perm[ii];
    if (where[bndlist[i]] == from && g.vwgt[bndlist[i]] <= mindiff)
      q.insert(bndlist[i], ed[bndlist[i]] - id[bndlist[i]]);
  }
  int mincut = g.mincut;
  for (int nswaps = 0; nswaps < n; ++nswaps) {
    const int higain = q.top();
    if (higain == -1) break;
    if (pwgts[to] + g.vwgt[higain] > tpwgts[to]) break;
    mincut -= ed[higain] - id[higain];
    pwgts[to] += g.vwgt[higain];
    pwgts[from] -= g.vwgt[higain];
    where[higain] = to;
    moved[higain] = nswaps;
    std::swap(id[higain], ed[higain]);
    if (ed[higain] == 0 && g.xadj[higain] < g.xadj[higain + 1]) listdelete(nbnd, bndlist, bndptr, higain);
    for (int j = g.xadj[higain]; j < g.xadj[higain + 1]; ++j) {
      const int k = g.adjncy[j];
      const int kwgt = to == where[k] ? g.adjwgt[j] : -g.adjwgt[j];
      id[k] += kwgt;
      ed[k] -= kwgt;
      if (bndptr[k] != -1) {
        if (ed[k] == 0) {
          listdelete(nbnd, bndlist, bndptr, k);
          if (moved[k] == -1 && where[k] == from && g.vwgt[k] <= mindiff) q.remove(k);
        } else if (moved[k] == -1 && where[k] == from && g.vwgt[k] <= mindiff) {
          q.update(k, ed[k] - id[k]);
        }
      } else if (ed[k] > 0) {
        listinsert(nbnd, bndlist, bndptr, k);
        if (moved[k] == -1 && where[k] == from && g.vwgt[k] <= mindiff) q.insert(k, ed[k] - id[k]);
      }
    }
  }
  g.mincut = mincut;
  g.nbnd = nbnd;
}

// cuMetis_2way_bal, cu:2328-2338.
void two_way_bal(Admin &a, HGraph &g, const float *ntpwgts) {
  if (compute_imbal(a, g) <= 0) return;
  if (std::fabs(ntpwgts[0] * g.tvwgt - g.pwgts[0]) < 3 * g.tvwgt / g.n) return;
  bndvertex_2way_bal(a, g, ntpwgts);
}

// Fiduccia-Mattheyses passes with rollback to the best prefix
// (cuMetis_cpu_2way_refine, cu:2343-2530).
void two_way_refine(Admin &a, HGraph &g, const float *ntpwgts, int iteration_num) {
  const int n = g.n;
  int *where = g.where.data(), *id = g.id.data(), *ed = g.ed.data(), *bndptr = g.bndptr.data(),
      *bndlist = g.bndlist.data(), *pwgts = g.pwgts;
  std::vector<int> moved(n, -1);
  std::unique_ptr<int[]> swaps(new int[n > 0 ? n : 1]), perm(new int[n > 0 ? n : 1]);  // written before read
  int tpwgts[2];
  tpwgts[0] = g.tvwgt * ntpwgts[0];
  tpwgts[1] = g.tvwgt - tpwgts[0];
  const int limit = (int)std::min(std::max(0.01 * n, 15.0), 100.0);
  const int avgvwgt = std::min((pwgts[0] + pwgts[1]) / 20, 2 * (pwgts[0] + pwgts[1]) / n);
  Queue queues[2] = {Queue(n), Queue(n)};
  const int origdiff = std::abs(tpwgts[0] - pwgts[0]);
  for (int pass = 0; pass < iteration_num; ++pass) {
    queues[0].reset();
    queues[1].reset();
    int mincutorder = -1;
    int newcut, mincut, initcut;
    newcut = mincut = initcut = g.mincut;
    int mindiff = std::abs(tpwgts[0] - pwgts[0]);
    int nbnd = g.nbnd;
    randarrayofp(a, nbnd, perm.get(), nbnd, true);
    for (int ii = 0; ii < nbnd; ++ii) {
      const int i = perm[ii];
      queues[where[bndlist[i]]].insert(bndlist[i], ed[bndlist[i]] - id[bndlist[i]]);
    }
    int nswaps;
    for (nswaps = 0; nswaps < n; ++nswaps) {
      const int from = tpwgts[0] - pwgts[0] < tpwgts[1] - pwgts[1] ? 0 : 1;
      const int to = (from + 1) % 2;
      const int higain = queues[from].top();
      if (higain == -1) break;
      newcut -= ed[higain] - id[higain];
      pwgts[to] += g.vwgt[higain];
      pwgts[from] -= g.vwgt[higain];
      if ((newcut < mincut && std::abs(tpwgts[0] - pwgts[0]) <= origdiff + avgvwgt) ||
          (newcut == mincut && std::abs(tpwgts[0] - pwgts[0]) < mindiff)) {
        mincut = newcut;
        mindiff = std::abs(tpwgts[0] - pwgts[0]);
        mincutorder = nswaps;
      } else if (nswaps - mincutorder > limit) {
        newcut += ed[higain] - id[higain];
        pwgts[from] += g.vwgt[higain];
        pwgts[to] -= g.vwgt[higain];
        break;
      }
      where[higain] = to;
      moved[higain] = nswaps;
      swaps[nswaps] = higain;
      std::swap(id[higain], ed[higain]);
      if (ed[higain] == 0 && g.xadj[higain] < g.xadj[higain + 1]) listdelete(nbnd, bndlist, bndptr, higain);
      for (int j = g.xadj[higain]; j < g.xadj[higain + 1]; ++j) {
        const int k = g.adjncy[j];
        const int kwgt = to == where[k] ? g.adjwgt[j] : -g.adjwgt[j];
        id[k] += kwgt;
        ed[k] -= kwgt;
        if (bndptr[k] != -1) {
          if (ed[k] == 0) {
            listdelete(nbnd, bndlist, bndptr, k);
            if (moved[k] == -1) queues[where[k]].remove(k);
          } else if (moved[k] == -1) {
            queues[where[k]].update(k, ed[k] - id[k]);
          }
        } else if (ed[k] > 0) {
          listinsert(nbnd, bndlist, bndptr, k);
          if (moved[k] == -1) queues[where[k]].insert(k, ed[k] - id[k]);
        }
      }
    }
    for (int i = 0; i < nswaps; ++i) moved[swaps[i]] = -1;
    for (nswaps--; nswaps > mincutorder; nswaps--) {  // roll back past the best prefix
      const int higain = swaps[nswaps];
      const int to = where[higain] = (where[higain] + 1) % 2;
      std::swap(id[higain], ed[higain]);
      if (ed[higain] == 0 && bndptr[higain] != -1 && g.xadj[higain] < g.xadj[higain + 1])
        listdelete(nbnd, bndlist, bndptr, higain);
      else if (ed[higain] > 0 && bndptr[higain] == -1)
        listinsert(nbnd, bndlist, bndptr, higain);
      pwgts[to] += g.vwgt[higain];
      pwgts[(to + 1) % 2] -= g.vwgt[higain];
      for (int j = g.xadj[higain]; j < g.xadj[higain + 1]; ++j) {
        const int k = g.adjncy[j];
        const int kwgt = to == where[k] ? g.adjwgt[j] : -g.adjwgt[j];
        id[k] += kwgt;
        ed[k] -= kwgt;
        if (bndptr[k] != -1 && ed[k] == 0) listdelete(nbnd, bndlist, bndptr, k);
        if (bndptr[k] == -1 && ed[k] > 0) listinsert(nbnd, bndlist, bndptr, k);
      }
    }
    g.mincut = mincut;
    g.nbnd = nbnd;
    if (mincutorder <= 0 || mincut == initcut) break;
  }
}

// Untraversed vertices as a Fenwick tree of 0/1 flags: kth(k) is the k-th
// (0-based) untraversed vertex in id order, the vertex the reference finds by
// a linear scan (cu:2588-2598) -- the same choice in O(log n), so graphs with
// many components (isolated vertices restart the search once each) do not
// turn the region growing quadratic.
class Untraversed {
 public:
  explicit Untraversed(int n) : n_(n), t_(n + 1, 0), log_(1) {
    for (int i = 1; i <= n; ++i) {
      t_[i] += 1;
      const int j = i + (i & -i);
      if (j <= n) t_[j] += t_[i];
    }
    while ((1 << log_) <= n) ++log_;
  }
  void take(int v) {
    for (int i = v + 1; i <= n_; i += i & -i) t_[i] -= 1;
  }
  int kth(int k) const {  // smallest v with (untraversed in [0, v]) == k + 1
    int pos = 0, rem = k + 1;
    for (int b = log_; b >= 0; --b) {
      const int nx = pos + (1 << b);
      if (nx <= n_ && t_[nx] < rem) {
        pos = nx;
        rem -= t_[nx];
      }
    }
    return pos;  // 0-based vertex id
  }

 private:
  int n_;
  std::vector<int> t_;
  int log_;
};

// Breadth-first region growing from random seeds, niparts tries, each
// balanced and refined; the best cut wins (cuMetis_cpu_growbisection,
// cu:2536-2660).
void grow_bisection(Admin &a, HGraph &g, const float *ntpwgts, int niparts) {
  const int n = g.n;
  g.alloc_2way();
  std::vector<int> bestwhere(n), queue(n), tra(n);
  const int onemaxpwgt = a.ubfactor * g.tvwgt * ntpwgts[1];
  const int oneminpwgt = (1.0 / a.ubfactor) * g.tvwgt * ntpwgts[1];
  int bestcut = 0;
  for (int iter = 0; iter < niparts; ++iter) {
    for (int i = 0; i < n; ++i) {
      g.where[i] = 1;
      tra[i] = 0;
    }
    int pw[2];
    pw[1] = g.tvwgt;
    pw[0] = 0;
    Untraversed un(n);
    queue[0] = a.randinrange(n);
    tra[queue[0]] = 1;
    un.take(queue[0]);
    int first = 0, last = 1, nleft = n - 1, dd = 0;
    for (;;) {
      if (first == last) {
        if (nleft == 0 || dd) break;
        const int i = un.kth(a.randinrange(nleft));
        queue[0] = i;
        tra[i] = 1;
        un.take(i);
        first = 0;
        last = 1;
        nleft--;
      }
      const int i = queue[first++];
      if (pw[0] > 0 && pw[1] - g.vwgt[i] < oneminpwgt) {
        dd = 1;
        continue;
      }
      g.where[i] = 0;
      pw[0] += g.vwgt[i];
      pw[1] -= g.vwgt[i];
      if (pw[1] <= onemaxpwgt) break;
      dd = 0;
      for (int j = g.xadj[i]; j < g.xadj[i + 1]; ++j) {
        const int k = g.adjncy[j];
        if (tra[k] == 0) {
          queue[last++] = k;
          tra[k] = 1;
          un.take(k);
          nleft--;
        }
      }
    }
    compute_2wayparam(g);
    two_way_bal(a, g, ntpwgts);
    two_way_refine(a, g, ntpwgts, a.iteration_num);
    if (iter == 0 || bestcut > g.mincut) {
      bestcut = g.mincut;
      bestwhere = g.where;
      if (bestcut == 0) break;
    }
  }
  g.mincut = bestcut;
  g.where = bestwhere;
}

// cuMetis_2way_project, cu:2690-2763: the finer graph takes the coarse
// sides; vertices of interior coarse vertices skip the neighbour scan.
void two_way_project(HGraph &g) {
  HGraph &cg = *g.coarser;
  g.alloc_2way();
  for (int i = 0; i < g.n; ++i) g.bndptr[i] = -1;
  for (int i = 0; i < g.n; ++i) {
    const int j = g.cmap[i];
    g.where[i] = cg.where[j];
    g.cmap[i] = cg.bndptr[j];
  }
  int nbnd = 0;
  for (int i = 0; i < g.n; ++i) {
    const int istart = g.xadj[i], iend = g.xadj[i + 1];
    int tid = 0, ted = 0;
    if (g.cmap[i] == -1) {
      for (int j = istart; j < iend; ++j) tid += g.adjwgt[j];
    } else {
      const int me = g.where[i];
      for (int j = istart; j < iend; ++j) {
        if (me == g.where[g.adjncy[j]]) tid += g.adjwgt[j];
        else ted += g.adjwgt[j];
      }
    }
    g.id[i] = tid;
    g.ed[i] = ted;
    if (ted > 0 || istart == iend) listinsert(nbnd, g.bndlist.data(), g.bndptr.data(), i);
  }
  g.mincut = cg.mincut;
  g.nbnd = nbnd;
  g.pwgts[0] = cg.pwgts[0];
  g.pwgts[1] = cg.pwgts[1];
  g.coarser.reset();
}

// cuMetis_cpu_refinement, cu:2769-2800.
void cpu_refinement(Admin &a, HGraph *orig, HGraph *g, const float *tpwgts) {
  compute_2wayparam(*g);
  for (;;) {
    two_way_bal(a, *g, tpwgts);
    two_way_refine(a, *g, tpwgts, a.iteration_num);
    if (g == orig) break;
    g = g->finer;
    two_way_project(*g);
  }
}

// cuMetis_cpu_mlevelbisect, cu:2806-2828.
int mlevel_bisect(Admin &a, HGraph &g, const float *tpwgts) {
  for (int i = 0; i < 2; ++i) a.part_balance[i] = g.tvwgt_rev / tpwgts[i];
  HGraph *cg = cpu_coarsen(a, &g);
  grow_bisection(a, *cg, tpwgts, 5);
  cpu_refinement(a, &g, cg, tpwgts);
  return g.mincut;
}

// cuMetis_splitgraph, cu:2858-2957: interior vertices copy their rows, boundary
// vertices keep only same-side entries; ids renamed per side.
void split_graph(const HGraph &g, std::unique_ptr<HGraph> &lg, std::unique_ptr<HGraph> &rg) {
  const int n = g.n;
  std::vector<int> rename(n);
  int snv[2] = {0, 0}, sne[2] = {0, 0};
  for (int i = 0; i < n; ++i) {
    const int k = g.where[i];
    rename[i] = snv[k]++;
    sne[k] += g.xadj[i + 1] - g.xadj[i];
  }
  HGraph *s[2];
  lg = std::make_unique<HGraph>();
  rg = std::make_unique<HGraph>();
  s[0] = lg.get();
  s[1] = rg.get();
  for (int p = 0; p < 2; ++p) {
    s[p]->n = snv[p];
    s[p]->xadj.assign(snv[p] + 1, 0);
    s[p]->vwgt.assign(snv[p], 0);
    s[p]->adjncy.assign(sne[p], 0);
    s[p]->adjwgt.assign(sne[p], 0);
    s[p]->label.assign(snv[p], 0);
  }
  snv[0] = snv[1] = sne[0] = sne[1] = 0;
  for (int i = 0; i < n; ++i) {
    const int p = g.where[i];
    const int istart = g.xadj[i], iend = g.xadj[i + 1];
    if (g.bndptr[i] == -1) {
      for (int j = istart; j < iend; ++j) {
        s[p]->adjncy[sne[p] + j - istart] = g.adjncy[j];
        s[p]->adjwgt[sne[p] + j - istart] = g.adjwgt[j];
      }
      sne[p] += iend - istart;
    } else {
      int l = sne[p];
      for (int j = istart; j < iend; ++j) {
        const int k = g.adjncy[j];
        if (g.where[k] == p) {
          s[p]->adjncy[l] = k;
          s[p]->adjwgt[l++] = g.adjwgt[j];
        }
      }
      sne[p] = l;
    }
    s[p]->vwgt[snv[p]] = g.vwgt[i];
    s[p]->label[snv[p]] = g.label[i];
    s[p]->xadj[++snv[p]] = sne[p];
  }
  for (int p = 0; p < 2; ++p) {
    for (int i = 0; i < s[p]->xadj[snv[p]]; ++i) s[p]->adjncy[i] = rename[s[p]->adjncy[i]];
    s[p]->m = sne[p];
    s[p]->adjncy.resize(sne[p]);
    s[p]->adjwgt.resize(sne[p]);
    s[p]->set_tvwgt();
  }
}

// cuMetis_mlevel_rbbisection, cu:2964-3028.
int mlevel_rbbisection(Admin &a, std::unique_ptr<HGraph> g, int nparts, int *part, float *tpwgts, int fpart) {
  if (g->n == 0) return 0;  // the reference prints a warning and returns 0
  float tpwgts2[2];
  float s = 0;
  for (int i = 0; i < (nparts >> 1); ++i) s += tpwgts[i];
  tpwgts2[0] = s;
  tpwgts2[1] = 1.0 - tpwgts2[0];
  int objval = mlevel_bisect(a, *g, tpwgts2);
  for (int i = 0; i < g->n; ++i) part[g->label[i]] = g->where[i] + fpart;
  std::unique_ptr<HGraph> lg, rg;
  if (nparts > 2) split_graph(*g, lg, rg);
  g.reset();
  float wsum = 0;
  for (int i = 0; i < (nparts >> 1); ++i) wsum += tpwgts[i];
  {
    const float f = 1.0 / wsum;
    for (int i = 0; i < (nparts >> 1); ++i) tpwgts[i] *= f;
    const float f2 = 1.0 / (1.0 - wsum);
    for (int i = 0; i < nparts - (nparts >> 1); ++i) tpwgts[(nparts >> 1) + i] *= f2;
  }
  if (nparts > 3) {
    objval += mlevel_rbbisection(a, std::move(lg), nparts >> 1, part, tpwgts, fpart);
    objval += mlevel_rbbisection(a, std::move(rg), nparts - (nparts >> 1), part, tpwgts + (nparts >> 1),
                                 fpart + (nparts >> 1));
  } else if (nparts == 3) {
    lg.reset();
    objval += mlevel_rbbisection(a, std::move(rg), nparts - (nparts >> 1), part, tpwgts + (nparts >> 1),
                                 fpart + (nparts >> 1));
  }
  return objval;
}

}  // namespace

int initial_partition(const cm_graph *g, int32_t nparts, uint32_t seed, int32_t *part, int32_t *objval) {
  auto hg = std::make_unique<HGraph>();
  const int n = g->nvtxs;
  hg->n = n;
  hg->m = (int)g->nedges;
  hg->xadj.assign(g->xadj, g->xadj + n + 1);
  hg->adjncy.assign(g->adjncy, g->adjncy + g->nedges);
  if (g->adjwgt) hg->adjwgt.assign(g->adjwgt, g->adjwgt + g->nedges);
  else hg->adjwgt.assign(g->nedges, 1);
  if (g->vwgt) hg->vwgt.assign(g->vwgt, g->vwgt + n);
  else hg->vwgt.assign(n, 1);
  hg->label.resize(n);
  for (int i = 0; i < n; ++i) hg->label[i] = i;
  hg->set_tvwgt();
  Admin a(seed);
  std::vector<float> tpwgts(nparts, 1.0f / nparts);
  const int obj = mlevel_rbbisection(a, std::move(hg), nparts, part, tpwgts.data(), 0);
  if (objval) *objval = obj;
  return CM_OK;
}

}  // namespace cm

extern "C" int cm_initial_partition(const cm_graph *g, int32_t nparts, uint32_t seed, int32_t *part,
                                    int32_t *objval) {
  if (!g || !part || nparts < 1) return ::cm_fail(CM_ERR_INVALID, "cm_initial_partition: bad arguments");
  if (g->nvtxs < 0 || g->nedges < 0 || (g->nvtxs > 0 && (!g->xadj || (g->nedges > 0 && !g->adjncy))))
    return ::cm_fail(CM_ERR_INVALID, "cm_initial_partition: bad graph");
  if (g->nvtxs == 0) {
    if (objval) *objval = 0;
    return CM_OK;
  }
  if (nparts == 1) {
    for (int i = 0; i < g->nvtxs; ++i) part[i] = 0;
    if (objval) *objval = 0;
    return CM_OK;
  }
  try {
    return cm::initial_partition(g, nparts, seed, part, objval);
  } catch (const std::bad_alloc &) {
    return ::cm_fail(CM_ERR_NOMEM, "cm_initial_partition: out of host memory");
  }
}
