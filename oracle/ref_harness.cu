// ref_harness.cu -- include-harness around the unmodified cuMetis sources.
// TEST INFRASTRUCTURE ONLY: oracle/build.py (build_ref) compiles it, with the
// reference tree on the include path, into oracle/_ref/libref.so (never
// committed, never shipped); tests/golden/make_golden.py calls it to record
// the reference's own CPU coarsening outputs as golden fixtures.
//
// Exposed (extern "C"), wrapping reference functions:
//   ref_srand               srand(seed) for the reference's rand() stream
//   ref_cpu_match_contract  cuMetis_cpu_match (cuMetis.cu:830), which runs
//                           cuMetis_cpu_create_cgraph (cu:737)
//   ref_cpu_contract        cuMetis_cpu_create_cgraph on a caller's matching
//   ref_rbbisection         cuMetis_rbbisection (cuMetis.cu:3046), the initial
//                           partition by multilevel recursive bisection
#define main cuMetis_reference_main
#include "cuMetis.cu"
#undef main

namespace {
cuMetis_admin_t *make_admin(int maxvwgt) {
  cuMetis_admin_t *a = (cuMetis_admin_t *)calloc(1, sizeof(cuMetis_admin_t));
  a->maxvwgt = (int *)malloc(sizeof(int));
  a->maxvwgt[0] = maxvwgt;
  a->Coarsen_threshold = 200;
  a->nparts = 2;
  a->mcore = cuMetis_create_mcore(0);  // every request falls back to malloc
  return a;
}

cuMetis_graph_t *make_graph(int n, const int *xadj, const int *adjncy, const int *adjwgt, const int *vwgt) {
  cuMetis_graph_t *g = cuMetis_create_cpu_graph();
  g->nvtxs = n;
  g->nedges = xadj[n];
  g->xadj = const_cast<int *>(xadj);
  g->adjncy = const_cast<int *>(adjncy);
  g->adjwgt = const_cast<int *>(adjwgt);
  g->vwgt = const_cast<int *>(vwgt);
  g->cmap = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  return g;
}

int export_coarse(cuMetis_graph_t *g, int *cmap_out, int *cxadj, int *cvwgt, int *cadjncy, int *cadjwgt,
                  int *cnedges) {
  cuMetis_graph_t *c = g->coarser;
  memcpy(cmap_out, g->cmap, sizeof(int) * g->nvtxs);
  memcpy(cxadj, c->xadj, sizeof(int) * (c->nvtxs + 1));
  memcpy(cvwgt, c->vwgt, sizeof(int) * c->nvtxs);
  memcpy(cadjncy, c->adjncy, sizeof(int) * c->nedges);
  memcpy(cadjwgt, c->adjwgt, sizeof(int) * c->nedges);
  *cnedges = c->nedges;
  return c->nvtxs;
}
}  // namespace

extern "C" void ref_srand(unsigned seed) { srand(seed); }

extern "C" int ref_cpu_match_contract(int n, const int *xadj, const int *adjncy, const int *adjwgt,
                                      const int *vwgt, int maxvwgt, int *cmap_out, int *cxadj, int *cvwgt,
                                      int *cadjncy, int *cadjwgt, int *cnedges) {
  cuMetis_admin_t *a = make_admin(maxvwgt);
  cuMetis_graph_t *g = make_graph(n, xadj, adjncy, adjwgt, vwgt);
  cuMetis_cpu_match(a, g, 1);
  return export_coarse(g, cmap_out, cxadj, cvwgt, cadjncy, cadjwgt, cnedges);
}

// The caller's matching (match[v] = partner or v) is numbered exactly as the
// reference's cuMetis_cpu_match numbers it (cuMetis.cu:873-883): coarse ids
// in increasing order of the pair's smaller vertex.
extern "C" int ref_cpu_contract(int n, const int *xadj, const int *adjncy, const int *adjwgt, const int *vwgt,
                                const int *match, int *cmap_out, int *cxadj, int *cvwgt, int *cadjncy,
                                int *cadjwgt, int *cnedges) {
  cuMetis_admin_t *a = make_admin(1 << 30);
  cuMetis_graph_t *g = make_graph(n, xadj, adjncy, adjwgt, vwgt);
  int cn = 0;
  for (int i = 0; i < n; ++i)
    if (i <= match[i]) g->cmap[i] = g->cmap[match[i]] = cn++;
  cuMetis_cpu_create_cgraph(a, g, cn, const_cast<int *>(match), 1);
  return export_coarse(g, cmap_out, cxadj, cvwgt, cadjncy, cadjwgt, cnedges);
}

// cuMetis_rbbisection frees the graph arrays it is given (cuMetis_free_graph
// in cuMetis_mlevel_rbbisection, cu:3000), so it gets malloc'ed copies.
extern "C" int ref_rbbisection(int n, const int *xadj, const int *adjncy, const int *vwgt, const int *adjwgt,
                               int nparts, int *part, int *objval) {
  int m = xadj[n];
  int *x = (int *)malloc(sizeof(int) * (n + 1)), *a = (int *)malloc(sizeof(int) * (m > 0 ? m : 1));
  int *vw = (int *)malloc(sizeof(int) * (n > 0 ? n : 1)), *aw = (int *)malloc(sizeof(int) * (m > 0 ? m : 1));
  memcpy(x, xadj, sizeof(int) * (n + 1));
  memcpy(a, adjncy, sizeof(int) * m);
  memcpy(vw, vwgt, sizeof(int) * n);
  memcpy(aw, adjwgt, sizeof(int) * m);
  float ub = 1.03f;
  float *tp = (float *)malloc(sizeof(float) * nparts);
  for (int i = 0; i < nparts; ++i) tp[i] = 1.0f / nparts;
  int nv = n, np_ = nparts;
  cuMetis_rbbisection(&nv, x, a, vw, aw, &np_, tp, &ub, objval, part);
  free(tp);
  return 0;
}
