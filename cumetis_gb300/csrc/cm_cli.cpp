// cm_cli.cpp -- the `cuMetis <graph> <k>` command (cuMetis.cu:3874-3920) on
// top of the C ABI only.
//
//   cuMetis <graph> <k> [--seed S] [--device D] [--coarsen-to N] [--passes P]
//                       [--lex-ties] [--no-write]
//   cuMetis convert <matrix.mtx> [<out.graph>]
//
// A <graph> ending in .mtx is read as a MatrixMarket matrix (the pattern of
// A + A^T without the diagonal).  `convert` writes that graph as a METIS file,
// by default <matrix>.graph -- the reference's mtx_to_graph builds this name
// without a terminating NUL, which garbles it.
//
// Reads a METIS .graph file, partitions it into k parts (cm_part_graph),
// prints the reference's report lines (timings, edge cut) plus the imbalance,
// and writes <graph>.part.<k> (one part id per line), which the reference has
// commented out (cu:3909).  Exit status 0 on success, 2 on bad usage, 1 on
// any library error (message on stderr) -- the reference exits -2 on IO
// errors only.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cm.h"

static int usage(const char *argv0) {
  std::fprintf(stderr,
               "usage: %s <graph> <k> [--seed S] [--device D] [--coarsen-to N] [--passes P] [--lex-ties] "
               "[--no-write]\n       %s convert <matrix.mtx> [<out.graph>]\n",
               argv0, argv0);
  return 2;
}

static bool ends_with(const char *s, const char *suffix) {
  const size_t n = std::strlen(s), k = std::strlen(suffix);
  return n >= k && std::strcmp(s + n - k, suffix) == 0;
}

static int read_input(const char *path, cm_graph *g) {
  return ends_with(path, ".mtx") ? cm_read_mtx(path, g) : cm_read_graph(path, g);
}

static int convert(int argc, char **argv) {
  if (argc < 3 || argc > 4) return usage(argv[0]);
  const char *in = argv[2];
  std::string out = argc == 4 ? std::string(argv[3]) : std::string(in);
  if (argc == 3) {
    if (ends_with(in, ".mtx")) out.resize(out.size() - 4);
    out += ".graph";
  }
  cm_graph g{};
  if (cm_read_mtx(in, &g) != CM_OK || cm_write_graph(out.c_str(), &g) != CM_OK) {
    std::fprintf(stderr, "%s\n", cm_last_error());
    cm_graph_free(&g);
    return 1;
  }
  std::printf("%s: %d vertices, %lld edges\n", out.c_str(), g.nvtxs, (long long)(g.nedges / 2));
  cm_graph_free(&g);
  return 0;
}

int main(int argc, char **argv) {
  if (argc >= 2 && !std::strcmp(argv[1], "convert")) return convert(argc, argv);
  if (argc < 3) return usage(argv[0]);
  const char *path = argv[1];
  const int k = std::atoi(argv[2]);
  if (k < 1) return usage(argv[0]);
  cm_part_params P;
  cm_part_default_params(&P);
  int device = 0;
  bool write = true;
  for (int i = 3; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--seed") && i + 1 < argc) P.seed = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "--device") && i + 1 < argc) device = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "--coarsen-to") && i + 1 < argc) P.coarsen_to = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "--passes") && i + 1 < argc) P.refine_passes = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "--lex-ties")) P.match_mode = CM_MATCH_HEM;
    else if (!std::strcmp(argv[i], "--no-write")) write = false;
    else return usage(argv[0]);
  }
  cm_graph g{};
  if (read_input(path, &g) != CM_OK) {
    std::fprintf(stderr, "%s\n", cm_last_error());
    return 1;
  }
  cm_ctx *ctx = nullptr;
  if (cm_ctx_create(device, &ctx) != CM_OK) {
    std::fprintf(stderr, "%s\n", cm_last_error());
    cm_graph_free(&g);
    return 1;
  }
  std::vector<int32_t> part(g.nvtxs > 0 ? g.nvtxs : 1);
  int32_t objval = 0;
  cm_part_stats st{};
  const int rc = cm_part_graph(ctx, g.nvtxs, g.xadj, g.adjncy, g.vwgt, g.adjwgt, k, nullptr, nullptr, &objval,
                               part.data(), &P, &st);
  if (rc != CM_OK) {
    std::fprintf(stderr, "%s\n", cm_last_error());
    cm_ctx_destroy(ctx);
    cm_graph_free(&g);
    return 1;
  }
  std::printf("Graph: %s \nVertex: %d Edge: %lld\n", path, g.nvtxs, (long long)g.nedges);
  std::printf("cuMetis-Partition-end\n");
  std::printf("cuMetis_Partition_time= %lf     ms\n", st.total_ms);
  std::printf("------Coarsen_time=          %lf     ms\n", st.coarsen_ms);
  std::printf("------Init_time=             %lf     ms\n", st.init_ms);
  std::printf("------Uncoarsen_time=        %lf     ms\n", st.uncoarsen_ms);
  std::printf("------------------------------------------\n");
  std::printf("Levels=                      %d (coarsest %d vertices)\n", st.levels, st.coarsest_nvtxs);
  std::printf("Initial-cut=                 %d\n", st.initial_cut);
  std::printf("Refinement-moves=            %lld\n", (long long)st.moves);
  std::printf("Edge-cut=                    %lld\n", (long long)cm_edge_cut(&g, part.data()));
  std::printf("Imbalance=                   %.4f\n", cm_imbalance(&g, k, part.data()));
  int out = 0;
  if (write && cm_write_partition(path, k, g.nvtxs, part.data()) != CM_OK) {
    std::fprintf(stderr, "%s\n", cm_last_error());
    out = 1;
  }
  cm_ctx_destroy(ctx);
  cm_graph_free(&g);
  return out;
}
