// cm_batch.h -- coarsening many independent graphs level by level in shared
// launches (internal; cm_coarsen_batch and the engine use it).
#pragma once

#include <utility>
#include <vector>

#include "cm_ctx.h"

namespace cm {

// Graphs coarsened together: add() uploads new graphs (their level 0), step()
// runs one level for every active graph -- graphs laid side by side as one
// union per tie order, matched and contracted in one set of launches, then
// split back -- and hands over, with their caller's tag, the graphs whose
// stop rule ended their coarsening.  Everything runs on one context and
// stream; graphs may join between steps.
class BatchCoarsener {
 public:
  // Largest union of one level (int32 CSR).
  static constexpr int64_t kMaxUnionVertices = 400000000, kMaxUnionEntries = 1800000000;
  BatchCoarsener(cm_ctx *ctx, cudaStream_t s);
  ~BatchCoarsener();
  BatchCoarsener(const BatchCoarsener &) = delete;
  BatchCoarsener &operator=(const BatchCoarsener &) = delete;
  // Host graphs; params[i].coarsen_to >= 1.  Graphs without vertices finish
  // at once (into `finished`).
  int add(int32_t count, const cm_graph *graphs, const cm_coarsen_params *params, const int64_t *tags,
          std::vector<std::pair<int64_t, cm_hierarchy *>> &finished);
  int step(std::vector<std::pair<int64_t, cm_hierarchy *>> &finished);
  bool empty() const { return active_.empty(); }
  size_t active() const { return active_.size(); }

 private:
  struct Active {
    int64_t tag = 0;
    cm_coarsen_params p{};
    cm_hierarchy *h = nullptr;
    int64_t row_bound = 0;  // bound of the next expanded row
  };
  int level(const std::vector<int> &grp, std::vector<char> &stop);
  cm_ctx *ctx_;
  cudaStream_t s_;
  std::vector<Active> active_;
};

}  // namespace cm
