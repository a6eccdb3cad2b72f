// Greedy element colouring used to order the scatter: no two elements of one
// colour share a node, so a colour can add its element matrices into the CSR
// values without atomics and the per-entry summation order is fixed.
//
// The algorithm is element_coloring! of src/MeshModificationModule.jl:1329-1365
// over the node -> element map of src/FENodeToFEMapModule.jl:44-74, so the
// colours are the ones a FinEtools user gets from element_coloring(fes, n2e):
//   - an element with no coloured neighbour takes the least-used colour
//     (first minimum);
//   - if every colour is used by a neighbour, a new colour is opened;
//   - otherwise the least-used colour not used by a neighbour is taken.
#include <cstdint>
#include <limits>
#include <vector>

#include "fegpu_internal.h"

namespace fegpu {

int64_t greedy_element_coloring(int64_t nelem, int nne, const int32_t *conn0,
                                int64_t nnodes, std::vector<int64_t> &colors) {
  // node -> elements, elements in increasing order (CSR)
  std::vector<int64_t> ptr(nnodes + 1, 0);
  for (int64_t i = 0; i < nelem * nne; ++i) ptr[conn0[i] + 1]++;
  for (int64_t n = 0; n < nnodes; ++n) ptr[n + 1] += ptr[n];
  std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
  std::vector<int64_t> adj(static_cast<size_t>(nelem) * nne);
  for (int64_t e = 0; e < nelem; ++e)
    for (int a = 0; a < nne; ++a) adj[fill[conn0[e * nne + a]]++] = e;

  colors.assign(nelem, 0);
  std::vector<int64_t> counts(1, 0), used(1, 0);
  for (int64_t e = 0; e < nelem; ++e) {
    std::fill(used.begin(), used.end(), 0);
    int64_t total = 0;
    for (int a = 0; a < nne; ++a) {
      const int32_t n = conn0[e * nne + a];
      for (int64_t q = ptr[n]; q < ptr[n + 1]; ++q) {
        const int64_t c = colors[adj[q]];
        if (c > 0) {
          used[c - 1]++;
          total++;
        }
      }
    }
    const int64_t ncol = static_cast<int64_t>(counts.size());
    int64_t pick = -1;
    if (total == 0) {
      pick = 0;
      for (int64_t c = 1; c < ncol; ++c)
        if (counts[c] < counts[pick]) pick = c;
    } else {
      bool any_free = false;
      for (int64_t c = 0; c < ncol; ++c)
        if (used[c] == 0) {
          any_free = true;
          break;
        }
      if (!any_free) {
        counts.push_back(0);
        used.push_back(0);
        pick = ncol;
      } else {
        int64_t best = std::numeric_limits<int64_t>::max();
        for (int64_t c = 0; c < ncol; ++c)
          if (used[c] == 0 && best > counts[c]) {
            best = counts[c];
            pick = c;
          }
      }
    }
    colors[e] = pick + 1;
    counts[pick]++;
  }
  return static_cast<int64_t>(counts.size());
}

}  // namespace fegpu
