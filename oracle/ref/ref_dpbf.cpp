// C entry points around the reference's own CPU group-Steiner-tree solvers,
// compiled from the reference's unmodified headers (oracle/build_ref.sh).
//
// TEST INFRASTRUCTURE ONLY: the resulting oracle/_ref/libref_dpbf.so is used
// by tests/ to validate the C restatement (oracle/dpbf_oracle.c) and to make
// the golden fixtures. Nothing in the product links or loads it.
//
// Solvers wrapped:
//   ref_dpbf_only_ec   -> graph_v_of_v_idealID_DPBF_only_ec
//                         (rucgraph/graph_v_of_v_idealID_DPBF_only_ec.h:133)
//   ref_pruned_dp_pp   -> graph_v_of_v_idealID_PrunedDPPlusPlus
//                         (rucgraph/graph_v_of_v_idealID_PrunedDPPlusPlus.h:497)
//
// The DPBF header adds a missing tree's cost INT_MAX to a finite cost
// (graph_v_of_v_idealID_DPBF_only_ec.h:278-293), a signed overflow that
// stores a negative cost and later dereferences a missing state; PrunedDP++
// computes best_cost * 2 / 3 with best_cost = INT_MAX
// (graph_v_of_v_idealID_PrunedDPPlusPlus.h:511,915), which overflows the
// same way and makes it miss feasible trees. Both solvers (and the
// shortest-path / MST helpers PrunedDP++ includes) are therefore compiled
// inside a namespace whose `std::numeric_limits<int>` reports INT_MAX/2 as
// max(): every `inf` they derive becomes 2^30-1, the sums no longer
// overflow, and an absent tree can never win a merge. No line of the
// reference is edited.
//
// Instances reach the solvers in the reference's own data model:
//   input_graph  graph_v_of_v_idealID with sorted adjacency (add_edge),
//                double weights truncated to int by the solvers themselves;
//   group_graph  graph_v_of_v_idealID of size V+k, group g has ID V+g and an
//                edge to each member (as graph_hash_of_mixed_weighted_to_
//                graph_v_of_v_idealID builds it);
//   cumpulsory_group_vertices = {V, ..., V+k-1}.
// Infeasible instances are detected here first, because both solvers call
// exit() when no tree exists.

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <limits>
#include <list>
#include <queue>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <boost/heap/fibonacci_heap.hpp>
#include <boost/heap/pairing_heap.hpp>
#include <graph_v_of_v_idealID/graph_v_of_v_idealID.h>
#include <graph_hash_of_mixed_weighted/graph_hash_of_mixed_weighted.h>
#include <graph_hash_of_mixed_weighted_sum_of_nw_ec.h>

namespace gst_ref_dpbf {
namespace std {
using namespace ::std;
template <class T>
struct numeric_limits : ::std::numeric_limits<T> {};
template <>
struct numeric_limits<int> : ::std::numeric_limits<int> {
  static constexpr int max() noexcept { return INT_MAX / 2; }
};
}  // namespace std
#include <graph_v_of_v_idealID_DPBF_only_ec.h>
#include <graph_v_of_v_idealID_PrunedDPPlusPlus.h>
}  // namespace gst_ref_dpbf

namespace {

struct Instance {
  graph_v_of_v_idealID input_graph;
  graph_v_of_v_idealID group_graph;
  std::unordered_set<int> groups;
};

bool build_instance(int V, const int64_t* row_ptr, const int32_t* col, const double* w, int k,
                    const int32_t* group_ptr, const int32_t* members, Instance& inst) {
  inst.input_graph.assign(V, {});
  for (int u = 0; u < V; ++u)
    for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
      int v = col[e];
      if (v < 0 || v >= V) return false;
      if (u < v) graph_v_of_v_idealID_add_edge(inst.input_graph, u, v, w[e]);
    }
  inst.group_graph.assign(V + k, {});
  for (int g = 0; g < k; ++g) {
    inst.groups.insert(V + g);
    for (int32_t i = group_ptr[g]; i < group_ptr[g + 1]; ++i) {
      int m = members[i];
      if (m < 0 || m >= V) return false;
      graph_v_of_v_idealID_add_edge(inst.group_graph, m, V + g, 1);
    }
  }
  return true;
}

// True when one connected component holds a member of every group.
bool feasible(const Instance& inst, int V, int k, const int32_t* group_ptr, const int32_t* members) {
  std::vector<int> comp(V, -1);
  int ncomp = 0;
  for (int s = 0; s < V; ++s) {
    if (comp[s] >= 0) continue;
    std::vector<int> stack{s};
    comp[s] = ncomp;
    while (!stack.empty()) {
      int u = stack.back();
      stack.pop_back();
      for (auto& e : inst.input_graph[u])
        if (comp[e.first] < 0) {
          comp[e.first] = ncomp;
          stack.push_back(e.first);
        }
    }
    ++ncomp;
  }
  std::vector<int> hits(ncomp, 0);
  for (int g = 0; g < k; ++g) {
    std::unordered_set<int> seen;
    for (int32_t i = group_ptr[g]; i < group_ptr[g + 1]; ++i) seen.insert(comp[members[i]]);
    for (int c : seen) hits[c]++;
  }
  for (int c = 0; c < ncomp; ++c)
    if (hits[c] == k) return true;
  return false;
}

int export_tree(graph_hash_of_mixed_weighted& tree, int32_t* out_nv, int32_t* out_vertices,
                int32_t* out_ne, int32_t* out_edges, int32_t cap) {
  int nv = 0, ne = 0;
  for (auto& kv : tree.hash_of_vectors) {
    int u = kv.first;
    if (nv < cap) out_vertices[nv] = u;
    ++nv;
    for (auto& a : tree.adj_v_and_ec(u)) {
      if (u < a.first) {
        if (ne < cap) {
          out_edges[3 * ne + 0] = u;
          out_edges[3 * ne + 1] = a.first;
          out_edges[3 * ne + 2] = static_cast<int32_t>(a.second);
        }
        ++ne;
      }
    }
  }
  *out_nv = nv;
  *out_ne = ne;
  return (nv > cap || ne > cap) ? -2 : 0;
}

}  // namespace

extern "C" {

// Returns 0 on success (tree exported), 1 if no feasible tree exists,
// -1 for malformed input, -2 if the tree does not fit in `cap`.
// *out_cost = graph_hash_of_mixed_weighted_sum_of_ec(tree), the figure the
// reference's harness reports (rucgraph/test_gpu.h:215).
int ref_dpbf_only_ec(int32_t V, const int64_t* row_ptr, const int32_t* col, const double* w,
                     int32_t k, const int32_t* group_ptr, const int32_t* members, int32_t* out_cost,
                     int32_t* out_nv, int32_t* out_vertices, int32_t* out_ne, int32_t* out_edges,
                     int32_t cap) {
  if (k < 1 || k >= 20 || V < 1) return -1;
  Instance inst;
  if (!build_instance(V, row_ptr, col, w, k, group_ptr, members, inst)) return -1;
  if (!feasible(inst, V, k, group_ptr, members)) return 1;
  int ram_mb = 0;
  graph_hash_of_mixed_weighted tree = gst_ref_dpbf::graph_v_of_v_idealID_DPBF_only_ec(
      inst.input_graph, inst.group_graph, inst.groups, ram_mb);
  *out_cost = graph_hash_of_mixed_weighted_sum_of_ec(tree);
  return export_tree(tree, out_nv, out_vertices, out_ne, out_edges, cap);
}

// Same contract, using the reference's PrunedDP++ solver with
// maximum_return_app_ratio = 1 (exact), as rucgraph/test_gpu.h:165 calls it.
int ref_pruned_dp_pp(int32_t V, const int64_t* row_ptr, const int32_t* col, const double* w,
                     int32_t k, const int32_t* group_ptr, const int32_t* members, int32_t* out_cost,
                     int32_t* out_nv, int32_t* out_vertices, int32_t* out_ne, int32_t* out_edges,
                     int32_t cap) {
  if (k < 1 || k >= 15 || V < 1) return -1;
  Instance inst;
  if (!build_instance(V, row_ptr, col, w, k, group_ptr, members, inst)) return -1;
  if (!feasible(inst, V, k, group_ptr, members)) return 1;
  int ram_mb = 0, counter = 0;
  graph_hash_of_mixed_weighted tree = gst_ref_dpbf::graph_v_of_v_idealID_PrunedDPPlusPlus(
      inst.input_graph, inst.group_graph, inst.groups, 1, ram_mb, &counter);
  *out_cost = graph_hash_of_mixed_weighted_sum_of_ec(tree);
  return export_tree(tree, out_nv, out_vertices, out_ne, out_edges, cap);
}

}  // extern "C"
