// Test-side stand-in for the reference's rucgraph/DPQ.cuh and the types it
// pulls in (csr_graph.hpp, graph_v_of_v_idealID.h,
// graph_hash_of_mixed_weighted.h), for hosts without the reference
// checkout. It declares only what include/gst_dpbf_dropin.hpp and the
// harness in dropin_main.cpp use, with the reference's names, field names
// and argument meanings:
//   node / non_overlapped_group_sets  DPQ.cuh:44-56 (scratch records the
//                                     drop-in accepts and ignores)
//   CSR_graph                         csr_graph.hpp:11-24 (all_pointer,
//                                     all_edge, all_edge_weight in managed
//                                     memory; V, E_all)
//   graph_v_of_v_idealID              graph_v_of_v_idealID.h:50 (adjacency
//                                     lists of (neighbour, weight))
//   graph_hash_of_mixed_weighted      vertex weights + adjacency with the
//                                     add_vertex / add_edge helpers
// Everything here is test infrastructure; the product is include/.
#pragma once
#include <cuda_runtime.h>

#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

typedef struct non_overlapped_group_sets {
  std::vector<int> non_overlapped_group_sets_IDs_pointer_host, non_overlapped_group_sets_IDs;
  int length = 0;
} non_overlapped_group_sets;

typedef struct node {
  int update = 0;
  int type = 0;
  int cost = 10000;
  int u = 0;
  int p1 = 0, p2 = 0;
} node;

typedef std::vector<std::vector<std::pair<int, double>>> graph_v_of_v_idealID;

class CSR_graph {
 public:
  int *all_pointer = nullptr, *all_edge = nullptr, *all_edge_weight = nullptr;
  int E_all = 0, V = 0;
};

// toCSR's upload (csr_graph.hpp:29-65): weights truncated to int, arrays in
// managed memory.
inline CSR_graph toCSR(const graph_v_of_v_idealID &graph) {
  CSR_graph a;
  a.V = (int)graph.size();
  std::vector<int> ptr(a.V + 1, 0), edge, weight;
  for (int i = 0; i < a.V; ++i) {
    ptr[i] = (int)edge.size();
    for (auto &e : graph[i]) {
      edge.push_back(e.first);
      weight.push_back((int)e.second);
    }
  }
  ptr[a.V] = (int)edge.size();
  a.E_all = (int)edge.size();
  cudaMallocManaged(&a.all_pointer, (a.V + 1) * sizeof(int));
  cudaMallocManaged(&a.all_edge, (a.E_all > 0 ? a.E_all : 1) * sizeof(int));
  cudaMallocManaged(&a.all_edge_weight, (a.E_all > 0 ? a.E_all : 1) * sizeof(int));
  cudaMemcpy(a.all_pointer, ptr.data(), (a.V + 1) * sizeof(int), cudaMemcpyHostToDevice);
  if (a.E_all) {
    cudaMemcpy(a.all_edge, edge.data(), a.E_all * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(a.all_edge_weight, weight.data(), a.E_all * sizeof(int), cudaMemcpyHostToDevice);
  }
  return a;
}

class graph_hash_of_mixed_weighted {
 public:
  std::unordered_map<int, double> hash_of_vectors;                         // vertex -> weight
  std::unordered_map<int, std::unordered_map<int, double>> hash_of_hashs;  // adjacency with weights
};

inline void graph_hash_of_mixed_weighted_add_vertex(graph_hash_of_mixed_weighted &g, int v, double w) {
  g.hash_of_vectors[v] = w;
  g.hash_of_hashs[v];
}

inline void graph_hash_of_mixed_weighted_add_edge(graph_hash_of_mixed_weighted &g, int a, int b, double w) {
  graph_hash_of_mixed_weighted_add_vertex(g, a, g.hash_of_vectors.count(a) ? g.hash_of_vectors[a] : 0);
  graph_hash_of_mixed_weighted_add_vertex(g, b, g.hash_of_vectors.count(b) ? g.hash_of_vectors[b] : 0);
  g.hash_of_hashs[a][b] = w;
  g.hash_of_hashs[b][a] = w;
}
