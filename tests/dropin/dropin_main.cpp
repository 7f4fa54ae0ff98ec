// Runs the C++ drop-in DPBF_GPU (include/gst_dpbf_dropin.hpp) the way the
// reference's harness calls it (rucgraph/test_gpu.h:188-223): one CSR per
// instance built by toCSR in managed memory, the host_tree scratch sized
// V x 2^k, DPBF_GPU, then the CSR freed with cudaFree (test_gpu.h:281-283)
// before the next instance is built, so a later toCSR may reuse the freed
// addresses.
//
// Input (argv[1..]): instance files, each
//   V E k
//   E lines "u v w"      (undirected edges)
//   k lines "n m1 ... mn" (group members)
// Output per instance, one line:
//   cost <c> states <n> rt <seconds> vertices <n> v1 .. vn edges <m> u v w ..
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>

#include "DPQ.cuh"
#include "gst_dpbf_dropin.hpp"

int main(int argc, char **argv) {
  for (int f = 1; f < argc; ++f) {
    std::ifstream in(argv[f]);
    int V = 0, E = 0, k = 0;
    in >> V >> E >> k;
    graph_v_of_v_idealID input_graph(V);
    for (int i = 0; i < E; ++i) {
      int u, v, w;
      in >> u >> v >> w;
      input_graph[u].push_back({v, (double)w});
      input_graph[v].push_back({u, (double)w});
    }
    // the group graph: group g is vertex V + g, joined to its members
    // (the reference's to_graph_v_of_v_idealID layout)
    graph_v_of_v_idealID group_graph(V + k);
    std::unordered_set<int> group_vertices;
    for (int g = 0; g < k; ++g) {
      int n;
      in >> n;
      for (int i = 0; i < n; ++i) {
        int m;
        in >> m;
        group_graph[V + g].push_back({m, 1.0});
        group_graph[m].push_back({V + g, 1.0});
      }
      group_vertices.insert(V + g);
    }
    CSR_graph csr = toCSR(input_graph);
    const int width = 1 << k;
    node *host_tree_one_d = new node[(size_t)V * width];
    node **host_tree = new node *[V];
    for (int i = 0; i < V; ++i) host_tree[i] = &host_tree_one_d[(size_t)i * width];
    non_overlapped_group_sets s;
    int cost = -1, pointer1 = 0, c_size[3] = {0, 0, 0};
    double rt = -1;
    graph_hash_of_mixed_weighted tree = DPBF_GPU(host_tree, host_tree_one_d, csr, group_vertices, group_graph,
                                                 input_graph, &pointer1, &cost, nullptr, c_size, s, &rt);
    std::cout << "cost " << cost << " states " << pointer1 << " rt " << rt << " vertices "
              << tree.hash_of_vectors.size();
    for (auto &v : tree.hash_of_vectors) std::cout << " " << v.first;
    int ne = 0;
    for (auto &a : tree.hash_of_hashs)
      for (auto &b : a.second) ne += a.first < b.first;
    std::cout << " edges " << ne;
    for (auto &a : tree.hash_of_hashs)
      for (auto &b : a.second)
        if (a.first < b.first) std::cout << " " << a.first << " " << b.first << " " << (int)b.second;
    std::cout << std::endl;
    delete[] host_tree;
    delete[] host_tree_one_d;
    cudaFree(csr.all_edge);
    cudaFree(csr.all_pointer);
    cudaFree(csr.all_edge_weight);
  }
  gst_dropin::release_all();
  return 0;
}
