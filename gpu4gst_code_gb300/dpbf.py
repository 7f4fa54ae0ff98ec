"""Host-side mirror of the reference's DPBF call surface, over libgst.

Names, arguments and results follow the reference so a caller (and the
tests) read like the reference's own harness (rucgraph/test_gpu.h:79-291):

  toCSR(input_graph)                      csr_graph.hpp:29-65
  graph_v_of_v_idealID_DPBF_non_overlapped_group_sets_gpu(range)
                                          test_gpu.h:19-44
  DPBF_GPU(csr, groups, group_graph, input_graph, ...)
                                          DPQ.cuh:57, DPQ.cu:501-768
  graph_hash_of_mixed_weighted_sum_of_ec(tree)
                                          graph_hash_of_mixed_weighted_sum_of_nw_ec.h:58-87
  this_is_a_feasible_solution_gpu(tree, group_graph, group_vertices)
                                          test_gpu.h:45-77

Data types: graph_v_of_v_idealID is a list (one entry per vertex) of
sorted (neighbour, weight) pairs; the group graph has one row per vertex
plus one per group vertex, group vertex g adjacent to its members;
graph_hash_of_mixed_weighted is a vertex -> {neighbour: weight} mapping.
All solving happens in libgst's CUDA kernels.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import native

inf = 10000  # the reference's node.cost default (DPQ.cuh:48); not used by the solver


@dataclass
class CSR_graph:
    """toCSR's result (csr_graph.hpp:11-26): all_pointer / all_edge /
    all_edge_weight, weights truncated from double to int as at :46. The
    device copy (a native.Graph) is created on first use and kept."""

    all_pointer: np.ndarray
    all_edge: np.ndarray
    all_edge_weight: np.ndarray
    V: int
    E_all: int
    _device: native.Graph | None = field(default=None, repr=False)

    def device(self) -> native.Graph:
        if self._device is None:
            self._device = native.Graph(self.all_pointer, self.all_edge, self.all_edge_weight)
        return self._device

    def free(self) -> None:
        """The caller frees the CSR arrays (test_gpu.h:281-283)."""
        if self._device is not None:
            self._device.close()
            self._device = None


def toCSR(graph) -> CSR_graph:
    V = len(graph)
    ptr = np.zeros(V + 1, np.int32)
    edges, weights = [], []
    for i, row in enumerate(graph):
        for (u, w) in row:
            edges.append(int(u))
            weights.append(int(w))  # double -> int truncation (csr_graph.hpp:46)
        ptr[i + 1] = len(edges)
    return CSR_graph(ptr, np.asarray(edges, np.int32), np.asarray(weights, np.int32), V, len(edges))


@dataclass
class non_overlapped_group_sets:
    non_overlapped_group_sets_IDs_pointer_host: list
    non_overlapped_group_sets_IDs: list
    length: int


def graph_v_of_v_idealID_DPBF_non_overlapped_group_sets_gpu(group_sets_ID_range: int) -> non_overlapped_group_sets:
    """For each non-empty mask i, every j in [1, range) with i & j == 0, as
    one flat list plus offsets (test_gpu.h:19-44). libgst enumerates the
    splits on the device and does not need it; it is kept for callers
    that pass it to DPBF_GPU."""
    ptr = [0] * (group_sets_ID_range + 3)
    ids = []
    for i in range(1, group_sets_ID_range + 1):
        ptr[i] = len(ids)
        for j in range(1, group_sets_ID_range):
            if i & j == 0:
                ids.append(j)
    ptr[group_sets_ID_range + 1] = len(ids)
    return non_overlapped_group_sets(ptr, ids, len(ids))


class graph_hash_of_mixed_weighted:
    """Vertex -> {neighbour: weight} with vertex weights (graph_hash_of_mixed_weighted.h:20)."""

    def __init__(self):
        self.hash_of_vectors: dict[int, dict[int, float]] = {}
        self.vertex_weight: dict[int, float] = {}

    def add_vertex(self, v: int, weight: float = 0.0) -> None:
        self.hash_of_vectors.setdefault(int(v), {})
        self.vertex_weight[int(v)] = weight

    def add_edge(self, a: int, b: int, w: float) -> None:
        self.hash_of_vectors.setdefault(int(a), {})[int(b)] = w
        self.hash_of_vectors.setdefault(int(b), {})[int(a)] = w

    def edges(self):
        for a, nb in self.hash_of_vectors.items():
            for b, w in nb.items():
                if a < b:
                    yield a, b, w


def graph_hash_of_mixed_weighted_sum_of_ec(g: graph_hash_of_mixed_weighted) -> int:
    s = 0
    for _, _, w in g.edges():
        s = s + int(w)  # int accumulation as sum_of_nw_ec.h:60-85
    return s


def _components(g: graph_hash_of_mixed_weighted) -> int:
    seen, n = set(), 0
    for s in g.hash_of_vectors:
        if s in seen:
            continue
        n += 1
        stack = [s]
        seen.add(s)
        while stack:
            x = stack.pop()
            for y in g.hash_of_vectors[x]:
                if y not in seen:
                    seen.add(y)
                    stack.append(y)
    return n


def _contains(graph, a: int, b: int) -> bool:
    return any(int(u) == b for (u, _) in graph[a])


def this_is_a_feasible_solution_gpu(solu: graph_hash_of_mixed_weighted, group_graph, group_vertices) -> bool:
    """Connected, and every group has a member in the tree (test_gpu.h:45-77)."""
    if _components(solu) != 1:
        return False
    for g in group_vertices:
        if not any(_contains(group_graph, g, v) for v in solu.hash_of_vectors):
            return False
    return True


def DPBF_GPU(graph: CSR_graph, cumpulsory_group_vertices, group_graph, input_graph=None, *, pointer1=None,
             upper_bound: int = 0, use_graph: bool = False):
    """One exact GST query on the GPU (DPBF_GPU, DPQ.cu:501-768).

    Group g of `cumpulsory_group_vertices` has the members listed in
    group_graph[g] (DPQ.cu:22-34); bit order is the iteration order of the
    given collection. Returns (solution_tree, real_cost, processed, rt):
    an empty tree and real_cost None when no tree exists (DPQ.cu:620-624),
    processed = states written (the *pointer1 counter), rt = growth-loop
    seconds (*rt). `input_graph` is accepted for signature parity; edge
    weights come from the CSR, as the reference's backtrack reads the same
    truncated weights (DPQ.cu:749)."""
    groups = [[int(u) for (u, _) in group_graph[g]] for g in cumpulsory_group_vertices]
    res = graph.device().solve(groups, upper_bound=upper_bound, use_graph=use_graph)
    tree = graph_hash_of_mixed_weighted()
    if res.status != native.Status.OK:
        return tree, None, res.states, res.times_ms[1] / 1e3
    for v in res.vertices:
        tree.add_vertex(int(v), 0)
    for u, v, w in res.edges:
        tree.add_edge(int(u), int(v), int(w))
    if pointer1 is not None:
        pointer1[0] += res.states
    return tree, res.cost, res.states, res.times_ms[1] / 1e3


def group_graph_from_groups(V: int, groups) -> tuple[list, list]:
    """Builds the reference's group graph (size V+k, group vertex V+g
    adjacent to its members, graph_hash_of_mixed_weighted_to_graph_v_of_v_idealID)
    and the group-vertex list {V, ..., V+k-1}."""
    gg = [[] for _ in range(V + len(groups))]
    for g, mem in enumerate(groups):
        for m in mem:
            gg[V + g].append((int(m), 1.0))
            gg[int(m)].append((V + g, 1.0))
    for row in gg:
        row.sort()
    return gg, [V + g for g in range(len(groups))]


def csr_to_graph_v_of_v(row_ptr, col, w) -> list:
    """CSR -> graph_v_of_v_idealID (sorted (neighbour, weight) rows)."""
    V = len(row_ptr) - 1
    return [sorted((int(col[e]), float(w[e])) for e in range(int(row_ptr[v]), int(row_ptr[v + 1]))) for v in range(V)]
