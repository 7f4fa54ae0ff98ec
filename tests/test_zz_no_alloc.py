"""gst_group_distances_noalloc against the regular solver.

The allocation-free entry point serves callers that must not allocate
device memory themselves through CUDA (their host framework owns every
device byte through its own pool, or they sit on a path that cannot take
cudaMalloc's implicit synchronisation). It computes each vertex's distance
to one group using a fixed scratch array inside the library.

This test hands it caller-owned device buffers (allocated here by torch, as
a pool-owning host would) and compares its distances, on two calls in a row
with different groups, against the group distances the regular solver
(gst_solve) computes for the same groups in the first wave of its DP, read
through gst_graph_debug_table, and against the CPU oracle's exact table.
Integer distances: equality, no tolerance. It also checks that repeated
calls leave the device's free memory unchanged and that out-of-range
sources and CSR entries are rejected. The file is named so that pytest
collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from gpu4gst_code_gb300 import native
from gpu4gst_code_gb300.native import Status

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.int32)).cuda()


def _noalloc(torch, rp_d, col_d, w_d, V, sources, stream=None, bufs=None):
    src_d = _dev(torch, sources if len(sources) else [0])
    if bufs is None:
        bufs = (torch.empty(V, dtype=torch.int32, device="cuda"), torch.empty(V, dtype=torch.int32, device="cuda"))
    dist_d, pred_d = bufs
    torch.cuda.synchronize()
    st = native.lib().gst_group_distances_noalloc(
        C.c_void_p(rp_d.data_ptr()), C.c_void_p(col_d.data_ptr()), C.c_void_p(w_d.data_ptr()), V,
        col_d.numel(), C.c_void_p(src_d.data_ptr()), len(sources), C.c_void_p(dist_d.data_ptr()), C.c_void_p(pred_d.data_ptr()),
        None if stream is None else C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return Status(st), dist_d.cpu().numpy(), pred_d.cpu().numpy()


def test_noalloc_distances_match_solver_on_two_calls():
    torch = pytest.importorskip("torch")
    g = native.gen_barabasi_albert(30000, 4, 1, 100, 77)
    (gp, mem) = native.gen_groups_zipf_degree(g, 2, 1.2, 5, 500, 78)
    groups = [mem[gp[0]:gp[1]], mem[gp[1]:gp[2]]]

    # the regular path: a k=2 solve grows both single-group columns to
    # their exact distances (wave 1 of the DP)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        res = dg.solve(gp, mem)
        assert res.status == Status.OK
        table = dg.debug_table(2)
    want = [table[:, 1], table[:, 2]]
    # the same distances from the CPU oracle's exact DP table
    exact = oracle.dp_table(g.row_ptr, g.col, g.w, gp, mem)
    for col in (1, 2):
        assert np.array_equal(np.where(exact[:, col] == 2**31 - 1, native.COST_LIMIT, exact[:, col]), want[col - 1])

    rp_d, col_d, w_d = _dev(torch, g.row_ptr), _dev(torch, g.col), _dev(torch, g.w)
    for call in range(2):  # two calls in a row, different groups
        st, dist, pred = _noalloc(torch, rp_d, col_d, w_d, g.V, groups[call])
        assert st == Status.OK
        assert np.array_equal(dist, want[call]), f"call {call}"
        # pred names a CSR entry of the vertex's own row on a shortest path
        src = set(int(x) for x in groups[call])
        for u in range(0, g.V, 97):
            e = int(pred[u])
            if u in src:
                assert e == -1 and dist[u] == 0
            else:
                assert g.row_ptr[u] <= e < g.row_ptr[u + 1]
                assert dist[u] == dist[g.col[e]] + g.w[e]


def test_noalloc_rejects_oversized_graph():
    torch = pytest.importorskip("torch")
    tiny = torch.zeros(4, dtype=torch.int32, device="cuda")
    p = C.c_void_p(tiny.data_ptr())
    st = native.lib().gst_group_distances_noalloc(p, p, p, native.NOALLOC_MAX_VERTICES + 1, 4, p, 1, p, p,
                                                  None)
    assert Status(st) == Status.TOO_LARGE


def test_noalloc_allocates_nothing_and_reports_bad_input():
    """After a first call (which looks up the scratch array's address), two
    more calls leave the device's free memory unchanged; a source or a CSR
    entry out of range is reported as GST_BAD_INPUT; no sources leave every
    vertex unreachable; a call on a side stream gives the default stream's
    distances."""
    torch = pytest.importorskip("torch")
    g = native.gen_barabasi_albert(20000, 4, 1, 100, 81)
    gp, mem = native.gen_groups_uniform(g.V, 1, 7, 82)
    rp_d, col_d, w_d = _dev(torch, g.row_ptr), _dev(torch, g.col), _dev(torch, g.w)
    bufs = (torch.empty(g.V, dtype=torch.int32, device="cuda"), torch.empty(g.V, dtype=torch.int32, device="cuda"))
    st, d0, p0 = _noalloc(torch, rp_d, col_d, w_d, g.V, mem, bufs=bufs)
    assert st == Status.OK
    src_d = _dev(torch, mem)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        st = native.lib().gst_group_distances_noalloc(
            C.c_void_p(rp_d.data_ptr()), C.c_void_p(col_d.data_ptr()), C.c_void_p(w_d.data_ptr()), g.V, g.nnz,
            C.c_void_p(src_d.data_ptr()), len(mem), C.c_void_p(bufs[0].data_ptr()), C.c_void_p(bufs[1].data_ptr()),
            None)
        assert Status(st) == Status.OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0

    # a side stream gives the same distances
    side = torch.cuda.Stream()
    st, d1, _ = _noalloc(torch, rp_d, col_d, w_d, g.V, mem, stream=side)
    assert st == Status.OK and np.array_equal(d1, d0)

    # no sources: every vertex unreachable
    st, d2, p2 = _noalloc(torch, rp_d, col_d, w_d, g.V, [])
    assert st == Status.OK
    assert np.all(d2 == native.COST_LIMIT) and np.all(p2 == -1)

    # a source out of range (checked by the seeding kernel)
    st, _, _ = _noalloc(torch, rp_d, col_d, w_d, g.V, [3, g.V + 5])
    assert st == Status.BAD_INPUT

    # a CSR entry out of range (checked by the round kernel before it is used)
    bad_col = g.col.copy()
    bad_col[len(bad_col) // 2] = g.V + 9
    st, _, _ = _noalloc(torch, rp_d, _dev(torch, bad_col), w_d, g.V, mem)
    assert st == Status.BAD_INPUT

    # the entry point still works after the rejected calls
    st, d3, _ = _noalloc(torch, rp_d, col_d, w_d, g.V, mem)
    assert st == Status.OK and np.array_equal(d3, d0)
