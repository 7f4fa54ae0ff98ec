"""GPU parity tests: libgst (CUDA, through the C ABI) against the oracle.

Costs must match the reference CPU DPBF bit-exactly (integer arithmetic:
no tolerance), every returned tree must be a valid group Steiner tree of
exactly that cost, and on small instances the whole V x 2^k state table
must equal the oracle's exact fixpoint."""
import numpy as np
import pytest

import oracle
from conftest import load_edge_cases, load_fixture, make_instance
from gpu4gst_code_gb300 import dpbf, native
from gpu4gst_code_gb300.native import Status

pytestmark = pytest.mark.gpu

ORACLE_INF = 2**31 - 1


def _check(g_rp, g_col, g_w, gp, mem, res, cost):
    assert res.status == Status.OK
    assert res.cost == cost
    err = oracle.check_tree(g_rp, g_col, g_w, gp, mem, res.vertices, res.edges, res.cost)
    assert err is None, err


def test_fixture_simple_iterative():
    rp, col, w, gp, mem, cost = load_fixture()
    with native.Graph(rp, col, w) as g:
        res = g.solve(gp, mem)
        _check(rp, col, w, gp, mem, res, cost)
        assert cost == 16


MODES = [pytest.param(False, id="host-loop"), pytest.param(True, id="cuda-graph")]


@pytest.mark.parametrize("use_graph", MODES)
def test_golden_costs_bit_exact(golden, use_graph):
    graphs = {}
    for case in golden["cases"]:
        g, gp, mem = make_instance(case)
        key = tuple(case["graph"])
        if key not in graphs:
            graphs[key] = native.Graph(g.row_ptr, g.col, g.w)
        res = graphs[key].solve(gp, mem, use_graph=use_graph)
        _check(g.row_ptr, g.col, g.w, gp, mem, res, case["dpbf"])
    for dg in graphs.values():
        dg.close()


@pytest.mark.parametrize("use_graph", MODES)
def test_edge_cases(use_graph):
    for name, c in load_edge_cases().items():
        with native.Graph(c["rp"], c["col"], c["w"]) as g:
            res = g.solve(c["gp"], c["mem"], use_graph=use_graph)
            if int(c["cost"]) < 0:
                assert res.status == Status.INFEASIBLE, name
                assert res.cost == -1 and len(res.vertices) == 0
            else:
                _check(c["rp"], c["col"], c["w"], c["gp"], c["mem"], res, int(c["cost"]))


def test_empty_group_is_infeasible():
    rp, col, w, gp, mem, _ = load_fixture()
    gp2 = np.concatenate([gp, [gp[-1]]]).astype(np.int32)  # a 5th group with no members
    with native.Graph(rp, col, w) as g:
        assert g.solve(gp2, mem).status == Status.INFEASIBLE


@pytest.mark.parametrize("use_graph", MODES)
@pytest.mark.parametrize("idx", [0, 1, 2, 3, 200, 201, 202, 203, 204, 206])
def test_full_state_table_matches_oracle(golden, idx, use_graph):
    case = golden["cases"][idx]
    g, gp, mem = make_instance(case)
    if g.V > 6000:
        pytest.skip("table check kept to small graphs")
    k = len(gp) - 1
    want = oracle.dp_table(g.row_ptr, g.col, g.w, gp, mem)
    want = np.where(want == ORACLE_INF, native.COST_LIMIT, want)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        res = dg.solve(gp, mem, use_graph=use_graph)
        assert res.status == Status.OK
        got = dg.debug_table(k)
    # the last wave is merged but not grown (growth cannot lower the optimum)
    full = (1 << k) - 1
    assert np.array_equal(got[:, 1:full], want[:, 1:full])
    assert got[:, full].min() == want[:, full].min() == case["dpbf"]
    assert np.all(got[:, full] >= want[:, full])


@pytest.mark.parametrize("use_graph", MODES)
def test_upper_bound_pruning_is_exact(golden, use_graph):
    for case in golden["cases"][::5] + golden["cases"][200:]:
        g, gp, mem = make_instance(case)
        opt = case["dpbf"]
        with native.Graph(g.row_ptr, g.col, g.w) as dg:
            for ub in (opt, opt + 1, opt + 50, 2 * opt + 1):
                if ub <= 0:
                    continue
                res = dg.solve(gp, mem, upper_bound=ub, use_graph=use_graph)
                _check(g.row_ptr, g.col, g.w, gp, mem, res, opt)
            if opt > 1:
                # a bound below the optimum prunes every full tree
                res = dg.solve(gp, mem, upper_bound=opt - 1, use_graph=use_graph)
                assert res.status == Status.INFEASIBLE


@pytest.mark.parametrize("use_graph", MODES)
def test_refined_bound_is_exact(golden, use_graph):
    """refine_bound lowers the bound between waves from partial trees; the
    cost stays exact with and without a starting bound, and the final bound
    is a feasible cost (>= the optimum)."""
    for case in golden["cases"][::7] + golden["cases"][200:]:
        g, gp, mem = make_instance(case)
        opt = case["dpbf"]
        with native.Graph(g.row_ptr, g.col, g.w) as dg:
            for ub in (0, opt, 2 * opt + 1):
                res = dg.solve(gp, mem, upper_bound=ub, refine_bound=True, use_graph=use_graph)
                _check(g.row_ptr, g.col, g.w, gp, mem, res, opt)
                assert res.upper_bound == 0 or res.upper_bound >= opt
                if ub:
                    assert res.upper_bound <= ub


def test_hub_rows_use_block_path():
    # star: hub 0 joined to 600 leaves (degree > 64 -> one CTA per row)
    V = 601
    edges = [(0, i, 1 + (i * 7) % 13) for i in range(1, V)] + [(i, i + 1, 50) for i in range(1, V - 1)]
    rows = [[] for _ in range(V)]
    for a, b, ww in edges:
        rows[a].append((b, ww))
        rows[b].append((a, ww))
    rp, col, w = [0], [], []
    for r in rows:
        r.sort()
        col += [x for x, _ in r]
        w += [y for _, y in r]
        rp.append(len(col))
    groups = [[5, 300], [77], [450, 12], [599], [3, 4]]
    gp, mem = native.groups_to_csr(groups)
    want = oracle.dpbf(rp, col, w, gp, mem)
    with native.Graph(rp, col, w) as g:
        res = g.solve(gp, mem)
        _check(rp, col, w, gp, mem, res, want.cost)


@pytest.mark.parametrize("k", [1, 2, 5, 8, 10])
def test_many_group_counts(k):
    g = native.gen_random_connected(700, 2500, 1, 60, 40 + k)
    gp, mem = native.gen_groups_uniform(700, k, 3, 50 + k)
    want = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        res = dg.solve(gp, mem)
        _check(g.row_ptr, g.col, g.w, gp, mem, res, want.cost)


@pytest.mark.parametrize("k", [9, 10, 11, 12])
def test_wide_masks_merge_per_state(k):
    """k = 9 and 10 merge a vertex per thread with the tour bounds
    (k_merge_vertex; at k = 10 the path table is built in global memory),
    k > 10 a state per thread (k_merge, mask-table lookups): exact against
    the oracle unpruned, with a starting bound and with refinement."""
    g = native.gen_random_connected(300, 900, 1, 40, 60 + k)
    gp, mem = native.gen_groups_uniform(300, k, 2, 70 + k)
    want = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
    assert want.status == oracle.OK
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        for kw in ({}, {"upper_bound": 2 * want.cost + 1}, {"upper_bound": want.cost}, {"refine_bound": True}):
            for use_graph in (False, True):
                res = dg.solve(gp, mem, use_graph=use_graph, **kw)
                _check(g.row_ptr, g.col, g.w, gp, mem, res, want.cost)
        if want.cost > 1:
            assert dg.solve(gp, mem, upper_bound=want.cost - 1).status == Status.INFEASIBLE


def test_batch_query_with_bad_k_fails_alone():
    """A query whose k is out of range fails by itself; the queries after it
    keep their own groups (their offsets count the bad query's k)."""
    g = native.gen_random_connected(600, 2000, 1, 50, 71)
    q1 = native.gen_groups_uniform(600, 3, 4, 72)
    bad = native.gen_groups_uniform(600, 17, 2, 73)
    q3 = native.gen_groups_uniform(600, 3, 4, 74)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        res = dg.solve_batch([q1, bad, q3], raise_on_error=False)
    assert res[1].status == Status.BAD_INPUT
    for (gp, mem), r in ((q1, res[0]), (q3, res[2])):
        _check(g.row_ptr, g.col, g.w, gp, mem, r, oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem).cost)


@pytest.mark.parametrize("use_graph", MODES)
def test_workspace_reuse_across_k_and_repeat(use_graph):
    g = native.gen_barabasi_albert(4000, 4, 1, 100, 3)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        for k, seed in [(3, 1), (6, 2), (4, 3), (6, 2), (2, 5), (7, 9), (6, 2)]:
            gp, mem = native.gen_groups_zipf_degree(g, k, 1.2, 5, 500, seed)
            want = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
            res = dg.solve(gp, mem, use_graph=use_graph)
            _check(g.row_ptr, g.col, g.w, gp, mem, res, want.cost)


def test_batch_matches_single(golden):
    g = native.gen_barabasi_albert(3000, 4, 1, 100, 17)
    queries = [native.gen_groups_zipf_degree(g, 3 + (i % 5), 1.2, 5, 500, 900 + i) for i in range(12)]
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        batch = dg.solve_batch(queries)
        for (gp, mem), res in zip(queries, batch):
            want = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
            _check(g.row_ptr, g.col, g.w, gp, mem, res, want.cost)


def test_reference_call_surface_on_fixture():
    # the reference's harness flow (rucgraph/test_gpu.h:116-223) through the mirror
    rp, col, w, gp, mem, cost = load_fixture()
    input_graph = dpbf.csr_to_graph_v_of_v(rp, col, w)
    groups = [list(mem[gp[i]:gp[i + 1]]) for i in range(len(gp) - 1)]
    group_graph, group_vertices = dpbf.group_graph_from_groups(len(input_graph), groups)
    csr = dpbf.toCSR(input_graph)
    counter = [0]
    tree, real_cost, processed, rt = dpbf.DPBF_GPU(csr, group_vertices, group_graph, input_graph, pointer1=counter)
    assert real_cost == cost == 16
    assert dpbf.graph_hash_of_mixed_weighted_sum_of_ec(tree) == real_cost
    assert dpbf.this_is_a_feasible_solution_gpu(tree, group_graph, group_vertices)
    assert processed > 0 and counter[0] == processed and rt >= 0
    csr.free()


def test_bad_member_is_rejected():
    rp, col, w, gp, mem, _ = load_fixture()
    bad = mem.copy()
    bad[0] = 10**6
    with native.Graph(rp, col, w) as g:
        with pytest.raises(native.GSTError) as e:
            g.solve(gp, bad)
        assert e.value.status == Status.BAD_INPUT


@pytest.mark.parametrize("use_graph", MODES)
def test_timeout_status_is_reported(use_graph):
    g = native.gen_random_connected(2000, 4000, 1, 100, 8)
    gp, mem = native.gen_groups_uniform(2000, 3, 2, 9)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        res = dg.solve(gp, mem, max_rounds=1, raise_on_error=False, use_graph=use_graph)
        assert res.status == Status.TIMEOUT
        # the graph stays usable after the error
        want = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
        _check(g.row_ptr, g.col, g.w, gp, mem, dg.solve(gp, mem, use_graph=use_graph), want.cost)


@pytest.mark.parametrize("use_graph", MODES)
def test_stats_and_launch_count(use_graph):
    g = native.gen_barabasi_albert(20000, 4, 1, 100, 5)
    gp, mem = native.gen_groups_zipf_degree(g, 5, 1.2, 5, 500, 6)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        res = dg.solve(gp, mem, use_graph=use_graph, collect_stats=True)
        assert res.status == Status.OK
        st = res.stats
        assert st["rounds"] > 0 and st["vertices"] > 0 and st["entries"] > 0 and st["bytes"] > 0
        # each state evaluates its unordered splits, except states of cost 0
        assert 0 < st["splits"] <= 20000 * (3**5 - 2**6 + 1) // 2
        assert res.launches >= 1 + 5 + st["rounds"] + 2


def _oracle_costs(g, qs):
    return [oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem).cost for gp, mem in qs]


def _ba_queries(V, n, seed):
    g = native.gen_barabasi_albert(V, 4, 1, 100, seed)
    rng = np.random.default_rng(seed)
    qs = [native.gen_groups_zipf_degree(g, int(rng.integers(3, 7)), 1.2, 5, 60, seed * 1000 + i) for i in range(n)]
    return g, qs


@pytest.mark.parametrize("concurrency", [1, 3, 0])
def test_concurrent_batch_matches_single(concurrency):
    """gst_solve_batch runs queries on concurrent solve contexts (lanes)
    over one resident graph: every result equals the single solve."""
    g, qs = _ba_queries(20_000, 12, 31)
    want = _oracle_costs(g, qs)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        assert [dg.solve(gp, mem, use_graph=True).cost for gp, mem in qs] == want
        for refine in (False, True):
            got = dg.solve_batch(qs, use_graph=True, refine_bound=refine, concurrency=concurrency)
            assert [r.cost for r in got] == want
            for (gp, mem), r in zip(qs, got):
                _check(g.row_ptr, g.col, g.w, gp, mem, r, r.cost)
                assert r.latency_ms[0] > 0 and r.latency_ms[1] >= r.latency_ms[0] * 0.999


@pytest.mark.parametrize("batch_graph", [2, 3, 8])
def test_batch_graphs_match_oracle(batch_graph):
    """gst_solve_batch with batch graphs: queries grouped by k, each chunk
    one launch of a CUDA graph whose parallel branches are the queries'
    whole solves. Every cost equals the oracle's, every tree is valid, on
    two batches in a row (the second reuses the captured graphs), with and
    without bound refinement; a query with k = 17 fails alone."""
    g, qs = _ba_queries(20_000, 13, 43)
    want = _oracle_costs(g, qs)
    bad = native.gen_groups_uniform(g.V, 17, 2, 44)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        for refine in (False, True, True):
            got = dg.solve_batch(qs[:6] + [bad] + qs[6:], refine_bound=refine, batch_graph=batch_graph,
                                 raise_on_error=False)
            assert got[6].status == Status.BAD_INPUT
            got = got[:6] + got[7:]
            assert [r.cost for r in got] == want
            for (gp, mem), r in zip(qs, got):
                _check(g.row_ptr, g.col, g.w, gp, mem, r, r.cost)


def test_autotune_keeps_results_exact():
    g, qs = _ba_queries(20_000, 16, 37)
    want = _oracle_costs(g, qs)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        lanes = dg.autotune(qs[:8], refine_bound=True)
        assert lanes in (1, 2, 4, 8)  # concurrent contexts or batch-graph size
        got = dg.solve_batch(qs, use_graph=True, refine_bound=True)
        assert [r.cost for r in got] == want
        assert [dg.solve(gp, mem, use_graph=True).cost for gp, mem in qs] == want


def test_autotune_cache_applies_the_stored_record(tmp_path):
    """autotune(cache=...) tunes once, stores the record under the graph's
    shape key, and a second graph of the same shape takes the record from
    the file instead of tuning; the batch results stay exact."""
    g, qs = _ba_queries(20_000, 8, 41)
    want = _oracle_costs(g, qs)
    cache = tmp_path / "tuning.json"
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        lanes = dg.autotune(qs[:6], refine_bound=True, cache=cache)
        rec = dg.tuning()
    assert cache.exists()
    key = native.tuning_key(g.V, g.nnz, [len(gp) - 1 for gp, _ in qs[:6]], True, True)
    assert native.load_tuning(cache, key) == rec
    assert lanes == (rec["batch_graph"] or rec["concurrency"])
    with native.Graph(g.row_ptr, g.col, g.w) as dg2:
        assert dg2.tuning()["concurrency"] == 0  # a fresh graph is untuned
        assert dg2.autotune(qs[:6], refine_bound=True, cache=cache) == lanes
        assert dg2.tuning() == rec
        assert [r.cost for r in dg2.solve_batch(qs, use_graph=True, refine_bound=True)] == want
        bad = dict(rec, batch_graph=99)
        with pytest.raises(native.GSTError):
            dg2.set_tuning(bad)
        assert dg2.tuning() == rec  # a rejected record changes nothing


def test_dataset_files_solve_like_the_reference_harness(tmp_path):
    """A dataset in the reference's file formats (.in/.g/.g7), read with the
    gst_io readers and solved query by query (rucgraph/test_gpu.h:115-215)."""
    from test_dataset_cpu import write_in

    g = native.gen_random_connected(400, 1600, 1, 100, 21)
    write_in(tmp_path / "d.in", g)
    groups = [native.gen_groups_uniform(g.V, 1, 6, 900 + i)[1].tolist() for i in range(6)]
    (tmp_path / "d.g").write_text("".join(f"g{i + 1}:{' '.join(map(str, m))}\n" for i, m in enumerate(groups)))
    (tmp_path / "d.g7").write_text(f"{g.V} {g.V + 3} {g.V + 5} \n{g.V + 1} {g.V + 2} {g.V + 4} \n")
    h, _ = native.read_graph_file(tmp_path / "d.in")
    all_groups = native.read_groups_file(tmp_path / "d.g")
    queries = native.read_queries_file(tmp_path / "d.g7", h.V)
    assert queries == [[0, 3, 5], [1, 2, 4]]
    with native.Graph(h.row_ptr, h.col, h.w) as dg:
        for ids in queries:
            gp, mem = native.query_groups(all_groups, ids)
            want = oracle.dpbf(h.row_ptr, h.col, h.w, gp, mem).cost
            _check(h.row_ptr, h.col, h.w, gp, mem, dg.solve(gp, mem, use_graph=True), want)


def test_replica_pool_matches_single():
    """gst_pool: replicas of the graph (here two on device 0; on a multi-GPU
    node one per device) share a batch by work stealing; results equal the
    single solves and both replicas take queries."""
    g, qs = _ba_queries(20_000, 24, 41)
    want = _oracle_costs(g, qs)
    with native.Pool(g.row_ptr, g.col, g.w, [0, 0]) as pool:
        assert pool.replicas == 2
        got = pool.solve_batch(qs, refine_bound=True, concurrency=2)
        assert [r.cost for r in got] == want
        assert {r.replica for r in got} == {0, 1}
        for (gp, mem), r in zip(qs, got):
            _check(g.row_ptr, g.col, g.w, gp, mem, r, r.cost)


@pytest.mark.parametrize("use_graph", MODES)
@pytest.mark.parametrize("k", [4, 6])
def test_full_state_table_with_hub_segments(use_graph, k):
    """The whole table of the grown waves equals the oracle's exact fixpoint
    on a BA graph whose hubs span one and several 256-entry segments (the
    hub rows are relaxed whole by one warp, or folded through a scratch row
    by several), with dense, flag-checked and sparse rounds all occurring;
    at k = 6 the waves of 15 and 20 masks also run their small-frontier
    sparse rounds by vertex teams."""
    g = native.gen_barabasi_albert(30000, 4, 1, 100, 77)
    deg = np.diff(g.row_ptr)
    assert (deg > 256).sum() > 0 and (deg > 64).sum() > 100
    gp, mem = native.gen_groups_zipf_degree(g, k, 1.2, 5, 500, 79)
    assert len(gp) - 1 == k
    want = oracle.dp_table(g.row_ptr, g.col, g.w, gp, mem)
    want = np.where(want == ORACLE_INF, native.COST_LIMIT, want)
    with native.Graph(g.row_ptr, g.col, g.w) as dg:
        res = dg.solve(gp, mem, use_graph=use_graph)
        assert res.status == Status.OK
        got = dg.debug_table(k)
    full = (1 << k) - 1
    assert np.array_equal(got[:, 1:full], want[:, 1:full])
    assert got[:, full].min() == want[:, full].min() == res.cost
