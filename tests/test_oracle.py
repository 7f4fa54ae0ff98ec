"""Pins the CPU oracle (the C restatement) against the reference's own
solvers: the golden costs in tests/golden were produced by the reference's
graph_v_of_v_idealID_DPBF_only_ec compiled from its unmodified headers."""
import hashlib

import numpy as np
import pytest

import oracle
from conftest import load_edge_cases, load_fixture, make_instance


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()[:16]


def test_fixture_simple_iterative():
    rp, col, w, gp, mem, cost = load_fixture()
    assert cost == 16  # the reference's shipped instance (simple_iterative_tests.text)
    r = oracle.dpbf(rp, col, w, gp, mem)
    assert r.status == oracle.OK and r.cost == cost
    assert oracle.check_tree(rp, col, w, gp, mem, r.vertices, r.edges, r.cost) is None


def test_golden_instances_regenerate_bit_identically(golden):
    for case in golden["cases"]:
        g, gp, mem = make_instance(case)
        assert _digest(g.row_ptr, g.col, g.w, gp, mem) == case["digest"], case["name"]


def test_golden_costs(golden):
    for case in golden["cases"]:
        g, gp, mem = make_instance(case)
        r = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
        assert r.status == oracle.OK, case["name"]
        assert r.cost == case["dpbf"], case["name"]
        assert oracle.check_tree(g.row_ptr, g.col, g.w, gp, mem, _dedup(r.vertices), _edges(r.edges),
                                 r.cost) is None, case["name"]


def test_edge_cases():
    for name, c in load_edge_cases().items():
        r = oracle.dpbf(c["rp"], c["col"], c["w"], c["gp"], c["mem"])
        if int(c["cost"]) < 0:
            assert r.status == oracle.INFEASIBLE, name
        else:
            assert r.status == oracle.OK and r.cost == int(c["cost"]), name


def test_layered_table_matches_dpbf(golden):
    # the layered DP (src/DP.cu formulation) reaches the same optimum
    for case in golden["cases"][:25]:
        g, gp, mem = make_instance(case)
        t = oracle.dp_table(g.row_ptr, g.col, g.w, gp, mem)
        assert int(t[:, -1].min()) == case["dpbf"], case["name"]


def test_one_label_lb_is_max_singleton_distance(golden):
    case = golden["cases"][0]
    g, gp, mem = make_instance(case)
    t = oracle.dp_table(g.row_ptr, g.col, g.w, gp, mem)
    lb = oracle.one_label_lb(g.row_ptr, g.col, g.w, gp, mem)
    k = len(gp) - 1
    singles = np.stack([t[:, 1 << i] for i in range(k)], axis=1)
    assert np.array_equal(lb, singles.max(axis=1))


@pytest.mark.parametrize("seed", range(6))
def test_port_matches_reference_live(seed):
    if oracle.ref_lib() is None:
        pytest.skip("reference checkout not present")
    from gpu4gst_code_gb300 import native as N

    g = N.gen_random_connected(400, 1600, 1, 50, 500 + seed)
    gp, mem = N.gen_groups_uniform(400, 3 + seed % 4, 4, 600 + seed)
    r = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
    ref = oracle.reference(g.row_ptr, g.col, g.w, gp, mem)
    assert r.cost == ref.cost


def test_bounded_sample_stops():
    from gpu4gst_code_gb300 import native as N

    g = N.gen_random_connected(1000, 5000, 1, 100, 3)
    gp, mem = N.gen_groups_uniform(1000, 3, 20, 1003)
    r = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem, max_pops=10)
    assert r.status == oracle.STOPPED and r.pops == 10


def _dedup(v):
    return np.unique(v)


def _edges(e):
    e = np.asarray(e).reshape(-1, 3)
    seen = {}
    for u, v, w in e:
        seen[(min(int(u), int(v)), max(int(u), int(v)))] = int(w)
    return np.array([[a, b, w] for (a, b), w in seen.items()], np.int32).reshape(-1, 3)


def test_large_golden_costs_agree_with_the_reference_solver():
    """tests/golden/large.json: wherever the reference's own DPBF
    (graph_v_of_v_idealID_DPBF_only_ec, compiled from its unmodified
    headers) was run on a benchmark query (ref_cost, recorded by
    make_large.py --reference), it returned the oracle's cost — the pin of
    the full-size golden costs on the reference itself."""
    import json
    from pathlib import Path

    cases = json.loads((Path(__file__).resolve().parent / "golden" / "large.json").read_text())["cases"]
    pinned = [c for c in cases if "ref_cost" in c]
    assert pinned, "no case carries the reference solver's cost"
    assert {c["workload"] for c in pinned} >= {"rc1k_k3", "ba1m_k6", "serve256"}
    for c in pinned:
        assert c["ref_cost"] == c["cost"], (c["workload"], c["index"], c["ref_cost"], c["cost"])

