"""Runs the queries of a dataset in the reference's file formats, as the
reference's experiment loop does (rucgraph/test_gpu.h:115-215): read
<name>.in, <name>.g and a query file, upload the graph once, solve every
query exactly and print cost, tree size and time per query.

    python -m gpu4gst_code_gb300.run_dataset /data/Amazon --queries g7 [--method plain|bounded|learned]

The reference's own datasets (Amazon, MovieLens, ...) are not shipped with
it; any files in these formats work.
"""
from __future__ import annotations

import argparse
import json
import time

from . import native as N


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("name", help="dataset path prefix: reads <name>.in and <name>.g")
    ap.add_argument("--queries", default="g7", help="query file suffix (<name>.<suffix>)")
    ap.add_argument("--method", default="plain", choices=["plain", "bounded", "learned"])
    ap.add_argument("--limit", type=int, default=0, help="solve only the first n queries")
    a = ap.parse_args()
    g, C = N.read_graph_file(a.name + ".in")
    groups = N.read_groups_file(a.name + ".g")
    queries = N.read_queries_file(a.name + "." + a.queries, g.V)
    if a.limit:
        queries = queries[: a.limit]
    print(json.dumps({"V": g.V, "entries": g.nnz, "communities": C, "groups": len(groups[0]) - 1,
                      "queries": len(queries)}), flush=True)
    scorer = None
    if a.method == "learned":
        from . import learn

        scorer = N.Scorer(learn.load_params())
    with N.Graph(g.row_ptr, g.col, g.w) as dg:
        for i, ids in enumerate(queries):
            gp, mem = N.query_groups(groups, ids)
            t = time.perf_counter()
            if a.method == "learned":
                r = dg.solve_learned(scorer, gp, mem, raise_on_error=False)
            else:
                r = dg.solve(gp, mem, use_graph=True, refine_bound=a.method == "bounded", raise_on_error=False)
            wall = time.perf_counter() - t
            print(json.dumps({"query": i, "k": len(ids), "status": r.status.name, "cost": r.cost,
                              "tree_vertices": len(r.vertices), "device_ms": r.times_ms[0],
                              "wall_ms": 1e3 * wall}), flush=True)
    if scorer:
        scorer.close()


if __name__ == "__main__":
    main()
