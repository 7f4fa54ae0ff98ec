"""Generates tests/golden/large.json: oracle costs of the benchmark's own
queries at the sizes the workloads name.

For every workload of bench.py listed below, the graph and the first N
queries (query i is seeded 1000 + i, exactly as bench.py makes them) are
built with the oracle's own build of the seeded generators (oracle.gen_*,
the same source as include/gst_gen.h) and solved by the CPU oracle's C
restatement of the reference DPBF (oracle.dpbf, pinned against the
reference's own graph_v_of_v_idealID_DPBF_only_ec by tests/test_oracle.py).
Each case records digests of the regenerated graph and groups, so a reader
can check that it rebuilt the same instance, the optimal cost, the states
the oracle popped and its single-core time.

The GPU machine never runs this script (it takes tens of minutes and ~10 GB of
host memory per 2M- or 4M-vertex query); bench.py and the -m gpu tests only
read the committed file.

  python tests/golden/make_large.py [--workloads ba1m_k6,ba2m_k8,...] [--jobs N] [--reference N]

--reference N also runs the reference's own DPBF (compiled from its headers in
this container, oracle/_ref) on the first N cases of each workload and
records its cost (ref_cost) beside the oracle's.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import json
import multiprocessing as mp
import os
import platform
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

OUT = HERE / "large.json"

# workload -> (query indices, parallel jobs; the 2M and 4M instances need ~10 GB each)
PLAN = {
    "rc1k_k3": (range(0, 40), 8),
    "ba1m_k6": (range(0, 30), 6),
    "serve256": (range(0, 48), 6),
    "ba2m_k8": (range(0, 3), 3),
    "ba4m_k7": (range(0, 3), 3),
}


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()[:16]


def _solve(args):
    name, i = args
    import bench
    import oracle

    wl = dict(bench.WORKLOADS[name], name=name)
    g = bench.make_graph(wl, oracle)
    gp, mem = bench.make_query(wl, g, i, oracle)
    t = time.perf_counter()
    r = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
    sec = time.perf_counter() - t
    if r.cost >= 0:
        err = oracle.check_tree(g.row_ptr, g.col, g.w, gp, mem, r.vertices, r.edges, r.cost)
        if err is not None:
            raise RuntimeError(f"{name} query {i}: oracle tree invalid: {err}")
    return {"workload": name, "index": i, "seed": 1000 + i, "k": int(len(gp) - 1),
            "graph_digest": digest(g.row_ptr, g.col, g.w), "groups_digest": digest(gp, mem),
            "cost": int(r.cost), "pops": int(r.pops), "oracle_s": round(sec, 3)}


def _reference(args):
    """The reference's own DPBF solver (graph_v_of_v_idealID_DPBF_only_ec,
    compiled from its unmodified headers into oracle/_ref) on one case."""
    name, i = args
    import bench
    import oracle

    wl = dict(bench.WORKLOADS[name], name=name)
    g = bench.make_graph(wl, oracle)
    gp, mem = bench.make_query(wl, g, i, oracle)
    t = time.perf_counter()
    r = oracle.reference(g.row_ptr, g.col, g.w, gp, mem, solver="dpbf")
    sec = time.perf_counter() - t
    if r is None:
        raise RuntimeError("the reference's solver library (oracle/_ref) is not available")
    return name, i, int(r.cost), round(sec, 3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workloads", default=",".join(PLAN))
    ap.add_argument("--jobs", type=int, default=0, help="parallel oracle processes (0: the plan's)")
    ap.add_argument("--reference", type=int, default=0,
                    help="also solve the first N cases of each workload with the reference's own DPBF (ref_cost)")
    ap.add_argument("--reference-jobs", type=int, default=2)
    args = ap.parse_args()
    import oracle

    oracle.build_oracle()  # once, before the workers start
    oracle.build_gen()
    done = json.loads(OUT.read_text()) if OUT.exists() else {"cases": []}
    have = {(c["workload"], c["index"]) for c in done["cases"]}
    for name in args.workloads.split(","):
        idx, jobs = PLAN[name]
        todo = [(name, i) for i in idx if (name, i) not in have]
        if not todo:
            continue
        ctx = mp.get_context("spawn")
        with cf.ProcessPoolExecutor(max_workers=args.jobs or jobs, mp_context=ctx) as ex:
            for case in ex.map(_solve, todo):
                done["cases"].append(case)
                print(json.dumps(case), flush=True)
                done["cases"].sort(key=lambda c: (c["workload"], c["index"]))
                done["generator"] = ("tests/golden/make_large.py: bench.py's workloads and query seeds, oracle.gen_* "
                                     "instances, oracle.dpbf costs")
                done["host"] = f"{platform.machine()}, {os.cpu_count()} threads"
                OUT.write_text(json.dumps(done, indent=1) + "\n")
    if args.reference:
        oracle.build_ref()
        byname = {(c["workload"], c["index"]): c for c in done["cases"]}
        todo = [(name, i) for name in args.workloads.split(",") for i in range(args.reference)
                if (name, i) in byname and "ref_cost" not in byname[(name, i)]]
        ctx = mp.get_context("spawn")
        with cf.ProcessPoolExecutor(max_workers=args.reference_jobs, mp_context=ctx) as ex:
            for name, i, cost, sec in ex.map(_reference, todo):
                byname[(name, i)].update(ref_cost=cost, ref_s=sec)
                print(json.dumps(byname[(name, i)]), flush=True)
                done["reference"] = ("ref_cost: the reference's own graph_v_of_v_idealID_DPBF_only_ec, compiled from its "
                                     "unmodified headers (oracle/build_ref.sh), single-threaded; ref_s its time")
                OUT.write_text(json.dumps(done, indent=1) + "\n")


if __name__ == "__main__":
    main()
