"""Generates tests/golden/ from the reference's own CPU solvers.

Run in a checkout that has the reference next to it (oracle/_ref builds from
its unmodified headers); the GPU machine never runs this script, it only reads
the committed fixtures.

  python tests/golden/make_golden.py [--reference /root/reference]

Writes:
  simple_iterative.npz   the reference's shipped GSTP instance
                         (simple_iterative_tests.text) as CSR + groups,
                         parsed the way graph_hash_of_mixed_weighted_read_for_GSTP
                         does (rucgraph/graph_hash_of_mixed_weighted_read_for_GSTP.h:9-73:
                         weights through stod then int), with its optimal cost
  golden.json            seeded instances (regenerated by the project's
                         generators at test time, checked by a digest) and
                         the costs the reference's DPBF and PrunedDP++ return
  edge_cases.npz         small hand-built instances (zero weights, parallel
                         entries, overlapping groups, one-vertex trees,
                         infeasible) with reference costs
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from gpu4gst_code_gb300 import native as N  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()[:16]


def read_gstp(path: Path):
    """GSTP text -> (row_ptr, col, w, group_ptr, members)."""
    edges = {}
    gedges = []
    group_ids = []
    V = 0
    for line in path.read_text().splitlines():
        p = line.split(" ")
        if len(p) >= 3 and p[0] == "input_graph" and p[1] == "Vertex":
            V = max(V, int(p[2]) + 1)
        elif len(p) >= 5 and p[0] == "input_graph" and p[1] == "Edge":
            a, b, ec = int(p[2]), int(p[3]), int(float(p[4]))
            V = max(V, a + 1, b + 1)
            edges[(min(a, b), max(a, b))] = ec  # add_edge replaces the weight
        elif len(p) >= 5 and p[0] == "group_graph" and p[1] == "Edge":
            gedges.append((int(p[2]), int(p[3])))
        elif len(p) >= 2 and p[0] == "group_vertices":
            group_ids.append(int(p[1]))
    group_ids.sort()
    members = {g: set() for g in group_ids}
    for a, b in gedges:
        if a in members and b < V:
            members[a].add(b)
        elif b in members and a < V:
            members[b].add(a)
    rows = [[] for _ in range(V)]
    for (a, b), ec in edges.items():
        rows[a].append((b, ec))
        rows[b].append((a, ec))
    rp = [0]
    col, w = [], []
    for r in rows:
        r.sort()
        col += [x for x, _ in r]
        w += [y for _, y in r]
        rp.append(len(col))
    gp = [0]
    mem = []
    for g in group_ids:
        mem += sorted(members[g])
        gp.append(len(mem))
    return (np.array(rp, np.int32), np.array(col, np.int32), np.array(w, np.int32), np.array(gp, np.int32),
            np.array(mem, np.int32))


def csr_from_edges(V, edge_list):
    rows = [[] for _ in range(V)]
    for a, b, ww in edge_list:
        rows[a].append((b, ww))
        if a != b:
            rows[b].append((a, ww))
    rp, col, w = [0], [], []
    for r in rows:
        r.sort()
        col += [x for x, _ in r]
        w += [y for _, y in r]
        rp.append(len(col))
    return np.array(rp, np.int32), np.array(col, np.int32), np.array(w, np.int32)


def _solve_worker(solver: str, path: str) -> None:
    """Child process: solve the instance saved at `path`, print the cost."""
    d = np.load(path)
    r = oracle.reference(d["rp"], d["col"], d["w"], d["gp"], d["mem"], solver)
    print(json.dumps({"cost": r.cost if r.status == oracle.OK else -1}))


def _run_ref(solver, rp, col, w, gp, mem):
    """Runs one reference solver in a child process: both solvers call
    getchar()/exit() when they find no tree, which must not take this
    script down. Returns the cost, -1 for "no tree", None if the solver
    died or timed out."""
    with tempfile.NamedTemporaryFile(suffix=".npz", delete=False) as f:
        np.savez(f, rp=rp, col=col, w=w, gp=gp, mem=mem)
        path = f.name
    try:
        # cwd: PrunedDP++ writes "PrunedDPPlusPlus_irregular.txt" into the
        # working directory when it finds no tree (PrunedDPPlusPlus.h:962)
        proc = subprocess.run([sys.executable, os.path.abspath(__file__), "--worker", solver, path],
                              stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=1800,
                              cwd=tempfile.gettempdir())
    except subprocess.TimeoutExpired:
        return None
    finally:
        os.unlink(path)
    for line in proc.stdout.splitlines()[::-1]:
        if line.startswith("{"):
            return json.loads(line)["cost"]
    return None


def ref_costs(rp, col, w, gp, mem):
    out = {"dpbf": _run_ref("dpbf", rp, col, w, gp, mem)}
    # PrunedDP++ rejects zero edge weights (rucgraph/test_gpu.h:85) and k >= 15
    if len(gp) - 1 < 15 and len(w) > 0 and int(np.min(w)) > 0:
        out["pruned_dp_pp"] = _run_ref("pp", rp, col, w, gp, mem)
    return out


def edge_cases():
    cases = []
    # 1. single vertex carrying both groups: cost 0, tree = that vertex
    cases.append(("one_vertex", 1, [], [[0], [0]]))
    # 2. path 0-1-2-3 with a zero-weight middle edge
    cases.append(("zero_weight_path", 4, [(0, 1, 3), (1, 2, 0), (2, 3, 4)], [[0], [3]]))
    # 3. zero-weight triangle plus a tail: cycles of cost 0
    cases.append(("zero_triangle", 5, [(0, 1, 0), (1, 2, 0), (2, 0, 0), (2, 3, 2), (3, 4, 1)], [[0], [4], [1]]))
    # 4. groups overlapping on a hub vertex
    cases.append(("overlap_hub", 6, [(0, 1, 5), (0, 2, 5), (0, 3, 5), (3, 4, 1), (4, 5, 1)],
                  [[1, 4], [2, 4], [4, 5]]))
    # 5. disconnected: the groups live in different components -> infeasible
    cases.append(("disconnected", 4, [(0, 1, 1), (2, 3, 1)], [[0], [3]]))
    # 6. k = 1: a single group -> cost 0
    cases.append(("k1", 3, [(0, 1, 7), (1, 2, 7)], [[2, 0]]))
    # 7. star with a heavy centre vs a cheap rim path
    cases.append(("star_vs_rim", 6, [(0, 1, 10), (0, 2, 10), (0, 3, 10), (1, 4, 1), (4, 2, 1), (2, 5, 1), (5, 3, 1)],
                  [[1], [2], [3]]))
    # 8. every vertex in every group (k=4): cost 0
    cases.append(("all_in_all", 3, [(0, 1, 2), (1, 2, 2)], [[0, 1, 2]] * 4))
    # 9. isolated vertices around the solution
    cases.append(("isolated", 7, [(1, 2, 4), (2, 3, 4), (3, 5, 1)], [[1], [5], [2, 6]]))
    out = {}
    for name, V, el, groups in cases:
        rp, col, w = csr_from_edges(V, el)
        gp, mem = N.groups_to_csr(groups)
        cost = _run_ref("dpbf", rp, col, w, gp, mem)
        out[name] = dict(rp=rp, col=col, w=w, gp=gp, mem=mem, cost=np.int32(cost))
        print(f"edge case {name}: cost {cost}")
    return out


def main():
    if len(sys.argv) == 4 and sys.argv[1] == "--worker":
        _solve_worker(sys.argv[2], sys.argv[3])
        return
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=str(oracle.REFERENCE_ROOT))
    ap.add_argument("--config1-seeds", type=int, default=200)
    args = ap.parse_args()
    oracle.REFERENCE_ROOT = Path(args.reference)
    if oracle.build_ref() is None:
        sys.exit("reference checkout not found: golden fixtures need the reference's own solvers")

    # --- the reference's shipped instance
    rp, col, w, gp, mem = read_gstp(Path(args.reference) / "simple_iterative_tests.text")
    costs = ref_costs(rp, col, w, gp, mem)
    print("simple_iterative_tests.text:", costs)
    np.savez_compressed(HERE / "simple_iterative.npz", row_ptr=rp, col=col, w=w, group_ptr=gp, members=mem,
                        cost=np.int32(costs["dpbf"]))

    gold = {"generator": "gst_gen (xoshiro256**/splitmix64)", "cases": []}
    # --- config 1: V=1000, E=5000, w U[1,100], k=3 x 20 uniform members
    def config1(seed):
        g = N.gen_random_connected(1000, 5000, 1, 100, seed)
        gp, mem = N.gen_groups_uniform(1000, 3, 20, 1000 + seed)
        c = ref_costs(g.row_ptr, g.col, g.w, gp, mem)
        return dict(name=f"config1_s{seed}", graph=["random_connected", 1000, 5000, 1, 100, seed],
                    groups=["uniform", 3, 20, 1000 + seed], digest=digest(g.row_ptr, g.col, g.w, gp, mem), **c)

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        gold["cases"] += list(ex.map(config1, range(args.config1_seeds)))
    # --- wider checks: more groups, larger graphs, BA graphs with Zipf groups
    extra = [
        (["random_connected", 2000, 8000, 1, 100, 7], ["uniform", 5, 8, 77]),
        (["random_connected", 10000, 50000, 1, 4, 3], ["uniform", 4, 3, 33]),
        (["random_connected", 500, 1500, 1, 1000, 11], ["uniform", 8, 4, 111]),
        (["random_connected", 300, 900, 0, 20, 12], ["uniform", 6, 3, 112]),
        (["barabasi_albert", 5000, 4, 1, 100, 21], ["zipf_degree", 6, 1.2, 5, 500, 121]),
        (["barabasi_albert", 20000, 4, 1, 100, 22], ["zipf_degree", 5, 1.2, 5, 500, 122]),
        (["barabasi_albert", 3000, 8, 1, 1000, 23], ["uniform", 7, 10, 123]),
    ]
    for gspec, qspec in extra:
        g = make_graph(gspec)
        gp, mem = make_groups(g, qspec)
        c = ref_costs(g.row_ptr, g.col, g.w, gp, mem)
        name = f"{gspec[0]}_V{gspec[1]}_{qspec[0]}_k{qspec[1]}"
        print(name, c)
        gold["cases"].append(dict(name=name, graph=gspec, groups=qspec, digest=digest(g.row_ptr, g.col, g.w, gp, mem),
                                  **c))
    (HERE / "golden.json").write_text(json.dumps(gold, indent=1) + "\n")
    np.savez_compressed(HERE / "edge_cases.npz", **{f"{n}__{k}": v for n, d in edge_cases().items()
                                                    for k, v in d.items()})


def make_graph(spec):
    kind, *a = spec
    if kind == "random_connected":
        return N.gen_random_connected(*a)
    if kind == "barabasi_albert":
        return N.gen_barabasi_albert(*a)
    raise ValueError(kind)


def make_groups(g, spec):
    kind, *a = spec
    if kind == "uniform":
        k, size, seed = a
        return N.gen_groups_uniform(g.V, k, size, seed)
    if kind == "zipf_degree":
        k, s, lo, hi, seed = a
        return N.gen_groups_zipf_degree(g, k, s, lo, hi, seed)
    raise ValueError(kind)


if __name__ == "__main__":
    main()
