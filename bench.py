"""Benchmark: exact GST queries/sec on one GB300 (DPBF, k=6, |V|=1M).

A step is one exact query on a resident synthetic graph: Barabasi-Albert
m=4, |V|=1,000,000 (~4M edges), integer weights U[1,100]; k=6 groups with
Zipf(1.2) sizes clipped to [5,500], members drawn proportionally to degree.
Every step uses a different seeded query on the same graph. The same K
queries run through three exact methods, each through the C ABI:

  plain     gst_solve: the DPBF of the reference, unpruned;
  bounded   gst_solve with refine_bound: the bound is lowered after every
            wave from partial trees (PrunedDP++'s best-solution update);
  learned   gst_solve_learned with the committed trained scorer: the
            bound-refined DP, with the cost of a proposal tree rooted at
            the network's top vertex injected as a bound while it runs.

`value` is the bound-refined method's throughput (the fastest exact method
on this workload); the plain and learned methods and their speedups over
plain ride along in the same line (`methods`, `speedup_vs_plain`).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Device time comes from CUDA events recorded on the solver's own stream
(the learned method's proposal runs on a second stream while the DP's
graph runs, and the solver's stream records its end event only after the
proposal returned, so the event span covers both; with the host driver
the proposal runs first and its host wall time is added). The state table of a query (1M x 63 int32 costs + parents,
504 MB) exceeds L2 (129 MB), and L2 is additionally flushed (a 256 MiB
device write) before every step. `e2e` is the wall time of the C-ABI call
with host group arrays in and the host tree out. The CPU baseline is the
oracle's C restatement of the reference's CPU DPBF on one host core, one
full query.

Reference arm: the reference's CPU DPBF (its C restatement: the reference's
own build needs a Boost it does not ship) on all host cores, one query per
thread, K timed queries.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GST queries/sec, k=6, |V|=1M, exact; learned-UB pruned vs plain DPBF speedup"
UNIT = "queries/s"
FALLBACK_HBM_GBS = 6800.0

METHOD_DESC = {
    "plain": "plain DPBF (gst_solve, unpruned); exact",
    "bounded": "pruned DPBF, bound refined between waves (gst_solve, refine_bound); exact",
    "learned": "learned-bound pruned DPBF (gst_solve_learned, trained scorer, refined bound); exact",
}

WORKLOADS = {
    # name: (graph generator args, group generator, description)
    "ba1m_k6": dict(V=1_000_000, m=4, wmin=1, wmax=100, k=6, zipf=(1.2, 5, 500), graph_seed=2,
                    desc="plain GPU DPBF, single query: BA m=4, |V|=1,000,000, w U[1,100], k=6, "
                         "Zipf(1.2) sizes in [5,500], degree-proportional members"),
    "ba400k_k6": dict(V=400_000, m=4, wmin=1, wmax=100, k=6, zipf=(1.2, 5, 500), graph_seed=2,
                      desc="profiling size of ba1m_k6: BA m=4, |V|=400,000, w U[1,100], k=6, Zipf(1.2) "
                           "sizes in [5,500], degree-proportional members"),
    "ba2m_k8": dict(V=2_000_000, m=8, wmin=1, wmax=1000, k=8, uniform=50, graph_seed=3,
                    desc="plain GPU DPBF, large mask: BA m=8, |V|=2,000,000, w U[1,1000], k=8 x 50 uniform"),
    "ba4m_k7": dict(V=4_000_000, m=8, wmin=1, wmax=100, k=7, zipf=(1.2, 5, 500), graph_seed=5,
                    desc="learned-bound evaluation graph: BA m=8, |V|=4,000,000, w U[1,100], k=7, Zipf(1.2) "
                         "sizes in [5,500], degree-proportional members"),
    "serve256": dict(V=1_000_000, m=4, wmin=1, wmax=100, k=(3, 7), zipf=(1.2, 5, 500), graph_seed=2, batch=256,
                     desc="batched serving: one resident BA m=4 |V|=1,000,000 graph, w U[1,100]; batches of 256 "
                          "queries, k uniform in {3..7}, Zipf(1.2) sizes in [5,500], degree-proportional members"),
    "rc1k_k3": dict(V=1000, E=5000, wmin=1, wmax=100, k=3, uniform=20, graph_seed=0,
                    desc="plain DPBF, single query: random connected |V|=1000 |E|=5000, w U[1,100], k=3 x 20"),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def _generators(gen):
    """The seeded instance generators: the product library's (ours) or the
    oracle's own build of the same source (the reference arm, which must not
    load the product library)."""
    if gen is None:
        from gpu4gst_code_gb300 import native as gen
    return gen


def make_graph(wl, gen=None):
    N = _generators(gen)
    if "E" in wl:
        return N.gen_random_connected(wl["V"], wl["E"], wl["wmin"], wl["wmax"], wl["graph_seed"])
    return N.gen_barabasi_albert(wl["V"], wl["m"], wl["wmin"], wl["wmax"], wl["graph_seed"])


def make_query(wl, g, i, gen=None):
    N = _generators(gen)
    seed = 1000 + i
    k = wl["k"]
    if isinstance(k, tuple):  # k uniform in [lo, hi], seeded per query
        k = int(np.random.default_rng(seed).integers(k[0], k[1] + 1))
    if "zipf" in wl:
        s, lo, hi = wl["zipf"]
        return N.gen_groups_zipf_degree(g, k, s, lo, hi, seed)
    return N.gen_groups_uniform(g.V, wl["k"], wl["uniform"], seed)


# ------------------------------------------------------------- replicas --
def rank_query_ids(rank: int, n: int) -> range:
    """Query indices of one replica's timed steps: every rank solves its own
    n queries (rank 0: 0 .. n-1, the indices tests/golden/large.json holds
    oracle costs for)."""
    return range(rank * n, (rank + 1) * n)


def warmup_query_ids(rank: int, n: int) -> range:
    """Query indices of the untimed warm-up steps, apart from every timed one."""
    return range(100_000 + rank * n, 100_000 + (rank + 1) * n)


def golden_costs(workload: str) -> dict:
    """{query index: oracle cost} of tests/golden/large.json for a workload."""
    p = ROOT / "tests" / "golden" / "large.json"
    try:
        cases = json.loads(p.read_text())["cases"]
    except (OSError, ValueError, KeyError):
        return {}
    return {c["index"]: (c["cost"], c["groups_digest"]) for c in cases if c["workload"] == workload}


def groups_digest(gp, mem) -> str:
    import hashlib

    h = hashlib.sha256()
    for a in (gp, mem):
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()[:16]


def parity_vs_golden(workload: str, indices, queries, costs) -> dict:
    """Compares the costs of timed queries with the oracle costs committed
    for the same query indices; raises on a mismatch."""
    gold = golden_costs(workload)
    checked, mism = 0, []
    for i, (gp, mem), c in zip(indices, queries, costs):
        if i not in gold:
            continue
        want, dig = gold[i]
        if dig != groups_digest(gp, mem):
            raise AssertionError(f"{workload} query {i}: regenerated groups differ from the golden instance")
        checked += 1
        if c != want:
            mism.append((i, c, want))
    if mism:
        raise AssertionError(f"{workload}: costs differ from the oracle: {mism}")
    return {"checked": checked, "mismatches": 0,
            "source": "tests/golden/large.json: oracle.dpbf (C restatement of the reference CPU DPBF) on the same "
                      "seeded queries"}


def max_over_ranks(values, dist=None):
    """This rank's timed totals -> the max over ranks (an all-reduce on the
    host process group); the slowest replica sets the job's time."""
    if dist is None:
        return [float(v) for v in values]
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


# --------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes (read + write) of all growth-kernel launches of one plain
# query, each from one ncu capture of that workload (profiles/
# grow_dram_ba1m_k6.md: every growth launch of query 0 at full size, one pass
# per launch; profiles/grow_dram_ba400k_k6.md); None where no capture exists.
TRAFFIC_PER_STEP = {"ba400k_k6": 2.4e9, "ba1m_k6": 9.78e9}


def table_bytes(V, k):
    """cost + parent tables: V x sum over waves of the padded row stride, int32 each."""
    from math import comb

    return 8 * V * sum((comb(k, l) + 3) // 4 * 4 for l in range(1, k + 1))


def sweep_bytes(V, nnz, k):
    """Bytes of one sweep per grown wave (waves 1 .. k-1): every vertex reads
    its row_ptr pair and its own row, every CSR entry its (col, w) and the
    neighbour's row once, and every row (cost + parent) is written once."""
    from math import comb

    tot = 0
    for l in range(1, k):
        s = (comb(k, l) + 3) // 4 * 4
        tot += V * (8 + 4 * s) + nnz * (8 + 4 * s) + V * 8 * s
    return tot


def traffic_per_step(wl):
    return TRAFFIC_PER_STEP.get(wl.get("name"))


def measured_hbm_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------------------ reference --
def run_reference(args, wl):
    """The reference's CPU DPBF (oracle C restatement) on all host cores."""
    import concurrent.futures as cf

    import oracle

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    g = make_graph(wl, oracle)
    threads = max(1, min(os.cpu_count() or 1, max(args.steps, args.warmup)))

    def one(i):
        gp, mem = make_query(wl, g, i, oracle)
        r = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
        return r.cost

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        if args.warmup:
            list(ex.map(one, warmup_query_ids(0, args.warmup)))
        t0 = time.perf_counter()
        costs = list(ex.map(one, rank_query_ids(0, args.steps)))
        wall = time.perf_counter() - t0
    value = args.steps / wall
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "desc": wl["desc"], "queries": args.steps, "threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full queries, one per thread, {threads} threads; the reference's "
                                   "CPU DPBF as the oracle's C restatement (its own build needs Boost, absent)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "costs": costs,
    }
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------- serving --
def run_serving(args, wl, world, rank, local_rank, dist):
    """Batched serving: a step is one gst_solve_batch of wl['batch'] queries
    (concurrent solve contexts over one resident graph), wall-clocked with
    the device synchronised on both sides; per-query latencies from the
    results. Methods: plain and bounded (value = bounded)."""
    import torch

    from gpu4gst_code_gb300 import native as N

    torch.cuda.set_device(0)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    g = make_graph(wl)
    B = wl["batch"]
    # timed batch j holds query indices rank_query_ids(rank, K * B)[j*B : (j+1)*B]
    # (rank 0's first batch starts at index 0, the indices the golden costs
    # cover); warm-up batches and the autotune sample use indices of their own
    timed_ids = list(rank_query_ids(rank, args.steps * B))
    warm_ids = list(warmup_query_ids(rank, args.warmup * B))
    sample = [make_query(wl, g, 200_000 + 32 * rank + i) for i in range(32)]
    timed_q = [make_query(wl, g, i) for i in timed_ids]
    warm_q = [make_query(wl, g, i) for i in warm_ids]
    queries = timed_q
    dg = N.Graph(g.row_ptr, g.col, g.w)
    t = time.perf_counter()
    lanes = dg.autotune(sample, refine_bound=True)
    tune_s = time.perf_counter() - t
    arms = {}
    clocks = None
    for method in ("plain", "bounded"):
        refine = method == "bounded"
        batches = [timed_q[i * B:(i + 1) * B] for i in range(args.steps)]
        for i in range(args.warmup):
            dg.solve_batch(warm_q[i * B:(i + 1) * B], use_graph=True, refine_bound=refine)
        if dist:
            dist.barrier()
        walls, lat_own, lat_done, costs, launches = [], [], [], [], 0
        with ClockSampler(local_rank) as clk:
            for b in batches:
                flush.fill_(len(walls) & 0xFF)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                res = dg.solve_batch(b, use_graph=True, refine_bound=refine)
                torch.cuda.synchronize()
                walls.append(time.perf_counter() - t0)
                for r in res:
                    assert r.status == N.Status.OK, r.status
                    lat_own.append(r.latency_ms[0])
                    lat_done.append(r.latency_ms[1])
                    costs.append(r.cost)
                    launches += r.launches
        if method == "bounded":
            clocks = clk.summary()
        (wall,) = max_over_ranks([sum(walls)], dist)
        arms[method] = dict(qps=world * B * args.steps / wall, wall=wall, costs=costs, launches=launches,
                            p50=float(np.percentile(lat_own, 50)), p99=float(np.percentile(lat_own, 99)),
                            c50=float(np.percentile(lat_done, 50)), c99=float(np.percentile(lat_done, 99)))
    assert arms["plain"]["costs"] == arms["bounded"]["costs"]
    parity = parity_vs_golden(args.workload, timed_ids, timed_q, arms["bounded"]["costs"]) if rank == 0 else None
    head = arms["bounded"]
    h2d = int(np.mean([(len(q[0]) + len(q[1])) * 4 for q in queries]))
    line = {
        "metric": "GST queries/sec (batched serving, k in {3..7}, |V|=1M, exact)", "value": head["qps"],
        "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * head["wall"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generators; no public dataset)",
        "config": {"workload": args.workload, "desc": wl["desc"], "batch": B, "lanes": lanes,
                   "tuned_shift_by_k": "gst_autotune on 32 separate queries", "autotune_s": tune_s,
                   "method": METHOD_DESC["bounded"], "driver": "graph",
                   "l2": "flushed before every batch (256 MiB device write)"},
        "methods": {m: {"value": a["qps"], "latency_ms_p50": a["p50"], "latency_ms_p99": a["p99"],
                        "completion_ms_p50": a["c50"], "completion_ms_p99": a["c99"]} for m, a in arms.items()},
        "speedup_vs_plain": {"bounded": head["qps"] / arms["plain"]["qps"]},
        "latency_ms": {"p50": head["p50"], "p99": head["p99"], "note": "each query's own solve, wall clock"},
        "e2e": {"value": head["qps"], "unit": UNIT, "h2d_bytes_per_step": h2d * B, "d2h_bytes_per_step": 400 * B},
        "gpu_launches": head["launches"],
        "clocks": clocks,
        "parity": parity,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    dg.close()


def serving_subrecord(dg, g, flush, batches=2, B=64):
    """Batched serving on the bench's resident 1M graph (the serve256
    workload's graph): gst_autotune on 16 sample queries, one warm-up batch,
    then `batches` timed gst_solve_batch calls of B queries (k uniform in
    {3..7}; serve256 query indices 0 .. batches*B-1, the first ones with
    oracle costs), bound-refined method. Wall clock with the device
    synchronised on both sides."""
    import torch

    from gpu4gst_code_gb300 import native as N

    wl = dict(WORKLOADS["serve256"], name="serve256")
    sample = [make_query(wl, g, 200_000 + i) for i in range(16)]
    t = time.perf_counter()
    lanes = dg.autotune(sample, refine_bound=True)
    tune_s = time.perf_counter() - t
    ids = list(range(batches * B))
    timed_q = [make_query(wl, g, i) for i in ids]
    dg.solve_batch([make_query(wl, g, 100_000 + i) for i in range(B)], use_graph=True, refine_bound=True)
    walls, lat, costs = [], [], []
    for j in range(batches):
        flush.fill_(j & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = dg.solve_batch(timed_q[j * B:(j + 1) * B], use_graph=True, refine_bound=True)
        torch.cuda.synchronize()
        walls.append(time.perf_counter() - t0)
        for r in res:
            assert r.status == N.Status.OK, r.status
            lat.append(r.latency_ms[0])
            costs.append(r.cost)
    return {"workload": "serve256: " + wl["desc"].split(":", 1)[1].strip(), "batch": B, "batches": batches,
            "autotuned_width": lanes,
            "autotuned_width_note": "concurrent solve contexts, or queries per batch graph when those won",
            "autotune_s": tune_s, "method": METHOD_DESC["bounded"],
            "value": batches * B / sum(walls), "unit": UNIT,
            "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
            "parity": parity_vs_golden("serve256", ids, timed_q, costs)}


# ------------------------------------------------------------------ ours --
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ba1m_k6", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the batched-serving sub-record")
    ap.add_argument("--methods", default="plain,learned,bounded",
                    help="comma-separated subset of plain,learned,bounded (profiling runs); value = the last of "
                         "plain, learned, bounded present")
    ap.add_argument("--driver", default="graph", choices=["graph", "host"],
                    help="graph: one captured CUDA graph per query; host: host-launched growth rounds")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    wl = dict(WORKLOADS[args.workload], name=args.workload)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # replicas: each rank drives its own GPU with its own queries
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local_rank))

    if args.impl == "reference":
        return run_reference(args, wl)
    if "batch" in wl:
        dist = None
        if world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
        run_serving(args, wl, world, rank, local_rank, dist)
        if dist:
            dist.destroy_process_group()
        return

    import torch

    from gpu4gst_code_gb300 import native as N

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    torch.cuda.set_device(0)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    t = time.perf_counter()
    g = make_graph(wl)
    log(f"graph: V={g.V} nnz={g.nnz} ({time.perf_counter() - t:.1f}s)")
    # steps 0 .. W-1 are warm-up queries, steps W .. W+K-1 the timed ones
    # (rank 0's timed query indices are 0 .. K-1: golden oracle costs exist)
    n_total = args.warmup + args.steps
    timed_ids = list(rank_query_ids(rank, args.steps))
    queries = [make_query(wl, g, i) for i in list(warmup_query_ids(rank, args.warmup)) + timed_ids]
    t = time.perf_counter()
    dg = N.Graph(g.row_ptr, g.col, g.w)
    upload_ms = 1e3 * (time.perf_counter() - t)

    from gpu4gst_code_gb300 import learn

    scorer = N.Scorer(learn.load_params())
    use_graph = args.driver == "graph"

    def step(i, method):
        flush.fill_(i & 0xFF)
        torch.cuda.synchronize()
        gp, mem = queries[i]
        t0 = time.perf_counter()
        if method == "plain":
            r = dg.solve(gp, mem, use_graph=use_graph)
        elif method == "bounded":
            r = dg.solve(gp, mem, refine_bound=True, use_graph=use_graph)
        else:
            r = dg.solve_learned(scorer, gp, mem, use_graph=use_graph)
        wall = time.perf_counter() - t0
        assert r.status == N.Status.OK, r.status
        return r, wall

    def dev_ms(r, method):
        # a proposal that ran beside the captured DP lies inside times_ms[0]
        # (the solve's stream records its end after the proposal returned);
        # one that ran before the DP (host driver) adds its wall time
        serial = method == "learned" and not r.proposal_concurrent
        return r.times_ms[0] + (r.proposal_ms if serial else 0.0)

    arms = {}
    clocks = None
    # the last method is the line's `value`: the bound-refined DP, the fastest exact method here
    methods = [m for m in ("plain", "learned", "bounded") if m in args.methods.split(",")]
    for method in methods:
        for i in range(args.warmup):
            step(i, method)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        res = []
        with ClockSampler(local_rank) as clk:
            for i in range(args.warmup, n_total):
                res.append(step(i, method))
        torch.cuda.synchronize()
        if method == methods[-1]:
            clocks = clk.summary()
        d_ms, w_s = max_over_ranks([sum(dev_ms(r, method) for r, _ in res), sum(w for _, w in res)], dist)
        arms[method] = dict(results=res, dev_ms=d_ms, wall_s=w_s, qps=world * args.steps / (d_ms / 1e3),
                            e2e=world * args.steps / w_s)
    # Roofline pass of the growth kernels: the same plain queries with
    # statistics on, through the same driver. Per-wave CUDA events on the
    # solver's stream bracket only the growth rounds (with the CUDA-graph
    # driver they are event nodes of the query's graph, captured for solves
    # with statistics on); algorithmic bytes from the kernels' own
    # counters. Not part of `value`.
    dg.solve(*queries[0], collect_stats=True, use_graph=use_graph)  # captures the timed graph
    roof = [dg.solve(*queries[i], collect_stats=True, use_graph=use_graph) for i in range(args.warmup, n_total)]
    costs = {m: [r.cost for r, _ in a["results"]] for m, a in arms.items()}
    assert all(c == [r.cost for r in roof] for c in costs.values()), costs
    head = arms[methods[-1]]  # the metric's method: learned unless restricted
    value = head["qps"]
    grow_ms = sum(r.times_ms[1] for r in roof)
    grow_bytes = sum(r.stats["bytes"] for r in roof)
    launches = sum(r.launches for r, _ in head["results"])
    peak, peak_kind = measured_hbm_peak()
    achieved = grow_bytes / (grow_ms / 1e3) / 1e9 if grow_ms > 0 else 0.0
    sweep = sweep_bytes(g.V, g.nnz, wl["k"])
    traffic = traffic_per_step(wl)
    parity = parity_vs_golden(args.workload, timed_ids, queries[args.warmup:], costs[methods[-1]]) \
        if rank == 0 else None
    h2d = int(np.mean([(len(q[0]) + len(q[1])) * 4 for q in queries[args.warmup:]]))
    d2h = int(np.mean([64 + 4 * len(r.vertices) + 12 * len(r.edges) for r, _ in head["results"]]))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["dev_ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generators; no public dataset)",
        "config": {
            "workload": args.workload, "desc": wl["desc"], "V": g.V, "nnz": g.nnz, "k": wl["k"],
            "method": METHOD_DESC[methods[-1]],
            "driver": args.driver,
            "l2": f"flushed before every step (256 MiB device write); state table "
                  f"{table_bytes(g.V, wl['k']) / 1e6:.0f} MB > L2 (129 MB)",
            "graph_upload_ms": upload_ms, "costs": costs[methods[-1]],
        },
        "methods": {
            m: {"value": a["qps"], "ms_per_step": a["dev_ms"] / args.steps, "e2e": a["e2e"]}
            for m, a in arms.items()
        },
        "speedup_vs_plain": {m: a["qps"] / arms["plain"]["qps"] for m, a in arms.items()
                             if m != "plain" and "plain" in arms},
        "roofline": {"kernel": "growth kernels (k_grow_team dense rounds, k_grow_thread + k_grow_hubs_team "
                                 "sparse rounds; k_grow_group / k_grow_hubs for wider rows), plain method, per step",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic_per_step(wl),
                     "traffic_note": "DRAM bytes of the growth kernels per query: an ncu capture of every growth "
                                     "launch of one plain query of this workload (profiles/grow_dram_ba1m_k6.md)",
                     "algorithmic_bytes_per_step": grow_bytes / args.steps,
                     "grow_ms_per_step": grow_ms / args.steps,
                     "rounds_per_grown_wave": sum(r.stats["rounds"] for r in roof) / len(roof) / max(1, wl["k"] - 1),
                     "dram_frac": (traffic / (grow_ms / args.steps / 1e3) / 1e9 / peak) if traffic else None,
                     "one_sweep_bytes_per_step": sweep,
                     "one_sweep_frac": sweep / (grow_ms / args.steps / 1e3) / 1e9 / peak,
                     "note": "achieved = the growth kernels' own count of the bytes each round moves (every round "
                             "counted); one_sweep = the bytes of a single sweep per grown wave, which no number of "
                             "rounds changes"},
        "parity": parity,
        "e2e": {"value": head["e2e"], "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if "learned" in arms:
        lr = arms["learned"]["results"]
        line["learned_detail"] = {
            "proposal_ms_mean": float(np.mean([r.proposal_ms for r, _ in lr])),
            "proposal_concurrent": all(r.proposal_concurrent for r, _ in lr),
            "call_wall_ms_mean": float(np.mean([r.wall_ms for r, _ in lr])),
            "proposals_landed": sum(1 for r, _ in lr if r.proposal_cost > 0),
            "proposal_over_opt_mean": float(np.mean([r.proposal_cost / r.cost for r, _ in lr
                                                     if r.cost > 0 and r.proposal_cost > 0] or [0.0])),
            "final_bound_over_opt_mean": float(np.mean([r.upper_bound / r.cost for r, _ in lr if r.cost > 0])),
        }
    if rank == 0 and args.workload == "ba1m_k6" and not args.no_serving:
        line["serving"] = serving_subrecord(dg, g, flush)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle

        gp, mem = queries[args.warmup]
        t = time.perf_counter()
        ref = oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem)
        cpu_s = time.perf_counter() - t
        line["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "1 full query (the first timed one), 1 thread; the oracle's C "
                                          "restatement of the reference CPU DPBF"}
        line["parity_first_query"] = bool(ref.cost == roof[0].cost)
    if rank == 0:
        print(json.dumps(line), flush=True)
    scorer.close()
    dg.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
