"""Training and use of the learned upper-bound proposal (include/gst_learn.h).

The proposal network is trained on optimal trees that the plain GPU DPBF
itself produces: each step solves one synthetic query exactly, then takes
one Adam step of the device's fp32 forward/backward kernels against the
vertices of that optimal tree (listwise softmax loss). Everything runs
through libgst.so; this module only drives it.

    python -m gpu4gst_code_gb300.learn --instances 20000 --out weights/scorer_ba.npy

Defaults follow the training set of the learned-bound workload: Barabasi-
Albert graphs m=4, |V|=100,000, weights U[1,100]; k uniform in {4,5,6};
group sizes Zipf(1.2) clipped to [5,500], members degree-proportional.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import native as N

WEIGHTS_DIR = Path(__file__).resolve().parent / "weights"
DEFAULT_WEIGHTS = WEIGHTS_DIR / "scorer_ba.npy"


def init_params(seed: int = 0) -> np.ndarray:
    """Glorot-uniform weights, zero biases, in the library's flat layout."""
    rng = np.random.default_rng(seed)
    F, H = N.SCORER_FEATURES, N.SCORER_HIDDEN

    def glorot(fan_out, fan_in):
        lim = np.sqrt(6.0 / (fan_in + fan_out))
        return rng.uniform(-lim, lim, size=(fan_out, fan_in))

    parts = [glorot(H, F).ravel(), np.zeros(H)]
    for _ in range(3):
        parts += [glorot(H, H).ravel(), glorot(H, H).ravel(), np.zeros(H)]
    parts += [glorot(1, H).ravel(), np.zeros(1)]
    p = np.concatenate(parts).astype(np.float32)
    assert p.shape == (N.SCORER_NUM_PARAMS,)
    return p


def load_params(path: Path | str = DEFAULT_WEIGHTS) -> np.ndarray:
    p = np.load(path).astype(np.float32)
    if p.shape != (N.SCORER_NUM_PARAMS,):
        raise ValueError(f"{path}: expected {N.SCORER_NUM_PARAMS} parameters, got {p.shape}")
    return p


def make_query(g: N.CSR, k: int, seed: int, s: float = 1.2, lo: int = 5, hi: int = 500):
    return N.gen_groups_zipf_degree(g, k, s, lo, hi, seed)


def train(instances: int = 20000, V: int = 100_000, graphs: int = 8, ks=(4, 5, 6), lr: float = 1e-3,
          seed: int = 7, params: np.ndarray | None = None, log_every: int = 500, verbose: bool = True):
    """Trains a scorer on `instances` DP-solved queries spread over `graphs`
    resident graphs; returns (params, log)."""
    rng = np.random.default_rng(seed)
    p0 = init_params(seed) if params is None else params
    csrs = [N.gen_barabasi_albert(V, 4, 1, 100, 1000 + seed * 100 + i) for i in range(graphs)]
    dgs = [N.Graph(c.row_ptr, c.col, c.w) for c in csrs]
    log = []
    t0 = time.time()
    losses = []
    with N.Scorer(p0) as sc:
        for it in range(instances):
            gi = int(rng.integers(graphs))
            k = int(rng.choice(ks))
            gp, mem = make_query(csrs[gi], k, int(rng.integers(1 << 62)))
            res = dgs[gi].solve(gp, mem, use_graph=True)
            if res.status != N.Status.OK or len(res.vertices) == 0:
                continue
            loss, _ = sc.train_step(dgs[gi], gp, mem, res.vertices, lr=lr)
            losses.append(loss)
            if verbose and (it + 1) % log_every == 0:
                entry = {"step": it + 1, "loss": float(np.mean(losses[-log_every:])), "s": round(time.time() - t0, 1)}
                log.append(entry)
                print(json.dumps(entry), flush=True)
        params = sc.params()
    for d in dgs:
        d.close()
    return params, log


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--instances", type=int, default=20000)
    ap.add_argument("--V", type=int, default=100_000)
    ap.add_argument("--graphs", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", type=Path, default=DEFAULT_WEIGHTS)
    a = ap.parse_args()
    params, log = train(a.instances, a.V, a.graphs, lr=a.lr, seed=a.seed)
    a.out.parent.mkdir(parents=True, exist_ok=True)
    np.save(a.out, params)
    meta = {"instances": a.instances, "V": a.V, "graphs": a.graphs, "lr": a.lr, "seed": a.seed, "log": log}
    a.out.with_suffix(".json").write_text(json.dumps(meta, indent=1))
    print(f"saved {a.out}")


if __name__ == "__main__":
    main()
