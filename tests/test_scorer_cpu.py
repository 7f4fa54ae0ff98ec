"""CPU checks of the learned proposal: the numpy oracle of the network
against finite differences, and the parameter layout shared by the header,
the bindings and the oracle."""
import re

import numpy as np
import pytest

from conftest import ROOT
from oracle import scorer_oracle as SO


def small_case(seed=0, V=40, k=3):
    from gpu4gst_code_gb300 import native as N

    g = N.gen_random_connected(V, 3 * V, 1, 100, seed)
    gp, mem = N.gen_groups_uniform(V, k, 4, seed + 1)
    return g, gp, mem


def test_layout_constants():
    from gpu4gst_code_gb300 import native as N

    hdr = (ROOT / "include" / "gst_learn.h").read_text()
    n = int(re.search(r"#define GST_SCORER_NUM_PARAMS (\d+)", hdr).group(1))
    assert n == SO.NUM_PARAMS == N.SCORER_NUM_PARAMS
    assert int(re.search(r"#define GST_SCORER_FEATURES (\d+)", hdr).group(1)) == SO.FEAT
    assert int(re.search(r"#define GST_SCORER_HIDDEN (\d+)", hdr).group(1)) == SO.HID
    p = np.arange(SO.NUM_PARAMS, dtype=np.float64)
    assert np.array_equal(SO.pack(SO.unpack(p)), p)


def test_init_params():
    from gpu4gst_code_gb300 import learn

    p = learn.init_params(3)
    assert p.dtype == np.float32 and p.shape == (SO.NUM_PARAMS,)
    d = SO.unpack(p)
    assert np.all(d["b0"] == 0) and np.abs(d["W0"]).max() > 0


def test_features_match_definition():
    g, gp, mem = small_case()
    x = SO.features(g.row_ptr, g.col, gp, mem)
    V = g.V
    assert x.shape == (V, SO.FEAT)
    assert np.all(x[:, 0] == 1) and np.all(x[:, 11:] == 0)
    # a member has its own group within 0, 1, 2, 3 hops
    for gi in range(len(gp) - 1):
        for m in mem[gp[gi]:gp[gi + 1]]:
            assert x[m, 2] > 0 and x[m, 10] == 1
    assert np.all(x[:, 3] <= x[:, 4]) and np.all(x[:, 4] <= x[:, 5])


def test_oracle_gradient_matches_finite_differences():
    g, gp, mem = small_case(seed=5)
    A = SO.adjacency(g.row_ptr, g.col)
    x = SO.features(g.row_ptr, g.col, gp, mem)
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, SO.NUM_PARAMS)
    tree = rng.choice(g.V, 6, replace=False)
    loss, grad = SO.loss_and_grad(p, A, x, tree)
    assert np.isfinite(loss)
    idx = rng.choice(SO.NUM_PARAMS, 60, replace=False)
    # every output-side parameter too
    idx = np.unique(np.concatenate([idx, np.arange(SO.NUM_PARAMS - SO.HID - 1, SO.NUM_PARAMS)]))
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp, _ = SO.loss_and_grad(q, A, x, tree)
        q[i] -= 2 * eps
        lm, _ = SO.loss_and_grad(q, A, x, tree)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - grad[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, grad[i])
