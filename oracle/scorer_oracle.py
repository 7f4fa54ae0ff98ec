"""CPU oracle of the learned proposal's network (test infrastructure only).

A float64 numpy restatement of the scorer defined in include/gst_learn.h
and gpu4gst_code_gb300/csrc/learn_kernels.cu: the 16 query features, the
forward pass (h0 = relu(W0 x + b0); three layers h = relu(Ws h + Wn
mean_N(h) + b); score = wo . h3 + bo), the listwise softmax loss against a
set of tree vertices and its gradient. The GPU's fp32 training kernels and
bf16 inference kernels are checked against it. The network has no
counterpart in the reference (it is an addition), so there is nothing of
the reference to pin it to; this module pins itself against finite
differences instead (tests/test_scorer_cpu.py).

Only tests/ may import this module.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

FEAT = 16
HID = 64
LAYERS = 3
NUM_PARAMS = HID * FEAT + HID + LAYERS * (2 * HID * HID + HID) + HID + 1


def unpack(p: np.ndarray) -> dict:
    """Views into the flat parameter vector, in the library's layout."""
    p = np.asarray(p, dtype=np.float64)
    assert p.shape == (NUM_PARAMS,)
    out, o = {}, 0

    def take(name, shape):
        nonlocal o
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n

    take("W0", (HID, FEAT))
    take("b0", (HID,))
    for l in range(1, LAYERS + 1):
        take(f"Ws{l}", (HID, HID))
        take(f"Wn{l}", (HID, HID))
        take(f"b{l}", (HID,))
    take("wo", (HID,))
    take("bo", (1,))
    assert o == NUM_PARAMS
    return out


def pack(d: dict) -> np.ndarray:
    parts = [d["W0"].ravel(), d["b0"].ravel()]
    for l in range(1, LAYERS + 1):
        parts += [d[f"Ws{l}"].ravel(), d[f"Wn{l}"].ravel(), d[f"b{l}"].ravel()]
    parts += [d["wo"].ravel(), d["bo"].ravel()]
    return np.concatenate(parts)


def adjacency(row_ptr, col) -> sp.csr_matrix:
    V = len(row_ptr) - 1
    return sp.csr_matrix((np.ones(len(col)), np.asarray(col), np.asarray(row_ptr)), shape=(V, V))


def features(row_ptr, col, group_ptr, members) -> np.ndarray:
    """The 16 query features of every vertex (caller IDs)."""
    row_ptr = np.asarray(row_ptr, np.int64)
    col = np.asarray(col, np.int64)
    V = len(row_ptr) - 1
    k = len(group_ptr) - 1
    deg = np.diff(row_ptr)
    src = np.repeat(np.arange(V), deg)
    m0 = np.zeros(V, np.uint64)
    for g in range(k):
        for m in members[group_ptr[g]:group_ptr[g + 1]]:
            m0[m] |= np.uint64(1 << g)

    def reach(m):
        out = m.copy()
        np.bitwise_or.at(out, src, m[col])
        return out

    r1 = reach(m0)
    r2 = reach(r1)
    r3 = reach(r2)
    mnb = np.bincount(src, weights=(m0[col] != 0).astype(np.float64), minlength=V)

    def popc(a):
        return np.array([bin(int(x)).count("1") for x in a], np.float64)

    c0, c1, c2, c3 = popc(m0), popc(r1), popc(r2), popc(r3)
    x = np.zeros((V, FEAT))
    x[:, 0] = 1.0
    x[:, 1] = np.log1p(deg) / 8.0
    x[:, 2] = c0 / k
    x[:, 3] = c1 / k
    x[:, 4] = c2 / k
    x[:, 5] = c3 / k
    x[:, 6] = c1 == k
    x[:, 7] = c2 == k
    x[:, 8] = c3 == k
    x[:, 9] = np.where(deg > 0, mnb / np.maximum(deg, 1), 0.0)
    x[:, 10] = c0 > 0
    return x


def forward(p, A: sp.csr_matrix, x: np.ndarray):
    """Scores and the saved activations."""
    d = unpack(p)
    deg = np.asarray(A.sum(axis=1)).ravel()
    inv = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)[:, None]
    h = [np.maximum(x @ d["W0"].T + d["b0"], 0.0)]
    a = [None]
    for l in range(1, LAYERS + 1):
        al = (A @ h[-1]) * inv
        a.append(al)
        h.append(np.maximum(h[-1] @ d[f"Ws{l}"].T + al @ d[f"Wn{l}"].T + d[f"b{l}"], 0.0))
    s = h[-1] @ d["wo"] + d["bo"][0]
    return s, h, a


def loss_and_grad(p, A: sp.csr_matrix, x: np.ndarray, tree_vertices):
    """Listwise loss -(1/n) sum_{v in T} log softmax(s)_v and its gradient."""
    d = unpack(p)
    s, h, a = forward(p, A, x)
    V = len(s)
    y = np.zeros(V)
    y[np.unique(np.asarray(tree_vertices))] = 1.0
    n = y.sum()
    m = s.max()
    e = np.exp(s - m)
    lse = m + np.log(e.sum())
    loss = -np.sum((s - lse) * y) / n
    ds = e / e.sum() - y / n
    deg = np.asarray(A.sum(axis=1)).ravel()
    inv = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)[:, None]
    g = {k: np.zeros_like(v) for k, v in d.items()}
    g["wo"] = ds @ h[LAYERS]
    g["bo"] = np.array([ds.sum()])
    dz = np.outer(ds, d["wo"]) * (h[LAYERS] > 0)
    for l in range(LAYERS, 0, -1):
        g[f"Ws{l}"] = dz.T @ h[l - 1]
        g[f"Wn{l}"] = dz.T @ a[l]
        g[f"b{l}"] = dz.sum(axis=0)
        dh = dz @ d[f"Ws{l}"] + A.T @ ((dz @ d[f"Wn{l}"]) * inv)
        dz = dh * (h[l - 1] > 0)
    g["W0"] = dz.T @ x
    g["b0"] = dz.sum(axis=0)
    return loss, pack(g)
