"""The tour lower bound of the pruned solves, restated in numpy and checked on
exact oracle tables (CPU only).

The solver caps a state (v, S) of waves 2..k-1 at UB - LB(v, X), X = the
groups outside S, where LB is the larger of the one-label bound and
PrunedDP++'s tour bound (rucgraph/graph_v_of_v_idealID_PrunedDPPlusPlus.h:
268-386; computed by k_tour_table and k_merge_staged). T(v, X) of the exact
table is the cheapest tree that contains v and touches every group of X, so
a valid bound satisfies LB(v, X) <= T(v, X) for every v and X, whatever UB
caps the wave-1 distances with. This pins the bound's formula: group-to-group
legs as the smallest capped member distance, made symmetric by the larger of
the two directions, the path table over subsets clamped at UB, and half the
cheapest walk from v through X back to v.
"""
import numpy as np
import pytest

import oracle


def tour_tables(d, group_ptr, members, ub):
    """(D, F): capped group-to-group legs and path[i][X][j], as k_tour_table builds them."""
    k = d.shape[1]
    beyond = ub // 2 + 1
    dc = np.minimum(d, beyond)
    D = np.full((k, k), beyond, np.int64)
    for b in range(k):
        ms = members[group_ptr[b]:group_ptr[b + 1]]
        D[:, b] = np.minimum(D[:, b], dc[ms].min(axis=0))
    D = np.maximum(D, D.T)
    W = 1 << k
    F = np.full((k, W, k), ub, np.int64)
    for i in range(k):
        F[i, 1 << i, i] = 0
    for p in range(2, k + 1):
        for X in range(W):
            if bin(X).count("1") != p:
                continue
            for i in range(k):
                for j in range(k):
                    if i == j or not (X >> i) & 1 or not (X >> j) & 1:
                        continue
                    prev = X ^ (1 << j)
                    best = ub
                    for l in range(k):
                        if (prev >> l) & 1:
                            best = min(best, F[i, prev, l] + D[l, j])
                    F[i, X, j] = best
    return dc, F


def path_from(F, X):
    """W2[i] = the cheapest order visiting every group of X from group i,
    ending anywhere: min over j != i of path[i][X][j] (0 when X = {i})."""
    k = F.shape[0]
    gs = [g for g in range(k) if (X >> g) & 1]
    out = {}
    for i in gs:
        out[i] = 0 if len(gs) == 1 else min(int(F[i, X, j]) for j in gs if j != i)
    return out


def second_bound(dc, F, X):
    """PrunedDP++'s lb2 (graph_v_of_v_idealID_PrunedDPPlusPlus.h:454-466):
    max over i in X of (d(v,i) + W2[i][X] + min_j d(v,j)) / 2."""
    gs = [g for g in range(dc.shape[1]) if (X >> g) & 1]
    w2 = path_from(F, X)
    dmin = dc[:, gs].min(axis=1)
    lb = np.zeros(dc.shape[0], np.int64)
    for i in gs:
        lb = np.maximum(lb, (dc[:, i] + w2[i] + dmin) // 2)
    return lb


def lower_bound(dc, F, X, pairs_only=False):
    """LB(v, X) for every v: max(one-label, tour) as the merge takes it.
    pairs_only: the end groups as unordered pairs i < j, which is what the
    merge evaluates: the path table is symmetric, and its i = j entries are
    not walks (they hold the clamp), so leaving them out keeps the bound
    valid and can only raise it."""
    gs = [g for g in range(dc.shape[1]) if (X >> g) & 1]
    lb = dc[:, gs].max(axis=1)
    if len(gs) >= 2:
        tour = np.full(dc.shape[0], np.iinfo(np.int64).max)
        for a, i in enumerate(gs):
            for j in (gs[a + 1:] if pairs_only else gs):
                tour = np.minimum(tour, (dc[:, i] + F[i, X, j] + dc[:, j]) // 2)
        lb = np.maximum(lb, tour)
    return lb


def instance(kind, V, k, seed):
    from gpu4gst_code_gb300 import native as N

    if kind == "ba":
        g = N.gen_barabasi_albert(V, 3, 1, 100, seed)
        gp, mem = N.gen_groups_zipf_degree(g, k, 1.2, 3, 40, seed + 7)
    else:
        g = N.gen_random_connected(V, 4 * V, 1, 100, seed)
        gp, mem = N.gen_groups_uniform(V, k, 6, seed + 7)
    return g, np.asarray(gp, np.int64), np.asarray(mem, np.int64)


@pytest.mark.parametrize("kind,V,k,seed", [("ba", 1500, 5, 1), ("ba", 1200, 6, 2), ("rc", 800, 5, 3)])
def test_tour_bound_never_exceeds_the_cheapest_completion(kind, V, k, seed):
    g, gp, mem = instance(kind, V, k, seed)
    T = oracle.dp_table(g.row_ptr, g.col, g.w, gp, mem).astype(np.int64)
    full = (1 << k) - 1
    opt = int(T[:, full].min())
    assert 0 < opt < oracle.INF
    d = T[:, [1 << i for i in range(k)]]
    stronger = 0
    for ub in (opt, 2 * opt, 1 << 29):  # any bound caps the distances validly
        dc, F = tour_tables(d, gp, mem, ub)
        # the path table is symmetric: the cheapest order from i to j reversed
        assert np.array_equal(F, F.transpose(2, 1, 0))
        for X in range(1, full + 1):
            lb_all = lower_bound(dc, F, X)
            lb = lower_bound(dc, F, X, pairs_only=True)
            assert np.all(lb >= lb_all)
            lb = np.maximum(lb, second_bound(dc, F, X))
            t = T[:, X]
            fin = t < oracle.INF
            assert np.all(lb[fin] <= t[fin]), (ub, X, int(np.argmax(lb - np.where(fin, t, 0))))
            stronger += int(np.sum(lb[fin] > dc[fin][:, [g for g in range(k) if (X >> g) & 1]].max(axis=1)))
    assert stronger > 0  # the tour bound is tighter than the one-label bound somewhere
