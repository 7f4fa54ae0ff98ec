"""GPU checks of the learned proposal through the C ABI (gst_learn.h):
fp32 forward and gradients of the device training kernels against the
numpy oracle, bf16 inference against the same, feasibility of the proposed
tree, and exactness of the proposal-pruned solve."""
import numpy as np
import pytest

import oracle
from oracle import scorer_oracle as SO

pytestmark = pytest.mark.gpu


def ba_case(V=3000, k=4, seed=0):
    from gpu4gst_code_gb300 import native as N

    g = N.gen_barabasi_albert(V, 4, 1, 100, seed)
    gp, mem = N.gen_groups_zipf_degree(g, k, 1.2, 5, 60, seed + 11)
    return g, gp, mem


def rel_err(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12))


@pytest.fixture(scope="module")
def case():
    from gpu4gst_code_gb300 import learn, native as N

    g, gp, mem = ba_case()
    p = learn.init_params(1)
    with N.Graph(g.row_ptr, g.col, g.w) as dg:
        tree = dg.solve(gp, mem).vertices
    A = SO.adjacency(g.row_ptr, g.col)
    x = SO.features(g.row_ptr, g.col, gp, mem)
    return g, gp, mem, p, tree, A, x


def test_fp32_scores_match_oracle(case):
    from gpu4gst_code_gb300 import native as N

    g, gp, mem, p, tree, A, x = case
    want, _, _ = SO.forward(p.astype(np.float64), A, x)
    with N.Graph(g.row_ptr, g.col, g.w) as dg, N.Scorer(p) as sc:
        got = sc.scores(dg, gp, mem, fp32=True)
    assert np.abs(got - want).max() <= 1e-4 * (1 + np.abs(want).max())


def test_bf16_inference_tracks_oracle(case):
    from gpu4gst_code_gb300 import native as N

    g, gp, mem, p, tree, A, x = case
    want, _, _ = SO.forward(p.astype(np.float64), A, x)
    with N.Graph(g.row_ptr, g.col, g.w) as dg, N.Scorer(p) as sc:
        got = sc.scores(dg, gp, mem)
    # bf16 keeps 8 significant bits: errors stay within a few percent of the score range
    assert np.abs(got - want).max() <= 0.03 * (np.abs(want).max() + 1e-6)
    assert np.corrcoef(got, want)[0, 1] > 0.999


@pytest.mark.parametrize("V", [60, 128, 1000])
def test_bf16_inference_on_partial_and_whole_tiles(V):
    """The layer GEMM works on 128-vertex tiles: one partial tile (V=60), one
    whole tile (128) and a partial last tile (1000 = 7 x 128 + 104) score
    like the oracle."""
    from gpu4gst_code_gb300 import learn, native as N

    g, gp, mem = ba_case(V=V, k=3, seed=V)
    p = learn.init_params(V)
    want, _, _ = SO.forward(p.astype(np.float64), SO.adjacency(g.row_ptr, g.col), SO.features(g.row_ptr, g.col, gp, mem))
    with N.Graph(g.row_ptr, g.col, g.w) as dg, N.Scorer(p) as sc:
        got = sc.scores(dg, gp, mem)
    assert np.abs(got - want).max() <= 0.03 * (np.abs(want).max() + 1e-6)
    assert np.corrcoef(got, want)[0, 1] > 0.999


def test_gradients_match_oracle(case):
    from gpu4gst_code_gb300 import native as N

    g, gp, mem, p, tree, A, x = case
    want_loss, want = SO.loss_and_grad(p.astype(np.float64), A, x, tree)
    with N.Graph(g.row_ptr, g.col, g.w) as dg, N.Scorer(p) as sc:
        loss, got = sc.train_step(dg, gp, mem, tree, apply=False, want_grads=True)
        assert np.array_equal(sc.params(), p)  # apply=False leaves the parameters
    assert abs(loss - want_loss) <= 1e-4 * max(1.0, abs(want_loss))
    gd, wd = SO.unpack(got), SO.unpack(want)
    floor = 1e-5 * np.linalg.norm(want)  # d/d bo is exactly 0 (softmax sums to one): fp32 leaves ~1e-7
    for name in wd:
        err = np.linalg.norm(gd[name] - wd[name])
        assert err <= 2e-3 * np.linalg.norm(wd[name]) + floor, (name, err)


def test_adam_step_matches_numpy(case):
    from gpu4gst_code_gb300 import native as N

    g, gp, mem, p, tree, A, x = case
    lr = 1e-3
    with N.Graph(g.row_ptr, g.col, g.w) as dg, N.Scorer(p) as sc:
        _, grad = sc.train_step(dg, gp, mem, tree, lr=lr, apply=True, want_grads=True)
        got = sc.params()
    grad = grad.astype(np.float64)
    m = 0.1 * grad  # first step from zero moments
    v = 0.001 * grad * grad
    want = p - lr * (m / 0.1) / (np.sqrt(v / 0.001) + 1e-8)
    assert np.abs(got - want).max() <= 1e-6


@pytest.mark.parametrize("use_scorer", [False, True])
def test_proposal_is_feasible_and_learned_solve_exact(use_scorer):
    from gpu4gst_code_gb300 import learn, native as N

    for seed in range(6):
        k = 3 + seed % 4
        g, gp, mem = ba_case(V=2000 + 500 * seed, k=k, seed=100 + seed)
        with N.Graph(g.row_ptr, g.col, g.w) as dg, N.Scorer(learn.init_params(seed)) as sc:
            s = sc if use_scorer else None
            plain = dg.solve(gp, mem, use_graph=True)
            assert plain.cost == oracle.dpbf(g.row_ptr, g.col, g.w, gp, mem).cost
            prop = dg.propose(s, gp, mem)
            assert prop.status == N.Status.OK
            err = oracle.check_tree(g.row_ptr, g.col, g.w, gp, mem, prop.vertices, prop.edges, prop.cost)
            assert err is None, err
            assert prop.cost >= plain.cost
            # host driver: the proposal first, then the DP under its bound
            seq = dg.solve_learned(s, gp, mem, use_graph=False)
            assert seq.status == N.Status.OK and seq.cost == plain.cost and not seq.proposal_concurrent
            # a proposal's root distances stop after a fixed number of rounds, so two proposals of
            # one query may differ (in-place updates run in no fixed order); each is a feasible tree
            assert seq.proposal_cost >= plain.cost
            # the refined bound only drops from the proposal's cost, and stays a feasible cost (a
            # zero-cost tree leaves it unchanged: 0 would read as "no bound")
            assert plain.cost <= seq.upper_bound <= seq.proposal_cost
            # captured: the proposal runs beside the DP; its bound lands unless the DP finished first
            res = dg.solve_learned(s, gp, mem)
            assert res.status == N.Status.OK and res.cost == plain.cost and res.proposal_concurrent
            assert res.wall_ms > 0 and res.times_ms[0] > 0
            assert res.proposal_cost == 0 or res.proposal_cost >= plain.cost
            if res.proposal_cost:
                assert res.upper_bound <= res.proposal_cost
            assert res.upper_bound >= plain.cost or res.upper_bound == 0  # 0: no bound was found
            for r in (seq, res):
                err = oracle.check_tree(g.row_ptr, g.col, g.w, gp, mem, r.vertices, r.edges, r.cost)
                assert err is None, err


def test_trained_network_gains_over_the_method_without_it():
    """The committed weights (trained on DP-solved queries, see
    gpu4gst_code_gb300/weights/scorer_ba.json) propose tighter bounds on
    held-out queries than the same pipeline without a network (fixed
    feature score) and than the untrained network; every solve stays exact."""
    from gpu4gst_code_gb300 import learn, native as N

    g = N.gen_barabasi_albert(100_000, 4, 1, 100, 4242)  # a graph not trained on
    rng = np.random.default_rng(5)
    ratios = {"trained": [], "none": [], "untrained": []}
    with N.Graph(g.row_ptr, g.col, g.w) as dg, N.Scorer(learn.load_params()) as tr, \
            N.Scorer(learn.init_params(0)) as un:
        for q in range(24):
            k = int(rng.choice([4, 5, 6]))
            gp, mem = N.gen_groups_zipf_degree(g, k, 1.2, 5, 500, 90_000 + q)
            opt = dg.solve(gp, mem, use_graph=True).cost
            for name, sc in (("trained", tr), ("none", None), ("untrained", un)):
                # the host driver proposes before it solves: every proposal is complete
                res = dg.solve_learned(sc, gp, mem, use_graph=False)
                assert res.cost == opt
                assert res.proposal_cost >= opt
                ratios[name].append(res.proposal_cost / opt)
    mean = {k: float(np.mean(v)) for k, v in ratios.items()}
    assert mean["trained"] < mean["none"] and mean["trained"] < mean["untrained"], mean


def test_layer_wait_that_runs_out_reports_and_leaves_the_device_usable(case):
    """The layer GEMM's waits are bounded: a first tile that waits for 16
    bytes more than its TMA loads deliver runs its wait out (about a second
    at most), the layer reports it through its error flag (GST_INTERNAL,
    flag 1), and the next inference on the same graph scores like the
    oracle."""
    import ctypes as C

    from gpu4gst_code_gb300 import native as N

    g, gp, mem, p, tree, A, x = case
    want, _, _ = SO.forward(p.astype(np.float64), A, x)
    with N.Graph(g.row_ptr, g.col, g.w) as dg, N.Scorer(p) as sc:
        flag = C.c_int32(-1)
        st = N.lib().gst_debug_scorer_wait_timeout(dg._h, sc._h, 0, C.byref(flag))
        assert N.Status(st) == N.Status.OK and flag.value == 0
        st = N.lib().gst_debug_scorer_wait_timeout(dg._h, sc._h, 16, C.byref(flag))
        assert N.Status(st) == N.Status.INTERNAL and flag.value == 1
        got = sc.scores(dg, gp, mem)
    assert np.abs(got - want).max() <= 0.03 * (np.abs(want).max() + 1e-6)

