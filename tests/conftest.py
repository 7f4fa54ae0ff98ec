import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden():
    return json.loads((GOLDEN / "golden.json").read_text())


def load_fixture():
    d = np.load(GOLDEN / "simple_iterative.npz")
    return d["row_ptr"], d["col"], d["w"], d["group_ptr"], d["members"], int(d["cost"])


def load_edge_cases():
    d = np.load(GOLDEN / "edge_cases.npz")
    cases = {}
    for key in d.files:
        name, field = key.split("__")
        cases.setdefault(name, {})[field] = d[key]
    return cases


def make_instance(case):
    """Regenerates a golden.json instance with the project's generators."""
    from gpu4gst_code_gb300 import native as N

    kind, *a = case["graph"]
    g = N.gen_random_connected(*a) if kind == "random_connected" else N.gen_barabasi_albert(*a)
    qk, *q = case["groups"]
    if qk == "uniform":
        k, size, seed = q
        gp, mem = N.gen_groups_uniform(g.V, k, size, seed)
    else:
        k, s, lo, hi, seed = q
        gp, mem = N.gen_groups_zipf_degree(g, k, s, lo, hi, seed)
    return g, gp, mem


@pytest.fixture(scope="session")
def golden():
    return load_golden()
