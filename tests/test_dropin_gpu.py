"""The C++ drop-in DPBF_GPU (include/gst_dpbf_dropin.hpp) executed as the
reference's harness calls it (rucgraph/test_gpu.h:188-223, DPQ.cuh:57).

tests/dropin/dropin_main.cpp builds each instance's CSR with toCSR in
managed memory, calls DPBF_GPU with the harness's host_tree scratch, prints
the tree, then frees the CSR with cudaFree before building the next one
(test_gpu.h:281-283), so a later CSR can reuse the freed addresses. The
reference's own types come from the test-side stand-in tests/dropin/DPQ.cuh
(the reference checkout is not needed). Costs must equal the oracle's and
every tree must pass the reference's feasibility and cost checks.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import load_fixture
from gpu4gst_code_gb300 import native

ROOT = Path(__file__).resolve().parents[1]
DROPIN = ROOT / "tests" / "dropin"


def _compile(tmp_path) -> Path:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    native.lib()  # builds libgst.so if needed
    exe = tmp_path / "dropin_main"
    lib = native.LIB_PATH
    proc = subprocess.run([nvcc, "-std=c++17", "-O1", "-I", str(DROPIN), "-I", str(ROOT / "include"),
                           str(DROPIN / "dropin_main.cpp"), str(lib), f"-Xlinker=-rpath={lib.parent}", "-o", str(exe)],
                          capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-3000:]
    return exe


def _write_instance(path, rp, col, w, gp, mem):
    rp, col, w = np.asarray(rp), np.asarray(col), np.asarray(w)
    V = len(rp) - 1
    edges = [(u, int(col[e]), int(w[e])) for u in range(V) for e in range(rp[u], rp[u + 1]) if u < int(col[e])]
    lines = [f"{V} {len(edges)} {len(gp) - 1}"] + [f"{a} {b} {c}" for a, b, c in edges]
    for g in range(len(gp) - 1):
        m = [int(x) for x in mem[gp[g]:gp[g + 1]]]
        lines.append(" ".join(map(str, [len(m)] + m)))
    path.write_text("\n".join(lines) + "\n")


def _parse(line):
    t = line.split()
    assert t[0] == "cost" and t[2] == "states" and t[4] == "rt" and t[6] == "vertices"
    cost, states, rt, nv = int(t[1]), int(t[3]), float(t[5]), int(t[7])
    verts = [int(x) for x in t[8:8 + nv]]
    assert t[8 + nv] == "edges"
    ne = int(t[9 + nv])
    e = np.array([int(x) for x in t[10 + nv:10 + nv + 3 * ne]], np.int32).reshape(-1, 3)
    return cost, states, rt, verts, e


def test_dropin_compiles_against_standin_types(tmp_path):
    """Compiling and linking needs no GPU."""
    assert _compile(tmp_path).exists()


@pytest.mark.gpu
def test_dropin_dpbf_gpu_runs_like_the_reference_harness(tmp_path):
    exe = _compile(tmp_path)
    rp, col, w, gp, mem, cost16 = load_fixture()
    g2 = native.gen_random_connected(700, 2600, 1, 60, 91)
    gp2, mem2 = native.gen_groups_uniform(700, 4, 5, 92)
    g3 = native.gen_barabasi_albert(3000, 4, 1, 100, 93)
    gp3, mem3 = native.gen_groups_zipf_degree(g3, 5, 1.2, 5, 60, 94)
    cases = [(rp, col, w, gp, mem), (g2.row_ptr, g2.col, g2.w, gp2, mem2), (g3.row_ptr, g3.col, g3.w, gp3, mem3),
             (rp, col, w, gp, mem)]
    files = []
    for i, c in enumerate(cases):
        f = tmp_path / f"inst{i}.txt"
        _write_instance(f, *c)
        files.append(str(f))
    proc = subprocess.run([str(exe)] + files, capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-2000:]
    lines = [ln for ln in proc.stdout.splitlines() if ln.startswith("cost ")]
    assert len(lines) == len(cases), proc.stdout[-2000:]
    for (c_rp, c_col, c_w, c_gp, c_mem), ln in zip(cases, lines):
        cost, states, rt, verts, edges = _parse(ln)
        want = oracle.dpbf(c_rp, c_col, c_w, c_gp, c_mem).cost
        assert cost == want
        assert states > 0 and rt >= 0
        err = oracle.check_tree(c_rp, c_col, c_w, c_gp, c_mem, verts, edges, cost)
        assert err is None, err
    assert _parse(lines[0])[0] == cost16 == 16
