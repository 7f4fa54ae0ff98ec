"""CPU-only checks of libgst: it loads, exports every symbol the headers
declare, and rejects bad input before touching the device. No call here
launches GPU work."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from gpu4gst_code_gb300 import dpbf, native
from gpu4gst_code_gb300.native import Status

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(gst_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = native.lib()
    names = declared_functions()
    assert "gst_solve" in names and "gst_graph_upload" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    assert set(declared_functions()) <= set(native.SIGNATURES)


def test_version_string():
    assert "sm_103a" in native.version()


def _upload(rp, col, w, V=None, nnz=None):
    rp, col, w = (np.ascontiguousarray(x, np.int32) for x in (rp, col, w))
    h = C.c_void_p()
    st = native.lib().gst_graph_upload(rp.ctypes.data_as(native.I32P), col.ctypes.data_as(native.I32P),
                                       w.ctypes.data_as(native.I32P), len(rp) - 1 if V is None else V,
                                       len(col) if nnz is None else nnz, C.byref(h))
    return st, h


@pytest.mark.parametrize(
    "rp,col,w,why",
    [
        ([1, 2], [0], [1], "row_ptr[0] != 0"),
        ([0, 2, 1], [1, 0], [1, 1], "decreasing row_ptr"),
        ([0, 1, 2], [1, 5], [1, 1], "col out of range"),
        ([0, 1, 2], [1, 0], [1, -3], "negative weight"),
        ([0, 1, 2], [1, 0], [1, native.COST_LIMIT], "weight at the cost limit"),
    ],
)
def test_upload_rejects_bad_csr(rp, col, w, why):
    st, h = _upload(rp, col, w)
    assert st == Status.BAD_INPUT, why
    assert not h.value
    assert native.last_error()


def test_upload_rejects_nnz_mismatch():
    st, _ = _upload([0, 1, 2], [1, 0], [1, 1], nnz=1)
    assert st == Status.BAD_INPUT


def test_solve_rejects_null_graph():
    gp = np.array([0, 1], np.int32)
    mem = np.array([0], np.int32)
    r = C.c_void_p()
    st = native.lib().gst_solve(None, gp.ctypes.data_as(native.I32P), mem.ctypes.data_as(native.I32P), 1, None,
                                C.byref(r))
    assert st == Status.BAD_INPUT and not r.value


def test_generators_are_deterministic():
    a = native.gen_barabasi_albert(2000, 4, 1, 100, 9)
    b = native.gen_barabasi_albert(2000, 4, 1, 100, 9)
    assert np.array_equal(a.col, b.col) and np.array_equal(a.w, b.w)
    assert a.nnz == 2 * (10 + (2000 - 5) * 4)
    # symmetric, sorted rows, no self loops
    for v in range(0, 2000, 97):
        row = a.col[a.row_ptr[v]:a.row_ptr[v + 1]]
        assert np.all(np.diff(row) > 0) and v not in row
        for u in row:
            assert v in a.col[a.row_ptr[u]:a.row_ptr[u + 1]]
    gp, mem = native.gen_groups_zipf_degree(a, 6, 1.2, 5, 500, 4)
    sizes = np.diff(gp)
    assert len(sizes) == 6 and sizes.min() >= 5 and sizes.max() <= 500
    for g in range(6):
        assert len(set(mem[gp[g]:gp[g + 1]])) == sizes[g]


def test_random_connected_shape():
    g = native.gen_random_connected(1000, 5000, 1, 100, 0)
    assert g.nnz == 10000 and g.w.min() >= 1 and g.w.max() <= 100


def test_reference_mirror_helpers():
    # toCSR truncates double weights like csr_graph.hpp:46
    gv = [[(1, 2.9)], [(0, 2.9), (2, 1.5)], [(1, 1.5)]]
    csr = dpbf.toCSR(gv)
    assert list(csr.all_pointer) == [0, 1, 3, 4]
    assert list(csr.all_edge_weight) == [2, 2, 1, 1]
    s = dpbf.graph_v_of_v_idealID_DPBF_non_overlapped_group_sets_gpu(7)
    # sum over masks i of (2^(k-|i|) - 1) = 3^k - 2^(k+1) + 1 for k=3
    assert s.length == 27 - 16 + 1
    tree = dpbf.graph_hash_of_mixed_weighted()
    for v in (0, 1, 2):
        tree.add_vertex(v)
    tree.add_edge(0, 1, 2)
    tree.add_edge(1, 2, 1)
    assert dpbf.graph_hash_of_mixed_weighted_sum_of_ec(tree) == 3
    gg, gids = dpbf.group_graph_from_groups(3, [[0], [2]])
    assert dpbf.this_is_a_feasible_solution_gpu(tree, gg, gids)
    lone = dpbf.graph_hash_of_mixed_weighted()
    lone.add_vertex(0)
    assert not dpbf.this_is_a_feasible_solution_gpu(lone, gg, gids)


def test_dropin_adapter_compiles_against_reference_headers(tmp_path):
    """include/gst_dpbf_dropin.hpp defines the reference's DPBF_GPU
    (rucgraph/DPQ.cuh:57) on libgst: compile it with the reference's own
    headers and link it against libgst.so (no GPU needed to link)."""
    import shutil
    import subprocess

    import oracle

    ref = oracle.REFERENCE_ROOT / "rucgraph"
    if not (ref / "DPQ.cuh").exists() or not shutil.which("g++"):
        pytest.skip("reference headers not present")
    native.lib()
    tu = tmp_path / "dropin.cpp"
    tu.write_text('#include "DPQ.cuh"\n#include "gst_dpbf_dropin.hpp"\n'
                  "int main(){ return &DPBF_GPU != nullptr ? 0 : 1; }\n")
    cuda_inc = "/usr/local/cuda/include"
    out = tmp_path / "dropin"
    proc = subprocess.run(["g++", "-std=c++17", "-w", "-I", str(ref), "-I", cuda_inc, "-I", str(ROOT / "include"),
                           str(tu), str(native.LIB_PATH), "-o", str(out), "-lpthread"],
                          capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-2000:]


def test_tuning_cache_file_round_trip(tmp_path):
    """The tuning cache: records keyed by the graph's shape, merged into one
    file, read back exactly; a missing file, key or foreign format reads as
    no record."""
    key = native.tuning_key(1_000_000, 7_999_980, [6, 5, 6], True, True)
    assert key == "V<=2^20|deg8|k5,6|bounded|graph"
    assert native.tuning_key(1_048_576, 8_388_608, [6], False, False) == "V<=2^20|deg8|k6|plain|host"
    assert native.tuning_key(1_048_577, 8_388_608, [6], False, False).startswith("V<=2^21|")
    f = tmp_path / "t.json"
    assert native.load_tuning(f, key) is None
    a = {"dense_shift": [0] * 6 + [2] + [0] * 10, "concurrency": 4, "batch_graph": 0}
    b = {"dense_shift": [1] * 17, "concurrency": 0, "batch_graph": 8}
    native.store_tuning(f, key, a)
    native.store_tuning(f, "other", b)
    assert native.load_tuning(f, key) == a and native.load_tuning(f, "other") == b
    native.store_tuning(f, key, b)
    assert native.load_tuning(f, key) == b
    assert native.load_tuning(f, "missing") is None
    f.write_text('{"format": "something-else", "entries": {}}')
    assert native.load_tuning(f, key) is None
    assert sorted(p.name for p in tmp_path.iterdir()) == ["t.json"]  # no temporary file left
