"""The readers of the reference's dataset formats (include/gst_io.h), on
files written here in those formats (rucgraph/test_gpu.h:115-121 reads
<name>.in, <name>.g and <name>.g7)."""
import numpy as np
import pytest

from conftest import GOLDEN, load_fixture
from gpu4gst_code_gb300 import native as N


def write_in(path, g, communities=3):
    """read_input_graph's format: 'V E C', then Vertex and Edge lines."""
    lines = [f"{g.V} {g.nnz // 2} {communities}"]
    lines += [f"input_graph Vertex {v} 0 {v % communities}" for v in range(g.V)]
    for v in range(g.V):
        for e in range(g.row_ptr[v], g.row_ptr[v + 1]):
            u = int(g.col[e])
            if v < u:
                lines.append(f"input_graph Edge {v} {u} {int(g.w[e])}.000000")
    path.write_text("\n".join(lines) + "\n")


def test_graph_file_round_trip(tmp_path):
    g = N.gen_random_connected(300, 1200, 1, 100, 4)
    write_in(tmp_path / "d.in", g)
    h, C = N.read_graph_file(tmp_path / "d.in")
    assert C == 3
    assert np.array_equal(h.row_ptr, g.row_ptr)
    assert np.array_equal(h.col, g.col) and np.array_equal(h.w, g.w)


def test_groups_and_queries(tmp_path):
    V = 50
    (tmp_path / "d.g").write_text("g1:5 3 9\ng3:7 1\ng2:4 \n")
    gp, mem = N.read_groups_file(tmp_path / "d.g")
    assert gp.tolist() == [0, 3, 4, 6]
    assert mem.tolist() == [3, 5, 9, 4, 1, 7]
    # read_inquire: the last token of each line is ignored; value x -> group x - V
    (tmp_path / "d.g7").write_text(f"{V} {V + 2} \n{V + 1} {V + 2} {V}\n")
    qs = N.read_queries_file(tmp_path / "d.g7", V)
    assert qs == [[0, 2], [1, 2]]
    qgp, qmem = N.query_groups((gp, mem), qs[0])
    assert qgp.tolist() == [0, 3, 5] and qmem.tolist() == [3, 5, 9, 1, 7]


def test_bad_files_are_rejected(tmp_path):
    (tmp_path / "x.in").write_text("3 1 1\ninput_graph Edge 0 7 5\n")
    with pytest.raises(N.GSTError) as e:
        N.read_graph_file(tmp_path / "x.in")
    assert e.value.status == N.Status.BAD_INPUT and "x.in:2" in str(e.value)
    with pytest.raises(N.GSTError):
        N.read_graph_file(tmp_path / "missing.in")
    (tmp_path / "x.g").write_text("5 3 9\n")
    with pytest.raises(N.GSTError):
        N.read_groups_file(tmp_path / "x.g")


def test_gstp_instance_matches_fixture(tmp_path):
    """The fixture's arrays written back as GSTP text read identically."""
    rp, col, w, gp, mem, cost = load_fixture()
    V = len(rp) - 1
    lines = ["SECTION Comments", "END", "", "lambda 1", "", f"input_graph |V|={V} |E|={len(col) // 2}"]
    lines += [f"input_graph Vertex {v} 0" for v in range(V)]
    for v in range(V):
        for e in range(rp[v], rp[v + 1]):
            if v <= col[e]:
                lines.append(f"input_graph Edge {v} {col[e]} {w[e]}")
    for gi in range(len(gp) - 1):
        gid = V + gi
        lines.append(f"group_vertices {gid}")
        lines += [f"group_graph Edge {gid} {m} 1" for m in mem[gp[gi]:gp[gi + 1]]]
    (tmp_path / "f.text").write_text("\n".join(lines) + "\n")
    g, qgp, qmem = N.read_gstp_instance(tmp_path / "f.text")
    assert np.array_equal(g.row_ptr, rp) and np.array_equal(g.col, col) and np.array_equal(g.w, w)
    assert np.array_equal(qgp, gp) and np.array_equal(qmem, np.sort(mem) if len(gp) == 2 else qmem)
    for gi in range(len(gp) - 1):
        assert sorted(qmem[qgp[gi]:qgp[gi + 1]]) == sorted(mem[gp[gi]:gp[gi + 1]])
