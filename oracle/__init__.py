"""CPU oracle for the GST path — TEST INFRASTRUCTURE, not part of the product.

Two checkers, both loaded with ctypes:
  * liboracle.so  — the project's plain-C restatement (dpbf_oracle.c) of the
    reference's CPU DPBF (rucgraph/graph_v_of_v_idealID_DPBF_only_ec.h:133)
    and of the layered DP (src/DP.cu:102-215). Built here and on any host
    with gcc.
  * libref_dpbf.so — the reference's own CPU solvers compiled from their
    unmodified headers (build_ref.sh). Only where the reference checkout
    exists; used to pin the restatement and to make tests/golden.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may import
this package. The product library never calls into it.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import platform
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE.parent / "_build" / "oracle"
ORACLE_LIB = BUILD_DIR / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_dpbf.so"
# The reference checkout: $GST_REFERENCE_ROOT, else a directory named
# "reference" beside this repository's checkout. Absent on hosts that only
# run the built library; everything that needs it is skipped there.
REFERENCE_ROOT = Path(os.environ["GST_REFERENCE_ROOT"]) if os.environ.get("GST_REFERENCE_ROOT") \
    else HERE.parent.parent / "reference"
GEN_LIB = BUILD_DIR / "liboracle_gen.so"
GEN_SRC = HERE.parent / "gpu4gst_code_gb300" / "csrc" / "gen.cpp"
GEN_INCLUDE = HERE.parent / "include"

INF = 2**31 - 1
I32P = C.POINTER(C.c_int32)
I64P = C.POINTER(C.c_int64)
F64P = C.POINTER(C.c_double)

OK, INFEASIBLE, STOPPED = 0, 1, 2


def _stamp_ok(out: Path, inputs: list[Path], flags: list[str]) -> tuple[bool, str]:
    """(out is current, digest): a SHA-256 of the inputs, the flags and the
    host architecture, kept in <out>.sha256."""
    h = hashlib.sha256(" ".join(flags + [platform.machine()]).encode())
    for p in inputs:
        h.update(p.read_bytes())
    d = h.hexdigest()
    stamp = out.with_suffix(out.suffix + ".sha256")
    return out.exists() and stamp.exists() and stamp.read_text().strip() == d, d


def _build_so(out: Path, cmd: list[str], inputs: list[Path], force: bool) -> Path:
    ok, d = _stamp_ok(out, inputs, cmd)
    if ok and not force:
        return out
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    tmp = out.with_suffix(f".so.{os.getpid()}.tmp")  # concurrent builders never share a temporary
    subprocess.run(cmd + ["-o", str(tmp)], check=True)
    os.replace(tmp, out)
    out.with_suffix(out.suffix + ".sha256").write_text(d + "\n")
    return out


def build_oracle(force: bool = False) -> Path:
    src = HERE / "dpbf_oracle.c"
    cc = shutil.which("gcc") or "cc"
    return _build_so(ORACLE_LIB, [cc, "-O2", "-std=c11", "-shared", "-fPIC", str(src)], [src], force)


def build_gen(force: bool = False) -> Path:
    """The seeded instance generators (the same source the product library
    compiles, include/gst_gen.h) as a library of their own, so that the
    reference arm of the benchmark builds its instances without loading the
    product library."""
    cxx = shutil.which("g++") or "c++"
    return _build_so(GEN_LIB, [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(GEN_INCLUDE), str(GEN_SRC)],
                     [GEN_SRC, GEN_INCLUDE / "gst_gen.h"], force)


def build_ref(force: bool = False) -> Path | None:
    """Builds oracle/_ref from the reference checkout when it is present."""
    if not (REFERENCE_ROOT / "rucgraph" / "graph_v_of_v_idealID_DPBF_only_ec.h").exists():
        return None
    deps = [HERE / "ref" / "ref_dpbf.cpp", *sorted((HERE / "ref" / "shim").rglob("*.hpp"))]
    if not force and REF_LIB.exists() and all(REF_LIB.stat().st_mtime >= p.stat().st_mtime for p in deps):
        return REF_LIB
    subprocess.run(["sh", str(HERE / "build_ref.sh"), str(REFERENCE_ROOT)], check=True, capture_output=True)
    return REF_LIB


_ORC = None
_REF = None


def lib() -> C.CDLL:
    global _ORC
    if _ORC is None:
        dll = C.CDLL(str(build_oracle()))
        dll.oracle_dpbf.restype = C.c_int
        dll.oracle_dpbf.argtypes = [C.c_int32, I64P, I32P, I32P, C.c_int32, I32P, I32P, C.c_int64, I32P, I32P,
                                    I32P, I32P, I32P, I32P, C.c_int32, I64P]
        dll.oracle_dp_table.restype = C.c_int
        dll.oracle_dp_table.argtypes = [C.c_int32, I64P, I32P, I32P, C.c_int32, I32P, I32P, I32P]
        dll.oracle_one_label_lb.restype = C.c_int
        dll.oracle_one_label_lb.argtypes = [C.c_int32, I64P, I32P, I32P, C.c_int32, I32P, I32P, I32P]
        _ORC = dll
    return _ORC


def ref_lib() -> C.CDLL | None:
    global _REF
    if _REF is None:
        if not REF_LIB.exists():
            build_ref()
        if not REF_LIB.exists():
            return None
        dll = C.CDLL(str(REF_LIB))
        for name in ("ref_dpbf_only_ec", "ref_pruned_dp_pp"):
            fn = getattr(dll, name)
            fn.restype = C.c_int
            fn.argtypes = [C.c_int32, I64P, I32P, F64P, C.c_int32, I32P, I32P, I32P, I32P, I32P, I32P, I32P,
                           C.c_int32]
        _REF = dll
    return _REF


def _p(a, t=I32P):
    return a.ctypes.data_as(t)


def _csr64(row_ptr):
    return np.ascontiguousarray(row_ptr, dtype=np.int64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class OracleResult:
    def __init__(self, status, cost, root, vertices, edges, pops):
        self.status, self.cost, self.root = status, cost, root
        self.vertices, self.edges, self.pops = vertices, edges, pops


def dpbf(row_ptr, col, w, group_ptr, members, max_pops: int = 0, cap: int | None = None) -> OracleResult:
    """C restatement of graph_v_of_v_idealID_DPBF_only_ec."""
    L = lib()
    rp, c, ww, gp, mem = _csr64(row_ptr), _i32(col), _i32(w), _i32(group_ptr), _i32(members)
    V = len(rp) - 1
    k = len(gp) - 1
    if cap is None:
        cap = 4 * V + 64
    cost, root, nv, ne = (C.c_int32(-1) for _ in range(4))
    pops = C.c_int64(0)
    vv = np.zeros(cap, np.int32)
    ee = np.zeros(3 * cap, np.int32)
    st = L.oracle_dpbf(V, _p(rp, I64P), _p(c), _p(ww), k, _p(gp), _p(mem), max_pops, C.byref(cost), C.byref(root),
                       _p(vv), C.byref(nv), _p(ee), C.byref(ne), cap, C.byref(pops))
    if st not in (OK, INFEASIBLE, STOPPED):
        raise RuntimeError(f"oracle_dpbf failed with status {st}")
    if st != OK:
        return OracleResult(st, -1, -1, np.zeros(0, np.int32), np.zeros((0, 3), np.int32), pops.value)
    return OracleResult(st, cost.value, root.value, vv[: nv.value].copy(), ee[: 3 * ne.value].reshape(-1, 3).copy(),
                        pops.value)


def dp_table(row_ptr, col, w, group_ptr, members) -> np.ndarray:
    """Exact fixpoint T(v,S) as a (V, 2^k) int32 array (INF where absent)."""
    L = lib()
    rp, c, ww, gp, mem = _csr64(row_ptr), _i32(col), _i32(w), _i32(group_ptr), _i32(members)
    V, k = len(rp) - 1, len(gp) - 1
    t = np.zeros(V * (1 << k), np.int32)
    st = L.oracle_dp_table(V, _p(rp, I64P), _p(c), _p(ww), k, _p(gp), _p(mem), _p(t))
    if st != OK:
        raise RuntimeError(f"oracle_dp_table failed with status {st}")
    return t.reshape(V, 1 << k)


def one_label_lb(row_ptr, col, w, group_ptr, members) -> np.ndarray:
    L = lib()
    rp, c, ww, gp, mem = _csr64(row_ptr), _i32(col), _i32(w), _i32(group_ptr), _i32(members)
    V, k = len(rp) - 1, len(gp) - 1
    out = np.zeros(V, np.int32)
    st = L.oracle_one_label_lb(V, _p(rp, I64P), _p(c), _p(ww), k, _p(gp), _p(mem), _p(out))
    if st != OK:
        raise RuntimeError(f"oracle_one_label_lb failed with status {st}")
    return out


def reference(row_ptr, col, w, group_ptr, members, solver: str = "dpbf") -> OracleResult | None:
    """The reference's own solver (None when oracle/_ref is unavailable).
    `w` may be float: the reference truncates to int itself."""
    R = ref_lib()
    if R is None:
        return None
    fn = R.ref_dpbf_only_ec if solver == "dpbf" else R.ref_pruned_dp_pp
    rp, c, gp, mem = _csr64(row_ptr), _i32(col), _i32(group_ptr), _i32(members)
    ww = np.ascontiguousarray(w, dtype=np.float64)
    V, k = len(rp) - 1, len(gp) - 1
    cap = V + 16
    cost, nv, ne = C.c_int32(-1), C.c_int32(0), C.c_int32(0)
    vv = np.zeros(cap, np.int32)
    ee = np.zeros(3 * cap, np.int32)
    st = fn(V, _p(rp, I64P), _p(c), _p(ww, F64P), k, _p(gp), _p(mem), C.byref(cost), C.byref(nv), _p(vv),
            C.byref(ne), _p(ee), cap)
    if st not in (OK, INFEASIBLE):
        raise RuntimeError(f"reference solver failed with status {st}")
    if st == INFEASIBLE:
        return OracleResult(st, -1, -1, np.zeros(0, np.int32), np.zeros((0, 3), np.int32), 0)
    return OracleResult(st, cost.value, -1, vv[: nv.value].copy(), ee[: 3 * ne.value].reshape(-1, 3).copy(), 0)


def check_tree(row_ptr, col, w, group_ptr, members, vertices, edges, cost) -> str | None:
    """Feasibility + cost check of a returned tree, as the reference's
    this_is_a_feasible_solution_gpu (rucgraph/test_gpu.h:45-77) and
    graph_hash_of_mixed_weighted_sum_of_ec (sum_of_nw_ec.h:58-87) do.
    Returns None when valid, else the reason."""
    rp = np.asarray(row_ptr)
    vs = set(int(x) for x in vertices)
    E = {}
    for u, v, ww in np.asarray(edges).reshape(-1, 3):
        u, v, ww = int(u), int(v), int(ww)
        if u not in vs or v not in vs:
            return f"edge ({u},{v}) leaves the vertex set"
        # the edge must exist in the graph with that weight (lightest entry)
        row = range(int(rp[u]), int(rp[u + 1]))
        ws = [int(w[e]) for e in row if int(col[e]) == v]
        if not ws or min(ws) != ww:
            return f"edge ({u},{v},{ww}) is not a graph edge"
        E[(min(u, v), max(u, v))] = ww
    if sum(E.values()) != cost:
        return f"tree weight {sum(E.values())} != cost {cost}"
    if len(vs) == 0:
        return "empty tree"
    # connected (one component) — BFS over the tree edges
    adj = {x: [] for x in vs}
    for (u, v) in E:
        adj[u].append(v)
        adj[v].append(u)
    start = next(iter(vs))
    seen = {start}
    stack = [start]
    while stack:
        x = stack.pop()
        for y in adj[x]:
            if y not in seen:
                seen.add(y)
                stack.append(y)
    if seen != vs:
        return "tree is disconnected"
    if len(E) != len(vs) - 1:
        return "edge set is not a tree"
    gp = np.asarray(group_ptr)
    mem = np.asarray(members)
    for g in range(len(gp) - 1):
        if not any(int(m) in vs for m in mem[gp[g]:gp[g + 1]]):
            return f"group {g} not covered"
    return None


# ------------------------------------------------------------- generators --
_GEN = None


def gen_lib() -> C.CDLL:
    global _GEN
    if _GEN is None:
        dll = C.CDLL(str(build_gen()))
        sig = {
            "gst_gen_random_connected": (C.c_void_p, [C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_uint64]),
            "gst_gen_barabasi_albert": (C.c_void_p, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64]),
            "gst_host_graph_num_vertices": (C.c_int32, [C.c_void_p]),
            "gst_host_graph_num_entries": (C.c_int64, [C.c_void_p]),
            "gst_host_graph_copy": (None, [C.c_void_p, I32P, I32P, I32P]),
            "gst_host_graph_free": (None, [C.c_void_p]),
            "gst_gen_groups_uniform": (C.c_void_p, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64]),
            "gst_gen_groups_zipf_degree": (C.c_void_p, [I32P, I32P, C.c_int32, C.c_int64, C.c_int32, C.c_double,
                                                        C.c_int32, C.c_int32, C.c_uint64]),
            "gst_host_groups_k": (C.c_int32, [C.c_void_p]),
            "gst_host_groups_num_members": (C.c_int64, [C.c_void_p]),
            "gst_host_groups_copy": (None, [C.c_void_p, I32P, I32P]),
            "gst_host_groups_free": (None, [C.c_void_p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(dll, name)
            fn.restype, fn.argtypes = res, args
        _GEN = dll
    return _GEN


class HostCSR:
    def __init__(self, row_ptr, col, w):
        self.row_ptr, self.col, self.w = row_ptr, col, w

    @property
    def V(self) -> int:
        return len(self.row_ptr) - 1

    @property
    def nnz(self) -> int:
        return len(self.col)


def _take_graph(h) -> HostCSR:
    L = gen_lib()
    if not h:
        raise ValueError("generator rejected its parameters")
    try:
        V, n = L.gst_host_graph_num_vertices(h), L.gst_host_graph_num_entries(h)
        rp, col, w = np.zeros(V + 1, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32)
        L.gst_host_graph_copy(h, _p(rp), _p(col), _p(w))
    finally:
        L.gst_host_graph_free(h)
    return HostCSR(rp, col, w)


def _take_groups(h):
    L = gen_lib()
    if not h:
        raise ValueError("group generator rejected its parameters")
    try:
        k, n = L.gst_host_groups_k(h), L.gst_host_groups_num_members(h)
        gp, mem = np.zeros(k + 1, np.int32), np.zeros(n, np.int32)
        L.gst_host_groups_copy(h, _p(gp), _p(mem))
    finally:
        L.gst_host_groups_free(h)
    return gp, mem


def gen_random_connected(V, E, wmin, wmax, seed) -> HostCSR:
    return _take_graph(gen_lib().gst_gen_random_connected(V, E, wmin, wmax, seed))


def gen_barabasi_albert(V, m, wmin, wmax, seed) -> HostCSR:
    return _take_graph(gen_lib().gst_gen_barabasi_albert(V, m, wmin, wmax, seed))


def gen_groups_uniform(V, k, size, seed):
    return _take_groups(gen_lib().gst_gen_groups_uniform(V, k, size, seed))


def gen_groups_zipf_degree(g, k, s, size_min, size_max, seed):
    rp, col = _i32(g.row_ptr), _i32(g.col)
    return _take_groups(gen_lib().gst_gen_groups_zipf_degree(_p(rp), _p(col), g.V, g.nnz, k, s, size_min, size_max,
                                                             seed))
