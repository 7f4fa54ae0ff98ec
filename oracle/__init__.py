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
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE.parent / "_build" / "oracle"
ORACLE_LIB = BUILD_DIR / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_dpbf.so"
REFERENCE_ROOT = Path(os.environ.get("GST_REFERENCE_ROOT", "/root/reference"))

INF = 2**31 - 1
I32P = C.POINTER(C.c_int32)
I64P = C.POINTER(C.c_int64)
F64P = C.POINTER(C.c_double)

OK, INFEASIBLE, STOPPED = 0, 1, 2


def build_oracle(force: bool = False) -> Path:
    src = HERE / "dpbf_oracle.c"
    if not force and ORACLE_LIB.exists() and ORACLE_LIB.stat().st_mtime >= src.stat().st_mtime:
        return ORACLE_LIB
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    cc = shutil.which("gcc") or "cc"
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    subprocess.run([cc, "-O2", "-std=c11", "-shared", "-fPIC", str(src), "-o", str(tmp)], check=True)
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


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
