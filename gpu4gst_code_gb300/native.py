"""ctypes binding of libgst.so (include/gst.h, gst_gen.h, gst_io.h, gst_learn.h, gst_debug.h).

The library is the product: every solve runs the CUDA kernels in libgst.so.
There is no Python or CPU fallback; if the library is missing this module
raises instead of degrading.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libgst.so"

I32P = C.POINTER(C.c_int32)
I64P = C.POINTER(C.c_int64)
F64P = C.POINTER(C.c_double)
F32P = C.POINTER(C.c_float)

MAX_K = 16
COST_LIMIT = 1073741823
NOALLOC_MAX_VERTICES = 1 << 20
SCORER_NUM_PARAMS = 25921
SCORER_FEATURES = 16
SCORER_HIDDEN = 64


class Status(enum.IntEnum):
    OK = 0
    INFEASIBLE = 1
    BAD_INPUT = 2
    OOM = 3
    TIMEOUT = 4
    CUDA_ERROR = 5
    OVERFLOW = 6
    INTERNAL = 7
    TOO_LARGE = 8


class GSTError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{Status(status).name}: {message}")
        self.status = Status(status)


class Opts(C.Structure):
    _fields_ = [
        ("struct_size", C.c_int32),
        ("upper_bound", C.c_int32),
        ("max_rounds", C.c_int32),
        ("use_graph", C.c_int32),
        ("collect_stats", C.c_int32),
        ("dense_shift", C.c_int32),
        ("refine_bound", C.c_int32),
        ("concurrency", C.c_int32),
        ("batch_graph", C.c_int32),
        ("reserved", C.c_int32 * 7),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("dense_shift", C.c_int32 * (MAX_K + 1)),
        ("concurrency", C.c_int32),
        ("batch_graph", C.c_int32),
        ("reserved", C.c_int32 * 6),
    ]


# name -> (restype, argtypes); every symbol include/*.h declares
SIGNATURES = {
    "gst_graph_upload": (C.c_int, [I32P, I32P, I32P, C.c_int32, C.c_int64, C.POINTER(C.c_void_p)]),
    "gst_graph_free": (None, [C.c_void_p]),
    "gst_graph_num_vertices": (C.c_int32, [C.c_void_p]),
    "gst_graph_num_entries": (C.c_int64, [C.c_void_p]),
    "gst_solve": (C.c_int, [C.c_void_p, I32P, I32P, C.c_int32, C.POINTER(Opts), C.POINTER(C.c_void_p)]),
    "gst_solve_batch": (
        C.c_int,
        [C.c_void_p, C.c_int32, I32P, I32P, I32P, C.POINTER(Opts), C.POINTER(C.c_void_p)],
    ),
    "gst_autotune": (C.c_int, [C.c_void_p, C.c_int32, I32P, I32P, I32P, C.POINTER(Opts), I32P]),
    "gst_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "gst_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "gst_pool_create": (C.c_int, [I32P, I32P, I32P, C.c_int32, C.c_int64, I32P, C.c_int32, C.POINTER(C.c_void_p)]),
    "gst_pool_free": (None, [C.c_void_p]),
    "gst_pool_num_replicas": (C.c_int32, [C.c_void_p]),
    "gst_pool_solve_batch": (
        C.c_int,
        [C.c_void_p, C.c_int32, I32P, I32P, I32P, C.POINTER(Opts), C.POINTER(C.c_void_p)],
    ),
    "gst_result_replica": (C.c_int32, [C.c_void_p]),
    "gst_result_latency": (None, [C.c_void_p, F64P]),
    "gst_result_free": (None, [C.c_void_p]),
    "gst_result_status": (C.c_int, [C.c_void_p]),
    "gst_result_cost": (C.c_int32, [C.c_void_p]),
    "gst_result_root": (C.c_int32, [C.c_void_p]),
    "gst_result_num_vertices": (C.c_int32, [C.c_void_p]),
    "gst_result_num_edges": (C.c_int32, [C.c_void_p]),
    "gst_result_vertices": (None, [C.c_void_p, I32P]),
    "gst_result_edges": (None, [C.c_void_p, I32P]),
    "gst_result_states": (C.c_int64, [C.c_void_p]),
    "gst_result_launches": (C.c_int64, [C.c_void_p]),
    "gst_result_times": (None, [C.c_void_p, F64P]),
    "gst_result_stats": (None, [C.c_void_p, I64P]),
    "gst_graph_debug_table": (C.c_int, [C.c_void_p, C.c_int32, I32P]),
    "gst_debug_scorer_wait_timeout": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, I32P]),
    "gst_group_distances_noalloc": (
        C.c_int,
        [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
         C.c_void_p],
    ),
    # learned proposal (include/gst_learn.h)
    "gst_scorer_num_params": (C.c_int64, []),
    "gst_scorer_create": (C.c_int, [F32P, C.POINTER(C.c_void_p)]),
    "gst_scorer_free": (None, [C.c_void_p]),
    "gst_scorer_get_params": (C.c_int, [C.c_void_p, F32P]),
    "gst_scorer_scores": (C.c_int, [C.c_void_p, C.c_void_p, I32P, I32P, C.c_int32, C.c_int32, F32P]),
    "gst_scorer_train_step": (
        C.c_int,
        [C.c_void_p, C.c_void_p, I32P, I32P, C.c_int32, I32P, C.c_int32, C.c_float, C.c_int32, F32P, F32P],
    ),
    "gst_propose": (C.c_int, [C.c_void_p, C.c_void_p, I32P, I32P, C.c_int32, C.POINTER(C.c_void_p)]),
    "gst_solve_learned": (
        C.c_int,
        [C.c_void_p, C.c_void_p, I32P, I32P, C.c_int32, C.POINTER(Opts), C.POINTER(C.c_void_p)],
    ),
    "gst_result_upper_bound": (C.c_int32, [C.c_void_p]),
    "gst_result_proposal_cost": (C.c_int32, [C.c_void_p]),
    "gst_result_proposal_ms": (C.c_double, [C.c_void_p]),
    "gst_result_proposal_concurrent": (C.c_int32, [C.c_void_p]),
    "gst_result_wall_ms": (C.c_double, [C.c_void_p]),
    "gst_last_error": (C.c_char_p, []),
    "gst_version": (C.c_char_p, []),
    # generators (include/gst_gen.h)
    "gst_gen_random_connected": (C.c_void_p, [C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_uint64]),
    "gst_gen_barabasi_albert": (C.c_void_p, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64]),
    "gst_host_graph_num_vertices": (C.c_int32, [C.c_void_p]),
    "gst_host_graph_num_entries": (C.c_int64, [C.c_void_p]),
    "gst_host_graph_copy": (None, [C.c_void_p, I32P, I32P, I32P]),
    "gst_host_graph_free": (None, [C.c_void_p]),
    "gst_gen_groups_uniform": (C.c_void_p, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64]),
    "gst_gen_groups_zipf_degree": (
        C.c_void_p,
        [I32P, I32P, C.c_int32, C.c_int64, C.c_int32, C.c_double, C.c_int32, C.c_int32, C.c_uint64],
    ),
    "gst_host_groups_k": (C.c_int32, [C.c_void_p]),
    "gst_host_groups_num_members": (C.c_int64, [C.c_void_p]),
    "gst_host_groups_copy": (None, [C.c_void_p, I32P, I32P]),
    "gst_host_groups_free": (None, [C.c_void_p]),
    # dataset readers (include/gst_io.h)
    "gst_read_graph_file": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p), I32P]),
    "gst_read_groups_file": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "gst_read_queries_file": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "gst_read_gstp_instance": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
}

_LIB = None


def lib() -> C.CDLL:
    """Loads libgst.so (building it first if the CUDA toolkit is present)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    from . import build

    if build.toolkit_available():
        build.build_library()  # no-op when up to date
    if not LIB_PATH.exists():
        raise RuntimeError(f"libgst.so not found at {LIB_PATH}; run gpu4gst_code_gb300.build")
    dll = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(dll, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = dll
    return dll


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a: np.ndarray, t=I32P):
    return a.ctypes.data_as(t)


def last_error() -> str:
    return lib().gst_last_error().decode()


def version() -> str:
    return lib().gst_version().decode()


@dataclass
class Result:
    """One query's answer (gst_result)."""

    status: Status
    cost: int
    root: int
    vertices: np.ndarray
    edges: np.ndarray  # (n, 3) int32: u < v, w
    states: int
    launches: int = 0
    times_ms: tuple = (0.0, 0.0, 0.0, 0.0)
    stats: dict = field(default_factory=dict)
    latency_ms: tuple = (0.0, 0.0)  # batch: own solve, completion since the batch began
    replica: int = -1  # pool: replica that solved the query
    upper_bound: int = 0  # pruning bound at the last wave (0: unpruned)
    proposal_cost: int = 0  # learned path: cost of the proposed tree (0: none)
    proposal_ms: float = 0.0
    # learned path: the proposal ran beside the DP (times_ms[0] spans both)
    proposal_concurrent: bool = False
    wall_ms: float = 0.0  # learned path: host wall time of the call

    @property
    def feasible(self) -> bool:
        return self.status == Status.OK


STAT_NAMES = ("rounds", "vertices", "entries", "rows", "gathered", "improved", "splits", "bytes")


def _read_result(r) -> Result:
    L = lib()
    st = Status(L.gst_result_status(r))
    nv = L.gst_result_num_vertices(r)
    ne = L.gst_result_num_edges(r)
    v = np.zeros(nv, np.int32)
    e = np.zeros((ne, 3), np.int32)
    if nv:
        L.gst_result_vertices(r, _ptr(v))
    if ne:
        L.gst_result_edges(r, _ptr(e))
    t = (C.c_double * 4)()
    L.gst_result_times(r, t)
    s = (C.c_int64 * 8)()
    L.gst_result_stats(r, s)
    lat = (C.c_double * 2)()
    L.gst_result_latency(r, lat)
    return Result(
        status=st,
        cost=int(L.gst_result_cost(r)),
        root=int(L.gst_result_root(r)),
        vertices=v,
        edges=e,
        states=int(L.gst_result_states(r)),
        launches=int(L.gst_result_launches(r)),
        times_ms=tuple(t),
        stats=dict(zip(STAT_NAMES, list(s))),
        latency_ms=tuple(lat),
        replica=int(L.gst_result_replica(r)),
        upper_bound=int(L.gst_result_upper_bound(r)),
        proposal_cost=int(L.gst_result_proposal_cost(r)),
        proposal_ms=float(L.gst_result_proposal_ms(r)),
        proposal_concurrent=bool(L.gst_result_proposal_concurrent(r)),
        wall_ms=float(L.gst_result_wall_ms(r)),
    )


def make_opts(upper_bound: int = 0, max_rounds: int = 0, use_graph: bool = False, collect_stats: bool = False,
              dense_shift: int = 0, refine_bound: bool = False, concurrency: int = 0, batch_graph: int = 0) -> Opts:
    o = Opts()
    o.struct_size = C.sizeof(Opts)
    o.upper_bound = int(upper_bound)
    o.max_rounds = int(max_rounds)
    o.use_graph = int(bool(use_graph))
    o.collect_stats = int(bool(collect_stats))
    o.dense_shift = int(dense_shift)
    o.refine_bound = int(bool(refine_bound))
    o.concurrency = int(concurrency)
    o.batch_graph = int(batch_graph)
    return o


TUNING_FORMAT = "gst-tuning-1"


def tuning_key(V: int, nnz: int, ks, refine_bound: bool, use_graph: bool) -> str:
    """The shape a tuning record applies to: the vertex count's power-of-two
    bucket, the rounded average degree, the set of k in the sample, the
    method (plain or bound-refined) and the driver (CUDA graph or host)."""
    vb = max(0, int(V) - 1).bit_length()
    deg = round(int(nnz) / max(int(V), 1))
    kset = ",".join(str(k) for k in sorted({int(k) for k in ks}))
    return f"V<=2^{vb}|deg{deg}|k{kset}|{'bounded' if refine_bound else 'plain'}|{'graph' if use_graph else 'host'}"


def load_tuning(path, key: str):
    """The record stored under key in a tuning cache file, or None (no file,
    no such key, or a file of another format)."""
    import json

    p = Path(path)
    if not p.exists():
        return None
    try:
        doc = json.loads(p.read_text())
    except (OSError, ValueError):
        return None
    if not isinstance(doc, dict) or doc.get("format") != TUNING_FORMAT:
        return None
    rec = doc.get("entries", {}).get(key)
    if not isinstance(rec, dict):
        return None
    return {"dense_shift": [int(x) for x in rec.get("dense_shift", [])], "concurrency": int(rec.get("concurrency", 0)),
            "batch_graph": int(rec.get("batch_graph", 0))}


def store_tuning(path, key: str, rec: dict) -> None:
    """Adds (or replaces) key's record in a tuning cache file, written
    through a temporary file and renamed into place."""
    import json
    import os

    p = Path(path)
    doc = {"format": TUNING_FORMAT, "entries": {}}
    if p.exists():
        try:
            old = json.loads(p.read_text())
            if isinstance(old, dict) and old.get("format") == TUNING_FORMAT:
                doc["entries"] = dict(old.get("entries", {}))
        except (OSError, ValueError):
            pass
    doc["entries"][key] = {"dense_shift": [int(x) for x in rec["dense_shift"]], "concurrency": int(rec["concurrency"]),
                           "batch_graph": int(rec["batch_graph"])}
    tmp = p.with_name(f".{p.name}.{os.getpid()}.tmp")
    tmp.write_text(json.dumps(doc, indent=1, sort_keys=True) + "\n")
    os.replace(tmp, p)


def groups_to_csr(groups) -> tuple[np.ndarray, np.ndarray]:
    """[[members of group 0], [members of group 1], ...] -> (group_ptr, members)."""
    ptr = [0]
    mem: list[int] = []
    for g in groups:
        mem.extend(int(x) for x in g)
        ptr.append(len(mem))
    return _i32(ptr), _i32(mem)


class Graph:
    """A graph resident on the current GPU (gst_graph)."""

    def __init__(self, row_ptr, col, w):
        L = lib()
        self.row_ptr = _i32(row_ptr)
        self.col = _i32(col)
        self.w = _i32(w)
        V = len(self.row_ptr) - 1
        h = C.c_void_p()
        st = L.gst_graph_upload(_ptr(self.row_ptr), _ptr(self.col), _ptr(self.w), V, len(self.col), C.byref(h))
        if st != Status.OK:
            raise GSTError(st, last_error())
        self._h = h
        self.V = V
        self.nnz = len(self.col)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().gst_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def solve(self, group_ptr, members=None, *, upper_bound=0, max_rounds=0, use_graph=False,
              collect_stats=False, dense_shift=0, refine_bound=False, raise_on_error=True) -> Result:
        """Solves one query. `group_ptr` may be a list of member lists."""
        if members is None:
            group_ptr, members = groups_to_csr(group_ptr)
        gp, mem = _i32(group_ptr), _i32(members)
        k = len(gp) - 1
        o = make_opts(upper_bound, max_rounds, use_graph, collect_stats, dense_shift, refine_bound)
        r = C.c_void_p()
        st = lib().gst_solve(self._h, _ptr(gp), _ptr(mem), k, C.byref(o), C.byref(r))
        msg = last_error()
        try:
            res = _read_result(r) if r.value else None
        finally:
            if r.value:
                lib().gst_result_free(r)
        if st not in (Status.OK, Status.INFEASIBLE) and raise_on_error:
            raise GSTError(st, msg)
        if res is None:
            res = Result(Status(st), -1, -1, np.zeros(0, np.int32), np.zeros((0, 3), np.int32), 0)
        return res

    def _call_result(self, fn, *args, raise_on_error=True) -> Result:
        r = C.c_void_p()
        st = fn(*args, C.byref(r))
        msg = last_error()
        try:
            res = _read_result(r) if r.value else None
        finally:
            if r.value:
                lib().gst_result_free(r)
        if st not in (Status.OK, Status.INFEASIBLE) and raise_on_error:
            raise GSTError(st, msg)
        if res is None:
            res = Result(Status(st), -1, -1, np.zeros(0, np.int32), np.zeros((0, 3), np.int32), 0)
        return res

    def propose(self, scorer, group_ptr, members=None) -> Result:
        """Feasible tree from the scorer's top vertex (scorer None: fixed feature score)."""
        if members is None:
            group_ptr, members = groups_to_csr(group_ptr)
        gp, mem = _i32(group_ptr), _i32(members)
        h = scorer._h if scorer is not None else None
        return self._call_result(lib().gst_propose, self._h, h, _ptr(gp), _ptr(mem), len(gp) - 1)

    def solve_learned(self, scorer, group_ptr, members=None, *, max_rounds=0, use_graph=True,
                      collect_stats=False, dense_shift=0, raise_on_error=True) -> Result:
        """Proposal, then the exact DP pruned by its cost (gst_solve_learned)."""
        if members is None:
            group_ptr, members = groups_to_csr(group_ptr)
        gp, mem = _i32(group_ptr), _i32(members)
        o = make_opts(0, max_rounds, use_graph, collect_stats, dense_shift)
        h = scorer._h if scorer is not None else None
        return self._call_result(lib().gst_solve_learned, self._h, h, _ptr(gp), _ptr(mem), len(gp) - 1, C.byref(o),
                                 raise_on_error=raise_on_error)

    def debug_table(self, k: int) -> np.ndarray:
        """(V, 2^k) table of the last solve with k groups (gst_graph_debug_table)."""
        out = np.zeros(self.V * (1 << k), np.int32)
        st = lib().gst_graph_debug_table(self._h, k, _ptr(out))
        if st != Status.OK:
            raise GSTError(st, last_error())
        return out.reshape(self.V, 1 << k)

    @staticmethod
    def _pack_batch(queries):
        ks, gptr, mem = [], [0], []
        for q in queries:
            gp, m = q if isinstance(q, tuple) else groups_to_csr(q)
            gp = _i32(gp)
            ks.append(len(gp) - 1)
            base = len(mem)
            mem.extend(int(x) for x in m)
            gptr.extend(int(base + x) for x in gp[1:])
        return _i32(ks), _i32(gptr), _i32(mem)

    def autotune(self, queries, *, use_graph=True, refine_bound=False, cache=None) -> int:
        """gst_autotune on a sample of queries; returns the tuned concurrency
        (or the batch graph size, when batch graphs solved the sample faster).
        cache: a JSON file of tuning records keyed by the graph's shape and
        the sample's k (tuning_key); a record found there is applied instead
        of tuning, a new one is added after tuning."""
        ks_a, gp_a, mem_a = self._pack_batch(queries)
        key = tuning_key(self.V, self.nnz, ks_a, refine_bound, use_graph) if cache is not None else None
        if key is not None:
            rec = load_tuning(cache, key)
            if rec is not None:
                self.set_tuning(rec)
                return int(rec["batch_graph"] or rec["concurrency"])
        o = make_opts(0, 0, use_graph, False, 0, refine_bound)
        lanes = C.c_int32(0)
        st = lib().gst_autotune(self._h, len(ks_a), _ptr(ks_a), _ptr(gp_a), _ptr(mem_a), C.byref(o), C.byref(lanes))
        if st != Status.OK:
            raise GSTError(st, last_error())
        if key is not None:
            store_tuning(cache, key, self.tuning())
        return int(lanes.value)

    def tuning(self) -> dict:
        """The graph's tuned values (gst_get_tuning) as a plain dict."""
        t = Tuning()
        st = lib().gst_get_tuning(self._h, C.byref(t))
        if st != Status.OK:
            raise GSTError(st, last_error())
        return {"dense_shift": [int(x) for x in t.dense_shift], "concurrency": int(t.concurrency),
                "batch_graph": int(t.batch_graph)}

    def set_tuning(self, rec: dict) -> None:
        """Applies a record of tuning() (gst_set_tuning; out-of-range values raise)."""
        t = Tuning()
        shifts = list(rec.get("dense_shift", []))
        for k in range(MAX_K + 1):
            t.dense_shift[k] = int(shifts[k]) if k < len(shifts) else 0
        t.concurrency = int(rec.get("concurrency", 0))
        t.batch_graph = int(rec.get("batch_graph", 0))
        st = lib().gst_set_tuning(self._h, C.byref(t))
        if st != Status.OK:
            raise GSTError(st, last_error())

    def solve_batch(self, queries, *, upper_bound=0, use_graph=False, collect_stats=False, refine_bound=False,
                    concurrency=0, batch_graph=0, raise_on_error=True) -> list[Result]:
        """queries: list of (group_ptr, members) or list of member-list lists.
        A query that fails alone (k out of range) has its status in its own
        result; raise_on_error=False returns the results instead of raising
        the batch's first error."""
        ks_a, gp_a, mem_a = self._pack_batch(queries)
        n = len(ks_a)
        outs = (C.c_void_p * n)()
        o = make_opts(upper_bound, 0, use_graph, collect_stats, 0, refine_bound, concurrency, batch_graph)
        st = lib().gst_solve_batch(self._h, n, _ptr(ks_a), _ptr(gp_a), _ptr(mem_a), C.byref(o), outs)
        msg = last_error()
        res = []
        for i in range(n):
            if outs[i]:
                res.append(_read_result(outs[i]))
                lib().gst_result_free(outs[i])
            else:
                res.append(None)
        if raise_on_error and st not in (Status.OK, Status.INFEASIBLE):
            raise GSTError(st, msg)
        return res


class Pool:
    """Replicas of one graph on several devices (gst_pool); a device may repeat."""

    def __init__(self, row_ptr, col, w, devices):
        rp, c, ww = _i32(row_ptr), _i32(col), _i32(w)
        dev = _i32(devices)
        h = C.c_void_p()
        st = lib().gst_pool_create(_ptr(rp), _ptr(c), _ptr(ww), len(rp) - 1, len(c), _ptr(dev), len(dev),
                                   C.byref(h))
        if st != Status.OK:
            raise GSTError(st, last_error())
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().gst_pool_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def replicas(self) -> int:
        return int(lib().gst_pool_num_replicas(self._h))

    def solve_batch(self, queries, *, use_graph=True, refine_bound=False, concurrency=0) -> list[Result]:
        ks_a, gp_a, mem_a = Graph._pack_batch(queries)
        n = len(ks_a)
        outs = (C.c_void_p * n)()
        o = make_opts(0, 0, use_graph, False, 0, refine_bound, concurrency)
        st = lib().gst_pool_solve_batch(self._h, n, _ptr(ks_a), _ptr(gp_a), _ptr(mem_a), C.byref(o), outs)
        msg = last_error()
        res = []
        for i in range(n):
            if outs[i]:
                res.append(_read_result(outs[i]))
                lib().gst_result_free(outs[i])
            else:
                res.append(None)
        if st not in (Status.OK, Status.INFEASIBLE):
            raise GSTError(st, msg)
        return res


class Scorer:
    """The proposal network's parameters on the current GPU (gst_scorer)."""

    def __init__(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.shape != (SCORER_NUM_PARAMS,):
            raise ValueError(f"expected {SCORER_NUM_PARAMS} parameters, got {p.shape}")
        h = C.c_void_p()
        st = lib().gst_scorer_create(_ptr(p, F32P), C.byref(h))
        if st != Status.OK:
            raise GSTError(st, last_error())
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().gst_scorer_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def params(self) -> np.ndarray:
        out = np.zeros(SCORER_NUM_PARAMS, np.float32)
        st = lib().gst_scorer_get_params(self._h, _ptr(out, F32P))
        if st != Status.OK:
            raise GSTError(st, last_error())
        return out

    def scores(self, graph: "Graph", group_ptr, members, *, fp32: bool = False) -> np.ndarray:
        gp, mem = _i32(group_ptr), _i32(members)
        out = np.zeros(graph.V, np.float32)
        st = lib().gst_scorer_scores(graph._h, self._h, _ptr(gp), _ptr(mem), len(gp) - 1, int(fp32), _ptr(out, F32P))
        if st != Status.OK:
            raise GSTError(st, last_error())
        return out

    def train_step(self, graph: "Graph", group_ptr, members, tree_vertices, *, lr: float = 1e-3,
                   apply: bool = True, want_grads: bool = False):
        """One Adam step on one solved query; returns (loss, grads or None)."""
        gp, mem = _i32(group_ptr), _i32(members)
        tv = _i32(tree_vertices)
        loss = C.c_float(0.0)
        grads = np.zeros(SCORER_NUM_PARAMS, np.float32) if want_grads else None
        st = lib().gst_scorer_train_step(graph._h, self._h, _ptr(gp), _ptr(mem), len(gp) - 1, _ptr(tv), len(tv),
                                         float(lr), int(apply), C.byref(loss),
                                         _ptr(grads, F32P) if grads is not None else None)
        if st != Status.OK:
            raise GSTError(st, last_error())
        return float(loss.value), grads


# ------------------------------------------------------------- generators --
@dataclass
class CSR:
    row_ptr: np.ndarray
    col: np.ndarray
    w: np.ndarray

    @property
    def V(self) -> int:
        return len(self.row_ptr) - 1

    @property
    def nnz(self) -> int:
        return len(self.col)


def _take_graph(h) -> CSR:
    L = lib()
    if not h:
        raise GSTError(Status.BAD_INPUT, "generator rejected its parameters")
    try:
        V = L.gst_host_graph_num_vertices(h)
        n = L.gst_host_graph_num_entries(h)
        rp = np.zeros(V + 1, np.int32)
        col = np.zeros(n, np.int32)
        w = np.zeros(n, np.int32)
        L.gst_host_graph_copy(h, _ptr(rp), _ptr(col), _ptr(w))
    finally:
        L.gst_host_graph_free(h)
    return CSR(rp, col, w)


def _take_groups(h) -> tuple[np.ndarray, np.ndarray]:
    L = lib()
    if not h:
        raise GSTError(Status.BAD_INPUT, "group generator rejected its parameters")
    try:
        k = L.gst_host_groups_k(h)
        n = L.gst_host_groups_num_members(h)
        gp = np.zeros(k + 1, np.int32)
        mem = np.zeros(n, np.int32)
        L.gst_host_groups_copy(h, _ptr(gp), _ptr(mem))
    finally:
        L.gst_host_groups_free(h)
    return gp, mem


def gen_random_connected(V: int, E: int, wmin: int, wmax: int, seed: int) -> CSR:
    return _take_graph(lib().gst_gen_random_connected(V, E, wmin, wmax, seed))


def gen_barabasi_albert(V: int, m: int, wmin: int, wmax: int, seed: int) -> CSR:
    return _take_graph(lib().gst_gen_barabasi_albert(V, m, wmin, wmax, seed))


def gen_groups_uniform(V: int, k: int, size: int, seed: int):
    return _take_groups(lib().gst_gen_groups_uniform(V, k, size, seed))


def gen_groups_zipf_degree(g: CSR, k: int, s: float, size_min: int, size_max: int, seed: int):
    """Zipf(s)-sized groups clipped to [size_min, size_max], members by degree."""
    rp, col = _i32(g.row_ptr), _i32(g.col)
    return _take_groups(
        lib().gst_gen_groups_zipf_degree(_ptr(rp), _ptr(col), g.V, g.nnz, k, s, size_min, size_max, seed)
    )


# ---------------------------------------------------------------- datasets --
def _fs(path) -> bytes:
    return str(path).encode()


def read_graph_file(path) -> tuple[CSR, int]:
    """<name>.in (the reference's read_input_graph) -> (CSR, number of communities)."""
    h = C.c_void_p()
    c = C.c_int32(0)
    st = lib().gst_read_graph_file(_fs(path), C.byref(h), C.byref(c))
    if st != Status.OK:
        raise GSTError(st, last_error())
    return _take_graph(h.value), int(c.value)


def _take_lists(h) -> tuple[np.ndarray, np.ndarray]:
    L = lib()
    try:
        k = L.gst_host_groups_k(h)
        n = L.gst_host_groups_num_members(h)
        gp = np.zeros(k + 1, np.int32)
        mem = np.zeros(n, np.int32)
        L.gst_host_groups_copy(h, _ptr(gp), _ptr(mem))
    finally:
        L.gst_host_groups_free(h)
    return gp, mem


def read_groups_file(path) -> tuple[np.ndarray, np.ndarray]:
    """<name>.g (read_Group) -> every group of the dataset as (group_ptr, members)."""
    h = C.c_void_p()
    st = lib().gst_read_groups_file(_fs(path), C.byref(h))
    if st != Status.OK:
        raise GSTError(st, last_error())
    return _take_lists(h.value)


def read_queries_file(path, V: int) -> list[list[int]]:
    """<name>.gK (read_inquire) -> per query, its group indices (value - V)."""
    h = C.c_void_p()
    st = lib().gst_read_queries_file(_fs(path), int(V), C.byref(h))
    if st != Status.OK:
        raise GSTError(st, last_error())
    qp, ids = _take_lists(h.value)
    return [ids[qp[i]:qp[i + 1]].tolist() for i in range(len(qp) - 1)]


def read_gstp_instance(path) -> tuple[CSR, np.ndarray, np.ndarray]:
    """A GSTP instance text (graph_hash_of_mixed_weighted_save_for_GSTP) -> (CSR, group_ptr, members)."""
    hg, hq = C.c_void_p(), C.c_void_p()
    st = lib().gst_read_gstp_instance(_fs(path), C.byref(hg), C.byref(hq))
    if st != Status.OK:
        raise GSTError(st, last_error())
    g = _take_graph(hg.value)
    gp, mem = _take_lists(hq.value)
    return g, gp, mem


def query_groups(all_groups: tuple[np.ndarray, np.ndarray], ids) -> tuple[np.ndarray, np.ndarray]:
    """The (group_ptr, members) of one query from the dataset's groups."""
    gp_all, mem_all = all_groups
    gp, mem = [0], []
    for i in ids:
        mem.extend(mem_all[gp_all[i]:gp_all[i + 1]].tolist())
        gp.append(len(mem))
    return _i32(gp), _i32(mem)
