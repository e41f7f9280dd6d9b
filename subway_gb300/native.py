"""ctypes binding of libsubwaygb (include/subway_gb300.h, include/sgw_graphgen.h).

The engine lives entirely in the native library; this module only declares
the C entry points and wraps graphs and engines in small Python objects with
numpy views of the host arrays.  Loading fails loudly if the library has not
been built: there is no Python fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libsubwaygb.so"

SGW_OK = 0
BFS, SSSP, SSWP, CC, PR = 0, 1, 2, 3, 4
SYNC, ASYNC = 0, 1
INF = 4294967294
OPT_PROFILE = 0x1
OPT_NO_OVERLAP = 0x2
OPT_NO_PACK = 0x4
OPT_SCALAR_GATHER = 0x8
OPT_CTA_TILES = 0x10
OPT_SPLIT_WEIGHTS = 0x20
OPT_BATCH_PERSISTENT = 0x40
OPT_BATCH_GRAPH = 0x80
OPT_PAGEABLE_COPY = 0x100
OPT_GRAPH_IN_PLACE = 0x200
SCHED_CAP_COMPACT = 0x1
SCHED_KEEP_IDLE = 0x2
ALGOS = {"bfs": BFS, "sssp": SSSP, "sswp": SSWP, "cc": CC, "pr": PR}
MODES = {"sync": SYNC, "async": ASYNC}


class EngineOpts(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("device", C.c_int32), ("flags", C.c_uint32),
                ("inner_batch", C.c_uint32), ("tile_degree_max", C.c_uint32),
                ("chunk_edges", C.c_uint32), ("gather_ctas", C.c_uint32), ("num_buffers", C.c_uint32),
                ("sched_inner", C.c_uint32), ("sched_active_permille", C.c_uint32),
                ("sched_flags", C.c_uint32), ("sched_defer_permille", C.c_uint32),
                ("transfer_chunk_log2", C.c_uint32), ("generate_edge_limit", C.c_uint32)]


class RunParams(C.Structure):
    _fields_ = [("algo", C.c_int32), ("mode", C.c_int32), ("source", C.c_uint32),
                ("pr_init", C.c_float), ("pr_acc", C.c_float), ("pr_damping", C.c_float),
                ("max_inner", C.c_uint32), ("reserved", C.c_uint32 * 7)]


class RunStats(C.Structure):
    _fields_ = [("global_iterations", C.c_uint32), ("partitions", C.c_uint32),
                ("inner_iterations", C.c_uint64), ("active_vertices", C.c_uint64),
                ("active_edges", C.c_uint64), ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("reached_edges", C.c_uint64), ("ms_device", C.c_double), ("ms_generate", C.c_double),
                ("ms_partition", C.c_double), ("ms_gather", C.c_double), ("ms_relax", C.c_double),
                ("launches", C.c_uint64), ("gather_launches", C.c_uint64),
                ("relax_launches", C.c_uint64), ("generate_launches", C.c_uint64),
                ("relaxed_edges", C.c_uint64), ("relaxed_sources", C.c_uint64),
                ("gather_bytes", C.c_uint64), ("ms_stream", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


_P = C.c_void_p
_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)

# name -> (restype, argtypes)
_PROTOS = {
    "sgw_strerror": (C.c_char_p, [C.c_int]),
    "sgw_last_error": (C.c_char_p, []),
    "sgw_graph_load": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "sgw_graph_map": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "sgw_graph_from_csr": (C.c_int, [C.c_uint32, C.c_uint32, _P, _P, C.c_int, C.POINTER(_P)]),
    "sgw_graph_from_csr64": (C.c_int, [C.c_uint32, C.c_uint64, _P, _P, C.c_int, C.POINTER(_P)]),
    "sgw_graph_info": (C.c_int, [_P, _u32p, _u32p, C.POINTER(C.c_int)]),
    "sgw_graph_info64": (C.c_int, [_P, _u32p, C.POINTER(C.c_uint64), C.POINTER(C.c_int)]),
    "sgw_graph_node_pointer": (_P, [_P]),
    "sgw_graph_node_pointer64": (_P, [_P]),
    "sgw_graph_edges": (_P, [_P]),
    "sgw_graph_out_degree": (C.c_int, [_P, _P]),
    "sgw_graph_save": (C.c_int, [_P, C.c_char_p]),
    "sgw_graph_free": (None, [_P]),
    "sgw_engine_opts_default": (None, [C.POINTER(EngineOpts)]),
    "sgw_engine_create": (C.c_int, [_P, C.POINTER(EngineOpts), C.POINTER(_P)]),
    "sgw_engine_destroy": (C.c_int, [_P]),
    "sgw_engine_max_partition_size": (C.c_int, [_P, _u64p]),
    "sgw_engine_device_bytes": (C.c_int, [_P, _u64p]),
    "sgw_engine_host_copy_bytes": (C.c_int, [_P, _u64p]),
    "sgw_run_params_default": (None, [C.POINTER(RunParams), C.c_int, C.c_int, C.c_uint32]),
    "sgw_run": (C.c_int, [_P, C.POINTER(RunParams), _P, C.POINTER(RunStats)]),
    "sgw_state_init": (C.c_int, [_P, C.POINTER(RunParams)]),
    "sgw_generate": (C.c_int, [_P, _u32p, _u64p]),
    "sgw_partition": (C.c_int, [_P, _u32p]),
    "sgw_partition_info": (C.c_int, [_P, C.c_uint32, _u32p, _u32p, _u32p, _u64p]),
    "sgw_process_partition": (C.c_int, [_P, C.c_uint32, _u32p]),
    "sgw_read_values": (C.c_int, [_P, _P]),
    "sgw_read_values_f64": (C.c_int, [_P, _P]),
    "sgw_read_active": (C.c_int, [_P, _P, _P, C.c_uint32, _u32p]),
    "sgw_get_stats": (C.c_int, [_P, C.POINTER(RunStats)]),
    "sgw_plan_partitions": (C.c_int, [_P, C.c_uint32, C.c_uint64, _P, _P, C.c_uint32, _u32p]),
    "sgw_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "sgw_device_info": (C.c_int, [C.c_int, _u32p, _u64p]),
    "sgw_probe_link": (C.c_int, [C.c_int, C.c_uint64, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "sgw_generate_noalloc": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_int, _P, _P, _P, _u32p, _u64p]),
    "sgw_mlp_create": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(_P)]),
    "sgw_mlp_destroy": (C.c_int, [_P]),
    "sgw_mlp_set_params": (C.c_int, [_P, _P]),
    "sgw_mlp_get_params": (C.c_int, [_P, _P]),
    "sgw_mlp_forward": (C.c_int, [_P, _P, C.c_uint32, _P]),
    "sgw_mlp_gradient": (C.c_int, [_P, _P, _P, C.c_uint32, _P, C.POINTER(C.c_float)]),
    "sgw_mlp_train": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_float, C.POINTER(C.c_float)]),
    "sgw_mlp_save": (C.c_int, [_P, C.c_char_p]),
    "sgw_mlp_load": (C.c_int, [C.c_int, C.c_char_p, C.POINTER(_P)]),
    "sgw_set_policy": (C.c_int, [_P, C.c_int, _P]),
    "sgw_sched_buffers": (C.c_int, [_P, C.c_uint64, _u32p]),
    "sgw_engine_dma_rate": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "sgw_batch_create": (C.c_int, [_P, C.POINTER(EngineOpts), C.c_uint32, C.POINTER(_P)]),
    "sgw_batch_destroy": (C.c_int, [_P]),
    "sgw_batch_device_bytes": (C.c_int, [_P, _u64p]),
    "sgw_batch_run": (C.c_int, [_P, C.c_int, _P, C.c_uint32, _P, _P]),
    "sgw_batch_results": (C.c_int, [_P, C.POINTER(_P)]),
    "sgw_batch_check_wait_timeout": (C.c_int, [_P, C.c_uint64]),
    "sgw_batch_run_u16": (C.c_int, [_P, C.c_int, _P, C.c_uint32, _P, _P]),
    "sgw_range_trace_count": (C.c_int, [_P, _u64p]),
    "sgw_range_trace_read": (C.c_int, [_P, _P, C.c_uint64, _u64p]),
    "sgw_trace_enable": (C.c_int, [_P, C.c_int]),
    "sgw_trace_count": (C.c_int, [_P, _u64p]),
    "sgw_trace_read": (C.c_int, [_P, _P, C.c_uint64, _u64p]),
    "sgw_trace_save": (C.c_int, [_P, C.c_char_p]),
    "sgw_trace_write_csv": (C.c_int, [_P, C.c_uint64, C.c_char_p]),
    "sgw_graph_clear_out_edges": (C.c_int, [_P, C.c_uint32]),
    "sgw_gen_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                               C.c_uint64, C.c_int, C.c_uint32, C.POINTER(_P)]),
    "sgw_gen_er": (C.c_int, [C.c_uint32, C.c_uint64, C.c_uint64, C.c_int, C.c_uint32, C.POINTER(_P)]),
    "sgw_graph_symmetrize": (C.c_int, [_P, C.POINTER(_P)]),
    "sgw_pick_sources": (C.c_int, [_P, C.c_uint32, C.c_uint64, _P]),
    "sgw_largest_wcc": (C.c_int, [_P, _u32p, _u64p]),
}

_lib = None


class SgwError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: status {status}")


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with subway_gb300.build.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _PROTOS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols() -> list[str]:
    return list(_PROTOS)


def check(status: int, what: str):
    if status != SGW_OK:
        L = lib()
        msg = L.sgw_last_error().decode(errors="replace")
        raise SgwError(status, f"{what} -> {L.sgw_strerror(status).decode()} ({msg})")


def device_count() -> int:
    c = C.c_int(0)
    check(lib().sgw_device_count(C.byref(c)), "sgw_device_count")
    return c.value


def device_info(device=0) -> dict:
    sms, mem = C.c_uint32(0), C.c_uint64(0)
    check(lib().sgw_device_info(device, C.byref(sms), C.byref(mem)), "sgw_device_info")
    return {"sm_count": sms.value, "total_bytes": mem.value}


def sched_buffers(graph, budget_bytes) -> int:
    """Edge buffers for a learned-policy engine on this graph and budget."""
    nb = C.c_uint32(0)
    check(lib().sgw_sched_buffers(graph.h, int(budget_bytes), C.byref(nb)), "sgw_sched_buffers")
    return nb.value


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Graph:
    """A host CSR graph owned by the native library (or wrapping numpy arrays)."""

    def __init__(self, handle: int, keep=None):
        self.h = C.c_void_p(handle)
        self._keep = keep
        n, m, w = C.c_uint32(), C.c_uint64(), C.c_int()
        check(lib().sgw_graph_info64(self.h, C.byref(n), C.byref(m), C.byref(w)), "sgw_graph_info64")
        self.n, self.m, self.weighted = n.value, m.value, bool(w.value)

    # ---- constructors
    @classmethod
    def rmat(cls, scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, weighted=False, wmax=64):
        h = _P()
        check(lib().sgw_gen_rmat(scale, edge_factor, a, b, c, seed, int(weighted), wmax, C.byref(h)),
              "sgw_gen_rmat")
        return cls(h.value)

    @classmethod
    def er(cls, n, m, seed=1, weighted=False, wmax=64):
        h = _P()
        check(lib().sgw_gen_er(n, m, seed, int(weighted), wmax, C.byref(h)), "sgw_gen_er")
        return cls(h.value)

    @classmethod
    def load(cls, path):
        h = _P()
        check(lib().sgw_graph_load(str(path).encode(), C.byref(h)), f"sgw_graph_load({path})")
        return cls(h.value)

    @classmethod
    def map(cls, path):
        """A .bcsr/.bwcsr(64) file mapped in place: edges stay in the page cache."""
        h = _P()
        check(lib().sgw_graph_map(str(path).encode(), C.byref(h)), f"sgw_graph_map({path})")
        return cls(h.value)

    @classmethod
    def from_csr(cls, node_pointer, edges, weighted):
        """Wraps numpy CSR arrays without copying; u64 node pointers (or more
        than 2^32 - 1 edges) give a graph with u64 node pointers."""
        wide = np.asarray(node_pointer).dtype == np.uint64 or int(np.asarray(node_pointer)[-1]) >= 2 ** 32
        npa = np.ascontiguousarray(node_pointer, dtype=np.uint64 if wide else np.uint32)
        eda = np.ascontiguousarray(edges, dtype=np.uint32)
        n = len(npa) - 1
        m = int(npa[-1])
        if weighted:
            eda = eda.reshape(-1, 2)
        if eda.shape[0] != m:
            raise ValueError("edge count does not match node_pointer[-1]")
        h = _P()
        fn = lib().sgw_graph_from_csr64 if wide else lib().sgw_graph_from_csr
        check(fn(n, m, _ptr(npa), _ptr(eda) if m else None, int(weighted), C.byref(h)),
              "sgw_graph_from_csr64" if wide else "sgw_graph_from_csr")
        return cls(h.value, keep=(npa, eda))

    # ---- views
    @property
    def node_pointer(self) -> np.ndarray:
        """(n + 1,) node pointers: u32, or u64 for a graph that holds u64 ones."""
        p = lib().sgw_graph_node_pointer(self.h)
        if p:
            return np.ctypeslib.as_array(C.cast(p, _u32p), shape=(self.n + 1,))
        p = lib().sgw_graph_node_pointer64(self.h)
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint64)), shape=(self.n + 1,))

    @property
    def edges(self) -> np.ndarray:
        """(m,) u32 destinations, or (m, 2) [dst, weight] for weighted graphs."""
        if self.m == 0:
            return np.zeros((0, 2) if self.weighted else (0,), np.uint32)
        p = lib().sgw_graph_edges(self.h)
        shape = (self.m, 2) if self.weighted else (self.m,)
        return np.ctypeslib.as_array(C.cast(p, _u32p), shape=shape)

    @property
    def ends(self) -> np.ndarray:
        e = self.edges
        return e[:, 0] if self.weighted else e

    def out_degree(self) -> np.ndarray:
        out = np.empty(self.n, np.uint32)
        check(lib().sgw_graph_out_degree(self.h, _ptr(out)), "sgw_graph_out_degree")
        return out

    def save(self, path):
        check(lib().sgw_graph_save(self.h, str(path).encode()), f"sgw_graph_save({path})")

    def clear_out_edges(self, v):
        """Removes vertex v's out-edges (graphs the library owns only)."""
        check(lib().sgw_graph_clear_out_edges(self.h, int(v)), "sgw_graph_clear_out_edges")
        n, m = C.c_uint32(), C.c_uint64()
        check(lib().sgw_graph_info64(self.h, C.byref(n), C.byref(m), None), "sgw_graph_info64")
        self.m = m.value

    def symmetrize(self) -> "Graph":
        h = _P()
        check(lib().sgw_graph_symmetrize(self.h, C.byref(h)), "sgw_graph_symmetrize")
        return Graph(h.value)

    def pick_sources(self, count, seed=1) -> np.ndarray:
        out = np.empty(count, np.uint32)
        check(lib().sgw_pick_sources(self.h, count, seed, _ptr(out)), "sgw_pick_sources")
        return out

    def largest_wcc(self):
        v, e = C.c_uint32(), C.c_uint64()
        check(lib().sgw_largest_wcc(self.h, C.byref(v), C.byref(e)), "sgw_largest_wcc")
        return v.value, e.value

    def close(self):
        if self.h and self.h.value:
            lib().sgw_graph_free(self.h)
            self.h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan_partitions(ptr: np.ndarray, cap: int, capacity: int | None = None):
    ptr = np.ascontiguousarray(ptr, dtype=np.uint32)
    count = len(ptr) - 1
    capacity = capacity if capacity is not None else max(count, 1)
    fr = np.zeros(capacity, np.uint32)
    sz = np.zeros(capacity, np.uint32)
    p = C.c_uint32()
    check(lib().sgw_plan_partitions(_ptr(ptr), count, cap, _ptr(fr), _ptr(sz), capacity, C.byref(p)),
          "sgw_plan_partitions")
    return fr[: p.value].copy(), sz[: p.value].copy()


def default_opts() -> EngineOpts:
    o = EngineOpts()
    lib().sgw_engine_opts_default(C.byref(o))
    return o


def run_params(algo, mode, source=0, **kw) -> RunParams:
    p = RunParams()
    lib().sgw_run_params_default(C.byref(p), ALGOS.get(algo, algo), MODES.get(mode, mode), source)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Engine:
    """A device engine over one graph under a device-memory budget."""

    def __init__(self, graph: Graph, budget_bytes=0, device=0, flags=0, **opts):
        o = default_opts()
        o.budget_bytes = int(budget_bytes)
        o.device = device
        o.flags = flags
        for k, v in opts.items():
            setattr(o, k, v)
        h = _P()
        check(lib().sgw_engine_create(graph.h, C.byref(o), C.byref(h)), "sgw_engine_create")
        self.h = C.c_void_p(h.value)
        self.graph = graph

    def max_partition_size(self) -> int:
        v = C.c_uint64()
        check(lib().sgw_engine_max_partition_size(self.h, C.byref(v)), "max_partition_size")
        return v.value

    def device_bytes(self) -> int:
        v = C.c_uint64()
        check(lib().sgw_engine_device_bytes(self.h, C.byref(v)), "device_bytes")
        return v.value

    def host_copy_bytes(self) -> int:
        """Bytes of the host transfer copy (0 when the records are read in place)."""
        v = C.c_uint64()
        check(lib().sgw_engine_host_copy_bytes(self.h, C.byref(v)), "host_copy_bytes")
        return v.value

    def dma_rate(self) -> float:
        """DMA rate (GB/s) from the transfer copy timed at creation, -1 if not timed."""
        g = C.c_double(0)
        check(lib().sgw_engine_dma_rate(self.h, C.byref(g)), "sgw_engine_dma_rate")
        return g.value

    def run(self, algo, mode, source=0, out=None, **kw):
        p = run_params(algo, mode, source, **kw)
        if out is None:
            out = np.empty(self.graph.n, np.float32 if p.algo == PR else np.uint32)
        st = RunStats()
        check(lib().sgw_run(self.h, C.byref(p), _ptr(out), C.byref(st)), "sgw_run")
        return out, st.as_dict()

    # ---- step API
    def state_init(self, algo, mode, source=0, **kw):
        p = run_params(algo, mode, source, **kw)
        check(lib().sgw_state_init(self.h, C.byref(p)), "sgw_state_init")

    def generate(self):
        a, e = C.c_uint32(), C.c_uint64()
        check(lib().sgw_generate(self.h, C.byref(a), C.byref(e)), "sgw_generate")
        return a.value, e.value

    def partition(self):
        p = C.c_uint32()
        check(lib().sgw_partition(self.h, C.byref(p)), "sgw_partition")
        out = []
        for i in range(p.value):
            fn, fe, ns, es = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint64()
            check(lib().sgw_partition_info(self.h, i, C.byref(fn), C.byref(fe), C.byref(ns), C.byref(es)),
                  "sgw_partition_info")
            out.append((fn.value, fe.value, ns.value, es.value))
        return out

    def process_partition(self, i) -> int:
        it = C.c_uint32()
        check(lib().sgw_process_partition(self.h, i, C.byref(it)), "sgw_process_partition")
        return it.value

    def read_values(self, dtype=np.uint32):
        out = np.empty(self.graph.n, dtype)
        check(lib().sgw_read_values(self.h, _ptr(out)), "sgw_read_values")
        return out

    def read_active(self):
        cnt = C.c_uint32()
        cap = self.graph.n
        nodes = np.empty(max(cap, 1), np.uint32)
        ptr = np.empty(cap + 1, np.uint32)
        check(lib().sgw_read_active(self.h, _ptr(nodes), _ptr(ptr), cap, C.byref(cnt)), "sgw_read_active")
        c = cnt.value
        return nodes[:c].copy(), ptr[: c + 1].copy()

    def stats(self) -> dict:
        st = RunStats()
        check(lib().sgw_get_stats(self.h, C.byref(st)), "sgw_get_stats")
        return st.as_dict()

    def close(self):
        if self.h and self.h.value:
            lib().sgw_engine_destroy(self.h)
            self.h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- learned scheduler ------------------------------------------------------------
POLICY_PLAIN, POLICY_LEARNED = 0, 1
MLP_INPUTS, MLP_PARAMS = 5, 4609
ACT_SKIP, ACT_RESIDENT, ACT_STREAM, ACT_COMPACT, ACT_SPLIT = 0, 1, 2, 3, 4

TRACE_REC = np.dtype([("global_iteration", "<u4"), ("partition", "<u4"), ("num_partitions", "<u4"),
                      ("inner_iterations", "<u4"), ("active_nodes", "<u4"), ("first_vertex", "<u4"),
                      ("active_edges", "<u8"), ("iteration_active_nodes", "<u8"),
                      ("iteration_active_edges", "<u8"), ("bytes_h2d", "<u8"), ("transfer", "<u4"),
                      ("reserved", "<u4")])


def write_trace_csv(recs: np.ndarray, path):
    """sgw_trace_write_csv over an array of TRACE_REC records."""
    r = np.ascontiguousarray(recs, dtype=TRACE_REC)
    check(lib().sgw_trace_write_csv(r.ctypes.data if len(r) else None, len(r), str(path).encode()),
          "sgw_trace_write_csv")


RANGE_REC = np.dtype([("global_iteration", "<u4"), ("range", "<u4"), ("active_nodes", "<u4"),
                      ("range_nodes", "<u4"), ("active_edges", "<u4"), ("range_edges", "<u4"),
                      ("action", "<u4"), ("inner_iterations", "<u4"), ("features", "<f4", (5,)),
                      ("predicted", "<f4"), ("bytes_h2d", "<u8")])


class Mlp:
    """The scheduler's network (BF16 weights on the device)."""

    def __init__(self, handle: int):
        self.h = C.c_void_p(handle)

    @classmethod
    def create(cls, device=0, seed=1):
        h = _P()
        check(lib().sgw_mlp_create(device, seed, C.byref(h)), "sgw_mlp_create")
        return cls(h.value)

    @classmethod
    def load(cls, path, device=0):
        h = _P()
        check(lib().sgw_mlp_load(device, str(path).encode(), C.byref(h)), f"sgw_mlp_load({path})")
        return cls(h.value)

    def save(self, path):
        check(lib().sgw_mlp_save(self.h, str(path).encode()), f"sgw_mlp_save({path})")

    def params(self) -> np.ndarray:
        out = np.empty(MLP_PARAMS, np.float32)
        check(lib().sgw_mlp_get_params(self.h, _ptr(out)), "sgw_mlp_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (MLP_PARAMS,)
        check(lib().sgw_mlp_set_params(self.h, _ptr(p)), "sgw_mlp_set_params")

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_INPUTS)
        y = np.empty(len(x), np.float32)
        check(lib().sgw_mlp_forward(self.h, _ptr(x), len(x), _ptr(y)), "sgw_mlp_forward")
        return y

    def gradient(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_INPUTS)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.empty(MLP_PARAMS, np.float32)
        loss = C.c_float()
        check(lib().sgw_mlp_gradient(self.h, _ptr(x), _ptr(t), len(x), _ptr(g), C.byref(loss)),
              "sgw_mlp_gradient")
        return g, loss.value

    def train(self, x, t, steps=500, lr=3e-3) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_INPUTS)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = C.c_float()
        check(lib().sgw_mlp_train(self.h, _ptr(x), _ptr(t), len(x), steps, lr, C.byref(loss)), "sgw_mlp_train")
        return loss.value

    def close(self):
        if self.h and self.h.value:
            lib().sgw_mlp_destroy(self.h)
            self.h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _engine_set_policy(self, policy, model: "Mlp | None" = None):
    p = {"plain": POLICY_PLAIN, "learned": POLICY_LEARNED}.get(policy, policy)
    check(lib().sgw_set_policy(self.h, p, model.h if model is not None else None), "sgw_set_policy")


def _engine_trace_enable(self, on=True):
    check(lib().sgw_trace_enable(self.h, int(on)), "sgw_trace_enable")


def _engine_range_trace(self) -> np.ndarray:
    cnt = C.c_uint64()
    check(lib().sgw_range_trace_count(self.h, C.byref(cnt)), "sgw_range_trace_count")
    out = np.zeros(cnt.value, RANGE_REC)
    got = C.c_uint64()
    check(lib().sgw_range_trace_read(self.h, out.ctypes.data if cnt.value else None, cnt.value, C.byref(got)),
          "sgw_range_trace_read")
    return out[: got.value]


class BatchStats(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("queries", C.c_uint32), ("ms_device", C.c_double),
                ("ms_wall", C.c_double), ("d2h_bytes", C.c_uint64), ("reserved", C.c_uint64 * 4)]


class Batch:
    """Up to 64 BFS/SSSP queries per traversal over a graph held in HBM."""

    def __init__(self, graph: Graph, lanes=64, budget_bytes=0, device=0, chunk_edges=0, flags=0):
        o = default_opts()
        o.budget_bytes = int(budget_bytes)
        o.device = device
        o.flags = flags
        o.chunk_edges = chunk_edges
        h = _P()
        check(lib().sgw_batch_create(graph.h, C.byref(o), lanes, C.byref(h)), "sgw_batch_create")
        self.h = C.c_void_p(h.value)
        self.graph = graph
        self.lanes = lanes

    def run(self, algo, sources, out=None, view=False, answers="u32"):
        """Distances of each query (rows).  view=True returns a read-only view of
        the batch's pinned buffer (no copy; valid until the next run).
        answers="u16": 16-bit answers, unreached = 0xffff."""
        src = np.ascontiguousarray(sources, dtype=np.uint32)
        n = self.graph.n
        dt = np.uint16 if answers == "u16" else np.uint32
        if out is None and not view:
            out = np.empty((len(src), n), dt)
        st = BatchStats()
        fn = lib().sgw_batch_run_u16 if answers == "u16" else lib().sgw_batch_run
        check(fn(self.h, ALGOS.get(algo, algo), _ptr(src), len(src), _ptr(out) if out is not None else None,
                 C.byref(st)), "sgw_batch_run")
        if out is None:
            p = _P()
            check(lib().sgw_batch_results(self.h, C.byref(p)), "sgw_batch_results")
            ptr_t = C.POINTER(C.c_uint16) if answers == "u16" else _u32p
            out = np.ctypeslib.as_array(C.cast(p, ptr_t), shape=(len(src), n))
            out.flags.writeable = False
        return out, {k: getattr(st, k) for k, _ in st._fields_ if k != "reserved"}

    def device_bytes(self) -> int:
        v = C.c_uint64()
        check(lib().sgw_batch_device_bytes(self.h, C.byref(v)), "sgw_batch_device_bytes")
        return v.value

    def check_wait_timeout(self, wait_ns=2_000_000) -> int:
        """Status of one persistent run whose grid barriers cannot fill (SGW_ETIMEOUT expected)."""
        return lib().sgw_batch_check_wait_timeout(self.h, int(wait_ns))

    def close(self):
        if self.h and self.h.value:
            lib().sgw_batch_destroy(self.h)
            self.h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


Engine.set_policy = _engine_set_policy
Engine.trace_enable = _engine_trace_enable
Engine.range_trace = _engine_range_trace
