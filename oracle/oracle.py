"""ctypes binding of the CPU oracle (sgw_oracle.c).

TEST INFRASTRUCTURE: imported only by the tests, the smoke check and the
benchmark's CPU-baseline leg.  Functions take a host CSR as numpy arrays
(node_pointer of n+1 u32 or u64, edges of m u32 or (m, 2) u32) and return
numpy arrays of final values.  The C side takes u64 node pointers: u32
arrays are widened on every call, so callers that repeat calls on a large
graph widen once (np.uint64) and pass that.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build_oracle import OUT, build_oracle

_lib = None
_P = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = build_oracle() if not OUT.exists() else OUT
        L = C.CDLL(str(path))
        for name in ("orc_bfs", "orc_sssp", "orc_sswp", "omp_bfs", "omp_sssp", "omp_sswp", "omp_sssp_frontier"):
            getattr(L, name).argtypes = [C.c_uint32, _P, _P, C.c_uint32, C.c_uint32, _P]
            getattr(L, name).restype = C.c_int
        for name in ("orc_cc", "omp_cc"):
            getattr(L, name).argtypes = [C.c_uint32, _P, _P, C.c_uint32, _P]
            getattr(L, name).restype = C.c_int
        for name in ("orc_pr", "omp_pr"):
            getattr(L, name).argtypes = [C.c_uint32, _P, _P, C.c_uint32, C.c_double, C.c_double,
                                         C.c_double, C.c_uint32, _P, C.POINTER(C.c_uint32)]
            getattr(L, name).restype = C.c_int
        L.orc_generate.argtypes = [C.c_uint32, _P, _P, _P, _P, _P]
        L.orc_generate.restype = C.c_uint32
        L.orc_partition.argtypes = [_P, C.c_uint32, C.c_uint64, _P, _P, C.c_uint32]
        L.orc_partition.restype = C.c_uint32
        L.orc_num_threads.restype = C.c_int
        L.orc_rmat_write.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                     C.c_uint64, C.c_int, C.c_uint32, C.c_char_p, C.POINTER(C.c_uint64)]
        L.orc_rmat_write.restype = C.c_int
        L.orc_pick_sources.argtypes = [C.c_uint32, _P, _P, C.c_uint32, C.c_uint32, C.c_uint64, _P]
        L.orc_pick_sources.restype = C.c_int
        L.omp_reach_multi.argtypes = [C.c_uint32, _P, _P, C.c_uint32, C.c_uint32, _P, _P]
        L.omp_reach_multi.restype = C.c_int
        _lib = L
    return _lib


def _csr(node_pointer, edges):
    npa = np.ascontiguousarray(node_pointer, dtype=np.uint64)
    eda = np.ascontiguousarray(edges, dtype=np.uint32)
    stride = 2 if eda.ndim == 2 else 1
    return npa, eda, stride


def run(algo: str, node_pointer, edges, source: int = 0, parallel: bool = False) -> np.ndarray:
    """Final values of bfs/sssp/sswp/cc (u32)."""
    npa, eda, stride = _csr(node_pointer, edges)
    n = len(npa) - 1
    out = np.empty(n, np.uint32)
    L = lib()
    pre = "omp_" if parallel else "orc_"
    if algo == "cc":
        st = getattr(L, pre + "cc")(n, npa.ctypes.data, eda.ctypes.data, stride, out.ctypes.data)
    else:
        st = getattr(L, pre + algo)(n, npa.ctypes.data, eda.ctypes.data, stride, source, out.ctypes.data)
    if st != 0:
        raise RuntimeError(f"oracle {algo} failed ({st})")
    return out


def pagerank(node_pointer, edges, init=0.15, acc=0.01, damping=0.85, max_rounds=100000,
             parallel=False):
    npa, eda, stride = _csr(node_pointer, edges)
    n = len(npa) - 1
    out = np.empty(n, np.float64)
    r = C.c_uint32()
    f = lib().omp_pr if parallel else lib().orc_pr
    if f(n, npa.ctypes.data, eda.ctypes.data, stride, init, acc, damping, max_rounds,
         out.ctypes.data, C.byref(r)) != 0:
        raise RuntimeError("oracle pr failed")
    return out, r.value


def generate(label1, label2, out_degree):
    """Reference-semantics compaction: (queue, ptr) over active vertices."""
    l1 = np.ascontiguousarray(label1, dtype=np.uint8)
    l2 = np.ascontiguousarray(label2, dtype=np.uint8)
    deg = np.ascontiguousarray(out_degree, dtype=np.uint32)
    n = len(deg)
    q = np.empty(max(n, 1), np.uint32)
    p = np.empty(n + 1, np.uint32)
    c = lib().orc_generate(n, l1.ctypes.data, l2.ctypes.data, deg.ctypes.data, q.ctypes.data, p.ctypes.data)
    return q[:c].copy(), p[: c + 1].copy()


def partition(ptr, max_partition_size):
    """Reference partitions (from_node, node_size) or None where it would not terminate."""
    ptr = np.ascontiguousarray(ptr, dtype=np.uint32)
    cnt = len(ptr) - 1
    cap = max(cnt, 1)
    fr = np.zeros(cap, np.uint32)
    sz = np.zeros(cap, np.uint32)
    p = lib().orc_partition(ptr.ctypes.data, cnt, max_partition_size, fr.ctypes.data, sz.ctypes.data, cap)
    if p == 0xFFFFFFFF:
        return None
    return fr[:p].copy(), sz[:p].copy()


def num_threads() -> int:
    return lib().orc_num_threads()


def rmat_write(path, scale, edge_factor=16, seed=1, weighted=False, wmax=64, a=0.57, b=0.19, c=0.19) -> int:
    """Writes the seeded R-MAT graph as a .bcsr/.bwcsr file; returns its edge count."""
    m = C.c_uint64()
    st = lib().orc_rmat_write(scale, edge_factor, a, b, c, seed, int(weighted), wmax, str(path).encode(),
                              C.byref(m))
    if st != 0:
        raise RuntimeError(f"oracle R-MAT writer failed ({st})")
    return m.value


def read_csr(path):
    """(node_pointer[n+1], edges) of a .bcsr/.bwcsr file (u32 node pointers) or of a
    .bcsr64/.bwcsr64 file (u64); edges map the file in place."""
    path = str(path)
    wide = path.endswith("64")
    if wide:
        n, m = (int(x) for x in np.fromfile(path, dtype=np.uint64, count=2))
        hdr, npw, npt = 16, 8, np.uint64
    else:
        n, m = (int(x) for x in np.fromfile(path, dtype=np.uint32, count=2))
        hdr, npw, npt = 8, 4, np.uint32
    npa = np.empty(n + 1, npt)
    npa[:n] = np.memmap(path, dtype=npt, mode="r", offset=hdr, shape=(n,))
    npa[n] = m
    weighted = path.endswith((".bwcsr", ".bwcsr64"))
    shape = (m, 2) if weighted else (m,)
    edges = np.memmap(path, dtype=np.uint32, mode="r", offset=hdr + npw * n, shape=shape) if m else \
        np.zeros(shape, np.uint32)
    return npa, edges


def pick_sources(node_pointer, edges, count, seed=1) -> np.ndarray:
    """count sources among the out-degree > 0 vertices of the largest WCC."""
    npa, eda, stride = _csr(node_pointer, edges)
    out = np.empty(count, np.uint32)
    if lib().orc_pick_sources(len(npa) - 1, npa.ctypes.data, eda.ctypes.data, stride, count, seed,
                              out.ctypes.data) != 0:
        raise RuntimeError("oracle source picker failed")
    return out


def reached_edges(node_pointer, edges, sources) -> np.ndarray:
    """m_reached (edges whose source is reachable) of each source, <= 64 per call."""
    npa, eda, stride = _csr(node_pointer, edges)
    src = np.ascontiguousarray(sources, dtype=np.uint32)
    out = np.zeros(len(src), np.uint64)
    for k in range(0, len(src), 64):
        part = np.ascontiguousarray(src[k:k + 64])
        res = np.zeros(len(part), np.uint64)
        if lib().omp_reach_multi(len(npa) - 1, npa.ctypes.data, eda.ctypes.data, stride, len(part),
                                 part.ctypes.data, res.ctypes.data) != 0:
            raise RuntimeError("oracle reachability failed")
        out[k:k + 64] = res
    return out


def sssp_frontier(node_pointer, edges, source) -> np.ndarray:
    """SSSP by unbucketed frontier rounds (a second exact method)."""
    npa, eda, stride = _csr(node_pointer, edges)
    out = np.empty(len(npa) - 1, np.uint32)
    if lib().omp_sssp_frontier(len(npa) - 1, npa.ctypes.data, eda.ctypes.data, stride, int(source),
                               out.ctypes.data) != 0:
        raise RuntimeError("oracle sssp failed")
    return out
