"""ctypes binding of the CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU legs (the cpu_baseline sample and ``--impl reference``), as the
checker and the CPU baseline.  The product package ``byo_gb300`` never imports
this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")
NONE = 0xFFFFFFFF

_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_c = ctypes


def build(force=False):
    """Compile oracle.c into oracle/liboracle.so (gcc, OpenMP)."""
    src = os.path.join(_HERE, "oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src),
                                                  os.path.getmtime(os.path.join(_HERE, "oracle.h")))):
        return LIB_PATH
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu11",
           "-o", LIB_PATH + ".tmp", src, "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        sig = {
            "orc_mix64": (_c.c_uint64, [_c.c_uint64]),
            "orc_rmat_thresholds": (None, [_c.c_double, _c.c_double, _c.c_double, _u32p]),
            "orc_rmat_edges": (None, [_c.c_uint64, _c.c_uint32, _c.c_uint64, _c.c_uint64, _u32p, _u32p, _u32p]),
            "orc_uniform_pairs": (None, [_c.c_uint64, _c.c_uint64, _c.c_uint64, _c.c_uint64, _u32p, _u32p]),
            "orc_grid_pairs": (_c.c_uint64, [_c.c_uint32, _c.c_uint32, _u32p, _u32p]),
            "orc_chung_lu_cdf": (None, [_c.c_uint64, _c.c_double, _u64p]),
            "orc_chung_lu_pairs": (None, [_c.c_uint64, _c.c_uint64, _u64p, _c.c_uint64, _c.c_uint64, _u32p, _u32p]),
            "orc_build_csr": (_c.c_uint64, [_c.c_uint64, _u32p, _u32p, _c.c_uint64, _c.c_int, _c.c_int, _u64p, _u32p]),
            "orc_sort_unique_u64": (_c.c_uint64, [_u64p, _c.c_uint64]),
            "orc_bfs": (_c.c_uint32, [_c.c_uint64, _u64p, _u32p, _c.c_uint32, _u32p, _c.c_void_p]),
            "orc_cc": (None, [_c.c_uint64, _u64p, _u32p, _u32p]),
            "orc_bfs_cc": (None, [_c.c_uint64, _u64p, _u32p, _u32p]),
            "orc_pagerank": (None, [_c.c_uint64, _u64p, _u32p, _c.c_double, _c.c_uint32, _f64p,
                                    _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_double)]),
            "orc_pagerank_delta": (None, [_c.c_uint64, _u64p, _u32p, _c.c_double, _c.c_double, _c.c_uint32,
                                          _f64p, _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_double)]),
            "orc_triangle_count": (_c.c_uint64, [_c.c_uint64, _u64p, _u32p]),
            "orc_map_sum": (_c.c_uint64, [_c.c_uint64, _u64p, _u32p]),
            "orc_bytepd_sizes": (_c.c_uint64, [_c.c_uint64, _u64p, _u32p, _c.c_uint32, _u64p]),
            "orc_bytepd_encode": (None, [_c.c_uint64, _u64p, _u32p, _c.c_uint32, _u64p, _c.c_void_p]),
            "orc_bytepd_decode": (_c.c_int, [_c.c_uint64, _u64p, _u32p, _c.c_void_p, _c.c_uint64, _c.c_uint32,
                                             _u64p, _u32p]),
            "orc_map_remote": (_c.c_uint64, [_c.c_uint64, _u64p, _u32p, _c.c_void_p, _c.c_uint32]),
            "orc_store_create": (_c.c_void_p, [_c.c_uint64, _u64p, _u32p]),
            "orc_store_destroy": (None, [_c.c_void_p]),
            "orc_store_num_edges": (_c.c_uint64, [_c.c_void_p]),
            "orc_store_insert_batch": (_c.c_uint64, [_c.c_void_p, _u64p, _c.c_uint64]),
            "orc_store_remove_batch": (_c.c_uint64, [_c.c_void_p, _u64p, _c.c_uint64]),
            "orc_store_export_csr": (None, [_c.c_void_p, _u64p, _u32p]),
            "orc_num_threads": (_c.c_int, []),
            "orc_set_num_threads": (None, [_c.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


# ---------------------------------------------------------------- generators

def rmat_thresholds(a=0.57, b=0.19, c=0.19):
    t = np.zeros(3, np.uint32)
    lib().orc_rmat_thresholds(a, b, c, t)
    return t


def rmat_edges(seed, lg_n, count, a=0.57, b=0.19, c=0.19, first=0):
    s = np.empty(count, np.uint32)
    d = np.empty(count, np.uint32)
    lib().orc_rmat_edges(seed, lg_n, first, count, rmat_thresholds(a, b, c), s, d)
    return s, d


def uniform_pairs(seed, n, count, first=0):
    s = np.empty(count, np.uint32)
    d = np.empty(count, np.uint32)
    lib().orc_uniform_pairs(seed, n, first, count, s, d)
    return s, d


def grid_pairs(rows, cols):
    cap = max(2 * rows * cols, 1)
    s = np.empty(cap, np.uint32)
    d = np.empty(cap, np.uint32)
    k = lib().orc_grid_pairs(rows, cols, s, d)
    return s[:k].copy(), d[:k].copy()


def chung_lu_cdf(n, exponent):
    cdf = np.empty(n, np.uint64)
    lib().orc_chung_lu_cdf(n, exponent, cdf)
    return cdf


def chung_lu_pairs(seed, n, count, exponent=2.1, first=0, cdf=None):
    if cdf is None:
        cdf = chung_lu_cdf(n, exponent)
    s = np.empty(count, np.uint32)
    d = np.empty(count, np.uint32)
    lib().orc_chung_lu_pairs(seed, n, cdf, first, count, s, d)
    return s, d


def build_csr(n, src, dst, symmetrise=True, drop_self_loops=True):
    src, dst = _u32(src), _u32(dst)
    off = np.zeros(n + 1, np.uint64)
    nb = np.empty(max(len(src) * (2 if symmetrise else 1), 1), np.uint32)
    m = lib().orc_build_csr(n, src, dst, len(src), int(symmetrise), int(drop_self_loops), off, nb)
    return off, nb[:m].copy()


def sort_unique(keys):
    k = _u64(keys).copy()
    u = lib().orc_sort_unique_u64(k, len(k))
    return k[:u].copy()


# ---------------------------------------------------------------- algorithms

def bfs(offsets, nbrs, src):
    n = len(offsets) - 1
    par = np.empty(n, np.uint32)
    lev = np.empty(n, np.uint32)
    lib().orc_bfs(n, _u64(offsets), _u32(nbrs), src, par, lev.ctypes.data)
    return par, lev


def cc(offsets, nbrs):
    n = len(offsets) - 1
    lab = np.empty(n, np.uint32)
    lib().orc_cc(n, _u64(offsets), _u32(nbrs), lab)
    return lab


def bfs_cc(offsets, nbrs):
    n = len(offsets) - 1
    lab = np.empty(n, np.uint32)
    lib().orc_bfs_cc(n, _u64(offsets), _u32(nbrs), lab)
    return lab


def pagerank(offsets, nbrs, eps=1e-6, max_iters=100):
    n = len(offsets) - 1
    p = np.empty(n, np.float64)
    it = ctypes.c_uint32(0)
    l1 = ctypes.c_double(0)
    lib().orc_pagerank(n, _u64(offsets), _u32(nbrs), eps, max_iters, p, ctypes.byref(it), ctypes.byref(l1))
    return p, it.value, l1.value


def pagerank_delta(offsets, nbrs, eps=1e-6, local_eps=0.01, max_iters=100):
    n = len(offsets) - 1
    p = np.empty(n, np.float64)
    r = ctypes.c_uint32(0)
    l1 = ctypes.c_double(0)
    lib().orc_pagerank_delta(n, _u64(offsets), _u32(nbrs), eps, local_eps, max_iters, p, ctypes.byref(r),
                             ctypes.byref(l1))
    return p, r.value, l1.value


def bytepd_encode(offsets, nbrs, P=1000):
    """byte-PD amortized encoding: (byte_offsets[n+1], degrees[n], bytes)."""
    n = len(offsets) - 1
    off, nb = _u64(offsets), _u32(nbrs)
    sizes = np.zeros(max(n, 1), np.uint64)
    total = lib().orc_bytepd_sizes(n, off, nb, P, sizes)
    bo = np.zeros(n + 1, np.uint64)
    bo[1:] = np.cumsum(sizes[:n])
    out = np.zeros(max(total, 1), np.uint8)
    lib().orc_bytepd_encode(n, off, nb, P, bo, out.ctypes.data_as(ctypes.c_void_p))
    return bo, np.diff(off).astype(np.uint32), out[:total]


def bytepd_decode(byte_offsets, degrees, data, P=1000):
    n = len(degrees)
    off = np.zeros(n + 1, np.uint64)
    nb = np.zeros(max(int(np.sum(degrees, dtype=np.uint64)), 1), np.uint32)
    buf = np.ascontiguousarray(data, np.uint8)
    rc = lib().orc_bytepd_decode(n, _u64(byte_offsets), _u32(degrees), buf.ctypes.data_as(ctypes.c_void_p),
                                 len(buf), P, off, nb)
    if rc != 0:
        raise ValueError("malformed byte-PD data")
    return off, nb[:off[-1]]


def map_sum(offsets, nbrs):
    n = len(offsets) - 1
    return int(lib().orc_map_sum(n, _u64(offsets), _u32(nbrs)))


def map_remote(offsets, nbrs, remote, width):
    n = len(offsets) - 1
    buf = np.ascontiguousarray(remote)
    return int(lib().orc_map_remote(n, _u64(offsets), _u32(nbrs), buf.ctypes.data_as(ctypes.c_void_p), width))


def triangle_count(offsets, nbrs):
    n = len(offsets) - 1
    return int(lib().orc_triangle_count(n, _u64(offsets), _u32(nbrs)))


def num_threads():
    return int(lib().orc_num_threads())


def set_num_threads(t):
    lib().orc_set_num_threads(int(t))


class Store:
    """Container model: the sorted-set contents a CPMA / PMA_graph must hold."""

    def __init__(self, offsets, nbrs):
        self.n = len(offsets) - 1
        self._h = lib().orc_store_create(self.n, _u64(offsets), _u32(nbrs))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_store_destroy(self._h)
            self._h = None

    @property
    def num_edges(self):
        return int(lib().orc_store_num_edges(self._h))

    def insert_batch(self, keys):
        k = _u64(keys)
        return int(lib().orc_store_insert_batch(self._h, k, len(k)))

    def remove_batch(self, keys):
        k = _u64(keys)
        return int(lib().orc_store_remove_batch(self._h, k, len(k)))

    def export_csr(self):
        off = np.zeros(self.n + 1, np.uint64)
        nb = np.empty(max(self.num_edges, 1), np.uint32)
        lib().orc_store_export_csr(self._h, off, nb)
        return off, nb[:self.num_edges].copy()


def keys_from_pairs(src, dst, symmetrise=True):
    s = _u32(src).astype(np.uint64)
    d = _u32(dst).astype(np.uint64)
    k = (s << np.uint64(32)) | d
    if symmetrise:
        k = np.concatenate([k, (d << np.uint64(32)) | s])
    return k
