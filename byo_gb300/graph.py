"""Host-side mirror of the reference's container / edgeMap interface over the
C ABI, so code written against BYO's names reads the same.

Reference names kept (paths in the wheatman/BYO tree):
  Graph.N / M / num_vertices / num_edges / degree / out_degree /
  map_neighbors / map_neighbors_early_exit / insert_batch / remove_batch /
  write_adj                 gbbs/graph.h:2154-3150, run_csr.cc:28-175,
                            run_single_pma.cc:39-141
  vertexSubset, edgeMap     gbbs/vertex_subset.h:202-371,
                            gbbs/edge_map_data.h:254-315
  BFS_F, BFS                benchmarks/BFS/NonDeterministicBFS/BFS.h:30-64
  SimpleUnionAsync          benchmarks/Connectivity/SimpleUnionAsync/Connectivity.h:122-136
  bfs_cc                    benchmarks/Connectivity/BFSCC/Connectivity.h:79-88
  PageRank                  benchmarks/PageRank/PageRank.h:125-193
  Triangle_degree_ordering  benchmarks/TriangleCounting/ShunTangwongsan15/Triangle.h:167-204
Errors surface as ByoError carrying the library's status code.
"""
import atexit
import ctypes
import os
import weakref

import numpy as np

from . import _abi
from ._abi import ByoError, check, lib  # noqa: F401

UINT_E_MAX = _abi.NONE


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None and a.size else None


_live_contexts = weakref.WeakSet()


@atexit.register
def _close_all():
    # native objects must go before the CUDA runtime tears itself down
    for c in list(_live_contexts):
        c.close()


class Context:
    """One device, one stream (byo_gpu_init).  Closing a context first closes
    every graph, vertexSubset and functor created on it."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        rc = lib().byo_gpu_init(device, ctypes.byref(h))
        if rc != _abi.BYO_OK:
            raise ByoError(rc, "byo_gpu_init(%d) failed" % device)
        self.h = h
        self.device = device
        self._children = weakref.WeakSet()
        _live_contexts.add(self)

    def _adopt(self, obj):
        self._children.add(obj)
        return obj

    def close(self):
        if getattr(self, "h", None):
            kids = list(self._children)
            # subsets and functors before the graphs they belong to
            for k in sorted(kids, key=lambda o: 0 if not isinstance(o, Graph) else 1):
                k.close()
            lib().byo_gpu_shutdown(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @property
    def stream(self):
        return lib().byo_ctx_stream(self.h)

    @property
    def launches(self):
        return int(lib().byo_ctx_launches(self.h))

    def synchronize(self):
        check(lib().byo_ctx_synchronize(self.h), self.h)

    def kernel_timing(self, tag):
        check(lib().byo_ctx_kernel_timing(self.h, tag.encode() if tag else None), self.h)

    def kernel_time(self, tag=None):
        """(launches, total ms) of the timed launches of `tag` (None: all)."""
        n = ctypes.c_uint64(0)
        ms = ctypes.c_double(0)
        check(lib().byo_ctx_kernel_time(self.h, tag.encode() if tag else None, ctypes.byref(n),
                                        ctypes.byref(ms)), self.h)
        return int(n.value), float(ms.value)

    def set_round_timing(self, on):
        check(lib().byo_ctx_set_round_timing(self.h, int(bool(on))), self.h)

    def last_rounds(self):
        n = ctypes.c_uint64(0)
        check(lib().byo_last_rounds(self.h, None, 0, ctypes.byref(n)), self.h)
        arr = (_abi.RoundLog * max(n.value, 1))()
        check(lib().byo_last_rounds(self.h, arr, n.value, ctypes.byref(n)), self.h)
        return [dict(round=r.round, mode=r.mode, frontier=r.frontier, frontier_deg=r.frontier_deg,
                     unvisited=r.unvisited, ms=r.ms, features=list(r.features)) for r in arr[:n.value]]


def _container(name):
    """csr (static), pma (packed-memory array, CPMA / PMA_graph), vos (vector
    of per-vertex sorted runs, the vector-of-sets containers) or pcsr (Packed
    CSR: per-vertex sentinels and neighbour ids in one packed array)."""
    table = {"csr": _abi.CONTAINER_CSR, "pma": _abi.CONTAINER_PMA, "vos": _abi.CONTAINER_VOS,
             "pcsr": _abi.CONTAINER_PCSR}
    if name not in table:
        raise ValueError("container must be csr, pma, vos or pcsr")
    return table[name]


class Graph:
    """gbbs::Graph<Rep, symmetric=true, full_api> over a device container."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.h = handle
        ctx._adopt(self)

    # ------------------------------------------------------------ construction
    @classmethod
    def from_csr(cls, ctx, offsets, nbrs, container="csr"):
        off = np.ascontiguousarray(offsets, np.uint64)
        nb = np.ascontiguousarray(nbrs, np.uint32)
        n = len(off) - 1
        h = ctypes.c_void_p()
        check(lib().byo_graph_create(ctx.h, _container(container), n, len(nb), _ptr(off), _ptr(nb), ctypes.byref(h)),
              ctx.h)
        return cls(ctx, h)

    @classmethod
    def generate(cls, ctx, kind, seed=1, lg_n=0, n=0, draws=0, a=0.57, b=0.19, c=0.19,
                 exponent=2.1, container="csr"):
        kinds = {"rmat": _abi.GEN_RMAT, "er": _abi.GEN_ER, "grid": _abi.GEN_GRID,
                 "chung_lu": _abi.GEN_CHUNG_LU}
        spec = _abi.GenSpec(kinds[kind], seed, lg_n, n, draws, a, b, c, exponent)
        h = ctypes.c_void_p()
        cont = _container(container)
        check(lib().byo_graph_generate(ctx.h, cont, ctypes.byref(spec), ctypes.byref(h)), ctx.h)
        return cls(ctx, h)

    def close(self):
        if getattr(self, "h", None):
            lib().byo_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # ------------------------------------------------------------ container interface
    def N(self):
        return int(lib().byo_graph_num_vertices(self.h))

    num_vertices = N
    n = property(N)

    def M(self):
        return int(lib().byo_graph_num_edges(self.h))

    num_edges = M

    def nslots(self):
        """Slots of the traversal view (edges plus the PMA's gaps)."""
        return int(lib().byo_graph_num_slots(self.h))

    def tuning(self):
        """Launch shapes in effect for this graph (dict of byo_tuning fields)."""
        t = _abi.Tuning()
        check(lib().byo_graph_get_tuning(self.h, ctypes.byref(t)), self.ctx.h)
        return t.as_dict()

    def set_tuning(self, **fields):
        """Sets launch-shape fields (0 = automatic); others keep their values."""
        cur = self.tuning()
        cur.update(fields)
        t = _abi.Tuning(**cur)
        check(lib().byo_graph_set_tuning(self.h, ctypes.byref(t)), self.ctx.h)

    def autotune(self, bfs=True, multi=False, trials=3):
        """Times candidate launch shapes on this graph and installs the best."""
        what = (_abi.TUNE_BFS if bfs else 0) | (_abi.TUNE_MULTI if multi else 0)
        t = _abi.Tuning()
        check(lib().byo_graph_autotune(self.h, what, trials, ctypes.byref(t)), self.ctx.h)
        return t.as_dict()

    @property
    def container(self):
        names = {_abi.CONTAINER_PMA: "pma", _abi.CONTAINER_VOS: "vos", _abi.CONTAINER_PCSR: "pcsr"}
        return names.get(lib().byo_graph_container(self.h), "csr")

    def degrees(self):
        out = np.empty(self.N(), np.uint32)
        check(lib().byo_graph_degrees(self.h, _ptr(out)), self.ctx.h)
        return out

    def degree(self, i):
        d = ctypes.c_uint64(0)
        check(lib().byo_graph_neighbors(self.h, i, None, 0, ctypes.byref(d)), self.ctx.h)
        return int(d.value)

    out_degree = degree

    def neighbors(self, i):
        d = self.degree(i)
        out = np.empty(max(d, 1), np.uint32)
        dd = ctypes.c_uint64(0)
        check(lib().byo_graph_neighbors(self.h, i, _ptr(out), d, ctypes.byref(dd)), self.ctx.h)
        return out[:d]

    def map_neighbors(self, i, f):
        for u in self.neighbors(i):
            f(i, int(u), None)

    def map_neighbors_early_exit(self, i, f):
        for u in self.neighbors(i):
            if f(i, int(u), None):
                break

    def export_csr(self):
        off = np.empty(self.N() + 1, np.uint64)
        nb = np.empty(max(self.M(), 1), np.uint32)
        check(lib().byo_graph_export_csr(self.h, _ptr(off), _ptr(nb)), self.ctx.h)
        return off, nb[:self.M()]

    def write_adj(self, path, binary=False):
        """The sorted adjacency as an AdjacencyGraph text file (graph.h:3018-3044)
        or the binary CSR layout."""
        check(lib().byo_graph_write_adj(self.h, os.fsencode(path), int(binary)), self.ctx.h)

    @classmethod
    def read_adj(cls, ctx, path, binary=False, container="csr"):
        """read_unweighted_symmetric_graph (graph_io.h:98-124) into a container."""
        h = ctypes.c_void_p()
        cont = _container(container)
        check(lib().byo_graph_read_adj(ctx.h, os.fsencode(path), int(binary), cont, ctypes.byref(h)), ctx.h)
        return cls(ctx, h)

    @classmethod
    def read_bytepd(cls, ctx, path, block=1000, container="csr"):
        """read_compressed_symmetric_graph (graph_io.h:351-390): a byte-PD file,
        decoded on the GPU."""
        h = ctypes.c_void_p()
        cont = _container(container)
        check(lib().byo_graph_read_bytepd(ctx.h, os.fsencode(path), block, cont, ctypes.byref(h)), ctx.h)
        return cls(ctx, h)

    @classmethod
    def from_bytepd(cls, ctx, byte_offsets, degrees, data, block=1000, container="csr"):
        """A graph from byte-PD arrays (byte offsets [n+1], degrees [n], bytes)."""
        bo = np.ascontiguousarray(byte_offsets, np.uint64)
        dg = np.ascontiguousarray(degrees, np.uint32)
        by = np.ascontiguousarray(data, np.uint8)
        h = ctypes.c_void_p()
        cont = _container(container)
        check(lib().byo_graph_from_bytepd(ctx.h, len(dg), bo.ctypes.data, dg.ctypes.data, by.ctypes.data, len(by),
                                          block, cont, ctypes.byref(h)), ctx.h)
        return cls(ctx, h)

    def to_bytepd(self, block=1000):
        """(byte offsets, degrees, bytes) of the byte-PD encoding, made on the GPU."""
        n = self.N()
        bo = np.empty(n + 1, np.uint64)
        dg = np.empty(max(n, 1), np.uint32)
        size = ctypes.c_uint64(0)
        check(lib().byo_graph_encode_bytepd(self.h, block, None, None, None, ctypes.byref(size)), self.ctx.h)
        by = np.empty(max(size.value, 1), np.uint8)
        check(lib().byo_graph_encode_bytepd(self.h, block, bo.ctypes.data, dg.ctypes.data, by.ctypes.data,
                                            ctypes.byref(size)), self.ctx.h)
        return bo, dg[:n], by[:size.value]

    def write_bytepd(self, path, block=1000):
        check(lib().byo_graph_write_bytepd(self.h, os.fsencode(path), block), self.ctx.h)

    @staticmethod
    def _keys(batch):
        a = np.asarray(batch)
        if a.ndim == 2:  # (src, dst) pairs as std::tuple<uintE,uintE>
            a = (a[:, 0].astype(np.uint64) << np.uint64(32)) | a[:, 1].astype(np.uint64)
        return np.ascontiguousarray(a, np.uint64)

    def update_stream(self, batches, ops):
        """Applies update batches in order (ops[b]: True insert, False remove)
        through byo_graph_update_stream; returns each batch's changed count."""
        ks = [self._keys(b) for b in batches]
        off = np.zeros(len(ks) + 1, np.uint64)
        off[1:] = np.cumsum([len(k) for k in ks])
        keys = np.concatenate(ks) if ks else np.zeros(0, np.uint64)
        keys = np.ascontiguousarray(keys, np.uint64)
        o = np.ascontiguousarray([1 if x else 0 for x in ops], np.uint8)
        ch = np.zeros(max(len(ks), 1), np.uint64)
        check(lib().byo_graph_update_stream(self.h, keys.ctypes.data, off.ctypes.data, o.ctypes.data, len(ks),
                                            ch.ctypes.data), self.ctx.h)
        return ch[:len(ks)].astype(np.int64)

    def mixed_stream(self, ops, k, levels, device_keys=False):
        """A stream of update batches and k-source BFS queries, in order
        (byo_graph_mixed_stream).  ops: ("insert", keys), ("remove", keys)
        or ("query", sources) with k sources each; `levels` is a device array
        (anything with data_ptr(), e.g. a CUDA tensor) of nq * k * n uint32
        that receives query q's levels at [q * k * n, (q + 1) * k * n).
        Returns (changed per op, op times [nops, 2] in ns: device start and end
        of the ops run inside the PMA's persistent kernel, 0 for the others
        and on the other containers, which run the ops one by one)."""
        codes = {"remove": _abi.OP_REMOVE, "insert": _abi.OP_INSERT, "query": _abi.OP_QUERY}
        ks, srcs, o = [], [], []
        for kind, x in ops:
            o.append(codes[kind])
            if kind == "query":
                sv = np.ascontiguousarray(x, np.uint32)
                if len(sv) != k:
                    raise ValueError("a query takes exactly k sources")
                srcs.append(sv)
                ks.append(np.zeros(0, np.uint64))
            else:
                ks.append(self._keys(x))
        off = np.zeros(len(ks) + 1, np.uint64)
        off[1:] = np.cumsum([len(a) for a in ks])
        keys = np.ascontiguousarray(np.concatenate(ks) if ks else np.zeros(0, np.uint64), np.uint64)
        sv = np.ascontiguousarray(np.concatenate(srcs) if srcs else np.zeros(1, np.uint32), np.uint32)
        oc = np.ascontiguousarray(o, np.uint8)
        ch = np.zeros(max(len(o), 1), np.uint64)
        t = np.zeros(2 * max(len(o), 1), np.uint64)
        check(lib().byo_graph_mixed_stream(self.h, keys.ctypes.data if len(keys) else None, off.ctypes.data,
                                           oc.ctypes.data, len(o), sv.ctypes.data, k, levels.data_ptr(),
                                           ch.ctypes.data, t.ctypes.data), self.ctx.h)
        return ch[:len(o)].astype(np.int64), t[:2 * len(o)].reshape(-1, 2)

    def insert_batch(self, batch, sorted=False):
        k = self._keys(batch)
        ch = ctypes.c_uint64(0)
        check(lib().byo_graph_insert_batch(self.h, _ptr(k), len(k), int(sorted), ctypes.byref(ch)),
              self.ctx.h)
        return int(ch.value)

    def remove_batch(self, batch, sorted=False):
        k = self._keys(batch)
        ch = ctypes.c_uint64(0)
        check(lib().byo_graph_remove_batch(self.h, _ptr(k), len(k), int(sorted), ctypes.byref(ch)),
              self.ctx.h)
        return int(ch.value)

    insert_sorted_batch = insert_batch
    remove_sorted_batch = remove_batch

    def last_update_stats(self):
        """What the last insert/remove batch did: keys, changed, touched_leaves,
        touched_entries (keys those leaves held), leaf_slots, path."""
        st = _abi.UpdateStats()
        check(lib().byo_graph_last_update_stats(self.h, ctypes.byref(st)), self.ctx.h)
        return st.as_dict()


# ------------------------------------------------------------ vertexSubset / edgeMap

class vertexSubset:
    """vertexSubset(n, v) / vertexSubset(n, list) (vertex_subset.h:240-262)."""

    def __init__(self, G, vertices=None, _handle=None):
        self.G = G
        if _handle is not None:
            self.h = _handle
            G.ctx._adopt(self)
            return
        h = ctypes.c_void_p()
        if isinstance(vertices, (int, np.integer)):
            check(lib().byo_vs_create_single(G.h, int(vertices), ctypes.byref(h)), G.ctx.h)
        else:
            ids = np.ascontiguousarray(vertices if vertices is not None else [], np.uint32)
            check(lib().byo_vs_create_list(G.h, _ptr(ids), len(ids), ctypes.byref(h)), G.ctx.h)
        self.h = h
        G.ctx._adopt(self)

    def close(self):
        if getattr(self, "h", None):
            lib().byo_vs_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @classmethod
    def from_bitmap(cls, G, bits):
        """vertexSubset(n, m, BitArray&&) (vertex_subset.h:263-270): members are
        the set bits of `bits`, a device array of ceil(n/32) uint32 words
        (anything with data_ptr(), e.g. a CUDA tensor); None: every vertex."""
        h = ctypes.c_void_p()
        if bits is None:
            check(lib().byo_vs_create_all(G.h, ctypes.byref(h)), G.ctx.h)
        else:
            check(lib().byo_vs_create_bitmap(G.h, bits.data_ptr(), ctypes.byref(h)), G.ctx.h)
        return cls(G, _handle=h)

    @classmethod
    def all(cls, G):
        return cls.from_bitmap(G, None)

    def size(self):
        return int(lib().byo_vs_size(self.h))

    def isEmpty(self):
        return self.size() == 0

    @property
    def isDense(self):
        return bool(lib().byo_vs_is_dense(self.h))

    def to_list(self):
        s = self.size()
        out = np.empty(max(s, 1), np.uint32)
        check(lib().byo_vs_to_list(self.h, _ptr(out), s), self.G.ctx.h)
        return out[:s]


class BFS_F:
    """BFS_F (BFS.h:30-45) over a device Parents array."""

    def __init__(self, G, src):
        self.G = G
        h = ctypes.c_void_p()
        check(lib().byo_functor_bfs_create(G.h, src, ctypes.byref(h)), G.ctx.h)
        self.h = h
        G.ctx._adopt(self)

    def close(self):
        if getattr(self, "h", None):
            lib().byo_functor_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def parents(self):
        out = np.empty(self.G.N(), np.uint32)
        check(lib().byo_functor_bfs_parents(self.h, _ptr(out)), self.G.ctx.h)
        return out


class _DeviceFunctor:
    """A device functor over caller arrays (CUDA tensors, kept alive here)."""

    def __init__(self, G, create, *args):
        self.G = G
        self._keep = [a for a in args if hasattr(a, "data_ptr")]
        h = ctypes.c_void_p()
        conv = [a.data_ptr() if hasattr(a, "data_ptr") else a for a in args]
        check(create(G.h, *conv, ctypes.byref(h)), G.ctx.h)
        self.h = h
        G.ctx._adopt(self)

    def close(self):
        if getattr(self, "h", None):
            lib().byo_functor_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class BFS_ComponentLabel_F(_DeviceFunctor):
    """BFS_ComponentLabel_F (benchmarks/Connectivity/BFSCC/Connectivity.h:31-50)
    over a device Parents array of n uint32 (int32 tensor)."""

    def __init__(self, G, parents, src):
        super().__init__(G, lib().byo_functor_bfs_label_create, int(src), parents)


class PR_F(_DeviceFunctor):
    """PR_F (benchmarks/PageRank/PageRank.h:33-50) over device float64 arrays."""

    def __init__(self, G, p_curr, p_next):
        super().__init__(G, lib().byo_functor_pr_create, p_curr, p_next)


class PR_Delta_F(_DeviceFunctor):
    """delta::PR_Delta_F (benchmarks/PageRank/PageRank.h:200-226): delta is a
    device float64 array of n {delta, delta / degree} pairs, ngh_sum n float64."""

    def __init__(self, G, delta, ngh_sum):
        super().__init__(G, lib().byo_functor_pr_delta_create, delta, ngh_sum)


def _vop(kind, a=None, b=None, c=None, damping=0.85, eps2=0.0):
    ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    return _abi.VertexOp(kind, ptr(a), ptr(b), ptr(c), damping, eps2)


def vertexMap(vs, kind, a=None, b=None, c=None, damping=0.85, eps2=0.0):
    """vertexMap (vertex_subset.h:382-398) with a vertex function of the
    reference (_abi.VOP_*; arrays as include/byo_gpu.h byo_vertex_op says)."""
    op = _vop(kind, a, b, c, damping, eps2)
    check(lib().byo_vertex_map(vs.h, ctypes.byref(op)), vs.G.ctx.h)


def vertexFilter(vs, kind, a=None, b=None, c=None, damping=0.85, eps2=0.0):
    """vertexFilter (vertex_subset.h:441-485): the members the function keeps."""
    op = _vop(kind, a, b, c, damping, eps2)
    h = ctypes.c_void_p()
    check(lib().byo_vertex_filter(vs.h, ctypes.byref(op), ctypes.byref(h)), vs.G.ctx.h)
    return vertexSubset(vs.G, _handle=h)


def edgeMap(G, vs, F, threshold=-1, flags=0):
    h = ctypes.c_void_p()
    check(lib().byo_edge_map(G.h, vs.h, F.h, threshold, flags, ctypes.byref(h)), G.ctx.h)
    return vertexSubset(G, _handle=h)


# ------------------------------------------------------------ algorithms

def BFS(G, src, policy=_abi.POLICY_M20, levels=False, out=None):
    """Parents (and levels); `out` may supply the parents array (e.g. pinned)."""
    n = G.N()
    par = out if out is not None else np.empty(n, np.uint32)
    lev = np.empty(n, np.uint32) if levels else None
    r = ctypes.c_uint32(0)
    check(lib().byo_bfs(G.h, src, _ptr(par), _ptr(lev), policy, ctypes.byref(r)), G.ctx.h)
    return (par, lev) if levels else par


def BFS_multi(G, sources):
    """Levels from up to 64 sources in one bit-lane traversal: array [k, n]."""
    srcs = np.ascontiguousarray(sources, np.uint32)
    out = np.empty((len(srcs), G.N()), np.uint32)
    r = ctypes.c_uint32(0)
    check(lib().byo_bfs_multi(G.h, _ptr(srcs), len(srcs), _ptr(out), ctypes.byref(r)), G.ctx.h)
    return out


def SimpleUnionAsync(G, out=None):
    out = out if out is not None else np.empty(G.N(), np.uint32)
    check(lib().byo_cc(G.h, _ptr(out)), G.ctx.h)
    return out


def bfs_cc(G):
    out = np.empty(G.N(), np.uint32)
    check(lib().byo_bfs_cc(G.h, _ptr(out)), G.ctx.h)
    return out


def PageRank(G, eps=1e-6, max_iters=100, precision=_abi.PR_FP32_KAHAN, info=False, out=None):
    p = out if out is not None else np.empty(G.N(), np.float64)
    it = ctypes.c_uint32(0)
    l1 = ctypes.c_double(0)
    check(lib().byo_pagerank(G.h, eps, max_iters, precision, _ptr(p), ctypes.byref(it),
                             ctypes.byref(l1)), G.ctx.h)
    return (p, it.value, l1.value) if info else p


def read_adj_host(path, binary=False):
    """Parses a graph file on the host (no device): (offsets, nbrs)."""
    n, m = ctypes.c_uint64(0), ctypes.c_uint64(0)
    p = os.fsencode(path)
    check(lib().byo_adj_read(p, int(binary), ctypes.byref(n), ctypes.byref(m), None, None))
    off = np.empty(n.value + 1, np.uint64)
    nb = np.empty(max(m.value, 1), np.uint32)
    check(lib().byo_adj_read(p, int(binary), ctypes.byref(n), ctypes.byref(m), _ptr(off), _ptr(nb)))
    return off, nb[:m.value]


def PageRank_edgeMap(G, eps=1e-6, max_iters=100, info=False):
    """PageRank_edgeMap (PageRank.h:80-123): PageRank's recurrence in FP64."""
    p = np.empty(G.N(), np.float64)
    it = ctypes.c_uint32(0)
    l1 = ctypes.c_double(0)
    check(lib().byo_pagerank_edgemap(G.h, eps, max_iters, _ptr(p), ctypes.byref(it), ctypes.byref(l1)), G.ctx.h)
    return (p, it.value, l1.value) if info else p


def PageRankDelta(G, eps=1e-6, local_eps=0.01, max_iters=100, info=False):
    """delta::PageRankDelta (PageRank.h:340-398), FP64."""
    p = np.empty(G.N(), np.float64)
    r = ctypes.c_uint32(0)
    l1 = ctypes.c_double(0)
    check(lib().byo_pagerank_delta(G.h, eps, local_eps, max_iters, _ptr(p), ctypes.byref(r), ctypes.byref(l1)),
          G.ctx.h)
    return (p, r.value, l1.value) if info else p


def Test_Map(G):
    """Test_Map (benchmarks/Map/Base/Map.h:8-18): sum of every edge's destination."""
    c = ctypes.c_uint64(0)
    check(lib().byo_map_sum(G.h, ctypes.byref(c)), G.ctx.h)
    return int(c.value)


def Test_Map_Remote(G, remote, width):
    """Test_Map_Remote (benchmarks/Map/RemoteRead/Map.h:21-33): sum over every
    edge (u, v) of remote[v].  `remote` holds n elements of `width` bytes
    (0: a bitmap of uint64 words, least significant bit first; 16, 32: a
    uint64 at the start of each element), as a host array or a CUDA tensor."""
    c = ctypes.c_uint64(0)
    if hasattr(remote, "data_ptr"):
        check(lib().byo_map_remote_device(G.h, remote.data_ptr(), width, ctypes.byref(c)), G.ctx.h)
    else:
        buf = np.ascontiguousarray(remote)
        check(lib().byo_map_remote(G.h, buf.ctypes.data_as(ctypes.c_void_p), width, ctypes.byref(c)), G.ctx.h)
    return int(c.value)


def Triangle_degree_ordering(G):
    c = ctypes.c_uint64(0)
    check(lib().byo_triangle_count(G.h, ctypes.byref(c)), G.ctx.h)
    return int(c.value)
