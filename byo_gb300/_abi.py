"""ctypes binding of libbyo_gpu.so (the C ABI in include/byo_gpu.h).

The library is the product: there is no CPU fallback.  Importing works
without a GPU (so the ABI can be inspected), but every call that touches a
device fails with BYO_EDEVICE when none is present, and loading fails loudly
when the library has not been built.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libbyo_gpu.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "byo_gpu.h")

BYO_OK = 0
BYO_EINVAL = -1
BYO_ENOMEM = -2
BYO_EDEVICE = -3
BYO_ETIMEDOUT = -4
BYO_ENOTSUP = -5
NONE = 0xFFFFFFFF

CONTAINER_CSR = 0
CONTAINER_PMA = 1
CONTAINER_VOS = 2
CONTAINER_PCSR = 3

GEN_RMAT, GEN_ER, GEN_GRID, GEN_CHUNG_LU = 0, 1, 2, 3

POLICY_M20 = 0
POLICY_LEARNED = 1
POLICY_PUSH = 2
POLICY_PULL = 3
POLICY_BLOCKED = 4
POLICY_M20_BLOCKED = 5

PR_FP32_KAHAN = 0
PR_FP64 = 1
PR_FP32 = 2

FL_NO_OUTPUT = 1
FL_SPARSE_BLOCKED = 4
FL_DENSE_FORWARD = 8
FL_DENSE_PARALLEL = 16
FL_NO_DENSE = 64
FL_DENSE_ONLY = 1024

_c = ctypes
_vp = ctypes.c_void_p
_u32 = ctypes.c_uint32
_u64 = ctypes.c_uint64
_i64 = ctypes.c_int64
_int = ctypes.c_int
_dbl = ctypes.c_double
_P = ctypes.POINTER


TUNE_BFS = 1
TUNE_MULTI = 2


class Tuning(ctypes.Structure):
    _fields_ = [("push_group", _u32), ("hub_min", _u32), ("pull_cap", _u32), ("blocked_tile", _u32),
                ("ms_heavy_deg", _u32), ("ms_hub_deg", _u32), ("ms_push_div", _u32), ("pull_stage_words", _u32),
                ("tc_stage", _u32), ("reserved", _u32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class GenSpec(ctypes.Structure):
    _fields_ = [("kind", _int), ("seed", _u64), ("lg_n", _u32), ("n", _u64), ("draws", _u64),
                ("a", _dbl), ("b", _dbl), ("c", _dbl), ("exponent", _dbl)]


class RoundLog(ctypes.Structure):
    _fields_ = [("round", _u32), ("mode", _u32), ("frontier", _u64), ("frontier_deg", _u64),
                ("unvisited", _u64), ("ms", ctypes.c_float), ("features", ctypes.c_float * 16)]


F_BFS, F_BFS_LABEL, F_PR, F_PR_DELTA = 0, 1, 2, 3
OP_REMOVE, OP_INSERT, OP_QUERY = 0, 1, 2
VOP_PR_UPDATE, VOP_ZERO, VOP_PR_DELTA_FIRST, VOP_PR_DELTA = 0, 1, 2, 3


class VertexOp(ctypes.Structure):
    _fields_ = [("kind", _int), ("d_a", _vp), ("d_b", _vp), ("d_c", _vp), ("damping", _dbl), ("eps2", _dbl)]


class UpdateStats(ctypes.Structure):
    _fields_ = [("keys", _u64), ("changed", _u64), ("touched_leaves", _u64), ("touched_entries", _u64),
                ("leaf_slots", _u64), ("path", _u32), ("reserved", _u32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


# name -> (restype, argtypes)
SIGNATURES = {
    "byo_version": (ctypes.c_char_p, []),
    "byo_gpu_init": (_int, [_int, _P(_vp)]),
    "byo_gpu_shutdown": (None, [_vp]),
    "byo_last_error": (ctypes.c_char_p, [_vp]),
    "byo_ctx_stream": (_vp, [_vp]),
    "byo_ctx_launches": (_u64, [_vp]),
    "byo_ctx_synchronize": (_int, [_vp]),
    "byo_buffer_alloc": (_int, [_vp, _u64, _P(_vp)]),
    "byo_buffer_free": (None, [_vp, _vp]),
    "byo_buffer_write": (_int, [_vp, _vp, _u64, _vp, _u64]),
    "byo_buffer_read": (_int, [_vp, _vp, _u64, _vp, _u64]),
    "byo_buffer_fill32": (_int, [_vp, _vp, _u64, _u64, _u32]),
    "byo_ctx_set_round_timing": (_int, [_vp, _int]),
    "byo_ctx_set_barrier_test": (_int, [_vp, _u32, _u32]),
    "byo_ctx_set_pagerank_graphs": (_int, [_vp, _int]),
    "byo_gather_roof": (_int, [_vp, _u64, _P(_dbl)]),
    "byo_ctx_kernel_timing": (_int, [_vp, ctypes.c_char_p]),
    "byo_ctx_kernel_time": (_int, [_vp, ctypes.c_char_p, _P(_u64), _P(_dbl)]),
    "byo_graph_create_csr": (_int, [_vp, _u64, _u64, _vp, _vp, _P(_vp)]),
    "byo_graph_create_pma": (_int, [_vp, _u64, _u64, _vp, _vp, _P(_vp)]),
    "byo_graph_generate": (_int, [_vp, _int, _P(GenSpec), _P(_vp)]),
    "byo_graph_destroy": (None, [_vp]),
    "byo_graph_container": (_int, [_vp]),
    "byo_graph_num_vertices": (_u64, [_vp]),
    "byo_graph_num_edges": (_u64, [_vp]),
    "byo_graph_num_slots": (_u64, [_vp]),
    "byo_graph_degrees": (_int, [_vp, _vp]),
    "byo_graph_export_csr": (_int, [_vp, _vp, _vp]),
    "byo_graph_neighbors": (_int, [_vp, _u32, _vp, _u64, _P(_u64)]),
    "byo_graph_insert_batch": (_int, [_vp, _vp, _u64, _int, _P(_u64)]),
    "byo_graph_remove_batch": (_int, [_vp, _vp, _u64, _int, _P(_u64)]),
    "byo_graph_insert_batch_device": (_int, [_vp, _vp, _u64, _int, _P(_u64)]),
    "byo_graph_remove_batch_device": (_int, [_vp, _vp, _u64, _int, _P(_u64)]),
    "byo_graph_last_update_stats": (_int, [_vp, _P(UpdateStats)]),
    "byo_gen_rmat_pairs_device": (_int, [_vp, _u64, _u32, _dbl, _dbl, _dbl, _u64, _u64, _vp, _vp]),
    "byo_gen_uniform_pairs_device": (_int, [_vp, _u64, _u64, _u64, _u64, _vp, _vp]),
    "byo_gen_uniform_keys_device": (_int, [_vp, _u64, _u64, _u64, _vp]),
    "byo_bfs": (_int, [_vp, _u32, _vp, _vp, _int, _P(_u32)]),
    "byo_bfs_device": (_int, [_vp, _u32, _vp, _vp, _int, _P(_u32)]),
    "byo_bfs_multi": (_int, [_vp, _vp, _u32, _vp, _P(_u32)]),
    "byo_bfs_multi_device": (_int, [_vp, _vp, _u32, _vp, _P(_u32)]),
    "byo_adj_read": (_int, [ctypes.c_char_p, _int, _P(_u64), _P(_u64), _vp, _vp]),
    "byo_graph_read_adj": (_int, [_vp, ctypes.c_char_p, _int, _int, _P(_vp)]),
    "byo_graph_write_adj": (_int, [_vp, ctypes.c_char_p, _int]),
    "byo_graph_get_tuning": (_int, [_vp, _P(Tuning)]),
    "byo_graph_set_tuning": (_int, [_vp, _P(Tuning)]),
    "byo_graph_autotune": (_int, [_vp, _u32, _u32, _P(Tuning)]),
    "byo_cc": (_int, [_vp, _vp]),
    "byo_cc_device": (_int, [_vp, _vp]),
    "byo_bfs_cc": (_int, [_vp, _vp]),
    "byo_pagerank": (_int, [_vp, _dbl, _u32, _int, _vp, _P(_u32), _P(_dbl)]),
    "byo_pagerank_device": (_int, [_vp, _dbl, _u32, _int, _vp, _P(_u32), _P(_dbl)]),
    "byo_pagerank_edgemap": (_int, [_vp, _dbl, _u32, _vp, _P(_u32), _P(_dbl)]),
    "byo_pagerank_delta": (_int, [_vp, _dbl, _dbl, _u32, _vp, _P(_u32), _P(_dbl)]),
    "byo_pagerank_delta_device": (_int, [_vp, _dbl, _dbl, _u32, _vp, _P(_u32), _P(_dbl)]),
    "byo_triangle_count": (_int, [_vp, _P(_u64)]),
    "byo_map_sum": (_int, [_vp, _P(_u64)]),
    "byo_graph_create": (_int, [_vp, _int, _u64, _u64, _vp, _vp, _P(_vp)]),
    "byo_graph_update_stream": (_int, [_vp, _vp, _vp, _vp, _u64, _vp]),
    "byo_graph_update_stream_device": (_int, [_vp, _vp, _vp, _vp, _u64, _vp]),
    "byo_graph_mixed_stream": (_int, [_vp, _vp, _vp, _vp, _u64, _vp, _u32, _vp, _vp, _vp]),
    "byo_graph_mixed_stream_device": (_int, [_vp, _vp, _vp, _vp, _u64, _vp, _u32, _vp, _vp, _vp]),
    "byo_graph_from_bytepd": (_int, [_vp, _u64, _vp, _vp, _vp, _u64, _u32, _int, _P(_vp)]),
    "byo_graph_read_bytepd": (_int, [_vp, ctypes.c_char_p, _u32, _int, _P(_vp)]),
    "byo_graph_write_bytepd": (_int, [_vp, ctypes.c_char_p, _u32]),
    "byo_graph_encode_bytepd": (_int, [_vp, _u32, _vp, _vp, _vp, _P(_u64)]),
    "byo_map_remote": (_int, [_vp, _vp, _u32, _P(_u64)]),
    "byo_map_remote_device": (_int, [_vp, _vp, _u32, _P(_u64)]),
    "byo_functor_bfs_create": (_int, [_vp, _u32, _P(_vp)]),
    "byo_functor_bfs_parents": (_int, [_vp, _vp]),
    "byo_functor_destroy": (None, [_vp]),
    "byo_functor_bfs_label_create": (_int, [_vp, _u32, _vp, _P(_vp)]),
    "byo_functor_pr_create": (_int, [_vp, _vp, _vp, _P(_vp)]),
    "byo_functor_pr_delta_create": (_int, [_vp, _vp, _vp, _P(_vp)]),
    "byo_functor_kind": (_int, [_vp]),
    "byo_vs_create_bitmap": (_int, [_vp, _vp, _P(_vp)]),
    "byo_vs_create_all": (_int, [_vp, _P(_vp)]),
    "byo_vertex_map": (_int, [_vp, _P(VertexOp)]),
    "byo_vertex_filter": (_int, [_vp, _P(VertexOp), _P(_vp)]),
    "byo_vs_create_single": (_int, [_vp, _u32, _P(_vp)]),
    "byo_vs_create_list": (_int, [_vp, _vp, _u64, _P(_vp)]),
    "byo_vs_destroy": (None, [_vp]),
    "byo_vs_size": (_u64, [_vp]),
    "byo_vs_is_dense": (_int, [_vp]),
    "byo_vs_to_list": (_int, [_vp, _vp, _u64]),
    "byo_edge_map": (_int, [_vp, _vp, _vp, _i64, _u32, _P(_vp)]),
    "byo_last_rounds": (_int, [_vp, _P(RoundLog), _u64, _P(_u64)]),
    "byo_bfs_csr_noalloc": (_int, [_vp, _vp, _u64, _u64, _u32, _vp, _vp, _vp, _P(_u32)]),
    "byo_ctx_set_update_policy": (_int, [_vp, _int]),
    "byo_ctx_last_update_strategy": (_int, [_vp]),
    "byo_policy_init_params": (_int, [_u64, _vp]),
    "byo_policy_set_params": (_int, [_vp, _vp]),
    "byo_policy_get_params": (_int, [_vp, _vp]),
    "byo_policy_clear": (_int, [_vp]),
    "byo_policy_forward": (_int, [_vp, _vp, _vp, _u64, _vp]),
    "byo_policy_loss_grad": (_int, [_vp, _vp, _vp, _vp, _vp, _u64, _P(ctypes.c_float), _vp]),
    "byo_policy_train": (_int, [_vp, _vp, _vp, _vp, _vp, _u64, _u32, ctypes.c_float, _u64, _vp]),
    "byo_update_sample": (_int, [_vp, _vp, _u64, _vp, _vp, _vp]),
}
POLICY_NFEATURES, POLICY_NOUTPUTS, POLICY_NPARAMS = 16, 5, 1765
UPDATE_MERGE, UPDATE_LEARNED, UPDATE_REBUILD = 0, 1, 2
NOALLOC_MAX_VERTICES = 1 << 20

_lib = None


class ByoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("byo_gpu error %d: %s" % (code, msg))
        self.code = code


def lib():
    """Loads libbyo_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libbyo_gpu.so not built (run `python -m byo_gb300.build` or "
                              "__graft_entry__.build()): " + LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, ctx=None):
    if rc != BYO_OK:
        msg = lib().byo_last_error(ctx).decode() if ctx else ""
        raise ByoError(rc, msg)
    return rc
