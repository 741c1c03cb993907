"""GB300-native set-intersection pattern engine (EmptyHeaded's hot path).

Thin ctypes binding over the C ABI in include/eh_gb300.h, used by the tests and
the benchmark.  The engine itself is libeh_gb300.so (CUDA for sm_103a + host
C++); this module holds no compute.  Loading fails loudly when the library is
missing: there is no fallback path.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))

# Layout codes (the reference's common::type values, src/common.hpp:171-181).
BITSET, PSHORT, UINTEGER, HYBRID, HYBRID3 = 0, 1, 2, 5, 16
LAYOUTS = {"bs": BITSET, "bitset": BITSET, "pshort": PSHORT, "uint": UINTEGER,
           "uinteger": UINTEGER, "hybrid": HYBRID, "hybrid3": HYBRID3}
SELECT_ALL, SELECT_LOWER, SELECT_MASK = 0, 1, 2
SELECTIONS = {"all": SELECT_ALL, "lower": SELECT_LOWER, "mask": SELECT_MASK}

STATUS = {0: "EH_OK", 1: "EH_ERR_INVALID_ARGUMENT", 2: "EH_ERR_CUDA", 3: "EH_ERR_OUT_OF_MEMORY",
          4: "EH_ERR_UNSUPPORTED", 5: "EH_ERR_IO", 6: "EH_ERR_DEVICE_CHECK", 7: "EH_ERR_TIMEOUT",
          8: "EH_ERR_ADMISSION"}


class EHError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Tuning(C.Structure):
    _fields_ = [("light_max", C.c_uint32), ("unit_span", C.c_uint32), ("ctas_per_sm", C.c_uint32),
                ("core_rows", C.c_uint32), ("ms", C.c_float), ("configs_tried", C.c_uint32),
                ("core_hot_words", C.c_uint32), ("core_filter_words", C.c_uint32)]


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("hbm_cap_bytes", C.c_uint64)]


class QueryResult(C.Structure):
    _fields_ = [("count", C.c_uint64), ("status", C.c_int32), ("slot", C.c_int32),
                ("submit_ns", C.c_int64), ("start_ns", C.c_int64), ("done_ns", C.c_int64)]


class ServerCounters(C.Structure):
    _fields_ = [("graphs", C.c_uint32), ("slots", C.c_uint32), ("queued", C.c_uint64), ("completed", C.c_uint64),
                ("launched", C.c_uint64), ("max_inflight", C.c_uint64), ("resident_bytes", C.c_uint64),
                ("scratch_bytes", C.c_uint64), ("hbm_cap_bytes", C.c_uint64)]


QUERY_TRIANGLES, QUERY_CLIQUES, QUERY_SIMILAR_NODES = 0, 1, 2


class MatrixInfo(C.Structure):
    _fields_ = [("matrix_size", C.c_uint64), ("cardinality", C.c_uint64),
                ("row_total_bytes_used", C.c_uint64), ("max_nbrhood_size", C.c_uint64),
                ("max_row_cardinality", C.c_uint64), ("num_uint_rows", C.c_uint64),
                ("num_pshort_rows", C.c_uint64), ("num_bitset_rows", C.c_uint64),
                ("device_bytes", C.c_uint64), ("layout", C.c_int32), ("selection", C.c_int32)]


_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Loads libeh_gb300.so (building it first if absent and allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError("libeh_gb300.so is not built; run simdgraphprocessing_gb300.build.build()")
        _build.build()
    L = C.CDLL(path)
    P, U64, U32, I = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int
    sig = {
        "eh_last_error": (C.c_char_p, []),
        "eh_status_string": (C.c_char_p, [I]),
        "eh_version": (C.c_char_p, []),
        "eh_hgraph_from_csr": (I, [U64, P, P, P, C.POINTER(P)]),
        "eh_hgraph_read_binary": (I, [C.c_char_p, C.POINTER(P)]),
        "eh_hgraph_write_binary": (I, [P, C.c_char_p]),
        "eh_hgraph_read_edge_list": (I, [C.c_char_p, C.POINTER(P)]),
        "eh_hgraph_reorder_by_degree": (I, [P]),
        "eh_hgraph_view": (I, [P, C.POINTER(U64), C.POINTER(U64), C.POINTER(C.POINTER(U64)),
                               C.POINTER(C.POINTER(U32)), C.POINTER(C.POINTER(U64)), C.POINTER(U64)]),
        "eh_hgraph_free": (None, [P]),
        "eh_hgraph_read_directed_binary": (I, [C.c_char_p, C.POINTER(P)]),
        "eh_hgraph_write_directed_binary": (I, [P, C.c_char_p]),
        "eh_hgraph_read_directed_edge_list": (I, [C.c_char_p, C.POINTER(P)]),
        "eh_hgraph_directed_from_csr": (I, [U64, P, P, P, C.POINTER(P)]),
        "eh_hgraph_in_view": (I, [P, C.POINTER(I), C.POINTER(U64), C.POINTER(C.POINTER(U64)),
                                  C.POINTER(C.POINTER(U32))]),
        "eh_generate_directed_rmat": (I, [U32, U64, C.c_double, C.c_double, C.c_double, U64, C.POINTER(P)]),
        "eh_generate_rmat": (I, [U32, U64, C.c_double, C.c_double, C.c_double, U64, C.POINTER(P)]),
        "eh_generate_er": (I, [U64, U64, U64, C.POINTER(P)]),
        "eh_generate_ba": (I, [U64, U32, U64, C.POINTER(P)]),
        "eh_generate_planted_cliques": (I, [U64, U64, U32, U32, U32, U64, C.POINTER(P)]),
        "eh_matrix_build": (I, [U64, P, P, P, I, I, P, C.POINTER(P)]),
        "eh_matrix_build_device": (I, [U64, P, P, P, I, I, P, C.POINTER(P)]),
        "eh_matrix_get_info": (I, [P, C.POINTER(MatrixInfo)]),
        "eh_matrix_row_meta": (I, [P, P, P, P]),
        "eh_matrix_export_row": (I, [P, U32, P, U64, C.POINTER(U64)]),
        "eh_matrix_export_flattened": (I, [P, P, U64, C.POINTER(U64)]),
        "eh_matrix_get_max_row_id": (I, [P, C.POINTER(U32)]),
        "eh_matrix_triangle_bytes": (I, [P, C.POINTER(U64)]),
        "eh_matrix_free": (None, [P]),
        "eh_count_triangles": (I, [P, C.POINTER(U64), P]),
        "eh_count_triangles_async": (I, [P, P, P]),
        "eh_count_cliques": (I, [P, U32, C.POINTER(U64), P]),
        "eh_count_cliques_async": (I, [P, U32, P, P]),
        "eh_count_lollipops": (I, [P, C.POINTER(U64), P]),
        "eh_count_lollipops_async": (I, [P, P, P]),
        "eh_similar_nodes": (I, [P, U32, C.POINTER(U64), P]),
        "eh_similar_nodes_async": (I, [P, U32, P, P]),
        "eh_intersect_rows": (I, [P, P, P, U64, P, P]),
        "eh_symbiosity": (I, [P, P, C.c_double, C.POINTER(U64), P]),
        "eh_symbiosity_async": (I, [P, P, C.c_double, P, P]),
        "eh_bfs_path_length": (I, [P, U32, U64, C.POINTER(U64), C.POINTER(U64), P]),
        "eh_selftest_bounded_wait": (I, [U32, C.POINTER(U32)]),
        "eh_list_triangles": (I, [P, P, U64, P, P]),
        "eh_list_cliques": (I, [P, U32, P, U64, P, P]),
        "eh_matrix_tune": (I, [P, P, C.POINTER(Tuning)]),
        "eh_matrix_tune_for": (I, [P, C.c_uint32, P, C.POINTER(Tuning)]),
        "eh_matrix_set_shape": (I, [P, C.POINTER(Tuning), P]),
        "eh_batch_build": (I, [U32, P, U64, P, P, I, P, C.POINTER(P)]),
        "eh_batch_count": (I, [P, U32, P, P]),
        "eh_batch_run": (I, [P, P, P, I, P]),
        "eh_batch_tune": (I, [P, P, C.POINTER(Tuning)]),
        "eh_batch_matrix": (I, [P, C.POINTER(P)]),
        "eh_batch_free": (None, [P]),
        "eh_dcsr_from_edges": (I, [U64, U64, P, P, I, I, P, C.POINTER(P)]),
        "eh_dcsr_view": (I, [P, C.POINTER(U64), C.POINTER(U64), C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
        "eh_dcsr_free": (None, [P]),
        "eh_server_create": (I, [C.POINTER(ServerConfig), C.POINTER(P)]),
        "eh_server_add_graph": (I, [P, U64, P, P, I, C.POINTER(U32)]),
        "eh_server_submit": (I, [P, U32, I, U32, C.POINTER(U64)]),
        "eh_server_wait": (I, [P, U64, U32, C.POINTER(QueryResult)]),
        "eh_server_run_alone": (I, [P, U32, I, U32, C.POINTER(U64)]),
        "eh_server_stats": (I, [P, C.POINTER(ServerCounters)]),
        "eh_server_free": (None, [P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status):
    if status != 0:
        raise EHError(status, load().eh_last_error().decode(errors="replace"))


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _stream(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class HostGraph:
    """The reference's MutableGraph: symmetric adjacency in CSR form on the host,
    or the out- and in-neighbourhoods of a directed graph."""

    def __init__(self, handle):
        self.h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            load().eh_hgraph_free(self.h)
            self.h = None

    @classmethod
    def from_csr(cls, offsets, nbrs, ext_ids=None):
        offsets = np.ascontiguousarray(offsets, np.uint64)
        nbrs = np.ascontiguousarray(nbrs, np.uint32)
        ext = None if ext_ids is None else np.ascontiguousarray(ext_ids, np.uint64)
        h = C.c_void_p()
        check(load().eh_hgraph_from_csr(len(offsets) - 1, _p(offsets), _p(nbrs), _p(ext), C.byref(h)))
        return cls(h)

    @classmethod
    def read_binary(cls, path):
        h = C.c_void_p()
        check(load().eh_hgraph_read_binary(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def read_edge_list(cls, path):
        h = C.c_void_p()
        check(load().eh_hgraph_read_edge_list(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def read_directed_binary(cls, path):
        h = C.c_void_p()
        check(load().eh_hgraph_read_directed_binary(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def read_directed_edge_list(cls, path):
        h = C.c_void_p()
        check(load().eh_hgraph_read_directed_edge_list(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def directed_from_csr(cls, offsets, nbrs, ext_ids=None):
        offsets = np.ascontiguousarray(offsets, np.uint64)
        nbrs = np.ascontiguousarray(nbrs, np.uint32)
        ext = None if ext_ids is None else np.ascontiguousarray(ext_ids, np.uint64)
        h = C.c_void_p()
        check(load().eh_hgraph_directed_from_csr(len(offsets) - 1, _p(offsets), _p(nbrs), _p(ext), C.byref(h)))
        return cls(h)

    @classmethod
    def directed_rmat(cls, scale, num_edges, seed, a=0.57, b=0.19, c=0.19):
        h = C.c_void_p()
        check(load().eh_generate_directed_rmat(scale, num_edges, a, b, c, seed, C.byref(h)))
        return cls(h)

    @classmethod
    def rmat(cls, scale, num_edges, seed, a=0.57, b=0.19, c=0.19):
        h = C.c_void_p()
        check(load().eh_generate_rmat(scale, num_edges, a, b, c, seed, C.byref(h)))
        return cls(h)

    @classmethod
    def er(cls, n, num_edges, seed):
        h = C.c_void_p()
        check(load().eh_generate_er(n, num_edges, seed, C.byref(h)))
        return cls(h)

    @classmethod
    def ba(cls, n, m, seed):
        h = C.c_void_p()
        check(load().eh_generate_ba(n, m, seed, C.byref(h)))
        return cls(h)

    @classmethod
    def planted_cliques(cls, n, background_edges, num_cliques, min_size, max_size, seed):
        h = C.c_void_p()
        check(load().eh_generate_planted_cliques(n, background_edges, num_cliques, min_size, max_size,
                                                 seed, C.byref(h)))
        return cls(h)

    def reorder_by_degree(self):
        check(load().eh_hgraph_reorder_by_degree(self.h))
        return self

    def write_binary(self, path):
        check(load().eh_hgraph_write_binary(self.h, os.fsencode(path)))

    def write_directed_binary(self, path):
        check(load().eh_hgraph_write_directed_binary(self.h, os.fsencode(path)))

    @property
    def directed(self):
        d = C.c_int()
        check(load().eh_hgraph_in_view(self.h, C.byref(d), None, None, None))
        return bool(d.value)

    def in_csr(self, copy=True):
        """(in_offsets u64[n+1], in_nbrs u32[m]): the columns (= csr() when undirected)."""
        n = int(self.csr(copy=False)[0].shape[0] - 1)
        d, m = C.c_int(), C.c_uint64()
        off, nb = C.POINTER(C.c_uint64)(), C.POINTER(C.c_uint32)()
        check(load().eh_hgraph_in_view(self.h, C.byref(d), C.byref(m), C.byref(off), C.byref(nb)))
        o = np.ctypeslib.as_array(off, (n + 1,))
        b = np.ctypeslib.as_array(nb, (m.value,)) if m.value else np.zeros(0, np.uint32)
        return (o.copy(), b.copy()) if copy else (o, b)

    def csr(self, copy=True):
        """(offsets u64[n+1], nbrs u32[m], ext_ids u64[n], max_nbrhood_size)."""
        n, m, mx = C.c_uint64(), C.c_uint64(), C.c_uint64()
        off, nb, ex = C.POINTER(C.c_uint64)(), C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint64)()
        check(load().eh_hgraph_view(self.h, C.byref(n), C.byref(m), C.byref(off), C.byref(nb),
                                    C.byref(ex), C.byref(mx)))
        o = np.ctypeslib.as_array(off, (n.value + 1,))
        b = np.ctypeslib.as_array(nb, (m.value,)) if m.value else np.zeros(0, np.uint32)
        e = np.ctypeslib.as_array(ex, (n.value,)) if n.value else np.zeros(0, np.uint64)
        if copy:
            o, b, e = o.copy(), b.copy(), e.copy()
        return o, b, e, mx.value


class Matrix:
    """The reference's SparseMatrix<T,R>, resident in device memory."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            load().eh_matrix_free(self.h)
            self.h = None

    @classmethod
    def build(cls, offsets, nbrs, selection="lower", layout="hybrid", mask=None, stream=None):
        """Host CSR arrays -> upload -> device select / optimize / encode."""
        offsets = np.ascontiguousarray(offsets, np.uint64)
        nbrs = np.ascontiguousarray(nbrs, np.uint32)
        mask = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        h = C.c_void_p()
        check(load().eh_matrix_build(len(offsets) - 1, _p(offsets), _p(nbrs), _p(mask),
                                     SELECTIONS.get(selection, selection), LAYOUTS.get(layout, layout),
                                     _stream(stream), C.byref(h)))
        return cls(h)

    @classmethod
    def build_device(cls, n, d_offsets, d_nbrs, selection="lower", layout="hybrid", d_mask=None,
                     stream=None):
        """Device pointers (ints) of offsets / nbrs already resident in HBM."""
        h = C.c_void_p()
        check(load().eh_matrix_build_device(n, C.c_void_p(d_offsets), C.c_void_p(d_nbrs),
                                            None if d_mask is None else C.c_void_p(d_mask),
                                            SELECTIONS.get(selection, selection),
                                            LAYOUTS.get(layout, layout), _stream(stream), C.byref(h)))
        return cls(h)

    def info(self):
        i = MatrixInfo()
        check(load().eh_matrix_get_info(self.h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in MatrixInfo._fields_}

    def row_meta(self):
        n = self.info()["matrix_size"]
        t = np.zeros(n, np.uint8)
        c = np.zeros(n, np.uint32)
        b = np.zeros(n, np.uint64)
        check(load().eh_matrix_row_meta(self.h, _p(t), _p(c), _p(b)))
        return t, c, b

    def export_row(self, row):
        nb = C.c_uint64()
        st = load().eh_matrix_export_row(self.h, row, None, 0, C.byref(nb))
        buf = np.zeros(max(1, nb.value), np.uint8)
        check(load().eh_matrix_export_row(self.h, row, _p(buf), len(buf), C.byref(nb)))
        del st
        return bytes(buf[:nb.value])

    def export_flattened(self):
        """All rows' flattened bytes back to back (the reference's row_arrays contents)."""
        nb = C.c_uint64()
        check(load().eh_matrix_export_flattened(self.h, None, 0, C.byref(nb)))
        buf = np.zeros(max(1, nb.value), np.uint8)
        check(load().eh_matrix_export_flattened(self.h, _p(buf), len(buf), C.byref(nb)))
        return bytes(buf[:nb.value])

    def dump(self):
        """All rows in the format of oracle/ref_rowdump.cpp (type, card, bytes, payload)."""
        t, c, b = self.row_meta()
        flat = self.export_flattened()
        out = bytearray()
        pos = 0
        for i in range(len(t)):
            nb = int(b[i])
            out += bytes([int(t[i])]) + int(c[i]).to_bytes(4, "little") + nb.to_bytes(8, "little")
            out += flat[pos:pos + nb]
            pos += nb
        return bytes(out)

    def max_row_id(self):
        r = C.c_uint32()
        check(load().eh_matrix_get_max_row_id(self.h, C.byref(r)))
        return r.value

    def triangle_bytes(self):
        b = C.c_uint64()
        check(load().eh_matrix_triangle_bytes(self.h, C.byref(b)))
        return b.value

    def count_triangles(self, stream=None):
        c = C.c_uint64()
        check(load().eh_count_triangles(self.h, C.byref(c), _stream(stream)))
        return c.value

    def count_triangles_async(self, d_out, stream=None):
        check(load().eh_count_triangles_async(self.h, C.c_void_p(d_out), _stream(stream)))

    def count_cliques(self, k=4, stream=None):
        c = C.c_uint64()
        check(load().eh_count_cliques(self.h, k, C.byref(c), _stream(stream)))
        return c.value

    def count_cliques_async(self, k, d_out, stream=None):
        check(load().eh_count_cliques_async(self.h, k, C.c_void_p(d_out), _stream(stream)))

    def count_lollipops(self, stream=None):
        c = C.c_uint64()
        check(load().eh_count_lollipops(self.h, C.byref(c), _stream(stream)))
        return c.value

    def count_lollipops_async(self, d_out, stream=None):
        check(load().eh_count_lollipops_async(self.h, C.c_void_p(d_out), _stream(stream)))

    def similar_nodes(self, threshold=10, stream=None):
        c = C.c_uint64()
        check(load().eh_similar_nodes(self.h, threshold, C.byref(c), _stream(stream)))
        return c.value

    def similar_nodes_async(self, threshold, d_out, stream=None):
        check(load().eh_similar_nodes_async(self.h, threshold, C.c_void_p(d_out), _stream(stream)))

    def symbiosity(self, cols=None, threshold=0.5, stream=None):
        """Rows whose out-row (this matrix) and in-row (`cols`; None = this
        matrix, as for an undirected graph) have Jaccard ratio > threshold."""
        c = C.c_uint64()
        check(load().eh_symbiosity(self.h, (cols or self).h, float(threshold), C.byref(c), _stream(stream)))
        return c.value

    def symbiosity_async(self, cols, threshold, d_out, stream=None):
        check(load().eh_symbiosity_async(self.h, (cols or self).h, float(threshold), C.c_void_p(d_out),
                                         _stream(stream)))

    def bfs(self, start, depth=0xEFFFFFF, stream=None):
        """n_path BFS from row `start`: (path_length, vertices reached)."""
        p, r = C.c_uint64(), C.c_uint64()
        check(load().eh_bfs_path_length(self.h, int(start), int(depth), C.byref(p), C.byref(r), _stream(stream)))
        return p.value, r.value

    def list_triangles(self, d_out, capacity, d_total, stream=None):
        check(load().eh_list_triangles(self.h, C.c_void_p(d_out), capacity, C.c_void_p(d_total),
                                       _stream(stream)))

    def list_cliques(self, k, d_out, capacity, d_total, stream=None):
        """eh_list_cliques: k-clique tuples (k = 3 or 4) into device memory."""
        check(load().eh_list_cliques(self.h, k, C.c_void_p(d_out), capacity, C.c_void_p(d_total),
                                     _stream(stream)))

    def tune(self, stream=None, counts_per_build=0):
        """eh_matrix_tune, or eh_matrix_tune_for when counts_per_build > 0."""
        t = Tuning()
        if counts_per_build:
            check(load().eh_matrix_tune_for(self.h, counts_per_build, _stream(stream), C.byref(t)))
        else:
            check(load().eh_matrix_tune(self.h, _stream(stream), C.byref(t)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def set_shape(self, light_max, unit_span, ctas_per_sm, core_rows, core_hot_words=0, core_filter_words=0,
                  stream=None):
        """Uses this work shape for later counts (eh_matrix_set_shape)."""
        t = Tuning(light_max=light_max, unit_span=unit_span, ctas_per_sm=ctas_per_sm, core_rows=core_rows,
                   core_hot_words=core_hot_words, core_filter_words=core_filter_words)
        check(load().eh_matrix_set_shape(self.h, C.byref(t), _stream(stream)))

    def intersect_rows(self, d_a, d_b, npairs, d_counts, stream=None):
        check(load().eh_intersect_rows(self.h, C.c_void_p(d_a), C.c_void_p(d_b), npairs,
                                       C.c_void_p(d_counts), _stream(stream)))


class DeviceCSR:
    """Symmetric CSR built on the device from raw edge arrays (eh_dcsr_*)."""

    def __init__(self, n, d_src, d_dst, num_edges, drop_self_loops=False, degree_order=True, stream=None):
        self.h = C.c_void_p()
        check(load().eh_dcsr_from_edges(n, num_edges, C.c_void_p(d_src), C.c_void_p(d_dst), int(drop_self_loops),
                                        int(degree_order), _stream(stream), C.byref(self.h)))

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            load().eh_dcsr_free(self.h)
            self.h = None

    def view(self):
        """(n, entries, d_offsets, d_nbrs, d_new2old) as device addresses (ints; 0 = none)."""
        n, m = C.c_uint64(), C.c_uint64()
        o, b, r = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(load().eh_dcsr_view(self.h, C.byref(n), C.byref(m), C.byref(o), C.byref(b), C.byref(r)))
        return n.value, m.value, o.value or 0, b.value or 0, r.value or 0

    def matrix(self, selection="lower", layout="hybrid", stream=None):
        n, _, o, b, _ = self.view()
        return Matrix.build_device(n, o, b, selection, layout, stream=stream)


class Batch:
    """Many graphs counted in one launch (block-diagonal union of their rows)."""

    def __init__(self, graph_rows, offsets, nbrs, layout="hybrid", stream=None):
        self.graph_rows = np.ascontiguousarray(graph_rows, np.uint64)
        offsets = np.ascontiguousarray(offsets, np.uint64)
        nbrs = np.ascontiguousarray(nbrs, np.uint32)
        self.num_graphs = len(self.graph_rows) - 1
        self.h = C.c_void_p()
        check(load().eh_batch_build(self.num_graphs, _p(self.graph_rows), len(offsets) - 1, _p(offsets),
                                    _p(nbrs), LAYOUTS.get(layout, layout), _stream(stream), C.byref(self.h)))

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            load().eh_batch_free(self.h)
            self.h = None

    def count(self, k, d_counts, stream=None):
        check(load().eh_batch_count(self.h, k, C.c_void_p(d_counts), _stream(stream)))

    def run(self, d_triangles, d_cliques4, use_graph=True, stream=None):
        check(load().eh_batch_run(self.h, C.c_void_p(d_triangles), C.c_void_p(d_cliques4), int(use_graph),
                                  _stream(stream)))

    def tune(self, stream=None):
        t = Tuning()
        check(load().eh_batch_tune(self.h, _stream(stream), C.byref(t)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def matrix_info(self):
        m = C.c_void_p()
        check(load().eh_batch_matrix(self.h, C.byref(m)))
        i = MatrixInfo()
        check(load().eh_matrix_get_info(m, C.byref(i)))
        return {k: getattr(i, k) for k, _ in MatrixInfo._fields_}


class Server:
    """Device-resident graphs answering triangle / clique / similar_nodes queries
    with continuous batching (see eh_server_* in include/eh_gb300.h)."""

    def __init__(self, slots=8, hbm_cap_bytes=150 << 30):
        cfg = ServerConfig(slots, hbm_cap_bytes)
        self.h = C.c_void_p()
        check(load().eh_server_create(C.byref(cfg), C.byref(self.h)))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            load().eh_server_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def add_graph(self, offsets, nbrs, layout="hybrid"):
        offsets = np.ascontiguousarray(offsets, np.uint64)
        nbrs = np.ascontiguousarray(nbrs, np.uint32)
        gid = C.c_uint32()
        check(load().eh_server_add_graph(self.h, len(offsets) - 1, _p(offsets), _p(nbrs),
                                         LAYOUTS.get(layout, layout), C.byref(gid)))
        return gid.value

    def submit(self, graph_id, kind, param=0):
        t = C.c_uint64()
        check(load().eh_server_submit(self.h, graph_id, kind, param, C.byref(t)))
        return t.value

    def wait(self, ticket, timeout_ms=60000):
        r = QueryResult()
        check(load().eh_server_wait(self.h, ticket, timeout_ms, C.byref(r)))
        return {k: getattr(r, k) for k, _ in QueryResult._fields_}

    def run_alone(self, graph_id, kind, param=0):
        c = C.c_uint64()
        check(load().eh_server_run_alone(self.h, graph_id, kind, param, C.byref(c)))
        return c.value

    def stats(self):
        c = ServerCounters()
        check(load().eh_server_stats(self.h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in ServerCounters._fields_}


def concat_graphs(csrs):
    """Block-diagonal union of (offsets, nbrs) pairs -> (graph_rows, offsets, nbrs)."""
    rows = [len(o) - 1 for o, _ in csrs]
    graph_rows = np.zeros(len(csrs) + 1, np.uint64)
    graph_rows[1:] = np.cumsum(rows)
    offs, nbs = [np.zeros(1, np.uint64)], []
    base_e = 0
    for g, (o, b) in enumerate(csrs):
        offs.append(o[1:].astype(np.uint64) + np.uint64(base_e))
        nbs.append(b.astype(np.uint32) + np.uint32(graph_rows[g]))
        base_e += len(b)
    return graph_rows, np.concatenate(offs), (np.concatenate(nbs) if nbs else np.zeros(0, np.uint32))


def _splitmix_np(x):
    """SplitMix64 output function on a u64 array (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = np.asarray(x, np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def orient(undirected, p_both, seed):
    """Directed graph from an undirected one: each edge {u, v} (u < v) becomes
    u->v and v->u with probability p_both, else one of the two with equal
    probability, decided by SplitMix64 of (u << 32 | v) keyed by `seed`."""
    off, nbr, _, _ = undirected.csr()
    n = len(off) - 1
    src = np.repeat(np.arange(n, dtype=np.uint64), np.diff(off).astype(np.int64))
    dst = nbr.astype(np.uint64)
    keep = src < dst
    u, v = src[keep], dst[keep]
    r = _splitmix_np(((u << np.uint64(32)) | v) ^ _splitmix_np(np.uint64(seed)))
    x = (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    fwd = (x < p_both) | (x < p_both + (1.0 - p_both) / 2.0)
    bwd = (x < p_both) | ~fwd
    s_all = np.concatenate([u[fwd], v[bwd]])
    d_all = np.concatenate([v[fwd], u[bwd]])
    order = np.lexsort((d_all, s_all))
    s_all, d_all = s_all[order], d_all[order]
    offs = np.zeros(n + 1, np.uint64)
    np.add.at(offs, s_all.astype(np.int64) + 1, 1)
    return HostGraph.directed_from_csr(np.cumsum(offs, dtype=np.uint64), d_all.astype(np.uint32))


def graph(kind, seed, **kw):
    """Seeded, degree-ordered generator graph -> HostGraph."""
    if kind == "rmat":
        g = HostGraph.rmat(kw["scale"], kw["edges"], seed, kw.get("a", 0.57), kw.get("b", 0.19),
                           kw.get("c", 0.19))
    elif kind == "er":
        g = HostGraph.er(kw["n"], kw["edges"], seed)
    elif kind == "ba":
        g = HostGraph.ba(kw["n"], kw["m"], seed)
    elif kind == "planted":
        g = HostGraph.planted_cliques(kw["n"], kw["edges"], kw["cliques"], kw["min_size"],
                                      kw["max_size"], seed)
    elif kind == "recip":
        # Directed: a degree-ordered undirected generator graph, oriented by orient().
        base = graph(kw["base"], seed, **kw["base_params"])
        return orient(base, kw["p_both"], seed)
    elif kind == "drmat":
        # Directed graphs keep their generated ids (degree reordering is undirected-only).
        return HostGraph.directed_rmat(kw["scale"], kw["edges"], seed, kw.get("a", 0.57), kw.get("b", 0.19),
                                       kw.get("c", 0.19))
    else:
        raise ValueError(kind)
    return g.reorder_by_degree()
