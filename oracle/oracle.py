"""ctypes binding of the C oracle (oracle/eh_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference legs of bench.py, where it is the checker or the timed
CPU baseline.  The product package never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SRC = [os.path.join(HERE, "eh_oracle.c"), os.path.join(HERE, "eh_gen.c")]

# Layout and selection codes shared with the engine (common::type values).
BITSET, PSHORT, UINTEGER, HYBRID, HYBRID3 = 0, 1, 2, 5, 16
SELECT_ALL, SELECT_LOWER, SELECT_MASK = 0, 1, 2
LAYOUTS = {"bs": BITSET, "pshort": PSHORT, "uint": UINTEGER, "hybrid": HYBRID, "hybrid3": HYBRID3}
SELECTIONS = {"all": SELECT_ALL, "lower": SELECT_LOWER, "mask": SELECT_MASK}


def build(force=False):
    """Compiles the oracle with the host gcc (no GPU needed)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and \
            all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(s) for s in SRC):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-std=gnu99", "-fPIC", "-shared", "-fopenmp", "-o", tmp, *SRC])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.oracle_build.restype = P
        L.oracle_build.argtypes = [C.c_uint64, P, P, P, C.c_int, C.c_int, C.c_int]
        L.oracle_free.argtypes = [P]
        L.oracle_info.argtypes = [P, P]
        L.oracle_row_meta.argtypes = [P, P, P, P]
        L.oracle_row_bytes.restype = C.POINTER(C.c_uint8)
        L.oracle_row_bytes.argtypes = [P, C.c_uint64, C.POINTER(C.c_uint64)]
        L.oracle_max_row_id.restype = C.c_uint32
        L.oracle_max_row_id.argtypes = [P]
        for f in ("oracle_triangles", "oracle_lollipops"):
            getattr(L, f).restype = C.c_uint64
            getattr(L, f).argtypes = [P, C.c_int]
        L.oracle_cliques.restype = C.c_uint64
        L.oracle_cliques.argtypes = [P, C.c_int, C.c_int]
        L.oracle_similar_nodes.restype = C.c_uint64
        L.oracle_similar_nodes.argtypes = [P, C.c_uint32, C.c_int]
        L.oracle_intersect_rows.argtypes = [P, P, P, C.c_uint64, P, C.c_int]
        L.oracle_triangles_range.restype = C.c_uint64
        L.oracle_triangles_range.argtypes = [P, C.c_uint64, C.c_uint64, C.c_int]
        L.oracle_max_threads.restype = C.c_int
        L.oracle_dump.restype = C.c_uint64
        L.oracle_dump.argtypes = [P, P]
        L.oracle_symbiosity.restype = C.c_uint64
        L.oracle_symbiosity.argtypes = [P, P, C.c_double, C.c_int]
        L.oracle_n_path.restype = C.c_uint64
        L.oracle_n_path.argtypes = [P, C.c_uint32, C.c_uint64, C.POINTER(C.c_uint64)]
        L.oracle_list_triangles.restype = C.c_uint64
        L.oracle_list_triangles.argtypes = [P, P, C.c_uint64]
        L.oracle_list_cliques.restype = C.c_uint64
        L.oracle_list_cliques.argtypes = [P, C.c_int, P, C.c_uint64]
        L.oracle_rmat.restype = C.c_uint64
        L.oracle_rmat.argtypes = [C.c_uint32, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                  C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        L.oracle_gen_free.argtypes = [P]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Matrix:
    """The oracle's SparseMatrix<T,R>: rows selected and encoded on the CPU."""

    def __init__(self, offsets, nbrs, selection, layout, mask=None, threads=0):
        self.offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        self.nbrs = np.ascontiguousarray(nbrs, dtype=np.uint32)
        self.mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        self.n = len(self.offsets) - 1
        self.threads = threads
        self.h = lib().oracle_build(self.n, _ptr(self.offsets), _ptr(self.nbrs), _ptr(self.mask),
                                    selection, layout, threads)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_free(self.h)
            self.h = None

    def info(self):
        out = np.zeros(6, np.uint64)
        lib().oracle_info(self.h, _ptr(out))
        keys = ("matrix_size", "cardinality", "row_total_bytes_used", "num_uint_rows",
                "num_pshort_rows", "num_bitset_rows")
        return {k: int(v) for k, v in zip(keys, out)}

    def row_meta(self):
        t = np.zeros(self.n, np.uint8)
        c = np.zeros(self.n, np.uint32)
        b = np.zeros(self.n, np.uint64)
        lib().oracle_row_meta(self.h, _ptr(t), _ptr(c), _ptr(b))
        return t, c, b

    def row_bytes(self, i):
        nb = C.c_uint64()
        p = lib().oracle_row_bytes(self.h, i, C.byref(nb))
        return bytes(np.ctypeslib.as_array(p, (nb.value,))) if nb.value else b""

    def max_row_id(self):
        return int(lib().oracle_max_row_id(self.h))

    def dump(self):
        """All rows in the format of oracle/ref_rowdump.cpp (type, card, bytes, payload)."""
        size = lib().oracle_dump(self.h, None)
        buf = np.zeros(max(1, size), np.uint8)
        lib().oracle_dump(self.h, _ptr(buf))
        return bytes(buf[:size])

    def triangles(self):
        return int(lib().oracle_triangles(self.h, self.threads))

    def list_triangles(self):
        """(T, 3) u32 array of (i, j, k) triangle tuples, i > j > k, pivot order."""
        total = lib().oracle_list_triangles(self.h, None, 0)
        out = np.zeros((max(total, 1), 3), np.uint32)
        lib().oracle_list_triangles(self.h, _ptr(out), total)
        return out[:total]

    def list_cliques(self, k=4):
        """(Q, k) u32 array of k-clique tuples, descending ids, in the reference's loop order."""
        total = lib().oracle_list_cliques(self.h, k, None, 0)
        out = np.zeros((max(total, 1), k), np.uint32)
        lib().oracle_list_cliques(self.h, k, _ptr(out), total)
        return out[:total]

    def triangles_range(self, lo, hi):
        return int(lib().oracle_triangles_range(self.h, lo, hi, self.threads))

    def cliques(self, k=4):
        return int(lib().oracle_cliques(self.h, k, self.threads))

    def lollipops(self):
        return int(lib().oracle_lollipops(self.h, self.threads))

    def similar_nodes(self, threshold=10):
        return int(lib().oracle_similar_nodes(self.h, threshold, self.threads))

    def symbiosity(self, cols=None, threshold=0.5):
        """symbiosity over this matrix's rows and `cols`' rows (the columns;
        None = this matrix, as for an undirected graph)."""
        c = self if cols is None else cols
        return int(lib().oracle_symbiosity(self.h, c.h, float(threshold), self.threads))

    def n_path(self, start, depth=0xEFFFFFF):
        """(path_length, reached) of the n_path BFS from row `start`."""
        r = C.c_uint64(0)
        n = int(lib().oracle_n_path(self.h, int(start), int(depth), C.byref(r)))
        return n, int(r.value)

    def intersect_rows(self, a, b):
        a = np.ascontiguousarray(a, np.uint32)
        b = np.ascontiguousarray(b, np.uint32)
        out = np.zeros(len(a), np.uint32)
        lib().oracle_intersect_rows(self.h, _ptr(a), _ptr(b), len(a), _ptr(out), self.threads)
        return out


def rmat_graph(scale, edges, seed, a=0.57, b=0.19, c=0.19):
    """(offsets, nbrs) of the library's seeded R-MAT graph, degree-ordered,
    regenerated on the CPU by oracle/eh_gen.c (same CSR, byte for byte)."""
    po, pn = C.c_void_p(), C.c_void_p()
    n = int(lib().oracle_rmat(scale, edges, a, b, c, seed, C.byref(po), C.byref(pn)))
    if n == 0:
        raise RuntimeError("R-MAT scale %d could not reach %d distinct edges" % (scale, edges))
    off = np.ctypeslib.as_array(C.cast(po, C.POINTER(C.c_uint64)), (n + 1,)).copy()
    nbr = np.ctypeslib.as_array(C.cast(pn, C.POINTER(C.c_uint32)), (int(off[n]),)).copy()
    lib().oracle_gen_free(po)
    lib().oracle_gen_free(pn)
    return off, nbr


def read_binary(path):
    """MutableGraph::undirectedFromBinary (src/MutableGraph.hpp:316-360) in numpy:
    u64 n, then per row u64 external id, u64 length, u32[length]."""
    raw = np.fromfile(path, dtype=np.uint8)
    n = int(raw[:8].view(np.uint64)[0])
    pos = 8
    offsets = np.zeros(n + 1, np.uint64)
    ext = np.zeros(n, np.uint64)
    chunks = []
    for i in range(n):
        e, ln = raw[pos:pos + 16].view(np.uint64)
        pos += 16
        ext[i] = e
        ln = int(ln)
        chunks.append(raw[pos:pos + 4 * ln].view(np.uint32))
        pos += 4 * ln
        offsets[i + 1] = offsets[i] + ln
    nbrs = np.concatenate(chunks) if chunks else np.zeros(0, np.uint32)
    return offsets, nbrs, ext


def read_directed_binary(path):
    """MutableGraph::directedFromBinary (src/MutableGraph.hpp:656-714) in numpy:
    u64 n, then per row u64 external id, u64 out length, u32[out length],
    u64 in length, u32[in length].  Returns (out_off, out_nbr, in_off, in_nbr, ext)."""
    raw = np.fromfile(path, dtype=np.uint8)
    n = int(raw[:8].view(np.uint64)[0])
    pos = 8
    oo = np.zeros(n + 1, np.uint64)
    io = np.zeros(n + 1, np.uint64)
    ext = np.zeros(n, np.uint64)
    outs, ins = [], []
    for i in range(n):
        e, ln = raw[pos:pos + 16].view(np.uint64)
        pos += 16
        ext[i] = e
        ln = int(ln)
        outs.append(raw[pos:pos + 4 * ln].view(np.uint32))
        pos += 4 * ln
        oo[i + 1] = oo[i] + ln
        ln = int(raw[pos:pos + 8].view(np.uint64)[0])
        pos += 8
        ins.append(raw[pos:pos + 4 * ln].view(np.uint32))
        pos += 4 * ln
        io[i + 1] = io[i] + ln
    cat = lambda c: np.concatenate(c) if c else np.zeros(0, np.uint32)
    return oo, cat(outs), io, cat(ins), ext


def counts(offsets, nbrs, layout="hybrid", threads=0, k=4, threshold=10):
    """The four app counts for one symmetric graph, as the reference apps compute them."""
    lay = LAYOUTS[layout]
    low = Matrix(offsets, nbrs, SELECT_LOWER, lay, threads=threads)
    full = Matrix(offsets, nbrs, SELECT_ALL, lay, threads=threads)
    return {
        "triangles": low.triangles(),
        "cliques%d" % k: low.cliques(k),
        "lollipops": full.lollipops(),
        "similar_nodes": full.similar_nodes(threshold),
    }
