"""eh_count_cliques_noalloc: the clique count for callers that may not
allocate device memory at call time (a serving loop with a device-memory
budget fixed at start-up, or a host framework that owns all device
allocations).  Its scratch is a fixed 16 MiB device array instead of memory
the call allocates; its counts must equal eh_count_cliques's, exactly
(integer counts, tolerance 0), on two calls in a row that share that array.

Kept in its own file, collected last."""
import ctypes as C
from math import comb

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def complete_graphs(sizes, seed=9):
    rng = np.random.default_rng(seed)
    n = sum(sizes)
    perm = rng.permutation(n)
    rows = [[] for _ in range(n)]
    start = 0
    for s in sizes:
        ids = perm[start:start + s]
        start += s
        for v in ids:
            rows[v] = sorted(int(u) for u in ids if u != v)
    off = np.zeros(n + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in rows])
    nbr = np.array([x for r in rows for x in r], np.uint32)
    return off, nbr


SIZES = [1900, 600, 200, 30]


def graphs(eh):
    g = eh.HostGraph.from_csr(*complete_graphs(SIZES)).reorder_by_degree()
    yield "complete", g.csr()[:2]  # pivots above ~1,850 entries (too big for shared memory) use the fixed scratch
    yield "rmat", eh.graph("rmat", 12, scale=12, edges=40000).csr()[:2]


def _entry(L):
    f = L.eh_count_cliques_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    return f


def test_noalloc_counts_equal_the_allocating_entry_point(eh):
    torch = pytest.importorskip("torch")
    L = eh.load()
    f = _entry(L)
    for name, (off, nbr) in graphs(eh):
        m = eh.Matrix.build(off, nbr, selection="lower", layout="hybrid")
        fresh = torch.zeros(1, dtype=torch.int64, device="cuda")
        # before the matrix has a work plan the call refuses instead of allocating one
        assert f(m.h, 4, C.c_void_p(fresh.data_ptr()), None) == 1
        assert b"work plan" in L.eh_last_error()
        for k in ((3, 4) if name == "complete" else (3, 4, 5)):
            want = m.count_cliques(k)  # existing entry point; builds the plan on first use
            out = torch.full((2,), -1, dtype=torch.int64, device="cuda")
            for call in range(2):
                st = f(m.h, k, C.c_void_p(out[call:].data_ptr()), None)
                assert st == 0, L.eh_last_error()
            torch.cuda.synchronize()
            assert out.tolist() == [want, want], (name, k)
            if name == "complete":  # disjoint complete graphs: sum of C(s, k)
                assert want == sum(comb(s, k) for s in SIZES), k


def test_noalloc_rejects_a_pivot_beyond_the_fixed_scratch(eh):
    """A star whose hub has the highest id has one pivot of 16,400 entries: its
    4-clique working set (about 16.9 MB) is larger than the 16 MiB array, so the
    call refuses with EH_ERR_UNSUPPORTED and names the limit; the allocating
    entry point counts it (0 cliques)."""
    torch = pytest.importorskip("torch")
    L = eh.load()
    f = _entry(L)
    leaves = 16400
    hub = leaves
    off = np.concatenate([np.arange(leaves + 1, dtype=np.uint64), [2 * leaves]]).astype(np.uint64)
    nbr = np.concatenate([np.full(leaves, hub, np.uint32), np.arange(leaves, dtype=np.uint32)])
    m = eh.Matrix.build(off, nbr, selection="lower", layout="hybrid")
    assert m.count_cliques(4) == 0  # builds the plan; the allocating path has no such limit
    out = torch.full((1,), 7, dtype=torch.int64, device="cuda")
    assert f(m.h, 4, C.c_void_p(out.data_ptr()), None) == 4  # EH_ERR_UNSUPPORTED
    assert b"fixed scratch" in L.eh_last_error()
    torch.cuda.synchronize()
    assert out.item() == 0  # the count was cleared before the size check
    # the array is still usable: a graph that fits counts right after the refusal
    g = eh.HostGraph.from_csr(*complete_graphs([40])).csr()[:2]
    m2 = eh.Matrix.build(*g, selection="lower", layout="hybrid")
    m2.count_cliques(4)
    assert f(m2.h, 4, C.c_void_p(out.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert out.item() == comb(40, 4)
