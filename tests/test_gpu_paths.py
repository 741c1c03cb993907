"""CUDA symbiosity and n_path BFS vs the oracle and the reference binaries.

Both are integer results: the bar is exact equality.  The fixture
(tests/golden/reference_directed.json) holds the reference apps' own outputs
(apps/symbiosity.cpp, apps/n_path.cpp built from unmodified sources) on seeded
directed graphs in every layout; the oracle comparisons add the number of
vertices the BFS reached, several starts and depths, and the edge cases.
"""
import numpy as np
import pytest

import _golden

pytestmark = pytest.mark.gpu

LAYOUTS = ["hybrid", "uint", "bs", "pshort", "hybrid3"]


def _pair(eh, arrays, layout):
    off, nbr, ioff, inbr = arrays
    rows = eh.Matrix.build(off, nbr, selection="all", layout=layout)
    cols = eh.Matrix.build(ioff, inbr, selection="all", layout=layout)
    return rows, cols


def _opair(oracle, arrays, layout):
    off, nbr, ioff, inbr = arrays
    return (oracle.Matrix(off, nbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout]),
            oracle.Matrix(ioff, inbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout]))


@pytest.mark.parametrize("spec", _golden.directed_graphs(), ids=lambda s: s["name"])
def test_reference_fixture(eh, spec):
    arrays = _golden.generate_directed(eh, spec)
    doc = _golden.load_directed()
    key = "n_path_s%d_d%d" % (doc["n_path_start"], doc["n_path_depth"])
    for layout in ["hybrid", "uint", "bs", "pshort"]:
        rows, cols = _pair(eh, arrays, layout)
        want = spec["counts"][layout]
        assert rows.symbiosity(cols) == want["symbiosity"], layout
        assert rows.max_row_id() == want["n_path_start"], layout
        assert rows.bfs(want["n_path_start"])[0] == want["n_path"], layout
        assert rows.bfs(doc["n_path_start"], doc["n_path_depth"])[0] == want[key], layout


GRAPHS = {
    "drmat12": ("drmat", 31, dict(scale=12, edges=30000)),
    "recip_ba": ("recip", 32, dict(base="ba", base_params=dict(n=5000, m=6), p_both=0.4)),
    "recip_planted": ("recip", 33, dict(base="planted", base_params=dict(n=6000, edges=15000, cliques=6,
                                                                         min_size=20, max_size=150), p_both=0.8)),
    "recip_dense": ("recip", 34, dict(base="er", base_params=dict(n=500, edges=50000), p_both=0.5)),
}
_cache = {}


def arrays_of(eh, name):
    if name not in _cache:
        kind, seed, kw = GRAPHS[name]
        g = eh.graph(kind, seed, **kw)
        off, nbr, _, _ = g.csr()
        _cache[name] = (off, nbr) + g.in_csr()
    return _cache[name]


@pytest.mark.parametrize("name", list(GRAPHS))
@pytest.mark.parametrize("layout", LAYOUTS)
def test_symbiosity_vs_oracle(eh, oracle, name, layout):
    a = arrays_of(eh, name)
    rows, cols = _pair(eh, a, layout)
    orows, ocols = _opair(oracle, a, layout)
    for thr in (0.5, 0.0, 0.25, 0.9, -1.0):
        assert rows.symbiosity(cols, thr) == orows.symbiosity(ocols, thr), thr
    # Undirected use: the rows are their own columns.
    assert rows.symbiosity() == orows.symbiosity()


@pytest.mark.parametrize("name", list(GRAPHS))
@pytest.mark.parametrize("layout", LAYOUTS)
def test_bfs_vs_oracle(eh, oracle, name, layout):
    a = arrays_of(eh, name)
    off = a[0]
    n = len(off) - 1
    rows = eh.Matrix.build(a[0], a[1], selection="all", layout=layout)
    orows = oracle.Matrix(a[0], a[1], oracle.SELECT_ALL, oracle.LAYOUTS[layout])
    deg = np.diff(off)
    starts = {orows.max_row_id(), 0, n // 2, n - 1}
    if (deg == 0).any():
        starts.add(int(np.flatnonzero(deg == 0)[0]))
    for s in sorted(starts):
        for depth in (0, 1, 3, 0xEFFFFFF):
            assert rows.bfs(s, depth) == orows.n_path(s, depth), (s, depth)


def test_bfs_and_symbiosity_edge_cases(eh, oracle):
    # A path 0 -> 1 -> 2, an isolated vertex 3, and a self-loop on 4.
    off = np.array([0, 1, 2, 2, 2, 3], np.uint64)
    nbr = np.array([1, 2, 4], np.uint32)
    g = eh.HostGraph.directed_from_csr(off, nbr)
    ioff, inbr = g.in_csr()
    for layout in LAYOUTS:
        rows, cols = _pair(eh, (off, nbr, ioff, inbr), layout)
        assert rows.bfs(0) == (2, 3)
        assert rows.bfs(0, 1) == (1, 3)
        assert rows.bfs(2) == (0, 1)
        assert rows.bfs(3) == (0, 1)
        assert rows.bfs(4) == (0, 1)
        # Only vertex 4 (out {4}, in {4}) has ratio 1; 0/0 rows do not count.
        assert rows.symbiosity(cols) == 1
        with pytest.raises(eh.EHError):
            rows.bfs(5)
    one = eh.Matrix.build(np.array([0, 0], np.uint64), np.zeros(0, np.uint32), selection="all")
    assert one.bfs(0) == (0, 1)
    assert one.symbiosity() == 0
    empty = eh.Matrix.build(np.array([0], np.uint64), np.zeros(0, np.uint32), selection="all")
    assert empty.symbiosity() == 0
    with pytest.raises(eh.EHError):
        empty.bfs(0)
    other = eh.Matrix.build(np.array([0, 0, 0], np.uint64), np.zeros(0, np.uint32), selection="all")
    with pytest.raises(eh.EHError):
        one.symbiosity(other)


def test_pshort_u16_quirk(eh, oracle):
    """The reference's pshort ∩ pshort keeps a partition's intersection size in
    a uint16_t (intersection.hpp:857-865), so a fully shared 2^16 block counts
    0; the fixture holds the reference binaries' own counts on these graphs."""
    import torch
    quirks = _golden.load_directed()["quirks"]
    off, nbr = _golden.full_block_directed()
    g = eh.HostGraph.directed_from_csr(off, nbr)
    a = (off, nbr) + g.in_csr()
    for layout in ["pshort", "hybrid", "uint", "bs"]:
        rows, cols = _pair(eh, a, layout)
        orows, ocols = _opair(oracle, a, layout)
        assert rows.symbiosity(cols) == quirks["symbiosity_full_block"][layout] == orows.symbiosity(ocols), layout
        assert rows.bfs(65536) == orows.n_path(65536)
    uoff, unbr = _golden.full_block_undirected()
    pa = np.array([65536, 65536, 0], np.uint32)
    pb = np.array([65537, 65536, 1], np.uint32)
    for layout in ["pshort", "hybrid", "uint", "bs"]:
        m = eh.Matrix.build(uoff, unbr, selection="all", layout=layout)
        o = oracle.Matrix(uoff, unbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout])
        assert m.similar_nodes(10) == quirks["similar_nodes_full_block"][layout] == o.similar_nodes(10), layout
        da, db = torch.from_numpy(pa).cuda(), torch.from_numpy(pb).cuda()
        dc = torch.zeros(3, dtype=torch.int32, device="cuda")
        m.intersect_rows(da.data_ptr(), db.data_ptr(), 3, dc.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(dc.cpu().numpy().view(np.uint32), o.intersect_rows(pa, pb)), layout


def test_hub_rows_take_the_cta_path(eh, oracle):
    """A hub h with out-edges to the even ids and in-edges from the multiples of
    3 below 2^19: long bitset, uint and pshort rows on both sides, so every
    heavy-row branch of the symbiosity kernels and the grid-split BFS rows run."""
    n = (1 << 19) + 1
    h = n - 1
    outs = np.arange(0, h, 2, dtype=np.uint32)
    ins = np.arange(0, h, 3, dtype=np.uint32)
    src = np.concatenate([np.full(len(outs), h, np.uint32), ins])
    dst = np.concatenate([outs, np.full(len(ins), h, np.uint32)])
    # A second, smaller hub so that more than one heavy row is listed.
    src = np.concatenate([src, np.full(5000, 7, np.uint32), np.arange(1, 5001, dtype=np.uint32) * 13])
    dst = np.concatenate([dst, np.arange(1, 5001, dtype=np.uint32) * 13, np.full(5000, 7, np.uint32)])
    key = np.unique((src.astype(np.uint64) << np.uint64(32)) | dst.astype(np.uint64))
    s, d = (key >> np.uint64(32)).astype(np.int64), (key & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    off = np.zeros(n + 1, np.uint64)
    np.add.at(off, s + 1, 1)
    off = np.cumsum(off, dtype=np.uint64)
    g = eh.HostGraph.directed_from_csr(off, d)
    a = (off, d) + g.in_csr()
    for layout in ["bs", "hybrid", "uint", "pshort"]:
        rows, cols = _pair(eh, a, layout)
        orows, ocols = _opair(oracle, a, layout)
        for thr in (0.5, 0.0, 0.2):
            assert rows.symbiosity(cols, thr) == orows.symbiosity(ocols, thr), (layout, thr)
        for start in (h, 0, 7, 13):
            assert rows.bfs(start) == orows.n_path(start), (layout, start)
