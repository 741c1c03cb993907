"""CUDA path vs the oracle, through the C ABI, on seeded graphs.

Counts are integers: the bar is exact equality (tolerance 0).  Every layout the
reference offers (uint, pshort, bs, hybrid) plus the optional three-tier
hybrid is covered, with graphs that exercise uint, bitset and pshort rows,
empty rows, hubs split across CTAs, and rows long enough to need the decoded
giant-pivot path.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAPHS = {
    "rmat10": ("rmat", 11, dict(scale=10, edges=6000)),
    "rmat12": ("rmat", 12, dict(scale=12, edges=40000)),
    "er": ("er", 13, dict(n=3000, edges=30000)),
    "ba": ("ba", 14, dict(n=4000, m=8)),
    "planted": ("planted", 15, dict(n=6000, edges=20000, cliques=6, min_size=20, max_size=120)),
    "dense": ("er", 16, dict(n=400, edges=40000)),
}
LAYOUTS = ["hybrid", "uint", "bs", "pshort", "hybrid3"]

_cache = {}


def csr(eh, name):
    if name not in _cache:
        kind, seed, kw = GRAPHS[name]
        g = eh.graph(kind, seed, **kw)
        _cache[name] = g.csr()[:2]
    return _cache[name]


@pytest.mark.parametrize("name", list(GRAPHS))
@pytest.mark.parametrize("layout", LAYOUTS)
def test_triangles(eh, oracle, name, layout):
    off, nbr = csr(eh, name)
    m = eh.Matrix.build(off, nbr, selection="lower", layout=layout)
    o = oracle.Matrix(off, nbr, oracle.SELECT_LOWER, oracle.LAYOUTS[layout])
    assert m.count_triangles() == o.triangles()


@pytest.mark.parametrize("name", list(GRAPHS))
@pytest.mark.parametrize("layout", LAYOUTS)
def test_lollipops_and_similar(eh, oracle, name, layout):
    off, nbr = csr(eh, name)
    m = eh.Matrix.build(off, nbr, selection="all", layout=layout)
    o = oracle.Matrix(off, nbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout])
    assert m.count_lollipops() == o.lollipops()
    assert m.max_row_id() == o.max_row_id()
    for thr in (0, 10, 50):
        assert m.similar_nodes(thr) == o.similar_nodes(thr)


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("selection", ["lower", "all"])
def test_row_bytes_match_reference_format(eh, oracle, layout, selection):
    off, nbr = csr(eh, "planted")
    m = eh.Matrix.build(off, nbr, selection=selection, layout=layout)
    o = oracle.Matrix(off, nbr, oracle.SELECTIONS[selection], oracle.LAYOUTS[layout])
    info, oinfo = m.info(), o.info()
    for k in ("matrix_size", "cardinality", "row_total_bytes_used", "num_uint_rows",
              "num_pshort_rows", "num_bitset_rows"):
        assert info[k] == oinfo[k], k
    t, c, b = m.row_meta()
    ot, oc, ob = o.row_meta()
    assert np.array_equal(c, oc)
    assert np.array_equal(b, ob)
    nonempty = c > 0
    assert np.array_equal(t[nonempty], ot[nonempty])
    rng = np.random.default_rng(3)
    rows = np.concatenate([np.argsort(-c.astype(np.int64))[:20], rng.integers(0, len(c), 60)])
    for r in rows:
        assert m.export_row(int(r)) == o.row_bytes(int(r)), int(r)


def test_intersect_rows_all_layout_pairs(eh, oracle):
    torch = pytest.importorskip("torch")
    off, nbr = csr(eh, "planted")
    for layout in LAYOUTS:
        m = eh.Matrix.build(off, nbr, selection="all", layout=layout)
        o = oracle.Matrix(off, nbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout])
        rng = np.random.default_rng(5)
        n = len(off) - 1
        a = rng.integers(0, n, 5000).astype(np.uint32)
        b = rng.integers(0, n, 5000).astype(np.uint32)
        a[:100] = np.arange(100)  # hubs against everything
        da = torch.from_numpy(a.astype(np.int32)).cuda()
        db = torch.from_numpy(b.astype(np.int32)).cuda()
        dc = torch.zeros(len(a), dtype=torch.int32, device="cuda")
        m.intersect_rows(da.data_ptr(), db.data_ptr(), len(a), dc.data_ptr())
        torch.cuda.synchronize()
        got = dc.cpu().numpy().astype(np.uint32)
        assert np.array_equal(got, o.intersect_rows(a, b)), layout


@pytest.mark.parametrize("selection", ["all", "lower", "mask"])
def test_pshort_rows_over_several_partitions(eh, oracle, selection):
    """pshort payloads written by a warp or a CTA at once (rows over 32 and
    over 4,096 entries) equal the reference encoder's bytes when rows span
    several 2^16 partitions, partitions cross the warps' slices, and a mask
    drops elements anywhere in a row."""
    off, nbr = eh.graph("rmat", 25, scale=18, edges=3000000).csr()[:2]
    mask = None
    if selection == "mask":
        mask = (np.random.default_rng(5).random(len(nbr)) < 0.7).astype(np.uint8)
    m = eh.Matrix.build(off, nbr, selection=selection, layout="pshort", mask=mask)
    o = oracle.Matrix(off, nbr, oracle.SELECTIONS[selection], oracle.PSHORT, mask=mask)
    t, c, b = m.row_meta()
    ot, oc, ob = o.row_meta()
    assert np.array_equal(c, oc) and np.array_equal(b, ob)
    assert c.max() > (4096 if selection != "lower" else 256)  # pruned hub rows are short
    rng = np.random.default_rng(7)
    rows = np.concatenate([np.argsort(-c.astype(np.int64))[:60], rng.integers(0, len(c), 200)])
    for r in rows:
        assert m.export_row(int(r)) == o.row_bytes(int(r)), int(r)


def test_rejects_unsorted_rows_without_fault(eh):
    off = np.array([0, 2, 4, 6], np.uint64)
    nbr = np.array([2, 1, 0, 2, 0, 1], np.uint32)  # row 0 descending
    with pytest.raises(eh.EHError) as ei:
        eh.Matrix.build(off, nbr, selection="lower", layout="hybrid")
    assert ei.value.status == 1
    nbr2 = np.array([1, 7, 0, 2, 0, 1], np.uint32)  # id out of range
    with pytest.raises(eh.EHError):
        eh.Matrix.build(off, nbr2, selection="all", layout="uint")
    # the context is still usable afterwards
    m = eh.Matrix.build(off, np.array([1, 2, 0, 2, 0, 1], np.uint32), selection="lower", layout="hybrid")
    assert m.count_triangles() == 1


def test_rejects_bad_offsets_without_fault(eh):
    import torch
    nbr = np.array([1, 2, 0, 2, 0, 1], np.uint32)
    # falling offsets (row 1 would be [5, 2)), from host and from device buffers
    bad = np.array([0, 5, 2, 6], np.uint64)
    with pytest.raises(eh.EHError) as ei:
        eh.Matrix.build(bad, nbr, selection="lower", layout="hybrid")
    assert "offsets" in str(ei.value)
    d_nbr = torch.from_numpy(nbr.view(np.int32)).cuda()
    for off in (bad, np.array([0, 9, 9, 6], np.uint64)):  # the second runs past offsets[n]
        d_off = torch.from_numpy(off.view(np.int64)).cuda()
        with pytest.raises(eh.EHError):
            eh.Matrix.build_device(3, d_off.data_ptr(), d_nbr.data_ptr(), selection="all", layout="uint")
    good = torch.from_numpy(np.array([0, 2, 4, 6], np.uint64).view(np.int64)).cuda()
    m = eh.Matrix.build_device(3, good.data_ptr(), d_nbr.data_ptr(), selection="lower", layout="hybrid")
    assert m.count_triangles() == 1


def test_chunked_host_upload_equals_device_build(eh):
    """A build from host arrays uploads the adjacency in chunks of rows (about
    16 M entries each) and measures each chunk as it lands.  At about 42 M
    entries (three chunks, the long rows in the first) it must encode byte for
    byte as the single-pass build from device buffers, and falling offsets in a
    later chunk must still be rejected."""
    import hashlib
    import torch
    g = eh.graph("rmat", 21, scale=21, edges=21 << 20)
    off, nbr = g.csr()[:2]
    assert int(off[-1]) > 2 * (16 << 20)
    d_off = torch.from_numpy(off.view(np.int64)).cuda()
    d_nbr = torch.from_numpy(nbr.view(np.int32)).cuda()
    for layout in ("hybrid", "pshort"):
        a = eh.Matrix.build(off, nbr, selection="lower", layout=layout)
        b = eh.Matrix.build_device(len(off) - 1, d_off.data_ptr(), d_nbr.data_ptr(), selection="lower",
                                   layout=layout)
        assert a.info() == b.info()
        assert hashlib.sha256(a.export_flattened()).digest() == hashlib.sha256(b.export_flattened()).digest()
        assert a.count_triangles() == b.count_triangles()
        del a, b
    bad = off.copy()
    k = int(np.searchsorted(off, off[-1] * 3 // 4))  # a row in the last chunk
    assert off[k + 1] < off[-1]
    bad[k] = bad[k + 1] + 1  # row k falls; row k - 1 stays within the neighbour array
    with pytest.raises(eh.EHError) as ei:
        eh.Matrix.build(bad, nbr, selection="lower", layout="hybrid")
    assert "offsets" in str(ei.value)


def test_clique_pivot_limit_is_an_error_before_any_launch(eh):
    """A star whose centre has the highest id keeps all n - 1 > 2^18 leaves in
    one selected row: clique counts reject it (EH_ERR_UNSUPPORTED) before any
    kernel runs, since the packed masks' 32-bit offsets are exact only below
    2^18 entries; the triangle count of the same matrix is still 0."""
    n = (1 << 18) + 8
    hub = n - 1
    deg = np.ones(n, np.uint64)
    deg[hub] = n - 1
    off = np.zeros(n + 1, np.uint64)
    off[1:] = np.cumsum(deg)
    nbr = np.empty(int(off[-1]), np.uint32)
    nbr[:n - 1] = hub
    nbr[n - 1:] = np.arange(n - 1, dtype=np.uint32)
    m = eh.Matrix.build(off, nbr, selection="lower", layout="hybrid")
    assert m.info()["max_row_cardinality"] == n - 1
    with pytest.raises(eh.EHError) as ei:
        m.count_cliques(4)
    assert ei.value.status == 4
    assert m.count_triangles() == 0


def test_empty_and_tiny_graphs(eh, oracle):
    for off, nbr in [(np.zeros(1, np.uint64), np.zeros(0, np.uint32)),
                     (np.zeros(5, np.uint64), np.zeros(0, np.uint32)),
                     (np.array([0, 1, 2], np.uint64), np.array([1, 0], np.uint32))]:
        for layout in LAYOUTS:
            m = eh.Matrix.build(off, nbr, selection="lower", layout=layout)
            assert m.count_triangles() == 0
            f = eh.Matrix.build(off, nbr, selection="all", layout=layout)
            assert f.count_lollipops() == 0
            o = oracle.Matrix(off, nbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout])
            assert f.similar_nodes(0) == o.similar_nodes(0)


@pytest.mark.parametrize("layout", ["uint", "hybrid"])
def test_config1_graph_with_giant_pivots(eh, oracle, layout):
    """The 2^16-vertex, 1M-edge R-MAT graph: hubs of >6144 entries take the
    decoded giant-pivot path in the full-row (lollipop) matrix."""
    g = eh.graph("rmat", 1, scale=16, edges=1000000)
    off, nbr = g.csr()[:2]
    low = eh.Matrix.build(off, nbr, selection="lower", layout=layout)
    olow = oracle.Matrix(off, nbr, oracle.SELECT_LOWER, oracle.LAYOUTS[layout])
    assert low.count_triangles() == olow.triangles()
    full = eh.Matrix.build(off, nbr, selection="all", layout=layout)
    assert full.info()["max_row_cardinality"] > 6144
    ofull = oracle.Matrix(off, nbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout])
    assert full.count_lollipops() == ofull.lollipops()
    assert full.similar_nodes(10) == ofull.similar_nodes(10)


@pytest.mark.parametrize("name", ["rmat10", "rmat12", "er", "ba", "planted", "dense"])
@pytest.mark.parametrize("layout", LAYOUTS)
def test_cliques(eh, oracle, name, layout):
    off, nbr = csr(eh, name)
    m = eh.Matrix.build(off, nbr, selection="lower", layout=layout)
    o = oracle.Matrix(off, nbr, oracle.SELECT_LOWER, oracle.LAYOUTS[layout])
    ks = (3, 4) if name == "dense" else (3, 4, 5)
    for k in ks:
        assert m.count_cliques(k) == o.cliques(k), k


def complete_graphs(sizes):
    """Disjoint union of complete graphs K_s (vertex ids interleaved so that each
    clique spans the id range), degree-ordered."""
    import numpy as np
    rng = np.random.default_rng(9)
    n = sum(sizes)
    perm = rng.permutation(n)
    rows = [[] for _ in range(n)]
    start = 0
    for s in sizes:
        ids = perm[start:start + s]
        start += s
        for v in ids:
            rows[v] = [int(u) for u in ids if u != v]
    off = np.zeros(n + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in rows])
    nbr = np.array([x for r in rows for x in sorted(r)], np.uint32)
    return off, nbr


@pytest.mark.parametrize("layout", LAYOUTS)
def test_cliques_closed_form_all_tiers(eh, layout):
    from math import comb
    # Pivots of K_1900 above ~1,850 entries do not fit shared memory and use the
    # global-scratch tier; the rest of K_1900, K_1100 and K_600 cover the
    # shared-memory size bands, K_30 and K_5 the warp tier.
    sizes = [1900, 1100, 600, 200, 30, 5] if layout == "hybrid" else [1100, 600, 200, 30, 5]
    off, nbr = complete_graphs(sizes)
    g = eh.HostGraph.from_csr(off, nbr).reorder_by_degree()
    off, nbr = g.csr()[:2]
    m = eh.Matrix.build(off, nbr, selection="lower", layout=layout)
    assert m.info()["max_row_cardinality"] > 1024
    for k in (3, 4):
        assert m.count_cliques(k) == sum(comb(s, k) for s in sizes), k
    assert m.count_triangles() == sum(comb(s, 3) for s in sizes)
    # Work grows with the number of (k-1)-cliques: k = 5 on K_1100 is ~2e8 search
    # nodes (run for one layout; the masks, not the layout, carry the search).
    if layout == "hybrid":
        sizes5 = [1100, 600, 200, 30, 5]
        off5, nbr5 = complete_graphs(sizes5)
        g5 = eh.HostGraph.from_csr(off5, nbr5).reorder_by_degree()
        m5 = eh.Matrix.build(*g5.csr()[:2], selection="lower", layout=layout)
        assert m5.count_cliques(5) == sum(comb(s, 5) for s in sizes5)
    # Deeper k on small cliques: the search visits every (k-1)-clique, so K_40 with
    # k <= 8 (about 2e7 nodes, shared-memory tier) and K_20 up to k = 16 (warp tier).
    for small, ks in (([40, 33], (6, 8)), ([20, 18, 12, 7], (12, 16))):
        off2, nbr2 = complete_graphs(small)
        g2 = eh.HostGraph.from_csr(off2, nbr2).reorder_by_degree()
        m2 = eh.Matrix.build(*g2.csr()[:2], selection="lower", layout=layout)
        for k in ks:
            assert m2.count_cliques(k) == sum(comb(s, k) for s in small), k


def test_clique_size_limits(eh):
    off, nbr = csr(eh, "rmat10")
    m = eh.Matrix.build(off, nbr, selection="lower", layout="hybrid")
    assert m.count_cliques(2) == 0 and m.count_cliques(1) == 0  # the reference never reaches depth n < 3
    with pytest.raises(eh.EHError):
        m.count_cliques(17)
    full = eh.Matrix.build(off, nbr, selection="all", layout="hybrid")
    with pytest.raises(eh.EHError):
        full.count_cliques(4)


def test_device_waits_are_bounded(eh):
    """A device-side wait that nothing completes gives up after its poll limit
    and reports it (no hang, no fault); the context stays usable."""
    import ctypes as C
    flag = C.c_uint32(0)
    eh.check(eh.load().eh_selftest_bounded_wait(64, C.byref(flag)))
    assert flag.value == 1
    off, nbr = csr(eh, "rmat10")
    assert eh.Matrix.build(off, nbr, selection="lower").count_triangles() > 0


def test_bitset_pairs_at_every_word_alignment(eh):
    """Bitset ∩ bitset over 16-byte word pairs: rows whose first words differ by
    even and odd amounts, odd and even word counts, single words and long
    sparse rows, against numpy (integer counts, tolerance 0)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    n = 1 << 17
    rows = []
    for r in range(96):
        first = int(rng.integers(0, 40)) * 64 + int(rng.integers(0, 64))
        span = int(rng.choice([1, 63, 64, 65, 130, 700, 5000, 60000]))
        k = max(1, min(span, int(rng.integers(1, 300))))
        vals = np.unique(np.concatenate([[first], first + rng.integers(0, span, k)]))
        rows.append(vals[vals < n].astype(np.uint32))
    rows += [np.zeros(0, np.uint32)] * (n - len(rows))
    off = np.zeros(n + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in rows])
    nbr = np.concatenate(rows).astype(np.uint32)
    m = eh.Matrix.build(off, nbr, selection="all", layout="bs")
    a = np.repeat(np.arange(96, dtype=np.uint32), 96)
    b = np.tile(np.arange(96, dtype=np.uint32), 96)
    da = torch.from_numpy(a.astype(np.int32)).cuda()
    db = torch.from_numpy(b.astype(np.int32)).cuda()
    dc = torch.zeros(len(a), dtype=torch.int32, device="cuda")
    m.intersect_rows(da.data_ptr(), db.data_ptr(), len(a), dc.data_ptr())
    torch.cuda.synchronize()
    got = dc.cpu().numpy()
    want = np.array([len(np.intersect1d(rows[x], rows[y])) for x, y in zip(a, b)])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("filter_words", [0, 16, 32, 64])
def test_core_filters_keep_counts(eh, oracle, filter_words):
    """The hashed filters in front of the dense core's rows (a work-shape
    choice) never change a count: a set bit still reads the core word, a clear
    bit means the element is absent.  Triangles and lollipops on a graph whose
    core spans rows [0, 8192), so rows [4096, 8192) have filters, and a batch."""
    torch = pytest.importorskip("torch")
    off, nbr = eh.graph("rmat", 23, scale=14, edges=200000).csr()[:2]
    low = eh.Matrix.build(off, nbr, "lower", "hybrid")
    full = eh.Matrix.build(off, nbr, "all", "hybrid")
    low.set_shape(96, 128, 4, 8192, 64, filter_words)
    full.set_shape(96, 128, 4, 8192, 0, filter_words)
    assert low.count_triangles() == oracle.Matrix(off, nbr, oracle.SELECT_LOWER, oracle.HYBRID).triangles()
    assert full.count_lollipops() == oracle.Matrix(off, nbr, oracle.SELECT_ALL, oracle.HYBRID).lollipops()
    csrs = [eh.graph("rmat", 40 + k, scale=12, edges=30000).csr()[:2] for k in range(3)]
    gr, boff, bnbr = eh.concat_graphs(csrs)
    b = eh.Batch(gr, boff, bnbr, layout="hybrid")
    bm = eh.C.c_void_p()
    eh.check(eh.load().eh_batch_matrix(b.h, eh.C.byref(bm)))
    t = eh.Tuning(light_max=96, unit_span=128, ctas_per_sm=4, core_rows=8192, core_filter_words=filter_words)
    eh.check(eh.load().eh_matrix_set_shape(bm, eh.C.byref(t), None))
    tri = torch.zeros(len(csrs), dtype=torch.int64, device="cuda")
    b.count(3, tri.data_ptr())
    torch.cuda.synchronize()
    assert tri.cpu().tolist() == [oracle.Matrix(o, n, oracle.SELECT_LOWER, oracle.HYBRID).triangles() for o, n in csrs]


def test_set_shape_rejects_bad_filter_width(eh):
    off, nbr = eh.graph("rmat", 22, scale=10, edges=5000).csr()[:2]
    m = eh.Matrix.build(off, nbr, "lower", "hybrid")
    with pytest.raises(eh.EHError):
        m.set_shape(96, 128, 4, 0, 0, 24)
