"""Triangle tuples (eh_list_triangles) vs the oracle's tuples from the
reference's loop: the same set of (i, j, k), exactly; capacity handling."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def tuples(eh, torch, m, cap=None):
    total = torch.zeros(1, dtype=torch.int64, device="cuda")
    m.list_triangles(0, 0, total.data_ptr())
    torch.cuda.synchronize()
    t = int(total.item())
    cap = t if cap is None else cap
    out = torch.zeros((max(cap, 1), 3), dtype=torch.int32, device="cuda")
    m.list_triangles(out.data_ptr(), cap, total.data_ptr())
    torch.cuda.synchronize()
    return int(total.item()), out[:min(cap, t)].cpu().numpy().astype(np.uint32)


def canon(a):
    a = np.ascontiguousarray(a, np.uint32)
    return a[np.lexsort((a[:, 2], a[:, 1], a[:, 0]))] if len(a) else a


@pytest.mark.parametrize("layout", ["hybrid", "uint", "bs", "pshort"])
@pytest.mark.parametrize("graph", [("rmat", 31, dict(scale=11, edges=20000)),
                                   ("planted", 32, dict(n=3000, edges=6000, cliques=4, min_size=30, max_size=90)),
                                   ("rmat", 1, dict(scale=16, edges=1000000))])
def test_tuples_equal_oracle(eh, oracle, layout, graph):
    torch = pytest.importorskip("torch")
    kind, seed, kw = graph
    off, nbr = eh.graph(kind, seed, **kw).csr()[:2]
    m = eh.Matrix.build(off, nbr, "lower", layout)
    total, got = tuples(eh, torch, m)
    want = oracle.Matrix(off, nbr, oracle.SELECT_LOWER, oracle.LAYOUTS[layout]).list_triangles()
    assert total == len(want) == m.count_triangles()
    assert np.all(got[:, 0] > got[:, 1]) and np.all(got[:, 1] > got[:, 2])
    assert np.array_equal(canon(got), canon(want))


def test_capacity_truncates_but_counts(eh):
    torch = pytest.importorskip("torch")
    off, nbr = eh.graph("rmat", 33, scale=10, edges=6000).csr()[:2]
    m = eh.Matrix.build(off, nbr, "lower", "hybrid")
    total, got = tuples(eh, torch, m, cap=100)
    assert total == m.count_triangles() > 100 and len(got) == 100
    assert len({tuple(r) for r in got.tolist()}) == 100  # 100 distinct tuples


def clique_tuples(eh, torch, m, k, cap=None):
    total = torch.zeros(1, dtype=torch.int64, device="cuda")
    m.list_cliques(k, 0, 0, total.data_ptr())
    torch.cuda.synchronize()
    t = int(total.item())
    cap = t if cap is None else cap
    out = torch.zeros((max(cap, 1), k), dtype=torch.int32, device="cuda")
    m.list_cliques(k, out.data_ptr(), cap, total.data_ptr())
    torch.cuda.synchronize()
    return int(total.item()), out[:min(cap, t)].cpu().numpy().astype(np.uint32)


def canon_k(a):
    a = np.ascontiguousarray(a, np.uint32)
    return a[np.lexsort(a.T[::-1])] if len(a) else a


@pytest.mark.parametrize("layout", ["hybrid", "uint", "bs", "pshort"])
@pytest.mark.parametrize("graph", [("rmat", 31, dict(scale=11, edges=20000)),
                                   ("planted", 32, dict(n=3000, edges=6000, cliques=4, min_size=30, max_size=90))])
@pytest.mark.parametrize("k", [3, 4])
def test_clique_tuples_equal_oracle(eh, oracle, layout, graph, k):
    """eh_list_cliques writes the reference's n_clique table (WRITE_TABLE) as a
    set: pivots of up to 32 entries in the warp tier, larger ones in the CTA
    tier; the total equals the count."""
    torch = pytest.importorskip("torch")
    kind, seed, kw = graph
    off, nbr = eh.graph(kind, seed, **kw).csr()[:2]
    m = eh.Matrix.build(off, nbr, "lower", layout)
    total, got = clique_tuples(eh, torch, m, k)
    want = oracle.Matrix(off, nbr, oracle.SELECT_LOWER, oracle.LAYOUTS[layout]).list_cliques(k)
    assert total == len(want) == m.count_cliques(k)
    assert all(np.all(got[:, d] > got[:, d + 1]) for d in range(k - 1))
    assert np.array_equal(canon_k(got), canon_k(want))


def test_clique_tuples_in_every_tier(eh):
    """Complete graphs reach every tier (K_1900: pivots above the shared-memory
    limit in global scratch; K_1100 / K_600: the 1,024- and 256-thread bands;
    K_30: the warp tier).  Totals equal comb(s, k); the written tuples (up to the
    capacity) are distinct and descending within one clique."""
    from math import comb
    from test_gpu_parity import complete_graphs
    torch = pytest.importorskip("torch")
    for sizes, k in (([1900, 600, 30], 3), ([1100, 600, 30], 4)):
        off, nbr = complete_graphs(sizes)
        g = eh.HostGraph.from_csr(off, nbr).reorder_by_degree()
        off, nbr = g.csr()[:2]
        m = eh.Matrix.build(off, nbr, "lower", "hybrid")
        total, got = clique_tuples(eh, torch, m, k, cap=1 << 20)
        assert total == sum(comb(s, k) for s in sizes) == m.count_cliques(k)
        assert len(got) == 1 << 20
        assert all(np.all(got[:, d] > got[:, d + 1]) for d in range(k - 1))
        assert len({tuple(r) for r in got.tolist()}) == len(got)
        # Each tuple's ids are pairwise adjacent.
        rows = [set(nbr[off[v]:off[v + 1]].tolist()) for v in range(len(off) - 1)]
        sample = got[:: max(1, len(got) // 2000)]
        assert all(int(t[b]) in rows[int(t[a])] for t in sample for a in range(k) for b in range(a + 1, k))


def test_clique_tuples_reject_other_k(eh):
    torch = pytest.importorskip("torch")
    off, nbr = eh.graph("rmat", 33, scale=10, edges=6000).csr()[:2]
    m = eh.Matrix.build(off, nbr, "lower", "hybrid")
    total = torch.zeros(1, dtype=torch.int64, device="cuda")
    with pytest.raises(eh.EHError):
        m.list_cliques(5, 0, 0, total.data_ptr())
