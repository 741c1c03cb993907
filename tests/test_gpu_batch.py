"""Batched counting (many graphs, one launch) and CUDA-graph replay: every
graph's triangle and 4-clique count in the batch equals its count alone and
the oracle's (integers, tolerance 0); the autotuner changes no count."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_batch(eh):
    from simdgraphprocessing_gb300 import workloads as W
    specs = W.batch_specs(num_graphs=48, seed=40, n_lo=40, n_hi=3000)  # BA needs n > m + 1 (m <= 32)
    csrs = [eh.graph(kind, s, **kw).csr()[:2] for kind, s, kw in specs]
    csrs.append((np.zeros(1, np.uint64), np.zeros(0, np.uint32)))  # an empty graph
    csrs.append((np.array([0, 1, 2], np.uint64), np.array([1, 0], np.uint32)))  # one edge
    return csrs, eh.concat_graphs(csrs)


def test_batch_counts_equal_per_graph_counts(eh, oracle):
    torch = pytest.importorskip("torch")
    csrs, (gr, off, nbr) = small_batch(eh)
    G = len(csrs)
    b = eh.Batch(gr, off, nbr, layout="hybrid")
    tri = torch.zeros(G, dtype=torch.int64, device="cuda")
    clq = torch.zeros(G, dtype=torch.int64, device="cuda")
    b.count(3, tri.data_ptr())
    b.count(4, clq.data_ptr())
    torch.cuda.synchronize()
    want_t, want_c = [], []
    for o, n in csrs:
        om = oracle.Matrix(o, n, oracle.SELECT_LOWER, oracle.HYBRID)
        want_t.append(om.triangles())
        want_c.append(om.cliques(4))
        m = eh.Matrix.build(o, n, "lower", "hybrid")
        assert m.count_triangles() == want_t[-1]
    assert tri.cpu().tolist() == want_t
    assert clq.cpu().tolist() == want_c
    assert b.matrix_info()["matrix_size"] == int(gr[-1])


@pytest.mark.parametrize("layout", ["hybrid", "uint", "bs", "pshort"])
def test_batch_graph_replay_and_tuning(eh, oracle, layout):
    torch = pytest.importorskip("torch")
    csrs, (gr, off, nbr) = small_batch(eh)
    G = len(csrs)
    b = eh.Batch(gr, off, nbr, layout=layout)
    s = torch.cuda.Stream()
    tri = torch.zeros(G, dtype=torch.int64, device="cuda")
    clq = torch.zeros(G, dtype=torch.int64, device="cuda")
    ref_t = torch.zeros(G, dtype=torch.int64, device="cuda")
    ref_c = torch.zeros(G, dtype=torch.int64, device="cuda")
    b.run(ref_t.data_ptr(), ref_c.data_ptr(), use_graph=False, stream=s)
    for _ in range(3):
        b.run(tri.data_ptr(), clq.data_ptr(), use_graph=True, stream=s)
        s.synchronize()
        assert torch.equal(tri, ref_t) and torch.equal(clq, ref_c)
    shape = b.tune(stream=s)
    assert shape["ctas_per_sm"] >= 1 and shape["configs_tried"] >= 1
    b.run(tri.data_ptr(), clq.data_ptr(), use_graph=True, stream=s)
    s.synchronize()
    assert torch.equal(tri, ref_t) and torch.equal(clq, ref_c)
    want = [oracle.Matrix(o, n, oracle.SELECT_LOWER, oracle.LAYOUTS[layout]).triangles() for o, n in csrs]
    assert ref_t.cpu().tolist() == want


@pytest.mark.timeout(300)
def test_tuning_a_fresh_matrix(eh):
    # Tuning before any count builds the plan inside the tuner.
    off, nbr = eh.graph("rmat", 13, scale=13, edges=80000).csr()[:2]
    m = eh.Matrix.build(off, nbr, "lower", "hybrid")
    shape = m.tune()
    assert shape["configs_tried"] >= 1
    fresh = eh.Matrix.build(off, nbr, "lower", "hybrid")  # picks the cached shape up at plan time
    assert fresh.count_triangles() == m.count_triangles()


def test_single_matrix_tuning_keeps_counts(eh, oracle):
    off, nbr = eh.graph("rmat", 12, scale=12, edges=40000).csr()[:2]
    m = eh.Matrix.build(off, nbr, "lower", "hybrid")
    want = m.count_triangles()
    shape = m.tune()
    assert shape["light_max"] in (32, 64, 96, 128, 160) and shape["unit_span"] in (32, 64, 128, 256, 512, 1024, 2048)
    assert m.count_triangles() == want
    assert m.count_cliques(4) == oracle.Matrix(off, nbr, oracle.SELECT_LOWER, oracle.HYBRID).cliques(4)


def test_full_row_matrix_tunes_on_lollipops(eh, oracle):
    off, nbr = eh.graph("rmat", 14, scale=12, edges=40000).csr()[:2]
    m = eh.Matrix.build(off, nbr, "all", "hybrid")
    want = oracle.Matrix(off, nbr, oracle.SELECT_ALL, oracle.HYBRID).lollipops()
    assert m.count_lollipops() == want
    shape = m.tune()
    assert shape["configs_tried"] >= 1
    assert m.count_lollipops() == want


@pytest.mark.timeout(300)
def test_one_shot_tuning_and_explicit_shape(eh, oracle):
    """eh_matrix_tune_for ranks shapes with their one-shot plan cost; its shape,
    given to a fresh matrix with eh_matrix_set_shape, is not replaced by the
    cached shape of eh_matrix_tune when the plan is built (seen in the dense
    core's memory), and counts stay exact."""
    off, nbr = eh.graph("rmat", 15, scale=13, edges=80000).csr()[:2]
    want = oracle.Matrix(off, nbr, oracle.SELECT_LOWER, oracle.HYBRID).triangles()
    m = eh.Matrix.build(off, nbr, "lower", "hybrid")
    once = m.tune(counts_per_build=1)
    assert once["configs_tried"] >= 1 and m.count_triangles() == want
    many = m.tune()
    assert m.count_triangles() == want
    sizes = {}
    for core in (0, 8192):
        fresh = eh.Matrix.build(off, nbr, "lower", "hybrid")
        fresh.set_shape(once["light_max"], once["unit_span"], once["ctas_per_sm"], core)
        assert fresh.count_triangles() == want
        sizes[core] = fresh.info()["device_bytes"]
    assert sizes[8192] - sizes[0] >= 8192 * 8191 // 128  # the 8,192-row core is there, whatever the cache says
    assert many["configs_tried"] >= 1
