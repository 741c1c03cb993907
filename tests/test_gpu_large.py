"""Benchmark-size parity: the GPU counts on the configurations' own graphs equal
the reference binaries' counts committed in tests/golden/reference_large.json
(made by tests/golden/make_golden.py --large from the unmodified reference
sources; integer counts, tolerance 0).

* R-MAT scale 22, edge factor 16, seed 2: triangles (the headline graph);
* R-MAT scale 20, edge factor 16, seed 3 and the planted-clique graph
  (2^20 vertices, 1,024 cliques of 64..512 vertices over G(n, p=1e-4)):
  triangles, 4-cliques and lollipops;
* the 4,096-graph batch: every graph's triangle and 4-clique count (the first
  512 graphs here; bench.py --workload batch checks all 4,096).
Each generated CSR is first checked against the fixture's SHA-256."""
import pytest

import _golden

pytestmark = pytest.mark.gpu


def generate(eh, spec):
    if spec["kind"] == "planted_workload":
        from simdgraphprocessing_gb300 import workloads as W
        g = W.planted_graph(spec["seed"])
    else:
        g = eh.graph(spec["kind"], spec["seed"], **spec["params"])
    off, nbr = g.csr()[:2]
    assert _golden.csr_sha(off, nbr) == spec["csr_sha256"], "generator drifted from the fixture graph"
    return off, nbr


@pytest.mark.timeout(900)
def test_headline_triangles_equal_reference_binary(eh):
    spec = _golden.large_graph("rmat_s22_ef16_seed2")
    off, nbr = generate(eh, spec)
    m = eh.Matrix.build(off, nbr, "lower", "hybrid")
    assert m.count_triangles() == spec["counts"]["triangles"]
    assert m.count_triangles() == spec["counts"]["triangles"]  # plan reused, same answer


@pytest.mark.timeout(900)
@pytest.mark.parametrize("name", ["rmat_s20_ef16_seed3", "planted_2^20_p1e-4_1024cliques_seed3"])
def test_clique_workloads_equal_reference_binary(eh, name):
    spec = _golden.large_graph(name)
    off, nbr = generate(eh, spec)
    low = eh.Matrix.build(off, nbr, "lower", "hybrid")
    assert low.count_triangles() == spec["counts"]["triangles"]
    assert low.count_cliques(4) == spec["counts"]["cliques4"]
    del low
    full = eh.Matrix.build(off, nbr, "all", "hybrid")
    assert full.count_lollipops() == spec["counts"]["lollipops"]


@pytest.mark.timeout(900)
def test_batch_graphs_equal_reference_binary(eh):
    torch = pytest.importorskip("torch")
    from simdgraphprocessing_gb300 import workloads as W
    fx = _golden.load_large()["batch"]
    G = 512
    csrs = [eh.graph(kind, s, **kw).csr()[:2] for kind, s, kw in W.batch_specs()[:G]]
    gr, off, nbr = eh.concat_graphs(csrs)
    s = torch.cuda.Stream()
    b = eh.Batch(gr, off, nbr, layout="hybrid", stream=s)
    tri = torch.zeros(G, dtype=torch.int64, device="cuda")
    clq = torch.zeros(G, dtype=torch.int64, device="cuda")
    b.run(tri.data_ptr(), clq.data_ptr(), use_graph=True, stream=s)  # captured and replayed
    s.synchronize()
    assert tri.cpu().tolist() == fx["triangles"][:G]
    assert clq.cpu().tolist() == fx["cliques4"][:G]
