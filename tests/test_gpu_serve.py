"""Serving loop: continuous batching over device-resident graphs.  Every
query's answer in the concurrent mix equals the same query run alone and the
oracle's (integers, tolerance 0); admission and waits are bounded."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(eh):
    graphs = [eh.graph("rmat", 100 + k, scale=s, edges=16 << s).csr()[:2] for k, s in enumerate([10, 11, 12, 13])]
    graphs.append(eh.graph("planted", 7, n=3000, edges=9000, cliques=4, min_size=20, max_size=60).csr()[:2])
    srv = eh.Server(slots=6, hbm_cap_bytes=8 << 30)
    ids = [srv.add_graph(o, n, "hybrid") for o, n in graphs]
    yield eh, srv, ids, graphs
    srv.close()


def test_mix_equals_alone_and_oracle(served, oracle):
    eh, srv, ids, graphs = served
    rng = np.random.default_rng(1)
    kinds = [(eh.QUERY_TRIANGLES, 0), (eh.QUERY_CLIQUES, 4), (eh.QUERY_CLIQUES, 3), (eh.QUERY_SIMILAR_NODES, 10),
             (eh.QUERY_CLIQUES, 5)]
    mix = [(int(rng.integers(len(ids))), *kinds[int(rng.integers(len(kinds)))]) for _ in range(120)]
    tickets = [srv.submit(ids[g], k, p) for g, k, p in mix]
    results = [srv.wait(t) for t in tickets]
    st = srv.stats()
    assert st["completed"] >= len(mix) and st["max_inflight"] >= 2  # work overlapped on the device
    alone = {}
    for (g, k, p), r in zip(mix, results):
        assert r["status"] == 0 and r["done_ns"] >= r["start_ns"] >= r["submit_ns"]
        key = (g, k, p)
        if key not in alone:
            alone[key] = srv.run_alone(ids[g], k, p)
        assert r["count"] == alone[key], key
    for (g, k, p), want in alone.items():
        o, n = graphs[g]
        if k == eh.QUERY_SIMILAR_NODES:
            assert want == oracle.Matrix(o, n, oracle.SELECT_ALL, oracle.HYBRID).similar_nodes(p)
        else:
            kk = 3 if k == eh.QUERY_TRIANGLES else p
            assert want == oracle.Matrix(o, n, oracle.SELECT_LOWER, oracle.HYBRID).cliques(kk)


def test_admission_and_bounded_waits(eh):
    o, n = eh.graph("rmat", 5, scale=11, edges=20000).csr()[:2]
    srv = eh.Server(slots=2, hbm_cap_bytes=1 << 16)  # far too small for any graph
    with pytest.raises(eh.EHError) as e:
        srv.add_graph(o, n)
    assert e.value.status == 8  # EH_ERR_ADMISSION
    srv.close()
    srv = eh.Server(slots=1, hbm_cap_bytes=1 << 30)
    g = srv.add_graph(o, n)
    t = srv.submit(g, eh.QUERY_TRIANGLES)
    r = srv.wait(t, timeout_ms=60000)
    assert r["count"] == srv.run_alone(g, eh.QUERY_TRIANGLES)
    with pytest.raises(eh.EHError):
        srv.wait(t)  # a ticket is released by its wait
    with pytest.raises(eh.EHError):
        srv.submit(99, eh.QUERY_TRIANGLES)
    srv.close()
