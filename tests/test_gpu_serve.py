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


def _complete_graph(n):
    off = np.arange(0, n * n, n - 1, dtype=np.uint64)[: n + 1]
    nbr = np.array([u for v in range(n) for u in range(n) if u != v], np.uint32)
    return off, nbr


def test_memory_blocked_query_lets_small_queries_pass(eh):
    """A 4-clique query whose pivots need global scratch waits while another
    such query holds the memory under the cap; small queries submitted after
    it start before it (bounded bypass, no head-of-line blocking); a query that
    can never fit is refused; every answer equals the query run alone."""
    big_g = _complete_graph(1900)  # pivots of up to 1,899 entries: above the shared-memory tier
    small_g = eh.graph("rmat", 6, scale=10, edges=6000).csr()[:2]
    probe = eh.Server(slots=2, hbm_cap_bytes=8 << 30)
    b0, s0 = probe.add_graph(*big_g), probe.add_graph(*small_g)
    probe.wait(probe.submit(b0, eh.QUERY_CLIQUES, 4))
    st = probe.stats()
    need, resident = st["scratch_bytes"], st["resident_bytes"]
    want_big = probe.run_alone(b0, eh.QUERY_CLIQUES, 4)
    want_small = probe.run_alone(s0, eh.QUERY_TRIANGLES)
    probe.close()
    assert need > 0 and want_big == 1900 * 1899 * 1898 * 1897 // 24

    srv = eh.Server(slots=6, hbm_cap_bytes=resident + need + need // 2)  # room for one big query's scratch
    b, s = srv.add_graph(*big_g), srv.add_graph(*small_g)
    first = srv.submit(b, eh.QUERY_CLIQUES, 4)
    second = srv.submit(b, eh.QUERY_CLIQUES, 4)
    smalls = [srv.submit(s, eh.QUERY_TRIANGLES) for _ in range(12)]
    r1, r2 = srv.wait(first), srv.wait(second)
    rs = [srv.wait(t) for t in smalls]
    assert r1["count"] == r2["count"] == want_big
    assert all(r["count"] == want_small and r["status"] == 0 for r in rs)
    assert r2["start_ns"] >= r1["done_ns"]  # the two big queries never held scratch at once
    assert any(r["start_ns"] < r2["start_ns"] for r in rs)  # smaller queries passed the waiting one
    srv.close()

    tight = eh.Server(slots=2, hbm_cap_bytes=resident + need // 2)
    b, s = tight.add_graph(*big_g), tight.add_graph(*small_g)
    t_big, t_small = tight.submit(b, eh.QUERY_CLIQUES, 4), tight.submit(s, eh.QUERY_TRIANGLES)
    with pytest.raises(eh.EHError) as e:
        tight.wait(t_big)
    assert e.value.status == 8  # EH_ERR_ADMISSION: its scratch can never fit under the cap
    assert tight.wait(t_small)["count"] == want_small
    tight.close()


def test_gpu_filling_queries_run_one_at_a_time(eh):
    """Counts on a graph of at least 8M pruned edges fill the GPU by themselves:
    the server runs them one after another (never side by side), while a small
    query submitted after them starts before the last of them; every answer
    equals the query run alone."""
    big_g = eh.graph("rmat", 31, scale=19, edges=9 << 20).csr()[:2]
    small_g = eh.graph("rmat", 32, scale=10, edges=6000).csr()[:2]
    srv = eh.Server(slots=4, hbm_cap_bytes=32 << 30)
    b, s = srv.add_graph(*big_g), srv.add_graph(*small_g)
    want_big, want_small = srv.run_alone(b, eh.QUERY_TRIANGLES), srv.run_alone(s, eh.QUERY_TRIANGLES)
    bigs = [srv.submit(b, eh.QUERY_TRIANGLES) for _ in range(3)]
    small = srv.submit(s, eh.QUERY_TRIANGLES)
    rb = [srv.wait(t) for t in bigs]
    rs = srv.wait(small)
    srv.close()
    assert all(r["count"] == want_big for r in rb) and rs["count"] == want_small
    for x, y in zip(rb, rb[1:]):
        assert y["start_ns"] >= x["done_ns"]  # in submission order, never overlapping
    assert rs["start_ns"] < rb[-1]["start_ns"]  # the small query did not wait behind them
