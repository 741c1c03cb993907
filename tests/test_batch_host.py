"""Host-side batch logic: deterministic workload specs and input validation
(rejected before any device work)."""
import numpy as np
import pytest


def test_batch_specs_are_deterministic_and_in_range():
    from simdgraphprocessing_gb300 import workloads as W
    a = W.batch_specs(256)
    assert a == W.batch_specs(256)
    ns = [kw["n"] for _, _, kw in a]
    assert min(ns) >= 200 and max(ns) <= 50000
    kinds = [k for k, _, _ in a]
    assert kinds.count("er") == kinds.count("ba") == 128
    for kind, s, kw in a:
        if kind == "ba":
            assert 2 <= kw["m"] <= 32
        else:
            assert 4 * kw["n"] / 2 - 1 <= kw["edges"] <= 64 * kw["n"] / 2 + 1
    # log-uniform: about as many graphs below the geometric midpoint (3162) as above
    lo = sum(n < 3162 for n in ns)
    assert 90 < lo < 166


def test_serving_specs_cover_scales():
    from simdgraphprocessing_gb300 import workloads as W
    sp = W.serving_specs()
    assert len(sp) == 32 and {s for s, _, _ in sp} == set(range(14, 24))


def test_concat_graphs_block_diagonal(eh):
    g1 = (np.array([0, 1, 2], np.uint64), np.array([1, 0], np.uint32))
    g2 = (np.array([0, 2, 3, 4], np.uint64), np.array([1, 2, 0, 0], np.uint32))
    gr, off, nbr = eh.concat_graphs([g1, g2])
    assert gr.tolist() == [0, 2, 5]
    assert off.tolist() == [0, 1, 2, 4, 5, 6]
    assert nbr.tolist() == [1, 0, 3, 4, 2, 2]


def test_batch_rejects_edges_that_leave_their_graph(eh):
    gr = np.array([0, 2, 4], np.uint64)
    off = np.array([0, 1, 2, 3, 4], np.uint64)
    nbr = np.array([1, 0, 0, 2], np.uint32)  # row 2 (graph 1) points into graph 0
    with pytest.raises(eh.EHError) as e:
        eh.Batch(gr, off, nbr)
    assert e.value.status == 1 and "leaves" in str(e.value)
    with pytest.raises(eh.EHError):
        eh.Batch(np.array([0, 3], np.uint64), off, np.array([1, 0, 3, 2], np.uint32))  # rows end at 4, not 3
