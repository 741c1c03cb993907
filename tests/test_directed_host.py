"""Directed graphs on the host and the oracle's symbiosity / n_path.

* MutableGraph::directedFromBinary / writeDirectedToBinary /
  directedFromEdgeList (src/MutableGraph.hpp:634-714, 893-986) restated by
  eh_hgraph_*_directed_*; checked against a plain-Python reading of the format
  and byte for byte on the reference's test/data/dfacebook.bin (committed as
  tests/golden/dfacebook.bin.gz).
* The oracle's symbiosity (apps/symbiosity.cpp:39-58) and n_path
  (apps/n_path.cpp:30-88) pinned to the reference's gtest goldens
  (test/symbiosity_test.cpp:6-20, test/n_path_test.cpp:6-12) and to the
  reference binaries' outputs on seeded directed graphs
  (tests/golden/reference_directed.json).
"""
import os
import tempfile

import numpy as np
import pytest

import _golden

LAYOUTS = ["hybrid", "uint", "bs", "pshort"]


def _oracle_pair(oracle, spec_arrays, layout):
    off, nbr, ioff, inbr = spec_arrays
    rows = oracle.Matrix(off, nbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout])
    cols = oracle.Matrix(ioff, inbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout])
    return rows, cols


def test_directed_binary_roundtrip(eh, oracle):
    g = eh.graph("drmat", 11, scale=9, edges=3000)
    assert g.directed
    off, nbr, ext, mx = g.csr()
    ioff, inbr = g.in_csr()
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "g.dbin")
        g.write_directed_binary(p)
        oo, on, io, inn, ex = oracle.read_directed_binary(p)
        assert np.array_equal(oo, off) and np.array_equal(on, nbr)
        assert np.array_equal(io, ioff) and np.array_equal(inn, inbr)
        h = eh.HostGraph.read_directed_binary(p)
        assert h.directed
        for a, b in zip(h.csr()[:3], (off, nbr, ext)):
            assert np.array_equal(a, b)
        assert h.csr()[3] == max(np.diff(off).max(), np.diff(ioff).max())


def test_in_csr_is_the_transpose(eh):
    g = eh.graph("drmat", 12, scale=10, edges=6000)
    off, nbr, _, _ = g.csr()
    ioff, inbr = g.in_csr()
    n = len(off) - 1
    src = np.repeat(np.arange(n), np.diff(off).astype(np.int64))
    pairs = sorted(zip(nbr.tolist(), src.tolist()))
    want_nbr = np.array([s for _, s in pairs], np.uint32)
    want_off = np.zeros(n + 1, np.uint64)
    np.add.at(want_off, np.array([d for d, _ in pairs], np.int64) + 1, 1)
    assert np.array_equal(ioff, np.cumsum(want_off))
    assert np.array_equal(inbr, want_nbr)


def test_directed_edge_list_semantics(eh):
    # ids interned in order of first appearance (src before dst); rows sorted
    # and deduplicated; self-loops kept.
    text = "10 20\n20 10\n10 30\n30 30\n10 20\n40 10\n"
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "e.txt")
        with open(p, "w") as f:
            f.write(text)
        g = eh.HostGraph.read_directed_edge_list(p)
    off, nbr, ext, mx = g.csr()
    ioff, inbr = g.in_csr()
    assert list(ext) == [10, 20, 30, 40]
    outs = [list(nbr[off[i]:off[i + 1]]) for i in range(4)]
    ins = [list(inbr[ioff[i]:ioff[i + 1]]) for i in range(4)]
    assert outs == [[1, 2], [0], [2], [0]]
    assert ins == [[1, 3], [0], [0, 2], []]
    assert mx == 3  # row 0's out-list [20, 30, 20] before deduplication


def test_undirected_in_view_and_reorder_guard(eh):
    u = eh.graph("rmat", 1, scale=9, edges=2000)
    assert not u.directed
    assert np.array_equal(u.in_csr()[1], u.csr()[1])
    d = eh.graph("drmat", 1, scale=9, edges=2000)
    with pytest.raises(eh.EHError):
        d.reorder_by_degree()


def test_directed_from_csr_rejects_bad_rows(eh):
    with pytest.raises(eh.EHError):
        eh.HostGraph.directed_from_csr(np.array([0, 2, 2], np.uint64), np.array([1, 1], np.uint32))
    with pytest.raises(eh.EHError):
        eh.HostGraph.directed_from_csr(np.array([0, 1, 1], np.uint64), np.array([5], np.uint32))


def test_dfacebook_read_write_bytes(eh, tmp_path):
    DFB = _golden.fixture_graph("dfacebook.bin", tmp_path)
    g = eh.HostGraph.read_directed_binary(DFB)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "d.bin")
        g.write_directed_binary(p)
        with open(p, "rb") as a, open(DFB, "rb") as b:
            assert a.read() == b.read()


def test_oracle_gtest_goldens(oracle, tmp_path):
    DFB = _golden.fixture_graph("dfacebook.bin", tmp_path)
    FB = _golden.fixture_graph("facebook.bin", tmp_path)
    want = _golden.load_directed()["reference_gtest_goldens"]
    oo, on, io, inn, _ = oracle.read_directed_binary(DFB)
    rows, cols = _oracle_pair(oracle, (oo, on, io, inn), "hybrid")
    assert rows.symbiosity(cols) == want["symbiosity_dfacebook_hybrid"]
    off, nbr, _ = oracle.read_binary(FB)
    und = oracle.Matrix(off, nbr, oracle.SELECT_ALL, oracle.LAYOUTS["hybrid"])
    assert und.symbiosity() == want["symbiosity_facebook_hybrid"]
    uint = oracle.Matrix(oo, on, oracle.SELECT_ALL, oracle.LAYOUTS["uint"])
    assert uint.n_path(0, 4)[0] == want["n_path_dfacebook_uint_start0_n4"]


@pytest.mark.parametrize("spec", _golden.directed_graphs(), ids=lambda s: s["name"])
def test_oracle_matches_reference_binaries(eh, oracle, spec):
    arrays = _golden.generate_directed(eh, spec)
    doc = _golden.load_directed()
    key = "n_path_s%d_d%d" % (doc["n_path_start"], doc["n_path_depth"])
    for layout in LAYOUTS:
        rows, cols = _oracle_pair(oracle, arrays, layout)
        want = spec["counts"][layout]
        assert rows.symbiosity(cols) == want["symbiosity"], layout
        assert rows.max_row_id() == want["n_path_start"], layout
        assert rows.n_path(want["n_path_start"])[0] == want["n_path"], layout
        assert rows.n_path(doc["n_path_start"], doc["n_path_depth"])[0] == want[key], layout


def test_oracle_full_block_quirks(eh, oracle):
    quirks = _golden.load_directed()["quirks"]
    off, nbr = _golden.full_block_directed()
    g = eh.HostGraph.directed_from_csr(off, nbr)
    ioff, inbr = g.in_csr()
    uoff, unbr = _golden.full_block_undirected()
    for layout in LAYOUTS:
        rows, cols = _oracle_pair(oracle, (off, nbr, ioff, inbr), layout)
        assert rows.symbiosity(cols) == quirks["symbiosity_full_block"][layout], layout
        u = oracle.Matrix(uoff, unbr, oracle.SELECT_ALL, oracle.LAYOUTS[layout])
        assert u.similar_nodes(10) == quirks["similar_nodes_full_block"][layout], layout
