"""Pins the C oracle to the reference.

1. The reference's own gtest goldens on its test/data/facebook.bin
   (test/undirected_triangle_counting_test.cpp:6-13, test/n_clique_test.cpp:6-12,
   test/undirected_lollipop_counting_test.cpp:6-13, test/similar_nodes_test.cpp:6-13);
   the graph file is committed as tests/golden/facebook.bin.gz.
2. Counts and encoded rows produced by the reference binaries themselves on the
   seeded generator graphs (tests/golden/reference_counts.json, made by
   tests/golden/make_golden.py from oracle/build_ref.sh builds).
"""
import hashlib

import pytest

import _golden

LAYOUTS = ["hybrid", "uint", "bs", "pshort"]


@pytest.mark.parametrize("layout", LAYOUTS + ["hybrid3"])
def test_facebook_gtest_goldens(oracle, layout, tmp_path):
    off, nbr, _ = oracle.read_binary(_golden.fixture_graph("facebook.bin", tmp_path))
    want = _golden.load()["reference_gtest_goldens"]
    got = oracle.counts(off, nbr, layout)
    for k in ("triangles", "cliques4", "lollipops", "similar_nodes"):
        assert got[k] == want[k], k


@pytest.mark.parametrize("spec", _golden.graphs(), ids=lambda s: s["name"])
def test_reference_fixture_counts(eh, oracle, spec):
    off, nbr = _golden.generate(eh, spec)
    for layout in LAYOUTS:
        assert oracle.counts(off, nbr, layout) == spec["counts"][layout], layout


@pytest.mark.parametrize("spec", _golden.graphs(), ids=lambda s: s["name"])
def test_reference_fixture_row_bytes(eh, oracle, spec):
    off, nbr = _golden.generate(eh, spec)
    for layout in LAYOUTS:
        for sel in ("lower", "all"):
            m = oracle.Matrix(off, nbr, oracle.SELECTIONS[sel], oracle.LAYOUTS[layout])
            got = hashlib.sha256(m.dump()).hexdigest()
            assert got == spec["rows_sha256"]["%s/%s" % (layout, sel)], (layout, sel)


def test_three_tier_mode_agrees(eh, oracle):
    spec = _golden.graphs()[5]
    off, nbr = _golden.generate(eh, spec)
    assert oracle.counts(off, nbr, "hybrid3") == spec["counts"]["hybrid"]


@pytest.mark.parametrize("layout", ["hybrid", "pshort"])
def test_oracle_clique_tables_match_counts(oracle, layout, tmp_path):
    """The oracle's n_clique table output (WRITE_TABLE) on the reference's
    facebook graph: as many 4-clique tuples as the gtest golden count, each
    descending; the 3-clique table is the triangle table."""
    import numpy as np
    off, nbr, _ = oracle.read_binary(_golden.fixture_graph("facebook.bin", tmp_path))
    m = oracle.Matrix(off, nbr, oracle.SELECT_LOWER, oracle.LAYOUTS[layout])
    t4 = m.list_cliques(4)
    assert len(t4) == _golden.load()["reference_gtest_goldens"]["cliques4"]
    assert all(np.all(t4[:, d] > t4[:, d + 1]) for d in range(3))
    t3 = m.list_cliques(3)
    tt = m.list_triangles()
    assert np.array_equal(t3, tt)
