"""CUDA path vs the reference's own outputs (tests/golden/reference_counts.json):
counts per layout and a SHA-256 of every encoded row in the reference's
flattened byte format.  Integer results: exact equality."""
import hashlib

import pytest

import _golden

pytestmark = pytest.mark.gpu
LAYOUTS = ["hybrid", "uint", "bs", "pshort"]


@pytest.mark.parametrize("spec", _golden.graphs(), ids=lambda s: s["name"])
def test_counts_match_reference(eh, spec):
    off, nbr = _golden.generate(eh, spec)
    for layout in LAYOUTS:
        want = spec["counts"][layout]
        low = eh.Matrix.build(off, nbr, "lower", layout)
        assert low.count_triangles() == want["triangles"], layout
        assert low.count_cliques(4) == want["cliques4"], layout
        full = eh.Matrix.build(off, nbr, "all", layout)
        assert full.count_lollipops() == want["lollipops"], layout
        assert full.similar_nodes(10) == want["similar_nodes"], layout


@pytest.mark.parametrize("spec", _golden.graphs(), ids=lambda s: s["name"])
def test_rows_match_reference_bytes(eh, spec):
    off, nbr = _golden.generate(eh, spec)
    for layout in LAYOUTS:
        for sel in ("lower", "all"):
            m = eh.Matrix.build(off, nbr, sel, layout)
            assert hashlib.sha256(m.dump()).hexdigest() == spec["rows_sha256"]["%s/%s" % (layout, sel)], \
                (layout, sel)
