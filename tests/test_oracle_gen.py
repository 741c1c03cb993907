"""oracle/eh_gen.c regenerates the library's seeded R-MAT graphs on the CPU
(for bench.py's CPU baseline arm, which must not load the GPU library).  Its
degree-ordered CSR must equal the library generator's byte for byte."""
import pytest

import _golden


@pytest.mark.parametrize("scale,edges,seed", [(8, 300, 5), (10, 8000, 101), (12, 50000, 102), (14, 200000, 103)])
def test_oracle_rmat_equals_library_generator(eh, oracle, scale, edges, seed):
    want = eh.graph("rmat", seed, scale=scale, edges=edges).csr()[:2]
    got = oracle.rmat_graph(scale, edges, seed)
    assert _golden.csr_sha(*got) == _golden.csr_sha(*want)


def test_oracle_rmat_equals_fixture_graph(oracle):
    spec = next(g for g in _golden.graphs() if g["name"] == "rmat_s16_1m")
    off, nbr = oracle.rmat_graph(spec["params"]["scale"], spec["params"]["edges"], spec["seed"])
    assert _golden.csr_sha(off, nbr) == spec["csr_sha256"]


def test_oracle_rmat_dense_case_needs_more_draws(eh, oracle):
    # All 28 pairs of 8 vertices: R-MAT's skew makes the last pairs rare, so both
    # generators draw several rounds; the graph is complete either way.
    want = eh.graph("rmat", 1, scale=3, edges=28).csr()[:2]
    got = oracle.rmat_graph(3, 28, 1)
    assert _golden.csr_sha(*got) == _golden.csr_sha(*want)
    assert len(got[1]) == 56
