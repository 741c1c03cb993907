"""Host-side graph logic (the reference's MutableGraph) against numpy
restatements and the reference's documented behaviour."""
import os

import numpy as np
import pytest

import _golden


def degree_order_numpy(off, nbr, ext):
    """OrderNeighborhoodByDegree (src/MutableGraph.hpp:20-32) + reassign_ids (:100-123)."""
    n = len(off) - 1
    deg = np.diff(off.astype(np.int64))
    new2old = np.lexsort((np.arange(n), -deg))  # degree desc, id asc
    old2new = np.empty(n, np.int64)
    old2new[new2old] = np.arange(n)
    rows = [np.sort(old2new[nbr[off[o]:off[o + 1]]]) for o in new2old]
    noff = np.zeros(n + 1, np.uint64)
    noff[1:] = np.cumsum([len(r) for r in rows])
    return noff, np.concatenate(rows).astype(np.uint32), ext[new2old]


def test_reorder_by_degree_matches_restatement(eh):
    g = eh.HostGraph.rmat(11, 15000, 77)
    off, nbr, ext, _ = g.csr()
    g.reorder_by_degree()
    off2, nbr2, ext2, _ = g.csr()
    roff, rnbr, rext = degree_order_numpy(off, nbr, ext)
    assert np.array_equal(off2, roff) and np.array_equal(nbr2, rnbr) and np.array_equal(ext2, rext)


def test_binary_round_trip(eh, tmp_path):
    g = eh.graph("ba", 3, n=500, m=4)
    p = str(tmp_path / "g.bin")
    g.write_binary(p)
    h = eh.HostGraph.read_binary(p)
    a, b = g.csr(), h.csr()
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    # layout of the file: u64 n, then per row u64 ext id, u64 length, u32 ids
    raw = open(p, "rb").read()
    assert int.from_bytes(raw[:8], "little") == 500
    assert len(raw) == 8 + 500 * 16 + 4 * len(a[1])


def test_truncated_binary_is_an_io_error(eh, tmp_path):
    g = eh.graph("er", 4, n=100, edges=300)
    p = str(tmp_path / "g.bin")
    g.write_binary(p)
    data = open(p, "rb").read()
    open(p, "wb").write(data[:-7])
    with pytest.raises(eh.EHError) as e:
        eh.HostGraph.read_binary(p)
    assert e.value.status == 5


def test_malformed_binary_headers_are_io_errors(eh, tmp_path):
    """Record counts and row lengths that the file cannot hold are rejected
    before anything of that size is allocated; a missing file is an I/O error
    too; trailing bytes after the last record are ignored, as before."""
    import struct
    p = str(tmp_path / "bad.bin")
    cases = [
        struct.pack("<Q", 1 << 31),                                   # 2^31 rows, no records
        struct.pack("<QQQ", 1, 0, 1 << 60),                          # one row of 2^60 entries
        struct.pack("<QQQ", 2, 0, 1) + struct.pack("<I", 1),         # second record missing
        struct.pack("<Q", 1 << 40),                                   # n beyond the u32 id space
        b"\x01\x00",                                                  # shorter than the header
    ]
    for blob in cases:
        open(p, "wb").write(blob)
        for reader in (eh.HostGraph.read_binary, eh.HostGraph.read_directed_binary):
            with pytest.raises(eh.EHError) as e:
                reader(p)
            assert e.value.status == 5, (blob, reader)
    with pytest.raises(eh.EHError) as e:
        eh.HostGraph.read_binary(str(tmp_path / "missing.bin"))
    assert e.value.status == 5
    g = eh.graph("er", 4, n=100, edges=300)
    g.write_binary(p)
    open(p, "ab").write(b"trailing bytes")
    h = eh.HostGraph.read_binary(p)
    assert all(np.array_equal(x, y) for x, y in zip(g.csr()[:3], h.csr()[:3]))


def test_edge_list_semantics(eh, tmp_path):
    # undirectedFromEdgeList (src/MutableGraph.hpp:517-599): ids in order of first
    # appearance, both directions, sorted + deduplicated rows, self-loops kept,
    # max_nbrhood_size taken before deduplication.
    p = tmp_path / "e.txt"
    p.write_text("10 20\n20 10\n10 30\n30 30\n40\t10\n")
    g = eh.HostGraph.read_edge_list(str(p))
    off, nbr, ext, mx = g.csr()
    assert list(ext) == [10, 20, 30, 40]
    rows = [list(nbr[off[i]:off[i + 1]]) for i in range(4)]
    assert rows == [[1, 2, 3], [0], [0, 2], [0]]
    assert mx == 4  # row of 10 held [1, 1, 2, 3] before dedup


@pytest.mark.parametrize("spec", _golden.graphs(), ids=lambda s: s["name"])
def test_generators_are_deterministic_and_clean(eh, spec):
    off, nbr = _golden.generate(eh, spec)  # asserts the fixture's CSR hash
    n = len(off) - 1
    row = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
    assert not np.any(nbr == row), "self-loop"
    d = np.diff(nbr.astype(np.int64))
    same = row[1:] == row[:-1]
    assert np.all(d[same] > 0), "row not strictly ascending"
    # symmetric
    fwd = set(zip(row.tolist(), nbr.tolist()))
    assert all((b, a) in fwd for a, b in list(fwd)[:2000])


def test_rmat_edge_count_is_exact(eh):
    g = eh.HostGraph.rmat(12, 30000, 5)
    off, nbr, _, _ = g.csr()
    assert len(nbr) == 2 * 30000
