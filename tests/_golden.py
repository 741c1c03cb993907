"""Shared helpers for the committed reference fixtures (tests/golden/)."""
import gzip
import hashlib
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "reference_counts.json")
LARGE_FIXTURE = os.path.join(HERE, "golden", "reference_large.json")
# The reference source tree, for the tests that compile its sources (set
# EH_REFERENCE to its path; those tests are skipped without it).
REFERENCE_TREE = os.environ.get("EH_REFERENCE") or None

# The reference's own test graphs (its test/data/facebook.bin and
# test/data/dfacebook.bin, byte for byte, gzip-compressed) and their SHA-256.
FACEBOOK = {
    "facebook.bin": "7be683d99952d5ff0ade026151d2f42d576fc9373309688e65ccdcfee183843e",
    "dfacebook.bin": "e6100bd8fe240b283f4679de69175acf93ea400ecc46f6e0b33ffadc0960c286",
}


def reference_file(*parts):
    """Path of a file in the reference tree, or None without EH_REFERENCE."""
    if not REFERENCE_TREE:
        return None
    p = os.path.join(REFERENCE_TREE, *parts)
    return p if os.path.exists(p) else None


def fixture_graph(name, directory):
    """Writes the reference test graph `name` (facebook.bin / dfacebook.bin)
    into `directory` and returns its path, after checking its SHA-256."""
    with gzip.open(os.path.join(HERE, "golden", name + ".gz"), "rb") as f:
        data = f.read()
    assert hashlib.sha256(data).hexdigest() == FACEBOOK[name], name
    path = os.path.join(str(directory), name)
    with open(path, "wb") as f:
        f.write(data)
    return path


def load_large():
    with open(LARGE_FIXTURE) as f:
        return json.load(f)


def large_graph(name):
    return next(g for g in load_large()["graphs"] if g["name"] == name)


def load():
    with open(FIXTURE) as f:
        return json.load(f)


def graphs():
    return load()["graphs"]


def csr_sha(off, nbr):
    h = hashlib.sha256()
    h.update(off.astype("<u8").tobytes())
    h.update(nbr.astype("<u4").tobytes())
    return h.hexdigest()


def generate(eh, spec):
    g = eh.graph(spec["kind"], spec["seed"], **spec["params"])
    off, nbr, _, _ = g.csr()
    assert csr_sha(off, nbr) == spec["csr_sha256"], "generator drifted from the fixture graph"
    return off, nbr


DIRECTED_FIXTURE = os.path.join(HERE, "golden", "reference_directed.json")


def load_directed():
    with open(DIRECTED_FIXTURE) as f:
        return json.load(f)


def directed_graphs():
    return load_directed()["graphs"]


def directed_sha(g):
    off, nbr, _, _ = g.csr()
    ioff, inbr = g.in_csr()
    h = hashlib.sha256()
    for a, t in ((off, "<u8"), (nbr, "<u4"), (ioff, "<u8"), (inbr, "<u4")):
        h.update(a.astype(t).tobytes())
    return h.hexdigest()


def generate_directed(eh, spec):
    """(out_off, out_nbr, in_off, in_nbr) of a directed fixture graph."""
    g = eh.graph(spec["kind"], spec["seed"], **spec["params"])
    assert directed_sha(g) == spec["sha256"], "generator drifted from the fixture graph"
    off, nbr, _, _ = g.csr()
    ioff, inbr = g.in_csr()
    return off, nbr, ioff, inbr


def full_block_directed():
    """Directed (out_off, out_nbr): vertex h = 65536 with out- and in-edges to
    every vertex of [0, 65536), so out(h) and in(h) each fill the 2^16 block 0."""
    import numpy as np
    h = 65536
    off = np.zeros(h + 2, np.uint64)
    off[1:h + 1] = np.arange(1, h + 1)
    off[h + 1] = 2 * h
    nbr = np.concatenate([np.full(h, h, np.uint32), np.arange(h, dtype=np.uint32)])
    return off, nbr


def full_block_undirected():
    """Symmetric (off, nbr): rows 65536 and 65537 both adjacent to all of [0, 65536)."""
    import numpy as np
    deg = np.concatenate([np.full(65536, 2), [65536, 65536]]).astype(np.uint64)
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint64)
    nbr = np.concatenate([np.tile(np.array([65536, 65537], np.uint32), 65536),
                          np.arange(65536, dtype=np.uint32), np.arange(65536, dtype=np.uint32)])
    return off, nbr
