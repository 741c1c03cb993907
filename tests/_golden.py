"""Shared helpers for the committed reference fixtures (tests/golden/)."""
import hashlib
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "reference_counts.json")
REFERENCE_TREE = os.environ.get("EH_REFERENCE", "/root/reference")


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
