"""Regenerates tests/golden/reference_counts.json.

Runs the reference's own binaries -- compiled from its unmodified sources by
oracle/build_ref.sh into oracle/_ref/ -- on seeded generator graphs written in
the reference's binary format, and records:
  * the app counts per layout (undirected_triangle_counting, n_clique n=4,
    undirected_lollipop_counting, similar_nodes), parsed from their output;
  * a SHA-256 of the reference's encoded rows (oracle/ref_rowdump.cpp) per
    layout and edge selection, for byte-format parity;
  * a SHA-256 of the generated CSR, so that a host that regenerates the graph
    (x86-64 or aarch64) can prove it got the same input.
With --directed it writes tests/golden/reference_directed.json instead: the
symbiosity and n_path apps on seeded directed graphs (directed binary format).
With --large it writes tests/golden/reference_large.json: the reference
binaries' counts on the benchmark-size graphs (R-MAT scale 22 edge factor 16
triangles; R-MAT scale 20 and the planted-clique graph on 2^20 vertices,
4-cliques and lollipops) and on every graph of the 4,096-graph batch
(triangles and 4-cliques), each keyed by the SHA-256 of the generated CSR.
Needs an x86-64 host with the reference tree (the reference uses SSE/AVX).
Usage: python tests/golden/make_golden.py [--directed | --large]
"""
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import simdgraphprocessing_gb300 as eh  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
OUT = os.path.join(HERE, "reference_counts.json")
OUT_DIRECTED = os.path.join(HERE, "reference_directed.json")

GRAPHS = [
    {"name": "rmat_s10", "kind": "rmat", "seed": 101, "params": {"scale": 10, "edges": 8000}},
    {"name": "rmat_s12", "kind": "rmat", "seed": 102, "params": {"scale": 12, "edges": 50000}},
    {"name": "rmat_s14", "kind": "rmat", "seed": 103, "params": {"scale": 14, "edges": 200000}},
    {"name": "er_2000", "kind": "er", "seed": 104, "params": {"n": 2000, "edges": 20000}},
    {"name": "ba_3000", "kind": "ba", "seed": 105, "params": {"n": 3000, "m": 6}},
    {"name": "planted_5000", "kind": "planted", "seed": 106,
     "params": {"n": 5000, "edges": 15000, "cliques": 5, "min_size": 16, "max_size": 80}},
    {"name": "dense_er_300", "kind": "er", "seed": 107, "params": {"n": 300, "edges": 20000}},
    # The 2^16-vertex, 1M-edge R-MAT graph of the uint triangle-count workload.
    {"name": "rmat_s16_1m", "kind": "rmat", "seed": 1, "params": {"scale": 16, "edges": 1000000}},
]
LAYOUTS = ["hybrid", "uint", "bs", "pshort"]
APPS = {
    "triangles": ("undirected_triangle_counting", r"Number of triangles:\s*(\d+)"),
    "cliques4": ("n_clique", r"Number of cliques:\s*(\d+)"),
    "lollipops": ("undirected_lollipop_counting", r"Count:\s*(\d+)"),
    "similar_nodes": ("similar_nodes", r"Count:\s*(\d+)"),
}


# Graphs for the directed apps (symbiosity, n_path), written in the directed
# binary format and run with --asymmetric; "undirected" entries use the
# undirected format and loader.
DIRECTED = [
    {"name": "drmat_s10", "kind": "drmat", "seed": 201, "params": {"scale": 10, "edges": 6000}},
    {"name": "drmat_s13", "kind": "drmat", "seed": 202, "params": {"scale": 13, "edges": 80000}},
    {"name": "recip_rmat_s12", "kind": "recip", "seed": 203,
     "params": {"base": "rmat", "base_params": {"scale": 12, "edges": 50000}, "p_both": 0.5}},
    {"name": "recip_er_3000", "kind": "recip", "seed": 204,
     "params": {"base": "er", "base_params": {"n": 3000, "edges": 30000}, "p_both": 0.7}},
    # Rows longer than 4,096 entries (the GPU BFS splits those over the grid).
    {"name": "recip_rmat_s15", "kind": "recip", "seed": 205,
     "params": {"base": "rmat", "base_params": {"scale": 15, "edges": 1000000}, "p_both": 0.6}},
    {"name": "rmat_s12_undirected", "kind": "rmat", "seed": 102, "params": {"scale": 12, "edges": 50000},
     "undirected": True},
]
NPATH_START, NPATH_DEPTH = 7, 2


def directed_sha(g):
    off, nbr, _, _ = g.csr()
    ioff, inbr = g.in_csr()
    h = hashlib.sha256()
    for a, t in ((off, "<u8"), (nbr, "<u4"), (ioff, "<u8"), (inbr, "<u4")):
        h.update(a.astype(t).tobytes())
    return h.hexdigest()


def run_directed(binary, graph, layout, undirected, extra=()):
    args = [os.path.join(REF, binary), "--graph=" + graph, "--input_type=binary", "--t=4", "--layout=" + layout]
    if not undirected:
        args.append("--asymmetric")
    return subprocess.run(args + list(extra), stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                          check=True).stdout


def make_directed(td):
    entries = []
    for spec in DIRECTED:
        g = eh.graph(spec["kind"], spec["seed"], **spec["params"])
        path = os.path.join(td, spec["name"] + ".dbin")
        und = spec.get("undirected", False)
        if und:
            g.write_binary(path)
        else:
            g.write_directed_binary(path)
        e = dict(spec)
        off, nbr, _, _ = g.csr()
        e["n"] = int(len(off) - 1)
        e["out_entries"] = int(len(nbr))
        e["sha256"] = directed_sha(g)
        e["counts"] = {}
        for layout in LAYOUTS:
            c = {}
            out = run_directed("symbiosity", path, layout, und)
            c["symbiosity"] = int(re.search(r"Count:\s*(\d+)", out).group(1))
            out = run_directed("n_path", path, layout, und)
            c["n_path_start"] = int(re.search(r"Internal:\s*(\d+)", out).group(1))
            c["n_path"] = int(re.search(r"path length:\s*(\d+)", out).group(1))
            out = run_directed("n_path", path, layout, und,
                               ("--start_node=%d" % NPATH_START, "--n=%d" % NPATH_DEPTH))
            c["n_path_s%d_d%d" % (NPATH_START, NPATH_DEPTH)] = int(re.search(r"path length:\s*(\d+)", out).group(1))
            e["counts"][layout] = c
        print(spec["name"], e["counts"]["hybrid"], flush=True)
        entries.append(e)
    return entries


def csr_sha(off, nbr):
    h = hashlib.sha256()
    h.update(off.astype("<u8").tobytes())
    h.update(nbr.astype("<u4").tobytes())
    return h.hexdigest()


def run_app(binary, graph, layout):
    out = subprocess.run([os.path.join(REF, binary), "--graph=" + graph, "--input_type=binary",
                          "--t=4", "--layout=" + layout], stdout=subprocess.PIPE,
                         stderr=subprocess.STDOUT, text=True, check=True).stdout
    return out


def full_block_quirks(td):
    """The pshort u16 partition-count quirk (intersection.hpp:857-865) as the
    reference binaries show it on the two full-block graphs of tests/_golden.py."""
    sys.path.insert(0, os.path.dirname(HERE))
    import _golden
    out = {"symbiosity_full_block": {}, "similar_nodes_full_block": {}}
    off, nbr = _golden.full_block_directed()
    dpath = os.path.join(td, "full_block.dbin")
    eh.HostGraph.directed_from_csr(off, nbr).write_directed_binary(dpath)
    off, nbr = _golden.full_block_undirected()
    upath = os.path.join(td, "full_block.bin")
    eh.HostGraph.from_csr(off, nbr).write_binary(upath)
    for layout in LAYOUTS:
        o = run_directed("symbiosity", dpath, layout, False)
        out["symbiosity_full_block"][layout] = int(re.search(r"Count:\s*(\d+)", o).group(1))
        o = run_app("similar_nodes", upath, layout)
        out["similar_nodes_full_block"][layout] = int(re.search(r"Count:\s*(\d+)", o).group(1))
    return out


def main_directed():
    with tempfile.TemporaryDirectory() as td:
        entries = make_directed(td)
        quirks = full_block_quirks(td)
    doc = {
        "generated_by": "tests/golden/make_golden.py --directed",
        "reference_binaries": "oracle/build_ref.sh (unmodified reference sources): apps symbiosity, n_path",
        "reference_gtest_goldens": {
            "source": "reference test/symbiosity_test.cpp, test/n_path_test.cpp",
            "symbiosity_dfacebook_hybrid": 0, "symbiosity_facebook_hybrid": 4039,
            "n_path_dfacebook_uint_start0_n4": 4,
        },
        "n_path_start": NPATH_START, "n_path_depth": NPATH_DEPTH,
        "graphs": entries,
        "quirks": quirks,
    }
    with open(OUT_DIRECTED, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)
    print("wrote", OUT_DIRECTED)


OUT_LARGE = os.path.join(HERE, "reference_large.json")

# Benchmark-size graphs: (name, how to generate, apps).  Counts do not depend on
# the layout (the reference's own cross-layout agreement), so the reference
# runs the hybrid layout, the one these workloads use.
LARGE = [
    {"name": "rmat_s22_ef16_seed2", "kind": "rmat", "seed": 2, "params": {"scale": 22, "edges": 16 << 22},
     "apps": ["triangles"]},
    {"name": "rmat_s20_ef16_seed3", "kind": "rmat", "seed": 3, "params": {"scale": 20, "edges": 16 << 20},
     "apps": ["triangles", "cliques4", "lollipops"]},
    {"name": "planted_2^20_p1e-4_1024cliques_seed3", "kind": "planted_workload", "seed": 3, "params": {},
     "apps": ["triangles", "cliques4", "lollipops"]},
]


def large_graph(spec):
    if spec["kind"] == "planted_workload":
        from simdgraphprocessing_gb300 import workloads as W
        return W.planted_graph(spec["seed"])
    return eh.graph(spec["kind"], spec["seed"], **spec["params"])


def run_app_threads(binary, graph, layout, threads):
    return subprocess.run([os.path.join(REF, binary), "--graph=" + graph, "--input_type=binary",
                           "--t=%d" % threads, "--layout=" + layout], stdout=subprocess.PIPE,
                          stderr=subprocess.STDOUT, text=True, check=True).stdout


def batch_reference_counts(td, threads):
    """The reference's triangle and 4-clique counts of every graph of the
    4,096-graph batch workload (seeds 4 + k), in batch order."""
    import concurrent.futures as cf
    from simdgraphprocessing_gb300 import workloads as W
    specs = W.batch_specs()
    h = hashlib.sha256()
    tri, clq = [0] * len(specs), [0] * len(specs)

    def one(k):
        kind, s, kw = specs[k]
        g = eh.graph(kind, s, **kw)
        path = os.path.join(td, "batch_%d.bin" % k)
        g.write_binary(path)
        t = int(re.search(APPS["triangles"][1], run_app_threads("undirected_triangle_counting", path, "hybrid",
                                                                1)).group(1))
        c = int(re.search(APPS["cliques4"][1], run_app_threads("n_clique", path, "hybrid", 1)).group(1))
        os.unlink(path)
        off, nbr, _, _ = g.csr()
        return k, t, c, csr_sha(off, nbr)

    shas = [None] * len(specs)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for k, t, c, sha in ex.map(one, range(len(specs))):
            tri[k], clq[k], shas[k] = t, c, sha
            if k % 256 == 0:
                print("batch", k, t, c, flush=True)
    for sha in shas:
        h.update(bytes.fromhex(sha))
    return {"num_graphs": len(specs), "seed": 4, "layout": "hybrid",
            "csr_sha256_of_shas": h.hexdigest(), "triangles": tri, "cliques4": clq,
            "total_triangles": sum(tri), "total_cliques4": sum(clq)}


def main_large():
    threads = os.cpu_count() or 4
    entries = []
    with tempfile.TemporaryDirectory(dir=os.environ.get("EH_GOLDEN_TMP")) as td:
        for spec in LARGE:
            g = large_graph(spec)
            off, nbr, _, _ = g.csr()
            path = os.path.join(td, spec["name"] + ".bin")
            g.write_binary(path)
            e = dict(spec)
            e["n"] = int(len(off) - 1)
            e["directed_edges"] = int(len(nbr))
            e["csr_sha256"] = csr_sha(off, nbr)
            del g, off, nbr
            e["counts"] = {}
            for key in spec["apps"]:
                binary, pat = APPS[key]
                out = run_app_threads(binary, path, "hybrid", threads)
                e["counts"][key] = int(re.search(pat, out).group(1))
                print(spec["name"], key, e["counts"][key], flush=True)
            os.unlink(path)
            entries.append(e)
        batch = batch_reference_counts(td, threads)
    doc = {
        "generated_by": "tests/golden/make_golden.py --large",
        "reference_binaries": "oracle/build_ref.sh (unmodified reference sources), hybrid layout",
        "graphs": entries,
        "batch": batch,
    }
    with open(OUT_LARGE, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)
    print("wrote", OUT_LARGE)


def main():
    if not os.path.exists(os.path.join(REF, "ref_rowdump")):
        sys.exit("oracle/_ref is not built; run: sh oracle/build_ref.sh <reference tree>")
    eh.load()
    if "--directed" in sys.argv:
        return main_directed()
    if "--large" in sys.argv:
        return main_large()
    entries = []
    with tempfile.TemporaryDirectory() as td:
        for spec in GRAPHS:
            g = eh.graph(spec["kind"], spec["seed"], **spec["params"])
            off, nbr, _, _ = g.csr()
            path = os.path.join(td, spec["name"] + ".bin")
            g.write_binary(path)
            e = dict(spec)
            e["n"] = int(len(off) - 1)
            e["directed_edges"] = int(len(nbr))
            e["csr_sha256"] = csr_sha(off, nbr)
            e["counts"] = {}
            for layout in LAYOUTS:
                c = {}
                for key, (binary, pat) in APPS.items():
                    m = re.search(pat, run_app(binary, path, layout))
                    c[key] = int(m.group(1))
                e["counts"][layout] = c
            e["rows_sha256"] = {}
            for layout in LAYOUTS:
                for sel in ("lower", "all"):
                    dump = os.path.join(td, "rows.bin")
                    subprocess.run([os.path.join(REF, "ref_rowdump"), path, layout, sel, dump],
                                   check=True, stdout=subprocess.DEVNULL)
                    with open(dump, "rb") as f:
                        e["rows_sha256"]["%s/%s" % (layout, sel)] = hashlib.sha256(f.read()).hexdigest()
            print(spec["name"], e["counts"]["hybrid"], flush=True)
            entries.append(e)
    doc = {
        "generated_by": "tests/golden/make_golden.py",
        "reference_binaries": "oracle/build_ref.sh (unmodified reference sources)",
        "reference_gtest_goldens": {
            "source": "reference test/*.cpp on test/data/facebook.bin (hybrid layout, 4 threads)",
            "triangles": 1612010, "cliques4": 30004668, "lollipops": 713455740, "similar_nodes": 904,
        },
        "graphs": entries,
    }
    with open(OUT, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
