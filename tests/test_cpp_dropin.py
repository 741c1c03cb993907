"""The drop-in C++ host API (simdgraphprocessing_gb300/host + apps).

CPU: the reference's own gtest sources for the hot path compile unmodified
against the drop-in headers (with EH_REFERENCE naming the reference tree).
GPU: the reference's seven gtests restated without gtest (tests/cpp/
dropin_gtests.cpp: same loaders, Parser arguments, app classes and expected
values) run on the reference's own test graphs (committed under tests/golden/),
and a C++ driver that uses the app classes the same way reproduces the
reference binaries' counts on the seeded fixture graphs.
"""
import os
import subprocess
import sys

import pytest

import _golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "simdgraphprocessing_gb300", "host")
APPS = os.path.join(ROOT, "simdgraphprocessing_gb300", "apps")
CUDA_INC = "/usr/local/cuda/include"
REF_TESTS = ["undirected_triangle_counting_test", "n_clique_test", "undirected_lollipop_counting_test",
             "similar_nodes_test", "symbiosity_test", "n_path_test"]


@pytest.mark.skipif(_golden.reference_file("test") is None,
                    reason="EH_REFERENCE does not name the reference tree")
@pytest.mark.parametrize("name", REF_TESTS)
def test_reference_gtests_compile_against_dropin_headers(name):
    ref = _golden.REFERENCE_TREE
    cmd = ["g++", "-std=c++11", "-fsyntax-only", "-fopenmp", "-DGOOGLE_TEST", "-I", HOST, "-I", APPS,
           "-I", os.path.join(ref, "lib", "gtest-1.7.0", "include"), "-I", CUDA_INC,
           os.path.join(ref, "test", name + ".cpp")]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-3000:]


def _build_driver(tmp_path, eh, name="dropin_apps"):
    exe = str(tmp_path / name)
    libdir = os.path.dirname(eh.lib_path())
    cmd = ["g++", "-std=c++11", "-O2", "-fopenmp", "-I", HOST, "-I", APPS, "-I", CUDA_INC,
           os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-o", exe,
           "-L", libdir, "-leh_gb300", "-Wl,-rpath," + libdir, "-L/usr/local/cuda/lib64", "-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-3000:]
    return exe


def test_host_set_ops(tmp_path):
    """ops::set_intersect / set_union / set_difference of the drop-in headers
    (host-side compat for code that combines rows read back with get_row)."""
    exe = str(tmp_path / "set_ops")
    cmd = ["g++", "-std=c++11", "-O1", "-fopenmp", "-I", HOST, "-I", CUDA_INC,
           os.path.join(ROOT, "tests", "cpp", "set_ops.cpp"), "-o", exe]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-3000:]
    out = subprocess.run([exe], stdout=subprocess.PIPE, text=True, check=True).stdout
    got = {l.split()[0]: [int(x) for x in l.split()[1:]] for l in out.splitlines()}
    both = [5, 9, 127, 70001]
    for k in ("uu", "up", "pb", "bb", "pp"):
        assert got[k] == [len(both)] + both, k
    assert got["pp_full"] == [1, 70000]       # the shared full 2^16 block counts 0 (u16)
    assert got["up_full"][0] == 65537          # mixed layouts count it
    assert got["diff"] == [3, 6, 128, 90000]  # bits set by the second union only


def test_dropin_driver_compiles(tmp_path, eh):
    _build_driver(tmp_path, eh)
    _build_driver(tmp_path, eh, "dropin_directed")
    _build_driver(tmp_path, eh, "dropin_gtests")


@pytest.mark.gpu
def test_reference_gtests_on_gpu(tmp_path, eh):
    """The reference's gtest goldens (1,612,010 triangles; 30,004,668
    4-cliques; 713,455,740 lollipops; 904 similar nodes; symbiosity 0 directed
    and 4,039 undirected; BFS path length 4) from the GPU through the drop-in
    C++ API."""
    exe = _build_driver(tmp_path, eh, "dropin_gtests")
    for name in _golden.FACEBOOK:
        _golden.fixture_graph(name, tmp_path)
    r = subprocess.run([exe, str(tmp_path)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "7 of 7 passed" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("layout", ["hybrid", "uint", "bs", "pshort"])
def test_dropin_directed_apps_reproduce_reference(tmp_path, eh, layout):
    exe = _build_driver(tmp_path, eh, "dropin_directed")
    doc = _golden.load_directed()
    start, depth = doc["n_path_start"], doc["n_path_depth"]
    for spec in doc["graphs"]:
        g = eh.graph(spec["kind"], spec["seed"], **spec["params"])
        assert _golden.directed_sha(g) == spec["sha256"]
        path = str(tmp_path / (spec["name"] + ".bin"))
        directed = not spec.get("undirected", False)
        if directed:
            g.write_directed_binary(path)
        else:
            g.write_binary(path)
        want = spec["counts"][layout]
        args = [exe, path, layout, str(int(directed)), str(want["symbiosity"]), str(want["n_path"]), str(start),
                str(depth), str(want["n_path_s%d_d%d" % (start, depth)])]
        r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, (spec["name"], r.stdout[-2000:])
        assert "Start node - External: %d Internal: %d" % (want["n_path_start"], want["n_path_start"]) in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("layout", ["hybrid", "uint", "bs", "pshort"])
def test_dropin_apps_reproduce_reference_counts(tmp_path, eh, layout):
    exe = _build_driver(tmp_path, eh)
    for spec in _golden.graphs()[:6]:
        off, nbr = _golden.generate(eh, spec)
        path = str(tmp_path / (spec["name"] + ".bin"))
        eh.HostGraph.from_csr(off, nbr).write_binary(path)
        want = spec["counts"][layout]
        args = [exe, path, layout] + [str(want[k]) for k in ("triangles", "cliques4", "lollipops",
                                                             "similar_nodes")]
        r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, (spec["name"], r.stdout[-2000:])
        assert "Number of triangles: %d" % want["triangles"] in r.stdout
