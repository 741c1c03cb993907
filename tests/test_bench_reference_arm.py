"""bench.py's reference arm on the host cores (no GPU): the JSON line keeps the
contract's keys, the count it times is the oracle's, and the CPU it ran on is
named."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "12",
                        "--edges", "40000", "--steps", "2", "--warmup", "1"],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["cpu"]
    assert cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0


def test_cpu_model_names_the_host():
    sys.path.insert(0, ROOT)
    import bench
    name = bench.cpu_model()
    assert isinstance(name, str) and name


def test_reference_arm_never_loads_the_gpu_library():
    """The reference arm regenerates its graph with the oracle's CPU generator:
    neither the product package nor libeh_gb300.so is loaded in that process."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--scale', '10', '--edges', '8000', "
            "'--steps', '1', '--warmup', '1']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "assert 'libeh_gb300' not in maps, 'GPU library mapped'; "
            "assert 'simdgraphprocessing_gb300' not in sys.modules, 'product package imported'; print('clean')")
    r = subprocess.run([sys.executable, "-c", code], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().endswith("clean")


def test_headline_config_has_a_reference_binary_fixture():
    """Both arms build `config` with bench.workload (nothing run-specific in it),
    and the headline graph has the reference binary's count to check against."""
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    ns = argparse.Namespace(scale=22, edge_factor=16, edges=0, seed=2, layout="hybrid")
    cfg = bench.workload(ns, 1)
    assert cfg["scale"] == 22 and cfg["undirected_edges"] == 16 << 22 and "work_shape" not in cfg
    fx = bench.fixture_for(ns)
    assert fx is not None and fx["counts"]["triangles"] == 2333984842
