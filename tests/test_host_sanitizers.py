"""The host half of the engine (loaders, generators, reordering, directed
graphs: csrc/eh_host.cpp) and the C oracle (oracle/eh_oracle.c) under
AddressSanitizer + UndefinedBehaviorSanitizer, built apart from the CUDA code.
(compute-sanitizer, the device-side counterpart, is not available on the GPU
pool.)"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_host_code_is_clean_under_asan_ubsan(tmp_path):
    exe = str(tmp_path / "host_asan")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fopenmp", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "simdgraphprocessing_gb300", "csrc", "eh_host.cpp"),
           os.path.join(ROOT, "tests", "cpp", "host_asan.cpp"), "-o", exe]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0 and ("cannot find -lasan" in r.stdout or "libasan" in r.stdout):
        pytest.skip("sanitizer runtime not installed")
    assert r.returncode == 0, r.stdout[-3000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", OMP_NUM_THREADS="2")
    r = subprocess.run([exe, str(tmp_path)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-3000:]


def test_oracle_is_clean_under_asan_ubsan(tmp_path):
    exe = str(tmp_path / "oracle_asan")
    cmd = ["gcc", "-std=c99", "-O1", "-g", "-fopenmp", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", os.path.join(ROOT, "oracle", "eh_oracle.c"),
           os.path.join(ROOT, "tests", "cpp", "oracle_asan.c"), "-o", exe]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0 and ("cannot find -lasan" in r.stdout or "libasan" in r.stdout):
        pytest.skip("sanitizer runtime not installed")
    assert r.returncode == 0, r.stdout[-3000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", OMP_NUM_THREADS="2")
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, env=env, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().splitlines()[-1].startswith("ok"), r.stdout[-3000:]


def test_upload_chunk_plan(tmp_path):
    """The split of a host adjacency into uploads (eh::plan_upload_chunks) on
    random degree sequences, with and without bad offsets."""
    exe = str(tmp_path / "upload_chunks")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fopenmp", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "simdgraphprocessing_gb300", "csrc"),
           os.path.join(ROOT, "simdgraphprocessing_gb300", "csrc", "eh_host.cpp"),
           os.path.join(ROOT, "tests", "cpp", "upload_chunks.cpp"), "-o", exe]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0 and ("cannot find -lasan" in r.stdout or "libasan" in r.stdout):
        pytest.skip("sanitizer runtime not installed")
    assert r.returncode == 0, r.stdout[-3000:]
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-3000:]
