#!/usr/bin/env python3
"""Benchmark of the set-intersection pattern engine on GB300.

Workload (the metric's headline configuration): undirected triangle counting
with the hybrid per-set layout optimizer on a seeded R-MAT graph, scale 22,
edge factor 16 (67,108,864 distinct undirected edges after dedup and self-loop
removal; a=0.57, b=0.19, c=0.19, seed 2), degree-ordered, nbr < node pruning,
u32 ids, u64 count.

One step = one triangle-count pass over the encoded graph.  `value` is pruned
edges per second with the encoded graph resident in HBM (count phase only, as
the reference's own "Time[UNDIRECTED TRIANGLE COUNTING]" timer measures).
`e2e` (the median of its timed passes) runs the same pass through the C ABI
from pinned host CSR buffers: upload,
device select/optimize/encode, the plan with the work shape tuned for a matrix
built and counted once (eh_matrix_tune_for, counts_per_build = 1), count, and
the u64 result copied back.  `value` uses the shape tuned for a resident matrix
(eh_matrix_tune): a larger dense core that saves count time but costs more to
build than a single count saves.

--impl reference times the reference's algorithm on the host cores instead: the
C oracle port (oracle/eh_oracle.c) over the same graph, regenerated on the CPU by
oracle/eh_gen.c (the GPU library is not loaded), the whole graph counted in
every step.  The reference's own sources use x86 SSE/AVX and do not build on the
aarch64 host of the GPU machine.

Multi-GPU: every rank counts its own replica of the graph (the count does not
need an exchange); value = total edges over all ranks / slowest rank's time.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
NOMINAL_HBM_GBS = 7900.0  # GB300 HBM3e nominal; the roofline's `peak` is the measured copy bandwidth
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 256 << 20


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--scale", type=int, default=22)
    p.add_argument("--edge-factor", type=int, default=16)
    p.add_argument("--edges", type=int, default=0,
                   help="exact undirected edge count (overrides the edge factor; e.g. the uint workload: "
                        "--scale 16 --edges 1000000 --seed 1 --layout uint)")
    p.add_argument("--seed", type=int, default=2)
    p.add_argument("--layout", default="hybrid")
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--profile", action="store_true", help="minimal run for ncu captures")
    p.add_argument("--workload", default="triangles", choices=["triangles", "cliques", "batch", "serve", "paths"],
                   help="triangles: the headline; cliques: 4-clique + lollipop on R-MAT s20 and the "
                        "planted-clique graph; batch: 4,096 graphs in one launch vs one launch per graph; "
                        "serve: Poisson query stream against 32 resident graphs; paths: symbiosity and "
                        "n_path BFS on a directed R-MAT graph")
    p.add_argument("--graphs", type=int, default=0, help="batch / serve: number of graphs (0 = configured)")
    p.add_argument("--queries", type=int, default=400, help="serve: queries in the stream")
    p.add_argument("--slots", type=int, default=8, help="serve: concurrent queries on the device")
    return p.parse_args()


def cpu_model():
    """The host CPU as /proc/cpuinfo names it (x86: model name; Arm: implementer / part)."""
    import platform
    fields = {}
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                fields.setdefault(k.strip(), v.strip())
    except OSError:
        pass
    if "model name" in fields:
        return fields["model name"]
    part = fields.get("CPU part")
    names = {"0xd4f": "Neoverse V2 (Grace)", "0xd40": "Neoverse V1", "0xd0c": "Neoverse N1"}
    if part:
        return "%s %s (implementer %s, part %s)" % (platform.machine(), names.get(part, "Arm core"),
                                                     fields.get("CPU implementer", "?"), part)
    return platform.machine()


def edge_count(a):
    return a.edges if a.edges else a.edge_factor << a.scale


def workload(a, world=1):
    """The config object, identical for both arms of the same run."""
    size = ("%d edges" % a.edges) if a.edges else ("edge factor %d" % a.edge_factor)
    return {
        "workload": "undirected triangle count, R-MAT scale %d %s (a=.57,b=.19,c=.19), "
                    "seed %d, %s layout, degree-ordered, nbr<node pruning" % (a.scale, size, a.seed, a.layout),
        "graph": "rmat", "scale": a.scale, "undirected_edges": edge_count(a), "seed": a.seed,
        "layout": a.layout,
        "l2": "GPU: a 256 MiB L2 flush is written before every timed step (and the encoded rows are larger "
              "than the 129 MB L2 at scale 22)",
        "parallelism": "replicas" if world > 1 else "single GPU",
    }


def fixture_counts():
    """Reference-binary counts of the benchmark graphs (tests/golden/reference_large.json),
    keyed by graph name, with the CSR SHA-256 they were made on."""
    try:
        with open(os.path.join(ROOT, "tests", "golden", "reference_large.json")) as f:
            return {g["name"]: g for g in json.load(f)["graphs"]}
    except (OSError, ValueError, KeyError):
        return {}


def fixture_for(a):
    name = "rmat_s%d_ef%d_seed%d" % (a.scale, edge_count(a) >> a.scale, a.seed)
    g = fixture_counts().get(name)
    return g if g and g["params"]["edges"] == edge_count(a) else None


def csr_sha(off, nbr):
    import hashlib
    h = hashlib.sha256()
    h.update(off.astype("<u8").tobytes())
    h.update(nbr.astype("<u4").tobytes())
    return h.hexdigest()


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_launch(work):
    """DRAM bytes (read + write) per launch of the count kernel from the committed
    ncu summary for this workload, or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        key = "rmat_s%d_ef%d_seed%d_%s" % (work["scale"], work["undirected_edges"] >> work["scale"],
                                            work["seed"], work["layout"])
        return t[key]["dram_bytes_per_launch"]
    except Exception:
        return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, device=None):
    """Max of a float over all ranks of the default process group (identity when
    torch.distributed is not initialised).  Works with nccl (device tensor) and
    gloo (host tensor)."""
    import torch
    import torch.distributed as tdist
    if not (tdist.is_available() and tdist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def aggregate(units_per_rank, ms_per_rank, world, device=None):
    """Whole-job throughput of replicas: every rank processed units_per_rank units;
    the job takes as long as the slowest rank."""
    ms = max_over_ranks(ms_per_rank, device)
    return world * units_per_rank / (ms / 1e3), ms


def make_graph(a):
    import simdgraphprocessing_gb300 as eh
    g = eh.graph("rmat", a.seed, scale=a.scale, edges=edge_count(a))
    off, nbr, _, _ = g.csr()
    return off, nbr


def cpu_count(off, nbr, layout, max_seconds=20.0):
    """Oracle port of the reference's triangle count on all host cores.  Returns
    (edges/s, seconds, threads, sample description, count or None, build seconds)."""
    from oracle import oracle as O
    t = time.perf_counter()
    m = O.Matrix(off, nbr, O.SELECT_LOWER, O.LAYOUTS[layout])
    tb = time.perf_counter() - t
    _, cards, _ = m.row_meta()
    threads = O.lib().oracle_max_threads()
    n = len(off) - 1
    # Calibrate on a 1/64 strided sample, then take the full graph if it fits the budget.
    lo_hi = (0, n)
    t = time.perf_counter()
    m.triangles_range(0, n // 64)
    est = (time.perf_counter() - t) * 64
    if est <= max_seconds:
        # Median of up to 5 full passes (while they fit the time budget).
        times, c, spent = [], None, 0.0
        while len(times) < 5 and (not times or spent + times[-1] <= max_seconds):
            t = time.perf_counter()
            c = m.triangles()
            times.append(time.perf_counter() - t)
            spent += times[-1]
        dt = statistics.median(times)
        return (float(cards.sum()) / dt, dt, threads, "full graph, median of %d passes" % len(times), c, tb)
    hi = max(1, int(n * max_seconds / est))
    lo_hi = (0, hi)
    t = time.perf_counter()
    m.triangles_range(*lo_hi)
    dt = time.perf_counter() - t
    return float(cards[:hi].sum()) / dt, dt, threads, "rows [0, %d) of %d, one pass" % lo_hi, None, tb


def run_reference(a, rank, world):
    """The reference's triangle count (the C oracle port of apps/
    undirected_triangle_counting.cpp, OpenMP over all host cores) on the whole
    graph in every step.  The graph comes from oracle/eh_gen.c, the CPU copy of
    the library's generator, and is checked against the reference-binary
    fixture's CSR SHA-256 and count when one exists for the configuration."""
    work = workload(a, world)
    if rank != 0:
        return
    from oracle import oracle as O
    t = time.perf_counter()
    off, nbr = O.rmat_graph(a.scale, edge_count(a), a.seed)
    t_gen = time.perf_counter() - t
    fx = fixture_for(a)
    if fx and csr_sha(off, nbr) != fx["csr_sha256"]:
        raise SystemExit("regenerated graph differs from the fixture graph %s" % fx["name"])
    t = time.perf_counter()
    m = O.Matrix(off, nbr, O.SELECT_LOWER, O.LAYOUTS[a.layout])
    t_build = time.perf_counter() - t
    _, cards, _ = m.row_meta()
    threads = O.lib().oracle_max_threads()
    edges = float(cards.sum())
    count = None
    for _ in range(a.warmup):
        count = m.triangles()
    times = []
    for _ in range(a.steps):
        t = time.perf_counter()
        c = m.triangles()
        times.append(time.perf_counter() - t)
        if count is not None and c != count:
            raise SystemExit("nondeterministic CPU count: %d vs %d" % (c, count))
        count = c
    if fx and count != fx["counts"]["triangles"]:
        raise SystemExit("CPU count %d differs from the reference binary's %d" % (count, fx["counts"]["triangles"]))
    ms = 1e3 * statistics.mean(times)
    value = edges / (ms / 1e3)
    sample = "full graph per step (%d pruned edges), mean of %d steps" % (edges, len(times))
    out = {
        "impl": "reference", "metric": "triangle-count edges/s (pruned undirected edges per second)",
        "value": value, "unit": "edges/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded R-MAT generator)", "config": work,
        "cpu_baseline": {"value": value, "unit": "edges/s", "cores": threads, "kind": "port",
                         "cpu": cpu_model(),
                         "sample": sample + "; C oracle port of the reference algorithm (OpenMP)"},
        "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "count": count,
        "count_matches_reference_binary": (count == fx["counts"]["triangles"]) if fx else None,
        "setup_s": {"generate": t_gen, "build": t_build},
    }
    print(json.dumps(out), flush=True)


def run_ours(a, rank, world, local_rank):
    import torch
    import simdgraphprocessing_gb300 as eh
    dist = world > 1
    torch.cuda.set_device(local_rank)
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    work = workload(a, world)
    L = eh.load()
    off, nbr = make_graph(a)
    stream = torch.cuda.current_stream()
    st = eh._stream(stream)
    m = eh.Matrix.build(off, nbr, "lower", a.layout, stream=stream)
    # Autotuned work shapes (cached for later builds): one for a matrix built and
    # counted once (the e2e passes), then the one for a resident matrix counted
    # many times (the timed counts), which stays applied to m.
    shape1 = m.tune(stream=stream, counts_per_build=1) if not (a.profile or a.no_e2e) else None
    shape = m.tune(stream=stream) if not a.profile else None
    info = m.info()
    pruned = info["cardinality"]
    btc = m.triangle_bytes()
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    count_ref = m.count_triangles(stream=stream)

    def step():
        check_status = L.eh_count_triangles_async(m.h, C.c_void_p(out.data_ptr()), st)
        if check_status:
            eh.check(check_status)

    for w in range(max(a.warmup, 0)):
        flush.fill_(w & 0xff)
        step()
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    sampler = ClockSampler(local_rank) if rank == 0 else None
    if sampler:
        time.sleep(0.5)  # let nvidia-smi start sampling before the timed region
    events = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(a.steps):
        flush.fill_(k & 0xff)  # 256 MiB write between steps: nothing of the last step stays in L2
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        events.append((e0, e1))
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    wall = time.perf_counter() - t0
    clocks = sampler.stop() if sampler else None
    times = [e0.elapsed_time(e1) for e0, e1 in events]
    ms = statistics.mean(times)
    count = int(out.item())
    if count != count_ref:
        raise SystemExit("nondeterministic count: %d vs %d" % (count, count_ref))
    fx0 = fixture_for(a)
    if fx0 and count != fx0["counts"]["triangles"]:
        raise SystemExit("GPU count %d differs from the reference binary's %d on %s"
                         % (count, fx0["counts"]["triangles"], fx0["name"]))
    value, ms_max = aggregate(pruned, ms, world, "cuda")

    # End to end through the C ABI from pinned host buffers.  The passes stand
    # alone: the resident matrix of the timed counts (and its dense core) is
    # released first.
    del m
    torch.cuda.synchronize()
    e2e = None
    if not a.no_e2e and not a.profile:
        h_off = torch.from_numpy(off.view("int64")).pin_memory()
        h_nbr = torch.from_numpy(nbr.view("int32")).pin_memory()
        e2e_times, e2e_phases = [], []
        t1 = eh.Tuning(**{k: shape1[k] for k in ("light_max", "unit_span", "ctas_per_sm", "core_rows",
                                                 "core_hot_words", "core_filter_words")})
        torch.cuda.synchronize()
        e2e_warm = 2  # untimed passes: the first maps the library's memory pools
        for k in range(a.e2e_steps + e2e_warm):
            flush.fill_(k & 0xff)
            torch.cuda.synchronize()
            t = time.perf_counter()
            h = C.c_void_p()
            eh.check(L.eh_matrix_build(len(off) - 1, C.c_void_p(h_off.data_ptr()), C.c_void_p(h_nbr.data_ptr()),
                                       None, eh.SELECT_LOWER, eh.LAYOUTS[a.layout], st, C.byref(h)))
            tb = time.perf_counter()  # each call below returns after its work is done
            eh.check(L.eh_matrix_set_shape(h, C.byref(t1), st))
            tp = time.perf_counter()
            c = C.c_uint64()
            eh.check(L.eh_count_triangles(h, C.byref(c), st))
            dt = time.perf_counter() - t
            L.eh_matrix_free(h)  # outside the timed region, as a caller frees a matrix it is done with
            if c.value != count_ref:
                raise SystemExit("e2e count mismatch %d vs %d" % (c.value, count_ref))
            if k >= e2e_warm:
                e2e_times.append(dt)
                e2e_phases.append((tb - t, tp - tb, t + dt - tp))
        # The median pass: on a box whose previous job has just ended, the first
        # passes of a process have been seen to take up to 20x longer (host or
        # driver work outside this process); every pass is listed in step_ms.
        e2e_value, e2e_ms = aggregate(pruned, 1e3 * statistics.median(e2e_times), world, "cuda")
        e2e = {"value": e2e_value, "unit": "edges/s",
               "h2d_bytes_per_step": int(off.nbytes + nbr.nbytes), "d2h_bytes_per_step": 8,
               "ms_per_step": e2e_ms, "steps": len(e2e_times), "statistic": "median of the timed passes",
               "mean_ms": 1e3 * statistics.mean(e2e_times),
               "includes": "pinned H2D of the full symmetric CSR, device select/optimize/encode/plan, "
                           "triangle count, u64 result D2H",
               "work_shape": shape1,
               "step_ms": [round(1e3 * x, 3) for x in e2e_times],
               "step_phase_ms": [[round(1e3 * x, 3) for x in p] for p in e2e_phases],
               "phase_ms_median": {k: round(1e3 * statistics.median(p[i] for p in e2e_phases), 3)
                                   for i, k in enumerate(("build", "plan", "count"))}}

    if rank != 0:
        if dist:
            tdist.destroy_process_group()
        return
    peak, peak_kind = measured_peak()
    # A count launches the heavy-pivot kernel when some row is longer than the
    # light-pivot limit and the light-pivot kernel when some row is not.
    light_max = (shape or {}).get("light_max", 96)
    kernels_per_count = 1 + (info["max_row_cardinality"] > light_max)
    traffic = traffic_per_launch(work)
    fx = fixture_for(a)
    cpu = None
    if not a.no_cpu and not a.profile and world == 1:
        v, dt, threads, sample, ccount, tb = cpu_count(off, nbr, a.layout)
        cpu = {"value": v, "unit": "edges/s", "cores": threads, "kind": "port", "cpu": cpu_model(),
               "sample": sample +
               "; C oracle port of the reference algorithm (OpenMP, build %.2f s untimed)" % tb,
               "count_matches_gpu": (ccount == count) if ccount is not None else None}
    # Roofline: the physical HBM figure is the count's DRAM traffic (ncu, the
    # two pivot kernels of one count) over the event-timed count.  The
    # algorithmic bytes B_tc charge every neighbour row in full per edge while
    # the kernels probe words of it (much of it from L2), so B_tc / time is an
    # effective bandwidth above what HBM can deliver, reported beside it.
    algo_gbs = btc / (ms / 1e3) / 1e9
    dram_gbs = (traffic / (ms / 1e3) / 1e9) if traffic else None
    roofline = {"bound": "hbm", "achieved": dram_gbs, "peak": peak, "unit": "GB/s",
                "frac": (dram_gbs / peak) if dram_gbs else None, "traffic": traffic, "peak_kind": peak_kind,
                "achieved_basis": "ncu DRAM bytes (read + write) of one count's kernels / CUDA-event count time",
                "nominal_gbs": NOMINAL_HBM_GBS,
                "frac_of_nominal": (dram_gbs / NOMINAL_HBM_GBS) if dram_gbs else None,
                "algorithmic_bytes_per_launch": btc,
                "algorithmic_formula": "sum_i [8 + bytes(A_i)] + sum_{(i,j) in E<} bytes(B_j), bytes = layout "
                                       "payload (every neighbour row charged in full per edge)",
                "effective_gbs": algo_gbs,
                "effective_note": "algorithmic bytes / count time: an effective bandwidth, not an HBM fraction "
                                  "(the kernels read words of the rows, many from L2)"}
    res = {
        "metric": "triangle-count edges/s (pruned undirected edges per second)",
        "value": value, "unit": "edges/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded R-MAT generator)",
        "config": work,
        "work_shape": shape,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clocks,
        "gpu_launches": a.steps * kernels_per_count,
        "count": count,
        "count_matches_reference_binary": (count == fx["counts"]["triangles"]) if fx else None,
        "wall_s_timed_region": wall,
        "graph": {"vertices": info["matrix_size"], "pruned_edges": pruned,
                  "bitset_rows": info["num_bitset_rows"], "uint_rows": info["num_uint_rows"],
                  "row_bytes": info["row_total_bytes_used"], "device_bytes": info["device_bytes"]},
    }
    print(json.dumps(res), flush=True)
    if dist:
        tdist.destroy_process_group()


def _events_ms(fn, stream, reps, flush=None):
    import torch
    ts = []
    for r in range(reps):
        if flush is not None:
            flush.fill_(r & 0xff)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return ts


def run_cliques(a):
    """4-clique and lollipop counts on R-MAT scale 20 ef16 seed 3 and on the
    planted-clique graph (2^20 vertices, G(n, M) background with p = 1e-4, 1,024
    cliques of 64..512 vertices)."""
    import torch
    import simdgraphprocessing_gb300 as eh
    from simdgraphprocessing_gb300 import workloads as W
    from oracle import oracle as O
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    lines = []
    for name, g in (("rmat_s20_ef16_seed3", eh.graph("rmat", 3, scale=20, edges=16 << 20)),
                    ("planted_2^20_p1e-4_1024cliques_seed3", W.planted_graph(3))):
        off, nbr = g.csr()[:2]
        low = eh.Matrix.build(off, nbr, "lower", a.layout, stream=stream)
        full = eh.Matrix.build(off, nbr, "all", a.layout, stream=stream)
        # Work shapes: the pruned matrix tuned on triangles (its dense core also
        # serves the clique kernels), the full one on lollipops.
        low.tune(stream=stream)
        full.tune(stream=stream)
        res = {"graph": name, "pruned_edges": low.info()["cardinality"], "layout": a.layout,
               "bitset_rows_lower": low.info()["num_bitset_rows"]}
        c4 = low.count_cliques(4, stream=stream)
        t4 = _events_ms(lambda: low.count_cliques_async(4, out.data_ptr(), stream.cuda_stream), stream, a.steps, flush)
        lp = full.count_lollipops(stream=stream)
        tl = _events_ms(lambda: full.count_lollipops_async(out.data_ptr(), stream.cuda_stream), stream, a.steps, flush)
        res.update({"cliques4": c4, "cliques4_ms": statistics.median(t4[a.warmup:] or t4),
                    "lollipops": lp, "lollipops_ms": statistics.median(tl[a.warmup:] or tl)})
        fx = fixture_counts().get(name)
        if fx and a.layout in ("hybrid", "uint", "bs", "pshort", "hybrid3"):
            if csr_sha(off, nbr) != fx["csr_sha256"]:
                raise SystemExit("generated graph differs from the fixture graph %s" % name)
            res["cliques4_matches_reference_binary"] = c4 == fx["counts"]["cliques4"]
            res["lollipops_match_reference_binary"] = lp == fx["counts"]["lollipops"]
            if c4 != fx["counts"]["cliques4"] or lp != fx["counts"]["lollipops"]:
                print(json.dumps(res), flush=True)
                raise SystemExit("count differs from the reference binary on %s" % name)
        if not a.no_cpu:
            t = time.perf_counter()
            om = O.Matrix(off, nbr, O.SELECT_LOWER, O.LAYOUTS[a.layout])
            t = time.perf_counter()
            oc4 = om.cliques(4)
            res["cpu_cliques4_s"] = time.perf_counter() - t
            res["cliques4_matches_cpu"] = oc4 == c4
            of = O.Matrix(off, nbr, O.SELECT_ALL, O.LAYOUTS[a.layout])
            t = time.perf_counter()
            olp = of.lollipops()
            res["cpu_lollipops_s"] = time.perf_counter() - t
            res["lollipops_match_cpu"] = olp == lp
            res["cpu_threads"] = O.lib().oracle_max_threads()
        lines.append(res)
    print(json.dumps({"workload": "cliques", "metric": "4-clique / lollipop count time", "unit": "ms",
                      "higher_is_better": False, "data": "synthetic (seeded generators)", "results": lines}),
          flush=True)


def run_paths(a):
    """symbiosity and the n_path BFS on a directed R-MAT graph: scale 22, the
    first 64M distinct ordered pairs (edge factor 16), seed 5; BFS from the
    largest row with no depth limit."""
    import torch
    import simdgraphprocessing_gb300 as eh
    from oracle import oracle as O
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    t = time.perf_counter()
    g = eh.HostGraph.directed_rmat(a.scale, a.edge_factor << a.scale, 5)
    off, nbr, _, _ = g.csr()
    ioff, inbr = g.in_csr()
    t_gen = time.perf_counter() - t
    rows = eh.Matrix.build(off, nbr, "all", a.layout, stream=stream)
    cols = eh.Matrix.build(ioff, inbr, "all", a.layout, stream=stream)
    res = {"graph": "directed_rmat_s%d_ef%d_seed5" % (a.scale, a.edge_factor), "vertices": len(off) - 1,
           "out_entries": int(len(nbr)), "layout": a.layout, "generate_s": t_gen}
    sym = rows.symbiosity(cols, 0.5, stream=stream)
    ts = _events_ms(lambda: rows.symbiosity_async(cols, 0.5, out.data_ptr(), stream.cuda_stream), stream,
                    a.steps + a.warmup, flush)
    res.update({"symbiosity": sym, "symbiosity_ms": statistics.median(ts[a.warmup:])})
    start = rows.max_row_id()
    path, reached = rows.bfs(start, stream=stream)
    tb = []
    for r in range(a.steps + a.warmup):
        flush.fill_(r & 0xff)
        torch.cuda.synchronize()
        t = time.perf_counter()
        rows.bfs(start, stream=stream)
        tb.append((time.perf_counter() - t) * 1e3)
    res.update({"bfs_start": start, "n_path": path, "bfs_reached": reached,
                "bfs_ms": statistics.median(tb[a.warmup:]), "bfs_timing": "host wall clock per call (the call "
                "synchronises once per 8 levels), L2 flushed before each"})
    if not a.no_cpu:
        orows = O.Matrix(off, nbr, O.SELECT_ALL, O.LAYOUTS[a.layout])
        ocols = O.Matrix(ioff, inbr, O.SELECT_ALL, O.LAYOUTS[a.layout])
        t = time.perf_counter()
        res["symbiosity_matches_cpu"] = orows.symbiosity(ocols) == sym
        res["cpu_symbiosity_s"] = time.perf_counter() - t
        t = time.perf_counter()
        res["bfs_matches_cpu"] = orows.n_path(start) == (path, reached)
        res["cpu_bfs_s"] = time.perf_counter() - t
        res["cpu_threads"] = {"symbiosity": O.lib().oracle_max_threads(), "bfs": 1}
    print(json.dumps({"workload": "paths", "metric": "symbiosity / n_path BFS time", "unit": "ms",
                      "higher_is_better": False, "data": "synthetic (seeded directed R-MAT generator)",
                      "results": [res]}), flush=True)


def run_batch(a):
    """4,096 graphs (half G(n, M), half Barabasi-Albert; n log-uniform in
    [200, 50000]; mean degree uniform in [4, 64]; seeds 4+k): triangles and
    4-cliques of every graph in one persistent launch each, captured in a CUDA
    graph and replayed, with the autotuned work shape, against one launch per
    graph on the same GPU."""
    import torch
    import simdgraphprocessing_gb300 as eh
    from simdgraphprocessing_gb300 import workloads as W
    G = a.graphs or 4096
    t = time.perf_counter()
    csrs, (gr, off, nbr) = W.batch_union(G, 4)
    t_gen = time.perf_counter() - t
    s = torch.cuda.Stream()
    b = eh.Batch(gr, off, nbr, layout=a.layout, stream=s)
    info = b.matrix_info()
    tri = torch.zeros(G, dtype=torch.int64, device="cuda")
    clq = torch.zeros(G, dtype=torch.int64, device="cuda")
    shape = b.tune(stream=s)
    for _ in range(a.warmup):
        b.run(tri.data_ptr(), clq.data_ptr(), use_graph=True, stream=s)
    s.synchronize()
    times = _events_ms(lambda: b.run(tri.data_ptr(), clq.data_ptr(), use_graph=True, stream=s), s, a.steps)
    batched_ms = statistics.median(times)
    bt, bc = tri.cpu().tolist(), clq.cpu().tolist()
    # One launch per graph (each graph its own matrix, counted on its own).
    mats = [eh.Matrix.build(o, n, "lower", a.layout, stream=s) for o, n in csrs]
    pt = torch.zeros(G, dtype=torch.int64, device="cuda")
    pc = torch.zeros(G, dtype=torch.int64, device="cuda")
    L = eh.load()

    def per_graph():
        for g, m in enumerate(mats):
            eh.check(L.eh_count_triangles_async(m.h, C.c_void_p(pt[g:].data_ptr()), C.c_void_p(s.cuda_stream)))
            eh.check(L.eh_count_cliques_async(m.h, 4, C.c_void_p(pc[g:].data_ptr()), C.c_void_p(s.cuda_stream)))

    per_graph()
    s.synchronize()
    ptimes = _events_ms(per_graph, s, max(3, a.steps // 4))
    per_ms = statistics.median(ptimes)
    same = pt.cpu().tolist() == bt and pc.cpu().tolist() == bc
    edges = info["cardinality"]
    fx = None
    try:
        with open(os.path.join(ROOT, "tests", "golden", "reference_large.json")) as f:
            fx = json.load(f)["batch"]
    except (OSError, ValueError, KeyError):
        pass
    ref_match = None
    if fx and G <= fx["num_graphs"]:
        ref_match = bt == fx["triangles"][:G] and bc == fx["cliques4"][:G]
        if not ref_match:
            raise SystemExit("batched counts differ from the reference binaries' per-graph counts")
    print(json.dumps({
        "workload": "batch", "metric": "graphs counted per second (triangles + 4-cliques)", "unit": "graphs/s",
        "value": G / (batched_ms / 1e3), "higher_is_better": True, "n_graphs": G,
        "batched_ms": batched_ms, "per_graph_launch_ms": per_ms, "speedup_vs_per_graph": per_ms / batched_ms,
        "counts_identical": same, "counts_match_reference_binary": ref_match, "pruned_edges": edges, "edges_per_s": edges / (batched_ms / 1e3),
        "total_triangles": int(sum(bt)), "total_cliques4": int(sum(bc)), "tuned_shape": shape,
        "generation_s": t_gen, "data": "synthetic (seeded G(n,M) / Barabasi-Albert generators)",
        "cuda_graph_replay": True}), flush=True)


def run_serve(a):
    """32 device-resident R-MAT graphs (scales 14..23, ef16, seeds 100+k); a
    stream of triangle / 4-clique / similar_nodes queries (uniform mix, uniform
    graph) served with continuous batching under a 150 GB HBM cap.
    1. one at a time: each query alone (the answers for the identity check);
    2. capacity: every query submitted at once, queries/s to drain them;
    3. open-loop Poisson arrivals at 0.5x and 0.8x of that capacity: p50/p99
       latency (submit to result) below saturation.
    Every served answer must equal the same query run alone."""
    import random
    import threading
    import simdgraphprocessing_gb300 as eh
    from simdgraphprocessing_gb300 import workloads as W
    specs = W.serving_specs(a.graphs or 32)
    srv = eh.Server(slots=a.slots, hbm_cap_bytes=150 << 30)
    ids = []
    t = time.perf_counter()
    for scale, seed, ef in specs:
        o, n = eh.graph("rmat", seed, scale=scale, edges=ef << scale).csr()[:2]
        ids.append(srv.add_graph(o, n, a.layout))
    t_load = time.perf_counter() - t
    rnd = random.Random(5)
    kinds = [(eh.QUERY_TRIANGLES, 0), (eh.QUERY_CLIQUES, 4), (eh.QUERY_SIMILAR_NODES, 10)]
    mix = [(rnd.randrange(len(ids)), *kinds[rnd.randrange(3)]) for _ in range(a.queries)]
    alone, alone_ms = [], {}
    t = time.perf_counter()
    for q in mix:
        t1 = time.perf_counter()
        alone.append(srv.run_alone(ids[q[0]], q[1], q[2]))
        key = "%s/s%d" % (("triangles", "cliques4", "similar")[q[1]], specs[q[0]][0])
        alone_ms.setdefault(key, []).append(1e3 * (time.perf_counter() - t1))
    serial_s = time.perf_counter() - t
    serial_qps = len(mix) / serial_s

    def served(arrivals):
        tickets = [None] * len(mix)

        def submitter():
            t0 = time.perf_counter()
            for i, q in enumerate(mix):
                d = arrivals[i] - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
                tickets[i] = srv.submit(ids[q[0]], q[1], q[2])

        t0 = time.perf_counter()
        th = threading.Thread(target=submitter)
        th.start()
        th.join()
        res = [srv.wait(tk, timeout_ms=600000) for tk in tickets]
        wall = time.perf_counter() - t0
        lat = sorted((r["done_ns"] - r["submit_ns"]) / 1e6 for r in res)
        wait = sorted((r["start_ns"] - r["submit_ns"]) / 1e6 for r in res)
        pct = lambda v, p: v[min(len(v) - 1, int(p * len(v)))]
        return {"qps": len(mix) / wall, "p50_ms": pct(lat, 0.5), "p99_ms": pct(lat, 0.99),
                "queue_wait_p50_ms": pct(wait, 0.5), "queue_wait_p99_ms": pct(wait, 0.99),
                "identical_to_alone": all(r["count"] == c for r, c in zip(res, alone))}

    capacity = served([0.0] * len(mix))
    loads = {}
    for frac in (0.5, 0.8):
        rate = frac * capacity["qps"]
        arr, tt = [], 0.0
        for _ in mix:
            tt += rnd.expovariate(rate)
            arr.append(tt)
        loads["%.1fx" % frac] = dict(served(arr), arrival_rate_per_s=rate)
    st = srv.stats()
    srv.close()
    # Upper bound of any overlap: the served wall time cannot drop below the
    # largest single query, nor below the queries that each fill the GPU.
    longest = max(max(v) for v in alone_ms.values())
    same = capacity["identical_to_alone"] and all(v["identical_to_alone"] for v in loads.values())
    print(json.dumps({
        "workload": "serve", "metric": "queries/s at capacity, p50/p99 latency at 0.5x and 0.8x of capacity",
        "unit": "queries/s", "value": capacity["qps"], "higher_is_better": True,
        "queries": len(mix), "slots": a.slots, "one_at_a_time_qps": serial_qps,
        "speedup_vs_one_at_a_time": capacity["qps"] / serial_qps, "capacity": capacity, "latency": loads,
        "results_identical_alone_and_in_mix": same, "one_at_a_time_s": serial_s,
        "longest_single_query_ms": longest,
        "alone_ms_by_query": {k: [len(v), round(statistics.median(v), 3), round(sum(v), 1)]
                              for k, v in sorted(alone_ms.items())},
        "max_inflight": st["max_inflight"], "resident_bytes": st["resident_bytes"], "hbm_cap_bytes": st["hbm_cap_bytes"],
        "graphs": len(ids), "graph_load_s": t_load, "query_mix": "uniform: triangles / 4-cliques / similar_nodes(10)",
        "data": "synthetic (seeded R-MAT generator)"}), flush=True)
    if not same:
        raise SystemExit("a served answer differs from the same query run alone")


def main():
    a = parse_args()
    if a.workload != "triangles":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        {"cliques": run_cliques, "batch": run_batch, "serve": run_serve, "paths": run_paths}[a.workload](a)
        return
    if a.profile:
        a.warmup, a.steps, a.no_e2e, a.no_cpu = 1, 1, True, True
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(a.gpus if a.gpus == 1 else 1)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank, world)
    else:
        run_ours(a, rank, world, local_rank)


if __name__ == "__main__":
    main()
