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
`e2e` runs the same pass through the C ABI from pinned host CSR buffers: upload,
device select/optimize/encode, count, and the u64 result copied back.

--impl reference times the reference's algorithm on the host cores instead (the
C oracle port; the reference's own sources use x86 SSE/AVX and do not build on
the aarch64 host of the GPU machine).

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
    p.add_argument("--seed", type=int, default=2)
    p.add_argument("--layout", default="hybrid")
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--profile", action="store_true", help="minimal run for ncu captures")
    return p.parse_args()


def workload(a):
    return {
        "workload": "undirected triangle count, R-MAT scale %d edge factor %d (a=.57,b=.19,c=.19), "
                    "seed %d, %s layout, degree-ordered, nbr<node pruning" % (a.scale, a.edge_factor, a.seed, a.layout),
        "graph": "rmat", "scale": a.scale, "undirected_edges": a.edge_factor << a.scale, "seed": a.seed,
        "layout": a.layout,
    }


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


def make_graph(a):
    import simdgraphprocessing_gb300 as eh
    g = eh.graph("rmat", a.seed, scale=a.scale, edges=a.edge_factor << a.scale)
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
        t = time.perf_counter()
        c = m.triangles()
        dt = time.perf_counter() - t
        return float(cards.sum()) / dt, dt, threads, "full graph, one pass", c, tb
    hi = max(1, int(n * max_seconds / est))
    lo_hi = (0, hi)
    t = time.perf_counter()
    m.triangles_range(*lo_hi)
    dt = time.perf_counter() - t
    return float(cards[:hi].sum()) / dt, dt, threads, "rows [0, %d) of %d, one pass" % lo_hi, None, tb


def run_reference(a, rank, world):
    work = workload(a)
    if rank != 0:
        return
    off, nbr = make_graph(a)
    from oracle import oracle as O
    m = O.Matrix(off, nbr, O.SELECT_LOWER, O.LAYOUTS[a.layout])
    _, cards, _ = m.row_meta()
    threads = O.lib().oracle_max_threads()
    total_edges = float(cards.sum())
    n = len(off) - 1
    # Size each step: full graph if one pass takes <= 10 s, else a prefix of rows.
    t = time.perf_counter()
    m.triangles_range(0, n // 64)
    est = (time.perf_counter() - t) * 64
    hi = n if est <= 10.0 else max(1, int(n * 10.0 / est))
    edges = float(cards[:hi].sum())
    for _ in range(a.warmup):
        m.triangles_range(0, hi)
    times = []
    for _ in range(a.steps):
        t = time.perf_counter()
        m.triangles_range(0, hi)
        times.append(time.perf_counter() - t)
    ms = 1e3 * statistics.mean(times)
    value = edges / (ms / 1e3)
    sample = "full graph per step" if hi == n else "rows [0, %d) of %d per step" % (hi, n)
    out = {
        "impl": "reference", "metric": "triangle-count edges/s (pruned undirected edges per second)",
        "value": value, "unit": "edges/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded R-MAT generator)", "config": work,
        "cpu_baseline": {"value": value, "unit": "edges/s", "cores": threads, "kind": "port",
                         "sample": sample + "; C oracle port of the reference algorithm (OpenMP)"},
        "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "pruned_edges_total": total_edges,
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
    work = workload(a)
    L = eh.load()
    off, nbr = make_graph(a)
    stream = torch.cuda.current_stream()
    st = eh._stream(stream)
    m = eh.Matrix.build(off, nbr, "lower", a.layout, stream=stream)
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
    if dist:
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        ms_max = float(t.item())
    else:
        ms_max = ms
    value = world * pruned / (ms_max / 1e3)

    # End to end through the C ABI from pinned host buffers.
    e2e = None
    if not a.no_e2e and not a.profile:
        h_off = torch.from_numpy(off.view("int64")).pin_memory()
        h_nbr = torch.from_numpy(nbr.view("int32")).pin_memory()
        res = torch.zeros(1, dtype=torch.int64).pin_memory()
        keep = []
        e2e_times = []
        torch.cuda.synchronize()
        for k in range(a.e2e_steps + 1):
            flush.fill_(k & 0xff)
            torch.cuda.synchronize()
            t = time.perf_counter()
            h = C.c_void_p()
            eh.check(L.eh_matrix_build(len(off) - 1, C.c_void_p(h_off.data_ptr()), C.c_void_p(h_nbr.data_ptr()),
                                       None, eh.SELECT_LOWER, eh.LAYOUTS[a.layout], st, C.byref(h)))
            c = C.c_uint64()
            eh.check(L.eh_count_triangles(h, C.byref(c), st))
            dt = time.perf_counter() - t
            keep.append(h)
            if c.value != count_ref:
                raise SystemExit("e2e count mismatch %d vs %d" % (c.value, count_ref))
            if k > 0:  # the first pass warms the allocator pools
                e2e_times.append(dt)
        for h in keep:
            L.eh_matrix_free(h)
        e2e_ms = 1e3 * statistics.mean(e2e_times)
        if dist:
            t = torch.tensor([e2e_ms], dtype=torch.float64, device="cuda")
            tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
            e2e_ms = float(t.item())
        e2e = {"value": world * pruned / (e2e_ms / 1e3), "unit": "edges/s",
               "h2d_bytes_per_step": int(off.nbytes + nbr.nbytes), "d2h_bytes_per_step": 8,
               "ms_per_step": e2e_ms, "steps": len(e2e_times),
               "includes": "pinned H2D of the full symmetric CSR, device select/optimize/encode/plan, "
                           "triangle count, u64 result D2H"}

    if rank != 0:
        if dist:
            tdist.destroy_process_group()
        return
    peak, peak_kind = measured_peak()
    achieved = btc / (ms / 1e3) / 1e9
    traffic = traffic_per_launch(work)
    cpu = None
    if not a.no_cpu and not a.profile and world == 1:
        v, dt, threads, sample, ccount, tb = cpu_count(off, nbr, a.layout)
        cpu = {"value": v, "unit": "edges/s", "cores": threads, "kind": "port", "sample": sample +
               "; C oracle port of the reference algorithm (OpenMP, build %.2f s untimed)" % tb,
               "count_matches_gpu": (ccount == count) if ccount is not None else None}
    res = {
        "metric": "triangle-count edges/s (pruned undirected edges per second)",
        "value": value, "unit": "edges/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded R-MAT generator)",
        "config": dict(work, l2="256 MiB L2 flush written before every timed step; encoded rows "
                                "%.0f MB > 129 MB L2" % (info["row_total_bytes_used"] / 1e6),
                       parallelism="replicas" if world > 1 else "single GPU"),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": btc,
                     "formula": "sum_i [8 + bytes(A_i)] + sum_{(i,j) in E<} bytes(B_j), bytes = layout payload"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clocks,
        "gpu_launches": a.steps,
        "count": count,
        "wall_s_timed_region": wall,
        "graph": {"vertices": info["matrix_size"], "pruned_edges": pruned,
                  "bitset_rows": info["num_bitset_rows"], "uint_rows": info["num_uint_rows"],
                  "row_bytes": info["row_total_bytes_used"], "device_bytes": info["device_bytes"]},
    }
    print(json.dumps(res), flush=True)
    if dist:
        tdist.destroy_process_group()


def main():
    a = parse_args()
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
