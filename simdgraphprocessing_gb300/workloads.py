"""Seeded synthetic workloads of the benchmark configurations.

The reference measures no public dataset; these generators stand in for the
configurations' graphs.  Parameters are drawn with integer SplitMix64 and plain
IEEE arithmetic (no libm calls) so every host derives the same graphs.

* headline: R-MAT scale 22, edge factor 16, seed 2 (triangles, hybrid layout)
* uint workload: R-MAT scale 16 with 1,000,000 edges, seed 1
* clique / lollipop workloads: R-MAT scale 20 ef16 seed 3, and 2^20 vertices of
  G(n, M) background (M = 1e-4 * n(n-1)/2) with 1,024 planted cliques of
  64..512 vertices
* batch: 4,096 graphs, seeds 4+k, half G(n, M) / half Barabasi-Albert, n
  log-uniform in [200, 50000], mean degree uniform in [4, 64] (BA m = round(d/2))
* serving: 32 R-MAT graphs of scales 14..23 (edge factor 16, seeds 100+k)
"""
import bisect

import numpy as np

from . import HostGraph, concat_graphs, graph

MASK64 = (1 << 64) - 1


def splitmix(x):
    """SplitMix64 output function of state x (Steele, Lea, Flood 2014)."""
    z = (x + 0x9E3779B97F4A7C15) & MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def uniform01(seed, tag):
    return (splitmix((seed * 0x100000001B3 + tag) & MASK64) >> 11) * (1.0 / 9007199254740992.0)


_LOGU = {}


def log_uniform_int(lo, hi, u):
    """Integer in [lo, hi] with P(n) proportional to 1/n (discrete log-uniform)."""
    key = (lo, hi)
    if key not in _LOGU:
        acc, cdf = 0.0, []
        for n in range(lo, hi + 1):
            acc += 1.0 / n
            cdf.append(acc)
        _LOGU[key] = cdf
    cdf = _LOGU[key]
    return lo + min(bisect.bisect_left(cdf, u * cdf[-1]), hi - lo)


def batch_specs(num_graphs=4096, seed=4, n_lo=200, n_hi=50000, d_lo=4.0, d_hi=64.0):
    specs = []
    for k in range(num_graphs):
        s = seed + k
        n = log_uniform_int(n_lo, n_hi, uniform01(s, 1))
        d = d_lo + (d_hi - d_lo) * uniform01(s, 2)
        if k % 2 == 0:
            m = min(int(round(n * d / 2.0)), n * (n - 1) // 2)
            specs.append(("er", s, dict(n=n, edges=m)))
        else:
            specs.append(("ba", s, dict(n=n, m=max(1, int(round(d / 2.0))))))
    return specs


def batch_graphs(num_graphs=4096, seed=4):
    """[(offsets, nbrs)] of the batch configuration, each degree-ordered."""
    out = []
    for kind, s, kw in batch_specs(num_graphs, seed):
        off, nbr = graph(kind, s, **kw).csr()[:2]
        out.append((off, nbr))
    return out


def batch_union(num_graphs=4096, seed=4):
    csrs = batch_graphs(num_graphs, seed)
    return csrs, concat_graphs(csrs)


def serving_specs(num_graphs=32, seed=100, lo=14, hi=23, edge_factor=16):
    return [(lo + (k * (hi - lo + 1)) // num_graphs, seed + k, edge_factor) for k in range(num_graphs)]


def planted_graph(seed=3):
    n = 1 << 20
    m = int(round(1e-4 * n * (n - 1) / 2))
    return HostGraph.planted_cliques(n, m, 1024, 64, 512, seed).reorder_by_degree()


def rmat(scale, edge_factor=16, seed=2, edges=None):
    return graph("rmat", seed, scale=scale, edges=edges if edges is not None else edge_factor << scale)


__all__ = ["batch_specs", "batch_graphs", "batch_union", "serving_specs", "planted_graph", "rmat", "splitmix",
           "uniform01", "log_uniform_int", "np"]
