"""Device ingestion (eh_dcsr_from_edges): raw edge arrays -> symmetric,
sorted, deduplicated CSR, optionally degree-ordered, on the GPU.  Checked
against the host loader's semantics and the host degree ordering (exact)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class _DevicePtr:
    """Expose a raw device allocation to torch via __cuda_array_interface__."""

    def __init__(self, addr, count, dtype, typestr):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": typestr, "data": (addr, False),
                                         "version": 3}


def download(torch, dcsr):
    n, m, o, b, r = dcsr.view()
    off = torch.as_tensor(_DevicePtr(o, n + 1, None, "<u8"), device="cuda").cpu().numpy().astype(np.uint64)
    nbr = (torch.as_tensor(_DevicePtr(b, m, None, "<u4"), device="cuda").cpu().numpy().astype(np.uint32)
           if m else np.zeros(0, np.uint32))
    n2o = (torch.as_tensor(_DevicePtr(r, n, None, "<u4"), device="cuda").cpu().numpy().astype(np.uint32)
           if r else None)
    return off, nbr, n2o


def upload(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()


def test_generator_graph_round_trips_with_identity_order(eh):
    torch = pytest.importorskip("torch")
    off, nbr = eh.graph("rmat", 21, scale=12, edges=40000).csr()[:2]
    n = len(off) - 1
    row = np.repeat(np.arange(n, dtype=np.uint32), np.diff(off.astype(np.int64)))
    up = nbr > row
    src, dst = row[up], nbr[up]
    rng = np.random.default_rng(2)
    flip = rng.random(len(src)) < 0.5
    src, dst = np.where(flip, dst, src), np.where(flip, src, dst)
    dup = rng.integers(0, len(src), len(src) // 5)  # duplicated edges
    src, dst = np.concatenate([src, dst[dup]]), np.concatenate([dst, src[dup]])
    perm = rng.permutation(len(src))
    s_d, d_d = upload(torch, src[perm]), upload(torch, dst[perm])
    g = eh.DeviceCSR(n, s_d.data_ptr(), d_d.data_ptr(), len(src), degree_order=True)
    o2, b2, n2o = download(torch, g)
    assert np.array_equal(o2, off) and np.array_equal(b2, nbr)
    assert np.array_equal(n2o, np.arange(n))  # already degree-ordered: identity
    m = g.matrix("lower", "hybrid")
    assert m.count_triangles() == eh.Matrix.build(off, nbr, "lower", "hybrid").count_triangles()


def test_random_ids_match_host_degree_order_and_self_loops(eh):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    n = 3000
    src = rng.integers(0, n, 20000).astype(np.uint32)
    dst = rng.integers(0, n, 20000).astype(np.uint32)
    src[:50] = dst[:50]  # self-loops
    s_d, d_d = upload(torch, src), upload(torch, dst)
    for drop in (False, True):
        keys = set()
        for u, v in zip(src.tolist(), dst.tolist()):
            if u == v and drop:
                continue
            keys.add((u, v))
            keys.add((v, u))
        rows = [[] for _ in range(n)]
        for u, v in keys:
            rows[u].append(v)
        off = np.zeros(n + 1, np.uint64)
        off[1:] = np.cumsum([len(r) for r in rows])
        nbr = np.array([x for r in rows for x in sorted(r)], np.uint32)
        want = eh.HostGraph.from_csr(off, nbr).reorder_by_degree().csr()
        g = eh.DeviceCSR(n, s_d.data_ptr(), d_d.data_ptr(), len(src), drop_self_loops=drop, degree_order=True)
        o2, b2, n2o = download(torch, g)
        assert np.array_equal(o2, want[0]) and np.array_equal(b2, want[1])
        assert np.array_equal(n2o.astype(np.uint64), want[2])  # ext ids of the host path = input ids
        g2 = eh.DeviceCSR(n, s_d.data_ptr(), d_d.data_ptr(), len(src), drop_self_loops=drop, degree_order=False)
        o3, b3, n2o3 = download(torch, g2)
        assert n2o3 is None and np.array_equal(o3, off) and np.array_equal(b3, nbr)


def test_out_of_range_endpoint_is_rejected(eh):
    torch = pytest.importorskip("torch")
    s_d = upload(torch, np.array([0, 1, 7], np.uint32))
    d_d = upload(torch, np.array([1, 2, 3], np.uint32))
    with pytest.raises(eh.EHError) as e:
        eh.DeviceCSR(5, s_d.data_ptr(), d_d.data_ptr(), 3)
    assert e.value.status == 1
