"""The allocation-free Morton ordering entry point (sph_morton_order_noalloc).

It exists for callers that cannot let the library allocate device memory: a
host that runs under a fixed device-memory budget (its own pool allocator owns
the rest of the GPU) or that may not take a cudaFree's device-wide
synchronisation in the middle of its step.  Its scratch is a file-scope
device array shared by all calls, so every case below calls it at least twice
in a row and checks each result against the existing entry point (the key
order the octree build of sph_run_pass(ctx, 0) reports through
sph_get_order, and the CPU oracle's Morton sort): integer work, so equality
is exact.  This file is collected
last on purpose; it passes alone and after the other tests."""
import ctypes as C

import numpy as np
import pytest

from helpers import device_context, small_impact, tillotson_materials

pytestmark = pytest.mark.gpu

SPH_ERR_NONFINITE = -5
SPH_ERR_CAPACITY = -6


def _tree_order(F, ids, mats):
    """the existing entry point's order: slot and key of every sorted position"""
    ctx = device_context(tillotson_materials())
    try:
        ctx.upload(F, ids, mats)
        ctx.run_pass(0)
        return ctx.order()
    finally:
        ctx.close()


def _oracle_order(F):
    """the CPU oracle's Morton sort (root cube, keys, stable radix sort)"""
    import ctypes

    from oracle import pyoracle as po

    L = po.lib()
    n = F.shape[1]
    x, y, z = (np.ascontiguousarray(F[c]) for c in range(3))
    rb = po.RootBox()
    L.or_root_box(po._p(x), po._p(y), po._p(z), n, ctypes.byref(rb))
    keys = np.zeros(n, dtype=np.uint64)
    L.or_morton_keys(po._p(x), po._p(y), po._p(z), n, ctypes.byref(rb), po._p(keys, ctypes.c_uint64))
    perm = np.zeros(n, dtype=np.int64)
    L.or_sort_perm(po._p(keys, ctypes.c_uint64), n, po._p(perm, ctypes.c_int64))
    return perm.astype(np.int32), keys[perm]


def _noalloc(L, x, y, z, n, k_out, o_out, stream=None):
    return L.sph_morton_order_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(z.data_ptr()),
                                      n, C.c_void_p(k_out.data_ptr()), C.c_void_p(o_out.data_ptr()),
                                      None if stream is None else C.c_void_p(stream))


def _check_twice(F, ids, mats, against_tree=True):
    import torch

    from fdps_sph_gb300 import lib

    n = F.shape[1]
    slot, keys = _oracle_order(F)
    if against_tree:
        t_slot, t_keys = _tree_order(F, ids, mats)
        assert np.array_equal(t_slot, slot) and np.array_equal(t_keys, keys)
    L = lib.load()
    dev = torch.device("cuda:0")
    x, y, z = (torch.tensor(F[c], dtype=torch.float64, device=dev) for c in range(3))
    for call in range(2):
        k_out = torch.full((n,), -1, dtype=torch.int64, device=dev)
        o_out = torch.full((n,), -1, dtype=torch.int32, device=dev)
        rc = _noalloc(L, x, y, z, n, k_out, o_out)
        assert rc == lib.SPH_OK, (n, call, rc)
        torch.cuda.synchronize()
        assert np.array_equal(k_out.cpu().numpy().view(np.uint64), keys), (n, call)
        assert np.array_equal(o_out.cpu().numpy(), slot), (n, call)
    return L, x, y, z, k_out, o_out


def test_morton_order_without_allocation_matches_tree_build():
    from fdps_sph_gb300 import lib

    F, ids, mats, _ = small_impact(18000, 2000, seed=21)
    assert F.shape[1] <= lib.NOALLOC_MAX_N
    L, x, y, z, k_out, o_out = _check_twice(F, ids, mats)
    # beyond the scratch capacity: refused before any device work
    assert _noalloc(L, x, y, z, lib.NOALLOC_MAX_N + 1, k_out, o_out) == SPH_ERR_CAPACITY


def test_morton_order_without_allocation_at_the_capacity():
    # n == SPH_NOALLOC_MAX_N fills every scratch region and the last radix tile
    from fdps_sph_gb300 import lib

    nmax = lib.NOALLOC_MAX_N
    F, ids, mats, _ = small_impact(nmax - nmax // 10, nmax // 10, seed=23)
    assert F.shape[1] == nmax
    _check_twice(F, ids, mats)


def test_morton_order_without_allocation_of_one_particle():
    F, ids, mats, _ = small_impact(1800, 200, seed=24)
    F1 = np.ascontiguousarray(F[:, :1])
    _check_twice(F1, ids[:1], mats[:1], against_tree=False)


def test_morton_order_without_allocation_rejects_a_nonfinite_position():
    # a NaN position is reported; the next clean call clears the error word and succeeds
    import torch

    from fdps_sph_gb300 import lib

    F, ids, mats, _ = small_impact(1800, 200, seed=25)
    n = F.shape[1]
    L = lib.load()
    dev = torch.device("cuda:0")
    bad = F.copy()
    bad[1, n // 2] = np.nan
    x, y, z = (torch.tensor(bad[c], dtype=torch.float64, device=dev) for c in range(3))
    k_out = torch.empty((n,), dtype=torch.int64, device=dev)
    o_out = torch.empty((n,), dtype=torch.int32, device=dev)
    assert _noalloc(L, x, y, z, n, k_out, o_out) == SPH_ERR_NONFINITE
    _check_twice(F, ids, mats)


def test_morton_order_without_allocation_recorded_into_a_cuda_graph():
    """captured on a side stream into a CUDA graph (after an eager call has looked the scratch up),
    the call only records its work and returns SPH_OK; two replays, each into freshly cleared
    outputs, give the oracle's order exactly"""
    import torch

    from fdps_sph_gb300 import lib

    F, ids, mats, _ = small_impact(9000, 1000, seed=26)
    n = F.shape[1]
    slot, keys = _oracle_order(F)
    L = lib.load()
    dev = torch.device("cuda:0")
    x, y, z = (torch.tensor(F[c], dtype=torch.float64, device=dev) for c in range(3))
    k_out = torch.full((n,), -1, dtype=torch.int64, device=dev)
    o_out = torch.full((n,), -1, dtype=torch.int32, device=dev)
    assert _noalloc(L, x, y, z, n, k_out, o_out) == lib.SPH_OK   # eager: resolves the scratch array
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc = _noalloc(L, x, y, z, n, k_out, o_out, stream=s.cuda_stream)
    assert rc == lib.SPH_OK
    for replay in range(2):
        k_out.fill_(-1)
        o_out.fill_(-1)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(k_out.cpu().numpy().view(np.uint64), keys), replay
        assert np.array_equal(o_out.cpu().numpy(), slot), replay
    # an eager call after the replays still reads its status back
    assert _noalloc(L, x, y, z, n, k_out, o_out) == lib.SPH_OK
