"""The allocation-free Morton ordering entry point (sph_morton_order_noalloc).

It exists for callers that cannot let the library allocate device memory:
a host that records its own step into a CUDA graph (an allocation inside the
capture breaks it) or one that runs under a fixed device-memory budget.  Its
scratch is a file-scope device array shared by all calls, so this test calls
it twice in a row and checks both results against the existing entry point
(the key order the octree build of sph_run_pass(ctx, 0) reports through
sph_get_order): integer work, so equality is exact.  This file is collected
last on purpose; it passes alone and after the other tests."""
import ctypes as C

import numpy as np
import pytest

from helpers import device_context, small_impact, tillotson_materials

pytestmark = pytest.mark.gpu


def test_morton_order_without_allocation_matches_tree_build():
    import torch

    from fdps_sph_gb300 import lib

    F, ids, mats, _ = small_impact(18000, 2000, seed=21)
    n = F.shape[1]
    assert n <= lib.NOALLOC_MAX_N
    ctx = device_context(tillotson_materials())
    ctx.upload(F, ids, mats)
    ctx.run_pass(0)
    slot, keys = ctx.order()

    L = lib.load()
    dev = torch.device("cuda:0")
    x = torch.tensor(F[0], dtype=torch.float64, device=dev)
    y = torch.tensor(F[1], dtype=torch.float64, device=dev)
    z = torch.tensor(F[2], dtype=torch.float64, device=dev)
    for call in range(2):
        k_out = torch.full((n,), -1, dtype=torch.int64, device=dev)
        o_out = torch.full((n,), -1, dtype=torch.int32, device=dev)
        rc = L.sph_morton_order_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                        C.c_void_p(z.data_ptr()), n, C.c_void_p(k_out.data_ptr()),
                                        C.c_void_p(o_out.data_ptr()), None)
        assert rc == lib.SPH_OK, (call, rc)
        torch.cuda.synchronize()
        assert np.array_equal(k_out.cpu().numpy().view(np.uint64), keys), call
        assert np.array_equal(o_out.cpu().numpy(), slot), call

    # beyond the scratch capacity: refused before any device work
    big = lib.NOALLOC_MAX_N + 1
    rc = L.sph_morton_order_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(z.data_ptr()),
                                    big, C.c_void_p(k_out.data_ptr()), C.c_void_p(o_out.data_ptr()), None)
    assert rc == -6   # SPH_ERR_CAPACITY
    ctx.close()
