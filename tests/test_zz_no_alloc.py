"""cfx_reduce_noalloc: the reduction entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc: a host application whose
own memory pool has reserved the whole GPU, or one held to a fixed
device-memory budget.  Its block partials live in a static device array, so it has a
size limit (33,554,432 elements).  The test compares it, through the C ABI,
with the allocating entry point cfx_reduce on two calls in a row (the static
scratch is reused), within the reduction tolerance the other tests use, and
checks that a size beyond the limit is refused before any launch.  This file
sorts after the solver and operator tests so that a run stopping at the first
failure has run them.
"""
import ctypes

import numpy as np
import pytest

from openfoam_dev_gb300 import ldu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAX_N = 33_554_432


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def test_noalloc_reduction_matches_cfx_reduce_twice():
    rng = np.random.default_rng(11)
    n = 3_000_017
    a = torch.from_numpy(rng.uniform(-1, 1, n)).cuda()
    b = torch.from_numpy(rng.uniform(-1, 1, n)).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    ctx = ldu.default_context()
    lib = ldu.lib()
    for which in (0, 1, 2, 3):
        ref = ctx.reduce(which, a, b if which == 3 else None)
        for _ in range(2):
            out.fill_(np.nan)
            torch.cuda.synchronize()
            rc = lib.cfx_reduce_noalloc(which, n, _p(a), _p(b if which == 3 else None), _p(out), None)
            assert rc == 0, lib.cfx_last_error()
            torch.cuda.synchronize()
            assert out.item() == pytest.approx(ref, rel=1e-12, abs=1e-12), (which, out.item(), ref)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    a = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    lib = ldu.lib()
    rc = lib.cfx_reduce_noalloc(0, MAX_N + 1, _p(a), None, _p(out), None)
    assert rc == -1
    assert b"exceeds the maximum" in lib.cfx_last_error()
