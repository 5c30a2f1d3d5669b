"""changa_cell_forces_mixed_noalloc: the cell-list evaluation of the FP32-mixed
form with its scratch in the library's fixed device array instead of a
stream-ordered allocation.  It serves callers that must not let a library
allocate device memory (all of it handed to their own pool allocator, or a
thread that must not wait on cudaMalloc/cudaFree synchronising the device).

Checked through the C-ABI against the allocating entry point,
changa_cell_forces_mixed, on two calls in a row (the second call finds the
first one's contents in the shared array and must not depend on them), and
against the CPU oracle's nodeBucketForce on the same cell lists.
This file sorts last so that a run stopping at its first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

import oracle
from changa_gb300 import _native as N
from changa_gb300 import gravity, ics, tree

pytestmark = pytest.mark.gpu

TOL = 1e-6  # the FP64-form bar; both entries run the same kernels
# FP32-mixed arithmetic against the FP64 oracle (relative force error)
ORACLE_MEDIAN, ORACLE_MAX = 1e-6, 1e-4


def _call(fn, ds, vars):
    import torch
    vars.zero_()
    rc = fn(ds.moments.data_ptr(), ds.moments.shape[0], ds.parts.data_ptr(), ds.n,
            C.byref(ds.reqs[0]["c"]), float(ds.lists.period), vars.data_ptr(),
            torch.cuda.current_stream().cuda_stream)
    N.check(rc, fn.__name__)
    return vars.cpu().numpy().copy()


def _rel(a, b):
    return np.linalg.norm(a[:, :3] - b[:, :3], axis=1) / np.linalg.norm(b[:, :3], axis=1)


def test_noalloc_matches_allocating_entry(cuda_ok):
    import torch
    lib = N.cuda_lib()
    p = ics.plummer(20000, ics.rng_for(31), soft=0.01)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7)
    # fits the fixed scratch: 64 B per moment + 32 B per target
    assert 64 * L.moments.shape[0] + 32 * L.n < 16 * 2 ** 20
    ds = gravity.DeviceSystem(L)
    vars = torch.zeros((L.n, 5), dtype=torch.float64, device="cuda")
    ref = _call(lib.changa_cell_forces_mixed, ds, vars)
    orc = oracle.cell_forces(L.moments, L.parts, L.cells, fperiod=L.period)
    for _ in range(2):
        out = _call(lib.changa_cell_forces_mixed_noalloc, ds, vars)
        assert _rel(out, ref).max() < TOL
        np.testing.assert_allclose(out[:, 3], ref[:, 3], rtol=TOL)
        np.testing.assert_allclose(out[:, 4], ref[:, 4], rtol=TOL)
        e = _rel(out, orc)
        assert np.median(e) < ORACLE_MEDIAN and e.max() < ORACLE_MAX, (np.median(e), e.max())


def test_noalloc_rejects_oversize(cuda_ok):
    """Sizes beyond the fixed scratch are refused before anything is
    enqueued (the pointers are never dereferenced)."""
    lib = N.cuda_lib()
    lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_RECORD)
    try:
        req = N.ChangaListRequest()
        req.list = req.markers = req.starts = req.sizes = 1  # never read
        req.n_buckets = 1
        req.n_entries = 1
        lib.changa_gb300_last_error()  # the first error since the last read is kept: clear it
        before = lib.changa_gb300_kernel_launches()
        rc = lib.changa_cell_forces_mixed_noalloc(8, 300000, 8, 1, C.byref(req), 0.0, 8, None)
        assert rc == 1003
        assert lib.changa_gb300_last_error() == 1003
        # counts whose byte sizes would wrap around 64 bits are refused too
        for nm, nt in ((1 << 58, 1), (1, 1 << 59), (1 << 62, 1 << 62)):
            rc = lib.changa_cell_forces_mixed_noalloc(8, nm, 8, nt, C.byref(req), 0.0, 8, None)
            assert rc == 1003, (nm, nt, rc)
            assert lib.changa_gb300_last_error() == 1003
        assert lib.changa_gb300_kernel_launches() == before
    finally:
        lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_ABORT)
