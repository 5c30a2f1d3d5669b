"""Walk and forces in one pass (changa_walk_forces): the two-phase walk's
second phase evaluates each block of accepted cells and opened particles as
it decides them, with no interaction lists.  The interactions are the list
walk's, so the forces equal the list path's FP32-mixed forces up to FP32
summation order, and sit as close to the FP64 form as those do."""
import numpy as np
import pytest

from changa_gb300 import gravity, ics, tree
from changa_gb300.walk import walk_forces
from helpers import force_rel_err, force_rms_err, pot_rel_err

pytestmark = pytest.mark.gpu


def _compare(L, ewald=None, periodic=False):
    ds = gravity.DeviceSystem(L, ewald=ewald)
    f64 = ds.step("fp64").cpu().numpy()
    mix = ds.step("mixed").cpu().numpy()
    fused = walk_forces(L, ewald=ds.ewald_params).cpu().numpy()
    err = force_rms_err if periodic else force_rel_err
    e_f, e_m = err(fused, f64), err(mix, f64)
    print("fused vs FP64: median %.2e max %.2e; list mixed vs FP64: median %.2e max %.2e"
          % (np.median(e_f), e_f.max(), np.median(e_m), e_m.max()))
    # the same FP32 arithmetic in another summation order
    assert np.median(e_f) < 1.5 * np.median(e_m) + 1e-9
    assert e_f.max() < 3.0 * e_m.max() + 1e-7
    assert np.median(err(fused, mix)) < 2.0 * np.median(e_m) + 1e-9
    if not periodic:
        assert np.median(pot_rel_err(fused, f64)) < 1e-6
    else:  # the periodic potential crosses zero: against its rms
        dp = np.abs(fused[:, 3] - f64[:, 3]) / np.sqrt((f64[:, 3] ** 2).mean())
        assert np.median(dp) < 1e-5
    # dtGrav: a maximum over the same per-pair values
    rel_dt = np.abs(fused[:, 4] - mix[:, 4]) / np.maximum(mix[:, 4], 1e-300)
    assert np.median(rel_dt) < 1e-6 and rel_dt.max() < 1e-4
    return fused


def test_walk_forces_plummer(cuda_ok):
    p = ics.plummer(32768, ics.rng_for(0), soft=0.01)
    _compare(tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7))


def test_walk_forces_periodic_clustered_ewald(cuda_ok):
    p = ics.nfw_halos(65536, ics.rng_for(8), soft=2e-4)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=32, theta=0.7, period=1.0,
                         n_replicas=1)
    _compare(L, ewald=gravity.EwaldConfig(1.0, 1, 2.6, 2.8), periodic=True)


@pytest.mark.parametrize("nb", [1, 5, 33, 64])
def test_walk_forces_ragged_buckets(cuda_ok, nb):
    """Buckets of 1 and 5 targets (several lane groups per warp) and of 33
    and 64 (walked once per chunk of 32 targets)."""
    p = ics.plummer(6000, ics.rng_for(5), soft=0.05)
    _compare(tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=nb, theta=0.6))


def test_walk_forces_stack_rerun(cuda_ok):
    """A 32-entry first stack runs out; the launch runs again with the large
    stack and rewrites every target: the same bits as a normal run."""
    from changa_gb300 import _native as N
    lib = N.cuda_lib()
    p = ics.plummer(16384, ics.rng_for(2), soft=0.01)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=8, theta=0.5)
    ref = walk_forces(L).cpu().numpy()
    before = lib.changa_walk_stack_reruns()
    lib.changa_walk_set_test_small_stack(1)
    try:
        got = walk_forces(L).cpu().numpy()
    finally:
        lib.changa_walk_set_test_small_stack(0)
    assert lib.changa_walk_stack_reruns() > before
    assert np.array_equal(got, ref)


def test_walk_forces_device_tree(cuda_ok):
    """Positions on the device to forces: the GPU-built tree, walked and
    evaluated in one pass, against its own list path."""
    import torch
    from changa_gb300.gputree import DeviceTree
    from changa_gb300.walk import gpu_walk
    p = ics.nfw_halos(131072, ics.rng_for(9), soft=2e-4)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    T = DeviceTree(t(p["pos"]), t(p["mass"]), t(p["soft"]), n_bucket=32, theta=0.7)
    cells, plist, _ = gpu_walk(T)
    ds = gravity.DeviceSystem(T, device_reqs=[cells, plist])
    f64 = ds.step("fp64").cpu().numpy()
    mix = ds.step("mixed").cpu().numpy()
    fused = walk_forces(T).cpu().numpy()
    e_f, e_m = force_rel_err(fused, f64), force_rel_err(mix, f64)
    assert np.median(e_f) < 1.5 * np.median(e_m) + 1e-9
    assert e_f.max() < 3.0 * e_m.max() + 1e-7


def test_walk_forces_rejects_hexadecapole(cuda_ok):
    from changa_gb300 import _native as N
    lib = N.cuda_lib()
    p = ics.plummer(2048, ics.rng_for(3))
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, order=4)
    lib.changa_gb300_last_error()  # clear
    with pytest.raises(RuntimeError, match="1001"):  # CHANGA_E_INVALID_ARG
        walk_forces(L)
    assert lib.changa_gb300_last_error() == 1001  # read, and so cleared


def test_walk_forces_rejects_short_particle_array(cuda_ok):
    """A particle count below the tree's: the buckets past it are refused
    by the kernel's range check (nothing is read past the array) and the
    call returns CHANGA_E_INVALID_ARG."""
    import ctypes as C

    import torch
    from changa_gb300 import _native as N
    lib = N.cuda_lib()
    p = ics.plummer(4096, ics.rng_for(4), soft=0.01)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    m = L.meta
    geom, bbox, info = t(m["node_geom"]), t(m["node_bbox"]), t(m["node_info"])
    parent, bnode = t(m["parent"]), t(m["bucket_node"])
    moments, parts = t(L.moments), t(L.parts)
    tv = N.ChangaTreeView(geom.data_ptr(), bbox.data_ptr(), info.data_ptr(), parent.data_ptr(),
                          int(geom.shape[0]), bnode.data_ptr(), int(bnode.shape[0]))
    wp = N.ChangaWalkParams(0.7, 2, 0.0, 0)
    out = torch.zeros((L.n, 5), dtype=torch.float64, device="cuda")
    lib.changa_gb300_last_error()  # clear
    rc = lib.changa_walk_forces(C.byref(tv), C.byref(wp), moments.data_ptr(), parts.data_ptr(),
                                L.n // 2, None, out.data_ptr(),
                                torch.cuda.current_stream().cuda_stream)
    assert rc == 1001
    assert lib.changa_gb300_last_error() == 1001


def test_walk_forces_two_replica_layers(cuda_ok):
    """Two replica layers (5^3 replica roots on the root check list) and the
    Ewald term with nReps = 2, walked and evaluated in one pass."""
    p = ics.nfw_halos(16384, ics.rng_for(10), soft=1e-3)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         n_replicas=2)
    _compare(L, ewald=gravity.EwaldConfig(1.0, 2, 2.6, 2.8), periodic=True)
