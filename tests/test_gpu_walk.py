"""The interaction-list walk on the GPU: every bucket gets the same entries
as the host walk (ChaNGa's dual walk restated in host/tree.cpp), for open
and periodic trees, quadrupole and hexadecapole rules (with softened
cells), ragged buckets; and forces from the device lists equal those from
the host lists up to summation order."""
import numpy as np
import pytest

from changa_gb300 import gravity, ics, tree
from changa_gb300.walk import gpu_walk, same_entries
from helpers import force_rel_err, force_rms_err

pytestmark = pytest.mark.gpu


def _identical(a, b):
    """Two device requests hold the same arrays (entries in the same order)."""
    la, ma = a.to_host()
    lb, mb = b.to_host()
    return np.array_equal(la, lb) and np.array_equal(ma, mb)


def _check(L, ewald=None):
    cells, plist, soft = gpu_walk(L)
    # changa_walk writes exactly what count + fill write
    two = gpu_walk(L, method="two_pass")
    for k in range(3 if L.order == 4 else 2):
        assert _identical((cells, plist, soft)[k], two[k])
    nb = len(L.bucket_starts)
    assert same_entries(L.cells, cells, nb)
    assert same_entries(L.plist, plist, nb)
    if L.order == 4:
        assert same_entries(L.softcells, soft, nb)
    reqs = [cells, plist] + ([soft] if L.order == 4 else [])
    host = gravity.DeviceSystem(L, ewald=ewald).step("fp64").cpu().numpy()
    dev = gravity.DeviceSystem(L, ewald=ewald, device_reqs=reqs).step("fp64").cpu().numpy()
    assert force_rel_err(dev, host).max() < 1e-12
    vm = gravity.DeviceSystem(L, ewald=ewald, device_reqs=reqs).step("mixed").cpu().numpy()
    if ewald is None:
        assert np.median(force_rel_err(vm, host)) < 2e-6
    else:  # near-uniform periodic lattice: measured against rms|a|, as the Ewald tests are
        assert np.median(force_rms_err(vm, host)) < 5e-5


def test_walk_plummer(cuda_ok):
    p = ics.plummer(32768, ics.rng_for(0), soft=0.01)
    _check(tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7))


def test_walk_periodic_lattice(cuda_ok):
    p = ics.lattice_grf(24, ics.rng_for(1))
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0)
    _check(L, ewald=gravity.EwaldConfig(1.0, 1, 2.6, 2.8))


def test_walk_hexadecapole_softened(cuda_ok):
    p = ics.plummer(16384, ics.rng_for(3))
    p["soft"][:] = 0.3
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, order=4)
    assert L.softcells.n_entries > 0
    _check(L)


@pytest.mark.parametrize("nb", [1, 5, 33])
def test_walk_ragged_buckets(cuda_ok, nb):
    p = ics.plummer(3000, ics.rng_for(5), soft=0.05)
    _check(tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=nb, theta=0.6))


def test_walk_single_traversal_path(cuda_ok):
    """A tree of more than 16384 buckets takes changa_walk's single
    traversal (sampled pool sizes, append, gather): the same arrays as count
    + fill, the host walk's entries; and with pools too small it falls back
    to the fill pass with the same result."""
    from changa_gb300 import _native as N
    p = ics.plummer(65536, ics.rng_for(6), soft=0.01)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=2, theta=0.7)
    nb = len(L.bucket_starts)
    assert nb >= 16384
    tm = {}
    one = gpu_walk(L, timings=tm)
    assert tm["passes"] == 1
    two = gpu_walk(L, method="two_pass")
    lib = N.cuda_lib()
    lib.changa_walk_set_pool_factor(0.0)
    try:
        tm3 = {}
        short = gpu_walk(L, timings=tm3)
    finally:
        lib.changa_walk_set_pool_factor(1.2)
    assert tm3["passes"] == 3
    # this tree takes the two-phase walk: count + fill (one phase) holds the
    # same entries per bucket in another order; the fill-pass fallback writes
    # the append pass's arrays
    for k in range(2):
        assert _identical(short[k], one[k])
    assert same_entries(L.cells, one[0], nb) and same_entries(L.plist, one[1], nb)
    assert same_entries(L.cells, two[0], nb) and same_entries(L.plist, two[1], nb)


@pytest.mark.parametrize("gmax", [1, 2, 8, 32, 256])
def test_walk_two_phase(cuda_ok, gmax):
    """The two-phase walk (each group of at most gmax buckets walked once
    down to its group node, then each bucket from the group's frontier, its
    lists starting with the group's prefix lists) gives every bucket the
    host walk's entries: open and periodic trees (one and two replica
    shells), small and large buckets, the hexadecapole rules with softened
    cells (split per bucket from the group's cells), single traversal and
    count + fill, and the forces of the one-phase lists."""
    from changa_gb300 import _native as N
    lib = N.cuda_lib()
    p = ics.plummer(65536, ics.rng_for(6), soft=0.01)
    g = ics.lattice_grf(16, ics.rng_for(7))
    h = ics.plummer(16384, ics.rng_for(3))
    h["soft"][:] = 0.3  # hexadecapole rules with many softened cells
    cases = [tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=4, theta=0.7),
             tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=32, theta=0.5),
             tree.build_lists(g["pos"], g["mass"], g["soft"], n_bucket=8, theta=0.7, period=1.0),
             tree.build_lists(g["pos"], g["mass"], g["soft"], n_bucket=8, theta=0.7, period=1.0,
                              n_replicas=2),
             tree.build_lists(h["pos"], h["mass"], h["soft"], n_bucket=8, theta=0.7, order=4)]
    lib.changa_walk_set_groups(gmax, 1)
    try:
        for L in cases:
            nb = len(L.bucket_starts)
            for method in ("single", "two_pass"):
                cells, plist, soft = gpu_walk(L, method=method)
                assert same_entries(L.cells, cells, nb) and same_entries(L.plist, plist, nb)
                if L.order == 4:
                    assert L.softcells.n_entries > 0 and same_entries(L.softcells, soft, nb)
            reqs = [cells, plist] + ([soft] if L.order == 4 else [])
            host = gravity.DeviceSystem(L).step("fp64").cpu().numpy()
            dev = gravity.DeviceSystem(L, device_reqs=reqs).step("fp64").cpu().numpy()
            assert force_rel_err(dev, host).max() < 1e-12
    finally:
        lib.changa_walk_set_groups(32, 4096)


def test_walk_stack_rerun(cuda_ok):
    """A warp that exhausts its traversal stack makes the launch run once
    more with the large stack: with the first traversal forced onto a
    64-entry stack, the single traversal (append, periodic lattice) and the
    count + fill passes (Plummer) give the host walk's entries."""
    from changa_gb300 import _native as N
    lib = N.cuda_lib()
    p = ics.plummer(65536, ics.rng_for(6), soft=0.01)
    Lp = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=2, theta=0.7)
    g = ics.lattice_grf(16, ics.rng_for(7))
    Lg = tree.build_lists(g["pos"], g["mass"], g["soft"], n_bucket=8, theta=0.7, period=1.0)
    # two replica shells: 125 replica roots start on the stack, more than the
    # 64-entry first stack holds, so every warp hands over to the re-run
    h = ics.lattice_grf(8, ics.rng_for(8))
    Lh = tree.build_lists(h["pos"], h["mass"], h["soft"], n_bucket=8, theta=0.7, period=1.0,
                          n_replicas=2)
    ref_p = gpu_walk(Lp)
    ref_g = gpu_walk(Lg, method="two_pass")
    ref_h = [gpu_walk(Lh, method=m) for m in ("two_pass", "single")]
    before = lib.changa_walk_stack_reruns()
    lib.changa_walk_set_test_small_stack(1)
    try:
        one = gpu_walk(Lp)
        two = gpu_walk(Lg, method="two_pass")
        before_h = lib.changa_walk_stack_reruns()
        three = [gpu_walk(Lh, method=m) for m in ("two_pass", "single")]
        assert lib.changa_walk_stack_reruns() >= before_h + 2
    finally:
        lib.changa_walk_set_test_small_stack(0)
    assert lib.changa_walk_stack_reruns() > before
    for k in range(2):
        assert _identical(one[k], ref_p[k]) and _identical(two[k], ref_g[k])
        for t3, r3 in zip(three, ref_h):
            assert _identical(t3[k], r3[k])
    nbp, nbg, nbh = len(Lp.bucket_starts), len(Lg.bucket_starts), len(Lh.bucket_starts)
    assert same_entries(Lp.cells, one[0], nbp) and same_entries(Lp.plist, one[1], nbp)
    assert same_entries(Lg.cells, two[0], nbg) and same_entries(Lg.plist, two[1], nbg)
    for t3 in three:
        assert same_entries(Lh.cells, t3[0], nbh) and same_entries(Lh.plist, t3[1], nbh)


def test_device_lists_outlive_their_call(cuda_ok):
    """Tree arrays and lists come back as torch views of library memory;
    each view keeps its owner alive.  Five trees built one after another
    (only their DeviceSystems kept), each evaluated after all were built,
    give the host-built trees' FP64 forces: no tree's memory was handed on
    to the next build while still in use."""
    import torch
    from changa_gb300.gputree import DeviceTree
    p = ics.plummer(65536, ics.rng_for(4), soft=0.01)
    systems, hosts = [], []
    for k in range(5):
        pos = p["pos"] * (1.0 + 0.01 * k)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
        T = DeviceTree(t(pos), t(p["mass"]), t(p["soft"]), n_bucket=16, theta=0.7)
        cells, plist, _ = gpu_walk(T)
        systems.append(gravity.DeviceSystem(T, device_reqs=[cells, plist]))
        del T, cells, plist
        hosts.append(tree.build_lists(pos, p["mass"], p["soft"], n_bucket=16, theta=0.7))
    for ds, L in zip(systems, hosts):
        dev = ds.step("fp64").cpu().numpy()
        host = gravity.DeviceSystem(L).step("fp64").cpu().numpy()
        assert force_rel_err(dev, host).max() < 1e-10
