"""Tree build on the GPU against the host build: same key order, the same
breadth-first topology, bucket order and particle ranges, the same
bounding boxes, moments and radii, bit for bit; and the GPU walk over the
device tree gives the host walk's lists, so forces agree."""
import numpy as np
import pytest

from changa_gb300 import gravity, ics, tree
from changa_gb300.gputree import DeviceTree
from changa_gb300.walk import gpu_walk, same_entries
from helpers import force_rel_err, force_rms_err

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _compare(p, n_bucket, theta, period=0.0, ewald=None):
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=n_bucket, theta=theta,
                         period=period)
    T = DeviceTree(_dev(p["pos"]), _dev(p["mass"]), _dev(p["soft"]), n_bucket=n_bucket,
                   theta=theta, period=period)
    try:
        assert np.array_equal(T.perm.cpu().numpy(), L.perm)
        assert T.n_nodes == L.moments.shape[0] and T.n_buckets == len(L.bucket_starts)
        assert np.array_equal(T.meta["node_info"].cpu().numpy(), L.meta["node_info"])
        assert np.array_equal(T.meta["parent"].cpu().numpy(), L.meta["parent"])
        assert np.array_equal(T.meta["bucket_node"].cpu().numpy(), L.meta["bucket_node"])
        assert np.array_equal(T.meta["leaf"].cpu().numpy(), L.meta["leaf"])
        assert np.array_equal(T.meta["node_bbox"].cpu().numpy(), L.meta["node_bbox"])
        assert np.array_equal(T.parts.cpu().numpy(), L.parts)
        # the device sums are the host's, in its order, without FMA
        # contraction: bit for bit
        assert np.array_equal(T.moments.cpu().numpy(), L.moments)
        assert np.array_equal(T.meta["node_geom"].cpu().numpy(), L.meta["node_geom"])
        cells, plist, _ = gpu_walk(T)
        nb = T.n_buckets
        assert same_entries(L.cells, cells, nb) and same_entries(L.plist, plist, nb)
        host = gravity.DeviceSystem(L, ewald=ewald).step("fp64").cpu().numpy()
        dev = gravity.DeviceSystem(T, ewald=ewald, device_reqs=[cells, plist]).step("fp64")
        err = force_rms_err if ewald else force_rel_err
        assert err(dev.cpu().numpy(), host).max() < 1e-10
    finally:
        T.close()


def test_treebuild_plummer(cuda_ok):
    _compare(ics.plummer(32768, ics.rng_for(0), soft=0.01), 16, 0.7)


def test_treebuild_periodic_nfw(cuda_ok):
    _compare(ics.nfw_halos(32768, ics.rng_for(2), soft=1e-3), 32, 0.7, period=1.0,
             ewald=gravity.EwaldConfig(1.0, 1, 2.6, 2.8))


def test_treebuild_coincident_and_tiny(cuda_ok):
    """Coincident particles (equal keys keep input order) and 1-particle
    buckets."""
    rng = np.random.default_rng(4)
    pos = rng.uniform(-1, 1, (3000, 3))
    pos[1000:1100] = pos[5]
    p = dict(pos=pos, mass=np.full(3000, 1 / 3000), soft=np.full(3000, 0.02))
    _compare(p, 1, 0.6)
    _compare(p, 7, 0.6)
