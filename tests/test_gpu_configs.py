"""GPU parity at the stated sizes of two workloads.

* lattice1m: the periodic 128^3 perturbed lattice (128^3 = 2^21 particles;
  P(k) ~ k^-2, rms displacement 0.2 of the spacing), eps 1/(50*128), theta
  0.7, bucket 16, Ewald with 1 replica, cut 2.6, h-cut 2.8.  The FP64 form
  against the oracle (gravity.h nodeBucketForce / partBucketForce +
  Ewald.cpp BucketEwald) per particle on a few thousand sampled buckets,
  and both forms against the FP64 Ewald direct sum on 4096 random
  particles.  On a near-uniform lattice the net force is a small residual
  of large cancelling terms, so ChaNGa's algorithm itself (the quadrupole
  tree at theta 0.7, and the root expansion for the replicas beyond the
  first shell) lies far from the direct sum there: its truncation does not
  shrink with N while the net force does (as N^(-1/3)).  The test records
  that error, checks that the FP32-mixed form adds nothing to it, and, on a
  32^3 lattice, that the tree converges to the direct sum as theta shrinks
  and as replica shells are added.
* clusters512: 512 isolated Plummer clusters (N log-uniform in [1024,
  65536], theta 0.6, bucket 16) evaluated by one CUDA-graph replay of the
  concatenated requests; every cluster checked against its own oracle
  evaluation on a sample of its buckets, and the FP64 form of the batch
  against the oracle.
"""
import numpy as np
import pytest

from helpers import force_rel_err, sampled_oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-6        # the plain FP64 form, relative per particle
MIX_MEDIAN_TOL = 2e-6  # FP32-mixed against the FP64 oracle, relative
MIX_P99_TOL = 1e-4
# periodic lattice: forces are small residuals of O(1) replica terms, so the
# FP32-mixed form is measured against the rms force (as for the smaller
# lattice of test_gpu_forces); measured at 128^3: median 3.7e-5, max 1.4e-4,
# set by the FP32 rounding of the O(1) Ewald hole terms
MIX_RMS_MEDIAN = 1e-4
MIX_RMS_MAX = 5e-4


@pytest.fixture(scope="module")
def lattice1m(cuda_ok):
    from changa_gb300 import gravity
    from changa_gb300.workloads import WORKLOADS
    wl = WORKLOADS["lattice1m"]
    L = wl.lists()
    ew = wl.ewald_config()
    ds = gravity.DeviceSystem(L, ewald=ew)
    v64 = ds.step("fp64").cpu().numpy().copy()
    vmx = ds.step("mixed").cpu().numpy().copy()
    return L, ew, ds, v64, vmx


def test_lattice1m_against_oracle(lattice1m):
    L, ew, _, v64, vmx = lattice1m
    assert L.n == 128 ** 3
    rng = np.random.default_rng(11)
    nb = len(L.bucket_starts)
    buckets = np.sort(rng.choice(nb, 3000, replace=False))
    ref, rows = sampled_oracle(L, ew, buckets)
    e64 = force_rel_err(v64[rows], ref[rows])
    # the periodic potential crosses zero: its error is taken against the rms
    pot64 = np.abs(v64[rows, 3] - ref[rows, 3]) / np.sqrt(np.mean(ref[rows, 3] ** 2))
    rms = np.sqrt((ref[rows, :3] ** 2).sum(1).mean())
    emx = np.linalg.norm(vmx[rows, :3] - ref[rows, :3], axis=1) / rms
    print("lattice1m, %d particles of %d buckets: FP64 max rel %.2e (pot %.2e); mixed / rms "
          "median %.2e max %.2e" % (len(rows), len(buckets), e64.max(), pot64.max(),
                                    np.median(emx), emx.max()))
    assert e64.max() < FP64_TOL
    assert pot64.max() < FP64_TOL
    np.testing.assert_allclose(v64[rows, 4], ref[rows, 4], rtol=FP64_TOL)
    assert np.median(emx) < MIX_RMS_MEDIAN and emx.max() < MIX_RMS_MAX


def test_lattice1m_against_direct_sum(lattice1m):
    from changa_gb300 import gravity
    L, _, ds, v64, vmx = lattice1m
    idx = np.sort(np.random.default_rng(12).choice(L.n, 4096, replace=False)).astype(np.int32)
    ref = gravity.direct_forces(ds.parts, idx, period=1.0)
    rms = np.sqrt((ref[:, :3] ** 2).sum(1).mean())
    e64 = np.linalg.norm(v64[idx, :3] - ref[:, :3], axis=1) / rms
    emx = np.linalg.norm(vmx[idx, :3] - ref[:, :3], axis=1) / rms
    rel = force_rel_err(v64[idx], ref)
    print("lattice1m vs direct Ewald sum, 4096 particles: FP64 / rms median %.2e p99 %.2e; "
          "mixed / rms median %.2e; relative median %.2e p99 %.2e" % (
              np.median(e64), np.percentile(e64, 99), np.median(emx), np.median(rel),
              np.percentile(rel, 99)))
    # the mixed arithmetic adds nothing visible on top of the algorithm's error
    assert abs(np.median(emx) - np.median(e64)) < 0.01 * np.median(e64)
    assert abs(np.percentile(emx, 99) - np.percentile(e64, 99)) < 0.01 * np.percentile(e64, 99)


def test_lattice_tree_converges_to_direct_sum(cuda_ok):
    """On a 32^3 perturbed lattice (same spectrum and softening rule), the
    FP64 tree + Ewald approaches the direct Ewald sum as theta shrinks, and
    with theta small the rest is the replica treatment: a second explicit
    replica shell removes most of it."""
    from changa_gb300 import gravity, ics, tree
    p = ics.lattice_grf(32, ics.rng_for(1))
    idx = np.random.default_rng(5).choice(len(p["mass"]), 1024, replace=False)
    med = {}
    for theta, nrep in ((0.7, 1), (0.4, 1), (0.2, 1), (0.2, 2)):
        L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=theta,
                             period=1.0, n_replicas=nrep)
        gi = np.argsort(L.perm)[idx].astype(np.int32)
        ds = gravity.DeviceSystem(L, ewald=gravity.EwaldConfig(1.0, nrep, max(2.6, nrep), 2.8))
        v = ds.step("fp64").cpu().numpy()[gi]
        ref = gravity.direct_forces(ds.parts, gi, period=1.0)
        rms = np.sqrt((ref[:, :3] ** 2).sum(1).mean())
        med[(theta, nrep)] = float(np.median(np.linalg.norm(v[:, :3] - ref[:, :3], axis=1)) / rms)
        print("lattice 32^3 theta %.1f nReps %d: tree+Ewald vs direct, median / rms %.2e" % (
            theta, nrep, med[(theta, nrep)]))
    assert med[(0.2, 1)] < med[(0.4, 1)] < med[(0.7, 1)]
    assert med[(0.2, 1)] < med[(0.7, 1)] / 5
    assert med[(0.2, 2)] < med[(0.2, 1)] / 2


def test_clusters512_graph_against_oracle(cuda_ok):
    import oracle
    from changa_gb300 import gravity, tree
    from changa_gb300.workloads import WORKLOADS
    wl = WORKLOADS["clusters512"]
    systems = wl.systems()
    assert len(systems) == 512
    ns = np.array([s.n for s in systems])
    assert ns.min() >= 1024 and ns.max() <= 65536
    B = tree.concat_systems(systems)
    ds = gravity.DeviceSystem(B)
    g = gravity.GravityGraph(ds, "mixed")
    try:
        g.launch()
        vmx = ds.vars.cpu().numpy().copy()
    finally:
        g.close()
    v64 = ds.step("fp64").cpu().numpy().copy()
    off = B.meta["offsets"]
    rng = np.random.default_rng(13)
    worst_med, worst_p99, worst64 = 0.0, 0.0, 0.0
    for k, s in enumerate(systems):
        nb = len(s.bucket_starts)
        buckets = np.sort(rng.choice(nb, max(1, nb // 8), replace=False))
        ref, rows = sampled_oracle(s, None, buckets)
        e = force_rel_err(vmx[off[k] + rows], ref[rows])
        e64 = force_rel_err(v64[off[k] + rows], ref[rows])
        worst_med = max(worst_med, float(np.median(e)))
        worst_p99 = max(worst_p99, float(np.percentile(e, 99)))
        worst64 = max(worst64, float(e64.max()))
        assert np.median(e) < MIX_MEDIAN_TOL and np.percentile(e, 99) < MIX_P99_TOL, k
        assert e64.max() < FP64_TOL, k
    print("clusters512 (%d particles): per cluster, worst median %.2e, worst p99 %.2e of the "
          "graph replay; FP64 worst max %.2e" % (B.n, worst_med, worst_p99, worst64))
