"""The batching form: many independent systems concatenated into one request
pair, evaluated by one CUDA-graph replay whose persistent kernels share a
device work queue.  Each system must match its own FP64 CPU tree result, and
the replay must match the plain (captured-free) evaluation."""
import numpy as np
import pytest

import oracle
from changa_gb300 import gravity, ics, tree
from helpers import force_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch(cuda_ok):
    rng = ics.rng_for(40)
    systems = []
    for p in ics.plummer_clusters(12, rng, nmin=256, nmax=4096):
        systems.append(tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.6))
    return systems, tree.concat_systems(systems)


def test_batched_graph_matches_each_system(batch):
    systems, cat = batch
    ds = gravity.DeviceSystem(cat)
    g = gravity.GravityGraph(ds, "mixed")
    try:
        v1 = g.launch().cpu().numpy().copy()
        v2 = g.launch().cpu().numpy().copy()  # replays zero and recompute
    finally:
        g.close()
    np.testing.assert_array_equal(v1, v2)
    plain = gravity.DeviceSystem(cat).step("mixed").cpu().numpy()
    np.testing.assert_allclose(v1, plain, rtol=1e-12, atol=0)
    off = cat.meta["offsets"]
    for k, s in enumerate(systems):
        ref = oracle.cell_forces(s.moments, s.parts, s.cells)
        ref = oracle.part_forces(s.parts, s.parts, s.plist, vars=ref)
        e = force_rel_err(v1[off[k]:off[k + 1]], ref)
        assert np.median(e) < 2e-6 and np.percentile(e, 99) < 1e-4, k


def test_batched_fp64_graph(batch):
    systems, cat = batch
    ds = gravity.DeviceSystem(cat)
    g = gravity.GravityGraph(ds, "fp64")
    try:
        v = g.launch().cpu().numpy()
    finally:
        g.close()
    off = cat.meta["offsets"]
    for k in (0, len(systems) - 1):
        s = systems[k]
        ref = oracle.cell_forces(s.moments, s.parts, s.cells)
        ref = oracle.part_forces(s.parts, s.parts, s.plist, vars=ref)
        assert force_rel_err(v[off[k]:off[k + 1]], ref).max() < 1e-6
