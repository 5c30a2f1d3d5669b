"""Host tree structure exports used by the device moment up-pass and the
adjoint (no GPU): parent / leaf / particle ranges are consistent, and the
moment sums the device up-pass forms over each node's range reproduce the
host build's incremental moments (MultipoleMoments.h:206-352 order)."""
import numpy as np
import pytest

from changa_gb300 import ics, tree


@pytest.fixture(scope="module")
def small_tree(built):
    p = ics.plummer(3000, ics.rng_for(0))
    return tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7)


def test_ranges_partition(small_tree):
    t = small_tree
    parent, leaf = t.meta["parent"], t.meta["leaf"]
    first, count = t.meta["first"], t.meta["count"]
    nm = t.moments.shape[0]
    assert parent[0] == -1 and first[0] == 0 and count[0] == t.n
    assert (parent[1:] >= 0).all() and (parent[1:] < np.arange(1, nm)).all()
    # children tile their parent's range
    kids = np.zeros(nm, np.int64)
    np.add.at(kids, parent[1:], count[1:])
    internal = kids > 0
    assert (kids[internal] == count[internal]).all()
    for i in np.nonzero(parent >= 0)[0]:
        p = parent[i]
        assert first[p] <= first[i] and first[i] + count[i] <= first[p] + count[p]
    # every particle's leaf range holds it, and the leaves are the buckets
    k = np.arange(t.n)
    assert ((first[leaf] <= k) & (k < first[leaf] + count[leaf])).all()
    assert sorted(set(leaf.tolist())) == sorted(np.nonzero(~internal & (count > 0))[0].tolist())


def test_range_moments_match_host(small_tree):
    t = small_tree
    first, count = t.meta["first"], t.meta["count"]
    m, s, x = t.parts[:, 0], t.parts[:, 1], t.parts[:, 2:5]
    for i in range(t.moments.shape[0]):
        sl = slice(first[i], first[i] + count[i])
        M = m[sl].sum()
        cm = (m[sl, None] * x[sl]).sum(0) / M
        d = x[sl] - cm
        q = np.einsum("k,ka,kb->ab", m[sl], d, d)
        got = np.array([(m[sl] * s[sl]).sum() / M, M, *cm, q[0, 0], q[0, 1], q[0, 2], q[1, 1],
                        q[1, 2], q[2, 2]])
        ref = t.moments[i, 1:]
        scale = np.array([1, M, 1, 1, 1] + [max(q.trace(), 1e-300)] * 6)
        np.testing.assert_allclose(got / scale, ref / scale, rtol=0, atol=1e-12)
