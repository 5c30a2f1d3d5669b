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


def test_concat_systems_shifts_indices():
    """The batched request of several systems: each system's buckets keep
    their entries, with source indices shifted by the system's first moment
    (cells) or particle (particles) and targets by its first particle."""
    from changa_gb300 import ics, tree
    rng = ics.rng_for(9)
    systems = []
    for n in (300, 1000, 77):
        p = ics.plummer(n, rng, soft=0.02)
        systems.append(tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=8, theta=0.6))
    B = tree.concat_systems(systems)
    assert B.n == sum(s.n for s in systems)
    assert B.interactions == sum(s.interactions for s in systems)
    p_off = np.cumsum([0] + [s.n for s in systems])
    m_off = np.cumsum([0] + [s.moments.shape[0] for s in systems])
    for kind, off in (("cells", m_off), ("plist", p_off)):
        R = getattr(B, kind)
        b0 = 0
        for k, s in enumerate(systems):
            r = getattr(s, kind)
            for j in range(r.n_buckets):
                lo, hi = R.markers[b0 + j], R.markers[b0 + j + 1]
                got = R.list[lo:hi]
                want = r.list[r.markers[j]:r.markers[j + 1]]
                np.testing.assert_array_equal(got[:, 0], want[:, 0] + off[k])
                np.testing.assert_array_equal(got[:, 1], want[:, 1])
                assert R.starts[b0 + j] == r.starts[j] + p_off[k]
                assert R.sizes[b0 + j] == r.sizes[j]
            b0 += r.n_buckets
        assert b0 == R.n_buckets


def test_part_runs_round_trip():
    """Particle lists as runs (the reference's ILPart form): expanding the
    runs gives the flat list back entry for entry, every run stays inside its
    bucket, and runs are far fewer than entries."""
    from changa_gb300 import ics, tree
    p = ics.plummer(8000, ics.rng_for(3), soft=0.02)
    g = ics.lattice_grf(12, ics.rng_for(4))
    for q, period in ((p, 0.0), (g, 1.0)):
        L = tree.build_lists(q["pos"], q["mass"], q["soft"], n_bucket=16, theta=0.7,
                             period=period)
        pr = tree.part_runs(L.plist)
        np.testing.assert_array_equal(tree.expand_runs(pr), L.plist.list)
        rm = pr.run_markers.astype(np.int64)
        assert rm[0] == 0 and rm[-1] == pr.n_runs and np.all(np.diff(rm) >= 0)
        per_bucket = np.add.reduceat(pr.runs[:, 2].astype(np.int64), rm[:-1]) * (np.diff(rm) > 0)
        np.testing.assert_array_equal(per_bucket, np.diff(L.plist.markers.astype(np.int64)))
        assert pr.n_runs * 4 < L.plist.n_entries


@pytest.mark.parametrize("case", ["open", "periodic1", "periodic2", "hexadecapole"])
def test_walk_accounts_every_source_once(built, case):
    """Each bucket's lists (accepted cells, opened particles and, in the
    hexadecapole build, softened cells, over every replica) account for
    every source particle exactly once: their masses
    sum to the total mass times the number of replicas walked, (2 n + 1)^3.
    A missed or repeated subtree of the walk (TreeWalk.cpp:297-434) shows
    here; unequal random masses keep swapped entries from cancelling."""
    rng = np.random.Generator(np.random.PCG64(21))
    if case == "open" or case == "hexadecapole":
        # softening 0.3: the hexadecapole walk sends cells whose softening
        # overlaps the bucket to its third list, as softened point masses
        p = ics.plummer(8192, ics.rng_for(0), soft=0.3 if case == "hexadecapole" else 0.01)
        kw = dict(order=4) if case == "hexadecapole" else {}
        reps = 1
    else:
        p = ics.nfw_halos(16384, ics.rng_for(3), soft=1e-3)
        nr = 1 if case == "periodic1" else 2
        kw = dict(period=1.0, n_replicas=nr)
        reps = (2 * nr + 1) ** 3
    mass = rng.uniform(0.5, 1.5, len(p["mass"])) / len(p["mass"])
    L = tree.build_lists(p["pos"], mass, p["soft"], n_bucket=16, theta=0.7, **kw)
    reqs = [(L.cells, L.moments[:, 2]), (L.plist, L.parts[:, 0])]
    if case == "hexadecapole":
        assert L.softcells.n_entries > 0
        reqs.append((L.softcells, L.moments[:, 2]))
    total = np.zeros(int(max(r.bucket_ids.max() for r, _ in reqs)) + 1)
    for req, w in reqs:
        seg = w[req.list[:, 0]]
        s = np.add.reduceat(seg, req.markers[:-1]) if len(seg) else np.zeros(req.n_buckets)
        s[req.markers[1:] == req.markers[:-1]] = 0.0
        np.add.at(total, req.bucket_ids, s)
    np.testing.assert_allclose(total, reps * mass.sum(), rtol=1e-12)


@pytest.mark.parametrize("n_replicas", [1, 2])
def test_walk_accounts_every_replica_once(built, n_replicas):
    """Per replica: each entry's offsetID carries its replica in bits 22-30
    (x + 3, y + 3, z + 3 in three bits each; TreePiece.cpp:3631-3652), and
    each bucket's entries of every one of the (2 n + 1)^3 replicas account
    for every source particle exactly once (masses summing to the total)."""
    rng = np.random.Generator(np.random.PCG64(21))
    p = ics.nfw_halos(16384, ics.rng_for(3), soft=1e-3)
    mass = rng.uniform(0.5, 1.5, len(p["mass"])) / len(p["mass"])
    L = tree.build_lists(p["pos"], mass, p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         n_replicas=n_replicas)
    side = 2 * n_replicas + 1
    nb = int(max(L.cells.bucket_ids.max(), L.plist.bucket_ids.max())) + 1
    total = np.zeros((nb, side ** 3))
    for req, w in ((L.cells, L.moments[:, 2]), (L.plist, L.parts[:, 0])):
        code = (req.list[:, 1].astype(np.int64) >> 22) & 0x1FF
        off = [((code >> (3 * k)) & 7) - 3 for k in range(3)]
        assert max(np.abs(o).max() for o in off) <= n_replicas
        rep = ((off[0] + n_replicas) * side + (off[1] + n_replicas)) * side + off[2] + n_replicas
        b = np.repeat(req.bucket_ids, np.diff(req.markers))
        np.add.at(total, (b, rep), w[req.list[:, 0]])
    np.testing.assert_allclose(total, mass.sum(), rtol=1e-12)


@pytest.mark.parametrize("case", ["open", "open_theta04", "periodic1"])
def test_walk_decisions_follow_opening_criterion(built, case):
    """The walk's decisions against ChaNGa's opening criterion, restated here
    apart from the host walk: a node opens when it holds 6 particles or
    fewer, or when the sphere of radius max(2/sqrt(3) R / theta, R) about
    its centre of mass plus the replica offset meets the box of the local
    node tested (gravity.h:597-723).  Every accepted cell of a bucket holds
    more than 6 particles and its sphere misses the bucket's box (accepted
    at any local level above, it missed a larger box), and its parent was
    opened for that bucket.  A source bucket that only partially meets a
    local ancestor is opened into particles for every bucket below it
    (Compute.cpp:717-760 with codes.h:21-22 and the local table of
    Opt.h:85-123), so particle entries are checked one level up: the parent
    of each source leaf was opened for the bucket."""
    if case == "periodic1":
        p = ics.nfw_halos(16384, ics.rng_for(3), soft=1e-3)
        theta, kw, period = 0.7, dict(period=1.0, n_replicas=1), 1.0
    else:
        p = ics.plummer(8192, ics.rng_for(0), soft=0.01)
        theta, kw, period = (0.4 if case == "open_theta04" else 0.7), {}, 0.0
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=theta, **kw)
    g, bb, cnt, par = L.meta["node_geom"], L.meta["node_bbox"], L.meta["count"], L.meta["parent"]
    leaf, bnode = L.meta["leaf"], L.meta["bucket_node"]

    def ratio(nodes, off, buckets):
        """squared distance from the node's sphere centre to the bucket's box
        over the squared opening radius"""
        c = g[nodes, :3] + off
        box = bb[bnode[buckets]]
        d = np.maximum(np.maximum(box[:, :3] - c, c - box[:, 3:]), 0.0)
        r = np.maximum(2.0 / np.sqrt(3.0) * g[nodes, 3] / theta, g[nodes, 3])
        return (d * d).sum(1) / (r * r)

    def entries(req):
        code = (req.list[:, 1].astype(np.int64) >> 22) & 0x1FF
        off = np.stack([((code >> (3 * k)) & 7) - 3 for k in range(3)], 1) * period
        return req.list[:, 0], off, np.repeat(req.bucket_ids, np.diff(req.markers))

    idx, off, b = entries(L.cells)
    assert (cnt[idx] > 6).all()
    assert (ratio(idx, off, b) > 1.0 - 1e-12).all()
    up = par[idx]
    has = up >= 0
    assert ((ratio(up[has], off[has], b[has]) <= 1.0 + 1e-12) | (cnt[up[has]] <= 6)).all()
    idx, off, b = entries(L.plist)
    up = par[leaf[idx]]
    has = up >= 0
    assert ((ratio(up[has], off[has], b[has]) <= 1.0 + 1e-12) | (cnt[up[has]] <= 6)).all()


def test_hexadecapole_walk_decisions(built):
    """The hexadecapole walk's accepted cells against its rules, restated
    apart from the walk: every cell and softened cell of a bucket holds
    more than 6 particles and its theta sphere misses the bucket's box
    (gravity.h:597-633), and the two lists split on openSoftening
    (gravity.h:251-260: the cell's and the bucket's spheres of twice their
    softening meet, or the cell's meets the bucket's box): true for every
    softened cell, false for every cell.  (Parents are not checked: there a
    local node is opened for every bucket below it when the monopole sphere
    meets its box, gravity.h:705-717.)"""
    p = ics.plummer(8192, ics.rng_for(0), soft=0.3)
    theta = 0.7
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=theta, order=4)
    g, bb, cnt = L.meta["node_geom"], L.meta["node_bbox"], L.meta["count"]
    bnode = L.meta["bucket_node"]

    def box_d2(c, buckets):
        box = bb[bnode[buckets]]
        d = np.maximum(np.maximum(box[:, :3] - c, c - box[:, 3:]), 0.0)
        return (d * d).sum(1)

    for req, soft_expected in ((L.cells, False), (L.softcells, True)):
        assert req.n_entries > 0
        idx = req.list[:, 0]
        b = np.repeat(req.bucket_ids, np.diff(req.markers))
        c = g[idx, :3]
        r = np.maximum(2.0 / np.sqrt(3.0) * g[idx, 3] / theta, g[idx, 3])
        assert (cnt[idx] > 6).all()
        assert (box_d2(c, b) > r * r * (1.0 - 1e-12)).all()
        rs, rb = 2.0 * g[idx, 4], 2.0 * g[bnode[b], 4]
        soft = (((c - g[bnode[b], :3]) ** 2).sum(1) <= (rs + rb) ** 2) | (box_d2(c, b) <= rs * rs)
        assert (soft == soft_expected).all()


@pytest.mark.parametrize("case", ["open", "periodic"])
def test_tree_nodes_follow_reference_rules(built, case):
    """The host build's nodes against ChaNGa's rules, restated apart from
    the build: a node is a bucket when it holds nBucket particles or fewer
    (Compute.cpp:2476-2482, no node reaching the depth limit here), its box
    is the tight box of its particles, its centre of mass the mass-weighted
    mean; a bucket of several distinct particles takes the distance from
    its centre of mass to its farthest particle as its radius
    (GenericTreeNode.h:219-256, MultipoleMoments.h:487-504), an internal
    node the distance to its box's farthest corner (Compute.cpp:2576,
    MultipoleMoments.h:460-471).  (A one-particle bucket keeps half the
    diagonal of its spatial cell, which is not exported.)  The softening is
    the mass-weighted mean and the second moments are raw, sum m dx dx about
    the centre of mass, not trace-free (MultipoleMoments.h:207-225,
    330-348); unequal masses and softenings keep each rule distinct."""
    if case == "open":
        p, kw, nb = ics.plummer(8192, ics.rng_for(0), soft=0.01), {}, 16
    else:
        p, kw, nb = ics.nfw_halos(16384, ics.rng_for(3), soft=1e-3), dict(period=1.0), 8
    rng = np.random.Generator(np.random.PCG64(4))
    n = len(p["mass"])
    mass = rng.uniform(0.5, 1.5, n) / n
    soft = p["soft"] * rng.uniform(0.5, 5.0, n)
    L = tree.build_lists(p["pos"], mass, soft, n_bucket=nb, theta=0.7, **kw)
    g, bb, info = L.meta["node_geom"], L.meta["node_bbox"], L.meta["node_info"]
    first, count = L.meta["first"], L.meta["count"]
    pos, m = L.parts[:, 2:5], L.parts[:, 0]
    leaf = (info[:, 0] < 0) & (info[:, 1] < 0)  # an empty child is -1 as well
    live = count > 0
    assert set(np.where(leaf & live)[0]) == set(L.meta["bucket_node"])
    assert count[leaf & live].max() <= nb and count[~leaf & live].min() > nb
    for i in np.where(live)[0]:
        x, w = pos[first[i]:first[i] + count[i]], m[first[i]:first[i] + count[i]]
        assert np.array_equal(x.min(0), bb[i, :3]) and np.array_equal(x.max(0), bb[i, 3:])
        np.testing.assert_allclose(g[i, :3], (w[:, None] * x).sum(0) / w.sum(), rtol=1e-12,
                                   atol=1e-14)
        np.testing.assert_allclose(g[i, 5], w.sum(), rtol=1e-13)
        sf = L.parts[first[i]:first[i] + count[i], 1]
        np.testing.assert_allclose(g[i, 4], (w * sf).sum() / w.sum(), rtol=1e-13)
        dx = x - L.moments[i, 3:6]
        q = [(w * dx[:, a] * dx[:, b]).sum() for a, b in ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2),
                                                          (2, 2))]
        # the build accumulates child by child with parallel-axis shifts, so
        # its rounding scales with m |x|^2 about the origin, not with the
        # node's own trace (which a trace-free Q would miss by a third)
        tr = (w * (dx * dx).sum(1)).sum()
        tol = 1e-12 * (w * (x * x).sum(1)).sum()
        assert tol < 0.01 * tr or count[i] == 1 or tr == 0
        np.testing.assert_allclose(L.moments[i, 6:12], q, rtol=0, atol=tol + 1e-300)
        if leaf[i]:
            far = np.sqrt(((x - g[i, :3]) ** 2).sum(1).max())
            if count[i] > 1 and far > 0:
                np.testing.assert_allclose(g[i, 3], far, rtol=1e-13)
            else:
                assert g[i, 3] > 0
        else:
            d = np.maximum(g[i, :3] - bb[i, :3], bb[i, 3:] - g[i, :3])
            np.testing.assert_allclose(g[i, 3], np.sqrt((d * d).sum()), rtol=1e-13)
