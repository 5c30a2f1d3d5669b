"""The CPU oracle: the restated port against ChaNGa's own CPU force code and
against the committed golden fixtures (which that code produced)."""
import numpy as np
import pytest

import oracle
from changa_gb300 import ics, tree
from helpers import FIXTURES, load_golden, lists_from_golden
import sys, os
sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_golden import list_digest  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


@pytest.mark.parametrize("name", FIXTURES)
def test_port_matches_golden(name):
    g = load_golden(name)
    L = lists_from_golden(g)
    assert list_digest(L) == str(g["digest"]), "host tree/walk changed the lists"
    per = float(g["period"])
    v = oracle.cell_forces(L.moments, L.parts, L.cells, fperiod=per, kind="port")
    v = oracle.part_forces(L.parts, L.parts, L.plist, fperiod=per, vars=v, kind="port")
    rows = g["rows"]
    # the golden came from gravity.h itself; the port is the same arithmetic
    np.testing.assert_allclose(v[rows], g["tree_vars"], rtol=1e-13, atol=1e-300)
    if "ewald_vars" in g:
        cut, hcut = g["ewald_cfg"]
        ew = oracle.ewald_forces(L.parts, L.root, per, 1, cut, hcut, idx=rows, kind="port")
        np.testing.assert_allclose(ew, g["ewald_vars"], rtol=1e-12, atol=1e-15)
        tb = oracle.ewald_table(L.root, per, hcut, kind="port")
        np.testing.assert_allclose(tb, g["ewt"], rtol=1e-14, atol=1e-300)


@pytest.mark.skipif(not oracle.available("ref"), reason="reference sources not built here")
@pytest.mark.parametrize("period,bucket,theta", [(0.0, 16, 0.7), (0.0, 8, 0.4), (1.0, 16, 0.7)])
def test_port_bitexact_vs_reference(period, bucket, theta):
    rng = ics.rng_for(7)
    if period:
        p = ics.lattice_grf(12, rng)
    else:
        p = ics.plummer(3000, rng, soft=0.03)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=bucket, theta=theta, period=period)
    out = {}
    for kind in ("port", "ref"):
        v = oracle.cell_forces(L.moments, L.parts, L.cells, fperiod=period, kind=kind)
        v = oracle.part_forces(L.parts, L.parts, L.plist, fperiod=period, vars=v, kind=kind)
        if period:
            v = oracle.ewald_forces(L.parts, L.root, period, 1, 2.6, 2.8, vars=v, kind=kind)
        out[kind] = v
    assert np.array_equal(out["port"], out["ref"])


def test_two_body_known_answer():
    """Unit masses at distance 1, far outside softening: a = +-1, pot = -1
    (partBucketForce, gravity.h:267-303)."""
    parts = np.array([[1.0, 1e-3, 0.0, 0.0, 0.0], [1.0, 1e-3, 1.0, 0.0, 0.0]])
    code = (3 | 3 << 3 | 3 << 6) << 22  # replica (0, 0, 0)
    req = tree.ListRequest(np.array([[1, code], [0, code]], np.int32), np.array([0, 1, 2], np.int32),
                           np.array([0, 1], np.int32), np.array([1, 1], np.int32),
                           np.array([0, 1], np.int32))
    v = oracle.part_forces(parts, parts, req)
    np.testing.assert_allclose(v[0, :4], [1.0, 0.0, 0.0, -1.0], rtol=1e-15)
    np.testing.assert_allclose(v[1, :4], [-1.0, 0.0, 0.0, -1.0], rtol=1e-15)
    np.testing.assert_allclose(v[:, 4], [2.0, 2.0], rtol=1e-15)


def test_spline_branches_continuous():
    """The softened pair force is continuous across u = 1 and r = twoh."""
    twoh = 0.1
    r = np.array([0.05 * (1 - 1e-9), 0.05 * (1 + 1e-9), 0.1 * (1 - 1e-9), 0.1 * (1 + 1e-9)])
    a, b = oracle.spline_ab(r * r, np.full(4, twoh))
    assert abs(a[0] - a[1]) < 1e-6 * a[0] and abs(b[0] - b[1]) < 1e-6 * b[0]
    assert abs(a[2] - a[3]) < 1e-6 * a[2] and abs(b[2] - b[3]) < 1e-6 * b[2]


def test_tree_force_accuracy_vs_direct_sum():
    """theta = 0.7 quadrupole tree forces are within the expected ~1e-3 of an
    FP64 direct sum (median), on the oracle."""
    rng = ics.rng_for(8)
    p = ics.plummer(8192, rng, soft=0.01)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7)
    v = oracle.cell_forces(L.moments, L.parts, L.cells)
    v = oracle.part_forces(L.parts, L.parts, L.plist, vars=v)
    idx = rng.choice(L.n, 200, replace=False)
    acc, pot = oracle.direct_sum(L.parts, idx)
    err = np.linalg.norm(v[idx, :3] - acc, axis=1) / np.linalg.norm(acc, axis=1)
    assert np.median(err) < 3e-3
    assert np.percentile(err, 99) < 3e-2
    assert np.median(np.abs(v[idx, 3] - pot) / np.abs(pot)) < 1e-3


def test_plummer_sphere_analytic_profile():
    """A Plummer sphere (a = 1, M = 1, G = 1, truncated at r = 20 and
    renormalised, as ics.plummer draws it) against its analytic profile:
    shell means of the tree's radial acceleration follow -G M(<r) / r^2 =
    -r / (1 + r^2)^(3/2) / f, and of its potential
    -(1 / sqrt(1 + r^2) - (1 + 20^2)^(-3/2)) / f, with f = 20^3 / 401^(3/2)
    the mass fraction inside the truncation.  Measured (32768 particles,
    theta 0.7): radial force within 0.5% over 0.6 < r < 8, potential within
    0.3% over 0.2 < r < 8; the bounds leave room for the enclosed-mass noise
    of the inner shells."""
    p = ics.plummer(32768, ics.rng_for(14), soft=0.01, velocities=False)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7)
    v = oracle.cell_forces(L.moments, L.parts, L.cells)
    v = oracle.part_forces(L.parts, L.parts, L.plist, vars=v)
    x = L.parts[:, 2:5]
    r = np.linalg.norm(x, axis=1)
    f = 20.0 ** 3 / 401.0 ** 1.5
    a_r = (v[:, :3] * x).sum(1) / r
    a_ana = -r / (1.0 + r * r) ** 1.5 / f
    phi_ana = -(1.0 / np.sqrt(1.0 + r * r) - 401.0 ** -1.5) / f
    edges = np.geomspace(0.2, 8.0, 11)
    for lo, hi in zip(edges[:-1], edges[1:]):
        s = (r >= lo) & (r < hi)
        assert abs(v[s, 3].mean() / phi_ana[s].mean() - 1.0) < 0.01, (lo, hi)
        if lo >= 0.6:
            assert abs(a_r[s].mean() / a_ana[s].mean() - 1.0) < 0.03, (lo, hi)


def test_ewald_single_particle_no_self_force():
    """A single particle in a periodic box feels no net force from its own
    replicas (tree replicas + Ewald correction cancel by symmetry)."""
    p = dict(pos=np.array([[0.3, 0.6, 0.45]]), mass=np.array([1.0]), soft=np.array([1e-3]))
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0)
    v = oracle.cell_forces(L.moments, L.parts, L.cells, fperiod=1.0)
    v = oracle.part_forces(L.parts, L.parts, L.plist, fperiod=1.0, vars=v)
    v = oracle.ewald_forces(L.parts, L.root, 1.0, 1, 2.6, 2.8, vars=v)
    assert np.abs(v[0, :3]).max() < 1e-6


def test_perfect_lattice_known_answer():
    """A perfect periodic lattice (8^3) feels no net force, and every
    particle sees the same potential, by symmetry.  The tree over one
    replica shell plus the Ewald term (ChaNGa's algorithm, run by the
    oracle) leaves a residual that falls with theta until the root-moment
    expansion the Ewald term uses for the replicas beyond the first shell,
    which theta does not refine, is what remains: 0.40 of a neighbour's
    force m/h^2 at theta 0.7, 0.019 at 0.2."""
    m, h = 1.0 / 512, 1.0 / 8
    res = {}
    for theta in (0.7, 0.2):
        p = ics.lattice_grf(8, ics.rng_for(1), rms_frac=0.0)
        L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=theta, period=1.0)
        v = oracle.cell_forces(L.moments, L.parts, L.cells, fperiod=1.0)
        v = oracle.part_forces(L.parts, L.parts, L.plist, fperiod=1.0, vars=v)
        v = oracle.ewald_forces(L.parts, L.root, 1.0, 1, 2.6, 2.8, vars=v)
        a = np.linalg.norm(v[:, :3], axis=1) / (m / h ** 2)
        res[theta] = (a.max(), np.ptp(v[:, 3]) / (m / h))
    assert res[0.7][0] < 0.5
    assert res[0.2][0] < 0.03 and res[0.2][1] < 0.06
    assert res[0.2][0] < 0.1 * res[0.7][0]


def _hex_lists(n=8192, soft=0.3, seed=3):
    from changa_gb300 import ics, tree
    p = ics.plummer(n, ics.rng_for(seed))
    p["soft"][:] = soft
    return tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, order=4)


@pytest.mark.skipif(not os.path.exists(oracle.REF_HEX_LIB), reason="reference not built here")
def test_hex_port_bitexact_vs_reference(built):
    """The port's hexadecapole cell evaluation (momEvalFmomrcm and the
    openSoftening point-mass path) is bit-identical to the reference's own
    gravity.h + moments.c built with HEXADECAPOLE, on both lists the
    hexadecapole walk emits."""
    L = _hex_lists()
    assert L.cells.n_entries > 0 and L.softcells.n_entries > 0
    for req in (L.cells, L.softcells):
        g = oracle.bucket_geometry(L, req)
        a = oracle.cell_forces_hex(L.moments, L.parts, req, g, kind="port")
        b = oracle.cell_forces_hex(L.moments, L.parts, req, g, kind="ref")
        assert np.array_equal(a, b)


def test_hex_more_accurate_than_quadrupole(built):
    """Same tree, same opening angle: the hexadecapole evaluation sits an
    order of magnitude closer to the direct sum than the quadrupole one."""
    from changa_gb300 import ics, tree
    p = ics.plummer(16384, ics.rng_for(0), soft=0.01)
    idx = np.random.default_rng(0).choice(16384, 256, replace=False)
    med = {}
    for order in (2, 4):
        L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, order=order)
        if order == 4:
            v = oracle.cell_forces_hex(L.moments, L.parts, L.cells, oracle.bucket_geometry(L, L.cells))
            if L.softcells.n_buckets:
                v = oracle.cell_forces_hex(L.moments, L.parts, L.softcells,
                                           oracle.bucket_geometry(L, L.softcells), vars=v)
        else:
            v = oracle.cell_forces(L.moments, L.parts, L.cells)
        v = oracle.part_forces(L.parts, L.parts, L.plist, vars=v)
        gi = np.argsort(L.perm)[idx]
        acc, _ = oracle.direct_sum(L.parts, gi)
        e = np.linalg.norm(v[gi, :3] - acc, axis=1) / np.linalg.norm(acc, axis=1)
        med[order] = np.median(e)
    assert med[4] < med[2] / 4 and med[4] < 3e-4, med


@pytest.mark.skipif(not os.path.exists(oracle.REF_HEX_LIB), reason="reference not built here")
def test_hex_ewald_port_bitexact_vs_reference(built):
    """The port's hexadecapole Ewald (EwaldInit's complete root moments and
    h-table, BucketEwald to fourth order) is bit-identical to the reference's
    Ewald.cpp built with HEXADECAPOLE, on a clustered periodic root with
    sizeable octupole and hexadecapole moments."""
    p = ics.nfw_halos(16384, ics.rng_for(2), soft=1e-3)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         order=4)
    root = L.moments[0]
    tp, mp = oracle.ewald_table_hex(root, 1.0, 2.8, kind="port")
    tr, mr = oracle.ewald_table_hex(root, 1.0, 2.8, kind="ref")
    assert np.array_equal(tp, tr) and np.array_equal(mp, mr)
    assert np.abs(tr[:, 4]).max() > 0
    idx = np.arange(0, L.n, 61).astype(np.int32)
    a = oracle.ewald_forces_hex(L.parts, root, 1.0, 1, 2.6, 2.8, idx=idx, kind="port")
    b = oracle.ewald_forces_hex(L.parts, root, 1.0, 1, 2.6, 2.8, idx=idx, kind="ref")
    assert np.array_equal(a, b)


def test_hex_ewald_single_particle_no_self_force():
    """Hexadecapole build: a lone particle feels no force from its own
    replicas, tree replicas plus the Ewald correction."""
    p = dict(pos=np.array([[0.3, 0.6, 0.45]]), mass=np.array([1.0]), soft=np.array([1e-3]))
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         order=4)
    v = np.zeros((1, 5))
    for req in (L.cells, L.softcells):
        if req.n_buckets:
            v = oracle.cell_forces_hex(L.moments, L.parts, req, oracle.bucket_geometry(L, req),
                                       fperiod=1.0, vars=v)
    v = oracle.part_forces(L.parts, L.parts, L.plist, fperiod=1.0, vars=v)
    v = oracle.ewald_forces_hex(L.parts, L.moments[0], 1.0, 1, 2.6, 2.8, vars=v)
    assert np.abs(v[0, :3]).max() < 1e-6
