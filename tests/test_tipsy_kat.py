"""Tipsy reader, and the reference's own known answer for its test model
(teststep/king_soft.bin, the 36000-particle King model; teststep/
pkdtest.log line 36 gives T = 32.65580 and U = -64.84776 at t = 0 from
PKDGRAV with hexadecapole moments, nBucket 8, theta 0.7, open boundaries).
T checks the reader exactly; U is a loose check of the quadrupole tree and
the oracle's force arithmetic on real data.  The model file is only read
where the reference tree exists."""
import os

import numpy as np
import pytest

from changa_gb300 import tipsy
from helpers import reference_root

_REF = reference_root()
KING = os.path.join(_REF, "teststep", "king_soft.bin") if _REF else ""


def test_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    n = 100
    pos, vel = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    mass, soft = rng.uniform(1, 2, n) / n, np.full(n, 0.01)
    p = tmp_path / "t.bin"
    tipsy.write(str(p), pos, vel, mass, soft, time=0.5)
    d = tipsy.read(str(p))
    assert d["n"] == n and d["ndark"] == n and d["time"] == 0.5
    np.testing.assert_allclose(d["pos"], pos.astype(np.float32), rtol=0, atol=0)
    np.testing.assert_allclose(d["soft"], np.float32(0.01))


@pytest.mark.skipif(not KING or not os.path.exists(KING),
                    reason="reference test data not present (set CHANGA_REFERENCE)")
def test_king_model_energies(built):
    import oracle
    from changa_gb300 import tree
    d = tipsy.read(KING)
    assert d["n"] == 36000 and d["ndark"] == 36000
    T = 0.5 * (d["mass"] * (d["vel"] ** 2).sum(1)).sum()
    assert abs(T / 32.65580 - 1) < 2e-6, T
    L = tree.build_lists(d["pos"], d["mass"], d["soft"], n_bucket=8, theta=0.7)
    v = oracle.cell_forces(L.moments, L.parts, L.cells)
    v = oracle.part_forces(L.parts, L.parts, L.plist, vars=v)
    U = 0.5 * (L.parts[:, 0] * v[:, 3]).sum()
    assert abs(U / -64.84776 - 1) < 2e-4, U  # measured 4.0e-5


@pytest.mark.skipif(not KING or not os.path.exists(KING),
                    reason="reference test data not present (set CHANGA_REFERENCE)")
def test_king_model_integration_energy(built):
    """The reference's integrator test (teststep/Makefile:8): the King model
    integrated to t = 1 keeps its total energy at -32.19 +- 0.005
    (teststep/README: 10 big steps of 0.1, about one central dynamical
    time).  ChaNGa runs it with multistepping; here a kick-drift-kick with
    a global step of 0.05 over the quadrupole tree (nBucket 8, theta 0.7)
    rebuilt every step, with the oracle's force arithmetic, meets the same
    criterion (measured: E(1) = -32.18945, drift under 1e-3 throughout)."""
    import oracle
    from changa_gb300 import tree
    d = tipsy.read(KING)
    x, v = d["pos"].astype(np.float64), d["vel"].astype(np.float64)
    m, s = d["mass"].astype(np.float64), d["soft"].astype(np.float64)

    def accel(x):
        L = tree.build_lists(x, m, s, n_bucket=8, theta=0.7)
        w = oracle.cell_forces(L.moments, L.parts, L.cells)
        w = oracle.part_forces(L.parts, L.parts, L.plist, vars=w)
        a, pot = np.empty((len(x), 3)), np.empty(len(x))
        a[L.perm], pot[L.perm] = w[:, :3], w[:, 3]
        return a, pot

    def energy(pot):
        return 0.5 * (m * (v ** 2).sum(1)).sum() + 0.5 * (m * pot).sum()

    dt, sub = 0.05, 2
    a, pot = accel(x)
    e0 = energy(pot)
    for k in range(10 * sub):
        v += 0.5 * dt * a
        x += dt * v
        a, pot = accel(x)
        v += 0.5 * dt * a
        if (k + 1) % sub == 0:
            assert abs(energy(pot) - e0) < 2e-3, (k, energy(pot), e0)
    assert abs(energy(pot) + 32.19) < 0.005, energy(pot)


@pytest.mark.skipif(not KING or not os.path.exists(KING),
                    reason="reference test data not present (set CHANGA_REFERENCE)")
def test_king_model_direct_energy(built):
    """pkdtest.log's U = -64.84776 at t = 0 (PKDGRAV) against the exact
    potential energy of the model as the reader returns it: an FP64 direct
    sum over all 36000 x 35999 / 2 pairs with the P-P spline softening and
    the per-particle softenings of the file.  They agree to 6.7e-6 (the
    last digits of the log and PKDGRAV's own expansion error); the
    quadrupole tree (nBucket 8, theta 0.7) sits 3.3e-5 from the exact
    value."""
    import oracle
    from changa_gb300 import tree
    d = tipsy.read(KING)
    L = tree.build_lists(d["pos"], d["mass"], d["soft"], n_bucket=8, theta=0.7)
    U = oracle.direct_energy(L.parts)
    assert abs(U / -64.84776 - 1) < 2e-5, U
    v = oracle.cell_forces(L.moments, L.parts, L.cells)
    v = oracle.part_forces(L.parts, L.parts, L.plist, vars=v)
    U_tree = 0.5 * (L.parts[:, 0] * v[:, 3]).sum()
    assert abs(U_tree / U - 1) < 1e-4, (U_tree, U)
