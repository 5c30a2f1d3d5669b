"""The hexadecapole build (ChaNGa's default configuration) on the GPU: FP64
and FP32-mixed forms against the oracle (the port, itself bit-identical to
the reference's gravity.h + moments.c built with HEXADECAPOLE), including
the softened cells evaluated as point masses, and its accuracy against the
direct sum next to the quadrupole build."""
import numpy as np
import pytest

import oracle
from changa_gb300 import _native as N
from changa_gb300 import gravity, ics, tree
from helpers import force_rel_err, force_rms_err, pot_rel_err

pytestmark = pytest.mark.gpu


def _oracle_hex(L):
    v = oracle.cell_forces_hex(L.moments, L.parts, L.cells, oracle.bucket_geometry(L, L.cells))
    if L.softcells.n_buckets:
        v = oracle.cell_forces_hex(L.moments, L.parts, L.softcells,
                                   oracle.bucket_geometry(L, L.softcells), vars=v)
    return oracle.part_forces(L.parts, L.parts, L.plist, vars=v)


@pytest.mark.parametrize("soft,n_bucket", [(0.01, 16), (0.3, 16), (0.05, 32)])
def test_hex_forms_match_oracle(cuda_ok, soft, n_bucket):
    p = ics.plummer(32768, ics.rng_for(0))
    p["soft"][:] = soft
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=n_bucket, theta=0.7, order=4)
    if soft >= 0.3:
        assert L.softcells.n_entries > 0
    ref = _oracle_hex(L)
    ds = gravity.DeviceSystem(L)
    v64 = ds.step("fp64").cpu().numpy()
    assert force_rel_err(v64, ref).max() < 1e-6
    assert pot_rel_err(v64, ref).max() < 1e-6
    np.testing.assert_allclose(v64[:, 4], ref[:, 4], rtol=1e-6)
    lib = N.cuda_lib()
    default = lib.changa_gb300_get_hex_variant()
    try:
        # every shape of the mixed hexadecapole cell kernel: synchronous
        # staging (0) and the paired .f32x2 kernel at 1 and 2 blocks per SM
        for variant in (0, 1, 2):
            N.check(lib.changa_gb300_set_hex_variant(variant), "set_hex_variant")
            vmx = ds.step("mixed").cpu().numpy()
            e = force_rel_err(vmx, ref)
            print("hex soft %g variant %d: fp64 max %.2e, mixed median %.2e p99 %.2e" % (
                soft, variant, force_rel_err(v64, ref).max(), np.median(e),
                np.percentile(e, 99)))
            assert np.median(e) < 2e-6 and np.percentile(e, 99) < 1e-4
            assert np.median(pot_rel_err(vmx, ref)) < 2e-6
            np.testing.assert_allclose(vmx[:, 4], ref[:, 4], rtol=2e-5)
    finally:
        lib.changa_gb300_set_hex_variant(default)


def test_hex_closer_to_direct_sum_than_quadrupole(cuda_ok):
    p = ics.plummer(65536, ics.rng_for(4))
    idx = np.random.default_rng(9).choice(65536, 2048, replace=False)
    med = {}
    for order in (2, 4):
        L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, order=order)
        ds = gravity.DeviceSystem(L)
        v = ds.step("mixed").cpu().numpy()
        gi = np.argsort(L.perm)[idx].astype(np.int32)
        ref = gravity.direct_forces(ds.parts, gi)
        e = np.linalg.norm(v[gi, :3] - ref[:, :3], axis=1) / np.linalg.norm(ref[:, :3], axis=1)
        med[order] = float(np.median(e))
        print("plummer64k theta 0.7 order %d: median %.2e p99 %.2e" % (
            order, med[order], np.percentile(e, 99)))
    assert med[4] < med[2] / 4


def _f32(a):
    return np.asarray(a, np.float32).astype(np.float64)


def _dropin_reference(L, ewald=None):
    """What the HEXADECAPOLE drop-in computes, by the oracle on the FP32
    inputs it receives: the cell list (cells whose softening misses the
    bucket; ChaNGa evaluates the softened ones on the CPU) with
    momEvalFmomrcm, the particle list, and the hexadecapole Ewald term."""
    mom, parts = _f32(L.moments), _f32(L.parts)
    v = oracle.cell_forces_hex(mom, parts, L.cells, oracle.bucket_geometry(L, L.cells),
                               fperiod=L.period)
    v = oracle.part_forces(parts, parts, L.plist, fperiod=L.period, vars=v)
    if ewald is not None:
        v = oracle.ewald_forces_hex(parts, L.moments[0], ewald.L, ewald.n_reps, ewald.fEwCut,
                                    ewald.dEwhCut, vars=v)
    return v


def test_hex_dropin_matches_oracle(cuda_ok):
    """The boundary of ChaNGa's hexadecapole build (libchanga_gb300_hex.so:
    108-byte CudaMultipoleMoments through DataManagerTransferLocalTree and
    TreePieceCellListDataTransferLocal) against the oracle."""
    p = ics.plummer(32768, ics.rng_for(0), soft=0.01)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, order=4)
    ref = _dropin_reference(L)
    inp = gravity.DropInInputs(L)
    try:
        assert inp.moments.nbytes == 108 * L.moments.shape[0]
        v = gravity.dropin_step(inp).astype(np.float64)
    finally:
        inp.free()
    e = force_rel_err(v, ref)
    print("hex drop-in: median %.2e p99 %.2e" % (np.median(e), np.percentile(e, 99)))
    assert np.median(e) < 2e-6 and np.percentile(e, 99) < 1e-4
    assert np.median(pot_rel_err(v, ref)) < 2e-6
    np.testing.assert_allclose(v[:, 4], ref[:, 4], rtol=1e-4)


def test_hex_dropin_ewald(cuda_ok):
    """EwaldHost of the hexadecapole build (the root's complete moments in
    EwaldReadOnlyData.momcRoot, octupole sine terms in the h-table) on a
    clustered periodic box, with the tree replicas, against the oracle."""
    p = ics.nfw_halos(32768, ics.rng_for(2), soft=1e-3)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         order=4)
    ew = gravity.EwaldConfig(1.0, 1, 2.6, 2.8)
    ref = _dropin_reference(L, ew)
    inp = gravity.DropInInputs(L, ewald=ew)
    try:
        v = gravity.dropin_step(inp).astype(np.float64)
    finally:
        inp.free()
    e = force_rms_err(v, ref)
    dpot = np.abs(v[:, 3] - ref[:, 3])
    # the quadrupole build's drop-in on the same box, for scale
    Lq = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0)
    mq, pq = _f32(Lq.moments), _f32(Lq.parts)
    refq = oracle.cell_forces(mq, pq, Lq.cells, fperiod=1.0)
    refq = oracle.part_forces(pq, pq, Lq.plist, fperiod=1.0, vars=refq)
    refq = oracle.ewald_forces(pq, _f32(Lq.root), 1.0, 1, 2.6, 2.8, vars=refq)
    inq = gravity.DropInInputs(Lq, ewald=ew)
    try:
        vq = gravity.dropin_step(inq).astype(np.float64)
    finally:
        inq.free()
    dpot_q = np.abs(vq[:, 3] - refq[:, 3])
    worst = int(np.argmax(dpot))
    r2 = ((L.parts[worst, 2:5] - L.moments[0, 3:6]) ** 2).sum()
    print("hex drop-in with Ewald: median %.2e max %.2e; pot max %.2e (r^2 to the root %.2e), "
          "quadrupole build pot max %.2e" % (np.median(e), e.max(), dpot.max(), r2, dpot_q.max()))
    # FP32 rounding of O(10) hole and replica terms of size G M / L = 1
    # against the rms force, as for the quadrupole drop-in
    assert np.median(e) < 5e-5 and e.max() < 2e-3
    # the potential carries the reference's single-precision two-term series
    # inside fInner2 = 1.1e-2 L^2 (Ewald.cpp:508-516), where the dropped
    # (alpha r)^4 term of g0 alone reaches ka (alpha r)^4 / 10 = 4.5e-4 of
    # G M / L; the oracle (CPU constants) switches at 1.2e-3 L^2
    assert dpot.max() < 1e-3 and dpot_q.max() < 1e-3


def test_hex_forms_with_ewald(cuda_ok):
    """changa_gravity_step_hexa with its Ewald term (the root's complete
    moments to fourth order) on a clustered periodic box: the FP64 form
    against the oracle per particle, the FP32-mixed form as the quadrupole
    mixed Ewald is measured (rms|a| and G M / L units)."""
    p = ics.nfw_halos(32768, ics.rng_for(2), soft=1e-3)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         order=4)
    ew = gravity.EwaldConfig(1.0, 1, 2.6, 2.8)
    ref = np.zeros((L.n, 5))
    for req in (L.cells, L.softcells):
        if req.n_buckets:
            ref = oracle.cell_forces_hex(L.moments, L.parts, req, oracle.bucket_geometry(L, req),
                                         fperiod=1.0, vars=ref)
    ref = oracle.part_forces(L.parts, L.parts, L.plist, fperiod=1.0, vars=ref)
    ref = oracle.ewald_forces_hex(L.parts, L.moments[0], 1.0, 1, 2.6, 2.8, vars=ref)
    ds = gravity.DeviceSystem(L, ewald=ew)
    v64 = ds.step("fp64").cpu().numpy()
    e64 = force_rel_err(v64, ref)
    vmx = ds.step("mixed").cpu().numpy()
    e = force_rms_err(vmx, ref)
    print("hex + Ewald: fp64 max %.2e, pot max %.2e; mixed rms median %.2e max %.2e, rel median "
          "%.2e, pot max %.2e" % (e64.max(), np.abs(v64[:, 3] - ref[:, 3]).max(), np.median(e),
                                  e.max(), np.median(force_rel_err(vmx, ref)),
                                  np.abs(vmx[:, 3] - ref[:, 3]).max()))
    assert e64.max() < 1e-6
    assert np.abs(v64[:, 3] - ref[:, 3]).max() < 1e-9
    assert np.median(e) < 5e-5 and e.max() < 2e-3
    assert np.median(force_rel_err(vmx, ref)) < 1e-4
    assert np.abs(vmx[:, 3] - ref[:, 3]).max() < 5e-5


def test_hex_two_replica_layers_with_ewald(cuda_ok):
    """The hexadecapole build over two replica layers (5^3 replica roots)
    with its Ewald term at nReps = 2: the FP64 form against the oracle, the
    FP32-mixed form against the FP64 oracle."""
    p = ics.nfw_halos(16384, ics.rng_for(11), soft=1e-3)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         n_replicas=2, order=4)
    ew = gravity.EwaldConfig(1.0, 2, 2.6, 2.8)
    ref = np.zeros((L.n, 5))
    for req in (L.cells, L.softcells):
        if req.n_buckets:
            ref = oracle.cell_forces_hex(L.moments, L.parts, req, oracle.bucket_geometry(L, req),
                                         fperiod=1.0, vars=ref)
    ref = oracle.part_forces(L.parts, L.parts, L.plist, fperiod=1.0, vars=ref)
    ref = oracle.ewald_forces_hex(L.parts, L.moments[0], 1.0, 2, 2.6, 2.8, vars=ref)
    ds = gravity.DeviceSystem(L, ewald=ew)
    v64 = ds.step("fp64").cpu().numpy()
    vmx = ds.step("mixed").cpu().numpy()
    e64, e = force_rel_err(v64, ref), force_rms_err(vmx, ref)
    print("hex two replica layers: fp64 max %.2e; mixed rms median %.2e max %.2e" % (
        e64.max(), np.median(e), e.max()))
    assert e64.max() < 1e-6
    assert np.median(e) < 5e-5 and e.max() < 2e-3
