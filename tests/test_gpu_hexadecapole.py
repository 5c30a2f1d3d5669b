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
from helpers import force_rel_err, pot_rel_err

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
