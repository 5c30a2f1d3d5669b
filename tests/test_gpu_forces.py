"""GPU parity: every form of the list kernels and the Ewald kernels against
the CPU oracle on the same lists (and against the committed fixtures that
ChaNGa's own CPU code produced)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from changa_gb300 import _native as N
from changa_gb300 import gravity, ics, tree
from changa_gb300.walk import gpu_walk
from helpers import (FIXTURES, force_rel_err, force_rms_err, load_golden, lists_from_golden,
                     pot_rel_err, pot_rms_err)

pytestmark = pytest.mark.gpu

# Tolerances (per particle, |da|/|a| and |dpot|/|pot|):
FP64_TOL = 1e-6        # the plain FP64 form (stated bar: 1e-6 relative)
F32_MEDIAN_TOL = 2e-6  # FP32 drop-in vs FP64 oracle on the same FP32 inputs
F32_P99_TOL = 1e-4
MIX_MEDIAN_TOL = 2e-6  # FP32-mixed vs the FP64 form
MIX_P99_TOL = 1e-4


def oracle_vars(L, period=0.0, ewald=None, f32_inputs=False):
    mom, parts = L.moments, L.parts
    if f32_inputs:
        mom = mom.astype(np.float32).astype(np.float64)
        parts = parts.astype(np.float32).astype(np.float64)
    v = oracle.cell_forces(mom, parts, L.cells, fperiod=period)
    v = oracle.part_forces(parts, parts, L.plist, fperiod=period, vars=v)
    if ewald is not None:
        root = L.root if not f32_inputs else L.root.astype(np.float32).astype(np.float64)
        v = oracle.ewald_forces(parts, root, ewald.L, ewald.n_reps, ewald.fEwCut, ewald.dEwhCut,
                                vars=v)
    return v


@pytest.fixture(scope="module")
def plummer(cuda_ok):
    p = ics.plummer(32768, ics.rng_for(0), soft=0.01)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7)
    return L, oracle_vars(L), oracle_vars(L, f32_inputs=True)


@pytest.fixture(scope="module")
def lattice(cuda_ok):
    p = ics.lattice_grf(24, ics.rng_for(1))
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0)
    ew = gravity.EwaldConfig(1.0, 1, 2.6, 2.8)
    return L, ew, oracle_vars(L, 1.0, ew)


def test_fp64_form_matches_oracle(plummer):
    L, ref, _ = plummer
    before = N.cuda_lib().changa_gb300_kernel_launches()
    v = gravity.DeviceSystem(L).step("fp64").cpu().numpy()
    assert N.cuda_lib().changa_gb300_kernel_launches() > before
    assert force_rel_err(v, ref).max() < FP64_TOL
    assert pot_rel_err(v, ref).max() < FP64_TOL
    np.testing.assert_allclose(v[:, 4], ref[:, 4], rtol=FP64_TOL)


def test_fp32_dropin_matches_oracle(plummer):
    L, _, ref32 = plummer
    inp = gravity.DropInInputs(L)
    try:
        v = gravity.dropin_step(inp).astype(np.float64)
    finally:
        inp.free()
    e = force_rel_err(v, ref32)
    assert np.median(e) < F32_MEDIAN_TOL
    assert np.percentile(e, 99) < F32_P99_TOL
    assert np.median(pot_rel_err(v, ref32)) < F32_MEDIAN_TOL
    np.testing.assert_allclose(v[:, 4], ref32[:, 4], rtol=1e-4)


def test_mixed_form_matches_fp64(plummer):
    L, ref, _ = plummer
    v = gravity.DeviceSystem(L).step("mixed").cpu().numpy()
    e = force_rel_err(v, ref)
    assert np.median(e) < MIX_MEDIAN_TOL
    assert np.percentile(e, 99) < MIX_P99_TOL
    assert np.median(pot_rel_err(v, ref)) < MIX_MEDIAN_TOL


def test_mixed_form_far_from_origin(cuda_ok):
    """The FP32-mixed form keeps its accuracy for a system far from the
    origin: coordinates split into hi + lo and differences formed relative
    to the target bucket, so a Plummer sphere shifted by ~1e3 (where one
    FP32 coordinate resolves 6e-5, against a softening of 0.01) matches
    the FP64 oracle as closely as the same sphere at the origin."""
    p = ics.plummer(16384, ics.rng_for(12), soft=0.01)
    shift = np.array([1000.25, -3000.5, 777.125])
    errs = []
    for pos in (p["pos"], p["pos"] + shift):
        L = tree.build_lists(pos, p["mass"], p["soft"], n_bucket=16, theta=0.7)
        ref = oracle_vars(L)
        v = gravity.DeviceSystem(L).step("mixed").cpu().numpy()
        e = force_rel_err(v, ref)
        assert np.median(e) < MIX_MEDIAN_TOL and np.percentile(e, 99) < MIX_P99_TOL
        assert np.median(pot_rel_err(v, ref)) < MIX_MEDIAN_TOL
        errs.append(np.median(e))
    assert errs[1] < 3.0 * errs[0]


def test_host_entry_matches_device_entry(plummer):
    L, ref, _ = plummer
    v = gravity.gravity_step_host(L, "fp64")
    assert force_rel_err(v, ref).max() < FP64_TOL


def test_host_entry_pipelined_chunks(plummer, lattice):
    """Host-array entry with the lists uploaded in many small chunks (cell
    and particle lists, with and without Ewald, accumulate and overwrite):
    bit-identical to the device-resident evaluation without Ewald, since
    every bucket is computed by the same kernel whichever chunk carries it
    (with Ewald the host entry adds the Ewald term first, so sums differ in
    their last bits)."""
    lib = N.cuda_lib()
    lib.changa_gb300_set_host_chunk_bytes(64 * 1024)
    try:
        for (L, ew) in ((plummer[0], None), (lattice[0], lattice[1])):
            for form in ("mixed", "fp64"):
                dev = gravity.DeviceSystem(L, ewald=ew).step(form).cpu().numpy()
                host = gravity.gravity_step_host(L, form, ewald=ew, overwrite=True)
                if ew is None:
                    assert np.array_equal(host, dev), form
                else:
                    np.testing.assert_allclose(host, dev, rtol=1e-12,
                                               atol=1e-13 * np.abs(dev).max())
                acc = gravity.gravity_step_host(L, form, ewald=ew, vars=np.ones((L.n, 5)))
                np.testing.assert_allclose(acc[:, :4], dev[:, :4] + 1.0, rtol=1e-12, atol=1e-12)
    finally:
        lib.changa_gb300_set_host_chunk_bytes(0)  # the default


def test_host_entry_particle_slices(cuda_ok):
    """The host entry uploads the particles in slices (a quarter chunk,
    started on multiples of 32) and gives each its Ewald term as it lands.
    Every warp of the Ewald kernel then holds the particles it holds in one
    launch over all, so the slicing changes no bit: a clustered periodic set
    of a particle count that is no multiple of 32, both forms, overwriting
    and accumulating, in slices of 96 particles against one slice."""
    lib = N.cuda_lib()
    p = ics.nfw_halos(20001, ics.rng_for(11), soft=1e-3)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         n_replicas=1)
    ew = gravity.EwaldConfig(1.0, 1, 2.6, 2.8)
    start = np.random.Generator(np.random.PCG64(3)).standard_normal((L.n, 5))
    for form in ("mixed", "fp64"):
        one = gravity.gravity_step_host(L, form, ewald=ew, overwrite=True)
        acc_one = gravity.gravity_step_host(L, form, ewald=ew, vars=start.copy())
        lib.changa_gb300_set_host_chunk_bytes(16 * 1024)  # 96-particle slices
        try:
            many = gravity.gravity_step_host(L, form, ewald=ew, overwrite=True)
            acc_many = gravity.gravity_step_host(L, form, ewald=ew, vars=start.copy())
        finally:
            lib.changa_gb300_set_host_chunk_bytes(0)  # the default
        assert np.array_equal(many, one), form
        assert np.array_equal(acc_many, acc_one), form


def _reordered(req, order):
    """The request with its buckets taken in `order` (a subset or a
    permutation of the bucket indices), entries moved with them."""
    seg = [req.list[req.markers[b]:req.markers[b + 1]] for b in order]
    lst = np.concatenate(seg) if seg else req.list[:0]
    markers = np.zeros(len(order) + 1, dtype=np.int32)
    markers[1:] = np.cumsum([len(x) for x in seg])
    return tree.ListRequest(np.ascontiguousarray(lst, dtype=np.int32), markers,
                            np.ascontiguousarray(req.starts[order]),
                            np.ascontiguousarray(req.sizes[order]),
                            np.ascontiguousarray(req.bucket_ids[order]))


def test_host_entry_early_readback(plummer, lattice):
    """Host-array entry into page-locked vars, where each chunk's particles
    are read back as soon as their last kernel is done: bit-identical to
    the device-resident evaluation for the particle list as built, for one
    with every other bucket dropped (particles no chunk writes), and for one
    with its buckets shuffled (overlapping chunk ranges: one read-back at
    the end), each chunked finely and with Ewald."""
    import dataclasses
    lib = N.cuda_lib()
    rng = np.random.Generator(np.random.PCG64(7))
    lib.changa_gb300_set_host_chunk_bytes(16 * 1024)
    try:
        for (L0, ew) in ((plummer[0], None), (lattice[0], lattice[1])):
            nb = L0.plist.n_buckets
            for order in (np.arange(nb), np.arange(0, nb, 2), rng.permutation(nb)):
                L = dataclasses.replace(L0, plist=_reordered(L0.plist, order))
                for form in ("mixed", "fp64"):
                    dev = gravity.DeviceSystem(L, ewald=ew).step(form).cpu().numpy()
                    out = gravity.PinnedArray(np.zeros((L.n, 5)))
                    try:
                        host = gravity.gravity_step_host(L, form, ewald=ew, vars=out.array,
                                                         overwrite=True)
                        if ew is None:
                            assert np.array_equal(host, dev), form
                        else:
                            np.testing.assert_allclose(host, dev, rtol=1e-12,
                                                       atol=1e-13 * np.abs(dev).max())
                        out.array[...] = 1.0
                        acc = gravity.gravity_step_host(L, form, ewald=ew, vars=out.array)
                        np.testing.assert_allclose(acc[:, :4], dev[:, :4] + 1.0, rtol=1e-12,
                                                   atol=1e-12)
                    finally:
                        out.free()
    finally:
        lib.changa_gb300_set_host_chunk_bytes(0)  # the default


@pytest.mark.parametrize("name", FIXTURES)
def test_fp64_form_matches_golden(cuda_ok, name):
    g = load_golden(name)
    L = lists_from_golden(g)
    per = float(g["period"])
    ew = None
    if "ewald_vars" in g:
        cut, hcut = g["ewald_cfg"]
        ew = gravity.EwaldConfig(per, 1, float(cut), float(hcut))
    v = gravity.DeviceSystem(L, ewald=ew).step("fp64").cpu().numpy()[g["rows"]]
    ref = g["tree_vars"] + (g["ewald_vars"] if ew else 0.0)
    if ew:
        ref[:, 4] = g["tree_vars"][:, 4]
    assert force_rel_err(v, ref).max() < FP64_TOL
    assert pot_rel_err(v, ref).max() < FP64_TOL


def test_ewald_forms(lattice):
    """Tree + Ewald on a perturbed periodic lattice.  The FP64 form matches
    the oracle per particle; FP32 forms are measured against rms|a| and
    rms(pot) because the net lattice force is a small residual of O(1)
    replica terms (the FP32 forms are still ~1e-5 relative per particle)."""
    L, ew, ref = lattice
    v64 = gravity.DeviceSystem(L, ewald=ew).step("fp64").cpu().numpy()
    assert force_rel_err(v64, ref).max() < FP64_TOL
    assert pot_rms_err(v64, ref).max() < FP64_TOL
    vmx = gravity.DeviceSystem(L, ewald=ew).step("mixed").cpu().numpy()
    e = force_rms_err(vmx, ref)
    # FP32 rounding of ~27 O(1) hole/replica terms against an rms force of
    # ~0.04: about 1e-6 absolute, 2e-5 of rms|a|
    assert np.median(e) < 5e-5 and e.max() < 2e-3
    assert np.median(force_rel_err(vmx, ref)) < 1e-4
    # the periodic potential of a near-uniform lattice (~3e-3) is the residual
    # of O(10) replica terms of size G M / L = 1: measure it in those units
    assert np.abs(vmx[:, 3] - ref[:, 3]).max() < 5e-5


def test_perfect_lattice_forms(cuda_ok):
    """A perfect periodic lattice (8^3, Ewald): every coordinate an exact
    float, both halves of each split equal across rows, and the net force
    only the residual of cancelling replica terms (zero by symmetry; about
    0.4 of a neighbour's force from ChaNGa's algorithm at theta 0.7).  The
    FP64 form equals the oracle to the 1e-6 bar of the rms force and the
    rms potential; the FP32-mixed form stays within the rounding of the
    O(1) terms, as on the perturbed lattice."""
    p = ics.lattice_grf(8, ics.rng_for(1), rms_frac=0.0)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0)
    ew = gravity.EwaldConfig(1.0, 1, 2.6, 2.8)
    ref = oracle_vars(L, 1.0, ew)
    v64 = gravity.DeviceSystem(L, ewald=ew).step("fp64").cpu().numpy()
    assert force_rms_err(v64, ref).max() < FP64_TOL
    assert pot_rms_err(v64, ref).max() < FP64_TOL
    vmx = gravity.DeviceSystem(L, ewald=ew).step("mixed").cpu().numpy()
    e = force_rms_err(vmx, ref)
    assert np.median(e) < 5e-5 and e.max() < 2e-3
    assert np.abs(vmx[:, 3] - ref[:, 3]).max() < 5e-5


def test_ewald_dropin(lattice):
    L, ew, _ = lattice
    ref32 = oracle_vars(L, 1.0, ew, f32_inputs=True)
    inp = gravity.DropInInputs(L, ewald=ew)
    try:
        v = gravity.dropin_step(inp).astype(np.float64)
    finally:
        inp.free()
    e = force_rms_err(v, ref32)
    # FP32 rounding of ~27 O(1) hole/replica terms against an rms force of
    # ~0.04: about 1e-6 absolute, 2e-5 of rms|a|
    assert np.median(e) < 5e-5 and e.max() < 2e-3
    # G M / L = 1 units; the reference's FP32 Ewald keeps its two-term series
    # up to fInner2 = 1.1e-2 L^2 (Ewald.cpp:508-516), which bounds this
    assert np.abs(v[:, 3] - ref32[:, 3]).max() < 2e-4


def test_ragged_and_tiny_buckets(cuda_ok):
    """Buckets above 32 targets (chunked), buckets of 1, and a 1-particle
    system."""
    p = ics.plummer(3000, ics.rng_for(5), soft=0.05)
    for nb in (1, 5, 33, 64, 100):
        L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=nb, theta=0.6)
        ref = oracle_vars(L)
        v = gravity.DeviceSystem(L).step("fp64").cpu().numpy()
        assert force_rel_err(v, ref).max() < FP64_TOL, nb
        vm = gravity.DeviceSystem(L).step("mixed").cpu().numpy()
        assert np.median(force_rel_err(vm, ref)) < MIX_MEDIAN_TOL, nb
    one = tree.build_lists(np.zeros((1, 3)), np.ones(1), np.full(1, 0.1))
    v = gravity.DeviceSystem(one).step("mixed").cpu().numpy()
    assert np.all(v == 0)


def test_empty_request_and_validation(cuda_ok):
    """numBucketsPlusOne == 1 enqueues nothing; with validation on, a
    request with an out-of-range index is rejected on the host before any
    copy or launch and reported through the error code."""
    lib = N.cuda_lib()
    p = ics.plummer(512, ics.rng_for(6))
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16)
    inp = gravity.DropInInputs(L)
    rt = gravity._cudart()
    d_m, d_p, d_v = C.c_void_p(), C.c_void_p(), C.c_void_p()
    lib.DataManagerTransferLocalTree(inp.moments.ptr, inp.moments.nbytes, inp.parts.ptr,
                                     inp.parts.nbytes, inp.vars.ptr, inp.vars.nbytes,
                                     C.byref(d_m), C.byref(d_p), C.byref(d_v), None, L.n, None)
    try:
        lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_RECORD)
        lib.changa_gb300_set_validate(1)
        lst, mk, st, sz, req = inp.reqs[0]
        r = N.CudaRequest()
        r.d_localMoments, r.d_localParts, r.d_localVars = d_m, d_p, d_v
        r.list, r.bucketMarkers, r.bucketStarts, r.bucketSizes = lst.ptr, mk.ptr, st.ptr, sz.ptr
        r.numInteractions = req.n_entries
        r.numBucketsPlusOne = 1
        before = lib.changa_gb300_kernel_launches()
        lib.TreePieceCellListDataTransferLocal(C.byref(r))
        assert lib.changa_gb300_kernel_launches() == before
        assert lib.changa_gb300_last_error() == 0
        lst.array[0, 0] = L.moments.shape[0] + 7  # out of range
        r.numBucketsPlusOne = req.n_buckets + 1
        lib.TreePieceCellListDataTransferLocal(C.byref(r))
        assert lib.changa_gb300_kernel_launches() == before
        assert lib.changa_gb300_last_error() == 1002
    finally:
        lib.changa_gb300_set_validate(0)
        lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_ABORT)
        rt.cudaStreamSynchronize(None)
        for q in (d_m, d_p, d_v):
            rt.cudaFree(q)
        inp.free()


def test_every_list_variant(plummer):
    """Every shape variant of the FP32-form list kernels (source-parallel,
    target-parallel, paired, and paired with TMA-staged cell records), on
    the Plummer lists, on ragged buckets and on GPU-walk lists (every
    bucket, some lists empty), holds the same tolerances as the default
    one."""
    L, ref, ref32 = plummer
    lib = N.cuda_lib()
    ids = [N.KERNEL_IDS[k] for k in ("list_f32_cell", "list_f32_part", "list_mixed_cell",
                                     "list_mixed_part")]
    saved = [lib.changa_gb300_get_list_variant(k) for k in ids]
    p = ics.plummer(3000, ics.rng_for(5), soft=0.05)
    ragged = [tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=nb, theta=0.6)
              for nb in (1, 5, 33, 64)]
    ragged_ref = [oracle_vars(R) for R in ragged]
    try:
        for var in range(lib.changa_gb300_list_variant_count()):
            for k in ids:
                assert lib.changa_gb300_set_list_variant(k, var) == 0
            v = gravity.DeviceSystem(L).step("mixed").cpu().numpy()
            e = force_rel_err(v, ref)
            assert np.median(e) < MIX_MEDIAN_TOL and np.percentile(e, 99) < MIX_P99_TOL, var
            assert np.median(pot_rel_err(v, ref)) < MIX_MEDIAN_TOL, var
            np.testing.assert_allclose(v[:, 4], ref[:, 4], rtol=1e-4, err_msg=str(var))
            inp = gravity.DropInInputs(L)
            try:
                v32 = gravity.dropin_step(inp).astype(np.float64)
            finally:
                inp.free()
            e = force_rel_err(v32, ref32)
            assert np.median(e) < F32_MEDIAN_TOL and np.percentile(e, 99) < F32_P99_TOL, var
            for R, rr in zip(ragged, ragged_ref):
                vm = gravity.DeviceSystem(R).step("mixed").cpu().numpy()
                assert np.median(force_rel_err(vm, rr)) < MIX_MEDIAN_TOL, (var, R.n_bucket)
                assert np.percentile(force_rel_err(vm, rr), 99) < MIX_P99_TOL, (var, R.n_bucket)
            # lists from the GPU walk hold every bucket, some with empty lists
            cells, plist, _ = gpu_walk(ragged[0])
            vd = gravity.DeviceSystem(ragged[0], device_reqs=[cells, plist]).step("mixed")
            e = force_rel_err(vd.cpu().numpy(), ragged_ref[0])
            assert np.median(e) < MIX_MEDIAN_TOL and np.percentile(e, 99) < MIX_P99_TOL, var
    finally:
        for k, s in zip(ids, saved):
            lib.changa_gb300_set_list_variant(k, s)


def test_dropin_remote_resume_and_small_phase(plummer):
    """The other request paths of the drop-in boundary: remote chunks
    (DataManagerTransferRemoteChunk + *Remote), resume requests carrying the
    missed nodes / particles on the host (*RemoteResume), the small-phase
    particle request and TreePieceDataTransferBasic/Cleanup.  Fed the same
    moments and particles as the local path, each gives the same result."""
    L, _, _ = plummer
    lib = N.cuda_lib()
    rt = gravity._cudart()
    inp = gravity.DropInInputs(L)
    try:
        ref = gravity.dropin_step(inp).copy()
        d_m, d_p, d_v = C.c_void_p(), C.c_void_p(), C.c_void_p()
        r_m, r_p = C.c_void_p(), C.c_void_p()

        def fresh():
            inp.vars.array[...] = 0
            lib.DataManagerTransferLocalTree(inp.moments.ptr, inp.moments.nbytes, inp.parts.ptr,
                                             inp.parts.nbytes, inp.vars.ptr, inp.vars.nbytes,
                                             C.byref(d_m), C.byref(d_p), C.byref(d_v), None, L.n,
                                             None)

        def request(k, moments=None, parts=None):
            lst, mk, st, sz, req = inp.reqs[k]
            r = N.CudaRequest()
            r.d_localMoments, r.d_localParts, r.d_localVars = d_m, d_p, d_v
            r.d_remoteMoments, r.d_remoteParts = moments, parts
            r.list, r.bucketMarkers, r.bucketStarts, r.bucketSizes = lst.ptr, mk.ptr, st.ptr, sz.ptr
            r.numInteractions = req.n_entries
            r.numBucketsPlusOne = req.n_buckets + 1
            r.fperiod = 0.0
            return r

        def result():
            lib.TransferParticleVarsBack(inp.out.ptr, inp.out.nbytes, d_v, None, None)
            rt.cudaStreamSynchronize(None)
            return inp.out.array.copy()

        def free_all(*ptrs):
            for q in ptrs:
                rt.cudaFree(q)

        # remote chunk: the same moments and particles uploaded as remote data
        fresh()
        lib.DataManagerTransferRemoteChunk(inp.moments.ptr, inp.moments.nbytes, inp.parts.ptr,
                                           inp.parts.nbytes, C.byref(r_m), C.byref(r_p), None, None)
        lib.TreePieceCellListDataTransferRemote(C.byref(request(0, r_m, r_p)))
        lib.TreePiecePartListDataTransferRemote(C.byref(request(1, r_m, r_p)))
        assert np.array_equal(result(), ref)
        free_all(d_m, d_p, d_v, r_m, r_p)

        # resume: the missed nodes / particles travel with the request
        fresh()
        rc = request(0)
        rc.missedNodes, rc.sMissed = inp.moments.ptr, inp.moments.nbytes
        lib.TreePieceCellListDataTransferRemoteResume(C.byref(rc))
        rp = request(1)
        rp.missedParts, rp.sMissed = inp.parts.ptr, inp.parts.nbytes
        lib.TreePiecePartListDataTransferRemoteResume(C.byref(rp))
        assert np.array_equal(result(), ref)
        free_all(d_m, d_p, d_v)

        # small phase: the source particles passed from the host
        fresh()
        lib.TreePieceCellListDataTransferLocal(C.byref(request(0)))
        lib.TreePiecePartListDataTransferLocalSmallPhase(C.byref(request(1)), inp.parts.ptr, L.n)
        assert np.array_equal(result(), ref)
        free_all(d_m, d_p, d_v)

        # Basic + Cleanup upload a request's arrays and release them
        fresh()
        ptrs = N.CudaDevPtr()
        lib.TreePieceDataTransferBasic(C.byref(request(0)), C.byref(ptrs))
        rt.cudaStreamSynchronize(None)
        assert ptrs.d_list and ptrs.d_bucketMarkers
        lib.TreePieceDataTransferBasicCleanup(C.byref(ptrs))
        rt.cudaStreamSynchronize(None)
        free_all(d_m, d_p, d_v)
    finally:
        inp.free()


def test_dropin_concurrent_streams(plummer, lattice):
    """ChaNGa calls the boundary from several PE threads at once, each
    TreePiece on its own stream (TreePiece.cpp:5380).  Four threads with
    their own streams and host buffers, mixing cell/particle lists with
    Ewald requests, call the drop-in concurrently (ctypes releases the GIL);
    every result equals its serial result bit for bit (no shared mutable
    state on the path; the Ewald parameters travel with each launch)."""
    import threading
    import torch
    L, _, _ = plummer
    Ll, ew, _ = lattice
    cases = [(L, None), (Ll, ew), (L, None), (Ll, ew)]
    serial = []
    for Lc, e in cases:
        inp = gravity.DropInInputs(Lc, ewald=e)
        try:
            serial.append(gravity.dropin_step(inp).copy())
        finally:
            inp.free()
    inputs = [gravity.DropInInputs(Lc, ewald=e) for Lc, e in cases]
    streams = [torch.cuda.Stream() for _ in cases]
    out = [None] * len(cases)
    errors = []

    def run(i):
        try:
            for _ in range(3):
                out[i] = gravity.dropin_step(inputs[i], stream=streams[i].cuda_stream).copy()
        except Exception as ex:  # reported below
            errors.append(ex)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(len(cases))]
    try:
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    finally:
        for inp in inputs:
            inp.free()
    assert not errors, errors
    for i in range(len(cases)):
        assert np.array_equal(out[i], serial[i]), i


def test_tma_wait_timeout_reports_error(plummer):
    """The TMA-staged cell variant waits for its copies with an iteration
    limit.  With the limit at 0 polls every wait runs out at once: each warp
    still drains its copy in flight (long limit) and stops, the kernel
    returns, and the device status reads CHANGA_E_DEVICE_WAIT once (then it
    is cleared).  The GPU stays usable: the next evaluation with the default
    limit matches the oracle and leaves the status clear.  The same holds
    through changa_gravity_step_host, which reads the status itself."""
    L, ref, _ = plummer
    lib = N.cuda_lib()
    k = N.KERNEL_IDS["list_mixed_cell"]
    saved = lib.changa_gb300_get_list_variant(k)
    assert lib.changa_gb300_device_status() == 0
    lib.changa_gb300_last_error()
    try:
        assert lib.changa_gb300_set_list_variant(k, 11) == 0
        lib.changa_gb300_set_test_wait_limit(0)
        ds = gravity.DeviceSystem(L)
        ds.step("mixed")
        assert lib.changa_gb300_device_status() == 1004
        assert lib.changa_gb300_last_error() == 1004
        assert lib.changa_gb300_device_status() == 0
        # through the host-array entry, which checks the word after its sync
        with pytest.raises(RuntimeError, match="1004"):
            gravity.gravity_step_host(L, "mixed")
        assert lib.changa_gb300_last_error() == 1004
        assert lib.changa_gb300_device_status() == 0
        lib.changa_gb300_set_test_wait_limit(-1)
        v = gravity.DeviceSystem(L).step("mixed").cpu().numpy()
        assert lib.changa_gb300_device_status() == 0
        e = force_rel_err(v, ref)
        assert np.median(e) < MIX_MEDIAN_TOL and np.percentile(e, 99) < MIX_P99_TOL
    finally:
        lib.changa_gb300_set_test_wait_limit(-1)
        lib.changa_gb300_set_list_variant(k, saved)
        lib.changa_gb300_last_error()


def test_dropin_chunked_upload(plummer, lattice):
    """A drop-in request whose list is longer than two upload chunks streams
    its list in chunks on the copy stream, each chunk's buckets launched as
    the chunk lands.  Every bucket is still evaluated by one warp with the
    same arithmetic, so the result equals the single-upload result bit for
    bit (cell and particle lists, with Ewald on the lattice); with the
    completion hook counting, each request still signals once."""
    lib = N.cuda_lib()
    for L, ew in ((plummer[0], None), (lattice[0], lattice[1])):
        inp = gravity.DropInInputs(L, ew)
        try:
            whole = gravity.dropin_step(inp).copy()
            n_entries = min(L.cells.n_entries, L.plist.n_entries)
            # chunks of ~1/5 of the shorter list: both requests take the chunked path
            chunk = max(4096, n_entries * 8 // 5)
            lib.changa_gb300_set_host_chunk_bytes(chunk)
            try:
                chunked = gravity.dropin_step(inp).copy()
            finally:
                lib.changa_gb300_set_host_chunk_bytes(0)  # the default
        finally:
            inp.free()
        assert n_entries * 8 > 2 * chunk
        np.testing.assert_array_equal(chunked, whole)


def test_host_entry_particle_runs(plummer, lattice):
    """changa_gravity_step_host_runs: the particle lists travel as runs
    (ILPart, 12 bytes per run), are expanded on the device chunk by chunk
    and evaluated as they land.  The expanded lists are the flat lists, and
    each bucket is evaluated by one warp in the same order, so the result
    equals the flat-list entry's bit for bit: both forms, with Ewald on the
    lattice, with one chunk and with chunks of a few hundred runs."""
    from changa_gb300 import tree as T
    lib = N.cuda_lib()
    for L, ew in ((plummer[0], None), (lattice[0], lattice[1])):
        pr = T.part_runs(L.plist)
        for form in ("fp64", "mixed"):
            flat = gravity.gravity_step_host(L, form, ewald=ew)
            runs = gravity.gravity_step_host(L, form, ewald=ew, runs=pr)
            np.testing.assert_array_equal(runs, flat)
        lib.changa_gb300_set_host_chunk_bytes(4096)  # 341 runs per chunk
        try:
            small = gravity.gravity_step_host(L, "mixed", ewald=ew, runs=pr)
        finally:
            lib.changa_gb300_set_host_chunk_bytes(0)  # the default
        np.testing.assert_array_equal(small, gravity.gravity_step_host(L, "mixed", ewald=ew))


def test_two_replica_layers_with_ewald(cuda_ok):
    """Lists over 5^3 replica roots (two replica layers: offset codes with
    components of magnitude 2) and the Ewald term with nReps = 2 (its hole
    spans those 125 replicas), on a clustered periodic box: the FP64 form
    against the oracle per particle, the FP32-mixed form against the FP64
    oracle, and the FP32 drop-in against the oracle on its FP32 inputs."""
    p = ics.nfw_halos(16384, ics.rng_for(10), soft=1e-3)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         n_replicas=2)
    codes = np.concatenate([(L.cells.list[:, 1] >> 22) & 0x1ff, (L.plist.list[:, 1] >> 22) & 0x1ff])
    assert ((codes & 7) == 5).any() and ((codes & 7) == 1).any()  # x offsets of +2 and -2
    ew = gravity.EwaldConfig(1.0, 2, 2.6, 2.8)
    ref = oracle_vars(L, 1.0, ew)
    v64 = gravity.DeviceSystem(L, ewald=ew).step("fp64").cpu().numpy()
    assert force_rel_err(v64, ref).max() < FP64_TOL
    assert pot_rms_err(v64, ref).max() < FP64_TOL
    vmx = gravity.DeviceSystem(L, ewald=ew).step("mixed").cpu().numpy()
    e = force_rms_err(vmx, ref)
    assert np.median(e) < 5e-5 and e.max() < 2e-3
    assert np.median(force_rel_err(vmx, ref)) < 1e-4
    ref32 = oracle_vars(L, 1.0, ew, f32_inputs=True)
    inp = gravity.DropInInputs(L, ewald=ew)
    try:
        v = gravity.dropin_step(inp).astype(np.float64)
    finally:
        inp.free()
    e32 = force_rms_err(v, ref32)
    print("two replica layers: fp64 max rel %.2e; mixed rms median %.2e max %.2e; drop-in rms "
          "median %.2e max %.2e" % (force_rel_err(v64, ref).max(), np.median(e), e.max(),
                                    np.median(e32), e32.max()))
    assert np.median(e32) < 5e-5 and e32.max() < 2e-3


def test_coincident_particles(cuda_ok):
    """Every particle twice at the same position: the pairs at r = 0 are
    skipped (partBucketForce's rsq = 0 test, gravity.h:276-301) in every
    form, and the rest matches the oracle."""
    p = ics.plummer(4096, ics.rng_for(12), soft=0.01)
    pos = np.concatenate([p["pos"], p["pos"]])
    mass = np.concatenate([p["mass"], p["mass"]]) / 2
    soft = np.concatenate([p["soft"], p["soft"]])
    L = tree.build_lists(pos, mass, soft, n_bucket=16, theta=0.7)
    ref = oracle_vars(L)
    assert np.isfinite(ref).all()
    v64 = gravity.DeviceSystem(L).step("fp64").cpu().numpy()
    assert force_rel_err(v64, ref).max() < FP64_TOL
    vmx = gravity.DeviceSystem(L).step("mixed").cpu().numpy()
    assert np.isfinite(vmx).all()
    assert np.median(force_rel_err(vmx, ref)) < MIX_MEDIAN_TOL
    assert np.percentile(force_rel_err(vmx, ref), 99) < MIX_P99_TOL
    ref32 = oracle_vars(L, f32_inputs=True)
    inp = gravity.DropInInputs(L)
    try:
        v32 = gravity.dropin_step(inp).astype(np.float64)
    finally:
        inp.free()
    assert np.isfinite(v32).all()
    assert np.median(force_rel_err(v32, ref32)) < F32_MEDIAN_TOL
