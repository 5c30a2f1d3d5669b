"""The C-ABI library: loads without a GPU, exports every declared symbol
(C names and the reference's C++-mangled names), and its structs have the
reference's byte layouts."""
import os
import re
import subprocess

import numpy as np
import pytest

from changa_gb300 import _native as N

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


@pytest.fixture(scope="module")
def lib(built):
    return N.cuda_lib()


def _declared(header):
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"typedef[^;]*;", "", src)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?[\s\*]([A-Za-z_]\w*)\s*\([^;{]*\)\s*;",
                       src, flags=re.M)
    return sorted(set(n for n in names if not n.startswith("_")))


def _exported(path=None):
    out = subprocess.run(["nm", "-D", "--defined-only", path or N._build.CUDA_LIB],
                         capture_output=True, text=True, check=True).stdout
    return set(l.split()[-1] for l in out.splitlines() if " T " in l)


@pytest.mark.parametrize("build", ["quadrupole", "hexadecapole"])
@pytest.mark.parametrize("header", ["HostCUDA.h", "EwaldCUDA.h", "changa_gb300.h"])
def test_every_declared_symbol_exported(lib, header, build):
    """Both builds of the library (the quadrupole one and the HEXADECAPOLE
    one) export the whole boundary."""
    names = _declared(header)
    assert len(names) >= 3
    hexa = build == "hexadecapole"
    exported = _exported(N._build.HEX_LIB if hexa else None)
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    loaded = N.cuda_lib_hex() if hexa else lib
    for n in names:
        assert hasattr(loaded, n)


def test_reference_mangled_names_exported(lib):
    """The reference's header has C++ linkage; these are the names an
    unmodified ChaNGa object refers to."""
    exported = _exported()
    for sym in ["_Z34TreePieceCellListDataTransferLocalP12_CudaRequest",
                "_Z34TreePiecePartListDataTransferLocalP12_CudaRequest",
                "_Z41TreePieceCellListDataTransferRemoteResumeP12_CudaRequest",
                "_Z44TreePiecePartListDataTransferLocalSmallPhaseP12_CudaRequestP15CompactPartDatai",
                "_Z28DataManagerTransferLocalTreePvmS_mS_mPS_S0_S0_P11CUstream_stiS_",
                "_Z24TransferParticleVarsBackP16VariablePartDatamPvP11CUstream_stS1_",
                "_Z9EwaldHostP15CompactPartDataP16VariablePartDataP9EwaldDataP11CUstream_stPvii",
                "_Z24allocatePinnedHostMemoryPPvm"]:
        assert sym in exported, sym


LAYOUT_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "HostCUDA.h"
#include "EwaldCUDA.h"
#define P(T) printf(#T " %zu\n", sizeof(T))
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
  P(CudaMultipoleMoments); P(CompactPartData); P(VariablePartData); P(ILCell); P(ILPart);
  P(EwtData); P(MultipoleMomentsData); P(MomcData); P(EwaldReadOnlyData); P(EwaldData);
  P(CudaRequest); P(CudaDevPtr);
  O(CudaMultipoleMoments, cm); O(CudaMultipoleMoments, xx); O(CudaMultipoleMoments, zz);
  O(CompactPartData, position); O(VariablePartData, potential); O(VariablePartData, dtGrav);
  O(EwaldReadOnlyData, n); O(EwaldReadOnlyData, L); O(EwaldReadOnlyData, fInner2);
  O(CudaRequest, list); O(CudaRequest, numInteractions); O(CudaRequest, cb); O(CudaRequest, fperiod);
  O(CudaRequest, node); O(CudaRequest, remote);
  return 0;
}
"""


def test_struct_layouts(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(LAYOUT_PROBE)
    exe = tmp_path / "probe"
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    subprocess.run(["gcc", "-I", INCLUDE, "-I", cuda_inc, str(src), "-o", str(exe)], check=True)
    got = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    got = {k: int(v) for k, v in got.items()}
    # quadrupole, no GPU walk (cuda_typedef.h:104-272, EwaldCUDA.h:11-57)
    assert got["CudaMultipoleMoments"] == 48
    assert got["CompactPartData"] == 20
    assert got["VariablePartData"] == 20
    assert got["ILCell"] == 8 and got["ILPart"] == 12
    assert got["EwtData"] == 20
    assert got["MultipoleMomentsData"] == 40
    assert got["MomcData"] == 32 * 4
    assert got["EwaldReadOnlyData"] == 40 + 128 + 16 + 32
    assert got["CudaMultipoleMoments.cm"] == 12 and got["CudaMultipoleMoments.xx"] == 24
    assert got["CompactPartData.position"] == 8
    assert got["VariablePartData.dtGrav"] == 16
    # the ctypes mirror used by the Python harness agrees
    import ctypes as C
    assert C.sizeof(N.CudaRequest) == got["CudaRequest"]
    assert C.sizeof(N.EwaldReadOnlyData) == got["EwaldReadOnlyData"]
    assert C.sizeof(N.EwaldData) == got["EwaldData"]
    assert N.CudaRequest.fperiod.offset == got["CudaRequest.fperiod"]
    assert N.CudaRequest.remote.offset == got["CudaRequest.remote"]
    assert N.CudaRequest.cb.offset == got["CudaRequest.cb"]


LAYOUT_PROBE_HEX = r"""
#include <stdio.h>
#include <stddef.h>
#include "HostCUDA.h"
#include "EwaldCUDA.h"
#define P(T) printf(#T " %zu\n", sizeof(T))
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
  P(CudaMultipoleMoments); P(MultipoleMomentsData); P(MomcData); P(EwaldReadOnlyData);
  O(CudaMultipoleMoments, xx); O(CudaMultipoleMoments, xxx); O(CudaMultipoleMoments, xxxx);
  O(CudaMultipoleMoments, xyyz); O(EwaldReadOnlyData, momcRoot); O(EwaldReadOnlyData, n);
  O(EwaldReadOnlyData, fInner2);
  return 0;
}
"""


def test_struct_layouts_hexadecapole(tmp_path):
    """The boundary headers compiled with -DHEXADECAPOLE give the reference's
    hexadecapole layouts (cuda_typedef.h:104-128, EwaldCUDA.h:18-47)."""
    src = tmp_path / "probe_hex.c"
    src.write_text(LAYOUT_PROBE_HEX)
    exe = tmp_path / "probe_hex"
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    subprocess.run(["gcc", "-DHEXADECAPOLE", "-I", INCLUDE, "-I", cuda_inc, str(src), "-o",
                    str(exe)], check=True)
    got = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    got = {k: int(v) for k, v in got.items()}
    assert got["CudaMultipoleMoments"] == 108
    assert got["CudaMultipoleMoments.xx"] == 24
    assert got["CudaMultipoleMoments.xxx"] == 44
    assert got["CudaMultipoleMoments.xxxx"] == 72
    assert got["CudaMultipoleMoments.xyyz"] == 104
    assert got["MultipoleMomentsData"] == 16
    assert got["MomcData"] == 128
    assert got["EwaldReadOnlyData"] == 16 + 128 + 16 + 32
    assert got["EwaldReadOnlyData.momcRoot"] == 16
    import ctypes as C
    assert C.sizeof(N.EwaldReadOnlyDataHex) == got["EwaldReadOnlyData"]
    assert N.EwaldReadOnlyDataHex.n.offset == got["EwaldReadOnlyData.n"]
    assert N.EwaldReadOnlyDataHex.fInner2.offset == got["EwaldReadOnlyData.fInner2"]


def _hex_root():
    from changa_gb300 import ics, tree
    p = ics.nfw_halos(8000, ics.rng_for(2), soft=1e-3)
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0,
                         order=4)
    return L.moments[0].copy()


def test_ewald_table_hex_matches_oracle(lib):
    """changa_ewald_table_hex (our restatement of EwaldInit with
    HEXADECAPOLE) against the oracle: the complete root moments exactly, the
    table to rounding (the contractions are summed in another order)."""
    import oracle
    from changa_gb300.gravity import EwaldConfig
    root = _hex_root()
    tb, momc = EwaldConfig(1.0, 1, 2.6, 2.8).table_hex(root)
    ref, ref_momc = oracle.ewald_table_hex(root, 1.0, 2.8)
    assert tb.shape == (80, 5)
    np.testing.assert_array_equal(momc, ref_momc)
    np.testing.assert_array_equal(tb[:, :3], ref[:, :3])
    scale = np.abs(ref[:, 3:]).max(axis=0)
    assert (np.abs(tb[:, 3:] - ref[:, 3:]).max(axis=0) <= 1e-14 * scale).all()
    assert np.abs(ref[:, 4]).max() > 0  # the octupole gives a sine term


def test_ewald_table_matches_oracle(lib):
    import oracle
    root = np.array([0.5, 0.0, 1.0, 0.49, 0.51, 0.5, 0.08, 0.001, -0.002, 0.081, 0.0005, 0.079])
    from changa_gb300.gravity import EwaldConfig
    tb = EwaldConfig(1.0, 1, 2.6, 2.8).table(root)
    assert tb.shape == (80, 5)
    np.testing.assert_array_equal(tb, oracle.ewald_table(root, 1.0, 2.8))


def test_host_validator(lib):
    """changa_validate_request rejects out-of-range indices, markers and
    bucket ranges on the host, without touching a GPU."""
    import ctypes as C
    lst = np.array([[0, 0], [5, 0], [2, 0]], np.int32)
    mk = np.array([0, 2, 3], np.int32)
    st = np.array([0, 4], np.int32)
    sz = np.array([4, 4], np.int32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    ok = lib.changa_validate_request(p(lst), 3, p(mk), p(st), p(sz), 2, 6, 8)
    assert ok == 0
    assert lib.changa_validate_request(p(lst), 3, p(mk), p(st), p(sz), 2, 5, 8) == 1002  # index 5
    assert lib.changa_validate_request(p(lst), 3, p(mk), p(st), p(sz), 2, 6, 7) == 1002  # targets
    bad_mk = np.array([0, 3, 2], np.int32)
    assert lib.changa_validate_request(p(lst), 3, p(bad_mk), p(st), p(sz), 2, 6, 8) == 1002
    assert lib.changa_validate_request(p(lst), 3, p(mk), p(st), p(sz), 0, 6, 8) == 0  # empty


def test_ewald_vjp_rejects_hexadecapole_tables():
    """The Ewald adjoint is the quadrupole root expansion's: a table with
    sine terms (the hexadecapole build's) or a massless root is refused
    before anything runs on the device."""
    import ctypes as C
    lib = N.cuda_lib()
    lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_RECORD)
    try:
        lib.changa_gb300_last_error()
        ewt = np.zeros((2, 5))
        ewt[:, 3] = 1.0
        ewt[1, 4] = 0.5  # a sine term
        p = N.ChangaEwaldParams()
        p.root[2] = 1.0
        p.L = 1.0
        p.nReps = 1
        p.fEwCut = 2.6
        p.nEwhLoop = 2
        p.ewt = ewt.ctypes.data
        dummy = C.c_void_p(8)  # never dereferenced
        assert lib.changa_ewald_vjp(dummy, 4, C.byref(p), dummy, dummy, None) == 1001
        assert lib.changa_gb300_last_error() == 1001
        ewt[1, 4] = 0.0
        p.root[2] = 0.0  # no mass
        assert lib.changa_ewald_vjp(dummy, 4, C.byref(p), dummy, dummy, None) == 1001
        assert lib.changa_gb300_last_error() == 1001
    finally:
        lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_ABORT)


def test_walk_forces_argument_checks():
    """changa_walk_forces refuses a missing tree, the hexadecapole rules
    (order 4) and missing arrays before anything runs on the device."""
    import ctypes as C
    lib = N.cuda_lib()
    lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_RECORD)
    try:
        lib.changa_gb300_last_error()
        dummy = C.c_void_p(8)  # never dereferenced
        wp = N.ChangaWalkParams(0.7, 2, 0.0, 0)
        assert lib.changa_walk_forces(None, C.byref(wp), dummy, dummy, 16, None, dummy, None) == 1001
        assert lib.changa_gb300_last_error() == 1001
        tv = N.ChangaTreeView(8, 8, 8, 8, 3, 8, 1)
        wp4 = N.ChangaWalkParams(0.7, 4, 0.0, 0)
        assert lib.changa_walk_forces(C.byref(tv), C.byref(wp4), dummy, dummy, 16, None, dummy,
                                      None) == 1001
        assert lib.changa_gb300_last_error() == 1001
        assert lib.changa_walk_forces(C.byref(tv), C.byref(wp), None, dummy, 16, None, dummy,
                                      None) == 1001
        assert lib.changa_gb300_last_error() == 1001
        assert lib.changa_walk_forces(C.byref(tv), C.byref(wp), dummy, dummy, 0, None, dummy,
                                      None) == 1001
        assert lib.changa_gb300_last_error() == 1001
    finally:
        lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_ABORT)
