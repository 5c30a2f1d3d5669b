"""ctypes bindings of the two native libraries.

The CUDA library is the product path: if it is missing or fails to load,
every GPU entry point raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_cuda = None
_host = None


class ILCell(C.Structure):
    _fields_ = [("index", C.c_int), ("offsetID", C.c_int)]


class CudaRequest(C.Structure):
    """Layout of CudaRequest (include/HostCUDA.h)."""
    _fields_ = [
        ("stream", C.c_void_p),
        ("d_localMoments", C.c_void_p),
        ("d_remoteMoments", C.c_void_p),
        ("d_localParts", C.c_void_p),
        ("d_remoteParts", C.c_void_p),
        ("d_localVars", C.c_void_p),
        ("sMoments", C.c_size_t),
        ("sCompactParts", C.c_size_t),
        ("sVarParts", C.c_size_t),
        ("list", C.c_void_p),
        ("bucketMarkers", C.c_void_p),
        ("bucketStarts", C.c_void_p),
        ("bucketSizes", C.c_void_p),
        ("numInteractions", C.c_int),
        ("numBucketsPlusOne", C.c_int),
        ("tp", C.c_void_p),
        ("missedNodes", C.c_void_p),
        ("missedParts", C.c_void_p),
        ("sMissed", C.c_size_t),
        ("affectedBuckets", C.c_void_p),
        ("cb", C.c_void_p),
        ("state", C.c_void_p),
        ("fperiod", C.c_float),
        ("node", C.c_bool),
        ("remote", C.c_bool),
    ]


class CudaDevPtr(C.Structure):
    _fields_ = [("d_list", C.c_void_p), ("d_bucketMarkers", C.c_void_p),
                ("d_bucketStarts", C.c_void_p), ("d_bucketSizes", C.c_void_p)]


class EwtData(C.Structure):
    _fields_ = [("hx", C.c_float), ("hy", C.c_float), ("hz", C.c_float),
                ("hCfac", C.c_float), ("hSfac", C.c_float)]


class MultipoleMomentsData(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("xx", "xy", "xz", "yy", "yz", "zz", "totalMass",
                                         "cmx", "cmy", "cmz")]


class MomcData(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "m", "xx", "yy", "xy", "xz", "yz", "xxx", "xyy", "xxy", "yyy", "xxz", "yyz", "xyz",
        "xxxx", "xyyy", "xxxy", "yyyy", "xxxz", "yyyz", "xxyy", "xxyz", "xyyz", "zz",
        "xzz", "yzz", "zzz", "xxzz", "xyzz", "xzzz", "yyzz", "yzzz", "zzzz")]


class EwaldReadOnlyData(C.Structure):
    _fields_ = [("mm", MultipoleMomentsData), ("momcRoot", MomcData),
                ("n", C.c_int), ("nReps", C.c_int), ("nEwReps", C.c_int), ("nEwhLoop", C.c_int),
                ("L", C.c_float), ("fEwCut", C.c_float), ("alpha", C.c_float),
                ("alpha2", C.c_float), ("k1", C.c_float), ("ka", C.c_float),
                ("fEwCut2", C.c_float), ("fInner2", C.c_float)]


class MultipoleMomentsDataHex(C.Structure):
    """MultipoleMomentsData of the HEXADECAPOLE build (no quadrupole terms)."""
    _fields_ = [(n, C.c_float) for n in ("totalMass", "cmx", "cmy", "cmz")]


class EwaldReadOnlyDataHex(C.Structure):
    """EwaldReadOnlyData of the HEXADECAPOLE build."""
    _fields_ = [("mm", MultipoleMomentsDataHex), ("momcRoot", MomcData),
                ("n", C.c_int), ("nReps", C.c_int), ("nEwReps", C.c_int), ("nEwhLoop", C.c_int),
                ("L", C.c_float), ("fEwCut", C.c_float), ("alpha", C.c_float),
                ("alpha2", C.c_float), ("k1", C.c_float), ("ka", C.c_float),
                ("fEwCut2", C.c_float), ("fInner2", C.c_float)]


# CudaMultipoleMoments: 12 floats (quadrupole build), 27 (HEXADECAPOLE)
MOMENT_FLOATS = {"quadrupole": 12, "hexadecapole": 27}


class EwaldData(C.Structure):
    _fields_ = [("EwaldRange", C.c_int * 2), ("EwaldMarkers", C.c_void_p),
                ("ewt", C.c_void_p), ("cachedData", C.c_void_p)]


class ChangaListRequest(C.Structure):
    _fields_ = [("list", C.c_void_p), ("markers", C.c_void_p), ("starts", C.c_void_p),
                ("sizes", C.c_void_p), ("n_buckets", C.c_int), ("n_entries", C.c_longlong)]


class ChangaPartRuns(C.Structure):
    _fields_ = [("runs", C.c_void_p), ("run_markers", C.c_void_p), ("markers", C.c_void_p),
                ("starts", C.c_void_p), ("sizes", C.c_void_p), ("n_buckets", C.c_int),
                ("n_runs", C.c_longlong)]


class ChangaTreeView(C.Structure):
    _fields_ = [("geom", C.c_void_p), ("bbox", C.c_void_p), ("info", C.c_void_p),
                ("parent", C.c_void_p), ("n_nodes", C.c_longlong), ("bucket_node", C.c_void_p),
                ("n_buckets", C.c_int)]


class ChangaWalkParams(C.Structure):
    _fields_ = [("theta", C.c_double), ("order", C.c_int), ("period", C.c_double),
                ("n_replicas", C.c_int)]


class ChangaWalkLists(C.Structure):
    _fields_ = [("n_buckets", C.c_int), ("order", C.c_int), ("passes", C.c_int),
                ("n_entries", C.c_longlong * 3), ("list", C.c_void_p * 3),
                ("markers", C.c_void_p * 3)]


class ChangaTreeArrays(C.Structure):
    _fields_ = [("n", C.c_longlong), ("n_nodes", C.c_longlong), ("n_buckets", C.c_int),
                ("perm", C.c_void_p), ("parts", C.c_void_p), ("moments", C.c_void_p),
                ("geom", C.c_void_p), ("bbox", C.c_void_p), ("info", C.c_void_p),
                ("parent", C.c_void_p), ("bucket_node", C.c_void_p), ("leaf", C.c_void_p),
                ("box", C.c_void_p)]


class ChangaEwaldParams(C.Structure):
    _fields_ = [("root", C.c_double * 12), ("L", C.c_double), ("nReps", C.c_int),
                ("fEwCut", C.c_double), ("nEwhLoop", C.c_int), ("ewt", C.c_void_p),
                ("momc", C.c_void_p)]


CHANGA_ERRORS_ABORT = 0
CHANGA_ERRORS_RECORD = 1
CHANGA_FORM_FP32 = 0
CHANGA_FORM_FP64 = 1
CHANGA_FORM_MIXED = 2
CHANGA_STEP_OVERWRITE = 0x100
CHANGA_MAX_EWH = 256

# kernel ids of changa_gb300_kernel_time
KERNEL_IDS = {"list_f32_cell": 0, "list_f32_part": 1, "list_f64_cell": 2, "list_f64_part": 3,
              "list_mixed_cell": 4, "list_mixed_part": 5, "ewald_f32": 6, "ewald_f64": 7,
              "ewald_mixed": 8, "pack": 9, "vjp_cell": 10, "vjp_part": 11,
              "moments": 12}


def kernel_time(name):
    """(total ms, launches) of one kernel since its last read (timing on)."""
    ms, n = C.c_double(), C.c_longlong()
    check(cuda_lib().changa_gb300_kernel_time(KERNEL_IDS[name], C.byref(ms), C.byref(n)),
          "kernel_time")
    return ms.value, n.value

# Every C-ABI function of include/HostCUDA.h, include/EwaldCUDA.h and
# include/changa_gb300.h with (restype, argtypes).
_VP, _SZ, _I, _LL, _D = C.c_void_p, C.c_size_t, C.c_int, C.c_longlong, C.c_double
_REQ = C.POINTER(CudaRequest)
CUDA_SIGNATURES = {
    "allocatePinnedHostMemory": (None, [C.POINTER(C.c_void_p), _SZ]),
    "freePinnedHostMemory": (None, [_VP]),
    "DataManagerTransferLocalTree": (None, [_VP, _SZ, _VP, _SZ, _VP, _SZ, C.POINTER(C.c_void_p),
                                            C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _VP, _I, _VP]),
    "DataManagerTransferRemoteChunk": (None, [_VP, _SZ, _VP, _SZ, C.POINTER(C.c_void_p),
                                              C.POINTER(C.c_void_p), _VP, _VP]),
    "TransferParticleVarsBack": (None, [_VP, _SZ, _VP, _VP, _VP]),
    "TreePieceCellListDataTransferLocal": (None, [_REQ]),
    "TreePieceCellListDataTransferRemote": (None, [_REQ]),
    "TreePieceCellListDataTransferRemoteResume": (None, [_REQ]),
    "TreePiecePartListDataTransferLocal": (None, [_REQ]),
    "TreePiecePartListDataTransferLocalSmallPhase": (None, [_REQ, _VP, _I]),
    "TreePiecePartListDataTransferRemote": (None, [_REQ]),
    "TreePiecePartListDataTransferRemoteResume": (None, [_REQ]),
    "TreePieceDataTransferBasic": (None, [_REQ, C.POINTER(CudaDevPtr)]),
    "TreePieceDataTransferBasicCleanup": (None, [C.POINTER(CudaDevPtr)]),
    "EwaldHostMemorySetup": (None, [C.POINTER(EwaldData), _I, _I, _I]),
    "EwaldHostMemoryFree": (None, [C.POINTER(EwaldData), _I]),
    "EwaldHost": (None, [_VP, _VP, C.POINTER(EwaldData), _VP, _VP, _I, _I]),
    "changa_gb300_set_error_mode": (None, [_I]),
    "changa_gb300_last_error": (_I, []),
    "changa_gb300_error_string": (C.c_char_p, [_I]),
    "changa_gb300_set_completion_hook": (None, [_VP]),
    "changa_gb300_set_validate": (None, [_I]),
    "changa_validate_request": (_I, [_VP, _LL, _VP, _VP, _VP, _I, _LL, _LL]),
    "changa_gb300_version": (_I, []),
    "changa_gb300_fp32_fma_peak": (_I, [C.POINTER(C.c_double)]),
    "changa_gb300_kernel_launches": (C.c_ulonglong, []),
    "changa_gb300_set_timing": (None, [_I]),
    "changa_gb300_set_host_chunk_bytes": (None, [_SZ]),
    "changa_gb300_list_variant_count": (_I, []),
    "changa_gb300_set_list_variant": (_I, [_I, _I]),
    "changa_gb300_get_list_variant": (_I, [_I]),
    "changa_gb300_set_hex_variant": (_I, [_I]),
    "changa_gb300_get_hex_variant": (_I, []),
    "changa_gb300_device_status": (_I, []),
    "changa_gb300_set_test_wait_limit": (None, [_I]),
    "changa_gb300_kernel_time": (_I, [_I, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
    "changa_cell_forces_fp64": (_I, [_VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest), _D, _VP, _VP]),
    "changa_part_forces_fp64": (_I, [_VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest), _D, _VP, _VP]),
    "changa_cell_forces_mixed": (_I, [_VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest), _D, _VP, _VP]),
    "changa_part_forces_mixed": (_I, [_VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest), _D, _VP, _VP]),
    "changa_cell_forces_mixed_noalloc": (_I, [_VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest), _D,
                                              _VP, _VP]),
    "changa_gravity_step": (_I, [_I, _VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest),
                                 C.POINTER(ChangaListRequest), _D, C.POINTER(ChangaEwaldParams),
                                 _VP, _VP]),
    "changa_gravity_step_host": (_I, [_I, _VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest),
                                      C.POINTER(ChangaListRequest), _D,
                                      C.POINTER(ChangaEwaldParams), _VP, _VP]),
    "changa_gravity_step_host_runs": (_I, [_I, _VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest),
                                           C.POINTER(ChangaPartRuns), _D,
                                           C.POINTER(ChangaEwaldParams), _VP, _VP]),
    "changa_gravity_graph_create": (_VP, [_I, _VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest),
                                         C.POINTER(ChangaListRequest), _D,
                                         C.POINTER(ChangaEwaldParams), _VP, _I]),
    "changa_gravity_graph_launch": (_I, [_VP, _VP]),
    "changa_gravity_vjp_mixed": (_I, [_VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest),
                                      C.POINTER(ChangaListRequest), _D, _VP, _VP, _VP, _VP, _VP]),
    "changa_gravity_graph_destroy": (None, [_VP]),
    "changa_ewald_vjp": (_I, [_VP, _LL, C.POINTER(ChangaEwaldParams), _VP, _VP, _VP]),
    "changa_tree_moments": (_I, [_VP, _LL, _VP, _VP, _LL, _VP, _VP]),
    "changa_direct_forces": (_I, [_VP, _LL, _VP, _LL, _D, _D, _VP, _VP]),
    "changa_tree_build": (_VP, [_VP, _VP, _VP, _LL, _I, _VP]),
    "changa_tree_view": (_I, [_VP, C.POINTER(ChangaTreeArrays)]),
    "changa_tree_free": (None, [_VP]),
    "changa_walk_count": (_I, [C.POINTER(ChangaTreeView), C.POINTER(ChangaWalkParams), _VP, _VP,
                               _VP, _VP]),
    "changa_walk_fill": (_I, [C.POINTER(ChangaTreeView), C.POINTER(ChangaWalkParams), _VP, _VP,
                              _VP, _VP, _VP, _VP, _VP]),
    "changa_walk": (_I, [C.POINTER(ChangaTreeView), C.POINTER(ChangaWalkParams),
                         C.POINTER(ChangaWalkLists), _VP]),
    "changa_walk_lists_free": (None, [C.POINTER(ChangaWalkLists)]),
    "changa_walk_set_pool_factor": (None, [_D]),
    "changa_walk_set_test_small_stack": (None, [C.c_int]),
    "changa_walk_set_groups": (None, [C.c_int, C.c_int]),
    "changa_walk_forces": (_I, [C.POINTER(ChangaTreeView), C.POINTER(ChangaWalkParams), _VP, _VP,
                                _LL, C.POINTER(ChangaEwaldParams), _VP, _VP]),
    "changa_walk_stack_reruns": (C.c_longlong, []),
    "changa_gravity_step_hexa": (_I, [_I, _VP, _LL, _VP, _LL, C.POINTER(ChangaListRequest),
                                      C.POINTER(ChangaListRequest),
                                      C.POINTER(ChangaListRequest), _D,
                                      C.POINTER(ChangaEwaldParams), _VP, _VP]),
    "changa_ewald_forces": (_I, [_I, _VP, _LL, _VP, _LL, C.POINTER(ChangaEwaldParams), _VP, _VP]),
    "changa_ewald_table": (_I, [_VP, _D, _D, _VP, _I]),
    "changa_ewald_table_hex": (_I, [_VP, _D, _D, _VP, _I, _VP]),
}

HOST_SIGNATURES = {
    "chg_tree_build": (_VP, [_VP, _VP, _VP, C.c_long, _I, _D, _D, _I]),
    "chg_tree_free": (None, [_VP]),
    "chg_tree_num_moments": (C.c_long, [_VP]),
    "chg_tree_num_buckets": (C.c_long, [_VP]),
    "chg_tree_num_nodes": (C.c_long, [_VP]),
    "chg_tree_get_order": (None, [_VP, _VP]),
    "chg_tree_get_moments": (None, [_VP, _VP]),
    "chg_tree_get_root": (None, [_VP, _VP]),
    "chg_tree_get_buckets": (None, [_VP, _VP, _VP, _VP, _VP]),
    "chg_tree_walk": (_I, [_VP, _I]),
    "chg_tree_list_lengths": (None, [_VP, _VP, _VP]),
    "chg_tree_serialize": (C.c_long, [_VP, _I, C.c_long, C.c_long, _VP, _VP, _VP, _VP, _VP,
                                      C.c_long, C.c_long]),
    "chg_tree_drop_lists": (None, [_VP]),
    "chg_tree_get_structure": (None, [_VP, _VP, _VP]),
    "chg_tree_get_ranges": (None, [_VP, _VP, _VP]),
    "chg_tree_set_order": (_I, [_VP, _I]),
    "chg_tree_soft_lengths": (None, [_VP, _VP]),
    "chg_tree_get_moments_hex": (None, [_VP, _VP]),
    "chg_tree_get_nodes": (None, [_VP, _VP, _VP, _VP]),
}


def _bind(lib, sigs):
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def host_lib():
    """The host tree/walk library (builds it on first use if absent)."""
    global _host
    if _host is None:
        path = _build.HOST_LIB
        if not os.path.exists(path):
            _build.build_host()
        _host = _bind(C.CDLL(path), HOST_SIGNATURES)
    return _host


def cuda_lib():
    """The CUDA gravity library.  Raises if it was not built: the GPU path
    has no fallback."""
    global _cuda
    if _cuda is None:
        path = _build.CUDA_LIB
        if not os.path.exists(path):
            raise RuntimeError("libchanga_gb300.so is not built (run __graft_entry__.build() or "
                               "python changa_gb300/build.py); the GPU path has no fallback")
        _cuda = _bind(C.CDLL(path, mode=C.RTLD_GLOBAL), CUDA_SIGNATURES)
    return _cuda


_cuda_hex = None


def cuda_lib_hex():
    """The same library built with -DHEXADECAPOLE: the boundary of ChaNGa's
    hexadecapole build (108-byte CudaMultipoleMoments, the hexadecapole
    EwaldReadOnlyData).  Loaded with local symbol scope next to cuda_lib()."""
    global _cuda_hex
    if _cuda_hex is None:
        path = _build.HEX_LIB
        if not os.path.exists(path):
            raise RuntimeError("libchanga_gb300_hex.so is not built (run __graft_entry__.build() "
                               "or python changa_gb300/build.py); the GPU path has no fallback")
        _cuda_hex = _bind(C.CDLL(path, mode=C.RTLD_LOCAL), CUDA_SIGNATURES)
    return _cuda_hex


def check(rc, what="changa_gb300"):
    if rc:
        msg = cuda_lib().changa_gb300_error_string(rc)
        raise RuntimeError("%s failed: %d (%s)" % (what, rc, msg.decode() if msg else "?"))
