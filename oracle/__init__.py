"""CPU oracle for the gravity hot path -- TEST INFRASTRUCTURE ONLY.

Loads one of the two implementations of oracle/oracle_api.h:
  "ref"  ChaNGa's own gravity.h + Ewald.cpp compiled unchanged (oracle/_ref,
         only where the reference sources were available at build time);
  "port" this project's plain-C restatement (oracle/_build).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package; the product never does.  Also holds FP64 direct sums
(numpy) used as accuracy yardsticks.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libchanga_port.so")
REF_LIB = os.path.join(HERE, "_ref", "libchanga_ref.so")
REF_HEX_LIB = os.path.join(HERE, "_ref", "libchanga_ref_hex.so")

_libs = {}


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def available(kind):
    return os.path.exists(REF_LIB if kind == "ref" else PORT_LIB)


def load(kind="port"):
    if kind == "auto":
        kind = "ref" if available("ref") else "port"
    if kind not in _libs:
        path = REF_LIB if kind == "ref" else PORT_LIB
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        vp, i, l, d = C.c_void_p, C.c_int, C.c_long, C.c_double
        lib.oracle_cell_list_forces.argtypes = [vp, l, vp, l, vp, vp, vp, vp, i, vp, i, d, vp, i]
        lib.oracle_part_list_forces.argtypes = [vp, l, vp, l, vp, vp, vp, vp, i, vp, i, d, vp, i]
        lib.oracle_ewald_table.argtypes = [vp, d, d, vp, i]
        lib.oracle_ewald_forces.argtypes = [vp, l, vp, l, vp, d, i, d, d, vp, i]
        for f in (lib.oracle_cell_list_forces, lib.oracle_part_list_forces, lib.oracle_ewald_table,
                  lib.oracle_ewald_forces):
            f.restype = i
        if kind == "port":
            _bind_hex(lib)
            lib.oracle_direct_energy.argtypes = [vp, l, i]
            lib.oracle_direct_energy.restype = d
        _libs[kind] = lib
    return _libs[kind]


def _bind_hex(lib):
    vp, i, l, d = C.c_void_p, C.c_int, C.c_long, C.c_double
    lib.oracle_cell_list_forces_hex.argtypes = [vp, l, vp, l, vp, vp, vp, vp, i, vp, d, vp, i]
    lib.oracle_ewald_table_hex.argtypes = [vp, d, d, vp, i, vp]
    lib.oracle_ewald_forces_hex.argtypes = [vp, l, vp, l, vp, d, i, d, d, vp, i]
    for f in (lib.oracle_cell_list_forces_hex, lib.oracle_ewald_table_hex,
              lib.oracle_ewald_forces_hex):
        f.restype = i


def _load_hex(kind):
    """The hexadecapole cell-list oracle: the port, or the reference's own
    gravity.h + moments.c compiled with HEXADECAPOLE (kind "ref")."""
    if kind == "auto":
        kind = "ref" if os.path.exists(REF_HEX_LIB) else "port"
    if kind == "port":
        return load("port")
    key = "ref_hex"
    if key not in _libs:
        if not os.path.exists(REF_HEX_LIB):
            build()
        lib = C.CDLL(REF_HEX_LIB)
        _bind_hex(lib)
        _libs[key] = lib
    return _libs[key]


def bucket_geometry(lists, req):
    """{cm.xyz, soft, bbox lesser xyz, greater xyz} of every bucket of a
    request (the bucket's own moments and particle box), for the
    hexadecapole softening test."""
    ids = np.asarray(req.bucket_ids, dtype=np.int64)
    mom = lists.moments[lists.meta["leaf"][lists.bucket_starts[ids]]]
    g = np.empty((len(ids), 10))
    g[:, 0:3] = mom[:, 3:6]
    g[:, 3] = mom[:, 1]
    g[:, 4:10] = lists.bucket_bbox[ids]
    return g


def cell_forces_hex(moments, parts, req, geom, fperiod=0.0, vars=None, kind="port", nthreads=0):
    """nodeBucketForce of the hexadecapole build over a cell request
    (moments M x 27; geom from bucket_geometry); returns vars (N x 5)."""
    lib = _load_hex(kind)
    moments = _c(moments, np.float64)
    parts = _c(parts, np.float64)
    geom = _c(geom, np.float64)
    if vars is None:
        vars = np.zeros((parts.shape[0], 5))
    lst, mk, st, sz = (_c(req.list, np.int32), _c(req.markers, np.int32),
                       _c(req.starts, np.int32), _c(req.sizes, np.int32))
    rc = lib.oracle_cell_list_forces_hex(_p(moments), moments.shape[0], _p(parts), parts.shape[0],
                                         _p(lst), _p(mk), _p(st), _p(sz), len(st), _p(geom),
                                         float(fperiod), _p(vars), int(nthreads))
    assert rc == 0
    return vars


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


def cell_forces(moments, parts, req, fperiod=0.0, vars=None, bucket_ids=None, kind="port",
                nthreads=0):
    """nodeBucketForce over a cell request; returns vars (N x 5, FP64)."""
    lib = load(kind)
    moments = _c(moments, np.float64)
    parts = _c(parts, np.float64)
    if vars is None:
        vars = np.zeros((parts.shape[0], 5))
    ids = _c(bucket_ids, np.int32)
    lst, mk, st, sz = (_c(req.list, np.int32), _c(req.markers, np.int32),
                       _c(req.starts, np.int32), _c(req.sizes, np.int32))
    rc = lib.oracle_cell_list_forces(_p(moments), moments.shape[0], _p(parts), parts.shape[0],
                                     _p(lst), _p(mk), _p(st), _p(sz), len(st), _p(ids),
                                     0 if ids is None else len(ids), float(fperiod), _p(vars),
                                     int(nthreads))
    assert rc == 0
    return vars


def part_forces(sources, targets, req, fperiod=0.0, vars=None, bucket_ids=None, kind="port",
                nthreads=0):
    """partBucketForce over a flattened particle request."""
    lib = load(kind)
    sources = _c(sources, np.float64)
    targets = _c(targets, np.float64)
    if vars is None:
        vars = np.zeros((targets.shape[0], 5))
    ids = _c(bucket_ids, np.int32)
    lst, mk, st, sz = (_c(req.list, np.int32), _c(req.markers, np.int32),
                       _c(req.starts, np.int32), _c(req.sizes, np.int32))
    rc = lib.oracle_part_list_forces(_p(sources), sources.shape[0], _p(targets), targets.shape[0],
                                     _p(lst), _p(mk), _p(st), _p(sz), len(st), _p(ids),
                                     0 if ids is None else len(ids), float(fperiod), _p(vars),
                                     int(nthreads))
    assert rc == 0
    return vars


def ewald_table(root, L, dEwhCut, kind="port"):
    lib = load(kind)
    root = _c(root, np.float64)
    out = np.zeros((4096, 5))
    n = lib.oracle_ewald_table(_p(root), float(L), float(dEwhCut), _p(out), 4096)
    assert n >= 0
    return out[:n].copy()


def ewald_forces(parts, root, L, nReps, fEwCut, dEwhCut, idx=None, vars=None, kind="port",
                 nthreads=0):
    """BucketEwald for parts[idx] (all when idx is None); returns vars rows
    in idx order."""
    lib = load(kind)
    parts = _c(parts, np.float64)
    root = _c(root, np.float64)
    idx = _c(idx, np.int32)
    n_idx = parts.shape[0] if idx is None else len(idx)
    if vars is None:
        vars = np.zeros((n_idx, 5))
    rc = lib.oracle_ewald_forces(_p(parts), parts.shape[0], _p(idx), n_idx, _p(root), float(L),
                                 int(nReps), float(fEwCut), float(dEwhCut), _p(vars), int(nthreads))
    assert rc == 0
    return vars


def ewald_table_hex(root, L, dEwhCut, kind="port"):
    """EwaldInit of the hexadecapole build for a 27-value root: (h-table rows,
    the root's complete moments in MomcData order)."""
    lib = _load_hex(kind)
    root = _c(root, np.float64)
    out = np.zeros((4096, 5))
    momc = np.zeros(32)
    n = lib.oracle_ewald_table_hex(_p(root), float(L), float(dEwhCut), _p(out), 4096, _p(momc))
    assert n >= 0
    return out[:n].copy(), momc


def ewald_forces_hex(parts, root, L, nReps, fEwCut, dEwhCut, idx=None, vars=None, kind="port",
                     nthreads=0):
    """BucketEwald of the hexadecapole build for parts[idx]; returns vars
    rows in idx order."""
    lib = _load_hex(kind)
    parts = _c(parts, np.float64)
    root = _c(root, np.float64)
    idx = _c(idx, np.int32)
    n_idx = parts.shape[0] if idx is None else len(idx)
    if vars is None:
        vars = np.zeros((n_idx, 5))
    rc = lib.oracle_ewald_forces_hex(_p(parts), parts.shape[0], _p(idx), n_idx, _p(root),
                                     float(L), int(nReps), float(fEwCut), float(dEwhCut),
                                     _p(vars), int(nthreads))
    assert rc == 0
    return vars


def spline_ab(r2, twoh):
    """SPLINE (gravity.h:147-182) vectorised in numpy FP64."""
    r = np.sqrt(r2)
    a = np.empty_like(r)
    b = np.empty_like(r)
    far = r >= twoh
    with np.errstate(divide="ignore", invalid="ignore"):
        a[far] = 1.0 / r[far]
        b[far] = a[far] ** 3
        near = ~far
        dih = 2.0 / twoh[near]
        u = r[near] * dih
        inner = u < 1.0
        ui, di = u[inner], dih[inner]
        an = np.empty_like(u)
        bn = np.empty_like(u)
        an[inner] = di * (7 / 5 - 2 / 3 * ui ** 2 + 3 / 10 * ui ** 4 - 1 / 10 * ui ** 5)
        bn[inner] = di ** 3 * (4 / 3 - 6 / 5 * ui ** 2 + 1 / 2 * ui ** 3)
        uo, do = u[~inner], dih[~inner]
        diro = 1.0 / r[near][~inner]
        an[~inner] = -1 / 15 * diro + do * (8 / 5 - 4 / 3 * uo ** 2 + uo ** 3 - 3 / 10 * uo ** 4 +
                                            1 / 30 * uo ** 5)
        bn[~inner] = -1 / 15 * diro ** 3 + do ** 3 * (8 / 3 - 3 * uo + 6 / 5 * uo ** 2 -
                                                      1 / 6 * uo ** 3)
        a[near] = an
        b[near] = bn
    return a, b


def direct_energy(parts, nthreads=0):
    """Potential energy 0.5 sum_i m_i phi_i of an open system, by FP64
    direct summation over every pair with the P-P spline softening (the C
    port, all host cores)."""
    parts = np.ascontiguousarray(parts, dtype=np.float64)
    return float(load("port").oracle_direct_energy(_p(parts), parts.shape[0], nthreads))


def direct_sum(parts, targets_idx, chunk=4096):
    """FP64 spline-softened direct sum (open boundaries) on the selected
    targets: returns (acc (k x 3), pot (k,))."""
    parts = np.asarray(parts, dtype=np.float64)
    src_m, src_s, src_x = parts[:, 0], parts[:, 1], parts[:, 2:5]
    acc = np.zeros((len(targets_idx), 3))
    pot = np.zeros(len(targets_idx))
    for k0 in range(0, len(targets_idx), 64):
        ti = np.asarray(targets_idx[k0:k0 + 64])
        tx = parts[ti, 2:5]
        ts = parts[ti, 1]
        for j0 in range(0, parts.shape[0], chunk):
            r = src_x[None, j0:j0 + chunk, :] - tx[:, None, :]
            r2 = (r * r).sum(axis=2)
            twoh = ts[:, None] + src_s[None, j0:j0 + chunk]
            m = np.broadcast_to(src_m[None, j0:j0 + chunk], r2.shape)
            mask = r2 > 0
            a = np.zeros_like(r2)
            b = np.zeros_like(r2)
            aa, bb = spline_ab(r2[mask], twoh[mask])
            a[mask] = aa
            b[mask] = bb
            acc[k0:k0 + 64] += ((b * m)[:, :, None] * r).sum(axis=1)
            pot[k0:k0 + 64] -= (a * m).sum(axis=1)
    return acc, pot
