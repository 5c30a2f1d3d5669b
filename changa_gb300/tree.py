"""Host side of the gravity path: tree, walk and the boundary arrays.

``build_lists`` runs the native tree build and dual walk
(changa_gb300/host/tree.cpp) and returns every array the GPU entry points
consume, in the reference's layouts:

* ``parts``     N x 5 FP64  {mass, soft, x, y, z} in bucket (key) order
* ``moments``   M x 12 FP64 {radius, soft, totalMass, cm, xx..zz}, BFS order
* ``cells``     the cell-list request: list (L x 2 int32 ILCell), markers,
                starts, sizes, bucket ids (only buckets with a non-empty list)
* ``plist``     the particle-list request, flattened to one ILCell per source
                particle
* ``perm``      GPU order -> caller order

``interactions`` follows the reference's counter (Compute.cpp:1643-1651):
sum over buckets of n_b (|cell list| + |particle list|).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._native import host_lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


@dataclass
class ListRequest:
    list: np.ndarray      # (L, 2) int32
    markers: np.ndarray   # (nb + 1,) int32
    starts: np.ndarray    # (nb,) int32
    sizes: np.ndarray     # (nb,) int32
    bucket_ids: np.ndarray

    @property
    def n_buckets(self):
        return int(len(self.starts))

    @property
    def n_entries(self):
        return int(self.list.shape[0])

    def interactions(self):
        lens = np.diff(self.markers.astype(np.int64))
        return int((lens * self.sizes.astype(np.int64)).sum())


@dataclass
class TreeLists:
    n: int
    parts: np.ndarray
    moments: np.ndarray
    root: np.ndarray
    perm: np.ndarray
    bucket_starts: np.ndarray
    bucket_sizes: np.ndarray
    bucket_bbox: np.ndarray
    cells: ListRequest
    plist: ListRequest
    period: float
    n_replicas: int
    theta: float
    n_bucket: int
    meta: dict = field(default_factory=dict)
    order: int = 2
    softcells: ListRequest | None = None  # order 4: cells evaluated as softened points

    @property
    def interactions(self):
        n = self.cells.interactions() + self.plist.interactions()
        if self.softcells is not None:
            n += self.softcells.interactions()
        return n

    def abi_moments(self):
        """CudaMultipoleMoments array: M x 12 float32 (quadrupole build) or
        M x 27 float32 (order 4: the HEXADECAPOLE build's 108-byte struct)."""
        return np.ascontiguousarray(self.moments, dtype=np.float32)

    def abi_parts(self):
        """CompactPartData array (N x 5 float32)."""
        return np.ascontiguousarray(self.parts, dtype=np.float32)


def _serialize(lib, h, kind, nb_total, lens):
    n_entries = int(lens.sum())
    filled = int((lens > 0).sum())
    lst = np.empty((n_entries, 2), dtype=np.int32)
    markers = np.empty(filled + 1, dtype=np.int32)
    starts = np.empty(filled, dtype=np.int32)
    sizes = np.empty(filled, dtype=np.int32)
    ids = np.empty(filled, dtype=np.int32)
    got = lib.chg_tree_serialize(h, kind, 0, nb_total, _ptr(lst), _ptr(markers), _ptr(starts),
                                 _ptr(sizes), _ptr(ids), 0, 0)
    assert got == filled
    return ListRequest(lst, markers, starts, sizes, ids)


def build_lists(pos, mass, soft, n_bucket=16, theta=0.7, period=0.0, n_replicas=0,
                nthreads=0, order=2) -> TreeLists:
    """Tree + walk + serialisation for one system (FP64 inputs).  order 2:
    quadrupole cells (moments M x 12); order 4: hexadecapole cells (moments
    M x 27, the walk's softening and monopole tests, and the softened cells
    in their own request, `softcells`, indexing the moments)."""
    if order not in (2, 4):
        raise ValueError("order must be 2 or 4")
    lib = host_lib()
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    soft = np.ascontiguousarray(soft, dtype=np.float64)
    n = pos.shape[0]
    if n >= 2 ** 31 - 1:
        raise ValueError("at most 2^31-2 particles per system")
    if period and n_replicas == 0:
        n_replicas = 1
    h = lib.chg_tree_build(_ptr(pos), _ptr(mass), _ptr(soft), n, int(n_bucket), float(theta),
                           float(period), int(n_replicas))
    if not h:
        raise ValueError("tree build rejected its arguments")
    try:
        perm = np.empty(n, dtype=np.int64)
        lib.chg_tree_get_order(h, _ptr(perm))
        nm = lib.chg_tree_num_moments(h)
        if order == 4:
            lib.chg_tree_set_order(h, 4)
            moments = np.empty((nm, 27), dtype=np.float64)
            lib.chg_tree_get_moments_hex(h, _ptr(moments))
        else:
            moments = np.empty((nm, 12), dtype=np.float64)
            lib.chg_tree_get_moments(h, _ptr(moments))
        root = np.empty(12, dtype=np.float64)
        lib.chg_tree_get_root(h, _ptr(root))
        nb = lib.chg_tree_num_buckets(h)
        bstarts = np.empty(nb, dtype=np.int32)
        bsizes = np.empty(nb, dtype=np.int32)
        bbox = np.empty((nb, 6), dtype=np.float64)
        bnode = np.empty(nb, dtype=np.int32)
        lib.chg_tree_get_buckets(h, _ptr(bstarts), _ptr(bsizes), _ptr(bbox), _ptr(bnode))
        ngeom = np.empty((nm, 6), dtype=np.float64)
        nbbox = np.empty((nm, 6), dtype=np.float64)
        ninfo = np.empty((nm, 4), dtype=np.int32)
        lib.chg_tree_get_nodes(h, _ptr(ngeom), _ptr(nbbox), _ptr(ninfo))
        parent = np.empty(nm, dtype=np.int32)
        leaf = np.empty(n, dtype=np.int32)
        lib.chg_tree_get_structure(h, _ptr(parent), _ptr(leaf))
        first = np.empty(nm, dtype=np.int32)
        count = np.empty(nm, dtype=np.int32)
        lib.chg_tree_get_ranges(h, _ptr(first), _ptr(count))
        lib.chg_tree_walk(h, int(nthreads))
        nc = np.empty(nb, dtype=np.int64)
        npl = np.empty(nb, dtype=np.int64)
        lib.chg_tree_list_lengths(h, _ptr(nc), _ptr(npl))
        cells = _serialize(lib, h, 0, nb, nc)
        plist = _serialize(lib, h, 1, nb, npl)
        softcells = None
        if order == 4:
            ns = np.empty(nb, dtype=np.int64)
            lib.chg_tree_soft_lengths(h, _ptr(ns))
            softcells = _serialize(lib, h, 2, nb, ns)
    finally:
        lib.chg_tree_free(h)
    parts = np.empty((n, 5), dtype=np.float64)
    parts[:, 0] = mass[perm]
    parts[:, 1] = soft[perm]
    parts[:, 2:5] = pos[perm]
    return TreeLists(n=n, parts=parts, moments=moments, root=root, perm=perm,
                     bucket_starts=bstarts, bucket_sizes=bsizes, bucket_bbox=bbox,
                     cells=cells, plist=plist, period=float(period), n_replicas=int(n_replicas),
                     theta=float(theta), n_bucket=int(n_bucket),
                     meta={"parent": parent, "leaf": leaf, "first": first, "count": count,
                           "bucket_node": bnode, "node_geom": ngeom, "node_bbox": nbbox,
                           "node_info": ninfo},
                     order=order, softcells=softcells)


@dataclass
class PartRuns:
    """A particle request as runs of consecutive source particles: runs (R x
    3 int32: first particle, offsetID, num; the reference's ILPart) with
    their per-bucket CSR run_markers, next to the flat request's markers,
    starts and sizes."""
    runs: np.ndarray
    run_markers: np.ndarray
    markers: np.ndarray
    starts: np.ndarray
    sizes: np.ndarray

    @property
    def n_buckets(self):
        return int(len(self.starts))

    @property
    def n_runs(self):
        return int(self.runs.shape[0])


def part_runs(req: ListRequest) -> PartRuns:
    """Runs of a flat particle request: a run ends where the next entry is
    not the next particle with the same replica code, or at a bucket's end.
    Expanding the runs gives back req.list exactly (expand_runs)."""
    lst = req.list
    n = lst.shape[0]
    idx, off = lst[:, 0], lst[:, 1]
    brk = np.ones(n, dtype=bool)
    if n > 1:
        np.not_equal(idx[1:], idx[:-1] + 1, out=brk[1:])
        brk[1:] |= off[1:] != off[:-1]
    mk = req.markers.astype(np.int64)
    brk[mk[:-1][mk[:-1] < n]] = True
    first = np.flatnonzero(brk)
    num = np.diff(np.append(first, n))
    runs = np.empty((len(first), 3), dtype=np.int32)
    runs[:, 0] = idx[first]
    runs[:, 1] = off[first]
    runs[:, 2] = num
    run_markers = np.searchsorted(first, mk).astype(np.int32)
    return PartRuns(runs, run_markers, req.markers, req.starts, req.sizes)


def expand_runs(pr: PartRuns) -> np.ndarray:
    """The flat (L x 2) entries of a PartRuns (numpy; the check of part_runs)."""
    num = pr.runs[:, 2].astype(np.int64)
    rep = np.repeat(np.arange(len(num)), num)
    first = np.repeat(np.cumsum(num) - num, num)
    out = np.empty((int(num.sum()), 2), dtype=np.int32)
    out[:, 0] = pr.runs[rep, 0] + (np.arange(len(rep)) - first)
    out[:, 1] = pr.runs[rep, 1]
    return out


def concat_systems(systems):
    """Concatenates independent systems into one TreeLists with one pair of
    requests (list indices and bucket starts shifted), for one batched
    evaluation.  meta["offsets"] holds each system's first particle."""
    parts = np.concatenate([s.parts for s in systems], axis=0)
    moments = np.concatenate([s.moments for s in systems], axis=0)
    p_off = np.cumsum([0] + [s.n for s in systems])
    m_off = np.cumsum([0] + [s.moments.shape[0] for s in systems])

    def cat(reqs, idx_off):
        ne = np.cumsum([0] + [r.n_entries for r in reqs])
        nb = np.cumsum([0] + [r.n_buckets for r in reqs])
        if ne[-1] >= 2 ** 31:
            raise ValueError("batched list exceeds int32 markers")
        lst = np.empty((int(ne[-1]), 2), np.int32)
        mk = np.empty(int(nb[-1]) + 1, np.int32)
        starts = np.empty(int(nb[-1]), np.int32)
        sizes = np.empty(int(nb[-1]), np.int32)
        ids = np.empty(int(nb[-1]), np.int32)
        mk[0] = 0
        for k, r in enumerate(reqs):
            e0, e1, b0, b1 = ne[k], ne[k + 1], nb[k], nb[k + 1]
            np.add(r.list[:, 0], np.int32(idx_off[k]), out=lst[e0:e1, 0])
            lst[e0:e1, 1] = r.list[:, 1]
            mk[b0 + 1:b1 + 1] = r.markers[1:] + np.int32(e0)
            starts[b0:b1] = r.starts + np.int32(p_off[k])
            sizes[b0:b1] = r.sizes
            ids[b0:b1] = r.bucket_ids
        return ListRequest(lst, mk, starts, sizes, ids)

    cells = cat([s.cells for s in systems], m_off)
    plist = cat([s.plist for s in systems], p_off)
    n = int(p_off[-1])
    return TreeLists(n=n, parts=parts, moments=moments, root=None,
                     perm=np.concatenate([s.perm + p_off[k] for k, s in enumerate(systems)]),
                     bucket_starts=np.concatenate([s.bucket_starts + p_off[k]
                                                   for k, s in enumerate(systems)]),
                     bucket_sizes=np.concatenate([s.bucket_sizes for s in systems]),
                     bucket_bbox=np.concatenate([s.bucket_bbox for s in systems]),
                     cells=cells, plist=plist, period=0.0, n_replicas=0,
                     theta=systems[0].theta, n_bucket=systems[0].n_bucket,
                     meta={"offsets": p_off, "moment_offsets": m_off})
