"""Interaction lists built on the GPU (changa_walk_count / changa_walk_fill).

``gpu_walk(lists)`` takes the tree of a TreeLists (node arrays exported by
the host build) and returns device-resident requests for every bucket: the
same per-bucket entries as the host walk, in depth-first order, ready for
DeviceSystem.  torch supplies device memory and the prefix sums only.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _native as N


class DeviceListRequest:
    """A list request whose arrays live on the device (torch tensors)."""

    def __init__(self, list, markers, starts, sizes):
        self.list, self.markers, self.starts, self.sizes = list, markers, starts, sizes
        self.n_buckets = int(starts.shape[0])
        self.n_entries = int(list.shape[0])

    def interactions(self):
        lens = (self.markers[1:] - self.markers[:-1]).long()
        return int((lens * self.sizes.long()).sum().item())

    def to_host(self):
        """(list, markers) as numpy arrays."""
        return self.list.cpu().numpy(), self.markers.cpu().numpy()


class _WalkLists:
    """Owns the device lists of one changa_walk call until collected."""

    def __init__(self, lib, res):
        self.lib, self.res = lib, res

    def __del__(self):
        try:
            self.lib.changa_walk_lists_free(C.byref(self.res))
        except Exception:
            pass


def gpu_walk(lists, device="cuda", stream=None, timings=None, method="single"):
    """Walks lists' tree on the GPU; returns (cells, plist, softcells or None)
    as DeviceListRequests over all buckets (bucket b at position b).

    method "single": one library call (changa_walk: counts, prefix sums and
    entries, library-owned lists); "two_pass": changa_walk_count, torch
    prefix sums, changa_walk_fill into torch-owned lists."""
    import torch
    lib = N.cuda_lib()
    m = lists.meta
    t = lambda a: (a.to(device) if isinstance(a, torch.Tensor)
                   else torch.from_numpy(np.ascontiguousarray(a)).to(device))
    t0 = time.perf_counter()
    geom, bbox, info = t(m["node_geom"]), t(m["node_bbox"]), t(m["node_info"])
    parent, bnode = t(m["parent"]), t(m["bucket_node"])
    tv = N.ChangaTreeView(geom.data_ptr(), bbox.data_ptr(), info.data_ptr(), parent.data_ptr(),
                          int(geom.shape[0]), bnode.data_ptr(), int(bnode.shape[0]))
    order = getattr(lists, "order", 2)
    wp = N.ChangaWalkParams(float(lists.theta), int(order), float(lists.period),
                            int(lists.n_replicas))
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    nb = int(bnode.shape[0])
    if method == "single":
        from .gputree import _view
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        res = N.ChangaWalkLists()
        N.check(lib.changa_walk(C.byref(tv), C.byref(wp), C.byref(res), s), "changa_walk")
        owner = _WalkLists(lib, res)
        t2 = time.perf_counter()
        starts = info[bnode.long(), 2].contiguous()
        sizes = info[bnode.long(), 3].contiguous()
        reqs = []
        for k in range(3 if order == 4 else 2):
            n = int(res.n_entries[k])
            # the views keep `owner` (and so the lists) alive
            lst = _view(res.list[k], (n, 2), "<i4", owner)
            mk = _view(res.markers[k], (nb + 1,), "<i4", owner)
            reqs.append(DeviceListRequest(lst, mk, starts, sizes))
        if timings is not None:
            timings.update(upload_s=t1 - t0, walk_s=t2 - t1, passes=int(res.passes))
        return reqs[0], reqs[1], (reqs[2] if order == 4 else None)
    if method != "two_pass":
        raise ValueError("method must be 'single' or 'two_pass'")
    counts = [torch.zeros(nb, dtype=torch.int32, device=device) for _ in range(3)]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    N.check(lib.changa_walk_count(C.byref(tv), C.byref(wp), counts[0].data_ptr(),
                                  counts[1].data_ptr(), counts[2].data_ptr() if order == 4 else None,
                                  s), "changa_walk_count")
    offs, lists_out, markers = [], [], []
    for k in range(3):
        c = counts[k].long()
        off = torch.zeros(nb + 1, dtype=torch.int64, device=device)
        off[1:] = torch.cumsum(c, 0)
        total = int(off[-1].item())
        if total >= 2 ** 31:
            raise ValueError("walk lists exceed int32 markers")
        offs.append(off)
        markers.append(off.to(torch.int32))
        lists_out.append(torch.empty((max(total, 1), 2), dtype=torch.int32, device=device)[:total])
    N.check(lib.changa_walk_fill(C.byref(tv), C.byref(wp), offs[0].data_ptr(), offs[1].data_ptr(),
                                 offs[2].data_ptr() if order == 4 else None,
                                 lists_out[0].data_ptr(), lists_out[1].data_ptr(),
                                 lists_out[2].data_ptr() if order == 4 else None, s),
            "changa_walk_fill")
    t2 = time.perf_counter()
    starts = info[bnode.long(), 2].contiguous()
    sizes = info[bnode.long(), 3].contiguous()
    reqs = [DeviceListRequest(lists_out[k], markers[k], starts, sizes) for k in range(3)]
    if timings is not None:
        timings.update(upload_s=t1 - t0, walk_s=t2 - t1)
    return reqs[0], reqs[1], (reqs[2] if order == 4 else None)


def same_entries(host_req, dev_req, n_buckets):
    """True when every bucket holds the same multiset of (index, replica)
    entries in both requests (the host request lists only non-empty
    buckets, by bucket id; the device request lists all buckets)."""
    hl, hm = host_req.list, host_req.markers
    dl, dm = dev_req.to_host()
    ids = np.asarray(host_req.bucket_ids)
    host_of = {int(b): i for i, b in enumerate(ids)}
    for b in range(n_buckets):
        d = dl[dm[b]:dm[b + 1]]
        i = host_of.get(b)
        h = hl[hm[i]:hm[i + 1]] if i is not None else np.empty((0, 2), np.int32)
        if len(d) != len(h):
            return False
        key = lambda a: np.sort(a[:, 0].astype(np.int64) * 1024 + ((a[:, 1] >> 22) & 0x1ff))
        if not np.array_equal(key(d), key(h)):
            return False
    return True


def walk_forces(lists, ewald=None, device="cuda", stream=None, out=None):
    """Forces straight from the tree, with no interaction lists
    (changa_walk_forces: the two-phase walk's second phase evaluates each
    block of accepted cells and opened particles as it decides them,
    FP32-mixed form, quadrupole trees).  lists: a TreeLists or a DeviceTree
    (its node arrays, moments and particles); ewald: a ChangaEwaldParams for
    a periodic tree.  Returns the N x 5 FP64 device array {a.xyz, potential,
    dtGrav} in the tree's particle order (written, then the Ewald term
    added)."""
    import torch
    lib = N.cuda_lib()
    m = lists.meta
    t = lambda a: (a.to(device) if isinstance(a, torch.Tensor)
                   else torch.from_numpy(np.ascontiguousarray(a)).to(device))
    geom, bbox, info = t(m["node_geom"]), t(m["node_bbox"]), t(m["node_info"])
    parent, bnode = t(m["parent"]), t(m["bucket_node"])
    moments, parts = t(lists.moments).contiguous(), t(lists.parts).contiguous()
    tv = N.ChangaTreeView(geom.data_ptr(), bbox.data_ptr(), info.data_ptr(), parent.data_ptr(),
                          int(geom.shape[0]), bnode.data_ptr(), int(bnode.shape[0]))
    wp = N.ChangaWalkParams(float(lists.theta), int(getattr(lists, "order", 2)),
                            float(lists.period), int(lists.n_replicas))
    n = int(parts.shape[0])
    if out is None:
        out = torch.empty((n, 5), dtype=torch.float64, device=device)
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    N.check(lib.changa_walk_forces(C.byref(tv), C.byref(wp), moments.data_ptr(), parts.data_ptr(),
                                   n, C.byref(ewald) if ewald is not None else None,
                                   out.data_ptr(), s), "changa_walk_forces")
    return out
