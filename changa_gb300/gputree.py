"""Tree built on the GPU (changa_tree_build), wrapped so the GPU walk and
DeviceSystem take it like a host TreeLists: positions to forces without
leaving the device.

    tree = DeviceTree(pos, mass, soft, n_bucket=16, theta=0.7)  # device FP64 tensors
    cells, plist, _ = walk.gpu_walk(tree)
    vars = gravity.DeviceSystem(tree, device_reqs=[cells, plist]).step("mixed")
    acc = vars[:, :3][tree.inverse_perm()]                      # caller order

The arrays stay owned by the library handle; torch tensors view them
(CUDA array interface), and every view keeps the handle alive, so the
device memory outlives the last view (or an explicit close()).
"""
from __future__ import annotations

import ctypes as C

from . import _native as N


class _CudaArray:
    """A CUDA array interface provider; torch keeps the provider (and so
    `owner`, the holder of the memory) alive as long as the tensor."""

    def __init__(self, ptr, shape, typestr, owner):
        self.owner = owner
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3}


def _view(ptr, shape, typestr, owner):
    import torch
    return torch.as_tensor(_CudaArray(ptr, shape, typestr, owner), device="cuda")


class _TreeHandle:
    """Owns one changa_tree_build result; frees it once."""

    def __init__(self, handle):
        self.handle = handle

    def free(self):
        if self.handle:
            N.cuda_lib().changa_tree_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DeviceTree:
    order = 2

    def __init__(self, pos, mass, soft, n_bucket=16, theta=0.7, period=0.0, n_replicas=0,
                 stream=None):
        import torch
        lib = N.cuda_lib()
        pos = pos.contiguous().to(torch.float64)
        mass = mass.contiguous().to(torch.float64)
        soft = soft.contiguous().to(torch.float64)
        self._keep = (pos, mass, soft)
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        handle = lib.changa_tree_build(pos.data_ptr(), mass.data_ptr(), soft.data_ptr(),
                                       pos.shape[0], int(n_bucket), s)
        if not handle:
            N.check(lib.changa_gb300_last_error() or N.CHANGA_ERRORS_RECORD, "changa_tree_build")
        self._h = _TreeHandle(handle)
        a = N.ChangaTreeArrays()
        N.check(lib.changa_tree_view(handle, C.byref(a)), "changa_tree_view")
        h = self._h
        n, nm, nb = int(a.n), int(a.n_nodes), int(a.n_buckets)
        self.n, self.n_nodes, self.n_buckets = n, nm, nb
        self.n_bucket, self.theta = int(n_bucket), float(theta)
        self.period, self.n_replicas = float(period), int(n_replicas if period else 0)
        if period and not self.n_replicas:
            self.n_replicas = 1
        self.perm = _view(a.perm, (n,), "<i4", h)
        self.parts = _view(a.parts, (n, 5), "<f8", h)
        self.moments = _view(a.moments, (nm, 12), "<f8", h)
        self.meta = {"node_geom": _view(a.geom, (nm, 6), "<f8", h),
                     "node_bbox": _view(a.bbox, (nm, 6), "<f8", h),
                     "node_info": _view(a.info, (nm, 4), "<i4", h),
                     "parent": _view(a.parent, (nm,), "<i4", h),
                     "bucket_node": _view(a.bucket_node, (nb,), "<i4", h),
                     "leaf": _view(a.leaf, (n,), "<i4", h)}
        self.box = _view(a.box, (6,), "<f8", h)
        self.root = None

    def inverse_perm(self):
        """Index array taking GPU-order rows to caller order."""
        import torch
        inv = torch.empty_like(self.perm, dtype=torch.int64)
        inv[self.perm.long()] = torch.arange(self.n, device=self.perm.device)
        return inv

    @property
    def handle(self):
        return self._h.handle

    def close(self):
        """Frees the device arrays now (the views must not be used after)."""
        self._h.free()
