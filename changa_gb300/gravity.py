"""Python wrappers over the C-ABI of the gravity library.

Three ways in, all through ``libchanga_gb300.so``:

* ``dropin_step``     -- the reference-facing path: HostCUDA.h / EwaldCUDA.h
                         entry points with HOST buffers in the FP32 ABI
                         structs, the call sequence ChaNGa's DataManager and
                         ListCompute make (transfer tree, cell request,
                         particle request, Ewald, transfer results back).
* ``gravity_step_host`` -- the FP64 / FP32-mixed forms from host arrays
                         (changa_gravity_step_host).
* ``DeviceSystem``    -- the same forms on device-resident inputs held in
                         torch tensors (changa_gravity_step); torch provides
                         device memory and streams only.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N

FORMS = {"fp64": N.CHANGA_FORM_FP64, "mixed": N.CHANGA_FORM_MIXED}


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _cudart():
    """The CUDA runtime (for cudaFree / cudaStreamSynchronize of buffers the
    drop-in entry points allocate, as ChaNGa's DataManager does)."""
    import ctypes.util
    import os
    for name in ("/usr/local/cuda/lib64/libcudart.so", "libcudart.so.13", "libcudart.so"):
        try:
            lib = C.CDLL(name if os.path.isabs(name) else (ctypes.util.find_library("cudart") or name))
            lib.cudaFree.argtypes = [C.c_void_p]
            lib.cudaStreamSynchronize.argtypes = [C.c_void_p]
            return lib
        except OSError:
            continue
    raise RuntimeError("CUDA runtime library not found")


class EwaldConfig:
    """Periodic Ewald parameters (Ewald.cpp / ParallelGravity.cpp:432-440
    defaults: fEwCut 2.6, dEwhCut 2.8)."""

    def __init__(self, L=1.0, n_reps=1, fEwCut=2.6, dEwhCut=2.8):
        self.L, self.n_reps, self.fEwCut, self.dEwhCut = float(L), int(n_reps), float(fEwCut), float(dEwhCut)

    def table(self, root):
        out = np.zeros((N.CHANGA_MAX_EWH, 5))
        n = N.cuda_lib().changa_ewald_table(_p(np.ascontiguousarray(root, np.float64)), self.L,
                                            self.dEwhCut, _p(out), N.CHANGA_MAX_EWH)
        if n < 0:
            raise ValueError("Ewald h-table larger than %d rows" % N.CHANGA_MAX_EWH)
        return out[:n].copy()

    def params(self, root):
        """ChangaEwaldParams (keeps the table alive on the returned object)."""
        p = N.ChangaEwaldParams()
        for i in range(12):
            p.root[i] = float(root[i])
        p.L = self.L
        p.nReps = self.n_reps
        p.fEwCut = self.fEwCut
        tb = np.ascontiguousarray(self.table(root))
        p.nEwhLoop = tb.shape[0]
        p.ewt = tb.ctypes.data
        p._keep = tb
        return p

    def params_hex(self, root):
        """ChangaEwaldParams of the hexadecapole build for a 27-value root:
        mass and centre in root[2..5], the complete moments in momc."""
        p = N.ChangaEwaldParams()
        for i in range(6):
            p.root[i] = float(root[i])
        p.L = self.L
        p.nReps = self.n_reps
        p.fEwCut = self.fEwCut
        tb, momc = self.table_hex(root)
        tb = np.ascontiguousarray(tb)
        momc = np.ascontiguousarray(momc)
        p.nEwhLoop = tb.shape[0]
        p.ewt = tb.ctypes.data
        p.momc = momc.ctypes.data
        p._keep = (tb, momc)
        return p

    def table_hex(self, root):
        """The hexadecapole build's table for a 27-value root, and the root's
        complete moments (MomcData order)."""
        out = np.zeros((N.CHANGA_MAX_EWH, 5))
        momc = np.zeros(32)
        n = N.cuda_lib().changa_ewald_table_hex(_p(np.ascontiguousarray(root, np.float64)), self.L,
                                                self.dEwhCut, _p(out), N.CHANGA_MAX_EWH, _p(momc))
        if n < 0:
            raise ValueError("Ewald h-table larger than %d rows" % N.CHANGA_MAX_EWH)
        return out[:n].copy(), momc

    def readonly_f32_hex(self, root, n_active, momc):
        """EwaldReadOnlyData of the hexadecapole build as TreePiece::EwaldGPU
        fills it (Ewald.cpp:452-516): the complete root moments, mass and
        centre rounded to float."""
        q = self.readonly_f32(np.concatenate([root[:6], np.zeros(6)]), n_active)
        ro = N.EwaldReadOnlyDataHex()
        for f, _ in N.EwaldReadOnlyDataHex._fields_:
            if f not in ("mm", "momcRoot"):
                setattr(ro, f, getattr(q, f))
        ro.mm.totalMass = q.mm.totalMass
        ro.mm.cmx, ro.mm.cmy, ro.mm.cmz = q.mm.cmx, q.mm.cmy, q.mm.cmz
        for k, (f, _) in enumerate(N.MomcData._fields_):
            setattr(ro.momcRoot, f, float(np.float32(momc[k])))
        return ro

    def readonly_f32(self, root, n_active):
        """EwaldReadOnlyData as TreePiece::EwaldGPU fills it (Ewald.cpp:470-516)."""
        ro = N.EwaldReadOnlyData()
        mm = ro.mm
        mm.xx, mm.xy, mm.xz, mm.yy, mm.yz, mm.zz = [float(np.float32(root[k])) for k in range(6, 12)]
        mm.totalMass = float(np.float32(root[2]))
        mm.cmx, mm.cmy, mm.cmz = [float(np.float32(root[k])) for k in (3, 4, 5)]
        L = np.float32(self.L)
        alpha = np.float32(2.0) / L
        ro.n = int(n_active)
        ro.fEwCut = float(np.float32(self.fEwCut))
        ro.nReps = self.n_reps
        ro.nEwReps = int(math.ceil(self.fEwCut))
        ro.L = float(L)
        ro.alpha = float(alpha)
        ro.alpha2 = float(np.float32(alpha * alpha))
        ro.k1 = float(np.float32(math.pi / (float(alpha) * float(alpha) * float(L) ** 3)))
        ro.ka = float(np.float32(2.0 * float(alpha) / math.sqrt(math.pi)))
        ro.fEwCut2 = float(np.float32(self.fEwCut * self.fEwCut * float(L) * float(L)))
        ro.fInner2 = float(np.float32(1.1e-2 * float(L) * float(L)))
        return ro


def _host_req(req):
    """ChangaListRequest over host numpy arrays (kept alive by the caller)."""
    r = N.ChangaListRequest()
    r.list = req.list.ctypes.data
    r.markers = req.markers.ctypes.data
    r.starts = req.starts.ctypes.data
    r.sizes = req.sizes.ctypes.data
    r.n_buckets = req.n_buckets
    r.n_entries = req.n_entries
    return r


def host_runs(pr):
    """ChangaPartRuns over a tree.PartRuns (host numpy arrays, kept alive by
    the caller)."""
    r = N.ChangaPartRuns()
    r.runs = pr.runs.ctypes.data
    r.run_markers = pr.run_markers.ctypes.data
    r.markers = pr.markers.ctypes.data
    r.starts = pr.starts.ctypes.data
    r.sizes = pr.sizes.ctypes.data
    r.n_buckets = pr.n_buckets
    r.n_runs = pr.n_runs
    return r


def gravity_step_host(lists, form="mixed", ewald: EwaldConfig | None = None, stream=None,
                      vars=None, overwrite=False, runs=None):
    """One force evaluation from host arrays; returns vars (N x 5 FP64).
    Results accumulate into vars unless overwrite (then vars is not read).
    With runs (a tree.PartRuns of lists.plist) the particle lists travel as
    runs (changa_gravity_step_host_runs)."""
    lib = N.cuda_lib()
    if vars is None:
        vars = np.empty((lists.n, 5)) if overwrite else np.zeros((lists.n, 5))
    cr = _host_req(lists.cells)
    ep = ewald.params(lists.root) if ewald else None
    f = FORMS[form] | (N.CHANGA_STEP_OVERWRITE if overwrite else 0)
    if runs is not None:
        rr = host_runs(runs)
        rc = lib.changa_gravity_step_host_runs(f, _p(lists.moments), lists.moments.shape[0],
                                               _p(lists.parts), lists.n, C.byref(cr), C.byref(rr),
                                               float(lists.period), C.byref(ep) if ep else None,
                                               _p(vars), stream)
        N.check(rc, "changa_gravity_step_host_runs")
        return vars
    pr = _host_req(lists.plist)
    rc = lib.changa_gravity_step_host(f, _p(lists.moments), lists.moments.shape[0],
                                      _p(lists.parts), lists.n, C.byref(cr), C.byref(pr),
                                      float(lists.period), C.byref(ep) if ep else None, _p(vars),
                                      stream)
    N.check(rc, "changa_gravity_step_host")
    return vars


class PinnedArray:
    """Host array in page-locked memory from allocatePinnedHostMemory."""

    def __init__(self, arr):
        arr = np.ascontiguousarray(arr)
        self.nbytes = max(arr.nbytes, 1)
        self.ptr = C.c_void_p()
        N.cuda_lib().allocatePinnedHostMemory(C.byref(self.ptr), self.nbytes)
        if not self.ptr.value:
            raise MemoryError("pinned allocation failed")
        buf = (C.c_char * self.nbytes).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=arr.dtype, count=arr.size).reshape(arr.shape)
        self.array[...] = arr

    def free(self):
        if self.ptr.value:
            N.cuda_lib().freePinnedHostMemory(self.ptr)
            self.ptr = C.c_void_p()


class DropInInputs:
    """The host buffers ChaNGa would hand the drop-in boundary for one
    force evaluation (pinned, FP32 ABI structs), built once.  Lists of
    order 4 go to the HEXADECAPOLE build of the library (108-byte moments,
    the hexadecapole Ewald data); their softened cells are the caller's
    (ChaNGa evaluates them on the CPU, Compute.cpp:1683-1698)."""

    def __init__(self, lists, ewald: EwaldConfig | None = None):
        self.lists = lists
        self.n = lists.n
        self.hex = getattr(lists, "order", 2) == 4
        self.lib = N.cuda_lib_hex() if self.hex else N.cuda_lib()
        self.moments = PinnedArray(lists.abi_moments())
        self.parts = PinnedArray(lists.abi_parts())
        self.vars = PinnedArray(np.zeros((lists.n, 5), np.float32))
        self.out = PinnedArray(np.zeros((lists.n, 5), np.float32))
        self.reqs = []
        for req in (lists.cells, lists.plist):
            self.reqs.append((PinnedArray(req.list), PinnedArray(req.markers),
                              PinnedArray(req.starts), PinnedArray(req.sizes), req))
        self.ewald = ewald
        self.ewald_data = None
        if ewald is not None:
            ed = N.EwaldData()
            lib = self.lib
            lib.EwaldHostMemorySetup(C.byref(ed), self.n, N.CHANGA_MAX_EWH, 1)
            if self.hex:
                tb, momc = ewald.table_hex(lists.moments[0])
            else:
                tb = ewald.table(lists.root)
            ewt = (N.EwtData * tb.shape[0]).from_address(ed.ewt)
            for i in range(tb.shape[0]):
                ewt[i].hx, ewt[i].hy, ewt[i].hz, ewt[i].hCfac, ewt[i].hSfac = [float(np.float32(x)) for x in tb[i]]
            if self.hex:
                ro = ewald.readonly_f32_hex(lists.moments[0], self.n, momc)
            else:
                ro = ewald.readonly_f32(lists.root, self.n)
            ro.nEwhLoop = tb.shape[0]
            C.memmove(ed.cachedData, C.byref(ro), C.sizeof(ro))
            mk = (C.c_int * self.n).from_address(ed.EwaldMarkers)
            np.frombuffer(mk, dtype=np.int32)[:] = np.arange(self.n, dtype=np.int32)
            ed.EwaldRange[0] = 0
            ed.EwaldRange[1] = self.n - 1
            self.ewald_data = ed
        self.h2d_bytes = (self.moments.nbytes + self.parts.nbytes + self.vars.nbytes +
                          sum(a.nbytes for r in self.reqs for a in r[:4]) +
                          (self.n * 4 if ewald else 0))
        self.d2h_bytes = self.out.nbytes

    def free(self):
        for a in (self.moments, self.parts, self.vars, self.out):
            a.free()
        for r in self.reqs:
            for a in r[:4]:
                a.free()
        if self.ewald_data is not None:
            self.lib.EwaldHostMemoryFree(C.byref(self.ewald_data), 1)
            self.ewald_data = None


def dropin_step(inp: DropInInputs, stream=None, cudart=None):
    """Runs one force evaluation through the reference-facing boundary and
    returns the VariablePartData rows (N x 5 float32, a view of pinned
    memory, valid until the next call).  All device memory is released."""
    lib = inp.lib
    rt = cudart or _cudart()
    d_m, d_p, d_v = C.c_void_p(), C.c_void_p(), C.c_void_p()
    lib.DataManagerTransferLocalTree(inp.moments.ptr, inp.moments.nbytes, inp.parts.ptr,
                                     inp.parts.nbytes, inp.vars.ptr, inp.vars.nbytes,
                                     C.byref(d_m), C.byref(d_p), C.byref(d_v), stream, inp.n, None)
    # ChaNGa queues the Ewald launch right after the local tree transfer
    # (DataManager.cpp:495-510, TreePiece::calculateEwald -> EwaldGPU), so
    # it runs while the walk produces the lists and they are uploaded
    if inp.ewald_data is not None:
        lib.EwaldHost(d_p, d_v, C.byref(inp.ewald_data), stream, None, 0, 1)
    for k, (lst, mk, st, sz, req) in enumerate(inp.reqs):
        if req.n_buckets == 0:
            continue
        r = N.CudaRequest()
        r.stream = stream
        r.d_localMoments = d_m
        r.d_localParts = d_p
        r.d_localVars = d_v
        r.list = lst.ptr
        r.bucketMarkers = mk.ptr
        r.bucketStarts = st.ptr
        r.bucketSizes = sz.ptr
        r.numInteractions = req.n_entries
        r.numBucketsPlusOne = req.n_buckets + 1
        r.fperiod = float(inp.lists.period)
        r.node = k == 0
        if k == 0:
            lib.TreePieceCellListDataTransferLocal(C.byref(r))
        else:
            lib.TreePiecePartListDataTransferLocal(C.byref(r))
    lib.TransferParticleVarsBack(inp.out.ptr, inp.out.nbytes, d_v, stream, None)
    rt.cudaStreamSynchronize(stream)
    for p in (d_m, d_p, d_v):
        rt.cudaFree(p)
    return inp.out.array


class DeviceSystem:
    """Device-resident inputs of one force evaluation (torch tensors)."""

    def __init__(self, lists, device="cuda", ewald: EwaldConfig | None = None,
                 device_reqs=None):
        """device_reqs: requests built on the device (walk.gpu_walk) to use
        instead of the host lists' (cells, plist[, softcells])."""
        import torch
        self.torch = torch
        self.lists = lists
        self.n = lists.n
        t = lambda a: (a.to(device) if isinstance(a, torch.Tensor)
                       else torch.from_numpy(np.ascontiguousarray(a)).to(device))
        self.moments = t(lists.moments)
        self.parts = t(lists.parts)
        self.reqs = []
        self.order = getattr(lists, "order", 2)
        reqs = list(device_reqs) if device_reqs is not None else [lists.cells, lists.plist]
        if self.order == 4 and device_reqs is None:
            reqs.append(lists.softcells)
        for req in reqs:
            d = dict(list=t(req.list), markers=t(req.markers), starts=t(req.starts), sizes=t(req.sizes))
            r = N.ChangaListRequest()
            r.list = d["list"].data_ptr()
            r.markers = d["markers"].data_ptr()
            r.starts = d["starts"].data_ptr()
            r.sizes = d["sizes"].data_ptr()
            r.n_buckets = req.n_buckets
            r.n_entries = req.n_entries
            d["c"] = r
            self.reqs.append(d)
        self.vars = torch.zeros((lists.n, 5), dtype=torch.float64, device=device)
        self.ewald = ewald
        root = lists.root
        if ewald is not None and (root is None or self.order == 4):
            # a device-built tree or the hexadecapole build: the root moments
            root = self.moments[0].cpu().numpy()
        if ewald is None:
            self.ewald_params = None
        elif self.order == 4:
            self.ewald_params = ewald.params_hex(root)
        else:
            self.ewald_params = ewald.params(root)

    def step(self, form="mixed", stream=None, zero=True):
        """Enqueues one evaluation on `stream` (torch stream handle or None for
        the current torch stream); results accumulate into self.vars."""
        torch = self.torch
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        if zero:
            self.vars.zero_()
        if self.order == 4:
            rc = N.cuda_lib().changa_gravity_step_hexa(
                FORMS[form], self.moments.data_ptr(), self.moments.shape[0],
                self.parts.data_ptr(), self.n, C.byref(self.reqs[0]["c"]),
                C.byref(self.reqs[1]["c"]), C.byref(self.reqs[2]["c"]),
                float(self.lists.period),
                C.byref(self.ewald_params) if self.ewald_params else None,
                self.vars.data_ptr(), s)
            N.check(rc, "changa_gravity_step_hexa")
            return self.vars
        ep = self.ewald_params
        rc = N.cuda_lib().changa_gravity_step(
            FORMS[form], self.moments.data_ptr(), self.moments.shape[0], self.parts.data_ptr(),
            self.n, C.byref(self.reqs[0]["c"]), C.byref(self.reqs[1]["c"]), float(self.lists.period),
            C.byref(ep) if ep else None, self.vars.data_ptr(), s)
        N.check(rc, "changa_gravity_step")
        return self.vars


class GravityGraph:
    """One evaluation of a DeviceSystem captured into a CUDA graph
    (changa_gravity_graph_create) and replayed with one launch."""

    def __init__(self, ds: DeviceSystem, form="mixed"):
        if ds.order != 2:
            raise ValueError("the graph form captures the quadrupole evaluation")
        self.ds = ds
        ep = ds.ewald_params
        self.handle = N.cuda_lib().changa_gravity_graph_create(
            FORMS[form], ds.moments.data_ptr(), ds.moments.shape[0], ds.parts.data_ptr(), ds.n,
            C.byref(ds.reqs[0]["c"]), C.byref(ds.reqs[1]["c"]), float(ds.lists.period),
            C.byref(ep) if ep else None, ds.vars.data_ptr(), 1)
        if not self.handle:
            N.check(N.cuda_lib().changa_gb300_last_error() or N.CHANGA_ERRORS_RECORD,
                    "changa_gravity_graph_create")

    def launch(self, stream=None):
        torch = self.ds.torch
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        N.check(N.cuda_lib().changa_gravity_graph_launch(self.handle, s), "graph launch")
        return self.ds.vars

    def close(self):
        if self.handle:
            N.cuda_lib().changa_gravity_graph_destroy(self.handle)
            self.handle = None


def direct_forces(parts, idx, period=0.0, rcut_frac=0.0, stream=None):
    """The direct-sum yardstick (changa_direct_forces) on the particles idx
    of `parts` (device FP64 tensor, parts layout): returns a numpy array
    len(idx) x 4 {ax, ay, az, pot (open boundaries only)}."""
    import torch
    i = torch.from_numpy(np.ascontiguousarray(idx, dtype=np.int32)).to(parts.device)
    out = torch.empty((len(idx), 4), dtype=torch.float64, device=parts.device)
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = N.cuda_lib().changa_direct_forces(parts.data_ptr(), parts.shape[0], i.data_ptr(),
                                           len(idx), float(period), float(rcut_frac),
                                           out.data_ptr(), s)
    N.check(rc, "changa_direct_forces")
    return out.cpu().numpy()
