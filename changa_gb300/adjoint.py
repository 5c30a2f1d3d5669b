"""Differentiated tree gravity: the adjoint kernels behind a leapfrog.

ChaNGa itself has no gradient path; this module adds one on top of the
same tree, walk and interaction lists:

* ``TreeStep``  -- one tree (topology + lists) built at one set of positions
  and held on the device.  ``accel`` runs the list forces
  (changa_gravity_step), ``vjp`` the hand-written adjoint kernels
  (changa_gravity_vjp_mixed: dL/dx and dL/dm from lambda = dL/da; for a
  periodic system changa_ewald_vjp adds the Ewald term's part), and
  ``load`` moves the particles while keeping the topology (the device moment
  up-pass changa_tree_moments refreshes the moments), which is the function
  the adjoint differentiates: lists and topology fixed, moments exact.
* ``Leapfrog``  -- kick-drift-kick integration (the reference's
  Main::advanceBigStep order: half kick, drift, half kick;
  ParallelGravity.cpp) with the tree rebuilt every step (on the host, or on
  the GPU with builder="device"), and its reverse pass with checkpoints every k steps: the forward keeps only
  (x, v) at every k-th step; the reverse pass re-runs each k-step segment
  from its checkpoint (rebuilding the same trees, since the build and the
  forces are deterministic) and walks it backwards.

The reverse pass of one KDK step (x_k, v_k) -> (x_{k+1}, v_{k+1}) with
adjoints xb, vb:  vb += dt xb (drift), then one VJP at x_k with
lambda = dt vb (dt/2 vb at x_0), as the half kicks of two consecutive steps
share a(x_k); the final position gets lambda = dt/2 vb_T.  All state is
FP64 on the device in the caller's particle order; torch supplies device
memory and the elementwise updates only.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .gravity import DeviceSystem
from .tree import build_lists


class TreeStep:
    """Tree, lists and device arrays for one set of positions.

    builder "host": the host tree build, walk and serialisation
    (tree.build_lists), uploaded.  builder "device": the tree built on the
    GPU (gputree.DeviceTree) and walked there (walk.gpu_walk); the positions
    never leave the device.  Both give the same tree and the same
    per-bucket entries."""

    def __init__(self, x, mass, soft, theta=0.7, n_bucket=16, device="cuda", nthreads=0,
                 builder="host", period=0.0, ewald=None):
        """period, ewald: a periodic system (host builder): the walk covers
        one replica shell and ewald (gravity.EwaldConfig) adds the Ewald
        term, whose root parameters follow every load."""
        import torch
        self.torch = torch
        self.period = float(period)
        if builder == "device":
            if period:
                raise ValueError("the device builder walks isolated systems")
            self._init_device(x, mass, soft, theta, n_bucket, device)
            return
        if builder != "host":
            raise ValueError("builder must be 'host' or 'device'")
        x_h = x.detach().cpu().numpy() if hasattr(x, "detach") else np.asarray(x)
        m_h = mass.detach().cpu().numpy() if hasattr(mass, "detach") else np.asarray(mass)
        s_h = soft.detach().cpu().numpy() if hasattr(soft, "detach") else np.asarray(soft)
        lists = build_lists(x_h, m_h, s_h, n_bucket=n_bucket, theta=theta, nthreads=nthreads,
                            period=self.period, n_replicas=1 if self.period else 0)
        self.lists = lists
        self.n = lists.n
        self.ds = DeviceSystem(lists, device=device, ewald=ewald if self.period else None)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
        self.perm = t(lists.perm)
        self.parent = t(lists.meta["parent"])
        self.leaf = t(lists.meta["leaf"])
        self.first = t(lists.meta["first"])
        self.count = t(lists.meta["count"])
        self.interactions = lists.interactions

    def _init_device(self, x, mass, soft, theta, n_bucket, device):
        from .gputree import DeviceTree
        from .walk import gpu_walk
        torch = self.torch
        f = lambda a: torch.as_tensor(a, dtype=torch.float64, device=device).detach()
        tree = DeviceTree(f(x), f(mass), f(soft), n_bucket=n_bucket, theta=theta)
        cells, plist, _ = gpu_walk(tree)
        self.tree = tree
        self.lists = tree
        self.n = tree.n
        self.ds = DeviceSystem(tree, device=device, device_reqs=[cells, plist])
        self.perm = tree.perm.long()
        self.parent = tree.meta["parent"]
        self.leaf = tree.meta["leaf"]
        info = tree.meta["node_info"]
        self.first = info[:, 2].contiguous()
        self.count = info[:, 3].contiguous()
        self.interactions = cells.interactions() + plist.interactions()

    def _stream(self, stream):
        return stream if stream is not None else self.torch.cuda.current_stream().cuda_stream

    def load(self, x, mass, soft, stream=None):
        """Places the particles (caller order, device FP64) into this tree's
        order and recomputes its moments over the fixed topology."""
        p = self.ds.parts
        p[:, 0] = mass[self.perm]
        p[:, 1] = soft[self.perm]
        p[:, 2:5] = x[self.perm]
        mo = self.ds.moments
        rc = N.cuda_lib().changa_tree_moments(p.data_ptr(), self.n, self.first.data_ptr(),
                                              self.count.data_ptr(), mo.shape[0], mo.data_ptr(),
                                              self._stream(stream))
        N.check(rc, "changa_tree_moments")
        if self.ds.ewald_params is not None:
            # the Ewald term expands about the refreshed root
            self.ds.ewald_params = self.ds.ewald.params(mo[0].cpu().numpy())

    def accel(self, form="mixed", stream=None):
        """Accelerations (caller order, N x 3 FP64) from the current arrays."""
        v = self.ds.step(form, stream=stream)
        a = self.torch.empty((self.n, 3), dtype=self.torch.float64, device=v.device)
        a[self.perm] = v[:, :3]
        return a

    def vjp(self, lam, stream=None):
        """(dL/dx (N x 3), dL/dm (N,)) in caller order for lam = dL/da
        (caller order, N x 3), through the FP32-mixed adjoint kernels."""
        torch = self.torch
        ds = self.ds
        lam_g = lam[self.perm].contiguous()
        grad = torch.zeros((self.n, 4), dtype=torch.float64, device=lam.device)
        rc = N.cuda_lib().changa_gravity_vjp_mixed(
            ds.moments.data_ptr(), ds.moments.shape[0], ds.parts.data_ptr(), self.n,
            C.byref(ds.reqs[0]["c"]), C.byref(ds.reqs[1]["c"]), self.period,
            self.parent.data_ptr(), self.leaf.data_ptr(), lam_g.data_ptr(), grad.data_ptr(),
            self._stream(stream))
        N.check(rc, "changa_gravity_vjp_mixed")
        if ds.ewald_params is not None:
            rc = N.cuda_lib().changa_ewald_vjp(ds.parts.data_ptr(), self.n,
                                               C.byref(ds.ewald_params), lam_g.data_ptr(),
                                               grad.data_ptr(), self._stream(stream))
            N.check(rc, "changa_ewald_vjp")
        gx = torch.empty((self.n, 3), dtype=torch.float64, device=lam.device)
        gm = torch.empty(self.n, dtype=torch.float64, device=lam.device)
        gx[self.perm] = grad[:, :3]
        gm[self.perm] = grad[:, 3]
        return gx, gm


class Leapfrog:
    """KDK leapfrog over tree forces with a checkpointed adjoint.

    mass, soft: device FP64 (N,).  form: force form of the forward pass
    ("mixed" or "fp64"); the adjoint kernels are FP32-mixed.
    """

    def __init__(self, mass, soft, dt, n_steps, theta=0.7, n_bucket=16, checkpoint_every=4,
                 form="mixed", nthreads=0, builder="host"):
        self.mass = mass
        self.soft = soft
        self.dt = float(dt)
        self.n_steps = int(n_steps)
        self.theta = float(theta)
        self.n_bucket = int(n_bucket)
        self.every = max(1, int(checkpoint_every))
        self.form = form
        self.nthreads = nthreads
        self.builder = builder
        self.checkpoints = {}
        self.trees = None
        self.tree_builds = 0
        self.force_evals = 0

    def _tree(self, k, x, trees):
        if trees is not None:
            t = trees[k]
            t.load(x, self.mass, self.soft)
            return t
        self.tree_builds += 1
        return TreeStep(x, self.mass, self.soft, self.theta, self.n_bucket, device=x.device,
                        nthreads=self.nthreads, builder=self.builder)

    def _accel(self, tree):
        self.force_evals += 1
        return tree.accel(self.form)

    def forward(self, x0, v0, trees=None, keep_trees=False):
        """Integrates n_steps; returns (x_T, v_T).  trees: one TreeStep per
        position to reuse (fixed topology) instead of rebuilding;
        keep_trees: keep every position's tree in self.trees."""
        dt = self.dt
        x, v = x0.clone(), v0.clone()
        self.checkpoints = {0: (x.clone(), v.clone())}
        kept = [] if keep_trees else None
        t = self._tree(0, x, trees)
        if kept is not None:
            kept.append(t)
        a = self._accel(t)
        for k in range(self.n_steps):
            v += 0.5 * dt * a
            x += dt * v
            t = self._tree(k + 1, x, trees)
            if kept is not None:
                kept.append(t)
            a = self._accel(t)
            v += 0.5 * dt * a
            if (k + 1) % self.every == 0 and k + 1 < self.n_steps:
                self.checkpoints[k + 1] = (x.clone(), v.clone())
        if keep_trees:
            self.trees = kept
        return x, v

    def backward(self, xbar_T, vbar_T, trees=None):
        """Reverse pass: given dL/dx_T and dL/dv_T, returns
        (dL/dx_0, dL/dv_0, dL/dm).  Uses the checkpoints of the last
        forward; trees as in forward."""
        import torch
        dt = self.dt
        xb = xbar_T.clone()
        vb = vbar_T.clone()
        mb = torch.zeros_like(self.mass)
        starts = sorted(self.checkpoints)
        for s in reversed(starts):
            e = min(s + self.every, self.n_steps)
            seg = self._replay(s, e, trees)
            if e == self.n_steps:
                gx, gm = seg[e - s].vjp(0.5 * dt * vb)
                xb += gx
                mb += gm
            for k in range(e - 1, s - 1, -1):
                vb += dt * xb
                lam = (dt if k > 0 else 0.5 * dt) * vb
                gx, gm = seg[k - s].vjp(lam)
                xb += gx
                mb += gm
        return xb, vb, mb

    def _replay(self, s, e, trees):
        """Trees of positions s..e (the last only when e is the final
        position), re-integrated from checkpoint s."""
        dt = self.dt
        x, v = (c.clone() for c in self.checkpoints[s])
        t = self._tree(s, x, trees)
        seg = [t]
        last = e if e == self.n_steps else e - 1
        k = s
        if k < last:
            a = self._accel(t)
        while k < last:
            v += 0.5 * dt * a
            x += dt * v
            t = self._tree(k + 1, x, trees)
            seg.append(t)
            k += 1
            if k < last:
                a = self._accel(t)
                v += 0.5 * dt * a
        return seg


def loss_weights(n, seed, device="cuda"):
    """w_i ~ N(0, 1)^3 of the loss L = sum_i w_i . x_i(T) (seeded PCG64)."""
    import torch
    rng = np.random.Generator(np.random.PCG64(seed))
    return torch.from_numpy(rng.standard_normal((n, 3))).to(device)
