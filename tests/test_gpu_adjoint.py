"""Adjoint (VJP) kernels and the checkpointed leapfrog reverse pass.

The torch.autograd.Function below exists only in this test harness: it
wraps the hand-written VJP kernels so that torch can compose a leapfrog
whose gradient is compared with the library's own reverse pass.  The
references are central finite differences of the FP64 form over the same
(fixed) trees and lists, and torch FP64 autograd of a spline-softened
direct sum (the softening of gravity.h SPLINE)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plummer(n, seed_index=4):
    from changa_gb300 import ics
    return ics.plummer(n, ics.rng_for(seed_index))


def _dev(p):
    import torch
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    return t(p["pos"]), t(p["vel"]), t(p["mass"]), t(p["soft"])


def _spline_b(r2, twoh):
    """b(r) of SPLINE (gravity.h:147-182) in torch FP64, r2 > 0."""
    import torch
    r = torch.sqrt(r2)
    dih = 2.0 / twoh
    u = r * dih
    b_in = dih ** 3 * (4.0 / 3.0 - 1.2 * u ** 2 + 0.5 * u ** 3)
    b_mid = -1.0 / 15.0 / r ** 3 + dih ** 3 * (8.0 / 3.0 - 3.0 * u + 1.2 * u ** 2 - u ** 3 / 6.0)
    b_far = 1.0 / r ** 3
    return torch.where(u < 1.0, b_in, torch.where(u < 2.0, b_mid, b_far))


def direct_accel(x, m, soft):
    """FP64 direct-sum accelerations a_i = sum_j m_j b(r_ij) (x_j - x_i)."""
    import torch
    n = x.shape[0]
    r = x[None, :, :] - x[:, None, :]
    r2 = (r * r).sum(-1)
    eye = torch.eye(n, dtype=torch.bool, device=x.device)
    r2s = torch.where(eye, torch.ones_like(r2), r2)
    b = _spline_b(r2s, soft[:, None] + soft[None, :])
    b = torch.where(eye, torch.zeros_like(b), b)
    return ((b * m[None, :])[:, :, None] * r).sum(1)


def _tree_accel_fn():
    import torch

    class TreeAccel(torch.autograd.Function):
        """a(x, m) through one fixed tree; backward = the VJP kernels."""

        @staticmethod
        def forward(ctx, x, m, tree, soft):
            tree.load(x.detach(), m.detach(), soft)
            ctx.tree = tree
            return tree.accel("mixed")

        @staticmethod
        def backward(ctx, g):
            gx, gm = ctx.tree.vjp(g.contiguous())
            return gx, gm, None, None

    return TreeAccel


def _kdk(accel, x, v, dt, n_steps):
    """Plain torch KDK leapfrog; accel(k, x) gives a(x_k)."""
    a = accel(0, x)
    for k in range(n_steps):
        v = v + 0.5 * dt * a
        x = x + dt * v
        a = accel(k + 1, x)
        v = v + 0.5 * dt * a
    return x, v


def test_tree_moments_refresh(cuda_ok):
    from changa_gb300.adjoint import TreeStep
    x, v, m, s = _dev(_plummer(4096))
    t = TreeStep(x, m, s)
    host = t.ds.moments.clone()
    t.load(x, m, s)
    got = t.ds.moments
    tr = (host[:, 6] + host[:, 9] + host[:, 11]).abs().clamp_min(1e-300)
    assert (got[:, 0] == host[:, 0]).all()  # radius kept
    assert ((got[:, 2] - host[:, 2]).abs() / host[:, 2]).max().item() < 1e-12
    assert (got[:, 3:6] - host[:, 3:6]).abs().max().item() < 1e-12
    assert ((got[:, 6:12] - host[:, 6:12]).abs() / tr[:, None]).max().item() < 1e-10
    assert ((got[:, 1] - host[:, 1]).abs() / host[:, 1]).max().item() < 1e-12


def test_vjp_matches_direct_sum_autograd_all_pp(cuda_ok):
    """Tiny theta opens every cell: the lists become the full particle-particle
    sum and the VJP must equal torch FP64 autograd of the direct sum."""
    import torch
    from changa_gb300.adjoint import TreeStep
    x, v, m, s = _dev(_plummer(2048))
    t = TreeStep(x, m, s, theta=1e-3)
    assert t.lists.cells.n_entries == 0
    lam = torch.randn(x.shape, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    gx, gm = t.vjp(lam)
    xr = x.clone().requires_grad_(True)
    mr = m.clone().requires_grad_(True)
    (direct_accel(xr, mr, s) * lam).sum().backward()
    ex = ((gx - xr.grad).norm() / xr.grad.norm()).item()
    em = ((gm - mr.grad).norm() / mr.grad.norm()).item()
    print("all-pp vjp rel err: x %.3e m %.3e" % (ex, em))
    assert ex < 1e-5 and em < 1e-5


def test_vjp_matches_fd_single_evaluation(cuda_ok):
    """sum(lambda . a) through one fixed tree (theta 0.7, cells + particles):
    VJP vs central differences of the FP64 form with refreshed moments."""
    import torch
    from changa_gb300.adjoint import TreeStep
    x, v, m, s = _dev(_plummer(4096))
    t = TreeStep(x, m, s, theta=0.7)
    assert t.lists.cells.n_entries > 0
    lam = torch.randn(x.shape, dtype=torch.float64, device="cuda",
                      generator=torch.Generator("cuda").manual_seed(2))
    t.load(x, m, s)
    gx, gm = t.vjp(lam)

    def f(xx, mm):
        t.load(xx, mm, s)
        return (t.accel("fp64") * lam).sum().item()

    rng = np.random.default_rng(5)
    h = 1e-4
    errs_x, errs_m = [], []
    for i in rng.choice(x.shape[0], 12, replace=False):
        for c in range(3):
            xp, xm_ = x.clone(), x.clone()
            xp[i, c] += h
            xm_[i, c] -= h
            fd = (f(xp, m) - f(xm_, m)) / (2 * h)
            errs_x.append(abs(fd - gx[i, c].item()) / (abs(fd) + 1e-3 * gx.abs().max().item()))
    for i in rng.choice(x.shape[0], 12, replace=False):
        hm = 1e-4 * m[i].item()
        mp, mm_ = m.clone(), m.clone()
        mp[i] += hm
        mm_[i] -= hm
        fd = (f(x, mp) - f(x, mm_)) / (2 * hm)
        errs_m.append(abs(fd - gm[i].item()) / (abs(fd) + 1e-3 * gm.abs().max().item()))
    print("single-eval FD: x max %.3e, m max %.3e" % (max(errs_x), max(errs_m)))
    assert max(errs_x) < 1e-4 and max(errs_m) < 1e-4


def test_leapfrog_reverse_pass_matches_autograd(cuda_ok):
    """The checkpointed reverse pass equals torch autograd composing the
    same VJP kernels (TreeAccel) over the same trees."""
    import torch
    from changa_gb300.adjoint import Leapfrog, loss_weights
    x0, v0, m, s = _dev(_plummer(4096))
    dt, ns = 0.005, 8
    w = loss_weights(x0.shape[0], 7)
    lf = Leapfrog(m, s, dt, ns, theta=0.7, checkpoint_every=4)
    xT, vT = lf.forward(x0, v0, keep_trees=True)
    gx, gv, gm = lf.backward(w, torch.zeros_like(w))
    # forward: ns + 1 trees; reverse pass: the same ns + 1 positions rebuilt
    assert lf.tree_builds == 2 * (ns + 1)
    TreeAccel = _tree_accel_fn()
    trees = lf.trees
    xr = x0.clone().requires_grad_(True)
    vr = v0.clone().requires_grad_(True)
    mr = m.clone().requires_grad_(True)
    xT2, _ = _kdk(lambda k, xx: TreeAccel.apply(xx, mr, trees[k], s), xr, vr, dt, ns)
    assert (xT2.detach() - xT).abs().max().item() < 1e-9
    (xT2 * w).sum().backward()
    for name, a, b in (("x", gx, xr.grad), ("v", gv, vr.grad), ("m", gm, mr.grad)):
        e = ((a - b).norm() / b.norm()).item()
        print("reverse pass vs autograd %s: %.3e" % (name, e))
        assert e < 1e-6, name


def test_leapfrog_device_builder_matches_host(cuda_ok):
    """Trees built and walked on the GPU at every step give the host-built
    leapfrog's trajectory and gradients: the same trees and per-bucket
    entries, summed in another order (FP32-mixed forces)."""
    import torch
    from changa_gb300.adjoint import Leapfrog, loss_weights
    x0, v0, m, s = _dev(_plummer(4096))
    dt, ns = 0.005, 8
    w = loss_weights(x0.shape[0], 7)
    out = {}
    for builder in ("host", "device"):
        lf = Leapfrog(m, s, dt, ns, theta=0.7, checkpoint_every=4, builder=builder)
        xT, vT = lf.forward(x0, v0)
        grads = lf.backward(w, torch.zeros_like(w))
        out[builder] = (xT, vT) + grads
        assert lf.tree_builds == 2 * (ns + 1)
    for name, a, b in zip(("xT", "vT", "gx", "gv", "gm"), out["device"], out["host"]):
        e = ((a - b).norm() / b.norm()).item()
        print("device vs host builder %s: %.3e" % (name, e))
        assert e < 1e-6, name


def _direct_sum_grads(x0, v0, m, s, w, dt, ns):
    import torch
    from torch.utils.checkpoint import checkpoint
    xr = x0.clone().requires_grad_(True)
    vr = v0.clone().requires_grad_(True)
    mr = m.clone().requires_grad_(True)
    acc = lambda k, xx: checkpoint(direct_accel, xx, mr, s, use_reentrant=False)
    xT, _ = _kdk(acc, xr, vr, dt, ns)
    (xT * w).sum().backward()
    return xr.grad, vr.grad, mr.grad


@pytest.mark.parametrize("theta,tol", [(1e-3, 1e-5), (0.7, 2e-2)])
def test_leapfrog_gradient_vs_direct_sum_autograd(cuda_ok, theta, tol):
    """16 KDK steps (dt 0.005) at N=4096: the tree adjoint vs torch FP64
    autograd of the direct sum.  Compared are the force-driven parts of the
    gradients (dL/dx0 - w, dL/dv0 - T w, dL/dm): with theta -> 0 the tree is
    the direct sum; at theta 0.7 the gap is the multipole truncation."""
    import torch
    from changa_gb300.adjoint import Leapfrog, loss_weights
    x0, v0, m, s = _dev(_plummer(4096))
    dt, ns = 0.005, 16
    w = loss_weights(x0.shape[0], 11)
    lf = Leapfrog(m, s, dt, ns, theta=theta, checkpoint_every=4)
    lf.forward(x0, v0)
    gx, gv, gm = lf.backward(w, torch.zeros_like(w))
    rx, rv, rm = _direct_sum_grads(x0, v0, m, s, w, dt, ns)
    T = dt * ns
    for name, a, b in (("x", gx - w, rx - w), ("v", gv - T * w, rv - T * w), ("m", gm, rm)):
        e = ((a - b).norm() / b.norm()).item()
        print("theta %g leapfrog vs direct-sum autograd %s: %.3e" % (theta, name, e))
        assert e < tol, name


def test_leapfrog_gradient_vs_fd_plummer64k(cuda_ok):
    """The differentiation workload: Plummer N=65536, 16 KDK steps, dt 0.005,
    theta 0.7, tree rebuilt each step, FP32-mixed forces, checkpoints every 4
    steps, L = sum w . x(T).  64 sampled coordinates (24 positions, 24
    velocities, 16 masses) against central differences (h = 1e-4; 1e-4
    relative for masses) of the FP64 form over the forward pass's trees."""
    import torch
    from changa_gb300.adjoint import Leapfrog, loss_weights
    x0, v0, m, s = _dev(_plummer(65536))
    dt, ns = 0.005, 16
    w = loss_weights(x0.shape[0], 13)
    lf = Leapfrog(m, s, dt, ns, theta=0.7, checkpoint_every=4)
    lf.forward(x0, v0, keep_trees=True)
    trees = lf.trees
    assert sorted(lf.checkpoints) == [0, 4, 8, 12]
    gx, gv, gm = lf.backward(w, torch.zeros_like(w))
    fd_lf = Leapfrog(m, s, dt, ns, form="fp64")

    def final(xx, vv, mm):
        fd_lf.mass = mm
        xT, _ = fd_lf.forward(xx, vv, trees=trees)
        return xT

    def diff(a, b):
        # w . (x_T(+) - x_T(-)): differencing before the sum keeps the FP64
        # rounding of sum(w . x_T) (~1e-13 here) out of the difference
        return ((a - b) * w).sum().item()

    rng = np.random.default_rng(17)
    h = 1e-4
    rows = []
    for kind, count in (("x", 24), ("v", 24), ("m", 16)):
        for i in rng.choice(x0.shape[0], count, replace=False):
            c = int(rng.integers(3))
            xp, xm_, vp, vm_, mp, mm_ = x0.clone(), x0.clone(), v0.clone(), v0.clone(), m.clone(), m.clone()
            if kind == "x":
                xp[i, c] += h
                xm_[i, c] -= h
                hh, g = h, gx[i, c].item()
            elif kind == "v":
                vp[i, c] += h
                vm_[i, c] -= h
                hh, g = h, gv[i, c].item()
            else:
                hh = h * m[i].item()
                mp[i] += hh
                mm_[i] -= hh
                g = gm[i].item()
            fd = diff(final(xp, vp, mp), final(xm_, vm_, mm_)) / (2 * hh)
            rows.append((kind, fd, g))
    for kind in ("x", "v", "m"):
        fd = np.array([r[1] for r in rows if r[0] == kind])
        g = np.array([r[2] for r in rows if r[0] == kind])
        e = np.abs(g - fd) / (np.abs(fd) + 1e-3 * np.abs(fd).max())
        print("plummer64k FD %s: max rel %.3e median %.3e" % (kind, e.max(), np.median(e)))
        assert e.max() < 1e-3, kind


def _root(parts):
    """Root moments (moments layout) of FP64 parts {m, soft, x, y, z}: mass,
    centre of mass and the raw second moment about it."""
    m, x = parts[:, 0], parts[:, 2:5]
    M = m.sum()
    cm = (m[:, None] * x).sum(0) / M
    e = x - cm
    Q = np.einsum("i,ij,ik->jk", m, e, e)
    return np.array([0.0, 0.0, M, cm[0], cm[1], cm[2], Q[0, 0], Q[0, 1], Q[0, 2], Q[1, 1],
                     Q[1, 2], Q[2, 2]])


def test_ewald_vjp_matches_fd(cuda_ok):
    """changa_ewald_vjp against central differences of the FP64 Ewald term
    (changa_ewald_forces) with its root moments and h-table recomputed at
    every perturbed configuration: the derivative through each particle's
    own position and through the root's mass, centre and quadrupole, on a
    clustered periodic set whose particles reach the series branch near the
    centre of mass and the erf hole."""
    import ctypes as C

    import torch
    from changa_gb300 import _native as N
    from changa_gb300 import gravity, ics
    lib = N.cuda_lib()
    p = ics.nfw_halos(512, ics.rng_for(8), soft=1e-3)
    parts = np.concatenate([p["mass"][:, None], p["soft"][:, None], p["pos"]], axis=1)
    ew = gravity.EwaldConfig(1.0, 1, 2.6, 2.8)
    rng = np.random.default_rng(3)
    lam = rng.normal(size=(len(parts), 3))

    def accel(pp):
        ep = ew.params(_root(pp))
        dp = torch.from_numpy(np.ascontiguousarray(pp)).cuda()
        v = torch.zeros((len(pp), 5), dtype=torch.float64, device="cuda")
        N.check(lib.changa_ewald_forces(N.CHANGA_FORM_FP64, dp.data_ptr(), len(pp), None, len(pp),
                                        C.byref(ep), v.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream), "ewald_forces")
        return v[:, :3].cpu().numpy()

    def f(pp):
        return float((accel(pp) * lam).sum())

    ep = ew.params(_root(parts))
    dp = torch.from_numpy(np.ascontiguousarray(parts)).cuda()
    dl = torch.from_numpy(np.ascontiguousarray(lam)).cuda()
    grad = torch.zeros((len(parts), 4), dtype=torch.float64, device="cuda")
    N.check(lib.changa_ewald_vjp(dp.data_ptr(), len(parts), C.byref(ep), dl.data_ptr(),
                                 grad.data_ptr(), torch.cuda.current_stream().cuda_stream),
            "ewald_vjp")
    g = grad.cpu().numpy()
    h = 1e-5
    errs = []
    for i in rng.choice(len(parts), 24, replace=False):
        for c in (2, 3, 4, 0):  # x, y, z, then the mass
            hh = h if c else h * parts[i, 0]
            pp, pm = parts.copy(), parts.copy()
            pp[i, c] += hh
            pm[i, c] -= hh
            fd = (f(pp) - f(pm)) / (2 * hh)
            got = g[i, c - 2] if c else g[i, 3]
            scale = np.abs(g[:, :3]).max() if c else np.abs(g[:, 3]).max()
            errs.append(abs(fd - got) / (abs(fd) + 1e-4 * scale))
    print("ewald vjp vs FD: max %.2e, median %.2e" % (max(errs), np.median(errs)))
    assert max(errs) < 1e-5


def test_vjp_periodic_matches_fd(cuda_ok):
    """A periodic evaluation (cell and particle lists with replica offsets,
    plus the Ewald term) through one fixed tree: the list adjoint at the
    period plus changa_ewald_vjp against central differences of the FP64
    form, with the moments and the Ewald root refreshed at every perturbed
    configuration."""
    import torch
    from changa_gb300 import gravity, ics
    from changa_gb300.adjoint import TreeStep
    p = ics.nfw_halos(4096, ics.rng_for(9), soft=1e-3)
    t_ = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    x, m, s = t_(p["pos"]), t_(p["mass"]), t_(p["soft"])
    ew = gravity.EwaldConfig(1.0, 1, 2.6, 2.8)
    t = TreeStep(x, m, s, theta=0.7, period=1.0, ewald=ew)
    assert t.lists.cells.n_entries > 0 and t.ds.ewald_params is not None
    lam = torch.randn(x.shape, dtype=torch.float64, device="cuda",
                      generator=torch.Generator("cuda").manual_seed(4))
    t.load(x, m, s)
    gx, gm = t.vjp(lam)

    def f(xx, mm):
        t.load(xx, mm, s)
        return (t.accel("fp64") * lam).sum().item()

    # close pairs in the halo cores: the central difference's truncation
    # error reaches 5e-4 at h = 1e-5 and 4e-6 at h = 1e-6 (isolated or not)
    rng = np.random.default_rng(6)
    h = 1e-6
    errs_x, errs_m = [], []
    for i in rng.choice(x.shape[0], 12, replace=False):
        for c in range(3):
            xp, xm_ = x.clone(), x.clone()
            xp[i, c] += h
            xm_[i, c] -= h
            fd = (f(xp, m) - f(xm_, m)) / (2 * h)
            errs_x.append(abs(fd - gx[i, c].item()) / (abs(fd) + 1e-3 * gx.abs().max().item()))
    for i in rng.choice(x.shape[0], 12, replace=False):
        hm = 1e-4 * m[i].item()
        mp, mm_ = m.clone(), m.clone()
        mp[i] += hm
        mm_[i] -= hm
        fd = (f(x, mp) - f(x, mm_)) / (2 * hm)
        errs_m.append(abs(fd - gm[i].item()) / (abs(fd) + 1e-3 * gm.abs().max().item()))
    print("periodic single-eval FD: x max %.3e, m max %.3e" % (max(errs_x), max(errs_m)))
    assert max(errs_x) < 3e-5 and max(errs_m) < 3e-5
