#!/usr/bin/env python
"""Gravity-force benchmark: interactions/s of the FP32-mixed form.

One "step" is one complete force evaluation of the workload: the cell
(quadrupole) interaction lists, the particle interaction lists and the
periodic Ewald correction, over lists that are already resident in HBM
(the host tree walk that builds them runs once, outside the timed region,
as it does on ChaNGa's CPU).  Interactions follow ChaNGa's own counter
(Compute.cpp:1643-1651): per bucket, targets x (cell-list + particle-list
entries).

Default workload: nfw8m (N = 2^23 NFW halos + background, periodic, Ewald,
bucket 32, theta 0.7).  Other lines of the JSON:
  e2e          the same metric through changa_gravity_step_host with host
               (pinned) buffers, host<->device copies inside the timed region;
  roofline     the dominant kernel (FP32-mixed cell-list kernel) against the
               FP32 FMA peak of the GPU (roofline_pp: the particle-list kernel);
  cpu_baseline the CPU oracle (ChaNGa's own gravity.h/Ewald.cpp when it was
               built here, else its C restatement) on a bounded sample;
  adjoint      plummer64k: one adjoint (VJP) evaluation against one forward
               evaluation on the same tree, and the 16-step leapfrog forward /
               checkpointed reverse pass (--no-adjoint skips it).
--impl reference times that CPU implementation alone on the same workload.

Launch: python bench.py [--gpus N --steps K --warmup W]; for N > 1 under
torch.distributed.run, one rank per GPU; every rank evaluates its own copy
of the workload (weak scaling) and value = all ranks' interactions / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOP_PC = 67  # FLOP per quadrupole cell interaction (counted convention)
FLOP_PP = 23  # FLOP per particle-particle interaction
METRIC = "gravity interactions/s at N=8M, FP32-mixed vs FP64 form at rel force err ≤1e-3"


def metric_for(workload):
    if workload == "nfw8m":
        return METRIC
    return "gravity interactions/s, FP32-mixed form (%s)" % workload


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="nfw8m")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=9)
    ap.add_argument("--cpu-sample", type=float, default=1.5e10,
                    help="interactions in the bounded CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false",
                    help="skip the adjoint / forward cost measurement (plummer64k)")
    ap.add_argument("--no-adjoint-leapfrog", dest="adjoint_leapfrog", action="store_false")
    ap.add_argument("--no-direct", dest="direct", action="store_false",
                    help="skip the direct-sum error of the sampled particles")
    ap.add_argument("--no-hexadecapole", dest="hexadecapole", action="store_false",
                    help="skip the hexadecapole-build measurement on the same particles")
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip the clusters512 batching-form measurement")
    ap.add_argument("--variants", default=None,
                    help="CELL,PART list-kernel shape variants to use instead of the autotuner")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.out = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=5)
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                mhz.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not mhz:
            return None
        mhz.sort()
        return {"sm_mhz": mhz[len(mhz) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(mhz)}


def dist_setup(args):
    from changa_gb300 import replicas
    return replicas.setup()


def barrier(world):
    from changa_gb300 import replicas
    replicas.barrier(world)


def max_over_ranks(world, x):
    from changa_gb300 import replicas
    return replicas.max_over_ranks(world, x)


def sum_over_ranks(world, x):
    from changa_gb300 import replicas
    return replicas.sum_over_ranks(world, x)


def cpu_sample(lists, target, seed=12345):
    """A random subset of buckets whose interactions add up to ~target:
    returns (bucket ids of the cell request, of the particle request, count)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    nb = len(lists.bucket_starts)
    order = rng.permutation(nb)
    cl, pl = lists.cells, lists.plist
    c_of = {int(b): i for i, b in enumerate(cl.bucket_ids)}
    p_of = {int(b): i for i, b in enumerate(pl.bucket_ids)}
    c_len = np.diff(cl.markers.astype(np.int64)) * cl.sizes
    p_len = np.diff(pl.markers.astype(np.int64)) * pl.sizes
    cid, pid, tot = [], [], 0
    for b in order:
        b = int(b)
        if b in c_of:
            cid.append(c_of[b])
            tot += int(c_len[c_of[b]])
        if b in p_of:
            pid.append(p_of[b])
            tot += int(p_len[p_of[b]])
        if tot >= target:
            break
    return np.array(cid, np.int32), np.array(pid, np.int32), tot


def ewald_terms_per_particle(parts, root, ew, sample=4096):
    """Mean number of real-space Ewald terms one particle evaluates (the
    replicas inside the cut or the hole, Ewald.cpp BucketEwald's test), over
    a seeded sample of the particles."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(20261205))
    idx = rng.choice(parts.shape[0], size=min(sample, parts.shape[0]), replace=False)
    d = parts[idx, 2:5] - np.asarray(root[3:6], dtype=np.float64)
    ne = max(int(np.ceil(ew.fEwCut)), ew.n_reps)
    r = np.arange(-ne, ne + 1)
    g = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    hole = (np.abs(g) <= ew.n_reps).all(1)
    cut2 = (ew.fEwCut * ew.L) ** 2
    terms = 0
    for chunk in np.array_split(d, 16):
        x = chunk[:, None, :] + g[None, :, :] * ew.L
        terms += int((((x * x).sum(-1) <= cut2) | hole[None, :]).sum())
    return terms / len(idx)


def measure_dropin(lists, ew, interactions, steps):
    """End to end through the reference-facing boundary (HostCUDA.h /
    EwaldCUDA.h) with pinned FP32 ABI host buffers, as ChaNGa calls it:
    DataManagerTransferLocalTree, the cell and particle list transfers,
    EwaldHost and TransferParticleVarsBack in ChaNGa's order (EwaldHost right
    after the tree transfer), synchronised per step (wall clock, after one
    untimed step).  A failure is reported, not raised."""
    import time
    from changa_gb300 import _native as N
    from changa_gb300 import gravity
    lib = N.cuda_lib()
    lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_RECORD)  # an error is reported, not abort()
    inp = None

    def step():
        gravity.dropin_step(inp)
        code = lib.changa_gb300_last_error()
        if code:
            raise RuntimeError("drop-in step: error %d" % code)
    try:
        lib.changa_gb300_last_error()  # clear
        inp = gravity.DropInInputs(lists, ew)
        step()
        tt = []
        for _ in range(max(1, steps)):
            t1 = time.perf_counter()
            step()
            tt.append(time.perf_counter() - t1)
        t = sorted(tt)[len(tt) // 2]  # median step
        # where the time goes: the drop-in kernels of one more step, by events
        lib.changa_gb300_set_timing(1)
        for k in N.KERNEL_IDS:
            N.kernel_time(k)
        t1 = time.perf_counter()
        step()
        t_one = time.perf_counter() - t1
        kt = {k: N.kernel_time(k)[0] for k in ("list_f32_cell", "list_f32_part", "ewald_f32")}
        lib.changa_gb300_set_timing(0)
        return {"value": interactions / t, "unit": "interactions/s", "ms_per_step": 1e3 * t,
                "ms_steps": [round(1e3 * x, 3) for x in tt],
                "kernel_ms_one_step": kt, "timed_step_ms": 1e3 * t_one,
                "h2d_bytes_per_step": int(inp.h2d_bytes), "d2h_bytes_per_step": int(inp.d2h_bytes),
                "form": "FP32 (the reference's arithmetic on its ABI structs)",
                "api": "DataManagerTransferLocalTree, EwaldHost (queued after the tree "
                       "transfer, as DataManager.cpp:495-510 queues it), "
                       "TreePieceCellListDataTransferLocal, TreePiecePartListDataTransferLocal, "
                       "TransferParticleVarsBack; one request per list"}
    except Exception as e:  # noqa: BLE001 - reported in the JSON line
        return {"error": "%s: %s" % (type(e).__name__, e)}
    finally:
        if inp is not None:
            inp.free()
        lib.changa_gb300_set_error_mode(N.CHANGA_ERRORS_ABORT)


def run_cpu(lists, ewald, target, kind_pref="auto", reps=1, want_vars=False):
    """Times the CPU oracle on a bounded sample; returns dict (and, with
    want_vars, the oracle's vars and the rows whose result is complete: the
    particles of the sampled buckets, which received their whole cell list,
    particle list and Ewald term)."""
    import numpy as np

    import oracle
    kind = "ref" if (kind_pref == "auto" and oracle.available("ref")) else "port"
    oracle.load(kind)
    cid, pid, tot = cpu_sample(lists, target)
    cores = os.cpu_count() or 1
    # Ewald targets: the particles of the sampled buckets
    rows = []
    for i in pid:
        s, n = int(lists.plist.starts[i]), int(lists.plist.sizes[i])
        rows.extend(range(s, s + n))
    rows = np.array(sorted(set(rows)), np.int32)
    times = []
    for _ in range(reps):
        v = np.zeros((lists.n, 5))
        t0 = time.perf_counter()
        oracle.cell_forces(lists.moments, lists.parts, lists.cells, fperiod=lists.period, vars=v,
                           bucket_ids=cid, kind=kind, nthreads=cores)
        oracle.part_forces(lists.parts, lists.parts, lists.plist, fperiod=lists.period, vars=v,
                           bucket_ids=pid, kind=kind, nthreads=cores)
        ve = None
        if ewald is not None and len(rows):
            ve = oracle.ewald_forces(lists.parts, lists.root, ewald.L, ewald.n_reps, ewald.fEwCut,
                                     ewald.dEwhCut, idx=rows, kind=kind, nthreads=cores)
        times.append(time.perf_counter() - t0)
        if ve is not None:  # the Ewald rows (idx order) onto the sampled particles
            v[rows, :4] += ve[:, :4]
    dt = min(times)
    out = {"value": tot / dt, "unit": "interactions/s", "cores": cores,
           "kind": "reference" if kind == "ref" else "port",
           "sample": "%d random buckets of the workload (%.3g interactions, cell+particle lists"
                     "%s), FP64, OpenMP over buckets, best of %d" %
                     (len(set(cid.tolist()) | set(pid.tolist())), tot,
                      " + Ewald on their %d particles" % len(rows) if ewald else "", reps),
           "seconds": dt,
           "note": "scalar FP64 restatement of gravity.h/Ewald.cpp (the reference's CMK_SSE "
                   "vector path needs its absent SSE-Double.h), one OpenMP thread per core"}
    if want_vars:
        return out, v, rows
    return out


def rel_err(a, ref):
    """Per-particle relative force error |a - ref| / |ref|."""
    import numpy as np
    return np.linalg.norm(a[:, :3] - ref[:, :3], axis=1) / np.linalg.norm(ref[:, :3], axis=1)


def stats(e):
    import numpy as np
    return {"median": float(np.median(e)), "p99": float(np.percentile(e, 99)),
            "max": float(np.max(e))}


def parity_block(lists, v_oracle, rows, v64, v_mixed, kind):
    """The GPU forms against the CPU oracle (ChaNGa's gravity.h/Ewald.cpp or
    its C restatement) per particle, on the particles whose sampled buckets
    the oracle evaluated completely (same lists, same inputs)."""
    import numpy as np
    ref = v_oracle[rows]
    out = {"oracle": kind, "particles": int(len(rows)),
           "fp64_vs_oracle": stats(rel_err(v64[rows], ref)),
           "mixed_vs_oracle": stats(rel_err(v_mixed[rows], ref))}
    pot = lambda v: np.abs(v[rows, 3] - ref[:, 3]) / np.abs(ref[:, 3])
    out["fp64_pot_vs_oracle_max"] = float(pot(v64).max())
    out["mixed_pot_vs_oracle_median"] = float(np.median(pot(v_mixed)))
    out["fp64_vs_oracle_max"] = out["fp64_vs_oracle"]["max"]
    out["bar"] = "FP64 form: 1e-6 relative per particle"
    return out


def accuracy_block(lists, samp, v_mixed, v64, dsum):
    """Force error against the FP64 direct sum on the sampled particles:
    relative per particle, normalised by the sample's rms force, and the
    relative error binned by |a| and by local density (the particle's
    bucket: targets / box volume), to show where the tail sits."""
    import numpy as np
    a_ref = np.linalg.norm(dsum[:, :3], axis=1)
    rms = float(np.sqrt(np.mean(a_ref ** 2)))
    out = {"particles": int(len(samp)), "rms_force": rms}
    for name, v in (("mixed", v_mixed), ("fp64", v64)):
        e = rel_err(v[samp], dsum)
        out[name + "_rel"] = stats(e)
        out[name + "_over_rms"] = stats(np.linalg.norm(v[samp, :3] - dsum[:, :3], axis=1) / rms)
    e = rel_err(v_mixed[samp], dsum)
    # |a| quartiles
    q = np.quantile(a_ref, [0.25, 0.5, 0.75])
    bins = np.digitize(a_ref, q)
    out["mixed_rel_by_force_quartile"] = [
        {"force_range": [float(a_ref[bins == k].min()), float(a_ref[bins == k].max())],
         "median": float(np.median(e[bins == k])), "p99": float(np.percentile(e[bins == k], 99))}
        for k in range(4)]
    # local density: the particle's bucket (targets / bounding-box volume)
    bstart = lists.bucket_starts.astype(np.int64)
    b = np.searchsorted(bstart, samp, side="right") - 1
    bb = lists.bucket_bbox[b]
    ext = np.maximum(bb[:, 3:6] - bb[:, 0:3], 1e-9)
    dens = lists.bucket_sizes[b] / np.prod(ext, axis=1)
    qd = np.quantile(dens, [0.25, 0.5, 0.75])
    bd = np.digitize(dens, qd)
    out["mixed_rel_by_density_quartile"] = [
        {"median": float(np.median(e[bd == k])), "p99": float(np.percentile(e[bd == k], 99))}
        for k in range(4)]
    worst = e >= np.percentile(e, 99)
    out["worst_1pct"] = {"median_force_over_rms": float(np.median(a_ref[worst]) / rms),
                         "share_below_tenth_median_force":
                             float(np.mean(a_ref[worst] < 0.1 * np.median(a_ref)))}
    return out


def fp32_peak_tflops():
    """FP32 FMA peak, measured on this GPU (changa_gb300_fp32_fma_peak: every
    SM running independent fma.rn.f32 chains, best of 5), with the derived
    figure SMs x 128 lanes x 2 FLOP x max SM clock beside it."""
    import ctypes as C

    import torch
    from changa_gb300 import _native as N
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = None
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            mhz = json.load(f).get("sm_max_mhz")
    derived = sms * 128 * 2 * (mhz or 2070.0) * 1e6 / 1e12
    got = C.c_double(0.0)
    rc = N.cuda_lib().changa_gb300_fp32_fma_peak(C.byref(got))
    if rc == 0 and got.value > 0:
        return got.value, ("measured: changa_gb300_fp32_fma_peak, %d SMs x 8 blocks x 256 threads "
                           "of independent fma.rn.f32 chains, best of 5 (derived %d x 128 x 2 x "
                           "%.0f MHz = %.1f TFLOP/s)" % (sms, sms, mhz or 2070.0, derived))
    return derived, "derived: %d SMs x 128 FP32 lanes x 2 x %.0f MHz" % (sms, mhz or 2070.0)


def traffic_from_profiles():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def main_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from changa_gb300 import build as b
    from changa_gb300.workloads import WORKLOADS
    b.build_host()
    b.build_oracle()
    wl = WORKLOADS[args.workload]
    lists = wl.lists()
    ew = wl.ewald_config()
    per_step = args.cpu_sample / 5  # a few seconds of CPU work per step
    for _ in range(args.warmup):
        run_cpu(lists, ew, per_step / 4)
    vals = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        r = run_cpu(lists, ew, per_step)
        vals.append(r)
    wall = time.perf_counter() - t_all
    value = sum(r["value"] for r in vals) / len(vals)
    ms = 1e3 * sum(r["seconds"] for r in vals) / len(vals)
    cb = dict(vals[0])
    cb["value"] = value
    out = {"metric": metric_for(args.workload), "value": value, "unit": "interactions/s", "impl": "reference",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded %s)" % wl.name,
           "config": dict(wl.describe(), l2="inputs larger than L2 and a 256 MB flush write "
                                            "between timed steps"),
           "workload_detail": {"sample": vals[0]["sample"], "wall_s": wall},
           "cpu_baseline": cb,
           "e2e": {"value": value, "unit": "interactions/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


def measure_adjoint(leapfrog=True, reps=20, tune=True):
    """The differentiation workload (plummer64k): one FP32-mixed force
    evaluation vs one adjoint (VJP) evaluation on the same tree, by kernel
    time and by CUDA events around the whole call; optionally the 16-step
    KDK leapfrog forward and its checkpointed reverse pass (wall clock,
    host tree builds included)."""
    import numpy as np
    import torch
    from changa_gb300 import _native as N
    from changa_gb300 import autotune
    from changa_gb300.adjoint import Leapfrog, TreeStep, loss_weights
    from changa_gb300.workloads import WORKLOADS
    wl = WORKLOADS["plummer64k"]
    p = wl.particles()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    x, v, m, s = t(p["pos"]), t(p["vel"]), t(p["mass"]), t(p["soft"])
    ts = TreeStep(x, m, s, theta=wl.theta, n_bucket=wl.n_bucket)
    if tune:
        autotune.tune(ts.ds, "mixed")
    lam = loss_weights(wl.n, 99)
    for _ in range(3):
        ts.accel("mixed")
        ts.vjp(lam)
    torch.cuda.synchronize()
    lib = N.cuda_lib()
    lib.changa_gb300_set_timing(1)
    for k in N.KERNEL_IDS:
        N.kernel_time(k)
    for _ in range(reps):
        ts.ds.step("mixed")
    torch.cuda.synchronize()
    fw = {k: N.kernel_time(k)[0] / reps for k in ("list_mixed_cell", "list_mixed_part", "pack")}
    for _ in range(reps):
        ts.vjp(lam)
    torch.cuda.synchronize()
    bw = {k: N.kernel_time(k)[0] / reps for k in ("vjp_cell", "vjp_part", "pack", "moments")}
    lib.changa_gb300_set_timing(0)
    ev = []
    for fn in (lambda: ts.ds.step("mixed"), lambda: ts.vjp(lam)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        ev.append(e0.elapsed_time(e1) / reps)
    out = {"workload": wl.name, "n": wl.n, "interactions": ts.interactions,
           "forward_kernel_ms": fw, "vjp_kernel_ms": bw,
           "forward_ms": sum(fw.values()), "vjp_ms": sum(bw.values()),
           "vjp_over_forward": sum(bw.values()) / sum(fw.values()),
           "event_forward_ms": ev[0], "event_vjp_ms": ev[1],
           "event_vjp_over_forward": ev[1] / ev[0]}
    if leapfrog:
        w = loss_weights(wl.n, 13)
        out["leapfrog"] = {"steps": 16, "dt": 0.005, "checkpoint_every": 4}
        # trees rebuilt every step on the host (build, walk, serialise,
        # upload) or on the GPU (DeviceTree + gpu_walk)
        for builder in ("host", "device"):
            lf = Leapfrog(m, s, 0.005, 16, theta=wl.theta, n_bucket=wl.n_bucket,
                          checkpoint_every=4, builder=builder)
            if builder == "device":  # first-use costs (module loads) out of the timing
                TreeStep(x, m, s, theta=wl.theta, n_bucket=wl.n_bucket, builder="device")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            lf.forward(x, v)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            lf.backward(w, torch.zeros_like(w))
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            out["leapfrog"][builder + "_trees"] = {
                "forward_wall_s": t1 - t0, "reverse_wall_s": t2 - t1,
                "tree_builds": lf.tree_builds, "force_evals": lf.force_evals}
    return out


def measure_device_pipeline(wl, pts, interactions, ew=None, reps=3):
    """Positions already on the device to device-resident lists: the tree
    built on the GPU (changa_tree_build) and walked there (changa_walk);
    best of `reps` after one untimed run.  The interaction count must equal
    the host lists'.  Then the fused route on the last tree
    (changa_walk_forces: walk and FP32-mixed forces in one pass, no lists,
    with the Ewald term), best of `reps`, against the list route's forces
    on the same tree (walk + changa_gravity_step)."""
    import numpy as np
    import torch
    from changa_gb300 import gravity
    from changa_gb300.gputree import DeviceTree
    from changa_gb300.walk import gpu_walk, walk_forces
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    pos, m, s = t(pts["pos"]), t(pts["mass"]), t(pts["soft"])
    best = None
    tree = None
    for rep in range(reps + 1):
        if tree is not None:
            tree.close()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tree = DeviceTree(pos, m, s, n_bucket=wl.n_bucket, theta=wl.theta, period=wl.period)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        cells, plist, _ = gpu_walk(tree)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        n_int = cells.interactions() + plist.interactions()
        if rep and (best is None or t2 - t0 < best["tree_build_s"] + best["walk_s"]):
            best = {"tree_build_s": t1 - t0, "walk_s": t2 - t1, "n_nodes": tree.n_nodes,
                    "n_buckets": tree.n_buckets}
        if rep < reps:
            del cells, plist
    best["interactions_match"] = n_int == interactions
    ds = gravity.DeviceSystem(tree, device_reqs=[cells, plist], ewald=ew)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    list_ms = []
    for _ in range(reps + 1):
        ev0.record()
        ref = ds.step("mixed")
        ev1.record()
        torch.cuda.synchronize()
        list_ms.append(ev0.elapsed_time(ev1))
    best["list_forces_s"] = min(list_ms[1:]) * 1e-3
    out = torch.empty((tree.n, 5), dtype=torch.float64, device="cuda")
    fused = []
    for _ in range(reps + 1):
        torch.cuda.synchronize()
        f0 = time.perf_counter()
        walk_forces(tree, ewald=ds.ewald_params, out=out)
        torch.cuda.synchronize()
        fused.append(time.perf_counter() - f0)
    da = (out[:, :3] - ref[:, :3]).norm(dim=1) / ref[:, :3].norm(dim=1)
    best["fused"] = {"walk_forces_s": min(fused[1:]),
                     "vs_walk_plus_list_forces_s": best["walk_s"] + best["list_forces_s"],
                     "interactions_per_s": interactions / min(fused[1:]),
                     "max_rel_diff_vs_lists": float(da.max().item()),
                     "median_rel_diff_vs_lists": float(da.median().item())}
    tree.close()
    return best


def measure_hexadecapole(wl, pts, samp=None, dsum=None, steps=5, fp64_steps=1):
    """ChaNGa's default build on the same particles: the hexadecapole lists
    (host tree and walk, order 4) evaluated in the FP32-mixed form with the
    hexadecapole Ewald term; same timing rules as the headline (warm-up, a
    256 MB flush between steps, CUDA events on the stream).  The tree and
    particle order are the quadrupole build's, so the sampled particles'
    direct sums compare directly."""
    import numpy as np
    import torch
    from changa_gb300 import _native as N
    from changa_gb300 import gravity, tree
    lib = N.cuda_lib()
    t0 = time.perf_counter()
    L = tree.build_lists(pts["pos"], pts["mass"], pts["soft"], n_bucket=wl.n_bucket,
                         theta=wl.theta, period=wl.period, n_replicas=1 if wl.period else 0,
                         order=4)
    host_s = time.perf_counter() - t0
    # the same tree's lists walked on the GPU (two phases; the entries
    # counted against the host walk's)
    from changa_gb300.walk import gpu_walk
    gpu_walk(L)
    wt = {}
    dc, dp, dsoft = gpu_walk(L, timings=wt)
    walk_match = (dc.interactions() + dp.interactions() + dsoft.interactions() ==
                  L.cells.interactions() + L.plist.interactions() + L.softcells.interactions())
    del dc, dp, dsoft
    ds = gravity.DeviceSystem(L, device="cuda", ewald=wl.ewald_config())
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")
    for _ in range(3):
        ds.step("mixed")
    torch.cuda.synchronize()
    lib.changa_gb300_set_timing(1)
    for k in N.KERNEL_IDS:
        N.kernel_time(k)
    evs = []
    for _ in range(steps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ds.step("mixed")
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    kt = {k: N.kernel_time(k)[0] / steps for k in ("list_mixed_cell", "list_mixed_part",
                                                   "ewald_mixed", "pack")}
    lib.changa_gb300_set_timing(0)
    ms = sum(a.elapsed_time(b) for a, b in evs) / steps
    Ic, Ip, Is = (L.cells.interactions(), L.plist.interactions(), L.softcells.interactions())
    I = Ic + Ip + Is
    out = {"moments": "hexadecapole (scaled reduced, to fourth order)", "form": "FP32-mixed",
           "interactions": I, "cell_interactions": Ic, "particle_interactions": Ip,
           "softened_cell_interactions": Is, "ms_per_step": ms,
           "interactions_per_s": I / (ms / 1e3), "kernel_ms": kt,
           "cell_tflops_counted": Ic * 196 / (kt["list_mixed_cell"] / 1e3) / 1e12,
           "host_tree_walk_s": host_s, "gpu_walk_s": wt.get("walk_s"),
           "gpu_walk_interactions_match": bool(walk_match)}
    if samp is not None and dsum is not None:
        v = ds.vars.cpu().numpy()[samp]
        e = np.linalg.norm(v[:, :3] - dsum[:, :3], axis=1) / np.linalg.norm(dsum[:, :3], axis=1)
        out.update({"median_rel_force_err_vs_direct": float(np.median(e)),
                    "p99_rel_force_err_vs_direct": float(np.percentile(e, 99))})
    if fp64_steps > 0:
        # the FP64 form of the same build (its denominator), one warm step timed
        ds.step("fp64")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.fill_(1.0)
        e0.record(stream)
        for _ in range(fp64_steps):
            ds.step("fp64")
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1) / fp64_steps
        out.update({"fp64_ms_per_step": ms64, "fp64_interactions_per_s": I / (ms64 / 1e3),
                    "mixed_over_fp64": ms64 / ms})
        if samp is not None and dsum is not None:
            v = ds.vars.cpu().numpy()[samp]
            e = np.linalg.norm(v[:, :3] - dsum[:, :3], axis=1) / np.linalg.norm(dsum[:, :3], axis=1)
            out["fp64_median_rel_force_err_vs_direct"] = float(np.median(e))
    del ds, L
    torch.cuda.empty_cache()
    return out


def batched_workload(wl):
    return hasattr(wl, "systems")


def measure_batched(steps=5, seq_reps=2):
    """The batching form on clusters512 (512 independent Plummer clusters,
    N log-uniform in [1024, 65536]): one CUDA-graph replay of the
    concatenated requests (one persistent launch per list kind, its work
    queue balancing every cluster's buckets) against the 512 clusters
    evaluated one after another as plain evaluations.  Same timing rules as
    the headline: warm-up, a 256 MB flush between steps, CUDA events on the
    stream.  The two results must agree (same lists, same kernels)."""
    import numpy as np
    import torch
    from changa_gb300 import autotune, gravity, tree
    from changa_gb300.workloads import WORKLOADS
    wl = WORKLOADS["clusters512"]
    t0 = time.perf_counter()
    systems = wl.systems()
    L = tree.concat_systems(systems)
    host_s = time.perf_counter() - t0
    I = L.interactions
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")
    ds = gravity.DeviceSystem(L, device="cuda")
    tuning = autotune.tune(ds, "mixed")
    graph = gravity.GravityGraph(ds, "mixed")
    for _ in range(3):
        graph.launch()
    torch.cuda.synchronize()
    evs = []
    for _ in range(steps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        graph.launch()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / steps
    v_graph = ds.vars.cpu().numpy()
    graph.close()
    del ds
    singles = [gravity.DeviceSystem(s, device="cuda") for s in systems]
    for x in singles:
        x.step("mixed")
    torch.cuda.synchronize()
    ms_seq = []
    for _ in range(seq_reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for x in singles:
            x.step("mixed")
        e1.record(stream)
        torch.cuda.synchronize()
        ms_seq.append(e0.elapsed_time(e1))
    v_seq = np.concatenate([x.vars.cpu().numpy() for x in singles], axis=0)
    del singles
    torch.cuda.empty_cache()
    ms_s = sum(ms_seq) / len(ms_seq)
    e = rel_err(v_graph, v_seq)
    return {"workload": "clusters512", "clusters": len(systems), "n": int(L.n),
            "n_range": [int(min(x.n for x in systems)), int(max(x.n for x in systems))],
            "interactions": int(I), "form": "FP32-mixed",
            "graph_ms_per_step": ms, "graph_interactions_per_s": I / (ms / 1e3),
            "sequential_ms_per_step": ms_s, "sequential_interactions_per_s": I / (ms_s / 1e3),
            "graph_over_sequential": ms_s / ms,
            "graph_vs_sequential_max_rel_force_diff": float(e.max()),
            "autotune": {k: v.get("variant") for k, v in tuning.items() if isinstance(v, dict)},
            "host_tree_walk_s": host_s}


def timed_steps(step, steps, stream, flush):
    """CUDA-event time of each of `steps` calls of step(), a flush write
    before each."""
    import torch
    evs = []
    for _ in range(steps):
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


def measure_e2e(lists, ew, stream, steps, world, runs=None):
    """End to end through changa_gravity_step_host with pinned host buffers:
    the upload of every input and the read-back of the result are inside
    the timed region (wall clock per step, after one untimed step).  With
    runs (a tree.PartRuns of the particle lists) the call is
    changa_gravity_step_host_runs and the particle lists travel as runs."""
    import ctypes as C

    import numpy as np
    from changa_gb300 import _native as N
    from changa_gb300 import gravity
    lib = N.cuda_lib()
    arrays = [("moments", lists.moments), ("parts", lists.parts),
              ("cl", lists.cells.list), ("cm", lists.cells.markers), ("cs", lists.cells.starts),
              ("cz", lists.cells.sizes), ("pm", lists.plist.markers), ("ps", lists.plist.starts),
              ("pz", lists.plist.sizes)]
    if runs is None:
        arrays.append(("pl", lists.plist.list))
    else:
        arrays += [("pr", runs.runs), ("prm", runs.run_markers)]
    pin = {k: gravity.PinnedArray(a) for k, a in arrays}
    out = gravity.PinnedArray(np.zeros((lists.n, 5)))
    h2d = sum(int(a.nbytes) for _, a in arrays)

    def req(l, m, s, z, r):
        q = N.ChangaListRequest()
        q.list, q.markers, q.starts, q.sizes = pin[l].ptr, pin[m].ptr, pin[s].ptr, pin[z].ptr
        q.n_buckets, q.n_entries = r.n_buckets, r.n_entries
        return q
    cq = req("cl", "cm", "cs", "cz", lists.cells)
    if runs is None:
        pq = req("pl", "pm", "ps", "pz", lists.plist)
    else:
        pq = N.ChangaPartRuns()
        pq.runs, pq.run_markers = pin["pr"].ptr, pin["prm"].ptr
        pq.markers, pq.starts, pq.sizes = pin["pm"].ptr, pin["ps"].ptr, pin["pz"].ptr
        pq.n_buckets, pq.n_runs = runs.n_buckets, runs.n_runs
    ep = ew.params(lists.root) if ew else None
    sh = stream.cuda_stream
    fn = lib.changa_gravity_step_host if runs is None else lib.changa_gravity_step_host_runs

    def one():
        # overwrite: the result replaces out (no host zeroing, no vars upload)
        rc = fn(N.CHANGA_FORM_MIXED | N.CHANGA_STEP_OVERWRITE, pin["moments"].ptr,
                lists.moments.shape[0], pin["parts"].ptr, lists.n, C.byref(cq), C.byref(pq),
                float(lists.period), C.byref(ep) if ep else None, out.ptr, sh)
        N.check(rc, fn.__name__)
    try:
        one()
        tt = []
        for _ in range(steps):
            t1 = time.perf_counter()
            one()
            tt.append(time.perf_counter() - t1)
        result = out.array.copy()
    finally:
        for a in list(pin.values()) + [out]:
            a.free()
    t_e2e = max_over_ranks(world, sorted(tt)[len(tt) // 2])  # median step
    I = lists.interactions
    api = ("changa_gravity_step_host (include/changa_gb300.h), pinned host buffers, "
           "CHANGA_STEP_OVERWRITE; particles uploaded first in 64 MiB slices, each packed and given "
           "its Ewald term as it lands; lists in 256 MiB chunks (halving toward the end) on a "
           "copy stream overlapping the list kernels; each chunk's particles read back on a "
           "second copy stream once final")
    if runs is not None:
        api = ("changa_gravity_step_host_runs (include/changa_gb300.h): as "
               "changa_gravity_step_host, with the particle lists as runs (ILPart, 12 B per run of "
               "consecutive source particles, %d runs for %d entries) expanded on the device "
               "chunk by chunk" % (runs.n_runs, lists.plist.n_entries))
    return {"value": sum_over_ranks(world, float(I)) / t_e2e, "unit": "interactions/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(lists.parts.nbytes),
            "ms_per_step": 1e3 * t_e2e, "ms_steps": [round(1e3 * x, 3) for x in tt],
            "timing": "wall clock per call (each call returns with the results in host "
                      "memory), median of the steps after one untimed call",
            "api": api}, result


def main_ours(args):
    import numpy as np
    import torch

    import __graft_entry__
    __graft_entry__.build()
    from changa_gb300 import _native as N
    from changa_gb300 import gravity
    from changa_gb300.workloads import WORKLOADS

    world, rank, local = dist_setup(args)
    lib = N.cuda_lib()
    wl = WORKLOADS[args.workload]
    batched = batched_workload(wl)
    pts = None if batched else wl.particles()
    t0 = time.perf_counter()
    lists = wl.lists(particles=pts) if not batched else wl.lists()
    t_walk = time.perf_counter() - t0
    ew = wl.ewald_config()
    I = lists.interactions
    walk_gpu = None
    device_pipeline = None
    if not batched:
        # the same lists built on the GPU (changa_walk), timed
        from changa_gb300.walk import gpu_walk
        gpu_walk(lists)
        walk_gpu = {}
        gpu_walk(lists, timings=walk_gpu)
        device_pipeline = measure_device_pipeline(wl, pts, I, ew=ew)
        device_pipeline["walk_on_host_lists_s"] = walk_gpu.get("walk_s")
        device_pipeline["host_tree_walk_serialise_s"] = t_walk
    I_c, I_p = lists.cells.interactions(), lists.plist.interactions()
    ds = gravity.DeviceSystem(lists, device="cuda", ewald=ew)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")  # > L2
    from changa_gb300 import autotune
    if args.variants:
        # fixed shapes (profiling runs): no autotuner launches
        cv, pv = (int(x) for x in args.variants.split(","))
        tuning = {"list_mixed_cell": {"variant": cv}, "list_mixed_part": {"variant": pv},
                  "fixed": True}
        autotune.apply({k: v for k, v in tuning.items() if k != "fixed"})
    else:
        tuning = autotune.tune(ds, "mixed")  # untimed: selects the list-kernel shapes
    graph = gravity.GravityGraph(ds, "mixed") if batched else None

    def step():
        if graph is not None:
            graph.launch()
        else:
            ds.step("mixed")

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    lib.changa_gb300_set_timing(1)
    for k in N.KERNEL_IDS:
        N.kernel_time(k)
    launches0 = lib.changa_gb300_kernel_launches()
    ms_steps = timed_steps(step, args.steps, stream, flush)
    barrier(world)
    torch.cuda.synchronize()
    launches = lib.changa_gb300_kernel_launches() - launches0
    ktimes = {k: N.kernel_time(k) for k in N.KERNEL_IDS}
    lib.changa_gb300_set_timing(0)
    clk = clocks.stop()
    ms = sum(ms_steps) / len(ms_steps)
    ms_max = max_over_ranks(world, ms)
    value = sum_over_ranks(world, float(I)) / (ms_max / 1e3)
    v_mixed = ds.vars.cpu().numpy().copy()
    if graph is not None:
        graph.close()

    # FP64 form on the same lists (the precision yardstick and the 3x target)
    fp64, acc, v64, samp, dsum = None, None, None, None, None
    if args.fp64_steps > 0:
        ds.step("fp64")
        torch.cuda.synchronize()
        ms64 = sum(timed_steps(lambda: ds.step("fp64"), args.fp64_steps, stream, flush)) / \
            args.fp64_steps
        v64 = ds.vars.cpu().numpy()
        rng = np.random.default_rng(7)
        samp = np.sort(rng.choice(lists.n, min(16384, lists.n), replace=False))
        e = rel_err(v_mixed[samp], v64[samp])
        fp64 = {"ms_per_step": ms64, "interactions_per_s": I / (ms64 / 1e3),
                "mixed_ms_per_step": ms, "mixed_interactions_per_s": I / (ms / 1e3),
                "mixed_over_fp64": ms64 / ms,
                "mixed_vs_fp64": stats(e), "sampled_particles": int(len(samp))}
        if args.direct and not batched:
            # the same sample against the direct sum (Ewald-summed when periodic)
            t0 = time.perf_counter()
            dsum = gravity.direct_forces(ds.parts, samp, period=float(lists.period))
            acc = accuracy_block(lists, samp, v_mixed, v64, dsum)
            acc["direct_sum"] = "changa_direct_forces, FP64-accumulated%s, %.1f s" % (
                " Ewald sum" if lists.period else "", time.perf_counter() - t0)
        for k in N.KERNEL_IDS:
            N.kernel_time(k)
    del ds
    torch.cuda.empty_cache()

    # ChaNGa's default build (hexadecapole) on the same particles
    hexa = None
    if args.hexadecapole and pts is not None:
        hexa = measure_hexadecapole(wl, pts, samp, dsum)
        if acc is not None and "median_rel_force_err_vs_direct" in hexa:
            acc["hexadecapole_rel"] = {"median": hexa["median_rel_force_err_vs_direct"],
                                       "p99": hexa["p99_rel_force_err_vs_direct"]}
    pts = None

    # end to end through the public C-ABI with pinned host buffers: the
    # particle lists as runs (the headline), and as flat lists
    e2e = None
    if args.e2e_steps > 0:
        from changa_gb300 import tree as T
        runs = T.part_runs(lists.plist)
        e2e, r = measure_e2e(lists, ew, stream, args.e2e_steps, world, runs=runs)
        e2e["max_rel_force_diff_vs_device_step"] = float(rel_err(r, v_mixed).max())
        del runs
        flat, r = measure_e2e(lists, ew, stream, args.e2e_steps, world)
        e2e["flat_lists"] = {"value": flat["value"], "ms_per_step": flat["ms_per_step"],
                             "h2d_bytes_per_step": flat["h2d_bytes_per_step"],
                             "max_rel_force_diff_vs_device_step":
                                 float(rel_err(r, v_mixed).max()),
                             "api": flat["api"]}

    dropin = None
    if args.e2e_steps > 0 and getattr(lists, "order", 2) == 2 and not batched:
        # 32 ms steps with occasional host-side outliers: a median of at least 9
        dropin = measure_dropin(lists, ew, I, max(9, args.e2e_steps))
        if e2e is not None and "ms_per_step" in dropin:
            # the same bytes cross the host link on both paths (flat particle lists)
            dropin["ratio_to_e2e_flat_lists"] = (dropin["ms_per_step"] /
                                                 e2e["flat_lists"]["ms_per_step"])

    # roofline of the dominant kernel (FP32-mixed cell lists) and the P-P kernel.
    # The bound is the FP32 FMA pipe (no tensor-core or HBM bound applies:
    # DRAM traffic is under 5% of peak); traffic comes from the committed ncu
    # capture, valid for the nfw8m workload it was scaled to.
    peak, peak_src = fp32_peak_tflops()
    tr = traffic_from_profiles() if args.workload == "nfw8m" else {}
    lib_v = [lib.changa_gb300_get_list_variant(N.KERNEL_IDS[k])
             for k in ("list_mixed_cell", "list_mixed_part")]
    roof = None
    ms_pc, n_pc = ktimes["list_mixed_cell"]
    ms_pp, n_pp = ktimes["list_mixed_part"]
    if n_pc:
        t_pc = ms_pc / n_pc / 1e3
        ach = I_c * FLOP_PC / t_pc / 1e12
        roof = {"bound": "fp32", "kernel": "FP32-mixed cell-list kernel, shape variant %d" % lib_v[0],
                "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                "peak_source": peak_src,
                "algorithmic_flop_per_launch": I_c * FLOP_PC,
                "flop_per_interaction": FLOP_PC, "interactions_per_launch": I_c,
                "avg_launch_ms": 1e3 * t_pc,
                "traffic": tr.get("list_mixed_cell_bytes_per_launch"),
                "fma_pipe_active_ncu_pct": tr.get("list_mixed_cell_fma_pipe_pct"),
                "traffic_note": tr.get("note")}
    roof_pp = None
    if n_pp:
        t_pp = ms_pp / n_pp / 1e3
        ach = I_p * FLOP_PP / t_pp / 1e12
        roof_pp = {"bound": "fp32",
                   "kernel": "FP32-mixed particle-list kernel, shape variant %d" % lib_v[1],
                   "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                   "algorithmic_flop_per_launch": I_p * FLOP_PP, "flop_per_interaction": FLOP_PP,
                   "interactions_per_launch": I_p, "avg_launch_ms": 1e3 * t_pp,
                   "traffic": tr.get("list_mixed_part_bytes_per_launch"),
                   "fma_pipe_active_ncu_pct": tr.get("list_mixed_part_fma_pipe_pct")}
    kshare = {k: {"ms_per_step": v[0] / max(1, args.steps), "launches": v[1]}
              for k, v in ktimes.items() if v[1]}
    # Ewald on its own: particle evaluations/s and the reference's per-particle
    # work score (Ewald.cpp:153-159, 259-264: 333 per real-space term, 58 per
    # h-vector; it weighs erfc and exp far above one FLOP, so it is no
    # roofline figure)
    ewald_info = None
    ms_ew, n_ew = ktimes.get("ewald_mixed", (0.0, 0))
    if ew is not None and n_ew:
        t_ew = ms_ew / n_ew / 1e3
        terms = ewald_terms_per_particle(lists.parts, lists.root, ew)
        nh = int(ew.params(lists.root).nEwhLoop)
        fl = 333.0 * terms + 58.0 * nh
        ewald_info = {"particles_per_launch": int(lists.n), "avg_launch_ms": 1e3 * t_ew,
                      "particle_evals_per_s": lists.n / t_ew,
                      "real_space_terms_per_particle": terms, "h_vectors": nh,
                      "reference_score_per_particle": fl}

    # the CPU oracle on a bounded sample: the reported baseline, and the
    # per-particle parity of both GPU forms on the particles it evaluated
    cpu, parity = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, v_orc, rows = run_cpu(lists, ew, args.cpu_sample, want_vars=True)
        if v64 is not None:
            parity = parity_block(lists, v_orc, rows, v64, v_mixed, cpu["kind"])
        del v_orc
    list_bytes = int(lists.cells.list.nbytes + lists.plist.list.nbytes)
    del lists, v64
    torch.cuda.empty_cache()

    bat = None
    if rank == 0 and args.batched and not batched:
        try:
            bat = measure_batched()
        except Exception as ex:  # noqa: BLE001 - reported in the JSON line
            bat = {"error": "%s: %s" % (type(ex).__name__, ex)}

    adj = None
    if rank == 0 and args.adjoint:
        adj = measure_adjoint(args.adjoint_leapfrog, tune=not args.variants)

    if rank == 0:
        cfg = dict(wl.describe(), l2="inputs larger than L2 and a 256 MB flush write between "
                                     "timed steps")
        out = {"metric": metric_for(args.workload), "value": value, "unit": "interactions/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded %s; no dataset)" % wl.name,
               "config": cfg,
               "workload_detail": {"form": "FP32-mixed", "interactions": I,
                                   "cell_interactions": I_c, "particle_interactions": I_p,
                                   "list_bytes": list_bytes, "host_walk_s": t_walk,
                                   "autotune": tuning, "kernels": kshare,
                                   "parallelism": "replicas x%d" % world},
               "roofline": roof, "roofline_pp": roof_pp, "cpu_baseline": cpu, "e2e": e2e,
               "gpu_launches": int(launches), "clocks": clk,
               "fp64_form": fp64, "parity": parity, "accuracy": acc, "hexadecapole": hexa,
               "dropin_e2e": dropin, "batched": bat, "ewald": ewald_info,
               "device_pipeline": device_pipeline, "adjoint": adj}
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return main_reference(args)
    return main_ours(args)


if __name__ == "__main__":
    sys.exit(main())
