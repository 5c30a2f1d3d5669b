"""Autotuner for the list-kernel shapes.

The FP32-form list kernels are compiled in several shapes (resident blocks
per SM, i.e. the register cap, x list entries per reduction tile; see
kVariants in csrc/grav_lists.cu).  Which one is fastest depends on the
workload: bucket occupancy, list lengths and the share of softened pairs
shift the balance between occupancy and spills.  ``tune`` times every shape
on the actual device-resident lists with the library's per-kernel CUDA-event
timing, selects the fastest for the cell and the particle kernel separately,
and caches the choice per (GPU, form, workload signature) in
``_build/tuning.json``.
"""
from __future__ import annotations

import json
import os

from . import _native as N
from . import build as _build

CACHE = os.path.join(_build.BUILD, "tuning.json")
KERNELS = {"mixed": ("list_mixed_cell", "list_mixed_part")}


def signature(ds, form):
    import torch
    name = torch.cuda.get_device_name()
    L = ds.lists
    nb = max(1, L.cells.n_buckets)
    return "%s|%s|n=%d|cells=%d|parts=%d|nb=%d" % (
        name, form, L.n, L.cells.n_entries // nb, L.plist.n_entries // max(1, L.plist.n_buckets),
        round(L.n / max(1, len(L.bucket_starts))))


def _load():
    if os.path.exists(CACHE):
        try:
            with open(CACHE) as f:
                return json.load(f)
        except (OSError, ValueError):
            return {}
    return {}


def _save(cache):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def apply(choice):
    lib = N.cuda_lib()
    for kname, v in choice.items():
        N.check(lib.changa_gb300_set_list_variant(N.KERNEL_IDS[kname], int(v["variant"])),
                "set_list_variant")


def tune(ds, form="mixed", reps=3, use_cache=True):
    """Selects the fastest shape for the form's cell and particle kernels on
    this DeviceSystem; returns {kernel: {"variant", "ms", "all_ms"}}."""
    import torch
    lib = N.cuda_lib()
    sig = signature(ds, form)
    cache = _load() if use_cache else {}
    if sig in cache:
        apply(cache[sig])
        return dict(cache[sig], cached=True)
    kernels = KERNELS[form]
    nvar = lib.changa_gb300_list_variant_count()
    times = {k: [] for k in kernels}
    lib.changa_gb300_set_timing(1)
    try:
        for v in range(nvar):
            for k in kernels:
                N.check(lib.changa_gb300_set_list_variant(N.KERNEL_IDS[k], v), "set_list_variant")
            ds.step(form)  # warm this shape
            torch.cuda.synchronize()
            for k in N.KERNEL_IDS:
                N.kernel_time(k)
            for _ in range(reps):
                ds.step(form)
            torch.cuda.synchronize()
            for k in kernels:
                ms, n = N.kernel_time(k)
                times[k].append(ms / max(1, n))
    finally:
        lib.changa_gb300_set_timing(0)
    choice = {}
    for k in kernels:
        best = min(range(nvar), key=lambda v: times[k][v])
        choice[k] = {"variant": best, "ms": times[k][best], "all_ms": times[k]}
    apply(choice)
    cache[sig] = choice
    _save(cache)
    return choice
