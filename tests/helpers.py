"""Shared helpers of the test suite (fixtures, error metrics)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["plummer_1k", "plummer_ragged_2k", "lattice_8", "plummer_32k_sample"]


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def lists_from_golden(g):
    from changa_gb300 import tree
    return tree.build_lists(g["pos"].astype(np.float64), g["mass"], g["soft"],
                            n_bucket=int(g["n_bucket"]), theta=float(g["theta"]),
                            period=float(g["period"]))


def force_rel_err(a, ref):
    """Per-particle |a - ref| / |ref| over the acceleration rows."""
    num = np.linalg.norm(a[:, :3] - ref[:, :3], axis=1)
    den = np.linalg.norm(ref[:, :3], axis=1)
    return num / np.maximum(den, 1e-300)


def pot_rel_err(a, ref):
    return np.abs(a[:, 3] - ref[:, 3]) / np.maximum(np.abs(ref[:, 3]), 1e-300)


def force_rms_err(a, ref):
    """Per-particle |a - ref| / rms|ref|: the metric for periodic sets, where
    net forces on a near-uniform lattice are a small residual of O(1)
    replica terms and per-particle relative errors lose meaning."""
    num = np.linalg.norm(a[:, :3] - ref[:, :3], axis=1)
    return num / np.sqrt((ref[:, :3] ** 2).sum(axis=1).mean())


def pot_rms_err(a, ref):
    """|dpot| / rms(pot); the periodic potential's zero point is arbitrary."""
    return np.abs(a[:, 3] - ref[:, 3]) / np.sqrt((ref[:, 3] ** 2).mean())


def reference_root():
    """The reference checkout for tests that read its data files:
    CHANGA_REFERENCE, else a checkout named "reference" beside this
    repository; None when neither exists (those tests then skip)."""
    root = os.environ.get("CHANGA_REFERENCE")
    if not root:
        here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        root = os.path.join(os.path.dirname(here), "reference")
    return root if os.path.isdir(root) else None


def sampled_oracle(L, ew, bucket_ids, kind="port"):
    """The oracle on a subset of buckets: nodeBucketForce over their cell
    lists, partBucketForce over their particle lists and (ew given)
    BucketEwald on their particles.  Returns (vars N x 5, rows): rows are
    the particles of those buckets, whose results are complete."""
    import oracle
    b = np.asarray(bucket_ids)
    c_of = {int(x): i for i, x in enumerate(L.cells.bucket_ids)}
    p_of = {int(x): i for i, x in enumerate(L.plist.bucket_ids)}
    cid = np.array([c_of[int(x)] for x in b if int(x) in c_of], np.int32)
    pid = np.array([p_of[int(x)] for x in b if int(x) in p_of], np.int32)
    v = np.zeros((L.n, 5))
    oracle.cell_forces(L.moments, L.parts, L.cells, fperiod=L.period, vars=v, bucket_ids=cid,
                       kind=kind)
    oracle.part_forces(L.parts, L.parts, L.plist, fperiod=L.period, vars=v, bucket_ids=pid,
                       kind=kind)
    rows = np.concatenate([np.arange(L.bucket_starts[x], L.bucket_starts[x] + L.bucket_sizes[x])
                           for x in b]).astype(np.int32)
    rows.sort()
    if ew is not None:
        ve = oracle.ewald_forces(L.parts, L.root, ew.L, ew.n_reps, ew.fEwCut, ew.dEwhCut, idx=rows,
                                 kind=kind)
        v[rows, :4] += ve[:, :4]
    return v, rows
