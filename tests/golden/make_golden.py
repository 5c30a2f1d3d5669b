"""Generates the committed golden fixtures from ChaNGa's own CPU force code.

Run where the reference sources are present (oracle/_ref is built from
them): ``python tests/golden/make_golden.py``.  Each fixture stores the
particle set, the tree parameters, a checksum of the serialised lists and
the reference's forces (gravity.h nodeBucketForce/partBucketForce and
Ewald.cpp BucketEwald run on those lists), so the restated oracle, the host
walk and the GPU path can all be checked against it without the reference.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from changa_gb300 import ics, tree  # noqa: E402


def list_digest(lists):
    h = hashlib.sha256()
    for req in (lists.cells, lists.plist):
        for a in (req.list, req.markers, req.starts, req.sizes):
            h.update(np.ascontiguousarray(a).tobytes())
    h.update(np.ascontiguousarray(lists.moments).tobytes())
    return h.hexdigest()


def make(name, p, kind, n_bucket, theta, period=0.0, ewald=None, sample=None):
    # inputs are stored (and used) as float32-valued positions to keep fixtures small
    p = dict(p, pos=p["pos"].astype(np.float32).astype(np.float64))
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=n_bucket, theta=theta,
                         period=period)
    v = oracle.cell_forces(L.moments, L.parts, L.cells, fperiod=period, kind=kind)
    v = oracle.part_forces(L.parts, L.parts, L.plist, fperiod=period, vars=v, kind=kind)
    ew = None
    if ewald:
        ew = oracle.ewald_forces(L.parts, L.root, period, 1, ewald[0], ewald[1], kind=kind)
    rows = np.arange(L.n) if sample is None else np.sort(sample)
    out = dict(pos=p["pos"].astype(np.float32), mass=p["mass"], soft=p["soft"], n_bucket=n_bucket, theta=theta,
               period=period, perm=L.perm, rows=rows, tree_vars=v[rows],
               digest=np.array(list_digest(L)), interactions=L.interactions,
               oracle=np.array(kind))
    if ew is not None:
        out["ewald_vars"] = ew[rows]
        out["ewald_cfg"] = np.array(ewald)
        out["ewt"] = oracle.ewald_table(L.root, period, ewald[1], kind=kind)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, L.n, "interactions", L.interactions, "digest", out["digest"])


def main():
    kind = "ref" if oracle.available("ref") else None
    if kind is None:
        oracle.build()
        kind = "ref" if oracle.available("ref") else None
    if kind is None:
        sys.exit("the reference oracle (oracle/_ref) is not available here")
    make("plummer_1k", ics.plummer(1024, ics.rng_for(100), soft=0.01), kind, 16, 0.7)
    make("plummer_ragged_2k", ics.plummer(2048, ics.rng_for(101), soft=0.05), kind, 48, 0.5)
    make("lattice_8", ics.lattice_grf(8, ics.rng_for(102)), kind, 16, 0.7, period=1.0,
         ewald=(2.6, 2.8))
    rng = ics.rng_for(103)
    p = ics.plummer(32768, ics.rng_for(0), soft=0.01)
    make("plummer_32k_sample", p, kind, 16, 0.7, sample=rng.choice(32768, 512, replace=False))


if __name__ == "__main__":
    main()
