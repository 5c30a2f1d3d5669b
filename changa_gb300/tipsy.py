"""Minimal Tipsy reader: the particle format ChaNGa loads its initial
conditions from (TreePiece::loadTipsy, InOutput.cpp:183-; the format
library itself, N-BodyShop's TipsyFile, is not part of the reference).

Layout: a header {double time; int nbodies, ndim, nsph, ndark, nstar; pad}
followed by nsph gas records {mass, pos[3], vel[3], rho, temp, hsmooth,
metals, phi}, ndark dark records {mass, pos[3], vel[3], eps, phi} and nstar
star records {mass, pos[3], vel[3], metals, tform, eps, phi}, all float32.
"Standard" files are big-endian (XDR) with the 4-byte pad after the
header; native files use the machine's byte order.  Gas particles carry no
eps; ChaNGa then softens them with the run's dSoft (passed as gas_soft).
"""
from __future__ import annotations

import numpy as np

_GAS = ["mass", "x", "y", "z", "vx", "vy", "vz", "rho", "temp", "hsmooth", "metals", "phi"]
_DARK = ["mass", "x", "y", "z", "vx", "vy", "vz", "eps", "phi"]
_STAR = ["mass", "x", "y", "z", "vx", "vy", "vz", "metals", "tform", "eps", "phi"]


def _header(raw, order):
    h = np.frombuffer(raw[:28], dtype=np.dtype([("time", order + "f8"), ("nbodies", order + "i4"),
                                                ("ndim", order + "i4"), ("nsph", order + "i4"),
                                                ("ndark", order + "i4"), ("nstar", order + "i4")]))[0]
    return {k: h[k].item() for k in h.dtype.names}


def read(path, gas_soft=0.0):
    """Returns dict(time, n, nsph, ndark, nstar, pos (n x 3), vel (n x 3),
    mass (n,), soft (n,)) in file order (gas, dark, star), FP64."""
    with open(path, "rb") as f:
        raw = f.read()
    for order, hdr_bytes in ((">", 32), ("<", 32), ("<", 28), (">", 28)):
        h = _header(raw, order)
        n = h["nbodies"]
        if not (0 <= h["nsph"] <= n and 0 <= h["ndark"] <= n and 0 <= h["nstar"] <= n and
                h["nsph"] + h["ndark"] + h["nstar"] == n and h["ndim"] in (2, 3)):
            continue
        size = hdr_bytes + 4 * (12 * h["nsph"] + 9 * h["ndark"] + 11 * h["nstar"])
        if size == len(raw):
            break
    else:
        raise ValueError("%s: not a Tipsy file (header and size disagree)" % path)
    off = hdr_bytes
    parts = []
    for fields, count in ((_GAS, h["nsph"]), (_DARK, h["ndark"]), (_STAR, h["nstar"])):
        dt = np.dtype([(name, order + "f4") for name in fields])
        rec = np.frombuffer(raw, dtype=dt, count=count, offset=off)
        off += dt.itemsize * count
        parts.append((fields, rec))
    pos = np.concatenate([np.stack([r["x"], r["y"], r["z"]], 1) for _, r in parts]).astype(np.float64)
    vel = np.concatenate([np.stack([r["vx"], r["vy"], r["vz"]], 1) for _, r in parts]).astype(np.float64)
    mass = np.concatenate([r["mass"] for _, r in parts]).astype(np.float64)
    soft = np.concatenate([r["eps"] if "eps" in f else np.full(len(r), gas_soft, np.float32)
                           for f, r in parts]).astype(np.float64)
    return dict(time=h["time"], n=n, nsph=h["nsph"], ndark=h["ndark"], nstar=h["nstar"], pos=pos,
                vel=vel, mass=mass, soft=soft)


def write(path, pos, vel, mass, soft, time=0.0):
    """Writes dark-matter particles as a standard (big-endian) Tipsy file."""
    n = len(mass)
    with open(path, "wb") as f:
        np.array([(time, n, 3, 0, n, 0)],
                 dtype=[("t", ">f8"), ("n", ">i4"), ("d", ">i4"), ("g", ">i4"), ("k", ">i4"),
                        ("s", ">i4")]).tofile(f)
        np.zeros(1, ">i4").tofile(f)
        rec = np.empty(n, dtype=np.dtype([(k, ">f4") for k in _DARK]))
        rec["mass"] = mass
        rec["x"], rec["y"], rec["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
        rec["vx"], rec["vy"], rec["vz"] = vel[:, 0], vel[:, 1], vel[:, 2]
        rec["eps"] = soft
        rec["phi"] = 0.0
        rec.tofile(f)
