"""Seeded synthetic particle sets for the gravity workloads.

No public dataset is involved: every workload is generated from a numpy
PCG64 stream seeded with ``20261203 + workload_index``.

* ``plummer``      isolated Plummer sphere (inverse-CDF radii truncated at
                   ``rmax`` scale radii, isotropic directions, velocities by
                   rejection sampling of the distribution function,
                   Aarseth, Henon & Wielen 1974).
* ``lattice_grf``  periodic unit cube: a cubic lattice displaced by a Gaussian
                   random field with P(k) ~ k^-2, normalised to a given rms.
* ``nfw_halos``    periodic unit cube: NFW halos with lognormal masses plus a
                   uniform background.
* ``plummer_clusters`` many independent Plummer spheres with log-uniform N.
"""
from __future__ import annotations

import numpy as np

SEED_BASE = 20261203


def rng_for(index: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(SEED_BASE + index))


def _isotropic(rng, n):
    u = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - u * u)
    return np.stack([s * np.cos(phi), s * np.sin(phi), u], axis=1)


def plummer(n: int, rng, a: float = 1.0, mass: float = 1.0, rmax: float = 20.0,
            soft: float = 0.01, velocities: bool = True):
    """Returns dict(pos, vel, mass, soft) for a Plummer sphere (G = 1)."""
    r = np.empty(n)
    filled = 0
    while filled < n:
        x = rng.uniform(0.0, 1.0, 2 * (n - filled) + 16)
        x = x[x > 0]
        rr = a / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
        rr = rr[rr <= rmax * a]
        take = min(len(rr), n - filled)
        r[filled:filled + take] = rr[:take]
        filled += take
    pos = r[:, None] * _isotropic(rng, n)
    vel = np.zeros((n, 3))
    if velocities:
        # q = v / v_esc from g(q) = q^2 (1 - q^2)^(7/2), max 0.092 at q^2 = 2/9
        q = np.empty(n)
        filled = 0
        while filled < n:
            m = 2 * (n - filled) + 16
            qq = rng.uniform(0.0, 1.0, m)
            yy = rng.uniform(0.0, 0.1, m)
            ok = yy < qq * qq * (1.0 - qq * qq) ** 3.5
            qq = qq[ok]
            take = min(len(qq), n - filled)
            q[filled:filled + take] = qq[:take]
            filled += take
        vesc = np.sqrt(2.0 * mass / a) * (1.0 + (r / a) ** 2) ** (-0.25)
        vel = (q * vesc)[:, None] * _isotropic(rng, n)
    # centre of mass / momentum at the origin
    pos -= pos.mean(axis=0)
    vel -= vel.mean(axis=0)
    return dict(pos=pos, vel=vel, mass=np.full(n, mass / n), soft=np.full(n, soft))


def lattice_grf(ngrid: int, rng, rms_frac: float = 0.2, soft: float | None = None):
    """Periodic unit cube, ngrid^3 particles on a lattice plus a Gaussian
    displacement field with P(k) ~ k^-2 per component; 3-D rms displacement
    = rms_frac of the lattice spacing; positions wrapped into [0, 1)."""
    n = ngrid ** 3
    h = 1.0 / ngrid
    k = np.fft.fftfreq(ngrid) * ngrid
    kx, ky, kz = np.meshgrid(k, k, k, indexing="ij")
    k2 = kx * kx + ky * ky + kz * kz
    amp = np.zeros_like(k2)
    amp[k2 > 0] = 1.0 / np.sqrt(k2[k2 > 0])  # sqrt(P), P ~ k^-2
    disp = np.empty((3, ngrid, ngrid, ngrid))
    for c in range(3):
        noise = rng.standard_normal((ngrid, ngrid, ngrid))
        f = np.fft.fftn(noise) * amp
        disp[c] = np.real(np.fft.ifftn(f))
    rms = np.sqrt((disp ** 2).sum(axis=0).mean())
    disp *= rms_frac * h / rms
    g = (np.arange(ngrid) + 0.5) * h
    gx, gy, gz = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([gx + disp[0], gy + disp[1], gz + disp[2]], axis=-1).reshape(n, 3)
    pos = np.mod(pos, 1.0)
    if soft is None:
        soft = 1.0 / (50.0 * ngrid)
    return dict(pos=pos, vel=np.zeros((n, 3)), mass=np.full(n, 1.0 / n), soft=np.full(n, soft))


def _nfw_radii(rng, n, c):
    """Inverse of mu(x) = ln(1+x) - x/(1+x) on [0, c] by bisection."""
    mu_c = np.log1p(c) - c / (1.0 + c)
    target = rng.uniform(0.0, 1.0, n) * mu_c
    lo = np.zeros(n)
    hi = np.full(n, c)
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        mu = np.log1p(mid) - mid / (1.0 + mid)
        below = mu < target
        lo = np.where(below, mid, lo)
        hi = np.where(below, hi, mid)
    return 0.5 * (lo + hi) / c  # in units of r_vir


def nfw_halos(n: int, rng, n_halos: int = 64, halo_frac: float = 0.8, sigma_ln: float = 1.0,
              conc: float = 10.0, r_median: float = 0.02, soft: float = 2e-4):
    """Periodic unit cube: halo_frac of the particles in NFW halos (lognormal
    masses with the given sigma in ln, median 1/100 of the total before
    renormalisation, r_vir ~ M^(1/3) with the median halo at r_median,
    uniform centres), the rest uniform.  Equal particle masses summing to 1."""
    mh = np.exp(rng.normal(np.log(0.01), sigma_ln, n_halos))
    med = np.median(mh)
    rvir = r_median * (mh / med) ** (1.0 / 3.0)
    mh = mh / mh.sum() * halo_frac
    n_in = int(round(halo_frac * n))
    counts = np.floor(mh / halo_frac * n_in).astype(np.int64)
    rem = n_in - counts.sum()
    order = np.argsort(-(mh / halo_frac * n_in - counts))
    counts[order[:rem]] += 1
    centres = rng.uniform(0.0, 1.0, (n_halos, 3))
    parts = []
    for h in range(n_halos):
        nh = int(counts[h])
        if nh == 0:
            continue
        r = _nfw_radii(rng, nh, conc) * rvir[h]
        parts.append(centres[h] + r[:, None] * _isotropic(rng, nh))
    parts.append(rng.uniform(0.0, 1.0, (n - n_in, 3)))
    pos = np.mod(np.concatenate(parts, axis=0), 1.0)
    return dict(pos=pos, vel=np.zeros((n, 3)), mass=np.full(n, 1.0 / n), soft=np.full(n, soft))


def plummer_clusters(n_clusters: int, rng, nmin: int = 1024, nmax: int = 65536):
    """Independent Plummer spheres: N log-uniform in [nmin, nmax], mass 1,
    scale radius uniform in [0.5, 2], softening 0.01 x scale radius."""
    out = []
    for _ in range(n_clusters):
        n = int(np.floor(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        a = rng.uniform(0.5, 2.0)
        out.append(plummer(n, rng, a=a, mass=1.0, soft=0.01 * a, velocities=False))
    return out
