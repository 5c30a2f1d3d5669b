"""The gravity workloads (seeded synthetic particle sets + tree parameters).

* ``plummer32k``  isolated Plummer sphere, N = 32768, eps 0.01, theta 0.7,
                  bucket 16, quadrupole, open boundaries.
* ``lattice1m``   periodic unit cube, 128^3 perturbed lattice (P(k) ~ k^-2,
                  rms 0.2 of the spacing), eps 1/(50*128), theta 0.7,
                  bucket 16, Ewald (1 replica, cut 2.6, h-cut 2.8).
* ``nfw8m``       periodic unit cube, N = 2^23: 64 NFW halos (lognormal
                  masses, c = 10) + 20% uniform background, eps 2e-4,
                  theta 0.7, bucket 32, Ewald on.  The headline workload.
* ``clusters512`` 512 independent Plummer clusters, N log-uniform in
                  [1024, 65536], theta 0.6, bucket 16 (batched form).
* ``plummer64k``  Plummer sphere, N = 65536 (with velocities), eps 0.01,
                  theta 0.7, bucket 16: the differentiated leapfrog
                  (16 KDK steps, dt 0.005, L = sum w . x(T)).
Seeds: PCG64(20261203 + index) with the index listed per workload.
"""
from __future__ import annotations

from dataclasses import dataclass

from . import ics, tree


@dataclass
class Workload:
    name: str
    index: int
    n: int
    n_bucket: int
    theta: float
    period: float
    ewald: tuple | None  # (fEwCut, dEwhCut)
    soft: float | None = None

    def particles(self):
        rng = ics.rng_for(self.index)
        if self.name.startswith("plummer"):
            return ics.plummer(self.n, rng, soft=self.soft)
        if self.name.startswith("lattice"):
            ng = round(self.n ** (1.0 / 3.0))
            return ics.lattice_grf(ng, rng)
        if self.name.startswith("nfw"):
            return ics.nfw_halos(self.n, rng, soft=self.soft)
        raise ValueError(self.name)

    def lists(self, nthreads=0, particles=None):
        p = particles if particles is not None else self.particles()
        return tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=self.n_bucket,
                                theta=self.theta, period=self.period,
                                n_replicas=1 if self.period else 0, nthreads=nthreads)

    def ewald_config(self):
        if not self.ewald:
            return None
        from .gravity import EwaldConfig
        return EwaldConfig(self.period, 1, self.ewald[0], self.ewald[1])

    def describe(self):
        return dict(workload=self.name, n=self.n, bucket=self.n_bucket, theta=self.theta,
                    periodic=bool(self.period), ewald=bool(self.ewald),
                    moments="quadrupole", seed=ics.SEED_BASE + self.index)


@dataclass
class ClusterBatch:
    """Many independent isolated Plummer clusters evaluated as one batch:
    N per cluster log-uniform in [nmin, nmax], mass 1, scale radius uniform
    in [0.5, 2], softening 0.01 x scale radius."""
    name: str
    index: int
    n_clusters: int
    nmin: int
    nmax: int
    n_bucket: int = 16
    theta: float = 0.6
    period: float = 0.0
    ewald: tuple | None = None

    def clusters(self):
        return ics.plummer_clusters(self.n_clusters, ics.rng_for(self.index), self.nmin, self.nmax)

    def systems(self, nthreads=0):
        """Each cluster's host tree, walk and lists.  The clusters are small,
        so they are built concurrently, one host thread each (the tree
        library's calls release the interpreter lock)."""
        import os
        from concurrent.futures import ThreadPoolExecutor
        cl = self.clusters()
        workers = nthreads if nthreads > 0 else (os.cpu_count() or 1)

        def one(p):
            return tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=self.n_bucket,
                                    theta=self.theta, nthreads=1)
        with ThreadPoolExecutor(max_workers=workers) as ex:
            return list(ex.map(one, cl))

    def lists(self, nthreads=0):
        return tree.concat_systems(self.systems(nthreads))

    def ewald_config(self):
        return None

    def describe(self):
        return dict(workload=self.name, clusters=self.n_clusters, n_range=[self.nmin, self.nmax],
                    bucket=self.n_bucket, theta=self.theta, periodic=False, ewald=False,
                    moments="quadrupole", seed=ics.SEED_BASE + self.index)


WORKLOADS = {
    "clusters512": ClusterBatch("clusters512", 3, 512, 1024, 65536),
    "plummer32k": Workload("plummer32k", 0, 32768, 16, 0.7, 0.0, None, soft=0.01),
    "lattice1m": Workload("lattice1m", 1, 128 ** 3, 16, 0.7, 1.0, (2.6, 2.8)),
    "nfw8m": Workload("nfw8m", 2, 2 ** 23, 32, 0.7, 1.0, (2.6, 2.8), soft=2e-4),
    "nfw1m": Workload("nfw1m", 2, 2 ** 20, 32, 0.7, 1.0, (2.6, 2.8), soft=2e-4),
    "plummer64k": Workload("plummer64k", 4, 65536, 16, 0.7, 0.0, None, soft=0.01),
}
