"""bench.py on the CPU: the reference arm's JSON line (the CPU
implementation of the path, timed on a bounded sample) carries the keys of
the benchmark contract, and the Ewald term count it reports matches a
direct count over the replica lattice."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line(built):
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload",
                          "plummer32k", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference" and d["n_gpus"] == 1
    assert d["unit"] == "interactions/s" and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 0 and d["ms_per_step"] > 0
    assert d["higher_is_better"] is True and d["scaling"] in ("weak", "strong")
    assert d["config"]["workload"] == "plummer32k"
    cpu = d["cpu_baseline"]
    assert cpu["value"] == d["value"] and cpu["cores"] >= 1
    assert cpu["kind"] in ("reference", "port") and cpu["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_ewald_terms_per_particle():
    sys.path.insert(0, ROOT)
    import bench
    from changa_gb300 import gravity
    rng = np.random.default_rng(3)
    n = 64
    parts = np.zeros((n, 5))
    parts[:, 2:5] = rng.uniform(0, 1, (n, 3))
    root = np.zeros(12)
    root[3:6] = 0.5
    ew = gravity.EwaldConfig(1.0, 1, 2.6, 2.8)
    got = bench.ewald_terms_per_particle(parts, root, ew, sample=n)
    total = 0
    for p in parts:
        d = p[2:5] - root[3:6]
        for ix in range(-3, 4):
            for iy in range(-3, 4):
                for iz in range(-3, 4):
                    x = d + np.array([ix, iy, iz], dtype=float)
                    hole = max(abs(ix), abs(iy), abs(iz)) <= 1
                    total += hole or x @ x <= 2.6 ** 2
    assert abs(got - total / n) < 1e-12


def test_oracle_sample_rows_are_complete(built):
    """bench.py's CPU baseline evaluates a sample of buckets; the rows it
    reports for the parity check hold the whole evaluation (cell list,
    particle list and Ewald term) of their particles: equal to the oracle run
    over every bucket."""
    sys.path.insert(0, ROOT)
    import bench
    import oracle
    from changa_gb300 import gravity, ics, tree
    p = ics.lattice_grf(10, ics.rng_for(1))
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7, period=1.0)
    ew = gravity.EwaldConfig(1.0, 1, 2.6, 2.8)
    full = oracle.cell_forces(L.moments, L.parts, L.cells, fperiod=1.0)
    full = oracle.part_forces(L.parts, L.parts, L.plist, fperiod=1.0, vars=full)
    full = oracle.ewald_forces(L.parts, L.root, 1.0, 1, 2.6, 2.8, vars=full)
    _, v, rows = bench.run_cpu(L, ew, L.interactions / 3, kind_pref="port", want_vars=True)
    assert 0 < len(rows) < L.n
    np.testing.assert_allclose(v[rows, :4], full[rows, :4], rtol=1e-12, atol=1e-14)
    np.testing.assert_array_equal(v[rows, 4], full[rows, 4])
    par = bench.parity_block(L, v, rows, full, full * (1 + 1e-7), "port")
    assert par["fp64_vs_oracle_max"] < 1e-12
    assert abs(par["mixed_vs_oracle"]["median"] - 1e-7) < 1e-9
    acc = bench.accuracy_block(L, rows[:200], full, full, full[rows[:200]])
    assert acc["mixed_rel"]["max"] == 0.0 and len(acc["mixed_rel_by_force_quartile"]) == 4
