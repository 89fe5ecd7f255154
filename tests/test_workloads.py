"""The seeded synthetic workloads of bench.py (no GPU): the clusters obey the
reference's non-overlap rule (Geometry.cpp:41-49, with a 20 nm gap) inside
their cube, the nMax rule of the spectral sweep, and the sizes, ranges and
mix of the sweep and the request stream."""
import numpy as np
import pytest

import bench

nm = 1e-9


def _gaps(xyz, rad):
    d = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=2)
    g = d - rad[:, None] - rad[None, :]
    np.fill_diagonal(g, np.inf)
    return g


@pytest.mark.parametrize("name", ["c1", "c2", "small"])
def test_fixed_clusters(name):
    w = bench.WORKLOADS[name]
    xyz, rad = bench.cluster(w)
    assert xyz.shape == (w["N"], 3) and rad.shape == (w["N"],)
    assert rad.min() >= w["rmin"] and rad.max() <= w["rmax"]
    assert _gaps(xyz, rad).min() >= 20 * nm * (1 - 1e-12)
    # every sphere inside the cube
    assert np.all(np.abs(xyz) + rad[:, None] <= w["edge"] / 2 * (1 + 1e-12))
    # seeded: the same cluster every time, a different one per replica rank
    xyz2, rad2 = bench.cluster(w)
    assert np.array_equal(xyz, xyz2) and np.array_equal(rad, rad2)
    xyz3, _ = bench.cluster(w, rank=1)
    assert not np.array_equal(xyz, xyz3)


def test_nmax_rule():
    lam = 600 * nm
    # x = 2 pi a / lambda; nMax = clamp(ceil(x + 4 x^(1/3) + 2), 4, 12), the
    # largest over the cluster's spheres
    for a in (10 * nm, 60 * nm, 120 * nm, 1000 * nm):
        x = 2 * np.pi * a / lam
        want = int(min(12, max(4, np.ceil(x + 4 * np.cbrt(x) + 2))))
        assert bench.nmax_rule([a], lam) == want
    assert bench.nmax_rule([10 * nm, 120 * nm], lam) == bench.nmax_rule([120 * nm], lam)
    assert bench.nmax_rule([1e-9], lam) == 4 and bench.nmax_rule([5000 * nm], lam) == 12


def test_ragged_cluster_volume_fraction_and_gaps():
    rng = np.random.default_rng(5)
    frac = bench.c1_volume_fraction()
    xyz, rad, edge = bench.ragged_cluster(rng, 40, 30 * nm, 120 * nm, frac)
    assert _gaps(xyz, rad).min() >= 20 * nm * (1 - 1e-12)
    assert np.all(np.abs(xyz) + rad[:, None] <= edge / 2 * (1 + 1e-12))
    got = np.sum(4 / 3 * np.pi * rad ** 3) / edge ** 3
    # the smallest edge giving the c1 volume fraction (grown by 10 % steps
    # only when the spheres do not fit)
    assert got <= frac * (1 + 1e-12) and got >= frac / 1.1 ** 3 / 1.5


def test_spectral_sweep_cases():
    cases = bench.c3_cases(8, 16)
    assert len(cases) == 8 * 16
    Ns = {c["N"] for c in cases}
    assert min(Ns) >= 2 and max(Ns) <= 64
    assert all(4 <= c["nmax"] <= 12 for c in cases)
    assert all(c["wave"].sh for c in cases)
    lams = sorted({c["wave"].wavelength for c in cases})
    assert len(lams) == 16 and lams[0] == pytest.approx(400 * nm) and lams[-1] == pytest.approx(900 * nm)
    # the same seed gives the same sweep
    again = bench.c3_cases(8, 16)
    assert [c["N"] for c in again] == [c["N"] for c in cases]
    assert [c["nmax"] for c in again] == [c["nmax"] for c in cases]


def test_request_stream_mix():
    reqs = bench.c4_requests(200.0, 1.5)
    n = len(reqs)
    # Poisson arrivals at 200/s for 1.5 s: 300 expected
    assert 240 <= n <= 360
    t = np.array([r["t"] for r in reqs])
    assert np.all(np.diff(t) > 0) and t[-1] < 1.5
    Ns = np.array([r["N"] for r in reqs])
    assert Ns.min() >= 1 and Ns.max() <= 300
    # log-uniform sizes: about half of them below sqrt(300) ~ 17
    assert 0.3 < np.mean(Ns < 17) < 0.7
    sh = np.mean([bool(r["wave"].sh) for r in reqs])
    assert 0.2 < sh < 0.4
    assert all(400 * nm <= r["wave"].wavelength <= 900 * nm for r in reqs)
