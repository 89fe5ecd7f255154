"""Serving / batching runtime (om_server_*): results are the same whether a
request runs alone or in a mix of requests that overlap on the device, the
HBM budget is enforced, and memory pressure releases resident problems
instead of deadlocking."""
import time

import numpy as np
import pytest

from helpers import nm, random_cluster

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    return G


def _requests(G):
    """Mixed sizes, both precision forms, LU / GMRES / FGMRES, SH on some, and
    a wavelength scan sharing one cluster key."""
    rng = np.random.default_rng(77)
    out = []
    lu = G.options(G.SOLVE_LU)
    gm = G.options(G.SOLVE_GMRES, tol=1e-11, max_iter=200)
    mx = G.options(G.SOLVE_FGMRES_MIXED, tol=1e-9, max_iter=30, restarts=4, inner_iter=60,
                   inner_tol=1e-4)
    specs = [(2, 4, lu, G.C128, True, 0), (6, 5, gm, G.C128, False, 0), (12, 4, mx, G.C64, False, 0),
             (5, 6, gm, G.C128, True, 0), (9, 5, mx, G.C64, True, 0)]
    for N, nmax, opts, prec, sh, key in specs:
        xyz, rad = random_cluster(rng, N, 900 * nm, 40 * nm, 80 * nm, 20 * nm)
        sp = G.spheres_array(xyz, rad, (2.5 + 0.05j) ** 2, nmax, eps_sh=(2.7 + 0.08j) ** 2,
                             ksippp=1.0 if sh else 0.0, ksiparppar=0.25 if sh else 0.0)
        wave = G.plane_wave(rng.uniform(500, 800) * nm, theta=rng.uniform(0, np.pi),
                            phi=rng.uniform(-np.pi, np.pi), e_theta=0.6, e_phi=0.8j, sh=sh)
        out.append((sp, G.medium(1.2), wave, opts, prec, key))
    # a scan of one cluster: same key, three wavelengths
    xyz, rad = random_cluster(rng, 8, 800 * nm, 40 * nm, 70 * nm, 20 * nm)
    sp = G.spheres_array(xyz, rad, (2.0 + 0.05j) ** 2, 5)
    for lam in (600, 610, 620):
        out.append((sp, G.medium(1.0), G.plane_wave(lam * nm), gm, G.C128, 42))
    return out


def _wait_all(srv, tickets, limit_s=300):
    res = {}
    deadline = time.time() + limit_s
    while len(res) < len(tickets):
        for t in tickets:
            if t not in res:
                r = srv.poll(t, wait=False)
                if r is not None:
                    res[t] = r
        if time.time() > deadline:
            raise AssertionError("server did not finish within the time limit")
        time.sleep(0.002)
    return [res[t] for t in tickets]


def test_alone_equals_in_the_mix(G):
    reqs = _requests(G)
    # alone: one slot, one request at a time
    srv = G.Server(0, 0, 1)
    alone = []
    for rq in reqs:
        alone.append(srv.poll(srv.submit(*rq)))
    srv.close()
    # in the mix: three slots, everything submitted at once
    srv = G.Server(0, 0, 3)
    mixed = _wait_all(srv, [srv.submit(*rq) for rq in reqs])
    srv.close()
    assert len({r["slot"] for r in mixed}) > 1
    for a, b, rq in zip(alone, mixed, reqs):
        assert a["status"] == G.OK and b["status"] == G.OK
        # fixed-order reductions everywhere: bitwise identical
        assert np.array_equal(a["xsec"], b["xsec"])
        assert np.array_equal(a["xsec_sh"], b["xsec_sh"])
        assert a["ff"]["iterations"] == b["ff"]["iterations"]
    # and the same as the single-context entry points
    ctx = G.Context(0)
    for r, (sp, bg, wave, opts, prec, key) in zip(alone, reqs):
        if wave.sh:
            xs, xsh, _ = G.wavelength_solve_sh(ctx, sp, bg, wave, opts, prec)
            assert np.array_equal(xsh, r["xsec_sh"])
        else:
            xs = G.wavelength_solve(ctx, sp, bg, wave, opts, prec)[0]
        assert np.array_equal(xs, r["xsec"])
    ctx.close()


def test_budget_refuses_what_can_never_fit(G):
    rng = np.random.default_rng(5)
    xyz, rad = random_cluster(rng, 30, 1500 * nm, 40 * nm, 60 * nm, 20 * nm)
    big = G.spheres_array(xyz, rad, 4.0, 8)        # n = 4,800: ~370 MB matrix
    small = G.spheres_array(xyz[:2], rad[:2], 4.0, 3)
    srv = G.Server(0, 300 << 20, 2)
    t_big = srv.submit(big, G.medium(), G.plane_wave(600 * nm), G.options(G.SOLVE_GMRES))
    t_small = srv.submit(small, G.medium(), G.plane_wave(600 * nm), G.options(G.SOLVE_LU))
    r_big, r_small = _wait_all(srv, [t_big, t_small])
    srv.close()
    assert r_big["status"] == G.ERR_BUDGET
    assert r_small["status"] == G.OK


def test_memory_pressure_releases_resident_problems(G):
    """Budget for about one request at a time and four distinct clusters on
    two slots: every request still finishes (resident problems are dropped
    when the queue head needs their memory)."""
    rng = np.random.default_rng(6)
    reqs = []
    for i in range(4):
        xyz, rad = random_cluster(rng, 20, 1400 * nm, 40 * nm, 60 * nm, 20 * nm)
        sp = G.spheres_array(xyz, rad, 4.0, 6)     # n = 1,920: 59 MB complex128
        reqs.append((sp, G.medium(), G.plane_wave((600 + 10 * i) * nm), G.options(G.SOLVE_GMRES),
                     G.C128, 100 + i))
    srv = G.Server(0, 600 << 20, 2)
    res = _wait_all(srv, [srv.submit(*rq) for rq in reqs])
    srv.close()
    assert all(r["status"] == G.OK for r in res)
    ctx = G.Context(0)
    for r, (sp, bg, wave, opts, prec, key) in zip(res, reqs):
        assert np.array_equal(G.wavelength_solve(ctx, sp, bg, wave, opts, prec)[0], r["xsec"])
    ctx.close()


def test_batched_service(G):
    """With batching on, runs of batchable requests go through om_batch_solve
    (results bitwise equal to a direct om_batch_solve call on the same
    requests) and the rest (an LU request) through the single-request path."""
    reqs = [rq for rq in _requests(G) if rq[3].method != G.SOLVE_LU]
    lu = next(rq for rq in _requests(G) if rq[3].method == G.SOLVE_LU)
    srv = G.Server(0, 0, 2)
    srv.batching(16)
    tickets = [srv.submit(*rq) for rq in reqs] + [srv.submit(*lu)]
    res = _wait_all(srv, tickets)
    srv.close()
    assert all(r["status"] == G.OK for r in res)
    ctx = G.Context(0)
    direct = G.batch_solve(ctx, [rq[:5] for rq in reqs])
    for r, d in zip(res, direct):
        assert np.array_equal(r["xsec"], d["xsec"])
        assert np.array_equal(r["xsec_sh"], d["xsec_sh"])
    sp, bg, wave, opts, prec, key = lu
    xs, xsh, _ = G.wavelength_solve_sh(ctx, sp, bg, wave, opts, prec)
    assert np.array_equal(res[-1]["xsec"], xs)
    ctx.close()
