"""Batching form (om_batch_solve): batched results agree with the golden
vectors of the oracle and with the single-request entry points, a request's
results are bitwise the same alone and in any batch, and failures stay with
the request that caused them.

Tolerances: the plain form (complex128 GMRES to 1e-13) within 1e-10 of the
golden cross sections, as the single-request entry point; both forms against
the single-request FP64 path within 1e-10 (plain) and 1e-6 (precision form)."""
import numpy as np
import pytest

from helpers import gpu_inputs, load_golden, nm, oracle_cluster, random_cluster, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    return G


@pytest.fixture(scope="module")
def ctx(G):
    c = G.Context(0)
    yield c
    c.close()


def plain(G, tol=1e-13):
    return G.options(G.SOLVE_GMRES, tol=tol, max_iter=150, restarts=6)


def mixed(G):
    return G.options(G.SOLVE_FGMRES_MIXED, tol=1e-10, max_iter=30, restarts=4, inner_iter=40,
                     inner_tol=1e-4)


def ragged_requests(G, opts, prec, seed=11):
    """Uneven N and nMax (several requests per size class), SH on every other
    request, random incidence."""
    rng = np.random.default_rng(seed)
    specs = [(1, 4), (2, 4), (2, 4), (3, 4), (5, 4), (6, 4), (7, 5), (2, 5), (12, 4), (11, 4),
             (9, 6), (4, 3), (16, 4), (6, 5)]
    out = []
    for i, (N, nmax) in enumerate(specs):
        xyz, rad = random_cluster(rng, N, 1000 * nm, 40 * nm, 80 * nm, 20 * nm)
        sh = i % 2 == 0
        sp = G.spheres_array(xyz, rad, (2.2 + 0.05j) ** 2, nmax, eps_sh=(2.4 + 0.07j) ** 2,
                             ksippp=1.0 if sh else 0.0, ksiparppar=0.25 if sh else 0.0)
        wave = G.plane_wave(rng.uniform(500, 800) * nm, theta=rng.uniform(0, np.pi),
                            phi=rng.uniform(-np.pi, np.pi), e_theta=0.6, e_phi=0.8j, sh=sh)
        out.append((sp, G.medium(1.2), wave, opts, prec))
    return out


def test_golden_vectors_through_the_batch(G, ctx, oracle):
    """The committed golden fixtures (oracle cross sections, FF and SH) as one
    batched call spanning several size classes."""
    names = ["c0", "metal5", "diel3", "single_sh", "pair_sh"]
    reqs, gs = [], []
    for name in names:
        g = load_golden(name)
        sp, bg, wave = gpu_inputs(G, oracle_cluster(oracle, g))
        wave.sh = int("xsec_sh" in g.files)
        reqs.append((sp, bg, wave, plain(G), G.C128))
        gs.append(g)
    res = G.batch_solve(ctx, reqs)
    for name, g, r in zip(names, gs, res):
        assert r["status"] == G.OK, name
        assert np.max(np.abs(r["xsec"] - g["xsec"]) / np.abs(g["xsec"])) < 1e-10, name
        if "xsec_sh" in g.files:
            assert np.max(np.abs(r["xsec_sh"] - g["xsec_sh"]) / np.abs(g["xsec_sh"])) < 1e-10, name


def test_plain_batch_matches_single_requests(G, ctx):
    reqs = ragged_requests(G, plain(G), G.C128)
    res = G.batch_solve(ctx, reqs)
    for r, (sp, bg, wave, opts, prec) in zip(res, reqs):
        assert r["status"] == G.OK
        xs, xsh, _ = G.wavelength_solve_sh(ctx, sp, bg, wave, opts, prec)
        assert rel(r["xsec"], xs) < 1e-10
        if wave.sh:
            assert rel(r["xsec_sh"], xsh) < 1e-10
        assert r["ff"]["rel_residual"] <= 1e-13


def test_precision_form_batch_within_1e6_of_fp64(G, ctx):
    reqs = ragged_requests(G, mixed(G), G.C64)
    res = G.batch_solve(ctx, reqs)
    for r, (sp, bg, wave, opts, prec) in zip(res, reqs):
        assert r["status"] == G.OK
        xs, xsh, _ = G.wavelength_solve_sh(ctx, sp, bg, wave, plain(G), G.C128)
        assert rel(r["xsec"], xs) < 1e-6
        if wave.sh:
            assert rel(r["xsec_sh"], xsh) < 1e-6
        # refinement: a few cycles, each an FP32 Arnoldi run
        assert 1 <= r["ff"]["iterations"] <= 8 and r["ff"]["inner_iterations"] >= 1


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_alone_equals_in_the_batch(G, ctx, form):
    """Every kernel reduces in a fixed order per slot, so a request gives the
    same bits alone, in a full batch, and in batches cut small by the arena."""
    reqs = ragged_requests(G, plain(G) if form == "plain" else mixed(G),
                           G.C128 if form == "plain" else G.C64, seed=5)
    together = G.batch_solve(ctx, reqs)
    tiny = G.batch_solve(ctx, reqs, arena_bytes=1 << 20)  # one request per batch
    for i, rq in enumerate(reqs):
        alone = G.batch_solve(ctx, [rq])[0]
        for other in (together[i], tiny[i]):
            assert np.array_equal(alone["xsec"], other["xsec"])
            assert np.array_equal(alone["xsec_sh"], other["xsec_sh"])
            assert alone["ff"]["iterations"] == other["ff"]["iterations"]
            assert alone["sh"]["inner_iterations"] == other["sh"]["inner_iterations"]
    assert len({r["slot"] for r in together}) > 1


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_autotuned_tiles_do_not_change_the_bits(G, form):
    """The batched matvecs' tile configurations (rows per tile, tile order,
    CTAs per SM) fixed one at a time, and chosen by the autotuner: the same
    bits, and the autotuner reports one choice per size class."""
    reqs = ragged_requests(G, plain(G) if form == "plain" else mixed(G),
                           G.C128 if form == "plain" else G.C64, seed=9)
    runs = []
    for cand in [0] + list(range(1, 9)):
        c = G.Context(0)
        c.tune(batch_tiles=cand, batch_fused=0)  # the lockstep form (the fused solve has no tiles)
        runs.append(G.batch_solve(c, reqs))
        if cand == 0:
            chosen = G.batch_tiles(c)
            assert len(chosen) >= 3  # the ragged requests span several size classes
            assert len({(t["precision"], t["nmax"], t["Npad"]) for t in chosen}) == len(chosen)
            assert all(t["rows"] in (128, 256) and t["ctas_per_sm"] in (2, 4, 8, 16) and t["matvec_us"] >= 0
                       for t in chosen)
        else:
            assert G.batch_tiles(c) == []
        c.close()
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            assert a["status"] == b["status"] == G.OK
            assert np.array_equal(a["xsec"], b["xsec"]) and np.array_equal(a["xsec_sh"], b["xsec_sh"])
            assert a["ff"]["iterations"] == b["ff"]["iterations"]


def blocky_requests(G, opts, prec, seed=13):
    """Size classes whose slots span several 512-row blocks (fused groups of
    2 to 7 CTAs) and several 1,024-column chunks."""
    rng = np.random.default_rng(seed)
    out = []
    for i, (N, nmax) in enumerate([(12, 8), (16, 9), (10, 6), (3, 12), (12, 8)]):
        xyz, rad = random_cluster(rng, N, 1400 * nm, 40 * nm, 80 * nm, 20 * nm)
        sh = i % 2 == 1
        sp = G.spheres_array(xyz, rad, (2.0 + 0.04j) ** 2, nmax, eps_sh=(2.2 + 0.06j) ** 2,
                             ksippp=1.0 if sh else 0.0, ksiparppar=0.25 if sh else 0.0)
        wave = G.plane_wave(rng.uniform(500, 800) * nm, theta=rng.uniform(0, np.pi),
                            phi=rng.uniform(-np.pi, np.pi), sh=sh)
        out.append((sp, G.medium(1.0), wave, opts, prec))
    return out


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_fused_solve_matches_the_lockstep_graphs(G, form):
    """The fused solve (one cooperative launch per solve, a group of CTAs per
    slot) against the lockstep Arnoldi steps replayed as graphs: the same
    bits, statistics included, in far fewer launches."""
    opts, prec = (plain(G), G.C128) if form == "plain" else (mixed(G), G.C64)
    reqs = ragged_requests(G, opts, prec, seed=21) + blocky_requests(G, opts, prec)
    runs, launches = [], []
    for fused in (2, 0):  # 2: every class of these requests through the fused solve
        c = G.Context(0)
        c.tune(batch_fused=fused)
        runs.append(G.batch_solve(c, reqs))
        launches.append(c.last_launches)
        c.close()
    for a, b in zip(*runs):
        assert a["status"] == b["status"] == G.OK
        assert np.array_equal(a["xsec"], b["xsec"]) and np.array_equal(a["xsec_sh"], b["xsec_sh"])
        for h in ("ff", "sh"):
            for f in ("iterations", "inner_iterations", "rel_residual"):
                assert a[h][f] == b[h][f]
    assert launches[0] < launches[1]


def test_fp16_copies_in_the_batch(G):
    """The precision form's Arnoldi products on the scaled fp16 copies
    (inner_half = 1, the default) and on the complex64 matrices (0): both
    within 1e-6 of the FP64 single-request path, a few refinement cycles
    each."""
    reqs = ragged_requests(G, mixed(G), G.C64, seed=31) + blocky_requests(G, mixed(G), G.C64, seed=32)
    runs = {}
    for half in (1, 0):
        c = G.Context(0)
        c.tune(inner_half=half)
        runs[half] = G.batch_solve(c, reqs)
        c.close()
    c = G.Context(0)
    for i, (sp, bg, wave, opts, prec) in enumerate(reqs):
        xs, xsh, _ = G.wavelength_solve_sh(c, sp, bg, wave, plain(G), G.C128)
        for half in (1, 0):
            r = runs[half][i]
            assert r["status"] == G.OK and 1 <= r["ff"]["iterations"] <= 8
            assert rel(r["xsec"], xs) < 1e-6
            if wave.sh:
                assert rel(r["xsec_sh"], xsh) < 1e-6
    c.close()


def test_fp16_copies_with_tiny_block_columns(G):
    """Small spheres at long wavelengths with a large nMax: the high-order
    block columns of S fall to 1e-35 and below, where an unclamped fp16 scale
    overflows (its zero entries then turned into NaN). The batched precision
    form must converge to the same cross sections with and without the
    copies."""
    rng = np.random.default_rng(41)
    reqs = []
    for N, nmax in [(20, 9), (12, 11), (30, 7)]:
        xyz, rad = random_cluster(rng, N, 900 * nm, 30 * nm, 34 * nm, 20 * nm)
        sp = G.spheres_array(xyz, rad, (1.6 + 0.002j) ** 2, nmax)
        reqs.append((sp, G.medium(1.0), G.plane_wave(890 * nm), mixed(G), G.C64))
    runs = {}
    for half in (1, 0):
        c = G.Context(0)
        c.tune(inner_half=half)
        runs[half] = G.batch_solve(c, reqs)
        c.close()
    for a, b in zip(runs[1], runs[0]):
        assert a["status"] == b["status"] == G.OK
        assert np.all(np.isfinite(a["xsec"])) and rel(a["xsec"], b["xsec"]) < 1e-6


def test_failures_stay_with_their_request(G, ctx):
    rng = np.random.default_rng(3)
    xyz, rad = random_cluster(rng, 4, 800 * nm, 40 * nm, 60 * nm, 20 * nm)
    good = G.spheres_array(xyz, rad, 4.0, 4)
    overlap = G.spheres_array([[0, 0, 0], [0, 0, 50 * nm]], [40 * nm, 40 * nm], 4.0, 4)
    w = G.plane_wave(600 * nm)
    starved = G.options(G.SOLVE_GMRES, tol=1e-14, max_iter=2, restarts=1)
    reqs = [(good, G.medium(), w, plain(G), G.C128),
            (overlap, G.medium(), w, plain(G), G.C128),
            (good, G.medium(), w, G.options(G.SOLVE_LU), G.C128),  # LU is not batched
            (good, G.medium(), w, starved, G.C128),
            (good, G.medium(), w, plain(G), G.C128)]
    res = G.batch_solve(ctx, reqs)
    assert [r["status"] for r in res] == [G.OK, G.ERR_OVERLAP, G.ERR_INVALID, G.ERR_NOT_CONVERGED,
                                          G.OK]
    assert np.array_equal(res[0]["xsec"], res[4]["xsec"])
    # the unconverged request still reports its (approximate) cross sections
    assert res[3]["ff"]["iterations"] == 2 and np.all(np.isfinite(res[3]["xsec"]))


@pytest.mark.parametrize("nmax", [1, 2, 12, 15])
def test_batch_extreme_nmax(G, ctx, nmax):
    """The batched assembly's table layouts at the ends of the nMax range
    (global factor tables from nMax 14), with a single sphere and a pair,
    FF + SH, against the single-request FP64 path (LU). The SH cross
    sections are compared up to nMax 8: from nMax 10 the SH source reads
    X_int = X_sca (.) Iaux, where |Iaux| reaches 1e20 on the high orders, so two
    independent solves (GMRES to 1e-13 and LU) give different SH sources there,
    in the reference as here; the same holds for the fourth cross section (the
    absorption from the internal coefficients and the Mie factors). The
    batch's GMRES stops at a residual of 1e-13; with the condition number the
    system reaches at nMax 12-15 that leaves the FF cross sections within
    5e-9 of LU (1e-10 up to nMax 8)."""
    rng = np.random.default_rng(nmax)
    reqs = []
    for N in (1, 2, 2):
        xyz, rad = random_cluster(rng, N, 600 * nm, 50 * nm, 70 * nm, 30 * nm)
        sp = G.spheres_array(xyz, rad, (1.9 + 0.03j) ** 2, nmax, eps_sh=(2.0 + 0.05j) ** 2,
                             ksippp=1.0, ksiparppar=0.25)
        wave = G.plane_wave(rng.uniform(500, 800) * nm, theta=rng.uniform(0, np.pi),
                            phi=rng.uniform(-np.pi, np.pi), e_theta=0.6, e_phi=0.8j, sh=True)
        reqs.append((sp, G.medium(1.1), wave, plain(G), G.C128))
    res = G.batch_solve(ctx, reqs)
    for r, (sp, bg, wave, opts, prec) in zip(res, reqs):
        assert r["status"] == G.OK
        xs, xsh, _ = G.wavelength_solve_sh(ctx, sp, bg, wave, G.options(G.SOLVE_LU), prec)
        assert rel(r["xsec"][:3], xs[:3]) < (1e-10 if nmax <= 8 else 5e-9)
        if nmax <= 8:
            assert rel(r["xsec"][3], xs[3]) < 1e-10
            assert rel(r["xsec_sh"], xsh) < 1e-9
