"""The tensor-core (tcgen05) complex64 trailing update of the precision form's
LU: exact on small integers (which the scaled fp16 parts and the FP32
accumulators hold exactly: this pins the operand layout, the descriptors, the
scales and the TMEM read-back), within the scaled fp16 hi/lo split's accuracy
on general data, and the LU-refined solve agrees with and without it."""
import numpy as np
import pytest

from helpers import load_golden, oracle_cluster, random_cluster, nm

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


# k > 32 runs in several chunks through the kernel's operand tiles (the
# LU's rank-128 trailing updates), with a ragged last chunk for 80 and 33
@pytest.mark.parametrize("m,n,k", [(128, 64, 32), (300, 200, 32), (257, 70, 17), (5, 3, 1),
                                   (300, 200, 128), (257, 70, 80), (130, 65, 33), (258, 70, 80),
                                   (1000, 1030, 128), (130, 66, 64)])
def test_update_exact_on_small_integers(G, ctx, m, n, k):
    rng = np.random.default_rng(m + n + k)
    A = (rng.integers(-8, 9, (m, k)) + 1j * rng.integers(-8, 9, (m, k))).astype(np.complex64)
    B = (rng.integers(-8, 9, (k, n)) + 1j * rng.integers(-8, 9, (k, n))).astype(np.complex64)
    C = (rng.integers(-100, 101, (m, n)) + 1j * rng.integers(-100, 101, (m, n))).astype(np.complex64)
    out = G.cgemm_sub_c64(ctx, A, B, C)
    ref = C.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    assert np.array_equal(out.astype(np.complex128), ref)


@pytest.mark.parametrize("k", [32, 128])
def test_update_accuracy_general(G, ctx, k):
    rng = np.random.default_rng(3)
    m, n = 600, 400
    A = (rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))).astype(np.complex64)
    B = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))).astype(np.complex64)
    C = (rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))).astype(np.complex64)
    out = G.cgemm_sub_c64(ctx, A, B, C)
    ref = C.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    scale = np.abs(A.astype(np.complex128)) @ np.abs(B.astype(np.complex128))
    err = np.max(np.abs(out - ref) / scale)
    assert err < 2e-6, err   # three products of scaled fp16 parts: about 21 significant bits
    assert err > 1e-9        # (and not an FP32 SIMT path in disguise)


# The persistent update (one CTA per SM walking its range of tiles, A resident
# up to k = 128 and streamed with B above, C through a ring, double-buffered
# accumulators) issues the same MMAs in the same order as the one-CTA-per-tile
# kernel and rounds the same epilogue, so the two agree bit for bit: a grid
# with fewer tiles than SMs, ranges that cross row tiles, long ranges that
# wrap every ring many times, and both A modes.
@pytest.mark.parametrize("m,n,k", [(256, 192, 128), (2050, 1500, 128), (4000, 4001, 128), (1998, 700, 96),
                                   (1000, 900, 256), (700, 1300, 160)])
def test_persistent_update_matches_tile_grid(G, ctx, m, n, k):
    rng = np.random.default_rng(m + 7 * n + k)
    A = (rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))).astype(np.complex64)
    B = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))).astype(np.complex64)
    C = (rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))).astype(np.complex64)
    out = {}
    for tc in (1, 2):
        ctx.tune(lu_tensor_cores=tc)
        out[tc] = G.cgemm_sub_c64(ctx, A, B, C)
    ctx.tune(lu_tensor_cores=3)
    assert np.array_equal(np.ascontiguousarray(out[1]).view(np.float32),
                          np.ascontiguousarray(out[2]).view(np.float32))
    ref = C.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    scale = np.abs(A.astype(np.complex128)) @ np.abs(B.astype(np.complex128))
    assert np.max(np.abs(out[1] - ref) / scale) < 2e-6


# n = 1,152: four blocks of 256 columns and a last one of 128; n = 450: a
# last block of 194 columns (inner panels of 32 and a last one of 2)
@pytest.mark.parametrize("N,nmax", [(12, 6), (15, 3)])
def test_lu_mixed_with_and_without_tensor_cores(G, ctx, N, nmax):
    rng = np.random.default_rng(21)
    xyz, rad = random_cluster(rng, N, 900 * nm, 40 * nm, 70 * nm, 20 * nm)
    sp = G.spheres_array(xyz, rad, (2.5 + 0.05j) ** 2, nmax)
    bg, wave = G.medium(1.0), G.plane_wave(600 * nm)
    ref = G.wavelength_solve(ctx, sp, bg, wave, G.options(G.SOLVE_LU), G.C128)[0]
    opts = G.options(G.SOLVE_LU_MIXED, tol=1e-10, max_iter=30, restarts=4)
    out = {}
    for tc in (3, 1, 2, 0):
        ctx.tune(lu_tensor_cores=tc)
        xs, _, _, st = G.wavelength_solve(ctx, sp, bg, wave, opts, G.C64)
        out[tc] = (xs, st.iterations)
    # the hybrid (3) takes the same bits as both single-kernel forms
    assert np.array_equal(out[3][0], out[1][0]) and np.array_equal(out[3][0], out[2][0])
    ctx.tune(lu_tensor_cores=3)
    for tc, (xs, it) in out.items():
        err = np.abs(xs - ref) / np.abs(ref)
        # C_ext, C_sca and C_ext - C_sca to 1e-6; C_abs comes from the internal
        # coefficients (X_sca times the Iaux factors, which amplify what the
        # 1e-10 residual leaves in X_sca by about 1e4 here), so 1e-5
        assert np.max(err[:3]) < 1e-6 and err[3] < 1e-5, (tc, xs, ref)
    # the FP64 refinement absorbs the weaker factorisation in a few more steps
    assert out[1][1] <= out[0][1] + 10


def test_lu_tall_panels(G, ctx):
    """n = 8,208 unknowns: the LU panels run on many CTAs (tall-panel path,
    from 8,192 rows). FP64 LU against FP64 GMRES, and the LU refinement role
    (complex64 LU with tensor-core updates, GMRES-based refinement) against
    FP64."""
    rng = np.random.default_rng(33)
    xyz, rad = random_cluster(rng, 171, 2400 * nm, 40 * nm, 60 * nm, 20 * nm)
    sp = G.spheres_array(xyz, rad, (1.8 + 0.02j) ** 2, 4)     # P = 24: n = 8,208
    bg, wave = G.medium(1.0), G.plane_wave(700 * nm)
    ref = G.wavelength_solve(ctx, sp, bg, wave, G.options(G.SOLVE_GMRES, tol=1e-13, max_iter=300), G.C128)[0]
    lu = G.wavelength_solve(ctx, sp, bg, wave, G.options(G.SOLVE_LU), G.C128)[0]
    assert np.max(np.abs(lu - ref) / np.abs(ref)) < 1e-10
    xs, _, _, st = G.wavelength_solve(ctx, sp, bg, wave,
                                      G.options(G.SOLVE_LU_MIXED, tol=1e-10, max_iter=30, restarts=4), G.C64)
    assert st.rel_residual <= 1e-10
    assert np.max(np.abs(xs - ref) / np.abs(ref)) < 1e-6


@pytest.mark.parametrize("N,nmax", [(15, 3), (12, 6), (40, 5)])
def test_one_launch_sweeps_match_block_launches(G, ctx, N, nmax):
    """The one-launch triangular sweeps (blocks published through flags)
    against one launch per 32-row block: the same bits for the FP64 LU role
    and the LU refinement role; n = 450 ends in a partial block, n = 1,152
    leaves most CTAs one block, n = 2,800 (88 blocks) gives some CTAs two."""
    rng = np.random.default_rng(N + nmax)
    xyz, rad = random_cluster(rng, N, 900 * nm * max(1, N // 15), 40 * nm, 70 * nm, 20 * nm)
    sp = G.spheres_array(xyz, rad, (2.5 + 0.05j) ** 2, nmax)
    bg, wave = G.medium(1.0), G.plane_wave(600 * nm)
    out = {}
    for mode in (1, 2):
        ctx.tune(lu_persistent=mode)
        pr = G.Problem(ctx, sp, bg, wave)
        pr.source_vector(copy=False)
        pr.assemble(G.FF, G.C128)
        pr.solve(G.options(G.SOLVE_LU))
        x64 = pr.coefficients()[0].copy()
        pr.assemble(G.FF, G.C64)
        # twice, so that the captured sweeps replay with a new epoch
        for _ in range(2):
            st = pr.solve(G.options(G.SOLVE_LU_MIXED, tol=1e-10, max_iter=30, restarts=4))
        out[mode] = (x64, pr.coefficients()[0].copy(), st.iterations)
        pr.close()
    ctx.tune(lu_persistent=1)
    assert np.array_equal(out[1][0], out[2][0])
    assert np.array_equal(out[1][1], out[2][1]) and out[1][2] == out[2][2]


def test_cooperative_panels_give_the_same_factors(G, ctx):
    """n = 9,600 (44 panels of 8,192 rows or more): the one-launch cooperative
    panel (a grid-wide barrier per column, row interchanges kept in a table and
    applied after the last column; the rows in shared memory, mode 1, or in
    global memory, mode 3) takes the same operations per entry as the
    two-launches-per-column panel, so both LU roles give bit-identical
    solutions; and the persistent trailing update with cooperative panels
    matches the one-CTA-per-tile update with per-column panels bit for bit."""
    rng = np.random.default_rng(35)
    xyz, rad = random_cluster(rng, 200, 2600 * nm, 40 * nm, 60 * nm, 20 * nm)
    sp = G.spheres_array(xyz, rad, (1.8 + 0.02j) ** 2, 4)     # P = 24: n = 9,600
    bg, wave = G.medium(1.0), G.plane_wave(700 * nm)
    out = {}
    for mode in (1, 2, 3):
        ctx.tune(lu_tensor_cores=min(mode, 2), lu_persistent=mode)
        pr = G.Problem(ctx, sp, bg, wave)
        pr.source_vector(copy=False)
        pr.assemble(G.FF, G.C128)
        pr.solve(G.options(G.SOLVE_LU))
        x64 = pr.coefficients()[0].copy()
        pr.assemble(G.FF, G.C64)
        st = pr.solve(G.options(G.SOLVE_LU_MIXED, tol=1e-10, max_iter=30, restarts=4))
        out[mode] = (x64, pr.coefficients()[0].copy(), st.iterations)
        pr.close()
    ctx.tune(lu_tensor_cores=3, lu_persistent=1)
    for mode in (2, 3):
        assert np.array_equal(out[1][0], out[mode][0])
        assert np.array_equal(out[1][1], out[mode][1]) and out[1][2] == out[mode][2]
    assert np.max(np.abs(out[1][1] - out[1][0])) / np.max(np.abs(out[1][0])) < 1e-8

