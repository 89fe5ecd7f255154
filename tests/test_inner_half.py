"""The precision form's inner FP32 GMRES on a bf16 copy of the complex64
matrix: the copy is S rounded to bf16 (round to nearest even, real and
imaginary parts apart), written by the first product as it reads S; later
products read the copy and accumulate in FP32 in the same order as the
complex64 product. The TMA-staged and the register-prefetching kernels give
the same bits. FGMRES with the copy stays within 1e-6 of FP64, as without it.

Tolerances: products within 1e-5 (relative 2-norm) of an FP64 product of the
same matrix (S, or S rounded to bf16 in numpy); TMA against plain kernels
bitwise."""
import numpy as np
import pytest

from helpers import gpu_inputs, nm, oracle_cluster, random_cluster, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    return G


def bf16(a):
    """complex64 -> complex64 with both parts rounded to bf16 (nearest even)."""
    f = np.ascontiguousarray(a, dtype=np.complex64).view(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).view(np.complex64).reshape(a.shape)


def matrix(rng, n):
    # magnitudes over twelve decades, as the coupling blocks' orders give
    mag = 10.0 ** rng.uniform(-6, 6, size=(n, n))
    ph = rng.uniform(0, 2 * np.pi, size=(n, n))
    return np.asfortranarray((mag * np.exp(1j * ph)).astype(np.complex64))


@pytest.mark.parametrize("n", [701, 1030, 2048])
def test_bf16_copy_products(G, n):
    rng = np.random.default_rng(n)
    S = matrix(rng, n)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    ref64 = S.astype(np.complex128) @ x.astype(np.complex128)
    ref16 = bf16(S).astype(np.complex128) @ x.astype(np.complex128)
    out = {}
    for tma in (1, 0):
        c = G.Context(0)
        c.tune(matvec_tma=tma, inner_half=1)
        out[tma] = [G.matvec_inner(c, S, x, p) for p in (1, 2, 3)]
        c.close()
    y1, y2, y3 = out[1]
    assert rel(y1, ref64) < 1e-5          # the copy-writing product is the complex64 one
    assert rel(y2, ref16) < 1e-5          # later products: S rounded to bf16
    assert np.array_equal(y2, y3)
    assert rel(y2, ref64) > 1e-5          # (they do read the copy)
    for a, b in zip(out[1], out[0]):
        assert np.array_equal(a, b)       # TMA-staged and plain kernels: the same bits
    c = G.Context(0)
    c.tune(inner_half=0)
    assert np.array_equal(G.matvec_inner(c, S, x, 2), y1)
    c.close()


def test_fgmres_with_bf16_inner(G, oracle):
    """FGMRES (FP64 outer on the complex64 matrix, FP32 inner GMRES) with and
    without the bf16 copy: both within 1e-6 of FP64; the inner products run
    on the copy (one product per solve writes it)."""
    rng = np.random.default_rng(17)
    xyz, rad = random_cluster(rng, 14, 1000 * nm, 40 * nm, 70 * nm, 20 * nm)
    cl = oracle.Cluster(xyz=xyz, radius=rad, eps=(2.0 + 0.05j) ** 2, nmax=6, wavelength=650 * nm,
                        theta=0.4, phi=0.1)
    c = G.Context(0)
    sp, bg, wave = gpu_inputs(G, cl)
    pr = G.Problem(c, sp, bg, wave)
    pr.source_vector(copy=False)
    pr.assemble(G.FF, G.C128)
    pr.solve(G.options(G.SOLVE_GMRES, tol=1e-12))
    ref = pr.cross_sections()
    pr.assemble(G.FF, G.C64)
    opts = G.options(G.SOLVE_FGMRES_MIXED, tol=1e-10, max_iter=30, restarts=4, inner_iter=40,
                     inner_tol=1e-4)
    res = {}
    for on in (1, 0):
        c.tune(inner_half=on)
        c.timers(True)
        st = pr.solve(opts)
        c.timers(False)
        res[on] = (pr.cross_sections(), st, c.inner_timers())
    for on in (1, 0):
        xs, st, _ = res[on]
        assert st.rel_residual <= 1e-10 and st.inner_iterations > 0
        assert np.max(np.abs(xs - ref) / np.abs(ref)) < 1e-6
    t16 = res[1][2]
    assert t16["copy"][1] == 1 and t16["bf16"][1] == res[1][1].inner_iterations - 1
    assert res[0][2]["copy"][1] == 0 and res[0][2]["bf16"][1] == 0
    pr.close()
    c.close()
