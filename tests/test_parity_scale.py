"""GPU parity at the configurations' full sizes.

C1 (N = 100, nMax = 8, 16,000 unknowns, metal-like spheres in water): the
GPU's FP64 solve end to end against tests/golden/c1.npz, the oracle's own
GMRES solution (relative residual 1e-13) of its own assembled S, through both
Bessel routes: the oracle's recurrences (the route the GPU kernels take) and
the reference's AMOS. Compared: the source vector, the scattering
coefficients, the four cross sections and the near field at 2,048 points of
the C1 grid (64 inside spheres).

C2 (N = 400, nMax = 8, 64,000 unknowns; the complex128 S is 65.5 GB, more
than the oracle can hold on the host): the GPU's FP64 solution against whole
sphere block rows assembled by the oracle, as the residual rows
Q_i - sum_j S_ij x_j, and the oracle's source vector.

Tolerances: 1e-10 relative (normwise for vectors) for the FP64 path; 1e-9 of
||Q|| for the C2 residual rows (GMRES stops at 1e-10); 1e-6 for the precision
form's cross sections against FP64."""
import numpy as np
import pytest

from helpers import gpu_inputs, load_golden, oracle_cluster, rel

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


def problem(G, ctx, cl):
    return G.Problem(ctx, *gpu_inputs(G, cl))


def test_c1_end_to_end(G, ctx, oracle):
    g = load_golden("c1")
    cl = oracle_cluster(oracle, g)
    pr = problem(G, ctx, cl)
    Q = pr.source_vector()
    assert rel(Q, g["Q_rec"]) < 1e-10
    assert rel(Q, g["Q_amos"]) < 1e-10
    pr.assemble(G.FF, G.C128)
    st = pr.solve(G.options(G.SOLVE_GMRES, tol=1e-13, max_iter=400, restarts=6))
    assert st.rel_residual <= 1e-13
    X, Xi = pr.coefficients()
    xs = pr.cross_sections()
    E, H = pr.near_field(g["points"])
    for route in ("rec", "amos"):
        assert rel(X, g[f"X_sca_{route}"]) < 1e-10, (route, rel(X, g[f"X_sca_{route}"]))
        err = np.max(np.abs(xs - g[f"xsec_{route}"]) / np.abs(g[f"xsec_{route}"]))
        assert err < 1e-10, (route, err)
        assert rel(E, g[f"E_{route}"]) < 1e-10, (route, rel(E, g[f"E_{route}"]))
        assert rel(H, g[f"H_{route}"]) < 1e-10, (route, rel(H, g[f"H_{route}"]))
    # the 64 interior points alone (regular waves at the interior wave number)
    inside = g["inside"]
    assert rel(E[inside], g["E_rec"][inside]) < 1e-10
    # precision form on the same cluster
    pr.assemble(G.FF, G.C64)
    pr.solve(G.options(G.SOLVE_FGMRES_MIXED, tol=1e-8, max_iter=30, restarts=8, inner_iter=80, inner_tol=1e-4))
    err = np.max(np.abs(pr.cross_sections() - g["xsec_rec"]) / np.abs(g["xsec_rec"]))
    assert err < 1e-6, err
    pr.close()


def test_c2_block_row_residuals(G, ctx, oracle):
    import bench
    w = bench.WORKLOADS["c2"]
    xyz, rad = bench.cluster(w)
    cl = oracle.Cluster(xyz=xyz, radius=rad, eps=complex(w["index"]) ** 2, nmax=w["nmax"],
                        wavelength=w["lam"], bg_eps=complex(w["host"]) ** 2)
    pr = problem(G, ctx, cl)
    Q = pr.source_vector()
    pr_o = oracle.Problem(cl)
    assert rel(Q, pr_o.source_vector()) < 1e-10
    pr.assemble(G.FF, G.C128)
    st = pr.solve(G.options(G.SOLVE_GMRES, tol=1e-10, max_iter=400, restarts=6))
    assert st.rel_residual <= 1e-10
    x, _ = pr.coefficients()
    ref = pr.cross_sections()
    N, P2 = cl.n_spheres, 2 * cl.P
    qn = np.linalg.norm(Q)
    for i in (0, 123, 399):
        others = [j for j in range(N) if j != i]
        blocks = oracle.assemble_pairs(pr_o, [(i, j) for j in others])
        r = Q[P2 * i:P2 * (i + 1)] - x[P2 * i:P2 * (i + 1)]  # S_ii = I
        for j, b in zip(others, blocks):
            r -= b @ x[P2 * j:P2 * (j + 1)]
        assert np.linalg.norm(r) / qn < 1e-9, (i, np.linalg.norm(r) / qn)
    # precision form, the headline settings of bench.py
    pr.assemble(G.FF, G.C64)
    pr.solve(G.options(G.SOLVE_FGMRES_MIXED, tol=1e-7, max_iter=30, restarts=4, inner_iter=80, inner_tol=1e-3))
    err = np.max(np.abs(pr.cross_sections() - ref) / np.abs(ref))
    assert err < 1e-6, err
    pr.close()
