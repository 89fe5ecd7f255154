"""GPU row blocks of the sharded solve (om_assemble_rows, om_matvec_rows), on
one GPU: the pieces of every rank of a 1-, 2- and 3-rank partition, computed
one after another, concatenate to the same product bit for bit (a row's sum
does not depend on the split) and match the full matrix's product; GMRES on
that product matches om_solve's GMRES. The collective itself (NCCL between
GPUs) is covered on the host by tests/test_sharded.py."""
import numpy as np
import pytest

from helpers import gpu_inputs, nm, random_cluster, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    return G


def test_row_blocks_and_sharded_gmres(G, oracle):
    import torch
    from optimet_gb300.sharded import gmres, partition
    xyz, rad = random_cluster(np.random.default_rng(31), 9, 1100 * nm, 40 * nm, 70 * nm, 20 * nm)
    cl = oracle.Cluster(xyz=xyz, radius=rad, eps=(2.0 + 0.05j) ** 2, nmax=5, wavelength=650 * nm,
                        theta=0.7, phi=-0.4)
    ctx = G.Context(0)
    pr = G.Problem(ctx, *gpu_inputs(G, cl))
    Q = pr.source_vector()
    pr.assemble(G.FF, G.C128)
    S = pr.matrix()
    P2 = 2 * cl.P
    rng = np.random.default_rng(2)
    v = rng.standard_normal(pr.n) + 1j * rng.standard_normal(pr.n)
    xd = torch.from_numpy(v).cuda()

    def product(world):
        pieces = []
        for r in range(world):
            g1, g2 = partition(cl.n_spheres, world, r)
            pr.assemble_rows(g1, g2)
            y = torch.zeros(P2 * (g2 - g1), dtype=torch.complex128, device="cuda")
            torch.cuda.synchronize()
            pr.matvec_rows(xd.data_ptr(), y.data_ptr())
            pieces.append(y.cpu().numpy())
        return np.concatenate(pieces)

    y1 = product(1)
    assert rel(y1, S @ v) < 1e-13
    for world in (2, 3):
        assert np.array_equal(product(world), y1)

    # GMRES around the row-block product (one rank holding all rows)
    pr.assemble_rows(0, cl.n_spheres)
    x_dev = torch.zeros(pr.n, dtype=torch.complex128, device="cuda")
    y_dev = torch.zeros(pr.n, dtype=torch.complex128, device="cuda")

    def matvec(u):
        x_dev.copy_(torch.from_numpy(np.ascontiguousarray(u)))
        torch.cuda.synchronize()
        pr.matvec_rows(x_dev.data_ptr(), y_dev.data_ptr())
        return y_dev.cpu().numpy()

    x, its, r = gmres(matvec, Q, tol=1e-12, max_iter=120, restarts=4)
    assert r <= 1e-12
    pr.solve(G.options(G.SOLVE_GMRES, tol=1e-12, max_iter=120, restarts=4))
    assert rel(x, pr.coefficients()[0]) < 1e-10
    pr.close()
    ctx.close()
