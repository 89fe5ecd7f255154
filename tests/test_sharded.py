"""Row-block sharded solve (optimet_gb300.sharded) as gloo ranks on the host:
the reference's sphere partition, the rank-order gather of the row pieces,
and GMRES with the distributed matvec against the single-rank solve and the
oracle's LU. Each rank's local matvec is its rows of the oracle's S."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from optimet_gb300.sharded import gmres, partition

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cluster(O):
    from helpers import nm, random_cluster
    xyz, rad = random_cluster(np.random.default_rng(21), 7, 900 * nm, 40 * nm, 70 * nm, 20 * nm)
    return O.Cluster(xyz=xyz, radius=rad, eps=(2.0 + 0.05j) ** 2, nmax=3, wavelength=650 * nm,
                     theta=0.4, phi=0.3)


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    from optimet_gb300.sharded import RowGather
    O.lib()
    O.set_threads(1)
    cl = _cluster(O)
    pr = O.Problem(cl)
    S, Q = pr.scattering_matrix(), pr.source_vector()
    P2 = 2 * cl.P
    parts = [partition(cl.n_spheres, world, r) for r in range(world)]
    g1, g2 = parts[rank]
    rows = S[P2 * g1:P2 * g2]
    gather = RowGather([P2 * (b - a) for a, b in parts])
    # gather order: rank r's piece lands in rows [P2 g1(r), P2 g2(r))
    order = gather(np.full(P2 * (g2 - g1), rank + 1.0, np.complex128))
    x, its, rel = gmres(lambda v: gather(rows @ v), Q, tol=1e-13, max_iter=60, restarts=4)
    out.put((rank, order, x, its, rel))
    dist.destroy_process_group()


def test_partition_is_the_references():
    for nobj in range(1, 40):
        for size in range(1, 9):
            got = [partition(nobj, size, r) for r in range(size)]
            q, rem = divmod(nobj, size)
            for r, (g1, g2) in enumerate(got):
                if r < rem:  # PreconditionedMatrix.cpp:1001-1007
                    assert (g1, g2) == (r * (q + 1), r * (q + 1) + q + 1)
                else:
                    assert (g1, g2) == (r * q + rem, r * q + rem + q)
            assert got[0][0] == 0 and got[-1][1] == nobj
            assert all(got[r][1] == got[r + 1][0] for r in range(size - 1))


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_gmres_gloo_ranks(oracle, world):
    cl = _cluster(oracle)
    pr = oracle.Problem(cl)
    S, Q = pr.scattering_matrix(), pr.source_vector()
    x1, its1, _ = gmres(lambda v: S @ v, Q, tol=1e-13, max_iter=60, restarts=4)
    x_lu = oracle.lu_solve(S, Q)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    P2 = 2 * cl.P
    want = np.concatenate([np.full(P2 * (b - a), r + 1.0) for r, (a, b) in
                           enumerate(partition(cl.n_spheres, world, r) for r in range(world))])
    for rank, order, x, its, rel in res:
        assert np.array_equal(order, want)
        assert rel <= 1e-13 and its == its1
        assert np.max(np.abs(x - x1)) / np.max(np.abs(x1)) < 1e-12
        assert np.max(np.abs(x - x_lu)) / np.max(np.abs(x_lu)) < 1e-10
    # every rank ends with the same iterate (the recurrence is replicated)
    assert all(np.array_equal(res[0][2], r[2]) for r in res[1:])
