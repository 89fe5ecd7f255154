"""One large solve sharded over several GPUs by sphere block rows.

The reference distributes its matrix by spheres (matvec_parallel,
PreconditionedMatrix.cpp:989-1054): rank r owns the block rows of spheres
gran1 .. gran2 - 1 (the first nobj % size ranks one sphere more, :1001-1007),
multiplies them with the full 2PN vector, and the row pieces are gathered in
rank order and broadcast (MPI_Gatherv + MPI_Bcast, :1044-1051); the GMRES
recurrence around it then runs on full vectors on every rank. This module does
the same with one process per GPU:

* ``partition`` is the reference's sphere split;
* ``RowGather`` all-gathers the ranks' row pieces in rank order over
  ``torch.distributed`` (NCCL between GPUs, gloo on the host);
* ``gmres`` is restarted GMRES (classical Gram-Schmidt with one
  re-orthogonalisation, Givens rotations, stop on the residual estimate
  relative to ||b||, as Gmres_Zcomp, PreconditionedMatrix.cpp:892-985) on
  full vectors, replicated on every rank; only the matrix-vector product is
  distributed, so the iterates do not depend on the number of ranks when each
  rank's rows sum in a split-independent order;
* ``GpuRows`` is a rank's device matvec: om_assemble_rows / om_matvec_rows on
  the rank's own GPU.
"""
from __future__ import annotations

import numpy as np


def partition(nobj: int, size: int, rank: int):
    """Spheres [gran1, gran2) of `rank` (PreconditionedMatrix.cpp:1001-1007)."""
    q, r = divmod(nobj, size)
    if rank < r:
        g1 = rank * (q + 1)
        return g1, g1 + q + 1
    g1 = rank * q + r
    return g1, g1 + q


class RowGather:
    """All-gather of per-rank row pieces (complex128) into the full vector in
    rank order. `counts[r]` is rank r's number of rows. Pieces are padded to
    the largest count for torch.distributed.all_gather."""

    def __init__(self, counts, device="cpu"):
        self.counts = list(counts)
        self.device = device
        import torch.distributed as dist
        self.dist = dist
        self.world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1

    def __call__(self, piece):
        import torch
        if self.world == 1:
            return piece.cpu().numpy() if torch.is_tensor(piece) else np.asarray(piece)
        m = max(self.counts)
        if not torch.is_tensor(piece):
            piece = torch.from_numpy(np.ascontiguousarray(piece))
        piece = piece.to(self.device)
        buf = torch.zeros(m, dtype=torch.complex128, device=self.device)
        buf[:piece.numel()] = piece
        # complex tensors travel as float64 pairs (gloo and NCCL both carry those)
        bufs = [torch.zeros(2 * m, dtype=torch.float64, device=self.device) for _ in range(self.world)]
        self.dist.all_gather(bufs, torch.view_as_real(buf).reshape(-1))
        parts = [torch.view_as_complex(b.reshape(-1, 2))[:c] for b, c in zip(bufs, self.counts)]
        return torch.cat(parts).cpu().numpy()


def _givens(a, b):
    """(c, s, r) with [c s; -conj(s) c] [a; b] = [r; 0], c real."""
    if b == 0:
        return 1.0, 0j, a
    if a == 0:
        return 0.0, np.conj(b) / abs(b), abs(b)
    t = np.hypot(abs(a), abs(b))
    c = abs(a) / t
    s = (a / abs(a)) * np.conj(b) / t
    return c, s, (a / abs(a)) * t


def gmres(matvec, b, tol=1e-10, max_iter=200, restarts=4):
    """Restarted GMRES on full vectors; matvec(x) returns S x (full length).
    Returns (x, iterations, relative residual estimate)."""
    b = np.asarray(b, dtype=np.complex128)
    n = b.size
    x = np.zeros(n, np.complex128)
    bnorm = np.linalg.norm(b)
    if bnorm == 0:
        return x, 0, 0.0
    its, rel = 0, 1.0
    for cycle in range(restarts):
        r = b - matvec(x) if cycle else b.copy()
        beta = np.linalg.norm(r)
        rel = beta / bnorm
        if rel <= tol:
            break
        V = np.zeros((max_iter + 1, n), np.complex128)
        H = np.zeros((max_iter + 1, max_iter), np.complex128)
        cs, sn = np.zeros(max_iter), np.zeros(max_iter, np.complex128)
        g = np.zeros(max_iter + 1, np.complex128)
        g[0] = beta
        V[0] = r / beta
        k = 0
        for k in range(max_iter):
            w = matvec(V[k])
            its += 1
            h = V[:k + 1].conj() @ w
            w = w - V[:k + 1].T @ h
            h2 = V[:k + 1].conj() @ w
            w = w - V[:k + 1].T @ h2
            h = h + h2
            hk1 = np.linalg.norm(w)
            col = np.concatenate([h, [hk1]])
            for i in range(k):
                t = cs[i] * col[i] + sn[i] * col[i + 1]
                col[i + 1] = -np.conj(sn[i]) * col[i] + cs[i] * col[i + 1]
                col[i] = t
            cs[k], sn[k], col[k] = _givens(col[k], col[k + 1])
            col[k + 1] = 0
            H[:k + 2, k] = col
            g[k + 1] = -np.conj(sn[k]) * g[k]
            g[k] = cs[k] * g[k]
            rel = abs(g[k + 1]) / bnorm
            if rel <= tol or k == max_iter - 1 or hk1 == 0:
                break
            V[k + 1] = w / hk1
        y = np.zeros(k + 1, np.complex128)
        for i in range(k, -1, -1):
            y[i] = (g[i] - H[i, i + 1:k + 1] @ y[i + 1:k + 1]) / H[i, i]
        x = x + V[:k + 1].T @ y
        if rel <= tol:
            break
    return x, its, rel


class GpuRows:
    """A rank's rows of S on its GPU: om_assemble_rows for the rank's spheres,
    om_matvec_rows on torch device tensors, the all-gather over NCCL."""

    def __init__(self, problem, rank, world, harmonic=0):
        import torch
        from . import FF
        self.pr = problem
        self.harmonic = harmonic if harmonic is not None else FF
        N, P = problem.N, problem.P
        self.g1, self.g2 = partition(N, world, rank)
        self.rows = 2 * P * (self.g2 - self.g1)
        problem.assemble_rows(self.g1, self.g2, self.harmonic)
        counts = [2 * P * (partition(N, world, r)[1] - partition(N, world, r)[0]) for r in range(world)]
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.gather = RowGather(counts, self.device)
        self.x = torch.zeros(problem.n, dtype=torch.complex128, device=self.device)
        self.y = torch.zeros(self.rows, dtype=torch.complex128, device=self.device)

    def __call__(self, v):
        import torch
        self.x.copy_(torch.from_numpy(np.ascontiguousarray(v, dtype=np.complex128)))
        torch.cuda.current_stream().synchronize()
        self.pr.matvec_rows(self.x.data_ptr(), self.y.data_ptr(), self.harmonic)
        return self.gather(self.y)
