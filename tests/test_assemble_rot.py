"""GPU tests of the precision form's assembly by rotations (assemble_rot.cu):
the complex64 matrix built from rotated z-axis translations against the FP64
assembly of the same problem, block by block, and against the general
translation's complex64 kernel.

Tolerance: each 2P x 2P block of the complex64 matrix within 1e-6 of its FP64
block, relative to the block's largest entry (complex64 rounding is 6e-8; the
FP32 rotation products add sums of up to 2 nMax + 1 terms)."""
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


@pytest.fixture(scope="module")
def ctx(G):
    c = G.Context(0)
    yield c
    c.tune(assemble_rotation=1)
    c.close()


def cluster(nsph, nmax, seed):
    """Random spheres plus two on the z axis of the first (theta = 0 and pi
    pair directions, where the Wigner d reduce to the identity and its mirror)."""
    rng = np.random.default_rng(seed)
    xyz, rad = random_cluster(rng, nsph, 1400 * nm, 40 * nm, 70 * nm, 20 * nm)
    top = xyz[0] + np.array([0, 0, rad[0] + 200 * nm])
    bot = xyz[0] - np.array([0, 0, rad[0] + 220 * nm])
    keep = [k for k in range(nsph) if min(np.linalg.norm(xyz[k] - top), np.linalg.norm(xyz[k] - bot))
            > rad[k] + 90 * nm]
    xyz = np.vstack([xyz[keep], top, bot])
    rad = np.concatenate([rad[keep], [50 * nm, 45 * nm]])
    return xyz, rad


def block_errors(S, R, P, N):
    worst = 0.0
    for i in range(N):
        for j in range(N):
            a = S[2 * P * i:2 * P * (i + 1), 2 * P * j:2 * P * (j + 1)]
            b = R[2 * P * i:2 * P * (i + 1), 2 * P * j:2 * P * (j + 1)]
            worst = max(worst, float(np.max(np.abs(a - b)) / np.max(np.abs(b))))
    return worst


def assemble_both(G, ctx, xyz, rad, eps, nmax, bg, harmonic, rotation):
    sp = G.spheres_array(xyz, rad, eps, nmax, eps_sh=eps)
    pr = G.Problem(ctx, sp, bg, G.plane_wave(650 * nm, 0.4, 0.9, sh=harmonic == G.SH))
    pr.assemble(harmonic, G.C128)
    S64 = pr.matrix(harmonic)
    ctx.tune(assemble_rotation=rotation)
    pr.assemble(harmonic, G.C64)
    S32 = pr.matrix(harmonic)
    ctx.tune(assemble_rotation=1)
    pr.close()
    return S32, S64


@pytest.mark.parametrize("nmax", [1, 2, 4, 8, 12, 15])
def test_rotation_assembly_matches_fp64(G, ctx, nmax):
    xyz, rad = cluster(6, nmax, 100 + nmax)
    N, P = len(rad), nmax * (nmax + 2)
    S32, S64 = assemble_both(G, ctx, xyz, rad, (2.0 + 0.05j) ** 2, nmax, G.medium(1.0), G.FF, 1)
    err = block_errors(S32, S64, P, N)
    assert err < 1e-6, err
    # identity diagonal blocks exactly
    for i in range(N):
        assert np.array_equal(S32[2 * P * i:2 * P * (i + 1), 2 * P * i:2 * P * (i + 1)], np.eye(2 * P))


def test_rotation_assembly_complex_wavenumber(G, ctx):
    """Lossy host medium: the m < 0 entries come from the conjugate-wave chain."""
    nmax = 6
    xyz, rad = cluster(5, nmax, 7)
    N, P = len(rad), nmax * (nmax + 2)
    S32, S64 = assemble_both(G, ctx, xyz, rad, (2.5 + 0.1j) ** 2, nmax, G.medium((1.4 + 0.02j) ** 2),
                             G.FF, 1)
    assert block_errors(S32, S64, P, N) < 1e-6


def test_rotation_assembly_second_harmonic(G, ctx):
    nmax = 5
    xyz, rad = cluster(5, nmax, 9)
    N, P = len(rad), nmax * (nmax + 2)
    S32, S64 = assemble_both(G, ctx, xyz, rad, (2.0 + 0.05j) ** 2, nmax, G.medium(1.0), G.SH, 1)
    assert block_errors(S32, S64, P, N) < 1e-6


def test_rotation_and_chain_assemblies_agree(G, ctx):
    """The two complex64 assemblies (rotations; all recurrence chains) are
    both within the tolerance of FP64 on the same problem."""
    nmax = 8
    xyz, rad = cluster(5, nmax, 11)
    N, P = len(rad), nmax * (nmax + 2)
    S_rot, S64 = assemble_both(G, ctx, xyz, rad, (2.0 + 0.05j) ** 2, nmax, G.medium(1.0), G.FF, 1)
    S_chain, _ = assemble_both(G, ctx, xyz, rad, (2.0 + 0.05j) ** 2, nmax, G.medium(1.0), G.FF, 0)
    assert block_errors(S_rot, S64, P, N) < 1e-6
    assert block_errors(S_chain, S64, P, N) < 1e-6
    assert block_errors(S_rot, S_chain, P, N) < 2e-6
