"""Generate the golden fixtures in tests/golden/ (run in a container that has
the reference tree, so the oracle can route its Bessel layer through the
reference's own AMOS build in oracle/_ref).

    OPTIMET_REFERENCE=<OPTIMET source tree> python tests/golden/make_golden.py [c1]

(`c1` writes only the full-size C1 fixture, a few minutes of host work.)

Each fixture is an .npz holding the inputs (cluster description) and the
oracle's outputs computed with the reference's AMOS Bessel arithmetic. The GPU
box has no reference tree; tests there compare against these files and against
the oracle's own (recurrence-based) Bessel layer.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

nm = 1e-9


def cases():
    """Small clusters covering the configs' shapes (C0 exactly, others scaled down)."""
    out = {}
    # C0: two spheres a=100 nm, n=3.5+0.01i, centres 250 nm apart on z, vacuum,
    # x-polarised plane wave along +z, lambda=600 nm, nMax=6.
    out["c0"] = O.Cluster(xyz=[[0, 0, -125 * nm], [0, 0, 125 * nm]], radius=100 * nm,
                          eps=(3.5 + 0.01j) ** 2, nmax=6, wavelength=600 * nm)
    # C1-like: metal-like spheres in water, oblique incidence, nMax=4.
    rng = np.random.default_rng(11)
    xyz, rad = random_cluster(rng, 5, 600 * nm, 50 * nm, 80 * nm, 20 * nm)
    out["metal5"] = O.Cluster(xyz=xyz, radius=rad, eps=(0.3 + 3.0j) ** 2, nmax=4,
                              wavelength=650 * nm, bg_eps=1.33 ** 2, theta=0.4, phi=1.1,
                              e_theta=0.6, e_phi=0.8j)
    # C2-like dielectric, nMax=5, three spheres.
    xyz, rad = random_cluster(np.random.default_rng(12), 3, 500 * nm, 40 * nm, 70 * nm, 20 * nm)
    out["diel3"] = O.Cluster(xyz=xyz, radius=rad, eps=(2.0 + 0.05j) ** 2, nmax=5,
                             wavelength=650 * nm, theta=2.0, phi=-0.7, e_theta=1.0, e_phi=0.0)
    # Single sphere off the origin with SH permittivity and surface + bulk chi(2), nMax=3.
    out["single_sh"] = O.Cluster(xyz=[[40 * nm, -30 * nm, 20 * nm]], radius=120 * nm,
                                 eps=(4.0 + 0.1j) ** 2, eps_sh=(4.2 + 0.2j) ** 2, nmax=3,
                                 wavelength=800 * nm, theta=0.9, phi=0.2, ksippp=1.0,
                                 ksiparppar=0.25, gamma=0.3)
    # Two spheres, C3-like chi(2) (perp-perp-perp 1.0, par-perp-par 0.25, no bulk term), nMax=4.
    out["pair_sh"] = O.Cluster(xyz=[[0, 0, 0], [180 * nm, 60 * nm, -90 * nm]], radius=[70 * nm, 90 * nm],
                               eps=[(2.5 + 0.05j) ** 2, (3.0 + 0.02j) ** 2],
                               eps_sh=[(2.6 + 0.06j) ** 2, (3.1 + 0.03j) ** 2], nmax=4,
                               wavelength=700 * nm, theta=0.5, phi=-0.4, e_theta=0.8, e_phi=0.6j,
                               ksippp=1.0, ksiparppar=0.25)
    return out


def random_cluster(rng, n, edge, rmin, rmax, gap):
    """Seeded rejection sampling: centres uniform in a cube of side `edge`
    (centred on the origin), radii uniform in [rmin, rmax], pairwise gap >= `gap`."""
    xyz, rad = [], []
    while len(xyz) < n:
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(-edge / 2 + r, edge / 2 - r, size=3)
        if all(np.linalg.norm(c - p) >= r + q + gap for p, q in zip(xyz, rad)):
            xyz.append(c)
            rad.append(r)
    return np.array(xyz), np.array(rad)


def field_points(cl, count, rng):
    lo = cl.xyz.min(axis=0) - 150 * nm
    hi = cl.xyz.max(axis=0) + 150 * nm
    pts = rng.uniform(lo, hi, size=(count, 3))
    pts[0] = cl.xyz[0] + np.array([0.3, -0.2, 0.1]) * cl.radius[0]  # one interior point
    return pts


def make(name, cl):
    pr = O.Problem(cl)
    n, P, N = pr.n, cl.P, cl.n_spheres
    S = pr.scattering_matrix()
    Q = pr.source_vector()
    X = O.lu_solve(S, Q)
    Xi = pr.internal(X)
    xsec = pr.cross_sections(X)
    pts = field_points(cl, 24, np.random.default_rng(5))
    E, H = pr.near_field(X, Xi, pts)
    # one off-diagonal block (sphere 1 rows, sphere 0 cols) and SH matrix block
    blk = (slice(0, 2 * P), slice(2 * P, 4 * P)) if N > 1 else (slice(0, 2 * P), slice(0, 2 * P))
    Ssh = pr.scattering_matrix(sh=True)
    rel = np.array(O.to_spherical(*(cl.xyz[-1] - cl.xyz[0]))) if N > 1 else np.array([150 * nm, 0.7, 0.4])
    k, omega = pr.wave_numbers()
    A_irr, B_irr = O.coupling(rel, k, cl.nmax, True)
    A_reg, B_reg = O.coupling(rel, k, cl.nmax, False)
    sh = {}
    if np.any(cl.chi != 0):
        tab = O.clg_tables(cl.nmax)
        K, K1, Xs, Xis = pr.sh_solve(tab, Xi)
        E_sh, H_sh = pr.near_field_sh(tab, Xi, Xs, Xis, pts)
        sh = dict(chi=cl.chi[0], K=K, K1ana=K1, X_sca_SH=Xs, X_int_SH=Xis, E_sh=E_sh, H_sh=H_sh,
                  xsec_sh=pr.sh_cross_sections(tab, Xi, Xs, Xis),
                  sh_factors=np.stack([pr.sh_factors(j) for j in range(N)]))
        if cl.nmax <= 3:
            sh["clg"] = tab
        print(name, "SH xsec", sh["xsec_sh"])
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"), **sh,
        xyz=cl.xyz, radius=cl.radius, eps=cl.eps, mu=cl.mu, eps_sh=cl.eps_sh,
        bg=np.array([cl.bg_eps, cl.bg_mu], np.complex128), nmax=cl.nmax,
        wavelength=cl.wavelength, angles=np.array([cl.theta, cl.phi]),
        pol=np.array([cl.e_theta, cl.e_phi], np.complex128),
        waveK=k, omega=omega, inc=pr.inc_coeffs(),
        T=np.stack([pr.tmatrix(j) for j in range(N)]),
        T_sh=np.stack([pr.tmatrix(j, sh=True) for j in range(N)]),
        Q=Q, S_block=S[blk], S_sh_block=Ssh[blk], X_sca=X, X_int=Xi, xsec=xsec,
        points=pts, E=E, H=H, rel=rel, A_irr=A_irr, B_irr=B_irr, A_reg=A_reg, B_reg=B_reg,
        S_full=S if n <= 200 else np.zeros(0),
    )
    print(name, "n =", n, "xsec", xsec)


def bessel_table():
    """Reference AMOS spherical Bessel/Hankel values at the argument kinds the
    path uses (real, negative real, complex interior arguments)."""
    zs = np.array([0.37, 1.0, 2.5, 6.0, 13.7, 44.0, 88.0, -3.0, -44.0, 0.24 + 2.4j,
                   2.1 + 0.05j, 7.5 + 0.19j, 1.5 + 0.001j, 0.05 + 0.5j, 30 + 1j], np.complex128)
    L = 25
    J = np.zeros((len(zs), L + 1), np.complex128)
    dJ = np.zeros_like(J)
    Hk = np.zeros_like(J)
    dH = np.zeros_like(J)
    for i, z in enumerate(zs):
        J[i], dJ[i] = O.bessel(0, complex(z), L)
        Hk[i], dH[i] = O.bessel(1, complex(z), L)
    np.savez_compressed(os.path.join(HERE, "bessel_amos.npz"), z=zs, J=J, dJ=dJ, H=Hk, dH=dH)


def make_c1():
    """c1.npz: the C1 configuration at full size (bench.py's seeded N = 100
    cluster, nMax = 8, 16,000 unknowns, metal-like spheres in water), solved by
    the oracle's GMRES to a relative residual of 1e-13 on its own assembled S,
    once through each Bessel route: the reference's AMOS (`_amos`) and the
    oracle's recurrences (`_rec`, the route the GPU kernels also take). Near
    field at 2,048 points of the C1 grid (256 x 256 x 2 over [-1, 1] um^2 at
    z = +-0.1 nm), 64 of them inside spheres."""
    sys.path.insert(0, ROOT)
    import bench
    w = bench.WORKLOADS["c1"]
    xyz, rad = bench.cluster(w)
    cl = O.Cluster(xyz=xyz, radius=rad, eps=complex(w["index"]) ** 2, nmax=w["nmax"],
                   wavelength=w["lam"], bg_eps=complex(w["host"]) ** 2)
    grid = O.grid_points([-1000 * nm, 1000 * nm, 256, -1000 * nm, 1000 * nm, 256, -0.1 * nm, 0.1 * nm, 2])
    inside = np.zeros(len(grid), bool)
    for c, r in zip(xyz, rad):
        inside |= np.linalg.norm(grid - c, axis=1) <= r
    rng = np.random.default_rng(2026)
    pick = np.concatenate([rng.choice(np.nonzero(inside)[0], 64, replace=False),
                           rng.choice(np.nonzero(~inside)[0], 2048 - 64, replace=False)])
    pts = grid[np.sort(pick)]
    out = {}
    for route, amos in (("rec", False), ("amos", True)):
        if not O.use_amos(amos):
            raise SystemExit("the reference's AMOS build (oracle/_ref) is required")
        pr = O.Problem(cl)
        S = pr.scattering_matrix()
        Q = pr.source_vector()
        X, it, rr = O.gmres(S, Q, tol=1e-13, maxit=400, restarts=6)
        del S
        Xi = pr.internal(X)
        E, H = pr.near_field(X, Xi, pts)
        out.update({f"X_sca_{route}": X, f"xsec_{route}": pr.cross_sections(X), f"E_{route}": E,
                    f"H_{route}": H, f"Q_{route}": Q, f"gmres_{route}": np.array([it, rr])})
        print("c1", route, "iterations", it, "residual", rr, "xsec", out[f"xsec_{route}"])
    O.use_amos(False)
    np.savez_compressed(
        os.path.join(HERE, "c1.npz"), **out,
        xyz=cl.xyz, radius=cl.radius, eps=cl.eps, mu=cl.mu, eps_sh=cl.eps_sh,
        bg=np.array([cl.bg_eps, cl.bg_mu], np.complex128), nmax=cl.nmax,
        wavelength=cl.wavelength, angles=np.array([cl.theta, cl.phi]),
        pol=np.array([cl.e_theta, cl.e_phi], np.complex128), points=pts, inside=inside[np.sort(pick)])


def main():
    O.build(ref=True)
    if not O.use_amos(True):
        raise SystemExit("the reference's AMOS build (oracle/_ref) is required")
    if sys.argv[1:] == ["c1"]:
        make_c1()
        return
    bessel_table()
    for name, cl in cases().items():
        make(name, cl)
    O.use_amos(False)


if __name__ == "__main__":
    main()
