"""CPU tests of the oracle: pinned against the reference's AMOS build (when the
reference tree is present), against the committed golden fixtures, against
scipy, and against physics identities (rotation/translation invariance, energy
balance). No GPU."""
import glob
import os

import numpy as np
import pytest
from scipy import special as sp
from scipy.spatial.transform import Rotation

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
nm = 1e-9


def load_cluster(O, g):
    from helpers import oracle_cluster
    return oracle_cluster(O, g)


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_bessel_against_reference_amos_table(oracle):
    g = np.load(os.path.join(GOLDEN, "bessel_amos.npz"))
    for i, z in enumerate(g["z"]):
        J, dJ = oracle.bessel(0, complex(z), 25)
        H, dH = oracle.bessel(1, complex(z), 25)
        # AMOS loses relative accuracy next to zeros of j_n; compare against the
        # local scale of the sequence.
        scale = np.maximum(np.abs(g["J"][i]), 1e-3 * np.max(np.abs(g["J"][i])))
        assert np.max(np.abs(J - g["J"][i]) / scale) < 1e-11, z
        assert np.max(np.abs(H - g["H"][i]) / np.abs(g["H"][i])) < 1e-12, z
        assert np.max(np.abs(dH[1:] - g["dH"][i][1:]) / np.abs(g["dH"][i][1:])) < 1e-12, z


@pytest.mark.skipif(not os.environ.get("OPTIMET_REFERENCE")
                    or not os.path.exists(os.path.join(os.environ["OPTIMET_REFERENCE"], "srcAna", "amos.c")),
                    reason="OPTIMET_REFERENCE unset: the live AMOS pin runs where a reference tree is given")
def test_bessel_against_live_amos(oracle):
    oracle.build(ref=True)
    rng = np.random.default_rng(3)
    zs = list(rng.uniform(0.05, 90, 20)) + list(rng.uniform(0.1, 8, 10) + 1j * rng.uniform(0, 3, 10))
    for z in zs:
        z = complex(z)
        oracle.use_amos(False)
        a, _ = oracle.bessel(1, z, 24)
        oracle.use_amos(True)
        b, _ = oracle.bessel(1, z, 24)
        oracle.use_amos(False)
        assert rel(a, b) < 1e-12


def test_bessel_against_scipy(oracle):
    n = np.arange(21)
    for z in (0.3, 2.0, 9.7, 44.0):
        J, dJ = oracle.bessel(0, complex(z), 20)
        H, _ = oracle.bessel(1, complex(z), 20)
        assert rel(J, sp.spherical_jn(n, z)) < 1e-13
        assert rel(dJ[:-1], sp.spherical_jn(n, z, derivative=True)[:-1]) < 1e-12
        assert rel(H, sp.spherical_jn(n, z) + 1j * sp.spherical_yn(n, z)) < 1e-13
    # real-axis fix-up of Bessel.h: zero imaginary part for real arguments
    J, _ = oracle.bessel(0, 3.0 + 0j, 8)
    assert np.all(J.imag == 0)
    # zero-argument branch
    J, dJ = oracle.bessel(0, 0j, 4)
    assert J[0] == 1 and np.all(J[1:] == 0) and np.all(dJ == 0)


def test_spherical_harmonics_against_scipy(oracle):
    rng = np.random.default_rng(0)
    for n in range(0, 25):
        for m in range(-n, n + 1):
            t, p = rng.uniform(0.01, np.pi - 0.01), rng.uniform(-np.pi, np.pi)
            y = oracle.ynm(n, m, t, p)
            ys = sp.sph_harm_y(n, m, t, p)
            assert abs(y - ys) <= 1e-12 * max(abs(ys), 1e-3)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))))
def test_golden_fixture(oracle, path):
    if path.endswith("bessel_amos.npz"):
        pytest.skip("bessel table")
    if path.endswith("c1.npz"):
        pytest.skip("full-size C1 fixture: test_c1_fixture_routes")
    g = np.load(path)
    cl = load_cluster(oracle, g)
    pr = oracle.Problem(cl)
    assert rel(pr.inc_coeffs(), g["inc"]) < 1e-12
    for j in range(cl.n_spheres):
        assert rel(pr.tmatrix(j), g["T"][j]) < 1e-11
        assert rel(pr.tmatrix(j, sh=True), g["T_sh"][j]) < 1e-11
    k, _ = pr.wave_numbers()
    A, B = oracle.coupling(g["rel"], k, cl.nmax, True)
    assert rel(A, g["A_irr"]) < 1e-11 and rel(B, g["B_irr"]) < 1e-11
    A, B = oracle.coupling(g["rel"], k, cl.nmax, False)
    assert rel(A, g["A_reg"]) < 1e-11 and rel(B, g["B_reg"]) < 1e-11
    Q = pr.source_vector()
    assert rel(Q, g["Q"]) < 1e-11
    S = pr.scattering_matrix()
    P = cl.P
    blk = (slice(0, 2 * P), slice(2 * P, 4 * P)) if cl.n_spheres > 1 else (slice(0, 2 * P),) * 2
    assert rel(S[blk], g["S_block"]) < 1e-11
    assert rel(pr.scattering_matrix(sh=True)[blk], g["S_sh_block"]) < 1e-11
    # Solution-level quantities. The fixture's Bessel values come from the
    # reference's AMOS and the oracle's from recurrences; measured differences
    # (x86-64 host, LU solve): X_sca 1e-15 to 3.6e-15, X_int (on the Iaux
    # scale) up to 1.8e-15, cross sections 3.7e-15 to 2.0e-14. The near field
    # evaluates Bessel functions at the field points as well: E up to 1.4e-12,
    # H up to 8.6e-11 (diel3), 4.5e-12 (c0), 2.4e-12 (pair_sh), 3e-15 (metal5,
    # single_sh). Bounds: 1e-13 for the solution and cross sections, the
    # measured near-field figure times about two.
    name = os.path.basename(path)[:-4]
    nf = {"c0": (1e-12, 1e-11), "diel3": (3e-12, 2e-10), "metal5": (1e-13, 1e-13),
          "pair_sh": (3e-13, 5e-12), "single_sh": (1e-13, 1e-13)}.get(name, (1e-10, 1e-10))
    X = oracle.lu_solve(S, Q)
    assert rel(X, g["X_sca"]) < 1e-13
    # Internal coefficients are X_sca times Iaux, whose high-order entries are
    # large (1/psi_n); errors are measured against that propagated scale.
    ia = np.concatenate([pr.iaux(j) for j in range(cl.n_spheres)])
    scale = np.abs(ia) * np.max(np.abs(g["X_sca"]))
    assert np.max(np.abs(pr.internal(X) - g["X_int"]) / scale) < 1e-13
    xs = pr.cross_sections(X)
    assert np.max(np.abs(xs - g["xsec"]) / np.abs(g["xsec"])) < 1e-13
    E, H = pr.near_field(X, pr.internal(X), g["points"])
    assert rel(E, g["E"]) < nf[0] and rel(H, g["H"]) < nf[1], (rel(E, g["E"]), rel(H, g["H"]))


def _solve(O, xyz, kdir, pol, nmax=5, eps=(2.0 + 0.1j) ** 2, radius=90 * nm):
    th = np.arccos(kdir[2])
    ph = np.arctan2(kdir[1], kdir[0])
    eth = np.array([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)])
    eph = np.array([-np.sin(ph), np.cos(ph), 0.0])
    cl = O.Cluster(xyz=xyz, radius=radius, eps=eps, nmax=nmax, wavelength=650 * nm, theta=th,
                   phi=ph, e_theta=pol @ eth, e_phi=pol @ eph)
    return O.Problem(cl).wavelength_solve("lu")[0]


def test_rotation_invariance_of_extinction(oracle):
    """Rotating spheres, incidence and polarisation together leaves C_ext and
    C_abs unchanged: pins the irregular and regular translation coefficients,
    the spherical harmonics and the T-matrices jointly."""
    pos = np.array([[0, 0, 0], [220, 30, -40], [-60, 210, 90]]) * nm
    k0 = np.array([0.3, -0.5, 0.8])
    k0 /= np.linalg.norm(k0)
    e0 = np.cross(k0, [0, 0, 1.0])
    e0 /= np.linalg.norm(e0)
    base = _solve(oracle, pos, k0, e0)
    R = Rotation.from_euler("zyz", [1.2, -0.3, 2.0]).as_matrix()
    rot = _solve(oracle, pos @ R.T, R @ k0, R @ e0)
    assert abs(rot[0] - base[0]) / abs(base[0]) < 1e-12
    assert abs(rot[3] - base[3]) / abs(base[3]) < 1e-12


def _wigner_small_d(n, theta):
    """d^n_{m' m}(theta) from the explicit sum (Wigner's formula), m', m = -n..n."""
    from math import factorial as f
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    d = np.zeros((2 * n + 1, 2 * n + 1))
    for mp in range(-n, n + 1):
        for m in range(-n, n + 1):
            tot = 0.0
            for k in range(0, 2 * n + 1):
                a, b, cc, dd = n + m - k, k, n - k - mp, k - m + mp
                if min(a, b, cc, dd) < 0:
                    continue
                tot += ((-1) ** (k - m + mp) * c ** (2 * n + m - mp - 2 * k) * s ** (2 * k - m + mp)
                        / (f(a) * f(b) * f(cc) * f(dd)))
            d[mp + n, m + n] = tot * np.sqrt(float(f(n + mp) * f(n - mp) * f(n + m) * f(n - m)))
    return d


@pytest.mark.parametrize("nmax,R", [(4, (300 * nm, 1.1, 0.7)), (6, (450 * nm, 2.6, -2.2)),
                                    (8, (260 * nm, 0.35, 4.0))])
def test_coupling_is_a_rotated_z_axis_translation(oracle, nmax, R):
    """A(R) = U A(|R| z) U^H and B(R) = U B(|R| z) U^H, U block-diagonal over
    the degree n with U[p(n, m'), p(n, m)] = d^n_{m' m}(theta) e^{i m' phi},
    and the z-axis blocks diagonal in m: an identity independent of the
    Stout recurrences, for both Bessel kinds (the rotation-based form of the
    translation, point-and-shoot)."""
    k = complex(2 * np.pi / 600e-9)
    P = nmax * (nmax + 2)
    U = np.zeros((P, P), complex)
    for n in range(1, nmax + 1):
        d = _wigner_small_d(n, R[1])
        for mp in range(-n, n + 1):
            for m in range(-n, n + 1):
                U[n * (n + 1) - mp - 1, n * (n + 1) - m - 1] = d[mp + n, m + n] * np.exp(1j * mp * R[2])
    mof = np.array([m for n in range(1, nmax + 1) for m in range(n, -n - 1, -1)])
    for regular in (False, True):
        A, B = oracle.coupling(R, k, nmax, regular)
        Az, Bz = oracle.coupling((R[0], 0.0, 0.0), k, nmax, regular)
        assert np.max(np.abs(Az[mof[:, None] != mof[None, :]])) == 0.0
        assert np.max(np.abs(Bz[mof[:, None] != mof[None, :]])) == 0.0
        scale = np.max(np.abs(A))
        assert np.max(np.abs(U @ Az @ U.conj().T - A)) / scale < 1e-12
        assert np.max(np.abs(U @ Bz @ U.conj().T - B)) / scale < 1e-12


def test_scattering_matrix_from_rotated_translations(oracle):
    """The oracle's S (PreconditionedMatrix.cpp:369-397) block by block from
    the rotated form: S_ij = -T_i [A^T B^T; B^T A^T] with A, B the coupling of
    r_i - r_j (the reference's inverted `regular` flag set) and
    A = U A(|R| z) U^H, B = U B(|R| z) U^H. Pins the layout, the transposes
    and the T scaling that a rotation-based assembly has to reproduce."""
    nmax = 4
    P = nmax * (nmax + 2)
    xyz = np.array([[0, 0, 0], [220, 30, -40], [-60, 210, 90]]) * nm
    cl = oracle.Cluster(xyz=xyz, radius=np.array([60, 50, 70]) * nm, eps=(2.0 + 0.05j) ** 2, nmax=nmax,
                        wavelength=650 * nm)
    pr = oracle.Problem(cl)
    S = pr.scattering_matrix()
    k0, _ = pr.wave_numbers()
    for i in range(3):
        for j in range(3):
            blk = S[2 * P * i:2 * P * (i + 1), 2 * P * j:2 * P * (j + 1)]
            if i == j:
                assert np.array_equal(blk, np.eye(2 * P))
                continue
            r, th, ph = oracle.to_spherical(*(xyz[i] - xyz[j]))
            U = np.zeros((P, P), complex)
            for n in range(1, nmax + 1):
                d = _wigner_small_d(n, th)
                for mp in range(-n, n + 1):
                    for m in range(-n, n + 1):
                        U[n * (n + 1) - mp - 1, n * (n + 1) - m - 1] = d[mp + n, m + n] * np.exp(1j * mp * ph)
            Az, Bz = oracle.coupling((r, 0.0, 0.0), k0, nmax, True)
            A, B = U @ Az @ U.conj().T, U @ Bz @ U.conj().T
            got = -pr.tmatrix(i)[:, None] * np.block([[A.T, B.T], [B.T, A.T]])
            assert np.max(np.abs(got - blk)) / np.max(np.abs(blk)) < 1e-12


def test_translation_convergence_single_sphere(oracle):
    k0 = np.array([0.3, -0.5, 0.8])
    k0 /= np.linalg.norm(k0)
    e0 = np.cross(k0, [0, 0, 1.0])
    e0 /= np.linalg.norm(e0)
    a = _solve(oracle, np.zeros((1, 3)), k0, e0, nmax=12)
    b = _solve(oracle, np.array([[80 * nm, -50 * nm, 60 * nm]]), k0, e0, nmax=12)
    assert abs(b[0] - a[0]) / abs(a[0]) < 1e-11


def test_single_sphere_energy_balance(oracle):
    cl = oracle.Cluster(xyz=[[0, 0, 0]], radius=100 * nm, eps=(3.5 + 0.01j) ** 2, nmax=6,
                        wavelength=600 * nm)
    xs = oracle.Problem(cl).wavelength_solve("lu")[0]
    assert abs(xs[0] - xs[1] - xs[3]) / xs[0] < 1e-12


def test_axial_incidence_parity_trap(oracle):
    """Incidence exactly along +z: the reference nudges theta after reflecting
    negative m, so its x-polarised wave expands as i * y-polarised. The oracle
    reproduces that (VIGdVIG, AuxCoefficients.cpp:217-240)."""
    cl = oracle.Cluster(xyz=[[900 * nm, 0, 0]], radius=10 * nm, eps=2.0, nmax=12,
                        wavelength=600 * nm)
    pr = oracle.Problem(cl)
    p = np.array([[30 * nm, 20 * nm, -50 * nm]])
    E, _ = pr.near_field(np.zeros(pr.n), np.zeros(pr.n), p)
    k = 2 * np.pi / (600 * nm)
    expect = 1j * np.array([0, 1, 0]) * np.exp(1j * k * p[0, 2])
    assert np.max(np.abs(E[0] - expect)) < 1e-4  # the 1e-6 theta nudge itself


def test_gmres_matches_lu(oracle):
    g = np.load(os.path.join(GOLDEN, "metal5.npz"))
    pr = oracle.Problem(load_cluster(oracle, g))
    S, Q = pr.scattering_matrix(), pr.source_vector()
    x, it, rr = oracle.gmres(S, Q, tol=1e-13, maxit=400, restarts=3)
    assert rr <= 1e-13 and it > 0
    assert rel(x, oracle.lu_solve(S, Q)) < 1e-10


def test_overlap_rejected(oracle):
    cl = oracle.Cluster(xyz=[[0, 0, 0], [0, 0, 150 * nm]], radius=100 * nm, eps=2.0, nmax=2,
                        wavelength=600 * nm)
    with pytest.raises(RuntimeError, match="overlaps"):
        oracle.Problem(cl)


def test_thread_count_does_not_change_results(oracle):
    g = np.load(os.path.join(GOLDEN, "diel3.npz"))
    pr = oracle.Problem(load_cluster(oracle, g))
    oracle.set_threads(1)
    a = pr.wavelength_solve("lu")[0]
    oracle.set_threads(4)
    b = pr.wavelength_solve("lu")[0]
    oracle.set_threads(1)
    assert np.array_equal(a, b)


def _w_table_entry_sympy(J1, M1, J2, M2, J, M, L1, L2):
    """Symbol.cpp's W(L1, J1, M1, L2, J2, M2, L, M) from sympy's exact symbols."""
    from sympy.physics.wigner import wigner_3j, wigner_6j

    def cg(j, m, j1, m1, j2, m2):
        return (-1.0) ** int(m + j1 - j2) * np.sqrt(2 * j + 1) * float(wigner_3j(j1, j2, j, m1, m2, -m))

    return ((-1.0) ** int(J2 + L1 + J) * np.sqrt((2 * J1 + 1) * (2 * J2 + 1) * (2 * L1 + 1) * (2 * L2 + 1)
                                             / (4 * np.pi * (2 * J + 1)))
            * float(wigner_6j(L1, L2, J, J2, J1, 1)) * cg(J, 0, L1, 0, L2, 0) * cg(J, M, J1, M1, J2, M2))


def test_sh_tables_against_sympy(oracle):
    """W_00 and W_10 entries of the SH coupling tables against sympy's exact Wigner symbols."""
    nmax = 3
    P = nmax * (nmax + 2)
    tab = oracle.clg_tables(nmax).reshape(9, P, P, P)

    def nm(p):
        n = int(np.sqrt(p + 1.0))
        return n, -(p + 1) + n * (n + 1)

    rng = np.random.default_rng(4)
    checked = 0
    for _ in range(60):
        k, p, q = rng.integers(0, P, 3)
        J, M = nm(k)
        J1, M1 = nm(p)
        J2, M2 = nm(q)
        if M != M1 + M2:
            assert tab[6, k, p, q] == 0.0
            continue
        w00 = _w_table_entry_sympy(J1, M1, J2, M2, J, M, J1, J2)
        assert abs(tab[6, k, p, q] - w00) < 1e-13 * max(1.0, abs(w00))
        a1, b1 = np.sqrt(J1 / (2 * J1 + 1)), np.sqrt((J1 + 1) / (2 * J1 + 1))
        w10 = b1 * _w_table_entry_sympy(J1, M1, J2, M2, J, M, J1 - 1, J2) + \
            a1 * _w_table_entry_sympy(J1, M1, J2, M2, J, M, J1 + 1, J2)
        assert abs(tab[7, k, p, q] - w10) < 1e-13 * max(1.0, abs(w10))
        checked += 1
    assert checked > 5


@pytest.mark.parametrize("name", ["single_sh", "pair_sh"])
def test_sh_golden(oracle, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    cl = load_cluster(oracle, g)
    pr = oracle.Problem(cl)
    tab = oracle.clg_tables(cl.nmax)
    if "clg" in g.files:
        assert np.max(np.abs(tab - g["clg"])) < 1e-13
    for j in range(cl.n_spheres):
        assert rel(pr.sh_factors(j), g["sh_factors"][j]) < 1e-11
    S, Q = pr.scattering_matrix(), pr.source_vector()
    X = oracle.lu_solve(S, Q)
    Xi = pr.internal(X)
    K, K1, Xs, Xis = pr.sh_solve(tab, Xi)
    # measured against the AMOS-route fixtures: single_sh 2e-15 to 1.1e-14 on
    # every quantity; pair_sh K 1.0e-13, K1ana 2.3e-13, X_sca_SH 1.1e-13,
    # X_int_SH 3.9e-13, cross sections 5.1e-14, E 6.3e-13, H 2.1e-13
    tol = 1e-13 if name == "single_sh" else 1e-12
    for a, b in ((K, g["K"]), (K1, g["K1ana"]), (Xs, g["X_sca_SH"]), (Xis, g["X_int_SH"])):
        assert rel(a, b) < tol
    xs = pr.sh_cross_sections(tab, Xi, Xs, Xis)
    assert np.max(np.abs(xs - g["xsec_sh"]) / np.abs(g["xsec_sh"])) < tol
    E, H = pr.near_field_sh(tab, Xi, Xs, Xis, g["points"])
    assert rel(E, g["E_sh"]) < 2 * tol and rel(H, g["H_sh"]) < 2 * tol


def test_sh_single_sphere_rotation_invariance(oracle):
    """Single sphere at the origin, surface chi(2) only: both SH cross sections
    are rotation invariant (pins the coupling tables and the SH factors). With
    two spheres the reference's source, built from conj(X_int), is not rotation
    covariant, so no such identity holds there."""
    def run(kdir, pol):
        th = np.arccos(kdir[2])
        ph = np.arctan2(kdir[1], kdir[0])
        eth = np.array([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)])
        eph = np.array([-np.sin(ph), np.cos(ph), 0.0])
        cl = oracle.Cluster(xyz=np.zeros((1, 3)), radius=80 * nm, eps=(2.0 + 0.1j) ** 2,
                            eps_sh=(2.2 + 0.15j) ** 2, nmax=4, wavelength=800 * nm, theta=th, phi=ph,
                            e_theta=pol @ eth, e_phi=pol @ eph, ksippp=1.0, ksiparppar=0.25)
        pr = oracle.Problem(cl)
        _, X, Xi, _ = pr.wavelength_solve("lu")
        tab = oracle.clg_tables(4)
        K, K1, Xs, Xis = pr.sh_solve(tab, Xi)
        return pr.sh_cross_sections(tab, Xi, Xs, Xis)
    k0 = np.array([0.3, -0.5, 0.8])
    k0 /= np.linalg.norm(k0)
    e0 = np.cross(k0, [0, 0, 1.0])
    e0 /= np.linalg.norm(e0)
    R = Rotation.from_euler("zyz", [1.2, -0.3, 2.0]).as_matrix()
    a, b = run(k0, e0), run(R @ k0, R @ e0)
    assert np.max(np.abs(a - b) / np.abs(a)) < 1e-12


def test_c1_fixture_routes(oracle):
    """The full-size C1 fixture (16,000 unknowns): the source vector and a
    sample of S blocks from the live oracle against the fixture's recurrence
    route, and the two Bessel routes' solutions against each other. The
    difference between the routes is what the reference's AMOS arithmetic does
    to the solution through the conditioning of S; the GPU is compared with
    both in tests/test_parity_scale.py."""
    g = np.load(os.path.join(GOLDEN, "c1.npz"))
    cl = load_cluster(oracle, g)
    pr = oracle.Problem(cl)
    assert rel(pr.source_vector(), g["Q_rec"]) < 1e-13
    assert rel(g["Q_amos"], g["Q_rec"]) < 5e-14
    assert g["gmres_rec"][1] <= 1e-13 and g["gmres_amos"][1] <= 1e-13
    # measured between the routes: Q 1.1e-14, X_sca 1.2e-14, cross sections
    # 4.2e-15, E 1.2e-14, H 1.1e-14 (both GMRES runs stop at 7.1e-14, 70 iterations)
    assert rel(g["X_sca_amos"], g["X_sca_rec"]) < 5e-14
    assert np.max(np.abs(g["xsec_amos"] - g["xsec_rec"]) / np.abs(g["xsec_rec"])) < 2e-14
    assert rel(g["E_amos"], g["E_rec"]) < 5e-14 and rel(g["H_amos"], g["H_rec"]) < 5e-14


def test_qr_solve_matches_lu(oracle):
    """The serial solver role (column-pivoted Householder QR) against the LU
    on the C0 fixture's matrix and a random complex system."""
    g = np.load(os.path.join(GOLDEN, "c0.npz"))
    S = g["S_full"]
    x_qr = oracle.qr_solve(S, g["Q"])
    assert rel(x_qr, oracle.lu_solve(S, g["Q"])) < 1e-13
    rng = np.random.default_rng(4)
    A = rng.standard_normal((60, 60)) + 1j * rng.standard_normal((60, 60))
    b = rng.standard_normal(60) + 1j * rng.standard_normal(60)
    assert rel(oracle.qr_solve(A, b), np.linalg.solve(A, b)) < 1e-12
    pr = oracle.Problem(load_cluster(oracle, g))
    xs_qr = pr.wavelength_solve("qr")[0]
    xs_lu = pr.wavelength_solve("lu")[0]
    assert np.max(np.abs(xs_qr - xs_lu) / np.abs(xs_lu)) < 1e-13

