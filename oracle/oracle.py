"""ctypes loader for the CPU oracle (test infrastructure only).

The oracle restates OPTIMET-3D's sphere path (srcAna/) on the CPU; see
optimet_oracle.cpp for what each routine follows. Only tests/, the smoke check
and bench.py's CPU-baseline leg use this module. Parity status: pinned at the
Bessel layer against the reference's AMOS build (oracle/_ref) and by physics
identities; otherwise unpinned (the reference ships no golden vectors).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboptimet_oracle.so")
AMOS_PATH = os.path.join(HERE, "_ref", "libamos_ref.so")

_lib = None
_dp = C.POINTER(C.c_double)


def reference_tree():
    """The OPTIMET source tree named by $OPTIMET_REFERENCE when it holds the
    vendored AMOS sources (srcAna/amos.c), else None."""
    root = os.environ.get("OPTIMET_REFERENCE")
    if root and os.path.exists(os.path.join(root, "srcAna", "amos.c")):
        return root
    return None


def build(ref: bool = False) -> None:
    """Compile the oracle and, with ref and a reference tree in
    $OPTIMET_REFERENCE, the reference's own AMOS Bessel code."""
    root = reference_tree() if ref else None
    targets = ["port"] + (["ref", f"REFERENCE={root}"] if root else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_last_error.restype = C.c_char_p
        L.orc_problem_create.restype = C.c_void_p
        L.orc_problem_create.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double,
                                         C.c_double, C.c_double, _dp, _dp, C.c_int, _dp]
        L.orc_clg_tables.argtypes = [C.c_int, _dp]
        L.orc_wigner.argtypes = [C.c_int, C.POINTER(C.c_int)]
        L.orc_wigner.restype = C.c_double
        L.orc_sh_factors.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_sh_solve.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_sh_cross_sections.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
        for name in ("orc_problem_destroy",):
            getattr(L, name).argtypes = [C.c_void_p]
        for name in ("orc_inc_coeffs", "orc_source_vector", "orc_wave_numbers"):
            getattr(L, name).argtypes = [C.c_void_p, _dp]
        L.orc_tmatrix.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        L.orc_iaux.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_inc_local.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_scattering_matrix.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_internal.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_cross_sections.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_near_field.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp, _dp, _dp]
        L.orc_near_field_sh.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp, _dp]
        L.orc_aca_block.argtypes = [_dp, C.c_int, _dp, _dp, C.POINTER(C.c_int)]
        L.orc_aca_matrix.argtypes = [C.c_void_p, C.c_int, _dp, C.POINTER(C.c_int)]
        L.orc_wavelength_solve.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int,
                                           _dp, _dp, _dp, C.POINTER(C.c_int)]
        L.orc_lu_solve.argtypes = [C.c_int, _dp, _dp, _dp]
        L.orc_gmres.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                C.POINTER(C.c_int), _dp]
        L.orc_bessel.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp]
        L.orc_ynm.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp]
        L.orc_ta.argtypes = [C.c_double] * 5 + [C.c_int] * 5 + [_dp]
        L.orc_coupling.argtypes = [C.c_double] * 5 + [C.c_int, C.c_int, _dp, _dp]
        L.orc_to_spherical.argtypes = [C.c_double] * 3 + [_dp]
        L.orc_grid_points.argtypes = [_dp, _dp]
        L.orc_use_amos.argtypes = [C.c_char_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_assemble_pairs.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), _dp]
        L.orc_matvec.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _c(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def use_amos(on: bool = True) -> bool:
    """Route the oracle's Bessel layer through the reference's AMOS build."""
    L = lib()
    if not on:
        L.orc_use_amos(None)
        return True
    if not os.path.exists(AMOS_PATH):
        return False
    return L.orc_use_amos(AMOS_PATH.encode()) == 0


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def bessel(kind: int, z: complex, L: int):
    out = np.zeros(L + 1, np.complex128)
    dout = np.zeros(L + 1, np.complex128)
    rc = lib().orc_bessel(kind, z.real, z.imag, L, _p(out), _p(dout))
    if rc:
        raise RuntimeError(lib().orc_last_error().decode())
    return out, dout


def ynm(n, m, the, phi) -> complex:
    out = np.zeros(1, np.complex128)
    lib().orc_ynm(n, m, the, phi, _p(out))
    return complex(out[0])


def coupling(rel_sph, k: complex, nmax: int, regular: bool):
    P = nmax * (nmax + 2)
    A = np.zeros((P, P), np.complex128, order="F")
    B = np.zeros((P, P), np.complex128, order="F")
    r, t, ph = rel_sph
    lib().orc_coupling(r, t, ph, k.real, k.imag, nmax, int(regular), _p(A), _p(B))
    return A, B


def to_spherical(x, y, z):
    out = np.zeros(3)
    lib().orc_to_spherical(x, y, z, _p(out))
    return tuple(out)


@dataclass
class Cluster:
    """Spheres + medium + plane wave, in the units of the XML reader after
    conversion: metres, relative eps/mu, radians."""
    xyz: np.ndarray            # (N, 3) metres
    radius: np.ndarray         # (N,) metres
    eps: np.ndarray            # (N,) complex relative permittivity (FF)
    nmax: int
    wavelength: float          # metres
    mu: np.ndarray | None = None
    eps_sh: np.ndarray | None = None
    bg_eps: complex = 1.0
    bg_mu: complex = 1.0
    theta: float = 0.0
    phi: float = 0.0
    e_theta: complex = 1.0
    e_phi: complex = 0.0
    ksippp: complex = 0.0      # surface chi(2) perp-perp-perp (XML <ksippp>)
    ksiparppar: complex = 0.0  # surface chi(2) par-perp-par (XML <ksiparppar>)
    gamma: complex = 0.0       # bulk chi(2) (XML <gamma>)

    def __post_init__(self):
        self.xyz = np.ascontiguousarray(self.xyz, dtype=np.float64).reshape(-1, 3)
        n = self.xyz.shape[0]
        self.radius = np.ascontiguousarray(np.broadcast_to(self.radius, (n,)), dtype=np.float64)
        self.eps = _c(np.broadcast_to(self.eps, (n,)))
        self.mu = _c(np.ones(n) if self.mu is None else np.broadcast_to(self.mu, (n,)))
        self.eps_sh = _c(self.eps if self.eps_sh is None else np.broadcast_to(self.eps_sh, (n,)))
        chi = np.zeros((n, 3), np.complex128)
        chi[:, 0] = np.broadcast_to(self.ksippp, (n,))
        chi[:, 1] = np.broadcast_to(self.ksiparppar, (n,))
        chi[:, 2] = np.broadcast_to(self.gamma, (n,))
        self.chi = np.ascontiguousarray(chi)

    @property
    def n_spheres(self):
        return self.xyz.shape[0]

    @property
    def P(self):
        return self.nmax * (self.nmax + 2)

    @property
    def n_unknowns(self):
        return 2 * self.P * self.n_spheres


class Problem:
    """Oracle handle for one cluster at one wavelength (Geometry + Excitation)."""

    def __init__(self, cl: Cluster):
        L = lib()
        self.cl = cl
        bg = np.array([cl.bg_eps.real, complex(cl.bg_eps).imag, complex(cl.bg_mu).real,
                       complex(cl.bg_mu).imag])
        et = np.array([complex(cl.e_theta).real, complex(cl.e_theta).imag])
        ep = np.array([complex(cl.e_phi).real, complex(cl.e_phi).imag])
        self._keep = (bg, et, ep)
        h = L.orc_problem_create(cl.n_spheres, _p(cl.xyz), _p(cl.radius), _p(cl.eps.view(np.float64)),
                                 _p(cl.mu.view(np.float64)), _p(cl.eps_sh.view(np.float64)), _p(bg),
                                 cl.wavelength, cl.theta, cl.phi, _p(et), _p(ep), cl.nmax,
                                 _p(cl.chi.view(np.float64)))
        if not h:
            raise RuntimeError(L.orc_last_error().decode())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_problem_destroy(self.h)
            self.h = None

    @property
    def n(self):
        return self.cl.n_unknowns

    def wave_numbers(self):
        out = np.zeros(3)
        lib().orc_wave_numbers(self.h, _p(out))
        return complex(out[0], out[1]), out[2]

    def inc_coeffs(self):
        out = np.zeros(2 * self.cl.P, np.complex128)
        lib().orc_inc_coeffs(self.h, _p(out))
        return out

    def tmatrix(self, j, sh=False):
        out = np.zeros(2 * self.cl.P, np.complex128)
        lib().orc_tmatrix(self.h, j, int(sh), _p(out))
        return out

    def iaux(self, j):
        out = np.zeros(2 * self.cl.P, np.complex128)
        lib().orc_iaux(self.h, j, _p(out))
        return out

    def inc_local(self, j):
        out = np.zeros(2 * self.cl.P, np.complex128)
        lib().orc_inc_local(self.h, j, _p(out))
        return out

    def source_vector(self):
        out = np.zeros(self.n, np.complex128)
        if lib().orc_source_vector(self.h, _p(out)):
            raise RuntimeError(lib().orc_last_error().decode())
        return out

    def scattering_matrix(self, sh=False):
        S = np.zeros((self.n, self.n), np.complex128, order="F")
        if lib().orc_scattering_matrix(self.h, int(sh), _p(S)):
            raise RuntimeError(lib().orc_last_error().decode())
        return S

    def internal(self, sca):
        sca = _c(sca)
        out = np.zeros_like(sca)
        lib().orc_internal(self.h, _p(sca), _p(out))
        return out

    def cross_sections(self, sca):
        """(C_ext, C_sca, C_ext - C_sca, C_abs via Mie) in m^2."""
        sca = _c(sca)
        out = np.zeros(4)
        lib().orc_cross_sections(self.h, _p(sca), _p(out))
        return out

    def near_field(self, sca, intc, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        sca, intc = _c(sca), _c(intc)
        E = np.zeros((xyz.shape[0], 3), np.complex128)
        H = np.zeros_like(E)
        if lib().orc_near_field(self.h, _p(sca), _p(intc), xyz.shape[0], _p(xyz), _p(E), _p(H)):
            raise RuntimeError(lib().orc_last_error().decode())
        return E, H

    def aca_matrix(self, sh=False):
        """Scattering matrix with the admissible blocks replaced by their ACA
        products (dense), and the block ranks (N x N: -2 diagonal, -1 dense)."""
        n = self.n
        S = np.zeros((n, n), np.complex128, order="F")
        ranks = np.zeros(self.cl.n_spheres ** 2, np.int32)
        if lib().orc_aca_matrix(self.h, int(sh), _p(S), ranks.ctypes.data_as(C.POINTER(C.c_int))):
            raise RuntimeError(lib().orc_last_error().decode())
        return S, ranks.reshape(self.cl.n_spheres, self.cl.n_spheres)

    def near_field_sh(self, tables, x_int, x_sca_sh, x_int_sh, xyz):
        """Second-harmonic E, H (3 complex per point) at Cartesian points."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        E = np.zeros((xyz.shape[0], 3), np.complex128)
        H = np.zeros_like(E)
        if lib().orc_near_field_sh(self.h, _p(tables), _p(_c(x_int)), _p(_c(x_sca_sh)),
                                   _p(_c(x_int_sh)), xyz.shape[0], _p(xyz), _p(E), _p(H)):
            raise RuntimeError(lib().orc_last_error().decode())
        return E, H

    def sh_factors(self, j):
        """T1_outer, T2_outer, IauxSH1, IauxSH2 of sphere j (2P each)."""
        out = np.zeros(8 * self.cl.P, np.complex128)
        lib().orc_sh_factors(self.h, j, _p(out))
        return out.reshape(4, 2 * self.cl.P)

    def sh_solve(self, tables, x_int):
        """SH half of the solve: (K, K1ana, X_sca_SH, X_int_SH)."""
        x_int = _c(x_int)
        outs = [np.zeros(self.n, np.complex128) for _ in range(4)]
        rc = lib().orc_sh_solve(self.h, _p(tables), _p(x_int), *[_p(o) for o in outs])
        if rc:
            raise RuntimeError(lib().orc_last_error().decode())
        return outs

    def sh_cross_sections(self, tables, x_int, x_sca_sh, x_int_sh):
        """(C_sca_SH, C_abs_SH) as Result::getScatteringCrossSection_SH / getAbsorptionCrossSection_SH."""
        out = np.zeros(2)
        rc = lib().orc_sh_cross_sections(self.h, _p(tables), _p(_c(x_int)), _p(_c(x_sca_sh)),
                                         _p(_c(x_int_sh)), _p(out))
        if rc:
            raise RuntimeError(lib().orc_last_error().decode())
        return out

    def wavelength_solve(self, method="lu", tol=1e-10, maxit=1000, restarts=4):
        xsec = np.zeros(4)
        xs = np.zeros(self.n, np.complex128)
        xi = np.zeros(self.n, np.complex128)
        it = C.c_int(0)
        rc = lib().orc_wavelength_solve(self.h, {"lu": 0, "gmres": 1, "qr": 2}[method], tol, maxit, restarts,
                                        _p(xsec), _p(xs), _p(xi), C.byref(it))
        if rc < 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return xsec, xs, xi, it.value


def max_threads() -> int:
    return int(lib().orc_max_threads())


def assemble_pairs(pr: Problem, pairs):
    """Off-diagonal blocks S_ij (i != j) for the given (i, j) pairs: the
    assembly's timing sample, and sampled parity at sizes where the full S is
    too large. The library writes each block column-major, so the C-ordered
    buffer is returned transposed back to S's orientation."""
    pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
    n2 = 2 * pr.cl.P
    out = np.zeros((pairs.shape[0], n2, n2), np.complex128)
    rc = lib().orc_assemble_pairs(pr.h, pairs.shape[0], pairs.ctypes.data_as(C.POINTER(C.c_int)),
                                  _p(out))
    if rc:
        raise RuntimeError(lib().orc_last_error().decode())
    return out.transpose(0, 2, 1)


def matvec(A, x):
    A = np.asfortranarray(A, dtype=np.complex128)
    x = _c(x)
    y = np.zeros(A.shape[0], np.complex128)
    lib().orc_matvec(A.shape[0], A.shape[1], _p(A), _p(x), _p(y))
    return y


def clg_tables(nmax: int) -> np.ndarray:
    """The nine SH coupling tables (9, P, P, P): C_10m1, C_11m1, C_00m1, C_01m1,
    W_m1m1, W_11, W_00, W_10, W_01, indexed [k][p][q]."""
    P = nmax * (nmax + 2)
    out = np.zeros(9 * P ** 3)
    lib().orc_clg_tables(nmax, _p(out))
    return out


def wigner(kind: int, *js) -> float:
    arr = (C.c_int * len(js))(*js)
    return float(lib().orc_wigner(kind, arr))


def lu_solve(A, b):
    A = np.asfortranarray(A, dtype=np.complex128)
    b = _c(b)
    x = np.zeros_like(b)
    rc = lib().orc_lu_solve(A.shape[0], _p(A), _p(b), _p(x))
    if rc:
        raise RuntimeError(f"singular matrix at column {rc}")
    return x


def qr_solve(A, b):
    """Column-pivoted Householder QR solve (the serial PreconditionedMatrix::solve role)."""
    A = np.asfortranarray(A, dtype=np.complex128)
    b = _c(b)
    x = np.zeros_like(b)
    rc = lib().orc_qr_solve(A.shape[0], _p(A), _p(b), _p(x))
    if rc:
        raise RuntimeError(f"rank-deficient matrix at column {rc}")
    return x


def gmres(A, b, tol=1e-10, maxit=240, restarts=2):
    A = np.asfortranarray(A, dtype=np.complex128)
    b = _c(b)
    x = np.zeros_like(b)
    it = C.c_int(0)
    rr = C.c_double(0)
    lib().orc_gmres(A.shape[0], _p(A), _p(b), _p(x), tol, maxit, restarts, C.byref(it),
                    C.byref(rr))
    return x, it.value, rr.value


def aca_block(M):
    """ACA_compression of one square block: (U kmax x r, V r x kmax, r)."""
    M = np.asfortranarray(M, dtype=np.complex128)
    k = M.shape[0]
    U = np.zeros(k * k, np.complex128)
    V = np.zeros(k * k, np.complex128)
    r = C.c_int(0)
    if lib().orc_aca_block(_p(M), k, _p(U), _p(V), C.byref(r)):
        raise RuntimeError(lib().orc_last_error().decode())
    r = r.value
    return U[:k * r].reshape(r, k).T, V[:k * r].reshape(r, k), r


def grid_points(params):
    params = np.ascontiguousarray(params, dtype=np.float64)
    n = int(params[2]) * int(params[5]) * int(params[8])
    out = np.zeros((n, 3))
    lib().orc_grid_points(_p(params), _p(out))
    return out
