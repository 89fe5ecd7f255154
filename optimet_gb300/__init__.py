"""optimet_gb300: GB300-native OPTIMET-3D sphere path (T-matrix multiple
scattering) behind the C ABI of include/optimet_gpu.h.

Low level: ``Context``, ``Problem``, ``coupling`` and ``wavelength_solve`` wrap
the C entry points one to one. The reference's own interface (Geometry,
Scatterer, Excitation, solver.factory, Result, simulation_input) is mirrored
in :mod:`optimet_gb300.optimet`.

The library must be built for sm_103a (``python -m optimet_gb300.build``);
there is no CPU fallback: loading fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboptimet_gpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "optimet_gpu.h")

OK, ERR_INVALID, ERR_OVERLAP, ERR_CUDA, ERR_BUDGET, ERR_NOT_CONVERGED, ERR_SINGULAR, ERR_STATE, PENDING = range(9)
FF, SH = 0, 1
C128, C64, ACA = 0, 1, 2
SOLVE_LU, SOLVE_GMRES, SOLVE_FGMRES_MIXED, SOLVE_LU_MIXED = 0, 1, 2, 3

ERROR_NAMES = {ERR_INVALID: "invalid argument", ERR_OVERLAP: "overlapping spheres",
               ERR_CUDA: "CUDA failure", ERR_BUDGET: "device-memory budget exceeded",
               ERR_NOT_CONVERGED: "not converged", ERR_SINGULAR: "singular matrix",
               ERR_STATE: "call out of order"}


class OptimetError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


class Sphere(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("radius", C.c_double),
                ("eps_r", C.c_double * 2), ("mu_r", C.c_double * 2), ("eps_r_sh", C.c_double * 2),
                ("ksippp", C.c_double * 2), ("ksiparppar", C.c_double * 2), ("gamma", C.c_double * 2),
                ("nmax", C.c_int), ("reserved", C.c_int)]


class Medium(C.Structure):
    _fields_ = [("eps_r", C.c_double * 2), ("mu_r", C.c_double * 2)]


class PlaneWave(C.Structure):
    _fields_ = [("wavelength", C.c_double), ("theta", C.c_double), ("phi", C.c_double),
                ("e_theta", C.c_double * 2), ("e_phi", C.c_double * 2), ("sh", C.c_int),
                ("reserved", C.c_int)]


class SolveOptions(C.Structure):
    _fields_ = [("method", C.c_int), ("max_iter", C.c_int), ("restarts", C.c_int),
                ("inner_iter", C.c_int), ("tol", C.c_double), ("inner_tol", C.c_double)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("inner_iterations", C.c_int),
                ("rel_residual", C.c_double), ("seconds", C.c_double)]


class Tuning(C.Structure):
    _fields_ = [("matvec_ctas_per_sm", C.c_int), ("matvec_df_ctas_per_sm", C.c_int),
                ("assemble_carveout", C.c_int), ("matvec_carveout", C.c_int),
                ("lu_tensor_cores", C.c_int), ("matvec_tma", C.c_int),
                ("assemble_rotation", C.c_int), ("lu_persistent", C.c_int), ("batch_tiles", C.c_int),
                ("batch_fused", C.c_int), ("inner_half", C.c_int)]


class Request(C.Structure):
    _fields_ = [("spheres", C.POINTER(Sphere)), ("n_spheres", C.c_int), ("precision", C.c_int),
                ("background", Medium), ("wave", PlaneWave), ("opts", SolveOptions),
                ("cluster_key", C.c_ulonglong)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("slot", C.c_int), ("xsec", C.c_double * 4),
                ("xsec_sh", C.c_double * 2), ("ff", SolveStats), ("sh", SolveStats),
                ("queue_ms", C.c_double), ("service_ms", C.c_double), ("latency_ms", C.c_double),
                ("device_bytes", C.c_size_t)]


_lib = None
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


def lib():
    """Load liboptimet_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m optimet_gb300.build`")
        L = C.CDLL(LIB_PATH)
        vp, pvp = C.c_void_p, C.POINTER(C.c_void_p)
        L.om_context_create.argtypes = [C.c_int, C.c_size_t, pvp]
        L.om_context_destroy.argtypes = [vp]
        L.om_context_last_error.argtypes = [vp]
        L.om_context_last_error.restype = C.c_char_p
        L.om_context_last_launches.argtypes = [vp]
        L.om_context_synchronize.argtypes = [vp]
        L.om_context_timers.argtypes = [vp, C.c_int, _dp]
        L.om_context_lu_timers.argtypes = [vp, _dp]
        L.om_context_inner_timers.argtypes = [vp, _dp]
        L.om_batch_tiles.argtypes = [vp, C.POINTER(C.c_int), C.c_int]
        L.om_context_mark.argtypes = [vp, _dp]
        L.om_context_tune.argtypes = [vp, C.POINTER(Tuning)]
        L.om_aca_info.argtypes = [vp, C.c_int, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp,
                                  C.POINTER(C.c_int)]
        L.om_matvec_inner_c64.argtypes = [vp, C.c_long, _fp, _fp, _fp, C.c_int]
        L.om_cgemm_sub_c64.argtypes = [vp, C.c_long, C.c_long, C.c_int, _fp, C.c_long, _fp,
                                       C.c_long, _fp, C.c_long]
        L.om_problem_create.argtypes = [vp, C.POINTER(Sphere), C.c_int, C.POINTER(Medium),
                                        C.POINTER(PlaneWave), pvp]
        L.om_problem_destroy.argtypes = [vp]
        L.om_problem_set_wavelength.argtypes = [vp, C.c_double]
        L.om_problem_size.argtypes = [vp]
        L.om_problem_size.restype = C.c_long
        L.om_coupling.argtypes = [vp, _dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, _dp, _dp]
        L.om_tmatrix.argtypes = [vp, C.c_int, _dp]
        L.om_incident_coefficients.argtypes = [vp, _dp]
        L.om_assemble.argtypes = [vp, C.c_int, C.c_int]
        L.om_copy_matrix.argtypes = [vp, C.c_int, _dp]
        L.om_source_vector.argtypes = [vp, _dp]
        L.om_solve.argtypes = [vp, C.POINTER(SolveOptions), C.POINTER(SolveStats)]
        L.om_solve_rhs.argtypes = [vp, C.c_int, C.POINTER(SolveOptions), _dp, _dp,
                                   C.POINTER(SolveStats)]
        L.om_get_coefficients.argtypes = [vp, _dp, _dp]
        L.om_assemble_rows.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.om_matvec_rows.argtypes = [vp, C.c_int, vp, vp]
        L.om_cross_sections.argtypes = [vp, _dp]
        L.om_near_field.argtypes = [vp, _dp, C.c_int, _dp, _dp]
        L.om_near_field_sh.argtypes = [vp, _dp, C.c_int, _dp, _dp]
        L.om_wavelength_solve.argtypes = [vp, C.POINTER(Sphere), C.c_int, C.POINTER(Medium),
                                          C.POINTER(PlaneWave), C.POINTER(SolveOptions), C.c_int,
                                          _dp, _dp, _dp, C.POINTER(SolveStats)]
        L.om_wavelength_solve_sh.argtypes = [vp, C.POINTER(Sphere), C.c_int, C.POINTER(Medium),
                                             C.POINTER(PlaneWave), C.POINTER(SolveOptions),
                                             C.c_int, _dp, _dp, C.POINTER(SolveStats)]
        L.om_solve_sh.argtypes = [vp, C.POINTER(SolveOptions), C.POINTER(SolveStats)]
        L.om_get_sh_vectors.argtypes = [vp, _dp, _dp, _dp, _dp]
        L.om_sh_cross_sections.argtypes = [vp, _dp]
        L.om_clg_tables.argtypes = [vp, C.c_int, _dp]
        L.om_problem_set_wave.argtypes = [vp, C.POINTER(PlaneWave)]
        L.om_server_create.argtypes = [C.c_int, C.c_size_t, C.c_int, pvp]
        L.om_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_ulonglong)]
        L.om_server_poll.argtypes = [vp, C.c_ulonglong, C.c_int, C.POINTER(Result)]
        L.om_server_drain.argtypes = [vp]
        L.om_server_tune.argtypes = [vp, C.POINTER(Tuning)]
        L.om_server_autotune.argtypes = [vp, C.POINTER(Request), C.c_int, C.c_double,
                                         C.POINTER(Tuning)]
        L.om_server_mark.argtypes = [vp, _dp]
        L.om_server_launches.argtypes = [vp]
        L.om_server_launches.restype = C.c_long
        L.om_server_last_error.argtypes = [vp]
        L.om_server_last_error.restype = C.c_char_p
        L.om_server_destroy.argtypes = [vp]
        L.om_server_batching.argtypes = [vp, C.c_int, C.c_size_t, C.c_size_t]
        L.om_batch_solve.argtypes = [vp, C.POINTER(Request), C.c_int, C.c_size_t, C.POINTER(Result)]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def options(method=SOLVE_GMRES, tol=1e-10, max_iter=200, restarts=10, inner_iter=40,
            inner_tol=1e-4) -> SolveOptions:
    return SolveOptions(method, max_iter, restarts, inner_iter, tol, inner_tol)


class Context:
    """One GPU, one stream, an optional device-memory budget in bytes."""

    def __init__(self, device: int = 0, budget: int = 0):
        h = C.c_void_p()
        rc = lib().om_context_create(device, budget, C.byref(h))
        if rc:
            raise OptimetError(rc, "cannot create a CUDA context on device %d" % device)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().om_context_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def check(self, rc):
        if rc not in (OK,):
            raise OptimetError(rc, lib().om_context_last_error(self.h).decode())
        return rc

    def synchronize(self):
        self.check(lib().om_context_synchronize(self.h))

    def mark(self) -> float:
        """Device milliseconds since the previous mark (CUDA events on the stream)."""
        out = np.zeros(1)
        self.check(lib().om_context_mark(self.h, _p(out)))
        return float(out[0])

    def tune(self, matvec_ctas_per_sm=0, matvec_df_ctas_per_sm=0, assemble_carveout=-1,
             matvec_carveout=-1, lu_tensor_cores=-1, matvec_tma=-1, assemble_rotation=-1, lu_persistent=-1, batch_tiles=-1,
             batch_fused=-1, inner_half=-1):
        """Launch tuning (om_context_tune); 0 / -1 keep the current value."""
        t = Tuning(matvec_ctas_per_sm, matvec_df_ctas_per_sm, assemble_carveout, matvec_carveout,
                   lu_tensor_cores, matvec_tma, assemble_rotation, lu_persistent, batch_tiles,
                   batch_fused, inner_half)
        self.check(lib().om_context_tune(self.h, C.byref(t)))

    def timers(self, enable=True):
        """Kernel times since the last call: dict of (milliseconds, launches)."""
        out = np.zeros(8)
        self.check(lib().om_context_timers(self.h, int(enable), _p(out)))
        return {"assemble": (out[0], int(out[1])), "matvec_c128": (out[2], int(out[3])),
                "matvec_c64": (out[4], int(out[5])), "matvec_c64_df": (out[6], int(out[7]))}

    def inner_timers(self):
        """Inner FP32 GMRES products of the precision form since the last
        call (recorded while timers() is on): dict of (milliseconds, launches)
        for the products on the bf16 copy and those that write it."""
        out = np.zeros(4)
        self.check(lib().om_context_inner_timers(self.h, _p(out)))
        return {"bf16": (out[0], int(out[1])), "copy": (out[2], int(out[3]))}

    def lu_timers(self):
        """LU phase times since the last call (recorded while timers() is on):
        dict of (milliseconds, count) for factorizations, panels, trailing
        updates and triangular solves."""
        out = np.zeros(8)
        self.check(lib().om_context_lu_timers(self.h, _p(out)))
        return {"factor": (out[0], int(out[1])), "panel": (out[2], int(out[3])),
                "update": (out[4], int(out[5])), "tri_solve": (out[6], int(out[7]))}

    @property
    def last_launches(self) -> int:
        return lib().om_context_last_launches(self.h)


def spheres_array(xyz, radius, eps, nmax, mu=None, eps_sh=None, ksippp=0.0, ksiparppar=0.0,
                  gamma=0.0):
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = xyz.shape[0]
    chi = [np.broadcast_to(np.asarray(v, dtype=np.complex128), (n,)) for v in (ksippp, ksiparppar, gamma)]
    radius = np.broadcast_to(np.asarray(radius, dtype=np.float64), (n,))
    eps = np.broadcast_to(np.asarray(eps, dtype=np.complex128), (n,))
    mu = np.broadcast_to(np.asarray(1.0 if mu is None else mu, dtype=np.complex128), (n,))
    eps_sh = eps if eps_sh is None else np.broadcast_to(np.asarray(eps_sh, dtype=np.complex128), (n,))
    arr = (Sphere * n)()
    for i in range(n):
        s = arr[i]
        s.x, s.y, s.z = xyz[i]
        s.radius = radius[i]
        s.eps_r[0], s.eps_r[1] = eps[i].real, eps[i].imag
        s.mu_r[0], s.mu_r[1] = mu[i].real, mu[i].imag
        s.eps_r_sh[0], s.eps_r_sh[1] = eps_sh[i].real, eps_sh[i].imag
        s.ksippp[0], s.ksippp[1] = chi[0][i].real, chi[0][i].imag
        s.ksiparppar[0], s.ksiparppar[1] = chi[1][i].real, chi[1][i].imag
        s.gamma[0], s.gamma[1] = chi[2][i].real, chi[2][i].imag
        s.nmax = int(nmax)
    return arr


def medium(eps=1.0, mu=1.0) -> Medium:
    eps, mu = complex(eps), complex(mu)
    return Medium((C.c_double * 2)(eps.real, eps.imag), (C.c_double * 2)(mu.real, mu.imag))


def plane_wave(wavelength, theta=0.0, phi=0.0, e_theta=1.0, e_phi=0.0, sh=False) -> PlaneWave:
    et, ep = complex(e_theta), complex(e_phi)
    return PlaneWave(wavelength, theta, phi, (C.c_double * 2)(et.real, et.imag),
                     (C.c_double * 2)(ep.real, ep.imag), int(sh), 0)


class Problem:
    """Geometry + Excitation of one cluster at one wavelength, device resident."""

    def __init__(self, ctx: Context, spheres, bg: Medium | None, wave: PlaneWave):
        self.ctx = ctx
        h = C.c_void_p()
        self._keep = (spheres, bg, wave)
        rc = lib().om_problem_create(ctx.h, spheres, len(spheres),
                                     None if bg is None else C.byref(bg), C.byref(wave), C.byref(h))
        ctx.check(rc)
        self.h = h
        self.n = lib().om_problem_size(h)
        self.nmax = spheres[0].nmax
        self.P = self.nmax * (self.nmax + 2)
        self.N = len(spheres)

    def close(self):
        if getattr(self, "h", None):
            # a closed context has already destroyed its problems
            if getattr(self.ctx, "h", None):
                lib().om_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_wavelength(self, wavelength):
        self.ctx.check(lib().om_problem_set_wavelength(self.h, wavelength))

    def set_wave(self, wave: PlaneWave):
        self.ctx.check(lib().om_problem_set_wave(self.h, C.byref(wave)))

    def tmatrix(self, harmonic=FF):
        out = np.zeros((self.N, 2 * self.P), np.complex128)
        self.ctx.check(lib().om_tmatrix(self.h, harmonic, _p(out)))
        return out

    def incident_coefficients(self):
        out = np.zeros(2 * self.P, np.complex128)
        self.ctx.check(lib().om_incident_coefficients(self.h, _p(out)))
        return out

    def assemble(self, harmonic=FF, precision=C128):
        self.ctx.check(lib().om_assemble(self.h, harmonic, precision))

    def matrix(self, harmonic=FF):
        S = np.zeros((self.n, self.n), np.complex128, order="F")
        self.ctx.check(lib().om_copy_matrix(self.h, harmonic, _p(S)))
        return S

    def source_vector(self, copy=True):
        Q = np.zeros(self.n, np.complex128) if copy else None
        self.ctx.check(lib().om_source_vector(self.h, _p(Q)))
        return Q

    def solve(self, opts: SolveOptions | None = None, allow_unconverged=False) -> SolveStats:
        st = SolveStats()
        rc = lib().om_solve(self.h, C.byref(opts or options()), C.byref(st))
        if not (allow_unconverged and rc == ERR_NOT_CONVERGED):
            self.ctx.check(rc)
        return st

    def solve_rhs(self, b, harmonic=FF, opts: SolveOptions | None = None):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b)
        st = SolveStats()
        self.ctx.check(lib().om_solve_rhs(self.h, harmonic, C.byref(opts or options()), _p(b),
                                          _p(x), C.byref(st)))
        return x, st

    def assemble_rows(self, sphere0, sphere1, harmonic=FF):
        """Block rows of S for spheres sphere0 .. sphere1 - 1 (complex128, on
        the device; om_assemble_rows)."""
        self.ctx.check(lib().om_assemble_rows(self.h, harmonic, int(sphere0), int(sphere1)))

    def matvec_rows(self, x_device_ptr, y_device_ptr, harmonic=FF):
        """y = S_rows x with x (n) and y (the block's rows) complex128 device
        buffers given by address (om_matvec_rows)."""
        self.ctx.check(lib().om_matvec_rows(self.h, harmonic, C.c_void_p(x_device_ptr),
                                            C.c_void_p(y_device_ptr)))

    def coefficients(self):
        xs = np.zeros(self.n, np.complex128)
        xi = np.zeros(self.n, np.complex128)
        self.ctx.check(lib().om_get_coefficients(self.h, _p(xs), _p(xi)))
        return xs, xi

    def cross_sections(self):
        out = np.zeros(4)
        self.ctx.check(lib().om_cross_sections(self.h, _p(out)))
        return out

    def solve_sh(self, opts: SolveOptions | None = None) -> SolveStats:
        """SH source, SH solve and SH internal coefficients (needs solve() and assemble(SH))."""
        st = SolveStats()
        self.ctx.check(lib().om_solve_sh(self.h, C.byref(opts or options()), C.byref(st)))
        return st

    def sh_vectors(self):
        """(K, K1ana, X_sca_SH, X_int_SH)."""
        outs = [np.zeros(self.n, np.complex128) for _ in range(4)]
        self.ctx.check(lib().om_get_sh_vectors(self.h, *[_p(o) for o in outs]))
        return outs

    def sh_cross_sections(self):
        """(C_sca_SH, C_abs_SH)."""
        out = np.zeros(2)
        self.ctx.check(lib().om_sh_cross_sections(self.h, _p(out)))
        return out

    def near_field(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        E = np.zeros((xyz.shape[0], 3), np.complex128)
        H = np.zeros_like(E)
        self.ctx.check(lib().om_near_field(self.h, _p(xyz), xyz.shape[0], _p(E), _p(H)))
        return E, H

    def aca_info(self, harmonic=FF):
        """Packed bytes, compressed / dense block counts, mean and max rank of
        an OM_ACA assembly."""
        b = C.c_double()
        nc, nd, mx = C.c_int(), C.c_int(), C.c_int()
        mr = C.c_double()
        self.ctx.check(lib().om_aca_info(self.h, harmonic, C.byref(b), C.byref(nc), C.byref(nd),
                                         C.byref(mr), C.byref(mx)))
        return {"store_bytes": b.value, "compressed": nc.value, "dense": nd.value,
                "mean_rank": mr.value, "max_rank": mx.value}

    def near_field_sh(self, xyz):
        """Second-harmonic E, H at Cartesian points (after solve_sh)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        E = np.zeros((xyz.shape[0], 3), np.complex128)
        H = np.zeros_like(E)
        self.ctx.check(lib().om_near_field_sh(self.h, _p(xyz), xyz.shape[0], _p(E), _p(H)))
        return E, H


def coupling(ctx: Context, rel_xyz, k: complex, nmax: int, regular: bool):
    """Coupling(relR, waveK, nMax, regular) for one or many Cartesian displacements."""
    rel = np.ascontiguousarray(rel_xyz, dtype=np.float64).reshape(-1, 3)
    P = nmax * (nmax + 2)
    A = np.zeros((rel.shape[0], P, P), np.complex128)
    B = np.zeros_like(A)
    ctx.check(lib().om_coupling(ctx.h, _p(rel), rel.shape[0], complex(k).real, complex(k).imag,
                                nmax, int(regular), _p(A), _p(B)))
    # (count, col, row) in memory -> (count, row, col)
    return A.transpose(0, 2, 1), B.transpose(0, 2, 1)


def wavelength_solve(ctx: Context, spheres, bg, wave, opts=None, precision=C128, want_coeffs=False):
    n = 2 * spheres[0].nmax * (spheres[0].nmax + 2) * len(spheres)
    xsec = np.zeros(4)
    xs = np.zeros(n, np.complex128) if want_coeffs else None
    xi = np.zeros(n, np.complex128) if want_coeffs else None
    st = SolveStats()
    rc = lib().om_wavelength_solve(ctx.h, spheres, len(spheres), None if bg is None else C.byref(bg),
                                   C.byref(wave), C.byref(opts or options()), precision, _p(xsec),
                                   _p(xs), _p(xi), C.byref(st))
    ctx.check(rc)
    return xsec, xs, xi, st


def cgemm_sub_c64(ctx: Context, A, B, C_):
    """C - A B for complex64 A (m x k), B (k x n), C (m x n), any k >= 1, on the
    tensor cores (om_cgemm_sub_c64); returns the new C."""
    A = np.asfortranarray(A, dtype=np.complex64)
    B = np.asfortranarray(B, dtype=np.complex64)
    out = np.array(C_, dtype=np.complex64, order="F")
    m, k = A.shape
    n = B.shape[1]
    fp = lambda a: a.ctypes.data_as(_fp)
    ctx.check(lib().om_cgemm_sub_c64(ctx.h, m, n, k, fp(A), m, fp(B), k, fp(out), m))
    return out


def matvec_inner(ctx: Context, S, x, products: int = 1) -> np.ndarray:
    """y = S x by the precision form's inner FP32 product, `products` times
    (om_matvec_inner_c64): the first on the complex64 matrix (it writes the
    bf16 copy when inner_half is on), the later ones on the copy."""
    S = np.asfortranarray(S, dtype=np.complex64)
    x = np.ascontiguousarray(x, dtype=np.complex64)
    n = S.shape[0]
    y = np.zeros(n, dtype=np.complex64)
    fp = lambda a: a.ctypes.data_as(_fp)
    ctx.check(lib().om_matvec_inner_c64(ctx.h, n, fp(S), fp(x), fp(y), products))
    return y


def clg_tables(ctx: Context, nmax: int) -> np.ndarray:
    """The nine SH coupling tables computed on the device, flattened (9 P^3)."""
    P = nmax * (nmax + 2)
    out = np.zeros(9 * P ** 3)
    ctx.check(lib().om_clg_tables(ctx.h, nmax, _p(out)))
    return out


def wavelength_solve_sh(ctx: Context, spheres, bg, wave, opts=None, precision=C128):
    xsec = np.zeros(4)
    xsh = np.zeros(2)
    st = SolveStats()
    rc = lib().om_wavelength_solve_sh(ctx.h, spheres, len(spheres), None if bg is None else C.byref(bg),
                                      C.byref(wave), C.byref(opts or options()), precision,
                                      _p(xsec), _p(xsh), C.byref(st))
    ctx.check(rc)
    return xsec, xsh, st


def _result_dict(r: Result) -> dict:
    st = lambda s: {"iterations": s.iterations, "inner_iterations": s.inner_iterations,
                    "rel_residual": s.rel_residual, "seconds": s.seconds}
    return {"status": r.status, "slot": r.slot, "xsec": np.array(r.xsec[:]),
            "xsec_sh": np.array(r.xsec_sh[:]), "ff": st(r.ff), "sh": st(r.sh),
            "queue_ms": r.queue_ms, "service_ms": r.service_ms, "latency_ms": r.latency_ms,
            "device_bytes": r.device_bytes}


def batch_solve(ctx: Context, requests, arena_bytes: int = 0):
    """Batched wavelength solves (om_batch_solve). `requests`: a list of
    (spheres, background, wave, opts, precision) tuples (a sixth element, the
    cluster key, is accepted and ignored). Returns one result dict per request,
    as Server.poll."""
    n = len(requests)
    rq = (Request * max(n, 1))()
    keep = []
    for i, r in enumerate(requests):
        sp, bg, wave, opts, prec = r[:5]
        keep.append(sp)
        rq[i] = Request(C.cast(sp, C.POINTER(Sphere)), len(sp), prec, bg or medium(), wave,
                        opts or options(), 0)
    out = (Result * max(n, 1))()
    ctx.check(lib().om_batch_solve(ctx.h, rq, n, arena_bytes, out))
    return [_result_dict(out[i]) for i in range(n)]


def batch_tiles(ctx: Context):
    """The batched matvec configurations the autotuner chose on this context
    (om_batch_tiles): one dict per size class."""
    k = lib().om_batch_tiles(ctx.h, None, 0)
    if k < 0:
        ctx.check(k)
    buf = (C.c_int * max(7 * k, 1))()
    lib().om_batch_tiles(ctx.h, buf, k)
    keys = ("precision", "nmax", "Npad", "rows", "order", "ctas_per_sm", "matvec_us")
    return [dict(zip(keys, buf[7 * i:7 * i + 7])) for i in range(k)]


class Server:
    """Serving / batching runtime (om_server_*): `slots` contexts on one GPU
    taking wavelength-solve requests in arrival order, admitted against an HBM
    budget in bytes (0 = the device's free memory less 1/16)."""

    def __init__(self, device: int = 0, budget: int = 0, slots: int = 2):
        h = C.c_void_p()
        rc = lib().om_server_create(device, budget, slots, C.byref(h))
        if rc:
            raise OptimetError(rc, "cannot create a server on device %d" % device)
        self.h = h
        self._keep = {}

    def close(self):
        if getattr(self, "h", None):
            lib().om_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def submit(self, spheres, bg, wave, opts=None, precision=C128, cluster_key=0) -> int:
        rq = Request(C.cast(spheres, C.POINTER(Sphere)), len(spheres), precision, bg, wave,
                     opts or options(), cluster_key)
        t = C.c_ulonglong()
        rc = lib().om_server_submit(self.h, C.byref(rq), C.byref(t))
        if rc:
            raise OptimetError(rc, lib().om_server_last_error(self.h).decode())
        return t.value

    def poll(self, ticket: int, wait: bool = True):
        """None while pending (wait=False), else a dict of the result."""
        r = Result()
        rc = lib().om_server_poll(self.h, ticket, int(wait), C.byref(r))
        if rc == PENDING:
            return None
        if rc:
            raise OptimetError(rc, "unknown ticket %d" % ticket)
        return _result_dict(r)

    def drain(self):
        lib().om_server_drain(self.h)

    def batching(self, max_requests=64, arena_bytes=0, max_request_bytes=0):
        """Serve runs of up to max_requests batchable requests (footprint at
        most max_request_bytes, 0 = any) through the batching form
        (om_server_batching); max_requests <= 1 turns it off."""
        rc = lib().om_server_batching(self.h, max_requests, arena_bytes, max_request_bytes)
        if rc:
            raise OptimetError(rc, "server batching")

    def tune(self, matvec_ctas_per_sm=0, matvec_df_ctas_per_sm=0, assemble_carveout=-1,
             matvec_carveout=-1, lu_tensor_cores=-1, matvec_tma=-1, assemble_rotation=-1, lu_persistent=-1, batch_tiles=-1,
             batch_fused=-1, inner_half=-1):
        t = Tuning(matvec_ctas_per_sm, matvec_df_ctas_per_sm, assemble_carveout, matvec_carveout,
                   lu_tensor_cores, matvec_tma, assemble_rotation, lu_persistent, batch_tiles,
                   batch_fused, inner_half)
        rc = lib().om_server_tune(self.h, C.byref(t))
        if rc:
            raise OptimetError(rc, "server tune")

    def mark(self) -> float:
        out = np.zeros(1)
        rc = lib().om_server_mark(self.h, _p(out))
        if rc:
            raise OptimetError(rc, "server mark")
        return float(out[0])

    def autotune(self, spheres, bg, wave, opts=None, precision=C128, cluster_key=1, count=4,
                 step=0.25e-9):
        """Pick the fastest built-in launch tuning for requests like this one;
        returns it as a dict."""
        rq = Request(C.cast(spheres, C.POINTER(Sphere)), len(spheres), precision, bg, wave,
                     opts or options(), cluster_key)
        t = Tuning()
        rc = lib().om_server_autotune(self.h, C.byref(rq), count, step, C.byref(t))
        if rc:
            raise OptimetError(rc, lib().om_server_last_error(self.h).decode())
        return {f: getattr(t, f) for f, _ in Tuning._fields_}

    def launches(self) -> int:
        return int(lib().om_server_launches(self.h))

    @property
    def last_error(self) -> str:
        return lib().om_server_last_error(self.h).decode()


def declared_symbols():
    """Entry points declared in include/optimet_gpu.h."""
    import re
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(om_[a-z0-9_]+)\s*\(", text)))
