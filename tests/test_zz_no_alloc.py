"""GPU test of om_solve_rhs_noalloc, the solve entry point that allocates no
device memory (for callers that cannot call cudaMalloc/cudaFree while they
solve: a serving loop whose HBM is already handed out, or code that must not
let an allocation synchronise the device). It must give the same solution as
the allocating entry point om_solve_rhs, call after call, although every call
reuses the same fixed device array."""
import ctypes as C

import numpy as np
import pytest

from helpers import load_golden, rel

pytestmark = pytest.mark.gpu


def _bind(G):
    L = G.lib()
    f = L.om_solve_rhs_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.POINTER(G.SolveOptions), C.POINTER(C.c_double),
                  C.POINTER(C.c_double), C.POINTER(G.SolveStats)]
    f.restype = C.c_int
    return f


def _problem(G, ctx):
    g = load_golden("metal5")
    cplx = lambda a: np.asarray(a, dtype=np.complex128)
    sp = G.spheres_array(g["xyz"], g["radius"], cplx(g["eps"]), int(g["nmax"]), mu=cplx(g["mu"]),
                         eps_sh=cplx(g["eps_sh"]))
    bg = G.medium(complex(g["bg"][0]), complex(g["bg"][1]))
    wave = G.plane_wave(float(g["wavelength"]), float(g["angles"][0]), float(g["angles"][1]),
                        complex(g["pol"][0]), complex(g["pol"][1]))
    return G.Problem(ctx, sp, bg, wave)


def test_no_alloc_solve_matches_allocating_solve():
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    solve_noalloc = _bind(G)
    ctx = G.Context(0)
    pr = _problem(G, ctx)
    b = pr.source_vector()
    pr.assemble(G.FF, G.C128)
    opts = G.options(G.SOLVE_GMRES, tol=1e-12, max_iter=120, restarts=6)
    x_ref, _ = pr.solve_rhs(b, G.FF, opts)
    dp = C.POINTER(C.c_double)
    for _ in range(2):  # two calls in a row share the same device array
        x = np.zeros_like(b)
        st = G.SolveStats()
        rc = solve_noalloc(pr.h, G.FF, C.byref(opts), b.ctypes.data_as(dp), x.ctypes.data_as(dp),
                           C.byref(st))
        assert rc == G.OK, G.lib().om_context_last_error(ctx.h)
        assert st.rel_residual <= 1e-12
        assert rel(x, x_ref) < 1e-10
    # independent of om_solve_rhs: the fixture's scattering coefficients
    # (the oracle's solution, through the reference's AMOS Bessel route)
    g = load_golden("metal5")
    assert rel(x, g["X_sca"]) < 1e-10
    # the complex64 matrix (the precision form's storage): the same GMRES over
    # the compensated complex64 x complex128 product, against om_solve_rhs on
    # that matrix; the complex64 rounding of S keeps it within 1e-6 of FP64
    pr.assemble(G.FF, G.C64)
    x64_ref, _ = pr.solve_rhs(b, G.FF, opts)
    for _ in range(2):
        x = np.zeros_like(b)
        st = G.SolveStats()
        rc = solve_noalloc(pr.h, G.FF, C.byref(opts), b.ctypes.data_as(dp), x.ctypes.data_as(dp),
                           C.byref(st))
        assert rc == G.OK, G.lib().om_context_last_error(ctx.h)
        assert st.rel_residual <= 1e-12 and st.seconds > 0
        assert rel(x, x64_ref) < 1e-10
        assert rel(x, g["X_sca"]) < 1e-6
    # a request larger than the fixed array is refused before any GPU work
    big = G.options(G.SOLVE_GMRES, tol=1e-12, max_iter=200000, restarts=1)
    x = np.zeros_like(b)
    rc = solve_noalloc(pr.h, G.FF, C.byref(big), b.ctypes.data_as(dp), x.ctypes.data_as(dp), None)
    assert rc == G.ERR_INVALID
    assert b"no-alloc scratch" in G.lib().om_context_last_error(ctx.h)
    pr.close()
    ctx.close()
