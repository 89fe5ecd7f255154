"""The C++ interface (include/optimet_gpu.hpp) as a reference-side caller
uses it: programs built with g++ against the header and the library.

On the CPU: both programs compile, and the solver-role mapping (plan: the
reference's solver::factory choice with each solver class's own parameters)
and the polarisation conversion (the reference's Cartesian Excitation::Einc
back to E_theta, E_phi) give the expected values. On the GPU: the metal5
fixture (oblique incidence, elliptical polarisation E_theta = 0.6,
E_phi = 0.8i, given to the program as its Cartesian field) under the direct
(serial and ScaLAPACK builds), Belos GMRES and ACA roles, against the golden
cross sections and coefficients."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "solver_case.cpp")
ROLES = os.path.join(ROOT, "tests", "cpp", "plan_roles.cpp")
INC = ["-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include"]


def _gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not available")
    return g


def test_header_and_program_compile(tmp_path):
    for src in (SRC, ROLES):
        out = tmp_path / (os.path.basename(src) + ".o")
        subprocess.run([_gxx(), "-std=c++17", "-Wall", "-Werror", "-c", src, *INC, "-o", str(out)], check=True)
        assert out.exists()


def test_solver_roles_and_polarisation(tmp_path):
    exe = tmp_path / "plan_roles"
    subprocess.run([_gxx(), "-std=c++17", "-Wall", "-Werror", ROLES, *INC, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    got = [tuple(ln.split(" : ")[1].split()) for ln in out[:-1]]
    C128, ACA, LU, GMRES = "0", "2", "0", "1"
    want = [(C128, LU, "0", "0", "0"), (C128, LU, "0", "0", "0"),  # serial QR, ScaLAPACK pzgesv
            (C128, GMRES, "300", "3", "1e-09"),                        # Belos: Num Blocks, Max Iterations, tol
            (C128, LU, "0", "0", "0"), (C128, LU, "0", "0", "0"),      # Belos list "eigen", "scalapack"
            (ACA, GMRES, "240", "2", "1e-06"), (ACA, GMRES, "250", "3", "1e-07"),
            (ACA, GMRES, "340", "1", "1e-06"), (ACA, GMRES, "240", "2", "1e-06")]
    assert got == want
    th, ph = 0.7, -1.1
    E = np.array([0.3 + 0.1j, -0.2 + 0.4j, 0.5 - 0.6j])
    eth = np.array([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)]) @ E
    eph = np.array([-np.sin(ph), np.cos(ph), 0.0]) @ E
    v = [float(x) for x in out[-1].split()[1:]]
    assert abs(complex(v[0], v[1]) - eth) < 1e-15 and abs(complex(v[2], v[3]) - eph) < 1e-15


def _case(g, role_lines):
    lines = []
    rad = np.broadcast_to(g["radius"], (len(g["xyz"]),))
    eps = np.broadcast_to(g["eps"], (len(g["xyz"]),))
    for c, r, e in zip(g["xyz"], rad, eps):
        lines.append("sphere %.17g %.17g %.17g %.17g %.17g %.17g" % (*map(float, c), float(r), e.real, e.imag))
    lines.append("nmax %d" % int(g["nmax"]))
    th, ph = (float(v) for v in g["angles"])
    lines.append("wave %.17g %.17g %.17g" % (float(g["wavelength"]), th, ph))
    et, ep = (complex(v) for v in g["pol"])
    # Tools::toProjection of (0, E_theta, E_phi): the Cartesian field the reference keeps
    E = et * np.array([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)]) + \
        ep * np.array([-np.sin(ph), np.cos(ph), 0.0])
    lines.append("einc " + " ".join("%.17g %.17g" % (z.real, z.imag) for z in E))
    b0, b1 = (complex(v) for v in g["bg"])
    lines.append("background %.17g %.17g %.17g %.17g" % (b0.real, b0.imag, b1.real, b1.imag))
    return "\n".join(lines + role_lines) + "\n"


@pytest.mark.gpu
@pytest.mark.parametrize("name,roles,tol", [
    ("c0", ["role serial"], 1e-10),
    ("metal5", ["role serial"], 1e-10),
    ("metal5", ["role scalapack"], 1e-10),
    ("metal5", ["role belos", "solver GMRES", "tolerance 1e-12", "iterations 400 200"], 1e-10),
    ("metal5", ["role belos", "solver eigen"], 1e-10),
    ("metal5", ["role serial", "aca yes"], 1e-2),
])
def test_roles_through_the_cpp_interface(tmp_path, name, roles, tol):
    from optimet_gb300 import build
    build.build()
    lib_dir = os.path.dirname(build.LIB)
    exe = tmp_path / "solver_case"
    subprocess.run([_gxx(), "-std=c++17", SRC, *INC, "-L", lib_dir, "-loptimet_gpu", "-Wl,-rpath," + lib_dir,
                    "-o", str(exe)], check=True)
    g = load_golden(name)
    case = tmp_path / "case.txt"
    case.write_text(_case(g, roles))
    run = subprocess.run([str(exe), str(case)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    lines = run.stdout.splitlines()
    xsec = np.array([float(v) for v in next(ln for ln in lines if ln.startswith("xsec")).split()[1:]])
    x = np.array([complex(*map(float, ln.split()[1:])) for ln in lines if ln.startswith("x ")])
    assert np.max(np.abs(xsec - g["xsec"]) / np.abs(g["xsec"])) < tol
    assert np.max(np.abs(x - g["X_sca"])) / np.max(np.abs(g["X_sca"])) < tol
    if "aca yes" in roles:
        assert next(ln for ln in lines if ln.startswith("plan")).split()[1] == "2"  # OM_ACA
