"""The C++ interface (include/optimet_gpu.hpp) as a reference-side caller
uses it: a program built with g++ against the header and the library. On the
CPU the program compiles; on the GPU it solves the C0 case (two spheres,
nMax = 6, direct LU) and matches the oracle's golden cross sections."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "solver_case.cpp")


def _gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not available")
    return g


def test_header_and_program_compile(tmp_path):
    out = tmp_path / "solver_case.o"
    subprocess.run([_gxx(), "-std=c++17", "-Wall", "-Werror", "-c", SRC, "-I", os.path.join(ROOT, "include"),
                    "-I", "/usr/local/cuda/include", "-o", str(out)], check=True)
    assert out.exists()


@pytest.mark.gpu
def test_c0_through_the_cpp_interface(tmp_path):
    from optimet_gb300 import build
    build.build()
    lib_dir = os.path.dirname(build.LIB)
    exe = tmp_path / "solver_case"
    subprocess.run([_gxx(), "-std=c++17", SRC, "-I", os.path.join(ROOT, "include"), "-I",
                    "/usr/local/cuda/include", "-L", lib_dir, "-loptimet_gpu", "-Wl,-rpath," + lib_dir,
                    "-o", str(exe)], check=True)
    g = load_golden("c0")
    lines = []
    for c, r, e in zip(g["xyz"], np.broadcast_to(g["radius"], (len(g["xyz"]),)),
                       np.broadcast_to(g["eps"], (len(g["xyz"]),))):
        lines.append("sphere %.17g %.17g %.17g %.17g %.17g %.17g" % (float(c[0]), float(c[1]), float(c[2]),
                                                                   float(r), float(e.real), float(e.imag)))
    lines.append("nmax %d" % int(g["nmax"]))
    th, ph = (float(v) for v in g["angles"])
    et, ep = (complex(v) for v in g["pol"])
    lines.append("wave %.17g %.17g %.17g %.17g %.17g %.17g %.17g" % (float(g["wavelength"]), th, ph, et.real,
                                                                   et.imag, ep.real, ep.imag))
    b0, b1 = (complex(v) for v in g["bg"])
    lines.append("background %.17g %.17g %.17g %.17g" % (b0.real, b0.imag, b1.real, b1.imag))
    lines.append("method lu")
    case = tmp_path / "c0.txt"
    case.write_text("\n".join(lines) + "\n")
    run = subprocess.run([str(exe), str(case)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    out = run.stdout
    xsec = np.array([float(v) for v in next(l for l in out.splitlines() if l.startswith("xsec")).split()[1:]])
    assert np.max(np.abs(xsec - g["xsec"]) / np.abs(g["xsec"])) < 1e-10
