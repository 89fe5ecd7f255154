"""CPU checks of the GPU library: it builds for sm_103a and exports every
entry point include/optimet_gpu.h declares. No GPU calls."""
import ctypes
import pytest


@pytest.fixture(scope="module")
def built():
    from optimet_gb300 import build
    return build.build()


def test_library_exports_declared_symbols(built):
    import optimet_gb300 as G
    declared = G.declared_symbols()
    assert len(declared) >= 20
    L = ctypes.CDLL(built)
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_build_targets_sm103a_only():
    from optimet_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_python_wrapper_loads(built):
    import optimet_gb300 as G
    assert G.lib() is not None


def test_python_structs_mirror_the_header(tmp_path):
    """Every ctypes mirror of a C-ABI struct has the header's size and the
    header's offset for each of its fields (compiled with the host C
    compiler against include/optimet_gpu.h)."""
    import os
    import shutil
    import subprocess
    import optimet_gb300 as G
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    pairs = {"om_sphere": G.Sphere, "om_medium": G.Medium, "om_plane_wave": G.PlaneWave,
             "om_solve_options": G.SolveOptions, "om_solve_stats": G.SolveStats, "om_tuning": G.Tuning,
             "om_request": G.Request, "om_result": G.Result}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "optimet_gpu.h"', 'int main(void) {']
    expect = []
    for cname, py in pairs.items():
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        expect.append(ctypes.sizeof(py))
        for f, _ in py._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {f}));')
            expect.append(getattr(py, f).offset)
    lines += ['  return 0;', '}']
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    exe = tmp_path / "abi"
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True, capture_output=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    assert got == expect
