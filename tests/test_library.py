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
