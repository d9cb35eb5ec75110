"""CPU-side checks of the drop-in boundary: the library loads and exports every entry point that
include/nbody.h declares (no compute calls: this machine may have no GPU)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "nbody.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nb_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def cuda_lib():
    import __graft_entry__  # noqa: F401  (puts the package on sys.path)
    from nbody import lib
    if not os.path.exists(lib.LIB_PATH):
        pytest.skip("library not built")
    return ctypes.CDLL(lib.LIB_PATH)


def test_header_declares_core_entry_points():
    names = declared_functions()
    for must in ("nb_ctx_create", "nb_ctx_destroy", "nb_naive_accel", "nb_leapfrog_kick_drift",
                 "nb_leapfrog_kick", "nb_energy", "nb_aabb", "nb_last_error_string", "nb_sync"):
        assert must in names


def test_library_exports_every_declared_symbol(cuda_lib):
    missing = [n for n in declared_functions() if not hasattr(cuda_lib, n)]
    assert not missing, f"declared in include/nbody.h but not exported: {missing}"


def test_python_binding_covers_every_symbol():
    from nbody import lib
    covered = set(lib.SIGNATURES) | set(lib.STRING_FUNCS)
    missing = [n for n in declared_functions() if n not in covered]
    assert not missing, f"no ctypes signature for {missing}"


def test_version_and_error_string_without_gpu(cuda_lib):
    cuda_lib.nb_version.restype = ctypes.c_char_p
    assert b"sm_103a" in cuda_lib.nb_version()
    cuda_lib.nb_last_error_string.restype = ctypes.c_char_p
    assert isinstance(cuda_lib.nb_last_error_string(), bytes)


def test_null_context_is_rejected_without_touching_the_gpu(cuda_lib):
    cuda_lib.nb_sync.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    assert cuda_lib.nb_sync(None, None) == 1  # NB_ERR_INVALID_ARG
