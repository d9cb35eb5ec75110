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


def header_defines():
    src = open(os.path.join(ROOT, "include", "nbody.h")).read()
    return {k: int(v.rstrip("u"), 0)
            for k, v in re.findall(r"#define\s+(NB_[A-Z0-9_]+)\s+([0-9xa-fA-Fu]+)\b", src)}


def test_python_constants_match_the_header():
    """The binding's copies of the header's counts and bit masks agree with include/nbody.h."""
    import __graft_entry__  # noqa: F401
    from nbody import lib
    h = header_defines()
    pairs = {"NB_PAIR_CONFIG_COUNT": lib.PAIR_CONFIGS, "NB_BATCH_CONFIG_COUNT": lib.BATCH_CONFIGS,
             "NB_REC_FP64": lib.REC_FP64, "NB_REC_DF": lib.REC_DF,
             "NB_REC_LEARNED": lib.REC_LEARNED, "NB_REC_ALL": lib.REC_ALL,
             "NB_BUILD_QUANTIZED_KEYS": lib.BUILD_QUANTIZED_KEYS,
             "NB_FAULT_DROP_LOOKBACK": lib.FAULT_DROP_LOOKBACK,
             "NB_LEARNED_STACK_CAP": lib.LEARNED_STACK_CAP,
             "NB_POLICY_BOUND_ACCEPT": lib.POLICY_BOUND_ACCEPT, "NB_MLP_PARAMS": lib.MLP_PARAMS}
    for name, value in pairs.items():
        assert h[name] == value, (name, h[name], value)
    assert h["NB_BATCH_CONFIG_COUNT"] == h["NB_PAIR_CONFIG_COUNT"] + h["NB_SYM_CONFIG_COUNT"]
    assert h["NB_REC_ALL"] & h["NB_BUILD_QUANTIZED_KEYS"] == 0


def test_record_sets_per_traversal():
    """records_for / build_mask_for: what each traversal reads, and quantized keys exactly for
    the traversals without FP64 records (no reference-exact cells needed)."""
    import __graft_entry__  # noqa: F401
    from nbody.lib import (BUILD_QUANTIZED_KEYS, REC_DF, REC_FP64, REC_LEARNED, build_mask_for,
                           records_for)
    assert records_for("theta", "f64") == REC_FP64
    assert records_for("theta", "f64_ieee") == REC_FP64
    assert records_for("group", "f64") == REC_FP64
    assert records_for("theta", "df64") == REC_FP64 | REC_DF
    assert records_for("theta", "f32c") == 0 and records_for("group", "f32c") == 0
    assert records_for("learned", "f32c") == REC_LEARNED
    for opening, precision in (("theta", "f64"), ("theta", "df64"), ("group", "f64")):
        assert not build_mask_for(opening, precision) & BUILD_QUANTIZED_KEYS
    for opening, precision in (("theta", "f32c"), ("group", "f32c"), ("learned", "f32c")):
        assert build_mask_for(opening, precision) & BUILD_QUANTIZED_KEYS


def test_policy_file_round_trip_and_rejections(tmp_path, cuda_lib):
    """nb_policy_save / nb_policy_load are host-side: a saved network and its settings load back
    bit for bit; files with another magic line, network shape, parameter count, a malformed value
    or unknown flags are rejected with NB_ERR_INVALID_ARG."""
    import numpy as np

    from nbody.lib import NBodyError, policy_load, policy_save
    rng = np.random.default_rng(4)
    params = rng.normal(size=1377).astype(np.float32) * np.float32(3.7)
    params[5] = np.float32(1e-38)  # subnormal-adjacent and extreme values survive the text form
    params[6] = np.float32(-3.4e38)
    path = str(tmp_path / "policy.txt")
    policy_save(path, params, -4.125, 0.3, 2 ** 31 - 1, 1)
    got, tau, theta, cap, flags = policy_load(path)
    np.testing.assert_array_equal(got, params)
    assert (tau, theta, cap, flags) == (-4.125, 0.3, 2 ** 31 - 1, 1)
    text = open(path).read().splitlines()
    assert text[0] == "nbody-gb300 opening policy 1" and text[6] == "params 1377"
    variants = {
        "magic": ["nbody opening policy 2"] + text[1:],
        "shape": text[:1] + ["network 8 64 64 1 relu"] + text[2:],
        "count": text[:6] + ["params 1376"] + text[7:-1],
        "value": text[:10] + ["nan-ish"] + text[11:],
        "flags": text[:5] + ["flags 6"] + text[6:],
        "short": text[:-1],
    }
    for name, lines in variants.items():
        bad = str(tmp_path / f"bad_{name}.txt")
        open(bad, "w").write("\n".join(lines) + "\n")
        with pytest.raises(NBodyError, match="INVALID_ARG"):
            policy_load(bad)
    with pytest.raises(ValueError):
        policy_save(path, params[:10], -4.0, 0.3, 1, 1)
