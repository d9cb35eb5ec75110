"""nb_energy_noalloc: the energy entry point for callers that cannot let the library allocate
device memory (for example an application that reserves the GPU's memory for its own pool up
front, or a time-critical loop that cannot afford cudaMalloc's device-wide synchronisation).

Calls the entry point through the C ABI twice in a row -- the second time with fewer bodies, so
partials left in the shared fixed scratch array by the first call must not leak into the second --
and checks each result against nb_energy and against the CPU oracle's energy (which restates
nBodyAlgorithm.cpp:11-86) within the energy tests' tolerance (1e-12 relative). The second call is
also checked to allocate nothing: every tensor the test needs exists before free memory is read,
which happens right around that call. Kept in a file pytest collects last: a failure here comes
after every other test has run.
"""

import ctypes

import numpy as np
import pytest

import oracle
from helpers import bodies, dev

pytestmark = pytest.mark.gpu

MAX_N = 1048576  # NB_ENERGY_NOALLOC_MAX_N in include/nbody.h
KEYS = ("m", "x", "y", "z", "vx", "vy", "vz")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_energy_matches_nb_energy_and_the_oracle_on_two_calls():
    import torch
    from nbody.lib import Context, load
    lib = load()
    ctx = Context(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n, seed in ((70001, 3), (1500, 4)):
        d = bodies("plummer", n, seed=seed)
        arrs = [dev(d[k]) for k in KEYS]
        out = torch.zeros(4, dtype=torch.float64, device="cuda")
        ref = torch.zeros(4, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = lib.nb_energy_noalloc(*[_ptr(a) for a in arrs], n, d["G"], _ptr(out), stream)
        assert st == 0, lib.nb_last_error_string()
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if seed == 4:  # the set-up happened on the first call; this call must not allocate
            assert free_after == free_before, (free_before, free_after)
        ctx.energy(*arrs, d["G"], ref)
        ctx.sync()
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        scale = max(abs(want[0]), abs(want[1]))
        assert np.all(np.abs(got - want) <= 1e-12 * scale), (got, want)
        o = oracle.energy(*[d[k] for k in KEYS], d["G"])
        expect = np.array([o["kinetic"], o["potential"], o["total"], o["virial"]])
        assert np.all(np.abs(got[:3] - expect[:3]) <= 1e-12 * scale), (got, expect)
        assert abs(got[3] - expect[3]) <= 1e-12 * abs(expect[3]), (got[3], expect[3])
    ctx.close()


def test_noalloc_energy_rejects_sizes_beyond_its_limit():
    import torch
    from nbody.lib import load
    lib = load()
    x = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = _ptr(x)
    st = lib.nb_energy_noalloc(p, p, p, p, p, p, p, MAX_N + 1, 1.0, p, ctypes.c_void_p(0))
    assert st == 1  # NB_ERR_INVALID_ARG
    assert b"exceeds the fixed scratch limit" in lib.nb_last_error_string()
