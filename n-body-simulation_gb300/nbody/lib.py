"""ctypes binding of libnbody_cuda.so (the C ABI declared in include/nbody.h).

Device arrays are passed as torch CUDA tensors (float64, contiguous); torch is only the
allocator and stream provider here. There is no CPU fallback: if the library is missing the
import-time load raises.
"""

from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "_build", "libnbody_cuda.so")

NB_OK = 0
STATUS_NAMES = {0: "NB_OK", 1: "NB_ERR_INVALID_ARG", 2: "NB_ERR_CUDA", 3: "NB_ERR_OOM",
                4: "NB_ERR_POOL_OVERFLOW", 5: "NB_ERR_DEPTH_OVERFLOW", 6: "NB_ERR_STACK_OVERFLOW",
                7: "NB_ERR_TIMEOUT", 8: "NB_ERR_UNSUPPORTED", 9: "NB_ERR_NOT_BUILT"}

NB_F64, NB_F64_IEEE, NB_F32C, NB_DF64 = 0, 1, 2, 3
PRECISIONS = {"f64": NB_F64, "f64_ieee": NB_F64_IEEE, "f32c": NB_F32C, "df64": NB_DF64}

_vp = C.c_void_p
_u32 = C.c_uint32
_d = C.c_double
_i = C.c_int


class NBodyError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# name -> (restype, argtypes); every function returns nb_status (int) unless stated.
SIGNATURES = {
    "nb_ctx_create": [_i, C.POINTER(_vp)],
    "nb_ctx_destroy": [_vp],
    "nb_sync": [_vp, _vp],
    "nb_naive_accel": [_vp] + [_vp] * 7 + [_u32, _d, _d, _i, _i, _vp],
    "nb_naive_accel_range": [_vp] + [_vp] * 7 + [_u32, _u32, _u32, _d, _d, _i, _vp],
    "nb_leapfrog_kick_drift": [_vp] + [_vp] * 12 + [_u32, _d, _vp],
    "nb_leapfrog_kick": [_vp] + [_vp] * 9 + [_u32, _d, _vp],
    "nb_leapfrog_kick_kick_drift": [_vp] + [_vp] * 12 + [_u32, _d, _vp],
    "nb_energy": [_vp] + [_vp] * 7 + [_u32, _d, _vp, _vp],
    "nb_aabb": [_vp] + [_vp] * 3 + [_u32, _vp, _vp],
    "nb_energy_noalloc": [_vp] * 7 + [_u32, _d, _vp, _vp],
    "nb_ctx_set_fault_hooks": [_vp, C.c_longlong, C.c_uint, C.c_uint],
}
STRING_FUNCS = ("nb_last_error_string", "nb_version")

_lib = None


def load() -> C.CDLL:
    """Loads the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not found: run n-body-simulation_gb300/build.py first")
        L = C.CDLL(LIB_PATH)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = argtypes
        for name in STRING_FUNCS:
            getattr(L, name).restype = C.c_char_p
            getattr(L, name).argtypes = []
        _lib = L
    return _lib


def check(status: int):
    if status != NB_OK:
        raise NBodyError(status, load().nb_last_error_string().decode())


def ptr(t) -> int:
    """Device pointer of a contiguous torch CUDA tensor (or None -> NULL)."""
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous(), "expected a contiguous CUDA tensor"
    return t.data_ptr()


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class Context:
    """Owns an nb_ctx (device id, scratch memory, device error word)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = _vp()
        check(self.lib.nb_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nb_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_fault_hooks(self, wait_limit=-1, flags=0, learned_stack_cap=0):
        """Failure-path test hooks of later launches (nb_ctx_set_fault_hooks): wait_limit polls
        before a bounded wait gives up (-1 = default), FAULT_DROP_LOOKBACK, stack capacity of the
        learned traversal (0 = full)."""
        check(self.lib.nb_ctx_set_fault_hooks(self.handle, wait_limit, flags, learned_stack_cap))

    def sync(self, stream=None):
        check(self.lib.nb_sync(self.handle, stream_ptr(stream)))

    # -- naive -----------------------------------------------------------------------------
    def naive_accel(self, m, x, y, z, ax, ay, az, G, eps2, precision="f64", block_size=0,
                    stream=None):
        n = m.numel()
        check(self.lib.nb_naive_accel(self.handle, ptr(m), ptr(x), ptr(y), ptr(z), ptr(ax),
                                      ptr(ay), ptr(az), n, G, eps2, PRECISIONS[precision],
                                      block_size, stream_ptr(stream)))

    def naive_accel_range(self, m, x, y, z, ax, ay, az, i_begin, i_end, G, eps2,
                          precision="f64", stream=None):
        n = m.numel()
        check(self.lib.nb_naive_accel_range(self.handle, ptr(m), ptr(x), ptr(y), ptr(z), ptr(ax),
                                            ptr(ay), ptr(az), n, i_begin, i_end, G, eps2,
                                            PRECISIONS[precision], stream_ptr(stream)))

    # -- integration -------------------------------------------------------------------------
    def kick_drift(self, vh, v, p, a, dt, stream=None):
        n = v[0].numel()
        check(self.lib.nb_leapfrog_kick_drift(self.handle, *map(ptr, vh), *map(ptr, v),
                                              *map(ptr, p), *map(ptr, a), n, dt,
                                              stream_ptr(stream)))

    def kick(self, v, vh, a, dt, stream=None):
        n = v[0].numel()
        check(self.lib.nb_leapfrog_kick(self.handle, *map(ptr, v), *map(ptr, vh), *map(ptr, a), n,
                                        dt, stream_ptr(stream)))

    def kick_kick_drift(self, v, vh, p, a, dt, stream=None):
        n = v[0].numel()
        check(self.lib.nb_leapfrog_kick_kick_drift(self.handle, *map(ptr, v), *map(ptr, vh),
                                                   *map(ptr, p), *map(ptr, a), n, dt,
                                                   stream_ptr(stream)))

    def energy(self, m, x, y, z, vx, vy, vz, G, out, stream=None):
        check(self.lib.nb_energy(self.handle, ptr(m), ptr(x), ptr(y), ptr(z), ptr(vx), ptr(vy),
                                 ptr(vz), m.numel(), G, ptr(out), stream_ptr(stream)))

    def naive_accel_targets(self, m, x, y, z, targets, ax, ay, az, G, eps2, stream=None):
        check(self.lib.nb_naive_accel_targets(self.handle, ptr(m), ptr(x), ptr(y), ptr(z),
                                              m.numel(), ptr(targets), targets.numel(), ptr(ax),
                                              ptr(ay), ptr(az), G, eps2, stream_ptr(stream)))

    def aabb(self, x, y, z, out, stream=None):
        check(self.lib.nb_aabb(self.handle, ptr(x), ptr(y), ptr(z), x.numel(), ptr(out),
                               stream_ptr(stream)))


# -- Barnes-Hut ---------------------------------------------------------------------------------
NB_OPEN_THETA, NB_OPEN_THETA_GROUP, NB_OPEN_LEARNED = 0, 1, 2
OPENINGS = {"theta": NB_OPEN_THETA, "group": NB_OPEN_THETA_GROUP, "learned": NB_OPEN_LEARNED}


class BHParams(C.Structure):
    _fields_ = [("theta", C.c_double), ("storage_size_param", C.c_uint32),
                ("stack_size_param", C.c_uint32), ("max_build_level", C.c_int),
                ("sort_bodies", C.c_int)]


class BHStats(C.Structure):
    _fields_ = [("n", C.c_uint32), ("node_count", C.c_uint32), ("max_depth", C.c_uint32),
                ("ref_node_count", C.c_uint32), ("aabb", C.c_double * 7)]


class BHRefLayout(C.Structure):
    _fields_ = [("capacity", C.c_uint32), ("node_count", C.c_uint32),
                ("octants", C.c_void_p), ("edge", C.c_void_p), ("min_x", C.c_void_p),
                ("min_y", C.c_void_p), ("min_z", C.c_void_p), ("body_of_node", C.c_void_p),
                ("node_is_leaf", C.c_void_p), ("sum_masses", C.c_void_p), ("com_x", C.c_void_p),
                ("com_y", C.c_void_p), ("com_z", C.c_void_p), ("body_count", C.c_void_p),
                ("sorted_bodies", C.c_void_p)]


SIGNATURES.update({
    "nb_bh_params_default": [C.POINTER(BHParams)],
    "nb_bh_tree_create": [_vp, _u32, C.POINTER(BHParams), C.POINTER(_vp)],
    "nb_bh_tree_destroy": [_vp],
    "nb_bh_tree_set_theta": [_vp, _d],
    "nb_bh_build": [_vp, _vp] + [_vp] * 4 + [_u32, _d, _vp],
    "nb_bh_accel": [_vp, _vp] + [_vp] * 6 + [_d, _d, _i, _i, _vp],
    "nb_bh_tree_stats": [_vp, C.POINTER(BHStats)],
    "nb_bh_export_ref_layout": [_vp, C.POINTER(BHRefLayout)],
    "nb_bh_export_order": [_vp, _vp, _vp],
    "nb_util_radix_sort_pairs": [_vp, _vp, _vp, _u32, _i, _i, _vp],
    "nb_util_exclusive_scan_u32": [_vp, _vp, _vp, _u32, _vp],
    "nb_bh_count_interactions": [_vp, _vp, _vp, _vp, _vp, _i, _vp, _vp],
    "nb_util_fma_peak": [_vp, _i, C.POINTER(_d)],
    "nb_bh_set_schedule": [_i],
    "nb_naive_set_pair_config": [_i],
    "nb_naive_set_symmetric": [_i, _i, _i, _i],
    "nb_batch_create": [_vp, _u32, _vp, C.POINTER(_vp)],
    "nb_batch_destroy": [_vp],
    "nb_batch_info": [_vp, C.POINTER(_u32), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i),
                      C.POINTER(_i)],
    "nb_batch_set_config": [_vp, _vp, _i],
    "nb_batch_naive_accel": [_vp, _vp] + [_vp] * 7 + [_d, _d, _vp],
    "nb_batch_autotune": [_vp, _vp] + [_vp] * 7 + [_d, _d, _i, _vp, C.POINTER(_i)],
    "nb_batch_graph_create": [_vp, _vp] + [_vp] * 13 + [_d, _d, _d, _i, C.POINTER(_vp)],
    "nb_graph_launch": [_vp, _vp],
    "nb_graph_destroy": [_vp],
    "nb_mlp_param_count": [C.POINTER(_u32)],
    "nb_mlp_loss_grad": [_vp] + [_vp] * 4 + [_u32, _vp, _vp, _vp],
    "nb_mlp_adam": [_vp] + [_vp] * 4 + [C.c_float] * 4 + [_i, _vp],
    "nb_mlp_predict": [_vp, _vp, _vp, _u32, _vp, _i, _vp],
    "nb_bh_generate_pairs": [_vp, _vp] + [_vp] * 7 + [_d, _d, _d, _d, _u32, _u32, _u32, _vp, _vp,
                                                     _vp, _vp, _vp],
    "nb_bh_export_node_ranges": [_vp, _vp, _vp, _vp, _vp],
    "nb_naive_accel_targets": [_vp] + [_vp] * 4 + [_u32, _vp, _u32] + [_vp] * 3 + [_d, _d, _vp],
    "nb_bh_set_policy": [_vp, _vp, C.c_float, _d, _u32, _u32],
    "nb_policy_save": [C.c_char_p, _vp, C.c_float, _d, _u32, _u32],
    "nb_policy_load": [C.c_char_p, _vp, C.POINTER(C.c_float), C.POINTER(_d), C.POINTER(_u32),
                       C.POINTER(_u32)],
    "nb_bh_set_phase_timing": [_vp, _i],
    "nb_bh_set_records": [_vp, C.c_uint],
    "nb_bh_graph_create": [_vp, _vp] + [_vp] * 13 + [_u32, _d, _d, _d, _i, _i, _i, _vp],
    "nb_bh_build_phase_ms": [_vp, _vp],
    "nb_bh_accel_learned_counted": [_vp, _vp] + [_vp] * 6 + [_d, _vp, _vp],
})


def default_bh_params(**kw) -> BHParams:
    p = BHParams()
    check(load().nb_bh_params_default(C.byref(p)))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class BHTree:
    """Owns an nb_bh_tree (device memory for up to n_max bodies)."""

    def __init__(self, ctx: Context, n_max: int, **params):
        self.ctx = ctx
        self.lib = load()
        self.params = default_bh_params(**params)
        h = _vp()
        check(self.lib.nb_bh_tree_create(ctx.handle, n_max, C.byref(self.params), C.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nb_bh_tree_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_theta(self, theta):
        check(self.lib.nb_bh_tree_set_theta(self.handle, theta))

    def build(self, m, x, y, z, G, stream=None):
        check(self.lib.nb_bh_build(self.ctx.handle, self.handle, ptr(m), ptr(x), ptr(y), ptr(z),
                                   m.numel(), G, stream_ptr(stream)))

    def graph(self, m, pos, vel, vh, acc, G, eps2, dt, steps, opening="theta", precision="f64"):
        """CUDA graph of `steps` leapfrog steps (kick-drift, build, traversal, kick)."""
        h = _vp()
        check(self.lib.nb_bh_graph_create(self.ctx.handle, self.handle, ptr(m), *map(ptr, pos),
                                          *map(ptr, vel), *map(ptr, vh), *map(ptr, acc),
                                          m.numel(), G, eps2, dt, steps, OPENINGS[opening],
                                          PRECISIONS[precision], C.byref(h)))
        return Graph(h)

    def set_records(self, mask):
        """Node record sets later builds compute (REC_* bits; records_for gives a traversal's)."""
        check(self.lib.nb_bh_set_records(self.handle, mask))

    def set_phase_timing(self, enable=True):
        check(self.lib.nb_bh_set_phase_timing(self.handle, 1 if enable else 0))

    def build_phase_ms(self):
        """Durations (ms) of the last build's phases: AABB, keys, sort, cells, centre of mass."""
        ms = (C.c_float * 5)()
        check(self.lib.nb_bh_build_phase_ms(self.handle, ms))
        return list(ms)

    def accel(self, x, y, z, ax, ay, az, G, eps2, opening="theta", precision="f64", stream=None):
        check(self.lib.nb_bh_accel(self.ctx.handle, self.handle, ptr(x), ptr(y), ptr(z), ptr(ax),
                                   ptr(ay), ptr(az), G, eps2, OPENINGS[opening],
                                   PRECISIONS[precision], stream_ptr(stream)))

    def stats(self) -> dict:
        s = BHStats()
        check(self.lib.nb_bh_tree_stats(self.handle, C.byref(s)))
        return {"n": s.n, "node_count": s.node_count, "max_depth": s.max_depth,
                "ref_node_count": s.ref_node_count, "aabb": list(s.aabb)}

    def count_interactions(self, x, y, z, opening="theta", stream=None):
        """(accepted, opened) cell totals of a traversal under a theta rule."""
        import torch
        out = torch.zeros(2, dtype=torch.int64, device="cuda")
        check(self.lib.nb_bh_count_interactions(self.ctx.handle, self.handle, ptr(x), ptr(y),
                                                ptr(z), OPENINGS[opening], ptr(out),
                                                stream_ptr(stream)))
        self.ctx.sync(stream)
        a, o = out.cpu().tolist()
        return int(a), int(o)

    def export_node_ranges(self):
        import numpy as np
        nc = self.stats()["node_count"]
        a = [np.zeros(nc, dtype=np.uint32) for _ in range(4)]
        check(self.lib.nb_bh_export_node_ranges(self.handle, *[v.ctypes.data for v in a]))
        return {"first": a[0], "count": a[1], "level": a[2], "body": a[3]}

    def set_policy(self, params, log10_tau, theta_fallback=0.5, count_cap=8192,
                   bound_accept=None):
        """bound_accept (default: on when a network is given) accepts cells whose analytic error
        bound is below tau before the network is asked."""
        self._policy = params  # keep the device tensor alive
        if bound_accept is None:
            bound_accept = params is not None
        check(self.lib.nb_bh_set_policy(self.handle, ptr(params), log10_tau, theta_fallback,
                                        count_cap, 1 if bound_accept else 0))

    def accel_learned_counted(self, x, y, z, ax, ay, az, eps2, stream=None):
        """NB_OPEN_LEARNED traversal; returns (interactions, policy decisions, cells visited,
        walk steps)."""
        import torch
        cnt = torch.zeros(4, dtype=torch.int64, device="cuda")
        check(self.lib.nb_bh_accel_learned_counted(self.ctx.handle, self.handle, ptr(x), ptr(y),
                                                   ptr(z), ptr(ax), ptr(ay), ptr(az), eps2,
                                                   ptr(cnt), stream_ptr(stream)))
        self.ctx.sync(stream)
        a, b, c, d = cnt.cpu().tolist()
        return int(a), int(b), int(c), int(d)

    def generate_pairs(self, m, x, y, z, ax, ay, az, G, eps2, theta_gen, sample_fraction, seed,
                       count_cap, max_pairs, with_ids=False, stream=None):
        """(features [k,8], labels [k], pair ids [k,2] or None, pairs found) on the device."""
        import torch
        f = torch.empty((max_pairs, 8), dtype=torch.float32, device="cuda")
        lab = torch.empty(max_pairs, dtype=torch.float32, device="cuda")
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        ids = torch.empty((max_pairs, 2), dtype=torch.int32, device="cuda") if with_ids else None
        check(self.lib.nb_bh_generate_pairs(self.ctx.handle, self.handle, ptr(m), ptr(x), ptr(y),
                                            ptr(z), ptr(ax), ptr(ay), ptr(az), G, eps2, theta_gen,
                                            sample_fraction, seed, count_cap, max_pairs, ptr(f),
                                            ptr(lab), ptr(cnt), ptr(ids) if with_ids else None,
                                            stream_ptr(stream)))
        self.ctx.sync(stream)
        found = int(cnt.item())
        k = min(found, max_pairs)
        return f[:k], lab[:k], (ids[:k] if with_ids else None), found

    def export_order(self, n):
        import numpy as np
        ids = np.zeros(n, dtype=np.uint32)
        lvl = np.zeros(n, dtype=np.uint32)
        check(self.lib.nb_bh_export_order(self.handle, ids.ctypes.data, lvl.ctypes.data))
        return ids, lvl

    def export_ref_layout(self, n):
        """The reference's linearised octree arrays (numpy), trimmed to node_count."""
        import numpy as np
        st = self.stats()
        cap = st["ref_node_count"]
        arrs = {"octants": np.zeros(8 * cap, np.uint32), "edge": np.zeros(cap), "min_x": np.zeros(cap),
                "min_y": np.zeros(cap), "min_z": np.zeros(cap),
                "body_of_node": np.zeros(cap, np.uint32), "node_is_leaf": np.zeros(cap, np.int32),
                "sum_masses": np.zeros(cap), "com_x": np.zeros(cap), "com_y": np.zeros(cap),
                "com_z": np.zeros(cap), "body_count": np.zeros(cap, np.uint32),
                "sorted_bodies": np.zeros(max(n, 1), np.uint32)}
        lay = BHRefLayout()
        lay.capacity = cap
        for k, a in arrs.items():
            setattr(lay, k, a.ctypes.data)
        check(self.lib.nb_bh_export_ref_layout(self.handle, C.byref(lay)))
        nc = lay.node_count
        out = {k: (v[:nc] if k not in ("octants", "sorted_bodies") else v) for k, v in arrs.items()}
        out["octants"] = arrs["octants"].reshape(8, cap)[:, :nc]
        out["sorted_bodies"] = arrs["sorted_bodies"][:n]
        out["node_count"] = nc
        return out


def set_bh_schedule(lockstep: bool):
    check(load().nb_bh_set_schedule(1 if lockstep else 0))


def fma_peak(ctx: Context, fp64: bool) -> float:
    v = C.c_double(0)
    check(load().nb_util_fma_peak(ctx.handle, 1 if fp64 else 0, C.byref(v)))
    return v.value


def util_radix_sort_pairs(ctx: Context, keys, vals, begin_bit=0, end_bit=64, stream=None):
    check(load().nb_util_radix_sort_pairs(ctx.handle, ptr(keys), ptr(vals), keys.numel(),
                                          begin_bit, end_bit, stream_ptr(stream)))


def util_exclusive_scan_u32(ctx: Context, inp, out, stream=None):
    check(load().nb_util_exclusive_scan_u32(ctx.handle, ptr(inp), ptr(out), inp.numel(),
                                            stream_ptr(stream)))


def set_naive_pair_config(config: int):
    check(load().nb_naive_set_pair_config(config))


SYM_NEVER, SYM_AUTO, SYM_ALWAYS = 0, 1, 2

# node record sets of a tree build (NB_REC_*) and the quantized-key build option
REC_FP64, REC_DF, REC_LEARNED = 1, 2, 4
REC_ALL = REC_FP64 | REC_DF | REC_LEARNED
BUILD_QUANTIZED_KEYS = 8


def records_for(opening: str, precision: str) -> int:
    """The record sets nb_bh_accel needs for an opening rule and precision."""
    if opening == "learned":
        return REC_LEARNED
    if precision == "f32c":
        return 0
    if precision == "df64":
        return REC_FP64 | REC_DF
    return REC_FP64


def build_mask_for(opening: str, precision: str) -> int:
    """records_for plus quantized keys for the traversals that need no reference-exact cells
    (every one without FP64 records: the FP32 rules and the learned policy)."""
    rec = records_for(opening, precision)
    return rec if rec & REC_FP64 else rec | BUILD_QUANTIZED_KEYS


def set_naive_symmetric(mode: int = SYM_AUTO, config: int = 0, config_f64: int = 0,
                        config_df: int = 0):
    """Selection of the symmetric pair kernel for full-range NB_F32C / NB_F64 / NB_DF64
    evaluations and its FP32, FP64 and double-float tile shapes."""
    check(load().nb_naive_set_symmetric(mode, config, config_f64, config_df))


class Batch:
    """Ensemble of independent systems in concatenated arrays (nb_batch)."""

    def __init__(self, ctx: Context, counts):
        import numpy as np
        self.ctx = ctx
        self.lib = load()
        self.counts = np.ascontiguousarray(counts, dtype=np.uint32)
        h = _vp()
        check(self.lib.nb_batch_create(ctx.handle, len(self.counts), self.counts.ctypes.data,
                                       C.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nb_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        n, c, t, ip, jt = _u32(), _i(), _i(), _i(), _i()
        check(self.lib.nb_batch_info(self.handle, C.byref(n), C.byref(c), C.byref(t), C.byref(ip),
                                     C.byref(jt)))
        return {"n_total": n.value, "config": c.value, "threads": t.value,
                "targets_per_thread": ip.value, "j_tile": jt.value}

    def set_config(self, config: int):
        check(self.lib.nb_batch_set_config(self.ctx.handle, self.handle, config))

    def accel(self, m, x, y, z, ax, ay, az, G, eps2, stream=None):
        check(self.lib.nb_batch_naive_accel(self.ctx.handle, self.handle, ptr(m), ptr(x), ptr(y),
                                            ptr(z), ptr(ax), ptr(ay), ptr(az), G, eps2,
                                            stream_ptr(stream)))

    def autotune(self, m, x, y, z, ax, ay, az, G, eps2, reps=3):
        ms = (C.c_float * BATCH_CONFIGS)()
        chosen = _i()
        check(self.lib.nb_batch_autotune(self.ctx.handle, self.handle, ptr(m), ptr(x), ptr(y),
                                         ptr(z), ptr(ax), ptr(ay), ptr(az), G, eps2, reps, ms,
                                         C.byref(chosen)))
        return chosen.value, list(ms)

    def graph(self, m, pos, vel, vh, acc, G, eps2, dt, steps):
        h = _vp()
        check(self.lib.nb_batch_graph_create(self.ctx.handle, self.handle, ptr(m), *map(ptr, pos),
                                             *map(ptr, vel), *map(ptr, vh), *map(ptr, acc), G,
                                             eps2, dt, steps, C.byref(h)))
        return Graph(h)


class Graph:
    def __init__(self, handle):
        self.lib = load()
        self.handle = handle

    def launch(self, stream=None):
        check(self.lib.nb_graph_launch(self.handle, stream_ptr(stream)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nb_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


POLICY_BOUND_ACCEPT = 1  # NB_POLICY_BOUND_ACCEPT
FAULT_DROP_LOOKBACK = 1  # NB_FAULT_DROP_LOOKBACK
LEARNED_STACK_CAP = 1024  # NB_LEARNED_STACK_CAP

MLP_PARAMS = 1377
PAIR_CONFIGS = 8  # NB_PAIR_CONFIG_COUNT
BATCH_CONFIGS = 16  # NB_BATCH_CONFIG_COUNT: the one-sided shapes, then the symmetric ones


def mlp_loss_grad(ctx, params, X, Y, idx, n, grad, loss, stream=None):
    check(load().nb_mlp_loss_grad(ctx.handle, ptr(params), ptr(X), ptr(Y), ptr(idx), n, ptr(grad),
                                  ptr(loss), stream_ptr(stream)))


def mlp_adam(ctx, params, m, v, grad, lr, beta1, beta2, eps, step, stream=None):
    check(load().nb_mlp_adam(ctx.handle, ptr(params), ptr(m), ptr(v), ptr(grad), lr, beta1, beta2,
                             eps, step, stream_ptr(stream)))


def mlp_predict(ctx, params, X, out, bf16=False, stream=None):
    check(load().nb_mlp_predict(ctx.handle, ptr(params), ptr(X), X.shape[0], ptr(out),
                                1 if bf16 else 0, stream_ptr(stream)))


def policy_save(path, params, log10_tau, theta_fallback, count_cap, flags):
    """Writes an opening-policy file (nb_policy_save) from a network (any array-like of
    MLP_PARAMS values, device or host) and its nb_bh_set_policy settings."""
    import numpy as np
    if hasattr(params, "detach"):
        params = params.detach().cpu().numpy()
    host = np.ascontiguousarray(params, dtype=np.float32)
    if host.size != MLP_PARAMS:
        raise ValueError(f"a network has {MLP_PARAMS} parameters, got {host.size}")
    check(load().nb_policy_save(os.fsencode(path), host.ctypes.data, log10_tau, theta_fallback,
                                count_cap, flags))


def policy_load(path):
    """(params as a float32 numpy array, log10_tau, theta_fallback, count_cap, flags) of an
    opening-policy file (nb_policy_load)."""
    import numpy as np
    host = np.zeros(MLP_PARAMS, dtype=np.float32)
    tau, theta = C.c_float(0), C.c_double(0)
    cap, flags = C.c_uint32(0), C.c_uint32(0)
    check(load().nb_policy_load(os.fsencode(path), host.ctypes.data, C.byref(tau),
                                C.byref(theta), C.byref(cap), C.byref(flags)))
    return host, tau.value, theta.value, cap.value, flags.value
