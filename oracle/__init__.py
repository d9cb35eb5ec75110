"""CPU oracle for the naive and Barnes-Hut force paths -- TEST INFRASTRUCTURE ONLY.

A ctypes binding of ``oracle/nbody_oracle.cpp``, a C++17/OpenMP restatement of the reference's
kernels (file:line citations in that file). Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU legs of ``bench.py`` import this package, and only as the parity reference or the timed CPU baseline;
the CUDA library and the host driver never load it.

Pinned against the reference's own known answers (tests/BarnesHutTest.cpp): AABB, node table,
subtree preparation, subtree body sort, root mass, in-order body sort. Parity unpinned for force,
centre-of-mass, leapfrog and energy values: no reference test covers them and the reference
(SYCL) cannot be compiled on these machines.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")

_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint32)
_ip = C.POINTER(C.c_int)
_u64p = C.POINTER(C.c_uint64)


class _TreeView(C.Structure):
    _fields_ = [
        ("n", C.c_uint32), ("S", C.c_uint32), ("node_count", C.c_uint32), ("pad", C.c_uint32),
        ("octants", _up),
        ("edge", _dp), ("min_x", _dp), ("min_y", _dp), ("min_z", _dp),
        ("body_of_node", _up),
        ("node_is_leaf", _ip),
        ("sum_masses", _dp), ("com_x", _dp), ("com_y", _dp), ("com_z", _dp),
        ("body_count", _up),
        ("sorted_bodies", _up),
        ("subtree_of_body", _up),
        ("aabb", C.c_double * 7),
    ]


def build(force: bool = False) -> str:
    """Compiles the oracle with its Makefile (g++ -fopenmp); returns the .so path."""
    if force or not os.path.exists(_SO):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_SO)
        L.orc_naive_accel.argtypes = [_dp] * 7 + [C.c_uint32, C.c_double, C.c_double, C.c_int]
        L.orc_naive_accel_subset.argtypes = [_dp] * 4 + [C.c_uint32, _up, C.c_uint32] + [_dp] * 3 + [
            C.c_double, C.c_double, C.c_int]
        L.orc_leapfrog_part1.argtypes = [_dp] * 12 + [C.c_uint32, C.c_double]
        L.orc_leapfrog_part2.argtypes = [_dp] * 9 + [C.c_uint32, C.c_double]
        L.orc_energy.argtypes = [_dp] * 7 + [C.c_uint32, C.c_double, _dp, C.c_int]
        L.orc_adjust_velocities.argtypes = [_dp] * 4 + [C.c_uint32]
        L.orc_aabb.argtypes = [_dp] * 3 + [C.c_uint32, C.c_int, _dp]
        L.orc_tree_create.restype = C.c_void_p
        L.orc_tree_create.argtypes = [C.c_uint32, C.c_uint32]
        L.orc_tree_destroy.argtypes = [C.c_void_p]
        L.orc_tree_view_get.argtypes = [C.c_void_p, C.POINTER(_TreeView)]
        L.orc_tree_build_subtrees.argtypes = [C.c_void_p] + [_dp] * 4 + [C.c_int] * 4
        L.orc_tree_build_sync.argtypes = [C.c_void_p] + [_dp] * 4 + [C.c_int] * 3
        L.orc_prepare_subtrees.argtypes = [_up, C.c_uint32, C.c_uint32, _up, _up, _up]
        L.orc_sort_bodies_for_subtrees.argtypes = [_up, C.c_uint32, _up, _up, C.c_uint32, _up, _up]
        L.orc_bh_accel.argtypes = [C.c_void_p] + [_dp] * 6 + [C.c_double] * 3 + [C.c_uint32, C.c_int,
                                                                                 C.c_int]
        L.orc_bh_accel_subset.argtypes = [C.c_void_p] + [_dp] * 3 + [_up, C.c_uint32] + [_dp] * 3 + [
            C.c_double] * 3 + [C.c_uint32, C.c_int]
        L.orc_bh_interaction_counts.argtypes = [C.c_void_p] + [_dp] * 3 + [C.c_double, C.c_uint32,
                                                                           _u64p, _u64p, C.c_int]
        L.orc_stack_size.restype = C.c_uint32
        L.orc_stack_size.argtypes = [C.c_uint32, C.c_uint32]
        _lib = L
    return _lib


def _d(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _u(a: np.ndarray):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(_up)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


# --------------------------------------------------------------------------------------------
def naive_accel(m, x, y, z, G, eps2, threads=0):
    m, x, y, z = map(_f64, (m, x, y, z))
    n = len(m)
    ax, ay, az = (np.empty(n) for _ in range(3))
    _check(lib().orc_naive_accel(_d(m), _d(x), _d(y), _d(z), _d(ax), _d(ay), _d(az), n, G, eps2,
                                 threads), "naive_accel")
    return ax, ay, az


def naive_accel_subset(m, x, y, z, targets, G, eps2, threads=0):
    m, x, y, z = map(_f64, (m, x, y, z))
    targets = np.ascontiguousarray(targets, dtype=np.uint32)
    k = len(targets)
    ax, ay, az = (np.empty(k) for _ in range(3))
    _check(lib().orc_naive_accel_subset(_d(m), _d(x), _d(y), _d(z), len(m), _u(targets), k,
                                        _d(ax), _d(ay), _d(az), G, eps2, threads), "subset")
    return ax, ay, az


def leapfrog_part1(v, p, a, dt):
    """v, p, a: lists of 3 float64 arrays; p is updated in place. Returns v_half."""
    n = len(v[0])
    vh = [np.empty(n) for _ in range(3)]
    lib().orc_leapfrog_part1(*[_d(q) for q in vh], *[_d(q) for q in v], *[_d(q) for q in p],
                             *[_d(q) for q in a], n, dt)
    return vh


def leapfrog_part2(v, vh, a, dt):
    """Writes v (in place) from v_half and a."""
    n = len(v[0])
    lib().orc_leapfrog_part2(*[_d(q) for q in v], *[_d(q) for q in vh], *[_d(q) for q in a], n, dt)


def energy(m, x, y, z, vx, vy, vz, G, threads=0):
    arrs = list(map(_f64, (m, x, y, z, vx, vy, vz)))
    out = np.zeros(4)
    lib().orc_energy(*[_d(a) for a in arrs], len(arrs[0]), G, _d(out), threads)
    return {"kinetic": out[0], "potential": out[1], "total": out[2], "virial": out[3]}


def adjust_velocities(m, vx, vy, vz):
    lib().orc_adjust_velocities(_d(m), _d(vx), _d(vy), _d(vz), len(m))


def aabb(x, y, z, work_items=1024):
    x, y, z = map(_f64, (x, y, z))
    out = np.zeros(7)
    _check(lib().orc_aabb(_d(x), _d(y), _d(z), len(x), work_items, _d(out)), "aabb")
    return {"min_x": out[0], "min_y": out[1], "min_z": out[2], "max_x": out[3], "max_y": out[4],
            "max_z": out[5], "edge": out[6]}


def stack_size(n, stack_size_param=16):
    return int(lib().orc_stack_size(n, stack_size_param))


@dataclass
class OracleTree:
    """Copies of the reference-layout octree arrays after a build (node_count entries each)."""
    n: int
    S: int
    node_count: int
    octants: np.ndarray        # [8, node_count] child ids per octant (0 = none)
    edge: np.ndarray
    min_x: np.ndarray
    min_y: np.ndarray
    min_z: np.ndarray
    body_of_node: np.ndarray   # n = empty or internal
    node_is_leaf: np.ndarray
    sum_masses: np.ndarray
    com_x: np.ndarray          # mass-weighted numerators
    com_y: np.ndarray
    com_z: np.ndarray
    body_count: np.ndarray
    sorted_bodies: np.ndarray
    subtree_of_body: np.ndarray
    aabb: np.ndarray
    handle: object = None


class _TreeHandle:
    def __init__(self, n, storage_param):
        self.ptr = lib().orc_tree_create(n, storage_param)

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().orc_tree_destroy(self.ptr)
            self.ptr = None


def _view(handle: _TreeHandle) -> OracleTree:
    v = _TreeView()
    lib().orc_tree_view_get(handle.ptr, C.byref(v))
    nc, S, n = v.node_count, v.S, v.n

    def arr(ptr, count, dt):
        if count == 0:
            return np.zeros(0, dtype=dt)
        return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dt, copy=True)

    octs = np.ctypeslib.as_array(v.octants, shape=(8 * S,)).reshape(8, S)[:, :nc].copy()
    return OracleTree(
        n=n, S=S, node_count=nc, octants=octs,
        edge=arr(v.edge, nc, np.float64), min_x=arr(v.min_x, nc, np.float64),
        min_y=arr(v.min_y, nc, np.float64), min_z=arr(v.min_z, nc, np.float64),
        body_of_node=arr(v.body_of_node, nc, np.uint32), node_is_leaf=arr(v.node_is_leaf, nc, np.int32),
        sum_masses=arr(v.sum_masses, nc, np.float64), com_x=arr(v.com_x, nc, np.float64),
        com_y=arr(v.com_y, nc, np.float64), com_z=arr(v.com_z, nc, np.float64),
        body_count=arr(v.body_count, nc, np.uint32), sorted_bodies=arr(v.sorted_bodies, n, np.uint32),
        subtree_of_body=arr(v.subtree_of_body, n, np.uint32), aabb=np.array(list(v.aabb)),
        handle=handle)


def build_subtrees(m, x, y, z, max_level=7, storage_param=16, aabb_work_items=1024, sort=True,
                   threads=0) -> OracleTree:
    """ParallelOctreeTopDownSubtrees::buildOctree (default builder) + centre of mass + sort."""
    m, x, y, z = map(_f64, (m, x, y, z))
    h = _TreeHandle(len(m), storage_param)
    _check(lib().orc_tree_build_subtrees(h.ptr, _d(m), _d(x), _d(y), _d(z), max_level,
                                         aabb_work_items, int(sort), threads), "build_subtrees")
    return _view(h)


def build_sync(m, x, y, z, storage_param=16, aabb_work_items=1024, sort=True, threads=0) -> OracleTree:
    """ParallelOctreeTopDownSynchronized::buildOctree + centre of mass + sort."""
    m, x, y, z = map(_f64, (m, x, y, z))
    h = _TreeHandle(len(m), storage_param)
    _check(lib().orc_tree_build_sync(h.ptr, _d(m), _d(x), _d(y), _d(z), aabb_work_items, int(sort),
                                     threads), "build_sync")
    return _view(h)


def prepare_subtrees(subtree_of_body, node_count):
    sob = np.ascontiguousarray(subtree_of_body, dtype=np.uint32)
    counts = np.zeros(node_count, dtype=np.uint32)
    subtrees = np.zeros(node_count, dtype=np.uint32)
    num = C.c_uint32(0)
    lib().orc_prepare_subtrees(_u(sob), len(sob), node_count, _u(counts), _u(subtrees), C.byref(num))
    return counts, subtrees[: num.value].copy(), num.value


def sort_bodies_for_subtrees(subtree_of_body, counts, subtrees):
    sob = np.ascontiguousarray(subtree_of_body, dtype=np.uint32)
    counts = np.ascontiguousarray(counts, dtype=np.uint32)
    subtrees = np.ascontiguousarray(subtrees, dtype=np.uint32)
    start = np.zeros(len(subtrees), dtype=np.uint32)
    total = int(sum(int(counts[s]) for s in subtrees))
    sorted_bodies = np.zeros(max(total, 1), dtype=np.uint32)
    lib().orc_sort_bodies_for_subtrees(_u(sob), len(sob), _u(counts), _u(subtrees), len(subtrees),
                                       _u(start), _u(sorted_bodies))
    return start, sorted_bodies[:total]


def bh_accel(tree: OracleTree, x, y, z, G, eps2, theta, stack_size_words=None, sorted_order=True,
             threads=0):
    x, y, z = map(_f64, (x, y, z))
    n = tree.n
    if stack_size_words is None:
        stack_size_words = stack_size(n)
    ax, ay, az = (np.zeros(n) for _ in range(3))
    _check(lib().orc_bh_accel(tree.handle.ptr, _d(x), _d(y), _d(z), _d(ax), _d(ay), _d(az), G, eps2,
                              theta, stack_size_words, int(sorted_order), threads), "bh_accel")
    return ax, ay, az


def bh_accel_subset(tree: OracleTree, x, y, z, targets, G, eps2, theta, stack_size_words=None,
                    threads=0):
    x, y, z = map(_f64, (x, y, z))
    targets = np.ascontiguousarray(targets, dtype=np.uint32)
    if stack_size_words is None:
        stack_size_words = stack_size(tree.n)
    k = len(targets)
    ax, ay, az = (np.zeros(k) for _ in range(3))
    _check(lib().orc_bh_accel_subset(tree.handle.ptr, _d(x), _d(y), _d(z), _u(targets), k, _d(ax),
                                     _d(ay), _d(az), G, eps2, theta, stack_size_words, threads),
           "bh_accel_subset")
    return ax, ay, az


def bh_interaction_counts(tree: OracleTree, x, y, z, theta, stack_size_words=None, threads=0):
    x, y, z = map(_f64, (x, y, z))
    if stack_size_words is None:
        stack_size_words = stack_size(tree.n)
    a = C.c_uint64(0)
    o = C.c_uint64(0)
    _check(lib().orc_bh_interaction_counts(tree.handle.ptr, _d(x), _d(y), _d(z), theta,
                                           stack_size_words, C.byref(a), C.byref(o), threads),
           "interaction_counts")
    return a.value, o.value
