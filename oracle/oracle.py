"""ORACLE — test infrastructure only.

ctypes wrapper of liboracle_astro.so, the CPU restatement of the osbo/astro
Barnes-Hut step (astro_oracle.h). Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use it, as the checker and the timed CPU
reference; the product never imports it.
"""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_uint32, c_uint64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle_astro.so"

# Layouts shared with the product (the reference's bridge.h records).
POSITION_MASS = np.dtype([("position", "<f4", (3,)), ("_pad0", "<f4"), ("mass", "<f4"),
                          ("_pad1", "<f4", (3,))])
VELOCITY_RADIUS = np.dtype([("velocity", "<f4", (3,)), ("_pad0", "<f4"), ("radius", "<f4"),
                            ("_pad1", "<f4", (3,))])
COLOR_TYPE = np.dtype([("color", "<f4", (4,)), ("type", "<u4"), ("_pad", "<u4", (3,))])
OCTREE_NODE = np.dtype([
    ("mortonCode", "<u8"), ("_pad0", "<u8"), ("centerOfMass", "<f4", (3,)), ("_pad1", "<f4"),
    ("totalMass", "<f4"), ("_pad2", "<f4", (3,)), ("emittedColor", "<f4", (4,)),
    ("emittedColorCenter", "<f4", (3,)), ("_pad3", "<f4"), ("children", "<u4", (8,)),
    ("layer", "<u4"), ("_pad4", "<u4", (3,)),
])


class Outputs(ctypes.Structure):
    _fields_ = [
        ("codes", c_void_p), ("sorted_codes", c_void_p), ("sorted_indices", c_void_p),
        ("layer_counts", c_void_p), ("layer_sizes", c_void_p), ("layer_offsets", c_void_p),
        ("nodes", c_void_p), ("acc4", c_void_p), ("interactions", c_uint64),
        ("node_visits", c_uint64), ("far_nodes", c_uint64), ("far_interactions", c_uint64),
        ("nodes_index", c_void_p), ("nodes_count", c_uint64),
    ]


_lib = None


def build() -> Path:
    res = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        l = ctypes.CDLL(str(LIB_PATH))
        l.oracle_set_threads.restype = c_int
        l.oracle_set_threads.argtypes = [c_int]
        l.oracle_interleave_bits.restype = c_uint64
        l.oracle_interleave_bits.argtypes = [c_uint32, c_uint32, c_uint32]
        l.oracle_generate_morton_codes.restype = None
        l.oracle_generate_morton_codes.argtypes = [c_void_p, c_void_p, c_void_p, c_uint32,
                                                   c_uint32, c_float]
        l.oracle_exclusive_scan.restype = None
        l.oracle_exclusive_scan.argtypes = [c_void_p, c_void_p, c_uint32]
        l.oracle_split_sort.restype = None
        l.oracle_split_sort.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_uint32]
        l.oracle_layer_layout.restype = c_uint64
        l.oracle_layer_layout.argtypes = [c_uint32, c_uint32, c_uint32, c_void_p, c_void_p]
        l.oracle_ref_run.restype = c_int
        l.oracle_ref_run.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_uint32,
                                     c_float, c_uint32, c_uint32, POINTER(Outputs)]
        l.oracle_phys_run.restype = c_int
        l.oracle_phys_run.argtypes = [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_uint32,
                                      c_float, c_uint32, c_uint32, c_void_p, POINTER(Outputs)]
        l.oracle_direct_accel_f64.restype = None
        l.oracle_direct_accel_f64.argtypes = [c_void_p, c_void_p, c_uint32, c_void_p, c_uint32,
                                              c_void_p, c_uint32, c_double, c_double, c_void_p]
        l.oracle_far_expand.restype = None
        l.oracle_far_expand.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p]
        l.oracle_splat.restype = None
        l.oracle_splat.argtypes = [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_void_p,
                                   c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p]
        l.oracle_lighting.restype = None
        l.oracle_lighting.argtypes = [c_void_p, c_void_p, c_uint32, c_uint32]
        _lib = l
    return _lib


def _p(a):
    return c_void_p(0) if a is None else c_void_p(a.ctypes.data)


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(n)


def interleave(x: int, y: int, z: int) -> int:
    return lib().oracle_interleave_bits(x, y, z)


def morton_codes(pm: np.ndarray, lbits: int = 6, offset: float = 1e6) -> np.ndarray:
    codes = np.zeros(len(pm), np.uint64)
    dup = np.zeros(len(pm), np.uint64)
    lib().oracle_generate_morton_codes(_p(pm), _p(codes), _p(dup), len(pm), lbits, offset)
    return codes


def exclusive_scan(values: np.ndarray) -> np.ndarray:
    v = np.ascontiguousarray(values, np.uint32)
    out = np.zeros_like(v)
    lib().oracle_exclusive_scan(_p(v), _p(out), len(v))
    return out


def split_sort(keys: np.ndarray, idx: np.ndarray | None = None, passes: int = 64):
    k = np.ascontiguousarray(keys, np.uint64)
    i = np.arange(len(k), dtype=np.uint32) if idx is None else np.ascontiguousarray(idx, np.uint32)
    ok = np.zeros_like(k)
    oi = np.zeros_like(i)
    lib().oracle_split_sort(_p(k), _p(i), _p(ok), _p(oi), len(k), passes)
    return ok, oi


def layer_layout(count: int, lbits: int):
    sizes = np.zeros(lbits + 1, np.uint32)
    offsets = np.zeros(lbits + 1, np.uint32)
    cap = lib().oracle_layer_layout(count, 1, lbits, _p(sizes), _p(offsets))
    return sizes, offsets, int(cap)


def _outputs(n_tree: int, n: int, layers: int, capacity: int):
    bufs = dict(
        codes=np.zeros(n_tree, np.uint64), sorted_codes=np.zeros(n_tree, np.uint64),
        sorted_indices=np.zeros(n_tree, np.uint32), layer_counts=np.zeros(layers, np.uint32),
        layer_sizes=np.zeros(layers, np.uint32), layer_offsets=np.zeros(layers, np.uint32),
        nodes=np.zeros(capacity, OCTREE_NODE), acc4=np.zeros((n, 4), np.float32))
    out = Outputs(**{k: _p(v) for k, v in bufs.items()})
    return bufs, out


def ref_run(params, pm, vr, ct=None, n_tree=None, dt=1.0 / 30.0, steps=1, split_passes=64):
    """REFERENCE preset: run `steps` frames in place; returns the outputs of
    the last frame's force evaluation."""
    n = len(pm)
    n_tree = n if n_tree is None else n_tree
    layers = params.lbits + 1
    _, _, cap = layer_layout(n_tree, params.lbits)
    bufs, out = _outputs(n_tree, n, layers, cap)
    r = lib().oracle_ref_run(ctypes.addressof(params), _p(pm), _p(vr), _p(ct), n, n_tree, dt,
                             steps, split_passes, ctypes.byref(out))
    if r != 0:
        raise RuntimeError(f"oracle_ref_run failed ({r})")
    return bufs


def phys_capacity(sizes, lbits: int) -> int:
    cap = 0
    for l in range(lbits + 1):
        possible = 1 << min(40, 3 * (lbits - l))
        cap += sum(min(int(s), possible) for s in sizes)
    return cap


def phys_run(params, pm, vr, sizes=None, dt=1e-3, steps=1, split_passes=0, want_pos64=False,
             nodes=None):
    """PHYSICAL preset: `steps` steps in place over one or several systems.
    nodes (an array of node slots) returns only those slots, in that order
    (for trees too large to hold whole as OctreeNode records)."""
    n = len(pm)
    sizes = [n] if sizes is None else [int(s) for s in sizes]
    layers = params.lbits + 1
    cap = phys_capacity(sizes, params.lbits)
    if nodes is not None:
        index = np.ascontiguousarray(nodes, np.uint64)
        bufs, out = _outputs(n, n, layers, len(index))
        bufs["_nodes_index"] = index
        out.nodes_index, out.nodes_count = _p(index), len(index)
    else:
        bufs, out = _outputs(n, n, layers, cap)
    sz = np.ascontiguousarray(sizes, np.uint32)
    pos64 = np.zeros((n, 3), np.float64) if want_pos64 else None
    r = lib().oracle_phys_run(ctypes.addressof(params), _p(pm), _p(vr), n, _p(sz), len(sz), dt,
                              steps, split_passes, _p(pos64), ctypes.byref(out))
    if r != 0:
        raise RuntimeError(f"oracle_phys_run failed ({r})")
    bufs["interactions"] = out.interactions
    bufs["node_visits"] = out.node_visits
    bufs["far_nodes"] = out.far_nodes
    bufs["far_interactions"] = out.far_interactions
    if want_pos64:
        bufs["pos64"] = pos64
    return bufs


def far_expand(params, cm4, q5, gc3, rho3):
    """(coefficients[19], G * expansion at rho3) of one far node about gc3."""
    f = lambda v: np.ascontiguousarray(v, np.float32)
    cm4, q5, gc3, rho3 = f(cm4), f(q5), f(gc3), f(rho3)
    co = np.zeros(19, np.float32)
    acc = np.zeros(3, np.float32)
    lib().oracle_far_expand(ctypes.addressof(params), _p(cm4), _p(q5), _p(gc3), _p(rho3), _p(co),
                            _p(acc))
    return co, acc


def direct_accel(pm, samples, g=1.0, eps=0.01, sizes=None, pos64=None) -> np.ndarray:
    s = np.ascontiguousarray(samples, np.uint32)
    out = np.zeros((len(s), 3), np.float64)
    sz = None if sizes is None else np.ascontiguousarray(sizes, np.uint32)
    lib().oracle_direct_accel_f64(_p(pm), _p(pos64), len(pm), _p(sz), 0 if sz is None else len(sz),
                                  _p(s), len(s), g, eps, _p(out))
    return out


def lighting(pm, ct, num_stars=5):
    """lightingPass on a copy of ct (ColorType[]); returns the new colours."""
    pm = np.ascontiguousarray(pm)
    out = np.array(ct, copy=True)
    lib().oracle_lighting(_p(pm), _p(out), len(pm), num_stars)
    return out


def splat(pm, vr, ct, camera, width, height, clear=(0.0, 0.0, 1.0 / 255.0, 1.0)):
    """The headless splat drawn sequentially: (rgba[h, w, 4], depth[h, w]).
    camera: astro_gb300.render.Camera (view, projection, position)."""
    n = len(pm)
    view = np.ascontiguousarray(camera.view, np.float32).reshape(16)
    proj = np.ascontiguousarray(camera.projection, np.float32).reshape(16)
    pos = np.ascontiguousarray(camera.position, np.float32).reshape(3)
    cl = np.ascontiguousarray(clear, np.float32)
    rgba = np.zeros((height, width, 4), np.float32)
    depth = np.zeros((height, width), np.float32)
    lib().oracle_splat(_p(np.ascontiguousarray(pm)), _p(np.ascontiguousarray(vr)),
                       _p(np.ascontiguousarray(ct)), n, _p(view), _p(proj), _p(pos), width, height,
                       _p(cl), _p(rgba), _p(depth))
    return rgba, depth
