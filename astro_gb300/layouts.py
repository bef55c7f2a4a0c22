"""Byte layouts of include/astro_cuda.h as numpy dtypes and ctypes structures.

The particle and node records keep the reference's layouts (Astro/bridge.h:
17-65): Metal's float3 occupies 16 bytes, so PositionMass, VelocityRadius and
ColorType are 32-byte records and OctreeNode is a 128-byte record.
"""
from __future__ import annotations

import ctypes

import numpy as np

INVALID_MORTON_CODE = 0xFFFFFFFFFFFFFFFF  # bridge.h:91-94
INVALID_CHILD = 0xFFFFFFFF  # Octree.metal:10
MAX_LBITS = 21
MAX_LAYERS = MAX_LBITS + 1

PRESET_REFERENCE = 0
PRESET_PHYSICAL = 1
FORM_PLAIN = 0
FORM_PRECISION = 1
FLAG_IEEE_EXACT = 0x1
FLAG_NO_GRAPH = 0x2
FLAG_PERSISTENT = 0x4
FLAG_OPEN_DELTA = 0x8
FLAG_QUADRUPOLE = 0x10
FLAG_PER_PARTICLE = 0x20
# astro_autotune_keep: knobs held at the context's values.
TUNE_KEEP_LBITS = 0x1
TUNE_KEEP_GROUP_SIZE = 0x2
TUNE_KEEP_ACCURACY = 0x4

IC_PLUMMER = 0
IC_DISK_BULGE = 1
IC_TWO_PLUMMER = 2
IC_UNIFORM_CUBE = 3
IC_REFERENCE_SCENE = 4

POSITION_MASS = np.dtype([("position", "<f4", (3,)), ("_pad0", "<f4"), ("mass", "<f4"),
                          ("_pad1", "<f4", (3,))], align=False)
VELOCITY_RADIUS = np.dtype([("velocity", "<f4", (3,)), ("_pad0", "<f4"), ("radius", "<f4"),
                            ("_pad1", "<f4", (3,))], align=False)
COLOR_TYPE = np.dtype([("color", "<f4", (4,)), ("type", "<u4"), ("_pad", "<u4", (3,))],
                      align=False)
OCTREE_NODE = np.dtype([
    ("mortonCode", "<u8"), ("_pad0", "<u8"),
    ("centerOfMass", "<f4", (3,)), ("_pad1", "<f4"),
    ("totalMass", "<f4"), ("_pad2", "<f4", (3,)),
    ("emittedColor", "<f4", (4,)),
    ("emittedColorCenter", "<f4", (3,)), ("_pad3", "<f4"),
    ("children", "<u4", (8,)),
    ("layer", "<u4"), ("_pad4", "<u4", (3,)),
], align=False)

assert POSITION_MASS.itemsize == 32 and VELOCITY_RADIUS.itemsize == 32
assert COLOR_TYPE.itemsize == 32 and OCTREE_NODE.itemsize == 128
assert OCTREE_NODE.fields["totalMass"][1] == 32 and OCTREE_NODE.fields["children"][1] == 80
assert OCTREE_NODE.fields["layer"][1] == 112


class Params(ctypes.Structure):
    """astro_params: every constant the reference hard-codes."""

    _fields_ = [
        ("preset", ctypes.c_uint32),
        ("form", ctypes.c_uint32),
        ("lbits", ctypes.c_uint32),
        ("flags", ctypes.c_uint32),
        ("theta", ctypes.c_float),
        ("g", ctypes.c_float),
        ("softening", ctypes.c_float),
        ("leaf_min_dist2", ctypes.c_float),
        ("force_clamp", ctypes.c_float),
        ("quant_offset", ctypes.c_float),
        ("damping", ctypes.c_float),
        ("type_accel_scale", ctypes.c_float * 3),
        ("bucket", ctypes.c_uint32),
        ("block_warps", ctypes.c_uint32),
        ("group_size", ctypes.c_uint32),
        ("sort_variant", ctypes.c_uint32),
        ("light_sources", ctypes.c_uint32),
        ("open_delta_weight", ctypes.c_float),
        ("far_ratio", ctypes.c_float),
        ("walk_frontier", ctypes.c_uint32),
    ]

    def replace(self, **kw) -> "Params":
        out = Params()
        ctypes.pointer(out)[0] = self
        for k, v in kw.items():
            if k == "type_accel_scale":
                out.type_accel_scale = (ctypes.c_float * 3)(*v)
            else:
                setattr(out, k, v)
        return out

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_ if not f.startswith("_")}
        d["type_accel_scale"] = list(self.type_accel_scale)
        return d


def host_default_params(preset: int = PRESET_PHYSICAL, **overrides) -> Params:
    """astro_params_default restated on the host (no library load): for
    callers that only hand parameters to a CPU implementation. A CPU test
    checks that both give the same bytes."""
    p = Params()
    p.preset = preset
    p.form = FORM_PLAIN
    p.lbits = 6                 # MortonCode.metal:47-50
    p.theta = 0.7               # Renderer.swift:864
    p.open_delta_weight = 1.0
    p.force_clamp = 1e5         # BarnesHut.metal:100
    if preset == PRESET_REFERENCE:
        p.g = 1e11              # BarnesHut.metal:39
        p.softening = 0.01      # BarnesHut.metal:40
        p.leaf_min_dist2 = 50.0  # BarnesHut.metal:70
        p.quant_offset = 1e6    # MortonCode.metal:35-37
        p.damping = 0.9995      # BarnesHut.metal:189
        p.type_accel_scale = (ctypes.c_float * 3)(5.0, 5.0, 1.0)  # BarnesHut.metal:181-187
        p.light_sources = 5     # numStars (Renderer.swift:26)
    elif preset == PRESET_PHYSICAL:
        p.g = 1.0
        p.softening = 0.01
        p.damping = 1.0
        p.type_accel_scale = (ctypes.c_float * 3)(1.0, 1.0, 1.0)
        p.bucket = 16
        p.flags = FLAG_OPEN_DELTA | FLAG_QUADRUPOLE
    else:
        raise ValueError(f"unknown preset {preset}")
    return p.replace(**overrides) if overrides else p


def empty_particles(n: int):
    """Zeroed PositionMass and VelocityRadius arrays of length n."""
    return np.zeros(n, POSITION_MASS), np.zeros(n, VELOCITY_RADIUS)


STATE_MAGIC = b"ASTROST1"
STATE_VERSION = 1
STATE_TYPES = 0x1
STATE_POS64 = 0x2


class StateHeader(ctypes.Structure):
    """astro_state_header: the fixed part of a state file."""

    _fields_ = [
        ("magic", ctypes.c_char * 8),
        ("version", ctypes.c_uint32),
        ("header_bytes", ctypes.c_uint32),
        ("params", Params),
        ("step", ctypes.c_uint64),
        ("time", ctypes.c_double),
        ("n", ctypes.c_uint32),
        ("n_tree", ctypes.c_uint32),
        ("nsys", ctypes.c_uint32),
        ("contents", ctypes.c_uint32),
    ]


def read_state(path):
    """Parse a state file on the host: (header, sys_sizes, pm, vr, ids, types
    or None, pos64 or None), arrays in the saved slot order."""
    import numpy as np

    raw = open(path, "rb").read()
    h = StateHeader.from_buffer_copy(raw[:ctypes.sizeof(StateHeader)])
    if h.magic != STATE_MAGIC or h.version != STATE_VERSION:
        raise ValueError("not an astro state file")
    off = h.header_bytes
    n = h.n

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off).copy()
        off += a.nbytes
        return a

    sizes = take(np.uint32, h.nsys)
    pm = take(POSITION_MASS, n)
    vr = take(VELOCITY_RADIUS, n)
    ids = take(np.uint32, n)
    types = take(np.uint32, n) if h.contents & STATE_TYPES else None
    pos64 = take(np.float64, 3 * n).reshape(n, 3) if h.contents & STATE_POS64 else None
    if off != len(raw):
        raise ValueError("state file size does not match its header")
    return h, sizes, pm, vr, ids, types, pos64


class CameraABI(ctypes.Structure):
    """astro_camera: column-major view and projection matrices, camera position."""

    _fields_ = [
        ("view", ctypes.c_float * 16),
        ("projection", ctypes.c_float * 16),
        ("position", ctypes.c_float * 3),
        ("_pad", ctypes.c_float),
    ]
