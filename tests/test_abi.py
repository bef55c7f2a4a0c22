"""The C ABI library: symbols, layouts, parameter defaults and host-only entry
points (no GPU needed)."""
import ctypes
import re
import subprocess
from ctypes import byref, c_size_t, c_void_p
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(astro_[a-z0-9_]+)\s*\(",
                             text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(native):
    from astro_gb300 import _native

    lib = _native.lib()
    declared = declared_functions()
    assert len(declared) >= 25
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    # The Python binding covers the same set.
    assert declared == set(_native.SIGNATURES), declared ^ set(_native.SIGNATURES)


def test_header_layouts_compile_with_gcc(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(f"""
#include <stddef.h>
#include "{ROOT / 'include' / 'astro_cuda.h'}"
_Static_assert(sizeof(PositionMass) == 32, "PositionMass");
_Static_assert(offsetof(PositionMass, mass) == 16, "mass");
_Static_assert(sizeof(VelocityRadius) == 32, "VelocityRadius");
_Static_assert(offsetof(VelocityRadius, radius) == 16, "radius");
_Static_assert(sizeof(ColorType) == 32, "ColorType");
_Static_assert(offsetof(ColorType, type) == 16, "type");
_Static_assert(sizeof(OctreeNode) == 128, "OctreeNode");
_Static_assert(offsetof(OctreeNode, centerOfMass) == 16, "com");
_Static_assert(offsetof(OctreeNode, totalMass) == 32, "mass");
_Static_assert(offsetof(OctreeNode, emittedColor) == 48, "ec");
_Static_assert(offsetof(OctreeNode, emittedColorCenter) == 64, "ecc");
_Static_assert(offsetof(OctreeNode, children) == 80, "children");
_Static_assert(offsetof(OctreeNode, layer) == 112, "layer");
_Static_assert(offsetof(astro_params, block_warps) == 60, "block_warps");
_Static_assert(offsetof(astro_params, group_size) == 64, "group_size");
_Static_assert(offsetof(astro_params, sort_variant) == 68, "sort_variant");
_Static_assert(offsetof(astro_params, open_delta_weight) == 76, "open_delta_weight");
_Static_assert(offsetof(astro_params, far_ratio) == 80, "far_ratio");
_Static_assert(offsetof(astro_params, walk_frontier) == 84, "walk_frontier");
_Static_assert(sizeof(astro_params) == 88, "astro_params");
_Static_assert(sizeof(astro_state_header) == 136, "astro_state_header");
_Static_assert(offsetof(astro_state_header, params) == 16, "state params");
_Static_assert(offsetof(astro_state_header, n) == 120, "state n");
int main(void) {{ return 0; }}
""")
    res = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-c", str(src), "-o",
                          str(tmp_path / "layout.o")], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


def test_python_layouts_match_header():
    from astro_gb300 import layouts as L

    assert ctypes.sizeof(L.Params) == 4 * 4 + 4 * 7 + 4 * 3 + 4 * 2 + 4 * 6 == 88
    assert L.Params.group_size.offset == 64 and L.Params.sort_variant.offset == 68
    assert ctypes.sizeof(L.StateHeader) == 136 and L.StateHeader.n.offset == 120


def test_load_state_rejects_bad_files_without_device(native, tmp_path):
    from astro_gb300 import layouts as L
    from astro_gb300._native import lib

    h = c_void_p()
    missing = str(tmp_path / "absent.state").encode()
    assert lib().astro_load_state(missing, 0, byref(h), None, None) == -1
    bad = tmp_path / "bad.state"
    bad.write_bytes(b"NOTSTATE" + bytes(200))
    assert lib().astro_load_state(str(bad).encode(), 0, byref(h), None, None) == -1
    # A valid header whose arrays are cut short.
    hdr = L.StateHeader(magic=L.STATE_MAGIC, version=L.STATE_VERSION,
                        header_bytes=ctypes.sizeof(L.StateHeader), n=10, n_tree=10, nsys=1)
    lib().astro_params_default(L.PRESET_PHYSICAL, byref(hdr.params))
    short = tmp_path / "short.state"
    short.write_bytes(bytes(hdr) + bytes(64))
    assert lib().astro_load_state(str(short).encode(), 0, byref(h), None, None) == -1
    assert not h.value
    assert L.OCTREE_NODE.itemsize == 128 and L.POSITION_MASS.itemsize == 32


def test_params_defaults(native):
    from astro_gb300 import layouts as L
    from astro_gb300._native import lib

    p = L.Params()
    assert lib().astro_params_default(L.PRESET_REFERENCE, byref(p)) == 0
    # The reference's literal constants (BarnesHut.metal:39-40,70,100,181-190;
    # MortonCode.metal:35-50; Renderer.swift:864).
    assert (p.lbits, p.theta, p.g, p.softening, p.leaf_min_dist2, p.force_clamp) == (
        6, pytest.approx(0.7), pytest.approx(1e11), pytest.approx(0.01), 50.0, 1e5)
    assert p.quant_offset == 1e6 and p.damping == pytest.approx(0.9995)
    assert list(p.type_accel_scale) == [5.0, 5.0, 1.0]
    assert p.light_sources == 5  # numStars (Renderer.swift:26)
    assert lib().astro_params_default(L.PRESET_PHYSICAL, byref(p)) == 0
    assert p.g == 1.0 and p.bucket == 16 and p.light_sources == 0 and p.open_delta_weight == 1.0
    assert lib().astro_params_default(7, byref(p)) == -1


def test_argument_errors_without_device(native):
    from astro_gb300 import layouts as L
    from astro_gb300._native import lib

    p = L.Params()
    lib().astro_params_default(L.PRESET_PHYSICAL, byref(p))
    h = c_void_p()
    bad = p.replace(lbits=0)
    assert lib().astro_create(byref(bad), 100, 1, byref(h)) == -1
    bad = p.replace(theta=-1.0)
    assert lib().astro_create(byref(bad), 100, 1, byref(h)) == -1
    bad = p.replace(group_size=65)
    assert lib().astro_create(byref(bad), 100, 1, byref(h)) == -1
    bad = p.replace(sort_variant=13)
    assert lib().astro_create(byref(bad), 100, 1, byref(h)) == -1
    bad = p.replace(open_delta_weight=-1.0)
    assert lib().astro_create(byref(bad), 100, 1, byref(h)) == -1
    bad = p.replace(walk_frontier=2)
    assert lib().astro_create(byref(bad), 100, 1, byref(h)) == -1
    for ratio in (-0.1, 0.6, float("nan")):
        bad = p.replace(far_ratio=ratio)
        assert lib().astro_create(byref(bad), 100, 1, byref(h)) == -1
    bad = p.replace(light_sources=5)  # lighting needs the REFERENCE preset
    assert lib().astro_create(byref(bad), 100, 1, byref(h)) == -1
    bad = L.Params()
    lib().astro_params_default(L.PRESET_REFERENCE, byref(bad))
    bad.form = L.FORM_PRECISION
    assert lib().astro_create(byref(bad), 100, 1, byref(h)) == -1
    assert lib().astro_create(byref(p), 0, 1, byref(h)) == -1
    assert lib().astro_destroy(None) == -1
    assert lib().astro_step(None, 0.1, 1) == -1
    assert lib().astro_radix_sort(None, None, None, None, 10, None, 64, None, 0, None) == -1
    assert lib().astro_radix_sort(None, None, None, None, 0, None, 64, None, 0, None) == 0
    assert lib().astro_status_string(-6) == b"device-side wait timed out"
    assert lib().astro_version().startswith(b"astro_gb300")


def test_sort_temp_bytes(native):
    from astro_gb300._native import lib

    b18, b64 = c_size_t(), c_size_t()
    assert lib().astro_radix_sort_temp_bytes(1 << 20, 18, byref(b18)) == 0
    assert lib().astro_radix_sort_temp_bytes(1 << 20, 64, byref(b64)) == 0
    # Ping-pong pairs (12 B each) plus per-pass histograms and look-back words.
    assert b18.value >= 12 * (1 << 20) and b64.value > b18.value
    assert lib().astro_radix_sort_temp_bytes(10, 65, byref(b18)) == -1


def test_generators_are_seeded_and_deterministic(native):
    from astro_gb300 import ic

    a, va = ic.plummer(5000, seed=1001)
    b, vb = ic.plummer(5000, seed=1001)
    c, _ = ic.plummer(5000, seed=1002)
    assert np.array_equal(a, b) and np.array_equal(va, vb)
    assert not np.array_equal(a, c)
    assert a["mass"].sum() == pytest.approx(1.0, rel=1e-5)
    # Plummer half-mass radius is about 1.305 a.
    r = np.linalg.norm(a["position"], axis=1)
    assert 1.15 < np.median(r) < 1.45
    # Virial ratio 2T/|W| of an equilibrium Plummer sphere is about 1
    # (T = 3 pi M^2 / 64 a with G = M = a = 1).
    T = 0.5 * np.sum(a["mass"] * np.sum(va["velocity"].astype(np.float64) ** 2, axis=1))
    assert T == pytest.approx(3 * np.pi / 64, rel=0.15)
    sizes, scales = ic.system_sizes(256, seed=1004)
    assert sizes.min() >= 1024 and sizes.max() <= 65536
    assert 2.0e6 < sizes.sum() < 6.5e6 and 0.5 <= scales.min() and scales.max() <= 2.0
    pm, vr = ic.uniform_cube(10000, seed=1005)
    assert pm["mass"].sum() == pytest.approx(1.0, rel=1e-4)
    assert pm["position"].min() >= 0 and pm["position"].max() <= 1
    pm, vr = ic.disk_bulge(10000, seed=1002)
    assert pm["mass"].sum() == pytest.approx(1.0, rel=1e-4)
    pm, vr = ic.two_plummer(10000, seed=1003)
    assert abs(pm["position"][:5000, 0].mean() + 5) < 0.5 and abs(pm["position"][5000:, 0].mean() - 5) < 0.5
