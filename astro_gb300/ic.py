"""Seeded initial conditions for the benchmark workloads (host C++ in the library).

Each workload is described by its sizes and distribution; the particles come
from astro_generate_ic (Philox4x32-10 streams keyed by seed, system and
particle), so every host generates the same set.
"""
from __future__ import annotations

from ctypes import c_void_p

import numpy as np

from . import layouts as L
from ._native import check, lib, ptr

# The library whose astro_generate_ic / astro_generate_system_sizes make the
# particles: libastro_cuda unless a caller names another build of the same
# host source (ic.cpp) with use_generator_library().
_generator = None


def use_generator_library(cdll) -> None:
    """Generate with `cdll` (a ctypes library exporting astro_generate_ic and
    astro_generate_system_sizes from the same source); None restores the
    default."""
    global _generator
    if cdll is not None:
        from ctypes import c_double, c_int, c_uint32, c_uint64

        cdll.astro_generate_ic.restype = c_int
        cdll.astro_generate_ic.argtypes = [c_uint32, c_uint64, c_uint32, c_uint32, c_double,
                                           c_double, c_void_p, c_void_p, c_void_p]
        cdll.astro_generate_system_sizes.restype = c_int
        cdll.astro_generate_system_sizes.argtypes = [c_uint64, c_uint32, c_uint32, c_uint32,
                                                     c_double, c_double, c_void_p, c_void_p]
    _generator = cdll


def _gen():
    return _generator if _generator is not None else lib()


def generate(kind: int, n: int, seed: int, system: int = 0, p0: float = 0.0, p1: float = 0.0,
             with_colors: bool = False):
    pm, vr = L.empty_particles(n)
    ct = np.zeros(n, L.COLOR_TYPE) if with_colors else None
    check(_gen().astro_generate_ic(kind, seed, system, n, p0, p1, ptr(pm), ptr(vr),
                                  ptr(ct) if ct is not None else c_void_p(0)))
    return (pm, vr, ct) if with_colors else (pm, vr)


def plummer(n: int, seed: int, a: float = 1.0, mass: float = 1.0, system: int = 0):
    return generate(L.IC_PLUMMER, n, seed, system, a, mass)


def disk_bulge(n: int, seed: int):
    return generate(L.IC_DISK_BULGE, n, seed)


def two_plummer(n: int, seed: int, separation: float = 10.0):
    return generate(L.IC_TWO_PLUMMER, n, seed, 0, separation)


def uniform_cube(n: int, seed: int, sigma_v: float = 0.1, sigma_logm: float = 0.5):
    return generate(L.IC_UNIFORM_CUBE, n, seed, 0, sigma_v, sigma_logm)


def reference_scene(n_stars: int = 5, n_planets: int = 200, n_dust: int = 500000, seed: int = 0):
    """The reference's scene (Renderer.swift:25-46): stars and planets in the
    tree, dust as tracers."""
    n = n_stars + n_planets + n_dust
    return generate(L.IC_REFERENCE_SCENE, n, seed, 0, n_stars, n_planets, with_colors=True)


def system_sizes(nsys: int, seed: int, n_min: int = 1024, n_max: int = 65536,
                 a_min: float = 0.5, a_max: float = 2.0):
    sizes = np.zeros(nsys, np.uint32)
    scales = np.zeros(nsys, np.float64)
    check(_gen().astro_generate_system_sizes(seed, nsys, n_min, n_max, a_min, a_max, ptr(sizes),
                                            ptr(scales)))
    return sizes, scales


def plummer_batch(nsys: int, seed: int, n_min: int = 1024, n_max: int = 65536):
    """Independent Plummer spheres (M = 1, a uniform in [0.5, 2]) of
    log-uniform sizes, back to back."""
    sizes, scales = system_sizes(nsys, seed, n_min, n_max)
    parts = [plummer(int(sz), seed, float(a), 1.0, system=s)
             for s, (sz, a) in enumerate(zip(sizes, scales))]
    pm = np.concatenate([p for p, _ in parts])
    vr = np.concatenate([v for _, v in parts])
    return pm, vr, sizes
