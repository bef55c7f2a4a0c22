"""Host-side mirror of the reference's per-frame compute (Renderer).

``Simulation`` owns one libastro_cuda context. Its methods follow the
reference's Renderer (Astro/Renderer.swift): ``make_buffers`` /
``make_spheres`` become the constructor and ``upload``, ``draw`` runs the
compute section of a frame, and the stage methods ``generate_morton_codes``,
``sort``, ``build_tree``, ``barnes_hut`` and ``update_spheres`` run one stage
each, in the reference's order (Renderer.swift:505-542).
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_uint32, c_uint64, c_void_p

import numpy as np

from . import layouts as L
from ._native import check, lib, ptr


def default_params(preset: int = L.PRESET_PHYSICAL, **overrides) -> L.Params:
    p = L.Params()
    check(lib().astro_params_default(preset, byref(p)))
    return p.replace(**overrides) if overrides else p


class Simulation:
    """One Barnes-Hut context on the current CUDA device."""

    def __init__(self, params: L.Params | None = None, max_n: int = 1 << 20,
                 max_systems: int = 1):
        self.params = params if params is not None else default_params()
        h = c_void_p()
        check(lib().astro_create(byref(self.params), max_n, max_systems, byref(h)))
        self._h = h
        self.max_n = max_n
        self.n = 0
        self.n_tree = 0
        self.sys_sizes: list[int] = []
        self._async_refs: list = []  # host arrays of queued asynchronous transfers

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if self._h:
            lib().astro_destroy(self._h)
            self._h = c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, status: int) -> None:
        check(status, self._h)

    # -- parameters -------------------------------------------------------
    def set_params(self, params: L.Params) -> None:
        self._check(lib().astro_set_params(self._h, byref(params)))
        self.params = params

    # -- state ------------------------------------------------------------
    def upload(self, pm: np.ndarray, vr: np.ndarray, ct: np.ndarray | None = None,
               n_tree: int | None = None) -> None:
        """Copy one system in (Renderer.makeSpheres' buffer copy)."""
        pm = np.ascontiguousarray(pm, dtype=L.POSITION_MASS)
        vr = np.ascontiguousarray(vr, dtype=L.VELOCITY_RADIUS)
        n = len(pm)
        n_tree = n if n_tree is None else n_tree
        if ct is not None:
            ct = np.ascontiguousarray(ct, dtype=L.COLOR_TYPE)
        self._check(lib().astro_upload(self._h, ptr(pm), ptr(vr), ptr(ct), n, n_tree))
        self.n, self.n_tree, self.sys_sizes = n, n_tree, [n_tree]

    def upload_systems(self, pm: np.ndarray, vr: np.ndarray, sizes) -> None:
        """Copy several independent systems in, laid out back to back."""
        pm = np.ascontiguousarray(pm, dtype=L.POSITION_MASS)
        vr = np.ascontiguousarray(vr, dtype=L.VELOCITY_RADIUS)
        sz = np.ascontiguousarray(sizes, dtype=np.uint32)
        arr = (c_uint32 * len(sz)).from_buffer(sz)
        self._check(lib().astro_upload_systems(self._h, ptr(pm), ptr(vr), arr, len(sz)))
        self.n = self.n_tree = int(sz.sum())
        self.sys_sizes = [int(s) for s in sz]

    def upload_async(self, pm: np.ndarray, vr: np.ndarray) -> None:
        """Replace the particles with len(pm) new ones in the last upload's
        layout, without waiting: the copy overlaps the steps queued before
        it. The arrays (pinned memory for the overlap) are kept alive until
        synchronize()."""
        if pm.dtype != L.POSITION_MASS or vr.dtype != L.VELOCITY_RADIUS or \
                not (pm.flags.c_contiguous and vr.flags.c_contiguous):
            raise TypeError("upload_async needs contiguous POSITION_MASS / VELOCITY_RADIUS arrays")
        self._check(lib().astro_upload_async(self._h, ptr(pm), ptr(vr), len(pm)))
        self._async_refs.extend((pm, vr))

    def download_async(self, pm: np.ndarray, vr: np.ndarray) -> None:
        """Queue a copy of the state (as after the steps queued so far) into
        pm and vr without waiting; they hold it once synchronize() returns."""
        if pm.dtype != L.POSITION_MASS or vr.dtype != L.VELOCITY_RADIUS or \
                not (pm.flags.c_contiguous and vr.flags.c_contiguous) or not pm.flags.writeable:
            raise TypeError("download_async needs writable contiguous POSITION_MASS / "
                            "VELOCITY_RADIUS arrays")
        self._check(lib().astro_download_async(self._h, ptr(pm), ptr(vr), self.n))
        self._async_refs.extend((pm, vr))

    def download(self, pm: np.ndarray | None = None, vr: np.ndarray | None = None):
        pm = np.zeros(self.n, L.POSITION_MASS) if pm is None else pm
        vr = np.zeros(self.n, L.VELOCITY_RADIUS) if vr is None else vr
        self._check(lib().astro_download(self._h, ptr(pm), ptr(vr), self.n))
        return pm, vr

    # -- state files (makeSpheres / resetSimulation without regeneration) --
    def save_state(self, path, step: int = 0, time: float = 0.0) -> None:
        """Write the state between steps (include/astro_cuda.h: state files)."""
        self._check(lib().astro_save_state(self._h, str(path).encode(), step, time))

    @classmethod
    def load_state(cls, path, max_n: int = 0) -> tuple["Simulation", int, float]:
        """A new context restored from a state file, with the saved step
        count and time."""
        h = c_void_p()
        step, t = c_uint64(), ctypes.c_double()
        check(lib().astro_load_state(str(path).encode(), max_n, byref(h), byref(step), byref(t)))
        sim = cls.__new__(cls)
        sim._h = h
        p = L.Params()
        sim._check(lib().astro_get_params(h, byref(p)))
        hdr, sizes, *_ = L.read_state(path)
        sim.params = p
        sim.max_n = max(max_n, hdr.n)
        sim.n, sim.n_tree = hdr.n, hdr.n_tree
        sim.sys_sizes = [int(s) for s in sizes]
        sim._async_refs = []
        return sim, step.value, t.value

    # -- stages (Renderer.draw order) -------------------------------------
    def generate_morton_codes(self) -> None:
        self._check(lib().astro_encode(self._h))

    def sort(self) -> None:
        self._check(lib().astro_sort(self._h))

    def build_tree(self) -> None:
        self._check(lib().astro_build(self._h))

    def barnes_hut(self) -> None:
        self._check(lib().astro_traverse(self._h))

    def update_spheres(self, dt: float) -> None:
        self._check(lib().astro_integrate(self._h, dt))

    def lighting_pass(self, num_stars: int = 5) -> None:
        """lightingPass (BarnesHut.metal:103-167), REFERENCE preset."""
        self._check(lib().astro_lighting(self._h, num_stars))

    def read_colors(self) -> np.ndarray:
        """ColorType of every particle in upload order (REFERENCE preset)."""
        ct = np.zeros(self.n, L.COLOR_TYPE)
        self._check(lib().astro_read_colors(self._h, ptr(ct), self.n))
        return ct

    def splat(self, camera, width: int, height: int, clear=None):
        """Headless scene pass (astro_splat): (rgba[h, w, 4], depth[h, w])."""
        from .render import to_abi

        cam = to_abi(camera)
        rgba = np.zeros((height, width, 4), np.float32)
        depth = np.zeros((height, width), np.float32)
        cl = None if clear is None else np.ascontiguousarray(clear, np.float32)
        self._check(lib().astro_splat(self._h, byref(cam), width, height, ptr(cl), ptr(rgba),
                                      ptr(depth)))
        return rgba, depth

    def draw(self, dt: float, steps: int = 1) -> None:
        """Run `steps` full steps (graph-replayed unless FLAG_NO_GRAPH)."""
        self._check(lib().astro_step(self._h, dt, steps))

    def draw_batched(self, dt: float, steps: int, sizes) -> None:
        """`steps` steps of the systems uploaded by upload_systems (sizes must
        equal them)."""
        sz = np.ascontiguousarray(sizes, dtype=np.uint32)
        self._check(lib().astro_step_batched(self._h, ptr(sz), len(sz), dt, steps))

    def autotune(self, path=None, target: float = 1e-3, samples: int = 1024, keep: int = 0) -> dict:
        """Native autotuner (astro_autotune_keep) on the current particles,
        holding the knobs of `keep` (TUNE_KEEP_* bits): the best knobs are
        applied to this context; returns the result record (knobs, step
        time, error, trials)."""
        import json
        import os
        import tempfile

        tmp = None
        if path is None:
            fd, tmp = tempfile.mkstemp(suffix=".json")
            os.close(fd)
            path = tmp
        try:
            self._check(lib().astro_autotune_keep(self._h, str(path).encode(), target, samples, keep))
            with open(path) as f:
                out = json.load(f)
        finally:
            if tmp:
                os.unlink(tmp)
        p = L.Params()
        self._check(lib().astro_get_params(self._h, byref(p)))
        self.params = p
        return out

    def synchronize(self) -> None:
        try:
            self._check(lib().astro_synchronize(self._h))
        finally:
            self._async_refs.clear()

    @property
    def stream(self) -> int:
        s = c_void_p()
        self._check(lib().astro_get_stream(self._h, byref(s)))
        return s.value or 0

    # -- readbacks --------------------------------------------------------
    def read_keys(self):
        n = self.n_tree
        codes = np.zeros(n, np.uint64)
        sorted_codes = np.zeros(n, np.uint64)
        idx = np.zeros(n, np.uint32)
        self._check(lib().astro_read_keys(self._h, ptr(codes), ptr(sorted_codes), ptr(idx), n))
        return codes, sorted_codes, idx

    def tree_info(self):
        nl = c_uint32()
        sizes = np.zeros(L.MAX_LAYERS, np.uint32)
        offsets = np.zeros(L.MAX_LAYERS, np.uint32)
        counts = np.zeros(L.MAX_LAYERS, np.uint32)
        self._check(lib().astro_read_tree_info(self._h, byref(nl), ptr(sizes), ptr(offsets),
                                               ptr(counts), L.MAX_LAYERS))
        k = nl.value
        return sizes[:k].copy(), offsets[:k].copy(), counts[:k].copy()

    def read_nodes(self, first: int = 0, count: int | None = None) -> np.ndarray:
        sizes, offsets, _ = self.tree_info()
        cap = int(offsets[-1]) + int(sizes[-1])
        count = cap - first if count is None else count
        out = np.zeros(count, L.OCTREE_NODE)
        self._check(lib().astro_read_nodes(self._h, ptr(out), first, count))
        return out

    def read_accel(self) -> np.ndarray:
        out = np.zeros((self.n, 4), np.float32)
        self._check(lib().astro_read_accel(self._h, ptr(out), self.n))
        return out

    def read_stats(self, cells: bool = False):
        """(interactions, node visits[, cell interactions]) of the last traversal."""
        i, v, c = c_uint64(), c_uint64(), c_uint64()
        self._check(lib().astro_read_stats(self._h, byref(i), byref(v), byref(c)))
        return (i.value, v.value, c.value) if cells else (i.value, v.value)

    def read_far_stats(self):
        """(far nodes expanded, far interactions) of the last group walk."""
        f, fi = c_uint64(), c_uint64()
        self._check(lib().astro_read_far_stats(self._h, byref(f), byref(fi)))
        return f.value, fi.value

    def traverse_times(self) -> tuple[float, float]:
        """(walk ms, evaluation ms) of the last group-walk barnes_hut() call."""
        w, e = ctypes.c_float(), ctypes.c_float()
        self._check(lib().astro_read_traverse_times(self._h, byref(w), byref(e)))
        return w.value, e.value

    def walk_buffers(self) -> tuple[int, int, int]:
        """(list pool blocks, frontier words per buffer, steps and
        traversals run again since creation because a group walk had
        outgrown its buffers). Waits for the context's stream."""
        b, f, r = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint64()
        self._check(lib().astro_read_walk_buffers(self._h, byref(b), byref(f), byref(r)))
        return b.value, f.value, r.value

    def direct_accel_f64(self, samples) -> np.ndarray:
        s = np.ascontiguousarray(samples, dtype=np.uint32)
        out = np.zeros((len(s), 3), np.float64)
        self._check(lib().astro_direct_accel_f64(self._h, ptr(s), len(s), ptr(out)))
        return out


def version() -> str:
    return lib().astro_version().decode()


__all__ = ["Simulation", "default_params", "version"]
_ = ctypes
