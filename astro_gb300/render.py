"""Camera matrices and images for the headless splat (astro_splat).

The reference renders from Camera (Astro/Camera.swift: position (0, 0, 1.8e6),
yaw pi, pitch 0; floatViewMatrix = lookAtD(0, forward, up) in FP64, cast to
FP32, applied to camera-relative positions) with createProjectionMatrix(fov =
pi / 2.5, aspect, near = 10, far = 1e7) (MathUtils.swift:3-13,
Renderer.swift:159). ``reference_camera`` builds the same matrices;
``Simulation.splat`` draws with any camera.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Camera:
    view: np.ndarray        # (16,) float32, column-major
    projection: np.ndarray  # (16,) float32, column-major
    position: np.ndarray    # (3,) float32


def _normalize(v):
    return v / np.linalg.norm(v)


def look_at(eye, center, up) -> np.ndarray:
    """lookAtD (Camera.swift:53-66) in FP64: column-major (16,) array."""
    eye, center, up = (np.asarray(a, np.float64) for a in (eye, center, up))
    z = _normalize(eye - center)
    x = _normalize(np.cross(up, z))
    y = np.cross(z, x)
    rot = np.array([[x[0], x[1], x[2], 0.0],
                    [y[0], y[1], y[2], 0.0],
                    [z[0], z[1], z[2], 0.0],
                    [0.0, 0.0, 0.0, 1.0]])          # row-major rows of rot
    trans = np.eye(4)
    trans[:3, 3] = -eye
    m = rot @ trans
    return m.T.reshape(16)                          # columns first


def projection(fov: float, aspect: float, near: float, far: float) -> np.ndarray:
    """createProjectionMatrix (MathUtils.swift:3-13) in FP32, column-major."""
    f32 = np.float32
    y = f32(1.0) / f32(math.tan(f32(fov) * f32(0.5)))
    x = y / f32(aspect)
    z = f32(far) / (f32(near) - f32(far))
    cols = [[x, 0, 0, 0], [0, y, 0, 0], [0, 0, z, -1], [0, 0, z * f32(near), 0]]
    return np.array(cols, np.float32).reshape(16)


def reference_camera(width: int, height: int, position=(0.0, 0.0, 1.8e6), yaw: float = math.pi,
                     pitch: float = 0.0) -> Camera:
    """The reference's initial camera and projection for a width x height view."""
    fwd = _normalize(np.array([math.cos(pitch) * math.sin(yaw), math.sin(pitch),
                               math.cos(pitch) * math.cos(yaw)]))
    right = _normalize(np.cross(fwd, [0.0, 1.0, 0.0]))
    up = np.cross(right, fwd)
    view = look_at([0.0, 0.0, 0.0], fwd, up).astype(np.float32)
    proj = projection(math.pi / 2.5, width / height, 10.0, 1e7)
    return Camera(view, proj, np.asarray(position, np.float32))


def to_abi(camera: Camera):
    from .layouts import CameraABI

    c = CameraABI()
    c.view[:] = [float(v) for v in np.asarray(camera.view, np.float32).reshape(16)]
    c.projection[:] = [float(v) for v in np.asarray(camera.projection, np.float32).reshape(16)]
    c.position[:] = [float(v) for v in np.asarray(camera.position, np.float32).reshape(3)]
    return c


def save_ppm(path, rgba: np.ndarray) -> None:
    """8-bit binary PPM of the RGB channels, clamped to [0, 1]."""
    h, w = rgba.shape[:2]
    rgb = (np.clip(rgba[..., :3], 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(f"P6\n{w} {h}\n255\n".encode())
        f.write(rgb.tobytes())
