"""Headless screen-space fluid renderer (render/fluidRender.ts) over the C
ABI, and the orbit camera of camera.ts that produces its uniforms.

The reference draws into a canvas through WebGPU; here the image is a
device buffer (float RGBA and RGBA8), read back with download().
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib as L
from .mlsmpm import _check, _stream_handle


def perspective(fov: float, aspect: float, near: float, far: float) -> np.ndarray:
    """WebGPU perspective projection (depth range [0, 1]), 4x4 row-major
    numpy array: x' = f/aspect x, y' = f y, z' = (far z + near far)/(near -
    far), w' = -z, with f = 1/tan(fov/2) (camera.ts:76)."""
    f = 1.0 / math.tan(fov / 2.0)
    r = 1.0 / (near - far)
    return np.array([[f / aspect, 0, 0, 0],
                     [0, f, 0, 0],
                     [0, 0, far * r, near * far * r],
                     [0, 0, -1, 0]], dtype=np.float64)


def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """View matrix of a camera at `eye` looking at `target` (camera.ts:91-95)."""
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    z = eye - target
    z /= np.linalg.norm(z)
    x = np.cross(up, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    y /= np.linalg.norm(y)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = x, y, z
    m[:3, 3] = -m[:3, :3] @ eye
    return m


def orbit_eye(target, distance: float, xtheta: float, ytheta: float) -> np.ndarray:
    """camera.ts:84-89: target + Ry(xtheta) Rx(ytheta) (0, 0, distance)."""
    cy, sy = math.cos(ytheta), math.sin(ytheta)
    cx, sx = math.cos(xtheta), math.sin(xtheta)
    p = np.array([0.0, -sy * distance, cy * distance])          # Rx(ytheta)
    p = np.array([cx * p[0] + sx * p[2], p[1], -sx * p[0] + cx * p[2]])  # Ry(xtheta)
    return np.asarray(target, dtype=np.float64) + p


def camera_uniforms(width: int, height: int, distance: float, target, fov: float,
                    sphere_size: float, xtheta: float = math.pi / 4,
                    ytheta: float = -math.pi / 12) -> L.RenderUniforms:
    """RenderUniforms of camera.ts:reset/recalculateView (near 0.1, far 500,
    initial angles pi/4 and -pi/12) and main.ts:106 (texel size)."""
    P = perspective(fov, width / height, 0.1, 500.0)
    V = look_at(orbit_eye(target, distance, xtheta, ytheta), target)
    u = L.RenderUniforms()
    u.texel_size[0], u.texel_size[1] = 1.0 / width, 1.0 / height
    u.sphere_size = sphere_size
    for name, m in (("inv_projection_matrix", np.linalg.inv(P)), ("projection_matrix", P),
                    ("view_matrix", V), ("inv_view_matrix", np.linalg.inv(V))):
        getattr(u, name)[:] = [float(np.float32(v)) for v in m.T.reshape(-1)]  # by columns
    return u


class FluidRenderer:
    """render/fluidRender.ts's FluidRenderer, headless."""

    def __init__(self, width: int, height: int, radius: float = 0.6,
                 fov: float = 45 * math.pi / 180):
        self._lib = L.load()
        self.width, self.height = int(width), int(height)
        self._handle = ctypes.c_void_p()
        _check(self._lib.mpm_renderer_create(self.width, self.height, float(radius), float(fov),
                                             ctypes.byref(self._handle)), "FluidRenderer")

    def setEnvmap(self, faces: np.ndarray) -> None:
        """faces: (6, S, S, 4) float32, order +x, -x, +y, -y, +z, -z."""
        f = np.ascontiguousarray(faces, dtype=np.float32)
        if f.ndim != 4 or f.shape[0] != 6 or f.shape[1] != f.shape[2] or f.shape[3] != 4:
            raise ValueError("faces must be (6, S, S, 4)")
        _check(self._lib.mpm_renderer_set_envmap(self._handle, f.shape[1],
                                                 f.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
               "setEnvmap")

    def execute(self, posvel, numParticles: int, uniforms: L.RenderUniforms,
                commandEncoder=None, sphereRenderFl: bool = False) -> None:
        """FluidRenderer.execute (render/fluidRender.ts:292-488).  posvel: a
        device pointer (int), a simulator (its posvel buffer) or a CUDA tensor
        of 32-byte records.  sphereRenderFl: draw every particle as a lit
        sphere coloured by its speed (render/sphere.wgsl) instead of the
        fluid surface."""
        if hasattr(posvel, "posvelDevicePtr"):
            ptr = posvel.posvelDevicePtr()
        elif hasattr(posvel, "data_ptr"):
            ptr = int(posvel.data_ptr())
        else:
            ptr = int(posvel)
        fn = (self._lib.mpm_renderer_execute_spheres if sphereRenderFl
              else self._lib.mpm_renderer_execute)
        _check(fn(self._handle, ctypes.c_void_p(ptr), int(numParticles), ctypes.byref(uniforms),
                  _stream_handle(commandEncoder)), "execute")

    def download(self, what: str = "color") -> np.ndarray:
        h, w = self.height, self.width
        code, shape, dtype = {
            "color": (L.MPM_RENDER_COLOR, (h, w, 4), np.float32),
            "color8": (L.MPM_RENDER_COLOR8, (h, w, 4), np.uint8),
            "depth": (L.MPM_RENDER_DEPTH, (h, w), np.float32),
            "thickness": (L.MPM_RENDER_THICKNESS, (h, w), np.float32),
        }[what]
        out = np.zeros(shape, dtype=dtype)
        _check(self._lib.mpm_renderer_download(self._handle, code,
                                               out.ctypes.data_as(ctypes.c_void_p)), "download")
        return out

    def colorDevicePtr(self) -> int:
        return int(self._lib.mpm_renderer_color_device_ptr(self._handle) or 0)

    def close(self) -> None:
        if self._handle:
            self._lib.mpm_renderer_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_ppm(path: str, rgba8: np.ndarray) -> None:
    """Binary PPM of an (H, W, 4) uint8 image (alpha dropped)."""
    h, w = rgba8.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(rgba8[:, :, :3]).tobytes())


def write_png(path: str, rgba8: np.ndarray) -> None:
    """PNG (8-bit RGBA, no filtering) of an (H, W, 4) uint8 image."""
    import struct
    import zlib
    h, w = rgba8.shape[:2]
    raw = b"".join(b"\x00" + np.ascontiguousarray(rgba8[y]).tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return (struct.pack(">I", len(data)) + tag + data +
                struct.pack(">I", zlib.crc32(tag + data) & 0xffffffff))
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))
