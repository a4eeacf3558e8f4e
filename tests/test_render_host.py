"""Host-side camera math of the renderer (webgpu-ocean_gb300/render.py) and
its image writers, on CPU."""
from __future__ import annotations

import math
import struct
import zlib

import numpy as np


def test_projection_maps_near_and_far_to_webgpu_depth(pkg):
    r = pkg.render
    P = r.perspective(math.pi / 4, 16 / 9, 0.1, 500.0)
    for z, want in ((-0.1, 0.0), (-500.0, 1.0)):
        clip = P @ np.array([0.0, 0.0, z, 1.0])
        assert abs(clip[2] / clip[3] - want) < 1e-12
    # a point on the view axis at the edge of the vertical field of view
    clip = P @ np.array([0.0, math.tan(math.pi / 8) * 10.0, -10.0, 1.0])
    assert abs(clip[1] / clip[3] - 1.0) < 1e-12


def test_look_at_and_orbit(pkg):
    r = pkg.render
    target = np.array([20.0, 7.5, 30.0])
    eye = r.orbit_eye(target, 70.0, math.pi / 4, -math.pi / 12)
    assert abs(np.linalg.norm(eye - target) - 70.0) < 1e-9
    assert eye[1] > target[1]  # ytheta < 0 looks down on the target
    V = r.look_at(eye, target)
    assert np.allclose(V[:3, :3] @ V[:3, :3].T, np.eye(3), atol=1e-12)  # rotation
    assert np.allclose(V @ np.append(eye, 1.0), [0, 0, 0, 1], atol=1e-9)  # eye at origin
    t_view = V @ np.append(target, 1.0)
    assert np.allclose(t_view[:2], 0.0, atol=1e-9) and t_view[2] < 0  # target straight ahead


def test_camera_uniforms_layout(pkg):
    r = pkg.render
    u = r.camera_uniforms(896, 504, 70.0, [20.0, 7.5, 30.0], math.pi / 4, 1.2)
    P = np.array(u.projection_matrix).reshape(4, 4).T   # stored by columns
    Pi = np.array(u.inv_projection_matrix).reshape(4, 4).T
    V = np.array(u.view_matrix).reshape(4, 4).T
    Vi = np.array(u.inv_view_matrix).reshape(4, 4).T
    assert np.allclose(P @ Pi, np.eye(4), atol=1e-5)
    assert np.allclose(V @ Vi, np.eye(4), atol=1e-4)
    assert abs(u.texel_size[0] - 1 / 896) < 1e-9 and abs(u.texel_size[1] - 1 / 504) < 1e-9
    assert abs(u.sphere_size - 1.2) < 1e-7


def test_png_writer(tmp_path, pkg):
    img = np.zeros((3, 5, 4), np.uint8)
    img[..., 0] = np.arange(5)[None, :] * 50
    img[..., 3] = 255
    path = tmp_path / "t.png"
    pkg.render.write_png(str(path), img)
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", data[16:24])
    assert (w, h) == (5, 3)
    idat_len = struct.unpack(">I", data[33:37])[0]
    raw = zlib.decompress(data[41:41 + idat_len])
    rows = [raw[i * (1 + 5 * 4) + 1:(i + 1) * (1 + 5 * 4)] for i in range(3)]
    assert np.array_equal(np.frombuffer(b"".join(rows), np.uint8).reshape(3, 5, 4), img)
