"""Generates tests/golden/render_splats.npz by running the reference's own
billboard shaders (render/depthMap.wgsl, render/thicknessMap.wgsl and
render/sphere.wgsl, read as text from the reference checkout) through
wgsl_interp.py: the vertex shader for the six vertices of every particle's
quad, then the fragment shader once per covered pixel.

What the graphics pipeline supplies (rasterisation, depth test, blending) is
not shader arithmetic and is fixed by the rules the library documents and
oracle/render_oracle.c follows:
  * a quad whose depth z/w (the same at all four corners) is outside [0, 1],
    or whose w is not positive, is clipped whole;
  * its corners (vertex 2: uv (0, 0), vertex 0: uv (1, 1)) map to the screen
    rectangle x = (ndc.x + 1) * W/2, y = (1 - ndc.y) * H/2; a pixel is
    covered when its centre lies in the rectangle (top-left rule: the left
    and top edges include centres on them, the right and bottom ones not);
  * uv is interpolated linearly across the rectangle (its four corners share
    one w, so perspective-correct interpolation is linear); view_position and
    speed are the same at every vertex and reach the fragment unchanged;
  * frag_depth is clamped to [0, 1]; the depth test is 'less' against a
    clear depth of 1, and of equal depths the first-drawn (lower instance
    index) fragment wins; depthMap's r32float target keeps the winner's
    colour (its x: the view-space z), sphere mode's the winner's colour over
    the clear colour (0.8, 0.8, 0.8, 1);
  * thicknessMap's additive blend into r16float is summed exactly (in 2^-32
    fixed point) and rounded once to half.

The scene: 800 particles (seeded) around the orbit camera's target at
distances that put some partly off screen, some beyond the far plane and a
few behind the camera, with speeds covering all five colour bands of
sphere.wgsl's value_to_color; a 64 x 48 image.

Run from the repository root (needs the reference checkout):
    python tests/golden/make_golden_splat.py --reference /path/to/WebGPU-Ocean
"""
from __future__ import annotations

import argparse
import ctypes
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import wgsl_interp as W  # noqa: E402
from make_golden_render import render_uniforms  # noqa: E402

W_PX, H_PX = 64, 48
F32 = np.float32


def scene(n: int = 800, seed: int = 5) -> np.ndarray:
    """posvel records (n, 8): position, pad, velocity, pad."""
    rng = np.random.default_rng(seed)
    pv = np.zeros((n, 8), np.float32)
    pv[:, 0:3] = rng.normal([20.0, 10.0, 30.0], [6.0, 4.0, 6.0], (n, 3))
    pv[:5, 0:3] = [[20.0, 10.0, 110.0], [20.0, 10.0, 108.0], [21.0, 11.0, 109.0],
                   [20.0, 10.0, 30.0], [20.0, 10.0, 30.0]]   # behind the camera; a tie
    pv[5:10, 0:3] = rng.uniform(-2000.0, -1500.0, (5, 3))    # beyond the far plane
    speed = rng.uniform(0.0, 2.0, n)
    d = rng.normal(size=(n, 3))
    pv[:, 4:7] = (d / np.linalg.norm(d, axis=1, keepdims=True) * speed[:, None]).astype(np.float32)
    return pv


def raster(vs_out):
    """Covered pixels of one quad: (x, y, uv) per pixel, or [] when clipped."""
    c0, c2 = vs_out[0]["position"], vs_out[2]["position"]
    if not (c0[3] > 0.0):
        return []
    zq = F32(c0[2] / c0[3])
    if not (F32(0.0) <= zq <= F32(1.0)):
        return []
    Wf, Hf = F32(W_PX), F32(H_PX)
    fxm = F32(F32(F32(c2[0] / c2[3]) + F32(1.0)) * F32(F32(0.5) * Wf))
    fxp = F32(F32(F32(c0[0] / c0[3]) + F32(1.0)) * F32(F32(0.5) * Wf))
    fym = F32(F32(F32(1.0) - F32(c2[1] / c2[3])) * F32(F32(0.5) * Hf))
    fyp = F32(F32(F32(1.0) - F32(c0[1] / c0[3])) * F32(F32(0.5) * Hf))
    X0, X1 = min(fxm, fxp), max(fxm, fxp)
    Y0, Y1 = min(fym, fyp), max(fym, fyp)
    if not (X1 > X0 and Y1 > Y0):
        return []
    x0 = int(min(max(np.ceil(F32(X0 - F32(0.5))), 0.0), W_PX))
    x1 = int(max(min(np.ceil(F32(X1 - F32(0.5))) - 1.0, W_PX - 1.0), -1.0))
    y0 = int(min(max(np.ceil(F32(Y0 - F32(0.5))), 0.0), H_PX))
    y1 = int(max(min(np.ceil(F32(Y1 - F32(0.5))) - 1.0, H_PX - 1.0), -1.0))
    out = []
    for py in range(y0, y1 + 1):
        for px in range(x0, x1 + 1):
            cx, cy = F32(F32(px) + F32(0.5)), F32(F32(py) + F32(0.5))
            uu = F32(F32(cx - fxm) / F32(fxp - fxm))
            vv = F32(F32(cy - fym) / F32(fyp - fym))
            out.append((px, py, (uu, vv)))
    return out


def draw(module, pv, U, kind):
    vs, _, _ = module.entry("vs")
    fs, _, _ = module.entry("fs")
    particles = [{"position": tuple(F32(x) for x in r[0:3]), "v": tuple(F32(x) for x in r[4:7])}
                 for r in pv]
    buffers = {"particles": particles, "uniforms": U}
    key = np.full((H_PX, W_PX), np.inf)
    win = {}
    tacc = np.zeros((H_PX, W_PX), np.int64)
    for i in range(len(pv)):
        outs = [vs(buffers, k, i) for k in range(6)]
        for px, py, uv in raster(outs):
            # the vertex outputs other than position reach the fragment; all
            # but uv are the same at every vertex
            inp = {f: v for f, v in outs[0].items() if f != "position"}
            inp["uv"] = uv
            r = fs(buffers, inp)
            if r is W.DISCARDED or (isinstance(r, str) and r == W.DISCARDED):
                continue
            if kind == "thickness":
                tacc[py, px] += int(np.rint(F32(F32(r[0]) * F32(4294967296.0))))
                continue
            depth = min(max(F32(r["frag_depth"]), F32(0.0)), F32(1.0))
            if depth < F32(1.0) and (depth, i) < (key[py, px], win.get((px, py), (0, 1 << 40))[1]):
                key[py, px] = depth
                win[(px, py)] = (r["frag_color"], i)
    if kind == "thickness":
        t = (tacc.astype(np.float32) * F32(2.3283064365386963e-10)).astype(np.float32)
        return t.astype(np.float16).astype(np.float32)
    if kind == "depth":
        d = np.zeros((H_PX, W_PX), np.float32)
        for (px, py), (col, _) in win.items():
            d[py, px] = F32(col[0])
        return d
    color = np.zeros((H_PX, W_PX, 4), np.float32)
    color[..., 0:3] = F32(0.8)
    color[..., 3] = F32(1.0)
    depth = np.ones((H_PX, W_PX), np.float32)
    for (px, py), (col, _) in win.items():
        color[py, px] = [F32(c) for c in col]
        depth[py, px] = F32(key[py, px])
    return color, depth


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("WEBGPU_OCEAN_REFERENCE"),
                    required="WEBGPU_OCEAN_REFERENCE" not in os.environ,
                    help="checkout of matsuoka-601/WebGPU-Ocean (or set "
                         "WEBGPU_OCEAN_REFERENCE)")
    args = ap.parse_args()
    import __graft_entry__ as entry
    pkg = entry.load_package()
    fov = 45 * math.pi / 180
    u = pkg.camera_uniforms(W_PX, H_PX, 45.0, [20.0, 10.0, 30.0], fov, 3.0)
    uf = np.frombuffer(ctypes.string_at(ctypes.addressof(u), ctypes.sizeof(u)),
                       dtype=np.float32).copy()
    U = render_uniforms(uf)
    pv = scene()
    src = os.path.join(args.reference, "render")
    mod = lambda name: W.Module(open(os.path.join(src, name)).read(), {})  # noqa: E731
    depth = draw(mod("depthMap.wgsl"), pv, U, "depth")
    thick = draw(mod("thicknessMap.wgsl"), pv, U, "thickness")
    color, sdepth = draw(mod("sphere.wgsl"), pv, U, "sphere")
    path = os.path.join(HERE, "render_splats.npz")
    np.savez_compressed(path, posvel=pv, uniforms=uf, depth=depth, thickness=thick,
                        sphere_color=color, sphere_depth=sdepth)
    print(f"render_splats: {len(pv)} particles, {W_PX}x{H_PX}, "
          f"{int((depth != 0).sum())} depth / {int((thick != 0).sum())} thickness / "
          f"{int((sdepth < 1).sum())} sphere pixels -> {os.path.relpath(path)} "
          f"({os.path.getsize(path)} B)")


if __name__ == "__main__":
    main()
