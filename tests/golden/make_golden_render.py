"""Generates tests/golden/render_filters.npz and render_shading.npz by
running the reference's own screen-space fragment shaders
(render/bilateral.wgsl, render/gaussian.wgsl and render/fluid.wgsl, read as
text from the reference checkout) through wgsl_interp.py, once per pixel,
over synthetic depth and thickness images: an X pass then a Y pass of each
filter, as fluidRender.ts runs them (blur_dir (1, 0) then (0, 1),
render/fluidRender.ts:230-235), then the shading of the filtered images.

What the graphics pipeline supplies is fixed as follows:
  * the fragment input interpolated from render/fullScreen.wgsl at a pixel
    centre: uv = ((x + 0.5) / W, (y + 0.5) / H), iuv = (x + 0.5, y + 0.5);
  * textureLoad outside the image reads the nearest edge texel (WGSL lets an
    out-of-bounds load return any texel within bounds);
  * the bilateral result lands in an r32float target, the gaussian result in
    an r16float one (rounded to the nearest half, ties to even);
  * exp and pow, whose precision WGSL leaves to the implementation, are the
    project's restatements (oracle/render_oracle.c exp_r / pow_r, also used
    by the CUDA renderer);
  * the environment cube is sampled by the restatement's lookup (bilinear
    within the face the direction selects): texture filtering is done by
    the sampling unit, not by shader arithmetic;
  * the shading's camera is the package's orbit camera (camera_uniforms) at
    distance 70 around (20, 10, 30) for a 40 x 28 image; the environment a
    seeded random 8 x 8 cube;
  * the pipeline constants depth_threshold, max_filter_size and
    projected_particle_constant are those of a 504-pixel-high screen with the
    reference's particle radius and field of view (main.ts:136-137).

Run from the repository root (needs the reference checkout):
    python tests/golden/make_golden_render.py --reference /path/to/WebGPU-Ocean
"""
from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import wgsl_interp as W  # noqa: E402

W_PX, H_PX = 40, 28
SCREEN_H, RADIUS, FOV = 504, 0.6, 45 * math.pi / 180


def images():
    """A depth image (background 0, one texel beyond the 1e4 cut-off, blobs
    at view depths 3-80 with noise and sharp steps) and a thickness image
    (zero outside the blobs, half-precision values inside)."""
    rng = np.random.default_rng(2024)
    yy, xx = np.mgrid[0:H_PX, 0:W_PX]
    depth = np.zeros((H_PX, W_PX), np.float32)
    thick = np.zeros((H_PX, W_PX), np.float32)
    for cx, cy, r, d in [(10, 9, 7, 60.0), (27, 15, 9, 4.0), (33, 6, 4, 15.0), (6, 22, 5, 3.0)]:
        m = (xx - cx) ** 2 + (yy - cy) ** 2 <= r * r
        depth[m] = (d + rng.normal(0.0, 0.2 * d / 10.0, m.sum())).astype(np.float32)
        thick[m] = rng.uniform(0.05, 1.5, m.sum()).astype(np.float32)
    depth[2, 37] = 2e4
    thick = thick.astype(np.float16).astype(np.float32)
    return depth, thick


def run_pass(module, img, blur_dir, half_target):
    run, _, _ = module.entry("fs")
    out = np.zeros_like(img)
    for y in range(H_PX):
        for x in range(W_PX):
            inp = {"uv": (np.float32((x + 0.5) / W_PX), np.float32((y + 0.5) / H_PX)),
                   "iuv": (np.float32(x + 0.5), np.float32(y + 0.5))}
            r = run({"texture": img, "uniforms": {"blur_dir": blur_dir}}, inp)[0]
            out[y, x] = np.float32(np.float16(r)) if half_target else np.float32(r)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("WEBGPU_OCEAN_REFERENCE"),
                    required="WEBGPU_OCEAN_REFERENCE" not in os.environ,
                    help="checkout of matsuoka-601/WebGPU-Ocean (or set "
                         "WEBGPU_OCEAN_REFERENCE)")
    args = ap.parse_args()
    from oracle import oracle as O
    W.EXP_F32 = lambda x: np.float32(O.render_scalar("exp", float(x)))
    dt, mf, ppc = O.filter_constants(SCREEN_H, RADIUS, FOV)
    overrides = {"depth_threshold": dt, "max_filter_size": mf, "projected_particle_constant": ppc}
    src = os.path.join(args.reference, "render")
    bil = W.Module(open(os.path.join(src, "bilateral.wgsl")).read(), overrides)
    gau = W.Module(open(os.path.join(src, "gaussian.wgsl")).read(), {})
    depth, thick = images()
    one, zero = np.float32(1.0), np.float32(0.0)
    depth_x = run_pass(bil, depth, (one, zero), False)
    depth_xy = run_pass(bil, depth_x, (zero, one), False)
    thick_x = run_pass(gau, thick, (one, zero), True)
    thick_xy = run_pass(gau, thick_x, (zero, one), True)
    path = os.path.join(HERE, "render_filters.npz")
    np.savez_compressed(path, depth=depth, thickness=thick, depth_x=depth_x, depth_xy=depth_xy,
                        thickness_x=thick_x, thickness_xy=thick_xy,
                        constants=np.array([dt, mf, ppc], np.float32))
    print(f"render_filters: {W_PX}x{H_PX}, constants {dt} {mf} {ppc} -> "
          f"{os.path.relpath(path)} ({os.path.getsize(path)} B)")

    # shading of the filtered images
    W.POW_F32 = lambda a, b: np.float32(O.render_scalar("pow", float(a), float(b)))
    W.CUBE_SAMPLE = lambda env, d: O.sample_cube(env, d)
    import ctypes
    import __graft_entry__ as entry
    pkg = entry.load_package()
    u = pkg.camera_uniforms(W_PX, H_PX, 70.0, [20.0, 10.0, 30.0], FOV, 2 * RADIUS)
    uf = np.frombuffer(ctypes.string_at(ctypes.addressof(u), ctypes.sizeof(u)),
                       dtype=np.float32).copy()
    env = np.random.default_rng(7).uniform(0.0, 1.0, (6, 8, 8, 4)).astype(np.float32)
    env[..., 3] = 1.0
    color = shade(W.Module(open(os.path.join(src, "fluid.wgsl")).read(), {}), depth_xy,
                  thick_xy, uf, env)
    path = os.path.join(HERE, "render_shading.npz")
    np.savez_compressed(path, depth=depth_xy, thickness=thick_xy, uniforms=uf, env=env,
                        color=color)
    print(f"render_shading: {W_PX}x{H_PX} -> {os.path.relpath(path)} "
          f"({os.path.getsize(path)} B)")


def render_uniforms(uf: np.ndarray) -> dict:
    """RenderUniforms (common.ts:1-9) from its 68 floats: texel size, sphere
    size, a pad, then four column-major 4 x 4 matrices."""
    def m4(o):
        return tuple(tuple(np.float32(x) for x in uf[o + 4 * c: o + 4 * c + 4]) for c in range(4))
    return {"texel_size": (np.float32(uf[0]), np.float32(uf[1])), "sphere_size": np.float32(uf[2]),
            "inv_projection_matrix": m4(4), "projection_matrix": m4(20), "view_matrix": m4(36),
            "inv_view_matrix": m4(52)}


def shade(module, depth, thick, uf, env):
    run, _, _ = module.entry("fs")
    buffers = {"texture": depth, "thickness_texture": thick, "envmap_texture": env,
               "texture_sampler": None, "uniforms": render_uniforms(uf)}
    out = np.zeros((H_PX, W_PX, 4), np.float32)
    w, h = np.float32(W_PX), np.float32(H_PX)
    for y in range(H_PX):
        for x in range(W_PX):
            inp = {"uv": (np.float32(np.float32(x + 0.5) / w), np.float32(np.float32(y + 0.5) / h)),
                   "iuv": (np.float32(x + 0.5), np.float32(y + 0.5))}
            out[y, x] = run(buffers, inp)
    return out


if __name__ == "__main__":
    main()
