"""GPU parity of the headless screen-space renderer (FluidRenderer, the
mpm_renderer_* C ABI) against the CPU restatement in oracle/render_oracle.c.

Both follow the same documented rasterisation, texture and precision rules
with the same operation order (explicitly rounded on the GPU, no FMA
contraction on the CPU) and the same exp/log/pow restatement, so every image
is compared bit for bit; NaN pixels (the shading reads the background depth
0 at silhouettes, fluid.wgsl:19-36) must sit at the same places.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FOV = 45 * math.pi / 180  # main.ts:136
RADIUS = 0.6              # main.ts:137


def uniforms_f32(u) -> np.ndarray:
    return np.frombuffer(ctypes.string_at(ctypes.addressof(u), ctypes.sizeof(u)), dtype=np.float32)


def same_bits(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, what
    if a.dtype.kind == "f":
        na, nb = np.isnan(a), np.isnan(b)
        assert np.array_equal(na, nb), f"{what}: NaN positions differ ({na.sum()} vs {nb.sum()})"
        a, b = np.where(na, 0, a), np.where(nb, 0, b)
        bad = np.argwhere(a.view(np.uint32) != b.view(np.uint32))
    else:
        bad = np.argwhere(a != b)
    assert len(bad) == 0, f"{what}: {len(bad)} pixels differ; first {tuple(bad[0])}: {a[tuple(bad[0])]} vs {b[tuple(bad[0])]}"


def env_faces(size=8, seed=0):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.0, 1.0, (6, size, size, 4)).astype(np.float32)
    f[..., 3] = 1.0
    return f


def render_both(pkg, oracle_mod, posvel, n, u, W, H, env=None):
    r = pkg.FluidRenderer(W, H, RADIUS, FOV)
    if env is not None:
        r.setEnvmap(env)
        e = env
    else:
        e = None
    import torch
    dev = torch.from_numpy(np.ascontiguousarray(posvel[:max(n, 1)], dtype=np.float32)).cuda()
    r.execute(dev, n, u)
    got = {k: r.download(k) for k in ("color", "color8", "depth", "thickness")}
    if e is None:  # the built-in sky: read it back through a 1-particle-free render
        e = default_env_from(pkg)
    want = oracle_mod.render(posvel[:n], uniforms_f32(u), W, H, RADIUS, FOV, e)
    r.close()
    return got, want


_ENV = {}


def default_env_from(pkg):
    """The renderer's built-in sky, regenerated on the host the same way
    (its formula is part of the library's documentation)."""
    if "sky" in _ENV:
        return _ENV["sky"]
    size = 32
    f = np.zeros((6, size, size, 4), np.float32)
    for face in range(6):
        for j in range(size):
            for i in range(size):
                s = np.float32(2.0) * (np.float32(i) + np.float32(0.5)) / np.float32(size) - np.float32(1.0)
                t = np.float32(2.0) * (np.float32(j) + np.float32(0.5)) / np.float32(size) - np.float32(1.0)
                d = {0: (1, -t, -s), 1: (-1, -t, s), 2: (s, 1, t), 3: (s, -1, -t),
                     4: (s, -t, 1), 5: (-s, -t, -1)}[face]
                d = np.array(d, dtype=np.float32)
                l = np.sqrt(np.float32(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), dtype=np.float32)
                y = np.float32(d[1] / l)
                h = max(y, np.float32(0))
                lo = lambda c: np.float32(c) * y if y < 0 else np.float32(0)
                f[face, j, i] = [np.float32(0.55) + np.float32(0.25) * h + lo(0.2),
                                 np.float32(0.65) + np.float32(0.25) * h + lo(0.2),
                                 np.float32(0.80) + np.float32(0.20) * h + lo(0.1), 1.0]
    _ENV["sky"] = f
    return f


def reference_scene(pkg, frames=20):
    """main.ts defaults: 70,000 particles in 40x30x60, camera distance 70."""
    box = [40.0, 30.0, 60.0]
    sim = pkg.MLSMPMSimulator(None, None, 2 * RADIUS, maxParticles=200000)
    sim.reset(70000, box)
    for _ in range(frames):
        sim.execute()
    pv = sim.downloadPosvel()
    n = sim.numParticles
    sim.close()
    target = [box[0] / 2, box[1] / 4, box[2] / 2]
    return pv, n, target


@pytest.mark.parametrize("size", [(192, 108), (160, 160)])
def test_reference_scene_matches_oracle(cuda, pkg, oracle_mod, size):
    W, H = size
    pv, n, target = reference_scene(pkg)
    u = pkg.camera_uniforms(W, H, 70.0, target, FOV, 2 * RADIUS)
    got, want = render_both(pkg, oracle_mod, pv, n, u, W, H, env=env_faces())
    for k in ("depth", "thickness", "color", "color8"):
        same_bits(got[k], want[k], k)
    fluid = want["depth"] > 0
    assert 0.05 < fluid.mean() < 0.9  # the fluid covers part of the image
    assert (want["thickness"][fluid] > 0).all()


def test_builtin_sky_and_close_camera(cuda, pkg, oracle_mod):
    pv, n, target = reference_scene(pkg, frames=5)
    W, H = 128, 96
    u = pkg.camera_uniforms(W, H, 30.0, target, FOV, 2 * RADIUS, xtheta=1.1, ytheta=-0.6)
    got, want = render_both(pkg, oracle_mod, pv, n, u, W, H)
    for k in ("depth", "thickness", "color", "color8"):
        same_bits(got[k], want[k], k)


def test_empty_and_clipped_particles(cuda, pkg, oracle_mod):
    W, H = 64, 48
    u = pkg.camera_uniforms(W, H, 20.0, [0.0, 0.0, 0.0], FOV, 1.2)
    # no particles: background everywhere
    got, want = render_both(pkg, oracle_mod, np.zeros((1, 8), np.float32), 0, u, W, H, env_faces())
    same_bits(got["color"], want["color"], "empty color")
    assert np.allclose(want["color"][..., :3], 0.8)
    # particles behind the camera, beyond the far plane, at the image edges
    eye = pkg.render.orbit_eye([0.0, 0.0, 0.0], 20.0, math.pi / 4, -math.pi / 12)
    pts = np.array([eye * 2.0, eye * -40.0, [0, 0, 0], [6.5, 0, -6.5], [-6.5, 3, 6.5],
                    [0, 9.9, 0], eye * 0.999], dtype=np.float32)
    pv = np.zeros((len(pts), 8), np.float32)
    pv[:, 0:3] = pts
    got, want = render_both(pkg, oracle_mod, pv, len(pv), u, W, H, env_faces(seed=3))
    for k in ("depth", "thickness", "color", "color8"):
        same_bits(got[k], want[k], k)


def test_render_reads_the_simulator_buffer(cuda, pkg):
    """execute() accepts the simulator itself (its posvel device buffer)."""
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=200000)
    sim.reset(20000, [30.0, 24.0, 40.0])
    sim.execute()
    r = pkg.FluidRenderer(96, 64)
    u = pkg.camera_uniforms(96, 64, 60.0, [15, 6, 20], FOV, 1.2)
    r.execute(sim, sim.numParticles, u)
    img = r.download("color8")
    assert img.shape == (64, 96, 4) and (img[..., 3] == 255).all()
    assert (r.download("depth") != 0).any()
    r.close()
    sim.close()


def test_sphere_mode_matches_restatement(cuda, pkg, oracle_mod):
    """FluidRenderer.execute(..., sphereRenderFl=True) (render/sphere.wgsl)
    against the restatement, which reproduces the reference's sphere shader
    run through the WGSL interpreter (tests/golden/render_splats.npz): the
    fixture's own scene and camera, then a simulated dam-break."""
    import os
    import torch
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "render_splats.npz"))
    H, W = g["sphere_depth"].shape
    u = pkg._lib.RenderUniforms.from_buffer_copy(g["uniforms"].astype(np.float32).tobytes())
    r = pkg.FluidRenderer(W, H, RADIUS, FOV)
    dev = torch.from_numpy(np.ascontiguousarray(g["posvel"], dtype=np.float32)).cuda()
    r.execute(dev, len(g["posvel"]), u, sphereRenderFl=True)
    same_bits(r.download("color"), g["sphere_color"], "sphere colour vs reference shader")
    same_bits(r.download("depth"), g["sphere_depth"], "sphere depth vs reference shader")
    r.close()
    # a simulated scene at another size
    sim = pkg.MLSMPMSimulator(None, None, 2 * RADIUS, maxParticles=20000, seed=4)
    sim.reset(20000, [40.0, 30.0, 60.0])
    for _ in range(20):
        sim.execute()
    sim.synchronize()
    pv = sim.downloadPosvel()
    W, H = 160, 96
    u = pkg.camera_uniforms(W, H, 60.0, [20.0, 10.0, 30.0], FOV, 2 * RADIUS)
    r = pkg.FluidRenderer(W, H, RADIUS, FOV)
    r.execute(sim, sim.numParticles, u, sphereRenderFl=True)
    want = oracle_mod.sphere(pv, uniforms_f32(u), W, H)
    for k in ("color", "color8", "depth"):
        same_bits(r.download(k), want[k], f"sphere {k}")
    assert (want["depth"] < 1).mean() > 0.03
    r.close()
    sim.close()
