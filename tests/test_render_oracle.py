"""CPU checks of the renderer restatement's scalar helpers (the same code
runs on the GPU): exp / log / pow against numpy in double precision, and the
half-precision rounding of r16float writes against numpy's float16."""
from __future__ import annotations

import numpy as np


def test_exp_log_pow_accuracy(oracle_mod):
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-100, 88, 4000), rng.uniform(-1, 1, 2000), [0.0, -0.0, 1e-30]])
    for x in xs.astype(np.float32):
        got = oracle_mod.render_scalar("exp", float(x))
        want = np.exp(np.float64(x))
        if want < 1.2e-38:  # subnormal results: absolute error of one subnormal step
            assert abs(got - want) <= 2e-45
        else:
            assert abs(got - want) <= 3e-7 * want, (x, got, want)
    for x in np.concatenate([rng.uniform(1e-30, 1e30, 2000), rng.uniform(0.5, 2.0, 2000),
                             [1.0, 2.0, 1e-40, 3.4e38]]).astype(np.float32):
        got = oracle_mod.render_scalar("log", float(x))
        want = np.log(np.float64(x))
        assert abs(got - want) <= 3e-7 * max(1.0, abs(want)), (x, got, want)
    for x, y in [(0.5, 250.0), (0.999, 250.0), (0.3, 5.0), (0.0, 5.0), (1.0, 250.0)]:
        got = oracle_mod.render_scalar("pow", x, y)
        want = np.float64(np.float32(x)) ** y
        assert abs(got - want) <= 2e-6 * max(want, 1e-30) + 1e-38, (x, y, got, want)
    assert np.isnan(oracle_mod.render_scalar("pow", -0.5, 5.0))
    assert oracle_mod.render_scalar("exp", 200.0) == np.inf
    assert oracle_mod.render_scalar("exp", -200.0) == 0.0


def test_half_rounding_matches_ieee(oracle_mod):
    rng = np.random.default_rng(1)
    vals = np.concatenate([
        rng.uniform(0, 1, 3000), rng.uniform(0, 70000, 1000), rng.uniform(0, 1e-4, 1000),
        rng.standard_normal(1000) * 1e-6,
        [0.0, 65504.0, 65519.0, 65520.0, 6.1035156e-05, 5.96e-08, 2.98e-08, 1.0 + 2**-11]]).astype(np.float32)
    for v in vals:
        got = np.float32(oracle_mod.render_scalar("half_round", float(v)))
        want = np.float32(np.float16(v))
        assert got == want or (np.isinf(got) and np.isinf(want)), (v, got, want)


def test_filter_passes_reproduce_wgsl_golden():
    """The renderer restatement's bilateral (depth) and gaussian (thickness)
    passes against the reference's own fragment shaders run per pixel by the
    WGSL interpreter (tests/golden/make_golden_render.py): X then Y pass, bit
    for bit.  The CUDA renderer equals the restatement end to end."""
    import os
    from oracle import oracle as O
    here = os.path.dirname(os.path.abspath(__file__))
    f = dict(np.load(os.path.join(here, "golden", "render_filters.npz")))
    dt, mf, ppc = (float(x) for x in f["constants"])
    bx = O.render_filter_pass("bilateral", f["depth"], (1, 0), dt, mf, ppc)
    by = O.render_filter_pass("bilateral", f["depth_x"], (0, 1), dt, mf, ppc)
    gx = O.render_filter_pass("gaussian", f["thickness"], (1, 0))
    gy = O.render_filter_pass("gaussian", f["thickness_x"], (0, 1))
    for got, key in ((bx, "depth_x"), (by, "depth_xy"), (gx, "thickness_x"), (gy, "thickness_xy")):
        assert np.array_equal(got.view(np.uint32), f[key].view(np.uint32)), key
    # coverage: background and the >= 1e4 texel pass through, filter sizes
    # reach the cap (depth < ppc / 100) and stay small elsewhere
    d = f["depth"]
    assert (f["depth_xy"][d == 0] == 0).all() and (d >= 1e4).any()
    fluid = (d > 0) & (d < 1e4)
    assert (ppc / d[fluid] > mf).any() and (ppc / d[fluid] < 10).any()
    assert (f["depth_xy"][fluid] != d[fluid]).any()


def test_shading_pass_reproduces_wgsl_golden():
    """The restatement's shading against the reference's fluid.wgsl fragment
    shader run per pixel by the WGSL interpreter over filtered depth and
    thickness images (tests/golden/make_golden_render.py): every colour bit
    for bit, the NaNs at silhouettes (a neighbour reads the background depth
    0) in the same places."""
    import os
    from oracle import oracle as O
    here = os.path.dirname(os.path.abspath(__file__))
    f = dict(np.load(os.path.join(here, "golden", "render_shading.npz")))
    got = O.render_shade_pass(f["depth"], f["thickness"], f["uniforms"], f["env"])
    want = f["color"]
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got.view(np.uint32)[~nan], want.view(np.uint32)[~nan])
    fluid = (f["depth"] > 0) & (f["depth"] < 1e4)
    assert fluid.any() and (~fluid).any() and nan.any()
    assert np.allclose(want[~fluid][:, :3], 0.8)  # background colour


def test_splats_and_sphere_mode_reproduce_wgsl_golden(oracle_mod):
    """The renderer restatement's depth splat, thickness splat and sphere
    mode against the reference's own depthMap.wgsl, thicknessMap.wgsl and
    sphere.wgsl run through the WGSL interpreter (vertex shader per quad
    vertex, fragment shader per covered pixel; the rasterisation, depth-test
    and blending rules are the documented ones,
    tests/golden/make_golden_splat.py): 800 particles at 64 x 48, every
    image bit for bit."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "render_splats.npz"))
    H, W = g["depth"].shape
    s = oracle_mod.splat(g["posvel"], g["uniforms"], W, H)
    assert np.array_equal(s["depth"].view(np.uint32), g["depth"].view(np.uint32))
    assert np.array_equal(s["thickness"].view(np.uint32), g["thickness"].view(np.uint32))
    assert (g["depth"] != 0).sum() > 1000  # the fixture covers a good part of the image
    sp = oracle_mod.sphere(g["posvel"], g["uniforms"], W, H)
    assert np.array_equal(sp["color"].view(np.uint32), g["sphere_color"].view(np.uint32))
    assert np.array_equal(sp["depth"].view(np.uint32), g["sphere_depth"].view(np.uint32))
