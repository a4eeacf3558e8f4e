"""The WGSL interpreter that produces the golden vectors
(tests/golden/wgsl_interp.py), checked on small shaders written here: the
typing, rounding and conversion rules the pins rely on."""
from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))

import wgsl_interp as W  # noqa: E402

F32 = np.float32


def run_compute(src, buffers, n=1, entry="main"):
    m = W.Module(src, {})
    W.dispatch(m, entry, buffers, n)
    return m


HEADER = """
@group(0) @binding(0) var<storage, read_write> fo: array<f32>;
@group(0) @binding(1) var<storage, read_write> io: array<i32>;
@group(0) @binding(2) var<storage, read_write> uo: array<u32>;
"""


def test_f32_rounding_and_abstract_literals():
    src = HEADER + """
@compute @workgroup_size(64)
fn main(@builtin(global_invocation_id) id: vec3<u32>) {
    if (id.x == 0u) {
        let a: f32 = 0.1;
        let b: f32 = 0.2;
        fo[0] = a + b;                 // one f32 rounding
        fo[1] = 0.1 + 0.2;             // abstract: folded exactly, then converted
        fo[2] = 1e-64;                 // underflows to 0 as an f32
        fo[3] = a * b + a;             // two roundings, no fused multiply-add
        let big: f32 = 3e38;
        fo[4] = big * 10.0;            // overflow to infinity
    }
}
"""
    b = {"fo": [F32(0)] * 5, "io": [0], "uo": [0]}
    run_compute(src, b)
    assert b["fo"][0] == F32(F32(0.1) + F32(0.2))
    assert b["fo"][1] == F32(0.1 + 0.2)
    assert b["fo"][2] == 0.0
    assert b["fo"][3] == F32(F32(F32(0.1) * F32(0.2)) + F32(0.1))
    assert np.isinf(b["fo"][4])


def test_integer_wraparound_and_saturating_conversions():
    src = HEADER + """
@compute @workgroup_size(64)
fn main(@builtin(global_invocation_id) id: vec3<u32>) {
    if (id.x == 0u) {
        let m: i32 = 2147483647;
        io[0] = m + 1;                 // i32 wraps
        let z: u32 = 0u;
        uo[0] = z - 1u;                // u32 wraps
        let h: f32 = 3e9;
        io[1] = i32(h);                // saturates
        io[2] = i32(-2.75);            // truncates toward zero
        let q: f32 = -1.5;
        uo[1] = u32(q);                // negative -> 0
    }
}
"""
    b = {"fo": [F32(0)], "io": [0] * 3, "uo": [0] * 2}
    run_compute(src, b)
    assert b["io"] == [-2147483648, 2147483647, -2]
    assert b["uo"] == [0xFFFFFFFF, 0]


def test_loops_continue_and_out_of_range_counting():
    src = HEADER + """
@compute @workgroup_size(64)
fn main(@builtin(global_invocation_id) id: vec3<u32>) {
    if (id.x < 2u) {
        var s: i32 = 0;
        for (var k: i32 = 0; k < 10; k++) {
            if (k % 3 == 0) {
                continue;
            }
            s += k;
        }
        io[id.x] = s;
        let bad = i32(id.x) - 5;
        io[bad] = 7;                   // dropped; one visit, counted once
        io[bad] += 1;                  // same element again: still the same visit
    }
}
"""
    b = {"fo": [F32(0)], "io": [0, 0], "uo": [0]}
    m = run_compute(src, b, n=2)
    assert b["io"] == [1 + 2 + 4 + 5 + 7 + 8] * 2
    assert m.oob == 2  # one per invocation


def test_vector_builtins_follow_the_documented_order():
    src = HEADER + """
@compute @workgroup_size(64)
fn main(@builtin(global_invocation_id) id: vec3<u32>) {
    if (id.x == 0u) {
        let a = vec3f(0.3, -1.7, 2.9);
        let b = vec3(1.1, 0.25, -0.6);
        fo[0] = dot(a, b);
        let n = normalize(a);
        fo[1] = n.x; fo[2] = n.y; fo[3] = n.z;
        let c = cross(a, b);
        fo[4] = c.y;
        let v4 = vec4f(a.xy, 5.0, 1.0);
        fo[5] = v4.z + v4.w;
        let r = reflect(a, n);
        fo[6] = r.x;
    }
}
"""
    b = {"fo": [F32(0)] * 7, "io": [0], "uo": [0]}
    run_compute(src, b)
    a = [F32(0.3), F32(-1.7), F32(2.9)]
    bb = [F32(1.1), F32(0.25), F32(-0.6)]
    dot = F32(F32(F32(a[0] * bb[0]) + F32(a[1] * bb[1])) + F32(a[2] * bb[2]))
    assert b["fo"][0] == dot
    ln = F32(np.sqrt(F32(F32(F32(a[0] * a[0]) + F32(a[1] * a[1])) + F32(a[2] * a[2]))))
    assert b["fo"][1:4] == [F32(x / ln) for x in a]
    assert b["fo"][4] == F32(F32(a[2] * bb[0]) - F32(a[0] * bb[2]))
    assert b["fo"][5] == F32(6.0)
    n = [F32(x / ln) for x in a]
    k = F32(F32(2.0) * F32(F32(F32(n[0] * a[0]) + F32(n[1] * a[1])) + F32(n[2] * a[2])))
    assert b["fo"][6] == F32(a[0] - F32(k * n[0]))


def test_fragment_entry_and_texture_edges():
    src = """
@group(0) @binding(1) var texture: texture_2d<f32>;
struct FragmentInput {
    @location(0) uv: vec2f,
    @location(1) iuv: vec2f
}
@fragment
fn fs(input: FragmentInput) -> @location(0) vec4f {
    let left = textureLoad(texture, vec2u(input.iuv + vec2f(-3.0, 0.0)), 0).r;
    let right = textureLoad(texture, vec2u(input.iuv + vec2f(3.0, 0.0)), 0).r;
    return vec4f(left, right, 0.0, 1.0);
}
"""
    img = np.arange(12, dtype=np.float32).reshape(3, 4)
    run, _, _ = W.Module(src, {}).entry("fs")
    out = run({"texture": img}, {"uv": (F32(0), F32(0)), "iuv": (F32(1.5), F32(1.5))})
    # x = 1 - 3 -> negative -> u32 0; x = 1 + 3 = 4 -> beyond the edge -> 3
    assert out[0] == img[1, 0] and out[1] == img[1, 3] and out[3] == 1.0


def test_vertex_and_fragment_features():
    """What the billboard shaders (render/depthMap.wgsl, thicknessMap.wgsl,
    sphere.wgsl) need: an array value built by array(...), inferred vec2 /
    vec4 constructors, struct constructors as return values, builtin vertex
    inputs, a struct fragment input and output, and discard."""
    src = """
struct VOut { @builtin(position) position: vec4f, @location(0) uv: vec2f, }
struct FIn { @location(0) uv: vec2f, }
struct FOut { @location(0) color: vec4f, @builtin(frag_depth) depth: f32, }
@vertex
fn vs(@builtin(vertex_index) vi: u32, @builtin(instance_index) ii: u32) -> VOut {
    var corners = array(vec2(0.5, 0.5), vec2(0.5, -0.5), vec2(-0.5, -0.5));
    let c = corners[vi] * 2.0;
    return VOut(vec4(c, f32(ii), 1.0), corners[vi] + 0.5);
}
@fragment
fn fs(input: FIn) -> FOut {
    var out: FOut;
    let r2 = dot(input.uv, input.uv);
    if (r2 > 1.0) {
        discard;
    }
    out.depth = r2 * 0.5;
    out.color = vec4(input.uv, r2, 1.);
    return out;
}
"""
    m = W.Module(src, {})
    vs, _, _ = m.entry("vs")
    fs, _, _ = m.entry("fs")
    o = vs({}, 2, 7)
    assert o["position"] == (F32(-1.0), F32(-1.0), F32(7.0), F32(1.0))
    assert o["uv"] == (F32(0.0), F32(0.0))
    assert fs({}, {"uv": (F32(1.0), F32(1.0))}) == W.DISCARDED
    r = fs({}, {"uv": (F32(0.5), F32(0.25))})
    r2 = F32(F32(F32(0.5) * F32(0.5)) + F32(F32(0.25) * F32(0.25)))
    assert r["depth"] == F32(r2 * F32(0.5))
    assert r["color"] == (F32(0.5), F32(0.25), r2, F32(1.0))
