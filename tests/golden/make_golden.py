"""Generates the golden vectors in tests/golden/*.npz by running the
reference's own WGSL kernels (mls-mpm/{clearGrid,p2g_1,p2g_2,updateGrid,g2p,
copyPosition}.wgsl, read as text from the reference checkout) through
wgsl_interp.py, dispatched in the order of MLSMPMSimulator.execute
(mls-mpm/mls-mpm.ts:245-268) with its pipeline constants
(mls-mpm/mls-mpm.ts:53-59).

Run from the repository root (needs the reference checkout; the fixtures it
writes are committed so that the tests never read the reference):
    python tests/golden/make_golden.py --reference /path/to/WebGPU-Ocean

Each fixture holds the inputs (particles in the 80-byte layout, init and real
box) and, for substep 0, the grid / particles / posvel after every one of the
six dispatches, then the state after each later substep.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import wgsl_interp as W  # noqa: E402

KERNELS = ["clearGrid", "p2g_1", "p2g_2", "updateGrid", "g2p", "copyPosition"]
# mls-mpm/mls-mpm.ts:53-59 (JS numbers; the interpreter converts each to the
# override's declared type)
OVERRIDES = {"stiffness": 3.0, "rest_density": 4.0, "dynamic_viscosity": 0.1, "dt": 0.20,
             "fixed_point_multiplier": 1e7}


def to_buffers(parts: np.ndarray, grid_count: int, init_box, real_box):
    particles = []
    for p in parts:
        particles.append({
            "position": tuple(np.float32(x) for x in p[0:3]),
            "v": tuple(np.float32(x) for x in p[4:7]),
            "C": tuple(tuple(np.float32(x) for x in p[8 + 4 * c: 11 + 4 * c]) for c in range(3)),
        })
    cells = [{"vx": 0, "vy": 0, "vz": 0, "mass": 0} for _ in range(grid_count)]
    posvel = [{"position": (np.float32(0),) * 3, "v": (np.float32(0),) * 3} for _ in parts]
    return {
        "particles": particles, "cells": cells, "posvel": posvel,
        "init_box_size": tuple(np.float32(x) for x in init_box),
        "real_box_size": tuple(np.float32(x) for x in real_box),
    }


def snapshot(buf):
    g = np.array([[c["vx"], c["vy"], c["vz"], c["mass"]] for c in buf["cells"]], dtype=np.int32)
    p = np.zeros((len(buf["particles"]), 20), dtype=np.float32)
    for i, r in enumerate(buf["particles"]):
        p[i, 0:3] = r["position"]
        p[i, 4:7] = r["v"]
        for c in range(3):
            p[i, 8 + 4 * c: 11 + 4 * c] = r["C"][c]
    pv = np.zeros((len(buf["posvel"]), 8), dtype=np.float32)
    for i, r in enumerate(buf["posvel"]):
        pv[i, 0:3] = r["position"]
        pv[i, 4:7] = r["v"]
    return g, p, pv


def run_case(modules, parts, init_box, real_box, substeps, per_kernel):
    import math
    grid_count = math.ceil(init_box[0]) * math.ceil(init_box[1]) * math.ceil(init_box[2])
    buf = to_buffers(parts, grid_count, init_box, real_box)
    n = len(parts)
    out = {}
    for s in range(substeps):
        for k in KERNELS:
            count = grid_count if k in ("clearGrid", "updateGrid") else n
            W.dispatch(modules[k], k, buf, count)
            if s == 0 and per_kernel:
                g, p, pv = snapshot(buf)
                out[f"s0_{k}_grid"], out[f"s0_{k}_particles"], out[f"s0_{k}_posvel"] = g, p, pv
        g, p, pv = snapshot(buf)
        out[f"s{s}_grid"], out[f"s{s}_particles"], out[f"s{s}_posvel"] = g, p, pv
    oob = sum(m.oob for m in modules.values())
    return out, oob


def cases():
    from oracle import scene
    rng = np.random.default_rng(20240607)
    out = {}
    # initDambreak (mls-mpm.ts:195-223) in a small box: rows start at y = 0,
    # so the first substeps exercise the flat-index aliasing (quirk Q1)
    out["dambreak"] = dict(parts=scene.dambreak([16.0, 14.0, 18.0], 120, 1),
                           init_box=[16.0, 14.0, 18.0], real_box=[16.0, 14.0, 18.0], substeps=3,
                           per_kernel=True)
    p = np.zeros((96, 20), dtype=np.float32)
    p[:, 0:3] = rng.uniform(3.0, 13.0, (96, 3))
    p[:, 4:7] = rng.uniform(-1.0, 1.0, (96, 3))
    for c in range(3):
        p[:, 8 + 4 * c: 11 + 4 * c] = rng.uniform(-0.5, 0.5, (96, 3))
    out["random_vc"] = dict(parts=p, init_box=[16.0, 16.0, 16.0], real_box=[16.0, 16.0, 16.0],
                            substeps=2, per_kernel=True)
    out["shrunk_box"] = dict(parts=p.copy(), init_box=[16.0, 16.0, 16.0],
                             real_box=[16.0, 16.0, 12.5], substeps=2, per_kernel=False)
    q = np.zeros((80, 20), dtype=np.float32)
    q[:, 0:3] = rng.uniform(3.0, 11.0, (80, 3))
    q[:, 4:7] = rng.uniform(-0.5, 0.5, (80, 3))
    for c in range(3):
        q[:, 8 + 4 * c: 11 + 4 * c] = rng.uniform(-0.2, 0.2, (80, 3))
    out["fractional_box"] = dict(parts=q, init_box=[15.5, 14.25, 16.75],
                                 real_box=[15.5, 14.25, 16.75], substeps=2, per_kernel=False)
    out["wall_impact"] = dict(parts=wall_impact_particles(), init_box=[16.0, 16.0, 16.0],
                              real_box=[16.0, 16.0, 16.0], substeps=3, per_kernel=True)
    return out


def wall_impact_particles() -> np.ndarray:
    """8 particles 0.6-2.5 cells from each of the six walls moving at it at
    2-6 cells per unit time (g2p's position clamp on both sides and wall
    push, updateGrid's boundary band; stencils that start outside the box
    alias (y, z) or fall out of range (x)), and a 4 x 4 x 3 cluster at
    spacing 0.3 (gathered density 4.3-6.5, above rest: positive pressure)
    with small random v and C."""
    rng = np.random.default_rng(20240611)
    p = np.zeros((96, 20), dtype=np.float32)
    i = 0
    for axis in range(3):
        for side in (0, 1):
            for _ in range(8):
                x = rng.uniform(4.0, 12.0, 3)
                gap = rng.uniform(0.6, 2.5)
                x[axis] = gap if side == 0 else 16.0 - gap
                v = rng.uniform(-0.5, 0.5, 3)
                v[axis] = -rng.uniform(2.0, 6.0) if side == 0 else rng.uniform(2.0, 6.0)
                p[i, 0:3], p[i, 4:7] = x, v
                i += 1
    for a in range(4):
        for b in range(4):
            for c in range(3):
                p[i, 0:3] = [7.0 + 0.3 * a, 7.0 + 0.3 * b, 7.2 + 0.3 * c]
                p[i, 4:7] = rng.uniform(-0.2, 0.2, 3)
                for col in range(3):
                    p[i, 8 + 4 * col: 11 + 4 * col] = rng.uniform(-0.1, 0.1, 3)
                i += 1
    return p


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("WEBGPU_OCEAN_REFERENCE"),
                    required="WEBGPU_OCEAN_REFERENCE" not in os.environ,
                    help="checkout of matsuoka-601/WebGPU-Ocean (or set "
                         "WEBGPU_OCEAN_REFERENCE)")
    ap.add_argument("--only", nargs="*", help="fixture names to (re)generate (default: all)")
    args = ap.parse_args()
    src_dir = os.path.join(args.reference, "mls-mpm")
    np.seterr(all="ignore")
    for name, c in cases().items():
        if args.only and name not in args.only:
            continue
        modules = {k: W.Module(open(os.path.join(src_dir, f"{k}.wgsl")).read(), OVERRIDES)
                   for k in KERNELS}
        res, oob = run_case(modules, c["parts"], c["init_box"], c["real_box"], c["substeps"],
                            c["per_kernel"])
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, particles=c["parts"],
                            init_box=np.array(c["init_box"], np.float32),
                            real_box=np.array(c["real_box"], np.float32),
                            substeps=np.int32(c["substeps"]), oob=np.int64(oob),
                            per_kernel=np.bool_(c["per_kernel"]), **res)
        print(f"{name}: {len(c['parts'])} particles, {c['substeps']} substeps, oob={oob} -> "
              f"{os.path.relpath(path)} ({os.path.getsize(path)} B)")


if __name__ == "__main__":
    main()
