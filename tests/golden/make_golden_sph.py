"""Generates the SPH golden vectors tests/golden/sph_*.npz by running the
reference's own SPH compute shaders (sph/grid/{gridClear,gridBuild,
reorderParticles}.wgsl and sph/{density,force,integrate,copyPosition}.wgsl,
read as text from the reference checkout) through wgsl_interp.py, dispatched
in the order of SPHSimulator.execute (sph/sph.ts:300-355) with the uniforms
its constructor writes (constants sph/sph.ts:58-77, environment :130-147,
parameters :150-176) and the real box of reset / changeBoxSize
(:284-296, :387-392).

What a GPU decides at run time is fixed here, each choice a legal execution
of the reference:
  * the prefix sum over the cell counts is the npm package webgpu-radix-sort
    (^1.0.7 in package.json; not vendored): PrefixSumKernel with
    data = cellParticleCount, count = gridCount + 1 (sph/sph.ts:309-312), an
    exclusive scan in place.  Restated as a plain exclusive scan: the sums
    are integers, exact in any order;
  * atomic arrival order in gridBuild (sph/grid/gridBuild.wgsl): its
    invocations run in descending particle index.  reorderParticles puts a
    cell's particles at end - 1 - arrival, so each cell then holds its
    particles in ascending index, the in-cell order the C oracle and the CUDA
    solver use;
  * params.n holds the particle count as a u32.  The reference writes it as
    the bit pattern of a float (sph/sph.ts:294-296), which makes its kernels
    also run the stale records of the last workgroup's ghost threads; the
    fixtures, like the library, simulate exactly n particles.

Run from the repository root (needs the reference checkout; the fixtures are
committed so the tests never read the reference):
    python tests/golden/make_golden_sph.py --reference /path/to/WebGPU-Ocean
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

F32 = np.float32
SHADERS = {"gridClear": ("grid/gridClear.wgsl", "main"),
           "gridBuild": ("grid/gridBuild.wgsl", "main"),
           "reorder": ("grid/reorderParticles.wgsl", "main"),
           "density": ("density.wgsl", "computeDensity"),
           "force": ("force.wgsl", "computeForce"),
           "integrate": ("integrate.wgsl", "integrate"),
           "copyPosition": ("copyPosition.wgsl", "copyPosition")}


def uniforms(n: int):
    """The environment and parameter uniforms of sph/sph.ts (JS doubles
    stored through Float32Array / Int32Array views)."""
    kr = 0.07
    cell = 1.0 * kr
    half = 2.0
    length = 2.0 * half
    sentinel = 4 * cell
    grids = math.ceil((length + sentinel) / cell)
    env = {"xGrids": grids, "yGrids": grids, "zGrids": grids, "cellSize": F32(cell),
           "xHalf": F32(half), "yHalf": F32(half), "zHalf": F32(half), "offset": F32(sentinel / 2)}
    params = {"mass": F32(1.0), "kernelRadius": F32(kr), "kernelRadiusPow2": F32(math.pow(kr, 2)),
              "kernelRadiusPow5": F32(math.pow(kr, 5)), "kernelRadiusPow6": F32(math.pow(kr, 6)),
              "kernelRadiusPow9": F32(math.pow(kr, 9)), "dt": F32(0.006), "stiffness": F32(20),
              "nearStiffness": F32(1.0), "restDensity": F32(15000), "viscosity": F32(100),
              "n": n}
    return env, params, grids ** 3


def to_particles(rec: np.ndarray):
    return [{"position": tuple(F32(x) for x in r[0:3]), "v": tuple(F32(x) for x in r[4:7]),
             "force": tuple(F32(x) for x in r[8:11]), "density": F32(r[11]),
             "nearDensity": F32(r[12])} for r in rec]


def records(parts) -> np.ndarray:
    out = np.zeros((len(parts), 16), np.float32)
    for i, p in enumerate(parts):
        out[i, 0:3] = p["position"]
        out[i, 4:7] = p["v"]
        out[i, 8:11] = p["force"]
        out[i, 11] = p["density"]
        out[i, 12] = p["nearDensity"]
    return out


def posvel_array(pv) -> np.ndarray:
    out = np.zeros((len(pv), 8), np.float32)
    for i, p in enumerate(pv):
        out[i, 0:3] = p["position"]
        out[i, 4:7] = p["v"]
    return out


def run_invocations(module, entry, buffers, count, descending=False):
    run, _, _ = module.entry(entry)
    total = -(-count // 64) * 64
    ids = range(total - 1, -1, -1) if descending else range(total)
    for i in ids:
        module._oob_last = None
        run(buffers, (i, 0, 0))


def run_case(modules, rec, real_halves):
    """Substep s uses real half box real_halves[s]; returns the state after
    every substep and, for substep 0, after each dispatch."""
    n = len(rec)
    env, params, total = uniforms(n)
    particles = to_particles(rec)
    sorted_particles = [dict(p) for p in particles]
    counts = [0] * (total + 1)
    offsets = [0] * n
    posvel = [{"position": (F32(0),) * 3, "v": (F32(0),) * 3} for _ in range(n)]
    out = {}
    for s, half in enumerate(real_halves):
        box = {"xHalf": F32(half[0]), "yHalf": F32(half[1]), "zHalf": F32(half[2])}
        steps = [
            ("gridClear", {"cellParticleCount": counts}, total + 1, False),
            ("gridBuild", {"cellParticleCount": counts, "particleCellOffset": offsets,
                           "particles": particles, "env": env, "params": params}, n, True),
            ("prefixSum", None, 0, False),
            ("reorder", {"sourceParticles": particles, "targetParticles": sorted_particles,
                         "cellParticleCount": counts, "particleCellOffset": offsets,
                         "env": env, "params": params}, n, False),
            ("density", {"particles": particles, "sortedParticles": sorted_particles,
                         "prefixSum": counts, "env": env, "params": params}, n, False),
            ("reorder", {"sourceParticles": particles, "targetParticles": sorted_particles,
                         "cellParticleCount": counts, "particleCellOffset": offsets,
                         "env": env, "params": params}, n, False),
            ("force", {"particles": particles, "sortedParticles": sorted_particles,
                       "prefixSum": counts, "env": env, "params": params}, n, False),
            ("integrate", {"particles": particles, "realBoxSize": box, "params": params}, n,
             False),
            ("copyPosition", {"particles": particles, "posvel": posvel, "env": params}, n, False),
        ]
        for name, buffers, count, descending in steps:
            if name == "prefixSum":
                run = 0
                for c in range(total + 1):
                    counts[c], run = run, (run + counts[c]) & 0xFFFFFFFF
                continue
            run_invocations(modules[name], SHADERS[name][1], buffers, count, descending)
            if s == 0 and name in ("density", "force"):
                out[f"s0_{name}_particles"] = records(particles)
        out[f"s{s}_particles"] = records(particles)
        out[f"s{s}_posvel"] = posvel_array(posvel)
    oob = sum(m.oob for m in modules.values())
    return out, oob


def cases():
    from oracle import scene
    out = {}
    # initDambreak (sph/sph.ts:357-381) in a small box, 2 frames of 2 substeps
    dam = scene.sph_dambreak([0.3, 0.6, 0.3], 800, 7)
    out["sph_dambreak"] = dict(rec=dam, real_halves=[[0.3, 0.6, 0.3]] * 4)
    # the same block in a box shrunk by changeBoxSize (wall forces of
    # integrate.wgsl), random velocities, and particles outside the grid:
    # one whose flat cell id aliases into another row, one below it (left out)
    rng = np.random.default_rng(11)
    walls = dam.copy()
    walls[:, 4:7] = rng.uniform(-0.5, 0.5, (len(walls), 3)).astype(np.float32)
    walls[0, 0:3] = [3.0, 0.1, 0.1]
    walls[1, 0:3] = [-3.0, 0.0, 0.05]
    walls[2, 0:3] = [0.0, -3.0, -3.0]
    out["sph_walls"] = dict(rec=walls, real_halves=[[0.2, 0.6, 0.2]] * 2 + [[0.15, 0.5, 0.25]] * 2)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("WEBGPU_OCEAN_REFERENCE"),
                    required="WEBGPU_OCEAN_REFERENCE" not in os.environ,
                    help="checkout of matsuoka-601/WebGPU-Ocean (or set "
                         "WEBGPU_OCEAN_REFERENCE)")
    ap.add_argument("--only", nargs="*", help="fixture names to (re)generate (default: all)")
    args = ap.parse_args()
    src_dir = os.path.join(args.reference, "sph")
    np.seterr(all="ignore")
    for name, c in cases().items():
        if args.only and name not in args.only:
            continue
        modules = {k: W.Module(open(os.path.join(src_dir, f)).read(), {})
                   for k, (f, _) in SHADERS.items()}
        res, oob = run_case(modules, c["rec"], c["real_halves"])
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, records=c["rec"],
                            real_halves=np.array(c["real_halves"], np.float32),
                            substeps=np.int32(len(c["real_halves"])), oob=np.int64(oob), **res)
        print(f"{name}: {len(c['rec'])} particles, {len(c['real_halves'])} substeps, oob={oob} "
              f"-> {os.path.relpath(path)} ({os.path.getsize(path)} B)")


if __name__ == "__main__":
    main()
