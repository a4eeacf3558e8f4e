"""GPU parity of the SPH solver (SPHSimulator over mpm_sph_*) against the
CPU restatement oracle/sph_oracle.c, bit for bit: particle records (position,
velocity, force, density, near density) and posvel."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import assert_bits_equal

pytestmark = pytest.mark.gpu


def run_pair(pkg, oracle_mod, half, n, frames, seed=7, box_changes=None, warp_max=-1):
    sim = pkg.SPHSimulator(None, None, 0.08, maxParticles=200000, seed=seed)
    sim.warpPerParticle = warp_max
    sim.reset(n, half)
    rec = sim.downloadParticles()
    assert len(rec) == n
    real = list(half)
    for f in range(frames):
        if box_changes and f in box_changes:
            real = box_changes[f]
            sim.changeBoxSize(real)
        sim.execute()
        rec, pv = oracle_mod.sph_execute(rec, real, 2)
    got = sim.downloadParticles()
    assert_bits_equal(got, rec, f"records after {frames} frames")
    assert_bits_equal(sim.downloadPosvel(), pv, "posvel")
    sim.close()
    return got


@pytest.mark.parametrize("warp_max", [-1, 0])
def test_default_scene(cuda, pkg, oracle_mod, warp_max):
    """main.ts's SPH defaults: 20,000 particles, half box (1.0, 2.0, 1.0);
    density and forces one warp per particle (the default at this size) and
    one thread per particle."""
    got = run_pair(pkg, oracle_mod, [1.0, 2.0, 1.0], 20000, 30, warp_max=warp_max)
    assert np.isfinite(got).all()
    assert (got[:, 11] > 0).all()  # every particle has neighbours in the grid


def test_warp_per_particle_dense_neighbourhoods(cuda, pkg, oracle_mod):
    """A compressed block (more neighbours than one staging round of 64)
    one warp per particle, and the knob's range."""
    run_pair(pkg, oracle_mod, [0.35, 1.0, 0.35], 20000, 8)
    sim = pkg.SPHSimulator(None, None, 0.08, maxParticles=1000)
    assert sim.warpPerParticle == 32768
    sim.warpPerParticle = 0
    assert sim.warpPerParticle == 0
    with pytest.raises(Exception):
        sim.warpPerParticle = -2
    sim.close()


@pytest.mark.parametrize("n,half", [(10000, [0.7, 2.0, 0.7]), (1, [1.0, 2.0, 1.0]),
                                    (63, [1.0, 2.0, 1.0])])
def test_ragged_counts(cuda, pkg, oracle_mod, n, half):
    run_pair(pkg, oracle_mod, half, n, 10)


def test_change_box_size(cuda, pkg, oracle_mod):
    run_pair(pkg, oracle_mod, [1.0, 2.0, 1.0], 20000, 24,
             box_changes={8: [0.8, 2.0, 1.0], 16: [1.2, 1.5, 0.9]})


def test_particles_outside_the_grid(cuda, pkg, oracle_mod):
    """Out-of-domain particles (flat id outside the grid, or aliasing into
    it) follow the documented rule in both implementations."""
    recs = pkg.sph_scene_dambreak([1.0, 2.0, 1.0], 5000, 3)
    extra = np.zeros((6, 16), np.float32)
    extra[:, 0:3] = [[0.0, -3.0, 0.0], [5.0, 0.0, 0.0], [-2.2, 0.1, 0.1],
                     [0.0, 2.3, 0.0], [np.nan, 0.0, 0.0], [1e30, -1e30, 0.0]]
    recs = np.concatenate([recs, extra])
    sim = pkg.SPHSimulator(None, None, 0.08, maxParticles=10000)
    sim.upload(recs, [1.0, 2.0, 1.0])
    ref = recs.copy()
    for _ in range(5):
        sim.execute()
        ref, pv = oracle_mod.sph_execute(ref, [1.0, 2.0, 1.0], 2)
    assert_bits_equal(sim.downloadParticles(), ref, "records")
    sim.close()


def test_posvel_feeds_the_renderer(cuda, pkg):
    import math
    sim = pkg.SPHSimulator(None, None, 0.08)
    sim.reset(20000, [1.0, 2.0, 1.0])
    for _ in range(5):
        sim.execute()
    r = pkg.FluidRenderer(128, 96, radius=0.04, fov=45 * math.pi / 180)
    u = pkg.camera_uniforms(128, 96, 3.0, [0.0, -1.5, 0.0], 45 * math.pi / 180, 0.08)
    r.execute(sim.posvelDevicePtr(), sim.numParticles, u)
    assert (r.download("depth") != 0).any()
    r.close()
    sim.close()


def test_graph_replay_equals_launches(cuda, pkg):
    """Frames replayed as CUDA graphs give the same records as launching every
    kernel, box changes between frames included."""
    outs = []
    for graph in (True, False):
        sim = pkg.SPHSimulator(None, None, 0.08, maxParticles=50000, seed=3)
        sim.setGraph(graph)
        sim.reset(12000, [1.0, 2.0, 1.0])
        for f in range(12):
            if f == 5:
                sim.changeBoxSize([0.8, 2.0, 1.0])
            sim.execute()
        outs.append(sim.downloadParticles())
        sim.close()
    assert_bits_equal(outs[0], outs[1], "graph vs launches")


@pytest.mark.parametrize("name", ["sph_dambreak", "sph_walls"])
def test_sph_solver_reproduces_wgsl_golden(cuda, pkg, name):
    """The CUDA SPH solver against the reference's SPH shaders run by the
    WGSL interpreter (tests/golden/make_golden_sph.py), one substep at a time
    with the fixture's real box: every record and posvel bit for bit."""
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    f = dict(np.load(os.path.join(here, "golden", f"{name}.npz")))
    recs = f["records"]
    sim = pkg.SPHSimulator(None, None, 0.08, maxParticles=len(recs))
    sim.upload(recs, [float(x) for x in f["real_halves"][0]])
    for s in range(int(f["substeps"])):
        sim.changeBoxSize([float(x) for x in f["real_halves"][s]])
        sim.execute(substeps=1)
        assert_bits_equal(sim.downloadParticles(), f[f"s{s}_particles"], f"{name} substep {s}")
        assert_bits_equal(sim.downloadPosvel(), f[f"s{s}_posvel"], f"{name} substep {s} posvel")
    sim.close()
