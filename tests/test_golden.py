"""Golden vectors made by executing the reference's own WGSL kernels
(tests/golden/make_golden.py + wgsl_interp.py): the C oracle (CPU) and
libmpm.so (GPU, both engines) must reproduce them bit for bit, kernel by
kernel where the fixture holds per-dispatch snapshots."""
from __future__ import annotations

import os

import numpy as np
import pytest

from helpers import assert_bits_equal

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["dambreak", "random_vc", "shrunk_box", "fractional_box", "wall_impact"]
KERNELS = ["clearGrid", "p2g_1", "p2g_2", "updateGrid", "g2p", "copyPosition"]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_wgsl_golden(oracle_mod, name):
    f = load(name)
    sim = oracle_mod.OracleSim(f["particles"], f["init_box"], real_box=f["real_box"])
    steps = [sim.clear_grid, sim.p2g_1, sim.p2g_2, sim.update_grid, sim.g2p, sim.copy_position]
    for s in range(int(f["substeps"])):
        for k, fn in zip(KERNELS, steps):
            fn()
            if s == 0 and bool(f["per_kernel"]):
                assert_bits_equal(sim.cells, f[f"s0_{k}_grid"], f"{name} after {k} grid")
                assert_bits_equal(sim.particles, f[f"s0_{k}_particles"], f"{name} after {k} particles")
                assert_bits_equal(sim.posvel, f[f"s0_{k}_posvel"], f"{name} after {k} posvel")
        assert_bits_equal(sim.cells, f[f"s{s}_grid"], f"{name} substep {s} grid")
        assert_bits_equal(sim.particles, f[f"s{s}_particles"], f"{name} substep {s} particles")
        assert_bits_equal(sim.posvel, f[f"s{s}_posvel"], f"{name} substep {s} posvel")
    assert sim.oob == int(f["oob"])


def test_golden_fixtures_cover_the_paths():
    """The fixtures exercise aliasing (dambreak starts at y = 0), a shrunk real
    box, a non-integer box, non-zero initial v and C, and particles hitting
    the walls (g2p's clamp on both sides, stencils out of range)."""
    d = load("dambreak")
    assert (np.floor(d["particles"][:, 1]) == 0).any()
    assert load("shrunk_box")["real_box"][2] < load("shrunk_box")["init_box"][2]
    fb = load("fractional_box")["init_box"]
    assert (fb != np.floor(fb)).all()
    assert np.abs(load("random_vc")["particles"][:, 8:19]).max() > 0
    w = load("wall_impact")
    x0 = w["s0_particles"][:, 0:3]
    assert (x0 == 1.0).any() and (x0 == w["real_box"][0] - 2.0).any()  # g2p.wgsl clamp
    assert int(w["oob"]) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_dispatch_engine_reproduces_wgsl_golden(cuda, pkg, name):
    f = load(name)
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=256, maxGrid=(32, 32, 32))
    sim.engine = "dispatch"
    sim.upload(f["particles"], f["init_box"])
    sim.changeBoxSize(f["real_box"])
    for s in range(int(f["substeps"])):
        for k in KERNELS:
            sim.dispatch(k)
            if s == 0 and bool(f["per_kernel"]):
                assert_bits_equal(sim.downloadGrid(), f[f"s0_{k}_grid"], f"{name} after {k} grid")
                assert_bits_equal(sim.downloadParticles(), f[f"s0_{k}_particles"],
                                  f"{name} after {k} particles")
        assert_bits_equal(sim.downloadGrid(), f[f"s{s}_grid"], f"{name} substep {s} grid")
        assert_bits_equal(sim.downloadParticles(), f[f"s{s}_particles"], f"{name} substep {s}")
        assert_bits_equal(sim.downloadPosvel(), f[f"s{s}_posvel"], f"{name} substep {s} posvel")
    sim.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_sorted_engine_reproduces_wgsl_golden(cuda, pkg, name):
    f = load(name)
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=256, maxGrid=(32, 32, 32))
    sim.engine = "sorted"
    sim.upload(f["particles"], f["init_box"])
    sim.changeBoxSize(f["real_box"])
    for s in range(int(f["substeps"])):
        sim.execute(substeps=1)
        assert_bits_equal(sim.downloadGrid(), f[f"s{s}_grid"], f"{name} substep {s} grid")
        assert_bits_equal(sim.downloadParticles(), f[f"s{s}_particles"], f"{name} substep {s}")
        assert_bits_equal(sim.downloadPosvel(), f[f"s{s}_posvel"], f"{name} substep {s} posvel")
    sim.close()
