"""CPU checks of the SPH path: the library's initDambreak (host code,
sph/sph.ts:357-381) against its restatement in oracle/scene.py, and known
answers of the SPH oracle (oracle/sph_oracle.c)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from helpers import assert_bits_equal


def test_sph_dambreak_matches_restatement(pkg):
    from oracle import scene
    for half, n, seed in [([1.0, 2.0, 1.0], 20000, 5), ([0.7, 2.0, 0.7], 10000, 1),
                          ([1.4, 2.0, 1.4], 40000, 9), ([1.0, 2.0, 1.0], 0, 3)]:
        got = pkg.sph_scene_dambreak(half, n, seed)
        want = scene.sph_dambreak(half, n, seed)
        assert len(got) == n
        assert_bits_equal(got, want, f"sph dambreak {half} {n}")
        if n:
            assert got[:, 0:3].min() >= -0.95 * max(half) - 1e-6
            assert (got[:, 2] < 0.001).all()  # z in [-0.95 h_z, 0) plus jitter


def test_sph_grid_constants(oracle_mod):
    # ceil((4 + 4 * 0.07) / 0.07) = 62 cells per axis (sph.ts:62-72)
    assert oracle_mod.sph_grid_count() == 62 ** 3


def test_sph_single_particle_free_fall(oracle_mod):
    """One particle: density = W_poly6(0) = 315/(64 pi h^9) h^6, no pressure
    partner, so it falls under gravity: v_y = -9.8 dt per substep."""
    rec = np.zeros((1, 16), np.float32)
    rec[0, 0:3] = [0.1, 0.5, -0.2]
    out, pv = oracle_mod.sph_execute(rec, [1.0, 2.0, 1.0], 1)
    h = np.float32(0.07)
    dens = out[0, 11]
    want = 315.0 / (64 * math.pi * 0.07 ** 9) * 0.07 ** 6
    assert abs(dens - want) / want < 1e-5
    assert abs(out[0, 5] - (-9.8 * 0.006)) < 1e-6
    assert abs(out[0, 1] - (0.5 - 9.8 * 0.006 * 0.006)) < 1e-6
    assert np.array_equal(pv[0, 0:3], out[0, 0:3]) and np.array_equal(pv[0, 4:7], out[0, 4:7])
    assert out[0, 12] > 0  # near density W_spiky(0)
    del h


def test_sph_walls_push_back(oracle_mod):
    """A particle outside the +x wall is accelerated back (integrate.wgsl)."""
    rec = np.zeros((1, 16), np.float32)
    rec[0, 0:3] = [1.05, 0.0, 0.0]
    out, _ = oracle_mod.sph_execute(rec, [1.0, 2.0, 1.0], 1)
    assert out[0, 4] < 0  # v_x points back inside
    # a particle outside the grid's domain has no density and does not move
    rec[0, 0:3] = [0.0, -3.0, 0.0]
    out2, _ = oracle_mod.sph_execute(rec, [1.0, 2.0, 1.0], 3)
    assert out2[0, 11] == 0 and np.array_equal(out2[0, 0:3], rec[0, 0:3])


SPH_GOLDEN = ["sph_dambreak", "sph_walls"]


def load_sph_golden(name):
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    return dict(np.load(os.path.join(here, "golden", f"{name}.npz")))


@pytest.mark.parametrize("name", SPH_GOLDEN)
def test_sph_oracle_reproduces_wgsl_golden(oracle_mod, name):
    """The reference's SPH shaders run by the WGSL interpreter
    (tests/golden/make_golden_sph.py): the C oracle reproduces every record
    and posvel after every substep bit for bit, box changes and particles
    outside the grid included."""
    f = load_sph_golden(name)
    rec = f["records"].copy()
    for s in range(int(f["substeps"])):
        rec, pv = oracle_mod.sph_execute(rec, [float(x) for x in f["real_halves"][s]], 1)
        assert_bits_equal(rec, f[f"s{s}_particles"], f"{name} substep {s} records")
        assert_bits_equal(pv, f[f"s{s}_posvel"], f"{name} substep {s} posvel")


def test_sph_golden_fixtures_cover_the_paths():
    d = load_sph_golden("sph_dambreak")
    assert (d["s0_particles"][:, 11] > 0).all()            # every particle has neighbours
    assert (d["s0_particles"][:, 11] > 15000).any()        # positive pressure somewhere
    w = load_sph_golden("sph_walls")
    assert (np.abs(w["records"][:, 0]) > w["real_halves"][0][0]).any()  # wall forces
    assert (w["real_halves"][1] != w["real_halves"][2]).any()          # box change
    assert (w["s3_particles"][:3, 11] == 0).all() and int(w["oob"]) > 0  # outside the grid
