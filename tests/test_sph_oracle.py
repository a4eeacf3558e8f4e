"""CPU checks of the SPH path: the library's initDambreak (host code,
sph/sph.ts:357-381) against its restatement in oracle/scene.py, and known
answers of the SPH oracle (oracle/sph_oracle.c)."""
from __future__ import annotations

import math

import numpy as np

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
