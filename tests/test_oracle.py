"""The C oracle against hand-derived known answers (CPU only).

The reference ships no tests or golden vectors, so these answers are derived
from the WGSL source by hand (mls-mpm/p2g_1.wgsl, p2g_2.wgsl,
updateGrid.wgsl, g2p.wgsl); tests/test_golden.py adds vectors produced by
running the WGSL source itself through an independent interpreter.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import assert_bits_equal

FM = 1e7


def one_particle(pos, v=(0.0, 0.0, 0.0), C=None):
    p = np.zeros((1, 20), dtype=np.float32)
    p[0, 0:3] = pos
    p[0, 4:7] = v
    if C is not None:
        C = np.asarray(C, dtype=np.float32)  # C[col][row]
        for c in range(3):
            p[0, 8 + 4 * c: 11 + 4 * c] = C[c]
    return p


def test_conversion_rules(oracle_mod):
    enc = oracle_mod.enc
    assert enc(0.5) == 5_000_000
    assert enc(-1.5e-7) == -1          # truncation toward zero
    assert enc(0.9e-7) == 0
    assert enc(float("nan")) == 0
    assert enc(float("inf")) == 2**31 - 1
    assert enc(float("-inf")) == -2**31
    assert enc(214.7483648) == 2**31 - 1  # 2^31 saturates
    assert enc(-214.7483648) == -2**31
    assert oracle_mod.dec(5_000_000) == np.float32(0.5)
    assert oracle_mod.dec(1) == np.float32(np.float32(1.0) / np.float32(1e7))


def test_single_particle_at_cell_centre(oracle_mod):
    """x = c + 0.5: d = 0 so the 1D weights are 1/8, 3/4, 1/8 exactly."""
    box = [16.0, 16.0, 16.0]
    sim = oracle_mod.OracleSim(one_particle([8.5, 7.5, 9.5]), box)
    sim.clear_grid()
    sim.p2g_1()
    w = [0.125, 0.75, 0.125]
    for gx in range(3):
        for gy in range(3):
            for gz in range(3):
                cx, cy, cz = 8 + gx - 1, 7 + gy - 1, 9 + gz - 1
                idx = cx * 16 * 16 + cy * 16 + cz
                want = int(np.float32(np.float32(w[gx] * w[gy]) * w[gz]) * np.float32(FM))
                assert sim.cells[idx, 3] == want
                assert tuple(sim.cells[idx, 0:3]) == (0, 0, 0)
    # the 27 weights sum to 1 exactly, but enc truncates: the 8 corners
    # (0.125^3 * 1e7 = 19531.25) lose 0.25 each, the 12 edges
    # (0.125^2 * 0.75 * 1e7 = 117187.5) lose 0.5 each
    assert sim.cells[:, 3].sum() == 10_000_000 - 8


def test_partition_of_unity_and_momentum(oracle_mod):
    """Grid mass sums to N*FM minus truncation; with C = 0 the momentum is
    sum over stencil of enc(w*v)."""
    rng = np.random.default_rng(3)
    n = 500
    p = np.zeros((n, 20), dtype=np.float32)
    p[:, 0:3] = rng.uniform(4, 20, (n, 3))
    p[:, 4:7] = rng.uniform(-1, 1, (n, 3))
    sim = oracle_mod.OracleSim(p, [24.0, 24.0, 24.0])
    sim.clear_grid()
    sim.p2g_1()
    total = int(sim.cells[:, 3].astype(np.int64).sum())
    assert n * FM - 27 * n <= total <= n * FM + 27 * n
    # momentum x: recompute per particle in numpy float32, same op order
    want = 0
    for i in range(n):
        x = p[i, 0:3]
        ci = np.floor(x)
        d = x - (ci + np.float32(0.5))
        w = [np.float32(0.5) * (np.float32(0.5) - d) * (np.float32(0.5) - d),
             np.float32(0.75) - d * d,
             np.float32(0.5) * (np.float32(0.5) + d) * (np.float32(0.5) + d)]
        for gx in range(3):
            for gy in range(3):
                for gz in range(3):
                    wt = np.float32(np.float32(w[gx][0] * w[gy][1]) * w[gz][2])
                    want += oracle_mod.enc(float(np.float32(wt * (p[i, 4] + np.float32(0.0)))))
    assert int(sim.cells[:, 0].astype(np.int64).sum()) == want


def test_update_grid_boundary_band(oracle_mod):
    """updateGrid.wgsl:26-44: v = p/m + gravity*dt in y, zeroed in the wall band
    (index < 2 or > ceil(real) - 3)."""
    box = [10.0, 10.0, 10.0]
    sim = oracle_mod.OracleSim(np.zeros((0, 20), np.float32), box)
    sim.cells[:] = 0
    for (x, y, z) in [(1, 5, 5), (2, 5, 5), (7, 5, 5), (8, 5, 5), (5, 1, 5), (5, 7, 7),
                      (5, 5, 8), (5, 5, 5)]:
        idx = x * 100 + y * 10 + z
        sim.cells[idx] = [oracle_mod.enc(0.2), oracle_mod.enc(0.4), oracle_mod.enc(-0.2),
                          oracle_mod.enc(2.0)]
    sim.cells[3 * 100 + 3 * 10 + 3] = [123, 456, 789, 0]   # mass 0: untouched
    sim.update_grid()
    vx = oracle_mod.enc(float(np.float32(oracle_mod.dec(oracle_mod.enc(0.2)) /
                                         oracle_mod.dec(oracle_mod.enc(2.0)))))
    c = sim.cells
    assert c[5 * 100 + 5 * 10 + 5, 0] == vx
    gy = np.float32(np.float32(-0.3) * np.float32(0.2))
    vy = np.float32(oracle_mod.dec(oracle_mod.enc(0.4)) / oracle_mod.dec(oracle_mod.enc(2.0)))
    assert c[5 * 100 + 5 * 10 + 5, 1] == oracle_mod.enc(float(np.float32(vy + gy)))
    assert c[1 * 100 + 5 * 10 + 5, 0] == 0      # x = 1 < 2
    assert c[2 * 100 + 5 * 10 + 5, 0] == vx     # x = 2 inside
    assert c[7 * 100 + 5 * 10 + 5, 0] == vx     # x = 7 = ceil(10) - 3 inside
    assert c[8 * 100 + 5 * 10 + 5, 0] == 0      # x = 8 > 7
    assert c[5 * 100 + 1 * 10 + 5, 1] == 0
    assert c[5 * 100 + 5 * 10 + 8, 2] == 0
    assert tuple(c[3 * 100 + 3 * 10 + 3]) == (123, 456, 789, 0)
    # a smaller real box moves the upper band (changeBoxSize)
    sim.cells[7 * 100 + 5 * 10 + 5] = [oracle_mod.enc(0.2), 0, 0, oracle_mod.enc(2.0)]
    sim.change_box_size([9.5, 10.0, 10.0])      # ceil(9.5) - 3 = 7
    sim.update_grid()
    assert sim.cells[7 * 100 + 5 * 10 + 5, 0] != 0
    sim.cells[7 * 100 + 5 * 10 + 5] = [oracle_mod.enc(0.2), 0, 0, oracle_mod.enc(2.0)]
    sim.change_box_size([8.9, 10.0, 10.0])      # ceil(8.9) - 3 = 6
    sim.update_grid()
    assert sim.cells[7 * 100 + 5 * 10 + 5, 0] == 0


def test_q1_index_aliasing(oracle_mod):
    """A particle with floor(y) = 0 writes its gy = 0 row to flat index
    x*Y*Z - Z + z, i.e. cell (x-1, Y-1, z) (no per-axis bounds check)."""
    box = [16.0, 12.0, 16.0]
    sim = oracle_mod.OracleSim(one_particle([8.5, 0.5, 8.5]), box)
    sim.clear_grid()
    sim.p2g_1()
    Y, Z = 12, 16
    for gx in range(3):
        for gz in range(3):
            cx, cz = 8 + gx - 1, 8 + gz - 1
            alias = (cx - 1) * Y * Z + (Y - 1) * Z + cz
            assert sim.cells[alias, 3] > 0
    assert sim.oob == 0


def test_out_of_range_is_dropped_and_counted(oracle_mod):
    box = [8.0, 8.0, 8.0]
    sim = oracle_mod.OracleSim(one_particle([0.5, 0.5, 0.5]), box)
    sim.clear_grid()
    sim.p2g_1()
    assert sim.oob > 0
    sim2 = oracle_mod.OracleSim(one_particle([100.0, 4.0, 4.0]), box)
    sim2.clear_grid()
    sim2.p2g_1()
    assert sim2.oob == 27 and not sim2.cells.any()


def test_stage_sequence_equals_execute_and_threads(oracle_mod):
    from oracle import scene
    box = [40.0, 30.0, 60.0]
    parts = scene.dambreak(box, 30000, 5)
    a = oracle_mod.OracleSim(parts, box)
    b = oracle_mod.OracleSim(parts, box)
    c = oracle_mod.OracleSim(parts, box)
    for _ in range(3):
        a.substep()
    b.execute(3, 1)
    c.execute(3, 4)
    for other in (b, c):
        assert_bits_equal(other.cells, a.cells, "grid")
        assert_bits_equal(other.particles, a.particles, "particles")
        assert_bits_equal(other.posvel, a.posvel, "posvel")


def test_g2p_clamp_and_walls(oracle_mod):
    """g2p.wgsl:72-90 on an empty grid: v = 0, C = 0, x clamped to
    [1, real-2], then the soft wall pushes v by 0.3*(wall - x_n)."""
    box = [16.0, 16.0, 16.0]
    sim = oracle_mod.OracleSim(one_particle([0.25, 15.5, 8.0], v=(5, 5, 5)), box)
    sim.clear_grid()
    sim.g2p()
    p = sim.particles[0]
    assert p[0] == 1.0 and p[1] == 14.0 and p[2] == 8.0
    assert p[4] == np.float32(np.float32(0.3) * (np.float32(3.0) - np.float32(1.0)))
    assert p[5] == np.float32(np.float32(0.3) * (np.float32(12.0) - np.float32(14.0)))
    assert p[6] == 0.0
    assert not p[8:20].any()


@pytest.mark.parametrize("seed", [0, 1])
def test_grid_is_permutation_invariant(oracle_mod, seed):
    from oracle import scene
    box = [32.0, 32.0, 32.0]
    parts = scene.lattice(14, 6.0, 0.5, 0.05, seed)
    perm = np.random.default_rng(seed).permutation(len(parts))
    a = oracle_mod.OracleSim(parts, box)
    b = oracle_mod.OracleSim(parts[perm], box)
    a.execute(2)
    b.execute(2)
    assert_bits_equal(a.cells, b.cells, "grid")
    assert_bits_equal(a.particles[perm], b.particles, "particles")


def test_fp64_model_tracks_the_fixed_point_oracle(oracle_mod):
    """The FP64 continuous restatement (finite-difference reference of the
    derivative path) stays within the fixed-point quantisation of the f32
    oracle over 20 substeps."""
    from oracle import scene
    recs = scene.lattice(12, 9.0, 0.5, 0.05, 3)
    box = [32.0, 32.0, 32.0]
    ref = oracle_mod.OracleSim(recs, box)
    ref.execute(20, 2)
    st = oracle_mod.run64(oracle_mod.records_to_state64(recs), oracle_mod.Params64.make(box), 20)
    assert np.abs(ref.particles[:, 0:3] - st[:, 0:3]).max() < 5e-4
    assert np.abs(ref.particles[:, 4:7] - st[:, 3:6]).max() < 5e-4
    # gravity vector and stiffness reach the FP64 model
    st2 = oracle_mod.run64(oracle_mod.records_to_state64(recs),
                           oracle_mod.Params64.make(box, gravity=(0.3, 0.0, 0.0)), 5)
    assert st2[:, 3].mean() > 0.0 > st[:, 4].mean()
