"""The C ABI without a GPU: the library loads, exports every function that
include/mpm.h declares, and its host-only scene builders match the oracle's
restatements bit for bit."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from helpers import assert_bits_equal


def test_exports_every_declared_symbol(pkg):
    lib = pkg._lib.load()
    declared = pkg._lib.declared_functions()
    assert len(declared) >= 20
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, f"not exported: {missing}"


def test_error_strings(pkg):
    lib = pkg._lib.load()
    assert lib.mpm_error_string(pkg._lib.MPM_E_GRID_CAPACITY) == \
        b"gridCount should be equal to or less than maxGridCount"
    assert lib.mpm_error_string(0) == b"ok"


def test_null_handles_are_rejected(pkg):
    lib = pkg._lib.load()
    assert lib.mpm_step(None, 2, None) == pkg._lib.MPM_E_INVALID
    assert lib.mpm_set_real_box(None, None) == pkg._lib.MPM_E_INVALID
    assert lib.mpm_num_particles(None) == 0
    assert lib.mpm_destroy(None) == 0
    E = pkg._lib.MPM_E_INVALID
    assert lib.mpm_download_posvel_async(None, None, None) == E
    assert lib.mpm_wait_posvel(None, None) == E
    assert lib.mpm_batch_upload(None, None) == E
    assert lib.mpm_backward(None, None, None, 0, None, None, None) == E
    assert lib.mpm_backward_list(None, None, None, 0, None, None, None) == E
    assert lib.mpm_sph_set_graph(None, 1) == E
    assert lib.mpm_set_lane_table_min(None, 128) == E
    assert lib.mpm_get_lane_table_min(None) == E
    assert lib.mpm_batch_set_lane_table_min(None, 128) == E
    assert lib.mpm_batch_get_lane_table_min(None) == E
    assert lib.mpm_batch_get_task_size(None) == E
    assert lib.mpm_adjoint_set_observations(None, 0, None, None) == E
    assert lib.mpm_adjoint_observation_loss(None, None, None) == E
    assert lib.mpm_backward_observed(None, None, None, None) == E


def test_default_params_are_the_reference_constants(pkg):
    p = pkg.default_params()
    assert (p.stiffness, p.rest_density, p.dt) == (3.0, 4.0, np.float32(0.2))
    assert np.float32(p.dynamic_viscosity) == np.float32(0.1)
    assert p.fixed_point_multiplier == 1e7


@pytest.mark.parametrize("box,n,seed", [
    ([40, 30, 60], 70000, 0),      # main.ts:128-129 defaults
    ([35, 25, 55], 40000, 1),
    ([50, 50, 80], 200000, 2),
    ([45.5, 40.25, 80.75], 120000, 3),
    ([12, 10, 14], 10**6, 4),       # fewer lattice sites than asked
])
def test_dambreak_scene_matches_restatement(pkg, box, n, seed):
    from oracle import scene
    got = pkg.scene_dambreak(box, n, seed)
    want = scene.dambreak(box, n, seed)
    assert_bits_equal(got, want, f"initDambreak {box} n={n}")


def test_lattice_scene_matches_restatement(pkg):
    from oracle import scene
    got = pkg.scene_lattice(12, 3.0, 0.5, 0.05, 2024)
    want = scene.lattice(12, 3.0, 0.5, 0.05, 2024)
    assert_bits_equal(got, want, "lattice")
    assert got.shape == (12 ** 3, 20)
    assert np.all(np.abs(got[:, 0:3] - np.round((got[:, 0:3] - 3.0) / 0.5) * 0.5 - 3.0) <= 0.0501)


def test_lattice_vectorised_equals_sequential_definition():
    """oracle/scene.py draws the lattice's jitter with a vectorised SplitMix64;
    it must equal the plain sequential loop draw for draw."""
    from oracle import scene
    for args in ((9, 3.0, 0.5, 0.05, 7), (16, 8.0, 0.5, 0.05, 3), (5, 4.0, 0.5, 0.05, 20240601)):
        assert_bits_equal(scene.lattice(*args), scene.lattice_sequential(*args), f"lattice {args}")


def test_benchmark_lattice_matches_restatement(pkg):
    """The 1,000,000-particle benchmark scene (100^3 points from 4, spacing
    0.5, jitter 0.05, seed 20240601): the library's builder and the oracle's
    give the same bits, so the CPU reference arm never needs the library."""
    from oracle import scene
    got = pkg.scene_lattice(100, 4.0, 0.5, 0.05, 20240601)
    want = scene.lattice(100, 4.0, 0.5, 0.05, 20240601)
    assert_bits_equal(got, want, "1M lattice")


def test_no_device_is_reported_not_faked(pkg):
    """Without a GPU, creating a simulator fails loudly (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.MPMError, match="no CUDA device"):
        pkg.MLSMPMSimulator(None, None, 1.2)


def test_batch_scene_generator_is_seeded_and_in_range(pkg):
    """batch_scenes: counts, sides, walls, gravity magnitude, stiffness range."""
    d1, r1 = pkg.batch_scenes(12, seed=3)
    d2, r2 = pkg.batch_scenes(12, seed=3)
    assert np.array_equal(r1, r2)
    assert [d.num_particles for d in d1] == [d.num_particles for d in d2]
    off = 0
    for d in d1:
        n = d.num_particles
        side = d.init_box[0]
        assert 4000 <= n <= 64000 and side in (32.0, 48.0, 64.0)
        assert tuple(d.init_box) == (side, side, side) == tuple(d.real_box)
        pos = r1[off:off + n, :3]
        assert pos.min() >= 3.0 and pos.max() <= side - 4.0
        assert np.all(r1[off:off + n, 3:] == 0)
        g = np.array(list(d.gravity), dtype=np.float64)
        assert abs(np.linalg.norm(g) - 0.3) < 1e-6
        assert 2.0 <= d.stiffness <= 4.0
        off += n
    assert off == len(r1)
