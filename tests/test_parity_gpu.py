"""GPU parity: libmpm.so (through its C ABI) against the CPU oracle.

Grid, particle state and posvel are compared bit for bit (integer grid sums
are exact; every per-particle float operation follows the same rounding
sequence), so the tolerance is zero.  Workloads: the reference's own scene
(initDambreak, mls-mpm/mls-mpm.ts:195-223, UI defaults main.ts:128-129,194)
and the benchmark lattices (64k particles on 64^3, 1M on 128^3).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import NTHREADS, assert_bits_equal, assert_state_equal

pytestmark = pytest.mark.gpu

ENGINES = ["sorted", "dispatch"]


def make_sim(pkg, engine, max_particles=200000, max_grid=(64, 64, 64), seed=11):
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=max_particles, maxGrid=max_grid,
                              seed=seed)
    sim.engine = engine
    return sim


def test_conversions_match_oracle(cuda, pkg, oracle_mod):
    special = np.array([0.0, -0.0, 1e-8, -1e-8, 0.9e-7, 1.0e-7, 1.1e-7, -1.1e-7, 0.5, -0.5,
                        214.7483647, 214.7483648, 214.75, -214.7483648, -214.75, 1e30, -1e30,
                        np.inf, -np.inf, np.nan, 1.4e-45, -1.4e-45, 3.4e38, 123.456789,
                        -987.654321], dtype=np.float32)
    rng = np.random.default_rng(5)
    rand = (rng.standard_normal(20000) * np.exp(rng.uniform(-20, 8, 20000))).astype(np.float32)
    bits = rng.integers(0, 2**32, 20000, dtype=np.uint64).astype(np.uint32).view(np.float32)
    vals = np.concatenate([special, rand, bits])
    enc, dec = pkg.probe_conversions(vals, 1e7)
    want_enc = np.array([oracle_mod.enc(float(v)) for v in vals], dtype=np.int32)
    ints = vals.view(np.int32)
    want_dec = np.array([oracle_mod.dec(int(i)) for i in ints], dtype=np.float32)
    assert_bits_equal(enc, want_enc, "enc")
    assert_bits_equal(dec, want_dec, "dec")


def test_each_wgsl_entry_point_matches_oracle(cuda, pkg, oracle_mod):
    """mpm_dispatch runs one kernel; compare after every kernel of 2 substeps."""
    box = [30.0, 24.0, 40.0]
    sim = make_sim(pkg, "dispatch")
    sim.reset(6000, box)
    ref = oracle_mod.OracleSim(sim.downloadParticles(), box)
    for sub in range(2):
        for kernel, step in [("clearGrid", ref.clear_grid), ("p2g_1", ref.p2g_1),
                             ("p2g_2", ref.p2g_2), ("updateGrid", ref.update_grid),
                             ("g2p", ref.g2p), ("copyPosition", ref.copy_position)]:
            sim.dispatch(kernel)
            step()
            assert_state_equal(sim, ref, f"substep {sub} after {kernel}")
    sim.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_reference_scene_frames(cuda, pkg, oracle_mod, engine):
    """The reference's default scene (70,000 particles, box 40x30x60, which
    also exercises quirk Q1: bottom particles start in cell row y = 0)."""
    box = [40.0, 30.0, 60.0]
    sim = make_sim(pkg, engine)
    sim.reset(70000, box)
    assert sim.numParticles == 70000
    assert sim.gridCount == 40 * 30 * 60
    ref = oracle_mod.OracleSim(sim.downloadParticles(), box)
    for frame in range(12):
        sim.execute()
        ref.execute(2, NTHREADS)
        assert_state_equal(sim, ref, f"{engine} frame {frame}")
    sim.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_lattice_64k_long_run(cuda, pkg, oracle_mod, engine):
    """The 64,000-particle lattice on a 64^3 grid for 100 frames (200 substeps)."""
    from oracle import scene
    box = [64.0, 64.0, 64.0]
    parts = scene.lattice(40, 3.0, 0.5, 0.05, 2024)
    sim = make_sim(pkg, engine)
    sim.upload(parts, box)
    ref = oracle_mod.OracleSim(parts, box)
    checkpoints = {0, 1, 9, 49, 99}
    done = 0
    for frame in range(100):
        sim.execute()
        if frame in checkpoints:
            ref.execute(2 * (frame + 1 - done), NTHREADS)
            done = frame + 1
            assert_state_equal(sim, ref, f"{engine} frame {frame}")
    sim.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_change_box_size(cuda, pkg, oracle_mod, engine):
    """changeBoxSize shrinks the walls (main.ts:249-262): updateGrid's BC band
    and g2p's clamp/walls follow real_box while indices keep init_box."""
    box = [32.0, 28.0, 48.0]
    sim = make_sim(pkg, engine)
    sim.reset(20000, box)
    ref = oracle_mod.OracleSim(sim.downloadParticles(), box)
    for frame, z in enumerate([48.0, 44.5, 40.0, 36.25, 36.25, 42.0]):
        real = [32.0, 28.0, z]
        sim.changeBoxSize(real)
        ref.change_box_size(real)
        sim.execute()
        ref.execute(2, NTHREADS)
        assert_state_equal(sim, ref, f"{engine} frame {frame} real_z={z}")
    sim.close()


def test_engines_agree_and_are_deterministic(cuda, pkg):
    box = [40.0, 30.0, 60.0]
    results = []
    for engine in ENGINES + ["sorted"]:
        sim = make_sim(pkg, engine, seed=3)
        sim.reset(50000, box)
        for _ in range(5):
            sim.execute()
        results.append((sim.downloadGrid(), sim.downloadParticles()))
        sim.close()
    for g, p in results[1:]:
        assert_bits_equal(g, results[0][0], "grid")
        assert_bits_equal(p, results[0][1], "particles")


def test_permutation_invariance(cuda, pkg, oracle_mod):
    """Integer grid sums do not depend on particle order."""
    from oracle import scene
    box = [48.0, 48.0, 48.0]
    parts = scene.lattice(24, 6.0, 0.5, 0.05, 77)
    perm = np.random.default_rng(1).permutation(len(parts))
    outs = []
    for p in (parts, parts[perm]):
        sim = make_sim(pkg, "sorted")
        sim.upload(p, box)
        for _ in range(3):
            sim.execute()
        outs.append((sim.downloadGrid(), sim.downloadParticles()))
        sim.close()
    assert_bits_equal(outs[0][0], outs[1][0], "grid under permutation")
    assert_bits_equal(outs[0][1][perm], outs[1][1], "particles under permutation")


@pytest.mark.parametrize("engine", ENGINES)
def test_small_and_ragged_counts(cuda, pkg, oracle_mod, engine):
    """N = 0, 1 and counts that are not multiples of 64 (quirk Q2: the
    reference dispatches ceil(N/64)*64 threads; this library runs exactly N)."""
    box = [20.0, 20.0, 20.0]
    for n in (0, 1, 63, 65, 1001):
        sim = make_sim(pkg, engine, max_particles=2048, max_grid=(32, 32, 32))
        sim.reset(n, box)
        assert sim.numParticles == n
        ref = oracle_mod.OracleSim(sim.downloadParticles(), box)
        for _ in range(3):
            sim.execute()
            ref.execute(2)
        assert_state_equal(sim, ref, f"{engine} n={n}")
        sim.close()


def test_capacity_errors(cuda, pkg):
    sim = make_sim(pkg, "sorted", max_particles=1000, max_grid=(16, 16, 16))
    with pytest.raises(pkg.GridCapacityError, match="gridCount should be equal to or less than maxGridCount"):
        sim.reset(100, [17.0, 16.0, 16.0])
    with pytest.raises(pkg.MPMError):
        sim.reset(1001, [16.0, 16.0, 16.0])
    with pytest.raises(pkg.MPMError):
        sim.execute()  # nothing loaded yet
    sim.reset(1000, [16.0, 16.0, 16.0])
    sim.execute()
    sim.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_out_of_box_and_nonfinite_particles(cuda, pkg, oracle_mod, engine):
    """Particles outside the box alias or fall off the grid (the global path)
    and NaN particles feed enc(NaN) = 0; both engines still match the oracle."""
    from oracle import scene
    box = [24.0, 24.0, 24.0]
    parts = scene.lattice(10, 6.0, 0.5, 0.05, 5)
    parts[0, 0:3] = [0.2, 12.0, 12.0]      # x stencil at -1
    parts[1, 0:3] = [12.0, 0.3, 12.0]      # y stencil at -1: aliases into x-1
    parts[2, 0:3] = [12.0, 12.0, 23.7]     # z stencil beyond the box
    parts[3, 0:3] = [30.0, 30.0, 30.0]     # far outside
    parts[4, 4:7] = [50.0, -40.0, 30.0]    # very fast
    parts[5, 8] = np.nan                   # NaN in C: absorbed, enc(NaN) = 0
    parts[6, 8:11] = [1e30, -1e30, 1e30]   # saturating encodes
    parts[7, 0] = np.nan                   # NaN position
    sim = make_sim(pkg, engine, max_particles=2048, max_grid=(32, 32, 32))
    sim.upload(parts, box)
    ref = oracle_mod.OracleSim(parts, box)
    for frame in range(3):
        sim.execute()
        ref.execute(2)
        g = sim.downloadGrid()
        assert_bits_equal(g, ref.cells, f"{engine} frame {frame} grid")
        p = sim.downloadParticles()
        finite = np.isfinite(ref.particles)
        assert np.array_equal(np.isfinite(p), finite), "non-finite pattern differs"
        assert_bits_equal(p[finite], ref.particles[finite], f"{engine} frame {frame} particles")
    health = sim.checkHealth()
    assert health["out_of_range_accesses"] > 0
    # g2p rebuilds v and C from the grid and the clamp maps a NaN position to
    # 1.0, so non-finite state heals within two substeps: the watchdog sees
    # it after a single one
    assert health["nonfinite_particles"] == 0 and health["ok"]
    bad = parts.copy()
    bad[7, 0] = np.nan
    sim.upload(bad, box)
    ref = oracle_mod.OracleSim(bad, box)
    sim.execute(substeps=1)
    ref.execute(1)
    health = sim.checkHealth()
    want = int((~np.isfinite(ref.particles)).any(axis=1).sum())
    assert want >= 1
    assert health["nonfinite_particles"] == want and not health["ok"]
    sim.close()


def test_caller_owned_posvel_buffer(cuda, pkg, oracle_mod):
    """posvelBuffer owned by the caller (main.ts:115-119), as a torch tensor."""
    torch = cuda
    box = [30.0, 24.0, 40.0]
    posvel = torch.zeros(8 * 10000, dtype=torch.float32, device="cuda")
    particles = torch.zeros(20 * 10000, dtype=torch.float32, device="cuda")
    sim = pkg.MLSMPMSimulator(particles, posvel, 1.2, maxParticles=10000, seed=9)
    sim.reset(8000, box)
    assert sim.posvelDevicePtr() == posvel.data_ptr()
    recs = particles[: 20 * sim.numParticles].cpu().numpy().reshape(-1, 20)
    ref = oracle_mod.OracleSim(recs, box)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        sim.execute(stream)
    stream.synchronize()
    ref.execute(2)
    got = posvel[: 8 * sim.numParticles].cpu().numpy().reshape(-1, 8)
    assert_bits_equal(got, ref.posvel, "caller-owned posvel")
    sim.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_lattice_1m_128(cuda, pkg, oracle_mod, engine):
    """The 1,000,000-particle lattice on a 128^3 grid (beyond the reference's
    64^3 / 200k caps): bit-exact against the oracle for 2 frames."""
    from oracle import scene
    box = [128.0, 128.0, 128.0]
    parts = scene.lattice(100, 4.0, 0.5, 0.05, 99)
    sim = make_sim(pkg, engine, max_particles=1_000_000, max_grid=(128, 128, 128))
    sim.upload(parts, box)
    ref = oracle_mod.OracleSim(parts, box)
    for frame in range(2):
        sim.execute()
        ref.execute(2, NTHREADS)
        assert_state_equal(sim, ref, f"{engine} 1M frame {frame}")
    sim.close()


def test_benchmark_workload_200_frames(cuda, pkg, oracle_mod):
    """The benchmarked configuration exactly: the 1,000,000-particle lattice
    (100^3 points from 4, spacing 0.5, jitter 0.05, seed 20240601) on 128^3,
    the sorted engine with CUDA graphs, for the configuration's full 200
    frames (400 substeps); grid, particles and posvel bit-exact against the
    oracle after frames 1, 5, 25, 100 and 200."""
    from oracle import scene
    box = [128.0, 128.0, 128.0]
    parts = scene.lattice(100, 4.0, 0.5, 0.05, 20240601)
    sim = make_sim(pkg, "sorted", max_particles=1_000_000, max_grid=(128, 128, 128))
    sim.upload(parts, box)
    ref = oracle_mod.OracleSim(parts, box)
    checks = {1, 5, 25, 100, 200}
    for frame in range(1, 201):
        sim.execute()
        ref.execute(2, NTHREADS)
        if frame in checks:
            assert_state_equal(sim, ref, f"benchmark workload frame {frame}")
    sim.close()


def test_packed_f32x2_matches_scalar_ieee(cuda, pkg):
    """The sorted engine pairs independent products in mul.rn.f32x2 and adds
    them with scalar add.rn.f32 (ptxas would contract a packed product that
    feeds a packed add into one FMA rounding); each lane must round exactly
    like the scalar ops, including subnormal inputs and results, signed
    zeros, infinities and NaN."""
    rng = np.random.default_rng(11)
    n = 1 << 16
    special = np.array([0.0, -0.0, 1e-45, -1e-45, 1.17549435e-38, 1e-38, 3e-39, np.inf, -np.inf,
                        np.nan, 1.0, -1.0, 3.4e38, 2 ** -75, 2 ** -60, 1.5, 1e7], dtype=np.float32)
    a = np.concatenate([np.repeat(special, len(special)), np.tile(special, len(special)),
                        (rng.standard_normal(n) * np.exp(rng.uniform(-90, 90, n))).astype(np.float32)])
    b = np.concatenate([np.tile(special, len(special)), np.repeat(special, len(special)),
                        (rng.standard_normal(n) * np.exp(rng.uniform(-90, 90, n))).astype(np.float32)])
    if len(a) % 2:
        a, b = a[:-1], b[:-1]
    pm, pa, pma, sm, sa, sma = pkg.probe_packed(a, b)
    with np.errstate(all="ignore"):
        want_m = (a * b).astype(np.float32)
        want_a = (a + b).astype(np.float32)
        want_ma = (want_m + a).astype(np.float32)
    for got, want, what in [(pm, want_m, "packed mul"), (pa, want_a, "packed add"),
                            (pma, want_ma, "packed mul then scalar add (no contraction)"),
                            (sm, want_m, "scalar mul"), (sa, want_a, "scalar add"),
                            (sma, want_ma, "scalar mul then add (no contraction)")]:
        nan = np.isnan(want)
        assert np.array_equal(np.isnan(got), nan), what
        assert_bits_equal(got[~nan], want[~nan], what)
    assert (np.abs(want_m[np.isfinite(want_m)]) < 1.17549435e-38).sum() > 0  # subnormals covered


@pytest.mark.parametrize("cap", [64, 200, 1024, 0])
def test_task_size_does_not_change_results(cuda, pkg, oracle_mod, cap):
    """Bins split into tasks of at most `cap` particles: same bits."""
    box = [40.0, 30.0, 60.0]
    sim = make_sim(pkg, "sorted")
    sim.reset(70000, box)
    sim.taskSize = cap
    assert cap == 0 or sim.taskSize == cap
    ref = oracle_mod.OracleSim(sim.downloadParticles(), box)
    for _ in range(5):
        sim.execute()
        ref.execute(2, NTHREADS)
    assert_state_equal(sim, ref, f"task size {cap}")
    sim.close()


def test_lane_table_threshold_does_not_change_results(cuda, pkg, oracle_mod):
    """The lane table on every task (1), on none (2^30), or from 32 / 128
    particles: same bits as the oracle."""
    box = [40.0, 30.0, 60.0]
    sims = []
    for lane in (1, 32, 128, 1 << 30):
        sim = make_sim(pkg, "sorted")
        sim.reset(70000, box)
        sim.laneTableMin = lane
        assert sim.laneTableMin == lane
        sims.append((lane, sim))
    ref = oracle_mod.OracleSim(sims[0][1].downloadParticles(), box)
    for _ in range(5):
        for _, sim in sims:
            sim.execute()
        ref.execute(2, NTHREADS)
    for lane, sim in sims:
        assert_state_equal(sim, ref, f"lane table from {lane} particles")
        sim.close()
    sim = make_sim(pkg, "sorted")
    sim.laneTableMin = 0
    assert sim.laneTableMin == 128
    with pytest.raises(Exception):
        sim.laneTableMin = -1
    sim.close()


@pytest.mark.parametrize("threads", [128, 256, 512])
def test_task_threads_do_not_change_results(cuda, pkg, oracle_mod, threads):
    """The task kernels at 128, 256 or 512 threads per block, with the
    smallest and the default task sizes and the lane table always or never:
    same bits as the oracle (the reference's UI scene and the 64k lattice)."""
    from oracle import scene
    cases = [([40.0, 30.0, 60.0], None), ([64.0, 64.0, 64.0], scene.lattice(40, 3.0, 0.5, 0.05, 8))]
    for box, parts in cases:
        for cap, lane in ((64, 1), (0, 1 << 30)):
            sim = make_sim(pkg, "sorted")
            if parts is None:
                sim.reset(70000, box)
            else:
                sim.upload(parts, box)
            sim.taskThreads = threads
            sim.taskSize = cap
            sim.laneTableMin = lane
            assert sim.taskThreads == threads
            ref = oracle_mod.OracleSim(sim.downloadParticles(), box)
            for _ in range(4):
                sim.execute()
                ref.execute(2, NTHREADS)
            assert_state_equal(sim, ref, f"{threads} threads, task size {cap}, lane table {lane}")
            sim.close()
    sim = make_sim(pkg, "sorted")
    sim.taskThreads = 0
    assert sim.taskThreads == 256
    with pytest.raises(Exception):
        sim.taskThreads = 192
    sim.close()


def _quirk_scene():
    """A lattice with particles past every wall, fast, NaN and saturating
    ones (the global path and the padding bricks around the grid)."""
    from oracle import scene
    parts = scene.lattice(10, 6.0, 0.5, 0.05, 5)
    parts[0, 0:3] = [0.2, 12.0, 12.0]
    parts[1, 0:3] = [12.0, 0.3, 12.0]
    parts[2, 0:3] = [12.0, 12.0, 23.7]
    parts[3, 0:3] = [30.0, 30.0, 30.0]
    parts[4, 4:7] = [50.0, -40.0, 30.0]
    parts[5, 8] = np.nan
    parts[6, 8:11] = [1e30, -1e30, 1e30]
    return parts


@pytest.mark.parametrize("pairing", [0, 256, 1 << 30])
def test_bin_pairing_does_not_change_results(cuda, pkg, oracle_mod, pairing):
    """One-brick tasks only (0), z pairs of at most 256 particles merged into
    one task, or every pair whose two bins hold particles (2^30), at every
    block size, with the smallest and the default task sizes and the lane
    table always or never: same bits as the oracle on the reference's UI
    scene (60 cells along z: an odd brick count), the 64k lattice, a box of
    odd sizes and particles past every wall."""
    from oracle import scene
    cases = [([40.0, 30.0, 60.0], None, 70000),
             ([64.0, 64.0, 64.0], scene.lattice(40, 3.0, 0.5, 0.05, 8), None),
             ([37.0, 23.0, 29.0], None, 20000),
             ([24.0, 24.0, 24.0], _quirk_scene(), None)]
    for box, parts, n in cases:
        for threads, cap, lane in ((256, 0, 128), (128, 64, 1), (512, 0, 1 << 30)):
            sim = make_sim(pkg, "sorted")
            if parts is None:
                sim.reset(n, box)
            else:
                sim.upload(parts, box)
            sim.binPairing = pairing
            sim.taskThreads = threads
            sim.taskSize = cap
            sim.laneTableMin = lane
            assert sim.binPairing == pairing
            ref = oracle_mod.OracleSim(sim.downloadParticles(), box)
            for _ in range(4):
                sim.execute()
                ref.execute(2, NTHREADS)
            what = f"box {box}, pairing {pairing}, {threads} threads, task size {cap}, lane {lane}"
            assert_bits_equal(sim.downloadGrid(), ref.cells, what + " grid")
            p = sim.downloadParticles()
            finite = np.isfinite(ref.particles)
            assert np.array_equal(np.isfinite(p), finite), what
            assert_bits_equal(p[finite], ref.particles[finite], what + " particles")
            sim.close()


def test_bin_pairing_switch_mid_run(cuda, pkg, oracle_mod):
    """Changing the z-pair threshold between frames keeps the run bit for
    bit, and the grid of the last frame stays readable."""
    box = [40.0, 30.0, 60.0]
    sim = make_sim(pkg, "sorted")
    sim.reset(70000, box)
    ref = oracle_mod.OracleSim(sim.downloadParticles(), box)
    ran = False
    for pairing in (0, 1 << 30, 200, 0, 600):
        sim.binPairing = pairing
        if ran:
            assert_bits_equal(sim.downloadGrid(), ref.cells, f"grid after switching to {pairing}")
        for _ in range(2):
            sim.execute()
            ref.execute(2, NTHREADS)
        ran = True
        assert_state_equal(sim, ref, f"pairing {pairing}")
    assert sim.binPairing == 600
    sim.binPairing = 2**31 - 1
    assert sim.binPairing == 512
    with pytest.raises(Exception):
        sim.binPairing = -1
    sim.close()


def test_autotune_cache_file(cuda, pkg, tmp_path):
    """autotune(cache=...) times once per workload key and reapplies the
    stored choice afterwards."""
    import json
    box = [40.0, 30.0, 60.0]
    path = str(tmp_path / "tuning.json")
    sim = make_sim(pkg, "sorted")
    sim.reset(70000, box)
    sim.autotune(2, cache=path)
    choice = sim.tuning()
    table = json.load(open(path))
    assert list(table.values()) == [choice]
    sim2 = make_sim(pkg, "sorted")
    sim2.reset(70000, box)
    sim2.autotune(2, cache=path)
    assert sim2.tuning() == choice
    sim.close()
    sim2.close()


def test_autotune_keeps_the_state(cuda, pkg, oracle_mod):
    box = [40.0, 30.0, 60.0]
    sim = make_sim(pkg, "sorted")
    sim.reset(70000, box)
    ref = oracle_mod.OracleSim(sim.downloadParticles(), box)
    for _ in range(3):
        sim.execute()
        ref.execute(2, NTHREADS)
    before = (sim.downloadParticles(), sim.downloadGrid(), sim.downloadPosvel())
    chosen = sim.autotune(4)
    assert chosen in (64, 128, 256, 512, 1024) and sim.taskSize == chosen
    assert sim.laneTableMin in (32, 128, 512, 1 << 30)
    assert sim.taskThreads in (128, 256, 512)
    assert sim.binPairing in (0, 256, 512, 1 << 30)
    assert_bits_equal(sim.downloadParticles(), before[0], "particles after autotune")
    assert_bits_equal(sim.downloadGrid(), before[1], "grid after autotune")
    assert_bits_equal(sim.downloadPosvel(), before[2], "posvel after autotune")
    for _ in range(3):
        sim.execute()
        ref.execute(2, NTHREADS)
    assert_state_equal(sim, ref, "after autotune")
    sim.close()


def test_pipelined_posvel_readback(cuda, pkg):
    """downloadPosvelAsync copies the posvel of the moment of the call, even
    while the next execute() runs on the same stream."""
    import torch
    from oracle import scene as scene_mod
    recs = scene_mod.lattice(20, 6.0, 0.5, 0.05, 9)
    box = [40.0, 40.0, 40.0]
    ref = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=len(recs), maxGrid=(40, 40, 40))
    ref.upload(recs, box)
    want = []
    for _ in range(4):
        ref.execute()
        want.append(ref.downloadPosvel().copy())
    ref.close()
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=len(recs), maxGrid=(40, 40, 40))
    sim.upload(recs, box)
    stream = torch.cuda.Stream()
    bufs = [torch.empty((len(recs), 8), dtype=torch.float32, pin_memory=True).numpy()
            for _ in range(2)]
    sim.execute(stream)
    for i in range(4):
        out = sim.downloadPosvelAsync(stream, out=bufs[i % 2])
        sim.execute(stream)  # overlaps the copy; must not change `out`
        sim.waitPosvel()
        assert np.array_equal(out.view(np.uint32), want[i].view(np.uint32)), f"step {i}"
    sim.waitPosvel(stream)
    stream.synchronize()
    sim.close()
