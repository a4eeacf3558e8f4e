"""GPU parity of batched scenes: MLSMPMBatch (mpm_batch_* through the C ABI)
against the CPU oracle run on each scene alone, bit for bit.

A batch advances all its scenes in the same launches; each scene must still
give exactly what the reference's six dispatches (mls-mpm/mls-mpm.ts:245-268)
give for that scene alone, with that scene's stiffness, gravity and boxes.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import NTHREADS, assert_bits_equal

pytestmark = pytest.mark.gpu


def oracle_params(oracle_mod, d):
    return oracle_mod.Params.make(stiffness=d.stiffness, rest_density=d.rest_density,
                                  dynamic_viscosity=d.dynamic_viscosity, dt=d.dt,
                                  fixed_point_multiplier=d.fixed_point_multiplier,
                                  gravity=tuple(d.gravity))


def oracle_scene(oracle_mod, d, recs):
    return oracle_mod.OracleSim(recs, list(d.init_box), oracle_params(oracle_mod, d),
                                real_box=list(d.real_box))


def check_scene(batch, s, ref, what):
    lo, hi = batch.sceneOffsets[s], batch.sceneOffsets[s + 1]
    parts = batch.downloadParticles()[lo:hi]
    assert_bits_equal(batch.downloadGrid(s), ref.cells, f"{what} scene {s} grid")
    assert_bits_equal(parts, ref.particles, f"{what} scene {s} particles")


def mixed_scenes(pkg, scene_mod):
    """Uneven scenes: the reference's dam-break (quirk Q1 aliasing at y = 0),
    lattices with rotated gravity and other stiffnesses, a non-cubic box."""
    descs, recs = [], []
    db = pkg.scene_dambreak([30.0, 24.0, 40.0], 5000, 11)
    descs.append(pkg.scene_desc(len(db), (30.0, 24.0, 40.0)))
    recs.append(db)
    lat = scene_mod.lattice(14, 6.0, 0.5, 0.05, 3)
    descs.append(pkg.scene_desc(len(lat), (32, 32, 32), stiffness=2.2,
                                gravity=(0.17320508, -0.17320508, 0.17320508)))
    recs.append(lat)
    lat2 = scene_mod.lattice(11, 9.0, 0.5, 0.05, 4)
    descs.append(pkg.scene_desc(len(lat2), (24, 40, 36), stiffness=3.9,
                                gravity=(-0.3, 0.0, 0.0)))
    recs.append(lat2)
    sub, srec = pkg.batch_scenes(3, seed=7, n_range=(1500, 6000), sides=(32, 48))
    descs += sub
    recs.append(srec)
    return descs, np.concatenate(recs)


@pytest.mark.parametrize("graph", [True, False])
def test_mixed_batch_matches_oracle_per_scene(cuda, pkg, oracle_mod, graph):
    from oracle import scene as scene_mod
    descs, recs = mixed_scenes(pkg, scene_mod)
    batch = pkg.MLSMPMBatch(descs, recs, graph=graph)
    offs = batch.sceneOffsets
    refs = [oracle_scene(oracle_mod, d, recs[offs[s]:offs[s + 1]]) for s, d in enumerate(descs)]
    for frame in range(6):
        batch.execute()
        for r in refs:
            r.execute(2, NTHREADS)
        if frame in (0, 5):
            for s, r in enumerate(refs):
                check_scene(batch, s, r, f"frame {frame}")
    assert batch.checkHealth()["ok"]
    batch.close()


def test_batch_equals_single_scene_simulators(cuda, pkg):
    """Default constants: each scene equals an MLSMPMSimulator run alone."""
    boxes = [(30.0, 24.0, 40.0), (40.0, 30.0, 60.0), (20.0, 20.0, 20.0)]
    counts = [4000, 9000, 1500]
    descs, recs = [], []
    for i, (b, n) in enumerate(zip(boxes, counts)):
        r = pkg.scene_dambreak(b, n, 100 + i)
        descs.append(pkg.scene_desc(len(r), b))
        recs.append(r)
    batch = pkg.MLSMPMBatch(descs, np.concatenate(recs))
    sims = []
    for b, r in zip(boxes, recs):
        sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=20000)
        sim.upload(r, b)
        sims.append(sim)
    for _ in range(10):
        batch.execute()
        for sim in sims:
            sim.execute()
    parts = batch.downloadParticles()
    for s, sim in enumerate(sims):
        lo, hi = batch.sceneOffsets[s], batch.sceneOffsets[s + 1]
        assert_bits_equal(parts[lo:hi], sim.downloadParticles(), f"scene {s} particles")
        assert_bits_equal(batch.downloadGrid(s), sim.downloadGrid(), f"scene {s} grid")
        sim.close()
    batch.close()


def test_batch_change_box_size_and_constants(cuda, pkg, oracle_mod):
    """changeBoxSize / new constants of one scene between steps."""
    from oracle import scene as scene_mod
    descs, recs = mixed_scenes(pkg, scene_mod)
    batch = pkg.MLSMPMBatch(descs, recs)
    offs = batch.sceneOffsets
    refs = [oracle_scene(oracle_mod, d, recs[offs[s]:offs[s + 1]]) for s, d in enumerate(descs)]
    for frame in range(4):
        if frame == 2:
            batch.changeBoxSize(0, (26.5, 24.0, 33.25))
            refs[0].change_box_size((26.5, 24.0, 33.25))
            d = descs[1]
            new = pkg.scene_desc(d.num_particles, list(d.init_box), list(d.real_box),
                                 stiffness=3.5, dynamic_viscosity=0.15, gravity=(0.0, 0.0, -0.3))
            batch.setScene(1, new)
            refs[1].params = oracle_params(oracle_mod, new)
        batch.execute()
        for r in refs:
            r.execute(2, NTHREADS)
    for s, r in enumerate(refs):
        check_scene(batch, s, r, "after box change")
    batch.close()


def test_batch_rejects_bad_scenes(cuda, pkg):
    good = pkg.scene_desc(10, (16, 16, 16))
    bad = pkg.scene_desc(10, (16, 0.5, 16))  # i32(Y) == 0
    recs = np.zeros((20, 20), np.float32) + 8.0
    with pytest.raises(pkg.MPMError):
        pkg.MLSMPMBatch([good, bad], recs)
    with pytest.raises(ValueError):
        pkg.MLSMPMBatch([good], recs)
    batch = pkg.MLSMPMBatch([good], recs[:10])
    other = pkg.scene_desc(10, (20, 16, 16))
    with pytest.raises(pkg.MPMError):
        batch.setScene(0, other)  # geometry is fixed at creation
    batch.close()


def test_full_size_batch_spot_check(cuda, pkg, oracle_mod):
    """256 scenes, 4k-64k particles, sides 32/48/64: three scenes against the
    oracle after 4 substeps; every scene finite and in range."""
    descs, recs = pkg.batch_scenes(256, seed=20240601)
    batch = pkg.MLSMPMBatch(descs, recs)
    batch.step(4)
    offs = batch.sceneOffsets
    for s in (0, 97, 255):
        ref = oracle_scene(oracle_mod, descs[s], recs[offs[s]:offs[s + 1]])
        ref.execute(4, NTHREADS)
        check_scene(batch, s, ref, "full batch")
    h = batch.checkHealth()
    assert h["ok"] and h["out_of_range_accesses"] == 0
    assert batch.launchCount() > 0
    batch.close()


def test_batch_task_size_and_autotune(cuda, pkg, oracle_mod):
    from oracle import scene as scene_mod
    descs, recs = mixed_scenes(pkg, scene_mod)
    offs = np.concatenate([[0], np.cumsum([d.num_particles for d in descs])])
    results = []
    configs = ((64, 256, 0), (1024, 256, 0), (128, 128, 0), (512, 512, 0), (64, 256, 1 << 30),
               (1024, 128, 1 << 30), (0, 512, 300))
    for cap, threads, pairing in configs:
        batch = pkg.MLSMPMBatch(descs, recs)
        batch.setTaskSize(cap)
        batch.taskThreads = threads
        batch.binPairing = pairing
        assert batch.binPairing == pairing
        batch.step(3)
        if pairing:  # and off, mid-run
            batch.binPairing = 0
            batch.step(3)
            batch.binPairing = pairing
        else:
            batch.step(3)
        results.append(batch.downloadParticles())
        batch.close()
    for r, cfg in zip(results[1:], configs[1:]):
        assert_bits_equal(results[0], r, f"task size 64 vs (task size, threads, pairing) {cfg}")
    batch = pkg.MLSMPMBatch(descs, recs)
    batch.step(2)
    before = batch.downloadParticles()
    chosen = batch.autotune(2)
    assert chosen in (64, 128, 256, 512, 1024) and batch.taskSize == chosen
    assert batch.laneTableMin in (32, 128, 512, 1 << 30)
    assert batch.binPairing in (0, 256, 512, 1 << 30)
    assert_bits_equal(batch.downloadParticles(), before, "particles after autotune")
    batch.step(4)
    assert_bits_equal(batch.downloadParticles(), results[0], "after autotune")
    batch.close()


def test_batch_kernel_stats(cuda, pkg):
    """Per-kernel event timing of a batch: every stage of a substep is
    counted and timed; the results equal an unprofiled batch's."""
    from oracle import scene as scene_mod
    descs, recs = mixed_scenes(pkg, scene_mod)
    plain = pkg.MLSMPMBatch(descs, recs)
    plain.step(3)
    timed = pkg.MLSMPMBatch(descs, recs)
    timed.setProfiling(True)
    timed.step(3)
    st = timed.kernelStats()
    for name in ("sorted_p2g_2", "updateGrid", "sorted_g2p_p2g_1", "scan", "scatter"):
        launches, timed_launches, ms = st[name]
        assert launches >= 3 and timed_launches == launches and ms > 0.0, (name, st[name])
    assert_bits_equal(timed.downloadParticles(), plain.downloadParticles(), "profiled batch")
    plain.close()
    timed.close()


def test_batch_upload_restarts_and_reuses_graphs(cuda, pkg):
    """upload() restarts every scene from new records exactly as a fresh batch
    would, with the CUDA graph captured before the upload replayed."""
    from oracle import scene as scene_mod
    descs, recs = mixed_scenes(pkg, scene_mod)
    fresh = pkg.MLSMPMBatch(descs, recs)
    fresh.step(5)
    want = fresh.downloadParticles()
    fresh.close()
    batch = pkg.MLSMPMBatch(descs, recs)
    other = recs.copy()
    other[:, 4:7] += np.float32(0.05)
    batch.upload(other)
    batch.step(5)
    moved = batch.downloadParticles()
    launches = batch.launchCount()
    batch.upload(recs)
    batch.step(5)
    assert_bits_equal(batch.downloadParticles(), want, "after upload")
    assert not np.array_equal(moved, want)
    assert batch.launchCount() > launches
    with pytest.raises(ValueError):
        batch.upload(recs[:-1])
    batch.close()


def test_simulator_reupload_replays_its_graph(cuda, pkg):
    """Re-uploading the same scene keeps the simulator's captured graph and
    gives the same trajectory as the first run."""
    from oracle import scene as scene_mod
    recs = scene_mod.lattice(16, 6.0, 0.5, 0.05, 5)
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=len(recs), maxGrid=(32, 32, 32))
    sim.setGraph(True)
    outs = []
    for _ in range(3):
        sim.upload(recs, [32.0, 32.0, 32.0])
        sim.execute(substeps=7)
        outs.append(sim.downloadParticles())
    assert_bits_equal(outs[1], outs[0], "second upload")
    assert_bits_equal(outs[2], outs[0], "third upload")
    sim.close()
