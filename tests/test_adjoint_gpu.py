"""GPU checks of the differentiation path (mpm_forward_ckpt / mpm_backward).

Gradients are checked against central finite differences of the FP64
continuous model (oracle/mpm_oracle64.c), the function the adjoint
differentiates.  That function is only piecewise smooth (walls, position
clamp and the pressure threshold, mls-mpm/g2p.wgsl:72-90 and
p2g_2.wgsl:61-63, switch as particles cross them), so a finite difference
averages the slopes of the pieces inside [p - eps, p + eps] and moves with
eps; the reference value is the median over a few eps, and the tolerance is
the 1e-3 relative the derivative path targets.  Directions in state space
(positions, velocities, C) are random unit vectors over all particles.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TARGET = np.array([30.0, 10.0, 30.0])


def lattice_with_velocity(scene_mod, npa, origin, seed=3, vseed=1):
    recs = scene_mod.lattice(npa, origin, 0.5, 0.05, seed)
    rng = np.random.default_rng(vseed)
    recs[:, 4:7] = rng.normal(0.0, 0.1, (len(recs), 3)).astype(np.float32)
    return recs


def loss64(oracle_mod, st0, box, T, k=3.0, mu=0.1, sl=None, u=None, eps=0.0):
    st = st0
    if sl is not None:
        st = st0.copy()
        st[:, sl] += eps * u
    out = oracle_mod.run64(st, oracle_mod.Params64.make(box, stiffness=k, dynamic_viscosity=mu), T)
    c = out[:, 0:3].mean(axis=0)
    return float(np.sum((c - TARGET) ** 2))


def fd_median(oracle_mod, st0, box, T, what, eps_list, u=None):
    """Median over eps of the central difference of the centroid loss."""
    sl = {"x": slice(0, 3), "v": slice(3, 6), "C": slice(6, 15)}.get(what)

    def one(eps, sign):
        if what == "k":
            return loss64(oracle_mod, st0, box, T, k=3.0 + sign * eps)
        if what == "mu":
            return loss64(oracle_mod, st0, box, T, mu=0.1 + sign * eps)
        return loss64(oracle_mod, st0, box, T, sl=sl, u=u, eps=sign * eps)

    with ThreadPoolExecutor(max(1, min(16, os.cpu_count() or 1))) as ex:
        jobs = [(ex.submit(one, e, 1.0), ex.submit(one, e, -1.0), e) for e in eps_list]
        vals = [(p.result() - m.result()) / (2 * e) for p, m, e in jobs]
    return float(np.median(vals)), vals


def directional(grad, what, u):
    if what == "x":
        return float(np.sum(grad[:, 0:3].astype(np.float64) * u))
    if what == "v":
        return float(np.sum(grad[:, 4:7].astype(np.float64) * u))
    gc = np.concatenate([grad[:, 8:11], grad[:, 12:15], grad[:, 16:19]], axis=1)
    return float(np.sum(gc.astype(np.float64) * u))


def run_gradient(pkg, recs, box, T, every, tape="fp64"):
    adj = pkg.MLSMPMAdjoint([pkg.scene_desc(len(recs), box)], T, every, tape=tape)
    adj.forward(recs, T)
    final = adj.state(T)
    L, seed = pkg.centroid_loss(final, TARGET)
    grad, pgrad = adj.backward({T: seed})
    adj.close()
    return L[0], grad, pgrad


def check_against_fd(oracle_mod, recs, box, T, grad, pgrad, eps_list, tol, ndir=2):
    st0 = oracle_mod.records_to_state64(recs)
    rng = np.random.default_rng(17)
    checks = [("k", None), ("mu", None)]
    for what, width in (("v", 3), ("v", 3), ("x", 3), ("C", 9))[:ndir + 2]:
        u = rng.normal(size=(len(recs), width))
        checks.append((what, u / np.linalg.norm(u)))
    report = []
    for what, u in checks:
        ref, vals = fd_median(oracle_mod, st0, box, T, what, eps_list, u)
        got = pgrad[0, 0] if what == "k" else pgrad[0, 1] if what == "mu" else directional(grad, what, u)
        rel = abs(got - ref) / abs(ref)
        report.append((what, got, ref, rel, vals))
    bad = [r for r in report if r[3] > tol]
    assert not bad, "\n".join(f"{w}: adjoint {g:.7g} fd {f:.7g} rel {r:.2e} (eps: {v})"
                              for w, g, f, r, v in report)
    return report


def test_adjoint_matches_fp64_fd_short_horizon(cuda, pkg, oracle_mod):
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 16, 8.0)
    box = [32.0, 32.0, 32.0]
    T = 40
    _, grad, pgrad = run_gradient(pkg, recs, box, T, 10)
    check_against_fd(oracle_mod, recs, box, T, grad, pgrad, (1e-3, 1e-4, 1e-5), 1e-3)


def test_adjoint_differentiable_config(cuda, pkg, oracle_mod):
    """32,768 particles (32^3 lattice, spacing 0.5) in a 48^3 grid, 200
    substeps, checkpoint every 20, centroid loss to (30, 10, 30), initial
    velocities N(0, 0.1): gradients w.r.t. stiffness, viscosity and the
    initial state."""
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 32, 8.0)
    box = [48.0, 48.0, 48.0]
    T = 200
    L, grad, pgrad = run_gradient(pkg, recs, box, T, 20)
    assert np.isfinite(grad).all() and np.isfinite(pgrad).all()
    # four state-space directions (two in velocity, one each in position and
    # C) plus both parameters; the median over eps is the reference, and the
    # report carries each eps's value (eps = 1e-4 first)
    check_against_fd(oracle_mod, recs, box, T, grad, pgrad, (1e-4, 3e-5, 1e-5), 1e-3, ndir=4)


def test_fixed_point_tape_short_horizon(cuda, pkg, oracle_mod):
    """Along the solver's own fixed-point trajectory the gradient is that of
    a slightly different path: within 2e-3 at 40 substeps."""
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 16, 8.0)
    box = [32.0, 32.0, 32.0]
    _, grad, pgrad = run_gradient(pkg, recs, box, 40, 10, tape="fixed")
    check_against_fd(oracle_mod, recs, box, 40, grad, pgrad, (1e-3, 1e-4, 1e-5), 2e-3)


@pytest.mark.parametrize("tape", ["fp64", "fixed"])
def test_checkpoint_interval_does_not_change_gradients(cuda, pkg, tape):
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 12, 9.0)
    box = [32.0, 32.0, 32.0]
    T = 30
    outs = [run_gradient(pkg, recs, box, T, every, tape)[1:] for every in (1, 7, 30)]
    # float atomics sum in a different order on every run: compare at the
    # gradient's own scale
    scale = float(np.abs(outs[0][0]).max())
    for g, p in outs[1:]:
        np.testing.assert_allclose(g, outs[0][0], rtol=1e-4, atol=1e-5 * scale)
        np.testing.assert_allclose(p, outs[0][1], rtol=1e-4)


def test_fixed_tape_forward_is_the_solver(cuda, pkg):
    """The fixed-point tape's states are the solver's, bit for bit."""
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 12, 9.0)
    box = [32.0, 32.0, 32.0]
    adj = pkg.MLSMPMAdjoint([pkg.scene_desc(len(recs), box)], 24, 8, tape="fixed")
    adj.forward(recs, 24)
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=len(recs), maxGrid=(32, 32, 32))
    sim.upload(recs, box)
    for t in (8, 16, 24):
        sim.execute(substeps=8)
        assert np.array_equal(adj.state(t).view(np.uint32), sim.downloadParticles().view(np.uint32))
    sim.close()
    adj.close()


def test_fp64_tape_forward_matches_oracle(cuda, pkg, oracle_mod):
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 12, 9.0)
    box = [32.0, 32.0, 32.0]
    adj = pkg.MLSMPMAdjoint([pkg.scene_desc(len(recs), box)], 30, 10)
    adj.forward(recs, 30)
    want = oracle_mod.run64(oracle_mod.records_to_state64(recs), oracle_mod.Params64.make(box), 30)
    got = adj.state(30)
    np.testing.assert_allclose(got[:, 0:3], want[:, 0:3], rtol=0, atol=2e-5)
    np.testing.assert_allclose(got[:, 4:7], want[:, 3:6], rtol=0, atol=2e-5)
    adj.close()


def test_batched_adjoint_equals_single_scenes(cuda, pkg):
    """Scenes differentiated together give each scene's own gradients."""
    from oracle import scene as scene_mod
    parts = [lattice_with_velocity(scene_mod, 10, 8.0, seed=s, vseed=s) for s in (1, 2, 3)]
    boxes = [[32.0, 32.0, 32.0], [28.0, 36.0, 30.0], [32.0, 32.0, 32.0]]
    ks = [2.5, 3.0, 3.7]
    descs = [pkg.scene_desc(len(p), b, stiffness=k) for p, b, k in zip(parts, boxes, ks)]
    T = 24
    adj = pkg.MLSMPMAdjoint(descs, T, 8)
    allp = np.concatenate(parts)
    adj.forward(allp, T)
    L, seed = pkg.centroid_loss(adj.state(T), TARGET, adj.sceneOffsets)
    g, pg = adj.backward({T: seed})
    adj.close()
    for s, (p, d) in enumerate(zip(parts, descs)):
        one = pkg.MLSMPMAdjoint([d], T, 8)
        one.forward(p, T)
        L1, seed1 = pkg.centroid_loss(one.state(T), TARGET)
        g1, pg1 = one.backward({T: seed1})
        one.close()
        lo, hi = adj.sceneOffsets[s], adj.sceneOffsets[s + 1]
        assert abs(L1[0] - L[s]) <= 1e-9 * max(1.0, abs(L1[0]))
        np.testing.assert_allclose(g[lo:hi], g1, rtol=1e-4, atol=1e-5 * float(np.abs(g1).max()))
        np.testing.assert_allclose(pg[s], pg1[0], rtol=1e-4)


def test_intermediate_seeds_are_linear(cuda, pkg):
    """Seeds at several substeps give the sum of the separate gradients."""
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 10, 9.0)
    box = [32.0, 32.0, 32.0]
    T = 30
    adj = pkg.MLSMPMAdjoint([pkg.scene_desc(len(recs), box)], T, 10)
    adj.forward(recs, T)
    _, s10 = pkg.centroid_loss(adj.state(10), TARGET)
    _, s30 = pkg.centroid_loss(adj.state(30), TARGET)
    g_both, p_both = adj.backward({10: s10, 30: s30})
    g_a, p_a = adj.backward({10: s10})
    g_b, p_b = adj.backward({30: s30})
    adj.close()
    np.testing.assert_allclose(g_both, g_a + g_b, rtol=1e-4,
                               atol=1e-5 * float(np.abs(g_both).max()))
    np.testing.assert_allclose(p_both, p_a + p_b, rtol=1e-4)


def test_inverse_problem_recovers_constants(cuda, pkg):
    """Batched forward + adjoint + Adam: hidden stiffness / viscosity of 4
    small scenes recovered from observed positions."""
    r = pkg.inverse.run_inverse_problem(4, seed=3, substeps=40, checkpoint_every=10, iters=30,
                                        lr=0.05, n_range=(3000, 5000), side=32, observe_every=10)
    h = r["history"]
    assert h[-1]["loss"].mean() < 0.1 * h[0]["loss"].mean()
    assert np.median(r["rel_err"][:, 0]) < 0.05
    assert np.isfinite(r["recovered"]).all()


@pytest.mark.parametrize("tape", ["fixed", "fp64"])
def test_observation_loss_matches_host_loss(cuda, pkg, tape):
    """observationLoss / backwardObserved (loss and seeds on the device)
    against the same loss, seeds and backward computed on the host from the
    read-back states."""
    inv = pkg.inverse
    descs, recs, _ = inv.inverse_scenes(3, seed=4, n_range=(3000, 5000), side=32)
    T, steps = 30, [10, 20, 30]
    adj = pkg.MLSMPMAdjoint(descs, T, 10, tape=tape)
    for s in range(3):
        adj.setScene(s, inv.with_constants(descs[s], 2.5, 0.15))
    observed = inv.observe(adj, recs, T, steps)
    for s in range(3):
        adj.setScene(s, descs[s])
    adj.setObservations(observed)
    adj.forward(recs, T)
    loss_dev = adj.observationLoss()
    g_dev, p_dev = adj.backwardObserved()

    offs = adj.sceneOffsets
    counts = np.diff(offs)
    scale = (2.0 / np.repeat(counts.astype(np.float64), counts)).astype(np.float32)[:, None]
    loss_host = np.zeros(3)
    seeds = {}
    for t in steps:
        x = adj.state(t)
        diff = x[:, 0:3] - observed[t].astype(np.float32)
        sq = np.einsum("ij,ij->i", diff, diff, dtype=np.float64)
        loss_host += np.add.reduceat(sq, offs[:-1]) / counts
        seeds[t] = np.zeros_like(x)
        seeds[t][:, 0:3] = diff * scale
    assert (loss_host > 0).all()
    np.testing.assert_allclose(loss_dev, loss_host, rtol=1e-12)
    g_host, p_host = adj.backward(seeds)
    # the same seeds; float atomics make the summation order differ
    np.testing.assert_allclose(g_dev, g_host, rtol=1e-4, atol=1e-5 * float(np.abs(g_host).max()))
    np.testing.assert_allclose(p_dev, p_host, rtol=1e-4)
    assert np.isfinite(g_dev).all()

    # the seeds belong to one forward; observed substeps must be checkpoints
    adj.forward(recs, T)
    with pytest.raises(pkg.MPMError):
        adj.backwardObserved()
    adj.setObservations({15: observed[10]})
    with pytest.raises(pkg.MPMError):
        adj.observationLoss()
    adj.close()


@pytest.mark.parametrize("tape", ["fixed", "fp64"])
def test_repeated_backward_after_one_forward(cuda, pkg, tape):
    """A second and third backward after the same forward (the first one used
    the forward's record of the last segment, later ones recompute it) give
    the same gradients as the first."""
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 10, 9.0)
    adj = pkg.MLSMPMAdjoint([pkg.scene_desc(len(recs), [32.0, 32.0, 32.0])], 25, 10, tape=tape)
    adj.forward(recs, 25)
    _, seed = pkg.centroid_loss(adj.state(25), TARGET)
    outs = [adj.backward({25: seed}) for _ in range(3)]
    adj.close()
    for g, p in outs[1:]:
        # float atomics make the summation order differ between runs
        np.testing.assert_allclose(g, outs[0][0], rtol=1e-4,
                                   atol=1e-5 * float(np.abs(outs[0][0]).max()))
        np.testing.assert_allclose(p, outs[0][1], rtol=1e-4)
    assert np.isfinite(outs[0][0]).all()


@pytest.mark.parametrize("tape", ["fixed", "fp64"])
def test_large_batch_uses_the_sorted_path(cuda, pkg, tape):
    """Above 512 particles per SM the adjoint kernels walk a per-substep
    brick sort with one thread per particle; below it they use three threads
    per particle in particle order.  Each scene of a large batch must get the
    gradients its own (small) adjoint gives."""
    import torch
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    descs, recs = pkg.batch_scenes(16, seed=11, n_range=(5000, 8000), sides=(32,))
    offs = np.concatenate([[0], np.cumsum([d.num_particles for d in descs])])
    assert offs[-1] >= 512 * nsm, "the batch must be large enough for the sorted path"
    T, every = 12, 4
    adj = pkg.MLSMPMAdjoint(descs, T, every, tape=tape)
    adj.forward(recs, T)
    L, seed = pkg.centroid_loss(adj.state(T), TARGET, adj.sceneOffsets)
    g, pg = adj.backward({T: seed})
    adj.close()
    assert np.isfinite(g).all()
    for s in (0, 7, 15):
        d = descs[s]
        one = pkg.MLSMPMAdjoint([d], T, every, tape=tape)
        one.forward(recs[offs[s]:offs[s + 1]], T)
        _, seed1 = pkg.centroid_loss(one.state(T), TARGET)
        g1, pg1 = one.backward({T: seed1})
        one.close()
        np.testing.assert_allclose(g[offs[s]:offs[s + 1]], g1, rtol=1e-4,
                                   atol=1e-5 * float(np.abs(g1).max()))
        np.testing.assert_allclose(pg[s], pg1[0], rtol=1e-4, atol=1e-9)


def test_contiguous_seed_block_abi(cuda, pkg):
    """mpm_backward (all seed blocks in one array) gives what the pointer-list
    entry point the Python class uses gives."""
    import ctypes
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 10, 9.0)
    adj = pkg.MLSMPMAdjoint([pkg.scene_desc(len(recs), [32.0, 32.0, 32.0])], 20, 10, tape="fixed")
    adj.forward(recs, 20)
    _, s10 = pkg.centroid_loss(adj.state(10), TARGET)
    _, s20 = pkg.centroid_loss(adj.state(20), TARGET)
    g_list, p_list = adj.backward({10: s10, 20: s20})
    n = len(recs)
    block = np.ascontiguousarray(np.stack([s10, s20]), dtype=np.float32)
    steps = (ctypes.c_int32 * 2)(10, 20)
    grad = np.zeros((n, 20), np.float32)
    pgrad = np.zeros((1, 2), np.float64)
    fp = ctypes.POINTER(ctypes.c_float)
    rc = adj._lib.mpm_backward(adj._handle, block.ctypes.data_as(fp), steps, 2,
                               grad.ctypes.data_as(fp),
                               pgrad.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    adj.close()
    assert rc == 0
    np.testing.assert_allclose(grad, g_list, rtol=1e-4, atol=1e-5 * float(np.abs(g_list).max()))
    np.testing.assert_allclose(pgrad, p_list, rtol=1e-4)


@pytest.mark.parametrize("T,every", [(1, 1), (12, 5), (40, 10)])
def test_backward_matches_cpu_tape_adjoint(cuda, pkg, oracle_mod, T, every):
    """The library's backward on the FP64 tape against the independent FP64
    tape adjoint on the CPU (oracle/mpm_adjoint64.c): the same trajectory,
    the same seeds (random adjoints of every state component at the final
    substep and of the velocities at an intermediate one), the reverse pass
    restated by hand in double precision.  T = 1 compares one substep's
    adjoint (p2g_1, p2g_2, updateGrid and g2p backward) term for term;
    longer runs add checkpointing and recompute.  The GPU's adjoint
    arithmetic is f32, so the tolerance is relative to the gradient's
    scale."""
    from oracle import scene as scene_mod
    recs = lattice_with_velocity(scene_mod, 16, 8.0)
    recs[:, 8:11] = np.random.default_rng(3).normal(0.0, 0.05, (len(recs), 3)).astype(np.float32)
    box = [32.0, 32.0, 32.0]
    n = len(recs)
    rng = np.random.default_rng(11)
    seed_T = np.zeros((n, 20), np.float32)
    for sl in (slice(0, 3), slice(4, 7), slice(8, 11), slice(12, 15), slice(16, 19)):
        seed_T[:, sl] = rng.normal(0.0, 1e-3, (n, 3)).astype(np.float32)
    mid = T // 2
    seed_m = np.zeros((n, 20), np.float32)
    seed_m[:, 4:7] = rng.normal(0.0, 1e-3, (n, 3)).astype(np.float32)
    seeds = {T: seed_T} if mid in (0, T) else {T: seed_T, mid: seed_m}
    adj = pkg.MLSMPMAdjoint([pkg.scene_desc(n, box)], T, every, tape="fp64")
    adj.forward(recs, T)
    g, pg = adj.backward(seeds)
    adj.close()
    st0 = oracle_mod.records_to_state64(recs)
    p = oracle_mod.Params64.make(box)
    cs = {t: oracle_mod.records_to_state64(v) for t, v in seeds.items()}
    want, pwant = oracle_mod.backward64(st0, p, T, cs, every=every)
    got = oracle_mod.records_to_state64(g)
    for name, sl in (("x", slice(0, 3)), ("v", slice(3, 6)), ("C", slice(6, 15))):
        scale = np.abs(want[:, sl]).max()
        err = np.abs(got[:, sl] - want[:, sl]).max() / scale
        assert err < 2e-4, f"{name}: max error {err:.2e} of the gradient's scale {scale:.3e}"
    for j, name in enumerate(("stiffness", "viscosity")):
        assert abs(pg[0, j] - pwant[j]) <= 2e-4 * abs(pwant[j]) + 1e-12, (name, pg[0, j], pwant[j])
