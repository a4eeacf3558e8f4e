"""The FP64 tape adjoint on the CPU (oracle/mpm_adjoint64.c) against FP64
central differences of the continuous model it differentiates
(oracle/mpm_oracle64.c): directional derivatives in state space, the
stiffness and viscosity derivatives, seeds at the final and at an
intermediate substep, checkpointed recompute.  This is the independent
adjoint the library's backward kernels are compared with (GPU tests)."""
from __future__ import annotations

import numpy as np
import pytest

TARGET = np.array([10.0, 5.0, 10.0])


def _scene(oracle_mod, spacing, seed):
    from oracle import scene
    rng = np.random.default_rng(seed)
    st = oracle_mod.records_to_state64(scene.lattice(8, 8.0, spacing, 0.05, 3))
    st[:, 3:6] = rng.normal(0, 0.1, (len(st), 3))
    st[:, 6:15] = rng.normal(0, 0.05, (len(st), 9))
    return st, rng


def _params(oracle_mod, k=None, mu=None):
    p = oracle_mod.Params64.make([20.0, 20.0, 20.0])
    if k is not None:
        p.stiffness = k
    if mu is not None:
        p.dynamic_viscosity = mu
    return p


@pytest.mark.parametrize("spacing", [0.5, 0.4])   # 8 and 15.6 particles per cell (rest: 4)
def test_cpu_tape_adjoint_matches_fp64_central_differences(oracle_mod, spacing):
    T, mid = 12, 5
    st, rng = _scene(oracle_mod, spacing, 1)
    p = _params(oracle_mod)
    k0, mu0 = p.stiffness, p.dynamic_viscosity

    def loss(s, k=k0, mu=mu0):
        pp = _params(oracle_mod, k, mu)
        out = oracle_mod.run64(s, pp, T)
        m = oracle_mod.run64(s, pp, mid)
        c = out[:, 0:3].mean(0)
        return ((c - TARGET) ** 2).sum() + 0.005 * (m[:, 3:6] ** 2).sum()

    out = oracle_mod.run64(st, p, T)
    m = oracle_mod.run64(st, p, mid)
    seed_t = np.zeros_like(st)
    seed_t[:, 0:3] = 2 * (out[:, 0:3].mean(0) - TARGET) / len(st)
    seed_m = np.zeros_like(st)
    seed_m[:, 3:6] = 0.01 * m[:, 3:6]
    g, pg = oracle_mod.backward64(st, p, T, {T: seed_t, mid: seed_m}, every=5)
    eps = 1e-6
    for _ in range(3):
        d = rng.normal(size=st.shape)
        d /= np.linalg.norm(d)
        fd = (loss(st + eps * d) - loss(st - eps * d)) / (2 * eps)
        # relative to the gradient's norm: a random direction can cancel most of it
        assert abs((g * d).sum() - fd) <= 1e-5 * np.linalg.norm(g), ((g * d).sum(), fd)
    fdk = (loss(st, k0 + eps) - loss(st, k0 - eps)) / (2 * eps)
    fdm = (loss(st, k0, mu0 + eps) - loss(st, k0, mu0 - eps)) / (2 * eps)
    assert abs(pg[1] - fdm) <= 1e-5 * abs(fdm), (pg[1], fdm)
    assert abs(pg[0] - fdk) <= 1e-5 * abs(fdk), (pg[0], fdk)


def test_cpu_tape_adjoint_independent_of_checkpoint_interval(oracle_mod):
    st, _ = _scene(oracle_mod, 0.4, 2)
    p = _params(oracle_mod)
    seed = np.zeros_like(st)
    seed[:, 0:6] = 1e-3
    ref = oracle_mod.backward64(st, p, 9, {9: seed}, every=1)
    for every in (2, 4, 9, 20):
        g, pg = oracle_mod.backward64(st, p, 9, {9: seed}, every=every)
        assert np.array_equal(g, ref[0]) and np.array_equal(pg, ref[1]), every
