"""Host logic of the batched inverse problem (webgpu-ocean_gb300/inverse.py)
on CPU: the per-scene trajectory loss, the seeds handed to the backward and
the Adam update, with a stand-in adjoint whose forward returns fixed states
and whose backward returns a known parameter gradient."""
from __future__ import annotations

import numpy as np


class FakeAdjoint:
    def __init__(self, pkg, counts, states, pgrad):
        self._descs = [pkg.scene_desc(int(c), [32.0, 32.0, 32.0]) for c in counts]
        self.numScenes = len(counts)
        self.sceneOffsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.states = states
        self.pgrad = pgrad
        self.set_calls = []
        self.seeds_seen = []

    def setScene(self, s, desc):
        self.set_calls.append((s, desc.stiffness, desc.dynamic_viscosity))

    def forward(self, init, substeps):
        pass

    def state(self, t, out=None):
        out[:] = self.states[t]
        return out

    def backward(self, seeds):
        self.seeds_seen.append({t: np.array(v) for t, v in seeds.items()})
        return np.zeros_like(next(iter(seeds.values()))), self.pgrad.copy()


def test_loss_seeds_and_adam_step(pkg):
    rng = np.random.default_rng(5)
    counts = [7, 3, 11]
    n = sum(counts)
    steps = [4, 8]
    states = {t: rng.normal(10.0, 2.0, (n, 20)).astype(np.float32) for t in steps}
    observed = {t: (states[t][:, 0:3] + rng.normal(0.0, 0.1, (n, 3))).astype(np.float32)
                for t in steps}
    pgrad = np.array([[0.5, -2.0], [-1.0, 0.25], [3.0, 1.0]])
    adj = FakeAdjoint(pkg, counts, states, pgrad)
    start = np.array([[3.0, 0.1], [2.0, 0.2], [2.5, 0.05]])
    fit = pkg.inverse.fit_parameters(adj, None, observed, 8, start, iters=2, lr=0.1,
                                     device_loss=False)

    offs = adj.sceneOffsets
    want_loss = np.zeros(3)
    for t in steps:
        for s in range(3):
            d = states[t][offs[s]:offs[s + 1], 0:3].astype(np.float64) - observed[t][offs[s]:offs[s + 1]]
            want_loss[s] += np.mean(np.sum(d * d, axis=1))
    np.testing.assert_allclose(fit["history"][0]["loss"], want_loss, rtol=1e-6)
    for t in steps:
        seed = adj.seeds_seen[0][t]
        assert not seed[:, 3:].any(), "only the position columns carry the loss gradient"
        for s in range(3):
            d = states[t][offs[s]:offs[s + 1], 0:3].astype(np.float64) - observed[t][offs[s]:offs[s + 1]]
            np.testing.assert_allclose(seed[offs[s]:offs[s + 1], 0:3], 2.0 * d / counts[s],
                                       rtol=1e-5, atol=1e-6)
    # first Adam step on log parameters: theta -= lr * sign(g) (m/v bias-corrected)
    g = pgrad * start
    theta1 = np.log(start) - 0.1 * g / (np.abs(g) + 1e-12)
    np.testing.assert_allclose(fit["history"][1]["params"], np.exp(theta1), rtol=1e-9)
    assert len(adj.set_calls) == 2 * 3


def test_centroid_loss_seed_is_its_gradient(pkg):
    rng = np.random.default_rng(2)
    state = rng.normal(10.0, 3.0, (12, 20)).astype(np.float32)
    offs = [0, 5, 12]
    target = [30.0, 10.0, 30.0]
    loss, seed = pkg.centroid_loss(state, target, offs)
    assert not seed[:, 3:].any()
    eps = 1e-3
    for i, a in ((0, 0), (4, 2), (7, 1), (11, 0)):
        up, dn = state.astype(np.float64).copy(), state.astype(np.float64).copy()
        up[i, a] += eps
        dn[i, a] -= eps
        lu, _ = pkg.centroid_loss(up, target, offs)
        ld, _ = pkg.centroid_loss(dn, target, offs)
        fd = (lu - ld).sum() / (2 * eps)
        assert abs(fd - seed[i, a]) < 1e-3 * max(1.0, abs(fd))
