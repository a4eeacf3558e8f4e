"""Batched parameter recovery with the adjoint (system identification).

Each scene of a batch has unknown stiffness k and dynamic viscosity mu.
Given observed particle positions at a few substeps of a rollout from a
known initial state, fit_parameters runs the batched forward with
checkpoints and the batched backward (mpm_forward_ckpt / mpm_backward) once
per iteration and takes an Adam step on (log k, log mu) of every scene.

Loss of scene s:  L_s = sum over observed substeps t of
                        mean over its particles of |x_p(t) - x_obs_p(t)|^2
"""
from __future__ import annotations

import time

import numpy as np

from . import _lib as L
from .mlsmpm import MLSMPMAdjoint, batch_scenes, scene_desc


def inverse_scenes(num_scenes: int = 64, seed: int = 0, n_range=(16000, 32000), side: int = 48,
                   stiffness_range=(2.0, 4.0), viscosity_range=(0.05, 0.2)):
    """Scenes with hidden constants: lattice blocks in side^3 grids (the
    batch_scenes layout, reference gravity), stiffness and viscosity drawn
    uniformly (numpy PCG64(seed + 1)).  Returns (descs with the hidden
    constants, (N, 20) initial records, hidden (S, 2) array)."""
    descs, recs = batch_scenes(num_scenes, seed=seed, n_range=n_range, sides=(side,),
                               gravity=(0.0, -0.3, 0.0))
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    hidden = np.stack([rng.uniform(*stiffness_range, num_scenes),
                       rng.uniform(*viscosity_range, num_scenes)], axis=1).astype(np.float32)
    out = [with_constants(d, hidden[s, 0], hidden[s, 1]) for s, d in enumerate(descs)]
    return out, recs, hidden


def with_constants(desc: L.SceneDesc, stiffness: float, viscosity: float) -> L.SceneDesc:
    return scene_desc(desc.num_particles, list(desc.init_box), list(desc.real_box),
                      stiffness=float(stiffness), rest_density=desc.rest_density,
                      dynamic_viscosity=float(viscosity), dt=desc.dt,
                      fixed_point_multiplier=desc.fixed_point_multiplier,
                      gravity=list(desc.gravity))


def observe(adj: MLSMPMAdjoint, init: np.ndarray, substeps: int, steps) -> dict:
    """Positions at `steps` of a forward from `init` with adj's constants."""
    adj.forward(init, substeps)
    return {t: adj.state(t)[:, 0:3].copy() for t in steps}


def _host_array(shape) -> np.ndarray:
    """A zeroed float32 host array, page-locked when CUDA is available (the
    state reads and seed uploads of every iteration then run at pinned-copy
    speed)."""
    try:
        import torch
        if torch.cuda.is_available():
            return torch.zeros(shape, dtype=torch.float32, pin_memory=True).numpy()
    except ImportError:
        pass
    return np.zeros(shape, dtype=np.float32)


def fit_parameters(adj: MLSMPMAdjoint, init: np.ndarray, observed: dict, substeps: int,
                   start, iters: int = 50, lr: float = 0.05, betas=(0.9, 0.999),
                   callback=None, device_loss: bool = True) -> dict:
    """Adam on (log k, log mu) per scene from `start` ((S, 2) array).  The
    loss, sum over observed substeps of each scene's mean squared distance to
    the observed positions, and its seeds are computed on the device
    (observationLoss / backwardObserved: the states stay there), or with
    device_loss=False on the host from the read-back states (same f32
    differences and seeds, FP64 sums)."""
    S = adj.numScenes
    offs = adj.sceneOffsets
    counts = np.diff(offs).astype(np.float64)
    base = [adj._descs[s] for s in range(S)]
    theta = np.log(np.asarray(start, dtype=np.float64).reshape(S, 2))
    m = np.zeros_like(theta)
    v = np.zeros_like(theta)
    steps = sorted(observed)
    n = int(offs[-1])
    if device_loss:
        adj.setObservations(observed)
    else:
        # dL/dx = 2 (x - x_obs) / (its scene's particle count); seed records
        # are zero except their position columns, so the buffers are made once
        scale = (2.0 / np.repeat(counts, np.diff(offs))).astype(np.float32)[:, None]
        obs32 = {t: np.asarray(observed[t], dtype=np.float32) for t in steps}
        seeds = {t: _host_array((n, 20)) for t in steps}
        x = _host_array((n, 20))
    history = []
    t0 = time.perf_counter()
    for it in range(iters):
        params = np.exp(theta)
        for s in range(S):
            adj.setScene(s, with_constants(base[s], params[s, 0], params[s, 1]))
        adj.forward(init, substeps)
        if device_loss:
            loss = adj.observationLoss()
            _, pgrad = adj.backwardObserved(grad_init=False)
        else:
            loss = np.zeros(S)
            for t in steps:
                adj.state(t, out=x)
                diff = x[:, 0:3] - obs32[t]
                sq = np.einsum("ij,ij->i", diff, diff, dtype=np.float64)
                loss += np.add.reduceat(sq, offs[:-1]) / counts
                np.multiply(diff, scale, out=seeds[t][:, 0:3])
            _, pgrad = adj.backward(seeds)
        g = pgrad * params  # d/d log(p) = p * d/dp
        m = betas[0] * m + (1 - betas[0]) * g
        v = betas[1] * v + (1 - betas[1]) * g * g
        mh = m / (1 - betas[0] ** (it + 1))
        vh = v / (1 - betas[1] ** (it + 1))
        theta -= lr * mh / (np.sqrt(vh) + 1e-12)
        history.append({"iter": it, "loss": loss.copy(), "params": params.copy()})
        if callback:
            callback(it, loss, params)
    return {"params": np.exp(theta), "history": history,
            "seconds": time.perf_counter() - t0}


def run_inverse_problem(num_scenes: int = 64, seed: int = 0, substeps: int = 100,
                        checkpoint_every: int = 20, iters: int = 50, lr: float = 0.05,
                        tape: str = "fixed", n_range=(16000, 32000), side: int = 48,
                        observe_every: int = 20, device_loss: bool = True) -> dict:
    """The whole experiment: hidden constants, observed rollouts, recovery
    from (k, mu) = (3, 0.1); returns the relative errors against the hidden
    values."""
    if observe_every % checkpoint_every:
        raise ValueError("observed substeps must be checkpoints (observe_every a multiple of "
                         "checkpoint_every)")
    descs, recs, hidden = inverse_scenes(num_scenes, seed, n_range, side)
    adj = MLSMPMAdjoint(descs, substeps, checkpoint_every, tape=tape)
    steps = list(range(observe_every, substeps + 1, observe_every))
    observed = {t: x.astype(np.float64) for t, x in observe(adj, recs, substeps, steps).items()}
    start = np.tile(np.array([[3.0, 0.1]]), (num_scenes, 1))
    fit = fit_parameters(adj, recs, observed, substeps, start, iters=iters, lr=lr,
                         device_loss=device_loss)
    adj.close()
    rel = np.abs(fit["params"] - hidden) / hidden
    return {"hidden": hidden, "recovered": fit["params"], "rel_err": rel,
            "history": fit["history"], "seconds": fit["seconds"],
            "particles": int(len(recs)), "scenes": num_scenes}
