"""Scene generators restated in Python (test infrastructure: the oracle side).

These produce particle arrays in the reference's 80-byte layout (20 float32
per particle: pos xyz pad, v xyz pad, C as three 16-byte columns).  The
product has its own C++ generators (libmpm.so `mpm_scene_*`); tests compare
the two bit for bit.

`dambreak` restates `MLSMPMSimulator.initDambreak` (mls-mpm/mls-mpm.ts:195-223).
JavaScript numbers are IEEE doubles and Python floats are too, so the loop
counters, the `+= spacing` accumulation and `i + jitter` reproduce the
reference exactly; `Float32Array.set` rounds to nearest float32, as
`np.float32(x)` does.  The one substitution is the random source:
`Math.random()` becomes SplitMix64 (Steele, Lea & Flood, OOPSLA 2014) so that
scenes are reproducible; a draw is the top 53 bits scaled by 2**-53.

`lattice` is the jittered lattice of the benchmark scenes: particle
(ix, iy, iz), x-major with z fastest, sits at origin + spacing*i on each axis
plus a per-component jitter uniform in [-jitter, jitter), three draws per
particle in x, y, z order.
"""
from __future__ import annotations

import numpy as np

MASK64 = (1 << 64) - 1
PARTICLE_FLOATS = 20  # mls-mpm/mls-mpm.ts:10 (80 bytes)


class SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def random(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)


def dambreak(init_box, num_particles: int, seed: int) -> np.ndarray:
    """mls-mpm/mls-mpm.ts:195-223 with Math.random -> SplitMix64(seed)."""
    rng = SplitMix64(seed)
    spacing = 0.65
    X, Y, Z = (float(b) for b in init_box)
    rows = []
    n = 0
    j = 0.0
    while j < Y * 0.80 and n < num_particles:
        i = 3.0
        while i < X - 4 and n < num_particles:
            k = 3.0
            while k < Z / 2 and n < num_particles:
                jitter = 2.0 * rng.random()
                rows.append((i + jitter, j + jitter, k + jitter))
                n += 1
                k += spacing
            i += spacing
        j += spacing
    out = np.zeros((n, PARTICLE_FLOATS), dtype=np.float32)
    if n:
        out[:, 0:3] = np.array(rows, dtype=np.float64).astype(np.float32)
    return out


def splitmix64_uniform(seed: int, count: int) -> np.ndarray:
    """The first `count` draws of SplitMix64(seed).random(), vectorised: draw
    k mixes the state seed + (k + 1) * gamma (mod 2**64), exactly as the
    sequential generator above advances it."""
    with np.errstate(over="ignore"):
        k = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed & MASK64) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def lattice(n_per_axis: int, origin: float, spacing: float, jitter: float, seed: int) -> np.ndarray:
    """Jittered cubic lattice, x-major (z fastest), jitter U[-jitter, jitter):
    coordinate a of particle (ix, iy, iz) is (origin + spacing*i_a) +
    jitter*(2u - 1), u the next draw, three draws per particle in x, y, z
    order (all in double precision, rounded once to float32)."""
    n = n_per_axis ** 3
    u = splitmix64_uniform(seed, 3 * n).reshape(n, 3)
    i = np.arange(n_per_axis, dtype=np.float64)
    idx = np.stack(np.meshgrid(i, i, i, indexing="ij"), axis=-1).reshape(n, 3)
    pos = (origin + spacing * idx) + jitter * (2.0 * u - 1.0)
    out = np.zeros((n, PARTICLE_FLOATS), dtype=np.float32)
    out[:, 0:3] = pos.astype(np.float32)
    return out


def lattice_sequential(n_per_axis: int, origin: float, spacing: float, jitter: float,
                       seed: int) -> np.ndarray:
    """`lattice` written as the plain loop over the sequential generator (the
    definition the vectorised version is tested against)."""
    rng = SplitMix64(seed)
    n = n_per_axis ** 3
    pos = np.empty((n, 3), dtype=np.float64)
    p = 0
    for ix in range(n_per_axis):
        for iy in range(n_per_axis):
            for iz in range(n_per_axis):
                for a, idx in enumerate((ix, iy, iz)):
                    u = rng.random()
                    pos[p, a] = (origin + spacing * idx) + jitter * (2.0 * u - 1.0)
                p += 1
    out = np.zeros((n, PARTICLE_FLOATS), dtype=np.float32)
    out[:, 0:3] = pos.astype(np.float32)
    return out


def sph_dambreak(init_half_box, num_particles: int, seed: int) -> np.ndarray:
    """SPHSimulator.initDambreak (sph/sph.ts:357-381) with Math.random ->
    SplitMix64(seed): 64-byte records (n, 16) float32."""
    rng = SplitMix64(seed)
    hx, hy, hz = (float(h) for h in init_half_box)
    step = 0.5 * 0.07
    rows = []
    y = -hy * 0.95
    while len(rows) < num_particles:
        before = len(rows)
        x = -0.95 * hx
        while x < 0.95 * hx and len(rows) < num_particles:
            z = -0.95 * hz
            while z < 0 * hz and len(rows) < num_particles:
                j = 0.001 * rng.random()
                rows.append((x + j, y + j, z + j))
                z += step
            x += step
        if len(rows) == before:
            break
        y += step
    out = np.zeros((len(rows), 16), np.float32)
    if rows:
        out[:, 0:3] = np.array(rows, dtype=np.float64).astype(np.float32)
    return out
