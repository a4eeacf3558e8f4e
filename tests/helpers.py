"""Shared helpers for the parity tests."""
from __future__ import annotations

import os

import numpy as np

NTHREADS = max(1, min(os.cpu_count() or 1, 32))


def first_mismatch(a: np.ndarray, b: np.ndarray) -> str:
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        return f"shape {a.shape} != {b.shape}"
    if a.dtype.kind == "f":
        av, bv = a.view(np.uint32), b.view(np.uint32)
    else:
        av, bv = a, b
    bad = np.argwhere(av != bv)
    if len(bad) == 0:
        return "equal"
    i = tuple(bad[0])
    return f"{len(bad)} mismatches; first at {i}: {a[i]!r} vs {b[i]!r}"


def assert_bits_equal(a: np.ndarray, b: np.ndarray, what: str) -> None:
    a = np.asarray(a)
    b = np.asarray(b)
    same = a.shape == b.shape and (
        np.array_equal(a.view(np.uint32), b.view(np.uint32)) if a.dtype.kind == "f"
        else np.array_equal(a, b))
    assert same, f"{what}: {first_mismatch(a, b)}"


def assert_state_equal(sim, ref, what: str, posvel: bool = True) -> None:
    assert_bits_equal(sim.downloadGrid(), ref.cells, f"{what} grid")
    assert_bits_equal(sim.downloadParticles(), ref.particles, f"{what} particles")
    if posvel:
        assert_bits_equal(sim.downloadPosvel(), ref.posvel, f"{what} posvel")


def lattice_scene(oracle_scene, n_per_axis: int, origin: float, seed: int = 1234) -> np.ndarray:
    return oracle_scene.lattice(n_per_axis, origin, 0.5, 0.05, seed)
