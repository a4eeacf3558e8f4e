"""mpm_count_nonfinite_noalloc: the watchdog scan for callers that cannot
allocate device memory (a per-frame host loop, a plugin host that owns all
device memory).  It reads a caller-owned device buffer and keeps its scratch
in a fixed array inside the library; its count must equal the one
mpm_check_health reports for the same particles, on consecutive calls.

This file is collected last so that a failure here never hides the others."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_watchdog_matches_check_health(cuda, pkg):
    torch = cuda
    from oracle import scene
    lib = pkg._lib.load()
    box = [32.0, 32.0, 32.0]
    parts = scene.lattice(12, 6.0, 0.5, 0.05, 21)
    parts[3, 0] = np.nan            # position
    parts[40, 5] = np.inf           # velocity
    parts[41, 13] = -np.inf         # C
    parts[41, 14] = np.nan          # same record twice
    parts[999, 18] = np.nan
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=len(parts), maxGrid=(32, 32, 32))
    sim.upload(parts, box)
    health = sim.checkHealth()                      # the existing entry point
    want = health["nonfinite_particles"]
    assert want == 4
    recs = torch.from_numpy(sim.downloadParticles()).cuda()   # caller-owned device buffer
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):                           # consecutive calls share the scratch
        out.fill_(-1)
        rc = lib.mpm_count_nonfinite_noalloc(ctypes.c_void_p(recs.data_ptr()), 20, len(parts),
                                             ctypes.c_void_p(out.data_ptr()),
                                             ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.mpm_last_error()
        torch.cuda.synchronize()
        assert int(out.item()) == want, f"call {call}"
    # a clean buffer right after: the previous call's counts must not leak
    clean = torch.from_numpy(scene.lattice(12, 6.0, 0.5, 0.05, 22)).cuda()
    rc = lib.mpm_count_nonfinite_noalloc(ctypes.c_void_p(clean.data_ptr()), 20, len(parts),
                                         ctypes.c_void_p(out.data_ptr()),
                                         ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert int(out.item()) == 0
    sim.close()


def test_noalloc_skips_padding_of_80_byte_records(cuda, pkg):
    """WGSL struct stores leave the padding of the 80-byte record unspecified:
    a NaN or Inf there is not a non-finite particle (mpm_check_health never
    sees padding: the upload drops it).  Any other stride checks every float."""
    torch = cuda
    from oracle import scene
    lib = pkg._lib.load()
    parts = scene.lattice(10, 6.0, 0.5, 0.05, 23)
    for j, rec in zip((3, 7, 11, 15, 19), (0, 17, 256, 511, 999)):
        parts[rec, j] = np.nan if j % 2 else np.inf        # padding only
    parts[5, 4] = np.nan                                   # one real state float
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=len(parts), maxGrid=(32, 32, 32))
    sim.upload(parts, [32.0, 32.0, 32.0])
    want = sim.checkHealth()["nonfinite_particles"]
    sim.close()
    assert want == 1
    recs = torch.from_numpy(parts).cuda()
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    for stride, n, expect in ((20, len(parts), want), (4, len(parts) * 5, 6)):
        for call in range(2):
            out.fill_(-1)
            rc = lib.mpm_count_nonfinite_noalloc(ctypes.c_void_p(recs.data_ptr()), stride, n,
                                                 ctypes.c_void_p(out.data_ptr()),
                                                 ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0, lib.mpm_last_error()
            torch.cuda.synchronize()
            assert int(out.item()) == expect, f"stride {stride}, call {call}"


def test_noalloc_rejects_oversized_calls(cuda, pkg):
    torch = cuda
    lib = pkg._lib.load()
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    dummy = torch.zeros(20, dtype=torch.float32, device="cuda")
    rc = lib.mpm_count_nonfinite_noalloc(ctypes.c_void_p(dummy.data_ptr()), 20, 16_777_217,
                                         ctypes.c_void_p(out.data_ptr()), None)
    assert rc == pkg._lib.MPM_E_CAPACITY
    assert b"16,777,216" in lib.mpm_last_error()
