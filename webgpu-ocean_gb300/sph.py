"""SPHSimulator: host mirror of the reference's second simulator
(sph/sph.ts:15-389) over the C ABI, with the same four methods as
MLSMPMSimulator: reset(numParticles, initHalfBoxSize), execute(),
changeBoxSize(realHalfBoxSize), numParticles / gridCount.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .mlsmpm import _check, _dev_ptr, _stream_handle

SPH_PARTICLE_STRUCT_SIZE = 64  # sph.ts:13
NUM_PARTICLES_MAX = 200000     # common.ts:11


class SPHSimulator:
    kernelRadius = 0.07  # sph.ts:41

    def __init__(self, particleBuffer=None, posvelBuffer=None, renderDiameter: float = 0.08,
                 device=None, *, maxParticles: int = NUM_PARTICLES_MAX, seed: int = 0):
        self._lib = L.load()
        self.renderDiameter = float(renderDiameter)
        self.particleBuffer = particleBuffer
        self.seed = int(seed)
        self.maxParticles = int(maxParticles)
        self._handle = ctypes.c_void_p()
        pv_ptr, pv_bytes = (None, 0)
        if posvelBuffer is not None:
            pv_ptr, pv_bytes = _dev_ptr(posvelBuffer)
        _check(self._lib.mpm_sph_create(self.maxParticles, self.renderDiameter, pv_ptr, pv_bytes,
                                        ctypes.byref(self._handle)), "SPHSimulator")
        self.sphere_size = None

    @property
    def numParticles(self) -> int:
        return int(self._lib.mpm_sph_num_particles(self._handle))

    @property
    def gridCount(self) -> int:
        return int(self._lib.mpm_sph_grid_count(self._handle))

    def reset(self, numParticles: int, initHalfBoxSize) -> None:
        """sph.ts:300-316."""
        self.sphere_size = self.renderDiameter
        h = (ctypes.c_double * 3)(*[float(b) for b in initHalfBoxSize])
        _check(self._lib.mpm_sph_reset_dambreak(self._handle, int(numParticles), h,
                                                ctypes.c_uint64(self.seed)), "reset")

    def execute(self, commandEncoder=None, substeps: int = 2) -> None:
        """sph.ts:318-356 (two substeps per frame)."""
        _check(self._lib.mpm_sph_step(self._handle, int(substeps), _stream_handle(commandEncoder)),
               "execute")

    def setGraph(self, enable: bool) -> None:
        """Replay frames as CUDA graphs (default) or launch every kernel."""
        _check(self._lib.mpm_sph_set_graph(self._handle, int(bool(enable))), "setGraph")

    @property
    def warpPerParticle(self) -> int:
        """Particle counts up to this run density and forces one warp per
        particle (default 32768; 0: never; -1 to set: the default)."""
        return _check(self._lib.mpm_sph_get_warp_per_particle(self._handle), "warpPerParticle")

    @warpPerParticle.setter
    def warpPerParticle(self, max_particles: int) -> None:
        _check(self._lib.mpm_sph_set_warp_per_particle(self._handle, int(max_particles)),
               "warpPerParticle")

    def changeBoxSize(self, realBoxSize) -> None:
        """sph.ts:383-388 (half sizes)."""
        b = (ctypes.c_float * 3)(*[float(x) for x in realBoxSize])
        _check(self._lib.mpm_sph_set_real_box(self._handle, b), "changeBoxSize")

    def upload(self, records: np.ndarray, realHalfBoxSize) -> None:
        r = np.ascontiguousarray(records, dtype=np.float32).reshape(-1, 16)
        b = (ctypes.c_float * 3)(*[float(x) for x in realHalfBoxSize])
        _check(self._lib.mpm_sph_upload(self._handle, r.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                        len(r), b), "upload")

    def downloadParticles(self) -> np.ndarray:
        out = np.zeros((self.numParticles, 16), dtype=np.float32)
        _check(self._lib.mpm_sph_download_particles(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "downloadParticles")
        return out

    def downloadPosvel(self) -> np.ndarray:
        """The 32-byte posvel records written by the last substep."""
        out = np.zeros((self.numParticles, 8), dtype=np.float32)
        _check(self._lib.mpm_sph_download_posvel(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "downloadPosvel")
        return out

    def posvelDevicePtr(self) -> int:
        return int(self._lib.mpm_sph_posvel_device_ptr(self._handle) or 0)

    def close(self) -> None:
        if self._handle:
            self._lib.mpm_sph_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sph_scene_dambreak(initHalfBoxSize, numParticles: int, seed: int) -> np.ndarray:
    """initDambreak (sph.ts:357-381) on the host: (n, 16) float32 records."""
    out = np.zeros((max(int(numParticles), 1), 16), dtype=np.float32)
    h = (ctypes.c_double * 3)(*[float(b) for b in initHalfBoxSize])
    n = _check(L.load().mpm_sph_scene_dambreak(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                               int(numParticles), h, ctypes.c_uint64(seed)))
    return out[:n].copy()
