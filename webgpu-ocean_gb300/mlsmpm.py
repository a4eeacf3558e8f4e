"""MLSMPMSimulator: the host-side mirror of WebGPU-Ocean's simulator class
(mls-mpm/mls-mpm.ts:12-276) over the C ABI of libmpm.so.

Names, arguments and error behaviour follow the TypeScript class:
  MLSMPMSimulator(particleBuffer, posvelBuffer, renderDiameter, device)
  reset(numParticles, initBoxSize)        -- throws on gridCount > capacity
  execute(commandEncoder)                 -- 2 substeps, asynchronous
  changeBoxSize(realBoxSize)
  numParticles, gridCount
Differences that come from the platform, not the algorithm:
  * buffers are CUDA device memory; posvelBuffer may be a torch CUDA tensor
    (or an object with data_ptr()/nbytes) or None, in which case the library
    allocates it; particleBuffer, if given, receives the 80-byte particle
    records at reset() and on writeParticleBuffer();
  * `commandEncoder` is the CUDA stream to enqueue on (a torch.cuda.Stream,
    a raw cudaStream_t integer, or None for the legacy default stream);
  * Math.random in initDambreak is SplitMix64(seed) (the `seed` keyword).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L

PARTICLE_STRUCT_SIZE = 80  # mlsmpmParticleStructSize, mls-mpm/mls-mpm.ts:10
NUM_PARTICLES_MAX = 200000  # common.ts:11


class MPMError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class GridCapacityError(MPMError):
    """The reference's `throw new Error("gridCount should be ...")`."""


def _check(code: int, what: str = "") -> int:
    if code >= 0:
        return code
    lib = L.load()
    msg = (lib.mpm_last_error() or b"").decode() or lib.mpm_error_string(code).decode()
    if what:
        msg = f"{what}: {msg}"
    cls = GridCapacityError if code == L.MPM_E_GRID_CAPACITY else MPMError
    raise cls(code, msg)


def _stream_handle(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream or None
    h = getattr(stream, "cuda_stream", None)
    if h is not None:
        return int(h) or None
    raise TypeError("commandEncoder must be a CUDA stream, an int handle or None")


def _dev_ptr(buf) -> tuple[int, int]:
    if hasattr(buf, "data_ptr"):
        ptr = int(buf.data_ptr())
        nbytes = int(buf.numel() * buf.element_size()) if hasattr(buf, "numel") else int(buf.nbytes)
        if hasattr(buf, "is_cuda") and not buf.is_cuda:
            raise ValueError("buffer must live in CUDA device memory")
        if hasattr(buf, "is_contiguous") and not buf.is_contiguous():
            raise ValueError("buffer must be contiguous")
        return ptr, nbytes
    raise TypeError("device buffers must expose data_ptr()")


def default_params() -> L.Params:
    p = L.Params()
    L.load().mpm_default_params(ctypes.byref(p))
    return p


def _cached_tuning(path, key: str, run, apply) -> dict:
    """The tuning choice for `key`: from the JSON file at `path` when it holds
    one (applied with apply(choice)), else run() -> choice, stored there."""
    import json
    import os
    table = {}
    if path and os.path.exists(path):
        with open(path) as f:
            table = json.load(f)
        if key in table:
            apply(table[key])
            return table[key]
    choice = run()
    if path:
        table[key] = choice
        tmp = f"{path}.tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    return choice


class MLSMPMSimulator:
    max_x_grids = 64  # mls-mpm/mls-mpm.ts:13-15
    max_y_grids = 64
    max_z_grids = 64
    cellStructSize = 16  # mls-mpm/mls-mpm.ts:16

    def __init__(self, particleBuffer=None, posvelBuffer=None, renderDiameter: float = 1.2,
                 device=None, *, maxParticles: int = NUM_PARTICLES_MAX,
                 maxGrid=(64, 64, 64), params: L.Params | None = None, seed: int = 0):
        self._lib = L.load()
        self.renderDiameter = float(renderDiameter)
        self.max_x_grids, self.max_y_grids, self.max_z_grids = (int(g) for g in maxGrid)
        self.maxParticles = int(maxParticles)
        self.particleBuffer = particleBuffer
        self.posvelBuffer = posvelBuffer
        self.seed = int(seed)
        self._device = device
        self._handle = ctypes.c_void_p()
        pv_ptr, pv_bytes = (None, 0)
        if posvelBuffer is not None:
            pv_ptr, pv_bytes = _dev_ptr(posvelBuffer)
        if particleBuffer is not None:
            _, pb = _dev_ptr(particleBuffer)
            if pb < PARTICLE_STRUCT_SIZE * self.maxParticles:
                raise ValueError("particleBuffer smaller than 80 * maxParticles bytes")
        prm = params if params is not None else default_params()
        with self._on_device():
            _check(self._lib.mpm_create(ctypes.byref(prm), self.maxParticles, self.max_x_grids,
                                        self.max_y_grids, self.max_z_grids,
                                        self.renderDiameter, pv_ptr, pv_bytes,
                                        ctypes.byref(self._handle)), "MLSMPMSimulator")
        self.params = prm
        self.sphere_size = None

    # -- device selection -------------------------------------------------
    def _on_device(self):
        dev = self._device
        if dev is None:
            import contextlib
            return contextlib.nullcontext()
        import torch
        return torch.cuda.device(dev)

    # -- the reference's interface ---------------------------------------
    @property
    def numParticles(self) -> int:
        return int(self._lib.mpm_num_particles(self._handle))

    @property
    def gridCount(self) -> int:
        return int(self._lib.mpm_grid_count(self._handle))

    def reset(self, numParticles: int, initBoxSize) -> None:
        """mls-mpm/mls-mpm.ts:225-243."""
        self.sphere_size = self.renderDiameter  # renderUniformsViews.sphere_size (:226)
        box = (ctypes.c_double * 3)(*[float(b) for b in initBoxSize])
        _check(self._lib.mpm_reset_dambreak(self._handle, int(numParticles), box,
                                            ctypes.c_uint64(self.seed)), "reset")
        if self.particleBuffer is not None:
            self.writeParticleBuffer()

    def execute(self, commandEncoder=None, substeps: int = 2) -> None:
        """mls-mpm/mls-mpm.ts:245-268 (two substeps per frame)."""
        _check(self._lib.mpm_step(self._handle, int(substeps), _stream_handle(commandEncoder)),
               "execute")

    def changeBoxSize(self, realBoxSize) -> None:
        """mls-mpm/mls-mpm.ts:270-275."""
        box = (ctypes.c_float * 3)(*[float(b) for b in realBoxSize])
        _check(self._lib.mpm_set_real_box(self._handle, box), "changeBoxSize")

    # -- beyond the reference: state access and diagnostics ---------------
    def upload(self, particles: np.ndarray, initBoxSize) -> None:
        arr = np.ascontiguousarray(particles, dtype=np.float32).reshape(-1, 20)
        box = (ctypes.c_float * 3)(*[float(b) for b in initBoxSize])
        _check(self._lib.mpm_upload(self._handle, arr.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                    len(arr), box), "upload")

    def downloadParticles(self) -> np.ndarray:
        out = np.zeros((self.numParticles, 20), dtype=np.float32)
        _check(self._lib.mpm_download_particles(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "downloadParticles")
        return out

    def downloadGrid(self) -> np.ndarray:
        out = np.zeros((self.gridCount, 4), dtype=np.int32)
        _check(self._lib.mpm_download_grid(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))), "downloadGrid")
        return out

    def downloadPosvel(self, commandEncoder=None, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.zeros((self.numParticles, 8), dtype=np.float32)
        _check(self._lib.mpm_download_posvel(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            _stream_handle(commandEncoder)), "downloadPosvel")
        if commandEncoder is None:
            self.synchronize()
        return out

    def downloadPosvelAsync(self, commandEncoder=None, out: np.ndarray | None = None) -> np.ndarray:
        """Pipelined read-back: snapshots posvel on the stream and copies it
        to `out` (pinned host memory for real overlap) on the library's copy
        stream; the next execute() overlaps the transfer.  `out` is valid
        after waitPosvel()."""
        if out is None:
            out = np.zeros((self.numParticles, 8), dtype=np.float32)
        _check(self._lib.mpm_download_posvel_async(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            _stream_handle(commandEncoder)), "downloadPosvelAsync")
        return out

    def waitPosvel(self, commandEncoder=None) -> None:
        """Waits for the last downloadPosvelAsync copy (on the host, or makes
        the given stream wait)."""
        _check(self._lib.mpm_wait_posvel(self._handle, _stream_handle(commandEncoder)),
               "waitPosvel")

    def writeParticleBuffer(self) -> None:
        """Copies the particle records (80-byte layout) into particleBuffer."""
        import torch
        recs = torch.from_numpy(self.downloadParticles().reshape(-1).view(np.uint8))
        dst = self.particleBuffer.view(torch.uint8).reshape(-1)[: recs.numel()]
        dst.copy_(recs)

    def dispatch(self, kernel: str, commandEncoder=None) -> None:
        """Runs one WGSL entry point alone (mls-mpm/mls-mpm.ts:248-265)."""
        _check(self._lib.mpm_dispatch(self._handle, L.KERNELS[kernel],
                                      _stream_handle(commandEncoder)), kernel)

    @property
    def engine(self) -> str:
        return "dispatch" if self._lib.mpm_get_engine(self._handle) == L.MPM_ENGINE_DISPATCH else "sorted"

    @engine.setter
    def engine(self, name: str) -> None:
        code = {"sorted": L.MPM_ENGINE_SORTED, "dispatch": L.MPM_ENGINE_DISPATCH}[name]
        _check(self._lib.mpm_set_engine(self._handle, code), "engine")

    def posvelDevicePtr(self) -> int:
        return int(self._lib.mpm_posvel_device_ptr(self._handle) or 0)

    def setGravity(self, gravity) -> None:
        """Body force per unit time (default (0, -0.3, 0), updateGrid.wgsl:34)."""
        g = (ctypes.c_float * 3)(*[float(x) for x in gravity])
        _check(self._lib.mpm_set_gravity(self._handle, g), "setGravity")

    def setGraph(self, enable: bool) -> None:
        """Run execute()'s substeps as one CUDA graph (sorted engine; on by
        default)."""
        _check(self._lib.mpm_set_graph(self._handle, int(bool(enable))), "setGraph")

    @property
    def taskSize(self) -> int:
        """Most particles per sorted-engine task (0 to set: automatic)."""
        return _check(self._lib.mpm_get_task_size(self._handle), "taskSize")

    @taskSize.setter
    def taskSize(self, cap: int) -> None:
        _check(self._lib.mpm_set_task_size(self._handle, int(cap)), "taskSize")

    @property
    def laneTableMin(self) -> int:
        """Smallest sorted-engine task that orders its particles by bank class
        (0 to set: the default; above 1024: never)."""
        return _check(self._lib.mpm_get_lane_table_min(self._handle), "laneTableMin")

    @laneTableMin.setter
    def laneTableMin(self, min_particles: int) -> None:
        _check(self._lib.mpm_set_lane_table_min(self._handle, int(min_particles)),
               "laneTableMin")

    @property
    def taskThreads(self) -> int:
        """Threads per block of the sorted engine's task kernels (128, 256,
        512; 0 to set: the default)."""
        return _check(self._lib.mpm_get_task_threads(self._handle), "taskThreads")

    @taskThreads.setter
    def taskThreads(self, threads: int) -> None:
        _check(self._lib.mpm_set_task_threads(self._handle, int(threads)), "taskThreads")

    @property
    def binPairing(self) -> int:
        """Two 4x4x4-cell bins stacked along z whose particles together
        number at most this share one task (default 512; 0: never; 2**30:
        every pair whose bins both hold particles; 2**31 - 1 to set: the
        default)."""
        return _check(self._lib.mpm_get_bin_pairing(self._handle), "binPairing")

    @binPairing.setter
    def binPairing(self, max_particles: int) -> None:
        _check(self._lib.mpm_set_bin_pairing(self._handle, int(max_particles)), "binPairing")

    def tuning(self) -> dict:
        """The engine's tunable configuration."""
        return {"bin_pairing": self.binPairing, "task_threads": self.taskThreads,
                "task_size": self.taskSize, "lane_table_min": self.laneTableMin}

    def autotune(self, substeps: int = 8, cache: str | None = None,
                 key: str | None = None) -> int:
        """Picks the fastest z-pair threshold, task-kernel block size, task
        size and lane-table threshold for the current scene (returns the task
        size); state unchanged.  cache: a JSON file of earlier choices by workload key
        (default key: particle count and grid size); a hit applies the
        stored choice without timing anything, a miss times and stores."""
        key = key or f"MLSMPMSimulator/n={self.numParticles}/cells={self.gridCount}"

        def run():
            out = ctypes.c_int(0)
            _check(self._lib.mpm_autotune(self._handle, int(substeps), ctypes.byref(out)),
                   "autotune")
            return self.tuning()

        choice = _cached_tuning(cache, key, run, self._apply_tuning)
        return int(choice["task_size"])

    def _apply_tuning(self, choice: dict) -> None:
        self.binPairing = choice.get("bin_pairing", 2**31 - 1)
        self.taskThreads = choice["task_threads"]
        self.taskSize = choice["task_size"]
        self.laneTableMin = choice["lane_table_min"]

    def checkHealth(self) -> dict:
        h = L.Health()
        code = self._lib.mpm_check_health(self._handle, ctypes.byref(h))
        if code not in (L.MPM_OK, L.MPM_E_NONFINITE):
            _check(code, "checkHealth")
        return {"nonfinite_particles": int(h.nonfinite_particles),
                "out_of_range_accesses": int(h.out_of_range_accesses),
                "ok": code == L.MPM_OK}

    def setProfiling(self, enable: bool) -> None:
        """Per-kernel CUDA-event timing on the launch stream (resets counters)."""
        _check(self._lib.mpm_set_profiling(self._handle, int(bool(enable))), "setProfiling")

    def kernelStats(self) -> dict:
        """{kernel name: (launches, timed launches, total device ms)}."""
        buf = (L.KernelStat * 32)()
        n = _check(self._lib.mpm_kernel_stats(self._handle, buf, 32), "kernelStats")
        return {buf[i].name.decode(): (int(buf[i].launches), int(buf[i].timed_launches),
                                       float(buf[i].total_ms)) for i in range(min(n, 32))}

    def launchCount(self) -> int:
        return int(self._lib.mpm_launch_count(self._handle))

    def synchronize(self) -> None:
        _check(self._lib.mpm_synchronize(self._handle), "synchronize")

    def close(self) -> None:
        if self._handle:
            self._lib.mpm_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def scene_dambreak(initBoxSize, numParticles: int, seed: int) -> np.ndarray:
    """initDambreak (mls-mpm/mls-mpm.ts:195-223) on the host, Math.random ->
    SplitMix64(seed); returns (n, 20) float32 records."""
    out = np.zeros((max(int(numParticles), 1), 20), dtype=np.float32)
    box = (ctypes.c_double * 3)(*[float(b) for b in initBoxSize])
    n = _check(L.load().mpm_scene_dambreak(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                           int(numParticles), box, ctypes.c_uint64(seed)))
    return out[:n].copy()


def scene_lattice(n_per_axis: int, origin: float, spacing: float = 0.5, jitter: float = 0.05,
                  seed: int = 0) -> np.ndarray:
    """Jittered cubic lattice of n_per_axis^3 particles (x-major)."""
    out = np.zeros((max(n_per_axis, 1) ** 3, 20), dtype=np.float32)
    n = _check(L.load().mpm_scene_lattice(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                          int(n_per_axis), float(origin), float(spacing),
                                          float(jitter), ctypes.c_uint64(seed)))
    return out[:n].copy()


def probe_conversions(values: np.ndarray, fm: float = 1e7):
    vals = np.ascontiguousarray(values, dtype=np.float32)
    enc = np.zeros(len(vals), dtype=np.int32)
    dec = np.zeros(len(vals), dtype=np.float32)
    _check(L.load().mpm_probe_conversions(vals.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                          len(vals), fm,
                                          enc.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                          dec.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
    return enc, dec


def probe_packed(a: np.ndarray, b: np.ndarray):
    """Packed f32x2 ops on the device vs the scalar ops: returns
    (packed_mul, packed_add, packed_muladd, scalar_mul, scalar_add,
    scalar_muladd), muladd = (a*b)+a with the product rounded first."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    n = len(a)
    out = np.zeros(6 * n, dtype=np.float32)
    fptr = ctypes.POINTER(ctypes.c_float)
    _check(L.load().mpm_probe_packed(a.ctypes.data_as(fptr), b.ctypes.data_as(fptr), n,
                                     out.ctypes.data_as(fptr)))
    return tuple(out[i * n:(i + 1) * n] for i in range(6))


# ---------------------------------------------------------------------------
# Batches of independent scenes
# ---------------------------------------------------------------------------

def scene_desc(num_particles: int, init_box, real_box=None, *, stiffness: float = 3.0,
               rest_density: float = 4.0, dynamic_viscosity: float = 0.1, dt: float = 0.2,
               fixed_point_multiplier: float = 1e7, gravity=(0.0, -0.3, 0.0)) -> L.SceneDesc:
    """One scene of a batch; the defaults are mls-mpm/mls-mpm.ts:53-59."""
    d = L.SceneDesc()
    d.num_particles = int(num_particles)
    real_box = init_box if real_box is None else real_box
    for a in range(3):
        d.init_box[a] = float(init_box[a])
        d.real_box[a] = float(real_box[a])
        d.gravity[a] = float(gravity[a])
    d.stiffness = stiffness
    d.rest_density = rest_density
    d.dynamic_viscosity = dynamic_viscosity
    d.dt = dt
    d.fixed_point_multiplier = fixed_point_multiplier
    return d


def batch_scenes(num_scenes: int = 256, seed: int = 0, n_range=(4000, 64000), sides=(32, 48, 64),
                 spacing: float = 0.5, jitter: float = 0.05, stiffness_range=(2.0, 4.0),
                 gravity_magnitude: float = 0.3, gravity=None):
    """Independent dam-break-like scenes of uneven sizes (numpy PCG64(seed)).

    Per scene: n uniform in n_range; a cubic grid whose side is drawn from
    `sides`; the first n points (x-major) of a jittered cubic lattice with
    ceil(cbrt(n)) points per axis, spacing `spacing`, placed at a uniform
    origin with the block inside the walls [3, side - 4]; gravity a uniform
    random direction times `gravity_magnitude` (or the fixed vector
    `gravity` when given); stiffness uniform in
    stiffness_range; the other constants are the reference's.
    Returns (list of SceneDesc, (sum n, 20) float32 records).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    descs, recs = [], []
    for _ in range(num_scenes):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        side = int(sides[int(rng.integers(0, len(sides)))])
        a = 1
        while a * a * a < n:
            a += 1
        extent = (a - 1) * spacing + 2 * jitter
        lo, hi = 3.0 + jitter, side - 4.0 - extent
        origin = lo + rng.random(3) * max(hi - lo, 0.0)
        idx = np.arange(n)
        lat = np.stack([idx // (a * a), (idx // a) % a, idx % a], axis=1).astype(np.float64)
        pos = origin + spacing * lat + jitter * (2.0 * rng.random((n, 3)) - 1.0)
        g = rng.normal(size=3)
        g = gravity_magnitude * g / np.linalg.norm(g) if gravity is None else np.asarray(gravity)
        k = float(rng.uniform(*stiffness_range))
        r = np.zeros((n, 20), dtype=np.float32)
        r[:, 0:3] = pos.astype(np.float32)
        descs.append(scene_desc(n, (side, side, side), stiffness=k, gravity=tuple(np.float32(g))))
        recs.append(r)
    return descs, np.concatenate(recs) if recs else np.zeros((0, 20), np.float32)


class MLSMPMBatch:
    """Many independent scenes advanced together: one launch per stage for
    all scenes, replayed as a CUDA graph.  Scene s behaves exactly like an
    MLSMPMSimulator holding it alone with the same constants."""

    def __init__(self, scenes, particles: np.ndarray, device=None, graph: bool = True):
        self._lib = L.load()
        self._device = device
        descs = list(scenes)
        self._descs = descs
        arr = (L.SceneDesc * len(descs))(*descs)
        recs = np.ascontiguousarray(particles, dtype=np.float32).reshape(-1, 20)
        counts = np.array([d.num_particles for d in descs], dtype=np.int64)
        if recs.shape[0] != int(counts.sum()):
            raise ValueError("particle array does not match the scenes' particle counts")
        self.sceneOffsets = np.concatenate([[0], np.cumsum(counts)])
        self._handle = ctypes.c_void_p()
        with self._on_device():
            _check(self._lib.mpm_batch_create(arr, len(descs),
                                              recs.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                              ctypes.byref(self._handle)), "MLSMPMBatch")
        self.setGraph(graph)

    def _on_device(self):
        if self._device is None:
            import contextlib
            return contextlib.nullcontext()
        import torch
        return torch.cuda.device(self._device)

    @property
    def numScenes(self) -> int:
        return int(self._lib.mpm_batch_num_scenes(self._handle))

    @property
    def numParticles(self) -> int:
        return int(self._lib.mpm_batch_num_particles(self._handle))

    def gridCount(self, scene: int) -> int:
        d = self._descs[scene]
        return int(np.prod([np.ceil(np.float64(d.init_box[a])) for a in range(3)]))

    def step(self, substeps: int = 2, commandEncoder=None) -> None:
        _check(self._lib.mpm_batch_step(self._handle, int(substeps),
                                        _stream_handle(commandEncoder)), "step")

    def upload(self, particles: np.ndarray) -> None:
        """Restarts every scene from new particle records (same counts and
        order as at construction); keeps the captured CUDA graphs."""
        recs = np.ascontiguousarray(particles, dtype=np.float32).reshape(-1, 20)
        if recs.shape[0] != int(self.sceneOffsets[-1]):
            raise ValueError("particle array does not match the scenes' particle counts")
        with self._on_device():
            _check(self._lib.mpm_batch_upload(self._handle,
                                              recs.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                   "upload")

    def execute(self, commandEncoder=None) -> None:
        """Two substeps of every scene (mls-mpm/mls-mpm.ts:245-268)."""
        self.step(2, commandEncoder)

    def setScene(self, scene: int, desc: L.SceneDesc) -> None:
        _check(self._lib.mpm_batch_set_scene(self._handle, int(scene), ctypes.byref(desc)),
               "setScene")
        self._descs[scene] = desc

    def changeBoxSize(self, scene: int, realBoxSize) -> None:
        d = L.SceneDesc.from_buffer_copy(self._descs[scene])
        for a in range(3):
            d.real_box[a] = float(realBoxSize[a])
        self.setScene(scene, d)

    def setGraph(self, enable: bool) -> None:
        _check(self._lib.mpm_batch_set_graph(self._handle, int(bool(enable))), "setGraph")

    def setTaskSize(self, cap: int) -> None:
        _check(self._lib.mpm_batch_set_task_size(self._handle, int(cap)), "setTaskSize")

    @property
    def taskSize(self) -> int:
        return _check(self._lib.mpm_batch_get_task_size(self._handle), "taskSize")

    @property
    def laneTableMin(self) -> int:
        """See MLSMPMSimulator.laneTableMin."""
        return _check(self._lib.mpm_batch_get_lane_table_min(self._handle), "laneTableMin")

    @laneTableMin.setter
    def laneTableMin(self, min_particles: int) -> None:
        _check(self._lib.mpm_batch_set_lane_table_min(self._handle, int(min_particles)),
               "laneTableMin")

    @property
    def taskThreads(self) -> int:
        """See MLSMPMSimulator.taskThreads."""
        return _check(self._lib.mpm_batch_get_task_threads(self._handle), "taskThreads")

    @taskThreads.setter
    def taskThreads(self, threads: int) -> None:
        _check(self._lib.mpm_batch_set_task_threads(self._handle, int(threads)), "taskThreads")

    @property
    def binPairing(self) -> int:
        """See MLSMPMSimulator.binPairing."""
        return _check(self._lib.mpm_batch_get_bin_pairing(self._handle), "binPairing")

    @binPairing.setter
    def binPairing(self, max_particles: int) -> None:
        _check(self._lib.mpm_batch_set_bin_pairing(self._handle, int(max_particles)), "binPairing")

    def tuning(self) -> dict:
        return {"bin_pairing": self.binPairing, "task_threads": self.taskThreads,
                "task_size": self.taskSize, "lane_table_min": self.laneTableMin}

    def autotune(self, substeps: int = 4, cache: str | None = None,
                 key: str | None = None) -> int:
        """Z-pair threshold, block size, task size and lane-table threshold,
        as MLSMPMSimulator.autotune (default key: scene and particle counts)."""
        key = key or f"MLSMPMBatch/scenes={self.numScenes}/n={self.numParticles}"

        def run():
            out = ctypes.c_int(0)
            _check(self._lib.mpm_batch_autotune(self._handle, int(substeps), ctypes.byref(out)),
                   "autotune")
            return self.tuning()

        def apply(choice):
            self.binPairing = choice.get("bin_pairing", 2**31 - 1)
            self.taskThreads = choice["task_threads"]
            self.taskSize = choice["task_size"]
            self.laneTableMin = choice["lane_table_min"]

        return int(_cached_tuning(cache, key, run, apply)["task_size"])

    def downloadParticles(self) -> np.ndarray:
        out = np.zeros((self.numParticles, 20), dtype=np.float32)
        _check(self._lib.mpm_batch_download_particles(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "downloadParticles")
        return out

    def downloadGrid(self, scene: int) -> np.ndarray:
        out = np.zeros((self.gridCount(scene), 4), dtype=np.int32)
        _check(self._lib.mpm_batch_download_grid(
            self._handle, int(scene), out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))),
            "downloadGrid")
        return out

    def posvelDevicePtr(self) -> int:
        return int(self._lib.mpm_batch_posvel_device_ptr(self._handle) or 0)

    def checkHealth(self) -> dict:
        h = L.Health()
        code = self._lib.mpm_batch_check_health(self._handle, ctypes.byref(h))
        if code not in (L.MPM_OK, L.MPM_E_NONFINITE):
            _check(code, "checkHealth")
        return {"nonfinite_particles": int(h.nonfinite_particles),
                "out_of_range_accesses": int(h.out_of_range_accesses),
                "ok": code == L.MPM_OK}

    def setProfiling(self, enable: bool) -> None:
        """Per-kernel CUDA-event timing on the launch stream (resets counters;
        CUDA graphs are bypassed while it is on)."""
        _check(self._lib.mpm_batch_set_profiling(self._handle, int(bool(enable))), "setProfiling")

    def kernelStats(self) -> dict:
        """{kernel name: (launches, timed launches, total device ms)}."""
        buf = (L.KernelStat * 32)()
        n = _check(self._lib.mpm_batch_kernel_stats(self._handle, buf, 32), "kernelStats")
        return {buf[i].name.decode(): (int(buf[i].launches), int(buf[i].timed_launches),
                                       float(buf[i].total_ms)) for i in range(min(n, 32))}

    def launchCount(self) -> int:
        return int(self._lib.mpm_batch_launch_count(self._handle))

    def close(self) -> None:
        if self._handle:
            self._lib.mpm_batch_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Differentiation
# ---------------------------------------------------------------------------

class MLSMPMAdjoint:
    """Forward with checkpoints and reverse-mode backward over a batch of
    scenes (pass one scene for a single simulation).

    forward(init, substeps) runs the fixed-point solver from `init` ((N, 20)
    particle records of all scenes) and keeps the state every
    `checkpointEvery` substeps.  backward(seeds) takes {substep: dL/dstate}
    ((N, 20) arrays in the particle-record layout) and returns
    (dL/d initial state (N, 20), dL/d (stiffness, dynamic_viscosity) per
    scene (S, 2)).  The derivative is that of the continuous model the solver
    discretises, along the solver's trajectory."""

    def __init__(self, scenes, maxSubsteps: int, checkpointEvery: int = 20, device=None,
                 tape: str = "fp64"):
        self._lib = L.load()
        self._device = device
        self._descs = list(scenes)
        arr = (L.SceneDesc * len(self._descs))(*self._descs)
        counts = np.array([d.num_particles for d in self._descs], dtype=np.int64)
        self.sceneOffsets = np.concatenate([[0], np.cumsum(counts)])
        self.numParticles = int(self.sceneOffsets[-1])
        self.maxSubsteps = int(maxSubsteps)
        self.checkpointEvery = min(int(checkpointEvery), self.maxSubsteps)
        self.substeps = None
        self._handle = ctypes.c_void_p()
        with self._on_device():
            _check(self._lib.mpm_adjoint_create(arr, len(self._descs), self.maxSubsteps,
                                                int(checkpointEvery), ctypes.byref(self._handle)),
                   "MLSMPMAdjoint")
        self.tape = tape

    @property
    def tape(self) -> str:
        return self._tape

    @tape.setter
    def tape(self, name: str) -> None:
        """"fp64": the continuous model integrated in FP64 (default);
        "fixed": the solver's own fixed-point trajectory."""
        code = {"fixed": L.MPM_TAPE_FIXED_POINT, "fp64": L.MPM_TAPE_FP64}[name]
        _check(self._lib.mpm_adjoint_set_tape(self._handle, code), "tape")
        self._tape = name
        self.substeps = None

    def _on_device(self):
        if self._device is None:
            import contextlib
            return contextlib.nullcontext()
        import torch
        return torch.cuda.device(self._device)

    @property
    def numScenes(self) -> int:
        return len(self._descs)

    def setScene(self, scene: int, desc: L.SceneDesc) -> None:
        _check(self._lib.mpm_adjoint_set_scene(self._handle, int(scene), ctypes.byref(desc)),
               "setScene")
        self._descs[scene] = desc
        self.substeps = None

    def forward(self, init: np.ndarray, substeps: int, commandEncoder=None) -> None:
        recs = np.ascontiguousarray(init, dtype=np.float32).reshape(-1, 20)
        if len(recs) != self.numParticles:
            raise ValueError("initial state does not match the scenes' particle counts")
        _check(self._lib.mpm_forward_ckpt(self._handle,
                                          recs.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                          int(substeps), _stream_handle(commandEncoder)),
               "forward")
        self.substeps = int(substeps)

    def state(self, substep: int, out: np.ndarray | None = None) -> np.ndarray:
        """The state after `substep` substeps of the last forward (a
        checkpoint), as (N, 20) records; written into `out` when given."""
        if out is None:
            out = np.empty((self.numParticles, 20), dtype=np.float32)
        elif (out.dtype != np.float32 or out.shape != (self.numParticles, 20)
              or not out.flags.c_contiguous):
            raise ValueError("out must be a C-contiguous float32 (N, 20) array")
        _check(self._lib.mpm_adjoint_state(self._handle, int(substep),
                                           out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
               "state")
        return out

    def backward(self, seeds: dict, commandEncoder=None):
        steps = sorted(seeds)
        n = self.numParticles
        blocks = [np.ascontiguousarray(seeds[t], dtype=np.float32).reshape(n, 20) for t in steps]
        fp = ctypes.POINTER(ctypes.c_float)
        ptrs = (fp * max(len(steps), 1))(*[b.ctypes.data_as(fp) for b in blocks])
        st = (ctypes.c_int32 * max(len(steps), 1))(*[int(t) for t in steps])
        grad = np.empty((n, 20), dtype=np.float32)
        pgrad = np.zeros((self.numScenes, 2), dtype=np.float64)
        _check(self._lib.mpm_backward_list(self._handle, ptrs, st, len(steps),
                                           grad.ctypes.data_as(fp),
                                           pgrad.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                           _stream_handle(commandEncoder)), "backward")
        return grad, pgrad

    def setObservations(self, observed: dict) -> None:
        """Observed positions {substep: (N, 3) array} for observationLoss; the
        substeps must be checkpoints of the forwards that follow."""
        steps = sorted(observed)
        n = self.numParticles
        blocks = [np.ascontiguousarray(observed[t], dtype=np.float32).reshape(n, 3)
                  for t in steps]
        fp = ctypes.POINTER(ctypes.c_float)
        ptrs = (fp * max(len(steps), 1))(*[b.ctypes.data_as(fp) for b in blocks])
        st = (ctypes.c_int32 * max(len(steps), 1))(*[int(t) for t in steps])
        _check(self._lib.mpm_adjoint_set_observations(self._handle, len(steps), st, ptrs),
               "setObservations")

    def observationLoss(self, commandEncoder=None) -> np.ndarray:
        """Per scene: the sum over observed substeps of the mean squared
        distance of its particles to the observed positions, for the last
        forward; leaves the seeds of backwardObserved on the device."""
        loss = np.zeros(self.numScenes, dtype=np.float64)
        _check(self._lib.mpm_adjoint_observation_loss(
            self._handle, loss.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            _stream_handle(commandEncoder)), "observationLoss")
        return loss

    def backwardObserved(self, commandEncoder=None, grad_init: bool = True):
        """backward() with the seeds of the last observationLoss; returns
        (dL/d initial state or None, (S, 2) dL/d(stiffness, viscosity))."""
        fp = ctypes.POINTER(ctypes.c_float)
        grad = np.empty((self.numParticles, 20), dtype=np.float32) if grad_init else None
        pgrad = np.zeros((self.numScenes, 2), dtype=np.float64)
        _check(self._lib.mpm_backward_observed(
            self._handle, grad.ctypes.data_as(fp) if grad is not None else None,
            pgrad.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            _stream_handle(commandEncoder)), "backwardObserved")
        return grad, pgrad

    def close(self) -> None:
        if self._handle:
            self._lib.mpm_adjoint_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def centroid_loss(state: np.ndarray, target, offsets=None):
    """Squared distance of each scene's particle centroid to `target`:
    returns (loss per scene, dL/dstate (N, 20) with the position columns set)."""
    state = np.asarray(state, dtype=np.float32).reshape(-1, 20)
    offsets = [0, len(state)] if offsets is None else list(offsets)
    t = np.asarray(target, dtype=np.float64)
    seed = np.zeros_like(state)
    losses = []
    for s in range(len(offsets) - 1):
        lo, hi = int(offsets[s]), int(offsets[s + 1])
        x = state[lo:hi, 0:3].astype(np.float64)
        c = x.mean(axis=0)
        losses.append(float(np.sum((c - t) ** 2)))
        seed[lo:hi, 0:3] = (2.0 * (c - t) / (hi - lo)).astype(np.float32)
    return np.array(losses), seed
