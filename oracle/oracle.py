"""ctypes front end of the C oracle (oracle/mpm_oracle.c, the FP64
continuous restatement oracle/mpm_oracle64.c used for finite differences,
the renderer restatement oracle/render_oracle.c and the SPH restatement
oracle/sph_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py (cpu_baseline leg and `--impl reference`) as the checker or the
CPU baseline.  The product never imports it.

Arrays use the reference's layouts: particles (n, 20) float32 (80 B each,
mls-mpm/mls-mpm.ts:10), cells (grid_count, 4) int32 {vx, vy, vz, mass}
(mls-mpm/p2g_1.wgsl:6-11), posvel (n, 8) float32 (copyPosition.wgsl:7-10).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "build")
LIB_PATH = os.path.join(BUILD_DIR, "libmpm_oracle.so")
SOURCES = [os.path.join(HERE, "mpm_oracle.c"), os.path.join(HERE, "mpm_oracle64.c"),
           os.path.join(HERE, "mpm_adjoint64.c"),
           os.path.join(HERE, "render_oracle.c"), os.path.join(HERE, "sph_oracle.c")]

# -ffp-contract=off: every float op rounds separately, as the WGSL restatement
# requires; no -ffast-math (keeps IEEE division, NaN and denormal semantics).
CFLAGS = ["-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
          "-pthread"]


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/build/libmpm_oracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", *CFLAGS, "-o", tmp, *SOURCES, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Params(ctypes.Structure):
    """orc_params; defaults are mls-mpm/mls-mpm.ts:53-59."""
    _fields_ = [
        ("stiffness", ctypes.c_float),
        ("rest_density", ctypes.c_float),
        ("dynamic_viscosity", ctypes.c_float),
        ("dt", ctypes.c_float),
        ("fixed_point_multiplier", ctypes.c_float),
        ("gravity", ctypes.c_float * 3),
    ]

    @classmethod
    def reference(cls) -> "Params":
        return cls.make()

    @classmethod
    def make(cls, stiffness=3.0, rest_density=4.0, dynamic_viscosity=0.1, dt=0.2,
             fixed_point_multiplier=1e7, gravity=(0.0, -0.3, 0.0)) -> "Params":
        """Scene constants; gravity (0, -0.3, 0) is updateGrid.wgsl:34."""
        p = cls(stiffness, rest_density, dynamic_viscosity, dt, fixed_point_multiplier)
        for a in range(3):
            p.gravity[a] = gravity[a]
        return p


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        box = ctypes.POINTER(ctypes.c_float)
        prm = ctypes.POINTER(Params)
        i64 = ctypes.c_int64
        L.orc_grid_count.argtypes = [box]
        L.orc_grid_count.restype = i64
        L.orc_clear_grid.argtypes = [i32p, i64]
        L.orc_p2g_1.argtypes = [f32p, i64, i32p, i64, box, prm]
        L.orc_p2g_1.restype = i64
        L.orc_p2g_2.argtypes = [f32p, i64, i32p, i64, box, prm]
        L.orc_p2g_2.restype = i64
        L.orc_update_grid.argtypes = [i32p, i64, box, box, prm]
        L.orc_g2p.argtypes = [f32p, i64, i32p, i64, box, box, prm]
        L.orc_g2p.restype = i64
        L.orc_copy_position.argtypes = [f32p, i64, f32p]
        L.orc_execute.argtypes = [f32p, i64, i32p, i64, box, box, prm, ctypes.c_void_p,
                                  ctypes.c_int, ctypes.c_int]
        L.orc_execute.restype = i64
        L.orc_enc.argtypes = [ctypes.c_float, ctypes.c_float]
        L.orc_enc.restype = ctypes.c_int32
        L.orc_dec.argtypes = [ctypes.c_int32, ctypes.c_float]
        L.orc_dec.restype = ctypes.c_float
        _lib = L
    return _lib


def _box(b) -> ctypes.Array:
    return (ctypes.c_float * 3)(*[float(np.float32(x)) for x in b])


def grid_count(init_box) -> int:
    return int(lib().orc_grid_count(_box(init_box)))


class OracleSim:
    """CPU mirror of MLSMPMSimulator's state (mls-mpm/mls-mpm.ts:12-276)."""

    def __init__(self, particles: np.ndarray, init_box, params: Params | None = None,
                 real_box=None):
        self.params = params or Params.reference()
        self.particles = np.ascontiguousarray(particles, dtype=np.float32).reshape(-1, 20).copy()
        self.init_box = [float(np.float32(x)) for x in init_box]
        self.real_box = list(self.init_box if real_box is None else
                             [float(np.float32(x)) for x in real_box])
        self.grid_count = grid_count(self.init_box)
        self.cells = np.zeros((self.grid_count, 4), dtype=np.int32)
        self.posvel = np.zeros((len(self.particles), 8), dtype=np.float32)
        self.oob = 0

    @property
    def n(self) -> int:
        return len(self.particles)

    def change_box_size(self, real_box):
        self.real_box = [float(np.float32(x)) for x in real_box]

    # one call per WGSL entry point
    def clear_grid(self):
        lib().orc_clear_grid(self.cells, self.grid_count)

    def p2g_1(self):
        self.oob += lib().orc_p2g_1(self.particles, self.n, self.cells, self.grid_count,
                                    _box(self.init_box), ctypes.byref(self.params))

    def p2g_2(self):
        self.oob += lib().orc_p2g_2(self.particles, self.n, self.cells, self.grid_count,
                                    _box(self.init_box), ctypes.byref(self.params))

    def update_grid(self):
        lib().orc_update_grid(self.cells, self.grid_count, _box(self.real_box),
                              _box(self.init_box), ctypes.byref(self.params))

    def g2p(self):
        self.oob += lib().orc_g2p(self.particles, self.n, self.cells, self.grid_count,
                                  _box(self.real_box), _box(self.init_box),
                                  ctypes.byref(self.params))

    def copy_position(self):
        lib().orc_copy_position(self.particles, self.n, self.posvel)

    def substep(self):
        self.clear_grid()
        self.p2g_1()
        self.p2g_2()
        self.update_grid()
        self.g2p()
        self.copy_position()

    def execute(self, substeps: int = 2, nthreads: int = 1):
        """mls-mpm/mls-mpm.ts:245-268 (2 substeps per call by default)."""
        r = lib().orc_execute(self.particles, self.n, self.cells, self.grid_count,
                              _box(self.real_box), _box(self.init_box),
                              ctypes.byref(self.params),
                              self.posvel.ctypes.data_as(ctypes.c_void_p), substeps, nthreads)
        if r < 0:
            raise RuntimeError("oracle thread error")
        self.oob += r


def enc(f: float, fm: float = 1e7) -> int:
    return int(lib().orc_enc(f, fm))


def dec(i: int, fm: float = 1e7) -> float:
    return float(lib().orc_dec(i, fm))


# ---------------------------------------------------------------------------
# FP64 continuous model (mpm_oracle64.c): the function the adjoint
# differentiates, for central finite differences.
# ---------------------------------------------------------------------------

class Params64(ctypes.Structure):
    _fields_ = [
        ("stiffness", ctypes.c_double),
        ("rest_density", ctypes.c_double),
        ("dynamic_viscosity", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("init_box", ctypes.c_double * 3),
        ("real_box", ctypes.c_double * 3),
    ]

    @classmethod
    def make(cls, init_box, real_box=None, stiffness=3.0, rest_density=4.0,
             dynamic_viscosity=0.1, dt=0.2, gravity=(0.0, -0.3, 0.0)) -> "Params64":
        """Constants as f32 values widened to double (the f32 solver's)."""
        f = lambda v: float(np.float32(v))
        p = cls(f(stiffness), f(rest_density), f(dynamic_viscosity), f(dt))
        real_box = init_box if real_box is None else real_box
        for a in range(3):
            p.gravity[a] = f(gravity[a])
            p.init_box[a] = f(init_box[a])
            p.real_box[a] = f(real_box[a])
        return p


def records_to_state64(recs: np.ndarray) -> np.ndarray:
    """(n, 20) float32 particle records -> (n, 15) float64 state
    (x, v, C by columns)."""
    r = np.asarray(recs, dtype=np.float32).reshape(-1, 20).astype(np.float64)
    out = np.empty((len(r), 15), dtype=np.float64)
    out[:, 0:3] = r[:, 0:3]
    out[:, 3:6] = r[:, 4:7]
    for c in range(3):
        out[:, 6 + 3 * c:9 + 3 * c] = r[:, 8 + 4 * c:11 + 4 * c]
    return out


def run64(state: np.ndarray, params: Params64, substeps: int) -> np.ndarray:
    """Returns the state after `substeps` substeps of the FP64 model."""
    L = lib()
    if not getattr(L, "_orc64_ready", False):
        L.orc64_run.argtypes = [np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS"),
                                ctypes.c_int64, ctypes.POINTER(Params64), ctypes.c_int]
        L.orc64_run.restype = ctypes.c_int64
        L._orc64_ready = True
    st = np.ascontiguousarray(state, dtype=np.float64).copy()
    if L.orc64_run(st, len(st), ctypes.byref(params), int(substeps)) < 0:
        raise MemoryError("orc64_run")
    return st


def backward64(state0: np.ndarray, params: Params64, substeps: int, seeds: dict,
               every: int = 20, f32_tape: bool = False):
    """FP64 tape adjoint on the CPU (mpm_adjoint64.c): gradient of a loss whose
    adjoint seeds are `seeds` = {substep t: (n, 15) adjoint of the state
    after t substeps}.  Returns (grad (n, 15) w.r.t. state0, [dL/d
    stiffness, dL/d dynamic viscosity]).  f32_tape: the trajectory is
    integrated in f32 (the reverse pass stays FP64)."""
    L = lib()
    f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    if not getattr(L, "_orc64_bwd_ready", False):
        L.orc64_backward_tape.argtypes = [f64p, ctypes.c_int64, ctypes.POINTER(Params64),
                                          ctypes.c_int, ctypes.c_int,
                                          np.ctypeslib.ndpointer(np.int32), f64p, ctypes.c_int,
                                          f64p, f64p, ctypes.c_int]
        L.orc64_backward_tape.restype = ctypes.c_int
        L._orc64_bwd_ready = True
    st = np.ascontiguousarray(state0, dtype=np.float64)
    n = len(st)
    ts = sorted(int(t) for t in seeds)
    vals = np.ascontiguousarray(np.stack([np.asarray(seeds[t], np.float64).reshape(n, 15)
                                          for t in ts]) if ts else np.zeros((0, n, 15)))
    grad = np.zeros((n, 15), np.float64)
    pgrad = np.zeros(2, np.float64)
    rc = L.orc64_backward_tape(st, n, ctypes.byref(params), int(substeps), int(every),
                               np.array(ts, np.int32), vals.reshape(-1) if vals.size else
                               np.zeros(1), len(ts), grad, pgrad, int(bool(f32_tape)))
    if rc != 0:
        raise MemoryError("orc64_backward")
    return grad, pgrad


# ---------------------------------------------------------------------------
# Screen-space renderer (render_oracle.c)
# ---------------------------------------------------------------------------

def _render_lib():
    L = lib()
    if not getattr(L, "_ro_ready", False):
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
        L.ro_render.argtypes = [f32p, ctypes.c_int64, f32p, ctypes.c_int, ctypes.c_int,
                                ctypes.c_float, ctypes.c_float, ctypes.c_float, f32p, ctypes.c_int,
                                f32p, u8p, f32p, f32p]
        L.ro_render.restype = ctypes.c_int
        fp = ctypes.POINTER(ctypes.c_float)
        L.ro_filter_constants.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, fp, fp, fp]
        for name in ("ro_exp", "ro_log", "ro_half_round"):
            getattr(L, name).argtypes = [ctypes.c_float]
            getattr(L, name).restype = ctypes.c_float
        L.ro_pow.argtypes = [ctypes.c_float, ctypes.c_float]
        L.ro_pow.restype = ctypes.c_float
        L.ro_bilateral_pass.argtypes = [f32p, f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                        ctypes.c_float]
        L.ro_bilateral_pass.restype = None
        L.ro_gaussian_pass.argtypes = [f32p, f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int]
        L.ro_gaussian_pass.restype = None
        L.ro_shade_pass.argtypes = [f32p, f32p, f32p, f32p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, f32p, u8p]
        L.ro_shade_pass.restype = None
        L.ro_sample_cube.argtypes = [f32p, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, f32p]
        L.ro_sample_cube.restype = None
        L.ro_splat.argtypes = [f32p, ctypes.c_int64, f32p, ctypes.c_int, ctypes.c_int, f32p, f32p]
        L.ro_splat.restype = ctypes.c_int
        L.ro_sphere.argtypes = [f32p, ctypes.c_int64, f32p, ctypes.c_int, ctypes.c_int, f32p, u8p,
                                f32p]
        L.ro_sphere.restype = ctypes.c_int
        L._ro_ready = True
    return L


def render(posvel: np.ndarray, uniforms_f32: np.ndarray, width: int, height: int, radius: float,
           fov: float, env: np.ndarray) -> dict:
    """The whole fluid path on the CPU.  uniforms_f32: the 272-byte
    RenderUniforms as 68 float32; env: (6, S, S, 4) float32."""
    L = _render_lib()
    pv = np.ascontiguousarray(posvel, dtype=np.float32).reshape(-1, 8)
    u = np.ascontiguousarray(uniforms_f32, dtype=np.float32).reshape(68)
    e = np.ascontiguousarray(env, dtype=np.float32)
    dt, mf, ppc = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
    L.ro_filter_constants(height, radius, fov, ctypes.byref(dt), ctypes.byref(mf), ctypes.byref(ppc))
    out = {"color": np.zeros((height, width, 4), np.float32),
           "color8": np.zeros((height, width, 4), np.uint8),
           "depth": np.zeros((height, width), np.float32),
           "thickness": np.zeros((height, width), np.float32)}
    if L.ro_render(pv, len(pv), u, width, height, dt, mf, ppc, e, e.shape[1], out["color"],
                   out["color8"], out["depth"], out["thickness"]) != 0:
        raise MemoryError("ro_render")
    return out


def splat(posvel: np.ndarray, uniforms_f32: np.ndarray, width: int, height: int) -> dict:
    """The depth and thickness splats alone (before the filters): depth =
    view-space z of the nearest fragment (0 where none), thickness rounded to
    half."""
    L = _render_lib()
    pv = np.ascontiguousarray(posvel, dtype=np.float32).reshape(-1, 8)
    u = np.ascontiguousarray(uniforms_f32, dtype=np.float32).reshape(68)
    out = {"depth": np.zeros((height, width), np.float32),
           "thickness": np.zeros((height, width), np.float32)}
    if L.ro_splat(pv, len(pv), u, width, height, out["depth"], out["thickness"]) != 0:
        raise MemoryError("ro_splat")
    return out


def sphere(posvel: np.ndarray, uniforms_f32: np.ndarray, width: int, height: int) -> dict:
    """Sphere mode (render/sphere.wgsl): colour, its rgba8 store and the
    winning fragment depth (1 where none)."""
    L = _render_lib()
    pv = np.ascontiguousarray(posvel, dtype=np.float32).reshape(-1, 8)
    u = np.ascontiguousarray(uniforms_f32, dtype=np.float32).reshape(68)
    out = {"color": np.zeros((height, width, 4), np.float32),
           "color8": np.zeros((height, width, 4), np.uint8),
           "depth": np.zeros((height, width), np.float32)}
    if L.ro_sphere(pv, len(pv), u, width, height, out["color"], out["color8"], out["depth"]) != 0:
        raise MemoryError("ro_sphere")
    return out


def render_scalar(name: str, *args) -> float:
    return float(getattr(_render_lib(), "ro_" + name)(*args))


def filter_constants(height: int, radius: float, fov: float):
    """(depth_threshold, max_filter_size, projected_particle_constant) of the
    filter passes for a screen height, particle radius and field of view."""
    L = _render_lib()
    dt, mf, ppc = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
    L.ro_filter_constants(height, radius, fov, ctypes.byref(dt), ctypes.byref(mf), ctypes.byref(ppc))
    return dt.value, mf.value, ppc.value


def render_shade_pass(depth: np.ndarray, thickness: np.ndarray, uniforms_f32: np.ndarray,
                      env: np.ndarray) -> np.ndarray:
    """The renderer's shading pass alone over filtered (H, W) depth and
    thickness images: (H, W, 4) float32 colour."""
    L = _render_lib()
    d = np.ascontiguousarray(depth, dtype=np.float32)
    t = np.ascontiguousarray(thickness, dtype=np.float32)
    h, w = d.shape
    u = np.ascontiguousarray(uniforms_f32, dtype=np.float32).reshape(68)
    e = np.ascontiguousarray(env, dtype=np.float32)
    color = np.zeros((h, w, 4), np.float32)
    color8 = np.zeros((h, w, 4), np.uint8)
    L.ro_shade_pass(d, t, u, e, e.shape[1], w, h, color, color8)
    return color


def sample_cube(env: np.ndarray, direction) -> np.ndarray:
    """The shading pass's cube-map lookup for one direction: rgb float32."""
    L = _render_lib()
    e = np.ascontiguousarray(env, dtype=np.float32)
    out = np.zeros(3, np.float32)
    L.ro_sample_cube(e, e.shape[1], float(direction[0]), float(direction[1]),
                     float(direction[2]), out)
    return out


def render_filter_pass(kind: str, img: np.ndarray, direction, depth_threshold: float = 0.0,
                       max_filter_size: float = 0.0, ppc: float = 0.0) -> np.ndarray:
    """One pass of the renderer's bilateral depth filter or gaussian thickness
    filter over an (H, W) float32 image along direction (1, 0) or (0, 1)."""
    L = _render_lib()
    src = np.ascontiguousarray(img, dtype=np.float32)
    h, w = src.shape
    dst = np.zeros_like(src)
    dx, dy = (int(direction[0]), int(direction[1]))
    if kind == "bilateral":
        L.ro_bilateral_pass(src, dst, w, h, dx, dy, depth_threshold, max_filter_size, ppc)
    elif kind == "gaussian":
        L.ro_gaussian_pass(src, dst, w, h, dx, dy)
    else:
        raise ValueError(kind)
    return dst


# ---------------------------------------------------------------------------
# SPH (sph_oracle.c)
# ---------------------------------------------------------------------------

def sph_execute(records: np.ndarray, real_half, substeps: int = 2):
    """Runs `substeps` SPH substeps on (n, 16) float32 records; returns
    (records, posvel (n, 8))."""
    L = lib()
    if not getattr(L, "_so_ready", False):
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        L.so_execute.argtypes = [f32p, ctypes.c_int64, ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                                 f32p]
        L.so_execute.restype = ctypes.c_int
        L.so_grid_count.restype = ctypes.c_int
        L._so_ready = True
    rec = np.ascontiguousarray(records, dtype=np.float32).reshape(-1, 16).copy()
    pv = np.zeros((max(len(rec), 1), 8), np.float32)
    half = (ctypes.c_float * 3)(*[float(np.float32(h)) for h in real_half])
    if L.so_execute(rec, len(rec), half, int(substeps), pv) != 0:
        raise MemoryError("so_execute")
    return rec, pv[:len(rec)]


def sph_grid_count() -> int:
    sph_execute(np.zeros((0, 16), np.float32), [1, 1, 1], 0)
    return int(lib().so_grid_count())
