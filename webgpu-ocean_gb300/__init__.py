"""GB300-native MLS-MPM solver: a drop-in for WebGPU-Ocean's MLSMPMSimulator
(mls-mpm/mls-mpm.ts).  The compute path is libmpm.so (csrc/, C ABI in
include/mpm.h); this package is its Python host mirror.

The directory name is not a Python identifier; load it with
`load_package()` from the repository root helpers, which registers it as
`webgpu_ocean_gb300`.
"""
from . import _lib, build
from .mlsmpm import (MLSMPMAdjoint, MLSMPMBatch, MLSMPMSimulator, MPMError, GridCapacityError,
                     batch_scenes, centroid_loss, default_params, probe_conversions, probe_packed,
                     scene_dambreak, scene_desc, scene_lattice)

from . import inverse, render, sph
from .sph import SPHSimulator, sph_scene_dambreak
from .render import FluidRenderer, camera_uniforms

__all__ = ["SPHSimulator", "sph_scene_dambreak", "sph", "FluidRenderer", "camera_uniforms", "render", "MLSMPMSimulator", "MLSMPMBatch", "MLSMPMAdjoint", "centroid_loss", "inverse",
           "MPMError", "GridCapacityError", "default_params", "scene_dambreak", "scene_lattice", "scene_desc", "batch_scenes", "probe_conversions",
           "probe_packed", "build", "_lib"]
