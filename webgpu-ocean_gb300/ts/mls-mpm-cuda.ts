// mls-mpm-cuda.ts -- drop-in replacement for MLSMPMSimulator
// (mls-mpm/mls-mpm.ts:12-276) that drives libmpm.so through its C ABI
// (include/mpm.h) from Node with the koffi FFI module.
//
// Same constructor parameters, the same reset-to-initial-box, the same
// per-frame execute() with two substeps, changeBoxSize(), numParticles and
// gridCount, and the same 32-byte posvel records handed to the renderer
// (as a device pointer).  main.ts changes only where it constructs the
// simulator (main.ts:141) and where the renderer reads posvel.
//
// This file is not run in this repository's build (no Node runtime there);
// the same C ABI is exercised from Python by every test.
import koffi from 'koffi';

const lib = koffi.load(process.env.LIBMPM_PATH ?? 'libmpm.so');

// mpm_params (include/mpm.h): the pipeline constants of mls-mpm.ts:53-59.
const MpmParams = koffi.struct('mpm_params', {
  stiffness: 'float',
  rest_density: 'float',
  dynamic_viscosity: 'float',
  dt: 'float',
  fixed_point_multiplier: 'float',
});

const mpm_create = lib.func(
  'int mpm_create(const mpm_params* params, int max_particles, int max_grid_x, ' +
  'int max_grid_y, int max_grid_z, float render_diameter, void* posvel_device, ' +
  'size_t posvel_bytes, _Out_ void** out)');
const mpm_destroy = lib.func('int mpm_destroy(void* sim)');
const mpm_reset_dambreak = lib.func(
  'int mpm_reset_dambreak(void* sim, int num_particles, const double* init_box, uint64_t seed)');
const mpm_step = lib.func('int mpm_step(void* sim, int substeps, void* stream)');
const mpm_set_real_box = lib.func('int mpm_set_real_box(void* sim, const float* real_box)');
const mpm_num_particles = lib.func('int mpm_num_particles(void* sim)');
const mpm_grid_count = lib.func('int64_t mpm_grid_count(void* sim)');
const mpm_posvel_device_ptr = lib.func('void* mpm_posvel_device_ptr(void* sim)');
const mpm_last_error = lib.func('const char* mpm_last_error()');

const MPM_E_GRID_CAPACITY = -3;

export interface RenderUniformViews {
  sphere_size: Float32Array;
}

export class MLSMPMSimulator {
  // mls-mpm.ts:13-15: the grid capacity the constructor sizes its cell buffer for.
  max_x_grids = 64;
  max_y_grids = 64;
  max_z_grids = 64;
  numParticlesMax = 200000;  // common.ts:11

  renderDiameter: number;
  private sim: unknown;
  private uniformViews: RenderUniformViews | null;

  // mls-mpm.ts:42.  The reference takes the app's particleBuffer and
  // posvelBuffer (GPUBuffers) and its GPUDevice; here the library owns the
  // particle state, posvelDevicePtr (optional) is a caller-owned CUDA
  // allocation of 32 * numParticlesMax bytes, and the current CUDA device is
  // used.
  constructor(posvelDevicePtr: unknown | null, renderDiameter: number,
              uniformViews: RenderUniformViews | null = null) {
    this.renderDiameter = renderDiameter;
    this.uniformViews = uniformViews;
    const out: unknown[] = [null];
    const rc = mpm_create(null, this.numParticlesMax, this.max_x_grids, this.max_y_grids,
                          this.max_z_grids, renderDiameter, posvelDevicePtr,
                          posvelDevicePtr ? 32 * this.numParticlesMax : 0, out);
    if (rc !== 0) throw new Error(mpm_last_error());
    this.sim = out[0];
  }

  // mls-mpm.ts:19-20
  get numParticles(): number { return mpm_num_particles(this.sim); }
  get gridCount(): number { return Number(mpm_grid_count(this.sim)); }

  // mls-mpm.ts:225-243: initDambreak + box uniforms + upload.  Math.random
  // becomes the library's seeded generator (the seed is the only change).
  reset(numParticles: number, initBoxSize: number[], seed: bigint = BigInt(Date.now())) {
    if (this.uniformViews) this.uniformViews.sphere_size.set([this.renderDiameter]);
    const rc = mpm_reset_dambreak(this.sim, numParticles, new Float64Array(initBoxSize), seed);
    if (rc === MPM_E_GRID_CAPACITY)
      throw new Error('gridCount should be equal to or less than maxGridCount');
    if (rc !== 0) throw new Error(mpm_last_error());
  }

  // mls-mpm.ts:245-268: two substeps of the six stages, asynchronous on
  // `stream` (a cudaStream_t, or null for the legacy stream) instead of a
  // GPUCommandEncoder.
  execute(stream: unknown = null) {
    if (mpm_step(this.sim, 2, stream) !== 0) throw new Error(mpm_last_error());
  }

  // mls-mpm.ts:270-275
  changeBoxSize(realBoxSize: number[]) {
    if (mpm_set_real_box(this.sim, new Float32Array(realBoxSize)) !== 0)
      throw new Error(mpm_last_error());
  }

  // posvelBuffer (main.ts:115-119): the renderer's input, 32-byte records.
  posvelDevicePtr(): unknown { return mpm_posvel_device_ptr(this.sim); }

  dispose() { mpm_destroy(this.sim); }
}
