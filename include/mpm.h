/*
 * mpm.h -- C ABI of libmpm.so, a GB300 (sm_103a) MLS-MPM fluid solver that
 * drops in for WebGPU-Ocean's MLSMPMSimulator (mls-mpm/mls-mpm.ts:12-276).
 *
 * Conventions
 *   - Every function returns MPM_OK (0) or a negative MPM_E_* code; no C++
 *     exception crosses the ABI.  mpm_last_error() gives a message for the
 *     last failing call on the calling thread.
 *   - The library owns its device state; handles are opaque.  A handle lives
 *     on the CUDA device that was current when it was created; every call
 *     switches to that device and restores the caller's device on return.
 *   - One handle serves one host thread at a time (the reference runs on a
 *     single-threaded JS event loop).  Calls that take a `stream` enqueue
 *     work on that cudaStream_t (NULL = the legacy default stream) and return
 *     without waiting, like WebGPU command submission.
 *   - Layouts are the reference's own:
 *       particle  80 B = pos vec3f @0, v vec3f @16, C mat3x3f @32 (three
 *                 16-byte columns)          mls-mpm/mls-mpm.ts:10,204-209
 *       cell      16 B = i32 vx, vy, vz, mass  mls-mpm/p2g_1.wgsl:6-11
 *       posvel    32 B = pos vec3f @0, v vec3f @16  copyPosition.wgsl:7-10
 */
#ifndef GB300_MPM_H
#define GB300_MPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpm_sim mpm_sim;

/* Pipeline override constants, mls-mpm/mls-mpm.ts:53-59. */
typedef struct mpm_params {
    float stiffness;              /* 3.0  */
    float rest_density;           /* 4.0  */
    float dynamic_viscosity;      /* 0.1  */
    float dt;                     /* 0.2  */
    float fixed_point_multiplier; /* 1e7  */
} mpm_params;

enum {
    MPM_OK = 0,
    MPM_E_INVALID = -1,       /* null handle or pointer, negative size, bad enum */
    MPM_E_CAPACITY = -2,      /* more particles than max_particles */
    MPM_E_GRID_CAPACITY = -3, /* gridCount > max grid (mls-mpm/mls-mpm.ts:230-232) */
    MPM_E_CUDA = -4,          /* a CUDA runtime call failed */
    MPM_E_NO_DEVICE = -5,     /* no CUDA device */
    MPM_E_STATE = -6,         /* no scene loaded yet */
    MPM_E_NONFINITE = -7      /* watchdog: non-finite particle state */
};

/* Engines.  Both give bit-identical results. */
enum {
    MPM_ENGINE_SORTED = 0,   /* default: binned particles, fused stages */
    MPM_ENGINE_DISPATCH = 1  /* one kernel per WGSL entry point, as the reference */
};

/* The six WGSL entry points, in the order execute() dispatches them
 * (mls-mpm/mls-mpm.ts:248-265). */
enum {
    MPM_KERNEL_CLEAR_GRID = 0,    /* mls-mpm/clearGrid.wgsl:10    */
    MPM_KERNEL_P2G_1 = 1,         /* mls-mpm/p2g_1.wgsl:24        */
    MPM_KERNEL_P2G_2 = 2,         /* mls-mpm/p2g_2.wgsl:30        */
    MPM_KERNEL_UPDATE_GRID = 3,   /* mls-mpm/updateGrid.wgsl:23   */
    MPM_KERNEL_G2P = 4,           /* mls-mpm/g2p.wgsl:26          */
    MPM_KERNEL_COPY_POSITION = 5  /* mls-mpm/copyPosition.wgsl:15 */
};

/* Fills the reference's constants (mls-mpm/mls-mpm.ts:53-59). */
void mpm_default_params(mpm_params* out);

/*
 * Replaces `new MLSMPMSimulator(particleBuffer, posvelBuffer, renderDiameter,
 * device)` (mls-mpm/mls-mpm.ts:42-193).  `params` NULL = the reference's
 * constants.  The grid capacity generalises the fixed 64^3 cell buffer
 * (mls-mpm.ts:13-15,122-130); `max_particles` generalises numParticlesMax
 * (common.ts:11).  `posvel_device` is the caller-owned posvelBuffer
 * (main.ts:115-119): a device pointer of at least 32*max_particles bytes
 * (`posvel_bytes`), or NULL to let the library allocate it.  The particle
 * state itself is library-owned (mpm_download_particles gives it back in the
 * 80-byte layout).  `render_diameter` is kept for the renderer hand-off
 * (reset() copies it to sphere_size, mls-mpm.ts:226).
 */
int mpm_create(const mpm_params* params, int max_particles, int max_grid_x, int max_grid_y,
               int max_grid_z, float render_diameter, void* posvel_device, size_t posvel_bytes,
               mpm_sim** out);
int mpm_destroy(mpm_sim* sim);

/*
 * Replaces reset(numParticles, initBoxSize) (mls-mpm/mls-mpm.ts:225-243):
 * builds the dam-break block of initDambreak (mls-mpm.ts:195-223) with
 * Math.random replaced by SplitMix64(seed), uploads it and sets both box
 * uniforms to init_box.  init_box is given in doubles because the reference's
 * loop bounds are JS numbers.  Returns MPM_E_GRID_CAPACITY (the reference's
 * throw) when ceil(X)*ceil(Y)*ceil(Z) exceeds the grid capacity.
 */
int mpm_reset_dambreak(mpm_sim* sim, int num_particles, const double init_box[3],
                       uint64_t seed);

/* Loads n particles in the reference's 80-byte layout (host memory) and sets
 * both box uniforms to init_box (the writeBuffer calls of mls-mpm.ts:239-241). */
int mpm_upload(mpm_sim* sim, const float* particles_aos80, int n, const float init_box[3]);

/* Replaces execute(commandEncoder) (mls-mpm/mls-mpm.ts:245-268): enqueues
 * `substeps` substeps (the reference runs 2) on `stream`; ends with posvel
 * holding the particles' positions and velocities. */
int mpm_step(mpm_sim* sim, int substeps, void* stream);

/* Replaces changeBoxSize(realBoxSize) (mls-mpm/mls-mpm.ts:270-275).  Takes
 * effect for work enqueued after the call. */
int mpm_set_real_box(mpm_sim* sim, const float real_box[3]);

/* The numParticles and gridCount fields (mls-mpm/mls-mpm.ts:19-20). */
int mpm_num_particles(const mpm_sim* sim);
int64_t mpm_grid_count(const mpm_sim* sim);
float mpm_render_diameter(const mpm_sim* sim);

/* posvelBuffer (main.ts:115-119): device pointer, 32 B per particle. */
void* mpm_posvel_device_ptr(mpm_sim* sim);

/* Synchronous copies back to host memory (for parity checks and tools). */
int mpm_download_particles(mpm_sim* sim, float* out_aos80);
int mpm_download_grid(mpm_sim* sim, int32_t* out_cells);
/* Asynchronous on `stream`: copies n*32 B of posvel into host memory
 * (pinned memory makes it truly asynchronous). */
int mpm_download_posvel(mpm_sim* sim, float* out_posvel, void* stream);
/* Pipelined read-back for a frame loop (no counterpart in the reference,
 * whose renderer reads posvel on the GPU): snapshots posvel on `stream` (a
 * device-to-device copy) and copies the snapshot into `out_posvel` (pinned
 * host memory) on the library's own copy stream, so the next mpm_execute on
 * `stream` overlaps the transfer.  `out_posvel` holds the posvel of the call
 * once mpm_wait_posvel returns. */
int mpm_download_posvel_async(mpm_sim* sim, float* out_posvel, void* stream);
/* Waits for the last mpm_download_posvel_async copy: on the host when
 * `stream` is NULL, else makes `stream` wait for it. */
int mpm_wait_posvel(mpm_sim* sim, void* stream);

/* Enqueues one WGSL entry point alone (mls-mpm/mls-mpm.ts:248-265) on the
 * dispatch engine's state.  Running the six in order equals one substep. */
int mpm_dispatch(mpm_sim* sim, int kernel, void* stream);

int mpm_set_engine(mpm_sim* sim, int engine);
int mpm_get_engine(const mpm_sim* sim);

/* Waits for all work of the handle (its streams and the legacy stream). */
int mpm_synchronize(mpm_sim* sim);

/* Watchdog (the reference only reports device loss, main.ts:185-188):
 * counts non-finite particle records and grid accesses that fell outside
 * [0, gridCount) since the last reset.  Synchronous. */
typedef struct mpm_health {
    int64_t nonfinite_particles;
    int64_t out_of_range_accesses;
} mpm_health;
int mpm_check_health(mpm_sim* sim, mpm_health* out);

/* Launch accounting (the reference only times JS encoding with
 * performance.now(), main.ts:209,278).  mpm_set_profiling(1) starts
 * bracketing every kernel with CUDA events on its launch stream and resets
 * the counters; mpm_kernel_stats waits for those events and fills up to
 * max_entries records, returning how many kernels have records.
 * mpm_launch_count is the number of kernels this handle has launched. */
typedef struct mpm_kernel_stat {
    const char* name;
    int64_t launches;
    int64_t timed_launches;
    double total_ms;
} mpm_kernel_stat;
int mpm_set_profiling(mpm_sim* sim, int enable);
int mpm_kernel_stats(mpm_sim* sim, mpm_kernel_stat* out, int max_entries);
int64_t mpm_launch_count(const mpm_sim* sim);

const char* mpm_error_string(int code);
const char* mpm_last_error(void);

/* Host-only scene builders (no GPU).  Each returns the particle count or a
 * negative code.
 * mpm_scene_dambreak: initDambreak (mls-mpm/mls-mpm.ts:195-223) with
 *   Math.random -> SplitMix64(seed); writes at most max_particles records.
 * mpm_scene_lattice: jittered cubic lattice, particle (ix,iy,iz) x-major at
 *   origin + spacing*i plus per-component jitter U[-jitter, jitter). */
int mpm_scene_dambreak(float* out_aos80, int max_particles, const double init_box[3],
                       uint64_t seed);
int mpm_scene_lattice(float* out_aos80, int n_per_axis, double origin, double spacing,
                      double jitter, uint64_t seed);

/* Diagnostic: evaluates the fixed-point conversions on the device.
 * enc_out[i] = i32(in[i] * fm) (p2g_1.wgsl:15-17), dec_out[i] =
 * f32(bits(in[i])) / fm (p2g_2.wgsl:22-24).  Synchronous, host arrays. */
int mpm_probe_conversions(const float* in, int n, float fm, int32_t* enc_out, float* dec_out);

/* Diagnostic: the packed f32x2 multiply and add the kernels use, against
 * the scalar IEEE operations.  n (even) floats in a and b; out holds 6n
 * floats: packed a*b, a+b, (a*b)+a, then scalar a*b, a+b, (a*b)+a (each
 * product rounded before the add).  Synchronous. */
int mpm_probe_packed(const float* a, const float* b, int n, float* out);

/* ------------------------------------------------------------------ */
/* Extensions beyond the reference's class                             */
/* ------------------------------------------------------------------ */

/* Body force (per unit time) added in updateGrid.  The reference hardcodes
 * (0, -0.3, 0) (mls-mpm/updateGrid.wgsl:34), the default; components that
 * are 0 are left untouched, so that default is bit-identical to it. */
int mpm_set_gravity(mpm_sim* sim, const float gravity[3]);

/* 1 (the default): mpm_step on the sorted engine runs its substeps as one
 * CUDA graph, captured on first use for each substep count and engine state
 * and recaptured after a change of constants (a changeBoxSize to a new
 * value); measured +3 % at 1M particles and +30 % at 64k.  0: plain
 * launches (also used while mpm_set_profiling times kernels). */
int mpm_set_graph(mpm_sim* sim, int enable);

/* Sorted engine: most particles per task.  A bin (4x4x4-cell brick) with
 * more particles is split into several tasks, so that small scenes still
 * spread over every SM.  0 (the default) picks it from the particle count:
 * particles per resident task-kernel block, rounded to the nearest power of
 * two within 64 ... 1024; otherwise 64 ... 2^30.  Results do not depend on
 * it. */
int mpm_set_task_size(mpm_sim* sim, int task_size);
int mpm_get_task_size(const mpm_sim* sim);
/* Sorted engine: tasks of at least `min_particles` particles spread them over
 * the warp lanes by shared-memory bank class before p2g_2 (the lane table:
 * fewer bank conflicts on the arena atomics, at the price of its barriers
 * and position loads); smaller tasks keep the bin order.  0 restores the
 * default (128); a value above 1024 turns the table off.  Results do not
 * depend on it. */
int mpm_set_lane_table_min(mpm_sim* sim, int min_particles);
int mpm_get_lane_table_min(const mpm_sim* sim);
/* Sorted engine: threads per block of its two task kernels (p2g_2; g2p with
 * the next p2g_1), the generalisation of the reference's
 * @workgroup_size(64) (mls-mpm/p2g_1.wgsl:24): 128, 256 (the default) or
 * 512; 0 restores the default.  A task is processed in chunks of this many
 * particles.  Results do not depend on it. */
int mpm_set_task_threads(mpm_sim* sim, int threads);
int mpm_get_task_threads(const mpm_sim* sim);
/* Sorted engine: the sort bins are 4x4x4-cell bricks; the bins of two bricks
 * stacked along z (an aligned pair) whose particles together number at most
 * `max_particles` (and at most the task size) form one task of 4x4x8 cells
 * with arenas four cells deeper, so that sparse bricks share a task's fixed
 * costs.  0 never pairs; 2^30 pairs every pair whose two bins hold
 * particles (4x4x8-cell bins throughout); INT_MAX restores the default,
 * 512.  Results do not depend on it. */
int mpm_set_bin_pairing(mpm_sim* sim, int max_particles);
int mpm_get_bin_pairing(const mpm_sim* sim);
/* Autotuner: times `substeps` substeps for each z-pair threshold in {0,
 * 256, 512, 2^30}, each task-kernel block size in {128, 256, 512}, each task
 * size in {128, 256, 512, 1024} and each lane-table threshold in {32, 128,
 * 512, off} from the current state (each combination once untimed first, so
 * its CUDA graphs are captured outside the timing), keeps the fastest and
 * restores the state (particles, posvel, counters and grid are as before
 * the call).  Writes the task size to *chosen_task_size when non-null (the
 * others: mpm_get_bin_pairing, mpm_get_task_threads,
 * mpm_get_lane_table_min).  Synchronizes. */
int mpm_autotune(mpm_sim* sim, int substeps, int* chosen_task_size);

/* Batches: many independent scenes that advance together, one launch per
 * stage for all of them (the sorted engine over the scenes' concatenated
 * particles, bricks and bins), replayed as a CUDA graph.  Each scene gives
 * the same results, bit for bit, as an mpm_sim holding it alone with the
 * same constants. */
typedef struct mpm_batch mpm_batch;

typedef struct mpm_scene_desc {
    int num_particles;            /* this scene's records in the particle array */
    float init_box[3];            /* reset()'s initBoxSize: grid extent, flat indices */
    float real_box[3];            /* changeBoxSize()'s realBoxSize: walls, clamp */
    float stiffness;              /* mpm_params fields, per scene */
    float rest_density;
    float dynamic_viscosity;
    float dt;
    float fixed_point_multiplier;
    float gravity[3];             /* see mpm_set_gravity */
} mpm_scene_desc;

/* Scene s's particles are records [sum of earlier num_particles, + its own)
 * of aos80 (80-byte records).  Grids must be non-degenerate
 * (i32(init_box.y), i32(init_box.z) >= 1). */
int mpm_batch_create(const mpm_scene_desc* scenes, int num_scenes, const float* aos80,
                     mpm_batch** out);
int mpm_batch_destroy(mpm_batch* batch);
int mpm_batch_num_scenes(const mpm_batch* batch);
int64_t mpm_batch_num_particles(const mpm_batch* batch);
/* `substeps` substeps of every scene; asynchronous on `stream`. */
int mpm_batch_step(mpm_batch* batch, int substeps, void* stream);
/* Replaces every scene's particles (same counts and order as at creation)
 * and restarts the scenes from them, as a fresh mpm_batch_create would;
 * captured graphs are kept (synchronizes). */
int mpm_batch_upload(mpm_batch* batch, const float* aos80);
/* Replaces scene s's constants (box sizes and num_particles must stay). */
int mpm_batch_set_scene(mpm_batch* batch, int scene, const mpm_scene_desc* desc);
int mpm_batch_set_graph(mpm_batch* batch, int enable); /* default 1 */
int mpm_batch_set_task_size(mpm_batch* batch, int task_size); /* see mpm_set_task_size */
int mpm_batch_get_task_size(const mpm_batch* batch);
int mpm_batch_set_lane_table_min(mpm_batch* batch, int min_particles); /* see mpm_set_lane_table_min */
int mpm_batch_get_lane_table_min(const mpm_batch* batch);
int mpm_batch_set_task_threads(mpm_batch* batch, int threads); /* see mpm_set_task_threads */
int mpm_batch_get_task_threads(const mpm_batch* batch);
int mpm_batch_set_bin_pairing(mpm_batch* batch, int max_particles); /* see mpm_set_bin_pairing */
int mpm_batch_get_bin_pairing(const mpm_batch* batch);
/* See mpm_autotune: the batch's particles and posvel are as before the call;
 * mpm_batch_download_grid returns zeros until the next step. */
int mpm_batch_autotune(mpm_batch* batch, int substeps, int* chosen_task_size);
/* All scenes' particles, in input order (synchronizes). */
int mpm_batch_download_particles(mpm_batch* batch, float* out_aos80);
/* Scene s's grid after its last updateGrid, reference layout (synchronizes). */
int mpm_batch_download_grid(mpm_batch* batch, int scene, int32_t* out_cells);
/* 32-byte posvel records of all particles, written by each step's last substep. */
void* mpm_batch_posvel_device_ptr(mpm_batch* batch);
int mpm_batch_check_health(mpm_batch* batch, mpm_health* out);
int64_t mpm_batch_launch_count(const mpm_batch* batch);
int mpm_batch_set_profiling(mpm_batch* batch, int enable);   /* see mpm_set_profiling */
int mpm_batch_kernel_stats(mpm_batch* batch, mpm_kernel_stat* out, int max_entries);

/* Differentiation: a forward / backward pair over a batch of scenes (one
 * scene for a single simulation).  The derivative is that of the continuous
 * model the fixed-point solver discretises (enc/dec taken as the identity),
 * evaluated along the solver's own trajectory.  mpm_forward_ckpt runs the
 * solver and keeps the state every `checkpoint_every` substeps; mpm_backward
 * recomputes each segment from its checkpoint (states and updated grids of
 * every substep) and runs the adjoint substeps in reverse; when max_substeps
 * > checkpoint_every it keeps two segment tapes (2 x checkpoint_every states
 * and grids) and recomputes segment j - 1 on a second stream while it
 * differentiates segment j.  checkpoint_every = 1 keeps every substep's state
 * and updated grid (max_substeps grids of device memory) and the backward
 * recomputes nothing. */
typedef struct mpm_adjoint mpm_adjoint;

/* Tapes (the trajectory the derivative is evaluated along):
 *   MPM_TAPE_FP64        the continuous model integrated in FP64 on the GPU
 *                        (double grid sums, no fixed point): its trajectory
 *                        tracks an FP64 reference over hundreds of substeps,
 *                        so gradients match FP64 finite differences (default)
 *   MPM_TAPE_FIXED_POINT the solver's own bit-exact fixed-point trajectory
 *                        (sorted engine); over long horizons it drifts from
 *                        the continuous model by the i32 truncation bias */
enum { MPM_TAPE_FIXED_POINT = 0, MPM_TAPE_FP64 = 1 };

int mpm_adjoint_create(const mpm_scene_desc* scenes, int num_scenes, int max_substeps,
                       int checkpoint_every, mpm_adjoint** out);
int mpm_adjoint_destroy(mpm_adjoint* adj);
/* Selects the tape (invalidates the forward). */
int mpm_adjoint_set_tape(mpm_adjoint* adj, int tape);
/* New constants for scene s (e.g. stiffness, viscosity between optimizer
 * steps); box sizes and num_particles must stay.  Invalidates the forward. */
int mpm_adjoint_set_scene(mpm_adjoint* adj, int scene, const mpm_scene_desc* desc);
/* Runs `substeps` substeps from init_aos80 (all scenes' 80-byte records). */
int mpm_forward_ckpt(mpm_adjoint* adj, const float* init_aos80, int substeps, void* stream);
/* The state after `substep` substeps of the last forward; substep must be a
 * multiple of checkpoint_every or the final substep (synchronizes). */
int mpm_adjoint_state(mpm_adjoint* adj, int substep, float* out_aos80);
/* seeds_aos80: num_seeds blocks of 80-byte records, block j = dL/d(state
 * after seed_substeps[j] substeps) (fields as in the particle record: position,
 * velocity, C).  Writes dL/d(initial state) to grad_init_aos80 and, per scene,
 * (dL/d stiffness, dL/d dynamic_viscosity) to grad_params[2 * s + 0/1]
 * (synchronizes). */
int mpm_backward(mpm_adjoint* adj, const float* seeds_aos80, const int* seed_substeps,
                 int num_seeds, float* grad_init_aos80, double* grad_params, void* stream);
/* The same with one pointer per seed block (no contiguous array of all
 * seeds needed). */
int mpm_backward_list(mpm_adjoint* adj, const float* const* seeds_aos80, const int* seed_substeps,
                      int num_seeds, float* grad_init_aos80, double* grad_params, void* stream);

/* Position observations for inverse problems, computed on the device so the
 * states and seeds never leave it.  mpm_adjoint_set_observations replaces
 * the observations: `count` blocks of n x 3 floats (positions in particle
 * order), block j observed after substeps[j] substeps.  After a forward,
 * mpm_adjoint_observation_loss writes per scene s
 *   loss[s] = sum_j (1 / n_s) sum_{i in s} |x_i(substeps[j]) - obs_j,i|^2
 * (FP64 sums of f32 differences; the observed substeps must be checkpoints
 * of that forward) and keeps the seeds dL/dx = f32(2 / n_s) * (x - obs) on
 * the device; mpm_backward_observed then runs mpm_backward with them.
 * Both synchronize. */
int mpm_adjoint_set_observations(mpm_adjoint* adj, int count, const int* substeps,
                                 const float* const* obs_xyz);
int mpm_adjoint_observation_loss(mpm_adjoint* adj, double* loss_per_scene, void* stream);
int mpm_backward_observed(mpm_adjoint* adj, float* grad_init_aos80, double* grad_params,
                          void* stream);

/* Headless screen-space renderer (render/fluidRender.ts, fluid path):
 * depth splat, 4 x bilateral filter, thickness splat, gaussian filter and
 * shading, from the posvel records the simulator writes, into an image in
 * device memory.  No window, swap chain or graphics API: the output is a
 * device buffer (RGBA float or 8-bit). */
typedef struct mpm_renderer mpm_renderer;

/* RenderUniforms (common.ts:1-9, 272 bytes): 4x4 matrices by columns. */
typedef struct mpm_render_uniforms {
    float texel_size[2];      /* 1 / width, 1 / height */
    float sphere_size;        /* billboard size (the simulator's render diameter) */
    float pad;
    float inv_projection_matrix[16];
    float projection_matrix[16];
    float view_matrix[16];
    float inv_view_matrix[16];
} mpm_render_uniforms;

enum {
    MPM_RENDER_COLOR = 0,     /* width*height float4, rows top to bottom */
    MPM_RENDER_COLOR8 = 1,    /* width*height RGBA8 */
    MPM_RENDER_DEPTH = 2,     /* filtered depth map, float */
    MPM_RENDER_THICKNESS = 3  /* filtered thickness map, float (r16float values) */
};

/* FluidRenderer constructor (fluidRender.ts:34-46): image size, particle
 * radius and vertical field of view (radians) set the filter constants.  The
 * environment map starts as a built-in sky gradient. */
int mpm_renderer_create(int width, int height, float radius, float fov, mpm_renderer** out);
int mpm_renderer_destroy(mpm_renderer* renderer);
/* Cube map faces +x, -x, +y, -y, +z, -z, each face_size^2 RGBA floats. */
int mpm_renderer_set_envmap(mpm_renderer* renderer, int face_size, const float* rgba);
/* FluidRenderer.execute (fluidRender.ts:292-488, sphereRenderFl false):
 * posvel_device = 32-byte records (mpm_posvel_device_ptr), asynchronous. */
int mpm_renderer_execute(mpm_renderer* renderer, const void* posvel_device, int num_particles,
                         const mpm_render_uniforms* uniforms, void* stream);
/* FluidRenderer.execute with sphereRenderFl true (fluidRender.ts:481-485,
 * render/sphere.wgsl): every particle's billboard drawn as a lit sphere
 * coloured by its speed, depth test 'less', over the clear colour
 * (0.8, 0.8, 0.8, 1).  MPM_RENDER_COLOR / _COLOR8 then hold the image and
 * MPM_RENDER_DEPTH the winning fragment depth (1 where none). */
int mpm_renderer_execute_spheres(mpm_renderer* renderer, const void* posvel_device,
                                 int num_particles, const mpm_render_uniforms* uniforms,
                                 void* stream);
/* Copies one of the MPM_RENDER_* images to host memory (synchronizes). */
int mpm_renderer_download(mpm_renderer* renderer, int what, void* out);
void* mpm_renderer_color_device_ptr(mpm_renderer* renderer);

/* The reference's second simulator, SPHSimulator (sph/sph.ts), behind the
 * same four methods.  Particle records are the reference's 64 bytes:
 * position vec3f @0, v vec3f @16, force vec3f @32, density f32 @44,
 * nearDensity f32 @48 (sph.ts:13,205-211).  Box sizes are HALF sizes, as
 * SPHSimulator.reset/changeBoxSize take them. */
typedef struct mpm_sph mpm_sph;

/* constructor(particleBuffer, posvelBuffer, renderDiameter, device), sph.ts:46 */
int mpm_sph_create(int max_particles, float render_diameter, void* posvel_device,
                   size_t posvel_bytes, mpm_sph** out);
int mpm_sph_destroy(mpm_sph* sph);
/* reset(numParticles, initHalfBoxSize), sph.ts:300-316 (initDambreak with
 * Math.random -> SplitMix64(seed)) */
int mpm_sph_reset_dambreak(mpm_sph* sph, int num_particles, const double init_half_box[3],
                           uint64_t seed);
int mpm_sph_upload(mpm_sph* sph, const float* rec64, int n, const float real_half_box[3]);
/* execute(commandEncoder), sph.ts:318-356: `substeps` (2 per frame) */
int mpm_sph_step(mpm_sph* sph, int substeps, void* stream);
/* Frames replay as CUDA graphs (captured once per substep and particle
 * count); 0 launches every kernel each frame.  Results are the same. */
int mpm_sph_set_graph(mpm_sph* sph, int enable); /* default 1 */
/* Up to max_particles particles, density and forces run one warp per
 * particle (the lanes share the neighbour terms; the sums keep the
 * one-thread order, so the results do not change); above it, one thread per
 * particle.  Default 32768; 0: always a thread per particle; -1: the
 * default. */
int mpm_sph_set_warp_per_particle(mpm_sph* sph, int max_particles);
int mpm_sph_get_warp_per_particle(const mpm_sph* sph);
/* changeBoxSize(realBoxSize), sph.ts:383-388 (half sizes) */
int mpm_sph_set_real_box(mpm_sph* sph, const float real_half_box[3]);
int mpm_sph_num_particles(const mpm_sph* sph);
int64_t mpm_sph_grid_count(const mpm_sph* sph);
void* mpm_sph_posvel_device_ptr(mpm_sph* sph);
/* All particle records / posvel records (synchronize). */
int mpm_sph_download_particles(mpm_sph* sph, float* out_rec64);
int mpm_sph_download_posvel(mpm_sph* sph, float* out_posvel);
/* initDambreak alone, into host memory; returns the record count. */
int mpm_sph_scene_dambreak(float* out_rec64, int num_particles, const double init_half_box[3],
                           uint64_t seed);

/*
 * No counterpart in the reference.  The watchdog scan of mpm_check_health
 * over a caller-owned device buffer, allocating nothing: for callers that
 * cannot call cudaMalloc, such as a host stepping the solver from its
 * per-frame loop (cudaMalloc/cudaFree may synchronize the device and take
 * unbounded time) or a plugin host that owns all device memory.  Counts the
 * records among n (each stride_floats floats, 20 for the 80-byte particle
 * layout) that hold a non-finite value and writes the count to *count_out
 * (device memory), asynchronously on `stream`, on the current device.  With
 * stride_floats == 20 the 16 state floats of each record are checked, as
 * mpm_check_health does, and the five padding floats (3, 7, 11, 15, 19) are
 * skipped; with any other stride every float is checked.
 * Limit: n <= 16,777,216 records; larger n returns MPM_E_CAPACITY.
 * Scratch: a fixed 512 KiB device array inside the library, which every GPU
 * that loads the library holds until exit.  Every call looks up that
 * array's device address in the current context (cudaGetSymbolAddress,
 * which allocates nothing); the first call on a device may load the
 * library's device code, so make it before any stream capture.
 * All calls share the array: calls that overlap on the GPU race.
 */
int mpm_count_nonfinite_noalloc(const float* records, int stride_floats, int n,
                                int64_t* count_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GB300_MPM_H */
