// sorted_engine.h -- the binned, fused MLS-MPM engine (kernels_sorted.cu).
#pragma once
#include <cuda_runtime.h>

#include "mpm_internal.h"

namespace mpm {

struct SortedEngine;

// Allocates the per-particle sort arrays; grids are sized at configure().
int sorted_create(SortedEngine** out, int max_particles);
void sorted_destroy(SortedEngine* e);

// Sizes the brick grid for a scene (box, grid_count).  Returns 0, or -1 when
// the box is degenerate (i32(Y) or i32(Z) == 0), in which case the caller
// must use the dispatch engine.
int sorted_configure(SortedEngine* e, const SimConsts& k);

// Sizes the engine for a batch of independent scenes (ks[s].n particles of
// scene s, stored after those of scenes 0..s-1).  Returns -1 when a box is
// degenerate or the batch exceeds max_particles.
int sorted_configure_batch(SortedEngine* e, const SimConsts* ks, int nscenes);

// Batch: replaces scene s's constants (real box, stiffness, gravity, ...);
// its geometry and particle count must stay.  Stream-ordered.
int sorted_set_scene_consts(SortedEngine* e, int scene, const SimConsts& k, cudaStream_t st);

// Most particles per task (a bin with more is split); 0 restores the
// automatic choice (enough tasks for every resident CTA, at most 1024).
// Results do not depend on it.
int sorted_set_task_cap(SortedEngine* e, int cap);
int sorted_task_cap(const SortedEngine* e);

// Tasks of at least `min_particles` particles order them into the bank-class
// lane table before p2g_2 (fewer shared-memory bank conflicts, at the price
// of the table's barriers and position loads); smaller tasks keep the bin
// order.  0 restores the default (128); a value above 1024 turns the table
// off.  Results do not depend on it.
int sorted_set_lane_table_min(SortedEngine* e, int min_particles);
int sorted_lane_table_min(const SortedEngine* e);

// Threads per CTA of the two task kernels (p2g_2; g2p + p2g_1): 128, 256 or
// 512 (0: the default, 256).  Results do not depend on it.
int sorted_set_threads(SortedEngine* e, int threads);
int sorted_threads(const SortedEngine* e);

// The bins of two bricks stacked along z (an aligned pair) whose particles
// together number at most max_particles (and at most the task size) share
// one task, with a 4x4x8-cell region and arenas 4 cells deeper: sparse
// bricks then share the fixed costs of a task.  0 never pairs; 2^30 pairs
// every pair whose two bins hold particles; INT_MAX restores the default
// (512).  Results do not depend on it.
int sorted_set_pair_max(SortedEngine* e, int max_particles);
int sorted_pair_max(const SortedEngine* e);

// Forgets the carried-over state (the next step re-bins and redoes p2g_1).
void sorted_invalidate(SortedEngine* e);

// Enqueues `substeps` substeps on ps->P[ps->cur]; each substep writes the
// particles, in bin order, to the other buffer and flips ps->cur.  posvel is
// written (in particle-id order) by the last substep.  k is the scene's
// constants (ignored for a batch, which uses its table).  With `graph` the
// substeps run as one CUDA graph, captured on first use for this substep
// count and engine state and replayed afterwards (not while prof times
// launches).
int sorted_step(SortedEngine* e, ParticleStore* ps, float4* posvel, unsigned long long* oob,
                const SimConsts& k, int substeps, cudaStream_t st, LaunchProfiler* prof,
                bool graph = false);

// True once a substep has run since configure/invalidate.
bool sorted_has_grid(const SortedEngine* e);

// Writes the last substep's grid, as updateGrid left it, in the reference's
// x-major layout (grid_count int4 cells) to device memory `out`.
int sorted_export_grid(SortedEngine* e, const SimConsts& k, int4* out, cudaStream_t st,
                       LaunchProfiler* prof);

// The same for scene `scene` of a batch.
int sorted_export_scene_grid(SortedEngine* e, int scene, int4* out, cudaStream_t st,
                             LaunchProfiler* prof);

// Batch: every scene's grid, as sorted_export_grid, into the concatenation of
// the scenes' reference-layout grids (scene order).
int sorted_export_all(SortedEngine* e, int4* out, cudaStream_t st, LaunchProfiler* prof);

// sorted_export_all plus the particles of `ps` (n of them) in index order
// into dst, in one launch.
int sorted_export_all_canonical(SortedEngine* e, int4* out, const ParticleStore& ps,
                                const Particles& dst, int n, cudaStream_t st,
                                LaunchProfiler* prof);

const char* sorted_error();

}  // namespace mpm
