// adjoint.h -- reverse-mode substep kernels (adjoint.cu).
#pragma once
#include <cuda_runtime.h>

#include "mpm_internal.h"

namespace mpm {

// Doubles per particle record of the FP64 tape: x[0..2], v[3..5], C[6..14]
// (C[c][r] at 6 + 3c + r), padding [15].
constexpr int kRec64 = 16;

// One scene of an adjoint batch: its constants, the first cell of its grid in
// the linear (reference-layout) concatenation of all scenes' grids, and its
// bricks (4^3 base cells, BX x BY x BZ of them) in the adjoint's spatial
// sort, numbered from bbase.
struct AdjScene {
    SimConsts k;
    int lbase;
    int bbase;
    int BY, BZ;
};

// Bricks per axis of a scene's grid (x extent ceil(grid_count / (Y Z))).
void adj_bricks(const SimConsts& k, int& BX, int& BY, int& BZ);

// Scratch of the adjoint's per-substep spatial sort: particles are ordered
// by the brick of their base cell (bin nbins - 1: stencils that leave the
// grid interior), and the particle kernels run in that order with `lanes`
// (1 or 3) threads per particle.
struct AdjSort {
    int2* key_rank = nullptr;   // n: (bin, rank in bin)
    int* perm = nullptr;        // n: particle ids in sorted order
    int* bin_count = nullptr;   // nbins
    int* bin_first = nullptr;   // nbins
    int* placed = nullptr;      // 1: particles placed so far
    int nbins = 0;
    int lanes = 1;
};

// One substep backward.  S: the substep's input state (particle order of the
// batch); G: its grid after updateGrid, reference layout, all scenes
// concatenated (ncells cells); Aout: adjoint of the substep's output state;
// Anew: receives the adjoint of S; gadj: ncells float4 of scratch; pgrad:
// per-scene (stiffness, dynamic_viscosity) adjoints, accumulated.
void launch_adjoint_substep(const Particles& S, const int4* G, const Particles& Aout,
                            const Particles& Anew, float4* gadj, const AdjScene* scenes,
                            int nscenes, const int* pscene, int n, int ncells, double* pgrad,
                            const AdjSort& so, cudaStream_t st);

// The same on the FP64 tape (S: kRec64 doubles per particle; G: double4
// cells {v or momentum, mass}).
void launch_adjoint_substep64(const double* S, const double4* G, const Particles& Aout,
                              const Particles& Anew, float4* gadj, const AdjScene* scenes,
                              int nscenes, const int* pscene, int n, int ncells, double* pgrad,
                              const AdjSort& so, cudaStream_t st);

// One FP64 substep of the continuous model: S -> Sout, leaving the updated
// grid in G (ncells double4, all scenes).
void launch_substep64(const double* S, double4* G, double* Sout, const AdjScene* scenes,
                      int nscenes, const int* pscene, int n, int ncells, cudaStream_t st);

// 80-byte reference records (device) <-> FP64 tape records.
void launch_records_to_rec64(const float* rec, double* S, int n, cudaStream_t st);
void launch_rec64_to_records(const double* S, float* rec, int n, cudaStream_t st);

// A += B, record-wise over n particles.
void launch_particles_axpy(const Particles& A, const Particles& B, int n, cudaStream_t st);

// Squared-distance loss of one observed substep: state X (fixed-point tape)
// or X64 (FP64 tape, when non-null) against obs (n float4, xyz), seeds into
// `seed` (position = scale[scene] * (x - obs), rest 0), |x - obs|^2 summed
// per scene into loss (FP64).
void launch_obs_loss(const Particles* X, const double* X64, const float4* obs, const int* pscene,
                     const float* scale, const Particles& seed, double* loss, int n,
                     cudaStream_t st);

}  // namespace mpm
