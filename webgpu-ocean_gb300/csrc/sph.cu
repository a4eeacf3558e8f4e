// sph.cu -- the reference's second simulator, SPHSimulator (sph/sph.ts),
// behind the same four-method API: counting-sort grid (sph/grid/*.wgsl),
// density and near density (sph/density.wgsl), pressure / near-pressure /
// viscosity forces (sph/force.wgsl), integration with penalty walls
// (sph/integrate.wgsl) and the posvel copy (sph/copyPosition.wgsl).
//
// Per substep (two per execute(), sph.ts:325-355):
//   k_sph_bin       cell of every particle (the grid's fixed [-2, 2]^3
//                   domain plus a sentinel), per-cell counts
//   k_sph_blocksum, k_sph_scan   exclusive prefix sum of the counts
//   k_sph_scatter   particle order by cell; each cell's run sorted by
//                   particle index (k_sph_cellsort)
//   k_sph_gather    sorted copies of positions and velocities
//   k_sph_density   per sorted slot: density and near density over the
//                   3x3x3 neighbouring cells (x runs merged, as the shader)
//   k_sph_force     per sorted slot: pressure, near pressure, viscosity,
//                   gravity
//   k_sph_integrate walls, velocity and position update, posvel
//
// Arithmetic restates the shaders with every f32 operation explicitly
// rounded (no contraction), in the shaders' operation order.  Two choices
// the reference leaves to its GPU are fixed: neighbours within a cell are
// visited in ascending particle index (the reference's order comes from
// atomic arrival and is arbitrary), and a particle whose flat cell id falls
// outside [0, gridCount) is left out of the grid (the reference indexes the
// count buffer out of bounds).  The reference's particle count uniform is
// written as a float bit pattern (sph.ts:303-306), so its kernels also run
// the ghost threads of the last workgroup; exactly numParticles particles
// are simulated here.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mpm.h"

namespace mpm {
void set_last_error(const std::string& msg);  // capi.cu
}

namespace {

__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float dvd(float a, float b) { return __fdiv_rn(a, b); }

// Environment (sph.ts:133-152) and SPHParams (sph.ts:154-179), as the
// shaders see them, plus the scale factors the kernel functions compute
// (density.wgsl:37-47, force.wgsl:37-56).
struct Env {
    int X, Y, Z;        // xGrids, yGrids, zGrids
    float cell;         // cellSize
    float half[3];      // xHalf, yHalf, zHalf (the grid's, not the walls')
    float offset;
    float mass, kr, kr2, kr5, kr6, kr9, dt, stiffness, near_stiffness, rest_density, viscosity;
    float s_density, s_near, s_grad, s_near_grad, s_lap;
    int total;          // X * Y * Z
};

__device__ __forceinline__ int f2i(float x) { return __float2int_rz(x); }  // saturating, NaN -> 0

__device__ __forceinline__ void cell_pos(const Env& e, float x, float y, float z, int& xi, int& yi,
                                         int& zi) {
    xi = f2i(floorf(dvd(add(add(x, e.half[0]), e.offset), e.cell)));
    yi = f2i(floorf(dvd(add(add(y, e.half[1]), e.offset), e.cell)));
    zi = f2i(floorf(dvd(add(add(z, e.half[2]), e.offset), e.cell)));
}

// xi + yi * X + zi * X * Y with i32 wraparound.
__device__ __forceinline__ int cell_number(const Env& e, int xi, int yi, int zi) {
    return (int)((unsigned)xi + (unsigned)yi * (unsigned)e.X +
                 (unsigned)zi * (unsigned)e.X * (unsigned)e.Y);
}

__global__ void k_sph_bin(float4* __restrict__ P, float4* __restrict__ V, float4* __restrict__ F,
                          int n, Env e, int* __restrict__ cell_of, unsigned* __restrict__ count,
                          unsigned* __restrict__ rank) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = P[i];
    int xi, yi, zi;
    cell_pos(e, p.x, p.y, p.z, xi, yi, zi);
    const int c = cell_number(e, xi, yi, zi);
    const bool in = c >= 0 && c < e.total;
    cell_of[i] = in ? c : -1;
    if (in) rank[i] = atomicAdd(count + c, 1u);
    // densities are recomputed this substep; particles outside the grid keep
    // zero (density.wgsl:58-59) and so a zero force (force.wgsl)
    p.w = 0.0f;
    P[i] = p;
    float4 v = V[i];
    v.w = 0.0f;
    V[i] = v;
    if (!in) F[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// Exclusive scan of count[0 .. m) into start[0 .. m] in two passes: per-CTA
// sums of kScan counts, then each CTA scans its own counts after adding the
// sums of the CTAs before it (at most a few hundred).
constexpr int kScan = 1024;

__device__ __forceinline__ unsigned block_exclusive(unsigned x, unsigned* s_w, unsigned& total) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane >= o) v += y;
    }
    if (lane == 31) s_w[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned w = s_w[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if ((int)lane >= o) w += y;
        }
        s_w[lane] = w;
    }
    __syncthreads();
    total = s_w[31];
    return v - x + (warp ? s_w[warp - 1] : 0u);
}

__global__ void __launch_bounds__(kScan) k_sph_blocksum(const unsigned* __restrict__ count, int m,
                                                        unsigned* __restrict__ sums) {
    __shared__ unsigned s_w[32];
    const int k = blockIdx.x * kScan + threadIdx.x;
    unsigned total;
    block_exclusive(k < m ? count[k] : 0u, s_w, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScan) k_sph_scan(const unsigned* __restrict__ count,
                                                    const unsigned* __restrict__ sums, int m,
                                                    unsigned* __restrict__ start) {
    __shared__ unsigned s_w[32];
    __shared__ unsigned s_pre;
    // sums of the CTAs before this one
    unsigned pre = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += kScan) pre += sums[b];
    unsigned tp;
    block_exclusive(pre, s_w, tp);
    if (threadIdx.x == 0) s_pre = tp;
    __syncthreads();
    const unsigned base = s_pre;
    const int k = blockIdx.x * kScan + threadIdx.x;
    const unsigned c = k < m ? count[k] : 0u;
    unsigned tot;
    const unsigned ex = block_exclusive(c, s_w, tot);
    if (k < m) start[k] = base + ex;
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) start[m] = base + tot;
}

__global__ void k_sph_scatter(const int* __restrict__ cell_of, const unsigned* __restrict__ rank,
                              const unsigned* __restrict__ start, int n, unsigned* __restrict__ order) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cell_of[i];
    if (c >= 0) order[start[c] + rank[i]] = (unsigned)i;
}

// Each cell's run in ascending particle index (insertion sort; runs are
// short at SPH densities).
__global__ void k_sph_cellsort(const unsigned* __restrict__ start, int total,
                               unsigned* __restrict__ order) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= total) return;
    const unsigned b = start[c], en = start[c + 1];
    for (unsigned k = b + 1; k < en; ++k) {
        const unsigned v = order[k];
        unsigned j = k;
        while (j > b && order[j - 1] > v) {
            order[j] = order[j - 1];
            --j;
        }
        order[j] = v;
    }
}

__global__ void k_sph_gather(const float4* __restrict__ P, const float4* __restrict__ V,
                             const unsigned* __restrict__ order, const unsigned* __restrict__ nbin,
                             float4* __restrict__ SP, float4* __restrict__ SV) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (int)*nbin) return;
    const unsigned i = order[s];
    SP[s] = P[i];
    SV[s] = V[i];
}

// density.wgsl:37-47
__device__ __forceinline__ float density_kernel(const Env& e, float r) {
    const float dd = sub(e.kr2, mul(r, r));
    return mul(mul(mul(e.s_density, dd), dd), dd);
}
__device__ __forceinline__ float near_density_kernel(const Env& e, float r) {
    const float d = sub(e.kr, r);
    return mul(mul(mul(e.s_near, d), d), d);
}

__device__ __forceinline__ bool in_grid(const Env& e, int xi, int yi, int zi) {
    return xi < e.X && 0 <= xi && yi < e.Y && 0 <= yi && zi < e.Z && 0 <= zi;
}

// density.wgsl:58-100, per sorted slot.
__global__ void k_sph_density(float4* __restrict__ P, float4* __restrict__ V,
                              float4* __restrict__ SP, float4* __restrict__ SV,
                              const unsigned* __restrict__ order, const unsigned* __restrict__ start,
                              Env e) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (int)start[e.total]) return;
    const float4 pi = SP[s];
    int vx, vy, vz;
    cell_pos(e, pi.x, pi.y, pi.z, vx, vy, vz);
    float dens = 0.0f, near = 0.0f;
    if (in_grid(e, vx, vy, vz)) {
        for (int dz = max(-1, -vz); dz <= min(1, e.Z - vz - 1); ++dz)
            for (int dy = max(-1, -vy); dy <= min(1, e.Y - vy - 1); ++dy) {
                const int dxmin = max(-1, -vx), dxmax = min(1, e.X - vx - 1);
                const int c0 = cell_number(e, vx + dxmin, vy + dy, vz + dz);
                const int c1 = cell_number(e, vx + dxmax, vy + dy, vz + dz);
                const unsigned b = start[c0], en = start[c1 + 1];
                for (unsigned j = b; j < en; ++j) {
                    const float4 pj = SP[j];
                    const float dx = sub(pi.x, pj.x), dyv = sub(pi.y, pj.y), dzv = sub(pi.z, pj.z);
                    const float r2 = add(add(mul(dx, dx), mul(dyv, dyv)), mul(dzv, dzv));
                    if (r2 < e.kr2) {
                        dens = add(dens, mul(e.mass, density_kernel(e, __fsqrt_rn(r2))));
                        near = add(near, mul(e.mass, near_density_kernel(e, __fsqrt_rn(r2))));
                    }
                }
            }
    }
    const unsigned i = order[s];
    SP[s].w = dens;
    SV[s].w = near;
    P[i].w = dens;
    V[i].w = near;
}

// force.wgsl:37-56
__device__ __forceinline__ float grad_kernel(const Env& e, float r) {
    const float d = sub(e.kr, r);
    return mul(mul(e.s_grad, d), d);
}
__device__ __forceinline__ float near_grad_kernel(const Env& e, float r) {
    const float d = sub(e.kr, r);
    return mul(mul(e.s_near_grad, d), d);
}
__device__ __forceinline__ float lap_kernel(const Env& e, float r) {
    return mul(e.s_lap, sub(e.kr, r));
}

// force.wgsl:64-128, per sorted slot.
__global__ void k_sph_force(const float4* __restrict__ SP, const float4* __restrict__ SV,
                            const unsigned* __restrict__ order, const unsigned* __restrict__ start,
                            Env e, float4* __restrict__ F) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (int)start[e.total]) return;
    const float4 pi = SP[s], vi = SV[s];
    const float dens_i = pi.w, near_i = vi.w;
    float fp[3] = {0.0f, 0.0f, 0.0f}, fv[3] = {0.0f, 0.0f, 0.0f};
    int vx, vy, vz;
    cell_pos(e, pi.x, pi.y, pi.z, vx, vy, vz);
    if (in_grid(e, vx, vy, vz)) {
        for (int dz = max(-1, -vz); dz <= min(1, e.Z - vz - 1); ++dz)
            for (int dy = max(-1, -vy); dy <= min(1, e.Y - vy - 1); ++dy) {
                const int dxmin = max(-1, -vx), dxmax = min(1, e.X - vx - 1);
                const int c0 = cell_number(e, vx + dxmin, vy + dy, vz + dz);
                const int c1 = cell_number(e, vx + dxmax, vy + dy, vz + dz);
                const unsigned b = start[c0], en = start[c1 + 1];
                for (unsigned j = b; j < en; ++j) {
                    const float4 pj = SP[j], vj = SV[j];
                    const float dens_j = pj.w, near_j = vj.w;
                    const float dx = sub(pi.x, pj.x), dyv = sub(pi.y, pj.y), dzv = sub(pi.z, pj.z);
                    const float r2 = add(add(mul(dx, dx), mul(dyv, dyv)), mul(dzv, dzv));
                    if (dens_j == 0.0f || near_j == 0.0f) continue;
                    if (r2 < e.kr2 && 0.0f < r2) {
                        const float r = __fsqrt_rn(r2);
                        const float p_i = mul(e.stiffness, sub(dens_i, e.rest_density));
                        const float p_j = mul(e.stiffness, sub(dens_j, e.rest_density));
                        const float np_i = mul(e.near_stiffness, near_i);
                        const float np_j = mul(e.near_stiffness, near_j);
                        const float sp = dvd(add(p_i, p_j), 2.0f);
                        const float nsp = dvd(add(np_i, np_j), 2.0f);
                        // normalize(pos_j - pos_i)
                        const float ux = sub(pj.x, pi.x), uy = sub(pj.y, pi.y), uz = sub(pj.z, pi.z);
                        const float len = __fsqrt_rn(add(add(mul(ux, ux), mul(uy, uy)), mul(uz, uz)));
                        const float dir[3] = {dvd(ux, len), dvd(uy, len), dvd(uz, len)};
                        const float g = grad_kernel(e, r), ng = near_grad_kernel(e, r);
                        const float a = mul(-e.mass, sp), an = mul(-e.mass, nsp);
                        const float lap = lap_kernel(e, r);
                        const float rel[3] = {sub(vj.x, vi.x), sub(vj.y, vi.y), sub(vj.z, vi.z)};
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            fp[c] = add(fp[c], dvd(mul(mul(a, dir[c]), g), dens_j));
                            fp[c] = add(fp[c], dvd(mul(mul(an, dir[c]), ng), near_j));
                            fv[c] = add(fv[c], dvd(mul(mul(e.mass, rel[c]), lap), dens_j));
                        }
                    }
                }
            }
    }
    const float grv[3] = {mul(dens_i, 0.0f), mul(dens_i, -9.8f), mul(dens_i, 0.0f)};
    float f[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] = add(add(fp[c], mul(fv[c], e.viscosity)), grv[c]);
    F[order[s]] = make_float4(f[0], f[1], f[2], 0.0f);
}


// ---------------------------------------------------------------------------
// Warp per particle (small particle counts: one thread per particle leaves
// the SMs with a few warps each, waiting on the neighbour loop).  The lanes
// compute the neighbour terms of up to kSphChunk neighbours at a time into
// shared memory, then one lane per accumulator adds them in the neighbours'
// order, so every sum is the thread kernel's, bit for bit.
// ---------------------------------------------------------------------------
constexpr int kSphChunk = 64;
constexpr int kSphWarps = 8;  // warps (particles) per 256-thread block

// The up to 9 runs of sorted slots (one per (dz, dy) row, x merged) that
// hold a particle's neighbours, in the thread kernels' visiting order.
struct NeighbourRows {
    unsigned b[9], len[9];
    int n = 0, total = 0;
};

__device__ __forceinline__ void neighbour_rows(const Env& e, const unsigned* __restrict__ start,
                                               int vx, int vy, int vz, NeighbourRows& nr) {
    nr.n = 0;
    nr.total = 0;
#pragma unroll
    for (int r = 0; r < 9; ++r) nr.b[r] = nr.len[r] = 0u;
    if (!in_grid(e, vx, vy, vz)) return;
    int r = 0;
    for (int dz = max(-1, -vz); dz <= min(1, e.Z - vz - 1); ++dz)
        for (int dy = max(-1, -vy); dy <= min(1, e.Y - vy - 1); ++dy) {
            const int dxmin = max(-1, -vx), dxmax = min(1, e.X - vx - 1);
            const int c0 = cell_number(e, vx + dxmin, vy + dy, vz + dz);
            const int c1 = cell_number(e, vx + dxmax, vy + dy, vz + dz);
            const unsigned b = start[c0], en = start[c1 + 1];
#pragma unroll
            for (int q = 0; q < 9; ++q)
                if (q == r) {
                    nr.b[q] = b;
                    nr.len[q] = en - b;
                }
            nr.total += (int)(en - b);
            ++r;
        }
    nr.n = r;
}

// Sorted slot of the k-th neighbour (k < total).
__device__ __forceinline__ unsigned neighbour_slot(const NeighbourRows& nr, int k) {
    unsigned j = 0u, off = 0u;
    bool found = false;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        if (!found && (unsigned)k < off + nr.len[r]) {
            j = nr.b[r] + ((unsigned)k - off);
            found = true;
        }
        off += nr.len[r];
    }
    return j;
}

// density.wgsl:58-100 as k_sph_density, one warp per sorted slot.
__global__ void __launch_bounds__(32 * kSphWarps)
    k_sph_density_warp(float4* __restrict__ P, float4* __restrict__ V, float4* __restrict__ SP,
                       float4* __restrict__ SV, const unsigned* __restrict__ order,
                       const unsigned* __restrict__ start, Env e) {
    __shared__ float s_t[kSphWarps][2][kSphChunk];
    __shared__ unsigned char s_ok[kSphWarps][kSphChunk];
    const int w = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31u);
    const int s = (int)blockIdx.x * kSphWarps + w;
    if (s >= (int)start[e.total]) return;  // uniform per warp
    const float4 pi = SP[s];
    int vx, vy, vz;
    cell_pos(e, pi.x, pi.y, pi.z, vx, vy, vz);
    NeighbourRows nr;
    neighbour_rows(e, start, vx, vy, vz, nr);
    float acc = 0.0f;  // lane 0: density, lane 1: near density
    for (int base = 0; base < nr.total; base += kSphChunk) {
        const int m = min(kSphChunk, nr.total - base);
        for (int q = lane; q < m; q += 32) {
            const float4 pj = SP[neighbour_slot(nr, base + q)];
            const float dx = sub(pi.x, pj.x), dyv = sub(pi.y, pj.y), dzv = sub(pi.z, pj.z);
            const float r2 = add(add(mul(dx, dx), mul(dyv, dyv)), mul(dzv, dzv));
            const bool ok = r2 < e.kr2;
            s_ok[w][q] = ok;
            if (ok) {
                s_t[w][0][q] = mul(e.mass, density_kernel(e, __fsqrt_rn(r2)));
                s_t[w][1][q] = mul(e.mass, near_density_kernel(e, __fsqrt_rn(r2)));
            }
        }
        __syncwarp();
        if (lane < 2)
            for (int q = 0; q < m; ++q)
                if (s_ok[w][q]) acc = add(acc, s_t[w][lane][q]);
        __syncwarp();
    }
    const float near = __shfl_sync(0xffffffffu, acc, 1);
    if (lane == 0) {
        const unsigned i = order[s];
        SP[s].w = acc;
        SV[s].w = near;
        P[i].w = acc;
        V[i].w = near;
    }
}

// force.wgsl:64-128 as k_sph_force, one warp per sorted slot.
__global__ void __launch_bounds__(32 * kSphWarps)
    k_sph_force_warp(const float4* __restrict__ SP, const float4* __restrict__ SV,
                     const unsigned* __restrict__ order, const unsigned* __restrict__ start,
                     Env e, float4* __restrict__ F) {
    __shared__ float s_t[kSphWarps][9][kSphChunk];
    __shared__ unsigned char s_ok[kSphWarps][kSphChunk];
    const int w = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31u);
    const int s = (int)blockIdx.x * kSphWarps + w;
    if (s >= (int)start[e.total]) return;  // uniform per warp
    const float4 pi = SP[s], vi = SV[s];
    const float dens_i = pi.w, near_i = vi.w;
    int vx, vy, vz;
    cell_pos(e, pi.x, pi.y, pi.z, vx, vy, vz);
    NeighbourRows nr;
    neighbour_rows(e, start, vx, vy, vz, nr);
    // lanes 0-2: pressure force component c (two terms per neighbour), lanes
    // 3-5: viscosity force component c
    float acc = 0.0f;
    for (int base = 0; base < nr.total; base += kSphChunk) {
        const int m = min(kSphChunk, nr.total - base);
        for (int q = lane; q < m; q += 32) {
            const unsigned j = neighbour_slot(nr, base + q);
            const float4 pj = SP[j], vj = SV[j];
            const float dens_j = pj.w, near_j = vj.w;
            const float dx = sub(pi.x, pj.x), dyv = sub(pi.y, pj.y), dzv = sub(pi.z, pj.z);
            const float r2 = add(add(mul(dx, dx), mul(dyv, dyv)), mul(dzv, dzv));
            const bool ok = !(dens_j == 0.0f || near_j == 0.0f) && r2 < e.kr2 && 0.0f < r2;
            s_ok[w][q] = ok;
            if (ok) {
                const float r = __fsqrt_rn(r2);
                const float p_i = mul(e.stiffness, sub(dens_i, e.rest_density));
                const float p_j = mul(e.stiffness, sub(dens_j, e.rest_density));
                const float np_i = mul(e.near_stiffness, near_i);
                const float np_j = mul(e.near_stiffness, near_j);
                const float sp = dvd(add(p_i, p_j), 2.0f);
                const float nsp = dvd(add(np_i, np_j), 2.0f);
                const float ux = sub(pj.x, pi.x), uy = sub(pj.y, pi.y), uz = sub(pj.z, pi.z);
                const float len = __fsqrt_rn(add(add(mul(ux, ux), mul(uy, uy)), mul(uz, uz)));
                const float dir[3] = {dvd(ux, len), dvd(uy, len), dvd(uz, len)};
                const float g = grad_kernel(e, r), ng = near_grad_kernel(e, r);
                const float a = mul(-e.mass, sp), an = mul(-e.mass, nsp);
                const float lap = lap_kernel(e, r);
                const float rel[3] = {sub(vj.x, vi.x), sub(vj.y, vi.y), sub(vj.z, vi.z)};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    s_t[w][c][q] = dvd(mul(mul(a, dir[c]), g), dens_j);
                    s_t[w][3 + c][q] = dvd(mul(mul(an, dir[c]), ng), near_j);
                    s_t[w][6 + c][q] = dvd(mul(mul(e.mass, rel[c]), lap), dens_j);
                }
            }
        }
        __syncwarp();
        if (lane < 3) {
            for (int q = 0; q < m; ++q)
                if (s_ok[w][q]) {
                    acc = add(acc, s_t[w][lane][q]);
                    acc = add(acc, s_t[w][3 + lane][q]);
                }
        } else if (lane < 6) {
            for (int q = 0; q < m; ++q)
                if (s_ok[w][q]) acc = add(acc, s_t[w][3 + lane][q]);
        }
        __syncwarp();
    }
    const float fv = __shfl_down_sync(0xffffffffu, acc, 3);  // lane c gets lane 3 + c's
    const float grv[3] = {mul(dens_i, 0.0f), mul(dens_i, -9.8f), mul(dens_i, 0.0f)};
    float f = 0.0f;
    if (lane < 3) f = add(add(acc, mul(fv, e.viscosity)), grv[lane]);
    const float f1 = __shfl_sync(0xffffffffu, f, 1), f2 = __shfl_sync(0xffffffffu, f, 2);
    if (lane == 0) F[order[s]] = make_float4(f, f1, f2, 0.0f);
}

// integrate.wgsl:37-64 and copyPosition.wgsl:27-37.
__global__ void k_sph_integrate(float4* __restrict__ P, float4* __restrict__ V,
                                const float4* __restrict__ F, int n, Env e,
                                const float* __restrict__ box, float4* __restrict__ posvel) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float rx = box[0], ry = box[1], rz = box[2];
    float4 p = P[i], v = V[i];
    const float dens = p.w;
    if (dens != 0.0f) {
        const float4 f = F[i];
        float a[3] = {dvd(f.x, dens), dvd(f.y, dens), dvd(f.z, dens)};
        const float ws = 8000.0f;
        const float half[3] = {rx, ry, rz};
        const float pos[3] = {p.x, p.y, p.z};
        float plus[3][3], minus[3][3];  // [axis][component]
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const float pd = fminf(sub(half[ax], pos[ax]), 0.0f);
            const float md = fminf(add(half[ax], pos[ax]), 0.0f);
#pragma unroll
            for (int c = 0; c < 3; ++c) {  // vec3f(1., 0., 0.) and vec3f(-1., 0., 0.)
                plus[ax][c] = mul(mul(c == ax ? 1.0f : 0.0f, ws), pd);
                minus[ax][c] = mul(mul(c == ax ? -1.0f : 0.0f, ws), md);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float xf = add(plus[0][c], minus[0][c]);
            const float yf = add(plus[1][c], minus[1][c]);
            const float zf = add(plus[2][c], minus[2][c]);
            a[c] = add(a[c], add(add(xf, yf), zf));
        }
        v.x = add(v.x, mul(e.dt, a[0]));
        v.y = add(v.y, mul(e.dt, a[1]));
        v.z = add(v.z, mul(e.dt, a[2]));
        p.x = add(p.x, mul(e.dt, v.x));
        p.y = add(p.y, mul(e.dt, v.y));
        p.z = add(p.z, mul(e.dt, v.z));
        P[i] = p;
        V[i] = v;
    }
    if (posvel) {
        posvel[2 * (size_t)i] = make_float4(p.x, p.y, p.z, 0.0f);
        posvel[2 * (size_t)i + 1] = make_float4(v.x, v.y, v.z, 0.0f);
    }
}

int fail(int code, const std::string& msg) {
    mpm::set_last_error(msg);
    return code;
}

int cuda_fail(cudaError_t err, const char* what) {
    return fail(MPM_E_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    double random() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
};

}  // namespace

// Default for mpm_sph::warp_max: below it a warp per particle, above it a
// thread per particle fills the GPU with fewer instructions.  Measured per
// 2-substep frame (warp / thread): 20k particles 0.285 / 0.359 ms, 40k
// 0.599 / 0.499 ms.
constexpr int kSphWarpMaxDefault = 32768;

struct mpm_sph {
    int device = 0;
    int max_particles = 0;
    int n = 0;
    float render_diameter = 0.0f;
    float real_half[3] = {0, 0, 0};
    Env e{};
    float4 *P = nullptr, *V = nullptr, *F = nullptr, *SP = nullptr, *SV = nullptr;
    float4* posvel = nullptr;
    bool posvel_owned = false;
    int* cell_of = nullptr;
    unsigned *count = nullptr, *start = nullptr, *rank = nullptr, *order = nullptr;
    unsigned* sums = nullptr;  // per-CTA count sums of the scan
    // the real box as the kernels read it (a device uniform, so that a
    // captured frame graph survives changeBoxSize)
    float* box_d = nullptr;
    float box_uploaded[3] = {NAN, NAN, NAN};
    bool graph = true;
    int warp_max = kSphWarpMaxDefault;  // particle counts up to this run a warp per particle
    struct FrameGraph {
        int substeps, n;
        cudaGraphExec_t exec;
    };
    std::vector<FrameGraph> graphs;
};

namespace {

void drop_graphs(mpm_sph* s) {
    for (auto& g : s->graphs) cudaGraphExecDestroy(g.exec);
    s->graphs.clear();
}

void free_sph(mpm_sph* s) {
    drop_graphs(s);
    cudaFree(s->box_d);
    cudaFree(s->P); cudaFree(s->V); cudaFree(s->F); cudaFree(s->SP); cudaFree(s->SV);
    if (s->posvel_owned) cudaFree(s->posvel);
    cudaFree(s->cell_of); cudaFree(s->count); cudaFree(s->start); cudaFree(s->rank);
    cudaFree(s->order); cudaFree(s->sums);
    delete s;
}

// sph.ts:58-86 and 154-179: grid and kernel constants (JS doubles, stored
// as f32 uniforms) and the scale factors of the kernel functions (f32
// arithmetic on the f32 uniforms; the literals' products are folded in
// double precision first, as WGSL folds abstract constants).
Env make_env() {
    Env e{};
    const double kr = 0.07;
    const double cell = 1.0 * kr;
    const double half = 2.0, len = 2.0 * half, sentinel = 4.0 * cell;
    const int grids = (int)std::ceil((len + sentinel) / cell);
    e.X = e.Y = e.Z = grids;
    e.cell = (float)cell;
    e.half[0] = e.half[1] = e.half[2] = (float)half;
    e.offset = (float)(sentinel / 2.0);
    e.mass = 1.0f;
    e.kr = (float)kr;
    e.kr2 = (float)std::pow(kr, 2);
    e.kr5 = (float)std::pow(kr, 5);
    e.kr6 = (float)std::pow(kr, 6);
    e.kr9 = (float)std::pow(kr, 9);
    e.dt = 0.006f;
    e.stiffness = 20.0f;
    e.near_stiffness = 1.0f;
    e.rest_density = 15000.0f;
    e.viscosity = 100.0f;
    const float pi = (float)3.1415926535;
    e.s_density = 315.0f / ((float)(64.0 * 3.1415926535) * e.kr9);
    e.s_near = 15.0f / (pi * e.kr6);
    e.s_grad = 45.0f / (pi * e.kr6);
    e.s_near_grad = 45.0f / (pi * e.kr5);
    e.s_lap = 45.0f / (pi * e.kr6);
    e.total = e.X * e.Y * e.Z;
    return e;
}

}  // namespace

extern "C" {

int mpm_sph_create(int max_particles, float render_diameter, void* posvel_device,
                   size_t posvel_bytes, mpm_sph** out) {
    if (!out) return fail(MPM_E_INVALID, "out is null");
    *out = nullptr;
    if (max_particles < 0) return fail(MPM_E_INVALID, "negative capacity");
    if (posvel_device && posvel_bytes < (size_t)32 * (size_t)max_particles)
        return fail(MPM_E_INVALID, "posvel buffer smaller than 32 * max_particles bytes");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(MPM_E_NO_DEVICE, "no CUDA device");
    }
    mpm_sph* s = new mpm_sph();
    cudaGetDevice(&s->device);
    s->max_particles = max_particles;
    s->render_diameter = render_diameter;
    s->e = make_env();
    const size_t np = (size_t)(max_particles > 0 ? max_particles : 1);
    cudaError_t err = cudaSuccess;
    float4** bufs[5] = {&s->P, &s->V, &s->F, &s->SP, &s->SV};
    for (int b = 0; b < 5 && err == cudaSuccess; ++b) err = cudaMalloc(bufs[b], sizeof(float4) * np);
    if (err == cudaSuccess) {
        if (posvel_device) {
            s->posvel = static_cast<float4*>(posvel_device);
        } else {
            err = cudaMalloc(&s->posvel, sizeof(float4) * 2 * np);
            s->posvel_owned = true;
        }
    }
    if (err == cudaSuccess) err = cudaMalloc(&s->cell_of, 4 * np);
    if (err == cudaSuccess) err = cudaMalloc(&s->rank, 4 * np);
    if (err == cudaSuccess) err = cudaMalloc(&s->order, 4 * np);
    if (err == cudaSuccess) err = cudaMalloc(&s->count, 4 * ((size_t)s->e.total + 1));
    if (err == cudaSuccess) err = cudaMalloc(&s->start, 4 * ((size_t)s->e.total + 1));
    if (err == cudaSuccess) err = cudaMalloc(&s->sums, 4 * ((size_t)s->e.total / kScan + 2));
    if (err == cudaSuccess) err = cudaMalloc(&s->box_d, sizeof(float) * 3);
    if (err != cudaSuccess) {
        const int rc = cuda_fail(err, "mpm_sph_create");
        free_sph(s);
        return rc;
    }
    *out = s;
    return MPM_OK;
}

int mpm_sph_destroy(mpm_sph* s) {
    if (!s) return MPM_OK;
    cudaDeviceSynchronize();
    free_sph(s);
    return MPM_OK;
}

int mpm_sph_upload(mpm_sph* s, const float* rec64, int n, const float real_half[3]) {
    if (!s || (n > 0 && !rec64) || !real_half) return fail(MPM_E_INVALID, "bad arguments");
    if (n < 0 || n > s->max_particles) return fail(MPM_E_CAPACITY, "numParticles exceeds the particle capacity");
    std::vector<float4> P((size_t)n), V((size_t)n), F((size_t)n);
    for (int i = 0; i < n; ++i) {
        const float* r = rec64 + 16 * (size_t)i;  // particle record, sph.ts:13,205-211
        P[(size_t)i] = make_float4(r[0], r[1], r[2], r[11]);
        V[(size_t)i] = make_float4(r[4], r[5], r[6], r[12]);
        F[(size_t)i] = make_float4(r[8], r[9], r[10], 0.0f);
    }
    cudaError_t err = cudaDeviceSynchronize();
    if (n && err == cudaSuccess) err = cudaMemcpy(s->P, P.data(), sizeof(float4) * n, cudaMemcpyHostToDevice);
    if (n && err == cudaSuccess) err = cudaMemcpy(s->V, V.data(), sizeof(float4) * n, cudaMemcpyHostToDevice);
    if (n && err == cudaSuccess) err = cudaMemcpy(s->F, F.data(), sizeof(float4) * n, cudaMemcpyHostToDevice);
    if (n && err == cudaSuccess) err = cudaMemset(s->posvel, 0, sizeof(float4) * 2 * (size_t)n);
    if (err != cudaSuccess) return cuda_fail(err, "mpm_sph_upload");
    s->n = n;
    for (int a = 0; a < 3; ++a) s->real_half[a] = real_half[a];
    return MPM_OK;
}

// SPHSimulator.initDambreak (sph.ts:357-381): y from -0.95 h_y upward without
// bound, x in [-0.95 h_x, 0.95 h_x), z in [-0.95 h_z, 0), step 0.035, one
// jitter 0.001 * Math.random() added to x, y and z (Math.random ->
// SplitMix64(seed)).  Writes 64-byte records; returns the count.
int mpm_sph_scene_dambreak(float* out_rec64, int num_particles, const double half[3], uint64_t seed) {
    if (!out_rec64 || !half || num_particles < 0) return fail(MPM_E_INVALID, "bad arguments");
    SplitMix64 rng(seed);
    const double kr = 0.07, step = 0.5 * kr;
    int n = 0;
    for (double y = -half[1] * 0.95; n < num_particles; y += step) {
        bool any = false;
        for (double x = -0.95 * half[0]; x < 0.95 * half[0] && n < num_particles; x += step)
            for (double z = -0.95 * half[2]; z < 0 * half[2] && n < num_particles; z += step) {
                const double jitter = 0.001 * rng.random();
                float* r = out_rec64 + 16 * (size_t)n;
                std::memset(r, 0, 64);
                r[0] = (float)(x + jitter);
                r[1] = (float)(y + jitter);
                r[2] = (float)(z + jitter);
                ++n;
                any = true;
            }
        if (!any) break;  // an empty layer never fills (degenerate box)
    }
    return n;
}

int mpm_sph_reset_dambreak(mpm_sph* s, int num_particles, const double half[3], uint64_t seed) {
    if (!s || !half) return fail(MPM_E_INVALID, "bad arguments");
    if (num_particles < 0 || num_particles > s->max_particles)
        return fail(MPM_E_CAPACITY, "numParticles exceeds the particle capacity");
    std::vector<float> buf((size_t)16 * (size_t)(num_particles > 0 ? num_particles : 1));
    const int n = mpm_sph_scene_dambreak(buf.data(), num_particles, half, seed);
    if (n < 0) return n;
    const float rh[3] = {(float)half[0], (float)half[1], (float)half[2]};
    return mpm_sph_upload(s, buf.data(), n, rh);
}

int mpm_sph_set_real_box(mpm_sph* s, const float real_half[3]) {
    if (!s || !real_half) return fail(MPM_E_INVALID, "bad arguments");
    for (int a = 0; a < 3; ++a) s->real_half[a] = real_half[a];
    return MPM_OK;
}

}  // extern "C"

namespace {

void enqueue_substeps(mpm_sph* s, int substeps, cudaStream_t st) {
    const int n = s->n;
    const Env& e = s->e;
    const int pb = (n + 255) / 256, cb = (e.total + 255) / 256;
    for (int k = 0; k < substeps; ++k) {
        cudaMemsetAsync(s->count, 0, 4 * ((size_t)e.total + 1), st);
        k_sph_bin<<<pb, 256, 0, st>>>(s->P, s->V, s->F, n, e, s->cell_of, s->count, s->rank);
        const int sb = (e.total + kScan - 1) / kScan;
        k_sph_blocksum<<<sb, kScan, 0, st>>>(s->count, e.total, s->sums);
        k_sph_scan<<<sb, kScan, 0, st>>>(s->count, s->sums, e.total, s->start);
        k_sph_scatter<<<pb, 256, 0, st>>>(s->cell_of, s->rank, s->start, n, s->order);
        k_sph_cellsort<<<cb, 256, 0, st>>>(s->start, e.total, s->order);
        // sorted slots: start[total] of them (read on the device); launched
        // over n, the most there can be
        k_sph_gather<<<pb, 256, 0, st>>>(s->P, s->V, s->order, s->start + e.total, s->SP, s->SV);
        if (n <= s->warp_max) {  // one warp per particle
            const int wb = (n + kSphWarps - 1) / kSphWarps;
            k_sph_density_warp<<<wb, 32 * kSphWarps, 0, st>>>(s->P, s->V, s->SP, s->SV, s->order,
                                                               s->start, e);
            k_sph_force_warp<<<wb, 32 * kSphWarps, 0, st>>>(s->SP, s->SV, s->order, s->start, e,
                                                             s->F);
        } else {
            k_sph_density<<<pb, 256, 0, st>>>(s->P, s->V, s->SP, s->SV, s->order, s->start, e);
            k_sph_force<<<pb, 256, 0, st>>>(s->SP, s->SV, s->order, s->start, e, s->F);
        }
        k_sph_integrate<<<pb, 256, 0, st>>>(s->P, s->V, s->F, n, e, s->box_d, s->posvel);
    }
}

// The frame's launches as a CUDA graph, captured once per (substeps,
// particle count) and replayed.
cudaError_t launch_graph(mpm_sph* s, int substeps, cudaStream_t st) {
    mpm_sph::FrameGraph* hit = nullptr;
    for (auto& g : s->graphs)
        if (g.substeps == substeps && g.n == s->n) hit = &g;
    if (!hit) {
        cudaStream_t cs = nullptr;
        cudaError_t err = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (err != cudaSuccess) return err;
        cudaGraph_t graph = nullptr;
        err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) {
            enqueue_substeps(s, substeps, cs);
            err = cudaStreamEndCapture(cs, &graph);
        }
        cudaGraphExec_t exec = nullptr;
        if (err == cudaSuccess) err = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        cudaStreamDestroy(cs);
        if (err != cudaSuccess) return err;
        s->graphs.push_back({substeps, s->n, exec});
        hit = &s->graphs.back();
    }
    return cudaGraphLaunch(hit->exec, st);
}

}  // namespace

extern "C" {

// execute (sph.ts:325-355): `substeps` x (grid clear, build, prefix sum,
// reorder, density, reorder, force, integrate, copyPosition).
int mpm_sph_step(mpm_sph* s, int substeps, void* stream) {
    if (!s || substeps < 0) return fail(MPM_E_INVALID, "bad arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (s->n == 0 || substeps == 0) return MPM_OK;
    if (std::memcmp(s->box_uploaded, s->real_half, sizeof(s->real_half)) != 0) {
        // pageable source: staged before the call returns
        const cudaError_t err =
            cudaMemcpyAsync(s->box_d, s->real_half, sizeof(s->real_half), cudaMemcpyHostToDevice, st);
        if (err != cudaSuccess) return cuda_fail(err, "mpm_sph_step");
        std::memcpy(s->box_uploaded, s->real_half, sizeof(s->real_half));
    }
    if (s->graph) {
        const cudaError_t err = launch_graph(s, substeps, st);
        if (err != cudaSuccess) return cuda_fail(err, "mpm_sph_step graph");
    } else {
        enqueue_substeps(s, substeps, st);
    }
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return cuda_fail(err, "mpm_sph_step");
    return MPM_OK;
}

int mpm_sph_set_graph(mpm_sph* s, int enable) {
    if (!s) return fail(MPM_E_INVALID, "bad arguments");
    s->graph = enable != 0;
    return MPM_OK;
}

int mpm_sph_set_warp_per_particle(mpm_sph* s, int max_particles) {
    if (!s || max_particles < -1) return fail(MPM_E_INVALID, "bad arguments");
    const int v = max_particles == -1 ? kSphWarpMaxDefault : max_particles;
    if (v != s->warp_max) drop_graphs(s);  // the captured frames hold the launches
    s->warp_max = v;
    return MPM_OK;
}

int mpm_sph_get_warp_per_particle(const mpm_sph* s) { return s ? s->warp_max : MPM_E_INVALID; }

int mpm_sph_num_particles(const mpm_sph* s) { return s ? s->n : 0; }
int64_t mpm_sph_grid_count(const mpm_sph* s) { return s ? s->e.total : 0; }
void* mpm_sph_posvel_device_ptr(mpm_sph* s) { return s ? s->posvel : nullptr; }

int mpm_sph_download_particles(mpm_sph* s, float* out_rec64) {
    if (!s || (!out_rec64 && s->n)) return fail(MPM_E_INVALID, "bad arguments");
    const int n = s->n;
    std::vector<float4> P((size_t)n), V((size_t)n), F((size_t)n);
    cudaError_t err = cudaDeviceSynchronize();
    if (n && err == cudaSuccess) err = cudaMemcpy(P.data(), s->P, sizeof(float4) * n, cudaMemcpyDeviceToHost);
    if (n && err == cudaSuccess) err = cudaMemcpy(V.data(), s->V, sizeof(float4) * n, cudaMemcpyDeviceToHost);
    if (n && err == cudaSuccess) err = cudaMemcpy(F.data(), s->F, sizeof(float4) * n, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_fail(err, "mpm_sph_download_particles");
    for (int i = 0; i < n; ++i) {
        float* r = out_rec64 + 16 * (size_t)i;
        std::memset(r, 0, 64);
        r[0] = P[(size_t)i].x; r[1] = P[(size_t)i].y; r[2] = P[(size_t)i].z;
        r[4] = V[(size_t)i].x; r[5] = V[(size_t)i].y; r[6] = V[(size_t)i].z;
        r[8] = F[(size_t)i].x; r[9] = F[(size_t)i].y; r[10] = F[(size_t)i].z;
        r[11] = P[(size_t)i].w;   // density
        r[12] = V[(size_t)i].w;   // nearDensity
    }
    return MPM_OK;
}

int mpm_sph_download_posvel(mpm_sph* s, float* out) {
    if (!s || (!out && s->n)) return fail(MPM_E_INVALID, "bad arguments");
    cudaError_t err = cudaDeviceSynchronize();
    if (s->n && err == cudaSuccess)
        err = cudaMemcpy(out, s->posvel, sizeof(float4) * 2 * (size_t)s->n, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_fail(err, "mpm_sph_download_posvel");
    return MPM_OK;
}

}  // extern "C"
