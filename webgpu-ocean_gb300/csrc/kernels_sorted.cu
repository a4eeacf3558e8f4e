// kernels_sorted.cu -- the binned, fused MLS-MPM engine.
//
// Same results as the reference's six dispatches (mls-mpm/mls-mpm.ts:245-268),
// bit for bit: every per-particle value is computed by the shared stage bodies
// of mpm_math.cuh, and the grid is an i32 sum, so the order in which
// contributions arrive does not matter.  What changes is where the work runs:
//
//  * The grid is stored brick-major: 4x4x4-cell bricks of 1 KB, contiguous,
//    so a particle neighbourhood is a handful of 64-byte runs.
//  * Particles are counting-sorted by brick every substep.  A task is up to
//    256 particles of one brick; a CTA runs one task at a time and keeps the
//    grid cells the task touches (its "arena", the particles' bounding box of
//    base cells plus a one-cell halo) in shared memory.  Gathers read the
//    arena; scatters are shared-memory i32 atomics, flushed with one
//    red.global.add per touched cell and component.
//  * Stage fusion per substep:
//      k_p2g2        p2g_2 (and clears the other grid's dirty bricks)
//      k_g2p_p2g1    updateGrid (applied while staging the arena) + g2p +
//                    copyPosition (last substep) + the next substep's
//                    clearGrid-free p2g_1 into the other grid + binning
//      k_scan, k_scatter   counting sort for the next substep
//    The updated grid is never written back: download recomputes updateGrid
//    from the raw post-p2g_2 grid, which is what the reference's buffer holds
//    once updateGrid has run.
//  * Particles whose 27-cell stencil leaves the box (quirk Q1 aliasing, NaN,
//    huge coordinates) and tasks whose arena would not fit take a global path
//    that uses the reference's flat indices directly.
#include <climits>
#include <cstdio>
#include <string>

#include "mpm_internal.h"
#include "sorted_engine.h"

namespace mpm {

namespace {

constexpr int kTask = 256;        // particles per task == threads per CTA
constexpr int kArenaMax = 1024;   // cells a shared-memory arena can hold
constexpr int kScanThreads = 1024;

thread_local std::string g_err;

struct Geo {
    int Y, Z, YZ;      // flat-index strides: i32(init.y), i32(init.z)
    int grid_count;
    int Xi;            // cells along x reachable by an in-range flat index
    int BX, BY, BZ;    // bricks per axis
    int nbricks;       // BX*BY*BZ; bin id nbricks collects irregular particles
};

struct Task {
    int first;
    int count;
};

struct Dev {
    int4* grid[2];
    uint32_t* dirty_flag[2];
    uint32_t* dirty_list[2];
    uint32_t* dirty_n;   // [2]
    uint32_t* ticket;    // [1]
    uint32_t* bin_of;
    uint32_t* rank_of;
    uint32_t* bin_count;  // [nbricks + 1]
    uint32_t* bin_start;  // [nbricks + 2]
    uint32_t* order;
    Task* tasks;
    uint32_t* ntasks;
};

__device__ __forceinline__ int brick_of(const Geo& g, int x, int y, int z) {
    return ((x >> 2) * g.BY + (y >> 2)) * g.BZ + (z >> 2);
}

__device__ __forceinline__ int brick_addr(const Geo& g, int x, int y, int z) {
    return brick_of(g, x, y, z) * 64 + ((x & 3) << 4) + ((y & 3) << 2) + (z & 3);
}

// Flat index (in [0, grid_count)) -> brick-major address.
__device__ __forceinline__ int flat_to_addr(const Geo& g, int idx) {
    const int x = idx / g.YZ;
    const int r = idx - x * g.YZ;
    const int y = r / g.Z;
    const int z = r - y * g.Z;
    return brick_addr(g, x, y, z);
}

__device__ __forceinline__ bool in_grid(const Geo& g, int idx) {
    return (unsigned)idx < (unsigned)g.grid_count;
}

// A particle is regular when all 27 stencil cells are in-range cells whose
// flat index equals their geometric position (no aliasing).
__device__ __forceinline__ bool regular_base(const Geo& g, int bx, int by, int bz) {
    if (bx < 1 || by < 1 || bz < 1) return false;
    if ((long long)by + 1 >= g.Y || (long long)bz + 1 >= g.Z) return false;
    const long long f = (((long long)bx + 1) * g.Y + (by + 1)) * (long long)g.Z + (bz + 1);
    return f < g.grid_count;
}

__device__ __forceinline__ void base_cell(const float x[3], int& bx, int& by, int& bz) {
    bx = f2i_sat(floorf(x[0]));
    by = f2i_sat(floorf(x[1]));
    bz = f2i_sat(floorf(x[2]));
}

__device__ __forceinline__ void mark_brick(const Dev& d, int gi, uint32_t b) {
    if (__ldcg(d.dirty_flag[gi] + b) != 0u) return;
    if (atomicExch(d.dirty_flag[gi] + b, 1u) == 0u) {
        const uint32_t pos = atomicAdd(d.dirty_n + gi, 1u);
        d.dirty_list[gi][pos] = b;
    }
}

// Bounding box of the valid base cells of the CTA's particles.
struct Box {
    int lo[3], hi[3];
    int dim[3];
    int cells;
    bool any, fits;
};

__device__ __forceinline__ Box block_box(bool valid, int bx, int by, int bz, int* s_box) {
    if (threadIdx.x < 6) s_box[threadIdx.x] = threadIdx.x < 3 ? INT_MAX : INT_MIN;
    __syncthreads();
    const int v[3] = {bx, by, bz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int mn = __reduce_min_sync(0xffffffffu, valid ? v[a] : INT_MAX);
        const int mx = __reduce_max_sync(0xffffffffu, valid ? v[a] : INT_MIN);
        if ((threadIdx.x & 31) == 0) {
            if (mn != INT_MAX) atomicMin(s_box + a, mn);
            if (mx != INT_MIN) atomicMax(s_box + 3 + a, mx);
        }
    }
    __syncthreads();
    Box b;
    b.any = s_box[0] <= s_box[3];
    long long cells = 0;
    if (b.any) {
        cells = 1;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = s_box[a] - 1;
            b.hi[a] = s_box[3 + a] + 1;
            const long long dd = (long long)b.hi[a] - b.lo[a] + 1;
            cells *= dd;
            b.dim[a] = dd > kArenaMax ? kArenaMax + 1 : (int)dd;
        }
    } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) b.lo[a] = b.hi[a] = 0, b.dim[a] = 0;
    }
    b.fits = b.any && cells <= kArenaMax;
    b.cells = b.fits ? (int)cells : 0;
    return b;
}

__device__ __forceinline__ void arena_coords(const Box& b, int li, int& x, int& y, int& z) {
    const int dyz = b.dim[1] * b.dim[2];
    const int ax = li / dyz;
    const int r = li - ax * dyz;
    const int ay = r / b.dim[2];
    const int az = r - ay * b.dim[2];
    x = b.lo[0] + ax;
    y = b.lo[1] + ay;
    z = b.lo[2] + az;
}

// Marks every brick overlapped by the arena as dirty in grid gi.
__device__ __forceinline__ void mark_arena_bricks(const Dev& d, const Geo& g, int gi, const Box& b) {
    const int b0[3] = {b.lo[0] >> 2, b.lo[1] >> 2, b.lo[2] >> 2};
    const int nb[3] = {(b.hi[0] >> 2) - b0[0] + 1, (b.hi[1] >> 2) - b0[1] + 1,
                       (b.hi[2] >> 2) - b0[2] + 1};
    const int total = nb[0] * nb[1] * nb[2];
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        const int ix = i / (nb[1] * nb[2]);
        const int r = i - ix * nb[1] * nb[2];
        const int iy = r / nb[2];
        const int iz = r - iy * nb[2];
        const uint32_t brick = ((b0[0] + ix) * g.BY + (b0[1] + iy)) * g.BZ + (b0[2] + iz);
        mark_brick(d, gi, brick);
    }
}

// Warp-aggregated counting-sort increment: bin_of/rank_of for the particle in
// `slot` (all 32 lanes call; inactive lanes pass active = false).
__device__ __forceinline__ void count_bin(const Dev& d, bool active, int slot, uint32_t key) {
    const uint32_t k = active ? key : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    const int leader = __ffs(peers) - 1;
    const unsigned lane = threadIdx.x & 31u;
    uint32_t base = 0;
    if (active && (int)lane == leader) base = atomicAdd(d.bin_count + k, (uint32_t)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (active) {
        d.bin_of[slot] = k;
        d.rank_of[slot] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
    }
}

__device__ __forceinline__ uint32_t bin_key(const Geo& g, bool reg, int bx, int by, int bz) {
    return reg ? (uint32_t)brick_of(g, bx, by, bz) : (uint32_t)g.nbricks;
}

// Clears the dirty bricks of grid gi (warp per brick, grid-stride over the
// list); the last CTA to finish resets the list.
__device__ __forceinline__ void clear_dirty(const Dev& d, int gi) {
    const uint32_t nd = __ldcg(d.dirty_n + gi);
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = warp; i < nd; i += nwarps) {
        const uint32_t b = __ldcg(d.dirty_list[gi] + i);
        int4* base = d.grid[gi] + (size_t)b * 64;
        base[lane] = make_int4(0, 0, 0, 0);
        base[lane + 32] = make_int4(0, 0, 0, 0);
        if (lane == 0) d.dirty_flag[gi][b] = 0u;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t t = atomicAdd(d.ticket, 1u);
        if (t == gridDim.x - 1) {
            d.dirty_n[gi] = 0u;
            *d.ticket = 0u;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------------------
// p2g_2 (p2g_2.wgsl:30-94) over tasks; also clears grid `cur ^ 1`.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTask) k_p2g2(Particles P, Geo g, SimConsts k, Dev d, int cur,
                                                unsigned long long* oob) {
    __shared__ __align__(16) int s_mem[4 * kArenaMax];
    __shared__ int s_box[6];
    float* s_mass = reinterpret_cast<float*>(s_mem);
    int* s_q = s_mem + kArenaMax;

    clear_dirty(d, cur ^ 1);

    int4* __restrict__ grid = d.grid[cur];
    unsigned bad = 0;
    const uint32_t ntasks = __ldcg(d.ntasks);
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const Task task = d.tasks[t];
        const bool active = (int)threadIdx.x < task.count;
        PState s;
        int bx = 0, by = 0, bz = 0;
        bool reg = false;
        if (active) {
            const int slot = (int)d.order[task.first + threadIdx.x];
            unpack_xC(P.p0[slot], P.p1[slot], P.p2[slot], s);
            base_cell(s.x, bx, by, bz);
            reg = regular_base(g, bx, by, bz);
        }
        const Box b = block_box(active && reg, bx, by, bz, s_box);
        for (int li = threadIdx.x; li < b.cells; li += blockDim.x) {
            int x, y, z;
            arena_coords(b, li, x, y, z);
            const int m = __ldcg(reinterpret_cast<const int*>(grid + brick_addr(g, x, y, z)) + 3);
            s_mass[li] = dec(m, k.fm);
            s_q[li] = 0;
            s_q[li + kArenaMax] = 0;
            s_q[li + 2 * kArenaMax] = 0;
        }
        __syncthreads();
        if (active) {
            if (reg && b.fits) {
                const int dz = b.dim[2], dyz = b.dim[1] * b.dim[2];
                const int li0 = ((bx - 1 - b.lo[0]) * b.dim[1] + (by - 1 - b.lo[1])) * dz +
                                (bz - 1 - b.lo[2]);
                p2g2_particle(
                    s, k,
                    [&](int, int gx, int gy, int gz) -> float {
                        return s_mass[li0 + gx * dyz + gy * dz + gz];
                    },
                    [&](int, int gx, int gy, int gz, int mx, int my, int mz) {
                        const int li = li0 + gx * dyz + gy * dz + gz;
                        if (mx) atomicAdd(s_q + li, mx);
                        if (my) atomicAdd(s_q + kArenaMax + li, my);
                        if (mz) atomicAdd(s_q + 2 * kArenaMax + li, mz);
                    });
            } else {
                p2g2_particle(
                    s, k,
                    [&](int idx, int, int, int) -> float {
                        if (!in_grid(g, idx)) { ++bad; return dec(0, k.fm); }
                        return dec(__ldcg(reinterpret_cast<const int*>(grid + flat_to_addr(g, idx)) + 3),
                                   k.fm);
                    },
                    [&](int idx, int, int, int, int mx, int my, int mz) {
                        if (!in_grid(g, idx)) { ++bad; return; }
                        const int a = flat_to_addr(g, idx);
                        int* c = reinterpret_cast<int*>(grid + a);
                        atomicAdd(c + 0, mx);
                        atomicAdd(c + 1, my);
                        atomicAdd(c + 2, mz);
                        mark_brick(d, cur, (uint32_t)(a >> 6));
                    });
            }
        }
        __syncthreads();
        for (int li = threadIdx.x; li < b.cells; li += blockDim.x) {
            const int q0 = s_q[li], q1 = s_q[li + kArenaMax], q2 = s_q[li + 2 * kArenaMax];
            if ((q0 | q1 | q2) == 0) continue;
            int x, y, z;
            arena_coords(b, li, x, y, z);
            int* c = reinterpret_cast<int*>(grid + brick_addr(g, x, y, z));
            if (q0) atomicAdd(c + 0, q0);
            if (q1) atomicAdd(c + 1, q1);
            if (q2) atomicAdd(c + 2, q2);
        }
        if (b.fits) mark_arena_bricks(d, g, cur, b);
        __syncthreads();
    }
    if (bad) atomicAdd(oob, (unsigned long long)bad);
}

// ---------------------------------------------------------------------------
// updateGrid + g2p + copyPosition + next p2g_1 + binning, over tasks.
// DO_G2P = false runs p2g_1 of the current positions only (first substep).
// ---------------------------------------------------------------------------
template <bool DO_G2P, bool POSVEL, bool COUNT>
__global__ void __launch_bounds__(kTask) k_g2p_p2g1(Particles P, float4* __restrict__ posvel,
                                                    Geo g, SimConsts k, Dev d, int src, int dst,
                                                    unsigned long long* oob) {
    __shared__ __align__(16) int s_mem[4 * kArenaMax];
    __shared__ int s_box[6];
    float* s_v = reinterpret_cast<float*>(s_mem);
    int* s_a = s_mem;

    const int4* __restrict__ gsrc = d.grid[src];
    int4* __restrict__ gdst = d.grid[dst];
    const int hx = wall_hi(k.real_box[0]), hy = wall_hi(k.real_box[1]),
              hz = wall_hi(k.real_box[2]);
    unsigned bad = 0;
    const uint32_t ntasks = __ldcg(d.ntasks);
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const Task task = d.tasks[t];
        const bool active = (int)threadIdx.x < task.count;
        const int slot = active ? (int)d.order[task.first + threadIdx.x] : 0;
        PState s;
        int bx = 0, by = 0, bz = 0;
        bool reg = false;
        if (DO_G2P) {
            if (active) {
                const float4 a = P.p0[slot];
                s.x[0] = a.x; s.x[1] = a.y; s.x[2] = a.z;
                base_cell(s.x, bx, by, bz);
                reg = regular_base(g, bx, by, bz);
            }
            const Box b = block_box(active && reg, bx, by, bz, s_box);
            for (int li = threadIdx.x; li < b.cells; li += blockDim.x) {
                int x, y, z;
                arena_coords(b, li, x, y, z);
                const int4 raw = __ldcg(gsrc + brick_addr(g, x, y, z));
                const int4 c = update_cell_xyz(raw, x, y, z, k, hx, hy, hz);
                s_v[li] = dec(c.x, k.fm);
                s_v[li + kArenaMax] = dec(c.y, k.fm);
                s_v[li + 2 * kArenaMax] = dec(c.z, k.fm);
            }
            __syncthreads();
            if (active) {
                if (reg && b.fits) {
                    const int dz = b.dim[2], dyz = b.dim[1] * b.dim[2];
                    const int li0 = ((bx - 1 - b.lo[0]) * b.dim[1] + (by - 1 - b.lo[1])) * dz +
                                    (bz - 1 - b.lo[2]);
                    g2p_particle(s, k, [&](int, int gx, int gy, int gz, float out[3]) {
                        const int li = li0 + gx * dyz + gy * dz + gz;
                        out[0] = s_v[li];
                        out[1] = s_v[li + kArenaMax];
                        out[2] = s_v[li + 2 * kArenaMax];
                    });
                } else {
                    g2p_particle(s, k, [&](int idx, int, int, int, float out[3]) {
                        int4 c = make_int4(0, 0, 0, 0);
                        if (in_grid(g, idx)) c = update_cell(__ldcg(gsrc + flat_to_addr(g, idx)), idx, k, hx, hy, hz);
                        else ++bad;
                        out[0] = dec(c.x, k.fm);
                        out[1] = dec(c.y, k.fm);
                        out[2] = dec(c.z, k.fm);
                    });
                }
                store_particle(P, slot, s);
                if (POSVEL) {
                    posvel[2 * (size_t)slot] = make_float4(s.x[0], s.x[1], s.x[2], 0.0f);
                    posvel[2 * (size_t)slot + 1] = make_float4(s.v[0], s.v[1], s.v[2], 0.0f);
                }
            }
            __syncthreads();  // s_v is reused as s_a below
        } else if (active) {
            load_particle(P, slot, s);
        }

        // p2g_1 of the (new) state into grid dst.
        bx = by = bz = 0;
        reg = false;
        if (active) {
            base_cell(s.x, bx, by, bz);
            reg = regular_base(g, bx, by, bz);
        }
        const Box b = block_box(active && reg, bx, by, bz, s_box);
        for (int li = threadIdx.x; li < b.cells; li += blockDim.x) {
            s_a[li] = 0;
            s_a[li + kArenaMax] = 0;
            s_a[li + 2 * kArenaMax] = 0;
            s_a[li + 3 * kArenaMax] = 0;
        }
        __syncthreads();
        if (active) {
            if (reg && b.fits) {
                const int dz = b.dim[2], dyz = b.dim[1] * b.dim[2];
                const int li0 = ((bx - 1 - b.lo[0]) * b.dim[1] + (by - 1 - b.lo[1])) * dz +
                                (bz - 1 - b.lo[2]);
                p2g1_particle(s, k, [&](int, int gx, int gy, int gz, int m, int vx, int vy, int vz) {
                    const int li = li0 + gx * dyz + gy * dz + gz;
                    if (m) atomicAdd(s_a + 3 * kArenaMax + li, m);
                    if (vx) atomicAdd(s_a + li, vx);
                    if (vy) atomicAdd(s_a + kArenaMax + li, vy);
                    if (vz) atomicAdd(s_a + 2 * kArenaMax + li, vz);
                });
            } else {
                p2g1_particle(s, k, [&](int idx, int, int, int, int m, int vx, int vy, int vz) {
                    if (!in_grid(g, idx)) { ++bad; return; }
                    const int a = flat_to_addr(g, idx);
                    int* c = reinterpret_cast<int*>(gdst + a);
                    atomicAdd(c + 3, m);
                    atomicAdd(c + 0, vx);
                    atomicAdd(c + 1, vy);
                    atomicAdd(c + 2, vz);
                    mark_brick(d, dst, (uint32_t)(a >> 6));
                });
            }
        }
        if (COUNT) count_bin(d, active, slot, bin_key(g, reg, bx, by, bz));
        __syncthreads();
        for (int li = threadIdx.x; li < b.cells; li += blockDim.x) {
            const int q0 = s_a[li], q1 = s_a[li + kArenaMax], q2 = s_a[li + 2 * kArenaMax],
                      q3 = s_a[li + 3 * kArenaMax];
            if ((q0 | q1 | q2 | q3) == 0) continue;
            int x, y, z;
            arena_coords(b, li, x, y, z);
            int* c = reinterpret_cast<int*>(gdst + brick_addr(g, x, y, z));
            if (q0) atomicAdd(c + 0, q0);
            if (q1) atomicAdd(c + 1, q1);
            if (q2) atomicAdd(c + 2, q2);
            if (q3) atomicAdd(c + 3, q3);
        }
        if (b.fits) mark_arena_bricks(d, g, dst, b);
        __syncthreads();
    }
    if (bad) atomicAdd(oob, (unsigned long long)bad);
}

// Bins the particles at their current positions (slot order).
__global__ void __launch_bounds__(kTask) k_bin(Particles P, Geo g, Dev d, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < n;
    int bx = 0, by = 0, bz = 0;
    bool reg = false;
    if (active) {
        const float4 a = P.p0[i];
        const float x[3] = {a.x, a.y, a.z};
        base_cell(x, bx, by, bz);
        reg = regular_base(g, bx, by, bz);
    }
    count_bin(d, active, active ? i : 0, bin_key(g, reg, bx, by, bz));
}

// Exclusive scan of the bin counts -> bin_start and the task list; zeroes the
// counts for the next binning.  One CTA.
__global__ void __launch_bounds__(kScanThreads) k_scan(Dev d, int nbins) {
    __shared__ uint32_t s_c[kScanThreads / 32], s_t[kScanThreads / 32];
    const int per = (nbins + kScanThreads - 1) / kScanThreads;
    const int b0 = min(nbins, (int)threadIdx.x * per), b1 = min(nbins, b0 + per);
    uint32_t sc = 0, stt = 0;
    for (int b = b0; b < b1; ++b) {
        const uint32_t c = d.bin_count[b];
        sc += c;
        stt += (c + kTask - 1) / kTask;
    }
    // block exclusive scan of (sc, stt)
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t ic = sc, it = stt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t yc = __shfl_up_sync(0xffffffffu, ic, o);
        const uint32_t yt = __shfl_up_sync(0xffffffffu, it, o);
        if ((int)lane >= o) { ic += yc; it += yt; }
    }
    if (lane == 31) { s_c[warp] = ic; s_t[warp] = it; }
    __syncthreads();
    if (warp == 0) {
        uint32_t wc = lane < kScanThreads / 32 ? s_c[lane] : 0u;
        uint32_t wt = lane < kScanThreads / 32 ? s_t[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t yc = __shfl_up_sync(0xffffffffu, wc, o);
            const uint32_t yt = __shfl_up_sync(0xffffffffu, wt, o);
            if ((int)lane >= o) { wc += yc; wt += yt; }
        }
        if (lane < kScanThreads / 32) { s_c[lane] = wc; s_t[lane] = wt; }
    }
    __syncthreads();
    uint32_t pc = ic - sc + (warp ? s_c[warp - 1] : 0u);
    uint32_t pt = it - stt + (warp ? s_t[warp - 1] : 0u);
    for (int b = b0; b < b1; ++b) {
        const uint32_t c = d.bin_count[b];
        d.bin_start[b] = pc;
        const uint32_t nt = (c + kTask - 1) / kTask;
        for (uint32_t j = 0; j < nt; ++j) {
            Task tk;
            tk.first = (int)(pc + j * kTask);
            tk.count = (int)min((uint32_t)kTask, c - j * kTask);
            d.tasks[pt + j] = tk;
        }
        pc += c;
        pt += nt;
        d.bin_count[b] = 0u;
    }
    if (threadIdx.x == kScanThreads - 1) {
        d.bin_start[nbins] = pc;
        *d.ntasks = pt;
    }
}

__global__ void k_scatter(Dev d, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    d.order[d.bin_start[d.bin_of[i]] + d.rank_of[i]] = (uint32_t)i;
}

// The last substep's grid as updateGrid left it, in the reference's layout.
__global__ void k_export(const int4* __restrict__ grid, Geo g, SimConsts k, int4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.grid_count) return;
    out[i] = update_cell(grid[flat_to_addr(g, i)], i, k, wall_hi(k.real_box[0]),
                         wall_hi(k.real_box[1]), wall_hi(k.real_box[2]));
}

}  // namespace

struct SortedEngine {
    int max_particles = 0;
    Geo geo{};
    bool configured = false;
    Dev d{};
    size_t grid_cells_alloc = 0;  // cells per grid buffer
    int bricks_alloc = 0;
    int max_tasks = 0;
    int cur = 0;          // grid holding p2g_1 of the next substep
    int last = 0;         // grid read by the last substep's g2p
    bool primed = false;
    bool has_grid = false;
    int blocks_p2g2 = 0, blocks_g2p = 0;
};

namespace {

#define SE_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) {                                             \
            g_err = std::string(#call) + ": " + cudaGetErrorString(e_);      \
            return -1;                                                       \
        }                                                                    \
    } while (0)

void free_grid_state(SortedEngine* e) {
    for (int b = 0; b < 2; ++b) {
        cudaFree(e->d.grid[b]);
        cudaFree(e->d.dirty_flag[b]);
        cudaFree(e->d.dirty_list[b]);
        e->d.grid[b] = nullptr;
        e->d.dirty_flag[b] = nullptr;
        e->d.dirty_list[b] = nullptr;
    }
    cudaFree(e->d.bin_count);
    cudaFree(e->d.bin_start);
    cudaFree(e->d.tasks);
    e->d.bin_count = e->d.bin_start = nullptr;
    e->d.tasks = nullptr;
    e->grid_cells_alloc = 0;
    e->bricks_alloc = 0;
    e->max_tasks = 0;
}

int occupancy_blocks(const void* fn) {
    int dev = 0, nsm = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kTask, 0) != cudaSuccess) return 0;
    if (per < 1) per = 1;
    return nsm * per;
}

}  // namespace

int sorted_create(SortedEngine** out, int max_particles) {
    *out = nullptr;
    SortedEngine* e = new SortedEngine();
    e->max_particles = max_particles;
    const size_t np = (size_t)(max_particles > 0 ? max_particles : 1);
    cudaError_t r = cudaMalloc(&e->d.bin_of, 4 * np);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.rank_of, 4 * np);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.order, 4 * np);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.dirty_n, 4 * 2);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.ticket, 4);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.ntasks, 4);
    if (r == cudaSuccess) {
        e->blocks_p2g2 = occupancy_blocks((const void*)k_p2g2);
        e->blocks_g2p = occupancy_blocks((const void*)k_g2p_p2g1<true, false, true>);
        if (e->blocks_p2g2 <= 0 || e->blocks_g2p <= 0) r = cudaErrorInvalidValue;
    }
    if (r != cudaSuccess) {
        g_err = std::string("sorted_create: ") + cudaGetErrorString(r);
        sorted_destroy(e);
        return -1;
    }
    *out = e;
    return 0;
}

void sorted_destroy(SortedEngine* e) {
    if (!e) return;
    free_grid_state(e);
    cudaFree(e->d.bin_of);
    cudaFree(e->d.rank_of);
    cudaFree(e->d.order);
    cudaFree(e->d.dirty_n);
    cudaFree(e->d.ticket);
    cudaFree(e->d.ntasks);
    delete e;
}

int sorted_configure(SortedEngine* e, const SimConsts& k) {
    e->configured = false;
    e->primed = false;
    e->has_grid = false;
    if (k.Y <= 0 || k.Z <= 0 || k.grid_count <= 0) return -1;
    Geo g{};
    g.Y = k.Y;
    g.Z = k.Z;
    const long long yz = (long long)k.Y * k.Z;
    if (yz > INT_MAX) return -1;
    g.YZ = (int)yz;
    g.grid_count = k.grid_count;
    g.Xi = (int)(((long long)k.grid_count + yz - 1) / yz);
    g.BX = (g.Xi + 3) / 4;
    g.BY = (g.Y + 3) / 4;
    g.BZ = (g.Z + 3) / 4;
    const long long nb = (long long)g.BX * g.BY * g.BZ;
    if (nb * 64 > INT_MAX) return -1;
    g.nbricks = (int)nb;
    const size_t cells = (size_t)nb * 64;
    const int max_tasks = e->max_particles / kTask + g.nbricks + 2;
    if (cells > e->grid_cells_alloc || g.nbricks > e->bricks_alloc || max_tasks > e->max_tasks) {
        free_grid_state(e);
        for (int b = 0; b < 2; ++b) {
            SE_CUDA(cudaMalloc(&e->d.grid[b], sizeof(int4) * cells));
            SE_CUDA(cudaMalloc(&e->d.dirty_flag[b], 4 * (size_t)g.nbricks));
            SE_CUDA(cudaMalloc(&e->d.dirty_list[b], 4 * (size_t)g.nbricks));
        }
        SE_CUDA(cudaMalloc(&e->d.bin_count, 4 * ((size_t)g.nbricks + 1)));
        SE_CUDA(cudaMalloc(&e->d.bin_start, 4 * ((size_t)g.nbricks + 2)));
        SE_CUDA(cudaMalloc(&e->d.tasks, sizeof(Task) * (size_t)max_tasks));
        e->grid_cells_alloc = cells;
        e->bricks_alloc = g.nbricks;
        e->max_tasks = max_tasks;
    }
    e->geo = g;
    e->configured = true;
    return 0;
}

void sorted_invalidate(SortedEngine* e) {
    if (!e) return;
    e->primed = false;
    e->has_grid = false;
}

bool sorted_has_grid(const SortedEngine* e) { return e && e->has_grid; }

#define LAUNCH(id, ...)          \
    do {                         \
        prof->before(st);        \
        __VA_ARGS__;             \
        prof->after((id), st);   \
    } while (0)

int sorted_step(SortedEngine* e, const Particles& P, float4* posvel, unsigned long long* oob,
                const SimConsts& k, int substeps, cudaStream_t st, LaunchProfiler* prof) {
    if (!e->configured) {
        g_err = "sorted engine is not configured for this scene";
        return -1;
    }
    const Geo& g = e->geo;
    const int n = k.n;
    const int nbins = g.nbricks + 1;
    if (n == 0 || substeps == 0) {
        if (n == 0 && substeps > 0) e->has_grid = false;
        return 0;
    }
    if (!e->primed) {
        const size_t cells = (size_t)g.nbricks * 64;
        for (int b = 0; b < 2; ++b) {
            SE_CUDA(cudaMemsetAsync(e->d.grid[b], 0, sizeof(int4) * cells, st));
            SE_CUDA(cudaMemsetAsync(e->d.dirty_flag[b], 0, 4 * (size_t)g.nbricks, st));
        }
        SE_CUDA(cudaMemsetAsync(e->d.dirty_n, 0, 8, st));
        SE_CUDA(cudaMemsetAsync(e->d.ticket, 0, 4, st));
        SE_CUDA(cudaMemsetAsync(e->d.bin_count, 0, 4 * (size_t)nbins, st));
        LAUNCH(KID_BIN, (k_bin<<<(n + kTask - 1) / kTask, kTask, 0, st>>>(P, g, e->d, n)));
        LAUNCH(KID_SCAN, (k_scan<<<1, kScanThreads, 0, st>>>(e->d, nbins)));
        LAUNCH(KID_SCATTER, (k_scatter<<<(n + 255) / 256, 256, 0, st>>>(e->d, n)));
        e->cur = 0;
        LAUNCH(KID_SORTED_P2G_1,
               (k_g2p_p2g1<false, false, false>
                <<<e->blocks_g2p, kTask, 0, st>>>(P, posvel, g, k, e->d, e->cur, e->cur, oob)));
        SE_CUDA(cudaGetLastError());
        e->primed = true;
    }
    for (int s = 0; s < substeps; ++s) {
        const int cur = e->cur, nxt = cur ^ 1;
        LAUNCH(KID_SORTED_P2G_2,
               (k_p2g2<<<e->blocks_p2g2, kTask, 0, st>>>(P, g, k, e->d, cur, oob)));
        if (s == substeps - 1)
            LAUNCH(KID_SORTED_G2P_P2G_1,
                   (k_g2p_p2g1<true, true, true>
                    <<<e->blocks_g2p, kTask, 0, st>>>(P, posvel, g, k, e->d, cur, nxt, oob)));
        else
            LAUNCH(KID_SORTED_G2P_P2G_1,
                   (k_g2p_p2g1<true, false, true>
                    <<<e->blocks_g2p, kTask, 0, st>>>(P, posvel, g, k, e->d, cur, nxt, oob)));
        LAUNCH(KID_SCAN, (k_scan<<<1, kScanThreads, 0, st>>>(e->d, nbins)));
        LAUNCH(KID_SCATTER, (k_scatter<<<(n + 255) / 256, 256, 0, st>>>(e->d, n)));
        e->last = cur;
        e->cur = nxt;
    }
    SE_CUDA(cudaGetLastError());
    e->has_grid = true;
    return 0;
}

int sorted_export_grid(SortedEngine* e, const SimConsts& k, int4* out, cudaStream_t st,
                       LaunchProfiler* prof) {
    if (!e->configured || !e->has_grid) {
        g_err = "no sorted-engine grid to export";
        return -1;
    }
    const Geo& g = e->geo;
    LAUNCH(KID_EXPORT,
           (k_export<<<(g.grid_count + 255) / 256, 256, 0, st>>>(e->d.grid[e->last], g, k, out)));
    SE_CUDA(cudaGetLastError());
    return 0;
}

const char* sorted_error() { return g_err.c_str(); }

}  // namespace mpm
