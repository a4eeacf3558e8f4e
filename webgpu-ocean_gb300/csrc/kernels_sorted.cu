// kernels_sorted.cu -- the binned, fused MLS-MPM engine.
//
// Same results as the reference's six dispatches (mls-mpm/mls-mpm.ts:245-268),
// bit for bit: every per-particle value is computed by the shared stage bodies
// of mpm_math.cuh, and the grid is an i32 sum, so the order in which
// contributions arrive does not matter.  What changes is where the work runs:
//
//  * The grid is stored brick-major: 4x4x4-cell bricks of 1 KB, contiguous,
//    with one brick of zero padding around the grid (two above it along z
//    when needed), so that every arena slot of every task addresses a stored
//    cell: padding and cells outside the reference grid are never written
//    and read as zero.
//  * Particles are counting-sorted by the bin of their base cell every
//    substep, and kept physically in that order: g2p writes each particle to
//    its position in the bin order of the other particle buffer (an id array
//    rides along), so the next substep reads nearly contiguous memory.  A bin
//    is one brick; the bins of the two bricks of an aligned z pair are
//    adjacent in the order.
//  * A task is one bin's particles, or the particles of both bins of a z
//    pair (4x4x8 cells) when together they number at most Dev::pair_max (a
//    runtime parameter, autotuned: sparse bricks then share one task's fixed
//    costs).  CTAs claim tasks from an atomic work counter and walk a task in
//    chunks of one particle per thread.  In tasks
//    of at least Dev::lane_min particles (a runtime parameter, autotuned),
//    p2g_2 first reorders the bin's particles into a lane table that puts
//    particles of 32 different shared-memory bank classes in the 32 lanes of
//    a warp (build_lane_table); g2p reuses that order.  The CTA keeps the
//    cells the task's stencils reach (its "arena") in shared memory: the
//    bin plus a one-cell halo (6x6x6 or 6x6x10 cells) for p2g_2 and g2p, plus
//    a two-cell halo (8x8x8 or 8x8x12) for the next substep's p2g_1, whose
//    particles have moved.  Gathers read the arena; scatters are shared-memory
//    i32 atomics, flushed once per task with one red.global.add per touched
//    cell and component.  Each thread owns fixed arena slots and keeps their
//    offsets (relative to the task's corner brick) in registers, so a task's
//    arena load and flush cost one add per slot.
//  * Per substep:
//      k_p2g2        p2g_2; also clears the other grid's dirty bricks
//      k_update      updateGrid over the bricks that hold contributions
//      k_g2p_p2g1    g2p + copyPosition (last substep) + the next substep's
//                    p2g_1 into the other (already cleared) grid + binning
//      k_scan, k_scatter   counting sort for the next substep
//  * Particles whose 27-cell stencil leaves the box (quirk Q1 aliasing, NaN,
//    huge coordinates) or leaves the task's arena take a global path that
//    uses the reference's flat indices directly.
//  * Batches: many independent scenes advance in the same launches.  Their
//    particles, bricks and bins are concatenated; a task belongs to one scene
//    and reads that scene's geometry and constants from a table (BATCH
//    instantiations).  The single-scene instantiations take them as kernel
//    parameters.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mpm_internal.h"
#include "mpm_math_x2.cuh"
#include "sorted_engine.h"

namespace mpm {

namespace {

// Particles per chunk == threads per CTA of the task kernels (TH below):
// 128, 256 (default) or 512, chosen per engine (sorted_set_threads) or by
// the autotuner.  Bricks at the free surface hold few particles, so smaller
// chunks leave fewer lanes idle; larger CTAs share one arena among more
// particles in flight.  Every variant asks for 1024 resident threads per SM
// (64 registers per thread); the 128-thread kernels keep one arena buffer
// instead of two so that their 8 blocks fit the SM's shared memory.
constexpr int kTask = 256;
// Arena strides: with x-stride = 16 and y-stride = 12 (mod 32) the 64 cells
// of a brick fall into 32 bank classes of exactly two cells each
// (class = (16*x + 12*y + z) mod 32 for brick-relative x, y, z).  When the
// 32 lanes of a warp hold particles of the 32 different classes (see
// build_lane_table), every stencil offset hits 32 different banks (and, for
// the float4 arena, 8 different 16-byte groups per quarter-warp), so the
// shared-memory gathers and atomics need one wavefront each.  The 8^3 arena
// uses congruent strides, so particles that stayed in their cell keep the
// property there.
constexpr int kA = 6;            // p2g_2 / g2p arena edge: brick + 1-cell halo
constexpr int kSYA = 12, kSXA = 80, kNA = kA * kSXA;
constexpr int kB = 8;            // next-p2g_1 arena edge: brick + 2-cell halo
constexpr int kSYB = 12, kSXB = 112, kNB = kB * kSXB;
constexpr int kMaxSort = 1024;   // tasks with more particles keep the bin order
// p2g_1 dirty-brick flags per task: the 3 x 3 x 4 stored bricks around a bin
// (a 4x4x8 bin's 8x8x12 arena reaches four bricks along z)
constexpr int kTouch = 36;
// Task::bin flag of a z-pair task; arena slot offset flag of the slots only
// a z-pair task's arena has (az >= 6 in the 6^3 arena, >= 8 in the 8^3 one).
constexpr int kPairBit = 1 << 30;
constexpr int kPairSlot = 1 << 30;
// Default z-pair threshold: on the 1M-particle dam-break, pairs of at most
// 512 particles gave the fastest whole run of the values tried (0, 128,
// 256, 512, all).
constexpr int kPairMaxDefault = 512;
constexpr int kPairDefaultRequest = INT_MAX;  // sorted_set_pair_max: restore the default
constexpr int kScanThreads = 1024;
// With more bin chunks (of kScanThreads bins) than this, k_chunk_sums sums
// each chunk once before k_scan.
constexpr int kChunkedScanMin = 64;
// A bin holding more than `task_cap` particles is split into tasks of at
// most task_cap particles (same brick, separate arena flushes), so that small
// scenes, whose bricks are few and full, still spread over every SM.
constexpr int kMinTaskCap = 64;
constexpr int kMaxTaskCap = 1 << 30;

// Minimum resident CTAs per SM requested from the register allocator: 1024
// threads per SM.  k_p2g2 at 4 CTAs of 256 (64 registers, some spilled to
// L1) measured ~5 % faster than at 3 on the 1M dam-break, early and late in
// the run.
// Default for Dev::lane_min: tasks with fewer particles skip the bank-class
// lane table (its barriers and position loads cost more than the bank
// conflicts it saves when a brick holds a few dozen particles) and keep the
// bin order.  The autotuner chooses it per workload.
#ifndef MPM_LANE_TABLE_MIN
#define MPM_LANE_TABLE_MIN 128
#endif
// 1: arena stage bodies use packed f32x2 products (mpm_math_x2.cuh).
#ifndef MPM_PACKED_MATH
#define MPM_PACKED_MATH 1
#endif


thread_local std::string g_err;

struct Geo {
    int Y, Z, YZ;      // flat-index strides: i32(init.y), i32(init.z)
    int grid_count;
    int Xi;            // cells along x reachable by an in-range flat index
    int BX, BY, BZ;    // bricks per axis covering the grid
    int PY, PZ;        // stored bricks along y and z (the grid's plus padding)
    int nbricks;       // stored bricks: (BX + 2) * PY * PZ
    int NZ;            // bins along z: BZ rounded up to even (z pairs)
    int nbins;         // BX * BY * NZ; bin nbins collects irregular particles and
                       // bin nbins + 1 stays empty (the scene's bins are an even count)
};

// A task: particles [first, first + count) of the bin order, all in `bin`
// (scene-local; -1: the scene's bin of irregular particles; kPairBit set:
// also in the next bin, the brick above along z) of `scene`.  (x0, y0, z0)
// is the bin's first cell; abase the int4 offset (scene-local) of the stored
// brick (x0/4 - 1, y0/4 - 1, z0/4 - 1), from which the arena slot offsets
// count.
struct __align__(16) Task {
    int first;
    int count;
    int bin;
    int scene;
    int x0, y0, z0;
    int abase;
};
// One scene of a batch: its geometry and constants, and where its bricks,
// bins and particles start in the concatenated arrays.  A scene's bins are
// its bricks followed by its irregular bin.
struct Scene {
    Geo g;
    int bbase;
    int binbase;
    int pbase;
    int lbase;   // first cell in the reference-layout concatenation of all grids
    // Batch: the index of the scene's (PY, PZ) among the batch's distinct
    // pairs.  Arena slot offsets depend on these two only, so a task kernel
    // keeps its offsets while consecutive tasks share the class; the bins
    // are laid out class by class for that reason.
    int gclass;
    SimConsts k;
};

struct Dev {
    int4* grid[2];
    float4* gv[2];       // decoded velocities of each grid's dirty bricks (k_update)
    uint32_t* dirty_flag[2];
    uint32_t* dirty_list[2];
    uint32_t* dirty_n;   // [2]
    uint32_t* ticket;    // [1]
    uint32_t* bin_of;
    uint32_t* rank_of;
    uint32_t* bin_count;  // [bins + 1]
    uint32_t* bin_start;  // [bins + 2]
    uint32_t* chunk_sum;  // [3 * chunks]: per 1024 bins, particles and multi-/single-chunk tasks
    uint32_t* order;
    Task* tasks;          // [task_slots]: multi-chunk tasks from the front, the others from the back
    uint32_t* ntasks;     // [2]: all tasks, multi-chunk tasks
    uint32_t* task_next;  // [3] work counters: p2g_2, g2p+p2g_1, first p2g_1
    // Batches only (null for one scene):
    const Scene* scenes;
    const uint32_t* brick_scene;  // global brick -> scene
    const uint32_t* bin_scene;    // global bin -> scene
    int nscenes;
    int task_cap;                 // most particles per task
    int cap_shift;                // log2(task_cap) when it is a power of two, else -1
    int chunk;                    // particles per chunk: the task kernels' block size
    int task_slots;               // entries of `tasks`
    int pair_max;                 // z pairs of at most this many particles share a task
    int lane_min;                 // tasks of at least this many particles use the lane table
};

// The scene of a task: the table entry in a batch, else the kernel's own.
template <bool BATCH>
__device__ __forceinline__ const Scene& scene_ref(const Dev& d, const Scene& one, int s) {
    if constexpr (BATCH) return d.scenes[s];
    else return one;
}
// First stored brick / bin of a scene (0 for a single scene).
template <bool BATCH>
__device__ __forceinline__ int brick_base(const Scene& s) {
    if constexpr (BATCH) return s.bbase;
    else return 0;
}
template <bool BATCH>
__device__ __forceinline__ uint32_t bin_base(const Scene& s) {
    if constexpr (BATCH) return (uint32_t)s.binbase;
    else return 0u;
}

enum { kCtrP2G2 = 0, kCtrG2P = 1, kCtrP2G1 = 2 };

// Dynamic task fetch: thread 0 claims task ids from a global counter, one
// ahead, through a two-slot shared buffer (see the loops below).
__device__ __forceinline__ int claim_task(const Dev& d, int ctr) {
    return (int)atomicAdd(d.task_next + ctr, 1u);
}

// Entry of claimed task t: the multi-chunk tasks (nbig of them, stored from
// the front) are handed out first and the single-chunk ones (stored from the
// back) last, so that the launch ends on short tasks.
__device__ __forceinline__ int task_slot(const Dev& d, int nbig, int t) {
    return t < nbig ? t : d.task_slots - 1 - (t - nbig);
}

// Cells along z of a task's region: 8 for a z pair, else 4.
__device__ __forceinline__ unsigned task_zext(const Task& t) {
    return (t.bin & kPairBit) ? 8u : 4u;
}

// Stored brick of cell (x, y, z); cells down to -4 and up to the padding's
// end along each axis have one.
__device__ __forceinline__ int brick_of(const Geo& g, int x, int y, int z) {
    return (((x >> 2) + 1) * g.PY + (y >> 2) + 1) * g.PZ + (z >> 2) + 1;
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

// Stored brick index -> brick coordinates of the grid (padding: -1 or past
// the end).
__device__ __forceinline__ void brick_coords(const Geo& g, int brick, int& x, int& y, int& z) {
    const int pyz = g.PY * g.PZ;
    x = brick / pyz;
    const int r = brick - x * pyz;
    y = r / g.PZ;
    z = r - y * g.PZ;
    x -= 1;
    y -= 1;
    z -= 1;
}

__device__ __forceinline__ void mark_brick(const Dev& d, int gi, uint32_t b) {
    if (__ldcg(d.dirty_flag[gi] + b) != 0u) return;
    if (atomicExch(d.dirty_flag[gi] + b, 1u) == 0u) {
        const uint32_t pos = atomicAdd(d.dirty_n + gi, 1u);
        d.dirty_list[gi][pos] = b;
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

__device__ __forceinline__ uint32_t bin_key(const Geo& g, uint32_t base, bool reg, int bx, int by,
                                           int bz) {
    return base + (reg ? (uint32_t)(((bx >> 2) * g.BY + (by >> 2)) * g.NZ + (bz >> 2))
                       : (uint32_t)g.nbins);
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
        float4* vbase = d.gv[gi] + (size_t)b * 64;
        vbase[lane] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        vbase[lane + 32] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
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

// int4 offset of arena slot li, counted from the stored brick (x0/4 - 1,
// y0/4 - 1, z0/4 - 1) of a task's bin at (x0, y0, z0).  The arena spans E
// cells along x and y and E + 4 along z (a z pair's) from (x0 - H, y0 - H,
// z0 - H) with strides (SX, SY, 1); slots past that extent (padding) and
// past N give -1, slots only a z pair's arena has carry kPairSlot.
template <int E, int SX, int SY, int H, int N>
__device__ __forceinline__ int slot_offset(const Geo& g, int li) {
    const int ax = li / SX;
    const int r = li - ax * SX;
    const int ay = r / SY;
    const int az = r - ay * SY;
    if (li >= N || ay >= E || az >= E + 4) return -1;
    const int tx = ax + 4 - H, ty = ay + 4 - H, tz = az + 4 - H;
    return ((((tx >> 2) * g.PY + (ty >> 2)) * g.PZ + (tz >> 2)) * 64 + ((tx & 3) << 4) +
            ((ty & 3) << 2) + (tz & 3)) |
           (az >= E ? kPairSlot : 0);
}

// The offsets of this thread's slots li = threadIdx.x + q * TH.
template <int E, int SX, int SY, int H, int N, int TH, int PER>
__device__ __forceinline__ void slot_offsets(const Geo& g, int (&off)[PER]) {
#pragma unroll
    for (int q = 0; q < PER; ++q) off[q] = slot_offset<E, SX, SY, H, N>(g, (int)threadIdx.x + q * TH);
}

// A slot the task's arena has: its offset (flag cleared), else -1.
__device__ __forceinline__ int task_offset(int off, bool pair) {
    return (off < 0 || (!pair && (off & kPairSlot))) ? -1 : (off & ~kPairSlot);
}

// Global-path mass source (flat indices, as the reference's shaders address).
struct GlobalMass {
    const Geo& g;
    const int4* grid;
    float fm;
    unsigned& bad;
    __device__ float operator()(int idx, int, int, int) const {
        if (!in_grid(g, idx)) { ++bad; return dec(0, fm); }
        return dec(__ldcg(reinterpret_cast<const int*>(grid + flat_to_addr(g, idx)) + 3), fm);
    }
};

// Async 16-byte global -> shared copies (L2 only), used to prefetch the next
// task's arena while the current task computes.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Shared-memory scratch of build_lane_table.
struct LaneTable {
    uint32_t slot[kMaxSort];    // particle slots in table order
    uint32_t key[kMaxSort];     // class | rank << 6, per particle in bin order
    uint32_t tmp[kMaxSort];     // particle slots in bin order
    int cnt[33];                // particles per bank class (32: not in the arena)
};

// Orders a bin's n particles into a table of ceil(n/32) rows of 32 lanes
// in which lane k of a row holds, where possible, a particle of bank class k
// (its base cell's class); particles of over-full classes (and particles
// outside the arena) fill the lanes that under-full classes leave empty, in
// order, and the unfilled lanes are the tail of the last row.  The table is
// written to order[first .. first + n) (g2p reuses it) and to lt.slot.
// Every thread calls it (it contains barriers).
template <int TH>
__device__ __forceinline__ void build_lane_table(const Particles& P, const Geo& g, const Dev& d,
                                                 const Task& task, LaneTable& lt) {
    const int n = task.count;
    // lt.cnt is zero here: zeroed at the kernel's start and after every table
    for (int j = threadIdx.x; j < n; j += TH) {
        const uint32_t slot = d.order[task.first + j];
        const float4 a = P.p0[slot];
        const float x[3] = {a.x, a.y, a.z};
        int bx, by, bz;
        base_cell(x, bx, by, bz);
        const int ax = bx - task.x0, ay = by - task.y0, az = bz - task.z0;
        const bool in = regular_base(g, bx, by, bz) && (unsigned)ax <= 3u && (unsigned)ay <= 3u &&
                        (unsigned)az < task_zext(task);
        const int cls = in ? ((16 * ax + 12 * ay + az) & 31) : 32;
        const int r = atomicAdd(&lt.cnt[cls], 1);
        lt.tmp[j] = slot;
        lt.key[j] = (uint32_t)cls | ((uint32_t)r << 6);
    }
    __syncthreads();
    // every warp scans the class counts itself (lane k: class k), so that no
    // warp waits for another's scan
    const unsigned full = 0xffffffffu;
    const int k = (int)(threadIdx.x & 31u);
    const int rows = (n + 31) >> 5;
    const int last = n - 32 * (rows - 1);            // lanes used in the last row
    const int v = rows - 1 + (k < last ? 1 : 0);     // rows lane k holds
    const int c = lt.cnt[k];
    const int core = min(c, v);
    const int e = v - core, o = c - core;            // empty lanes, overflow particles
    int ei = e, oi = o;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int ye = __shfl_up_sync(full, ei, off);
        const int yo = __shfl_up_sync(full, oi, off);
        if (k >= off) { ei += ye; oi += yo; }
    }
    const int empty_pre = ei - e, over_pre = oi - o;
    const int over_all = __shfl_sync(full, oi, 31);  // particles outside the arena overflow after these
    for (int base = 0; base < n; base += TH) {         // the same trip count in every warp
        const int j = base + (int)threadIdx.x;
        const bool active = j < n;
        const uint32_t key = active ? lt.key[j] : 0u;
        const int cls = (int)(key & 63u), r = (int)(key >> 6);
        const int v_c = __shfl_sync(full, v, cls & 31);
        const int op_c = __shfl_sync(full, over_pre, cls & 31);
        const bool direct = cls < 32 && r < v_c;
        const int i = cls < 32 ? op_c + (r - v_c) : over_all + r;
        int lo = 0;                                    // last lane with empty_pre <= i
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const int ep = __shfl_sync(full, empty_pre, lo + step);
            if (ep <= i) lo += step;
        }
        const int core_lo = __shfl_sync(full, core, lo);
        const int ep_lo = __shfl_sync(full, empty_pre, lo);
        const int pos = direct ? r * 32 + cls : (core_lo + (i - ep_lo)) * 32 + lo;
        if (active) {
            lt.slot[pos] = lt.tmp[j];
            d.order[task.first + pos] = lt.tmp[j];
        }
    }
    __syncthreads();
    if (threadIdx.x < 33) lt.cnt[threadIdx.x] = 0;  // every warp has read them
}

// ---------------------------------------------------------------------------
// p2g_2 (p2g_2.wgsl:30-94) over tasks; also clears grid `cur ^ 1`.
//
// One barrier per task: arenas are double-buffered.  While task i computes,
// the mass words of task i+1's arena are already loading into registers
// (decoded into the other buffer after the compute), and task i-1's momentum
// arena is flushed (each thread reads, flushes and zeroes its own slots).
// ---------------------------------------------------------------------------
template <bool BATCH, int TH>
__global__ void __launch_bounds__(TH, 1024 / TH)
    k_p2g2(Particles P, Scene one, Dev d, int cur, unsigned long long* oob) {
    constexpr bool DB = TH != 128;  // double-buffered arenas (128 threads: one, 8 blocks/SM)
    constexpr int NB = DB ? 2 : 1;
    __shared__ float s_mass[NB][kNA];
    __shared__ int s_q[NB][3][kNA];
    __shared__ int s_task[2];
    __shared__ LaneTable s_lt;
    constexpr int kPer = (kNA + TH - 1) / TH;  // arena slots per thread
    // 128 threads: this thread's slot offsets in shared memory (entry
    // [q][thread], written and read by that thread only), as in k_g2p_p2g1
    constexpr bool kTab = TH == 128;
    __shared__ int s_off[kTab ? kPer : 1][kTab ? TH : 1];
    // the task being computed (slot it & 1 of a double-buffered kernel: the
    // next task's record is written while this one computes)
    __shared__ Task s_cur[NB];

    clear_dirty(d, cur ^ 1);

    int4* __restrict__ grid_all = d.grid[cur];
    unsigned bad = 0;
    const int ntasks = (int)__ldcg(d.ntasks);
    const int nbig = (int)__ldcg(d.ntasks + 1);
    for (int i = threadIdx.x; i < NB * 3 * kNA; i += TH) (&s_q[0][0][0])[i] = 0;
    if (threadIdx.x < 33) s_lt.cnt[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        s_task[0] = claim_task(d, kCtrP2G2);
        s_task[1] = claim_task(d, kCtrP2G2);
    }

    // offsets of this thread's arena slots for geometry class off_class
    // (recomputed when a batch's task belongs to another class)
    int off_r[kTab ? 1 : kPer];
    auto set_offsets = [&](const Geo& g) {
        if constexpr (kTab) {
#pragma unroll
            for (int q = 0; q < kPer; ++q)
                s_off[q][threadIdx.x] = slot_offset<kA, kSXA, kSYA, 1, kNA>(g, (int)threadIdx.x + q * TH);
        } else {
            slot_offsets<kA, kSXA, kSYA, 1, kNA, TH, kPer>(g, off_r);
        }
    };
    auto off = [&](int q) -> int {
        if constexpr (kTab) return s_off[q][threadIdx.x];
        else return off_r[q];
    };
    int off_class = one.gclass;
    set_offsets(one.g);
    auto offsets_for = [&](int scene) {
        if (BATCH) {
            const Scene& ts = scene_ref<BATCH>(d, one, scene);
            if (ts.gclass != off_class) {
                set_offsets(ts.g);
                off_class = ts.gclass;
            }
        }
    };
    __syncthreads();

    // raw mass words of this thread's arena slots for a task, and its FM
    auto load_mass = [&](int t, int m[kPer], float& fm) {
#pragma unroll
        for (int q = 0; q < kPer; ++q) m[q] = 0;
        fm = one.k.fm;
        if (t >= ntasks) return;
        const Task tk = d.tasks[task_slot(d, nbig, t)];
        const Scene& ts = scene_ref<BATCH>(d, one, tk.scene);
        fm = ts.k.fm;
        if (tk.bin < 0) return;
        offsets_for(tk.scene);
        const int* grid = reinterpret_cast<const int*>(
            grid_all + (size_t)brick_base<BATCH>(ts) * 64 + tk.abase);
        const bool pair = (tk.bin & kPairBit) != 0;
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int o = task_offset(off(q), pair);
            if (o >= 0) m[q] = __ldcg(grid + 4 * o + 3);
        }
    };
    auto store_mass = [&](int buf, const int m[kPer], float fm) {
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int li = (int)threadIdx.x + q * TH;
            if (li < kNA) s_mass[buf][li] = dec(m[q], fm);
        }
    };
    auto flush = [&](int buf, const Task& tk) {
        if (tk.bin < 0) return;
        offsets_for(tk.scene);
        const Scene& ts = scene_ref<BATCH>(d, one, tk.scene);
        int* grid = reinterpret_cast<int*>(grid_all + (size_t)brick_base<BATCH>(ts) * 64 + tk.abase);
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int li = (int)threadIdx.x + q * TH;
            if (li >= kNA) continue;
            const int q0 = s_q[buf][0][li], q1 = s_q[buf][1][li], q2 = s_q[buf][2][li];
            if ((q0 | q1 | q2) == 0) continue;
            s_q[buf][0][li] = 0;
            s_q[buf][1][li] = 0;
            s_q[buf][2][li] = 0;
            const int oq = off(q);
            if (oq < 0) continue;  // unreachable: stencils stay inside the arena
            int* c = grid + 4 * (oq & ~kPairSlot);
            if (q0) atomicAdd(c + 0, q0);
            if (q1) atomicAdd(c + 1, q1);
            if (q2) atomicAdd(c + 2, q2);
        }
    };

    int t = s_task[0];
    if (DB) {
        int m[kPer];
        float fm;
        load_mass(t, m, fm);
        store_mass(0, m, fm);
        if (threadIdx.x == 0 && t < ntasks) s_cur[0] = d.tasks[task_slot(d, nbig, t)];
    }
    Task prev;
    prev.bin = -1;
    prev.count = 0;
    prev.scene = 0;
    bool have_prev = false;
    int it = 0;
    while (t < ntasks) {
        const int cb = it & 1;           // claim slot
        const int buf = DB ? cb : 0;     // arena buffer
        __syncthreads();  // DB: arena `buf` ready; task it-1 computed
        const int t_next = s_task[cb ^ 1];
        if (threadIdx.x == 0) s_task[cb] = claim_task(d, kCtrP2G2);
        int m_next[kPer];
        float fm_next = 0.0f;
        if (DB) {  // the next task's masses: loads issued before the flush, stored after it
            load_mass(t_next, m_next, fm_next);
            if (have_prev) flush(buf ^ 1, prev);
            store_mass(buf ^ 1, m_next, fm_next);
            if (threadIdx.x == 0 && t_next < ntasks) s_cur[buf ^ 1] = d.tasks[task_slot(d, nbig, t_next)];
        } else {  // one arena: flush task it-1's, load this task's, then wait
            if (have_prev) flush(0, prev);
            int m[kPer];
            float fm;
            load_mass(t, m, fm);
            store_mass(0, m, fm);
            if (threadIdx.x == 0) s_cur[0] = d.tasks[task_slot(d, nbig, t)];
            __syncthreads();
        }

        const Task& task = s_cur[buf];
        const Scene& sc = scene_ref<BATCH>(d, one, task.scene);
        const Geo& g = sc.g;
        const SimConsts& k = sc.k;
        const int bb = brick_base<BATCH>(sc);
        int4* __restrict__ grid = grid_all + (size_t)bb * 64;
        const bool table = task.bin >= 0 && task.count <= kMaxSort &&
                           task.count >= d.lane_min;  // uniform
        if (table) build_lane_table<TH>(P, g, d, task, s_lt);
        const unsigned zext = task_zext(task);
        for (int j = threadIdx.x; j < task.count; j += TH) {
            const int slot = table ? (int)s_lt.slot[j] : (int)d.order[task.first + j];
            PState s;
            unpack_xC(P.p0[slot], P.p1[slot], P.p2[slot], s);
            int bx, by, bz;
            base_cell(s.x, bx, by, bz);
            const int ax = bx - task.x0, ay = by - task.y0, az = bz - task.z0;
            const bool in_arena = task.bin >= 0 && regular_base(g, bx, by, bz) &&
                                  (unsigned)ax <= 3u && (unsigned)ay <= 3u && (unsigned)az < zext;
            if (in_arena) {
                // stencil corner (base - 1) relative to the arena origin (bin - 1)
                const int li0 = ax * kSXA + ay * kSYA + az;
                auto mass = [&](int gx, int gy, int gz) -> float {
                    return s_mass[buf][li0 + gx * kSXA + gy * kSYA + gz];
                };
                auto sink = [&](int gx, int gy, int gz, int mx, int my, int mz) {
                    const int li = li0 + gx * kSXA + gy * kSYA + gz;
                    atomicAdd(&s_q[buf][0][li], mx);
                    atomicAdd(&s_q[buf][1][li], my);
                    atomicAdd(&s_q[buf][2][li], mz);
                };
                if (MPM_PACKED_MATH) {
                    p2g2_particle_x2(s, k, mass, sink);
                } else {
                    p2g2_particle(
                        s, k, [&](int, int gx, int gy, int gz) { return mass(gx, gy, gz); },
                        [&](int, int gx, int gy, int gz, int mx, int my, int mz) {
                            sink(gx, gy, gz, mx, my, mz);
                        });
                }
            } else {
                p2g2_particle(
                    s, k, GlobalMass{g, grid, k.fm, bad},
                    [&](int idx, int, int, int, int mx, int my, int mz) {
                        if (!in_grid(g, idx)) { ++bad; return; }
                        const int a = flat_to_addr(g, idx);
                        int* c = reinterpret_cast<int*>(grid + a);
                        atomicAdd(c + 0, mx);
                        atomicAdd(c + 1, my);
                        atomicAdd(c + 2, mz);
                        mark_brick(d, cur, (uint32_t)(bb + (a >> 6)));
                    });
            }
        }
        prev = task;
        have_prev = true;
        t = t_next;
        ++it;
    }
    __syncthreads();
    if (have_prev) flush(DB ? (it - 1) & 1 : 0, prev);
    if (bad) atomicAdd(oob, (unsigned long long)bad);
}

// ---------------------------------------------------------------------------
// updateGrid (updateGrid.wgsl:23-46) on the dirty bricks of grid `cur`, in
// place, warp per brick, two cells per lane.  Also writes every cell of
// those bricks, decoded, to the float velocity grid g2p reads:
// (dec(vx), dec(vy), dec(vz), dec(vz)).
// ---------------------------------------------------------------------------
template <bool BATCH>
__global__ void __launch_bounds__(256) k_update(Scene one, Dev d, int cur) {
    const uint32_t nd = __ldcg(d.dirty_n + cur);
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    int4* __restrict__ grid = d.grid[cur];
    float4* __restrict__ gv = d.gv[cur];
    for (uint32_t i = warp; i < nd; i += nwarps) {
        const int b = (int)__ldcg(d.dirty_list[cur] + i);  // global brick
        const Scene& sc = scene_ref<BATCH>(d, one, BATCH ? (int)__ldg(d.brick_scene + b) : 0);
        const SimConsts& k = sc.k;
        const int hx = wall_hi(k.real_box[0]), hy = wall_hi(k.real_box[1]),
                  hz = wall_hi(k.real_box[2]);
        int bx, by, bz;
        brick_coords(sc.g, b - brick_base<BATCH>(sc), bx, by, bz);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int c = (int)lane + 32 * h;
            const size_t a = (size_t)b * 64 + c;
            int4 u = grid[a];
            if (u.w > 0) {
                const int x = 4 * bx + (c >> 4), y = 4 * by + ((c >> 2) & 3), z = 4 * bz + (c & 3);
                u = update_cell_xyz(u, x, y, z, k, hx, hy, hz);
                grid[a] = u;
            }
            const float vz = dec(u.z, k.fm);
            gv[a] = make_float4(dec(u.x, k.fm), dec(u.y, k.fm), vz, vz);
        }
    }
}

// ---------------------------------------------------------------------------
// g2p + copyPosition + next p2g_1 + binning, over tasks.  Reads particles
// from Pin through the bin order and writes them, in bin order, to Pout.
// DO_G2P = false runs p2g_1 of the current positions only (first substep;
// Pout is not written).
//
// One barrier per task: while task i computes, task i+1's g2p arena is
// copied in with cp.async and task i-1's p2g_1 arena is flushed (each thread
// reads, flushes and zeroes its own slots); the bricks task i-1's stencils
// reached are registered as dirty right after the barrier.
// ---------------------------------------------------------------------------
template <bool BATCH, bool DO_G2P, bool POSVEL, int TH>
__global__ void __launch_bounds__(TH, 1024 / TH)
    k_g2p_p2g1(Particles Pin, Particles Pout, const uint32_t* __restrict__ id_in,
               uint32_t* __restrict__ id_out, float4* __restrict__ posvel, Scene one, Dev d,
               int src, int dst, unsigned long long* oob) {
    constexpr bool DB = TH != 128;  // double-buffered arenas (128 threads: one, 8 blocks/SM)
    constexpr int NB = DB ? 2 : 1;
    __shared__ __align__(16) float4 s_v[DO_G2P ? NB : 1][DO_G2P ? kNA : 1];
    __shared__ int s_a[NB][4][kNB];
    __shared__ int s_touch[NB][kTouch];
    __shared__ int s_task[2];
    constexpr int kPerA = DO_G2P ? (kNA + TH - 1) / TH : 1;  // g2p arena slots per thread
    constexpr int kPerB = (kNB + TH - 1) / TH;                // p2g_1 arena slots per thread
    // 128 threads (one arena): the offsets of each thread's arena slots live
    // in shared memory (entry [q][thread], written and read by that thread
    // only) for the geometry class of the last task, which frees registers;
    // the larger blocks keep the g2p offsets in registers and compute the
    // p2g_1 ones at the flush (their spills grew with the tables).
    constexpr bool kTab = TH == 128;
    __shared__ int s_offB[kTab ? kPerB : 1][kTab ? TH : 1];
    __shared__ int s_offA[kTab ? kPerA : 1][kTab ? TH : 1];
    // the task being computed, read from shared memory (slot it & 1 of a
    // double-buffered kernel: the next task's record is written while this
    // one computes); a single scene's 128-thread kernel keeps it in
    // registers (it spilled more with it)
    constexpr bool kCur = BATCH || DB;
    __shared__ Task s_cur[kCur ? NB : 1];

    const float4* __restrict__ gv_all = d.gv[src];
    int4* __restrict__ gdst_all = d.grid[dst];
    const int ctr = DO_G2P ? kCtrG2P : kCtrP2G1;
    unsigned bad = 0;
    const int ntasks = (int)__ldcg(d.ntasks);
    const int nbig = (int)__ldcg(d.ntasks + 1);
    for (int i = threadIdx.x; i < NB * 4 * kNB; i += TH) (&s_a[0][0][0])[i] = 0;
    if (threadIdx.x < NB * kTouch) (&s_touch[0][0])[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        s_task[0] = claim_task(d, ctr);
        s_task[1] = claim_task(d, ctr);
    }

    // offsets of this thread's arena slots for geometry class off_class /
    // offB_class (recomputed when a batch's task belongs to another class)
    int offA[kTab ? 1 : kPerA];
    int off_class = one.gclass;
    auto offsetsA = [&](const Geo& g) {
        if constexpr (kTab) {
#pragma unroll
            for (int q = 0; q < kPerA; ++q)
                s_offA[q][threadIdx.x] = slot_offset<kA, kSXA, kSYA, 1, kNA>(g, (int)threadIdx.x + q * TH);
        } else {
            slot_offsets<kA, kSXA, kSYA, 1, kNA, TH, kPerA>(g, offA);
        }
    };
    auto offA_at = [&](int q) -> int {
        if constexpr (kTab) return s_offA[q][threadIdx.x];
        else return offA[q];
    };
    if (DO_G2P) offsetsA(one.g);
    int offB_class = one.gclass;
    auto offsetsB = [&](const Geo& g) {
        if constexpr (kTab) {
#pragma unroll
            for (int q = 0; q < kPerB; ++q)
                s_offB[q][threadIdx.x] = slot_offset<kB, kSXB, kSYB, 2, kNB>(g, (int)threadIdx.x + q * TH);
        }
    };
    offsetsB(one.g);
    auto offsets_for = [&](int scene) {
        if (BATCH && DO_G2P) {
            const Scene& ts = scene_ref<BATCH>(d, one, scene);
            if (ts.gclass != off_class) {
                offsetsA(ts.g);
                off_class = ts.gclass;
            }
        }
    };
    __syncthreads();

    // g2p arena of task t (velocities decoded by k_update) into s_v[buf]
    auto prefetch = [&](int t, int buf) {
        if (!DO_G2P || t >= ntasks) return;
        const Task tk = d.tasks[task_slot(d, nbig, t)];
        if (tk.bin < 0) return;
        offsets_for(tk.scene);
        const Scene& ts = scene_ref<BATCH>(d, one, tk.scene);
        const float4* gvsrc = gv_all + (size_t)brick_base<BATCH>(ts) * 64 + tk.abase;
        const bool pair = (tk.bin & kPairBit) != 0;
#pragma unroll
        for (int q = 0; q < kPerA; ++q) {
            const int o = task_offset(offA_at(q), pair);
            if (o >= 0) cp_async16(&s_v[buf][(int)threadIdx.x + q * TH], gvsrc + o);
        }
        cp_async_commit();
    };
    // flush the p2g_1 arena of task tk
    auto flush = [&](int buf, const Task& tk) {
        const Scene& ts = scene_ref<BATCH>(d, one, tk.scene);
        if (kTab && BATCH && ts.gclass != offB_class) {
            offsetsB(ts.g);
            offB_class = ts.gclass;
        }
        int* gdst = reinterpret_cast<int*>(gdst_all + (size_t)brick_base<BATCH>(ts) * 64 + tk.abase);
#pragma unroll
        for (int q = 0; q < kPerB; ++q) {
            const int li = (int)threadIdx.x + q * TH;
            if (li >= kNB) continue;
            const int q0 = s_a[buf][0][li], q1 = s_a[buf][1][li], q2 = s_a[buf][2][li],
                      q3 = s_a[buf][3][li];
            if ((q0 | q1 | q2 | q3) == 0) continue;
            s_a[buf][0][li] = 0;
            s_a[buf][1][li] = 0;
            s_a[buf][2][li] = 0;
            s_a[buf][3][li] = 0;
            const int o = kTab ? s_offB[q][threadIdx.x] : slot_offset<kB, kSXB, kSYB, 2, kNB>(ts.g, li);
            if (o < 0) continue;  // unreachable: stencils stay inside the arena
            int* c = gdst + 4 * (o & ~kPairSlot);
            if (q0) atomicAdd(c + 0, q0);
            if (q1) atomicAdd(c + 1, q1);
            if (q2) atomicAdd(c + 2, q2);
            if (q3) atomicAdd(c + 3, q3);
        }
    };
    // register the stored bricks flagged in s_touch[buf]: flag
    // (kx * 3 + ky) * 4 + kz is brick (x0/4 - 1 + kx, y0/4 - 1 + ky, z0/4 - 1 + kz)
    auto mark = [&](int buf, const Task& tk) {
        if (threadIdx.x < kTouch && s_touch[buf][threadIdx.x]) {
            const int i = threadIdx.x;
            const Scene& ts = scene_ref<BATCH>(d, one, tk.scene);
            const int kx = (i >> 2) / 3, ky = (i >> 2) - 3 * kx, kz = i & 3;
            const int off = (kx * ts.g.PY + ky) * ts.g.PZ + kz;
            mark_brick(d, dst, (uint32_t)(brick_base<BATCH>(ts) + (tk.abase >> 6) + off));
            s_touch[buf][i] = 0;
        }
    };

    int t = s_task[0];
    if (DB) {
        prefetch(t, 0);
        if (threadIdx.x == 0 && t < ntasks) s_cur[0] = d.tasks[task_slot(d, nbig, t)];
    }
    bool have_prev = false;
    Task prev;
    prev.bin = -1;
    prev.scene = 0;
    int it = 0;
    while (t < ntasks) {
        const int cb = it & 1;           // claim slot
        const int buf = DB ? cb : 0;     // arena buffer
        if (DB && DO_G2P) cp_async_wait_all();
        __syncthreads();  // DB: s_v[buf] arrived; task it-1 computed everywhere
        const int t_next = s_task[cb ^ 1];
        if (threadIdx.x == 0) s_task[cb] = claim_task(d, ctr);
        if (DB) {
            if (have_prev && prev.bin >= 0) mark(buf ^ 1, prev);
            prefetch(t_next, buf ^ 1);
            if (have_prev && prev.bin >= 0) flush(buf ^ 1, prev);
            if (threadIdx.x == 0 && t_next < ntasks) s_cur[buf ^ 1] = d.tasks[task_slot(d, nbig, t_next)];
        } else {  // one arena: flush task it-1's, copy in this task's, then wait
            if (have_prev && prev.bin >= 0) {
                mark(0, prev);
                flush(0, prev);
            }
            prefetch(t, 0);
            if (kCur && threadIdx.x == 0) s_cur[0] = d.tasks[task_slot(d, nbig, t)];
            if (DO_G2P) cp_async_wait_all();
            __syncthreads();
        }

        Task task_r;
        if (!kCur) task_r = d.tasks[task_slot(d, nbig, t)];
        const Task& task = kCur ? s_cur[buf] : task_r;
        const Scene& sc = scene_ref<BATCH>(d, one, task.scene);
        const Geo& g = sc.g;
        const SimConsts& k = sc.k;
        const int bb = brick_base<BATCH>(sc);
        const uint32_t binb = bin_base<BATCH>(sc);
        const float4* __restrict__ gvsrc = gv_all + (size_t)bb * 64;
        int4* __restrict__ gdst = gdst_all + (size_t)bb * 64;
        const unsigned zext = task_zext(task);
        for (int base = 0; base < task.count; base += TH) {
            const bool active = base + (int)threadIdx.x < task.count;
            const int jo = task.first + base + (active ? (int)threadIdx.x : 0);  // bin order
            const int slot = active ? (int)d.order[jo] : 0;
            PState s;
            if (DO_G2P) {
                if (active) {
                    const float4 a = Pin.p0[slot];
                    s.x[0] = a.x; s.x[1] = a.y; s.x[2] = a.z;
                    int bx, by, bz;
                    base_cell(s.x, bx, by, bz);
                    const int ax = bx - task.x0, ay = by - task.y0, az = bz - task.z0;
                    const bool in_arena = task.bin >= 0 && regular_base(g, bx, by, bz) &&
                                          (unsigned)ax <= 3u && (unsigned)ay <= 3u &&
                                          (unsigned)az < zext;
                    if (in_arena) {
                        const int li0 = ax * kSXA + ay * kSYA + az;
                        const float4* sv = s_v[DO_G2P ? buf : 0];
                        if (MPM_PACKED_MATH) {
                            g2p_particle_x2(s, k, [&](int gx, int gy, int gz, f2& gxy, f2& gzz) {
                                const float4 v = sv[li0 + gx * kSXA + gy * kSYA + gz];
                                gxy = pk(v.x, v.y);
                                gzz = pk(v.z, v.w);
                            });
                        } else {
                            g2p_particle(s, k, [&](int, int gx, int gy, int gz, float out[3]) {
                                const float4 v = sv[li0 + gx * kSXA + gy * kSYA + gz];
                                out[0] = v.x;
                                out[1] = v.y;
                                out[2] = v.z;
                            });
                        }
                    } else {
                        g2p_particle(s, k, [&](int idx, int, int, int, float out[3]) {
                            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                            if (in_grid(g, idx)) v = __ldcg(gvsrc + flat_to_addr(g, idx));
                            else ++bad;
                            out[0] = v.x;
                            out[1] = v.y;
                            out[2] = v.z;
                        });
                    }
                    store_particle(Pout, jo, s);
                    const uint32_t pid = id_in[slot];
                    id_out[jo] = pid;
                    if (POSVEL) {
                        posvel[2 * (size_t)pid] = make_float4(s.x[0], s.x[1], s.x[2], 0.0f);
                        posvel[2 * (size_t)pid + 1] = make_float4(s.v[0], s.v[1], s.v[2], 0.0f);
                    }
                }
            } else if (active) {
                load_particle(Pin, slot, s);
            }

            // p2g_1 of the (new) state into grid dst, arena = bin + 2-cell halo.
            int bx = 0, by = 0, bz = 0;
            bool reg = false;
            if (active) {
                base_cell(s.x, bx, by, bz);
                reg = regular_base(g, bx, by, bz);
                const int ax = bx + 1 - task.x0, ay = by + 1 - task.y0, az = bz + 1 - task.z0;
                const bool in_arena = task.bin >= 0 && reg && (unsigned)ax <= (unsigned)(kB - 3) &&
                                      (unsigned)ay <= (unsigned)(kB - 3) &&
                                      (unsigned)az <= zext + 1u;
                if (in_arena) {
                    const int li0 = ax * kSXB + ay * kSYB + az;
                    auto sink = [&](int gx, int gy, int gz, int m, int vx, int vy, int vz) {
                        const int li = li0 + gx * kSXB + gy * kSYB + gz;
                        atomicAdd(&s_a[buf][3][li], m);
                        atomicAdd(&s_a[buf][0][li], vx);
                        atomicAdd(&s_a[buf][1][li], vy);
                        atomicAdd(&s_a[buf][2][li], vz);
                    };
                    if (MPM_PACKED_MATH) {
                        p2g1_particle_x2(s, k, sink);
                    } else {
                        p2g1_particle(s, k,
                                      [&](int, int gx, int gy, int gz, int m, int vx, int vy,
                                          int vz) { sink(gx, gy, gz, m, vx, vy, vz); });
                    }
                    // bricks the stencil (base-1 .. base+1) reaches, from the bin's corner brick
                    const int cx = (task.x0 >> 2) - 1, cy = (task.y0 >> 2) - 1,
                              cz = (task.z0 >> 2) - 1;
                    const int x0 = ((bx - 1) >> 2) - cx, x1 = ((bx + 1) >> 2) - cx;
                    const int y0 = ((by - 1) >> 2) - cy, y1 = ((by + 1) >> 2) - cy;
                    const int z0 = ((bz - 1) >> 2) - cz, z1 = ((bz + 1) >> 2) - cz;
                    for (int xx = x0; xx <= x1; ++xx)
                        for (int yy = y0; yy <= y1; ++yy)
                            for (int zz = z0; zz <= z1; ++zz)
                                s_touch[buf][(xx * 3 + yy) * 4 + zz] = 1;
                } else {
                    p2g1_particle(s, k,
                                  [&](int idx, int, int, int, int m, int vx, int vy, int vz) {
                                      if (!in_grid(g, idx)) { ++bad; return; }
                                      const int a = flat_to_addr(g, idx);
                                      int* c = reinterpret_cast<int*>(gdst + a);
                                      atomicAdd(c + 3, m);
                                      atomicAdd(c + 0, vx);
                                      atomicAdd(c + 1, vy);
                                      atomicAdd(c + 2, vz);
                                      mark_brick(d, dst, (uint32_t)(bb + (a >> 6)));
                                  });
                }
            }
            if (DO_G2P) count_bin(d, active, jo, bin_key(g, binb, reg, bx, by, bz));
        }
        have_prev = true;
        prev = task;
        t = t_next;
        ++it;
    }
    __syncthreads();
    if (have_prev && prev.bin >= 0) {
        mark(DB ? (it - 1) & 1 : 0, prev);
        flush(DB ? (it - 1) & 1 : 0, prev);
    }
    if (bad) atomicAdd(oob, (unsigned long long)bad);
}

// Bins the particles at their current positions (slot order).  In a batch
// the scene of slot i is found by bisecting the scenes' first particles.
template <bool BATCH>
__global__ void __launch_bounds__(kTask) k_bin(Particles P, Scene one, Dev d, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < n;
    int s = 0;
    if (BATCH && active) {
        int lo = 0, hi = d.nscenes - 1;  // last scene with pbase <= i
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (d.scenes[mid].pbase <= i) lo = mid;
            else hi = mid - 1;
        }
        s = lo;
    }
    const Scene& sc = scene_ref<BATCH>(d, one, s);
    int bx = 0, by = 0, bz = 0;
    bool reg = false;
    if (active) {
        const float4 a = P.p0[i];
        const float x[3] = {a.x, a.y, a.z};
        base_cell(x, bx, by, bz);
        reg = regular_base(sc.g, bx, by, bz);
    }
    count_bin(d, active, active ? i : 0, bin_key(sc.g, bin_base<BATCH>(sc), reg, bx, by, bz));
}

// Exclusive scan of the bin counts -> bin_start and the task list: one task
// per non-empty bin, or several when it holds more than task_cap particles;
// tasks of more than one chunk are stored from the front of the list, the
// others from the back (task_slot).  one_g is a single scene's geometry;
// batches read theirs from the table.  CTA c scans bins [c*1024,
// (c+1)*1024); it finds its starting offsets by reducing all earlier counts
// itself (a few KB to a few hundred KB from L2), so no CTA waits on another.
// The counts are zeroed by k_scatter, which runs next.

// Block-wide exclusive scan of N values per thread, in place; tot gets the
// block's totals.  s: 32 * N words of shared scratch.
template <int N>
__device__ __forceinline__ void block_scan(uint32_t (&v)[N], uint32_t (&tot)[N], uint32_t* s) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t inc[N];
#pragma unroll
    for (int k = 0; k < N; ++k) inc[k] = v[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc[k], o);
            if ((int)lane >= o) inc[k] += y;
        }
    }
    if (lane == 31) {
#pragma unroll
        for (int k = 0; k < N; ++k) s[k * 32 + warp] = inc[k];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            uint32_t w = s[k * 32 + lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if ((int)lane >= o) w += y;
            }
            s[k * 32 + lane] = w;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) {
        tot[k] = s[k * 32 + 31];
        v[k] = inc[k] - v[k] + (warp ? s[k * 32 + warp - 1] : 0u);
    }
}

// Full tasks (task_cap particles) of a bin of c particles, and the rest.
__device__ __forceinline__ void bin_split(const Dev& d, uint32_t c, uint32_t& full, uint32_t& rem) {
    const uint32_t cap = (uint32_t)d.task_cap;
    full = d.cap_shift >= 0 ? c >> d.cap_shift : c / cap;
    rem = c - full * cap;
}

// Tasks of a bin of c particles: those of more than one chunk, and the others.
__device__ __forceinline__ void bin_tasks(const Dev& d, uint32_t c, uint32_t& big, uint32_t& small) {
    uint32_t full, rem;
    bin_split(d, c, full, rem);
    const uint32_t th = (uint32_t)d.chunk;
    const bool cap_big = (uint32_t)d.task_cap > th;
    big = (cap_big ? full : 0u) + (rem > th ? 1u : 0u);
    small = (cap_big ? 0u : full) + (rem != 0u && rem <= th ? 1u : 0u);
}

// The bins of a z pair (c0 and c1 particles) share one task: both hold
// particles and together at most pair_max and task_cap.  A scene's irregular
// bin is paired with its always-empty last bin, so it never merges.
__device__ __forceinline__ bool pair_merges(const Dev& d, uint32_t c0, uint32_t c1) {
    const uint32_t c = c0 + c1;
    return c0 != 0u && c1 != 0u && c <= (uint32_t)d.pair_max && c <= (uint32_t)d.task_cap;
}

// Tasks of the z pair of bins (c0, c1 particles), as bin_tasks.
__device__ __forceinline__ void pair_tasks(const Dev& d, uint32_t c0, uint32_t c1, uint32_t& big,
                                           uint32_t& small) {
    if (pair_merges(d, c0, c1)) {
        const bool b = c0 + c1 > (uint32_t)d.chunk;
        big = b ? 1u : 0u;
        small = b ? 0u : 1u;
        return;
    }
    uint32_t b0, s0, b1, s1;
    bin_tasks(d, c0, b0, s0);
    bin_tasks(d, c1, b1, s1);
    big = b0 + b1;
    small = s0 + s1;
}

// Sum of a range of bins' particles and tasks (four bins, two z pairs,
// per uint4), reduced over the block into pre[] (every thread gets it).
__device__ __forceinline__ void sum_bins(const Dev& d, int b0, int b1, uint32_t (&pre)[3],
                                         uint32_t* s_scan) {
    pre[0] = pre[1] = pre[2] = 0u;
    const uint4* c4 = reinterpret_cast<const uint4*>(d.bin_count) + b0 / 4;
    const int n4 = (b1 - b0) / 4;
    constexpr int kU = 8;  // loads in flight per thread
    for (int i0 = 0; i0 < n4; i0 += kU * kScanThreads) {
        uint4 q[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const int i = i0 + u * kScanThreads + (int)threadIdx.x;
            q[u] = i < n4 ? __ldcg(c4 + i) : make_uint4(0u, 0u, 0u, 0u);
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {  // two z pairs each
            uint32_t bg, sm;
            pair_tasks(d, q[u].x, q[u].y, bg, sm);
            pre[1] += bg;
            pre[2] += sm;
            pair_tasks(d, q[u].z, q[u].w, bg, sm);
            pre[1] += bg;
            pre[2] += sm;
            pre[0] += q[u].x + q[u].y + q[u].z + q[u].w;
        }
    }
    uint32_t tot[3];
    block_scan<3>(pre, tot, s_scan);
    pre[0] = tot[0];
    pre[1] = tot[1];
    pre[2] = tot[2];
}

// Per-chunk sums for k_scan when there are many chunks (otherwise each
// k_scan CTA reduces all earlier bins itself, which costs a quadratic
// number of reads).  The bin counts beyond nbins are zero.
__global__ void __launch_bounds__(kScanThreads) k_chunk_sums(Dev d) {
    __shared__ uint32_t s_scan[3 * 32];
    uint32_t pre[3];
    sum_bins(d, blockIdx.x * kScanThreads, (blockIdx.x + 1) * kScanThreads, pre, s_scan);
    if (threadIdx.x < 3) d.chunk_sum[3 * blockIdx.x + threadIdx.x] = pre[threadIdx.x];
}

// chunked: k_chunk_sums ran before (chunk_sum holds every chunk's sums).
__global__ void __launch_bounds__(kScanThreads) k_scan(Dev d, Geo one_g, int nbins, int chunked) {
    __shared__ uint32_t s_scan[3 * 32];
    const int base = blockIdx.x * kScanThreads;
    // counts of all bins before this CTA's range (particles, big and small tasks)
    uint32_t pre[3] = {0u, 0u, 0u};
    if (chunked) {
        for (int c = threadIdx.x; c < (int)blockIdx.x; c += kScanThreads)
#pragma unroll
            for (int k = 0; k < 3; ++k) pre[k] += __ldcg(d.chunk_sum + 3 * c + k);
        uint32_t tot[3];
        block_scan<3>(pre, tot, s_scan);
        pre[0] = tot[0];
        pre[1] = tot[1];
        pre[2] = tot[2];
    } else {
        sum_bins(d, 0, base, pre, s_scan);
    }
    __syncthreads();  // s_scan reused below
    const int bin = base + (int)threadIdx.x;
    const uint32_t c = bin < nbins ? __ldcg(d.bin_count + bin) : 0u;
    const uint32_t cpart = __shfl_xor_sync(0xffffffffu, c, 1);  // the other bin of the z pair
    const bool lead = (bin & 1) == 0;
    const bool merged = pair_merges(d, c, cpart);
    uint32_t v[3], tot[3];
    v[0] = c;
    if (merged) {  // the pair's task belongs to its first bin
        const bool b = c + cpart > (uint32_t)d.chunk;
        v[1] = lead && b ? 1u : 0u;
        v[2] = lead && !b ? 1u : 0u;
    } else {
        bin_tasks(d, c, v[1], v[2]);
    }
    block_scan<3>(v, tot, s_scan);
    if (bin < nbins) {
        const uint32_t start = pre[0] + v[0];
        d.bin_start[bin] = start;
        if (c && (lead || !merged)) {
            Task tk;
            tk.scene = d.bin_scene ? (int)__ldg(d.bin_scene + bin) : 0;
            const Geo& g = d.bin_scene ? d.scenes[tk.scene].g : one_g;
            const int local = d.bin_scene ? bin - d.scenes[tk.scene].binbase : bin;
            tk.bin = local == g.nbins ? -1 : local;
            tk.x0 = tk.y0 = tk.z0 = tk.abase = 0;
            if (tk.bin >= 0) {
                const int byz = g.BY * g.NZ;
                const int bx = local / byz;
                const int r = local - bx * byz;
                const int by = r / g.NZ;
                const int bz = r - by * g.NZ;
                tk.x0 = 4 * bx;
                tk.y0 = 4 * by;
                tk.z0 = 4 * bz;
                tk.abase = ((bx * g.PY + by) * g.PZ + bz) * 64;
            }
            uint32_t full, rem;
            if (merged) {
                tk.bin |= kPairBit;
                full = 0u;
                rem = c + cpart;
            } else {
                bin_split(d, c, full, rem);
            }
            const uint32_t cap = (uint32_t)d.task_cap;
            uint32_t jb = pre[1] + v[1], js = pre[2] + v[2];
            for (uint32_t q = 0; q < full + (rem ? 1u : 0u); ++q) {
                tk.first = (int)(start + q * cap);
                tk.count = (int)(q < full ? cap : rem);
                const int slot = tk.count > d.chunk ? (int)jb++ : d.task_slots - 1 - (int)js++;
                d.tasks[slot] = tk;
            }
        }
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        d.bin_start[nbins] = pre[0] + tot[0];
        d.ntasks[0] = pre[1] + tot[1] + pre[2] + tot[2];
        d.ntasks[1] = pre[1] + tot[1];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) d.task_next[0] = d.task_next[1] = d.task_next[2] = 0u;
}

// order[] from bin_start/bin_of/rank_of; also zeroes the bin counts for the
// next binning.
__global__ void k_scatter(Dev d, int n, int nbins) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nbins) d.bin_count[i] = 0u;
    if (i >= n) return;
    d.order[d.bin_start[d.bin_of[i]] + d.rank_of[i]] = (uint32_t)i;
}

// The last substep's grid (already updated in place) in the reference's
// x-major layout.
__global__ void k_export(const int4* __restrict__ grid, Geo g, int4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.grid_count) return;
    out[i] = grid[flat_to_addr(g, i)];
}

// The same for every scene of a batch, into the concatenation of their
// reference-layout grids (scene s at lbase): block row y exports scene
// s0 + y.
__global__ void k_export_scenes(const int4* __restrict__ grid, Dev d, int s0,
                                int4* __restrict__ out) {
    const Scene& sc = d.scenes[s0 + (int)blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.g.grid_count) return;
    out[sc.lbase + i] = grid[(size_t)sc.bbase * 64 + flat_to_addr(sc.g, i)];
}

}  // namespace

// A captured run of substeps and the engine state it starts from / ends in.
struct GraphEntry {
    int substeps = 0;
    int cur0 = 0, pcur0 = 0;     // e->cur, ps->cur before
    float4* posvel = nullptr;
    unsigned long long* oob = nullptr;
    int cur1 = 0, last1 = 0, pcur1 = 0;
    long long launches[KID_COUNT] = {};
    cudaGraphExec_t exec = nullptr;
};

struct SortedEngine {
    int max_particles = 0;
    bool configured = false;
    bool batch = false;
    Scene one{};                 // the scene (single) or scene 0 (batch)
    std::vector<Scene> scenes;   // batch: host copy of the table
    int nbins = 0;               // all scenes' bins
    int nbricks = 0;             // all scenes' bricks
    Dev d{};
    Scene* scenes_d = nullptr;
    uint32_t* brick_scene_d = nullptr;
    uint32_t* bin_scene_d = nullptr;
    size_t grid_cells_alloc = 0;  // cells per grid buffer
    int bricks_alloc = 0;
    int max_tasks = 0;
    int cur = 0;          // grid holding p2g_1 of the next substep
    int last = 0;         // grid read by the last substep's g2p
    bool primed = false;
    bool has_grid = false;
    int blocks_update = 0;
    int blocks_p2g2_v[3] = {0, 0, 0}, blocks_g2p_v[3] = {0, 0, 0};  // 128, 256, 512 threads
    int threads = kTask;         // CTA size of the task kernels
    int variant() const { return threads == 128 ? 0 : (threads == 512 ? 2 : 1); }
    int blocks_p2g2() const { return blocks_p2g2_v[variant()]; }
    int blocks_g2p() const { return blocks_g2p_v[variant()]; }
    int task_cap = kMaxSort;     // most particles per task (see kMinTaskCap)
    bool task_cap_auto = true;   // task_cap follows the particle count
    int ncells_linear = 0;       // batch: cells of all scenes' reference-layout grids
    int max_scene_cells = 0;     // batch: most cells of one scene's reference-layout grid
    std::vector<GraphEntry> graphs;
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

void drop_graphs(SortedEngine* e) {
    for (GraphEntry& g : e->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    e->graphs.clear();
}

void free_grid_state(SortedEngine* e) {
    drop_graphs(e);
    for (int b = 0; b < 2; ++b) {
        cudaFree(e->d.gv[b]);
        e->d.gv[b] = nullptr;
        cudaFree(e->d.grid[b]);
        cudaFree(e->d.dirty_flag[b]);
        cudaFree(e->d.dirty_list[b]);
        e->d.grid[b] = nullptr;
        e->d.dirty_flag[b] = nullptr;
        e->d.dirty_list[b] = nullptr;
    }
    cudaFree(e->d.bin_count);
    cudaFree(e->d.bin_start);
    cudaFree(e->d.chunk_sum);
    cudaFree(e->d.tasks);
    e->d.bin_count = e->d.bin_start = e->d.chunk_sum = nullptr;
    e->d.tasks = nullptr;
    e->grid_cells_alloc = 0;
    e->bricks_alloc = 0;
    e->max_tasks = 0;
}

void free_tables(SortedEngine* e) {
    cudaFree(e->scenes_d);
    cudaFree(e->brick_scene_d);
    cudaFree(e->bin_scene_d);
    e->scenes_d = nullptr;
    e->brick_scene_d = e->bin_scene_d = nullptr;
    e->d.scenes = nullptr;
    e->d.brick_scene = e->d.bin_scene = nullptr;
    e->d.nscenes = 1;
}

int occupancy_blocks(const void* fn, int threads) {
    int dev = 0, nsm = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0) != cudaSuccess) return 0;
    if (per < 1) per = 1;
    return nsm * per;
}

// Brick geometry of one scene; false for a degenerate box or one too large
// for i32 cell addresses.
bool make_geo(const SimConsts& k, Geo& g) {
    if (k.Y <= 0 || k.Z <= 0 || k.grid_count <= 0) return false;
    g = Geo{};
    g.Y = k.Y;
    g.Z = k.Z;
    const long long yz = (long long)k.Y * k.Z;
    if (yz > INT_MAX) return false;
    g.YZ = (int)yz;
    g.grid_count = k.grid_count;
    g.Xi = (int)(((long long)k.grid_count + yz - 1) / yz);
    g.BX = (g.Xi + 3) / 4;
    g.BY = (g.Y + 3) / 4;
    g.BZ = (g.Z + 3) / 4;
    // padding: one brick on each side, along z up to an even brick count
    // plus one more, so that a 4x4x8 bin's arena ends inside it
    g.PY = g.BY + 2;
    g.PZ = ((g.BZ + 1) & ~1) + 2;
    const long long nb = (long long)(g.BX + 2) * g.PY * g.PZ;
    if (nb * 64 > INT_MAX) return false;
    g.nbricks = (int)nb;
    g.NZ = (g.BZ + 1) & ~1;
    const long long nbins = (long long)g.BX * g.BY * g.NZ;
    if (nbins + 2 > INT_MAX / 2) return false;
    g.nbins = (int)nbins;
    return true;
}

// Bins of a scene: its bricks' (z rounded up to pairs), the irregular bin
// and an empty one.
long long scene_bins(const Geo& g) { return (long long)g.nbins + 2; }

// Grids, dirty lists, bin arrays and the task list for `bricks` bricks and
// `bins` bins (kept when large enough).
int ensure_grid_state(SortedEngine* e, long long bricks, long long bins) {
    const size_t cells = (size_t)bricks * 64;
    const long long max_tasks = bins + (long long)e->max_particles / kMinTaskCap + 2;
    if (cells <= e->grid_cells_alloc && bricks <= e->bricks_alloc && max_tasks <= e->max_tasks)
        return 0;
    free_grid_state(e);
    for (int b = 0; b < 2; ++b) {
        SE_CUDA(cudaMalloc(&e->d.grid[b], sizeof(int4) * cells));
        SE_CUDA(cudaMalloc(&e->d.gv[b], sizeof(float4) * cells));
        SE_CUDA(cudaMalloc(&e->d.dirty_flag[b], 4 * (size_t)bricks));
        SE_CUDA(cudaMalloc(&e->d.dirty_list[b], 4 * (size_t)bricks));
    }
    SE_CUDA(cudaMalloc(&e->d.bin_count, 4 * ((size_t)bins + kScanThreads)));
    SE_CUDA(cudaMalloc(&e->d.bin_start, 4 * ((size_t)bins + 1)));
    SE_CUDA(cudaMalloc(&e->d.chunk_sum, 4 * 3 * ((size_t)bins / kScanThreads + 2)));
    SE_CUDA(cudaMalloc(&e->d.tasks, sizeof(Task) * (size_t)max_tasks));
    e->grid_cells_alloc = cells;
    e->bricks_alloc = (int)bricks;
    e->max_tasks = (int)max_tasks;
    e->d.task_slots = (int)max_tasks;
    return 0;
}

// Default task size: enough tasks for every resident CTA of the task
// kernels, bins left whole when they already are.
// The automatic task size: the particles per resident task-kernel block,
// rounded to the nearest power of two (tasks then split by a shift) and
// clamped to [kMinTaskCap, kMaxSort].  64k particles on 608 blocks: 105 ->
// 128, 5 % faster per step than 105 on GB300.
int auto_task_cap(const SortedEngine* e, long long n) {
    const long long per = e->blocks_g2p() > 0 ? n / e->blocks_g2p() : kMaxSort;
    long long p = kMinTaskCap;
    while (p < kMaxSort && p * 2 <= per) p *= 2;              // largest power of two <= per
    if (p < kMaxSort && per * 1000 >= p * 1414) p *= 2;       // nearer the next one (log scale)
    return (int)p;
}

void apply_task_cap(SortedEngine* e, long long n) {
    const int cap = e->task_cap_auto ? auto_task_cap(e, n) : e->task_cap;
    if (cap != e->d.task_cap) drop_graphs(e);
    e->task_cap = cap;
    e->d.task_cap = cap;
    e->d.cap_shift = -1;
    if ((cap & (cap - 1)) == 0)
        for (int sh = 0; sh < 31; ++sh)
            if ((1 << sh) == cap) e->d.cap_shift = sh;
    e->d.chunk = e->threads;
}

}  // namespace

int sorted_create(SortedEngine** out, int max_particles) {
    *out = nullptr;
    SortedEngine* e = new SortedEngine();
    e->max_particles = max_particles;
    e->d.nscenes = 1;
    e->d.task_cap = kMaxSort;
    e->d.cap_shift = 10;
    e->d.chunk = kTask;
    e->d.pair_max = kPairMaxDefault;
    e->d.lane_min = MPM_LANE_TABLE_MIN;
    const size_t np = (size_t)(max_particles > 0 ? max_particles : 1);
    cudaError_t r = cudaMalloc(&e->d.bin_of, 4 * np);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.rank_of, 4 * np);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.order, 4 * np);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.dirty_n, 4 * 2);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.ticket, 4);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.ntasks, 4 * 2);
    if (r == cudaSuccess) r = cudaMalloc(&e->d.task_next, 4 * 3);
    if (r == cudaSuccess) {
        e->blocks_p2g2_v[0] = occupancy_blocks((const void*)k_p2g2<false, 128>, 128);
        e->blocks_p2g2_v[1] = occupancy_blocks((const void*)k_p2g2<false, 256>, 256);
        e->blocks_p2g2_v[2] = occupancy_blocks((const void*)k_p2g2<false, 512>, 512);
        e->blocks_g2p_v[0] = occupancy_blocks((const void*)k_g2p_p2g1<false, true, false, 128>, 128);
        e->blocks_g2p_v[1] = occupancy_blocks((const void*)k_g2p_p2g1<false, true, false, 256>, 256);
        e->blocks_g2p_v[2] = occupancy_blocks((const void*)k_g2p_p2g1<false, true, false, 512>, 512);
        e->blocks_update = occupancy_blocks((const void*)k_update<false>, 256);
        for (int v = 0; v < 3; ++v)
            if (e->blocks_p2g2_v[v] <= 0 || e->blocks_g2p_v[v] <= 0) r = cudaErrorInvalidValue;
        if (e->blocks_update <= 0) r = cudaErrorInvalidValue;
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
    free_tables(e);
    cudaFree(e->d.bin_of);
    cudaFree(e->d.rank_of);
    cudaFree(e->d.order);
    cudaFree(e->d.dirty_n);
    cudaFree(e->d.ticket);
    cudaFree(e->d.ntasks);
    cudaFree(e->d.task_next);
    delete e;
}

int sorted_configure(SortedEngine* e, const SimConsts& k) {
    e->configured = false;
    e->primed = false;
    e->has_grid = false;
    Geo g;
    if (!make_geo(k, g)) return -1;
    // Captured graphs hold the scene by value: they stay valid across a
    // reconfiguration with the same constants and geometry (a re-upload of
    // the same scene) and are dropped otherwise.
    Scene one{};
    one.g = g;
    one.k = k;
    if (e->batch || std::memcmp(&one, &e->one, sizeof(Scene)) != 0) drop_graphs(e);
    if (ensure_grid_state(e, g.nbricks, scene_bins(g))) return -1;
    free_tables(e);
    e->batch = false;
    e->scenes.clear();
    e->one = one;
    e->nbricks = g.nbricks;
    e->nbins = (int)scene_bins(g);
    apply_task_cap(e, k.n);
    e->configured = true;
    return 0;
}

int sorted_configure_batch(SortedEngine* e, const SimConsts* ks, int nscenes) {
    e->configured = false;
    e->primed = false;
    e->has_grid = false;
    if (nscenes < 1) {
        g_err = "a batch needs at least one scene";
        return -1;
    }
    std::vector<Scene> hs((size_t)nscenes);
    long long bricks = 0, bins = 0, parts = 0, lcells = 0;
    std::vector<std::pair<int, int>> classes;  // distinct (PY, PZ)
    for (int s = 0; s < nscenes; ++s) {
        if (!make_geo(ks[s], hs[s].g)) {
            g_err = "scene " + std::to_string(s) + " has a degenerate box";
            return -1;
        }
        const std::pair<int, int> pyz(hs[s].g.PY, hs[s].g.PZ);
        size_t c = 0;
        while (c < classes.size() && classes[c] != pyz) ++c;
        if (c == classes.size()) classes.push_back(pyz);
        hs[s].gclass = (int)c;
        hs[s].bbase = (int)bricks;
        hs[s].pbase = (int)parts;
        hs[s].lbase = (int)lcells;
        hs[s].k = ks[s];
        bricks += hs[s].g.nbricks;
        parts += ks[s].n;
        lcells += ks[s].grid_count;
        if (bricks * 64 > INT_MAX || parts > e->max_particles || lcells > INT_MAX) {
            g_err = "batch exceeds the engine's capacity";
            return -1;
        }
    }
    // bins class by class (scene order within a class)
    for (size_t c = 0; c < classes.size(); ++c)
        for (int s = 0; s < nscenes; ++s)
            if (hs[s].gclass == (int)c) {
                hs[s].binbase = (int)bins;
                bins += scene_bins(hs[s].g);
                if (bins > INT_MAX / 2) {
                    g_err = "batch exceeds the engine's capacity";
                    return -1;
                }
            }
    drop_graphs(e);
    if (bins > INT_MAX / 2) {
        g_err = "batch exceeds the engine's capacity";
        return -1;
    }
    if (ensure_grid_state(e, bricks, bins)) return -1;
    free_tables(e);
    std::vector<uint32_t> brick_scene((size_t)bricks), bin_scene((size_t)bins);
    for (int s = 0; s < nscenes; ++s) {
        for (int b = 0; b < hs[s].g.nbricks; ++b) brick_scene[(size_t)hs[s].bbase + b] = (uint32_t)s;
        for (long long b = 0; b < scene_bins(hs[s].g); ++b)
            bin_scene[(size_t)hs[s].binbase + b] = (uint32_t)s;
    }
    SE_CUDA(cudaMalloc(&e->scenes_d, sizeof(Scene) * (size_t)nscenes));
    SE_CUDA(cudaMalloc(&e->brick_scene_d, 4 * (size_t)bricks));
    SE_CUDA(cudaMalloc(&e->bin_scene_d, 4 * (size_t)bins));
    SE_CUDA(cudaMemcpy(e->scenes_d, hs.data(), sizeof(Scene) * (size_t)nscenes, cudaMemcpyHostToDevice));
    SE_CUDA(cudaMemcpy(e->brick_scene_d, brick_scene.data(), 4 * (size_t)bricks, cudaMemcpyHostToDevice));
    SE_CUDA(cudaMemcpy(e->bin_scene_d, bin_scene.data(), 4 * (size_t)bins, cudaMemcpyHostToDevice));
    e->d.scenes = e->scenes_d;
    e->d.brick_scene = e->brick_scene_d;
    e->d.bin_scene = e->bin_scene_d;
    e->d.nscenes = nscenes;
    e->batch = true;
    e->scenes = hs;
    e->one = hs[0];
    e->nbricks = (int)bricks;
    e->nbins = (int)bins;
    e->ncells_linear = (int)lcells;
    e->max_scene_cells = 0;
    for (int s = 0; s < nscenes; ++s) e->max_scene_cells = std::max(e->max_scene_cells, ks[s].grid_count);
    apply_task_cap(e, parts);
    e->configured = true;
    return 0;
}

int sorted_set_task_cap(SortedEngine* e, int cap) {
    if (cap != 0 && (cap < kMinTaskCap || cap > kMaxTaskCap)) {
        g_err = "task size outside [64, 2^30] (0: automatic)";
        return -1;
    }
    e->task_cap_auto = cap == 0;
    if (cap) e->task_cap = cap;
    long long n = e->one.k.n;
    if (e->batch) {
        n = 0;
        for (const Scene& sc : e->scenes) n += sc.k.n;
    }
    apply_task_cap(e, n);
    return 0;
}

int sorted_task_cap(const SortedEngine* e) { return e->d.task_cap; }

int sorted_set_lane_table_min(SortedEngine* e, int min_particles) {
    if (min_particles < 0) {
        g_err = "lane table threshold must be >= 0 (0: default)";
        return -1;
    }
    const int v = min_particles == 0 ? MPM_LANE_TABLE_MIN : min_particles;
    if (v != e->d.lane_min) drop_graphs(e);  // the captured launches carry it
    e->d.lane_min = v;
    return 0;
}

int sorted_lane_table_min(const SortedEngine* e) { return e->d.lane_min; }

int sorted_set_threads(SortedEngine* e, int threads) {
    if (threads == 0) threads = kTask;
    if (threads != 128 && threads != 256 && threads != 512) {
        g_err = "task-kernel block size must be 128, 256 or 512 (0: default 256)";
        return -1;
    }
    if (threads == e->threads) return 0;
    drop_graphs(e);  // the captured launches carry the CTA size
    e->threads = threads;
    long long n = e->one.k.n;
    if (e->batch) {
        n = 0;
        for (const Scene& sc : e->scenes) n += sc.k.n;
    }
    apply_task_cap(e, n);  // the automatic task size follows the resident CTAs
    return 0;
}

int sorted_threads(const SortedEngine* e) { return e->threads; }

int sorted_set_pair_max(SortedEngine* e, int max_particles) {
    if (max_particles < 0) {
        g_err = "z-pair threshold must be >= 0 (0: never pair)";
        return -1;
    }
    if (max_particles == kPairDefaultRequest) max_particles = kPairMaxDefault;
    if (max_particles == e->d.pair_max) return 0;
    drop_graphs(e);  // the captured launches carry it
    e->d.pair_max = max_particles;
    return 0;
}

int sorted_pair_max(const SortedEngine* e) { return e->d.pair_max; }

int sorted_set_scene_consts(SortedEngine* e, int scene, const SimConsts& k, cudaStream_t st) {
    if (!e->configured || !e->batch || scene < 0 || scene >= (int)e->scenes.size()) {
        g_err = "no such scene in the batch";
        return -1;
    }
    Scene& sc = e->scenes[(size_t)scene];
    if (k.Y != sc.k.Y || k.Z != sc.k.Z || k.grid_count != sc.k.grid_count || k.n != sc.k.n) {
        g_err = "a scene's geometry and particle count are fixed at batch creation";
        return -1;
    }
    sc.k = k;
    SE_CUDA(cudaMemcpyAsync(&e->scenes_d[scene].k, &sc.k, sizeof(SimConsts), cudaMemcpyHostToDevice, st));
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

namespace {

// The task kernels at the engine's CTA size.
template <bool BATCH, int TH>
void launch_p2g2_th(SortedEngine* e, const Particles& P, const Scene& one, int cur,
                    unsigned long long* oob, cudaStream_t st) {
    k_p2g2<BATCH, TH><<<e->blocks_p2g2(), TH, 0, st>>>(P, one, e->d, cur, oob);
}

template <bool BATCH>
void launch_p2g2(SortedEngine* e, const Particles& P, const Scene& one, int cur,
                 unsigned long long* oob, cudaStream_t st) {
    switch (e->threads) {
        case 128: launch_p2g2_th<BATCH, 128>(e, P, one, cur, oob, st); break;
        case 512: launch_p2g2_th<BATCH, 512>(e, P, one, cur, oob, st); break;
        default: launch_p2g2_th<BATCH, 256>(e, P, one, cur, oob, st); break;
    }
}

template <bool BATCH, bool DO_G2P, bool POSVEL, int TH>
void launch_g2p_th(SortedEngine* e, const Particles& Pin, const Particles& Pout,
                   const uint32_t* id_in, uint32_t* id_out, float4* posvel, const Scene& one,
                   int src, int dst, unsigned long long* oob, cudaStream_t st) {
    k_g2p_p2g1<BATCH, DO_G2P, POSVEL, TH><<<e->blocks_g2p(), TH, 0, st>>>(
        Pin, Pout, id_in, id_out, posvel, one, e->d, src, dst, oob);
}

template <bool BATCH, bool DO_G2P, bool POSVEL>
void launch_g2p(SortedEngine* e, const Particles& Pin, const Particles& Pout,
                const uint32_t* id_in, uint32_t* id_out, float4* posvel, const Scene& one,
                int src, int dst, unsigned long long* oob, cudaStream_t st) {
    switch (e->threads) {
        case 128:
            launch_g2p_th<BATCH, DO_G2P, POSVEL, 128>(e, Pin, Pout, id_in, id_out, posvel, one,
                                                      src, dst, oob, st);
            break;
        case 512:
            launch_g2p_th<BATCH, DO_G2P, POSVEL, 512>(e, Pin, Pout, id_in, id_out, posvel, one,
                                                      src, dst, oob, st);
            break;
        default:
            launch_g2p_th<BATCH, DO_G2P, POSVEL, 256>(e, Pin, Pout, id_in, id_out, posvel, one,
                                                      src, dst, oob, st);
            break;
    }
}

// The counting sort's scan (and, for many bins, the chunk sums before it).
void launch_scan(SortedEngine* e, const Scene& one, int nbins, cudaStream_t st,
                 LaunchProfiler* prof) {
    const int chunks = (nbins + kScanThreads - 1) / kScanThreads;
    const int chunked = chunks > kChunkedScanMin ? 1 : 0;
    if (chunked) LAUNCH(KID_SCAN, (k_chunk_sums<<<chunks, kScanThreads, 0, st>>>(e->d)));
    LAUNCH(KID_SCAN, (k_scan<<<chunks, kScanThreads, 0, st>>>(e->d, one.g, nbins, chunked)));
}

// Issues the kernels of `substeps` substeps and advances the engine state.
template <bool BATCH>
int enqueue_substeps(SortedEngine* e, ParticleStore* ps, float4* posvel, unsigned long long* oob,
                     const Scene& one, int n, int substeps, cudaStream_t st, LaunchProfiler* prof) {
    const int nbins = e->nbins;
    for (int s = 0; s < substeps; ++s) {
        const int cur = e->cur, nxt = cur ^ 1;
        const int pin = ps->cur, pout = pin ^ 1;
        LAUNCH(KID_SORTED_P2G_2, (launch_p2g2<BATCH>(e, ps->P[pin], one, cur, oob, st)));
        LAUNCH(KID_UPDATE_GRID, (k_update<BATCH><<<e->blocks_update, 256, 0, st>>>(one, e->d, cur)));
        if (s == substeps - 1)
            LAUNCH(KID_SORTED_G2P_P2G_1,
                   (launch_g2p<BATCH, true, true>(e, ps->P[pin], ps->P[pout], ps->id[pin],
                                                  ps->id[pout], posvel, one, cur, nxt, oob, st)));
        else
            LAUNCH(KID_SORTED_G2P_P2G_1,
                   (launch_g2p<BATCH, true, false>(e, ps->P[pin], ps->P[pout], ps->id[pin],
                                                   ps->id[pout], posvel, one, cur, nxt, oob, st)));
        launch_scan(e, one, nbins, st, prof);
        LAUNCH(KID_SCATTER, (k_scatter<<<(max(n, nbins) + 255) / 256, 256, 0, st>>>(e->d, n, nbins)));
        e->last = cur;
        e->cur = nxt;
        ps->cur = pout;
        ps->canonical = false;
    }
    SE_CUDA(cudaGetLastError());
    return 0;
}

template <bool BATCH>
int prime(SortedEngine* e, ParticleStore* ps, float4* posvel, unsigned long long* oob,
          const Scene& one, int n, cudaStream_t st, LaunchProfiler* prof) {
    const int nbins = e->nbins;
    const size_t cells = (size_t)e->nbricks * 64;
    for (int b = 0; b < 2; ++b) {
        SE_CUDA(cudaMemsetAsync(e->d.grid[b], 0, sizeof(int4) * cells, st));
        SE_CUDA(cudaMemsetAsync(e->d.gv[b], 0, sizeof(float4) * cells, st));
        SE_CUDA(cudaMemsetAsync(e->d.dirty_flag[b], 0, 4 * (size_t)e->nbricks, st));
    }
    SE_CUDA(cudaMemsetAsync(e->d.dirty_n, 0, 8, st));
    SE_CUDA(cudaMemsetAsync(e->d.ticket, 0, 4, st));
    SE_CUDA(cudaMemsetAsync(e->d.task_next, 0, 4 * 3, st));
    // k_chunk_sums reads the whole last chunk: the counts past nbins stay zero
    SE_CUDA(cudaMemsetAsync(e->d.bin_count, 0, 4 * ((size_t)nbins + kScanThreads), st));
    const Particles& P = ps->P[ps->cur];
    LAUNCH(KID_BIN, (k_bin<BATCH><<<(n + kTask - 1) / kTask, kTask, 0, st>>>(P, one, e->d, n)));
    launch_scan(e, one, nbins, st, prof);
    LAUNCH(KID_SCATTER, (k_scatter<<<(max(n, nbins) + 255) / 256, 256, 0, st>>>(e->d, n, nbins)));
    e->cur = 0;
    LAUNCH(KID_SORTED_P2G_1,
           (launch_g2p<BATCH, false, false>(e, P, P, ps->id[ps->cur], ps->id[ps->cur], posvel,
                                            one, e->cur, e->cur, oob, st)));
    SE_CUDA(cudaGetLastError());
    e->primed = true;
    return 0;
}

// Replays (capturing on first use) `substeps` substeps as one CUDA graph.
template <bool BATCH>
int enqueue_graph(SortedEngine* e, ParticleStore* ps, float4* posvel, unsigned long long* oob,
                  const Scene& one, int n, int substeps, cudaStream_t st, LaunchProfiler* prof) {
    GraphEntry* hit = nullptr;
    for (GraphEntry& g : e->graphs)
        if (g.substeps == substeps && g.cur0 == e->cur && g.pcur0 == ps->cur &&
            g.posvel == posvel && g.oob == oob)
            hit = &g;
    if (!hit) {
        GraphEntry ent;
        ent.substeps = substeps;
        ent.cur0 = e->cur;
        ent.pcur0 = ps->cur;
        ent.posvel = posvel;
        ent.oob = oob;
        const int cur0 = e->cur, last0 = e->last, pcur0 = ps->cur;
        const bool canon0 = ps->canonical;
        LaunchProfiler counter;  // counts the captured launches
        cudaStream_t cs = nullptr;
        SE_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t graph = nullptr;
        int rc = 0;
        cudaError_t r = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (r == cudaSuccess) {
            rc = enqueue_substeps<BATCH>(e, ps, posvel, oob, one, n, substeps, cs, &counter);
            r = cudaStreamEndCapture(cs, &graph);
        }
        if (r == cudaSuccess && rc == 0) r = cudaGraphInstantiate(&ent.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        cudaStreamDestroy(cs);
        ent.cur1 = e->cur;
        ent.last1 = e->last;
        ent.pcur1 = ps->cur;
        e->cur = cur0;  // the capture only recorded; the replay below runs it
        e->last = last0;
        ps->cur = pcur0;
        ps->canonical = canon0;
        if (r != cudaSuccess || rc != 0) {
            if (ent.exec) cudaGraphExecDestroy(ent.exec);
            if (r != cudaSuccess) g_err = std::string("graph capture: ") + cudaGetErrorString(r);
            cudaGetLastError();
            return -1;
        }
        for (int i = 0; i < KID_COUNT; ++i) ent.launches[i] = counter.launches[i];
        counter.release();
        e->graphs.push_back(ent);
        hit = &e->graphs.back();
    }
    SE_CUDA(cudaGraphLaunch(hit->exec, st));
    for (int i = 0; i < KID_COUNT; ++i) prof->launches[i] += hit->launches[i];
    e->cur = hit->cur1;
    e->last = hit->last1;
    ps->cur = hit->pcur1;
    ps->canonical = false;
    return 0;
}

template <bool BATCH>
int step_impl(SortedEngine* e, ParticleStore* ps, float4* posvel, unsigned long long* oob,
              const Scene& one, int n, int substeps, bool graph, cudaStream_t st,
              LaunchProfiler* prof) {
    if (!e->primed && prime<BATCH>(e, ps, posvel, oob, one, n, st, prof)) return -1;
    const int rc = (graph && !prof->enabled)
                       ? enqueue_graph<BATCH>(e, ps, posvel, oob, one, n, substeps, st, prof)
                       : enqueue_substeps<BATCH>(e, ps, posvel, oob, one, n, substeps, st, prof);
    if (rc) return rc;
    e->has_grid = true;
    return 0;
}

}  // namespace

int sorted_step(SortedEngine* e, ParticleStore* ps, float4* posvel, unsigned long long* oob,
                const SimConsts& k, int substeps, cudaStream_t st, LaunchProfiler* prof,
                bool graph) {
    if (!e->configured) {
        g_err = "sorted engine is not configured for this scene";
        return -1;
    }
    if (e->batch) {
        long long n = 0;
        for (const Scene& sc : e->scenes) n += sc.k.n;
        if (n == 0 || substeps == 0) return 0;
        return step_impl<true>(e, ps, posvel, oob, e->one, (int)n, substeps, graph, st, prof);
    }
    const int n = k.n;
    if (n == 0 || substeps == 0) {
        if (n == 0 && substeps > 0) e->has_grid = false;
        return 0;
    }
    // A single scene's constants are kernel parameters: graphs captured with
    // other constants are stale.
    if (graph && memcmp(&e->one.k, &k, sizeof(SimConsts)) != 0) drop_graphs(e);
    if (k.n != e->one.k.n) apply_task_cap(e, k.n);
    e->one.k = k;
    return step_impl<false>(e, ps, posvel, oob, e->one, n, substeps, graph, st, prof);
}

int sorted_export_grid(SortedEngine* e, const SimConsts& k, int4* out, cudaStream_t st,
                       LaunchProfiler* prof) {
    (void)k;
    return sorted_export_scene_grid(e, 0, out, st, prof);
}

int sorted_export_scene_grid(SortedEngine* e, int scene, int4* out, cudaStream_t st,
                             LaunchProfiler* prof) {
    if (!e->configured || !e->has_grid) {
        g_err = "no sorted-engine grid to export";
        return -1;
    }
    const Scene& sc = e->batch ? e->scenes.at((size_t)scene) : e->one;
    const Geo& g = sc.g;
    const int4* grid = e->d.grid[e->last] + (size_t)(e->batch ? sc.bbase : 0) * 64;
    LAUNCH(KID_EXPORT, (k_export<<<(g.grid_count + 255) / 256, 256, 0, st>>>(grid, g, out)));
    SE_CUDA(cudaGetLastError());
    return 0;
}

int sorted_export_all_canonical(SortedEngine* e, int4* out, const ParticleStore& ps,
                                const Particles& dst, int n, cudaStream_t st,
                                LaunchProfiler* prof) {
    if (sorted_export_all(e, out, st, prof) != 0) return -1;
    const int c = ps.cur;
    if (!ps.canonical) {
        if (n > 0)
            LAUNCH(KID_CANONICALIZE, launch_canonicalize(ps.P[c], ps.id[c], dst, nullptr, n, st));
        SE_CUDA(cudaGetLastError());
        return 0;
    }
    const float4* s[4] = {ps.P[c].p0, ps.P[c].p1, ps.P[c].p2, ps.P[c].p3};
    float4* d[4] = {dst.p0, dst.p1, dst.p2, dst.p3};
    for (int q = 0; q < 4 && n > 0; ++q)
        SE_CUDA(cudaMemcpyAsync(d[q], s[q], sizeof(float4) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    return 0;
}

int sorted_export_all(SortedEngine* e, int4* out, cudaStream_t st, LaunchProfiler* prof) {
    if (!e->configured || !e->has_grid || !e->batch) {
        g_err = "no batched sorted-engine grid to export";
        return -1;
    }
    const int S = (int)e->scenes.size();
    for (int s0 = 0; s0 < S; s0 += 65535) {
        const dim3 blocks((unsigned)((e->max_scene_cells + 255) / 256),
                          (unsigned)std::min(65535, S - s0));
        LAUNCH(KID_EXPORT,
               (k_export_scenes<<<blocks, 256, 0, st>>>(e->d.grid[e->last], e->d, s0, out)));
    }
    SE_CUDA(cudaGetLastError());
    return 0;
}

const char* sorted_error() { return g_err.c_str(); }

}  // namespace mpm
