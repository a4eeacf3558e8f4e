// adjoint.cu -- reverse-mode derivative of the MLS-MPM substep
// (mls-mpm/p2g_1.wgsl, p2g_2.wgsl, updateGrid.wgsl, g2p.wgsl), for batches
// of scenes.
//
// The forward is the fixed-point solver; its derivative is taken of the
// continuous model it discretises: enc/dec are treated as the identity
// (their truncation has zero derivative almost everywhere), floor() of the
// base cell is piecewise constant, and max/clamp/wall branches take the
// branch the forward took.  The adjoint of one substep runs in reverse stage
// order on the substep's input state S_t and its updated grid G_t (both
// recorded by a forward recompute from a checkpoint):
//
//   k_adj_g2p     particle-parallel; the g2p gather becomes a scatter of
//                 the grid-velocity adjoint (one float4 reduction per
//                 stencil cell)
//   k_adj_update  cell-parallel, elementwise: velocity adjoint -> momentum
//                 and mass adjoints
//   k_adj_p2g2    particle-parallel gather of the momentum adjoint through
//                 the stress term; the density gather becomes a scatter of
//                 the density adjoint onto the mass adjoint
//   k_adj_p2g1    particle-parallel gather of the mass and momentum adjoints
//
// Large batches run the particle kernels in the order of a per-substep
// spatial sort (k_adj_bin / k_adj_place / k_adj_perm), one thread per
// particle; small ones in particle order, three threads per particle.
//
// Two tapes: the fixed-point solver's own (S_t as f32 records, G_t as the
// i32 grid) or an FP64 integration of the continuous model on the GPU
// (k64_* below: double state records, double grid sums), whose trajectory
// stays close to an FP64 reference over hundreds of substeps.  The adjoint
// arithmetic is f32 in both cases; the Tape* accessors convert.
//
// Matrices: C is stored by columns, C[c][r] = M(r, c), as in the particle
// records; the adjoint records use the same packing.  Stencil cells whose
// flat index falls outside the grid were dropped (writes) or read as zero
// (reads) by the forward; their terms are dropped here too.
#include <cuda_runtime.h>

#include <climits>

#include "adjoint.h"

namespace mpm {

namespace {

constexpr int kThreads = 256;

// Resident CTAs per SM the particle kernels ask the register allocator for
// (one thread per particle, unbounded: k_adj_p2g2 ~160 registers, k_adj_g2p
// ~124; capped at 2 and 3 CTAs of 256 threads they spill 68 and 120 bytes
// and the 1.5M-particle backward runs ~5 % faster).
#ifndef MPM_ADJ_P2G2_MIN_BLOCKS
#define MPM_ADJ_P2G2_MIN_BLOCKS 2
#endif
#ifndef MPM_ADJ_G2P_MIN_BLOCKS
#define MPM_ADJ_G2P_MIN_BLOCKS 3
#endif

struct Sten {
    float cf[3];     // floor(x)
    float w[3][3];   // w[axis][g]
    float dw[3][3];  // d w[axis][g] / d x[axis]
};

__device__ __forceinline__ void make_sten(const float x[3], Sten& s) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float c = floorf(x[a]);
        const float d = x[a] - (c + 0.5f);
        const float lo = 0.5f - d, hi = 0.5f + d;
        s.cf[a] = c;
        s.w[a][0] = (0.5f * lo) * lo;
        s.w[a][1] = 0.75f - d * d;
        s.w[a][2] = (0.5f * hi) * hi;
        s.dw[a][0] = -lo;
        s.dw[a][1] = -2.0f * d;
        s.dw[a][2] = hi;
    }
}

// Stencil cell (gx, gy, gz) of a particle: its weight, weight gradient and
// dist.
struct Node {
    float w;
    float gw[3];
    float dist[3];
};

// Flat index of the stencil cell in the scene's grid, -1 where the forward
// dropped it (outside [0, grid_count)).
__device__ __forceinline__ int node_index(const Sten& s, int gx, int gy, int gz, const SimConsts& k) {
    const int idx = flat_index(s.cf[0] + (float)gx - 1.0f, s.cf[1] + (float)gy - 1.0f,
                               s.cf[2] + (float)gz - 1.0f, k.Y, k.Z);
    return (unsigned)idx < (unsigned)k.grid_count ? idx : -1;
}

struct Rec {
    float x[3], v[3];
    float C[3][3];  // C[c][r]
};

__device__ __forceinline__ Rec load_rec(const Particles& P, int i) {
    Rec r;
    const float4 a = P.p0[i], b = P.p1[i], c = P.p2[i], d = P.p3[i];
    r.x[0] = a.x; r.x[1] = a.y; r.x[2] = a.z;
    r.C[0][0] = a.w; r.C[0][1] = b.x; r.C[0][2] = b.y;
    r.C[1][0] = b.z; r.C[1][1] = b.w; r.C[1][2] = c.x;
    r.C[2][0] = c.y; r.C[2][1] = c.z; r.C[2][2] = c.w;
    r.v[0] = d.x; r.v[1] = d.y; r.v[2] = d.z;
    return r;
}

__device__ __forceinline__ void store_rec(const Particles& P, int i, const Rec& r) {
    P.p0[i] = make_float4(r.x[0], r.x[1], r.x[2], r.C[0][0]);
    P.p1[i] = make_float4(r.C[0][1], r.C[0][2], r.C[1][0], r.C[1][1]);
    P.p2[i] = make_float4(r.C[1][2], r.C[2][0], r.C[2][1], r.C[2][2]);
    P.p3[i] = make_float4(r.v[0], r.v[1], r.v[2], 0.0f);
}

__device__ __forceinline__ float dec_f(int i, float fm) { return (float)i / fm; }

// Tape of the fixed-point solver: f32 records and the updated i32 grid.
struct TapeFixed {
    Particles S;
    const int4* G;
    __device__ __forceinline__ Rec rec(int i) const { return load_rec(S, i); }
    __device__ __forceinline__ void pos(int i, float x[3]) const {
        const float4 a = S.p0[i];
        x[0] = a.x; x[1] = a.y; x[2] = a.z;
    }
    // cell j (all-scene linear index): velocity (or raw momentum), mass, mass > 0
    __device__ __forceinline__ void vel(int j, float fm, float v[3]) const {
        const int4 c = __ldg(G + j);
        v[0] = dec_f(c.x, fm); v[1] = dec_f(c.y, fm); v[2] = dec_f(c.z, fm);
    }
    __device__ __forceinline__ float mass(int j, float fm) const { return dec_f(__ldg(G + j).w, fm); }
    __device__ __forceinline__ bool updated(int j) const { return __ldg(G + j).w > 0; }
};

// FP64 tape: records of kRec64 doubles (x, v, C by columns) and double4
// cells (v or momentum, mass).
struct Tape64 {
    const double* S;
    const double4* G;
    __device__ __forceinline__ Rec rec(int i) const {
        const double* p = S + (size_t)kRec64 * i;
        Rec r;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            r.x[a] = (float)p[a];
            r.v[a] = (float)p[3 + a];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int q = 0; q < 3; ++q) r.C[c][q] = (float)p[6 + 3 * c + q];
        return r;
    }
    __device__ __forceinline__ void pos(int i, float x[3]) const {
        const double* p = S + (size_t)kRec64 * i;
        x[0] = (float)p[0]; x[1] = (float)p[1]; x[2] = (float)p[2];
    }
    __device__ __forceinline__ void vel(int j, float, float v[3]) const {
        const double4 c = G[j];
        v[0] = (float)c.x; v[1] = (float)c.y; v[2] = (float)c.z;
    }
    __device__ __forceinline__ float mass(int j, float) const { return (float)G[j].w; }
    __device__ __forceinline__ bool updated(int j) const { return G[j].w > 0.0; }
};

// Adds this thread's parameter adjoints to the scene's accumulators (warp
// sums when the whole warp is in one scene).
__device__ __forceinline__ void add_param_grads(double* pg, int scene, bool active, float gk,
                                                float gmu) {
    const unsigned full = 0xffffffffu;
    const int s0 = __shfl_sync(full, scene, 0);
    const bool uniform = __all_sync(full, !active || scene == s0);
    if (uniform) {
        float a = active ? gk : 0.0f, b = active ? gmu : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(full, a, o);
            b += __shfl_down_sync(full, b, o);
        }
        const bool any = __any_sync(full, active);
        if ((threadIdx.x & 31u) == 0 && any) {
            atomicAdd(pg + 2 * s0, (double)a);
            atomicAdd(pg + 2 * s0 + 1, (double)b);
        }
    } else if (active) {
        atomicAdd(pg + 2 * scene, (double)gk);
        atomicAdd(pg + 2 * scene + 1, (double)gmu);
    }
}

// ---------------------------------------------------------------------------
// Spatial sort of one substep's particles.  The particle-parallel kernels
// below walk the particles in the order of the brick (4^3 cells) of their
// base cell floor(x), so that the threads of a warp gather and scatter
// neighbouring cells: their loads hit L1 and their reductions land on a few
// L2 lines.  Particles whose stencil leaves the grid interior go to one
// extra bin at the end.
// ---------------------------------------------------------------------------
template <class Tape>
__global__ void __launch_bounds__(kThreads)
    k_adj_bin(Tape tp, const AdjScene* __restrict__ scenes, const int* __restrict__ pscene, int n,
              AdjSort so) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < n;
    int bin = -1;  // inactive lanes: a key no bin has
    if (active) {
        const AdjScene& sc = scenes[pscene[i]];
        const SimConsts& k = sc.k;
        float x[3];
        tp.pos(i, x);
        bin = so.nbins - 1;
        if (x[0] >= 1.0f && x[1] >= 1.0f && x[2] >= 1.0f && x[0] < 1.0e9f && x[1] < 1.0e9f &&
            x[2] < 1.0e9f) {
            const int cx = (int)floorf(x[0]), cy = (int)floorf(x[1]), cz = (int)floorf(x[2]);
            const long long top = ((long long)(cx + 1) * k.Y + (cy + 1)) * k.Z + (cz + 1);
            if (cy + 1 < k.Y && cz + 1 < k.Z && top < k.grid_count)
                bin = sc.bbase + ((cx >> 2) * sc.BY + (cy >> 2)) * sc.BZ + (cz >> 2);
        }
    }
    // warp-aggregated rank: one atomic per distinct bin of the warp
    const unsigned peers = __match_any_sync(0xffffffffu, bin);
    const int leader = __ffs(peers) - 1;
    const unsigned lane = threadIdx.x & 31u;
    int base = 0;
    if (active && (int)lane == leader) base = atomicAdd(so.bin_count + bin, __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (active) so.key_rank[i] = make_int2(bin, base + __popc(peers & ((1u << lane) - 1u)));
}

// One thread per bin: the bin's first slot in the sorted order (bins are
// placed in whatever order the warp-wide allocations from the counter come;
// only their contiguity matters).
__global__ void __launch_bounds__(kThreads) k_adj_place(AdjSort so) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = b < so.nbins ? so.bin_count[b] : 0;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int cs = c;  // inclusive warp scan
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(full, cs, o);
        if (lane >= o) cs += u;
    }
    int base = 0;
    if (lane == 31 && cs > 0) base = atomicAdd(so.placed, cs);
    base = __shfl_sync(full, base, 31);
    if (c > 0) so.bin_first[b] = base + cs - c;
}

__global__ void __launch_bounds__(kThreads) k_adj_perm(AdjSort so, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 kr = so.key_rank[i];
    so.perm[so.bin_first[kr.x] + kr.y] = i;
}

// ---------------------------------------------------------------------------
// Particle-parallel adjoint kernels.  L lanes per particle: L = 1 runs the
// whole 27-cell stencil in one thread; L = 3 gives lane q the nine cells of
// x-slab gx = q (groups of three lanes, ten particles per warp, lanes 30-31
// idle), for batches too small to fill the GPU one thread per particle.  A
// group sums its partial results in lane order, so every lane holds the same
// totals.  Each particle makes one gather pass over its stencil and at most
// one scatter pass; terms that depend on a gathered total enter after the
// gather by linearity.
// ---------------------------------------------------------------------------
template <int L>
struct Lanes {
    int q;        // this lane's slab (L = 3) or 0
    int j;        // particle slot in the sorted order
    bool active;  // a real particle (idle lanes repeat the last one)
};

template <int L>
__device__ __forceinline__ Lanes<L> lanes_of(int n) {
    Lanes<L> g;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (L == 1) {
        g.q = 0;
        g.j = t;
        g.active = t < n;
    } else {
        const int lane = threadIdx.x & 31;
        g.q = lane % 3;
        g.j = (t >> 5) * 10 + lane / 3;
        g.active = lane < 30 && g.j < n;
    }
    if (!g.active) g.j = n - 1;
    return g;
}

template <int L>
inline int lane_blocks(long long n) {
    const long long per = L == 1 ? kThreads : (kThreads / 32) * 10;
    return (int)((n + per - 1) / per);
}

// Sum over the lanes of a group, in lane order.
template <int L, int N>
__device__ __forceinline__ void lane_sum(float (&v)[N]) {
    if (L == 1) return;
    const int base = (threadIdx.x & 31) / 3 * 3;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const float a = __shfl_sync(0xffffffffu, v[j], base);
        const float b = __shfl_sync(0xffffffffu, v[j], base + 1);
        const float c = __shfl_sync(0xffffffffu, v[j], base + 2);
        v[j] = (a + b) + c;
    }
}

// The x-axis factors of slab gx of a particle's stencil.
struct Slab {
    int gx;
    float w, dw;
};

__device__ __forceinline__ Slab slab(const Sten& st, int gx) {
    Slab s;
    s.gx = gx;
    s.w = gx == 0 ? st.w[0][0] : (gx == 1 ? st.w[0][1] : st.w[0][2]);
    s.dw = gx == 0 ? st.dw[0][0] : (gx == 1 ? st.dw[0][1] : st.dw[0][2]);
    return s;
}

__device__ __forceinline__ void slab_node(const Sten& s, const float x[3], const Slab& sx, int gy,
                                          int gz, Node& nd) {
    const float wx = sx.w, wy = s.w[1][gy], wz = s.w[2][gz];
    nd.w = (wx * wy) * wz;
    nd.gw[0] = (sx.dw * wy) * wz;
    nd.gw[1] = (wx * s.dw[1][gy]) * wz;
    nd.gw[2] = (wx * wy) * s.dw[2][gz];
    nd.dist[0] = ((s.cf[0] + (float)sx.gx - 1.0f) + 0.5f) - x[0];
    nd.dist[1] = ((s.cf[1] + (float)gy - 1.0f) + 0.5f) - x[1];
    nd.dist[2] = ((s.cf[2] + (float)gz - 1.0f) + 0.5f) - x[2];
}

// The slabs lane q visits: all three (L = 1) or its own.
template <int L>
__device__ __forceinline__ int slab_count() { return L == 1 ? 3 : 1; }

template <int L>
__device__ __forceinline__ int slab_gx(int s, int q) { return L == 1 ? s : q; }

// ---------------------------------------------------------------------------
// g2p backward (g2p.wgsl:26-92).  Aout: adjoint of S_{t+1}; writes the g2p
// part of the position adjoint of S_t into Anew (velocity and C adjoints
// zeroed) and scatters the grid-velocity adjoint into gadj.xyz.  With
// u_n = Cbar v_n (rows of the C adjoint against the cell velocity) and
// q_n = vgbar + 4 Cbar^T d_n, the position adjoint
//   sum_n grad w_n (v_n . q_n) - 4 w_n u_n  =  G vgbar + H,
// G = sum_n grad w_n v_n^T, H = sum_n 4 grad w_n (d_n . u_n) - 4 w_n u_n.
// ---------------------------------------------------------------------------
template <class Tape, int L>
__global__ void __launch_bounds__(kThreads, MPM_ADJ_G2P_MIN_BLOCKS)
    k_adj_g2p(Tape tp, Particles Aout, Particles Anew, float4* __restrict__ gadj,
              const AdjScene* __restrict__ scenes, const int* __restrict__ pscene,
              const int* __restrict__ perm, int n) {
    const Lanes<L> ln = lanes_of<L>(n);
    const int i = perm ? perm[ln.j] : ln.j;
    const AdjScene& sc = scenes[pscene[i]];
    const SimConsts& k = sc.k;
    float4* ga = gadj + sc.lbase;
    float x[3];
    tp.pos(i, x);
    Sten st;
    make_sten(x, st);
    const Rec ao = load_rec(Aout, i);

    float acc[15] = {};  // vg (3), G row-major (9), H (3)
#pragma unroll
    for (int s = 0; s < slab_count<L>(); ++s) {
        const Slab sx = slab(st, slab_gx<L>(s, ln.q));
#pragma unroll
        for (int gy = 0; gy < 3; ++gy)
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const int c = node_index(st, sx.gx, gy, gz, k);
                if (c < 0) continue;
                float vi[3];
                tp.vel(sc.lbase + c, k.fm, vi);
                Node nd;
                slab_node(st, x, sx, gy, gz, nd);
                float u[3];
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    u[j] = ao.C[j][0] * vi[0] + ao.C[j][1] * vi[1] + ao.C[j][2] * vi[2];
                const float du = 4.0f * (nd.dist[0] * u[0] + nd.dist[1] * u[1] + nd.dist[2] * u[2]);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    acc[a] += nd.w * vi[a];
                    acc[12 + a] += nd.gw[a] * du - 4.0f * nd.w * u[a];
#pragma unroll
                    for (int r = 0; r < 3; ++r) acc[3 + 3 * a + r] += nd.gw[a] * vi[r];
                }
            }
    }
    lane_sum<L>(acc);

    float xbar[3], vgbar[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float vg = acc[a];
        const float xt = x[a] + vg * k.dt;
        const float hiw = k.real_box[a] - 2.0f;
        const bool inside = xt >= 1.0f && xt <= hiw;
        const float xc = fminf(fmaxf(xt, 1.0f), hiw);
        const float xn = xc + (vg * k.dt) * 3.0f;
        const float nw = (xn < 3.0f ? 1.0f : 0.0f) + (xn > k.real_box[a] - 4.0f ? 1.0f : 0.0f);
        const float xcbar = ao.x[a] - 0.3f * nw * ao.v[a];
        const float xtbar = inside ? xcbar : 0.0f;
        vgbar[a] = ao.v[a] * (1.0f - 0.9f * k.dt * nw) + k.dt * xtbar;
        xbar[a] = xtbar;
    }
    if (!ln.active) return;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        xbar[a] += acc[3 + 3 * a] * vgbar[0] + acc[4 + 3 * a] * vgbar[1] + acc[5 + 3 * a] * vgbar[2] +
                   acc[12 + a];

#pragma unroll
    for (int s = 0; s < slab_count<L>(); ++s) {
        const Slab sx = slab(st, slab_gx<L>(s, ln.q));
#pragma unroll
        for (int gy = 0; gy < 3; ++gy)
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const int c = node_index(st, sx.gx, gy, gz, k);
                if (c < 0) continue;
                Node nd;
                slab_node(st, x, sx, gy, gz, nd);
                float q[3];
#pragma unroll
                for (int r = 0; r < 3; ++r)
                    q[r] = nd.w * (vgbar[r] + 4.0f * (ao.C[0][r] * nd.dist[0] + ao.C[1][r] * nd.dist[1] +
                                                      ao.C[2][r] * nd.dist[2]));
                atomicAdd(ga + c, make_float4(q[0], q[1], q[2], 0.0f));
            }
    }
    if (ln.q == 0) {
        Rec an{};
#pragma unroll
        for (int a = 0; a < 3; ++a) an.x[a] = xbar[a];
        store_rec(Anew, i, an);
    }
}


// ---------------------------------------------------------------------------
// updateGrid backward (updateGrid.wgsl:23-46), per cell of all scenes:
// gadj.xyz = velocity adjoint -> (momentum adjoint, mass adjoint).
// ---------------------------------------------------------------------------
template <class Tape>
__global__ void __launch_bounds__(kThreads)
    k_adj_update(Tape tp, float4* __restrict__ gadj, const AdjScene* __restrict__ scenes,
                 int nscenes, int ncells) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncells) return;
    const float4 vb = gadj[j];
    // a cell no particle's g2p adjoint reached holds +0 and maps to +0 (with
    // a finite tape): most cells of an expanded scene, left as they are
    if ((__float_as_uint(vb.x) | __float_as_uint(vb.y) | __float_as_uint(vb.z) |
         __float_as_uint(vb.w)) == 0u)
        return;
    int lo = 0, hi = nscenes - 1;  // last scene with lbase <= j
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (scenes[mid].lbase <= j) lo = mid;
        else hi = mid - 1;
    }
    const SimConsts& k = scenes[lo].k;
    const int id = j - scenes[lo].lbase;
    if (!tp.updated(j)) {  // not updated: g2p read the raw momentum as velocity
        gadj[j] = make_float4(vb.x, vb.y, vb.z, 0.0f);
        return;
    }
    const float m = tp.mass(j, k.fm);
    float raw[3];
    tp.vel(j, k.fm, raw);
    const int x = (id / k.Z) / k.Y, y = (id / k.Z) % k.Y, z = id % k.Z;
    const int hx = wall_hi(k.real_box[0]), hy = wall_hi(k.real_box[1]), hz = wall_hi(k.real_box[2]);
    const bool keep[3] = {!(x < 2 || x > hx), !(y < 2 || y > hy), !(z < 2 || z > hz)};
    const float vin[3] = {vb.x, vb.y, vb.z};
    float mvbar[3], mbar = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!keep[a]) {
            mvbar[a] = 0.0f;
            continue;
        }
        const float vpre = raw[a] - (k.gravity[a] != 0.0f ? k.gravity[a] * k.dt : 0.0f);
        mvbar[a] = vin[a] / m;
        mbar -= vin[a] * vpre / m;
    }
    gadj[j] = make_float4(mvbar[0], mvbar[1], mvbar[2], mbar);
}


// ---------------------------------------------------------------------------
// p2g_2 backward (p2g_2.wgsl:30-94).  Accumulates into Anew (position and C
// adjoints), the scene's stiffness / viscosity adjoints, and scatters the
// density adjoint onto gadj.w.  The stress matrix T = beta sig,
// beta = -4 V dt, sig = -p I + mu S (S the symmetric strain), depends on the
// density being gathered, so T enters after the gather by linearity:
//   sum_n grad w_n (g_n . T d_n) - w_n T^T g_n
//     = beta (-p P1 + mu P2 + p Q - mu S Q)
// with P1 = sum_n grad w_n (g_n . d_n), P2 = sum_n grad w_n (g_n . S d_n) and
// Q = sum_n w_n g_n.
// ---------------------------------------------------------------------------
template <class Tape, int L>
__global__ void __launch_bounds__(kThreads, MPM_ADJ_P2G2_MIN_BLOCKS)
    k_adj_p2g2(Tape tp, Particles Anew, float4* __restrict__ gadj,
               const AdjScene* __restrict__ scenes, const int* __restrict__ pscene,
               const int* __restrict__ perm, int n, double* __restrict__ pgrad) {
    const Lanes<L> ln = lanes_of<L>(n);
    const int i = perm ? perm[ln.j] : ln.j;
    const int scene = pscene[i];
    const AdjScene& sc = scenes[scene];
    const SimConsts& k = sc.k;
    const int lb = sc.lbase;
    float4* ga = gadj + lb;
    const Rec p = tp.rec(i);
    Sten st;
    make_sten(p.x, st);
    float strain[3][3];  // [row][col], symmetric
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) strain[a][b] = p.C[b][a] + p.C[a][b];

    // rho (1), m grad w (3), sum w g d^T row-major (9), P1 (3), P2 (3), Q (3)
    float acc[22] = {};
#pragma unroll
    for (int s = 0; s < slab_count<L>(); ++s) {
        const Slab sx = slab(st, slab_gx<L>(s, ln.q));
#pragma unroll
        for (int gy = 0; gy < 3; ++gy)
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const int c = node_index(st, sx.gx, gy, gz, k);
                if (c < 0) continue;
                const float4 g4 = ga[c];
                const float g[3] = {g4.x, g4.y, g4.z};
                const float m = tp.mass(lb + c, k.fm);
                Node nd;
                slab_node(st, p.x, sx, gy, gz, nd);
                acc[0] += m * nd.w;
                const float gd = g[0] * nd.dist[0] + g[1] * nd.dist[1] + g[2] * nd.dist[2];
                float gsd = 0.0f;
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    gsd += g[a] * (strain[a][0] * nd.dist[0] + strain[a][1] * nd.dist[1] +
                                   strain[a][2] * nd.dist[2]);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    acc[1 + a] += m * nd.gw[a];
                    acc[13 + a] += nd.gw[a] * gd;
                    acc[16 + a] += nd.gw[a] * gsd;
                    acc[19 + a] += nd.w * g[a];
#pragma unroll
                    for (int b = 0; b < 3; ++b) acc[4 + 3 * a + b] += nd.w * g[a] * nd.dist[b];
                }
            }
    }
    lane_sum<L>(acc);
    const float rho = acc[0];
    const float V = 1.0f / rho;
    const float r = rho / k.rest_density;
    const float r4 = (r * r) * (r * r);
    const float pterm = k.stiffness * (r4 * r - 1.0f);
    const float pres = fmaxf(pterm, 0.0f);
    const float mu = k.dynamic_viscosity;
    const float beta = -4.0f * V * k.dt;
    float xb[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float sq = strain[a][0] * acc[19] + strain[a][1] * acc[20] + strain[a][2] * acc[21];
        xb[a] = beta * (-pres * acc[13 + a] + mu * acc[16 + a] + pres * acc[19 + a] - mu * sq);
    }
    float sb[3][3], Vbar = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float sig = (a == b ? -pres : 0.0f) + mu * strain[a][b];
            sb[a][b] = beta * acc[4 + 3 * a + b];
            Vbar += -4.0f * k.dt * sig * acc[4 + 3 * a + b];
        }
    float gk = 0.0f, gmu = 0.0f;
    float Cb[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            Cb[b][a] = mu * (sb[a][b] + sb[b][a]);  // M(a, b) = C[b][a]
            gmu += strain[a][b] * sb[a][b];
        }
    const float pbar = -(sb[0][0] + sb[1][1] + sb[2][2]);
    float rhobar = -Vbar / (rho * rho);
    if (pterm > 0.0f) {
        gk = pbar * (r4 * r - 1.0f);
        rhobar += pbar * k.stiffness * 5.0f * r4 / k.rest_density;
    }
    if (ln.active) {
#pragma unroll
        for (int s = 0; s < slab_count<L>(); ++s) {
            const Slab sx = slab(st, slab_gx<L>(s, ln.q));
#pragma unroll
            for (int gy = 0; gy < 3; ++gy)
#pragma unroll
                for (int gz = 0; gz < 3; ++gz) {
                    const int c = node_index(st, sx.gx, gy, gz, k);
                    if (c < 0) continue;
                    const float w = (sx.w * st.w[1][gy]) * st.w[2][gz];
                    atomicAdd(reinterpret_cast<float*>(ga + c) + 3, rhobar * w);
                }
        }
    }
    const bool leader = ln.active && ln.q == 0;
    if (leader) {
        Rec an = load_rec(Anew, i);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            an.x[a] += xb[a] + rhobar * acc[1 + a];
#pragma unroll
            for (int b = 0; b < 3; ++b) an.C[a][b] += Cb[a][b];
        }
        store_rec(Anew, i, an);
    }
    add_param_grads(pgrad, scene, leader, gk, gmu);
}

// ---------------------------------------------------------------------------
// p2g_1 backward (p2g_1.wgsl:24-65): gathers the mass and momentum adjoints;
// sets the velocity adjoint and adds to the position and C adjoints.
// ---------------------------------------------------------------------------
template <class Tape, int L>
__global__ void __launch_bounds__(kThreads)
    k_adj_p2g1(Tape tp, Particles Anew, const float4* __restrict__ gadj,
               const AdjScene* __restrict__ scenes, const int* __restrict__ pscene,
               const int* __restrict__ perm, int n) {
    const Lanes<L> ln = lanes_of<L>(n);
    const int i = perm ? perm[ln.j] : ln.j;
    const AdjScene& sc = scenes[pscene[i]];
    const SimConsts& k = sc.k;
    const float4* ga = gadj + sc.lbase;
    const Rec p = tp.rec(i);
    Sten st;
    make_sten(p.x, st);
    float acc[15] = {};  // v adjoint (3), C adjoint C[b][a] at 3 + 3b + a (9), x adjoint (3)
#pragma unroll
    for (int s = 0; s < slab_count<L>(); ++s) {
        const Slab sx = slab(st, slab_gx<L>(s, ln.q));
#pragma unroll
        for (int gy = 0; gy < 3; ++gy)
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const int c = node_index(st, sx.gx, gy, gz, k);
                if (c < 0) continue;
                const float4 g4 = __ldg(ga + c);
                Node nd;
                slab_node(st, p.x, sx, gy, gz, nd);
                const float g[3] = {g4.x, g4.y, g4.z};
                float s2 = g4.w;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const float q = p.v[a] + (p.C[0][a] * nd.dist[0] + p.C[1][a] * nd.dist[1] +
                                              p.C[2][a] * nd.dist[2]);
                    s2 += g[a] * q;
                    acc[a] += nd.w * g[a];
#pragma unroll
                    for (int b = 0; b < 3; ++b) acc[3 + 3 * b + a] += nd.w * g[a] * nd.dist[b];
                }
#pragma unroll
                for (int c2 = 0; c2 < 3; ++c2)
                    acc[12 + c2] += nd.gw[c2] * s2 -
                                    nd.w * (p.C[c2][0] * g[0] + p.C[c2][1] * g[1] + p.C[c2][2] * g[2]);
            }
    }
    lane_sum<L>(acc);
    if (!(ln.active && ln.q == 0)) return;
    Rec an = load_rec(Anew, i);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        an.v[a] = acc[a];
        an.x[a] += acc[12 + a];
#pragma unroll
        for (int b = 0; b < 3; ++b) an.C[b][a] += acc[3 + 3 * b + a];
    }
    store_rec(Anew, i, an);
}

// 80-byte reference records (x, v, C columns padded to four floats) <->
// FP64 tape records.
__global__ void k_records_to_rec64(const float* __restrict__ rec, double* __restrict__ S, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* P = rec + 20 * (size_t)i;
    double* q = S + (size_t)kRec64 * i;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        q[a] = P[a];
        q[3 + a] = P[4 + a];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) q[6 + 3 * c + r] = P[8 + 4 * c + r];
    q[15] = 0.0;
}

__global__ void k_rec64_to_records(const double* __restrict__ S, float* __restrict__ rec, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* q = S + (size_t)kRec64 * i;
    float* P = rec + 20 * (size_t)i;
#pragma unroll
    for (int j = 0; j < 20; ++j) P[j] = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        P[a] = (float)q[a];
        P[4 + a] = (float)q[3 + a];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) P[8 + 4 * c + r] = (float)q[6 + 3 * c + r];
}

// Squared-distance loss of one observed substep (inverse problems), per
// particle i of scene s: d = x_i - obs_i in f32, seed_i = the adjoint record
// whose position is scale[s] * d (scale = f32(2 / particles of s)) and whose
// other entries are 0, and loss[s] += |d|^2 summed in FP64.  A warp whose
// particles all belong to one scene adds one reduced term.
template <bool F64>
__global__ void k_obs_loss(Particles X, const double* __restrict__ X64,
                           const float4* __restrict__ obs, const int* __restrict__ pscene,
                           const float* __restrict__ scale, Particles seed,
                           double* __restrict__ loss, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < n;
    int s = -1;
    double sq = 0.0;
    if (act) {
        float x0, x1, x2;
        if (F64) {
            const double* q = X64 + (size_t)kRec64 * i;
            x0 = (float)q[0];
            x1 = (float)q[1];
            x2 = (float)q[2];
        } else {
            const float4 a = X.p0[i];
            x0 = a.x;
            x1 = a.y;
            x2 = a.z;
        }
        const float4 o = obs[i];
        const float dx = __fsub_rn(x0, o.x), dy = __fsub_rn(x1, o.y), dz = __fsub_rn(x2, o.z);
        s = pscene[i];
        const float c = scale[s];
        const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        seed.p0[i] = make_float4(__fmul_rn(dx, c), __fmul_rn(dy, c), __fmul_rn(dz, c), 0.0f);
        seed.p1[i] = zero;
        seed.p2[i] = zero;
        seed.p3[i] = zero;
        sq = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    }
    const int s0 = __shfl_sync(0xffffffffu, s, 0);
    if (__all_sync(0xffffffffu, !act || s == s0)) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, off);
        if ((threadIdx.x & 31) == 0 && s0 >= 0) atomicAdd(loss + s0, sq);
    } else if (act) {
        atomicAdd(loss + s, sq);
    }
}

// A += B over n records (all four streams).
__global__ void k_axpy(Particles A, Particles B, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4* a[4] = {A.p0, A.p1, A.p2, A.p3};
    const float4* b[4] = {B.p0, B.p1, B.p2, B.p3};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        float4 u = a[q][i];
        const float4 v = b[q][i];
        u.x += v.x; u.y += v.y; u.z += v.z; u.w += v.w;
        a[q][i] = u;
    }
}

// ---------------------------------------------------------------------------
// FP64 forward of the continuous model (the FP64 tape): the same stages,
// stencils, flat indices, boundary rules and branches as the fixed-point
// kernels, with double grid sums and no encode/decode.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int d2i_sat(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT_MAX;
    if (x <= -2147483648.0) return INT_MIN;
    return (int)x;
}

__device__ __forceinline__ int flat64(double cx, double cy, double cz, int Y, int Z) {
    const unsigned a = (unsigned)d2i_sat(cx) * (unsigned)Y * (unsigned)Z;
    const unsigned b = (unsigned)d2i_sat(cy) * (unsigned)Z;
    return (int)(a + b + (unsigned)d2i_sat(cz));
}

__device__ __forceinline__ void weights64(const double* x, double ci[3], double w[3][3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ci[a] = floor(x[a]);
        const double d = x[a] - (ci[a] + 0.5);
        w[a][0] = 0.5 * (0.5 - d) * (0.5 - d);
        w[a][1] = 0.75 - d * d;
        w[a][2] = 0.5 * (0.5 + d) * (0.5 + d);
    }
}

// One thread per particle: these kernels are bound by FP64 arithmetic, so
// splitting a particle's stencil over lanes (which repeats the weights)
// only adds work.
__global__ void __launch_bounds__(kThreads)
    k64_p2g(const double* __restrict__ S, double4* __restrict__ G,
            const AdjScene* __restrict__ scenes, const int* __restrict__ pscene, int n, int stage) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const AdjScene& sc = scenes[pscene[i]];
    const SimConsts& k = sc.k;
    double* grid = reinterpret_cast<double*>(G + sc.lbase);
    const double* P = S + (size_t)kRec64 * i;
    double x[3] = {P[0], P[1], P[2]};
    double ci[3], w[3][3];
    weights64(x, ci, w);
    double T[3][3];  // stage 2: [row][col]
    if (stage == 2) {
        double rho = 0.0;
#pragma unroll
        for (int gx = 0; gx < 3; ++gx)
#pragma unroll
            for (int gy = 0; gy < 3; ++gy)
#pragma unroll
                for (int gz = 0; gz < 3; ++gz) {
                    const double wt = w[0][gx] * w[1][gy] * w[2][gz];
                    const int idx = flat64(ci[0] + gx - 1.0, ci[1] + gy - 1.0, ci[2] + gz - 1.0,
                                           k.Y, k.Z);
                    if ((unsigned)idx >= (unsigned)k.grid_count) continue;
                    rho += grid[4 * (size_t)idx + 3] * wt;
                }
        const double V = 1.0 / rho;
        const double rr = rho / (double)k.rest_density;
        const double pterm = (double)k.stiffness * (rr * rr * rr * rr * rr - 1.0);
        const double pres = pterm > 0.0 ? pterm : 0.0;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const double strain = P[6 + 3 * b + a] + P[6 + 3 * a + b];
                const double sig = (a == b ? -pres : 0.0) + (double)k.dynamic_viscosity * strain;
                T[a][b] = -V * 4.0 * sig * (double)k.dt;
            }
    }
#pragma unroll
    for (int gx = 0; gx < 3; ++gx)
#pragma unroll
        for (int gy = 0; gy < 3; ++gy)
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const double wt = w[0][gx] * w[1][gy] * w[2][gz];
                const double c[3] = {ci[0] + gx - 1.0, ci[1] + gy - 1.0, ci[2] + gz - 1.0};
                double d[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) d[a] = (c[a] + 0.5) - x[a];
                const int idx = flat64(c[0], c[1], c[2], k.Y, k.Z);
                if ((unsigned)idx >= (unsigned)k.grid_count) continue;
                double* cell = grid + 4 * (size_t)idx;
                if (stage == 1) {
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        const double q = P[6 + r] * d[0] + P[9 + r] * d[1] + P[12 + r] * d[2];
                        atomicAdd(cell + r, wt * (P[3 + r] + q));
                    }
                    atomicAdd(cell + 3, wt);
                } else {
#pragma unroll
                    for (int r = 0; r < 3; ++r)
                        atomicAdd(cell + r, wt * (T[r][0] * d[0] + T[r][1] * d[1] + T[r][2] * d[2]));
                }
            }
}

__global__ void __launch_bounds__(kThreads)
    k64_update(double4* __restrict__ G, const AdjScene* __restrict__ scenes, int nscenes,
               int ncells) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncells) return;
    int lo = 0, hi = nscenes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (scenes[mid].lbase <= j) lo = mid;
        else hi = mid - 1;
    }
    const SimConsts& k = scenes[lo].k;
    double4 c = G[j];
    if (!(c.w > 0.0)) return;
    const int id = j - scenes[lo].lbase;
    const int xyz[3] = {(id / k.Z) / k.Y, (id / k.Z) % k.Y, id % k.Z};
    double v[3] = {c.x, c.y, c.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int hiw = d2i_sat(ceil((double)k.real_box[a]) - 3.0);
        double u = v[a] / c.w + (double)k.gravity[a] * (double)k.dt;
        if (xyz[a] < 2 || xyz[a] > hiw) u = 0.0;
        v[a] = u;
    }
    c.x = v[0];
    c.y = v[1];
    c.z = v[2];
    G[j] = c;
}

__global__ void __launch_bounds__(kThreads)
    k64_g2p(const double* __restrict__ S, const double4* __restrict__ G, double* __restrict__ Sout,
            const AdjScene* __restrict__ scenes, const int* __restrict__ pscene, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const AdjScene& sc = scenes[pscene[i]];
    const SimConsts& k = sc.k;
    const double4* grid = G + sc.lbase;
    const double* P = S + (size_t)kRec64 * i;
    double* Q = Sout + (size_t)kRec64 * i;
    const double x[3] = {P[0], P[1], P[2]};
    double ci[3], w[3][3];
    weights64(x, ci, w);
    double acc[12] = {};  // v (3), then B[c][r] at 3 + 3c + r
#pragma unroll
    for (int gx = 0; gx < 3; ++gx)
#pragma unroll
        for (int gy = 0; gy < 3; ++gy)
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const double wt = w[0][gx] * w[1][gy] * w[2][gz];
                const double c[3] = {ci[0] + gx - 1.0, ci[1] + gy - 1.0, ci[2] + gz - 1.0};
                double d[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) d[a] = (c[a] + 0.5) - x[a];
                const int idx = flat64(c[0], c[1], c[2], k.Y, k.Z);
                double gv[3] = {0.0, 0.0, 0.0};
                if ((unsigned)idx < (unsigned)k.grid_count) {
                    const double4 cc = grid[idx];
                    gv[0] = cc.x; gv[1] = cc.y; gv[2] = cc.z;
                }
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const double wv = gv[r] * wt;
#pragma unroll
                    for (int q = 0; q < 3; ++q) acc[3 + 3 * q + r] += wv * d[q];
                    acc[r] += wv;
                }
    }
    const double v[3] = {acc[0], acc[1], acc[2]};
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
        for (int r = 0; r < 3; ++r) Q[6 + 3 * q + r] = acc[3 + 3 * q + r] * 4.0;
    double xo[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double xx = x[a] + v[a] * (double)k.dt;
        const double hw = (double)k.real_box[a] - 2.0;
        xx = xx < 1.0 ? 1.0 : xx;
        xx = xx > hw ? hw : xx;
        xo[a] = xx;
        Q[a] = xx;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double xn = xo[a] + v[a] * (double)k.dt * 3.0;
        const double wmax = (double)k.real_box[a] - 4.0;
        double va = v[a];
        if (xn < 3.0) va += 0.3 * (3.0 - xn);
        if (xn > wmax) va += 0.3 * (wmax - xn);
        Q[3 + a] = va;
    }
    Q[15] = 0.0;
}

inline int blocks(long long n) { return (int)((n + kThreads - 1) / kThreads); }


template <class Tape, int L>
void adjoint_kernels(const Tape& tp, const Particles& Aout, const Particles& Anew, float4* gadj,
                     const AdjScene* scenes, int nscenes, const int* pscene, int n, int ncells,
                     double* pgrad, const int* perm, cudaStream_t st) {
    const int pb = lane_blocks<L>(n);
    k_adj_g2p<Tape, L><<<pb, kThreads, 0, st>>>(tp, Aout, Anew, gadj, scenes, pscene, perm, n);
    k_adj_update<Tape><<<blocks(ncells), kThreads, 0, st>>>(tp, gadj, scenes, nscenes, ncells);
    k_adj_p2g2<Tape, L><<<pb, kThreads, 0, st>>>(tp, Anew, gadj, scenes, pscene, perm, n, pgrad);
    k_adj_p2g1<Tape, L><<<pb, kThreads, 0, st>>>(tp, Anew, gadj, scenes, pscene, perm, n);
}

template <class Tape>
void adjoint_substep(const Tape& tp, const Particles& Aout, const Particles& Anew, float4* gadj,
                     const AdjScene* scenes, int nscenes, const int* pscene, int n, int ncells,
                     double* pgrad, const AdjSort& so, cudaStream_t st) {
    if (n <= 0) return;
    cudaMemsetAsync(gadj, 0, sizeof(float4) * (size_t)ncells, st);
    if (so.lanes == 3) {  // small batch: the sort's launches would cost more than it saves
        adjoint_kernels<Tape, 3>(tp, Aout, Anew, gadj, scenes, nscenes, pscene, n, ncells, pgrad,
                                 nullptr, st);
        return;
    }
    cudaMemsetAsync(so.bin_count, 0, sizeof(int) * (size_t)so.nbins, st);
    cudaMemsetAsync(so.placed, 0, sizeof(int), st);
    k_adj_bin<Tape><<<blocks(n), kThreads, 0, st>>>(tp, scenes, pscene, n, so);
    k_adj_place<<<blocks(so.nbins), kThreads, 0, st>>>(so);
    k_adj_perm<<<blocks(n), kThreads, 0, st>>>(so, n);
    adjoint_kernels<Tape, 1>(tp, Aout, Anew, gadj, scenes, nscenes, pscene, n, ncells, pgrad,
                             so.perm, st);
}

}  // namespace

void adj_bricks(const SimConsts& k, int& BX, int& BY, int& BZ) {
    const long long yz = (long long)k.Y * k.Z;
    const long long xi = yz > 0 ? ((long long)k.grid_count + yz - 1) / yz : 0;
    BX = (int)((xi + 3) / 4);
    BY = (k.Y + 3) / 4;
    BZ = (k.Z + 3) / 4;
}

void launch_adjoint_substep(const Particles& S, const int4* G, const Particles& Aout,
                            const Particles& Anew, float4* gadj, const AdjScene* scenes,
                            int nscenes, const int* pscene, int n, int ncells, double* pgrad,
                            const AdjSort& so, cudaStream_t st) {
    adjoint_substep(TapeFixed{S, G}, Aout, Anew, gadj, scenes, nscenes, pscene, n, ncells, pgrad,
                    so, st);
}

void launch_adjoint_substep64(const double* S, const double4* G, const Particles& Aout,
                              const Particles& Anew, float4* gadj, const AdjScene* scenes,
                              int nscenes, const int* pscene, int n, int ncells, double* pgrad,
                              const AdjSort& so, cudaStream_t st) {
    adjoint_substep(Tape64{S, G}, Aout, Anew, gadj, scenes, nscenes, pscene, n, ncells, pgrad,
                    so, st);
}

void launch_substep64(const double* S, double4* G, double* Sout, const AdjScene* scenes,
                      int nscenes, const int* pscene, int n, int ncells, cudaStream_t st) {
    cudaMemsetAsync(G, 0, sizeof(double4) * (size_t)ncells, st);
    if (n > 0) {
        k64_p2g<<<blocks(n), kThreads, 0, st>>>(S, G, scenes, pscene, n, 1);
        k64_p2g<<<blocks(n), kThreads, 0, st>>>(S, G, scenes, pscene, n, 2);
    }
    k64_update<<<blocks(ncells), kThreads, 0, st>>>(G, scenes, nscenes, ncells);
    if (n > 0) k64_g2p<<<blocks(n), kThreads, 0, st>>>(S, G, Sout, scenes, pscene, n);
}

void launch_records_to_rec64(const float* rec, double* S, int n, cudaStream_t st) {
    if (n <= 0) return;
    k_records_to_rec64<<<blocks(n), kThreads, 0, st>>>(rec, S, n);
}

void launch_rec64_to_records(const double* S, float* rec, int n, cudaStream_t st) {
    if (n <= 0) return;
    k_rec64_to_records<<<blocks(n), kThreads, 0, st>>>(S, rec, n);
}

void launch_obs_loss(const Particles* X, const double* X64, const float4* obs, const int* pscene,
                     const float* scale, const Particles& seed, double* loss, int n,
                     cudaStream_t st) {
    if (n <= 0) return;
    if (X64)
        k_obs_loss<true><<<blocks(n), kThreads, 0, st>>>(Particles{}, X64, obs, pscene, scale,
                                                         seed, loss, n);
    else
        k_obs_loss<false><<<blocks(n), kThreads, 0, st>>>(*X, nullptr, obs, pscene, scale, seed,
                                                          loss, n);
}

void launch_particles_axpy(const Particles& A, const Particles& B, int n, cudaStream_t st) {
    if (n <= 0) return;
    k_axpy<<<blocks(n), kThreads, 0, st>>>(A, B, n);
}

}  // namespace mpm
