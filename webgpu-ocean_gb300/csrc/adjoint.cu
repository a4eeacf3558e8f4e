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
//   k_adj_g2p     particle-parallel; the g2p gather becomes a float scatter
//                 of the grid-velocity adjoint (3 atomics per stencil cell)
//   k_adj_update  cell-parallel, elementwise: velocity adjoint -> momentum
//                 and mass adjoints
//   k_adj_p2g2    particle-parallel gather of the momentum adjoint through
//                 the stress term; the density gather becomes a scatter of
//                 the density adjoint onto the mass adjoint
//   k_adj_p2g1    particle-parallel gather of the mass and momentum adjoints
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

// Stencil cell (gx, gy, gz): its weight, weight gradient, dist and flat index
// (false when outside [0, grid_count)).
struct Node {
    float w;
    float gw[3];
    float dist[3];
    int idx;
};

__device__ __forceinline__ bool node(const Sten& s, const float x[3], int gx, int gy, int gz,
                                     const SimConsts& k, Node& nd) {
    const float wx = s.w[0][gx], wy = s.w[1][gy], wz = s.w[2][gz];
    nd.w = (wx * wy) * wz;
    nd.gw[0] = (s.dw[0][gx] * wy) * wz;
    nd.gw[1] = (wx * s.dw[1][gy]) * wz;
    nd.gw[2] = (wx * wy) * s.dw[2][gz];
    const float cx = s.cf[0] + (float)gx - 1.0f;
    const float cy = s.cf[1] + (float)gy - 1.0f;
    const float cz = s.cf[2] + (float)gz - 1.0f;
    nd.dist[0] = (cx + 0.5f) - x[0];
    nd.dist[1] = (cy + 0.5f) - x[1];
    nd.dist[2] = (cz + 0.5f) - x[2];
    nd.idx = flat_index(cx, cy, cz, k.Y, k.Z);
    return (unsigned)nd.idx < (unsigned)k.grid_count;
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

// Lanes per particle in the particle-parallel adjoint kernels: lane q of a
// group of kLanes consecutive lanes takes stencil cells q, q + kLanes, ...
// of the 27, and the group sums its partial results with shuffles.  Small
// scenes then still fill the GPU.
constexpr int kLanes = 4;

template <class R, int N>
__device__ __forceinline__ void group_sum(R (&v)[N]) {
#pragma unroll
    for (int o = 1; o < kLanes; o <<= 1)
#pragma unroll
        for (int j = 0; j < N; ++j) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
}

// ---------------------------------------------------------------------------
// g2p backward (g2p.wgsl:26-92).  Aout: adjoint of S_{t+1}; writes the g2p
// part of the position adjoint of S_t into Anew (velocity and C adjoints
// zeroed) and scatters the grid-velocity adjoint into gadj.xyz.
// ---------------------------------------------------------------------------
template <class Tape>
__global__ void __launch_bounds__(kThreads)
    k_adj_g2p(Tape tp, Particles Aout, Particles Anew, float4* __restrict__ gadj,
              const AdjScene* __restrict__ scenes, const int* __restrict__ pscene, int n) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = gi & (kLanes - 1);
    const bool active = gi / kLanes < n;
    const int i = active ? gi / kLanes : n - 1;
    const AdjScene& sc = scenes[pscene[i]];
    const SimConsts& k = sc.k;
    const int lb = sc.lbase;
    float4* ga = gadj + lb;
    float x[3];
    tp.pos(i, x);
    Sten st;
    make_sten(x, st);

    float vg[3] = {0.0f, 0.0f, 0.0f};
    for (int nn = lane; nn < 27; nn += kLanes) {
        Node nd;
        if (!node(st, x, nn / 9, (nn / 3) % 3, nn % 3, k, nd)) continue;
        float vi[3];
        tp.vel(lb + nd.idx, k.fm, vi);
        vg[0] += nd.w * vi[0];
        vg[1] += nd.w * vi[1];
        vg[2] += nd.w * vi[2];
    }
    group_sum(vg);

    const Rec ao = load_rec(Aout, i);
    float xbar[3], vgbar[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float xt = x[a] + vg[a] * k.dt;
        const float hiw = k.real_box[a] - 2.0f;
        const bool inside = xt >= 1.0f && xt <= hiw;
        const float xc = fminf(fmaxf(xt, 1.0f), hiw);
        const float xn = xc + (vg[a] * k.dt) * 3.0f;
        const float nw = (xn < 3.0f ? 1.0f : 0.0f) + (xn > k.real_box[a] - 4.0f ? 1.0f : 0.0f);
        const float xcbar = ao.x[a] - 0.3f * nw * ao.v[a];
        const float xtbar = inside ? xcbar : 0.0f;
        vgbar[a] = ao.v[a] * (1.0f - 0.9f * k.dt * nw) + k.dt * xtbar;
        xbar[a] = lane == 0 ? xtbar : 0.0f;
    }

    for (int nn = lane; nn < 27; nn += kLanes) {
        Node nd;
        if (!node(st, x, nn / 9, (nn / 3) % 3, nn % 3, k, nd)) continue;
        float vi[3];
        tp.vel(lb + nd.idx, k.fm, vi);
        float q[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
            q[r] = vgbar[r] + 4.0f * (ao.C[0][r] * nd.dist[0] + ao.C[1][r] * nd.dist[1] +
                                      ao.C[2][r] * nd.dist[2]);
        if (active) {
            float* cell = reinterpret_cast<float*>(ga + nd.idx);
            atomicAdd(cell + 0, nd.w * q[0]);
            atomicAdd(cell + 1, nd.w * q[1]);
            atomicAdd(cell + 2, nd.w * q[2]);
        }
        const float s = vi[0] * q[0] + vi[1] * q[1] + vi[2] * q[2];
#pragma unroll
        for (int a = 0; a < 3; ++a)
            xbar[a] += nd.gw[a] * s - 4.0f * nd.w *
                                          (ao.C[a][0] * vi[0] + ao.C[a][1] * vi[1] +
                                           ao.C[a][2] * vi[2]);
    }
    group_sum(xbar);

    if (active && lane == 0) {
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
    int lo = 0, hi = nscenes - 1;  // last scene with lbase <= j
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (scenes[mid].lbase <= j) lo = mid;
        else hi = mid - 1;
    }
    const SimConsts& k = scenes[lo].k;
    const int id = j - scenes[lo].lbase;
    const float4 vb = gadj[j];
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
// density adjoint onto gadj.w.
// ---------------------------------------------------------------------------
template <class Tape>
__global__ void __launch_bounds__(kThreads)
    k_adj_p2g2(Tape tp, Particles Anew, float4* __restrict__ gadj,
               const AdjScene* __restrict__ scenes, const int* __restrict__ pscene, int n,
               double* __restrict__ pgrad) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = gi & (kLanes - 1);
    const bool active = gi / kLanes < n;
    const int i = active ? gi / kLanes : n - 1;
    const int scene = pscene[i];
    const AdjScene& sc = scenes[scene];
    const SimConsts& k = sc.k;
    const int lb = sc.lbase;
    float4* ga = gadj + lb;
    const Rec p = tp.rec(i);
    Sten st;
    make_sten(p.x, st);
    float rho[1] = {0.0f};
    for (int nn = lane; nn < 27; nn += kLanes) {
        Node nd;
        if (!node(st, p.x, nn / 9, (nn / 3) % 3, nn % 3, k, nd)) continue;
        rho[0] += tp.mass(lb + nd.idx, k.fm) * nd.w;
    }
    group_sum(rho);
    const float V = 1.0f / rho[0];
    const float r = rho[0] / k.rest_density;
    const float r4 = (r * r) * (r * r);
    const float pterm = k.stiffness * (r4 * r - 1.0f);
    const float pres = fmaxf(pterm, 0.0f);
    float T[3][3], sig[3][3], strain[3][3];  // [row][col]
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            strain[a][b] = p.C[b][a] + p.C[a][b];
            sig[a][b] = (a == b ? -pres : 0.0f) + k.dynamic_viscosity * strain[a][b];
            T[a][b] = -4.0f * V * k.dt * sig[a][b];
        }
    float acc[12] = {};  // Tb (row-major 9), then the position adjoint (3)
    for (int nn = lane; nn < 27; nn += kLanes) {
        Node nd;
        if (!node(st, p.x, nn / 9, (nn / 3) % 3, nn % 3, k, nd)) continue;
        const float4 g4 = ga[nd.idx];
        const float g[3] = {g4.x, g4.y, g4.z};
        float s = 0.0f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float td = T[a][0] * nd.dist[0] + T[a][1] * nd.dist[1] + T[a][2] * nd.dist[2];
            s += g[a] * td;
#pragma unroll
            for (int b = 0; b < 3; ++b) acc[3 * a + b] += nd.w * g[a] * nd.dist[b];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
            acc[9 + c] += nd.gw[c] * s - nd.w * (T[0][c] * g[0] + T[1][c] * g[1] + T[2][c] * g[2]);
    }
    group_sum(acc);
    float sb[3][3], Vbar = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            sb[a][b] = -4.0f * V * k.dt * acc[3 * a + b];
            Vbar += -4.0f * k.dt * sig[a][b] * acc[3 * a + b];
        }
    float gk = 0.0f, gmu = 0.0f;
    float Cb[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            Cb[b][a] = k.dynamic_viscosity * (sb[a][b] + sb[b][a]);  // M(a, b) = C[b][a]
            gmu += strain[a][b] * sb[a][b];
        }
    const float pbar = -(sb[0][0] + sb[1][1] + sb[2][2]);
    float rhobar = -Vbar / (rho[0] * rho[0]);
    if (pterm > 0.0f) {
        gk = pbar * (r4 * r - 1.0f);
        rhobar += pbar * k.stiffness * 5.0f * r4 / k.rest_density;
    }
    float xb[3] = {0.0f, 0.0f, 0.0f};
    for (int nn = lane; nn < 27; nn += kLanes) {
        Node nd;
        if (!node(st, p.x, nn / 9, (nn / 3) % 3, nn % 3, k, nd)) continue;
        if (active) atomicAdd(reinterpret_cast<float*>(ga + nd.idx) + 3, rhobar * nd.w);
        const float m = tp.mass(lb + nd.idx, k.fm);
#pragma unroll
        for (int c = 0; c < 3; ++c) xb[c] += rhobar * m * nd.gw[c];
    }
    group_sum(xb);
    const bool leader = active && lane == 0;
    if (leader) {
        Rec an = load_rec(Anew, i);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            an.x[a] += acc[9 + a] + xb[a];
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
template <class Tape>
__global__ void __launch_bounds__(kThreads)
    k_adj_p2g1(Tape tp, Particles Anew, const float4* __restrict__ gadj,
               const AdjScene* __restrict__ scenes, const int* __restrict__ pscene, int n) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = gi & (kLanes - 1);
    const bool active = gi / kLanes < n;
    const int i = active ? gi / kLanes : n - 1;
    const AdjScene& sc = scenes[pscene[i]];
    const SimConsts& k = sc.k;
    const float4* ga = gadj + sc.lbase;
    const Rec p = tp.rec(i);
    Sten st;
    make_sten(p.x, st);
    float acc[15] = {};  // v adjoint (3), C adjoint C[b][a] at 3 + 3b + a (9), x adjoint (3)
    for (int nn = lane; nn < 27; nn += kLanes) {
        Node nd;
        if (!node(st, p.x, nn / 9, (nn / 3) % 3, nn % 3, k, nd)) continue;
        const float4 g4 = __ldg(ga + nd.idx);
        const float g[3] = {g4.x, g4.y, g4.z};
        float s = g4.w;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float q = p.v[a] + (p.C[0][a] * nd.dist[0] + p.C[1][a] * nd.dist[1] +
                                      p.C[2][a] * nd.dist[2]);
            s += g[a] * q;
            acc[a] += nd.w * g[a];
#pragma unroll
            for (int b = 0; b < 3; ++b) acc[3 + 3 * b + a] += nd.w * g[a] * nd.dist[b];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
            acc[12 + c] += nd.gw[c] * s -
                           nd.w * (p.C[c][0] * g[0] + p.C[c][1] * g[1] + p.C[c][2] * g[2]);
    }
    group_sum(acc);
    if (!(active && lane == 0)) return;
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

}  // namespace

template <class Tape>
void adjoint_substep(const Tape& tp, const Particles& Aout, const Particles& Anew, float4* gadj,
                     const AdjScene* scenes, int nscenes, const int* pscene, int n, int ncells,
                     double* pgrad, cudaStream_t st) {
    if (n <= 0) return;
    cudaMemsetAsync(gadj, 0, sizeof(float4) * (size_t)ncells, st);
    const int pb = blocks((long long)n * kLanes);
    k_adj_g2p<Tape><<<pb, kThreads, 0, st>>>(tp, Aout, Anew, gadj, scenes, pscene, n);
    k_adj_update<Tape><<<blocks(ncells), kThreads, 0, st>>>(tp, gadj, scenes, nscenes, ncells);
    k_adj_p2g2<Tape><<<pb, kThreads, 0, st>>>(tp, Anew, gadj, scenes, pscene, n, pgrad);
    k_adj_p2g1<Tape><<<pb, kThreads, 0, st>>>(tp, Anew, gadj, scenes, pscene, n);
}

void launch_adjoint_substep(const Particles& S, const int4* G, const Particles& Aout,
                            const Particles& Anew, float4* gadj, const AdjScene* scenes,
                            int nscenes, const int* pscene, int n, int ncells, double* pgrad,
                            cudaStream_t st) {
    adjoint_substep(TapeFixed{S, G}, Aout, Anew, gadj, scenes, nscenes, pscene, n, ncells, pgrad,
                    st);
}

void launch_adjoint_substep64(const double* S, const double4* G, const Particles& Aout,
                              const Particles& Anew, float4* gadj, const AdjScene* scenes,
                              int nscenes, const int* pscene, int n, int ncells, double* pgrad,
                              cudaStream_t st) {
    adjoint_substep(Tape64{S, G}, Aout, Anew, gadj, scenes, nscenes, pscene, n, ncells, pgrad,
                    st);
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

void launch_particles_axpy(const Particles& A, const Particles& B, int n, cudaStream_t st) {
    if (n <= 0) return;
    k_axpy<<<blocks(n), kThreads, 0, st>>>(A, B, n);
}

}  // namespace mpm
