// kernels_dispatch.cu -- one CUDA kernel per WGSL entry point of the
// reference's MLS-MPM substep, one thread per particle or per cell, global
// i32 atomics.  This engine keeps the reference's dispatch structure
// (mls-mpm/mls-mpm.ts:245-268) so each stage can be run and checked alone;
// the sorted engine (kernels_sorted.cu) is the fast path and must agree with
// it bit for bit.
#include "mpm_internal.h"
#include "mpm_math_x2.cuh"

namespace mpm {

namespace {

constexpr int kThreads = 256;

inline int blocks_for(long long n) { return (int)((n + kThreads - 1) / kThreads); }

__device__ __forceinline__ bool in_grid(int idx, int grid_count) {
    return (unsigned)idx < (unsigned)grid_count;
}

// clearGrid.wgsl:10-18
__global__ void k_clear_grid(int4* __restrict__ cells, int grid_count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < grid_count) cells[i] = make_int4(0, 0, 0, 0);
}

// p2g_1.wgsl:24-65
__global__ void k_p2g_1(Particles P, int4* __restrict__ cells, SimConsts k,
                        unsigned long long* __restrict__ oob) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    PState s;
    load_particle(P, i, s);
    unsigned bad = 0;
    p2g1_particle(s, k, [&](int idx, int, int, int, int m, int vx, int vy, int vz) {
        if (!in_grid(idx, k.grid_count)) { ++bad; return; }
        int* c = reinterpret_cast<int*>(cells + idx);
        atomicAdd(c + 3, m);
        atomicAdd(c + 0, vx);
        atomicAdd(c + 1, vy);
        atomicAdd(c + 2, vz);
    });
    if (bad) atomicAdd(oob, (unsigned long long)bad);
}

// p2g_2.wgsl:30-94
__global__ void k_p2g_2(Particles P, int4* __restrict__ cells, SimConsts k,
                        unsigned long long* __restrict__ oob) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    PState s;
    {
        float4 a = P.p0[i], b = P.p1[i], c = P.p2[i];
        unpack_xC(a, b, c, s);
    }
    unsigned bad = 0;
    p2g2_particle(
        s, k,
        [&](int idx, int, int, int) -> float {
            if (!in_grid(idx, k.grid_count)) { ++bad; return dec(0, k.fm); }
            return dec(__ldcg(reinterpret_cast<const int*>(cells + idx) + 3), k.fm);
        },
        [&](int idx, int, int, int, int mx, int my, int mz) {
            if (!in_grid(idx, k.grid_count)) { ++bad; return; }
            int* c = reinterpret_cast<int*>(cells + idx);
            atomicAdd(c + 0, mx);
            atomicAdd(c + 1, my);
            atomicAdd(c + 2, mz);
        });
    if (bad) atomicAdd(oob, (unsigned long long)bad);
}

// updateGrid.wgsl:23-46
__global__ void k_update_grid(int4* __restrict__ cells, SimConsts k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.grid_count) return;
    const int4 c = cells[i];
    if (!(c.w > 0)) return;
    cells[i] = update_cell(c, i, k, wall_hi(k.real_box[0]), wall_hi(k.real_box[1]),
                           wall_hi(k.real_box[2]));
}

// g2p.wgsl:26-92
__global__ void k_g2p(Particles P, const int4* __restrict__ cells, SimConsts k,
                      unsigned long long* __restrict__ oob) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    PState s;
    {
        float4 a = P.p0[i], b = P.p1[i], c = P.p2[i];
        unpack_xC(a, b, c, s);
    }
    unsigned bad = 0;
    g2p_particle(s, k, [&](int idx, int, int, int, float out[3]) {
        int4 c = make_int4(0, 0, 0, 0);
        if (in_grid(idx, k.grid_count)) c = cells[idx];
        else ++bad;
        out[0] = dec(c.x, k.fm);
        out[1] = dec(c.y, k.fm);
        out[2] = dec(c.z, k.fm);
    });
    store_particle(P, i, s);
    if (bad) atomicAdd(oob, (unsigned long long)bad);
}

// copyPosition.wgsl:15-21
__global__ void k_copy_position(Particles P, float4* __restrict__ posvel, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = P.p0[i];
    const float4 v = P.p3[i];
    posvel[2 * i + 0] = make_float4(a.x, a.y, a.z, 0.0f);
    posvel[2 * i + 1] = make_float4(v.x, v.y, v.z, 0.0f);
}

__global__ void k_canonicalize(Particles src, const uint32_t* __restrict__ id, Particles dst,
                               uint32_t* __restrict__ id_dst, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t i = id[j];
    dst.p0[i] = src.p0[j];
    dst.p1[i] = src.p1[j];
    dst.p2[i] = src.p2[j];
    dst.p3[i] = src.p3[j];
    if (id_dst) id_dst[j] = (uint32_t)j;
}

__global__ void k_iota(uint32_t* __restrict__ id, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) id[j] = (uint32_t)j;
}

// 80-byte reference records (20 floats: x, pad, v, pad, C columns padded to
// four) <-> the four float4 streams.  Record i is five aligned float4.
__global__ void k_records_to_streams(const float4* __restrict__ rec, Particles P, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* r = rec + 5 * (size_t)i;
    const float4 a = r[0], b = r[1], c = r[2], d = r[3], e = r[4];
    P.p0[i] = make_float4(a.x, a.y, a.z, c.x);
    P.p1[i] = make_float4(c.y, c.z, d.x, d.y);
    P.p2[i] = make_float4(d.z, e.x, e.y, e.z);
    P.p3[i] = make_float4(b.x, b.y, b.z, 0.0f);
}

__global__ void k_streams_to_records(Particles P, float4* __restrict__ rec, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = P.p0[i], b = P.p1[i], c = P.p2[i], d = P.p3[i];
    float4* r = rec + 5 * (size_t)i;
    r[0] = make_float4(a.x, a.y, a.z, 0.0f);
    r[1] = make_float4(d.x, d.y, d.z, 0.0f);
    r[2] = make_float4(a.w, b.x, b.y, 0.0f);
    r[3] = make_float4(b.z, b.w, c.x, 0.0f);
    r[4] = make_float4(c.y, c.z, c.w, 0.0f);
}

__global__ void k_count_nonfinite(Particles P, int n, unsigned long long* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned bad = 0;
    if (i < n) {
        const float4 q[4] = {P.p0[i], P.p1[i], P.p2[i], P.p3[i]};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            bad |= !isfinite(q[j].x) | !isfinite(q[j].y) | !isfinite(q[j].z) |
                   !isfinite(q[j].w);
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(out, (unsigned long long)__popc(m));
}

__global__ void k_convert_probe(const float* __restrict__ in, int n, float fm,
                                int* __restrict__ enc_out, float* __restrict__ dec_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    enc_out[i] = enc(in[i], fm);
    dec_out[i] = dec(__float_as_int(in[i]), fm);
}

// Packed (a[2i], a[2i+1]) op (b[2i], b[2i+1]) for op = mul, add and the
// pattern the kernels use for sums of products (packed multiply, scalar
// adds: a*b + a), each next to the scalar operations.
__global__ void k_packed_probe(const float* __restrict__ a, const float* __restrict__ b, int npairs,
                               float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npairs) return;
    const size_t n = 2 * (size_t)npairs;
    const f2 x = pk(a[2 * i], a[2 * i + 1]), y = pk(b[2 * i], b[2 * i + 1]);
    upk(mul2(x, y), out[2 * i], out[2 * i + 1]);
    upk(add2(x, y), out[n + 2 * i], out[n + 2 * i + 1]);
    {   // the kernels' pattern: packed product, scalar adds
        float p0, p1;
        upk(mul2(x, y), p0, p1);
        out[2 * n + 2 * i] = fadd(p0, a[2 * i]);
        out[2 * n + 2 * i + 1] = fadd(p1, a[2 * i + 1]);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float p = a[2 * i + h], q = b[2 * i + h];
        out[3 * n + 2 * i + h] = fmul(p, q);
        out[4 * n + 2 * i + h] = fadd(p, q);
        out[5 * n + 2 * i + h] = fadd(fmul(p, q), p);
    }
}

}  // namespace

void launch_packed_probe(const float* a, const float* b, int npairs, float* out6) {
    if (npairs <= 0) return;
    k_packed_probe<<<blocks_for(npairs), kThreads>>>(a, b, npairs, out6);
}

void launch_clear_grid(int4* cells, int grid_count, cudaStream_t st) {
    if (grid_count <= 0) return;
    k_clear_grid<<<blocks_for(grid_count), kThreads, 0, st>>>(cells, grid_count);
}

void launch_p2g_1(const Particles& P, int4* cells, const SimConsts& k, unsigned long long* oob,
                  cudaStream_t st) {
    if (k.n <= 0) return;
    k_p2g_1<<<blocks_for(k.n), kThreads, 0, st>>>(P, cells, k, oob);
}

void launch_p2g_2(const Particles& P, int4* cells, const SimConsts& k, unsigned long long* oob,
                  cudaStream_t st) {
    if (k.n <= 0) return;
    k_p2g_2<<<blocks_for(k.n), kThreads, 0, st>>>(P, cells, k, oob);
}

void launch_update_grid(int4* cells, const SimConsts& k, cudaStream_t st) {
    if (k.grid_count <= 0) return;
    k_update_grid<<<blocks_for(k.grid_count), kThreads, 0, st>>>(cells, k);
}

void launch_g2p(const Particles& P, const int4* cells, const SimConsts& k,
                unsigned long long* oob, cudaStream_t st) {
    if (k.n <= 0) return;
    k_g2p<<<blocks_for(k.n), kThreads, 0, st>>>(P, cells, k, oob);
}

void launch_copy_position(const Particles& P, float4* posvel, int n, cudaStream_t st) {
    if (n <= 0) return;
    k_copy_position<<<blocks_for(n), kThreads, 0, st>>>(P, posvel, n);
}

void launch_canonicalize(const Particles& src, const uint32_t* id, const Particles& dst,
                         uint32_t* id_dst, int n, cudaStream_t st) {
    if (n <= 0) return;
    k_canonicalize<<<blocks_for(n), kThreads, 0, st>>>(src, id, dst, id_dst, n);
}

void launch_iota(uint32_t* id, int n, cudaStream_t st) {
    if (n <= 0) return;
    k_iota<<<blocks_for(n), kThreads, 0, st>>>(id, n);
}

void launch_records_to_streams(const float* rec, const Particles& P, int n, cudaStream_t st) {
    if (n <= 0) return;
    k_records_to_streams<<<blocks_for(n), kThreads, 0, st>>>(reinterpret_cast<const float4*>(rec), P, n);
}

void launch_streams_to_records(const Particles& P, float* rec, int n, cudaStream_t st) {
    if (n <= 0) return;
    k_streams_to_records<<<blocks_for(n), kThreads, 0, st>>>(P, reinterpret_cast<float4*>(rec), n);
}

void launch_count_nonfinite(const Particles& P, int n, unsigned long long* out, cudaStream_t st) {
    if (n <= 0) return;
    k_count_nonfinite<<<blocks_for(n), kThreads, 0, st>>>(P, n, out);
}

void launch_convert_probe(const float* in, int n, float fm, int* enc_out, float* dec_out,
                          cudaStream_t st) {
    if (n <= 0) return;
    k_convert_probe<<<blocks_for(n), kThreads, 0, st>>>(in, n, fm, enc_out, dec_out);
}

}  // namespace mpm
