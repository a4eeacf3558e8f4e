// mpm_math.cuh -- exact f32 / i32 arithmetic shared by every MLS-MPM kernel.
//
// Every float operation goes through an explicitly rounded intrinsic
// (__fadd_rn, __fmul_rn, ...), so no pair of operations can be contracted
// into an FMA whatever the compiler flags; the library is also built with
// -fmad=false.  The rules restate the WGSL semantics of the reference's
// kernels (mls-mpm/p2g_1.wgsl, p2g_2.wgsl, updateGrid.wgsl, g2p.wgsl):
//   enc(f) = i32(f * FM)      p2g_1.wgsl:15-17  (round toward zero, saturating,
//                                                NaN -> 0: cvt.rzi.s32.f32)
//   dec(i) = f32(i) / FM      p2g_2.wgsl:22-24  (round-to-nearest conversion,
//                                                IEEE division)
//   weights                   p2g_1.wgsl:30-34
//   flat cell index           p2g_1.wgsl:53-56  (i32, wrapping)
//   mat3x3f * vec3f           (c0*v.x + c1*v.y) + c2*v.z, C stored by columns
//   pow(x, 5.)                ((x*x)*(x*x))*x
//   max / min                 WGSL: NaN operand -> the other operand
#pragma once
#include <cstdint>

namespace mpm {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// WGSL i32(f32).
__device__ __forceinline__ int f2i_sat(float x) { return __float2int_rz(x); }

__device__ __forceinline__ int enc(float f, float fm) { return f2i_sat(fmul(f, fm)); }

__device__ __forceinline__ float dec(int i, float fm) { return fdiv(__int2float_rn(i), fm); }

__device__ __forceinline__ float wmax(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (a < b) ? b : a;
}
__device__ __forceinline__ float wmin(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b < a) ? b : a;
}

__device__ __forceinline__ float pow5(float x) {
    float x2 = fmul(x, x);
    float x4 = fmul(x2, x2);
    return fmul(x4, x);
}

// Quadratic B-spline weights along one axis.  ci = floor(p); w[g] is the
// weight of cell ci + g - 1.
__device__ __forceinline__ void bspline(float p, float& ci, float w[3]) {
    ci = floorf(p);
    float d = fsub(p, fadd(ci, 0.5f));
    float a = fsub(0.5f, d);
    float b = fadd(0.5f, d);
    w[0] = fmul(fmul(0.5f, a), a);
    w[1] = fsub(0.75f, fmul(d, d));
    w[2] = fmul(fmul(0.5f, b), b);
}

// i32(cx)*Y*Z + i32(cy)*Z + i32(cz) with two's-complement wraparound.
__device__ __forceinline__ int flat_index(float cx, float cy, float cz, int Y, int Z) {
    unsigned a = (unsigned)f2i_sat(cx) * (unsigned)Y * (unsigned)Z;
    unsigned b = (unsigned)f2i_sat(cy) * (unsigned)Z;
    return (int)(a + b + (unsigned)f2i_sat(cz));
}

// Scene-wide constants (pipeline override constants, mls-mpm.ts:53-59, and
// the box uniforms, mls-mpm.ts:131-142).
struct SimConsts {
    float stiffness;
    float rest_density;
    float dynamic_viscosity;
    float dt;
    float fm;              // fixed_point_multiplier
    float init_box[3];
    float real_box[3];
    int Y, Z;              // i32(init_box.y), i32(init_box.z)
    int grid_count;
    int n;
    // Body force per unit time added in updateGrid.  The reference adds
    // -0.3*dt to vy only (updateGrid.wgsl:34); components that are 0 are not
    // touched, so (0, -0.3, 0) reproduces it exactly.
    float gravity[3];
};

// Particle state in HBM: four float4 streams (SoA, 64 B per particle).
//   P0 = (x, y, z, C00)   P1 = (C01, C02, C10, C11)
//   P2 = (C12, C20, C21, C22)   P3 = (vx, vy, vz, 0)
// C[c][r] is row r of column c (WGSL mat3x3f columns).
struct Particles {
    float4* p0;
    float4* p1;
    float4* p2;
    float4* p3;
};

struct PState {
    float x[3];
    float v[3];
    float C[3][3];
};

__device__ __forceinline__ void unpack_xC(float4 a, float4 b, float4 c, PState& s) {
    s.x[0] = a.x; s.x[1] = a.y; s.x[2] = a.z;
    s.C[0][0] = a.w; s.C[0][1] = b.x; s.C[0][2] = b.y;
    s.C[1][0] = b.z; s.C[1][1] = b.w; s.C[1][2] = c.x;
    s.C[2][0] = c.y; s.C[2][1] = c.z; s.C[2][2] = c.w;
}

__device__ __forceinline__ void load_particle(const Particles& P, int i, PState& s) {
    float4 a = P.p0[i], b = P.p1[i], c = P.p2[i], d = P.p3[i];
    unpack_xC(a, b, c, s);
    s.v[0] = d.x; s.v[1] = d.y; s.v[2] = d.z;
}

__device__ __forceinline__ void store_particle(const Particles& P, int i, const PState& s) {
    P.p0[i] = make_float4(s.x[0], s.x[1], s.x[2], s.C[0][0]);
    P.p1[i] = make_float4(s.C[0][1], s.C[0][2], s.C[1][0], s.C[1][1]);
    P.p2[i] = make_float4(s.C[1][2], s.C[2][0], s.C[2][1], s.C[2][2]);
    P.p3[i] = make_float4(s.v[0], s.v[1], s.v[2], 0.0f);
}

// ---------------------------------------------------------------------------
// Per-particle stages.  Each is the body of one WGSL entry point, written as a
// loop over the 27 stencil cells that hands each cell's contribution to a
// caller-supplied sink (global atomics, shared-memory arena, ...) or reads
// each cell from a caller-supplied source.  All engines share these bodies,
// so the arithmetic of every engine is the same instruction sequence.
// ---------------------------------------------------------------------------

// p2g_1.wgsl:24-65.  sink(idx, cx, cy, cz, mass, vx, vy, vz) with i32 values.
template <class Sink>
__device__ __forceinline__ void p2g1_particle(const PState& s, const SimConsts& k, Sink&& sink) {
    float ci[3], w[3][3];
    float wx[3], wy[3], wz[3];
    bspline(s.x[0], ci[0], wx);
    bspline(s.x[1], ci[1], wy);
    bspline(s.x[2], ci[2], wz);
    (void)w;
#pragma unroll
    for (int gx = 0; gx < 3; ++gx) {
        const float cx = fsub(fadd(ci[0], (float)gx), 1.0f);
        const float dx = fsub(fadd(cx, 0.5f), s.x[0]);
#pragma unroll
        for (int gy = 0; gy < 3; ++gy) {
            const float cy = fsub(fadd(ci[1], (float)gy), 1.0f);
            const float dy = fsub(fadd(cy, 0.5f), s.x[1]);
            const float wxy = fmul(wx[gx], wy[gy]);
            float qxy[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) qxy[r] = fadd(fmul(s.C[0][r], dx), fmul(s.C[1][r], dy));
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const float cz = fsub(fadd(ci[2], (float)gz), 1.0f);
                const float dz = fsub(fadd(cz, 0.5f), s.x[2]);
                const float weight = fmul(wxy, wz[gz]);
                const float mass = fmul(weight, 1.0f);
                float vel[3];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const float q = fadd(qxy[r], fmul(s.C[2][r], dz));
                    vel[r] = fmul(mass, fadd(s.v[r], q));
                }
                const int idx = flat_index(cx, cy, cz, k.Y, k.Z);
                sink(idx, gx, gy, gz, enc(mass, k.fm), enc(vel[0], k.fm), enc(vel[1], k.fm),
                     enc(vel[2], k.fm));
            }
        }
    }
}

// p2g_2.wgsl:30-94.  mass_src(idx, gx, gy, gz) -> f32 decoded mass of that
// cell (dec(cells[idx].mass)); sink(idx, gx, gy, gz, mx, my, mz).
template <class MassSrc, class Sink>
__device__ __forceinline__ void p2g2_particle(const PState& s, const SimConsts& k, MassSrc&& mass_src,
                                              Sink&& sink) {
    float ci[3], wx[3], wy[3], wz[3];
    bspline(s.x[0], ci[0], wx);
    bspline(s.x[1], ci[1], wy);
    bspline(s.x[2], ci[2], wz);

    float density = 0.0f;
#pragma unroll
    for (int gx = 0; gx < 3; ++gx) {
        const float cx = fsub(fadd(ci[0], (float)gx), 1.0f);
#pragma unroll
        for (int gy = 0; gy < 3; ++gy) {
            const float cy = fsub(fadd(ci[1], (float)gy), 1.0f);
            const float wxy = fmul(wx[gx], wy[gy]);
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const float cz = fsub(fadd(ci[2], (float)gz), 1.0f);
                const float weight = fmul(wxy, wz[gz]);
                const int idx = flat_index(cx, cy, cz, k.Y, k.Z);
                density = fadd(density, fmul(mass_src(idx, gx, gy, gz), weight));
            }
        }
    }

    const float volume = fdiv(1.0f, density);
    const float pr = fmul(k.stiffness, fsub(pow5(fdiv(density, k.rest_density)), 1.0f));
    const float pressure = wmax(-0.0f, pr);
    const float s0 = fmul(-volume, 4.0f);
    float T[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const float base = (c == r) ? -pressure : 0.0f;
            const float strain = fadd(s.C[c][r], s.C[r][c]);
            const float stress = fadd(base, fmul(k.dynamic_viscosity, strain));
            T[c][r] = fmul(fmul(s0, stress), k.dt);
        }

#pragma unroll
    for (int gx = 0; gx < 3; ++gx) {
        const float cx = fsub(fadd(ci[0], (float)gx), 1.0f);
        const float dx = fsub(fadd(cx, 0.5f), s.x[0]);
#pragma unroll
        for (int gy = 0; gy < 3; ++gy) {
            const float cy = fsub(fadd(ci[1], (float)gy), 1.0f);
            const float dy = fsub(fadd(cy, 0.5f), s.x[1]);
            const float wxy = fmul(wx[gx], wy[gy]);
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const float cz = fsub(fadd(ci[2], (float)gz), 1.0f);
                const float dz = fsub(fadd(cz, 0.5f), s.x[2]);
                const float weight = fmul(wxy, wz[gz]);
                float mom[3];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const float m0 = fmul(T[0][r], weight);
                    const float m1 = fmul(T[1][r], weight);
                    const float m2 = fmul(T[2][r], weight);
                    mom[r] = fadd(fadd(fmul(m0, dx), fmul(m1, dy)), fmul(m2, dz));
                }
                const int idx = flat_index(cx, cy, cz, k.Y, k.Z);
                sink(idx, gx, gy, gz, enc(mom[0], k.fm), enc(mom[1], k.fm), enc(mom[2], k.fm));
            }
        }
    }
}

// g2p.wgsl:26-92.  vel_src(idx, gx, gy, gz, float out[3]) -> decoded cell
// velocity (dec(vx), dec(vy), dec(vz)).  Updates s in place (x, v, C).
template <class VelSrc>
__device__ __forceinline__ void g2p_particle(PState& s, const SimConsts& k, VelSrc&& vel_src) {
    float ci[3], wx[3], wy[3], wz[3];
    bspline(s.x[0], ci[0], wx);
    bspline(s.x[1], ci[1], wy);
    bspline(s.x[2], ci[2], wz);
    float v[3] = {0.0f, 0.0f, 0.0f};
    float B[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
#pragma unroll
    for (int gx = 0; gx < 3; ++gx) {
        const float cx = fsub(fadd(ci[0], (float)gx), 1.0f);
        const float dx = fsub(fadd(cx, 0.5f), s.x[0]);
#pragma unroll
        for (int gy = 0; gy < 3; ++gy) {
            const float cy = fsub(fadd(ci[1], (float)gy), 1.0f);
            const float dy = fsub(fadd(cy, 0.5f), s.x[1]);
            const float wxy = fmul(wx[gx], wy[gy]);
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const float cz = fsub(fadd(ci[2], (float)gz), 1.0f);
                const float dz = fsub(fadd(cz, 0.5f), s.x[2]);
                const float weight = fmul(wxy, wz[gz]);
                const int idx = flat_index(cx, cy, cz, k.Y, k.Z);
                float gv[3];
                vel_src(idx, gx, gy, gz, gv);
                float wv[3];
#pragma unroll
                for (int r = 0; r < 3; ++r) wv[r] = fmul(gv[r], weight);
                const float d[3] = {dx, dy, dz};
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int r = 0; r < 3; ++r) B[c][r] = fadd(B[c][r], fmul(wv[r], d[c]));
#pragma unroll
                for (int r = 0; r < 3; ++r) v[r] = fadd(v[r], wv[r]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) s.C[c][r] = fmul(B[c][r], 4.0f);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float p = fadd(s.x[a], fmul(v[a], k.dt));
        s.x[a] = wmin(wmax(p, 1.0f), fsub(k.real_box[a], 2.0f));
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float xn = fadd(s.x[a], fmul(fmul(v[a], k.dt), 3.0f));
        const float wall_max = fsub(k.real_box[a], 4.0f);
        if (xn < 3.0f) v[a] = fadd(v[a], fmul(0.3f, fsub(3.0f, xn)));
        if (xn > wall_max) v[a] = fadd(v[a], fmul(0.3f, fsub(wall_max, xn)));
    }
    s.v[0] = v[0]; s.v[1] = v[1]; s.v[2] = v[2];
}

// updateGrid.wgsl:26-44 for one cell whose coordinates (x, y, z) are already
// known; returns the new (vx, vy, vz, mass).
__device__ __forceinline__ int4 update_cell_xyz(int4 c, int x, int y, int z, const SimConsts& k,
                                                int hx, int hy, int hz) {
    if (!(c.w > 0)) return c;
    const float m = dec(c.w, k.fm);
    const float fv0 = fdiv(dec(c.x, k.fm), m);
    const float fv1 = fdiv(dec(c.y, k.fm), m);
    const float fv2 = fdiv(dec(c.z, k.fm), m);
    int o0 = enc(k.gravity[0] != 0.0f ? fadd(fv0, fmul(k.gravity[0], k.dt)) : fv0, k.fm);
    int o1 = enc(k.gravity[1] != 0.0f ? fadd(fv1, fmul(k.gravity[1], k.dt)) : fv1, k.fm);
    int o2 = enc(k.gravity[2] != 0.0f ? fadd(fv2, fmul(k.gravity[2], k.dt)) : fv2, k.fm);
    if (x < 2 || x > hx) o0 = 0;
    if (y < 2 || y > hy) o1 = 0;
    if (z < 2 || z > hz) o2 = 0;
    return make_int4(o0, o1, o2, c.w);
}

// updateGrid.wgsl:23-46 for the cell with flat index `id`: coordinates come
// from the flat index with the truncated init box (updateGrid.wgsl:37-39).
__device__ __forceinline__ int4 update_cell(int4 c, int id, const SimConsts& k, int hx, int hy,
                                            int hz) {
    if (!(c.w > 0)) return c;
    const int x = (id / k.Z) / k.Y;
    const int y = (id / k.Z) % k.Y;
    const int z = id % k.Z;
    return update_cell_xyz(c, x, y, z, k, hx, hy, hz);
}

// i32(ceil(real_box_size.a) - 3), updateGrid.wgsl:41-43.
__device__ __forceinline__ int wall_hi(float real) { return f2i_sat(fsub(ceilf(real), 3.0f)); }

}  // namespace mpm
