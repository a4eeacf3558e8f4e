// mpm_math_x2.cuh -- the per-particle stage bodies of mpm_math.cuh written
// with Blackwell's packed f32x2 multiply (mul.rn.f32x2).
//
// A packed multiply rounds each of its two lanes exactly like a scalar
// mul.rn.f32, so computing two *independent* products in one instruction
// (two components of one vector, two entries of one matrix) gives exactly
// the scalar results.  Sums stay scalar: ptxas contracts a packed multiply
// whose only use is a packed add (add.rn.f32x2) into a packed FMA, even with
// --fmad=false, which would round once instead of twice.  A packed product
// is therefore only ever consumed by scalar adds (explicit .rn, never
// contracted), by further multiplies, or by conversions.  No sum is split
// or reassociated: every accumulator keeps the reference's order (gx, gy,
// gz loops, left to right), so these bodies are bit-identical to
// p2g1_particle, p2g2_particle and g2p_particle in mpm_math.cuh, which the
// tests check.
#pragma once
#include "mpm_math.cuh"

namespace mpm {

struct f2 {
    unsigned long long v;
};

__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(f2 x, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
}
__device__ __forceinline__ float lo(f2 x) {
    float a, b;
    upk(x, a, b);
    return a;
}
__device__ __forceinline__ float hi(f2 x) {
    float a, b;
    upk(x, a, b);
    return b;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
// Only for operands that are not packed products (see the file comment).
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 dup(float a) { return pk(a, a); }

// p2g_1.wgsl:24-65.  sink(gx, gy, gz, m, vx, vy, vz) with i32 values.
template <class Sink>
__device__ __forceinline__ void p2g1_particle_x2(const PState& s, const SimConsts& k, Sink&& sink) {
    float ci[3], wx[3], wy[3], wz[3];
    bspline(s.x[0], ci[0], wx);
    bspline(s.x[1], ci[1], wy);
    bspline(s.x[2], ci[2], wz);
    const f2 fm2 = dup(k.fm);
    const f2 C0_01 = pk(s.C[0][0], s.C[0][1]), C1_01 = pk(s.C[1][0], s.C[1][1]);
    const f2 C2_01 = pk(s.C[2][0], s.C[2][1]), C01_2 = pk(s.C[0][2], s.C[1][2]);
    // C[2][r] * dz per gz (third column of C * cell_dist)
    float c2dz[3][3];
    f2 wz2[3];
#pragma unroll
    for (int gz = 0; gz < 3; ++gz) {
        const float cz = fsub(fadd(ci[2], (float)gz), 1.0f);
        const float dz = fsub(fadd(cz, 0.5f), s.x[2]);
        upk(mul2(C2_01, dup(dz)), c2dz[gz][0], c2dz[gz][1]);
        c2dz[gz][2] = fmul(s.C[2][2], dz);
        wz2[gz] = dup(wz[gz]);
    }
#pragma unroll
    for (int gx = 0; gx < 3; ++gx) {
        const float cx = fsub(fadd(ci[0], (float)gx), 1.0f);
        const float dx = fsub(fadd(cx, 0.5f), s.x[0]);
#pragma unroll
        for (int gy = 0; gy < 3; ++gy) {
            const float cy = fsub(fadd(ci[1], (float)gy), 1.0f);
            const float dy = fsub(fadd(cy, 0.5f), s.x[1]);
            const f2 wxy2 = dup(fmul(wx[gx], wy[gy]));
            // (C0*dx + C1*dy) per row
            float a0, a1, b0, b1, e0, e1;
            upk(mul2(C0_01, dup(dx)), a0, a1);
            upk(mul2(C1_01, dup(dy)), b0, b1);
            upk(mul2(C01_2, pk(dx, dy)), e0, e1);
            const float qxy[3] = {fadd(a0, b0), fadd(a1, b1), fadd(e0, e1)};
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const f2 w2 = mul2(wxy2, wz2[gz]);                 // (weight, weight)
                float vq[3];
#pragma unroll
                for (int r = 0; r < 3; ++r) vq[r] = fadd(s.v[r], fadd(qxy[r], c2dz[gz][r]));
                const f2 vel01 = mul2(w2, pk(vq[0], vq[1]));       // mass * (v + Q), x y
                const f2 vel2m = mul2(w2, pk(vq[2], 1.0f));        // (mass * (v.z + Q.z), weight)
                const f2 e01 = mul2(vel01, fm2);
                const f2 e2m = mul2(vel2m, fm2);
                sink(gx, gy, gz, f2i_sat(hi(e2m)), f2i_sat(lo(e01)), f2i_sat(hi(e01)),
                     f2i_sat(lo(e2m)));
            }
        }
    }
}

// p2g_2.wgsl:30-94.  mass_src(gx, gy, gz) -> decoded cell mass;
// sink(gx, gy, gz, mx, my, mz).
template <class MassSrc, class Sink>
__device__ __forceinline__ void p2g2_particle_x2(const PState& s, const SimConsts& k,
                                                 MassSrc&& mass_src, Sink&& sink) {
    float ci[3], wx[3], wy[3], wz[3];
    bspline(s.x[0], ci[0], wx);
    bspline(s.x[1], ci[1], wy);
    bspline(s.x[2], ci[2], wz);

    float density = 0.0f;
#pragma unroll
    for (int gx = 0; gx < 3; ++gx)
#pragma unroll
        for (int gy = 0; gy < 3; ++gy) {
            const float wxy = fmul(wx[gx], wy[gy]);
#pragma unroll
            for (int gz = 0; gz < 3; ++gz)
                density = fadd(density, fmul(mass_src(gx, gy, gz), fmul(wxy, wz[gz])));
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
    const f2 T0_01 = pk(T[0][0], T[0][1]), T1_01 = pk(T[1][0], T[1][1]), T2_01 = pk(T[2][0], T[2][1]);
    const f2 T01_2 = pk(T[0][2], T[1][2]);
    const f2 fm2 = dup(k.fm);
    f2 wz2[3], dz2[3];
#pragma unroll
    for (int gz = 0; gz < 3; ++gz) {
        const float cz = fsub(fadd(ci[2], (float)gz), 1.0f);
        dz2[gz] = dup(fsub(fadd(cz, 0.5f), s.x[2]));
        wz2[gz] = dup(wz[gz]);
    }
#pragma unroll
    for (int gx = 0; gx < 3; ++gx) {
        const float cx = fsub(fadd(ci[0], (float)gx), 1.0f);
        const float dx = fsub(fadd(cx, 0.5f), s.x[0]);
        const f2 dx2 = dup(dx);
#pragma unroll
        for (int gy = 0; gy < 3; ++gy) {
            const float cy = fsub(fadd(ci[1], (float)gy), 1.0f);
            const float dy = fsub(fadd(cy, 0.5f), s.x[1]);
            const f2 dy2 = dup(dy);
            const f2 dxy = pk(dx, dy);
            const f2 wxy2 = dup(fmul(wx[gx], wy[gy]));
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const f2 w2 = mul2(wxy2, wz2[gz]);                 // (weight, weight)
                // M = T * weight; momentum = (M0*dx + M1*dy) + M2*dz per row
                float a0, a1, b0, b1, c0, c1, e0, e1;
                upk(mul2(mul2(T0_01, w2), dx2), a0, a1);
                upk(mul2(mul2(T1_01, w2), dy2), b0, b1);
                upk(mul2(mul2(T2_01, w2), dz2[gz]), c0, c1);
                upk(mul2(mul2(T01_2, w2), dxy), e0, e1);          // (M02*dx, M12*dy)
                const float m22dz = fmul(fmul(T[2][2], lo(w2)), lo(dz2[gz]));
                const float mom0 = fadd(fadd(a0, b0), c0);
                const float mom1 = fadd(fadd(a1, b1), c1);
                const float mom2 = fadd(fadd(e0, e1), m22dz);
                const f2 e01 = mul2(pk(mom0, mom1), fm2);
                sink(gx, gy, gz, f2i_sat(lo(e01)), f2i_sat(hi(e01)), f2i_sat(fmul(mom2, k.fm)));
            }
        }
    }
}

// g2p.wgsl:26-92.  vel_src(gx, gy, gz, f2& vxy, f2& vzz) -> decoded cell
// velocity as (vx, vy) and (vz, vz).  Updates s in place (x, v, C).
template <class VelSrc>
__device__ __forceinline__ void g2p_particle_x2(PState& s, const SimConsts& k, VelSrc&& vel_src) {
    float ci[3], wx[3], wy[3], wz[3];
    bspline(s.x[0], ci[0], wx);
    bspline(s.x[1], ci[1], wy);
    bspline(s.x[2], ci[2], wz);
    float v[3] = {0.0f, 0.0f, 0.0f};
    float B[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
    f2 wz2[3], dz2[3];
#pragma unroll
    for (int gz = 0; gz < 3; ++gz) {
        const float cz = fsub(fadd(ci[2], (float)gz), 1.0f);
        dz2[gz] = dup(fsub(fadd(cz, 0.5f), s.x[2]));
        wz2[gz] = dup(wz[gz]);
    }
#pragma unroll
    for (int gx = 0; gx < 3; ++gx) {
        const float cx = fsub(fadd(ci[0], (float)gx), 1.0f);
        const float dx = fsub(fadd(cx, 0.5f), s.x[0]);
        const f2 dx2 = dup(dx);
#pragma unroll
        for (int gy = 0; gy < 3; ++gy) {
            const float cy = fsub(fadd(ci[1], (float)gy), 1.0f);
            const float dy = fsub(fadd(cy, 0.5f), s.x[1]);
            const f2 dy2 = dup(dy);
            const f2 dxy = pk(dx, dy);
            const f2 wxy2 = dup(fmul(wx[gx], wy[gy]));
#pragma unroll
            for (int gz = 0; gz < 3; ++gz) {
                const f2 w2 = mul2(wxy2, wz2[gz]);                 // (weight, weight)
                f2 gxy, gzz;
                vel_src(gx, gy, gz, gxy, gzz);
                const f2 wv01 = mul2(gxy, w2);                     // weighted_velocity x, y
                const f2 wv22 = mul2(gzz, w2);                     // (wv.z, wv.z)
                // B += [wv*d.x | wv*d.y | wv*d.z]
                float p[8];
                upk(mul2(wv01, dx2), p[0], p[1]);
                upk(mul2(wv01, dy2), p[2], p[3]);
                upk(mul2(wv01, dz2[gz]), p[4], p[5]);
                upk(mul2(wv22, dxy), p[6], p[7]);
                B[0][0] = fadd(B[0][0], p[0]);
                B[0][1] = fadd(B[0][1], p[1]);
                B[0][2] = fadd(B[0][2], p[6]);
                B[1][0] = fadd(B[1][0], p[2]);
                B[1][1] = fadd(B[1][1], p[3]);
                B[1][2] = fadd(B[1][2], p[7]);
                B[2][0] = fadd(B[2][0], p[4]);
                B[2][1] = fadd(B[2][1], p[5]);
                B[2][2] = fadd(B[2][2], fmul(lo(wv22), lo(dz2[gz])));
                v[0] = fadd(v[0], lo(wv01));
                v[1] = fadd(v[1], hi(wv01));
                v[2] = fadd(v[2], lo(wv22));
            }
        }
    }
    const f2 four = dup(4.0f);
#pragma unroll
    for (int c = 0; c < 3; ++c) upk(mul2(pk(B[c][0], B[c][1]), four), s.C[c][0], s.C[c][1]);
    upk(mul2(pk(B[0][2], B[1][2]), four), s.C[0][2], s.C[1][2]);
    s.C[2][2] = fmul(B[2][2], 4.0f);
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

}  // namespace mpm
