// render_math.cuh -- f32 arithmetic of the headless screen-space renderer
// (render/*.wgsl), with every operation explicitly rounded so the result is
// a fixed function of the inputs.
//
// WGSL leaves exp/log/pow accuracy to the implementation (a few ULP), so any
// accurate restatement is a valid one; the renderer uses its own:
//   exp(x)   Cody-Waite range reduction x = k*ln2 + r (ln2 split into a
//            high part with trailing zero bits and a low correction),
//            exp(r) by its Taylor series to degree 8 (|r| <= ln2/2, error
//            below 1e-8 relative), then scaling by 2^k in two exact steps;
//   log2(x)  x = m * 2^e with m in [sqrt(1/2), sqrt(2)), log(m) from the
//            series 2*atanh(s) = 2*(s + s^3/3 + ... + s^11/11),
//            s = (m-1)/(m+1), |s| <= 0.172;
//   pow(x,y) exp(y * log2(x) * ln2), 0 for x == 0 and y > 0, NaN for x < 0.
// Vectors and 4x4 matrices follow WGSL (mat4x4f stored by columns;
// M * v = ((c0*v.x + c1*v.y) + c2*v.z) + c3*v.w).
#pragma once

#include <cstdint>

namespace mpm {
namespace rmath {

__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float dvd(float a, float b) { return __fdiv_rn(a, b); }

// 2^k for k in [-126, 127], exactly.
__device__ __forceinline__ float pow2i(int k) { return __int_as_float((k + 127) << 23); }

__device__ __forceinline__ float exp_r(float x) {
    if (x != x) return x;
    if (x > 88.8f) return __int_as_float(0x7f800000);
    if (x < -104.0f) return 0.0f;
    const float kf = rintf(mul(x, 1.44269502f));  // nearest integer of x / ln2
    const int k = (int)kf;
    const float r = sub(sub(x, mul(kf, 0.693145751953125f)), mul(kf, 1.42860677e-6f));
    // Taylor series of exp(r), Horner form
    float p = 2.48015873e-5f;                 // 1/8!
    p = add(mul(p, r), 1.98412698e-4f);       // 1/7!
    p = add(mul(p, r), 1.38888889e-3f);       // 1/6!
    p = add(mul(p, r), 8.33333333e-3f);       // 1/5!
    p = add(mul(p, r), 4.16666667e-2f);       // 1/4!
    p = add(mul(p, r), 1.66666667e-1f);       // 1/3!
    p = add(mul(p, r), 0.5f);
    p = add(mul(p, r), 1.0f);
    p = add(mul(p, r), 1.0f);
    // p * 2^k in two exact power-of-two steps (k in [-150, 128])
    const int k1 = k / 2, k2 = k - k1;
    return mul(mul(p, pow2i(k1)), pow2i(k2));
}

__device__ __forceinline__ float log_r(float x) {  // natural log
    if (x != x || x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return __int_as_float(0xff800000);
    if (x == __int_as_float(0x7f800000)) return x;
    int e = 0;
    float m = x;
    if (m < 1.17549435e-38f) {  // subnormal: scale into the normal range
        m = mul(m, 16777216.0f);
        e = -24;
    }
    const uint32_t b = (uint32_t)__float_as_int(m);
    e += (int)((b >> 23) & 0xffu) - 127;
    m = __int_as_float((int)((b & 0x007fffffu) | 0x3f800000u));  // [1, 2)
    if (m > 1.41421356f) {
        m = mul(m, 0.5f);
        e += 1;
    }
    const float s = dvd(sub(m, 1.0f), add(m, 1.0f));
    const float s2 = mul(s, s);
    float q = 9.09090909e-2f;                  // 1/11
    q = add(mul(q, s2), 1.11111111e-1f);       // 1/9
    q = add(mul(q, s2), 1.42857143e-1f);       // 1/7
    q = add(mul(q, s2), 2.0e-1f);              // 1/5
    q = add(mul(q, s2), 3.33333333e-1f);       // 1/3
    q = add(mul(q, s2), 1.0f);
    const float lm = mul(mul(2.0f, s), q);
    return add(mul((float)e, 0.693147181f), lm);
}

__device__ __forceinline__ float pow_r(float x, float y) {
    if (x == 0.0f && y > 0.0f) return 0.0f;
    return exp_r(mul(y, log_r(x)));
}

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return v3(add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)); }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return v3(sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)); }
__device__ __forceinline__ V3 vscale(V3 a, float s) { return v3(mul(a.x, s), mul(a.y, s), mul(a.z, s)); }
__device__ __forceinline__ float vdot(V3 a, V3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
__device__ __forceinline__ V3 vcross(V3 a, V3 b) {
    return v3(sub(mul(a.y, b.z), mul(a.z, b.y)), sub(mul(a.z, b.x), mul(a.x, b.z)),
              sub(mul(a.x, b.y), mul(a.y, b.x)));
}
__device__ __forceinline__ V3 vnormalize(V3 a) {
    const float l = __fsqrt_rn(vdot(a, a));
    return v3(dvd(a.x, l), dvd(a.y, l), dvd(a.z, l));
}

// 4x4 matrix (columns) times (x, y, z, w): ((c0*x + c1*y) + c2*z) + c3*w.
__device__ __forceinline__ float4 mat4_mul(const float* m, float x, float y, float z, float w) {
    float4 r;
    r.x = add(add(add(mul(m[0], x), mul(m[4], y)), mul(m[8], z)), mul(m[12], w));
    r.y = add(add(add(mul(m[1], x), mul(m[5], y)), mul(m[9], z)), mul(m[13], w));
    r.z = add(add(add(mul(m[2], x), mul(m[6], y)), mul(m[10], z)), mul(m[14], w));
    r.w = add(add(add(mul(m[3], x), mul(m[7], y)), mul(m[11], z)), mul(m[15], w));
    return r;
}

}  // namespace rmath
}  // namespace mpm
