// render.cu -- headless restatement of WebGPU-Ocean's screen-space fluid
// renderer (render/fluidRender.ts:292-488, fluid path), reading the posvel
// records the simulator writes and producing an image in device memory.
//
// Passes (reference shader in brackets):
//   k_splat           depth and thickness splats of every particle's
//                     screen-aligned billboard [depthMap.wgsl:34-79,
//                     thicknessMap.wgsl:27-62]
//   k_resolve         depth map (view z of the nearest fragment) and the
//                     thickness map (r16float)
//   k_bilateral x 8   separable bilateral filter of the depth map, 4 x (X, Y)
//                     [bilateral.wgsl:18-75]
//   k_gaussian x 2    separable gaussian of the thickness map, (X, Y)
//                     [gaussian.wgsl:14-42]
//   k_shade           normals, lighting, fresnel, transmittance, cube-map
//                     reflection [fluid.wgsl:37-98]
// and, for the sphere mode (sphereRenderFl, fluidRender.ts:481-485):
//   k_sphere_splat    the depth test of every billboard [sphere.wgsl:37-64]
//   k_sphere_shade    the winning particle's lit sphere, coloured by speed
//                     [sphere.wgsl:67-110]
//
// Rasterisation, restated for these billboards: with a perspective matrix
// without skew all four corners of a billboard share their clip w, so the
// quad covers an axis-aligned rectangle [X0, X1) x [Y0, Y1) of the
// framebuffer (x right, y down; pixel centres at +0.5), edges by the
// top-left rule, and the uv varying is linear in screen space.  A quad whose
// plane lies outside the depth range [0, 1] is clipped.  The depth test
// ('less' against a cleared 1.0, first-drawn fragment wins ties) is an
// atomicMin on (depth bits << 32 | particle index); frag_depth is clamped to
// [0, 1].  Thickness is the sum of every fragment's 0.05*sqrt(1 - r^2)
// (additive blending, no depth test), accumulated exactly in 2^-32 fixed
// point and rounded once to r16float, instead of the reference's blend-order
// dependent r16float additions.  Texture loads clamp their coordinates to the
// texture (WGSL's vec2u() saturates negative coordinates at 0; the far edge
// follows the clamping robustness of WebGPU implementations).  Every
// r16float texture write rounds to half precision.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mpm.h"
#include "render_math.cuh"

namespace mpm {
void set_last_error(const std::string& msg);  // capi.cu
}

using namespace mpm::rmath;

namespace {

struct Uni {
    float texel[2];
    float sphere_size;
    float pad;
    float invP[16];
    float P[16];
    float V[16];
    float invV[16];
};
static_assert(sizeof(Uni) == 272, "RenderUniforms layout (common.ts:1-9)");

struct Consts {
    int W, H;
    float depth_threshold;   // radius * 10           (fluidRender.ts:38-46)
    float max_filter_size;   // 100
    float ppc;               // projected_particle_constant
};

constexpr uint32_t kOneBits = 0x3f800000u;  // 1.0f
constexpr unsigned long long kClearKey = ((unsigned long long)kOneBits << 32) | 0xffffffffull;

__device__ __forceinline__ float half_round(float x) { return __half2float(__float2half_rn(x)); }

__device__ __forceinline__ float wmax(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return a < b ? b : a;
}
__device__ __forceinline__ float wmin(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return b < a ? b : a;
}

// Screen rectangle and per-fragment quantities of particle i.
struct Billboard {
    V3 view;
    float fxm, fxp, fym, fyp;  // framebuffer x of the uv.x = 0 / 1 edges, y of uv.y = 0 / 1
    int x0, x1, y0, y1;        // covered pixel range, inclusive; empty when x0 > x1
};

__device__ __forceinline__ bool billboard(const float4* posvel, int i, const Uni& u, const Consts& c,
                                          Billboard& b) {
    const float4 p = posvel[2 * (size_t)i];
    const float4 vp = mat4_mul(u.V, p.x, p.y, p.z, 1.0f);
    b.view = v3(vp.x, vp.y, vp.z);
    const float s = u.sphere_size;
    const float4 cm = mat4_mul(u.P, add(b.view.x, mul(-0.5f, s)), add(b.view.y, mul(-0.5f, s)), b.view.z, 1.0f);
    const float4 cp = mat4_mul(u.P, add(b.view.x, mul(0.5f, s)), add(b.view.y, mul(0.5f, s)), b.view.z, 1.0f);
    const float4 cc = mat4_mul(u.P, b.view.x, b.view.y, b.view.z, 1.0f);
    if (!(cc.w > 0.0f)) return false;
    const float zq = dvd(cc.z, cc.w);
    if (!(zq >= 0.0f && zq <= 1.0f)) return false;
    const float W = (float)c.W, H = (float)c.H;
    b.fxm = mul(add(dvd(cm.x, cm.w), 1.0f), mul(0.5f, W));
    b.fxp = mul(add(dvd(cp.x, cp.w), 1.0f), mul(0.5f, W));
    b.fym = mul(sub(1.0f, dvd(cm.y, cm.w)), mul(0.5f, H));
    b.fyp = mul(sub(1.0f, dvd(cp.y, cp.w)), mul(0.5f, H));
    const float X0 = fminf(b.fxm, b.fxp), X1 = fmaxf(b.fxm, b.fxp);
    const float Y0 = fminf(b.fym, b.fyp), Y1 = fmaxf(b.fym, b.fyp);
    if (!(X1 > X0) || !(Y1 > Y0)) return false;
    // pixel centres px + 0.5 in [X0, X1), clamped to the image before the
    // conversion to int
    const float lx = ceilf(sub(X0, 0.5f)), hx = sub(ceilf(sub(X1, 0.5f)), 1.0f);
    const float ly = ceilf(sub(Y0, 0.5f)), hy = sub(ceilf(sub(Y1, 0.5f)), 1.0f);
    b.x0 = (int)fminf(fmaxf(lx, 0.0f), W);
    b.x1 = (int)fmaxf(fminf(hx, W - 1.0f), -1.0f);
    b.y0 = (int)fminf(fmaxf(ly, 0.0f), H);
    b.y1 = (int)fmaxf(fminf(hy, H - 1.0f), -1.0f);
    return b.x0 <= b.x1 && b.y0 <= b.y1;
}

// Fragment of billboard b at pixel (px, py): false when discarded (r^2 > 1).
struct Frag {
    float depth;  // clamped frag_depth
    float vz;     // colour: view z of the sphere surface
    float nz;     // sqrt(1 - r^2)
};

__device__ __forceinline__ bool fragment(const Billboard& b, int px, int py, const Uni& u, Frag& f) {
    const float cx = add((float)px, 0.5f), cy = add((float)py, 0.5f);
    const float uu = dvd(sub(cx, b.fxm), sub(b.fxp, b.fxm));
    const float vv = dvd(sub(cy, b.fym), sub(b.fyp, b.fym));
    const float nx = sub(mul(uu, 2.0f), 1.0f), ny = sub(mul(vv, 2.0f), 1.0f);
    const float r2 = add(mul(nx, nx), mul(ny, ny));
    if (r2 > 1.0f) return false;
    const float nz = __fsqrt_rn(sub(1.0f, r2));
    const float radius = dvd(u.sphere_size, 2.0f);
    const V3 rv = vadd(b.view, vscale(v3(nx, ny, nz), radius));
    const float4 clip = mat4_mul(u.P, rv.x, rv.y, rv.z, 1.0f);
    f.depth = wmin(wmax(dvd(clip.z, clip.w), 0.0f), 1.0f);
    f.vz = rv.z;
    f.nz = nz;
    return true;
}

__global__ void k_clear(unsigned long long* dkey, unsigned long long* tacc, int npix) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    dkey[p] = kClearKey;
    tacc[p] = 0ull;
}

__global__ void __launch_bounds__(128) k_splat(const float4* __restrict__ posvel, int n, Uni u, Consts c,
                                               unsigned long long* __restrict__ dkey,
                                               unsigned long long* __restrict__ tacc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Billboard b;
    if (!billboard(posvel, i, u, c, b)) return;
    for (int py = b.y0; py <= b.y1; ++py)
        for (int px = b.x0; px <= b.x1; ++px) {
            Frag f;
            if (!fragment(b, px, py, u, f)) continue;
            const size_t p = (size_t)py * c.W + px;
            if (f.depth < 1.0f)
                atomicMin(dkey + p, ((unsigned long long)__float_as_uint(f.depth) << 32) | (unsigned)i);
            const float t = mul(0.05f, f.nz);
            atomicAdd(tacc + p, (unsigned long long)__float2ll_rn(mul(t, 4294967296.0f)));
        }
}

__global__ void k_resolve(const float4* __restrict__ posvel, Uni u, Consts c,
                          const unsigned long long* __restrict__ dkey,
                          const unsigned long long* __restrict__ tacc, float* __restrict__ depth,
                          float* __restrict__ thick) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= c.W * c.H) return;
    const unsigned long long key = dkey[p];
    float d = 0.0f;  // the depth map's clear colour
    if (key != kClearKey) {
        Billboard b;
        Frag f;
        const int i = (int)(key & 0xffffffffull);
        if (billboard(posvel, i, u, c, b) && fragment(b, p % c.W, p / c.W, u, f)) d = f.vz;
    }
    depth[p] = d;
    const float t = mul(__ll2float_rn((long long)tacc[p]), 2.3283064365386963e-10f);  // 2^-32
    thick[p] = half_round(t);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Spatial weights of the two filters, which depend only on the filter
// half-width and the tap offset: bilateral exp(-(x^2 + x^2) / (2 sigma^2)),
// sigma = fs / 3, for fs in [0, kMaxFs] and |x| <= fs (row fs at fs * kWRow);
// gaussian exp(-x^2 / (2 sigma^2)), sigma = 10, |x| <= 30.  Computed once
// with the same operations the filter bodies use, so a table read is
// bit-identical to evaluating the weight in place.
constexpr int kMaxFs = 100;
constexpr int kWRow = kMaxFs + 1;
constexpr int kGaussFs = 30;

__global__ void k_weight_tables(float* __restrict__ wtab, float* __restrict__ gtab) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < kWRow * kWRow) {
        const int fs = e / kWRow, x = e % kWRow;
        const float sigma = dvd((float)fs, 3.0f);
        const float two_sigma = mul(mul(2.0f, sigma), sigma);
        const float xf = (float)x;
        const float rr = add(mul(xf, xf), mul(xf, xf));
        wtab[e] = exp_r(dvd(-rr, two_sigma));
    }
    if (e <= kGaussFs) {
        const float sigma = dvd((float)kGaussFs, 3.0f);
        const float two_sigma = mul(mul(2.0f, sigma), sigma);
        const float xf = (float)e;
        gtab[e] = exp_r(dvd(mul(-xf, xf), two_sigma));
    }
}

__global__ void k_bilateral(const float* __restrict__ src, float* __restrict__ dst, Consts c,
                            const float* __restrict__ wtab, int dx, int dy) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= c.W * c.H) return;
    const int px = p % c.W, py = p / c.W;
    const float depth = fabsf(src[p]);
    if (depth >= 1e4f || depth <= 0.0f) {
        dst[p] = depth;
        return;
    }
    const int fs = min(__float2int_rz(c.max_filter_size), __float2int_rz(ceilf(dvd(c.ppc, depth))));
    const float* wrow = wtab + fs * kWRow;  // fs <= max_filter_size = kMaxFs
    const float sd = dvd(c.depth_threshold, 3.0f);
    const float two_sd = mul(mul(2.0f, sd), sd);
    float sum = 0.0f, wsum = 0.0f;
    for (int x = -fs; x <= fs; ++x) {
        const int ix = clampi(px + x * dx, 0, c.W - 1), iy = clampi(py + x * dy, 0, c.H - 1);
        const float sampled = fabsf(src[(size_t)iy * c.W + ix]);
        const float w = __ldg(wrow + (x < 0 ? -x : x));
        const float rd = sub(sampled, depth);
        const float wd = exp_r(dvd(mul(-rd, rd), two_sd));
        sum = add(sum, mul(mul(sampled, w), wd));
        wsum = add(wsum, mul(w, wd));
    }
    dst[p] = dvd(sum, wsum);
}

__global__ void k_gaussian(const float* __restrict__ src, float* __restrict__ dst, Consts c,
                           const float* __restrict__ gtab, int dx, int dy) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= c.W * c.H) return;
    const int px = p % c.W, py = p / c.W;
    const float t = src[p];
    if (t == 0.0f) {
        dst[p] = 0.0f;
        return;
    }
    constexpr int fs = kGaussFs;
    float sum = 0.0f, wsum = 0.0f;
    for (int x = -fs; x <= fs; ++x) {
        const int ix = clampi(px + x * dx, 0, c.W - 1), iy = clampi(py + x * dy, 0, c.H - 1);
        const float sampled = src[(size_t)iy * c.W + ix];
        const float w = __ldg(gtab + (x < 0 ? -x : x));
        sum = add(sum, mul(sampled, w));
        wsum = add(wsum, w);
    }
    dst[p] = half_round(dvd(sum, wsum));
}

// fluid.wgsl:19-27: view-space position from a texture coordinate and depth.
__device__ __forceinline__ V3 view_pos(const Uni& u, float tx, float ty, float depth) {
    const float nx = sub(mul(tx, 2.0f), 1.0f);
    const float ny = sub(1.0f, mul(2.0f, ty));
    const float nz = add(-u.P[10], dvd(u.P[14], depth));
    const float4 e = mat4_mul(u.invP, nx, ny, nz, 1.0f);
    return v3(dvd(e.x, e.w), dvd(e.y, e.w), dvd(e.z, e.w));
}

// Bilinear cube-map sample (level 0), faces +x, -x, +y, -y, +z, -z of
// size x size RGBA texels; face selection and (s, t) per the usual cube-map
// table; filtering within the face, clamped to its edge.
__device__ __forceinline__ V3 sample_cube(const float4* __restrict__ env, int size, V3 d) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int face;
    float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        if (d.x >= 0.0f) { face = 0; sc = -d.z; tc = -d.y; }
        else { face = 1; sc = d.z; tc = -d.y; }
    } else if (ay >= az) {
        ma = ay;
        if (d.y >= 0.0f) { face = 2; sc = d.x; tc = d.z; }
        else { face = 3; sc = d.x; tc = -d.z; }
    } else {
        ma = az;
        if (d.z >= 0.0f) { face = 4; sc = d.x; tc = -d.y; }
        else { face = 5; sc = -d.x; tc = -d.y; }
    }
    if (!(ma > 0.0f) || ma == __int_as_float(0x7f800000)) {
        const float q = __int_as_float(0x7fc00000);
        return v3(q, q, q);
    }
    const float s = mul(0.5f, add(dvd(sc, ma), 1.0f));
    const float t = mul(0.5f, add(dvd(tc, ma), 1.0f));
    const float fu = sub(mul(s, (float)size), 0.5f), fv = sub(mul(t, (float)size), 0.5f);
    const float iu = floorf(fu), iv = floorf(fv);
    const float a = sub(fu, iu), bb = sub(fv, iv);
    const int u0 = clampi((int)iu, 0, size - 1), u1 = clampi((int)iu + 1, 0, size - 1);
    const int v0 = clampi((int)iv, 0, size - 1), v1 = clampi((int)iv + 1, 0, size - 1);
    const float4* f = env + (size_t)face * size * size;
    const float4 c00 = f[v0 * size + u0], c10 = f[v0 * size + u1];
    const float4 c01 = f[v1 * size + u0], c11 = f[v1 * size + u1];
    const float ia = sub(1.0f, a), ib = sub(1.0f, bb);
    auto lerp2 = [&](float p00, float p10, float p01, float p11) {
        const float top = add(mul(p00, ia), mul(p10, a));
        const float bot = add(mul(p01, ia), mul(p11, a));
        return add(mul(top, ib), mul(bot, bb));
    };
    return v3(lerp2(c00.x, c10.x, c01.x, c11.x), lerp2(c00.y, c10.y, c01.y, c11.y),
              lerp2(c00.z, c10.z, c01.z, c11.z));
}

__global__ void k_shade(const float* __restrict__ depth_map, const float* __restrict__ thick_map,
                        const float4* __restrict__ env, int env_size, Uni u, Consts c,
                        float4* __restrict__ out, uchar4* __restrict__ out8) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= c.W * c.H) return;
    const int px = p % c.W, py = p / c.W;
    const float tx = dvd(add((float)px, 0.5f), (float)c.W);
    const float ty = dvd(add((float)py, 0.5f), (float)c.H);
    const V3 bg = v3(0.8f, 0.8f, 0.8f);
    const float depth = fabsf(depth_map[p]);
    V3 col;
    if (depth >= 1e4f || depth <= 0.0f) {
        col = bg;
    } else {
        const V3 vp = view_pos(u, tx, ty, depth);
        auto at = [&](int qx, int qy, float sx, float sy) {
            const int ix = clampi(qx, 0, c.W - 1), iy = clampi(qy, 0, c.H - 1);
            return view_pos(u, sx, sy, fabsf(depth_map[(size_t)iy * c.W + ix]));
        };
        V3 ddx = vsub(at(px + 1, py, add(tx, u.texel[0]), ty), vp);
        V3 ddy = vsub(at(px, py + 1, tx, add(ty, u.texel[1])), vp);
        const V3 ddx2 = vsub(vp, at(px - 1, py, sub(tx, u.texel[0]), ty));
        const V3 ddy2 = vsub(vp, at(px, py - 1, tx, sub(ty, u.texel[1])));
        if (fabsf(ddx.z) > fabsf(ddx2.z)) ddx = ddx2;
        if (fabsf(ddy.z) > fabsf(ddy2.z)) ddy = ddy2;
        const V3 nn = vnormalize(vcross(ddx, ddy));
        const V3 normal = v3(-nn.x, -nn.y, -nn.z);
        const V3 ray = vnormalize(vp);
        const float4 l4 = mat4_mul(u.V, 0.0f, 0.0f, -1.0f, 0.0f);
        const V3 light = vnormalize(v3(l4.x, l4.y, l4.z));
        const V3 hv = vnormalize(vsub(light, ray));
        const float specular = pow_r(wmax(0.0f, vdot(hv, normal)), 250.0f);
        const float density = 1.5f;
        const float thickness = thick_map[p];
        const V3 dc = v3(0.085f, 0.6375f, 0.9f);
        const float a = mul(-density, thickness);
        const V3 trans = v3(exp_r(mul(a, sub(1.0f, dc.x))), exp_r(mul(a, sub(1.0f, dc.y))),
                            exp_r(mul(a, sub(1.0f, dc.z))));
        const V3 refr = v3(mul(bg.x, trans.x), mul(bg.y, trans.y), mul(bg.z, trans.z));
        const float F0 = 0.02f;
        const float cosv = vdot(normal, v3(-ray.x, -ray.y, -ray.z));
        const float fres = wmin(wmax(add(F0, mul(sub(1.0f, F0), pow_r(sub(1.0f, cosv), 5.0f))), 0.0f), 1.0f);
        const V3 refl = vsub(ray, vscale(normal, mul(2.0f, vdot(normal, ray))));
        const float4 rw = mat4_mul(u.invV, refl.x, refl.y, refl.z, 0.0f);
        const V3 env_col = sample_cube(env, env_size, v3(rw.x, rw.y, rw.z));
        const float omf = sub(1.0f, fres);
        col = v3(add(mul(1.0f, specular), add(mul(refr.x, omf), mul(env_col.x, fres))),
                 add(mul(1.0f, specular), add(mul(refr.y, omf), mul(env_col.y, fres))),
                 add(mul(1.0f, specular), add(mul(refr.z, omf), mul(env_col.z, fres))));
    }
    out[p] = make_float4(col.x, col.y, col.z, 1.0f);
    auto u8 = [](float v) -> unsigned char {
        if (v != v) return 0;
        return (unsigned char)rintf(mul(wmin(wmax(v, 0.0f), 1.0f), 255.0f));
    };
    out8[p] = make_uchar4(u8(col.x), u8(col.y), u8(col.z), 255);
}

// Sphere mode (render/sphere.wgsl, fluidRender.ts:481-485): the depth test
// alone, then each pixel shaded from the winning particle.
__global__ void __launch_bounds__(128) k_sphere_splat(const float4* __restrict__ posvel, int n,
                                                      Uni u, Consts c,
                                                      unsigned long long* __restrict__ dkey) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Billboard b;
    if (!billboard(posvel, i, u, c, b)) return;
    for (int py = b.y0; py <= b.y1; ++py)
        for (int px = b.x0; px <= b.x1; ++px) {
            Frag f;
            if (!fragment(b, px, py, u, f)) continue;
            if (f.depth < 1.0f)
                atomicMin(dkey + (size_t)py * c.W + px,
                          ((unsigned long long)__float_as_uint(f.depth) << 32) | (unsigned)i);
        }
}

// sphere.wgsl:67-90 value_to_color: mix(col_k, col_k+1, t) = a*(1-t) + b*t.
__device__ __forceinline__ V3 value_to_color(float value) {
    float a[3], bb[3], t;
    if (0.0f <= value && value < 0.25f) {
        a[0] = 0.0f; a[1] = 0.4f; a[2] = 0.8f;
        bb[0] = 35.0f / 256.0f; bb[1] = 161.0f / 256.0f; bb[2] = 165.0f / 256.0f;
        t = dvd(value, 0.25f);
    } else if (0.25f <= value && value < 0.50f) {
        a[0] = 35.0f / 256.0f; a[1] = 161.0f / 256.0f; a[2] = 165.0f / 256.0f;
        bb[0] = 95.0f / 256.0f; bb[1] = 254.0f / 256.0f; bb[2] = 150.0f / 256.0f;
        t = dvd(sub(value, 0.25f), 0.25f);
    } else if (0.50f <= value && value < 0.75f) {
        a[0] = 95.0f / 256.0f; a[1] = 254.0f / 256.0f; a[2] = 150.0f / 256.0f;
        bb[0] = 243.0f / 256.0f; bb[1] = 250.0f / 256.0f; bb[2] = 49.0f / 256.0f;
        t = dvd(sub(value, 0.50f), 0.25f);
    } else {
        a[0] = 243.0f / 256.0f; a[1] = 250.0f / 256.0f; a[2] = 49.0f / 256.0f;
        bb[0] = 255.0f / 256.0f; bb[1] = 165.0f / 256.0f; bb[2] = 0.0f;
        t = dvd(sub(value, 0.75f), 0.25f);
    }
    const float om = sub(1.0f, t);
    return v3(add(mul(a[0], om), mul(bb[0], t)), add(mul(a[1], om), mul(bb[1], t)),
              add(mul(a[2], om), mul(bb[2], t)));
}

__global__ void k_sphere_shade(const float4* __restrict__ posvel, Uni u, Consts c,
                               const unsigned long long* __restrict__ dkey,
                               float4* __restrict__ out, uchar4* __restrict__ out8,
                               float* __restrict__ depth) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= c.W * c.H) return;
    const unsigned long long key = dkey[p];
    V3 col = v3(0.8f, 0.8f, 0.8f);  // the sphere pass's clear colour (fluidRender.ts:425)
    float d = 1.0f;
    if (key != kClearKey) {
        Billboard b;
        Frag f;
        const int i = (int)(key & 0xffffffffull);
        const int px = p % c.W, py = p / c.W;
        if (billboard(posvel, i, u, c, b) && fragment(b, px, py, u, f)) {
            const float4 v = posvel[2 * (size_t)i + 1];
            const float speed = __fsqrt_rn(vdot(v3(v.x, v.y, v.z), v3(v.x, v.y, v.z)));
            const float cx = add((float)px, 0.5f), cy = add((float)py, 0.5f);
            const float nx = sub(mul(dvd(sub(cx, b.fxm), sub(b.fxp, b.fxm)), 2.0f), 1.0f);
            const float ny = sub(mul(dvd(sub(cy, b.fym), sub(b.fyp, b.fym)), 2.0f), 1.0f);
            const float inv_len = dvd(1.0f, __fsqrt_rn(3.0f));  // normalize(vec3(1, 1, 1))
            const float diffuse = wmax(0.0f, vdot(v3(nx, ny, f.nz), v3(inv_len, inv_len, inv_len)));
            col = vscale(value_to_color(dvd(speed, 1.5f)), diffuse);
            d = f.depth;
        }
    }
    out[p] = make_float4(col.x, col.y, col.z, 1.0f);
    auto u8 = [](float x) -> unsigned char {
        if (x != x) return 0;
        return (unsigned char)rintf(mul(wmin(wmax(x, 0.0f), 1.0f), 255.0f));
    };
    out8[p] = make_uchar4(u8(col.x), u8(col.y), u8(col.z), 255);
    depth[p] = d;
}

int fail(int code, const std::string& msg) {
    mpm::set_last_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(MPM_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

struct mpm_renderer {
    int device = 0;
    Consts c{};
    unsigned long long* dkey = nullptr;
    unsigned long long* tacc = nullptr;
    float* depth[2] = {nullptr, nullptr};
    float* thick[2] = {nullptr, nullptr};
    float4* color = nullptr;
    uchar4* color8 = nullptr;
    float4* env = nullptr;
    int env_size = 0;
    float* wtab = nullptr;  // bilateral spatial weights, kWRow x kWRow
    float* gtab = nullptr;  // gaussian weights, kGaussFs + 1
};

namespace {

void free_renderer(mpm_renderer* r) {
    cudaFree(r->dkey);
    cudaFree(r->tacc);
    for (int i = 0; i < 2; ++i) {
        cudaFree(r->depth[i]);
        cudaFree(r->thick[i]);
    }
    cudaFree(r->color);
    cudaFree(r->color8);
    cudaFree(r->env);
    cudaFree(r->wtab);
    cudaFree(r->gtab);
    delete r;
}

// Default environment: a sky gradient (no image decoding here), bright above
// the horizon, darker below, 32 x 32 per face.
std::vector<float> default_env(int size) {
    std::vector<float> px((size_t)6 * size * size * 4);
    for (int f = 0; f < 6; ++f)
        for (int j = 0; j < size; ++j)
            for (int i = 0; i < size; ++i) {
                const float s = 2.0f * ((float)i + 0.5f) / (float)size - 1.0f;
                const float t = 2.0f * ((float)j + 0.5f) / (float)size - 1.0f;
                float d[3];
                switch (f) {  // inverse of the face table used by sample_cube
                    case 0: d[0] = 1; d[1] = -t; d[2] = -s; break;
                    case 1: d[0] = -1; d[1] = -t; d[2] = s; break;
                    case 2: d[0] = s; d[1] = 1; d[2] = t; break;
                    case 3: d[0] = s; d[1] = -1; d[2] = -t; break;
                    case 4: d[0] = s; d[1] = -t; d[2] = 1; break;
                    default: d[0] = -s; d[1] = -t; d[2] = -1; break;
                }
                const float l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                const float y = d[1] / l;
                float* q = px.data() + (((size_t)f * size + j) * size + i) * 4;
                const float h = y > 0.0f ? y : 0.0f;
                q[0] = 0.55f + 0.25f * h + (y < 0.0f ? 0.2f * y : 0.0f);
                q[1] = 0.65f + 0.25f * h + (y < 0.0f ? 0.2f * y : 0.0f);
                q[2] = 0.80f + 0.20f * h + (y < 0.0f ? 0.1f * y : 0.0f);
                q[3] = 1.0f;
            }
    return px;
}

int upload_env(mpm_renderer* r, int size, const float* rgba) {
    float4* e = nullptr;
    cudaError_t err = cudaMalloc(&e, sizeof(float4) * 6 * (size_t)size * size);
    if (err == cudaSuccess)
        err = cudaMemcpy(e, rgba, sizeof(float4) * 6 * (size_t)size * size, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
        cudaFree(e);
        return cuda_fail(err, "envmap");
    }
    cudaFree(r->env);
    r->env = e;
    r->env_size = size;
    return MPM_OK;
}

}  // namespace

extern "C" {

int mpm_renderer_create(int width, int height, float radius, float fov, mpm_renderer** out) {
    if (!out) return fail(MPM_E_INVALID, "out is null");
    *out = nullptr;
    if (width < 1 || height < 1 || (long long)width * height > (1LL << 28))
        return fail(MPM_E_INVALID, "image size outside [1, 2^28] pixels");
    if (!(radius > 0.0f) || !(fov > 0.0f) || !(fov < 3.14159f))
        return fail(MPM_E_INVALID, "radius must be positive and fov in (0, pi)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(MPM_E_NO_DEVICE, "no CUDA device");
    }
    mpm_renderer* r = new mpm_renderer();
    cudaGetDevice(&r->device);
    r->c.W = width;
    r->c.H = height;
    // fluidRender.ts:38-46 (computed in doubles, as JS does, then f32 constants)
    const double diameter = 2.0 * (double)radius;
    r->c.depth_threshold = (float)((double)radius * 10.0);
    r->c.max_filter_size = 100.0f;
    r->c.ppc = (float)((12.0 * diameter * 0.05 * ((double)height / 2.0)) / std::tan((double)fov / 2.0));
    const size_t np = (size_t)width * height;
    cudaError_t e = cudaMalloc(&r->dkey, 8 * np);
    if (e == cudaSuccess) e = cudaMalloc(&r->tacc, 8 * np);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaMalloc(&r->depth[i], 4 * np);
        if (e == cudaSuccess) e = cudaMalloc(&r->thick[i], 4 * np);
    }
    if (e == cudaSuccess) e = cudaMalloc(&r->color, sizeof(float4) * np);
    if (e == cudaSuccess) e = cudaMalloc(&r->color8, sizeof(uchar4) * np);
    if (e == cudaSuccess) e = cudaMalloc(&r->wtab, sizeof(float) * kWRow * kWRow);
    if (e == cudaSuccess) e = cudaMalloc(&r->gtab, sizeof(float) * (kGaussFs + 1));
    if (e == cudaSuccess) {
        k_weight_tables<<<(kWRow * kWRow + 255) / 256, 256>>>(r->wtab, r->gtab);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        const int rc = cuda_fail(e, "mpm_renderer_create");
        free_renderer(r);
        return rc;
    }
    const std::vector<float> env = default_env(32);
    if (int rc = upload_env(r, 32, env.data())) {
        free_renderer(r);
        return rc;
    }
    *out = r;
    return MPM_OK;
}

int mpm_renderer_destroy(mpm_renderer* r) {
    if (!r) return MPM_OK;
    cudaDeviceSynchronize();
    free_renderer(r);
    return MPM_OK;
}

int mpm_renderer_set_envmap(mpm_renderer* r, int face_size, const float* rgba) {
    if (!r || !rgba || face_size < 1 || face_size > 4096) return fail(MPM_E_INVALID, "bad envmap");
    cudaDeviceSynchronize();
    return upload_env(r, face_size, rgba);
}

int mpm_renderer_execute(mpm_renderer* r, const void* posvel, int n,
                         const mpm_render_uniforms* uniforms, void* stream) {
    if (!r || !uniforms || n < 0 || (n > 0 && !posvel)) return fail(MPM_E_INVALID, "bad arguments");
    Uni u;
    static_assert(sizeof(mpm_render_uniforms) == sizeof(Uni), "uniform layout");
    std::memcpy(&u, uniforms, sizeof(Uni));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Consts& c = r->c;
    const int npix = c.W * c.H;
    const int pb = (npix + 255) / 256;
    const float4* pv = static_cast<const float4*>(posvel);
    k_clear<<<pb, 256, 0, st>>>(r->dkey, r->tacc, npix);
    if (n > 0) k_splat<<<(n + 127) / 128, 128, 0, st>>>(pv, n, u, c, r->dkey, r->tacc);
    k_resolve<<<pb, 256, 0, st>>>(pv, u, c, r->dkey, r->tacc, r->depth[0], r->thick[0]);
    for (int it = 0; it < 4; ++it) {  // fluidRender.ts:455-466
        k_bilateral<<<pb, 256, 0, st>>>(r->depth[0], r->depth[1], c, r->wtab, 1, 0);
        k_bilateral<<<pb, 256, 0, st>>>(r->depth[1], r->depth[0], c, r->wtab, 0, 1);
    }
    k_gaussian<<<pb, 256, 0, st>>>(r->thick[0], r->thick[1], c, r->gtab, 1, 0);  // :474-486
    k_gaussian<<<pb, 256, 0, st>>>(r->thick[1], r->thick[0], c, r->gtab, 0, 1);
    k_shade<<<pb, 256, 0, st>>>(r->depth[0], r->thick[0], r->env, r->env_size, u, c, r->color,
                                r->color8);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mpm_renderer_execute");
    return MPM_OK;
}

int mpm_renderer_execute_spheres(mpm_renderer* r, const void* posvel, int n,
                                 const mpm_render_uniforms* uniforms, void* stream) {
    if (!r || !uniforms || n < 0 || (n > 0 && !posvel)) return fail(MPM_E_INVALID, "bad arguments");
    Uni u;
    std::memcpy(&u, uniforms, sizeof(Uni));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Consts& c = r->c;
    const int npix = c.W * c.H;
    const int pb = (npix + 255) / 256;
    const float4* pv = static_cast<const float4*>(posvel);
    k_clear<<<pb, 256, 0, st>>>(r->dkey, r->tacc, npix);
    if (n > 0) k_sphere_splat<<<(n + 127) / 128, 128, 0, st>>>(pv, n, u, c, r->dkey);
    k_sphere_shade<<<pb, 256, 0, st>>>(pv, u, c, r->dkey, r->color, r->color8, r->depth[0]);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mpm_renderer_execute_spheres");
    return MPM_OK;
}

int mpm_renderer_download(mpm_renderer* r, int what, void* out) {
    if (!r || !out) return fail(MPM_E_INVALID, "bad arguments");
    const size_t np = (size_t)r->c.W * r->c.H;
    const void* src = nullptr;
    size_t bytes = 0;
    switch (what) {
        case MPM_RENDER_COLOR: src = r->color; bytes = sizeof(float4) * np; break;
        case MPM_RENDER_COLOR8: src = r->color8; bytes = 4 * np; break;
        case MPM_RENDER_DEPTH: src = r->depth[0]; bytes = 4 * np; break;
        case MPM_RENDER_THICKNESS: src = r->thick[0]; bytes = 4 * np; break;
        default: return fail(MPM_E_INVALID, "unknown image");
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(out, src, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "mpm_renderer_download");
    return MPM_OK;
}

void* mpm_renderer_color_device_ptr(mpm_renderer* r) { return r ? r->color : nullptr; }

}  // extern "C"
