/*
 * render_oracle.c -- CPU restatement of WebGPU-Ocean's screen-space fluid
 * renderer (render/fluidRender.ts:292-488, fluid path).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/ as the checker of the headless
 * CUDA renderer, never by the product.
 *
 * The fullscreen passes are pinned to the reference itself:
 * tests/golden/make_golden_render.py runs its bilateral.wgsl, gaussian.wgsl
 * and fluid.wgsl fragment shaders (read as text) per pixel through the WGSL
 * interpreter, and bilateral_pass / gaussian_pass / shade_pass reproduce them
 * bit for bit.  The two splats are unpinned: they need rasterisation, depth
 * testing and blending, i.e. a WebGPU implementation and a graphics stack,
 * neither of which exists here (unavailable on this machine).  This file restates
 * the shader math of
 *   depthMap.wgsl:34-79      billboard depth splat, 'less' depth test
 *   thicknessMap.wgsl:27-62  additive thickness splat
 *   sphere.wgsl:37-110       sphere mode (ro_sphere)
 *   bilateral.wgsl:18-75     separable bilateral depth filter (4 x X, Y)
 *   gaussian.wgsl:14-42      separable gaussian thickness filter (X, Y)
 *   fluid.wgsl:19-98         shading
 * with the rasterisation and texture rules the library documents
 * (pixel-centre coverage of the billboard's screen rectangle, top-left edge
 * rule, first-drawn fragment wins depth ties, frag_depth clamped to [0, 1],
 * thickness summed in 2^-32 fixed point then rounded to half precision,
 * texture coordinates clamped to the texture, every r16float write rounded
 * to half), and the same exp / log / pow restatement (Cody-Waite reduction +
 * Taylor series; atanh series for log), operation for operation.  Build
 * with -ffp-contract=off.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct ro_uniforms { /* RenderUniforms, common.ts:1-9 */
    float texel[2];
    float sphere_size;
    float pad;
    float invP[16], P[16], V[16], invV[16];
} ro_uniforms;

static float fbits(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t bitsf(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

static float pow2i(int k) { return fbits((uint32_t)(k + 127) << 23); }

static float exp_r(float x) {
    if (x != x) return x;
    if (x > 88.8f) return fbits(0x7f800000u);
    if (x < -104.0f) return 0.0f;
    const float kf = rintf(x * 1.44269502f);
    const int k = (int)kf;
    const float r = (x - kf * 0.693145751953125f) - kf * 1.42860677e-6f;
    float p = 2.48015873e-5f;
    p = p * r + 1.98412698e-4f;
    p = p * r + 1.38888889e-3f;
    p = p * r + 8.33333333e-3f;
    p = p * r + 4.16666667e-2f;
    p = p * r + 1.66666667e-1f;
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    const int k1 = k / 2, k2 = k - k1;
    return (p * pow2i(k1)) * pow2i(k2);
}

static float log_r(float x) {
    if (x != x || x < 0.0f) return fbits(0x7fc00000u);
    if (x == 0.0f) return fbits(0xff800000u);
    if (x == fbits(0x7f800000u)) return x;
    int e = 0;
    float m = x;
    if (m < 1.17549435e-38f) {
        m = m * 16777216.0f;
        e = -24;
    }
    const uint32_t b = bitsf(m);
    e += (int)((b >> 23) & 0xffu) - 127;
    m = fbits((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float q = 9.09090909e-2f;
    q = q * s2 + 1.11111111e-1f;
    q = q * s2 + 1.42857143e-1f;
    q = q * s2 + 2.0e-1f;
    q = q * s2 + 3.33333333e-1f;
    q = q * s2 + 1.0f;
    const float lm = (2.0f * s) * q;
    return (float)e * 0.693147181f + lm;
}

static float pow_r(float x, float y) {
    if (x == 0.0f && y > 0.0f) return 0.0f;
    return exp_r(y * log_r(x));
}

/* float -> nearest-even half -> float */
static float half_round(float x) {
    const uint32_t b = bitsf(x);
    const uint32_t sign = b & 0x80000000u, ab = b & 0x7fffffffu;
    if (ab >= 0x7f800000u) return x;
    const float a = fbits(ab);
    if (a >= 65520.0f) return fbits(sign | 0x7f800000u);
    if (a < 6.103515625e-05f) {
        const float r = rintf(a * 16777216.0f) * 5.9604644775390625e-08f;
        return fbits(sign | bitsf(r));
    }
    uint32_t m = ab + 0xfffu + ((ab >> 13) & 1u);
    m &= ~0x1fffu;
    return fbits(sign | m);
}

static float wmax(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return a < b ? b : a;
}
static float wmin(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return b < a ? b : a;
}

static int f2i_sat(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int)(-2147483647 - 1);
    return (int)x;
}

typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } v4;

static v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 vscale(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static v3 vcross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static v3 vnormalize(v3 a) {
    const float l = sqrtf(vdot(a, a));
    return mk(a.x / l, a.y / l, a.z / l);
}
static v4 mat4_mul(const float* m, float x, float y, float z, float w) {
    v4 r;
    r.x = ((m[0] * x + m[4] * y) + m[8] * z) + m[12] * w;
    r.y = ((m[1] * x + m[5] * y) + m[9] * z) + m[13] * w;
    r.z = ((m[2] * x + m[6] * y) + m[10] * z) + m[14] * w;
    r.w = ((m[3] * x + m[7] * y) + m[11] * z) + m[15] * w;
    return r;
}

typedef struct {
    v3 view;
    float fxm, fxp, fym, fyp;
    int x0, x1, y0, y1;
} billboard_t;

static int billboard(const float* posvel, int64_t i, const ro_uniforms* u, int W, int H,
                     billboard_t* b) {
    const float* p = posvel + 8 * i;
    const v4 vp = mat4_mul(u->V, p[0], p[1], p[2], 1.0f);
    b->view = mk(vp.x, vp.y, vp.z);
    const float s = u->sphere_size;
    const v4 cm = mat4_mul(u->P, b->view.x + (-0.5f * s), b->view.y + (-0.5f * s), b->view.z, 1.0f);
    const v4 cp = mat4_mul(u->P, b->view.x + 0.5f * s, b->view.y + 0.5f * s, b->view.z, 1.0f);
    const v4 cc = mat4_mul(u->P, b->view.x, b->view.y, b->view.z, 1.0f);
    if (!(cc.w > 0.0f)) return 0;
    const float zq = cc.z / cc.w;
    if (!(zq >= 0.0f && zq <= 1.0f)) return 0;
    const float Wf = (float)W, Hf = (float)H;
    b->fxm = (cm.x / cm.w + 1.0f) * (0.5f * Wf);
    b->fxp = (cp.x / cp.w + 1.0f) * (0.5f * Wf);
    b->fym = (1.0f - cm.y / cm.w) * (0.5f * Hf);
    b->fyp = (1.0f - cp.y / cp.w) * (0.5f * Hf);
    const float X0 = fminf(b->fxm, b->fxp), X1 = fmaxf(b->fxm, b->fxp);
    const float Y0 = fminf(b->fym, b->fyp), Y1 = fmaxf(b->fym, b->fyp);
    if (!(X1 > X0) || !(Y1 > Y0)) return 0;
    const float lx = ceilf(X0 - 0.5f), hx = ceilf(X1 - 0.5f) - 1.0f;
    const float ly = ceilf(Y0 - 0.5f), hy = ceilf(Y1 - 0.5f) - 1.0f;
    b->x0 = (int)fminf(fmaxf(lx, 0.0f), Wf);
    b->x1 = (int)fmaxf(fminf(hx, Wf - 1.0f), -1.0f);
    b->y0 = (int)fminf(fmaxf(ly, 0.0f), Hf);
    b->y1 = (int)fmaxf(fminf(hy, Hf - 1.0f), -1.0f);
    return b->x0 <= b->x1 && b->y0 <= b->y1;
}

typedef struct { float depth, vz, nz; } frag_t;

static int fragment(const billboard_t* b, int px, int py, const ro_uniforms* u, frag_t* f) {
    const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
    const float uu = (cx - b->fxm) / (b->fxp - b->fxm);
    const float vv = (cy - b->fym) / (b->fyp - b->fym);
    const float nx = uu * 2.0f - 1.0f, ny = vv * 2.0f - 1.0f;
    const float r2 = nx * nx + ny * ny;
    if (r2 > 1.0f) return 0;
    const float nz = sqrtf(1.0f - r2);
    const float radius = u->sphere_size / 2.0f;
    const v3 rv = vadd(b->view, vscale(mk(nx, ny, nz), radius));
    const v4 clip = mat4_mul(u->P, rv.x, rv.y, rv.z, 1.0f);
    f->depth = wmin(wmax(clip.z / clip.w, 0.0f), 1.0f);
    f->vz = rv.z;
    f->nz = nz;
    return 1;
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

static v3 view_pos(const ro_uniforms* u, float tx, float ty, float depth) {
    const float nx = tx * 2.0f - 1.0f;
    const float ny = 1.0f - 2.0f * ty;
    const float nz = -u->P[10] + u->P[14] / depth;
    const v4 e = mat4_mul(u->invP, nx, ny, nz, 1.0f);
    return mk(e.x / e.w, e.y / e.w, e.z / e.w);
}

static v3 sample_cube(const float* env, int size, v3 d) {
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
    if (!(ma > 0.0f) || ma == fbits(0x7f800000u)) {
        const float q = fbits(0x7fc00000u);
        return mk(q, q, q);
    }
    const float s = 0.5f * (sc / ma + 1.0f);
    const float t = 0.5f * (tc / ma + 1.0f);
    const float fu = s * (float)size - 0.5f, fv = t * (float)size - 0.5f;
    const float iu = floorf(fu), iv = floorf(fv);
    const float a = fu - iu, bb = fv - iv;
    const int u0 = clampi((int)iu, 0, size - 1), u1 = clampi((int)iu + 1, 0, size - 1);
    const int v0 = clampi((int)iv, 0, size - 1), v1 = clampi((int)iv + 1, 0, size - 1);
    const float* f = env + (size_t)face * size * size * 4;
    const float* c00 = f + ((size_t)v0 * size + u0) * 4;
    const float* c10 = f + ((size_t)v0 * size + u1) * 4;
    const float* c01 = f + ((size_t)v1 * size + u0) * 4;
    const float* c11 = f + ((size_t)v1 * size + u1) * 4;
    const float ia = 1.0f - a, ib = 1.0f - bb;
    float o[3];
    for (int k = 0; k < 3; ++k) {
        const float top = c00[k] * ia + c10[k] * a;
        const float bot = c01[k] * ia + c11[k] * a;
        o[k] = top * ib + bot * bb;
    }
    return mk(o[0], o[1], o[2]);
}

/*
 * Renders n particles (posvel: n x 8 floats) into W x H images:
 * color (W*H*4 floats), color8 (W*H*4 bytes), depth and thickness (W*H
 * floats, after filtering).  env: 6 x size x size x 4 floats.  Filter
 * constants as fluidRender.ts:38-46.  Returns 0, or -1 on allocation failure.
 */
/* One pass of bilateral.wgsl:18-75 over a W x H depth image along (dx, dy):
 * texel coordinates outside the image are clamped to its edge (WGSL lets an
 * out-of-bounds textureLoad return any texel within bounds). */
static void bilateral_pass(const float* src, float* dst, int W, int H, int dx, int dy,
                           float depth_threshold, float max_filter_size, float ppc) {
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const size_t p = (size_t)py * W + px;
            const float depth = fabsf(src[p]);
            if (depth >= 1e4f || depth <= 0.0f) {
                dst[p] = depth;
                continue;
            }
            const int a = f2i_sat(max_filter_size), c = f2i_sat(ceilf(ppc / depth));
            const int fs = a < c ? a : c;
            const float sigma = (float)fs / 3.0f;
            const float two_sigma = (2.0f * sigma) * sigma;
            const float sd = depth_threshold / 3.0f;
            const float two_sd = (2.0f * sd) * sd;
            float sum = 0.0f, wsum = 0.0f;
            for (int x = -fs; x <= fs; ++x) {
                const float xf = (float)x;
                const int ix = clampi(px + x * dx, 0, W - 1), iy = clampi(py + x * dy, 0, H - 1);
                const float sampled = fabsf(src[(size_t)iy * W + ix]);
                const float rr = xf * xf + xf * xf;
                const float w = exp_r(-rr / two_sigma);
                const float rd = sampled - depth;
                const float wd = exp_r((-rd * rd) / two_sd);
                sum = sum + (sampled * w) * wd;
                wsum = wsum + w * wd;
            }
            dst[p] = sum / wsum;
        }
}

/* One pass of gaussian.wgsl:14-42 over a W x H thickness image along
 * (dx, dy), the result stored into the r16float target (rounded to half). */
static void gaussian_pass(const float* src, float* dst, int W, int H, int dx, int dy) {
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const size_t p = (size_t)py * W + px;
            const float t = src[p];
            if (t == 0.0f) {
                dst[p] = 0.0f;
                continue;
            }
            const int fs = 30;
            const float sigma = (float)fs / 3.0f;
            const float two_sigma = (2.0f * sigma) * sigma;
            float sum = 0.0f, wsum = 0.0f;
            for (int x = -fs; x <= fs; ++x) {
                const float xf = (float)x;
                const int ix = clampi(px + x * dx, 0, W - 1), iy = clampi(py + x * dy, 0, H - 1);
                const float sampled = src[(size_t)iy * W + ix];
                const float w = exp_r((-xf * xf) / two_sigma);
                sum = sum + sampled * w;
                wsum = wsum + w;
            }
            dst[p] = half_round(sum / wsum);
        }
}

/* fluid.wgsl:19-98 over W x H pixels: the filtered depth d0 and thickness
 * t0 in, colour (W*H*4 floats) and its rgba8unorm store (color8) out. */
static void shade_pass(const float* d0, const float* t0, const ro_uniforms* u, const float* env,
                       int env_size, int W, int H, float* color, uint8_t* color8) {
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const size_t p = (size_t)py * W + px;
            const float tx = ((float)px + 0.5f) / (float)W;
            const float ty = ((float)py + 0.5f) / (float)H;
            const v3 bg = mk(0.8f, 0.8f, 0.8f);
            const float depth = fabsf(d0[p]);
            v3 col;
            if (depth >= 1e4f || depth <= 0.0f) {
                col = bg;
            } else {
                const v3 vp = view_pos(u, tx, ty, depth);
#define AT(qx, qy, sx, sy) view_pos(u, (sx), (sy), fabsf(d0[(size_t)clampi((qy), 0, H - 1) * W + clampi((qx), 0, W - 1)]))
                v3 ddx = vsub(AT(px + 1, py, tx + u->texel[0], ty), vp);
                v3 ddy = vsub(AT(px, py + 1, tx, ty + u->texel[1]), vp);
                const v3 ddx2 = vsub(vp, AT(px - 1, py, tx - u->texel[0], ty));
                const v3 ddy2 = vsub(vp, AT(px, py - 1, tx, ty - u->texel[1]));
#undef AT
                if (fabsf(ddx.z) > fabsf(ddx2.z)) ddx = ddx2;
                if (fabsf(ddy.z) > fabsf(ddy2.z)) ddy = ddy2;
                const v3 nn = vnormalize(vcross(ddx, ddy));
                const v3 normal = mk(-nn.x, -nn.y, -nn.z);
                const v3 ray = vnormalize(vp);
                const v4 l4 = mat4_mul(u->V, 0.0f, 0.0f, -1.0f, 0.0f);
                const v3 light = vnormalize(mk(l4.x, l4.y, l4.z));
                const v3 hv = vnormalize(vsub(light, ray));
                const float specular = pow_r(wmax(0.0f, vdot(hv, normal)), 250.0f);
                const float density = 1.5f;
                const float thickness = t0[p];
                const v3 dc = mk(0.085f, 0.6375f, 0.9f);
                const float a = -density * thickness;
                const v3 trans = mk(exp_r(a * (1.0f - dc.x)), exp_r(a * (1.0f - dc.y)),
                                    exp_r(a * (1.0f - dc.z)));
                const v3 refr = mk(bg.x * trans.x, bg.y * trans.y, bg.z * trans.z);
                const float F0 = 0.02f;
                const float cosv = vdot(normal, mk(-ray.x, -ray.y, -ray.z));
                const float fres =
                    wmin(wmax(F0 + (1.0f - F0) * pow_r(1.0f - cosv, 5.0f), 0.0f), 1.0f);
                const v3 refl = vsub(ray, vscale(normal, 2.0f * vdot(normal, ray)));
                const v4 rw = mat4_mul(u->invV, refl.x, refl.y, refl.z, 0.0f);
                const v3 env_col = sample_cube(env, env_size, mk(rw.x, rw.y, rw.z));
                const float omf = 1.0f - fres;
                col = mk(1.0f * specular + (refr.x * omf + env_col.x * fres),
                         1.0f * specular + (refr.y * omf + env_col.y * fres),
                         1.0f * specular + (refr.z * omf + env_col.z * fres));
            }
            const float cv[3] = {col.x, col.y, col.z};
            for (int k = 0; k < 3; ++k) {
                color[4 * p + k] = cv[k];
                color8[4 * p + k] = cv[k] != cv[k] ? 0 : (uint8_t)rintf(wmin(wmax(cv[k], 0.0f), 1.0f) * 255.0f);
            }
            color[4 * p + 3] = 1.0f;
            color8[4 * p + 3] = 255;
        }
}

/* The depth and thickness splats and the depth resolve (depthMap.wgsl,
 * thicknessMap.wgsl): d0 = view-space z of the nearest fragment (0 where
 * none), t0 = the additive thickness rounded to half. */
static int splat(const float* posvel, int64_t n, const ro_uniforms* u, int W, int H, float* d0,
                 float* t0) {
    const size_t np = (size_t)W * H;
    uint64_t* dkey = (uint64_t*)malloc(8 * np);
    int64_t* tacc = (int64_t*)calloc(np, 8);
    if (!dkey || !tacc) {
        free(dkey); free(tacc);
        return -1;
    }
    const uint64_t clear_key = ((uint64_t)0x3f800000u << 32) | 0xffffffffu;
    for (size_t p = 0; p < np; ++p) dkey[p] = clear_key;
    /* splats */
    for (int64_t i = 0; i < n; ++i) {
        billboard_t b;
        if (!billboard(posvel, i, u, W, H, &b)) continue;
        for (int py = b.y0; py <= b.y1; ++py)
            for (int px = b.x0; px <= b.x1; ++px) {
                frag_t f;
                if (!fragment(&b, px, py, u, &f)) continue;
                const size_t p = (size_t)py * W + px;
                if (f.depth < 1.0f) {
                    const uint64_t key = ((uint64_t)bitsf(f.depth) << 32) | (uint32_t)i;
                    if (key < dkey[p]) dkey[p] = key;
                }
                const float t = 0.05f * f.nz;
                tacc[p] += (int64_t)llrintf(t * 4294967296.0f);
            }
    }
    /* resolve */
    for (size_t p = 0; p < np; ++p) {
        float d = 0.0f;
        if (dkey[p] != clear_key) {
            billboard_t b;
            frag_t f;
            const int64_t i = (int64_t)(dkey[p] & 0xffffffffu);
            if (billboard(posvel, i, u, W, H, &b) && fragment(&b, (int)(p % W), (int)(p / W), u, &f))
                d = f.vz;
        }
        d0[p] = d;
        t0[p] = half_round((float)tacc[p] * 2.3283064365386963e-10f);
    }
    free(dkey); free(tacc);
    return 0;
}

int ro_splat(const float* posvel, int64_t n, const ro_uniforms* u, int W, int H, float* depth_out,
             float* thick_out) {
    return splat(posvel, n, u, W, H, depth_out, thick_out);
}

int ro_render(const float* posvel, int64_t n, const ro_uniforms* u, int W, int H,
              float depth_threshold, float max_filter_size, float ppc, const float* env,
              int env_size, float* color, uint8_t* color8, float* depth_out, float* thick_out) {
    const size_t np = (size_t)W * H;
    float* d0 = (float*)malloc(4 * np);
    float* d1 = (float*)malloc(4 * np);
    float* t0 = (float*)malloc(4 * np);
    float* t1 = (float*)malloc(4 * np);
    if (!d0 || !d1 || !t0 || !t1 || splat(posvel, n, u, W, H, d0, t0) != 0) {
        free(d0); free(d1); free(t0); free(t1);
        return -1;
    }
    /* bilateral depth filter, 4 x (X, Y) */
    for (int it = 0; it < 8; ++it)
        bilateral_pass((it & 1) ? d1 : d0, (it & 1) ? d0 : d1, W, H, (it & 1) ? 0 : 1,
                       (it & 1) ? 1 : 0, depth_threshold, max_filter_size, ppc);
    /* gaussian thickness filter, X then Y */
    for (int it = 0; it < 2; ++it)
        gaussian_pass(it ? t1 : t0, it ? t0 : t1, W, H, it ? 0 : 1, it ? 1 : 0);
    /* shading */
    shade_pass(d0, t0, u, env, env_size, W, H, color, color8);
    memcpy(depth_out, d0, 4 * np);
    memcpy(thick_out, t0, 4 * np);
    free(d0); free(d1); free(t0); free(t1);
    return 0;
}

/* sphere.wgsl:67-90 value_to_color. */
static v3 value_to_color(float value) {
    const v3 col[5] = {mk(0.0f, 0.4f, 0.8f), mk(35.0f / 256.0f, 161.0f / 256.0f, 165.0f / 256.0f),
                       mk(95.0f / 256.0f, 254.0f / 256.0f, 150.0f / 256.0f),
                       mk(243.0f / 256.0f, 250.0f / 256.0f, 49.0f / 256.0f),
                       mk(255.0f / 256.0f, 165.0f / 256.0f, 0.0f / 256.0f)};
    int k;
    float t;
    if (0.0f <= value && value < 0.25f) { k = 0; t = value / 0.25f; }
    else if (0.25f <= value && value < 0.50f) { k = 1; t = (value - 0.25f) / 0.25f; }
    else if (0.50f <= value && value < 0.75f) { k = 2; t = (value - 0.50f) / 0.25f; }
    else { k = 3; t = (value - 0.75f) / 0.25f; }
    const float om = 1.0f - t;  /* mix(a, b, t) = a * (1 - t) + b * t */
    return mk(col[k].x * om + col[k + 1].x * t, col[k].y * om + col[k + 1].y * t,
              col[k].z * om + col[k + 1].z * t);
}

/* Sphere mode (render/sphere.wgsl, render/fluidRender.ts:481-485): each
 * particle's billboard shaded as a lit sphere coloured by its speed, with
 * the depth test 'less' (first-drawn fragment wins ties) over the clear
 * colour (0.8, 0.8, 0.8, 1).  color: W*H*4 floats, color8 its rgba8unorm
 * store, depth_out: the winning frag_depth (1 where none). */
int ro_sphere(const float* posvel, int64_t n, const ro_uniforms* u, int W, int H, float* color,
              uint8_t* color8, float* depth_out) {
    const size_t np = (size_t)W * H;
    uint64_t* dkey = (uint64_t*)malloc(8 * np);
    if (!dkey) return -1;
    const uint64_t clear_key = ((uint64_t)0x3f800000u << 32) | 0xffffffffu;
    for (size_t p = 0; p < np; ++p) dkey[p] = clear_key;
    for (int64_t i = 0; i < n; ++i) {
        billboard_t b;
        if (!billboard(posvel, i, u, W, H, &b)) continue;
        for (int py = b.y0; py <= b.y1; ++py)
            for (int px = b.x0; px <= b.x1; ++px) {
                frag_t f;
                if (!fragment(&b, px, py, u, &f)) continue;
                const size_t p = (size_t)py * W + px;
                if (f.depth < 1.0f) {
                    const uint64_t key = ((uint64_t)bitsf(f.depth) << 32) | (uint32_t)i;
                    if (key < dkey[p]) dkey[p] = key;
                }
            }
    }
    const float inv_len = 1.0f / sqrtf(3.0f);  /* normalize(vec3(1.0, 1.0, 1.0)) */
    for (size_t p = 0; p < np; ++p) {
        v3 col = mk(0.8f, 0.8f, 0.8f);
        float depth = 1.0f;
        if (dkey[p] != clear_key) {
            const int64_t i = (int64_t)(dkey[p] & 0xffffffffu);
            billboard_t b;
            frag_t f;
            if (billboard(posvel, i, u, W, H, &b) &&
                fragment(&b, (int)(p % W), (int)(p / W), u, &f)) {
                const float* pv = posvel + 8 * i;
                const v3 v = mk(pv[4], pv[5], pv[6]);
                const float speed = sqrtf(vdot(v, v));
                const float cx = (float)(p % W) + 0.5f, cy = (float)(p / W) + 0.5f;
                const float nx = ((cx - b.fxm) / (b.fxp - b.fxm)) * 2.0f - 1.0f;
                const float ny = ((cy - b.fym) / (b.fyp - b.fym)) * 2.0f - 1.0f;
                const float diffuse =
                    wmax(0.0f, vdot(mk(nx, ny, f.nz), mk(inv_len, inv_len, inv_len)));
                const v3 c = value_to_color(speed / 1.5f);
                col = vscale(c, diffuse);
                depth = f.depth;
            }
        }
        const float cv[3] = {col.x, col.y, col.z};
        for (int k = 0; k < 3; ++k) {
            color[4 * p + k] = cv[k];
            color8[4 * p + k] = cv[k] != cv[k] ? 0 : (uint8_t)rintf(wmin(wmax(cv[k], 0.0f), 1.0f) * 255.0f);
        }
        color[4 * p + 3] = 1.0f;
        color8[4 * p + 3] = 255;
        depth_out[p] = depth;
    }
    free(dkey);
    return 0;
}

/* The filter constants of fluidRender.ts:38-46 for an image height, radius
 * and field of view (doubles, as JS computes them). */
void ro_filter_constants(int H, double radius, double fov, float* depth_threshold,
                         float* max_filter_size, float* ppc) {
    const double diameter = 2.0 * radius;
    *depth_threshold = (float)(radius * 10.0);
    *max_filter_size = 100.0f;
    *ppc = (float)((12.0 * diameter * 0.05 * ((double)H / 2.0)) / tan(fov / 2.0));
}

/* The scalar helpers, for tests of the restatement itself. */
/* One filter pass alone (the golden tests run it against the reference's
 * own fragment shaders). */
void ro_bilateral_pass(const float* src, float* dst, int W, int H, int dx, int dy,
                       float depth_threshold, float max_filter_size, float ppc) {
    bilateral_pass(src, dst, W, H, dx, dy, depth_threshold, max_filter_size, ppc);
}
void ro_gaussian_pass(const float* src, float* dst, int W, int H, int dx, int dy) {
    gaussian_pass(src, dst, W, H, dx, dy);
}
void ro_shade_pass(const float* d0, const float* t0, const ro_uniforms* u, const float* env,
                   int env_size, int W, int H, float* color, uint8_t* color8) {
    shade_pass(d0, t0, u, env, env_size, W, H, color, color8);
}
/* The cube-map lookup of the shading pass (bilinear within the face the
 * direction selects), for the golden tests' interpreter. */
void ro_sample_cube(const float* env, int size, float x, float y, float z, float* out3) {
    const v3 c = sample_cube(env, size, mk(x, y, z));
    out3[0] = c.x;
    out3[1] = c.y;
    out3[2] = c.z;
}
float ro_exp(float x) { return exp_r(x); }
float ro_log(float x) { return log_r(x); }
float ro_pow(float x, float y) { return pow_r(x, y); }
float ro_half_round(float x) { return half_round(x); }
