/*
 * mpm_oracle.c -- CPU restatement of the WebGPU-Ocean MLS-MPM substep.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py (its
 * cpu_baseline leg and `--impl reference`) load it, always as the checker or
 * the baseline, never as the thing measured or shipped.  The product
 * (libmpm.so) neither links nor calls anything in oracle/.
 *
 * Parity pin: the reference ships no tests, fixtures or golden vectors, and
 * its kernels are WGSL that needs a WebGPU runtime (none exists here).  This
 * restatement is pinned against (1) golden vectors produced by executing the
 * reference's own WGSL source text with an independent float32 interpreter
 * (oracle/wgsl_interp.py, vectors under tests/golden/), and (2) hand-derived
 * known answers (tests/test_oracle.py).
 *
 * Each function follows one WGSL entry point of the reference, op for op:
 *   orc_clear_grid     mls-mpm/clearGrid.wgsl:10-18
 *   orc_p2g_1          mls-mpm/p2g_1.wgsl:24-65
 *   orc_p2g_2          mls-mpm/p2g_2.wgsl:30-94
 *   orc_update_grid    mls-mpm/updateGrid.wgsl:23-46
 *   orc_g2p            mls-mpm/g2p.wgsl:26-92
 *   orc_copy_position  mls-mpm/copyPosition.wgsl:15-21
 *   orc_execute        mls-mpm/mls-mpm.ts:245-268 (substeps x 6 dispatches)
 *
 * Arithmetic contract (shared bit for bit with the CUDA kernels):
 *   - every f32 `*`, `+`, `-`, `/` is rounded separately (build with
 *     -ffp-contract=off, never -ffast-math);
 *   - enc(f) = i32(f * FM): truncation toward zero, saturating, NaN -> 0
 *     (WGSL f32->i32 conversion);
 *   - dec(i) = f32(i) / FM: round-to-nearest conversion then IEEE division;
 *   - mat3x3f * vec3f = (c0*v.x + c1*v.y) + c2*v.z with C stored by columns;
 *   - pow(x, 5.) = ((x*x)*(x*x))*x, a fixed multiply chain (WGSL leaves pow's
 *     precision to the implementation);
 *   - max/min/clamp follow WGSL: max(a,b) = a < b ? b : a with NaN operands
 *     yielding the other operand;
 *   - i32 grid sums wrap (two's complement); flat cell indices are i32 with
 *     wraparound, computed with the truncated init_box_size, exactly as the
 *     shaders do (so out-of-box stencils alias, quirk Q1);
 *   - a flat index outside [0, grid_count) is dropped on write and reads as
 *     zero (WGSL leaves out-of-bounds behaviour to the implementation); each
 *     such access is counted in `oob`.
 *
 * Layouts (the reference's own, mls-mpm/mls-mpm.ts:10,204-209):
 *   particle = 20 floats (80 B): pos[0..2] pad, v[4..6] pad, C column c at
 *              [8+4c .. 10+4c] pad  (mat3x3f = 3 columns of 16 B)
 *   cell     = 4 x i32 (16 B): vx, vy, vz, mass
 *   posvel   = 8 floats (32 B): pos[0..2] pad, v[4..6] pad
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct orc_params {
    float stiffness;              /* mls-mpm.ts:54 */
    float rest_density;           /* mls-mpm.ts:55 */
    float dynamic_viscosity;      /* mls-mpm.ts:56 */
    float dt;                     /* mls-mpm.ts:57 */
    float fixed_point_multiplier; /* mls-mpm.ts:58 */
    /* Body force added per unit time in updateGrid.  The reference adds
       -0.3*dt to vy only (updateGrid.wgsl:34): zero components are left
       untouched, so (0, -0.3, 0) is the reference.  Other directions are the
       batched scenes' extension. */
    float gravity[3];
} orc_params;

/* ------------------------------------------------------------------ */
/* scalar helpers                                                      */
/* ------------------------------------------------------------------ */

/* WGSL i32(f32): round toward zero, saturate, NaN -> 0. */
static inline int32_t f2i_sat(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}

/* p2g_1.wgsl:15-17 */
static inline int32_t enc(float f, float fm) { return f2i_sat(f * fm); }

/* p2g_2.wgsl:22-24 */
static inline float dec(int32_t i, float fm) { return (float)i / fm; }

/* WGSL max/min (NaN operand -> the other operand). */
static inline float wmax(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (a < b) ? b : a;
}
static inline float wmin(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b < a) ? b : a;
}

static inline int32_t wrap_add(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a + (uint32_t)b);
}
static inline int32_t wrap_mul(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a * (uint32_t)b);
}

/* p2g_1.wgsl:53-56: i32(cx)*i32(Y)*i32(Z) + i32(cy)*i32(Z) + i32(cz) */
static inline int32_t flat_index(float cx, float cy, float cz, int32_t Y, int32_t Z) {
    int32_t a = wrap_mul(wrap_mul(f2i_sat(cx), Y), Z);
    int32_t b = wrap_mul(f2i_sat(cy), Z);
    return wrap_add(wrap_add(a, b), f2i_sat(cz));
}

/* Integer add into the grid, either plain (single thread) or atomic. */
static inline void grid_add(int32_t* p, int32_t v, int atomic) {
    if (atomic) {
        __atomic_fetch_add((uint32_t*)p, (uint32_t)v, __ATOMIC_RELAXED);
    } else {
        *p = wrap_add(*p, v);
    }
}

/* Quadratic B-spline weights, p2g_1.wgsl:30-34 (also p2g_2:36-40, g2p:33-37). */
static inline void bspline(const float* pos, float cell_idx[3], float w[3][3]) {
    for (int a = 0; a < 3; ++a) {
        float ci = floorf(pos[a]);
        float d = pos[a] - (ci + 0.5f);
        cell_idx[a] = ci;
        w[0][a] = (0.5f * (0.5f - d)) * (0.5f - d);
        w[1][a] = 0.75f - d * d;
        w[2][a] = (0.5f * (0.5f + d)) * (0.5f + d);
    }
}

typedef struct orc_box {
    int32_t Y, Z;        /* i32(init_box_size.y), i32(init_box_size.z) */
} orc_box;

static inline orc_box make_box(const float init_box[3]) {
    orc_box b;
    b.Y = f2i_sat(init_box[1]);
    b.Z = f2i_sat(init_box[2]);
    return b;
}

/* ------------------------------------------------------------------ */
/* kernels over index ranges                                           */
/* ------------------------------------------------------------------ */

/* clearGrid.wgsl:10-18 */
static void clear_range(int32_t* cells, int64_t c0, int64_t c1) {
    memset(cells + 4 * c0, 0, (size_t)(c1 - c0) * 16);
}

/* p2g_1.wgsl:24-65 */
static void p2g_1_range(const float* particles, int64_t i0, int64_t i1, int32_t* cells,
                        int64_t grid_count, orc_box box, float fm, int atomic,
                        int64_t* oob) {
    int64_t bad = 0;
    for (int64_t i = i0; i < i1; ++i) {
        const float* P = particles + 20 * i;
        const float pos[3] = {P[0], P[1], P[2]};
        const float v[3] = {P[4], P[5], P[6]};
        float C[3][3]; /* C[column][row] */
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) C[c][r] = P[8 + 4 * c + r];
        float ci[3], w[3][3];
        bspline(pos, ci, w);
        for (int gx = 0; gx < 3; ++gx)
            for (int gy = 0; gy < 3; ++gy)
                for (int gz = 0; gz < 3; ++gz) {
                    float weight = (w[gx][0] * w[gy][1]) * w[gz][2];
                    float cx = (ci[0] + (float)gx) - 1.0f;
                    float cy = (ci[1] + (float)gy) - 1.0f;
                    float cz = (ci[2] + (float)gz) - 1.0f;
                    float d[3] = {(cx + 0.5f) - pos[0], (cy + 0.5f) - pos[1],
                                  (cz + 0.5f) - pos[2]};
                    float Q[3];
                    for (int r = 0; r < 3; ++r)
                        Q[r] = (C[0][r] * d[0] + C[1][r] * d[1]) + C[2][r] * d[2];
                    float mass_contrib = weight * 1.0f;
                    float vel[3];
                    for (int r = 0; r < 3; ++r) vel[r] = mass_contrib * (v[r] + Q[r]);
                    int32_t idx = flat_index(cx, cy, cz, box.Y, box.Z);
                    if (idx < 0 || (int64_t)idx >= grid_count) { ++bad; continue; }
                    int32_t* cell = cells + 4 * (int64_t)idx;
                    grid_add(cell + 3, enc(mass_contrib, fm), atomic);
                    grid_add(cell + 0, enc(vel[0], fm), atomic);
                    grid_add(cell + 1, enc(vel[1], fm), atomic);
                    grid_add(cell + 2, enc(vel[2], fm), atomic);
                }
    }
    if (oob) *oob += bad;
}

/* Project-defined pow(x, 5.0). */
static inline float pow5(float x) {
    float x2 = x * x;
    float x4 = x2 * x2;
    return x4 * x;
}

/* p2g_2.wgsl:30-94 */
static void p2g_2_range(const float* particles, int64_t i0, int64_t i1, int32_t* cells,
                        int64_t grid_count, orc_box box, const orc_params* prm, int atomic,
                        int64_t* oob) {
    const float fm = prm->fixed_point_multiplier;
    int64_t bad = 0;
    for (int64_t i = i0; i < i1; ++i) {
        const float* P = particles + 20 * i;
        const float pos[3] = {P[0], P[1], P[2]};
        float C[3][3];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) C[c][r] = P[8 + 4 * c + r];
        float ci[3], w[3][3];
        bspline(pos, ci, w);

        float density = 0.0f;
        for (int gx = 0; gx < 3; ++gx)
            for (int gy = 0; gy < 3; ++gy)
                for (int gz = 0; gz < 3; ++gz) {
                    float weight = (w[gx][0] * w[gy][1]) * w[gz][2];
                    float cx = (ci[0] + (float)gx) - 1.0f;
                    float cy = (ci[1] + (float)gy) - 1.0f;
                    float cz = (ci[2] + (float)gz) - 1.0f;
                    int32_t idx = flat_index(cx, cy, cz, box.Y, box.Z);
                    int32_t m = 0;
                    if (idx < 0 || (int64_t)idx >= grid_count) ++bad;
                    else m = cells[4 * (int64_t)idx + 3];
                    density = density + dec(m, fm) * weight;
                }

        float volume = 1.0f / density;
        float pr = prm->stiffness * (pow5(density / prm->rest_density) - 1.0f);
        float pressure = wmax(-0.0f, pr);

        float T[3][3];
        float s0 = (-volume) * 4.0f;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) {
                float base = (c == r) ? -pressure : 0.0f;
                float strain = C[c][r] + C[r][c];
                float stress = base + prm->dynamic_viscosity * strain;
                T[c][r] = (s0 * stress) * prm->dt;
            }

        for (int gx = 0; gx < 3; ++gx)
            for (int gy = 0; gy < 3; ++gy)
                for (int gz = 0; gz < 3; ++gz) {
                    float weight = (w[gx][0] * w[gy][1]) * w[gz][2];
                    float cx = (ci[0] + (float)gx) - 1.0f;
                    float cy = (ci[1] + (float)gy) - 1.0f;
                    float cz = (ci[2] + (float)gz) - 1.0f;
                    float d[3] = {(cx + 0.5f) - pos[0], (cy + 0.5f) - pos[1],
                                  (cz + 0.5f) - pos[2]};
                    int32_t idx = flat_index(cx, cy, cz, box.Y, box.Z);
                    float M[3][3];
                    for (int c = 0; c < 3; ++c)
                        for (int r = 0; r < 3; ++r) M[c][r] = T[c][r] * weight;
                    float mom[3];
                    for (int r = 0; r < 3; ++r)
                        mom[r] = (M[0][r] * d[0] + M[1][r] * d[1]) + M[2][r] * d[2];
                    if (idx < 0 || (int64_t)idx >= grid_count) { ++bad; continue; }
                    int32_t* cell = cells + 4 * (int64_t)idx;
                    grid_add(cell + 0, enc(mom[0], fm), atomic);
                    grid_add(cell + 1, enc(mom[1], fm), atomic);
                    grid_add(cell + 2, enc(mom[2], fm), atomic);
                }
    }
    if (oob) *oob += bad;
}

/* updateGrid.wgsl:23-46 */
static void update_range(int32_t* cells, int64_t c0, int64_t c1, const float real_box[3],
                         orc_box box, const orc_params* prm) {
    const float fm = prm->fixed_point_multiplier;
    const float g0 = prm->gravity[0] * prm->dt;
    const float g1 = prm->gravity[1] * prm->dt;
    const float g2 = prm->gravity[2] * prm->dt;
    const int32_t hx = f2i_sat(ceilf(real_box[0]) - 3.0f);
    const int32_t hy = f2i_sat(ceilf(real_box[1]) - 3.0f);
    const int32_t hz = f2i_sat(ceilf(real_box[2]) - 3.0f);
    for (int64_t i = c0; i < c1; ++i) {
        int32_t* cell = cells + 4 * i;
        if (!(cell[3] > 0)) continue;
        float fv0 = dec(cell[0], fm), fv1 = dec(cell[1], fm), fv2 = dec(cell[2], fm);
        float m = dec(cell[3], fm);
        fv0 = fv0 / m;
        fv1 = fv1 / m;
        fv2 = fv2 / m;
        int32_t o0 = enc(prm->gravity[0] != 0.0f ? fv0 + g0 : fv0, fm);
        int32_t o1 = enc(prm->gravity[1] != 0.0f ? fv1 + g1 : fv1, fm);
        int32_t o2 = enc(prm->gravity[2] != 0.0f ? fv2 + g2 : fv2, fm);
        int32_t id = (int32_t)i;
        int32_t x = (box.Z != 0 && box.Y != 0) ? (id / box.Z) / box.Y : 0;
        int32_t y = (box.Z != 0 && box.Y != 0) ? (id / box.Z) % box.Y : 0;
        int32_t z = (box.Z != 0) ? id % box.Z : 0;
        if (x < 2 || x > hx) o0 = 0;
        if (y < 2 || y > hy) o1 = 0;
        if (z < 2 || z > hz) o2 = 0;
        cell[0] = o0;
        cell[1] = o1;
        cell[2] = o2;
    }
}

/* g2p.wgsl:26-92 */
static void g2p_range(float* particles, int64_t i0, int64_t i1, const int32_t* cells,
                      int64_t grid_count, const float real_box[3], orc_box box,
                      const orc_params* prm, int64_t* oob) {
    const float fm = prm->fixed_point_multiplier;
    const float dt = prm->dt;
    int64_t bad = 0;
    for (int64_t i = i0; i < i1; ++i) {
        float* P = particles + 20 * i;
        const float pos[3] = {P[0], P[1], P[2]};
        float v[3] = {0.0f, 0.0f, 0.0f};
        float ci[3], w[3][3];
        bspline(pos, ci, w);
        float B[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
        for (int gx = 0; gx < 3; ++gx)
            for (int gy = 0; gy < 3; ++gy)
                for (int gz = 0; gz < 3; ++gz) {
                    float weight = (w[gx][0] * w[gy][1]) * w[gz][2];
                    float cx = (ci[0] + (float)gx) - 1.0f;
                    float cy = (ci[1] + (float)gy) - 1.0f;
                    float cz = (ci[2] + (float)gz) - 1.0f;
                    float d[3] = {(cx + 0.5f) - pos[0], (cy + 0.5f) - pos[1],
                                  (cz + 0.5f) - pos[2]};
                    int32_t idx = flat_index(cx, cy, cz, box.Y, box.Z);
                    int32_t gv[3] = {0, 0, 0};
                    if (idx < 0 || (int64_t)idx >= grid_count) ++bad;
                    else {
                        const int32_t* cell = cells + 4 * (int64_t)idx;
                        gv[0] = cell[0];
                        gv[1] = cell[1];
                        gv[2] = cell[2];
                    }
                    float wv[3];
                    for (int r = 0; r < 3; ++r) wv[r] = dec(gv[r], fm) * weight;
                    for (int c = 0; c < 3; ++c)
                        for (int r = 0; r < 3; ++r) B[c][r] = B[c][r] + wv[r] * d[c];
                    for (int r = 0; r < 3; ++r) v[r] = v[r] + wv[r];
                }
        float np[3];
        for (int a = 0; a < 3; ++a) {
            float p = pos[a] + v[a] * dt;
            np[a] = wmin(wmax(p, 1.0f), real_box[a] - 2.0f);
        }
        for (int a = 0; a < 3; ++a) {
            float xn = np[a] + (v[a] * dt) * 3.0f;
            float wall_max = real_box[a] - 4.0f;
            if (xn < 3.0f) v[a] = v[a] + 0.3f * (3.0f - xn);
            if (xn > wall_max) v[a] = v[a] + 0.3f * (wall_max - xn);
        }
        P[0] = np[0];
        P[1] = np[1];
        P[2] = np[2];
        P[4] = v[0];
        P[5] = v[1];
        P[6] = v[2];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) P[8 + 4 * c + r] = B[c][r] * 4.0f;
    }
    if (oob) *oob += bad;
}

/* copyPosition.wgsl:15-21 */
static void copy_range(const float* particles, int64_t i0, int64_t i1, float* posvel) {
    for (int64_t i = i0; i < i1; ++i) {
        const float* P = particles + 20 * i;
        float* Q = posvel + 8 * i;
        Q[0] = P[0]; Q[1] = P[1]; Q[2] = P[2]; Q[3] = 0.0f;
        Q[4] = P[4]; Q[5] = P[5]; Q[6] = P[6]; Q[7] = 0.0f;
    }
}

/* ------------------------------------------------------------------ */
/* exported single-threaded kernels (one per WGSL entry point)         */
/* ------------------------------------------------------------------ */

void orc_default_params(orc_params* p) {
    p->stiffness = 3.0f;
    p->rest_density = 4.0f;
    p->dynamic_viscosity = 0.1f;
    p->dt = 0.2f;
    p->fixed_point_multiplier = 1e7f;
}

/* mls-mpm.ts:229: ceil(X) * ceil(Y) * ceil(Z) */
int64_t orc_grid_count(const float init_box[3]) {
    return (int64_t)ceil((double)init_box[0]) * (int64_t)ceil((double)init_box[1]) *
           (int64_t)ceil((double)init_box[2]);
}

void orc_clear_grid(int32_t* cells, int64_t grid_count) { clear_range(cells, 0, grid_count); }

int64_t orc_p2g_1(const float* particles, int64_t n, int32_t* cells, int64_t grid_count,
                  const float init_box[3], const orc_params* prm) {
    int64_t oob = 0;
    p2g_1_range(particles, 0, n, cells, grid_count, make_box(init_box),
                prm->fixed_point_multiplier, 0, &oob);
    return oob;
}

int64_t orc_p2g_2(const float* particles, int64_t n, int32_t* cells, int64_t grid_count,
                  const float init_box[3], const orc_params* prm) {
    int64_t oob = 0;
    p2g_2_range(particles, 0, n, cells, grid_count, make_box(init_box), prm, 0, &oob);
    return oob;
}

void orc_update_grid(int32_t* cells, int64_t grid_count, const float real_box[3],
                     const float init_box[3], const orc_params* prm) {
    update_range(cells, 0, grid_count, real_box, make_box(init_box), prm);
}

int64_t orc_g2p(float* particles, int64_t n, const int32_t* cells, int64_t grid_count,
                const float real_box[3], const float init_box[3], const orc_params* prm) {
    int64_t oob = 0;
    g2p_range(particles, 0, n, cells, grid_count, real_box, make_box(init_box), prm, &oob);
    return oob;
}

void orc_copy_position(const float* particles, int64_t n, float* posvel) {
    copy_range(particles, 0, n, posvel);
}

/* ------------------------------------------------------------------ */
/* execute: substeps x [clear, p2g_1, p2g_2, updateGrid, g2p, copy]    */
/* mls-mpm.ts:245-268, run on `nthreads` host threads                  */
/* ------------------------------------------------------------------ */

typedef struct exec_ctx {
    float* particles;
    int64_t n;
    int32_t* cells;
    int64_t grid_count;
    float real_box[3];
    orc_box box;
    orc_params prm;
    float* posvel;
    int substeps;
    int nthreads;
    pthread_barrier_t bar;
    int64_t oob[256];
} exec_ctx;

typedef struct exec_arg {
    exec_ctx* ctx;
    int tid;
} exec_arg;

static void split(int64_t n, int nt, int tid, int64_t* a, int64_t* b) {
    int64_t chunk = (n + nt - 1) / nt;
    *a = chunk * tid;
    *b = *a + chunk;
    if (*a > n) *a = n;
    if (*b > n) *b = n;
}

static inline void sync_all(exec_ctx* c) {
    if (c->nthreads > 1) pthread_barrier_wait(&c->bar);
}

static void* exec_worker(void* p) {
    exec_arg* arg = (exec_arg*)p;
    exec_ctx* c = arg->ctx;
    const int t = arg->tid, nt = c->nthreads;
    const int atomic = nt > 1;
    int64_t pa, pb, ca, cb;
    split(c->n, nt, t, &pa, &pb);
    split(c->grid_count, nt, t, &ca, &cb);
    int64_t oob = 0;
    for (int s = 0; s < c->substeps; ++s) {
        clear_range(c->cells, ca, cb);
        sync_all(c);
        p2g_1_range(c->particles, pa, pb, c->cells, c->grid_count, c->box,
                    c->prm.fixed_point_multiplier, atomic, &oob);
        sync_all(c);
        p2g_2_range(c->particles, pa, pb, c->cells, c->grid_count, c->box, &c->prm, atomic,
                    &oob);
        sync_all(c);
        update_range(c->cells, ca, cb, c->real_box, c->box, &c->prm);
        sync_all(c);
        g2p_range(c->particles, pa, pb, c->cells, c->grid_count, c->real_box, c->box, &c->prm,
                  &oob);
        if (c->posvel) copy_range(c->particles, pa, pb, c->posvel);
        sync_all(c);
    }
    c->oob[t] = oob;
    return NULL;
}

/*
 * Runs `substeps` substeps (the reference's execute() runs 2).  `posvel` may
 * be NULL.  Returns the number of out-of-range grid accesses, or -1 on a
 * thread error.  Results do not depend on `nthreads`: per-particle arithmetic
 * is independent and integer grid sums commute.
 */
int64_t orc_execute(float* particles, int64_t n, int32_t* cells, int64_t grid_count,
                    const float real_box[3], const float init_box[3], const orc_params* prm,
                    float* posvel, int substeps, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    exec_ctx* c = (exec_ctx*)calloc(1, sizeof(exec_ctx));
    if (!c) return -1;
    c->particles = particles;
    c->n = n;
    c->cells = cells;
    c->grid_count = grid_count;
    memcpy(c->real_box, real_box, sizeof(float) * 3);
    c->box = make_box(init_box);
    c->prm = *prm;
    c->posvel = posvel;
    c->substeps = substeps;
    c->nthreads = nthreads;
    int64_t total = 0;
    if (nthreads == 1) {
        exec_arg a = {c, 0};
        exec_worker(&a);
        total = c->oob[0];
        free(c);
        return total;
    }
    pthread_barrier_init(&c->bar, NULL, (unsigned)nthreads);
    pthread_t th[256];
    exec_arg args[256];
    int started = 0;
    for (int t = 0; t < nthreads; ++t) {
        args[t].ctx = c;
        args[t].tid = t;
        if (pthread_create(&th[t], NULL, exec_worker, &args[t]) != 0) break;
        ++started;
    }
    if (started != nthreads) {
        /* cannot make progress past the barrier with fewer threads */
        abort();
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    pthread_barrier_destroy(&c->bar);
    for (int t = 0; t < nthreads; ++t) total += c->oob[t];
    free(c);
    return total;
}

/* Exposed for tests of the conversion rules. */
int32_t orc_enc(float f, float fm) { return enc(f, fm); }
float orc_dec(int32_t i, float fm) { return dec(i, fm); }
