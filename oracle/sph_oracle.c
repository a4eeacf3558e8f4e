/*
 * sph_oracle.c -- CPU restatement of WebGPU-Ocean's SPH substep
 * (sph/sph.ts:325-355): grid build and reorder (sph/grid/*.wgsl), density
 * (sph/density.wgsl:58-100), force (sph/force.wgsl:64-128), integrate
 * (sph/integrate.wgsl:37-64) and copyPosition (sph/copyPosition.wgsl).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/ as the checker of the CUDA SPH
 * solver, never by the product.
 *
 * Pinned to the reference's own shaders: tests/golden/make_golden_sph.py
 * runs sph/grid/*.wgsl and sph/{density,force,integrate,copyPosition}.wgsl
 * (read as text) through the WGSL interpreter in the dispatch order of
 * SPHSimulator.execute, and this restatement reproduces those fixtures bit
 * for bit.  It follows the shaders operation for operation in f32 (build with
 * -ffp-contract=off), with the choices the library documents: neighbours
 * within a cell in ascending particle index (the reference's in-cell order
 * comes from atomic arrival; the fixtures take the legal schedule that gives
 * it), particles whose flat cell id is outside [0, gridCount) left out of the
 * grid, exactly n particles (no ghost threads), dot = (x*x + y*y) + z*z and
 * normalize(u) = u / sqrt(dot(u, u)).
 *
 * Particle records: 16 floats (64 bytes, sph.ts:13,205-211): position
 * [0..2], v [4..6], force [8..10], density [11], nearDensity [12].
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct so_env {
    int X, Y, Z;
    float cell, half[3], offset;
    float mass, kr, kr2, kr5, kr6, kr9, dt, stiffness, near_stiffness, rest_density, viscosity;
    float s_density, s_near, s_grad, s_near_grad, s_lap;
    int total;
} so_env;

/* sph.ts:58-86, 154-179 (JS doubles stored as f32) and the kernel scale
 * factors (density.wgsl:37-47, force.wgsl:37-56). */
static so_env make_env(void) {
    so_env e;
    memset(&e, 0, sizeof e);
    const double kr = 0.07, cell = 1.0 * kr, half = 2.0, len = 2.0 * half, sentinel = 4.0 * cell;
    const int grids = (int)ceil((len + sentinel) / cell);
    e.X = e.Y = e.Z = grids;
    e.cell = (float)cell;
    e.half[0] = e.half[1] = e.half[2] = (float)half;
    e.offset = (float)(sentinel / 2.0);
    e.mass = 1.0f;
    e.kr = (float)kr;
    e.kr2 = (float)pow(kr, 2);
    e.kr5 = (float)pow(kr, 5);
    e.kr6 = (float)pow(kr, 6);
    e.kr9 = (float)pow(kr, 9);
    e.dt = 0.006f;
    e.stiffness = 20.0f;
    e.near_stiffness = 1.0f;
    e.rest_density = 15000.0f;
    e.viscosity = 100.0f;
    const float pi = (float)3.1415926535;
    e.s_density = 315.0f / ((float)(64.0 * 3.1415926535) * e.kr9);
    e.s_near = 15.0f / (pi * e.kr6);
    e.s_grad = 45.0f / (pi * e.kr6);
    e.s_near_grad = 45.0f / (pi * e.kr5);
    e.s_lap = 45.0f / (pi * e.kr6);
    e.total = e.X * e.Y * e.Z;
    return e;
}

static int f2i(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int)(-2147483647 - 1);
    return (int)x;
}

static void cell_pos(const so_env* e, const float* p, int* xi, int* yi, int* zi) {
    *xi = f2i(floorf(((p[0] + e->half[0]) + e->offset) / e->cell));
    *yi = f2i(floorf(((p[1] + e->half[1]) + e->offset) / e->cell));
    *zi = f2i(floorf(((p[2] + e->half[2]) + e->offset) / e->cell));
}

static int cell_number(const so_env* e, int xi, int yi, int zi) {
    return (int)((uint32_t)xi + (uint32_t)yi * (uint32_t)e->X +
                 (uint32_t)zi * (uint32_t)e->X * (uint32_t)e->Y);
}

static int in_grid(const so_env* e, int x, int y, int z) {
    return x < e->X && 0 <= x && y < e->Y && 0 <= y && z < e->Z && 0 <= z;
}

static int imax(int a, int b) { return a > b ? a : b; }
static int imin(int a, int b) { return a < b ? a : b; }

/* Runs `substeps` substeps on n records (16 floats each) in place; writes
 * posvel (n x 8 floats) when non-null.  real_half: changeBoxSize's half
 * sizes.  Returns 0, or -1 on allocation failure. */
int so_execute(float* rec, int64_t n, const float real_half[3], int substeps, float* posvel) {
    so_env e = make_env();
    const so_env* E = &e;
    uint32_t* count = (uint32_t*)malloc(4 * ((size_t)e.total + 1));
    uint32_t* start = (uint32_t*)malloc(4 * ((size_t)e.total + 1));
    int* cell_of = (int*)malloc(4 * (size_t)(n > 0 ? n : 1));
    uint32_t* order = (uint32_t*)malloc(4 * (size_t)(n > 0 ? n : 1));
    float* sp = (float*)malloc(sizeof(float) * 8 * (size_t)(n > 0 ? n : 1)); /* x y z dens vx vy vz near */
    if (!count || !start || !cell_of || !order || !sp) {
        free(count); free(start); free(cell_of); free(order); free(sp);
        return -1;
    }
    for (int sub = 0; sub < substeps; ++sub) {
        /* grid clear + build; densities reset */
        memset(count, 0, 4 * ((size_t)e.total + 1));
        for (int64_t i = 0; i < n; ++i) {
            float* r = rec + 16 * i;
            int xi, yi, zi;
            cell_pos(E, r, &xi, &yi, &zi);
            const int c = cell_number(E, xi, yi, zi);
            const int in = c >= 0 && c < e.total;
            cell_of[i] = in ? c : -1;
            if (in) count[c]++;
            r[11] = 0.0f;
            r[12] = 0.0f;
            if (!in) r[8] = r[9] = r[10] = 0.0f;
        }
        /* exclusive prefix sum */
        uint32_t run = 0;
        for (int c = 0; c <= e.total; ++c) {
            start[c] = run;
            if (c < e.total) run += count[c];
        }
        /* reorder: cells in order, particles ascending within a cell */
        memset(count, 0, 4 * ((size_t)e.total + 1));
        for (int64_t i = 0; i < n; ++i) {
            const int c = cell_of[i];
            if (c >= 0) order[start[c] + count[c]++] = (uint32_t)i;
        }
        const uint32_t nb = start[e.total];
        for (uint32_t s = 0; s < nb; ++s) {
            const float* r = rec + 16 * (size_t)order[s];
            float* q = sp + 8 * (size_t)s;
            q[0] = r[0]; q[1] = r[1]; q[2] = r[2]; q[3] = 0.0f;
            q[4] = r[4]; q[5] = r[5]; q[6] = r[6]; q[7] = 0.0f;
        }
        /* density */
        for (uint32_t s = 0; s < nb; ++s) {
            const float* pi = sp + 8 * (size_t)s;
            int vx, vy, vz;
            cell_pos(E, pi, &vx, &vy, &vz);
            float dens = 0.0f, near = 0.0f;
            if (in_grid(E, vx, vy, vz)) {
                for (int dz = imax(-1, -vz); dz <= imin(1, e.Z - vz - 1); ++dz)
                    for (int dy = imax(-1, -vy); dy <= imin(1, e.Y - vy - 1); ++dy) {
                        const int dxmin = imax(-1, -vx), dxmax = imin(1, e.X - vx - 1);
                        const int c0 = cell_number(E, vx + dxmin, vy + dy, vz + dz);
                        const int c1 = cell_number(E, vx + dxmax, vy + dy, vz + dz);
                        for (uint32_t j = start[c0]; j < start[c1 + 1]; ++j) {
                            const float* pj = sp + 8 * (size_t)j;
                            const float dx = pi[0] - pj[0], dyv = pi[1] - pj[1], dzv = pi[2] - pj[2];
                            const float r2 = (dx * dx + dyv * dyv) + dzv * dzv;
                            if (r2 < e.kr2) {
                                const float r = sqrtf(r2);
                                const float dd = e.kr2 - r * r;
                                dens = dens + e.mass * (((e.s_density * dd) * dd) * dd);
                                const float d = e.kr - r;
                                near = near + e.mass * (((e.s_near * d) * d) * d);
                            }
                        }
                    }
            }
            float* r = rec + 16 * (size_t)order[s];
            r[11] = dens;
            r[12] = near;
            sp[8 * (size_t)s + 3] = dens;
            sp[8 * (size_t)s + 7] = near;
        }
        /* force */
        for (uint32_t s = 0; s < nb; ++s) {
            const float* pi = sp + 8 * (size_t)s;
            const float dens_i = pi[3], near_i = pi[7];
            float fp[3] = {0, 0, 0}, fv[3] = {0, 0, 0};
            int vx, vy, vz;
            cell_pos(E, pi, &vx, &vy, &vz);
            if (in_grid(E, vx, vy, vz)) {
                for (int dz = imax(-1, -vz); dz <= imin(1, e.Z - vz - 1); ++dz)
                    for (int dy = imax(-1, -vy); dy <= imin(1, e.Y - vy - 1); ++dy) {
                        const int dxmin = imax(-1, -vx), dxmax = imin(1, e.X - vx - 1);
                        const int c0 = cell_number(E, vx + dxmin, vy + dy, vz + dz);
                        const int c1 = cell_number(E, vx + dxmax, vy + dy, vz + dz);
                        for (uint32_t j = start[c0]; j < start[c1 + 1]; ++j) {
                            const float* pj = sp + 8 * (size_t)j;
                            const float dens_j = pj[3], near_j = pj[7];
                            const float dx = pi[0] - pj[0], dyv = pi[1] - pj[1], dzv = pi[2] - pj[2];
                            const float r2 = (dx * dx + dyv * dyv) + dzv * dzv;
                            if (dens_j == 0.0f || near_j == 0.0f) continue;
                            if (r2 < e.kr2 && 0.0f < r2) {
                                const float r = sqrtf(r2);
                                const float p_i = e.stiffness * (dens_i - e.rest_density);
                                const float p_j = e.stiffness * (dens_j - e.rest_density);
                                const float np_i = e.near_stiffness * near_i;
                                const float np_j = e.near_stiffness * near_j;
                                const float spr = (p_i + p_j) / 2.0f;
                                const float nsp = (np_i + np_j) / 2.0f;
                                const float ux = pj[0] - pi[0], uy = pj[1] - pi[1], uz = pj[2] - pi[2];
                                const float len = sqrtf((ux * ux + uy * uy) + uz * uz);
                                const float dir[3] = {ux / len, uy / len, uz / len};
                                const float d = e.kr - r;
                                const float g = (e.s_grad * d) * d, ng = (e.s_near_grad * d) * d;
                                const float a = -e.mass * spr, an = -e.mass * nsp;
                                const float lap = e.s_lap * d;
                                const float rel[3] = {pj[4] - pi[4], pj[5] - pi[5], pj[6] - pi[6]};
                                for (int c = 0; c < 3; ++c) {
                                    fp[c] = fp[c] + ((a * dir[c]) * g) / dens_j;
                                    fp[c] = fp[c] + ((an * dir[c]) * ng) / near_j;
                                    fv[c] = fv[c] + ((e.mass * rel[c]) * lap) / dens_j;
                                }
                            }
                        }
                    }
            }
            const float grv[3] = {dens_i * 0.0f, dens_i * -9.8f, dens_i * 0.0f};
            float* r = rec + 16 * (size_t)order[s];
            for (int c = 0; c < 3; ++c) r[8 + c] = (fp[c] + fv[c] * e.viscosity) + grv[c];
        }
        /* integrate + copyPosition */
        for (int64_t i = 0; i < n; ++i) {
            float* r = rec + 16 * i;
            const float dens = r[11];
            if (dens != 0.0f) {
                float a[3] = {r[8] / dens, r[9] / dens, r[10] / dens};
                const float ws = 8000.0f;
                float plus[3][3], minus[3][3];
                for (int ax = 0; ax < 3; ++ax) {
                    const float pd = fminf(real_half[ax] - r[ax], 0.0f);
                    const float md = fminf(real_half[ax] + r[ax], 0.0f);
                    for (int c = 0; c < 3; ++c) {
                        plus[ax][c] = ((c == ax ? 1.0f : 0.0f) * ws) * pd;
                        minus[ax][c] = ((c == ax ? -1.0f : 0.0f) * ws) * md;
                    }
                }
                for (int c = 0; c < 3; ++c) {
                    const float xf = plus[0][c] + minus[0][c];
                    const float yf = plus[1][c] + minus[1][c];
                    const float zf = plus[2][c] + minus[2][c];
                    a[c] = a[c] + ((xf + yf) + zf);
                }
                for (int c = 0; c < 3; ++c) r[4 + c] = r[4 + c] + e.dt * a[c];
                for (int c = 0; c < 3; ++c) r[c] = r[c] + e.dt * r[4 + c];
            }
            if (posvel) {
                float* q = posvel + 8 * i;
                q[0] = r[0]; q[1] = r[1]; q[2] = r[2]; q[3] = 0.0f;
                q[4] = r[4]; q[5] = r[5]; q[6] = r[6]; q[7] = 0.0f;
            }
        }
    }
    free(count); free(start); free(cell_of); free(order); free(sp);
    return 0;
}

int so_grid_count(void) { return make_env().total; }
