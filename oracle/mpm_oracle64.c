/*
 * mpm_oracle64.c -- FP64 restatement of the MLS-MPM substep as a continuous
 * model, for finite-difference checks of the derivative (adjoint) path.
 *
 * TEST INFRASTRUCTURE ONLY, like mpm_oracle.c: loaded by tests/ as the
 * checker, never by the product.
 *
 * Same stages, stencils, flat indices (with the reference's aliasing),
 * boundary rules and branch structure as mpm_oracle.c (which follows
 * mls-mpm/p2g_1.wgsl:24-65, p2g_2.wgsl:30-94, updateGrid.wgsl:23-46,
 * g2p.wgsl:26-92), but in double precision and without the fixed-point
 * grid: the grid holds double sums, so encode/decode are the identity.  This
 * is the function whose derivative the library's adjoint computes.
 *
 * State layout: 15 doubles per particle: x[0..2], v[3..5], C[6..14] with
 * C[c][r] at 6 + 3c + r (columns, as the 80-byte record stores them).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct orc64_params {
    double stiffness;
    double rest_density;
    double dynamic_viscosity;
    double dt;
    double gravity[3];
    double init_box[3];
    double real_box[3];
} orc64_params;

static int32_t d2i_sat(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return (int32_t)x;
}

static int32_t flat64(double cx, double cy, double cz, int32_t Y, int32_t Z) {
    uint32_t a = (uint32_t)d2i_sat(cx) * (uint32_t)Y * (uint32_t)Z;
    uint32_t b = (uint32_t)d2i_sat(cy) * (uint32_t)Z;
    return (int32_t)(a + b + (uint32_t)d2i_sat(cz));
}

static void weights64(const double* x, double ci[3], double w[3][3]) {
    for (int a = 0; a < 3; ++a) {
        ci[a] = floor(x[a]);
        const double d = x[a] - (ci[a] + 0.5);
        w[a][0] = 0.5 * (0.5 - d) * (0.5 - d);
        w[a][1] = 0.75 - d * d;
        w[a][2] = 0.5 * (0.5 + d) * (0.5 + d);
    }
}

int64_t orc64_grid_count(const orc64_params* p) {
    return (int64_t)ceil(p->init_box[0]) * (int64_t)ceil(p->init_box[1]) *
           (int64_t)ceil(p->init_box[2]);
}

/* One substep on state (n x 15 doubles) in place; the grid g (grid_count x 4
 * doubles, caller-owned) is left as updateGrid leaves it: per touched cell
 * the velocity (or, where the mass is not positive, the raw momentum) and
 * the mass.  Adds the number of stencil accesses outside the grid to *bad. */
void orc64_substep(double* state, int64_t n, const orc64_params* p, double* g, int64_t* bad_out) {
    const int64_t gc = orc64_grid_count(p);
    const int32_t Y = d2i_sat(p->init_box[1]), Z = d2i_sat(p->init_box[2]);
    int64_t bad = 0;
    {
        memset(g, 0, sizeof(double) * 4 * (size_t)gc);
        /* p2g_1 */
        for (int64_t i = 0; i < n; ++i) {
            const double* P = state + 15 * i;
            double ci[3], w[3][3];
            weights64(P, ci, w);
            for (int gx = 0; gx < 3; ++gx)
                for (int gy = 0; gy < 3; ++gy)
                    for (int gz = 0; gz < 3; ++gz) {
                        const double wt = w[0][gx] * w[1][gy] * w[2][gz];
                        const double c[3] = {ci[0] + gx - 1.0, ci[1] + gy - 1.0, ci[2] + gz - 1.0};
                        double d[3];
                        for (int a = 0; a < 3; ++a) d[a] = (c[a] + 0.5) - P[a];
                        const int32_t idx = flat64(c[0], c[1], c[2], Y, Z);
                        if (idx < 0 || idx >= gc) { ++bad; continue; }
                        double* cell = g + 4 * (int64_t)idx;
                        for (int r = 0; r < 3; ++r) {
                            const double q = P[6 + r] * d[0] + P[9 + r] * d[1] + P[12 + r] * d[2];
                            cell[r] += wt * (P[3 + r] + q);
                        }
                        cell[3] += wt;
                    }
        }
        /* p2g_2 */
        for (int64_t i = 0; i < n; ++i) {
            const double* P = state + 15 * i;
            double ci[3], w[3][3];
            weights64(P, ci, w);
            double rho = 0.0;
            for (int gx = 0; gx < 3; ++gx)
                for (int gy = 0; gy < 3; ++gy)
                    for (int gz = 0; gz < 3; ++gz) {
                        const double wt = w[0][gx] * w[1][gy] * w[2][gz];
                        const int32_t idx = flat64(ci[0] + gx - 1.0, ci[1] + gy - 1.0,
                                                   ci[2] + gz - 1.0, Y, Z);
                        if (idx < 0 || idx >= gc) { ++bad; continue; }
                        rho += g[4 * (int64_t)idx + 3] * wt;
                    }
            const double V = 1.0 / rho;
            const double rr = rho / p->rest_density;
            const double pterm = p->stiffness * (rr * rr * rr * rr * rr - 1.0);
            const double pres = pterm > 0.0 ? pterm : 0.0;
            double T[3][3]; /* [row][col] */
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    const double strain = P[6 + 3 * b + a] + P[6 + 3 * a + b];
                    const double sig = (a == b ? -pres : 0.0) + p->dynamic_viscosity * strain;
                    T[a][b] = -V * 4.0 * sig * p->dt;
                }
            for (int gx = 0; gx < 3; ++gx)
                for (int gy = 0; gy < 3; ++gy)
                    for (int gz = 0; gz < 3; ++gz) {
                        const double wt = w[0][gx] * w[1][gy] * w[2][gz];
                        const double c[3] = {ci[0] + gx - 1.0, ci[1] + gy - 1.0, ci[2] + gz - 1.0};
                        double d[3];
                        for (int a = 0; a < 3; ++a) d[a] = (c[a] + 0.5) - P[a];
                        const int32_t idx = flat64(c[0], c[1], c[2], Y, Z);
                        if (idx < 0 || idx >= gc) { ++bad; continue; }
                        double* cell = g + 4 * (int64_t)idx;
                        for (int r = 0; r < 3; ++r)
                            cell[r] += wt * (T[r][0] * d[0] + T[r][1] * d[1] + T[r][2] * d[2]);
                    }
        }
        /* updateGrid */
        int32_t hi[3];
        for (int a = 0; a < 3; ++a) hi[a] = d2i_sat(ceil(p->real_box[a]) - 3.0);
        for (int64_t j = 0; j < gc; ++j) {
            double* cell = g + 4 * j;
            if (!(cell[3] > 0.0)) continue;
            const int32_t id = (int32_t)j;
            const int32_t xyz[3] = {(id / Z) / Y, (id / Z) % Y, id % Z};
            for (int a = 0; a < 3; ++a) {
                double v = cell[a] / cell[3] + p->gravity[a] * p->dt;
                if (xyz[a] < 2 || xyz[a] > hi[a]) v = 0.0;
                cell[a] = v;
            }
        }
        /* g2p */
        for (int64_t i = 0; i < n; ++i) {
            double* P = state + 15 * i;
            double ci[3], w[3][3];
            weights64(P, ci, w);
            double v[3] = {0.0, 0.0, 0.0}, B[3][3] = {{0}}; /* B[c][r] */
            for (int gx = 0; gx < 3; ++gx)
                for (int gy = 0; gy < 3; ++gy)
                    for (int gz = 0; gz < 3; ++gz) {
                        const double wt = w[0][gx] * w[1][gy] * w[2][gz];
                        const double c[3] = {ci[0] + gx - 1.0, ci[1] + gy - 1.0, ci[2] + gz - 1.0};
                        double d[3];
                        for (int a = 0; a < 3; ++a) d[a] = (c[a] + 0.5) - P[a];
                        const int32_t idx = flat64(c[0], c[1], c[2], Y, Z);
                        double gv[3] = {0.0, 0.0, 0.0};
                        if (idx < 0 || idx >= gc) ++bad;
                        else for (int a = 0; a < 3; ++a) gv[a] = g[4 * (int64_t)idx + a];
                        for (int r = 0; r < 3; ++r) {
                            const double wv = gv[r] * wt;
                            for (int cc = 0; cc < 3; ++cc) B[cc][r] += wv * d[cc];
                            v[r] += wv;
                        }
                    }
            for (int cc = 0; cc < 3; ++cc)
                for (int r = 0; r < 3; ++r) P[6 + 3 * cc + r] = B[cc][r] * 4.0;
            for (int a = 0; a < 3; ++a) {
                double x = P[a] + v[a] * p->dt;
                const double lo = 1.0, hw = p->real_box[a] - 2.0;
                x = x < lo ? lo : x;
                x = x > hw ? hw : x;
                P[a] = x;
            }
            for (int a = 0; a < 3; ++a) {
                const double xn = P[a] + v[a] * p->dt * 3.0;
                const double wmax = p->real_box[a] - 4.0;
                double va = v[a];
                if (xn < 3.0) va += 0.3 * (3.0 - xn);
                if (xn > wmax) va += 0.3 * (wmax - xn);
                P[3 + a] = va;
            }
        }
    }
    *bad_out += bad;
}

static void weights32(const float* x, float ci[3], float w[3][3]) {
    for (int a = 0; a < 3; ++a) {
        ci[a] = floorf(x[a]);
        const float d = x[a] - (ci[a] + 0.5f);
        w[a][0] = 0.5f * (0.5f - d) * (0.5f - d);
        w[a][1] = 0.75f - d * d;
        w[a][2] = 0.5f * (0.5f + d) * (0.5f + d);
    }
}

/* The same substep with every value and grid sum in f32 (state n x 15
 * floats, grid grid_count x 4 floats): the continuous model integrated in
 * single precision, as the library's f32 tape integrates it (there the
 * grid sums arrive in atomic order). */
/* One substep on state (n x 15 floats) in place; the grid g (grid_count x 4
 * floats, caller-owned) is left as updateGrid leaves it: per touched cell
 * the velocity (or, where the mass is not positive, the raw momentum) and
 * the mass.  Adds the number of stencil accesses outside the grid to *bad. */
void orc32_substep(float* state, int64_t n, const orc64_params* p, float* g, int64_t* bad_out) {
    const int64_t gc = orc64_grid_count(p);
    const int32_t Y = d2i_sat(p->init_box[1]), Z = d2i_sat(p->init_box[2]);
    int64_t bad = 0;
    {
        memset(g, 0, sizeof(float) * 4 * (size_t)gc);
        /* p2g_1 */
        for (int64_t i = 0; i < n; ++i) {
            const float* P = state + 15 * i;
            float ci[3], w[3][3];
            weights32(P, ci, w);
            for (int gx = 0; gx < 3; ++gx)
                for (int gy = 0; gy < 3; ++gy)
                    for (int gz = 0; gz < 3; ++gz) {
                        const float wt = w[0][gx] * w[1][gy] * w[2][gz];
                        const float c[3] = {ci[0] + gx - 1.0f, ci[1] + gy - 1.0f, ci[2] + gz - 1.0f};
                        float d[3];
                        for (int a = 0; a < 3; ++a) d[a] = (c[a] + 0.5f) - P[a];
                        const int32_t idx = flat64(c[0], c[1], c[2], Y, Z);
                        if (idx < 0 || idx >= gc) { ++bad; continue; }
                        float* cell = g + 4 * (int64_t)idx;
                        for (int r = 0; r < 3; ++r) {
                            const float q = P[6 + r] * d[0] + P[9 + r] * d[1] + P[12 + r] * d[2];
                            cell[r] += wt * (P[3 + r] + q);
                        }
                        cell[3] += wt;
                    }
        }
        /* p2g_2 */
        for (int64_t i = 0; i < n; ++i) {
            const float* P = state + 15 * i;
            float ci[3], w[3][3];
            weights32(P, ci, w);
            float rho = 0.0f;
            for (int gx = 0; gx < 3; ++gx)
                for (int gy = 0; gy < 3; ++gy)
                    for (int gz = 0; gz < 3; ++gz) {
                        const float wt = w[0][gx] * w[1][gy] * w[2][gz];
                        const int32_t idx = flat64(ci[0] + gx - 1.0f, ci[1] + gy - 1.0f,
                                                   ci[2] + gz - 1.0f, Y, Z);
                        if (idx < 0 || idx >= gc) { ++bad; continue; }
                        rho += g[4 * (int64_t)idx + 3] * wt;
                    }
            const float V = 1.0f / rho;
            const float rr = rho / (float)p->rest_density;
            const float pterm = (float)p->stiffness * (rr * rr * rr * rr * rr - 1.0f);
            const float pres = pterm > 0.0f ? pterm : 0.0f;
            float T[3][3]; /* [row][col] */
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    const float strain = P[6 + 3 * b + a] + P[6 + 3 * a + b];
                    const float sig = (a == b ? -pres : 0.0f) + (float)p->dynamic_viscosity * strain;
                    T[a][b] = -V * 4.0f * sig * (float)p->dt;
                }
            for (int gx = 0; gx < 3; ++gx)
                for (int gy = 0; gy < 3; ++gy)
                    for (int gz = 0; gz < 3; ++gz) {
                        const float wt = w[0][gx] * w[1][gy] * w[2][gz];
                        const float c[3] = {ci[0] + gx - 1.0f, ci[1] + gy - 1.0f, ci[2] + gz - 1.0f};
                        float d[3];
                        for (int a = 0; a < 3; ++a) d[a] = (c[a] + 0.5f) - P[a];
                        const int32_t idx = flat64(c[0], c[1], c[2], Y, Z);
                        if (idx < 0 || idx >= gc) { ++bad; continue; }
                        float* cell = g + 4 * (int64_t)idx;
                        for (int r = 0; r < 3; ++r)
                            cell[r] += wt * (T[r][0] * d[0] + T[r][1] * d[1] + T[r][2] * d[2]);
                    }
        }
        /* updateGrid */
        int32_t hi[3];
        for (int a = 0; a < 3; ++a) hi[a] = d2i_sat(ceil(p->real_box[a]) - 3.0);
        for (int64_t j = 0; j < gc; ++j) {
            float* cell = g + 4 * j;
            if (!(cell[3] > 0.0f)) continue;
            const int32_t id = (int32_t)j;
            const int32_t xyz[3] = {(id / Z) / Y, (id / Z) % Y, id % Z};
            for (int a = 0; a < 3; ++a) {
                float v = cell[a] / cell[3] + (float)p->gravity[a] * (float)p->dt;
                if (xyz[a] < 2 || xyz[a] > hi[a]) v = 0.0f;
                cell[a] = v;
            }
        }
        /* g2p */
        for (int64_t i = 0; i < n; ++i) {
            float* P = state + 15 * i;
            float ci[3], w[3][3];
            weights32(P, ci, w);
            float v[3] = {0.0f, 0.0f, 0.0f}, B[3][3] = {{0}}; /* B[c][r] */
            for (int gx = 0; gx < 3; ++gx)
                for (int gy = 0; gy < 3; ++gy)
                    for (int gz = 0; gz < 3; ++gz) {
                        const float wt = w[0][gx] * w[1][gy] * w[2][gz];
                        const float c[3] = {ci[0] + gx - 1.0f, ci[1] + gy - 1.0f, ci[2] + gz - 1.0f};
                        float d[3];
                        for (int a = 0; a < 3; ++a) d[a] = (c[a] + 0.5f) - P[a];
                        const int32_t idx = flat64(c[0], c[1], c[2], Y, Z);
                        float gv[3] = {0.0f, 0.0f, 0.0f};
                        if (idx < 0 || idx >= gc) ++bad;
                        else for (int a = 0; a < 3; ++a) gv[a] = g[4 * (int64_t)idx + a];
                        for (int r = 0; r < 3; ++r) {
                            const float wv = gv[r] * wt;
                            for (int cc = 0; cc < 3; ++cc) B[cc][r] += wv * d[cc];
                            v[r] += wv;
                        }
                    }
            for (int cc = 0; cc < 3; ++cc)
                for (int r = 0; r < 3; ++r) P[6 + 3 * cc + r] = B[cc][r] * 4.0f;
            for (int a = 0; a < 3; ++a) {
                float x = P[a] + v[a] * (float)p->dt;
                const float lo = 1.0f, hw = (float)p->real_box[a] - 2.0f;
                x = x < lo ? lo : x;
                x = x > hw ? hw : x;
                P[a] = x;
            }
            for (int a = 0; a < 3; ++a) {
                const float xn = P[a] + v[a] * (float)p->dt * 3.0f;
                const float wmax = (float)p->real_box[a] - 4.0f;
                float va = v[a];
                if (xn < 3.0f) va += 0.3f * (3.0f - xn);
                if (xn > wmax) va += 0.3f * (wmax - xn);
                P[3 + a] = va;
            }
        }
    }
    *bad_out += bad;
}

/* Runs `substeps` substeps on state (n x 15 doubles) in place.  Returns the
 * number of stencil accesses outside the grid, or -1 on allocation failure. */
int64_t orc64_run(double* state, int64_t n, const orc64_params* p, int substeps) {
    const int64_t gc = orc64_grid_count(p);
    double* g = (double*)malloc(sizeof(double) * 4 * (size_t)(gc > 0 ? gc : 1));
    if (!g) return -1;
    int64_t bad = 0;
    for (int sub = 0; sub < substeps; ++sub) orc64_substep(state, n, p, g, &bad);
    free(g);
    return bad;
}
