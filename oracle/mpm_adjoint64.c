/*
 * mpm_adjoint64.c -- FP64 tape adjoint of the continuous MLS-MPM substep
 * (mpm_oracle64.c), on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY, like the other oracles: loaded by tests/ as the
 * checker of the library's backward kernels, never by the product.
 *
 * The forward is orc64_substep (the stages of mls-mpm/p2g_1.wgsl:24-65,
 * p2g_2.wgsl:30-94, updateGrid.wgsl:23-46 and g2p.wgsl:26-92 in double
 * precision with double grid sums).  Its reverse pass, for one substep with
 * input state S, updated grid G and output adjoint A' (all in the 15-double
 * layout x, v, C by columns):
 *
 *   g2p      v' = sum_i w_i u_i,  B[c][r] = sum_i w_i u_i[r] d_i[c],  C' = 4B,
 *            x' = clamp(x + dt v'),  x_n = x' + 3 dt v',  v'' = v' + walls(x_n)
 *            -> u_bar_j += w_i (v'_bar + B_bar d_i),  x_bar from w_i and d_i
 *   update   u_j = P_j / m_j + g dt (0 on the boundary band)
 *            -> P_bar_j = u_bar_j / m_j,  m_bar_j = -sum_a u_bar_j[a] (u_j[a] - g_a dt) / m_j
 *   p2g_2    rho = sum_i m_j w_i,  T = -4 dt sigma / rho,
 *            sigma = -max(k((rho/rho0)^5 - 1), 0) I + mu (C + C^T),
 *            P_j += w_i T d_i
 *            -> T_bar, rho_bar, k_bar, mu_bar, C_bar; m_bar_j += rho_bar w_i
 *   p2g_1    m_j += w_i,  P_j += w_i (v + C d_i)
 *            -> v_bar, C_bar, x_bar (gathers of P_bar_j and m_bar_j)
 *
 * with d_i = (c_i + 0.5) - x, dd_i/dx = -I, and w_i the product of the three
 * quadratic B-spline factors (their derivatives: -(0.5 - d), -2d, 0.5 + d).
 * floor(x) is piecewise constant; the clamp and the wall pushes take the
 * branch the forward took.  Stencil cells outside the grid carry nothing.
 *
 * orc64_backward runs the whole trajectory: a forward keeping the state
 * every `every` substeps, then per segment, last first, a recompute that
 * tapes each substep's input state and updated grid, and the reverse pass
 * of each of its substeps, adding the seeds given at that substep.
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

int64_t orc64_grid_count(const orc64_params* p);
void orc64_substep(double* state, int64_t n, const orc64_params* p, double* g, int64_t* bad);
void orc32_substep(float* state, int64_t n, const orc64_params* p, float* g, int64_t* bad);


/* One forward substep of the tape: in FP64, or (f32 != 0) in f32 through the
 * float buffers sf (n x 15) and gf (grid), the result widened to double. */
static void tape_substep(double* state, int64_t n, const orc64_params* p, double* g, int64_t* bad,
                         int f32, float* sf, float* gf) {
    if (!f32) {
        orc64_substep(state, n, p, g, bad);
        return;
    }
    const int64_t gc = orc64_grid_count(p);
    for (int64_t q = 0; q < 15 * n; ++q) sf[q] = (float)state[q];
    orc32_substep(sf, n, p, gf, bad);
    for (int64_t q = 0; q < 15 * n; ++q) state[q] = (double)sf[q];
    for (int64_t q = 0; q < 4 * gc; ++q) g[q] = (double)gf[q];
}

static int32_t sat_i32(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return (int32_t)x;
}

static int32_t flat_idx(double cx, double cy, double cz, int32_t Y, int32_t Z) {
    uint32_t a = (uint32_t)sat_i32(cx) * (uint32_t)Y * (uint32_t)Z;
    uint32_t b = (uint32_t)sat_i32(cy) * (uint32_t)Z;
    return (int32_t)(a + b + (uint32_t)sat_i32(cz));
}

/* Per stencil node: weight, its gradient, dist and the cell's flat index
 * (-1 outside the grid). */
typedef struct {
    double w, gw[3], d[3];
    int32_t idx;
} node64;

static void stencil64(const double* x, const orc64_params* p, int64_t gc, node64 nd[27]) {
    const int32_t Y = sat_i32(p->init_box[1]), Z = sat_i32(p->init_box[2]);
    double ci[3], w[3][3], dw[3][3];
    for (int a = 0; a < 3; ++a) {
        ci[a] = floor(x[a]);
        const double d = x[a] - (ci[a] + 0.5);
        w[a][0] = 0.5 * (0.5 - d) * (0.5 - d);
        w[a][1] = 0.75 - d * d;
        w[a][2] = 0.5 * (0.5 + d) * (0.5 + d);
        dw[a][0] = -(0.5 - d);
        dw[a][1] = -2.0 * d;
        dw[a][2] = 0.5 + d;
    }
    int i = 0;
    for (int gx = 0; gx < 3; ++gx)
        for (int gy = 0; gy < 3; ++gy)
            for (int gz = 0; gz < 3; ++gz, ++i) {
                node64* q = &nd[i];
                q->w = w[0][gx] * w[1][gy] * w[2][gz];
                q->gw[0] = dw[0][gx] * w[1][gy] * w[2][gz];
                q->gw[1] = w[0][gx] * dw[1][gy] * w[2][gz];
                q->gw[2] = w[0][gx] * w[1][gy] * dw[2][gz];
                const double c[3] = {ci[0] + gx - 1.0, ci[1] + gy - 1.0, ci[2] + gz - 1.0};
                for (int a = 0; a < 3; ++a) q->d[a] = (c[a] + 0.5) - x[a];
                const int32_t idx = flat_idx(c[0], c[1], c[2], Y, Z);
                q->idx = (idx < 0 || idx >= gc) ? -1 : idx;
            }
}

/* The reverse pass of one substep.  S: input state (n x 15); G: its updated
 * grid (gc x 4); Aout: adjoint of the output state; Ain: receives the
 * adjoint of S (overwritten); gadj: scratch (gc x 4: u_bar / P_bar xyz and
 * m_bar); pgrad[0..1] += (k_bar, mu_bar). */
void orc64_substep_adjoint(const double* S, const double* G, const double* Aout, double* Ain,
                           int64_t n, const orc64_params* p, double* gadj, double* pgrad) {
    const int64_t gc = orc64_grid_count(p);
    const int32_t Y = sat_i32(p->init_box[1]), Z = sat_i32(p->init_box[2]);
    const double dt = p->dt;
    memset(gadj, 0, sizeof(double) * 4 * (size_t)gc);
    memset(Ain, 0, sizeof(double) * 15 * (size_t)n);
    node64 nd[27];

    /* g2p backward: recompute v' and the output position, then scatter. */
    for (int64_t i = 0; i < n; ++i) {
        const double* P = S + 15 * i;
        const double* A = Aout + 15 * i;
        double* R = Ain + 15 * i;
        stencil64(P, p, gc, nd);
        double v[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < 27; ++k) {
            if (nd[k].idx < 0) continue;
            const double* u = G + 4 * (int64_t)nd[k].idx;
            for (int r = 0; r < 3; ++r) v[r] += u[r] * nd[k].w;
        }
        double vbar[3], xbar_out[3];
        for (int a = 0; a < 3; ++a) {
            const double xr = P[a] + v[a] * dt;
            const double hw = p->real_box[a] - 2.0;
            double xo = xr < 1.0 ? 1.0 : xr;
            xo = xo > hw ? hw : xo;
            const double xn = xo + v[a] * dt * 3.0;
            const double wmax = p->real_box[a] - 4.0;
            double s = 0.0;
            if (xn < 3.0) s += 0.3;
            if (xn > wmax) s += 0.3;
            const double vb2 = A[3 + a];          /* adjoint of v'' */
            const double xnbar = -s * vb2;         /* v'' = v' + 0.3 (wall - x_n) */
            double xob = A[a] + xnbar;             /* adjoint of the clamped x' */
            vbar[a] = vb2 + 3.0 * dt * xnbar;
            const int clamped = (xr < 1.0) || (xr > hw);
            xbar_out[a] = clamped ? 0.0 : xob;     /* adjoint of x + dt v' */
            vbar[a] += dt * xbar_out[a];
        }
        double Bbar[3][3]; /* [c][r] */
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) Bbar[c][r] = 4.0 * A[6 + 3 * c + r];
        double xb[3] = {xbar_out[0], xbar_out[1], xbar_out[2]};
        for (int k = 0; k < 27; ++k) {
            if (nd[k].idx < 0) continue;
            const double* u = G + 4 * (int64_t)nd[k].idx;
            double* ub = gadj + 4 * (int64_t)nd[k].idx;
            double dot = 0.0; /* sum_r u[r] (vbar[r] + sum_c Bbar[c][r] d[c]) */
            for (int r = 0; r < 3; ++r) {
                double h = vbar[r];
                for (int c = 0; c < 3; ++c) h += Bbar[c][r] * nd[k].d[c];
                ub[r] += nd[k].w * h;
                dot += u[r] * h;
            }
            for (int a = 0; a < 3; ++a) {
                double t = 0.0; /* d/dd[a]: sum_r w u[r] Bbar[a][r] */
                for (int r = 0; r < 3; ++r) t += u[r] * Bbar[a][r];
                xb[a] += nd[k].gw[a] * dot - nd[k].w * t;
            }
        }
        for (int a = 0; a < 3; ++a) R[a] = xb[a];
    }

    /* update backward: u_bar -> P_bar (xyz) and m_bar (w). */
    {
        int32_t hi[3];
        for (int a = 0; a < 3; ++a) hi[a] = sat_i32(ceil(p->real_box[a]) - 3.0);
        for (int64_t j = 0; j < gc; ++j) {
            double* ub = gadj + 4 * j;
            const double* c = G + 4 * j;
            const double m = c[3];
            if (!(m > 0.0)) { ub[3] = 0.0; continue; } /* untouched: u = P */
            const int32_t id = (int32_t)j;
            const int32_t xyz[3] = {(id / Z) / Y, (id / Z) % Y, id % Z};
            double mb = 0.0;
            for (int a = 0; a < 3; ++a) {
                if (xyz[a] < 2 || xyz[a] > hi[a]) { ub[a] = 0.0; continue; }
                const double pm = c[a] - p->gravity[a] * dt; /* P / m */
                mb -= ub[a] * pm / m;
                ub[a] = ub[a] / m;
            }
            ub[3] = mb;
        }
    }

    /* p2g_2 backward: momentum adjoint through the stress; the density
     * adjoint is scattered onto m_bar (complete before p2g_1 gathers it). */
    double kbar = 0.0, mubar = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double* P = S + 15 * i;
        double* R = Ain + 15 * i;
        stencil64(P, p, gc, nd);
        double rho = 0.0;
        for (int k = 0; k < 27; ++k)
            if (nd[k].idx >= 0) rho += G[4 * (int64_t)nd[k].idx + 3] * nd[k].w;
        const double V = 1.0 / rho;
        const double rr = rho / p->rest_density;
        const double r5 = rr * rr * rr * rr * rr;
        const double pterm = p->stiffness * (r5 - 1.0);
        const double pres = pterm > 0.0 ? pterm : 0.0;
        double sig[3][3], T[3][3]; /* [row][col] */
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const double strain = P[6 + 3 * b + a] + P[6 + 3 * a + b];
                sig[a][b] = (a == b ? -pres : 0.0) + p->dynamic_viscosity * strain;
                T[a][b] = -V * 4.0 * sig[a][b] * dt;
            }
        double Tbar[3][3] = {{0}};
        double xb[3] = {0.0, 0.0, 0.0};
        double wbar[27];
        for (int k = 0; k < 27; ++k) {
            wbar[k] = 0.0;
            if (nd[k].idx < 0) continue;
            const double* Pb = gadj + 4 * (int64_t)nd[k].idx;
            double td[3];
            for (int r = 0; r < 3; ++r) td[r] = T[r][0] * nd[k].d[0] + T[r][1] * nd[k].d[1] +
                                                T[r][2] * nd[k].d[2];
            for (int r = 0; r < 3; ++r) {
                wbar[k] += Pb[r] * td[r];
                for (int b = 0; b < 3; ++b) Tbar[r][b] += Pb[r] * nd[k].w * nd[k].d[b];
            }
            for (int b = 0; b < 3; ++b) {
                double t = 0.0;
                for (int r = 0; r < 3; ++r) t += T[r][b] * Pb[r];
                xb[b] -= nd[k].w * t;
            }
        }
        /* T = -4 dt V sigma */
        double Vbar = 0.0, sigbar[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                Vbar += -4.0 * dt * sig[a][b] * Tbar[a][b];
                sigbar[a][b] = -4.0 * dt * V * Tbar[a][b];
            }
        double presbar = 0.0;
        for (int a = 0; a < 3; ++a) presbar -= sigbar[a][a];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                mubar += sigbar[a][b] * (P[6 + 3 * b + a] + P[6 + 3 * a + b]);
                R[6 + 3 * b + a] += p->dynamic_viscosity * sigbar[a][b];
                R[6 + 3 * a + b] += p->dynamic_viscosity * sigbar[a][b];
            }
        double rhobar = -Vbar / (rho * rho);
        if (pterm > 0.0) {
            kbar += presbar * (r5 - 1.0);
            rhobar += presbar * p->stiffness * 5.0 * rr * rr * rr * rr / p->rest_density;
        }
        for (int k = 0; k < 27; ++k) {
            if (nd[k].idx < 0) continue;
            gadj[4 * (int64_t)nd[k].idx + 3] += rhobar * nd[k].w;  /* density -> m_bar */
            wbar[k] += rhobar * G[4 * (int64_t)nd[k].idx + 3];
            for (int a = 0; a < 3; ++a) xb[a] += wbar[k] * nd[k].gw[a];
        }
        for (int a = 0; a < 3; ++a) R[a] += xb[a];
    }
    pgrad[0] += kbar;
    pgrad[1] += mubar;

    /* p2g_1 backward: gather P_bar and m_bar. */
    for (int64_t i = 0; i < n; ++i) {
        const double* P = S + 15 * i;
        double* R = Ain + 15 * i;
        stencil64(P, p, gc, nd);
        double xb[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < 27; ++k) {
            if (nd[k].idx < 0) continue;
            const double* Pb = gadj + 4 * (int64_t)nd[k].idx;
            double wb = Pb[3];
            for (int r = 0; r < 3; ++r) {
                const double q = P[6 + r] * nd[k].d[0] + P[9 + r] * nd[k].d[1] +
                                 P[12 + r] * nd[k].d[2];
                wb += Pb[r] * (P[3 + r] + q);
                R[3 + r] += nd[k].w * Pb[r];
                for (int c = 0; c < 3; ++c) R[6 + 3 * c + r] += nd[k].w * Pb[r] * nd[k].d[c];
            }
            for (int c = 0; c < 3; ++c) {
                double t = 0.0;
                for (int r = 0; r < 3; ++r) t += P[6 + 3 * c + r] * Pb[r];
                xb[c] -= nd[k].w * t;
            }
            for (int a = 0; a < 3; ++a) xb[a] += wb * nd[k].gw[a];
        }
        for (int a = 0; a < 3; ++a) R[a] += xb[a];
    }
}

/* Reverse-mode gradient of a loss whose adjoint seeds are given at some
 * substeps: seed_t[s] in [0, T] (ascending, unique), seed_vals[s] an n x 15
 * adjoint of the state after seed_t[s] substeps.  state0: n x 15 initial
 * state.  Outputs: grad (n x 15, dL/d state0) and pgrad[2] (dL/d stiffness,
 * dL/d dynamic viscosity).  every: checkpoint interval.  Returns 0, or -1 on
 * allocation failure. */
int orc64_backward_tape(const double* state0, int64_t n, const orc64_params* p, int T, int every,
                        const int* seed_t, const double* seed_vals, int nseeds, double* grad,
                        double* pgrad, int f32);

int orc64_backward(const double* state0, int64_t n, const orc64_params* p, int T, int every,
                   const int* seed_t, const double* seed_vals, int nseeds, double* grad,
                   double* pgrad) {
    return orc64_backward_tape(state0, n, p, T, every, seed_t, seed_vals, nseeds, grad, pgrad, 0);
}

/* orc64_backward with the tape (the trajectory and its grids) integrated in
 * f32 when f32 != 0 (the state widened to double between substeps, exactly);
 * the reverse pass itself stays FP64.  The difference from orc64_backward is
 * what an f32 trajectory costs the gradient. */
int orc64_backward_tape(const double* state0, int64_t n, const orc64_params* p, int T, int every,
                        const int* seed_t, const double* seed_vals, int nseeds, double* grad,
                        double* pgrad, int f32) {
    if (every < 1) every = 1;
    const int64_t gc = orc64_grid_count(p);
    const size_t sbytes = sizeof(double) * 15 * (size_t)n;
    const size_t gbytes = sizeof(double) * 4 * (size_t)(gc > 0 ? gc : 1);
    const int nseg = (T + every - 1) / every;
    double* ckpt = (double*)malloc(sbytes * (size_t)(nseg > 0 ? nseg : 1) + 1);
    double* tape_s = (double*)malloc(sbytes * (size_t)every + 1);
    double* tape_g = (double*)malloc(gbytes * (size_t)every);
    double* work = (double*)malloc(sbytes + 1);
    double* a = (double*)malloc(sbytes + 1);
    double* a2 = (double*)malloc(sbytes + 1);
    double* gadj = (double*)malloc(gbytes);
    float* sf = f32 ? (float*)malloc(sbytes / 2 + 1) : NULL;
    float* gf = f32 ? (float*)malloc(gbytes / 2 + 1) : NULL;
    if (!ckpt || !tape_s || !tape_g || !work || !a || !a2 || !gadj || (f32 && (!sf || !gf))) {
        free(ckpt); free(tape_s); free(tape_g); free(work); free(a); free(a2); free(gadj);
        free(sf); free(gf);
        return -1;
    }
    int64_t bad = 0;
    /* forward, keeping the state at the start of every segment */
    memcpy(work, state0, sbytes);
    for (int t = 0; t < T; ++t) {
        if (t % every == 0) memcpy(ckpt + 15 * (size_t)n * (t / every), work, sbytes);
        tape_substep(work, n, p, gadj, &bad, f32, sf, gf);
    }
    pgrad[0] = pgrad[1] = 0.0;
    memset(a, 0, sbytes);
    int s = nseeds - 1;
    /* the seed at T (the final state) */
    if (s >= 0 && seed_t[s] == T) {
        for (size_t q = 0; q < 15 * (size_t)n; ++q) a[q] += seed_vals[15 * (size_t)n * s + q];
        --s;
    }
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int t0 = seg * every, t1 = (t0 + every < T) ? t0 + every : T;
        memcpy(work, ckpt + 15 * (size_t)n * seg, sbytes);
        for (int t = t0; t < t1; ++t) {
            memcpy(tape_s + 15 * (size_t)n * (t - t0), work, sbytes);
            tape_substep(work, n, p, tape_g + 4 * (size_t)gc * (t - t0), &bad, f32, sf, gf);
        }
        for (int t = t1 - 1; t >= t0; --t) {
            orc64_substep_adjoint(tape_s + 15 * (size_t)n * (t - t0),
                                  tape_g + 4 * (size_t)gc * (t - t0), a, a2, n, p, gadj, pgrad);
            double* sw = a; a = a2; a2 = sw;
            if (s >= 0 && seed_t[s] == t) {
                for (size_t q = 0; q < 15 * (size_t)n; ++q)
                    a[q] += seed_vals[15 * (size_t)n * s + q];
                --s;
            }
        }
    }
    memcpy(grad, a, sbytes);
    free(ckpt); free(tape_s); free(tape_g); free(work); free(a); free(a2); free(gadj);
    free(sf); free(gf);
    return 0;
}
