/*
 * lbm_oracle.c -- CPU restatement of lbc's D2Q9 step, used ONLY as a test checker.
 *
 * This file is test infrastructure. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load it. The product (lbc_gb300/liblbm_gpu.so)
 * never links or calls it.
 *
 * It restates, in plain C99 (+ optional OpenMP), the FP64 algorithm of lbc's
 * src/core and src/bc, with every floating-point expression evaluated in the same
 * order as the reference so that, compiled with -ffp-contract=off, results match
 * the reference bit for bit (signed zeros aside). Each function cites the
 * reference file:line it follows. Arrays use the reference layout: populations
 * f[Ny][Nx][Q] (AoS, k fastest), scalar fields [Ny][Nx], int solid mask.
 *
 * Exported names carry the prefix orc_ so this library can be loaded next to the
 * GPU drop-in (which exports the reference's own names).
 *
 * Pinned: bit for bit against lbc's own src/ compiled by oracle/build_ref.sh
 * (every function, 15 cases) and against fixtures made by lbc's build
 * (tests/golden/), and to 1e-15 against lbc's shipped drag record
 * cases/cylinder/sol/forces_IBB_res_20_Re_20.00_tau_0.90.bin.
 *
 * Extensions without a counterpart in lbc (moving-wall bounce-back and the
 * per-wall-node mass-spring-damper impedance wall) are at the end of the file and
 * are marked as such. The moving wall reduces to lbc's step when the walls are
 * still; the impedance wall's parity is unpinned against lbc (its eduction lives
 * in an external toolkit that is not present).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_RHO_FLOOR 1e-16 /* src/core/compute_macroscopic_fields.c:2 */
#define ORC_IBB_EPS 1e-12   /* src/bc/interpolated_bounce_back.c:2 */

typedef void (*orc_bc_fn)(int, int, int, int, const double *, const double *, double *, double *,
                          double *, double *, double *, int *, int *, int *, double *);

/* Mirror of lbc's Boundary (include/lbm_types.h:21-26). */
typedef struct {
    int index;
    const double *val1;
    const double *val2;
    orc_bc_fn apply;
} orc_boundary;

static inline size_t nid(int Nx, int j, int i) { return (size_t)j * (size_t)Nx + (size_t)i; }
static inline size_t pid(int Nx, int Q, int j, int i, int k) { return nid(Nx, j, i) * (size_t)Q + (size_t)k; }

/* Wrap (or reject) a neighbour coordinate. Returns 0 when the coordinate falls
 * outside a non-periodic axis. Follows the wrap blocks of
 * src/bc/bounce_back.c:26-40 and src/core/streaming.c:24-37. */
static inline int wrap_coord(int *c, int n, int periodic) {
    if (periodic) {
        if (*c < 0) *c += n;
        else if (*c >= n) *c -= n;
        return 1;
    }
    return (*c >= 0 && *c < n);
}

/* ---------------------------------------------------------------- collision
 * src/core/collision.c:1-41. In-place BGK with Guo forcing, stored rho/u/v,
 * solids skipped. */
void orc_collision(int Nx, int Ny, int Q, double *f, const double *rho, const double *u,
                   const double *v, const double *omega_eff, const int *solid_mask, const int *cx,
                   const int *cy, const double *w, double Fx, double Fy) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        for (int i = 0; i < Nx; i++) {
            size_t n = nid(Nx, j, i);
            if (solid_mask[n]) continue;
            double ux = u[n], uy = v[n];
            double usq = ux * ux + uy * uy;
            double uF = ux * Fx + uy * Fy;
            double om = omega_eff[n];
            for (int k = 0; k < Q; k++) {
                double cu = cx[k] * ux + cy[k] * uy;
                double feq = w[k] * rho[n] * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
                double cF = cx[k] * Fx + cy[k] * Fy;
                double Fk = w[k] * (3.0 * cF + 9.0 * cu * cF - 3.0 * uF);
                size_t p = n * (size_t)Q + (size_t)k;
                f[p] += -om * (f[p] - feq) + (1 - 0.5 * om) * Fk;
            }
        }
    }
}

/* ---------------------------------------------------------------- streaming
 * src/core/streaming.c:1-45. Pull into fluid destinations from in-range (or
 * wrapped) non-solid sources; every other slot of f_new is left untouched. */
void orc_streaming(int Nx, int Ny, int Q, const double *f, double *f_new, const int *solid_mask,
                   const int *cx, const int *cy, int isperiodic_x, int isperiodic_y) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        for (int i = 0; i < Nx; i++) {
            if (solid_mask[nid(Nx, j, i)]) continue;
            for (int k = 0; k < Q; k++) {
                int is = i - cx[k], js = j - cy[k];
                if (!wrap_coord(&is, Nx, isperiodic_x)) continue;
                if (!wrap_coord(&js, Ny, isperiodic_y)) continue;
                if (solid_mask[nid(Nx, js, is)]) continue;
                f_new[pid(Nx, Q, j, i, k)] = f[pid(Nx, Q, js, is, k)];
            }
        }
    }
}

/* ---------------------------------------------------------------- moments
 * src/core/compute_macroscopic_fields.c:4-49. Sums over k in order, floor on
 * the density, NaN at solids. */
void orc_compute_macroscopic_fields(int Nx, int Ny, int Q, const double *f_new,
                                    const int *solid_mask, const int *cx, const int *cy,
                                    double *rho, double *u, double *v, double Fx, double Fy) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        for (int i = 0; i < Nx; i++) {
            size_t n = nid(Nx, j, i);
            double s = 0.0, sx = 0.0, sy = 0.0;
            for (int k = 0; k < Q; k++) {
                double fk = f_new[n * (size_t)Q + (size_t)k];
                s += fk;
                sx += fk * cx[k];
                sy += fk * cy[k];
            }
            if (s < ORC_RHO_FLOOR) s = ORC_RHO_FLOOR;
            if (!solid_mask[n]) {
                rho[n] = s;
                u[n] = (sx + 0.5 * Fx) / s;
                v[n] = (sy + 0.5 * Fy) / s;
            } else {
                rho[n] = NAN;
                u[n] = NAN;
                v[n] = NAN;
            }
        }
    }
}

/* ---------------------------------------------------------------- MEM force
 * src/core/compute_force_mem.c:1-72. Sum over fluid->solid links of
 * (f_k + f_new_opp(k)) c_k. The reference reduces with OpenMP atomics (order not
 * fixed); here rows are reduced in order, so results agree to round-off. */
void orc_compute_force_mem(int Nx, int Ny, int Q, const double *f, const double *f_new,
                           const int *solid_mask, int isperiodic_x, int isperiodic_y,
                           const int *cx, const int *cy, const int *opp, double *Fx, double *Fy) {
    double *rowx = (double *)calloc((size_t)Ny, sizeof(double));
    double *rowy = (double *)calloc((size_t)Ny, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        double ax = 0.0, ay = 0.0;
        for (int i = 0; i < Nx; i++) {
            if (solid_mask[nid(Nx, j, i)]) continue;
            for (int k = 1; k < Q; k++) {
                int in = i + cx[k], jn = j + cy[k];
                if (!wrap_coord(&in, Nx, isperiodic_x)) continue;
                if (!wrap_coord(&jn, Ny, isperiodic_y)) continue;
                if (!solid_mask[nid(Nx, jn, in)]) continue;
                double df = f[pid(Nx, Q, j, i, k)] + f_new[pid(Nx, Q, j, i, opp[k])];
                ax += df * cx[k];
                ay += df * cy[k];
            }
        }
        rowx[j] = ax;
        rowy[j] = ay;
    }
    double sx = 0.0, sy = 0.0;
    for (int j = 0; j < Ny; j++) {
        sx += rowx[j];
        sy += rowy[j];
    }
    free(rowx);
    free(rowy);
    *Fx = sx;
    *Fy = sy;
}

/* ---------------------------------------------------------------- bounce-back
 * src/bc/bounce_back.c:1-50. Halfway BB: f_new(x, opp k) = f(x, k) for every
 * fluid x whose neighbour along c_k is solid. */
void orc_bounce_back(int Nx, int Ny, int Q, const double *f, double *f_new, const int *solid_mask,
                     const int *cx, const int *cy, const int *opp, int isperiodic_x,
                     int isperiodic_y) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        for (int i = 0; i < Nx; i++) {
            if (solid_mask[nid(Nx, j, i)]) continue;
            for (int k = 0; k < Q; k++) {
                int in = i + cx[k], jn = j + cy[k];
                if (!wrap_coord(&in, Nx, isperiodic_x)) continue;
                if (!wrap_coord(&jn, Ny, isperiodic_y)) continue;
                if (!solid_mask[nid(Nx, jn, in)]) continue;
                f_new[pid(Nx, Q, j, i, opp[k])] = f[pid(Nx, Q, j, i, k)];
            }
        }
    }
}

/* ------------------------------------------------------- interpolated BB
 * src/bc/interpolated_bounce_back.c:4-104. Linear Bouzidi on cut links with q
 * from the level set phi, clamped (:51-61); behind node x - c_k (:63-89); the
 * q > 1/2 branch reads f_opp at the behind node (:98) and falls back to simple
 * BB when the behind node is solid (:95-96) or out of range (:72-88). */
void orc_interpolated_bounce_back(int Nx, int Ny, int Q, const double *f, double *f_new,
                                  const int *solid_mask, const double *phi, const int *opp,
                                  const int *cx, const int *cy, int isperiodic_x,
                                  int isperiodic_y) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        for (int i = 0; i < Nx; i++) {
            size_t n = nid(Nx, j, i);
            if (solid_mask[n]) continue;
            for (int k = 0; k < Q; k++) {
                int in = i + cx[k], jn = j + cy[k];
                if (!wrap_coord(&in, Nx, isperiodic_x)) continue;
                if (!wrap_coord(&jn, Ny, isperiodic_y)) continue;
                if (!solid_mask[nid(Nx, jn, in)]) continue;
                double denom = phi[n] - phi[nid(Nx, jn, in)];
                if (fabs(denom) < ORC_IBB_EPS) denom = (denom >= 0.0) ? ORC_IBB_EPS : -ORC_IBB_EPS;
                double q = phi[n] / denom;
                if (q < ORC_IBB_EPS) q = ORC_IBB_EPS;
                if (q > 1.0 - ORC_IBB_EPS) q = 1.0 - ORC_IBB_EPS;
                size_t dst = pid(Nx, Q, j, i, opp[k]);
                double fk = f[pid(Nx, Q, j, i, k)];
                int ib = i - cx[k], jb = j - cy[k];
                if (!wrap_coord(&ib, Nx, isperiodic_x) || !wrap_coord(&jb, Ny, isperiodic_y)) {
                    f_new[dst] = fk;
                    continue;
                }
                if (q <= 0.5) {
                    f_new[dst] = (1.0 - 2.0 * q) * fk + 2.0 * q * f[pid(Nx, Q, jb, ib, k)];
                } else if (solid_mask[nid(Nx, jb, ib)]) {
                    f_new[dst] = fk;
                } else {
                    f_new[dst] = (1.0 / (2.0 * q)) * fk +
                                 (2.0 * q - 1.0) / (2.0 * q) * f[pid(Nx, Q, jb, ib, opp[k])];
                }
            }
        }
    }
}

/* ---------------------------------------------------------------- edge BCs
 * Common argument list of every lbc BC (BCFunction, include/lbm_types.h:4-19).
 * Edge lines: "column" BCs act on i = index for all j, "row" BCs on j = index
 * for all i. */
#define ORC_BC_ARGS                                                                           \
    int Nx, int Ny, int Q, int index, const double *val1, const double *val2, double *f,      \
        double *f_new, double *rho, double *u, double *v, int *solid_mask, int *cx, int *cy, \
        double *w

/* Regularized BC shared by the eight *_regularized files
 * (e.g. src/bc/velocity_inlet_regularized.c:18-71). Node b gets
 * f_eq(rho_b, u_b) + 3/2 w_k Q_k:Pi, with Pi the second moment of the
 * non-equilibrium part at the interior node n (previous-step rho/u/v at n,
 * current f_new at n). Velocity BCs: rho_b = rho_n, u_b = (val1, val2).
 * Pressure BCs: rho_b = val1, u_b = u_n. */
static void regularized_node(int Q, const int *cx, const int *cy, const double *w,
                             const double *fn, double rho_n, double u_n, double v_n,
                             double rho_b, double U_b, double V_b, double *fb) {
    double usq_n = u_n * u_n + v_n * v_n;
    double usq_b = U_b * U_b + V_b * V_b;
    double Pxx = 0.0, Pxy = 0.0, Pyy = 0.0;
    for (int k = 0; k < Q; k++) {
        double cu = cx[k] * u_n + cy[k] * v_n;
        double feq = w[k] * rho_n * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq_n);
        double fneq = fn[k] - feq;
        Pxx += cx[k] * cx[k] * fneq;
        Pxy += cx[k] * cy[k] * fneq;
        Pyy += cy[k] * cy[k] * fneq;
    }
    for (int k = 0; k < Q; k++) {
        double cu = cx[k] * U_b + cy[k] * V_b;
        double feq = w[k] * rho_b * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq_b);
        double Qxx = cx[k] * cx[k] - 1.0 / 3.0;
        double Qxy = cx[k] * cy[k];
        double Qyy = cy[k] * cy[k] - 1.0 / 3.0;
        double fneq = (3.0 / 2.0) * w[k] * (Qxx * Pxx + 2.0 * Qxy * Pxy + Qyy * Pyy);
        fb[k] = feq + fneq;
    }
}

/* side: 0 inlet (i=index, n=i+1), 1 outlet (i=index, n=i-1), 2 bottom (j=index,
 * n=j+1), 3 top (j=index, n=j-1). pressure: rho_b from val1 and u_b from n. */
static void regularized_line(ORC_BC_ARGS, int side, int pressure) {
    int along = (side < 2) ? Ny : Nx;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < along; t++) {
        int ib, jb, in_, jn;
        if (side < 2) {
            ib = index; jb = t; jn = t; in_ = (side == 0) ? index + 1 : index - 1;
        } else {
            jb = index; ib = t; in_ = t; jn = (side == 2) ? index + 1 : index - 1;
        }
        size_t b = nid(Nx, jb, ib), n = nid(Nx, jn, in_);
        if (solid_mask[b]) continue;
        double rho_b, U_b, V_b;
        if (pressure) {
            rho_b = val1[t]; U_b = u[n]; V_b = v[n];
        } else {
            rho_b = rho[n]; U_b = val1[t]; V_b = val2[t];
        }
        double fb[9];
        regularized_node(Q, cx, cy, w, f_new + n * (size_t)Q, rho[n], u[n], v[n], rho_b, U_b,
                         V_b, fb);
        for (int k = 0; k < Q; k++) f_new[b * (size_t)Q + (size_t)k] = fb[k];
    }
    (void)f;
}

/* src/bc/velocity_inlet_regularized.c:1-72 */
void orc_velocity_inlet_regularized(ORC_BC_ARGS) { regularized_line(Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, solid_mask, cx, cy, w, 0, 0); }
/* src/bc/velocity_outlet_regularized.c:1-72 */
void orc_velocity_outlet_regularized(ORC_BC_ARGS) { regularized_line(Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, solid_mask, cx, cy, w, 1, 0); }
/* src/bc/velocity_bottom_regularized.c:1-71 */
void orc_velocity_bottom_regularized(ORC_BC_ARGS) { regularized_line(Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, solid_mask, cx, cy, w, 2, 0); }
/* src/bc/velocity_top_regularized.c:1-71 */
void orc_velocity_top_regularized(ORC_BC_ARGS) { regularized_line(Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, solid_mask, cx, cy, w, 3, 0); }
/* src/bc/pressure_inlet_regularized.c:1-72 */
void orc_pressure_inlet_regularized(ORC_BC_ARGS) { regularized_line(Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, solid_mask, cx, cy, w, 0, 1); }
/* src/bc/pressure_outlet_regularized.c:1-72 */
void orc_pressure_outlet_regularized(ORC_BC_ARGS) { regularized_line(Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, solid_mask, cx, cy, w, 1, 1); }
/* src/bc/pressure_bottom_regularized.c:1-71 */
void orc_pressure_bottom_regularized(ORC_BC_ARGS) { regularized_line(Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, solid_mask, cx, cy, w, 2, 1); }
/* src/bc/pressure_top_regularized.c:1-71 */
void orc_pressure_top_regularized(ORC_BC_ARGS) { regularized_line(Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, solid_mask, cx, cy, w, 3, 1); }

/* Zou-He BCs. They use literal population numbers of lbc's D2Q9 ordering. */

/* src/bc/velocity_inlet.c:17-41 */
void orc_velocity_inlet(ORC_BC_ARGS) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        size_t b = nid(Nx, j, index);
        if (solid_mask[b]) continue;
        double *p = f_new + b * (size_t)Q;
        double U = val1[j], V = val2[j];
        double rh = (p[0] + p[2] + p[4] + 2.0 * (p[3] + p[6] + p[7])) / (1.0 - U);
        double f2 = p[2], f3 = p[3], f4 = p[4], f6 = p[6], f7 = p[7];
        p[1] = f3 + (2.0 / 3.0) * rh * U;
        p[5] = f7 + (1.0 / 6.0) * rh * U - 0.5 * (f2 - f4) + (1.0 / 2.0) * rh * V;
        p[8] = f6 + (1.0 / 6.0) * rh * U + 0.5 * (f2 - f4) - (1.0 / 2.0) * rh * V;
    }
}

/* src/bc/velocity_outlet.c:17-41 */
void orc_velocity_outlet(ORC_BC_ARGS) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        size_t b = nid(Nx, j, index);
        if (solid_mask[b]) continue;
        double *p = f_new + b * (size_t)Q;
        double U = val1[j], V = val2[j];
        double f1 = p[1], f2 = p[2], f4 = p[4], f5 = p[5], f8 = p[8];
        double rh = (p[0] + f2 + f4 + 2.0 * (f1 + f5 + f8)) / (1.0 + U);
        p[3] = f1 - (2.0 / 3.0) * rh * U;
        p[6] = f8 - 0.5 * (f2 - f4) - (1.0 / 6.0) * rh * U + (1.0 / 2.0) * rh * V;
        p[7] = f5 + 0.5 * (f2 - f4) - (1.0 / 6.0) * rh * U - (1.0 / 2.0) * rh * V;
    }
}

/* src/bc/velocity_top.c:17-40 */
void orc_velocity_top(ORC_BC_ARGS) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < Nx; i++) {
        size_t b = nid(Nx, index, i);
        if (solid_mask[b]) continue;
        double *p = f_new + b * (size_t)Q;
        double U = val1[i], V = val2[i];
        double f1 = p[1], f2 = p[2], f3 = p[3], f5 = p[5], f6 = p[6];
        double rh = (p[0] + f1 + f3 + 2 * (f2 + f5 + f6)) / (1 + V);
        p[4] = f2 - 2.0 / 3.0 * rh * V;
        p[7] = f5 + (f1 - f3) / 2.0 - 0.5 * rh * U - 1.0 / 6.0 * rh * V;
        p[8] = f6 - (f1 - f3) / 2.0 + 0.5 * rh * U - 1.0 / 6.0 * rh * V;
    }
}

/* src/bc/velocity_bottom.c:17-40. Keeps lbc's behaviour at :39, which writes
 * population 7 (not 6) a second time. */
void orc_velocity_bottom(ORC_BC_ARGS) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < Nx; i++) {
        size_t b = nid(Nx, index, i);
        if (solid_mask[b]) continue;
        double *p = f_new + b * (size_t)Q;
        double U = val1[i], V = val2[i];
        double f1 = p[1], f3 = p[3], f4 = p[4], f7 = p[7], f8 = p[8];
        double rh = (p[0] + f1 + f3 + 2 * (f4 + f7 + f8)) / (1 - V);
        p[2] = f4 + 2.0 / 3.0 * rh * V;
        p[5] = f7 - (f1 - f3) / 2.0 + 0.5 * rh * U + 1.0 / 6.0 * rh * V;
        p[7] = f8 + (f1 - f3) / 2.0 - 0.5 * rh * U + 1.0 / 6.0 * rh * V;
    }
}

/* Extension (no counterpart in lbc): velocity_bottom with the last Zou-He line
 * written to population 6, as the closure for a bottom wall has it (the mirror
 * of src/bc/velocity_top.c:37-39 in y). */
void orc_velocity_bottom_corrected(ORC_BC_ARGS) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < Nx; i++) {
        size_t b = nid(Nx, index, i);
        if (solid_mask[b]) continue;
        double *p = f_new + b * (size_t)Q;
        double U = val1[i], V = val2[i];
        double f1 = p[1], f3 = p[3], f4 = p[4], f7 = p[7], f8 = p[8];
        double rh = (p[0] + f1 + f3 + 2 * (f4 + f7 + f8)) / (1 - V);
        p[2] = f4 + 2.0 / 3.0 * rh * V;
        p[5] = f7 - (f1 - f3) / 2.0 + 0.5 * rh * U + 1.0 / 6.0 * rh * V;
        p[6] = f8 + (f1 - f3) / 2.0 - 0.5 * rh * U + 1.0 / 6.0 * rh * V;
    }
}

/* src/bc/pressure_inlet.c:17-41. Transverse velocity from the previous-step v at
 * i+1 (:35). */
void orc_pressure_inlet(ORC_BC_ARGS) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        size_t b = nid(Nx, j, index);
        if (solid_mask[b]) continue;
        double *p = f_new + b * (size_t)Q;
        double R = val1[j];
        double f2 = p[2], f4 = p[4], f3 = p[3], f6 = p[6], f7 = p[7];
        double U = 1.0 - (p[0] + f2 + f4 + 2.0 * (f3 + f6 + f7)) / R;
        double V = v[nid(Nx, j, index + 1)];
        p[1] = f3 + (2.0 / 3.0) * R * U;
        p[5] = f7 + (1.0 / 6.0) * R * U - 0.5 * (f2 - f4) + (1.0 / 2.0) * R * V;
        p[8] = f6 + (1.0 / 6.0) * R * U + 0.5 * (f2 - f4) - (1.0 / 2.0) * R * V;
    }
}

/* src/bc/pressure_outlet.c:17-41. Transverse velocity from the previous-step v
 * at i-1 (:35). */
void orc_pressure_outlet(ORC_BC_ARGS) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ny; j++) {
        size_t b = nid(Nx, j, index);
        if (solid_mask[b]) continue;
        double *p = f_new + b * (size_t)Q;
        double R = val1[j];
        double f1 = p[1], f2 = p[2], f4 = p[4], f5 = p[5], f8 = p[8];
        double U = (p[0] + f2 + f4 + 2.0 * (f1 + f5 + f8)) / R - 1.0;
        double V = v[nid(Nx, j, index - 1)];
        p[3] = f1 - (2.0 / 3.0) * R * U;
        p[6] = f8 - 0.5 * (f2 - f4) - (1.0 / 6.0) * R * U + (1.0 / 2.0) * R * V;
        p[7] = f5 + 0.5 * (f2 - f4) - (1.0 / 6.0) * R * U - (1.0 / 2.0) * R * V;
    }
}

/* Convective (zero-gradient) edges copy the current f_new of the interior
 * neighbour: src/bc/convective_inlet.c:17-29, src/bc/convective_outlet.c:17-29. */
void orc_convective_inlet(ORC_BC_ARGS) {
    for (int j = 0; j < Ny; j++) {
        if (solid_mask[nid(Nx, j, index)]) continue;
        memcpy(f_new + nid(Nx, j, index) * (size_t)Q, f_new + nid(Nx, j, index + 1) * (size_t)Q,
               sizeof(double) * (size_t)Q);
    }
}
void orc_convective_outlet(ORC_BC_ARGS) {
    for (int j = 0; j < Ny; j++) {
        if (solid_mask[nid(Nx, j, index)]) continue;
        memcpy(f_new + nid(Nx, j, index) * (size_t)Q, f_new + nid(Nx, j, index - 1) * (size_t)Q,
               sizeof(double) * (size_t)Q);
    }
}

/* Periodic edges re-copy wrapped populations from the post-collision f:
 * src/bc/periodic_x.c:17-51 (no wrap in y), src/bc/periodic_y.c:17-51 (no wrap
 * in x). */
void orc_periodic_x(ORC_BC_ARGS) {
    for (int k = 0; k < Q; k++) {
        if (cx[k] == 0) continue;
        int i = (cx[k] > 0) ? 0 : Nx - 1;
        int is = (cx[k] > 0) ? Nx - cx[k] : -cx[k] - 1;
        for (int j = 0; j < Ny; j++) {
            int js = j - cy[k];
            if (js < 0 || js >= Ny) continue;
            if (solid_mask[nid(Nx, j, i)] || solid_mask[nid(Nx, js, is)]) continue;
            f_new[pid(Nx, Q, j, i, k)] = f[pid(Nx, Q, js, is, k)];
        }
    }
}
void orc_periodic_y(ORC_BC_ARGS) {
    for (int k = 0; k < Q; k++) {
        if (cy[k] == 0) continue;
        int j = (cy[k] > 0) ? 0 : Ny - 1;
        int js = (cy[k] > 0) ? Ny - cy[k] : -cy[k] - 1;
        for (int i = 0; i < Nx; i++) {
            int is = i - cx[k];
            if (is < 0 || is >= Nx) continue;
            if (solid_mask[nid(Nx, j, i)] || solid_mask[nid(Nx, js, is)]) continue;
            f_new[pid(Nx, Q, j, i, k)] = f[pid(Nx, Q, js, is, k)];
        }
    }
}

/* ---------------------------------------------------------------- one step
 * src/core/main_lbm.c:5-62: collide -> BB or IBB -> MEM force (into D, L as
 * Fx, Fy, :43) -> stream -> BC list in order -> moments. */
void orc_main_lbm(int Nx, int Ny, int Q, double *f, double *f_new, double *rho, double *u,
                  double *v, int *cx, int *cy, double *w, int *opp, double *omega_eff,
                  int *solid_mask, orc_boundary *boundaries, int num_boundaries, int isperiodic_x,
                  int isperiodic_y, double Fx, double Fy, double *L, double *D, double *phi,
                  int use_IBB) {
    orc_collision(Nx, Ny, Q, f, rho, u, v, omega_eff, solid_mask, cx, cy, w, Fx, Fy);
    if (use_IBB)
        orc_interpolated_bounce_back(Nx, Ny, Q, f, f_new, solid_mask, phi, opp, cx, cy,
                                     isperiodic_x, isperiodic_y);
    else
        orc_bounce_back(Nx, Ny, Q, f, f_new, solid_mask, cx, cy, opp, isperiodic_x, isperiodic_y);
    orc_compute_force_mem(Nx, Ny, Q, f, f_new, solid_mask, isperiodic_x, isperiodic_y, cx, cy, opp,
                          D, L);
    orc_streaming(Nx, Ny, Q, f, f_new, solid_mask, cx, cy, isperiodic_x, isperiodic_y);
    for (int b = 0; b < num_boundaries; b++)
        boundaries[b].apply(Nx, Ny, Q, boundaries[b].index, boundaries[b].val1,
                            boundaries[b].val2, f, f_new, rho, u, v, solid_mask, cx, cy, w);
    orc_compute_macroscopic_fields(Nx, Ny, Q, f_new, solid_mask, cx, cy, rho, u, v, Fx, Fy);
}

/* Convenience driver for tests: n calls of orc_main_lbm with the caller-side
 * pointer swap of cases/nit/nit.c:309-311. After the call, f holds the newest
 * populations (the swap is applied to the arrays' contents when n is odd so the
 * caller's naming stays valid). */
void orc_run(int nsteps, int Nx, int Ny, int Q, double *f, double *f_new, double *rho, double *u,
             double *v, int *cx, int *cy, double *w, int *opp, double *omega_eff, int *solid_mask,
             orc_boundary *boundaries, int num_boundaries, int isperiodic_x, int isperiodic_y,
             double Fx, double Fy, double *L, double *D, double *phi, int use_IBB) {
    double *a = f, *b = f_new;
    for (int s = 0; s < nsteps; s++) {
        orc_main_lbm(Nx, Ny, Q, a, b, rho, u, v, cx, cy, w, opp, omega_eff, solid_mask, boundaries,
                     num_boundaries, isperiodic_x, isperiodic_y, Fx, Fy, L, D, phi, use_IBB);
        double *t = a; a = b; b = t;
    }
    if (a != f) {
        size_t n = (size_t)Nx * (size_t)Ny * (size_t)Q;
        double *tmp = (double *)malloc(n * sizeof(double));
        memcpy(tmp, f, n * sizeof(double));
        memcpy(f, f_new, n * sizeof(double));
        memcpy(f_new, tmp, n * sizeof(double));
        free(tmp);
    }
}

/* ---------------------------------------------------------------- Mei init
 * src/core/mei_initialization.c:7-143. Incompressible-equilibrium start, then
 * density moment / incompressible collision (all nodes, :92-108) / streaming
 * until max|d rho| <= tol. The swap at :114-116 only swaps the local names, so
 * after an odd number of completed iterations the newest populations sit in the
 * caller's f_new. Returns the number of completed iterations. */
int orc_mei_initialization(int Nx, int Ny, int Q, double *f, double *f_new, const double *rho_in,
                           const double *U_in, const double *V_in, double *rho, double *u,
                           double *v, const int *cx, const int *cy, const double *w,
                           const double *omega_eff, int isperiodic_x, int isperiodic_y,
                           int init_iter_max, double tol_rho, const int *solid_mask) {
    size_t N = (size_t)Nx * (size_t)Ny;
    memcpy(u, U_in, N * sizeof(double));
    memcpy(v, V_in, N * sizeof(double));
    memcpy(rho, rho_in, N * sizeof(double));
    double rho0 = 0.0;
    for (size_t n = 0; n < N; n++) rho0 += rho[n];
    rho0 /= (Nx * Ny);
    for (size_t n = 0; n < N; n++) {
        double ux = u[n], uy = v[n];
        double usq = ux * ux + uy * uy;
        for (int k = 0; k < Q; k++) {
            double cu = cx[k] * ux + cy[k] * uy;
            f[n * (size_t)Q + (size_t)k] = w[k] * rho[n] + w[k] * rho0 * (3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
        }
    }
    double *prev = (double *)malloc(N * sizeof(double));
    double *a = f, *b = f_new;
    double maxd = 0.0;
    int done = 0;
    for (int it = 0; it < init_iter_max; it++) {
        memcpy(prev, rho, N * sizeof(double));
        for (size_t n = 0; n < N; n++) {
            double s = 0.0;
            for (int k = 0; k < Q; k++) s += a[n * (size_t)Q + (size_t)k];
            rho[n] = s;
        }
        for (size_t n = 0; n < N; n++) {
            double ux = u[n], uy = v[n];
            double usq = ux * ux + uy * uy;
            for (int k = 0; k < Q; k++) {
                double cu = cx[k] * ux + cy[k] * uy;
                double feq = w[k] * rho[n] + w[k] * rho0 * (3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
                size_t p = n * (size_t)Q + (size_t)k;
                a[p] += -omega_eff[n] * (a[p] - feq);
            }
        }
        orc_streaming(Nx, Ny, Q, a, b, solid_mask, cx, cy, isperiodic_x, isperiodic_y);
        double *t = a; a = b; b = t;
        done = it + 1;
        maxd = 0.0;
        for (size_t n = 0; n < N; n++) {
            double d = fabs(rho[n] - prev[n]);
            if (d > maxd) maxd = d;
        }
        if (maxd <= tol_rho) break;
    }
    free(prev);
    return done;
}

/* ---------------------------------------------------------------- sponge
 * src/core/sponge_layer.c:3-45. Radial exponential ramp of tau, stored as
 * omega = 1/tau. */
void orc_sponge_layer(int Nx, int Ny, double dx, double xc, double yc, double r_inner,
                      double r_outer, double tau_base, double incr_tau, double exp_coeff,
                      double *omega_eff) {
    for (int j = 0; j < Ny; j++) {
        double y = j * dx - yc;
        for (int i = 0; i < Nx; i++) {
            double x = i * dx - xc;
            double r = sqrt(x * x + y * y);
            double tau;
            if (r <= r_inner) {
                tau = tau_base;
            } else if ((r > r_inner) & (r <= r_outer)) {
                tau = tau_base + (incr_tau - 1) * tau_base * (exp(exp_coeff * (r - r_inner)) - 1) /
                                     (exp(exp_coeff * (r_outer - r_inner)) - 1);
            } else {
                tau = tau_base * incr_tau;
            }
            omega_eff[nid(Nx, j, i)] = 1.0 / tau;
        }
    }
}

/* ======================================================================
 * Extensions with no counterpart in lbc (checked by their own tests).
 * ====================================================================== */

/* Moving-wall halfway bounce-back (Ladd): for a fluid node x whose neighbour
 * along c_k is a solid node with wall velocity (uw, vw), the reflected
 * population is f_new(x, opp k) = f(x, k) - 6 w_k rho_w (c_k . u_w), with
 * rho_w = 1. Applied after orc_bounce_back so it only corrects the moving
 * links; wall velocity arrays are per node (zero on fixed walls). */
void orc_ext_moving_wall(int Nx, int Ny, int Q, const double *f, double *f_new,
                         const int *solid_mask, const double *uw, const double *vw, const int *cx,
                         const int *cy, const double *w, const int *opp, int isperiodic_x,
                         int isperiodic_y) {
    for (int j = 0; j < Ny; j++) {
        for (int i = 0; i < Nx; i++) {
            if (solid_mask[nid(Nx, j, i)]) continue;
            for (int k = 1; k < Q; k++) {
                int in = i + cx[k], jn = j + cy[k];
                if (!wrap_coord(&in, Nx, isperiodic_x)) continue;
                if (!wrap_coord(&jn, Ny, isperiodic_y)) continue;
                size_t s = nid(Nx, jn, in);
                if (!solid_mask[s]) continue;
                double cuw = cx[k] * uw[s] + cy[k] * vw[s];
                if (cuw == 0.0) continue;
                f_new[pid(Nx, Q, j, i, opp[k])] = f[pid(Nx, Q, j, i, k)] - 6.0 * w[k] * cuw;
            }
        }
    }
}

/* One step with moving walls: the reference step with the moving-wall term
 * applied right after the plain bounce-back. */
void orc_ext_main_lbm_moving(int Nx, int Ny, int Q, double *f, double *f_new, double *rho,
                             double *u, double *v, int *cx, int *cy, double *w, int *opp,
                             double *omega_eff, int *solid_mask, orc_boundary *boundaries,
                             int num_boundaries, int isperiodic_x, int isperiodic_y, double Fx,
                             double Fy, double *L, double *D, const double *uw, const double *vw) {
    orc_collision(Nx, Ny, Q, f, rho, u, v, omega_eff, solid_mask, cx, cy, w, Fx, Fy);
    orc_bounce_back(Nx, Ny, Q, f, f_new, solid_mask, cx, cy, opp, isperiodic_x, isperiodic_y);
    orc_ext_moving_wall(Nx, Ny, Q, f, f_new, solid_mask, uw, vw, cx, cy, w, opp, isperiodic_x,
                        isperiodic_y);
    orc_compute_force_mem(Nx, Ny, Q, f, f_new, solid_mask, isperiodic_x, isperiodic_y, cx, cy, opp,
                          D, L);
    orc_streaming(Nx, Ny, Q, f, f_new, solid_mask, cx, cy, isperiodic_x, isperiodic_y);
    for (int b = 0; b < num_boundaries; b++)
        boundaries[b].apply(Nx, Ny, Q, boundaries[b].index, boundaries[b].val1,
                            boundaries[b].val2, f, f_new, rho, u, v, solid_mask, cx, cy, w);
    orc_compute_macroscopic_fields(Nx, Ny, Q, f_new, solid_mask, cx, cy, rho, u, v, Fx, Fy);
}

/* ---------------------------------------------------------------- impedance wall
 * Extension: per wall node a mass-spring-damper m v' + R v + K x = p' replaces
 * the single host-side ADE of cases/nit/nit.c:13-47,276-303 (which drives one
 * velocity for the whole outlet from the surface-averaged pressure). Each step,
 * before main_lbm, the pressure p' = (rho - rho_ref)/3 of the node above the
 * wall (previous-step density, as the regularized BC uses it) advances the
 * node's state with the exact zero-order-hold update, and the new wall-normal
 * velocity v (into the liner) goes to the bottom regularized BC as val2 = -v.
 * Layout of `imp` (shared with the GPU engine): field-major, n entries per
 * field: active, A11, A12, A21, A22, b1, b2, x, v, mean density, then per
 * frequency (phasor re, im, sum p' e^{-iwn} re, im, sum v e^{-iwn} re, im).
 * p' is taken about the node's running mean density, rhobar += alpha (rho -
 * rhobar) (alpha = 0: fixed reference). The DFT terms are weighted by a Hann
 * window 0.5 (1 - cos(2 pi n / L)) kept as a rotating phasor (wc, ws) turned
 * by (wcos, wsin) = (cos, sin)(2 pi / L) each step when windowed. */
enum { OI_ACT, OI_A11, OI_A12, OI_A21, OI_A22, OI_B1, OI_B2, OI_X, OI_V, OI_RHOBAR, OI_WC, OI_WS, OI_N };

int orc_ext_msd_zoh(double R, double m, double K, double *A, double *b) {
    if (!(m > 0.0) || !(K > 0.0) || !(R >= 0.0)) return 0;
    double km = K / m, rm = R / m;
    double a = -0.5 * rm;
    double d2 = a * a - km;
    double E0, E1;
    if (d2 > 0.0) {
        double d = sqrt(d2);
        double ep = exp(a + d), em = exp(a - d);
        E0 = 0.5 * (ep + em);
        E1 = 0.5 * (ep - em) / d;
    } else if (d2 < 0.0) {
        double wd = sqrt(-d2), ea = exp(a);
        E0 = ea * cos(wd);
        E1 = ea * sin(wd) / wd;
    } else {
        E0 = exp(a);
        E1 = exp(a);
    }
    A[0] = E0 + E1 * (0.0 - a);
    A[1] = E1 * 1.0;
    A[2] = E1 * (-km);
    A[3] = E0 + E1 * (-rm - a);
    double q1 = A[1] / m, q2 = (A[3] - 1.0) / m;
    b[0] = (-rm * q1 - q2) / km;
    b[1] = q1;
    return 1;
}

/* One step of every wall node; val2_out = -v on active nodes, val2_in
 * elsewhere. rho is the stored [Ny][Nx] density, the wall row is `index`. */
void orc_ext_impedance_step(int Nx, int index, const double *rho, double alpha, double *imp,
                            int nf, const double *cw, const double *sw, double wcos, double wsin,
                            int windowed, const int *solid_mask, const double *val2_in,
                            double *val2_out) {
    int n = Nx;
#define OIMP(f, t) imp[(size_t)(f) * (size_t)n + (size_t)(t)]
    for (int t = 0; t < n; t++) {
        val2_out[t] = val2_in ? val2_in[t] : 0.0;
        if (OIMP(OI_ACT, t) == 0.0 || solid_mask[nid(Nx, index, t)]) continue;
        double rn = rho[nid(Nx, index + 1, t)];
        double rb = OIMP(OI_RHOBAR, t);
        double p = (rn - rb) / 3.0;
        OIMP(OI_RHOBAR, t) = rb + alpha * (rn - rb);
        double win = 1.0;
        if (windowed) {
            double c = OIMP(OI_WC, t), s = OIMP(OI_WS, t);
            win = 0.5 * (1.0 - c);
            OIMP(OI_WC, t) = c * wcos - s * wsin;
            OIMP(OI_WS, t) = s * wcos + c * wsin;
        }
        double x = OIMP(OI_X, t), v = OIMP(OI_V, t);
        double xn = OIMP(OI_A11, t) * x + OIMP(OI_A12, t) * v + OIMP(OI_B1, t) * p;
        double vn = OIMP(OI_A21, t) * x + OIMP(OI_A22, t) * v + OIMP(OI_B2, t) * p;
        OIMP(OI_X, t) = xn;
        OIMP(OI_V, t) = vn;
        for (int f = 0; f < nf; f++) {
            int b0 = OI_N + 6 * f;
            double cr = OIMP(b0, t), ci = OIMP(b0 + 1, t);
            double wp = win * p, wv = win * vn;
            OIMP(b0 + 2, t) += wp * cr;
            OIMP(b0 + 3, t) += wp * ci;
            OIMP(b0 + 4, t) += wv * cr;
            OIMP(b0 + 5, t) += wv * ci;
            OIMP(b0, t) = cr * cw[f] + ci * sw[f];
            OIMP(b0 + 1, t) = ci * cw[f] - cr * sw[f];
        }
        val2_out[t] = -vn;
    }
#undef OIMP
}
