// bc_shifted.cuh -- lbc's edge boundary conditions on shifted populations
// g = f - w in FP32 (the FP32 / FP16 storage forms).
//
// Each BC is lbc's formula with f_k = g_k + w_k substituted. The weights of
// opposite directions are equal, so differences of populations carry over to
// g unchanged; the Zou-He density closures sum populations whose weights add
// up to exactly 1 (e.g. w0 + w2 + w4 + 2 (w3 + w6 + w7) = 1), so
// rho = (1 + G) / (1 - U) with G the same combination of g; the regularized
// BCs take the non-equilibrium part as g - (feq - w), which keeps its
// precision in FP32 (f - feq of unshifted FP32 values would lose most of it).
// The FP64 form (bc_apply in lbm_device.cuh) is the one checked bit for bit
// against lbc.
#pragma once
#include "lbm_device.cuh"

namespace lbm {

// feq_k - w_k = w_k (drho + rho (3 c.u + 4.5 (c.u)^2 - 1.5 u.u)), rho = 1 + drho.
__device__ __forceinline__ void feq_shifted(const float w[9], float dr, float ux, float uy, float out[9]) {
    const float rho = 1.0f + dr;
    const float uu = 1.5f * (ux * ux + uy * uy);
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const float cu = (float)cxk(k) * ux + (float)cyk(k) * uy;
        out[k] = w[k] * (dr + rho * (3.0f * cu + 4.5f * cu * cu - uu));
    }
}

// Regularized BC at boundary node b from interior neighbour n
// (src/bc/velocity_inlet_regularized.c:18-71 and its seven siblings): the
// previous-step moments of n, the current g of n; velocity BCs impose
// (U, V) with drho_b = drho_n, pressure BCs impose drho_b with u_b = u_n.
template <class A>
__device__ __forceinline__ void bc_regularized_s(A &a, const float w[9], int ib, int jb, int in, int jn,
                                                 bool pressure, float v1, float v2) {
    const float dr_n = a.drho(in, jn), u_n = a.ux(in, jn), v_n = a.uy(in, jn);
    float drb, U, V;
    if (pressure) {
        drb = v1; U = u_n; V = v_n;
    } else {
        drb = dr_n; U = v1; V = v2;
    }
    float fe[9];
    feq_shifted(w, dr_n, u_n, v_n, fe);
    float fneq[9];
#pragma unroll
    for (int k = 0; k < 9; k++) fneq[k] = a.get(in, jn, k) - fe[k];
    const float Pxx = ((((fneq[1] + fneq[3]) + fneq[5]) + fneq[6]) + fneq[7]) + fneq[8];
    const float Pxy = ((fneq[5] - fneq[6]) + fneq[7]) - fneq[8];
    const float Pyy = ((((fneq[2] + fneq[4]) + fneq[5]) + fneq[6]) + fneq[7]) + fneq[8];
    float fb[9];
    feq_shifted(w, drb, U, V, fb);
    const float third = 1.0f / 3.0f;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const float cx = (float)cxk(k), cy = (float)cyk(k);
        const float Qxx = cx * cx - third, Qxy = cx * cy, Qyy = cy * cy - third;
        a.set(ib, jb, k, fb[k] + 1.5f * w[k] * (Qxx * Pxx + 2.0f * Qxy * Pxy + Qyy * Pyy));
    }
}

// One point t of one Boundary entry (the FP32 counterpart of bc_apply).
// v1 / v2 are the entry's FP64 values at t; pressure values enter as
// rho - 1, formed in FP64.
template <class A>
__device__ __forceinline__ void bc_apply_s(A &a, const float w[9], int kind, int Nx, int Ny, int index, int t,
                                           double v1, double v2) {
    if (kind == BC_PERIODIC_X || kind == BC_PERIODIC_Y) {
        // src/bc/periodic_x.c:19-50 / periodic_y.c:19-50
        if (kind == BC_PERIODIC_X) {
            const int j = t % Ny;
            const bool left = t < Ny;
            const int i = left ? 0 : Nx - 1;
            if (a.solid(i, j)) return;
#pragma unroll
            for (int k = 1; k < 9; k++) {
                const int cx = cxk(k);
                if (left ? cx <= 0 : cx >= 0) continue;
                const int is = left ? Nx - cx : -cx - 1;
                const int js = j - cyk(k);
                if (js < 0 || js >= Ny) continue;
                if (a.solid(is, js)) continue;
                a.set(i, j, k, a.post(is, js, k));
            }
        } else {
            const int i = t % Nx;
            const bool bottom = t < Nx;
            const int j = bottom ? 0 : Ny - 1;
            if (a.solid(i, j)) return;
#pragma unroll
            for (int k = 1; k < 9; k++) {
                const int cy = cyk(k);
                if (bottom ? cy <= 0 : cy >= 0) continue;
                const int js = bottom ? Ny - cy : -cy - 1;
                const int is = i - cxk(k);
                if (is < 0 || is >= Nx) continue;
                if (a.solid(is, js)) continue;
                a.set(i, j, k, a.post(is, js, k));
            }
        }
        return;
    }
    int ib, jb;
    if (bc_is_column(kind)) { ib = index; jb = t; } else { ib = t; jb = index; }
    if (a.solid(ib, jb)) return;
    const float c23 = 2.0f / 3.0f, c16 = 1.0f / 6.0f;
    switch (kind) {
    case BC_VEL_IN_ZH: {  // src/bc/velocity_inlet.c:25-39
        const float U = (float)v1, V = (float)v2;
        const float g0 = a.get(ib, jb, 0), g2 = a.get(ib, jb, 2), g3 = a.get(ib, jb, 3),
                    g4 = a.get(ib, jb, 4), g6 = a.get(ib, jb, 6), g7 = a.get(ib, jb, 7);
        const float r = (1.0f + (g0 + g2 + g4 + 2.0f * (g3 + g6 + g7))) / (1.0f - U);
        a.set(ib, jb, 1, g3 + c23 * r * U);
        a.set(ib, jb, 5, g7 + c16 * r * U - 0.5f * (g2 - g4) + 0.5f * r * V);
        a.set(ib, jb, 8, g6 + c16 * r * U + 0.5f * (g2 - g4) - 0.5f * r * V);
    } break;
    case BC_VEL_OUT_ZH: {  // src/bc/velocity_outlet.c:25-39
        const float U = (float)v1, V = (float)v2;
        const float g0 = a.get(ib, jb, 0), g2 = a.get(ib, jb, 2), g4 = a.get(ib, jb, 4),
                    g1 = a.get(ib, jb, 1), g5 = a.get(ib, jb, 5), g8 = a.get(ib, jb, 8);
        const float r = (1.0f + (g0 + g2 + g4 + 2.0f * (g1 + g5 + g8))) / (1.0f + U);
        a.set(ib, jb, 3, g1 - c23 * r * U);
        a.set(ib, jb, 6, g8 - 0.5f * (g2 - g4) - c16 * r * U + 0.5f * r * V);
        a.set(ib, jb, 7, g5 + 0.5f * (g2 - g4) - c16 * r * U - 0.5f * r * V);
    } break;
    case BC_VEL_TOP_ZH: {  // src/bc/velocity_top.c:25-39
        const float U = (float)v1, V = (float)v2;
        const float g0 = a.get(ib, jb, 0), g1 = a.get(ib, jb, 1), g2 = a.get(ib, jb, 2),
                    g3 = a.get(ib, jb, 3), g5 = a.get(ib, jb, 5), g6 = a.get(ib, jb, 6);
        const float r = (1.0f + (g0 + g1 + g3 + 2.0f * (g2 + g5 + g6))) / (1.0f + V);
        a.set(ib, jb, 4, g2 - c23 * r * V);
        a.set(ib, jb, 7, g5 + 0.5f * (g1 - g3) - 0.5f * r * U - c16 * r * V);
        a.set(ib, jb, 8, g6 - 0.5f * (g1 - g3) + 0.5f * r * U - c16 * r * V);
    } break;
    case BC_VEL_BOT_ZH:      // src/bc/velocity_bottom.c:25-39 (second write to 7 kept, :39)
    case BC_VEL_BOT_ZH_FIX: {  // the same, the last line written to 6
        const float U = (float)v1, V = (float)v2;
        const float g0 = a.get(ib, jb, 0), g1 = a.get(ib, jb, 1), g3 = a.get(ib, jb, 3),
                    g4 = a.get(ib, jb, 4), g7 = a.get(ib, jb, 7), g8 = a.get(ib, jb, 8);
        const float r = (1.0f + (g0 + g1 + g3 + 2.0f * (g4 + g7 + g8))) / (1.0f - V);
        a.set(ib, jb, 2, g4 + c23 * r * V);
        a.set(ib, jb, 5, g7 - 0.5f * (g1 - g3) + 0.5f * r * U + c16 * r * V);
        a.set(ib, jb, kind == BC_VEL_BOT_ZH_FIX ? 6 : 7, g8 + 0.5f * (g1 - g3) - 0.5f * r * U + c16 * r * V);
    } break;
    case BC_PRES_IN_ZH: {  // src/bc/pressure_inlet.c:25-39
        const float R = (float)v1, dR = (float)(v1 - 1.0);
        const float g0 = a.get(ib, jb, 0), g2 = a.get(ib, jb, 2), g4 = a.get(ib, jb, 4),
                    g3 = a.get(ib, jb, 3), g6 = a.get(ib, jb, 6), g7 = a.get(ib, jb, 7);
        // U = 1 - (1 + G) / R = (dR - G) / R
        const float U = (dR - (g0 + g2 + g4 + 2.0f * (g3 + g6 + g7))) / R;
        const float V = a.uy(ib + 1, jb);
        a.set(ib, jb, 1, g3 + c23 * R * U);
        a.set(ib, jb, 5, g7 + c16 * R * U - 0.5f * (g2 - g4) + 0.5f * R * V);
        a.set(ib, jb, 8, g6 + c16 * R * U + 0.5f * (g2 - g4) - 0.5f * R * V);
    } break;
    case BC_PRES_OUT_ZH: {  // src/bc/pressure_outlet.c:25-39
        const float R = (float)v1, dR = (float)(v1 - 1.0);
        const float g0 = a.get(ib, jb, 0), g2 = a.get(ib, jb, 2), g4 = a.get(ib, jb, 4),
                    g1 = a.get(ib, jb, 1), g5 = a.get(ib, jb, 5), g8 = a.get(ib, jb, 8);
        // U = (1 + G) / R - 1 = (G - dR) / R
        const float U = ((g0 + g2 + g4 + 2.0f * (g1 + g5 + g8)) - dR) / R;
        const float V = a.uy(ib - 1, jb);
        a.set(ib, jb, 3, g1 - c23 * R * U);
        a.set(ib, jb, 6, g8 - 0.5f * (g2 - g4) - c16 * R * U + 0.5f * R * V);
        a.set(ib, jb, 7, g5 + 0.5f * (g2 - g4) - c16 * R * U - 0.5f * R * V);
    } break;
    case BC_CONV_IN:  // src/bc/convective_inlet.c:20-28
#pragma unroll
        for (int k = 0; k < 9; k++) a.set(ib, jb, k, a.get(ib + 1, jb, k));
        break;
    case BC_CONV_OUT:  // src/bc/convective_outlet.c:20-28
#pragma unroll
        for (int k = 0; k < 9; k++) a.set(ib, jb, k, a.get(ib - 1, jb, k));
        break;
    case BC_VEL_IN_REG: bc_regularized_s(a, w, ib, jb, ib + 1, jb, false, (float)v1, (float)v2); break;
    case BC_VEL_OUT_REG: bc_regularized_s(a, w, ib, jb, ib - 1, jb, false, (float)v1, (float)v2); break;
    case BC_VEL_BOT_REG: bc_regularized_s(a, w, ib, jb, ib, jb + 1, false, (float)v1, (float)v2); break;
    case BC_VEL_TOP_REG: bc_regularized_s(a, w, ib, jb, ib, jb - 1, false, (float)v1, (float)v2); break;
    case BC_PRES_IN_REG: bc_regularized_s(a, w, ib, jb, ib + 1, jb, true, (float)(v1 - 1.0), 0.f); break;
    case BC_PRES_OUT_REG: bc_regularized_s(a, w, ib, jb, ib - 1, jb, true, (float)(v1 - 1.0), 0.f); break;
    case BC_PRES_BOT_REG: bc_regularized_s(a, w, ib, jb, ib, jb + 1, true, (float)(v1 - 1.0), 0.f); break;
    case BC_PRES_TOP_REG: bc_regularized_s(a, w, ib, jb, ib, jb - 1, true, (float)(v1 - 1.0), 0.f); break;
    default: break;
    }
}

}  // namespace lbm
