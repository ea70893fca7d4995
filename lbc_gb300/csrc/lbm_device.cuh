// lbm_device.cuh -- shared device-side definitions of the D2Q9 engine.
//
// Populations live on the device as structure-of-arrays planes: population k of
// node (i, j) is at plane k, offset j * pitch + i. lbc's own ordering of the
// velocity set is the canonical one (cases/nit/nit.c:195-202):
//   c = (0,0) (1,0) (0,1) (-1,0) (0,-1) (1,1) (-1,1) (-1,-1) (1,-1), opp = 0 3 4 1 2 7 8 5 6.
#pragma once
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

namespace lbm {

constexpr int Q = 9;

__host__ __device__ constexpr int cxk(int k) {
    return k == 1 || k == 5 || k == 8 ? 1 : (k == 3 || k == 6 || k == 7 ? -1 : 0);
}
__host__ __device__ constexpr int cyk(int k) {
    return k == 2 || k == 5 || k == 6 ? 1 : (k == 4 || k == 7 || k == 8 ? -1 : 0);
}
__host__ __device__ constexpr int oppk(int k) {
    return k == 0 ? 0 : (k <= 4 ? ((k + 1) % 4) + 1 : ((k - 5 + 2) % 4) + 5);
}
static_assert(oppk(1) == 3 && oppk(2) == 4 && oppk(3) == 1 && oppk(4) == 2, "opp");
static_assert(oppk(5) == 7 && oppk(6) == 8 && oppk(7) == 5 && oppk(8) == 6, "opp");

// Per-node flag word (uint16), built once per geometry on the host.
enum : uint16_t {
    NF_SPECIAL_MASK = 0x01FF,  // bit k: the pull source x - c_k is solid or off a non-periodic edge
    NF_SOLID = 1u << 9,        // node is solid (never written)
    NF_BAND = 1u << 10,        // node's pre-collision populations feed the edge-BC pipeline
    NF_BCW = 1u << 11,         // node is written by an edge BC (collided by the stage launch)
    NF_LINKS = 1u << 12,       // node owns entries in the cut-link table (IBB / moving wall)
};

// One wall link entry, in the order of the node's special solid sources.
enum : uint8_t { LINK_BB = 0, LINK_IBB_LO = 1, LINK_IBB_HI = 2, LINK_MOVING = 3 };
struct Link {
    double c1, c2;   // interpolation weights (IBB) or wall term (moving wall: c2)
    int64_t behind;  // plane offset of the behind node x + c_k' (IBB), else -1
    uint8_t mode;
    uint8_t k;       // pulled population
    uint8_t pad[6];
};
static_assert(sizeof(Link) == 32, "Link layout");

// Edge-BC kinds (lbc's 18 BC functions that act on populations, then the
// extensions this library adds).
enum BCKind : int {
    BC_VEL_IN_ZH = 0, BC_VEL_OUT_ZH, BC_VEL_TOP_ZH, BC_VEL_BOT_ZH,
    BC_PRES_IN_ZH, BC_PRES_OUT_ZH,
    BC_CONV_IN, BC_CONV_OUT,
    BC_PERIODIC_X, BC_PERIODIC_Y,
    BC_VEL_IN_REG, BC_VEL_OUT_REG, BC_VEL_TOP_REG, BC_VEL_BOT_REG,
    BC_PRES_IN_REG, BC_PRES_OUT_REG, BC_PRES_TOP_REG, BC_PRES_BOT_REG,
    // velocity_bottom with the Zou-He closure written to population 6 (lbc's
    // src/bc/velocity_bottom.c:39 writes 7 a second time and leaves 6 as
    // streamed); an extension, opt-in by function (velocity_bottom_corrected)
    BC_VEL_BOT_ZH_FIX,
    BC_KIND_COUNT
};

// Impedance wall (time-domain impedance BC): per wall node of a bottom
// regularized entry, a mass-spring-damper m v' + R v + K x = p' advanced once
// per step with the exact zero-order-hold update of the 2x2 system, plus
// running DFTs of p' and v at nf frequencies for eduction. Layout: field-major
// [IMP_FIELDS + 4 nf][along] doubles, then the wall's phasor table: two slots
// (the step's band parity selects the one read; the other is written for the
// next step) of imp_tab_stride(nf) doubles: the window phasor (cos, sin of
// 2 pi n / window length), then e^{-i w_f n} (re, im) per frequency. Every
// node of a wall rotates the same phasors from the same start, so one copy
// per wall serves them all (and spares each node the rotations' FP64 work).
enum : int {
    IMP_ACTIVE = 0, IMP_A11, IMP_A12, IMP_A21, IMP_A22, IMP_B1, IMP_B2, IMP_X, IMP_V, IMP_RHOBAR,
    IMP_P,           // the pressure fluctuation p' of the last update (for the wall's trace)
    IMP_FIELDS
};
// per frequency f: sum p' e^{-i w n} (re, im), sum v e^{-i w n} (re, im)
__host__ __device__ inline int imp_field(int f, int q) { return IMP_FIELDS + 4 * f + q; }
__host__ __device__ inline int imp_tab_stride(int nf) { return 2 + 2 * nf; }
// Offset of the phasor table's slot `slot` in a wall's array; imp_doubles is
// the array's size.
__host__ __device__ inline size_t imp_tab_offset(int nf, int along, int slot) {
    return (size_t)(IMP_FIELDS + 4 * nf) * (size_t)along + (size_t)slot * imp_tab_stride(nf);
}
__host__ __device__ inline size_t imp_doubles(int nf, int along) { return imp_tab_offset(nf, along, 2); }

__host__ __device__ inline bool bc_is_column(int kind) {
    return kind == BC_VEL_IN_ZH || kind == BC_VEL_OUT_ZH || kind == BC_PRES_IN_ZH ||
           kind == BC_PRES_OUT_ZH || kind == BC_CONV_IN || kind == BC_CONV_OUT ||
           kind == BC_VEL_IN_REG || kind == BC_VEL_OUT_REG || kind == BC_PRES_IN_REG ||
           kind == BC_PRES_OUT_REG;
}

// Storage policies: FP64 stores f as is; FP32/FP16 store the shifted deviation
// g_k = f_k - w_k.
template <typename T> struct Store;
template <> struct Store<double> {
    static __device__ __forceinline__ double to_f64(double s, double) { return s; }
    static __device__ __forceinline__ double from_f64(double f, double) { return f; }
};
template <> struct Store<float> {
    static __device__ __forceinline__ double to_f64(float s, double w) { return (double)s + w; }
    static __device__ __forceinline__ float from_f64(double f, double w) { return (float)(f - w); }
};
template <> struct Store<__half> {
    static __device__ __forceinline__ double to_f64(__half s, double w) { return (double)__half2float(s) + w; }
    static __device__ __forceinline__ __half from_f64(double f, double w) { return __float2half_rn((float)(f - w)); }
};

// ---------------------------------------------------------------------------
// Exact FP64 arithmetic in lbc's operation order. The translation units that use
// these are compiled with --fmad=false, so no multiply-add is contracted.

// Moments of one node, src/core/compute_macroscopic_fields.c:23-41. The k-ordered
// sums with integer velocities reduce to these add chains (x + (+-0) == x).
__device__ __forceinline__ void moments_exact(const double f[9], double hFx, double hFy,
                                              double &rho, double &ux, double &uy) {
    double s = ((((((((f[0] + f[1]) + f[2]) + f[3]) + f[4]) + f[5]) + f[6]) + f[7]) + f[8]);
    double sx = ((((f[1] - f[3]) + f[5]) - f[6]) - f[7]) + f[8];
    double sy = ((((f[2] - f[4]) + f[5]) + f[6]) - f[7]) - f[8];
    if (s < 1e-16) s = 1e-16;
    rho = s;
    ux = (sx + hFx) / s;
    uy = (sy + hFy) / s;
}

// f_eq for the nine directions in the order of src/core/collision.c:31-32.
__device__ __forceinline__ void feq_exact(const double w[9], double rho, double ux, double uy,
                                          double feq[9]) {
    const double usq = ux * ux + uy * uy;
    const double t = 1.5 * usq;
    const double wr0 = w[0] * rho, wr1 = w[1] * rho, wr2 = w[2] * rho, wr3 = w[3] * rho,
                 wr4 = w[4] * rho, wr5 = w[5] * rho, wr6 = w[6] * rho, wr7 = w[7] * rho,
                 wr8 = w[8] * rho;
    feq[0] = wr0 * (1.0 - t);
    {
        const double c = ux, B = 3.0 * c, A = (4.5 * c) * c;
        feq[1] = wr1 * (((1.0 + B) + A) - t);
        feq[3] = wr3 * (((1.0 - B) + A) - t);
    }
    {
        const double c = uy, B = 3.0 * c, A = (4.5 * c) * c;
        feq[2] = wr2 * (((1.0 + B) + A) - t);
        feq[4] = wr4 * (((1.0 - B) + A) - t);
    }
    {
        const double c = ux + uy, B = 3.0 * c, A = (4.5 * c) * c;
        feq[5] = wr5 * (((1.0 + B) + A) - t);
        feq[7] = wr7 * (((1.0 - B) + A) - t);
    }
    {
        const double c = uy - ux, B = 3.0 * c, A = (4.5 * c) * c;
        feq[6] = wr6 * (((1.0 + B) + A) - t);
        feq[8] = wr8 * (((1.0 - B) + A) - t);
    }
}

// BGK + Guo forcing in place, src/core/collision.c:24-38.
__device__ __forceinline__ void collide_exact(double f[9], const double w[9], double rho, double ux,
                                              double uy, double om, bool force, double Fx,
                                              double Fy) {
    double feq[9];
    feq_exact(w, rho, ux, uy, feq);
    if (!force) {
#pragma unroll
        for (int k = 0; k < 9; k++) f[k] = f[k] + (-om * (f[k] - feq[k]));
        return;
    }
    const double uF = ux * Fx + uy * Fy;
    const double g = 1 - 0.5 * om;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int cx = cxk(k), cy = cyk(k);
        const double cu = cx * ux + cy * uy;
        const double cF = cx * Fx + cy * Fy;
        const double Fk = w[k] * (3.0 * cF + 9.0 * cu * cF - 3.0 * uF);
        f[k] = f[k] + (-om * (f[k] - feq[k]) + g * Fk);
    }
}

// ---------------------------------------------------------------------------
// FP64 with fused multiply-adds and the D2Q9 pair symmetry: the same physics
// as moments_exact / collide_exact (src/core/compute_macroscopic_fields.c:23-46,
// src/core/collision.c:24-38) in fewer FP64 instructions, rounded
// differently, so it agrees with lbc to rounding, not bit for bit. Over the
// 20,000 steps of the 256 x 64 channel both stay within 1e-12 of the same
// step in extended precision (lbc's own rounding: 3e-13 in u) and within about
// 1e-12 of each other in u and 1e-14 in rho. GB300 issues FP64 at about two
// lane operations per clock per SM, so on this part the FP64 step is bound by
// its FP64 instruction count, not by memory. Written with explicit fma()
// calls, which --fmad=false leaves alone.
//
// Needs lbc's weight symmetry: w1 = w2 = w3 = w4 (axes) and w5 = ... = w8
// (diagonals); the host checks it before choosing this arithmetic.

#ifdef __CUDACC__  // device-only: the host translation units see none of it
// 1/x by Newton-Raphson from the hardware's FP64 reciprocal seed (rcp.approx,
// relative error below 2^-20), finished with the third-order step
// r (1 + e + e^2), e = 1 - x r, whose error is about e^3: a result within an
// ulp or two of 1/x for the positive densities the step sees.
__device__ __forceinline__ double recip_fma(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    const double e = fma(-x, r, 1.0);
    return fma(r, fma(e, e, e), r);
}

// rho, (j + F / 2) / rho with shared partial sums: 14 additions for the three
// moments, one reciprocal, two multiplies.
__device__ __forceinline__ void moments_fma(const double f[9], double hFx, double hFy, bool force,
                                            double &rho, double &ux, double &uy) {
    const double a = (f[1] + f[5]) + f[8];   // c_x = +1
    const double b = (f[3] + f[6]) + f[7];   // c_x = -1
    const double c = (f[2] + f[5]) + f[6];   // c_y = +1
    const double d = (f[4] + f[7]) + f[8];   // c_y = -1
    double s = (((f[0] + f[2]) + f[4]) + a) + b;
    double jx = a - b, jy = c - d;
    if (force) { jx += hFx; jy += hFy; }
    // lbc's floor (compute_macroscopic_fields.c:27), compared on the bit
    // pattern: for doubles of either sign x < 1e-16 iff bits(x) < bits(1e-16)
    // as signed integers, which spares an FP64 compare.
    if (__double_as_longlong(s) < __double_as_longlong(1e-16)) s = 1e-16;
    rho = s;
    const double r = recip_fma(s);
    ux = jx * r;
    uy = jy * r;
}

// BGK collision, and with a body force Guo's term (1 - omega/2) w_k (3 c.F +
// 9 (c.u)(c.F) - 3 u.F), in lbc's relaxation form f' = f + (omega (f_eq - f)
// + G_k): f_eq - f is exact for populations near equilibrium (Sterbenz), so
// the only rounding at the populations' scale is the final addition, as in
// lbc (src/core/collision.c:36-37). That keeps the step's mass drift the one
// lbc's own FP64 run has (from the weights' FP64 sum), which a form
// (1 - omega) f + omega f_eq would change. f_eq of an opposite pair
// (k, opp k), cu = c_k . u, is E +- O: even part E = w rho (1 - 1.5 u.u +
// 4.5 cu^2), odd part O = 3 w rho cu; the forcing term splits the same way
// into g w (9 cu cF - 3 u.F) and 3 g w cF.
__device__ __forceinline__ void collide_fma(double f[9], double w0, double wa, double wd, double rho,
                                            double ux, double uy, double om, bool force, double Fx,
                                            double Fy) {
    const double base = fma(-1.5, fma(ux, ux, uy * uy), 1.0);
    const double wra = wa * rho, wrd = wd * rho;
    const double Ba = wra * base, Bd = wrd * base;      // even part, constant term
    const double Ca = 4.5 * wra, Cd = 4.5 * wrd;        // even part, c.u squared
    const double Da = 3.0 * wra, Dd = 3.0 * wrd;        // odd part
    const double B0 = (w0 * rho) * base;
    const double u5 = ux + uy, u6 = uy - ux;
    if (!force) {
        auto pair = [&](double &fp, double &fm, double cu, double B, double C, double D) {
            const double E = fma(C * cu, cu, B);
            const double O = D * cu;
            fp = fma(om, (E + O) - fp, fp);
            fm = fma(om, (E - O) - fm, fm);
        };
        f[0] = fma(om, B0 - f[0], f[0]);
        pair(f[1], f[3], ux, Ba, Ca, Da);
        pair(f[2], f[4], uy, Ba, Ca, Da);
        pair(f[5], f[7], u5, Bd, Cd, Dd);
        pair(f[6], f[8], u6, Bd, Cd, Dd);
        return;
    }
    const double g = fma(-0.5, om, 1.0);
    const double ga = g * wa, gd = g * wd;
    const double uF = fma(ux, Fx, uy * Fy);
    const double ga9 = 9.0 * ga, gd9 = 9.0 * gd, ga3 = 3.0 * ga, gd3 = 3.0 * gd;
    const double Ga = -ga3 * uF, Gd = -gd3 * uF;        // even forcing, constant term
    f[0] = f[0] + fma(om, B0 - f[0], (-3.0 * (g * w0)) * uF);
    const double F5 = Fx + Fy, F6 = Fy - Fx;
    auto pair = [&](double &fp, double &fm, double cu, double P, double Qo, double B, double C, double D,
                    double G) {
        const double E = fma(C * cu, cu, B);
        const double O = D * cu;
        const double GE = fma(P, cu, G);
        fp = fp + fma(om, (E + O) - fp, GE + Qo);
        fm = fm + fma(om, (E - O) - fm, GE - Qo);
    };
    pair(f[1], f[3], ux, ga9 * Fx, ga3 * Fx, Ba, Ca, Da, Ga);
    pair(f[2], f[4], uy, ga9 * Fy, ga3 * Fy, Ba, Ca, Da, Ga);
    pair(f[5], f[7], u5, gd9 * F5, gd3 * F5, Bd, Cd, Dd, Gd);
    pair(f[6], f[8], u6, gd9 * F6, gd3 * F6, Bd, Cd, Dd, Gd);
}
#endif  // __CUDACC__

// ---------------------------------------------------------------------------
// Edge BCs, generic over an accessor that reads/writes the current f_new of a
// node, the previous-step moments and (periodic only) the post-collision f.
// Accessor interface:
//   double get(int i, int j, int k); void set(int i, int j, int k, double v);
//   double rho(int i, int j), ux(...), uy(...);          previous-step fields
//   double post(int i, int j, int k);                    post-collision f
//   bool solid(int i, int j);

// Regularized node update shared by the eight *_regularized files
// (src/bc/velocity_inlet_regularized.c:26-70).
template <class A>
__device__ __forceinline__ void bc_regularized(A &a, const double w[9], int ib, int jb, int in,
                                               int jn, bool pressure, double val1, double val2) {
    const double rho_n = a.rho(in, jn), u_n = a.ux(in, jn), v_n = a.uy(in, jn);
    double rho_b, U, V;
    if (pressure) {
        rho_b = val1; U = u_n; V = v_n;
    } else {
        rho_b = rho_n; U = val1; V = val2;
    }
    double feq[9];
    feq_exact(w, rho_n, u_n, v_n, feq);
    double fneq[9];
#pragma unroll
    for (int k = 0; k < 9; k++) fneq[k] = a.get(in, jn, k) - feq[k];
    // Pi sums in k order; terms with a zero coefficient add +-0 (no effect).
    const double Pxx = ((((fneq[1] + fneq[3]) + fneq[5]) + fneq[6]) + fneq[7]) + fneq[8];
    const double Pxy = ((fneq[5] - fneq[6]) + fneq[7]) - fneq[8];
    const double Pyy = ((((fneq[2] + fneq[4]) + fneq[5]) + fneq[6]) + fneq[7]) + fneq[8];
    double fb[9];
    feq_exact(w, rho_b, U, V, fb);
    const double third = 1.0 / 3.0;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int cx = cxk(k), cy = cyk(k);
        const double Qxx = cx * cx - third;
        const double Qxy = cx * cy;
        const double Qyy = cy * cy - third;
        const double fr = (3.0 / 2.0) * w[k] * (Qxx * Pxx + 2.0 * Qxy * Pxy + Qyy * Pyy);
        a.set(ib, jb, k, fb[k] + fr);
    }
}

// One step of the impedance wall at position t of the line (FP64): pressure
// fluctuation p' = c_s^2 (rho_n - rhobar) from the previous-step density of the
// interior neighbour and the node's running mean density rhobar (an
// exponential average with rate alpha; alpha = 0 keeps the fixed reference the
// wall was set up with), state (x, v) <- A (x, v) + b p', DFT accumulation,
// and the wall-normal velocity into the liner returned (the BC imposes
// u_y = -v).
// The DFT sums are weighted by a Hann window over the eduction length
// (weight 0.5 (1 - cos(2 pi n / L)) from the window phasor; no window when
// the wall was set up without a length). tab: this step's slot of the wall's
// phasor table.
// FMA: the update with fused multiply-adds and p' = (rho - rho_bar) * (1/3)
// (about half the FP64 instructions: shifted storage, whose populations are
// FP32 or FP16 anyway); otherwise the oracle's sequence, bit for bit (FP64
// storage).
template <bool FMA = false>
__device__ __forceinline__ double impedance_step(double *imp, int along, int nf, int t, double rho_n,
                                                 double alpha, const double *tab, int windowed) {
#define IMP(f) imp[(size_t)(f) * along + t]
    // The fields share one array, so the compiler cannot move a load above an
    // earlier store to it: all loads of a group are issued before its stores
    // (the node's state, then the DFT in groups of four frequencies), which
    // keeps the chain to a few memory latencies. The arithmetic is the same
    // sequence as a field-by-field update.
    const double rb = IMP(IMP_RHOBAR);
    const double x = IMP(IMP_X), v = IMP(IMP_V);
    const double a11 = IMP(IMP_A11), a12 = IMP(IMP_A12), b1 = IMP(IMP_B1);
    const double a21 = IMP(IMP_A21), a22 = IMP(IMP_A22), b2 = IMP(IMP_B2);
    const double wc0 = tab[0];
    double cr[4], ci[4], ac[4][4];
    auto load_group = [&](int f0) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (f0 + q >= nf) break;
            cr[q] = tab[2 + 2 * (f0 + q)];
            ci[q] = tab[3 + 2 * (f0 + q)];
#pragma unroll
            for (int m = 0; m < 4; m++) ac[q][m] = IMP(imp_field(f0 + q, m));
        }
    };
    load_group(0);
    const double d = rho_n - rb;
    const double p = FMA ? d * (1.0 / 3.0) : d / 3.0;
    const double win = windowed ? 0.5 * (1.0 - wc0) : 1.0;
    IMP(IMP_RHOBAR) = FMA ? fma(alpha, d, rb) : rb + alpha * d;
    IMP(IMP_P) = p;
    const double xn = FMA ? fma(a11, x, fma(a12, v, b1 * p)) : a11 * x + a12 * v + b1 * p;
    const double vn = FMA ? fma(a21, x, fma(a22, v, b2 * p)) : a21 * x + a22 * v + b2 * p;
    IMP(IMP_X) = xn;
    IMP(IMP_V) = vn;
    const double wp = win * p, wv = win * vn;
    for (int f0 = 0; f0 < nf; f0 += 4) {
        if (f0 > 0) load_group(f0);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int f = f0 + q;
            if (f >= nf) break;
            IMP(imp_field(f, 0)) = FMA ? fma(wp, cr[q], ac[q][0]) : ac[q][0] + wp * cr[q];
            IMP(imp_field(f, 1)) = FMA ? fma(wp, ci[q], ac[q][1]) : ac[q][1] + wp * ci[q];
            IMP(imp_field(f, 2)) = FMA ? fma(wv, cr[q], ac[q][2]) : ac[q][2] + wv * cr[q];
            IMP(imp_field(f, 3)) = FMA ? fma(wv, ci[q], ac[q][3]) : ac[q][3] + wv * ci[q];
        }
    }
    return vn;
#undef IMP
}

// The wall's phasors one step on: from this step's slot `cur` into the other
// slot `next` (window phasor rotated by 2 pi / length, e^{-i w_f n} by
// e^{-i w_f}). One thread per wall per step.
__device__ __forceinline__ void impedance_advance(const double *cur, double *next, int nf, const double *cw,
                                                  const double *sw, double wcos, double wsin, int windowed) {
    const double wc0 = cur[0], ws0 = cur[1];
    if (windowed) {
        next[0] = wc0 * wcos - ws0 * wsin;
        next[1] = ws0 * wcos + wc0 * wsin;
    } else {
        next[0] = wc0;
        next[1] = ws0;
    }
    for (int f = 0; f < nf; f++) {
        const double cr = cur[2 + 2 * f], ci = cur[3 + 2 * f];
        next[2 + 2 * f] = cr * cw[f] + ci * sw[f];
        next[3 + 2 * f] = ci * cw[f] - cr * sw[f];
    }
}

template <class A>
__device__ __forceinline__ void bc_apply(A &a, const double w[9], int kind, int Nx, int Ny,
                                         int index, int t, double v1, double v2) {
    const bool col = bc_is_column(kind);
    int ib, jb;
    if (kind == BC_PERIODIC_X || kind == BC_PERIODIC_Y) {
        // src/bc/periodic_x.c:19-50 / periodic_y.c:19-50: t enumerates the two
        // edge lines (t < along: first edge, else second edge).
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
    if (col) { ib = index; jb = t; } else { ib = t; jb = index; }
    if (a.solid(ib, jb)) return;
    switch (kind) {
    case BC_VEL_IN_ZH: {  // src/bc/velocity_inlet.c:25-39
        const double U = v1, V = v2;
        const double f0 = a.get(ib, jb, 0), f2 = a.get(ib, jb, 2), f3 = a.get(ib, jb, 3),
                     f4 = a.get(ib, jb, 4), f6 = a.get(ib, jb, 6), f7 = a.get(ib, jb, 7);
        const double r = (f0 + f2 + f4 + 2.0 * (f3 + f6 + f7)) / (1.0 - U);
        a.set(ib, jb, 1, f3 + (2.0 / 3.0) * r * U);
        a.set(ib, jb, 5, f7 + (1.0 / 6.0) * r * U - 0.5 * (f2 - f4) + (1.0 / 2.0) * r * V);
        a.set(ib, jb, 8, f6 + (1.0 / 6.0) * r * U + 0.5 * (f2 - f4) - (1.0 / 2.0) * r * V);
    } break;
    case BC_VEL_OUT_ZH: {  // src/bc/velocity_outlet.c:25-39
        const double U = v1, V = v2;
        const double f0 = a.get(ib, jb, 0), f2 = a.get(ib, jb, 2), f4 = a.get(ib, jb, 4),
                     f1 = a.get(ib, jb, 1), f5 = a.get(ib, jb, 5), f8 = a.get(ib, jb, 8);
        const double r = (f0 + f2 + f4 + 2.0 * (f1 + f5 + f8)) / (1.0 + U);
        a.set(ib, jb, 3, f1 - (2.0 / 3.0) * r * U);
        a.set(ib, jb, 6, f8 - 0.5 * (f2 - f4) - (1.0 / 6.0) * r * U + (1.0 / 2.0) * r * V);
        a.set(ib, jb, 7, f5 + 0.5 * (f2 - f4) - (1.0 / 6.0) * r * U - (1.0 / 2.0) * r * V);
    } break;
    case BC_VEL_TOP_ZH: {  // src/bc/velocity_top.c:25-39
        const double U = v1, V = v2;
        const double f0 = a.get(ib, jb, 0), f1 = a.get(ib, jb, 1), f2 = a.get(ib, jb, 2),
                     f3 = a.get(ib, jb, 3), f5 = a.get(ib, jb, 5), f6 = a.get(ib, jb, 6);
        const double r = (f0 + f1 + f3 + 2 * (f2 + f5 + f6)) / (1 + V);
        a.set(ib, jb, 4, f2 - 2.0 / 3.0 * r * V);
        a.set(ib, jb, 7, f5 + (f1 - f3) / 2.0 - 0.5 * r * U - 1.0 / 6.0 * r * V);
        a.set(ib, jb, 8, f6 - (f1 - f3) / 2.0 + 0.5 * r * U - 1.0 / 6.0 * r * V);
    } break;
    case BC_VEL_BOT_ZH:      // src/bc/velocity_bottom.c:25-39 (second write to 7 kept, :39)
    case BC_VEL_BOT_ZH_FIX: {  // the same, the last line written to 6
        const double U = v1, V = v2;
        const double f0 = a.get(ib, jb, 0), f1 = a.get(ib, jb, 1), f3 = a.get(ib, jb, 3),
                     f4 = a.get(ib, jb, 4), f7 = a.get(ib, jb, 7), f8 = a.get(ib, jb, 8);
        const double r = (f0 + f1 + f3 + 2 * (f4 + f7 + f8)) / (1 - V);
        a.set(ib, jb, 2, f4 + 2.0 / 3.0 * r * V);
        a.set(ib, jb, 5, f7 - (f1 - f3) / 2.0 + 0.5 * r * U + 1.0 / 6.0 * r * V);
        a.set(ib, jb, kind == BC_VEL_BOT_ZH_FIX ? 6 : 7, f8 + (f1 - f3) / 2.0 - 0.5 * r * U + 1.0 / 6.0 * r * V);
    } break;
    case BC_PRES_IN_ZH: {  // src/bc/pressure_inlet.c:25-39
        const double R = v1;
        const double f0 = a.get(ib, jb, 0), f2 = a.get(ib, jb, 2), f4 = a.get(ib, jb, 4),
                     f3 = a.get(ib, jb, 3), f6 = a.get(ib, jb, 6), f7 = a.get(ib, jb, 7);
        const double U = 1.0 - (f0 + f2 + f4 + 2.0 * (f3 + f6 + f7)) / R;
        const double V = a.uy(ib + 1, jb);
        a.set(ib, jb, 1, f3 + (2.0 / 3.0) * R * U);
        a.set(ib, jb, 5, f7 + (1.0 / 6.0) * R * U - 0.5 * (f2 - f4) + (1.0 / 2.0) * R * V);
        a.set(ib, jb, 8, f6 + (1.0 / 6.0) * R * U + 0.5 * (f2 - f4) - (1.0 / 2.0) * R * V);
    } break;
    case BC_PRES_OUT_ZH: {  // src/bc/pressure_outlet.c:25-39
        const double R = v1;
        const double f0 = a.get(ib, jb, 0), f2 = a.get(ib, jb, 2), f4 = a.get(ib, jb, 4),
                     f1 = a.get(ib, jb, 1), f5 = a.get(ib, jb, 5), f8 = a.get(ib, jb, 8);
        const double U = (f0 + f2 + f4 + 2.0 * (f1 + f5 + f8)) / R - 1.0;
        const double V = a.uy(ib - 1, jb);
        a.set(ib, jb, 3, f1 - (2.0 / 3.0) * R * U);
        a.set(ib, jb, 6, f8 - 0.5 * (f2 - f4) - (1.0 / 6.0) * R * U + (1.0 / 2.0) * R * V);
        a.set(ib, jb, 7, f5 + 0.5 * (f2 - f4) - (1.0 / 6.0) * R * U - (1.0 / 2.0) * R * V);
    } break;
    case BC_CONV_IN:  // src/bc/convective_inlet.c:20-28
#pragma unroll
        for (int k = 0; k < 9; k++) a.set(ib, jb, k, a.get(ib + 1, jb, k));
        break;
    case BC_CONV_OUT:  // src/bc/convective_outlet.c:20-28
#pragma unroll
        for (int k = 0; k < 9; k++) a.set(ib, jb, k, a.get(ib - 1, jb, k));
        break;
    case BC_VEL_IN_REG: bc_regularized(a, w, ib, jb, ib + 1, jb, false, v1, v2); break;
    case BC_VEL_OUT_REG: bc_regularized(a, w, ib, jb, ib - 1, jb, false, v1, v2); break;
    case BC_VEL_BOT_REG: bc_regularized(a, w, ib, jb, ib, jb + 1, false, v1, v2); break;
    case BC_VEL_TOP_REG: bc_regularized(a, w, ib, jb, ib, jb - 1, false, v1, v2); break;
    case BC_PRES_IN_REG: bc_regularized(a, w, ib, jb, ib + 1, jb, true, v1, 0.0); break;
    case BC_PRES_OUT_REG: bc_regularized(a, w, ib, jb, ib - 1, jb, true, v1, 0.0); break;
    case BC_PRES_BOT_REG: bc_regularized(a, w, ib, jb, ib, jb + 1, true, v1, 0.0); break;
    case BC_PRES_TOP_REG: bc_regularized(a, w, ib, jb, ib, jb - 1, true, v1, 0.0); break;
    default: break;
    }
}

// ---------------------------------------------------------------------------
// Kernel parameter blocks (plain structs, passed by value).

struct StepParams {
    int Nx, Ny, pitch;
    int px, py;
    long long plane;          // pitch * Ny
    const void *src;          // post-collision populations of step n (planes)
    void *dst;                // output populations (also holds the stale slots)
    const uint16_t *flags;    // [Ny * pitch] or null (fully periodic, no solids, no BCs)
    const uint32_t *seg_clean; // bit per 64-node row segment whose 32 pairs are all clean; words per row: seg_words
    int seg_words;
    const int *link_off;      // [Ny * pitch]
    const Link *links;
    const double *omega;      // [Ny * Nx] per-node omega, or null -> omega0
    double omega0;
    int has_force;
    double Fx, Fy, hFx, hFy;  // hF = 0.5 F
    double w[9];
    // macroscopic output, dense [Ny * Nx]
    int write_macro;
    double *rho, *ux, *uy;
    // edge-BC band
    const int *colbase, *rowbase;
    int nslots;
    double *bandf;            // [9][nslots], pre-collision f_new of band nodes (FP64 storage)
    float *bandg;             // [9][nslots], the same as g = f - w (shifted storage)
    double *bandm_next;       // [3][nslots], their moments (for the next step's BCs)
    // momentum-exchange force (null when the geometry has no wall links).
    // FP64 storage: every 32-node row segment (j, i / 32) that contains wall
    // links has a slot (seg_slot >= 0, numbered in row-major order from the
    // geometry); the warp that steps it stores its sum at mem_partials[2 *
    // slot]. Shifted storage: wall-link nodes are special nodes, stepped from
    // the case's special-node list, and every 32-entry chunk of that list
    // that contains links has a slot (chunk_slot[chunk] >= 0). k_force_reduce
    // adds the slots up in order. Neither depends on the block or tile shape,
    // nor on whether the case runs alone or in a batch.
    double *mem_partials;
    const int *seg_slot;      // [Ny][(Nx + 31) / 32] (FP64 storage)
    const int *chunk_slot;    // [special list length / 32] (shifted storage)
};

struct FinishParams;

struct StageParams {
    int Nx, Ny, pitch;
    long long plane;
    int kind, index, along;
    const double *val1, *val2;
    double *imp;               // impedance-wall state or null
    int imp_nf;
    double imp_alpha;
    double imp_wcos, imp_wsin;     // window phasor rotation (2 pi / length)
    int imp_windowed;
    int imp_slot;                  // the phasor table slot this step reads (the step's band parity)
    double imp_cos[8], imp_sin[8];  // e^{-i w_f} per frequency
    const uint16_t *flags;
    const int *colbase, *rowbase;
    int nslots;
    double *bandf;             // FP64 storage
    float *bandg;              // shifted storage
    const double *bandm_prev;  // [3][nslots]
    const void *src;           // post-collision populations (periodic stages)
    double w[9];
    float wf[9];               // FP32 copies (shifted storage: no FP64 conversions per thread)
    // Finish in the same launch: the thread of a node whose last writer in
    // the Boundary list is this entry (last[slot] == entry) computes the
    // node's moments and collision right after the entry's BC.
    const short *last;
    int entry;
    const FinishParams *fin;   // batches: the case's finish parameters (solo: by value)
};

struct FinishParams {
    int Nx, Ny, pitch;
    long long plane;
    const int *colbase, *rowbase;
    int nslots;
    const double *bandf;       // FP64 storage
    const float *bandg;        // shifted storage
    double *bandm_next;
    void *dst;
    const double *omega;
    double omega0;
    int has_force;
    double Fx, Fy, hFx, hFy;
    double w[9];
    int write_macro;
    double *rho, *ux, *uy;
    // FP32 copies of the above (shifted storage)
    float wf[9];
    float omega0f, Fxf, Fyf, hFxf, hFyf;
};

// Special-node list entries (shifted storage): bit 30 of the column marks a
// solid node whose band values no BC reads, whose step only writes NaN
// moments on steps that write the fields (grids narrower than 2^30 columns).
constexpr int kSpecialSolid = 1 << 30;

// Both bases are loaded at once (rowbase[j] is in bounds whatever colbase[i]
// holds): one memory latency, not two dependent ones.
__device__ __forceinline__ int band_slot(const int *colbase, const int *rowbase, int i, int j) {
    const int c = colbase[i], r = rowbase[j];
    return c >= 0 ? c + j : r + i;
}

// The node that thread t of a Boundary entry works on (bc_apply's mapping:
// periodic entries enumerate both edge lines, t < along / 2 the first).
__device__ __forceinline__ int2 stage_node(int kind, int Nx, int Ny, int index, int t) {
    if (kind == BC_PERIODIC_X) return make_int2(t < Ny ? 0 : Nx - 1, t % Ny);
    if (kind == BC_PERIODIC_Y) return make_int2(t % Nx, t < Nx ? 0 : Ny - 1);
    return bc_is_column(kind) ? make_int2(index, t) : make_int2(t, index);
}

// The interior neighbour whose populations or moments a Boundary entry reads
// at node ij (the band's read lines), x = -1 for entries that read none.
__host__ __device__ __forceinline__ int2 stage_neighbour(int kind, int2 ij) {
    switch (kind) {
    case BC_PRES_IN_ZH: case BC_CONV_IN: case BC_VEL_IN_REG: case BC_PRES_IN_REG: return make_int2(ij.x + 1, ij.y);
    case BC_PRES_OUT_ZH: case BC_CONV_OUT: case BC_VEL_OUT_REG: case BC_PRES_OUT_REG: return make_int2(ij.x - 1, ij.y);
    case BC_VEL_BOT_REG: case BC_PRES_BOT_REG: return make_int2(ij.x, ij.y + 1);
    case BC_VEL_TOP_REG: case BC_PRES_TOP_REG: return make_int2(ij.x, ij.y - 1);
    default: return make_int2(-1, -1);
    }
}

// What stage thread t reads that the bulk kernel of the same step does not
// write: its node's solid flag and band slot, the neighbour's slot and
// previous-step moments, the entry's values at t, whether it finishes the
// node, and the impedance wall's update (which depends only on the
// neighbour's previous density and the wall's own state). Loaded before
// pdl_wait(), so that after the bulk kernel ends only the band populations,
// the BC arithmetic and the finish remain. The band accessors answer from it.
struct StagePre {
    int2 ij, nij;
    int slot, nslot;
    bool solid, fin, imp;
    double nrho, nux, nuy;
    double v1, v2;   // v2 = -(wall velocity) on impedance nodes (imp)
};

template <bool FMA = false>
__device__ __forceinline__ StagePre stage_preload(const StageParams &p, int t, int kind) {
    StagePre c;
    c.ij = stage_node(kind, p.Nx, p.Ny, p.index, t);
    c.nij = stage_neighbour(kind, c.ij);
    c.solid = (p.flags[(long long)c.ij.y * p.pitch + c.ij.x] & NF_SOLID) != 0;
    c.slot = band_slot(p.colbase, p.rowbase, c.ij.x, c.ij.y);
    c.nslot = 0;
    c.nrho = c.nux = c.nuy = 0.0;
    if (c.nij.x >= 0) {
        c.nslot = band_slot(p.colbase, p.rowbase, c.nij.x, c.nij.y);
        c.nrho = p.bandm_prev[c.nslot];
        c.nux = p.bandm_prev[(size_t)p.nslots + c.nslot];
        c.nuy = p.bandm_prev[2 * (size_t)p.nslots + c.nslot];
    }
    c.v1 = p.val1 ? p.val1[t] : 0.0;
    c.v2 = p.val2 ? p.val2[t] : 0.0;
    c.fin = !c.solid && p.last[c.slot] == p.entry;
    c.imp = false;
    if (kind == BC_VEL_BOT_REG && p.imp && t == 0)
        impedance_advance(p.imp + imp_tab_offset(p.imp_nf, p.along, p.imp_slot),
                          p.imp + imp_tab_offset(p.imp_nf, p.along, p.imp_slot ^ 1), p.imp_nf, p.imp_cos, p.imp_sin,
                          p.imp_wcos, p.imp_wsin, p.imp_windowed);
    if (kind == BC_VEL_BOT_REG && p.imp && p.imp[(size_t)IMP_ACTIVE * p.along + t] != 0.0 && !c.solid) {
        // Impedance wall on this node: the regularized bottom BC with the
        // normal velocity from the node's mass-spring-damper, advanced here,
        // before the stage waits for the bulk kernels (it depends only on the
        // previous step's moments). Batches did it once in a launch of its
        // own ahead of the special nodes: measured on 64 liner ducts, 195.4
        // vs 192.5 us per step here.
        c.v2 = -impedance_step<FMA>(p.imp, p.along, p.imp_nf, t, c.nrho, p.imp_alpha,
                               p.imp + imp_tab_offset(p.imp_nf, p.along, p.imp_slot), p.imp_windowed);
        c.imp = true;
    }
    return c;
}


}  // namespace lbm
