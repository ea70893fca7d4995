// kernels_shifted.cu -- fused step with populations stored as shifted deviations
// g_k = f_k - w_k in FP32 or FP16 and the collision done in FP32.
//
// Same pull structure as the exact FP64 step (kernels_exact.cu): stream, halfway /
// interpolated / moving-wall bounce-back, stale slots off non-periodic edges, MEM
// force, moments, BGK + Guo collision. Storing g instead of f keeps the relative
// precision of the small deviations from the rest state; FP64 is used only for the
// force reduction and the band values handed to the edge BCs.
#include <algorithm>
#include <cmath>

#include "bc_shifted.cuh"
#include "kernels.h"
#include "lbm_device.cuh"
#include "pdl.cuh"
#include "reduce.cuh"

namespace lbm {

template <typename T> struct SV;
// rnd: the value as the storage type would hold it. Pre-collision values that
// are computed rather than loaded (bounce-back interpolation, edge BCs) are
// rounded to the storage type before the collision, so a run split into
// chunks (whose boundaries store and reload them) gives the same bits.
// ld2 / st2: two adjacent nodes of one row (an even column: the pair is 8- or
// 4-byte aligned because the pitch and the planes are multiples of 64 nodes).
template <> struct SV<float> {
    static __device__ __forceinline__ float ld(const float *p) { return __ldg(p); }
    static __device__ __forceinline__ float ld_plain(const float *p) { return *p; }
    static __device__ __forceinline__ void st(float *p, float v) { *p = v; }
    static __device__ __forceinline__ float rnd(float v) { return v; }
    static __device__ __forceinline__ float2 ld2(const float *p) { return __ldg((const float2 *)p); }
    static __device__ __forceinline__ void st2(float *p, float2 v) { *(float2 *)p = v; }
};
template <> struct SV<__half> {
    static __device__ __forceinline__ float ld(const __half *p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ float ld_plain(const __half *p) { return __half2float(*p); }
    static __device__ __forceinline__ void st(__half *p, float v) { *p = __float2half_rn(v); }
    static __device__ __forceinline__ float rnd(float v) { return __half2float(__float2half_rn(v)); }
    static __device__ __forceinline__ float2 ld2(const __half *p) { return __half22float2(__ldg((const __half2 *)p)); }
    static __device__ __forceinline__ void st2(__half *p, float2 v) { *(__half2 *)p = __float22half2_rn(v); }
};

// ---------------------------------------------------------------- lane math
// The arithmetic of one node (float) or of two adjacent nodes at once (float2,
// Blackwell's packed FP32 instructions). Every operation is one correctly
// rounded IEEE operation with no contraction left to the compiler, so a node
// gets the same bits whichever form, kernel or launch shape computed it.
__device__ __forceinline__ float v_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float v_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float v_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float v_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float v_rcp(float a) { return __frcp_rn(a); }
__device__ __forceinline__ float v_floor_rho(float a) { return a < 1e-16f ? 1e-16f : a; }
__device__ __forceinline__ float2 v_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b rounded once: b * (-1) is exact.
__device__ __forceinline__ float2 v_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 v_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 v_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 v_rcp(float2 a) { return make_float2(__frcp_rn(a.x), __frcp_rn(a.y)); }
__device__ __forceinline__ float2 v_floor_rho(float2 a) { return make_float2(v_floor_rho(a.x), v_floor_rho(a.y)); }
template <class V> __device__ __forceinline__ V v_splat(float x);
template <> __device__ __forceinline__ float v_splat<float>(float x) { return x; }
template <> __device__ __forceinline__ float2 v_splat<float2>(float x) { return make_float2(x, x); }

// h1 = fl(3 w1), h5 = (1 - 2 h1) / 4, as the host computes them.
__device__ __forceinline__ void shifted_h(float w1, float &h1, float &h5) {
    h1 = __fmul_rn(3.0f, w1);
    h5 = __fmul_rn(__fsub_rn(1.0f, __fmul_rn(2.0f, h1)), 0.25f);
}

// Shifted moments: delta rho = sum g, j = sum c g (sum c w = 0). Jx, Jy are the
// momentum including half the body force (rho u of lbc); jx, jy without it.
template <class V>
__device__ __forceinline__ void moments_v(const V g[9], V hFx, V hFy, V &dr, V &rho, V &ux, V &uy, V &Jx,
                                          V &Jy, V &jx, V &jy) {
    dr = v_add(v_add(v_add(v_add(g[0], g[1]), v_add(g[2], g[3])), v_add(v_add(g[4], g[5]), v_add(g[6], g[7]))),
               g[8]);
    jx = v_add(v_add(v_sub(g[1], g[3]), v_sub(g[5], g[6])), v_sub(g[8], g[7]));
    jy = v_sub(v_add(v_sub(g[2], g[4]), v_add(g[5], g[6])), v_add(g[7], g[8]));
    rho = v_floor_rho(v_add(v_splat<V>(1.0f), dr));
    const V inv = v_rcp(rho);
    Jx = v_add(jx, hFx);
    Jy = v_add(jy, hFy);
    ux = v_mul(Jx, inv);
    uy = v_mul(Jy, inv);
}

// One pair of directions (k, opposite) of the equilibrium: X = w (dr + 4.5 J c
// - rt) is the even part, h o the odd part, added to X with one rounding
// (X +- h o as FMAs: rounding h o first doubles the FP32 velocity error of a
// Taylor-Green run against FP64). The odd part takes the momentum without
// the half force, o = c.j; the force enters the odd part separately (see
// collide_v).
template <class V>
__device__ __forceinline__ void geq_pair(float w, float h, V dr, V c, V J, V o, V nrt, V &a, V &b) {
    const V X = v_mul(v_splat<V>(w), v_add(dr, v_fma(v_mul(v_splat<V>(4.5f), J), c, nrt)));
    a = v_fma(v_splat<V>(h), o, X);
    b = v_fma(v_splat<V>(-h), o, X);
}

// BGK + Guo on shifted populations, g' = g + om (geq - g) + (1 - om/2) F_k,
// with geq_k = w_k (drho + rho (3 c.u + 4.5 (c.u)^2 - 1.5 u.u)) built so that
// its mass and momentum are the node's own by construction: the odd part of
// each pair is h (c.J) with FP32 coefficients h1 = fl(3 w1) and
// h5 = (1 - 2 h1) / 4 whose sum rule 2 h1 + 4 h5 = 1 holds exactly, the linear
// term uses J = rho u directly (no division), and the rest population closes
// the mass. Rounded weights would otherwise bias every collision's momentum by
// ~1e-8 in the same direction, an error that grows linearly with the steps.
//
// With a body force, J = j + F/2 would round F/2 (~1e-7) against j: an error of
// the same sign every step, which drove a forced channel 6.6e-5 away from FP64
// in 20,000 steps. Instead the odd part relaxes towards h (c.j) and the whole
// odd forcing, om h c.F/2 + (1 - om/2) 3 w c.F = h c.F (h = 3 w), is added as
// one small term; the even forcing is (1 - om/2) w S, S = 9 (c.u)(c.F) - 3 u.F.
// The relaxation and the forcing are summed first (one FMA) and added to g with
// a single rounding. Channel 256 x 64 against FP64 after 20,000 steps: u L2
// error 5.0e-7 (6.6e-5 before).
template <class V, bool FORCE>
__device__ __forceinline__ void collide_v(V g[9], const float w[9], float h1, float h5, V dr, V ux, V uy,
                                          V Jx, V Jy, V jx, V jy, V om, bool force, float Fx, float Fy) {
    const V nrt = v_mul(v_splat<V>(-1.5f), v_fma(Jx, ux, v_mul(Jy, uy)));  // -rho * 1.5 u.u
    // Without a body force j = J exactly: one set of momenta stays live.
    const bool forced = FORCE && force;
    if (!FORCE) {
        jx = Jx;
        jy = Jy;
    }
    V geq[9];
    geq_pair(w[1], h1, dr, ux, Jx, jx, nrt, geq[1], geq[3]);
    geq_pair(w[2], h1, dr, uy, Jy, jy, nrt, geq[2], geq[4]);
    geq_pair(w[5], h5, dr, v_add(ux, uy), v_add(Jx, Jy), v_add(jx, jy), nrt, geq[5], geq[7]);
    geq_pair(w[6], h5, dr, v_sub(uy, ux), v_sub(Jy, Jx), v_sub(jy, jx), nrt, geq[6], geq[8]);
    geq[0] = v_sub(dr, v_add(v_add(v_add(geq[1], geq[3]), v_add(geq[2], geq[4])),
                             v_add(v_add(geq[5], geq[7]), v_add(geq[6], geq[8]))));
    if (!forced) {
        // A force-free case: one FMA per population. Kernels that may see
        // forced cases (FORCE) take this branch per case at run time, so a
        // case gets the same bits alone and in any batch.
#pragma unroll
        for (int k = 0; k < 9; k++) g[k] = v_fma(om, v_sub(geq[k], g[k]), g[k]);
        return;
    }
    const V Fxv = v_splat<V>(Fx), Fyv = v_splat<V>(Fy);
    const V gf = v_fma(v_splat<V>(-0.5f), om, v_splat<V>(1.0f));
    const V n3uF = v_mul(v_splat<V>(-3.0f), v_fma(ux, Fxv, v_mul(uy, Fyv)));  // -3 u.F
    g[0] = v_add(g[0], v_fma(om, v_sub(geq[0], g[0]), v_mul(gf, v_mul(v_splat<V>(w[0]), n3uF))));
    const V cu[4] = {ux, uy, v_add(ux, uy), v_sub(uy, ux)};
    const float cFs[4] = {Fx, Fy, Fx + Fy, Fy - Fx};
    const float hs[4] = {h1, h1, h5, h5};
    const int ka[4] = {1, 2, 5, 6}, kb[4] = {3, 4, 7, 8};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const V cF = v_splat<V>(cFs[q]);
        const V S = v_fma(v_mul(v_splat<V>(9.0f), cu[q]), cF, n3uF);
        const V E = v_mul(gf, v_mul(v_splat<V>(w[ka[q]]), S));
        const V O = v_splat<V>(hs[q] * cFs[q]);
        const int a = ka[q], b = kb[q];
        g[a] = v_add(g[a], v_fma(om, v_sub(geq[a], g[a]), v_add(E, O)));
        g[b] = v_add(g[b], v_fma(om, v_sub(geq[b], g[b]), v_sub(E, O)));
    }
}

// Scalar entry points used by the per-node paths.
__device__ __forceinline__ void moments_shifted(const float g[9], float hFx, float hFy, float &dr,
                                                float &rho, float &ux, float &uy, float &Jx,
                                                float &Jy, float &jx, float &jy) {
    moments_v<float>(g, hFx, hFy, dr, rho, ux, uy, Jx, Jy, jx, jy);
}

// Rare per-node outputs, kept out of line so the compiler cannot hoist their
// FP64 conversions into every thread's path (FP64 issue is slow on GB300).
template <typename T>
__device__ __noinline__ void solid_node_outputs(const StepParams &p, int slot, long long node, size_t dn,
                                                uint16_t fl) {
    if (p.write_macro) { p.rho[dn] = NAN; p.ux[dn] = NAN; p.uy[dn] = NAN; }
    if (fl & NF_BAND) {
        // A BC may read a solid neighbour: lbc sees the untouched buffer
        // content and NaN moments there.
        const T *Dst = (const T *)p.dst;
#pragma unroll
        for (int k = 0; k < 9; k++) p.bandg[(size_t)k * p.nslots + slot] = SV<T>::ld_plain(Dst + k * p.plane + node);
        p.bandm_next[slot] = NAN;
        p.bandm_next[(size_t)p.nslots + slot] = NAN;
        p.bandm_next[2 * (size_t)p.nslots + slot] = NAN;
    }
}


// A solid node off the edge band (kSpecialSolid entries): NaN moments on steps
// that write the fields, as solid_node_outputs writes them.
__device__ __forceinline__ void solid_nan(const StepParams &p, int i, int j) {
    if (!p.write_macro) return;
    const size_t dn = (size_t)j * (size_t)p.Nx + (size_t)i;
    p.rho[dn] = NAN;
    p.ux[dn] = NAN;
    p.uy[dn] = NAN;
}

__device__ __noinline__ void macro_store(const StepParams &p, size_t dn, int slot, float dr, float ux,
                                         float uy) {
    if (p.write_macro) { p.rho[dn] = 1.0 + (double)dr; p.ux[dn] = ux; p.uy[dn] = uy; }
    if (slot >= 0) {
        p.bandm_next[slot] = 1.0 + (double)dr;
        p.bandm_next[(size_t)p.nslots + slot] = ux;
        p.bandm_next[2 * (size_t)p.nslots + slot] = uy;
    }
}

__device__ __noinline__ void macro_store_pair(const StepParams &p, size_t dn, float2 dr, float2 ux, float2 uy) {
    p.rho[dn] = 1.0 + (double)dr.x;
    p.rho[dn + 1] = 1.0 + (double)dr.y;
    p.ux[dn] = ux.x;
    p.ux[dn + 1] = ux.y;
    p.uy[dn] = uy.x;
    p.uy[dn + 1] = uy.y;
}

__device__ __noinline__ float2 omega_pair(const double *omega, size_t dn) {
    return make_float2((float)omega[dn], (float)omega[dn + 1]);
}

// One node of the fused step in shifted storage (solids, bounce-back links,
// stale slots, edge-BC band: everything). I is the element-offset type: int
// whenever all nine planes fit in 2^31 elements (fewer address instructions),
// long long otherwise. LINKS = false: no case of the launch has cut-link
// records (plain bounce-back on every solid link), and the record path is
// left out (measured: 116 -> 64 registers for the batched special-node
// kernel, twice the resident warps).
template <typename T, typename I, bool FLAGS, bool COLLIDE, bool FORCE, bool LINKS = true>
__device__ __forceinline__ void step_node_shifted(const FastStepParams &fp, int i, int j,
                                                  float &mfx, float &mfy, bool &link) {
    const StepParams &p = fp.s;
    const I node = (I)j * (I)p.pitch + (I)i;
    const size_t dn = (size_t)j * (size_t)p.Nx + (size_t)i;
    const T *S = (const T *)p.src;
    T *Dst = (T *)p.dst;
    const I pl = (I)p.plane;
    // The loads come in three waves of independent loads, not one chain: (1)
    // the flag word, the nine pulled populations, the node's eight own
    // opposite populations, its cut-link offset, its band bases and (without
    // cut-link records) the stale slots of off-grid sources, which the
    // position alone decides; (2) the cut-link records of its flagged
    // directions; (3) the populations behind interpolated links (and the
    // stale slots, with records). Source neighbours are wrapped on periodic axes and
    // clamped otherwise, so that every load of wave 1 is in bounds whatever
    // the flags say. (Measured: the own populations loaded in wave 2, for
    // flagged directions only, cost the channel and the cylinder 2-4 %.)
    int im = i - 1, ip = i + 1, jm = j - 1, jp = j + 1;
    if (p.px) { if (im < 0) im += p.Nx; if (ip >= p.Nx) ip -= p.Nx; }
    else { im = max(im, 0); ip = min(ip, p.Nx - 1); }
    if (p.py) { if (jm < 0) jm += p.Ny; if (jp >= p.Ny) jp -= p.Ny; }
    else { jm = max(jm, 0); jp = min(jp, p.Ny - 1); }
    const I r0 = (I)j * (I)p.pitch, rm = (I)jm * (I)p.pitch, rp = (I)jp * (I)p.pitch;
    const I so[9] = {r0 + i, r0 + im, rm + i, r0 + ip, rp + i, rm + im, rm + ip, rp + ip, rp + im};
    const uint16_t fl = FLAGS ? p.flags[node] : (uint16_t)0;
    float g[9];
#pragma unroll
    for (int k = 0; k < 9; k++) g[k] = SV<T>::ld(S + (I)k * pl + so[k]);
    int lo = 0, cb = -1, rb = -1;
    float own[9];
    bool off[9];
    if (FLAGS) {
#pragma unroll
        for (int k = 1; k < 9; k++) own[k] = SV<T>::ld(S + (I)oppk(k) * pl + node);
        if (LINKS && p.link_off) lo = p.link_off[node];
        // Without cut-link records, also the band bases and the stale slots
        // of off-grid sources (this node's own destination slots, written by
        // no other thread). With records they stay in the later waves: their
        // registers (96 -> 116 for the per-case kernel) cost more than the
        // latency saved.
        if (!LINKS && p.colbase) { cb = p.colbase[i]; rb = p.rowbase[j]; }
        if (!LINKS) {
#pragma unroll
            for (int k = 1; k < 9; k++) {
                const int si = i - cxk(k), sj = j - cyk(k);
                off[k] = (!p.px && (si < 0 || si >= p.Nx)) || (!p.py && (sj < 0 || sj >= p.Ny));
                if (off[k]) g[k] = SV<T>::ld_plain(Dst + (I)k * pl + node);
            }
        }
    }
    int slot = -1;
    if (FLAGS && (fl & NF_BAND)) slot = LINKS ? band_slot(p.colbase, p.rowbase, i, j) : (cb >= 0 ? cb + j : rb + i);
    if (FLAGS && (fl & NF_SOLID)) {
        solid_node_outputs<T>(p, slot, (long long)node, dn, fl);
        return;
    }
    if (FLAGS && (fl & NF_SPECIAL_MASK)) {
        const bool has_links = LINKS && (fl & NF_LINKS) != 0;
        Link L[9];
        int m = 0;
#pragma unroll
        for (int k = 1; k < 9; k++) {
            if (LINKS) {
                const int si = i - cxk(k), sj = j - cyk(k);
                off[k] = (!p.px && (si < 0 || si >= p.Nx)) || (!p.py && (sj < 0 || sj >= p.Ny));
            }
            // link records in direction order, one per flagged on-grid direction
            if ((fl & (1u << k)) && !off[k] && has_links) L[k] = p.links[lo + m++];
        }
        float behind[9];
#pragma unroll
        for (int k = 1; k < 9; k++) {
            behind[k] = 0.f;
            if (!(fl & (1u << k))) continue;
            if (off[k]) {
                if (LINKS) g[k] = SV<T>::ld_plain(Dst + (I)k * pl + node);
            } else if (has_links) {
                if (L[k].mode == LINK_IBB_LO) behind[k] = SV<T>::ld(S + (I)oppk(k) * pl + (I)L[k].behind);
                else if (L[k].mode == LINK_IBB_HI) behind[k] = SV<T>::ld(S + (I)k * pl + (I)L[k].behind);
            }
        }
#pragma unroll
        for (int k = 1; k < 9; k++) {
            if (!(fl & (1u << k)) || off[k]) continue;
            float val = own[k];
            if (has_links) {
                if (L[k].mode == LINK_IBB_LO || L[k].mode == LINK_IBB_HI)
                    val = (float)L[k].c1 * own[k] + (float)L[k].c2 * behind[k];
                else if (L[k].mode == LINK_MOVING)
                    val = own[k] - (float)L[k].c2;
            }
            g[k] = SV<T>::rnd(val);
            // Per-node link sum in FP32 (a few terms); chunk and case sums are FP64.
            const float df = (own[k] + val) + 2.0f * fp.wf[k];
            mfx -= df * cxk(k);
            mfy -= df * cyk(k);
            link = true;
        }
    }
    if (FLAGS && (fl & NF_BAND)) {
#pragma unroll
        for (int k = 0; k < 9; k++) p.bandg[(size_t)k * p.nslots + slot] = g[k];
    }
    if (FLAGS && (fl & NF_BCW)) return;
    float dr, rho, ux, uy, Jx, Jy, jx, jy;
    moments_v<float>(g, fp.hFxf, fp.hFyf, dr, rho, ux, uy, Jx, Jy, jx, jy);
    if (p.write_macro || slot >= 0) macro_store(p, dn, slot, dr, ux, uy);
    if (COLLIDE) {
        const float om = p.omega ? (float)p.omega[dn] : fp.omega0f;
        collide_v<float, FORCE>(g, fp.wf, fp.h1f, fp.h5f, dr, ux, uy, Jx, Jy, jx, jy, om, p.has_force != 0,
                                fp.Fxf, fp.Fyf);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) SV<T>::st(Dst + (I)k * pl + node, g[k]);
}

// Two adjacent nodes (i0, i0 + 1) of one row, neither of them special (no
// solid, link, stale slot, band or BC node): pair loads where the pull sources
// are adjacent (c_x = 0), a pair and a single load otherwise (c_x = +-1), packed
// FP32 arithmetic, pair stores. im = source column of i0 - 1, ip2 of i0 + 2
// (wrapped or clamped like the per-node path), so every load is in bounds
// whatever the nodes' flags say.
template <typename T, typename I>
__device__ __forceinline__ void load_pair_shifted(const StepParams &p, int i0, int j, int im, int ip2, int jm,
                                                  int jp, float2 g[9]) {
    const T *S = (const T *)p.src;
    const I pl = (I)p.plane;
    const I r0 = (I)j * (I)p.pitch + (I)i0, rm = (I)jm * (I)p.pitch, rp = (I)jp * (I)p.pitch;
    const I m0 = rm + (I)i0, p0 = rp + (I)i0;
    float2 a;
    g[0] = SV<T>::ld2(S + r0);
    a = SV<T>::ld2(S + pl + r0);
    g[1] = make_float2(SV<T>::ld(S + pl + (r0 - (I)i0 + (I)im)), a.x);
    g[2] = SV<T>::ld2(S + 2 * pl + m0);
    a = SV<T>::ld2(S + 3 * pl + r0);
    g[3] = make_float2(a.y, SV<T>::ld(S + 3 * pl + (r0 - (I)i0 + (I)ip2)));
    g[4] = SV<T>::ld2(S + 4 * pl + p0);
    a = SV<T>::ld2(S + 5 * pl + m0);
    g[5] = make_float2(SV<T>::ld(S + 5 * pl + rm + (I)im), a.x);
    a = SV<T>::ld2(S + 6 * pl + m0);
    g[6] = make_float2(a.y, SV<T>::ld(S + 6 * pl + rm + (I)ip2));
    a = SV<T>::ld2(S + 7 * pl + p0);
    g[7] = make_float2(a.y, SV<T>::ld(S + 7 * pl + rp + (I)ip2));
    a = SV<T>::ld2(S + 8 * pl + p0);
    g[8] = make_float2(SV<T>::ld(S + 8 * pl + rp + (I)im), a.x);
}

template <typename T, typename I, bool COLLIDE, bool FORCE>
__device__ __forceinline__ void collide_store_pair_shifted(const FastStepParams &fp, int i0, int j, float2 g[9]) {
    const StepParams &p = fp.s;
    T *Dst = (T *)p.dst;
    const I pl = (I)p.plane;
    const I r0 = (I)j * (I)p.pitch + (I)i0;
    float2 dr, rho, ux, uy, Jx, Jy, jx, jy;
    moments_v<float2>(g, v_splat<float2>(fp.hFxf), v_splat<float2>(fp.hFyf), dr, rho, ux, uy, Jx, Jy, jx, jy);
    const size_t dn = (size_t)j * (size_t)p.Nx + (size_t)i0;
    if (p.write_macro) macro_store_pair(p, dn, dr, ux, uy);
    if (COLLIDE) {
        const float2 om = p.omega ? omega_pair(p.omega, dn) : v_splat<float2>(fp.omega0f);
        collide_v<float2, FORCE>(g, fp.wf, fp.h1f, fp.h5f, dr, ux, uy, Jx, Jy, jx, jy, om, p.has_force != 0,
                                 fp.Fxf, fp.Fyf);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) SV<T>::st2(Dst + (I)k * pl + r0, g[k]);
}

// Flag bits that take a node off the pair path: a solid or off-grid pull
// source, solid, edge-BC band or BC-written, cut links.
constexpr uint32_t kSpecialFlags = NF_SPECIAL_MASK | NF_SOLID | NF_BAND | NF_BCW | NF_LINKS;

// The pair (i0, i0 + 1) of row j when both nodes exist and neither is
// special; nothing otherwise (those nodes are on the case's special-node
// list). A bit per 64-node row segment (one warp's pairs) says the whole
// segment is clean; only other segments read their flag words, issued
// together with the pair's loads (measured: 64 ducts 58.5 -> 62.0 GLUPS,
// channels +1-2 %).
template <typename T, typename I, bool FLAGS, bool COLLIDE, bool FORCE>
__device__ __forceinline__ void step_pair_clean(const FastStepParams &fp, int i0, int j) {
    const StepParams &p = fp.s;
    if (i0 + 1 >= p.Nx) return;
    uint32_t f2 = 0;
    bool clean = !FLAGS;
    if (FLAGS) {
        const uint32_t wrd = __ldg(p.seg_clean + (size_t)j * p.seg_words + (i0 >> 11));
        clean = (wrd >> ((i0 >> 6) & 31)) & 1u;
        if (!clean) f2 = *(const uint32_t *)(p.flags + ((I)j * (I)p.pitch + (I)i0));
    }
    int im = i0 - 1, ip2 = i0 + 2, jm = j - 1, jp = j + 1;
    if (p.px) { if (im < 0) im += p.Nx; if (ip2 >= p.Nx) ip2 -= p.Nx; }
    else { im = max(im, 0); ip2 = min(ip2, p.Nx - 1); }
    if (p.py) { if (jm < 0) jm += p.Ny; if (jp >= p.Ny) jp -= p.Ny; }
    else { jm = max(jm, 0); jp = min(jp, p.Ny - 1); }
    float2 g[9];
    load_pair_shifted<T, I>(p, i0, j, im, ip2, jm, jp, g);
    if (FLAGS && !clean && ((f2 | (f2 >> 16)) & kSpecialFlags) != 0) return;
    collide_store_pair_shifted<T, I, COLLIDE, FORCE>(fp, i0, j, g);
}

// Fully periodic grid without solids or edge BCs: no flag word. Each thread
// steps two adjacent nodes; the last column of an odd-width grid takes the
// per-node path. Five resident blocks per SM (48 registers, no spills) keep
// more loads in flight than the unconstrained 64 registers (measured: FP16
// 135 -> 147 GLUPS on 4096^2).
template <typename T, typename I, bool COLLIDE, bool FORCE>
__global__ void __launch_bounds__(256, 5) k_step_shifted_plain(const FastStepParams fp) {
    pdl_launch_dependents();
    const int i0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i0 >= fp.s.Nx || j >= fp.s.Ny) return;
    if (i0 + 1 < fp.s.Nx) {
        step_pair_clean<T, I, false, COLLIDE, FORCE>(fp, i0, j);
    } else {
        float mx = 0.f, my = 0.f;
        bool l = false;
        step_node_shifted<T, I, false, COLLIDE, FORCE>(fp, i0, j, mx, my, l);
    }
}

// General geometry (flag word per node): the clean pairs only. The per-node
// path is in k_step_special_shifted, over the case's list of special nodes
// (every node of a pair with a special node, and an odd last column); kept
// out of this kernel, it costs the common path no registers, spills or
// instruction-cache space (measured: cylinder 2048x512 step 21.3 -> 14.2 us
// with the special nodes left out).
template <typename T, typename I, bool COLLIDE, bool FORCE>
__global__ void __launch_bounds__(256, 5) k_step_shifted_geo(const FastStepParams fp) {
    pdl_launch_dependents();
    const int i0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i0 < fp.s.Nx && j < fp.s.Ny) step_pair_clean<T, I, true, COLLIDE, FORCE>(fp, i0, j);
}

// The special nodes of a case, one per thread, on the per-node path (same
// arithmetic as the pair path, so a node's bits do not depend on which path
// steps it). Wall-link force terms are summed per 32-entry chunk of the list.
// It reads and writes nothing the clean-pair kernel touches: a case alone
// launches it first, as an ordinary launch, with the clean pairs as its
// programmatic follower (pdl.cuh), so their blocks fill the SMs around its
// latency-bound ones; the launch after both is ordinary. (The trigger at the
// start lets the follower launch at once; the wait at the end is then a
// no-op.)
template <typename T, typename I, bool FLAGS, bool COLLIDE, bool FORCE, bool LINKS>
__global__ void __launch_bounds__(128) k_step_special_shifted(const FastStepParams fp,
                                                              const int2 *__restrict__ nodes, int n) {
    pdl_launch_dependents();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    float mx = 0.f, my = 0.f;
    bool link = false;
    if (q < n) {
        const int2 ij = nodes[q];
        if (ij.x & kSpecialSolid) solid_nan(fp.s, ij.x & ~kSpecialSolid, ij.y);
        else step_node_shifted<T, I, FLAGS, COLLIDE, FORCE, LINKS>(fp, ij.x, ij.y, mx, my, link);
    }
    if (fp.s.mem_partials)
        chunk_reduce2_store((double)mx, (double)my, link, q >> 5, fp.s.chunk_slot, fp.s.mem_partials);
    pdl_wait();
}

// Batched form (see k_step_batch_exact in kernels_exact.cu): tiles of
// 2^(tws + 1) x 2^(8 - tws) nodes, two adjacent nodes per thread, clean pairs
// only (the special nodes of all cases are k_step_batch_special_shifted's:
// blocks of them spread through this kernel's tile list, on 64 liner ducts
// without cut links, measured 57.4 vs 67.7 GLUPS). Blocks stride through the
// tile list, so the tiles in flight at any moment are neighbours in memory
// (sequential DRAM streams, halo rows shared through L2).
template <typename T, typename I, bool FORCE, bool ALLFLAGS>
__global__ void __launch_bounds__(256, 4) k_step_batch_shifted(const FastStepParams *__restrict__ sp,
                                                            const int4 *__restrict__ tiles,
                                                            int ntiles, int sel, int tws) {
    pdl_launch_dependents();
    const int tx = threadIdx.x & ((1 << tws) - 1), ty = threadIdx.x >> tws;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int4 td = tiles[t];
        const FastStepParams &fp = sp[2 * td.x + sel];
        const int i0 = td.y + 2 * tx, j = td.z + ty;
        // FORCE: some case of the batch has a body force; force-free cases
        // still take their own (force-free) arithmetic per case (collide_v).
        // ALLFLAGS: every case has a flag word, and the flag-free form of the
        // pair step is left out (measured on 64 ducts: 54.4 -> 57.8 GLUPS,
        // from 72 to 12 bytes of spills).
        if (i0 < fp.s.Nx && j < fp.s.Ny) {
            if (ALLFLAGS || fp.s.flags) step_pair_clean<T, I, true, true, FORCE>(fp, i0, j);
            else step_pair_clean<T, I, false, true, FORCE>(fp, i0, j);
        }
    }
}

// The special nodes of every case of a batch: nodes[q] = (case, i, j, chunk),
// each case's list padded to a multiple of 32 entries (padding: i = -1), so
// that a warp holds one chunk of one case and the force partials are those of
// the case alone. LINKS: some case of the batch has cut-link records.
template <typename T, typename I, bool FORCE, bool LINKS>
__global__ void __launch_bounds__(128) k_step_batch_special_shifted(const FastStepParams *__restrict__ sp,
                                                                    const int4 *__restrict__ nodes, int n,
                                                                    int sel) {
    pdl_launch_dependents();
    const int q = (int)blockIdx.x * (int)blockDim.x + (int)threadIdx.x;
    if (q < n) {  // n is a multiple of 32: whole warps
        const int4 e = nodes[q];
        const FastStepParams &fp = sp[2 * e.x + sel];
        float mx = 0.f, my = 0.f;
        bool link = false;
        if (e.y & kSpecialSolid) solid_nan(fp.s, e.y & ~kSpecialSolid, e.z);
        else if (e.y >= 0) {
            if (fp.s.flags) step_node_shifted<T, I, true, true, FORCE, LINKS>(fp, e.y, e.z, mx, my, link);
            else step_node_shifted<T, I, false, true, FORCE, LINKS>(fp, e.y, e.z, mx, my, link);
        }
        if (fp.s.mem_partials)
            chunk_reduce2_store((double)mx, (double)my, link, e.w, fp.s.chunk_slot, fp.s.mem_partials);
    }
    pdl_wait();
}

// Band populations are read at L2 (__ldcg), never from a possibly stale L1
// line.
template <typename T, bool COLLIDE>
__device__ __forceinline__ void finish_node_shifted(const FinishParams &p, int2 ij, int slot) {
    float g[9], wf[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
        g[k] = SV<T>::rnd(__ldcg(p.bandg + (size_t)k * p.nslots + slot));
        wf[k] = p.wf[k];
    }
    float dr, rho, ux, uy, Jx, Jy, jx, jy;
    moments_shifted(g, p.hFxf, p.hFyf, dr, rho, ux, uy, Jx, Jy, jx, jy);
    const size_t dn = (size_t)ij.y * p.Nx + ij.x;
    if (p.write_macro) { p.rho[dn] = 1.0 + (double)dr; p.ux[dn] = ux; p.uy[dn] = uy; }
    p.bandm_next[slot] = 1.0 + (double)dr;
    p.bandm_next[(size_t)p.nslots + slot] = ux;
    p.bandm_next[2 * (size_t)p.nslots + slot] = uy;
    if (COLLIDE) {
        const float om = p.omega ? (float)p.omega[dn] : p.omega0f;
        float h1, h5;
        shifted_h(wf[1], h1, h5);
        if (p.has_force) collide_v<float, true>(g, wf, h1, h5, dr, ux, uy, Jx, Jy, jx, jy, om, true, p.Fxf, p.Fyf);
        else collide_v<float, false>(g, wf, h1, h5, dr, ux, uy, Jx, Jy, jx, jy, om, false, 0.f, 0.f);
    }
    T *D = (T *)p.dst;
    const long long node = (long long)ij.y * p.pitch + ij.x;
#pragma unroll
    for (int k = 0; k < 9; k++) SV<T>::st(D + k * p.plane + node, g[k]);
}

// In-place collision of shifted populations with the stored (FP64) rho/u/v:
// the first step of a run (src/core/collision.c:18-40).
template <typename T>
__global__ void k_collide_shifted(const CollideParams p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= p.Nx || j >= p.Ny) return;
    const long long node = (long long)j * p.pitch + i;
    if (p.flags && (p.flags[node] & NF_SOLID)) return;
    const size_t dn = (size_t)j * p.Nx + i;
    T *F = (T *)p.f;
    float g[9], wf[9];
#pragma unroll
    for (int k = 0; k < 9; k++) { g[k] = SV<T>::ld_plain(F + k * p.plane + node); wf[k] = (float)p.w[k]; }
    const float om = p.omega ? (float)p.omega[dn] : (float)p.omega0;
    float dr, rho, ux, uy, Jx, Jy, jx, jy;
    if (p.from_pops) {
        moments_shifted(g, (float)(0.5 * p.Fx), (float)(0.5 * p.Fy), dr, rho, ux, uy, Jx, Jy, jx, jy);
    } else {
        // the stored fields: rho, u = (j + F/2) / rho
        rho = (float)p.rho[dn];
        dr = (float)(p.rho[dn] - 1.0);
        ux = (float)p.ux[dn];
        uy = (float)p.uy[dn];
        Jx = (float)(p.rho[dn] * p.ux[dn]);
        Jy = (float)(p.rho[dn] * p.uy[dn]);
        jx = (float)(p.rho[dn] * p.ux[dn] - 0.5 * p.Fx);
        jy = (float)(p.rho[dn] * p.uy[dn] - 0.5 * p.Fy);
    }
    float h1, h5;
    shifted_h(wf[1], h1, h5);
    if (p.has_force) collide_v<float, true>(g, wf, h1, h5, dr, ux, uy, Jx, Jy, jx, jy, om, true, (float)p.Fx,
                                            (float)p.Fy);
    else collide_v<float, false>(g, wf, h1, h5, dr, ux, uy, Jx, Jy, jx, jy, om, false, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 9; k++) SV<T>::st(F + k * p.plane + node, g[k]);
}

// ---------------------------------------------------------------- edge BCs
// The Boundary list on the band in FP32 (bc_shifted.cuh): band populations are
// g, previous-step moments come from the FP64 band moments (rho - 1 formed in
// FP64). The impedance wall's mass-spring-damper state and DFT stay FP64.
template <typename T> struct BandAccessorS {
    const StageParams &p;
    const StagePre &c;
    __device__ int slot(int i, int j) const {
        if (i == c.ij.x && j == c.ij.y) return c.slot;
        if (i == c.nij.x && j == c.nij.y) return c.nslot;
        return band_slot(p.colbase, p.rowbase, i, j);
    }
    __device__ bool nb(int i, int j) const { return i == c.nij.x && j == c.nij.y; }
    __device__ double m(int q, int i, int j) const { return p.bandm_prev[(size_t)q * p.nslots + slot(i, j)]; }
    __device__ float get(int i, int j, int k) const { return __ldcg(p.bandg + (size_t)k * p.nslots + slot(i, j)); }
    __device__ void set(int i, int j, int k, float v) const {
        p.bandg[(size_t)k * p.nslots + slot(i, j)] = v;
    }
    __device__ float drho(int i, int j) const { return (float)((nb(i, j) ? c.nrho : m(0, i, j)) - 1.0); }
    __device__ float ux(int i, int j) const { return (float)(nb(i, j) ? c.nux : m(1, i, j)); }
    __device__ float uy(int i, int j) const { return (float)(nb(i, j) ? c.nuy : m(2, i, j)); }
    __device__ float post(int i, int j, int k) const {
        return SV<T>::ld_plain((const T *)p.src + k * p.plane + (long long)j * p.pitch + i);
    }
    __device__ bool solid(int i, int j) const {
        if (i == c.ij.x && j == c.ij.y) return c.solid;
        return (p.flags[(long long)j * p.pitch + i] & NF_SOLID) != 0;
    }
};

// One point of one Boundary entry (src/core/main_lbm.c:49-58) after its
// preload, as stage_point in kernels_exact.cu.
template <typename T>
__device__ __forceinline__ void stage_point_s(const StageParams &p, const StagePre &c, int t, int kind) {
    BandAccessorS<T> a{p, c};
    float w[9];
#pragma unroll
    for (int k = 0; k < 9; k++) w[k] = p.wf[k];
    if (kind == BC_VEL_BOT_REG && c.imp) {
        bc_regularized_s(a, w, t, p.index, t, p.index + 1, false, (float)c.v1, (float)c.v2);
        return;
    }
    bc_apply_s(a, w, kind, p.Nx, p.Ny, p.index, t, c.v1, c.v2);
}

// One stage thread, specialised on the entry's kind (each kind one short
// region of code): preload, wait for the kernels before it, the BC, the
// finish. (Alone, the edge launch is an ordinary launch behind the special
// nodes and the clean pairs; in a batch it follows the special nodes.) An
// instruction-cache warm-up pass before the wait, the same code without its
// stores, paid off while the edge launch overlapped the clean pairs' last
// wave; measured without it: cylinder 2048x512 17.96 -> 16.42 us per step
// in the current order, 64 liner ducts 186.3 -> 184.7 us.
template <typename T, bool COLLIDE, int KIND>
__device__ __forceinline__ void stage_thread_s(const StageParams &p, const FinishParams &f, int t) {
    StagePre c = stage_preload<true>(p, t, KIND);
    pdl_wait();
    stage_point_s<T>(p, c, t, KIND);
    if (c.fin) finish_node_shifted<T, COLLIDE>(f, c.ij, c.slot);
}

template <typename T, bool COLLIDE>
__device__ __forceinline__ void stage_dispatch_s(const StageParams &p, const FinishParams &f, int t) {
    switch (p.kind) {
#define LBM_STAGE_KIND(K) \
    case K: stage_thread_s<T, COLLIDE, K>(p, f, t); break;
    LBM_STAGE_KIND(BC_VEL_IN_ZH) LBM_STAGE_KIND(BC_VEL_OUT_ZH) LBM_STAGE_KIND(BC_VEL_TOP_ZH)
    LBM_STAGE_KIND(BC_VEL_BOT_ZH) LBM_STAGE_KIND(BC_PRES_IN_ZH) LBM_STAGE_KIND(BC_PRES_OUT_ZH)
    LBM_STAGE_KIND(BC_CONV_IN) LBM_STAGE_KIND(BC_CONV_OUT) LBM_STAGE_KIND(BC_PERIODIC_X)
    LBM_STAGE_KIND(BC_PERIODIC_Y) LBM_STAGE_KIND(BC_VEL_IN_REG) LBM_STAGE_KIND(BC_VEL_OUT_REG)
    LBM_STAGE_KIND(BC_VEL_TOP_REG) LBM_STAGE_KIND(BC_VEL_BOT_REG) LBM_STAGE_KIND(BC_PRES_IN_REG)
    LBM_STAGE_KIND(BC_PRES_OUT_REG) LBM_STAGE_KIND(BC_PRES_TOP_REG) LBM_STAGE_KIND(BC_PRES_BOT_REG)
    LBM_STAGE_KIND(BC_VEL_BOT_ZH_FIX)
#undef LBM_STAGE_KIND
    default: pdl_wait(); break;
    }
}

// As k_stage_group / k_stage_batch in kernels_exact.cu.
template <typename T, bool COLLIDE>
__global__ void k_stage_group_shifted(const StageGroup g) {
    if ((int)blockIdx.y >= g.n) {
        pdl_wait();
        if (blockIdx.x == 0 && threadIdx.x < 32) force_reduce_warp(*g.fs, (int)threadIdx.x);
        return;
    }
    const StageParams &p = g.p[blockIdx.y];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.along) return;
    stage_dispatch_s<T, COLLIDE>(p, g.fin, t);
}

template <typename T>
__global__ void k_stage_batch_shifted(const StageParams *__restrict__ list,
                                      const int2 *__restrict__ blk, int sel, int n,
                                      const ForceSlot *__restrict__ fs) {
    const int2 b = blk[blockIdx.x];
    const int e = b.x;
    if (e >= n) {
        pdl_wait();
        if (threadIdx.x < 32) force_reduce_warp(fs[e - n], (int)threadIdx.x);
        return;
    }
    const StageParams &p = list[2 * e + sel];
    const int t = b.y + (int)threadIdx.x;
    if (t >= p.along) return;
    stage_dispatch_s<T, true>(p, *p.fin, t);
}

namespace launch {

cudaError_t stage_group_shifted(const StageGroup &g, int store, bool collide, bool after_bulk, cudaStream_t s) {
    const dim3 grid((g.max_along + 63) / 64, g.n + (g.nfs ? 1 : 0)), b(64);
    if (store == STORE_F32) {
        if (collide) return launch_follower(after_bulk, k_stage_group_shifted<float, true>, grid, b, s, g);
        return launch_follower(after_bulk, k_stage_group_shifted<float, false>, grid, b, s, g);
    }
    if (collide) return launch_follower(after_bulk, k_stage_group_shifted<__half, true>, grid, b, s, g);
    return launch_follower(after_bulk, k_stage_group_shifted<__half, false>, grid, b, s, g);
}

cudaError_t stage_batch_shifted(const StageParams *list, int n, const int2 *blocks, int nblocks,
                                int store, int sel, const ForceSlot *fs, bool after_bulk, cudaStream_t s) {
    if (nblocks == 0) return cudaSuccess;
    const dim3 g(nblocks), b(kStageBatchPoints);
    if (store == STORE_F32)
        return launch_follower(after_bulk, k_stage_batch_shifted<float>, g, b, s, list, blocks, sel, n, fs);
    return launch_follower(after_bulk, k_stage_batch_shifted<__half>, g, b, s, list, blocks, sel, n, fs);
}

cudaError_t collide_shifted(const CollideParams &p, int store, cudaStream_t s) {
    const dim3 b(64, 4);
    const dim3 g((p.Nx + 63) / 64, (p.Ny + 3) / 4);
    if (store == STORE_F32) k_collide_shifted<float><<<g, b, 0, s>>>(p);
    else k_collide_shifted<__half><<<g, b, 0, s>>>(p);
    return cudaGetLastError();
}


template <typename T, typename I, bool FORCE>
static cudaError_t step_shifted_tif(const FastStepParams &p, bool flags, bool collide, bool after, dim3 g, dim3 b,
                                    cudaStream_t s) {
    if (flags) {
        if (collide) return launch_follower(after, k_step_shifted_geo<T, I, true, FORCE>, g, b, s, p);
        return launch_follower(after, k_step_shifted_geo<T, I, false, FORCE>, g, b, s, p);
    }
    if (collide) return launch_follower(after, k_step_shifted_plain<T, I, true, FORCE>, g, b, s, p);
    return launch_follower(after, k_step_shifted_plain<T, I, false, FORCE>, g, b, s, p);
}

// The body force is a template parameter: force-free kernels carry no forcing
// code (fewer registers).
template <typename T, typename I>
static cudaError_t step_shifted_ti(const FastStepParams &p, bool flags, bool collide, bool after, dim3 g, dim3 b,
                                   cudaStream_t s) {
    if (p.s.has_force) return step_shifted_tif<T, I, true>(p, flags, collide, after, g, b, s);
    return step_shifted_tif<T, I, false>(p, flags, collide, after, g, b, s);
}

template <typename T>
static cudaError_t step_shifted_t(const FastStepParams &p, bool flags, bool collide, bool after, dim3 g, dim3 b,
                                  cudaStream_t s) {
    // 32-bit element offsets whenever all nine planes fit.
    if (9LL * p.s.plane < (1LL << 31)) return step_shifted_ti<T, int>(p, flags, collide, after, g, b, s);
    return step_shifted_ti<T, long long>(p, flags, collide, after, g, b, s);
}

cudaError_t step_shifted(const FastStepParams &p, int store, bool flags, bool collide, dim3 block,
                         cudaStream_t s, bool after) {
    // Two nodes per thread along x. after: the programmatic follower of the
    // special-node kernel launched just before it (the two touch disjoint
    // nodes, so it needs no wait).
    const dim3 g((p.s.Nx + 2 * block.x - 1) / (2 * block.x), (p.s.Ny + block.y - 1) / block.y);
    if (store == STORE_F32) return step_shifted_t<float>(p, flags, collide, after, g, block, s);
    return step_shifted_t<__half>(p, flags, collide, after, g, block, s);
}

template <typename T, typename I, bool FORCE, bool LINKS>
static cudaError_t special_shifted_tifl(const FastStepParams &p, const int2 *nodes, int n, bool flags, bool collide,
                                        bool after_bulk, cudaStream_t s) {
    const dim3 g((n + 127) / 128), b(128);
    if (flags) {
        if (collide)
            return launch_follower(after_bulk, k_step_special_shifted<T, I, true, true, FORCE, LINKS>, g, b, s, p,
                                   nodes, n);
        return launch_follower(after_bulk, k_step_special_shifted<T, I, true, false, FORCE, LINKS>, g, b, s, p, nodes,
                               n);
    }
    if (collide)
        return launch_follower(after_bulk, k_step_special_shifted<T, I, false, true, FORCE, LINKS>, g, b, s, p, nodes,
                               n);
    return launch_follower(after_bulk, k_step_special_shifted<T, I, false, false, FORCE, LINKS>, g, b, s, p, nodes, n);
}

template <typename T, typename I, bool FORCE>
static cudaError_t special_shifted_tif(const FastStepParams &p, const int2 *nodes, int n, bool flags, bool collide,
                                       bool after_bulk, cudaStream_t s) {
    if (p.s.links) return special_shifted_tifl<T, I, FORCE, true>(p, nodes, n, flags, collide, after_bulk, s);
    return special_shifted_tifl<T, I, FORCE, false>(p, nodes, n, flags, collide, after_bulk, s);
}

template <typename T>
static cudaError_t special_shifted_t(const FastStepParams &p, const int2 *nodes, int n, bool flags, bool collide,
                                     bool after_bulk, cudaStream_t s) {
    const bool wide = 9LL * p.s.plane >= (1LL << 31);
    if (p.s.has_force) {
        if (wide) return special_shifted_tif<T, long long, true>(p, nodes, n, flags, collide, after_bulk, s);
        return special_shifted_tif<T, int, true>(p, nodes, n, flags, collide, after_bulk, s);
    }
    if (wide) return special_shifted_tif<T, long long, false>(p, nodes, n, flags, collide, after_bulk, s);
    return special_shifted_tif<T, int, false>(p, nodes, n, flags, collide, after_bulk, s);
}

cudaError_t special_shifted(const FastStepParams &p, const int2 *nodes, int n, int store, bool flags, bool collide,
                            bool after_bulk, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (store == STORE_F32) return special_shifted_t<float>(p, nodes, n, flags, collide, after_bulk, s);
    return special_shifted_t<__half>(p, nodes, n, flags, collide, after_bulk, s);
}

template <typename T, bool FORCE, bool LINKS>
static cudaError_t special_batch_shifted_tfl(const FastStepParams *sp, const int4 *nodes, int n,
                                             int sel, bool wide, bool after, cudaStream_t s) {
    const dim3 g((n + 127) / 128), b(128);
    if (wide)
        return launch_follower(after, k_step_batch_special_shifted<T, long long, FORCE, LINKS>, g, b, s, sp, nodes,
                               n, sel);
    return launch_follower(after, k_step_batch_special_shifted<T, int, FORCE, LINKS>, g, b, s, sp, nodes, n, sel);
}

template <typename T>
static cudaError_t special_batch_shifted_t(const FastStepParams *sp, const int4 *nodes, int n,
                                           int sel, bool wide, bool force, bool links, bool after, cudaStream_t s) {
    if (force) {
        if (links) return special_batch_shifted_tfl<T, true, true>(sp, nodes, n, sel, wide, after, s);
        return special_batch_shifted_tfl<T, true, false>(sp, nodes, n, sel, wide, after, s);
    }
    if (links) return special_batch_shifted_tfl<T, false, true>(sp, nodes, n, sel, wide, after, s);
    return special_batch_shifted_tfl<T, false, false>(sp, nodes, n, sel, wide, after, s);
}

cudaError_t special_batch_shifted(const FastStepParams *sp, const int4 *nodes, int n, int sel,
                                  int store, bool wide, bool force, bool links, bool after, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (n % 32) return cudaErrorInvalidValue;
    if (store == STORE_F32) return special_batch_shifted_t<float>(sp, nodes, n, sel, wide, force, links, after, s);
    return special_batch_shifted_t<__half>(sp, nodes, n, sel, wide, force, links, after, s);
}

template <typename T, bool FORCE, bool ALLFLAGS>
static cudaError_t step_batch_shifted_tfa(const FastStepParams *sp, const int4 *tiles, int ntiles,
                                          int sel, int tws, bool wide, int grid, bool after, cudaStream_t s) {
    if (wide)
        return launch_follower(after, k_step_batch_shifted<T, long long, FORCE, ALLFLAGS>, dim3(grid), dim3(256), s,
                               sp, tiles, ntiles, sel, tws);
    return launch_follower(after, k_step_batch_shifted<T, int, FORCE, ALLFLAGS>, dim3(grid), dim3(256), s, sp, tiles,
                           ntiles, sel, tws);
}

template <typename T, bool FORCE>
static cudaError_t step_batch_shifted_tf(const FastStepParams *sp, const int4 *tiles, int ntiles,
                                         int sel, int tws, bool wide, bool all_flags, int grid, bool after,
                                         cudaStream_t s) {
    if (all_flags) return step_batch_shifted_tfa<T, FORCE, true>(sp, tiles, ntiles, sel, tws, wide, grid, after, s);
    return step_batch_shifted_tfa<T, FORCE, false>(sp, tiles, ntiles, sel, tws, wide, grid, after, s);
}

cudaError_t step_batch_shifted(const FastStepParams *sp, const int4 *tiles,
                               int ntiles, int sel, int tws, int store, bool wide, bool force, bool all_flags,
                               int grid, cudaStream_t s) {
    const bool after_special = false;  // an ordinary launch
    if (ntiles == 0) return cudaSuccess;
    if (tws < 5 || tws > 8) return cudaErrorInvalidValue;
    if (store == STORE_F32) {
        if (force)
            return step_batch_shifted_tf<float, true>(sp, tiles, ntiles, sel, tws, wide, all_flags, grid,
                                                      after_special, s);
        return step_batch_shifted_tf<float, false>(sp, tiles, ntiles, sel, tws, wide, all_flags, grid,
                                                   after_special, s);
    }
    if (force)
        return step_batch_shifted_tf<__half, true>(sp, tiles, ntiles, sel, tws, wide, all_flags, grid,
                                                   after_special, s);
    return step_batch_shifted_tf<__half, false>(sp, tiles, ntiles, sel, tws, wide, all_flags, grid,
                                                after_special, s);
}

int sm_count() {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return nsm > 0 ? nsm : 1;
}

int step_batch_shifted_grid(int store) {
    int nb = 0, dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (store == STORE_F32) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_step_batch_shifted<float, int, true, false>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_step_batch_shifted<__half, int, true, false>, 256, 0);
    return nsm * (nb > 0 ? nb : 1);
}

}  // namespace launch
}  // namespace lbm
