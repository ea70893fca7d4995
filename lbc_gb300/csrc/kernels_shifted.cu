// kernels_shifted.cu -- fused step with populations stored as shifted deviations
// g_k = f_k - w_k in FP32 or FP16 and the collision done in FP32.
//
// Same pull structure as the exact FP64 step (kernels_exact.cu): stream, halfway /
// interpolated / moving-wall bounce-back, stale slots off non-periodic edges, MEM
// force, moments, BGK + Guo collision. Storing g instead of f keeps the relative
// precision of the small deviations from the rest state; FP64 is used only for the
// force reduction and the band values handed to the edge BCs.
#include <cmath>

#include "kernels.h"
#include "lbm_device.cuh"
#include "reduce.cuh"

namespace lbm {

template <typename T> struct SV;
// rnd: the value as the storage type would hold it. Pre-collision values that
// are computed rather than loaded (bounce-back interpolation, edge BCs) are
// rounded to the storage type before the collision, so a run split into
// chunks (whose boundaries store and reload them) gives the same bits.
template <> struct SV<float> {
    static __device__ __forceinline__ float ld(const float *p) { return __ldg(p); }
    static __device__ __forceinline__ float ld_plain(const float *p) { return *p; }
    static __device__ __forceinline__ void st(float *p, float v) { *p = v; }
    static __device__ __forceinline__ float rnd(float v) { return v; }
};
template <> struct SV<__half> {
    static __device__ __forceinline__ float ld(const __half *p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ float ld_plain(const __half *p) { return __half2float(*p); }
    static __device__ __forceinline__ void st(__half *p, float v) { *p = __float2half_rn(v); }
    static __device__ __forceinline__ float rnd(float v) { return __half2float(__float2half_rn(v)); }
};

// Shifted moments: delta rho = sum g, j = sum c g (sum c w = 0). Jx, Jy are the
// momentum including half the body force (rho u of lbc).
__device__ __forceinline__ void moments_shifted(const float g[9], float hFx, float hFy, float &dr,
                                                float &rho, float &ux, float &uy, float &Jx,
                                                float &Jy) {
    dr = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + (g[6] + g[7])) + g[8];
    const float jx = (g[1] - g[3]) + (g[5] - g[6]) + (g[8] - g[7]);
    const float jy = (g[2] - g[4]) + (g[5] + g[6]) - (g[7] + g[8]);
    rho = 1.0f + dr;
    if (rho < 1e-16f) rho = 1e-16f;
    const float inv = 1.0f / rho;
    Jx = jx + hFx;
    Jy = jy + hFy;
    ux = Jx * inv;
    uy = Jy * inv;
}

// BGK + Guo on shifted populations, g' = g + om (geq - g) + (1 - om/2) F_k,
// with geq_k = w_k (drho + rho (3 c.u + 4.5 (c.u)^2 - 1.5 u.u)) built so that
// its mass and momentum are the node's own by construction: the odd part of
// each pair is h (c.J) with FP32 coefficients h1 = fl(3 w1) and
// h5 = (1 - 2 h1) / 4 whose sum rule 2 h1 + 4 h5 = 1 holds exactly, the linear
// term uses J = rho u directly (no division), and the rest population closes
// the mass. Rounded weights would otherwise bias every collision's momentum by
// ~1e-8 in the same direction, an error that grows linearly with the steps.
__device__ __forceinline__ void collide_shifted(float g[9], const float w[9], float dr, float rho,
                                                float ux, float uy, float Jx, float Jy, float om,
                                                bool force, float Fx, float Fy) {
    const float h1 = 3.0f * w[1];
    const float h5 = (1.0f - 2.0f * h1) * 0.25f;
    const float rt = 1.5f * (Jx * ux + Jy * uy);  // rho * 1.5 u.u
    float geq[9];
    {
        const float c = ux, J = Jx, X = w[1] * (dr + fmaf(4.5f * J, c, -rt)), Y = h1 * J;
        geq[1] = X + Y; geq[3] = X - Y;
    }
    {
        const float c = uy, J = Jy, X = w[2] * (dr + fmaf(4.5f * J, c, -rt)), Y = h1 * J;
        geq[2] = X + Y; geq[4] = X - Y;
    }
    {
        const float c = ux + uy, J = Jx + Jy, X = w[5] * (dr + fmaf(4.5f * J, c, -rt)), Y = h5 * J;
        geq[5] = X + Y; geq[7] = X - Y;
    }
    {
        const float c = uy - ux, J = Jy - Jx, X = w[6] * (dr + fmaf(4.5f * J, c, -rt)), Y = h5 * J;
        geq[6] = X + Y; geq[8] = X - Y;
    }
    geq[0] = dr - (((geq[1] + geq[3]) + (geq[2] + geq[4])) + ((geq[5] + geq[7]) + (geq[6] + geq[8])));
#pragma unroll
    for (int k = 0; k < 9; k++) g[k] = fmaf(om, geq[k] - g[k], g[k]);
    if (force) {
        const float uF = ux * Fx + uy * Fy;
        const float gf = 1.0f - 0.5f * om;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const float cu = cxk(k) * ux + cyk(k) * uy;
            const float cF = cxk(k) * Fx + cyk(k) * Fy;
            g[k] = fmaf(gf, w[k] * (3.0f * cF + 9.0f * cu * cF - 3.0f * uF), g[k]);
        }
    }
}

// Rare per-node outputs, kept out of line so the compiler cannot hoist their
// FP64 conversions into every thread's path (FP64 issue is slow on GB300).
template <typename T>
__device__ __noinline__ void solid_node_outputs(const StepParams &p, int i, int j, long long node,
                                                size_t dn, uint16_t fl) {
    if (p.write_macro) { p.rho[dn] = NAN; p.ux[dn] = NAN; p.uy[dn] = NAN; }
    if (fl & NF_BAND) {
        // A BC may read a solid neighbour: lbc sees the untouched buffer
        // content and NaN moments there.
        const int slot = band_slot(p.colbase, p.rowbase, i, j);
        const T *Dst = (const T *)p.dst;
#pragma unroll
        for (int k = 0; k < 9; k++)
            p.bandf[(size_t)k * p.nslots + slot] = (double)SV<T>::ld_plain(Dst + k * p.plane + node) + p.w[k];
        p.bandm_next[slot] = NAN;
        p.bandm_next[(size_t)p.nslots + slot] = NAN;
        p.bandm_next[2 * (size_t)p.nslots + slot] = NAN;
    }
}

__device__ __noinline__ void band_store_f(const StepParams &p, int slot, float g0, float g1, float g2,
                                          float g3, float g4, float g5, float g6, float g7, float g8) {
    const float g[9] = {g0, g1, g2, g3, g4, g5, g6, g7, g8};
#pragma unroll
    for (int k = 0; k < 9; k++) p.bandf[(size_t)k * p.nslots + slot] = (double)g[k] + p.w[k];
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

// One node of the fused step in shifted storage. I is the element-offset type:
// int whenever all nine planes fit in 2^31 elements (fewer address
// instructions), long long otherwise.
template <typename T, typename I, bool FLAGS, bool COLLIDE>
__device__ __forceinline__ void step_node_shifted(const FastStepParams &fp, int i, int j,
                                                  float &mfx, float &mfy, bool &link) {
    const StepParams &p = fp.s;
    const I node = (I)j * (I)p.pitch + (I)i;
    const uint16_t fl = FLAGS ? p.flags[node] : (uint16_t)0;
    const size_t dn = (size_t)j * (size_t)p.Nx + (size_t)i;
    if (FLAGS && (fl & NF_SOLID)) {
        solid_node_outputs<T>(p, i, j, (long long)node, dn, fl);
        return;
    }
    const T *S = (const T *)p.src;
    T *Dst = (T *)p.dst;
    const I pl = (I)p.plane;
    // Source neighbours: wrapped on periodic axes, clamped otherwise so that
    // all nine loads are in bounds and can be issued at once; the flag word
    // then says which of them to replace.
    int im = i - 1, ip = i + 1, jm = j - 1, jp = j + 1;
    if (p.px) { if (im < 0) im += p.Nx; if (ip >= p.Nx) ip -= p.Nx; }
    else { im = max(im, 0); ip = min(ip, p.Nx - 1); }
    if (p.py) { if (jm < 0) jm += p.Ny; if (jp >= p.Ny) jp -= p.Ny; }
    else { jm = max(jm, 0); jp = min(jp, p.Ny - 1); }
    const I r0 = (I)j * (I)p.pitch, rm = (I)jm * (I)p.pitch, rp = (I)jp * (I)p.pitch;
    const I so[9] = {r0 + i, r0 + im, rm + i, r0 + ip, rp + i, rm + im, rm + ip, rp + ip, rp + im};
    float g[9];
#pragma unroll
    for (int k = 0; k < 9; k++) g[k] = SV<T>::ld(S + (I)k * pl + so[k]);
    if (FLAGS && (fl & NF_SPECIAL_MASK)) {
        const Link *lk = (fl & NF_LINKS) ? p.links + p.link_off[node] : nullptr;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            if (!(fl & (1u << k))) continue;
            const int si = i - cxk(k), sj = j - cyk(k);
            const bool off = (!p.px && (si < 0 || si >= p.Nx)) || (!p.py && (sj < 0 || sj >= p.Ny));
            if (off) {
                g[k] = SV<T>::ld_plain(Dst + (I)k * pl + node);
                continue;
            }
            const int ko = oppk(k);
            const float own = SV<T>::ld(S + (I)ko * pl + node);
            float val = own;
            if (lk) {
                const Link L = *lk++;
                if (L.mode == LINK_IBB_LO)
                    val = (float)L.c1 * own + (float)L.c2 * SV<T>::ld(S + (I)ko * pl + (I)L.behind);
                else if (L.mode == LINK_IBB_HI)
                    val = (float)L.c1 * own + (float)L.c2 * SV<T>::ld(S + (I)k * pl + (I)L.behind);
                else if (L.mode == LINK_MOVING)
                    val = own - (float)L.c2;
            }
            g[k] = SV<T>::rnd(val);
            // Per-node link sum in FP32 (a few terms); block and case sums are FP64.
            const float df = (own + val) + 2.0f * fp.wf[k];
            mfx -= df * cxk(k);
            mfy -= df * cyk(k);
            link = true;
        }
    }
    int slot = -1;
    if (FLAGS && (fl & NF_BAND)) {
        slot = band_slot(p.colbase, p.rowbase, i, j);
        band_store_f(p, slot, g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7], g[8]);
    }
    if (FLAGS && (fl & NF_BCW)) return;
    float dr, rho, ux, uy, Jx, Jy;
    moments_shifted(g, fp.hFxf, fp.hFyf, dr, rho, ux, uy, Jx, Jy);
    if (FLAGS) {
        if (p.write_macro || slot >= 0) macro_store(p, dn, slot, dr, ux, uy);
    } else if (p.write_macro) {
        p.rho[dn] = 1.0 + (double)dr;
        p.ux[dn] = ux;
        p.uy[dn] = uy;
    }
    if (COLLIDE) {
        const float om = p.omega ? (float)p.omega[dn] : fp.omega0f;
        collide_shifted(g, fp.wf, dr, rho, ux, uy, Jx, Jy, om, p.has_force != 0, fp.Fxf, fp.Fyf);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) SV<T>::st(Dst + (I)k * pl + node, g[k]);
}

// Fully periodic grid without solids or edge BCs: no flag word, 32 registers.
template <typename T, typename I, bool COLLIDE>
__global__ void __launch_bounds__(256) k_step_shifted_plain(const FastStepParams fp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    float mfx = 0.f, mfy = 0.f;
    bool link = false;
    if (i < fp.s.Nx && j < fp.s.Ny) step_node_shifted<T, I, false, COLLIDE>(fp, i, j, mfx, mfy, link);
}

// General geometry (flag word per node). The occupancy hint keeps it at five
// resident blocks per SM (48 registers) without spills.
template <typename T, typename I, bool COLLIDE>
__global__ void __launch_bounds__(256, 5) k_step_shifted_geo(const FastStepParams fp) {
    const StepParams &p = fp.s;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    float mfx = 0.f, mfy = 0.f;
    bool link = false;
    if (i < p.Nx && j < p.Ny) step_node_shifted<T, I, true, COLLIDE>(fp, i, j, mfx, mfy, link);
    if (p.mem_partials) segment_reduce2_store(mfx, mfy, link, i, j, p.Nx, p.seg_slot, p.mem_partials);
}

// Batched form (see k_step_batch_exact in kernels_exact.cu).
template <typename T>
__global__ void __launch_bounds__(256, 4) k_step_batch_shifted(const FastStepParams *__restrict__ sp,
                                                            const int *__restrict__ phase,
                                                            const int4 *__restrict__ tiles,
                                                            int ntiles, int sel, int tws) {
    const int tx = threadIdx.x & ((1 << tws) - 1), ty = threadIdx.x >> tws;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int4 td = tiles[t];
        const FastStepParams &fp = sp[2 * td.x + (sel ^ phase[td.x])];
        const int i = td.y + tx, j = td.z + ty;
        float mfx = 0.f, mfy = 0.f;
        bool link = false;
        const bool in = i < fp.s.Nx && j < fp.s.Ny;
        if (fp.s.flags) {
            if (in) step_node_shifted<T, long long, true, true>(fp, i, j, mfx, mfy, link);
        } else {
            if (in) step_node_shifted<T, long long, false, true>(fp, i, j, mfx, mfy, link);
        }
        if (td.w) segment_reduce2_store(mfx, mfy, link, i, j, fp.s.Nx, fp.s.seg_slot, fp.s.mem_partials);
    }
}

template <typename T, bool COLLIDE>
__device__ __forceinline__ void finish_node_shifted(const FinishParams &p, int2 ij) {
    const int slot = band_slot(p.colbase, p.rowbase, ij.x, ij.y);
    float g[9], wf[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
        g[k] = SV<T>::rnd((float)(p.bandf[(size_t)k * p.nslots + slot] - p.w[k]));
        wf[k] = (float)p.w[k];
    }
    float dr, rho, ux, uy, Jx, Jy;
    moments_shifted(g, (float)p.hFx, (float)p.hFy, dr, rho, ux, uy, Jx, Jy);
    const size_t dn = (size_t)ij.y * p.Nx + ij.x;
    if (p.write_macro) { p.rho[dn] = 1.0 + (double)dr; p.ux[dn] = ux; p.uy[dn] = uy; }
    p.bandm_next[slot] = 1.0 + (double)dr;
    p.bandm_next[(size_t)p.nslots + slot] = ux;
    p.bandm_next[2 * (size_t)p.nslots + slot] = uy;
    if (COLLIDE) {
        const float om = p.omega ? (float)p.omega[dn] : (float)p.omega0;
        collide_shifted(g, wf, dr, rho, ux, uy, Jx, Jy, om, p.has_force != 0, (float)p.Fx, (float)p.Fy);
    }
    T *D = (T *)p.dst;
    const long long node = (long long)ij.y * p.pitch + ij.x;
#pragma unroll
    for (int k = 0; k < 9; k++) SV<T>::st(D + k * p.plane + node, g[k]);
}

template <typename T, bool COLLIDE>
__global__ void k_finish_shifted(const FinishParams p) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.nw) return;
    finish_node_shifted<T, COLLIDE>(p, p.wnodes[t]);
}

template <typename T>
__global__ void k_finish_batch_shifted(const FinishParams *__restrict__ fp, const int *__restrict__ phase,
                                       const int4 *__restrict__ nodes, int n, int sel) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int4 c = nodes[t];
    finish_node_shifted<T, true>(fp[2 * c.x + (sel ^ phase[c.x])], make_int2(c.y, c.z));
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
    float dr, rho, ux, uy, Jx, Jy;
    if (p.from_pops) {
        moments_shifted(g, (float)(0.5 * p.Fx), (float)(0.5 * p.Fy), dr, rho, ux, uy, Jx, Jy);
    } else {
        rho = (float)p.rho[dn];
        dr = (float)(p.rho[dn] - 1.0);
        ux = (float)p.ux[dn];
        uy = (float)p.uy[dn];
        Jx = (float)(p.rho[dn] * p.ux[dn]);
        Jy = (float)(p.rho[dn] * p.uy[dn]);
    }
    collide_shifted(g, wf, dr, rho, ux, uy, Jx, Jy, om, p.has_force != 0, (float)p.Fx, (float)p.Fy);
#pragma unroll
    for (int k = 0; k < 9; k++) SV<T>::st(F + k * p.plane + node, g[k]);
}

namespace launch {

cudaError_t collide_shifted(const CollideParams &p, int store, cudaStream_t s) {
    const dim3 b(64, 4);
    const dim3 g((p.Nx + 63) / 64, (p.Ny + 3) / 4);
    if (store == STORE_F32) k_collide_shifted<float><<<g, b, 0, s>>>(p);
    else k_collide_shifted<__half><<<g, b, 0, s>>>(p);
    return cudaGetLastError();
}


template <typename T, typename I>
static void step_shifted_ti(const FastStepParams &p, bool flags, bool collide, dim3 g, dim3 b,
                            cudaStream_t s) {
    if (flags) {
        if (collide) k_step_shifted_geo<T, I, true><<<g, b, 0, s>>>(p);
        else k_step_shifted_geo<T, I, false><<<g, b, 0, s>>>(p);
    } else {
        if (collide) k_step_shifted_plain<T, I, true><<<g, b, 0, s>>>(p);
        else k_step_shifted_plain<T, I, false><<<g, b, 0, s>>>(p);
    }
}

template <typename T>
static void step_shifted_t(const FastStepParams &p, bool flags, bool collide, dim3 g, dim3 b,
                           cudaStream_t s) {
    // 32-bit element offsets whenever all nine planes fit.
    if (9LL * p.s.plane < (1LL << 31)) step_shifted_ti<T, int>(p, flags, collide, g, b, s);
    else step_shifted_ti<T, long long>(p, flags, collide, g, b, s);
}

cudaError_t step_shifted(const FastStepParams &p, int store, bool flags, bool collide, dim3 block,
                         cudaStream_t s) {
    const dim3 g((p.s.Nx + block.x - 1) / block.x, (p.s.Ny + block.y - 1) / block.y);
    if (store == STORE_F32) step_shifted_t<float>(p, flags, collide, g, block, s);
    else step_shifted_t<__half>(p, flags, collide, g, block, s);
    return cudaGetLastError();
}

cudaError_t step_batch_shifted(const FastStepParams *sp, const int *phase, const int4 *tiles,
                               int ntiles, int sel, int tws, int store, int grid, cudaStream_t s) {
    if (ntiles == 0) return cudaSuccess;
    if (tws < 5 || tws > 8) return cudaErrorInvalidValue;
    if (store == STORE_F32) k_step_batch_shifted<float><<<grid, 256, 0, s>>>(sp, phase, tiles, ntiles, sel, tws);
    else k_step_batch_shifted<__half><<<grid, 256, 0, s>>>(sp, phase, tiles, ntiles, sel, tws);
    return cudaGetLastError();
}

int step_batch_shifted_grid(int store) {
    int nb = 0, dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (store == STORE_F32) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_step_batch_shifted<float>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_step_batch_shifted<__half>, 256, 0);
    return nsm * (nb > 0 ? nb : 1);
}

cudaError_t finish_batch_shifted(const FinishParams *fp, const int *phase, const int4 *nodes, int n,
                                 int sel, int store, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (store == STORE_F32) k_finish_batch_shifted<float><<<(n + 127) / 128, 128, 0, s>>>(fp, phase, nodes, n, sel);
    else k_finish_batch_shifted<__half><<<(n + 127) / 128, 128, 0, s>>>(fp, phase, nodes, n, sel);
    return cudaGetLastError();
}

cudaError_t finish_shifted(const FinishParams &p, int store, bool collide, cudaStream_t s) {
    if (p.nw == 0) return cudaSuccess;
    const int b = 128, g = (p.nw + b - 1) / b;
    if (store == STORE_F32) {
        if (collide) k_finish_shifted<float, true><<<g, b, 0, s>>>(p);
        else k_finish_shifted<float, false><<<g, b, 0, s>>>(p);
    } else {
        if (collide) k_finish_shifted<__half, true><<<g, b, 0, s>>>(p);
        else k_finish_shifted<__half, false><<<g, b, 0, s>>>(p);
    }
    return cudaGetLastError();
}

}  // namespace launch
}  // namespace lbm
