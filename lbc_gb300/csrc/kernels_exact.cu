// kernels_exact.cu -- FP64 kernels that reproduce lbc's arithmetic bit for bit.
//
// Compiled with --fmad=false: every multiply and add rounds separately, in the
// order the reference C code evaluates them, so results match lbc's FP64 CPU
// solver exactly (signed zeros aside) on identical inputs.
//
// Contents:
//   * k_step_exact      fused pull step (stream + halfway/interpolated/moving-wall
//                       bounce-back + stale slots + MEM force + moments + BGK/Guo
//                       collision), one thread per node, SoA planes
//   * k_stage_group     a group of edge BCs of the Boundary list on the band
//                       buffer; each thread then finishes (moments + collision)
//                       the node its entry writes last; k_stage_batch for batches
//   * k_force_reduce    per-case force from its partials
//   * k_collide_exact   in-place collision with stored rho/u/v (first step)
//   * AoS kernels       lbc's standalone functions on lbc's own layout
//   * transposes        lbc AoS <-> device SoA, with FP32/FP16 shifted storage
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "kernels.h"
#include "lbm_device.cuh"
#include "pdl.cuh"
#include "reduce.cuh"

namespace lbm {

// ---------------------------------------------------------------- fused step

// src/core/main_lbm.c:31-61 restructured as a pull: the state entering the
// kernel is the post-collision f of step n (what lbc's collision leaves in f),
// each fluid node gathers f_new from its neighbours (src/core/streaming.c:20-42),
// takes bounce-back values where the source is solid (src/bc/bounce_back.c:42-46,
// src/bc/interpolated_bounce_back.c:91-100), keeps the old content of its slot
// where the source is off a non-periodic edge (src/core/streaming.c:36-37), adds
// its momentum-exchange terms (src/core/compute_force_mem.c:51-58), computes
// moments (src/core/compute_macroscopic_fields.c:23-46) and, unless it is written
// by an edge BC, collides (src/core/collision.c:22-38) and stores.
// FMA: moments_fma / collide_fma instead of lbc's rounding sequence (the same
// step to rounding, in 74 FP64 instructions per node instead of 125).
template <bool FLAGS, bool COLLIDE, bool FMA = false>
__device__ __forceinline__ void step_node_exact(const StepParams &p, int i, int j, double &mfx,
                                                double &mfy, bool &link) {
    {
        const long long node = (long long)j * p.pitch + i;
        const uint16_t fl = FLAGS ? p.flags[node] : (uint16_t)0;
        const size_t dn = (size_t)j * (size_t)p.Nx + (size_t)i;
        if (FLAGS && (fl & NF_SOLID)) {
            if (p.write_macro) { p.rho[dn] = NAN; p.ux[dn] = NAN; p.uy[dn] = NAN; }
            if (fl & NF_BAND) {
                // A BC may read a solid neighbour: lbc sees the untouched buffer
                // content and NaN moments there.
                const int slot = band_slot(p.colbase, p.rowbase, i, j);
                const double *Dst = (const double *)p.dst;
#pragma unroll
                for (int k = 0; k < 9; k++) p.bandf[(size_t)k * p.nslots + slot] = Dst[k * p.plane + node];
                p.bandm_next[slot] = NAN;
                p.bandm_next[(size_t)p.nslots + slot] = NAN;
                p.bandm_next[2 * (size_t)p.nslots + slot] = NAN;
            }
        } else {
            const double *S = (const double *)p.src;
            double *Dst = (double *)p.dst;
            const long long pl = p.plane;
            // Wrapped on periodic axes, clamped otherwise (all loads in bounds,
            // issued together); the flag word says which ones to replace.
            int im = i - 1, ip = i + 1, jm = j - 1, jp = j + 1;
            if (p.px) { if (im < 0) im += p.Nx; if (ip >= p.Nx) ip -= p.Nx; }
            else { im = max(im, 0); ip = min(ip, p.Nx - 1); }
            if (p.py) { if (jm < 0) jm += p.Ny; if (jp >= p.Ny) jp -= p.Ny; }
            else { jm = max(jm, 0); jp = min(jp, p.Ny - 1); }
            const long long r0 = (long long)j * p.pitch, rm = (long long)jm * p.pitch,
                            rp = (long long)jp * p.pitch;
            const long long so[9] = {r0 + i, r0 + im, rm + i, r0 + ip, rp + i,
                                     rm + im, rm + ip, rp + ip, rp + im};
            double f[9];
#pragma unroll
            for (int k = 0; k < 9; k++) f[k] = S[k * pl + so[k]];
            if (FLAGS && (fl & NF_SPECIAL_MASK)) {
                const Link *lk = (fl & NF_LINKS) ? p.links + p.link_off[node] : nullptr;
#pragma unroll
                for (int k = 0; k < 9; k++) {
                    if (!(fl & (1u << k))) continue;
                    const int si = i - cxk(k), sj = j - cyk(k);
                    const bool off = (!p.px && (si < 0 || si >= p.Nx)) ||
                                     (!p.py && (sj < 0 || sj >= p.Ny));
                    if (off) {
                        f[k] = Dst[k * pl + node];
                        continue;
                    }
                    const int ko = oppk(k);
                    const double own = S[ko * pl + node];
                    double val = own;
                    if (lk) {
                        const Link L = *lk++;
                        if (L.mode == LINK_IBB_LO) val = L.c1 * own + L.c2 * S[ko * pl + L.behind];
                        else if (L.mode == LINK_IBB_HI) val = L.c1 * own + L.c2 * S[k * pl + L.behind];
                        else if (L.mode == LINK_MOVING) val = own - L.c2;
                    }
                    f[k] = val;
                    const double df = own + val;
                    mfx -= df * cxk(k);
                    mfy -= df * cyk(k);
                    link = true;
                }
            }
            int slot = -1;
            if (FLAGS && (fl & NF_BAND)) {
                slot = band_slot(p.colbase, p.rowbase, i, j);
#pragma unroll
                for (int k = 0; k < 9; k++) p.bandf[(size_t)k * p.nslots + slot] = f[k];
            }
            if (!(FLAGS && (fl & NF_BCW))) {
                double rho, ux, uy;
                if (FMA) moments_fma(f, p.hFx, p.hFy, p.has_force != 0, rho, ux, uy);
                else moments_exact(f, p.hFx, p.hFy, rho, ux, uy);
                if (p.write_macro) { p.rho[dn] = rho; p.ux[dn] = ux; p.uy[dn] = uy; }
                if (slot >= 0) {
                    p.bandm_next[slot] = rho;
                    p.bandm_next[(size_t)p.nslots + slot] = ux;
                    p.bandm_next[2 * (size_t)p.nslots + slot] = uy;
                }
                if (COLLIDE) {
                    const double om = p.omega ? p.omega[dn] : p.omega0;
                    if (FMA) collide_fma(f, p.w[0], p.w[1], p.w[5], rho, ux, uy, om, p.has_force != 0, p.Fx, p.Fy);
                    else collide_exact(f, p.w, rho, ux, uy, om, p.has_force != 0, p.Fx, p.Fy);
                }
#pragma unroll
                for (int k = 0; k < 9; k++) Dst[k * pl + node] = f[k];
            }
        }
    }
}

template <bool FLAGS, bool COLLIDE, bool FMA>
__global__ void __launch_bounds__(256) k_step_exact(const StepParams p) {
    pdl_launch_dependents();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double mfx = 0.0, mfy = 0.0;
    bool link = false;
    if (i < p.Nx && j < p.Ny) step_node_exact<FLAGS, COLLIDE, FMA>(p, i, j, mfx, mfy, link);
    if (FLAGS && p.mem_partials) segment_reduce2_store(mfx, mfy, link, i, j, p.Nx, p.seg_slot, p.mem_partials);
}

// Many cases in one launch: a persistent loop over a flattened list of
// 2D tiles (one tile = one thread block's worth of nodes of one case: 256
// threads as 2^tws x 2^(8 - tws) nodes). Each case brings its own parameters
// (sp[2 * c + sel]: the two ping-pong directions), so uneven
// grids and different geometries share the launch. Force partials go to each
// case's own segment slots (td.w != 0: the tile contains wall links), reduced
// per case by k_force_reduce exactly as when the case runs alone.
template <bool FMA>
__global__ void __launch_bounds__(256) k_step_batch_exact(const StepParams *__restrict__ sp,
                                                          const int4 *__restrict__ tiles, int ntiles,
                                                          int sel, int tws) {
    pdl_launch_dependents();
    const int tx = threadIdx.x & ((1 << tws) - 1), ty = threadIdx.x >> tws;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int4 td = tiles[t];
        const StepParams &p = sp[2 * td.x + sel];
        const int i = td.y + tx, j = td.z + ty;
        double mfx = 0.0, mfy = 0.0;
        bool link = false;
        const bool in = i < p.Nx && j < p.Ny;
        if (p.flags) {
            if (in) step_node_exact<true, true, FMA>(p, i, j, mfx, mfy, link);
        } else {
            if (in) step_node_exact<false, true, FMA>(p, i, j, mfx, mfy, link);
        }
        if (td.w && p.mem_partials) segment_reduce2_store(mfx, mfy, link, i, j, p.Nx, p.seg_slot, p.mem_partials);
    }
}

// ---------------------------------------------------------------- edge BCs

// The band as lbc's BC functions see it. Lookups of the thread's own node and
// of its interior neighbour come from the thread's preload (StagePre).
template <typename T> struct BandAccessor {
    const StageParams &p;
    const StagePre &c;
    bool live;  // false: no stores (instruction-cache warm-up pass)
    __device__ int slot(int i, int j) const {
        if (i == c.ij.x && j == c.ij.y) return c.slot;
        if (i == c.nij.x && j == c.nij.y) return c.nslot;
        return band_slot(p.colbase, p.rowbase, i, j);
    }
    __device__ bool nb(int i, int j) const { return i == c.nij.x && j == c.nij.y; }
    __device__ double get(int i, int j, int k) const { return __ldcg(p.bandf + (size_t)k * p.nslots + slot(i, j)); }
    __device__ void set(int i, int j, int k, double v) const {
        if (live) p.bandf[(size_t)k * p.nslots + slot(i, j)] = v;
    }
    __device__ double rho(int i, int j) const { return nb(i, j) ? c.nrho : p.bandm_prev[slot(i, j)]; }
    __device__ double ux(int i, int j) const {
        return nb(i, j) ? c.nux : p.bandm_prev[(size_t)p.nslots + slot(i, j)];
    }
    __device__ double uy(int i, int j) const {
        return nb(i, j) ? c.nuy : p.bandm_prev[2 * (size_t)p.nslots + slot(i, j)];
    }
    __device__ double post(int i, int j, int k) const {
        return Store<T>::to_f64(((const T *)p.src)[k * p.plane + (long long)j * p.pitch + i], p.w[k]);
    }
    __device__ bool solid(int i, int j) const {
        if (i == c.ij.x && j == c.ij.y) return c.solid;
        return (p.flags[(long long)j * p.pitch + i] & NF_SOLID) != 0;
    }
};

// One entry of lbc's Boundary list (src/core/main_lbm.c:49-58) at point t,
// applied to the pre-collision f_new of the band nodes, after the preload c.
// Entries in different launches see the writes of the earlier ones, as in lbc.
template <typename T>
__device__ __forceinline__ void stage_point(const StageParams &p, const StagePre &c, int t, int kind, bool live) {
    BandAccessor<T> a{p, c, live};
    if (kind == BC_VEL_BOT_REG && c.imp) {
        bc_regularized(a, p.w, t, p.index, t, p.index + 1, false, c.v1, c.v2);
        return;
    }
    bc_apply(a, p.w, kind, p.Nx, p.Ny, p.index, t, c.v1, c.v2);
}

// Moments and collision of a node an edge BC wrote (band slot `slot`).
// live = false: the same instructions without their stores (warm-up pass);
// band populations are read at L2, never from a possibly stale L1 line.
template <bool COLLIDE>
__device__ __forceinline__ void finish_node_exact(const FinishParams &p, int2 ij, int slot, bool live) {
    double f[9];
#pragma unroll
    for (int k = 0; k < 9; k++) f[k] = __ldcg(p.bandf + (size_t)k * p.nslots + slot);
    double rho, ux, uy;
    moments_exact(f, p.hFx, p.hFy, rho, ux, uy);
    const size_t dn = (size_t)ij.y * p.Nx + ij.x;
    if (live) {
        if (p.write_macro) { p.rho[dn] = rho; p.ux[dn] = ux; p.uy[dn] = uy; }
        p.bandm_next[slot] = rho;
        p.bandm_next[(size_t)p.nslots + slot] = ux;
        p.bandm_next[2 * (size_t)p.nslots + slot] = uy;
    }
    if (COLLIDE) {
        const double om = p.omega ? p.omega[dn] : p.omega0;
        collide_exact(f, p.w, rho, ux, uy, om, p.has_force != 0, p.Fx, p.Fy);
    }
    double *D = (double *)p.dst;
    const long long node = (long long)ij.y * p.pitch + ij.x;
    if (live) {
#pragma unroll
        for (int k = 0; k < 9; k++) D[k * p.plane + node] = f[k];
    }
}

// One stage thread, specialised on the entry's kind; with warm set, a
// store-free pass before the wait warms the instruction cache (as
// stage_thread_s in kernels_shifted.cu). In FP64 that pass repeats the BC's
// and the collision's FP64 work beside the FP64-bound bulk kernel, so the
// host sets warm only for small grids, where the bulk kernel is short and the
// fetch latency is exposed (measured: cylinder 512x128 36.0 -> 32.9 ms per
// 1000 steps with it, 35.0 without; 2048x512 82.2 -> 83.5 with it, 81.8
// without).
template <typename T, bool COLLIDE, int KIND>
__device__ __forceinline__ void stage_thread(const StageParams &p, const FinishParams &f, int t, int warm) {
    const StagePre c = stage_preload(p, t, KIND);
#pragma unroll 1
    for (int pass = warm ? 0 : 1; pass < 2; pass++) {
        const bool live = pass != 0;
        if (live) pdl_wait();
        stage_point<T>(p, c, t, KIND, live);
        if (c.fin) finish_node_exact<COLLIDE>(f, c.ij, c.slot, live);
    }
}

template <typename T, bool COLLIDE>
__device__ __forceinline__ void stage_dispatch(const StageParams &p, const FinishParams &f, int t, int warm) {
    switch (p.kind) {
#define LBM_STAGE_KIND(K) \
    case K: stage_thread<T, COLLIDE, K>(p, f, t, warm); break;
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

// One group of Boundary entries of a case (blockIdx.y = member); a member
// thread finishes its node when its entry is the node's last writer
// (StageParams.last); row n reduces the case's force. Launched right behind
// the bulk kernel (pdl.cuh): everything up to pdl_wait() reads only what the
// bulk kernel does not write.
template <typename T, bool COLLIDE>
__global__ void k_stage_group(const StageGroup g) {
    if ((int)blockIdx.y >= g.n) {
        pdl_wait();
        if (blockIdx.x == 0 && threadIdx.x < 32) force_reduce_warp(*g.fs, (int)threadIdx.x);
        return;
    }
    const StageParams &p = g.p[blockIdx.y];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.along) return;
    stage_dispatch<T, COLLIDE>(p, g.fin, t, g.warm);
}

// Stage level of every case of a batch: block b steps points blk[b].y ..
// of entry e = blk[b].x, list[2 * e + sel] its parameters for this
// ping-pong direction; e >= n: reduce force slot fs[e - n].
template <typename T>
__global__ void k_stage_batch(const StageParams *__restrict__ list,
                              const int2 *__restrict__ blk, int sel, int n, const ForceSlot *__restrict__ fs,
                              int warm) {
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
    stage_dispatch<T, true>(p, *p.fin, t, warm);
}

// Per-case force of a step from its segment partials (one warp per case).
__global__ void k_force_reduce(const ForceSlot *__restrict__ slots, int nslots) {
    pdl_wait();
    const int c = blockIdx.x;
    if (c >= nslots) return;
    force_reduce_warp(slots[c], (int)threadIdx.x);
}

// In-place collision with the stored rho/u/v (src/core/collision.c:18-40); used
// for the first step, whose stored fields are the caller's arrays.
__global__ void k_collide_exact(const CollideParams p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= p.Nx || j >= p.Ny) return;
    const long long node = (long long)j * p.pitch + i;
    const uint16_t fl = p.flags ? p.flags[node] : (uint16_t)0;
    if (fl & NF_SOLID) return;
    const size_t dn = (size_t)j * p.Nx + i;
    double f[9];
#pragma unroll
    for (int k = 0; k < 9; k++) f[k] = p.f[k * p.plane + node];
    const double om = p.omega ? p.omega[dn] : p.omega0;
    // In the fused FMA step the nodes an edge BC writes are collided by the
    // stage launch's finish in lbc's arithmetic, the others in the FMA form:
    // the same split here, so that run(a) + run(b) = run(a + b) bit for bit.
    if (p.fma && !(fl & NF_BCW))
        collide_fma(f, p.w[0], p.w[1], p.w[5], p.rho[dn], p.ux[dn], p.uy[dn], om, p.has_force != 0, p.Fx, p.Fy);
    else collide_exact(f, p.w, p.rho[dn], p.ux[dn], p.uy[dn], om, p.has_force != 0, p.Fx, p.Fy);
#pragma unroll
    for (int k = 0; k < 9; k++) p.f[k * p.plane + node] = f[k];
}

// Collision over lbc's AoS array in place (src/core/collision.c:18-40), with the
// result also stored in the device SoA planes. Blocks stage 128 consecutive
// nodes through shared memory so the AoS traffic (over NVLink-C2C when the
// array is host memory) is one contiguous run per block.
__global__ void __launch_bounds__(128) k_collide_aos_exact(const CollideAosParams p) {
    __shared__ double tile[128 * 9];
    const long long n0 = (long long)blockIdx.x * 128;
    const long long N = (long long)p.Nx * p.Ny;
    const int cnt = (int)min((long long)128, N - n0);
    for (int e = threadIdx.x; e < cnt * 9; e += blockDim.x) tile[e] = p.f_aos[n0 * 9 + e];
    __syncthreads();
    const int r = threadIdx.x;
    if (r < cnt) {
        const long long n = n0 + r;
        const int j = (int)(n / p.Nx), i = (int)(n - (long long)j * p.Nx);
        const long long node = (long long)j * p.pitch + i;
        double f[9];
#pragma unroll
        for (int k = 0; k < 9; k++) f[k] = tile[r * 9 + k];
        if (!(p.flags && (p.flags[node] & NF_SOLID))) {
            const double om = p.omega ? p.omega[n] : p.omega0;
            collide_exact(f, p.w, p.rho[n], p.ux[n], p.uy[n], om, p.has_force != 0, p.Fx, p.Fy);
#pragma unroll
            for (int k = 0; k < 9; k++) tile[r * 9 + k] = f[k];
        }
#pragma unroll
        for (int k = 0; k < 9; k++) p.soa[k * p.plane + node] = f[k];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * 9; e += blockDim.x) p.f_aos[n0 * 9 + e] = tile[e];
}

// ---------------------------------------------------------------- transposes

// lbc AoS [Ny][Nx][9] (dense) -> device SoA planes of type T.
template <typename T>
__global__ void k_aos_to_soa(const double *__restrict__ aos, T *__restrict__ soa, int Nx, int Ny,
                             int pitch, long long plane, Wt w) {
    __shared__ double tile[128 * 9];
    const long long n0 = (long long)blockIdx.x * 128;
    const long long N = (long long)Nx * Ny;
    const int cnt = (int)min((long long)128, N - n0);
    for (int e = threadIdx.x; e < cnt * 9; e += blockDim.x) tile[e] = aos[n0 * 9 + e];
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * 9; e += blockDim.x) {
        const int k = e / cnt, r = e - k * cnt;
        const long long n = n0 + r;
        const int j = (int)(n / Nx), i = (int)(n - (long long)j * Nx);
        soa[k * plane + (long long)j * pitch + i] = Store<T>::from_f64(tile[r * 9 + k], w.w[k]);
    }
}

template <typename T>
__global__ void k_soa_to_aos(const T *__restrict__ soa, double *__restrict__ aos, int Nx, int Ny,
                             int pitch, long long plane, Wt w) {
    __shared__ double tile[128 * 9];
    const long long n0 = (long long)blockIdx.x * 128;
    const long long N = (long long)Nx * Ny;
    const int cnt = (int)min((long long)128, N - n0);
    for (int e = threadIdx.x; e < cnt * 9; e += blockDim.x) {
        const int k = e / cnt, r = e - k * cnt;
        const long long n = n0 + r;
        const int j = (int)(n / Nx), i = (int)(n - (long long)j * Nx);
        tile[r * 9 + k] = Store<T>::to_f64(soa[k * plane + (long long)j * pitch + i], w.w[k]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * 9; e += blockDim.x) aos[n0 * 9 + e] = tile[e];
}

// Band moments of the first step come from the caller's stored rho/u/v.
__global__ void k_seed_band(const int2 *nodes, const int *slots, int n, int Nx, const double *rho,
                            const double *ux, const double *uy, double *bandm, int nslots) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const size_t dn = (size_t)nodes[t].y * Nx + nodes[t].x;
    const int s = slots[t];
    bandm[s] = rho[dn];
    bandm[(size_t)nslots + s] = ux[dn];
    bandm[2 * (size_t)nslots + s] = uy[dn];
}

// ---------------------------------------------------------------- AoS kernels
// lbc's standalone functions on lbc's own layout, one thread per node.

#define AOS_IDX(j, i, k) ((((size_t)(j)) * (size_t)Nx + (size_t)(i)) * 9 + (size_t)(k))

__device__ __forceinline__ bool wrapc(int &c, int n, int periodic) {
    if (periodic) {
        if (c < 0) c += n;
        else if (c >= n) c -= n;
        return true;
    }
    return c >= 0 && c < n;
}

// src/core/collision.c:18-40
__global__ void k_aos_collision(AosArgs a) {
    const int Nx = a.Nx;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.Nx || j >= a.Ny) return;
    const size_t n = (size_t)j * Nx + i;
    if (a.mask[n]) return;
    double f[9];
#pragma unroll
    for (int k = 0; k < 9; k++) f[k] = a.f[AOS_IDX(j, i, k)];
    collide_exact(f, a.w, a.rho[n], a.u[n], a.v[n], a.omega[n], a.Fx != 0.0 || a.Fy != 0.0, a.Fx, a.Fy);
#pragma unroll
    for (int k = 0; k < 9; k++) a.f[AOS_IDX(j, i, k)] = f[k];
}

// src/core/streaming.c:14-45
__global__ void k_aos_streaming(AosArgs a) {
    const int Nx = a.Nx, Ny = a.Ny;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= Nx || j >= Ny) return;
    if (a.mask[(size_t)j * Nx + i]) return;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        int is = i - cxk(k), js = j - cyk(k);
        if (!wrapc(is, Nx, a.px) || !wrapc(js, Ny, a.py)) continue;
        if (a.mask[(size_t)js * Nx + is]) continue;
        a.fnew[AOS_IDX(j, i, k)] = a.f[AOS_IDX(js, is, k)];
    }
}

// src/core/compute_macroscopic_fields.c:19-48
__global__ void k_aos_moments(AosArgs a) {
    const int Nx = a.Nx;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.Nx || j >= a.Ny) return;
    const size_t n = (size_t)j * Nx + i;
    double f[9];
#pragma unroll
    for (int k = 0; k < 9; k++) f[k] = a.fnew[AOS_IDX(j, i, k)];
    double rho, ux, uy;
    moments_exact(f, 0.5 * a.Fx, 0.5 * a.Fy, rho, ux, uy);
    if (!a.mask[n]) { a.rho[n] = rho; a.u[n] = ux; a.v[n] = uy; }
    else { a.rho[n] = NAN; a.u[n] = NAN; a.v[n] = NAN; }
}

// src/bc/bounce_back.c:15-49
__global__ void k_aos_bounce_back(AosArgs a) {
    const int Nx = a.Nx, Ny = a.Ny;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= Nx || j >= Ny) return;
    if (a.mask[(size_t)j * Nx + i]) return;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        int in = i + cxk(k), jn = j + cyk(k);
        if (!wrapc(in, Nx, a.px) || !wrapc(jn, Ny, a.py)) continue;
        if (!a.mask[(size_t)jn * Nx + in]) continue;
        a.fnew[AOS_IDX(j, i, oppk(k))] = a.f[AOS_IDX(j, i, k)];
    }
}

// src/bc/interpolated_bounce_back.c:19-103
__global__ void k_aos_ibb(AosArgs a) {
    const int Nx = a.Nx, Ny = a.Ny;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= Nx || j >= Ny) return;
    const size_t n = (size_t)j * Nx + i;
    if (a.mask[n]) return;
    const double eps = 1e-12;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        int in = i + cxk(k), jn = j + cyk(k);
        if (!wrapc(in, Nx, a.px) || !wrapc(jn, Ny, a.py)) continue;
        if (!a.mask[(size_t)jn * Nx + in]) continue;
        double denom = a.phi[n] - a.phi[(size_t)jn * Nx + in];
        if (fabs(denom) < eps) denom = (denom >= 0.0) ? eps : -eps;
        double q = a.phi[n] / denom;
        if (q < eps) q = eps;
        if (q > 1.0 - eps) q = 1.0 - eps;
        const size_t dst = AOS_IDX(j, i, oppk(k));
        const double fk = a.f[AOS_IDX(j, i, k)];
        int ib = i - cxk(k), jb = j - cyk(k);
        if (!wrapc(ib, Nx, a.px) || !wrapc(jb, Ny, a.py)) { a.fnew[dst] = fk; continue; }
        if (q <= 0.5) a.fnew[dst] = (1.0 - 2.0 * q) * fk + 2.0 * q * a.f[AOS_IDX(jb, ib, k)];
        else if (a.mask[(size_t)jb * Nx + ib]) a.fnew[dst] = fk;
        else a.fnew[dst] = (1.0 / (2.0 * q)) * fk + (2.0 * q - 1.0) / (2.0 * q) * a.f[AOS_IDX(jb, ib, oppk(k))];
    }
}

// src/core/compute_force_mem.c:19-67, reduced deterministically.
__global__ void k_aos_mem(AosArgs a) {
    const int Nx = a.Nx, Ny = a.Ny;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    double fx = 0.0, fy = 0.0;
    if (i < Nx && j < Ny && !a.mask[(size_t)j * Nx + i]) {
#pragma unroll
        for (int k = 1; k < 9; k++) {
            int in = i + cxk(k), jn = j + cyk(k);
            if (!wrapc(in, Nx, a.px) || !wrapc(jn, Ny, a.py)) continue;
            if (!a.mask[(size_t)jn * Nx + in]) continue;
            const double df = a.f[AOS_IDX(j, i, k)] + a.fnew[AOS_IDX(j, i, oppk(k))];
            fx += df * cxk(k);
            fy += df * cyk(k);
        }
    }
    reduce2_grid(fx, fy, a.partials, a.ticket, a.out2);
}

struct AosAccessor {
    const AosArgs &a;
    __device__ double get(int i, int j, int k) const { const int Nx = a.Nx; return a.fnew[AOS_IDX(j, i, k)]; }
    __device__ void set(int i, int j, int k, double v) const { const int Nx = a.Nx; a.fnew[AOS_IDX(j, i, k)] = v; }
    __device__ double rho(int i, int j) const { return a.rho[(size_t)j * a.Nx + i]; }
    __device__ double ux(int i, int j) const { return a.u[(size_t)j * a.Nx + i]; }
    __device__ double uy(int i, int j) const { return a.v[(size_t)j * a.Nx + i]; }
    __device__ double post(int i, int j, int k) const { const int Nx = a.Nx; return a.f[AOS_IDX(j, i, k)]; }
    __device__ bool solid(int i, int j) const { return a.mask[(size_t)j * a.Nx + i] != 0; }
};

// Any of lbc's edge BC functions on the AoS arrays (src/bc/*.c).
__global__ void k_aos_bc(AosArgs a, int kind, int index, int along, const double *val1,
                         const double *val2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= along) return;
    AosAccessor acc{a};
    bc_apply(acc, a.w, kind, a.Nx, a.Ny, index, t, val1 ? val1[t] : 0.0, val2 ? val2[t] : 0.0);
}

// ---- Mei initialisation (src/core/mei_initialization.c:50-127) on AoS arrays.

// :51-63 incompressible equilibrium
__global__ void k_mei_init(AosArgs a, double rho0) {
    const int Nx = a.Nx;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.Nx || j >= a.Ny) return;
    const size_t n = (size_t)j * Nx + i;
    const double ux = a.u[n], uy = a.v[n];
    const double usq = ux * ux + uy * uy;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const double cu = cxk(k) * ux + cyk(k) * uy;
        a.f[AOS_IDX(j, i, k)] = a.w[k] * a.rho[n] + a.w[k] * rho0 * (3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
    }
}

// :76-108 density moment, then incompressible collision on every node, and the
// max |rho - rho_prev| of :121-127 folded in.
__global__ void k_mei_iter(AosArgs a, double rho0, unsigned long long *maxbits) {
    const int Nx = a.Nx;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    double d = 0.0;
    if (i < a.Nx && j < a.Ny) {
        const size_t n = (size_t)j * Nx + i;
        double f[9];
#pragma unroll
        for (int k = 0; k < 9; k++) f[k] = a.f[AOS_IDX(j, i, k)];
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 9; k++) s += f[k];
        d = fabs(s - a.rho[n]);
        a.rho[n] = s;
        const double ux = a.u[n], uy = a.v[n];
        const double usq = ux * ux + uy * uy;
        const double om = a.omega[n];
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const double cu = cxk(k) * ux + cyk(k) * uy;
            const double feq = a.w[k] * s + a.w[k] * rho0 * (3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
            a.f[AOS_IDX(j, i, k)] = f[k] + -om * (f[k] - feq);
        }
    }
    // d >= 0, so the IEEE bit pattern orders like the value.
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d = fmax(d, __shfl_down_sync(0xffffffffu, d, o));
    if (((threadIdx.y * blockDim.x + threadIdx.x) & 31) == 0 && d > 0.0)
        atomicMax(maxbits, (unsigned long long)__double_as_longlong(d));
}

// ---------------------------------------------------------------- sponge

// src/core/sponge_layer.c:21-43 on the device, one thread per node: omega =
// 1 / tau with tau ramped exponentially in the radius between r_inner and
// r_outer, in lbc's operation order (--fmad=false, correctly rounded sqrt and
// division). exp is CUDA's (within 1 ulp of the exact value, not libm's bits),
// so ramp nodes can differ from lbc in the last bits; the rest are identical.
__global__ void k_sponge(int Nx, int Ny, double dx, double xc, double yc, double r_inner, double r_outer,
                         double tau_base, double incr_tau, double exp_coeff, double *omega) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= Nx || j >= Ny) return;
    const double y = j * dx - yc;
    const double x = i * dx - xc;
    const double r = sqrt(x * x + y * y);
    double tau;
    if (r <= r_inner) tau = tau_base;
    else if (r <= r_outer)
        tau = tau_base + (incr_tau - 1) * tau_base * (exp(exp_coeff * (r - r_inner)) - 1) /
                             (exp(exp_coeff * (r_outer - r_inner)) - 1);
    else tau = tau_base * incr_tau;
    omega[(size_t)j * Nx + i] = 1.0 / tau;
}

// ---------------------------------------------------------------- records

// One block per task. Every thread reads the step count before the barrier at
// the end, after which thread 0 advances it, so all of a task's values of a
// step land in the same ring slot.
template <typename T>
__global__ void __launch_bounds__(256) k_record(const RecordTask *__restrict__ tasks, const void *dst,
                                                const char *spbase, int spstride, int sel,
                                                int collided) {
    __shared__ double sp_[256], sv_[256];
    __shared__ int sn_[256];
    const RecordTask &r = tasks[blockIdx.x];
    const unsigned long long k = *r.count;
    const size_t slot = (size_t)(k % (unsigned long long)r.cap);
    if (r.kind == REC_PROBES) {
        const void *buf = dst;
        if (spbase)
            buf = ((const StepParams *)(spbase + (size_t)(2 * r.cs + sel) * spstride))->dst;
        const T *f = (const T *)buf;
        for (int q = threadIdx.x; q < r.n; q += blockDim.x) {
            const long long o = r.nodes[q];
            double rho = 0.0, jx = 0.0, jy = 0.0;
#pragma unroll
            for (int kk = 0; kk < 9; kk++) {
                const double fk = Store<T>::to_f64(f[kk * r.plane + o], r.w[kk]);
                rho += fk;
                jx += cxk(kk) * fk;
                jy += cyk(kk) * fk;
            }
            double *out = r.ring + (slot * r.n + q) * 3;
            out[0] = rho;
            out[1] = (collided ? jx - r.hFx : jx + r.hFx) / rho;
            out[2] = (collided ? jy - r.hFy : jy + r.hFy) / rho;
        }
    } else {
        // Mean p' and v over the active nodes, summed in a fixed order (a
        // strided partial per thread, then a tree over the block).
        double a = 0.0, b = 0.0;
        int na = 0;
        for (int t = threadIdx.x; t < r.n; t += blockDim.x) {
            if (r.imp[(size_t)IMP_ACTIVE * r.n + t] == 0.0) continue;
            a += r.imp[(size_t)IMP_P * r.n + t];
            b += r.imp[(size_t)IMP_V * r.n + t];
            na++;
        }
        sp_[threadIdx.x] = a;
        sv_[threadIdx.x] = b;
        sn_[threadIdx.x] = na;
        __syncthreads();
        for (int h = blockDim.x / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) {
                sp_[threadIdx.x] += sp_[threadIdx.x + h];
                sv_[threadIdx.x] += sv_[threadIdx.x + h];
                sn_[threadIdx.x] += sn_[threadIdx.x + h];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            const double cnt = sn_[0] > 0 ? (double)sn_[0] : 1.0;
            r.ring[slot * 2] = sp_[0] / cnt;
            r.ring[slot * 2 + 1] = sv_[0] / cnt;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *r.count = k + 1ull;
}

// ---------------------------------------------------------------- FP64 rate

// The device's FP64 FMA issue rate, the ceiling of the FP64 step kernels: each
// thread runs eight independent dependency chains of DFMA (enough in flight
// per warp to cover the pipe's latency). x <- a x + b with a < 1 stays bounded.
__global__ void __launch_bounds__(256) k_fp64_rate(double *sink, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = (threadIdx.x + q) * 1e-3;
#pragma unroll 1
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int q = 0; q < 8; q++) x[q] = fma(x[q], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) s += x[q];
    if (s == -1.0) sink[0] = s;  // never true; keeps the chains live
}

// ---------------------------------------------------------------- launchers

namespace launch {

cudaError_t record(const RecordTask *tasks, int n, int store, const void *dst, const char *spbase, int spstride,
                   int sel, bool collided, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int c = collided ? 1 : 0;
    if (store == STORE_F64) k_record<double><<<n, 256, 0, s>>>(tasks, dst, spbase, spstride, sel, c);
    else if (store == STORE_F32) k_record<float><<<n, 256, 0, s>>>(tasks, dst, spbase, spstride, sel, c);
    else k_record<__half><<<n, 256, 0, s>>>(tasks, dst, spbase, spstride, sel, c);
    return cudaGetLastError();
}

cudaError_t sponge(int Nx, int Ny, double dx, double xc, double yc, double r_inner, double r_outer,
                   double tau_base, double incr_tau, double exp_coeff, double *omega, cudaStream_t s) {
    const dim3 b(64, 4);
    const dim3 g((Nx + b.x - 1) / b.x, (Ny + b.y - 1) / b.y);
    k_sponge<<<g, b, 0, s>>>(Nx, Ny, dx, xc, yc, r_inner, r_outer, tau_base, incr_tau, exp_coeff, omega);
    return cudaGetLastError();
}

cudaError_t fp64_rate(int blocks, int iters, double *sink, cudaStream_t s) {
    k_fp64_rate<<<blocks, 256, 0, s>>>(sink, iters, 0.9999999, 1e-9);
    return cudaGetLastError();
}

static dim3 grid2(int Nx, int Ny, dim3 b) { return dim3((Nx + b.x - 1) / b.x, (Ny + b.y - 1) / b.y); }

template <bool FMA>
static void step_exact_t(const StepParams &p, bool flags, bool collide, dim3 g, dim3 block, cudaStream_t s) {
    if (flags) {
        if (collide) k_step_exact<true, true, FMA><<<g, block, 0, s>>>(p);
        else k_step_exact<true, false, FMA><<<g, block, 0, s>>>(p);
    } else {
        if (collide) k_step_exact<false, true, FMA><<<g, block, 0, s>>>(p);
        else k_step_exact<false, false, FMA><<<g, block, 0, s>>>(p);
    }
}

cudaError_t step_exact(const StepParams &p, bool flags, bool collide, dim3 block, cudaStream_t s, bool fma) {
    const dim3 g = grid2(p.Nx, p.Ny, block);
    if (fma) step_exact_t<true>(p, flags, collide, g, block, s);
    else step_exact_t<false>(p, flags, collide, g, block, s);
    return cudaGetLastError();
}

// Edge kernels are FP64 and short: 32-thread blocks spread a line over many SMs.
cudaError_t stage_group(const StageGroup &g, int store, bool collide, bool after_bulk, cudaStream_t s) {
    if (g.n < 1 || g.n > kStageGroupMax || (g.nfs && !g.fs)) return cudaErrorInvalidValue;
    if (store != STORE_F64) return stage_group_shifted(g, store, collide, after_bulk, s);
    const dim3 grid((g.max_along + 31) / 32, g.n + (g.nfs ? 1 : 0));
    if (collide) return launch_follower(after_bulk, k_stage_group<double, true>, grid, dim3(32), s, g);
    return launch_follower(after_bulk, k_stage_group<double, false>, grid, dim3(32), s, g);
}

cudaError_t step_batch_exact(const StepParams *sp, const int4 *tiles, int ntiles,
                             int sel, int tws, int grid, cudaStream_t s, bool fma) {
    if (ntiles == 0) return cudaSuccess;
    if (tws < 5 || tws > 8) return cudaErrorInvalidValue;
    if (fma) k_step_batch_exact<true><<<grid, 256, 0, s>>>(sp, tiles, ntiles, sel, tws);
    else k_step_batch_exact<false><<<grid, 256, 0, s>>>(sp, tiles, ntiles, sel, tws);
    return cudaGetLastError();
}

// One block per tile (the batch launches min(tiles, this)): the FP64 step is
// bound by the FP64 issue rate, not by memory parallelism, so it gains nothing
// from a persistent grid, and short-lived blocks let the block scheduler give
// SMs to a concurrent higher-priority batch (the server's FP32 lane) as they
// free up. Measured on 64 liner ducts: 4.03 GLUPS persistent, 4.10 per tile.
int step_batch_exact_grid() { return 1 << 30; }

cudaError_t stage_batch(const StageParams *list, int n, const int2 *blocks, int nblocks,
                        int store, int sel, const ForceSlot *fs, bool after_bulk, bool warm, cudaStream_t s) {
    if (nblocks == 0) return cudaSuccess;
    if (store != STORE_F64) return stage_batch_shifted(list, n, blocks, nblocks, store, sel, fs, after_bulk, s);
    return launch_follower(after_bulk, k_stage_batch<double>, dim3(nblocks), dim3(kStageBatchPointsF64), s, list,
                           blocks, sel, n, fs, warm ? 1 : 0);
}

cudaError_t force_reduce(const ForceSlot *slots, int n, bool after_bulk, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    return launch_follower(after_bulk, k_force_reduce, dim3(n), dim3(32), s, slots, n);
}

cudaError_t collide_exact(const CollideParams &p, cudaStream_t s) {
    const dim3 b(64, 4);
    k_collide_exact<<<grid2(p.Nx, p.Ny, b), b, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t collide_aos_exact(const CollideAosParams &p, cudaStream_t s) {
    const long long N = (long long)p.Nx * p.Ny;
    k_collide_aos_exact<<<(unsigned)((N + 127) / 128), 128, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t aos_to_soa(const double *aos, void *soa, int store, int Nx, int Ny, int pitch,
                       long long plane, const double w[9], cudaStream_t s) {
    Wt wt;
    for (int k = 0; k < 9; k++) wt.w[k] = w[k];
    const long long N = (long long)Nx * Ny;
    const unsigned g = (unsigned)((N + 127) / 128);
    if (store == STORE_F64) k_aos_to_soa<double><<<g, 256, 0, s>>>(aos, (double *)soa, Nx, Ny, pitch, plane, wt);
    else if (store == STORE_F32) k_aos_to_soa<float><<<g, 256, 0, s>>>(aos, (float *)soa, Nx, Ny, pitch, plane, wt);
    else k_aos_to_soa<__half><<<g, 256, 0, s>>>(aos, (__half *)soa, Nx, Ny, pitch, plane, wt);
    return cudaGetLastError();
}

cudaError_t soa_to_aos(const void *soa, double *aos, int store, int Nx, int Ny, int pitch,
                       long long plane, const double w[9], cudaStream_t s) {
    Wt wt;
    for (int k = 0; k < 9; k++) wt.w[k] = w[k];
    const long long N = (long long)Nx * Ny;
    const unsigned g = (unsigned)((N + 127) / 128);
    if (store == STORE_F64) k_soa_to_aos<double><<<g, 256, 0, s>>>((const double *)soa, aos, Nx, Ny, pitch, plane, wt);
    else if (store == STORE_F32) k_soa_to_aos<float><<<g, 256, 0, s>>>((const float *)soa, aos, Nx, Ny, pitch, plane, wt);
    else k_soa_to_aos<__half><<<g, 256, 0, s>>>((const __half *)soa, aos, Nx, Ny, pitch, plane, wt);
    return cudaGetLastError();
}

cudaError_t seed_band(const int2 *nodes, const int *slots, int n, int Nx, const double *rho,
                      const double *ux, const double *uy, double *bandm, int nslots,
                      cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_seed_band<<<(n + 127) / 128, 128, 0, s>>>(nodes, slots, n, Nx, rho, ux, uy, bandm, nslots);
    return cudaGetLastError();
}

cudaError_t aos_op(int op, const AosArgs &a, cudaStream_t s) {
    const dim3 b(64, 4);
    const dim3 g = grid2(a.Nx, a.Ny, b);
    switch (op) {
    case AOS_COLLISION: k_aos_collision<<<g, b, 0, s>>>(a); break;
    case AOS_STREAMING: k_aos_streaming<<<g, b, 0, s>>>(a); break;
    case AOS_MOMENTS: k_aos_moments<<<g, b, 0, s>>>(a); break;
    case AOS_BOUNCE_BACK: k_aos_bounce_back<<<g, b, 0, s>>>(a); break;
    case AOS_IBB: k_aos_ibb<<<g, b, 0, s>>>(a); break;
    case AOS_MEM: k_aos_mem<<<g, b, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

unsigned aos_mem_blocks(int Nx, int Ny) {
    const dim3 g = grid2(Nx, Ny, dim3(64, 4));
    return g.x * g.y;
}

cudaError_t aos_bc(const AosArgs &a, int kind, int index, int along, const double *val1,
                   const double *val2, cudaStream_t s) {
    k_aos_bc<<<(along + 127) / 128, 128, 0, s>>>(a, kind, index, along, val1, val2);
    return cudaGetLastError();
}

cudaError_t mei_init(const AosArgs &a, double rho0, cudaStream_t s) {
    const dim3 b(64, 4);
    k_mei_init<<<grid2(a.Nx, a.Ny, b), b, 0, s>>>(a, rho0);
    return cudaGetLastError();
}

cudaError_t mei_iter(const AosArgs &a, double rho0, unsigned long long *maxbits, cudaStream_t s) {
    const dim3 b(64, 4);
    k_mei_iter<<<grid2(a.Nx, a.Ny, b), b, 0, s>>>(a, rho0, maxbits);
    return cudaGetLastError();
}

}  // namespace launch
}  // namespace lbm
