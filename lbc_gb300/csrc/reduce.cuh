// reduce.cuh -- deterministic grid-wide reduction shared by the step kernels.
#pragma once
#include <cuda_runtime.h>

namespace lbm {

// Warp sum of two doubles into lane 0. Warps where no lane has a wall link
// (most of the grid) skip the FP64 shuffles, which are slow on GB300.
__device__ __forceinline__ void warp_reduce2(double &a, double &b, bool link) {
    if (!__any_sync(0xffffffffu, link)) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
}

// One case's force from its segment partials, by one full warp (every lane
// calls it): the sum of partials[2 t], partials[2 t + 1] over t in [t0, t1)
// into out[0..1] and the next history slot. The order is fixed and does not
// depend on the launch: lane l keeps the running sum of t = t0 + l + 32 k in
// increasing k, and a shuffle tree folds the 32 sums. FP64 adds are the cost
// on GB300 (about 64 cycles per warp instruction on one SM sub-partition), so
// the order is the one with the fewest: n / 32 + 5 per component.
template <class Slot>
__device__ __forceinline__ void force_reduce_warp(const Slot &fs, int lane) {
    const int t0 = fs.t0, t1 = fs.t1;
    const double2 *part = (const double2 *)fs.partials;
    double a = 0.0, b = 0.0;
    for (int t = t0 + lane; t < t1; t += 32) {
        const double2 v = part[t];
        a += v.x;
        b += v.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (lane != 0) return;
    fs.out[0] = a;
    fs.out[1] = b;
    if (fs.hist) {
        const unsigned long long k = *fs.hist_count;
        const int slot = (int)(k % (unsigned long long)fs.hist_cap);
        fs.hist[2 * slot] = a;
        fs.hist[2 * slot + 1] = b;
        *fs.hist_count = k + 1ull;
    }
}

// Deterministic block + grid reduction of two doubles. Every thread of every
// block must call it. Blocks write partials; the last block to arrive sums them
// in block order and writes out[0..1] (and, when a history ring is given, the
// next ring slot), then rearms the ticket.
__device__ __forceinline__ void reduce2_grid(double a, double b, double *partials, unsigned int *ticket,
                                             double *out, double *hist = nullptr,
                                             unsigned long long *hist_count = nullptr,
                                             int hist_cap = 0) {
    __shared__ double sa[32], sb[32];
    __shared__ bool last;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nthr = blockDim.x * blockDim.y;
    const int lane = tid & 31, warp = tid >> 5;
    warp_reduce2(a, b, a != 0.0 || b != 0.0);
    if (lane == 0) { sa[warp] = a; sb[warp] = b; }
    __syncthreads();
    const int nblk = gridDim.x * gridDim.y;
    const int bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (tid == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < (nthr + 31) / 32; w++) { ta += sa[w]; tb += sb[w]; }
        partials[2 * bid] = ta;
        partials[2 * bid + 1] = tb;
        __threadfence();
        const unsigned int t = atomicAdd(ticket, 1u);
        last = (t == (unsigned int)nblk - 1u);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double ta = 0.0, tb = 0.0;
    for (int q = tid; q < nblk; q += nthr) {
        ta += __ldcg(partials + 2 * q);
        tb += __ldcg(partials + 2 * q + 1);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ta += __shfl_down_sync(0xffffffffu, ta, o);
        tb += __shfl_down_sync(0xffffffffu, tb, o);
    }
    __syncthreads();
    if (lane == 0) { sa[warp] = ta; sb[warp] = tb; }
    __syncthreads();
    if (tid == 0) {
        double ra = 0.0, rb = 0.0;
        for (int w = 0; w < (nthr + 31) / 32; w++) { ra += sa[w]; rb += sb[w]; }
        out[0] = ra;
        out[1] = rb;
        if (hist) {
            const unsigned long long c = *hist_count;
            const int slot = (int)(c % (unsigned long long)hist_cap);
            hist[2 * slot] = ra;
            hist[2 * slot + 1] = rb;
            *hist_count = c + 1ull;
        }
        *ticket = 0u;
    }
}

// Sum of two doubles over the warp that holds the 32-node row segment
// (j, i0 .. i0 + 31), i0 = i & ~31, stored by lane 0 at partials[2 * slot],
// slot = seg_slot[j][i0 / 32]. Every lane of the warp must call it; lanes past
// the grid pass link = false. `link`: this lane's node has wall links (its
// terms are nonzero). Warps without links (most of the grid) return at once.
__device__ __forceinline__ void segment_reduce2_store(double a, double b, bool link, int i, int j, int Nx,
                                                      const int *__restrict__ seg_slot, double *partials) {
    if (!__any_sync(0xffffffffu, link)) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((i & 31) == 0) {
        const int slot = seg_slot[(size_t)j * ((Nx + 31) >> 5) + (i >> 5)];
        if (slot >= 0) {
            partials[2 * (size_t)slot] = a;
            partials[2 * (size_t)slot + 1] = b;
        }
    }
}

// Force partial of one 32-entry chunk of a special-node list (one warp;
// every lane must call it): the lanes' terms in a fixed shuffle tree, stored
// at the chunk's slot when the chunk contains wall links.
__device__ __forceinline__ void chunk_reduce2_store(double a, double b, bool link, int chunk,
                                                    const int *__restrict__ chunk_slot, double *partials) {
    if (!__any_sync(0xffffffffu, link)) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        const int slot = chunk_slot[chunk];
        if (slot >= 0) {
            partials[2 * (size_t)slot] = a;
            partials[2 * (size_t)slot + 1] = b;
        }
    }
}

}  // namespace lbm
