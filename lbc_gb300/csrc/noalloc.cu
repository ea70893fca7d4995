// noalloc.cu -- momentum-exchange force on caller-owned device arrays, with no
// memory allocation of any kind.
//
// lbm_gpu_compute_force_mem_noalloc is for callers that cannot let a library
// call cudaMalloc / cudaFree: a process whose device memory is already held by
// its own pool (a deep-learning framework's caching allocator, or a server
// that reserves memory up front), or a loop that must not stall the device
// (cudaFree synchronizes it). Its only scratch, the per-block partial sums of
// the deterministic reduction and the arrival counter, lives in the static
// device array below (1 MiB + 256 B). The array belongs to this file's module,
// which CUDA loads into a context the first time the context uses it (with
// lazy module loading, the default since CUDA 12.2, that is this entry
// point's first call there; with eager loading, when the library's modules
// load). From then on the device holds it until the context is destroyed.
//
// The first call in a context (with its device current) looks the array's
// device address up with cudaGetSymbolAddress; that first call should come
// before any stream capture, and in a process whose pool reserves nearly all
// device memory, before the pool does. The address is kept per device together
// with the identity of the context it was looked up in, and looked up again
// when the current context differs (after cudaDeviceReset, for instance, the
// module is loaded again and the array may sit elsewhere). All calls share the
// array and it keeps the last call's contents: each call clears the counter it
// needs, and calls whose kernels overlap on the GPU race on the array, so order
// them (one stream, or events).
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/lbm_gpu.h"
#include "engine.h"
#include "lbm_device.cuh"
#include "reduce.cuh"

namespace {

constexpr int kNoallocMaxBlocks = 65536;  // 64 x 4 node blocks: grids up to 16.7 M nodes
constexpr int kNoallocDoubles = 2 * kNoallocMaxBlocks + 32;

// Partials at [0, 2 * kNoallocMaxBlocks), the arrival counter in the last 256 bytes.
static __device__ __align__(256) double g_noalloc_scratch[kNoallocDoubles];

struct DeviceScratch {
    unsigned long long ctx_id = 0;   // context the address was looked up in (0: none yet)
    double *partials = nullptr;
    unsigned int *ticket = nullptr;
};
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
DeviceScratch g_noalloc_dev[kMaxDevices];

// The driver's cuCtxGetCurrent / cuCtxGetId through the runtime's entry-point
// query (no link against libcuda). Context ids are unique for the life of the
// process, so a context destroyed and made again gets a new one even when its
// handle is reused.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
std::once_flag g_ctx_once;

void resolve_ctx_entry_points() {
    void *a = nullptr, *b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qb == cudaDriverEntryPointSuccess) {
        g_ctx_current = (CtxGetCurrentFn)a;
        g_ctx_id = (CtxGetIdFn)b;
    }
    cudaGetLastError();  // a failed query leaves no sticky error behind
}

// Id of the context current on this thread, 0 when there is none or the
// driver cannot say (then the address is looked up on every call).
unsigned long long current_ctx_id() {
    std::call_once(g_ctx_once, resolve_ctx_entry_points);
    if (!g_ctx_current || !g_ctx_id) return 0;
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&c) != CUDA_SUCCESS || !c) return 0;
    if (g_ctx_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

bool scratch_for_current_device(DeviceScratch &out) {
    int dev = 0;
    if (!lbm::check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return false;
    if (dev < 0 || dev >= kMaxDevices) {
        lbm::set_error("device index out of range for the no-alloc scratch table");
        return false;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    DeviceScratch &d = g_noalloc_dev[dev];
    unsigned long long id = current_ctx_id();
    if (id != 0 && id == d.ctx_id && d.partials) {
        out = d;
        return true;
    }
    // First call in this context (or no context made current yet: the lookup
    // below makes the device's primary context current, as every runtime call
    // that needs one does).
    void *p = nullptr;
    if (!lbm::check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress")) return false;
    if (id == 0) id = current_ctx_id();
    d.ctx_id = id;
    d.partials = (double *)p;
    d.ticket = (unsigned int *)((double *)p + 2 * kNoallocMaxBlocks);
    out = d;
    return true;
}

// src/core/compute_force_mem.c:19-67 on lbc's AoS layout, one thread per node,
// reduced in a fixed order into out[0..1].
__global__ void __launch_bounds__(256) k_force_mem_noalloc(int Nx, int Ny, int px, int py,
                                                           const double *__restrict__ f,
                                                           const double *__restrict__ fnew,
                                                           const int *__restrict__ mask,
                                                           double *partials, unsigned int *ticket,
                                                           double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double fx = 0.0, fy = 0.0;
    if (i < Nx && j < Ny && !mask[(size_t)j * Nx + i]) {
#pragma unroll
        for (int k = 1; k < 9; k++) {
            int in = i + lbm::cxk(k), jn = j + lbm::cyk(k);
            if (px) { if (in < 0) in += Nx; else if (in >= Nx) in -= Nx; }
            else if (in < 0 || in >= Nx) continue;
            if (py) { if (jn < 0) jn += Ny; else if (jn >= Ny) jn -= Ny; }
            else if (jn < 0 || jn >= Ny) continue;
            if (!mask[(size_t)jn * Nx + in]) continue;
            const size_t b = ((size_t)j * Nx + i) * 9;
            const double df = f[b + k] + fnew[b + lbm::oppk(k)];
            fx += df * lbm::cxk(k);
            fy += df * lbm::cyk(k);
        }
    }
    lbm::reduce2_grid(fx, fy, partials, ticket, out);
}

}  // namespace

extern "C" int lbm_gpu_compute_force_mem_noalloc(int Nx, int Ny, int Q, const double *f,
                                                 const double *f_new, const int *solid_mask,
                                                 int isperiodic_x, int isperiodic_y, const int *cx,
                                                 const int *cy, const int *opp, double *out,
                                                 void *stream) {
    static const int kCX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    static const int kCY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    static const int kOPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
    if (Q != 9 || Nx < 1 || Ny < 1 || !f || !f_new || !solid_mask || !out) {
        lbm::set_error("force_mem_noalloc: need Q = 9, a non-empty grid and non-null arrays");
        return LBM_GPU_ERR_ARG;
    }
    for (int k = 0; k < 9; k++) {
        if ((cx && cx[k] != kCX[k]) || (cy && cy[k] != kCY[k]) || (opp && opp[k] != kOPP[k])) {
            lbm::set_error("force_mem_noalloc: cx/cy/opp must be lbc's D2Q9 ordering");
            return LBM_GPU_ERR_ARG;
        }
    }
    const dim3 block(64, 4);
    const dim3 grid((Nx + 63) / 64, (Ny + 3) / 4);
    if ((long long)grid.x * grid.y > kNoallocMaxBlocks || grid.y > 65535u) {
        lbm::set_error("force_mem_noalloc: grid too large for the fixed scratch (at most 65536 blocks "
                       "of 64 x 4 nodes, e.g. 4096 x 4096, and at most 262140 rows)");
        return LBM_GPU_ERR_ARG;
    }
    DeviceScratch sc;
    if (!scratch_for_current_device(sc)) return LBM_GPU_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    if (!lbm::check_cuda(cudaMemsetAsync(sc.ticket, 0, sizeof(unsigned int), s), "cudaMemsetAsync"))
        return LBM_GPU_ERR_CUDA;
    k_force_mem_noalloc<<<grid, block, 0, s>>>(Nx, Ny, isperiodic_x, isperiodic_y, f, f_new,
                                                solid_mask, sc.partials, sc.ticket, out);
    return lbm::check_cuda(cudaGetLastError(), "k_force_mem_noalloc") ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}
