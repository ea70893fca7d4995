// pdl.cuh -- programmatic dependent launch between consecutive kernels of a
// step in the same stream (clean pairs, special nodes, edge stages, force
// reduction).
//
// A kernel signals at its start that the next kernel may be launched
// (griddepcontrol.launch_dependents); a follower launched with programmatic
// stream serialization is then scheduled once every block of the kernel
// before it has started, so its launch latency hides behind that kernel's
// last wave, or (a case alone: the special nodes, then the clean pairs) so
// that the two run side by side. A follower calls pdl_wait()
// (griddepcontrol.wait: returns once the kernel before it has completed and
// its writes are visible) before it reads or writes anything that kernel
// touches. A kernel launched without the attribute passes through both
// instructions unaffected.
#pragma once
#include <cuda_runtime.h>

#include <utility>

namespace lbm {

__device__ __forceinline__ void pdl_launch_dependents() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch k<<<g, b, 0, s>>>(args...), with programmatic stream serialization
// when after_bulk is set (the previous kernel in s is a bulk step kernel).
template <typename... K, typename... A>
inline cudaError_t launch_follower(bool after_bulk, void (*k)(K...), dim3 g, dim3 b, cudaStream_t s,
                                   A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = after_bulk ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}

}  // namespace lbm
