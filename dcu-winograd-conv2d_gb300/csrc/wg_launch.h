// Kernel launches with programmatic dependent launch (PDL): each kernel of a
// convolution may be scheduled while the kernel before it on the stream is
// still finishing, runs its prologue (barrier set-up, descriptor prefetch),
// and waits in griddepcontrol.wait for the earlier grid's completion and
// memory flush before it touches any tensor.  Every kernel launched this way
// starts with that wait, so results and ordering are those of plain stream
// launches; only the launch gap and prologue overlap.  WG_CONV2D_PDL=0 turns
// it off (plain launches).
#pragma once
#include <cstdlib>
#include <utility>

#include <cuda_runtime.h>

namespace wg {

inline bool pdl_enabled() {
    static const bool on = [] {
        const char* v = std::getenv("WG_CONV2D_PDL");
        return !(v && v[0] == '0');
    }();
    return on;
}

template <class... KArgs, class... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace wg
