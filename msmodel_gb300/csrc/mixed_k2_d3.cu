// One variant of the mixed-precision engine: job kind 2 (amplitudes), media all of d = 3;
// its host entry sets the kernel's shared-memory limit (attr_only) or launches it.
#define MSG_MIXED_KERNEL_BODY
#include "mixed_engine.cuh"

namespace msg {
int mixed_variant_2_d3(const EngineParams& P, const MixScratch& X, int grid, size_t smem, cudaStream_t st,
                        bool attr_only) {
    if (attr_only)
        return cudaFuncSetAttribute(k_engine_mixed<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem) == cudaSuccess
                   ? 0
                   : MSGPU_E_CUDA;
    k_engine_mixed<2, true><<<grid, NT, smem, st>>>(P, X);
    return cudaGetLastError() == cudaSuccess ? 0 : MSGPU_E_CUDA;
}
}  // namespace msg
