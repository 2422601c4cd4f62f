// mixed.cu -- mixed-precision engine (placeholder until the tensor-core path lands).
#include "engine_internal.h"

namespace msg {
int mixed_run(const EngineParams&, int, int, cudaStream_t) { return MSGPU_E_ARG; }
int mixed_launches() { return 0; }
}  // namespace msg
