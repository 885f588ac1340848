// Certified split-BF16 coarse pass on tcgen05 (placeholder until the kernel lands).
#include "knn_tc.h"

namespace costal {
namespace tc {

bool supported(int, int) { return false; }
size_t workspace_bytes(int, int) { return 256; }
cudaError_t prepare(void*, const float*, int, int, int, int, cudaStream_t, Plan&) { return cudaErrorNotSupported; }
cudaError_t launch_coarse(const Plan&, int, uint32_t*, float*, float*, unsigned long long*, int, cudaStream_t) {
    return cudaErrorNotSupported;
}

}  // namespace tc
}  // namespace costal
