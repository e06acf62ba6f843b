// Tiled mixed-precision path (placeholder until the tiled kernels land).
#include <cuda_runtime.h>

#include "gpw_internal.h"

namespace gpw {
int mixed_build(TaskSet &, std::string &) { return 0; }
void mixed_free(TaskSet &) {}
cudaError_t launch_collocate_mixed(const TaskSet &, const GridPtrs &, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t launch_integrate_mixed(const TaskSet &, const GridPtrs &, cudaStream_t) { return cudaErrorNotSupported; }
}  // namespace gpw
