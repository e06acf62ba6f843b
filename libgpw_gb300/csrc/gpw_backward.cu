// Backward kernels (placeholder until the force / exponent kernels land).
#include <cuda_runtime.h>

#include "gpw_internal.h"

namespace gpw {
cudaError_t launch_backward(const TaskSet &, const double *, const GridPtrs &, double *, double *, double *,
                            double *, double *, cudaStream_t) {
    return cudaErrorNotSupported;
}
}  // namespace gpw
