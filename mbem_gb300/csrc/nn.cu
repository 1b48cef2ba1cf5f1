// Learned preconditioner (mesh-local network): forward, backward and
// optimiser kernels. The apply entry point is the FGMRES hook for
// precond == 2.
#include "common.cuh"

namespace mbem {

int nn_precond_apply(const void* state, const double* r, double* z, cudaStream_t st) {
    (void)state; (void)r; (void)z; (void)st;
    return set_error(MBEM_ERR_UNSUPPORTED, "the learned preconditioner is not built yet");
}

}  // namespace mbem
