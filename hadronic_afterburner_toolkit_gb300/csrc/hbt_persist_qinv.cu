// Persistent kernels of the batched path with the q_inv histograms
// (invariant_radius_flag = 1, src/HBT_correlation.cpp:331-356, :595-607),
// fast binning.
#include "hbt_persist.cuh"

namespace hbt {

using namespace persist;

cudaError_t persistent_same_qinv(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                                 int grid, cudaStream_t st) {
    return launch_same_mode<MODE_FAST, true>(d, b, base, end, grid, st);
}

cudaError_t persistent_mixed_qinv(const Device &d, const BatchDev &b, int grid, cudaStream_t st) {
    return launch_mixed_mode<MODE_FAST, true>(d, b, grid, st);
}

}  // namespace hbt
