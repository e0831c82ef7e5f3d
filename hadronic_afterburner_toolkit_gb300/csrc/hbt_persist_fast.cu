// Persistent kernels of the batched path, fast binning (no pair cap can
// bind, no q_inv histograms): the default kernel of every fast call.
#include "hbt_persist.cuh"

namespace hbt {

using namespace persist;

cudaError_t persistent_same_fast(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                                 int grid, cudaStream_t st) {
    return launch_same_mode<MODE_FAST, false>(d, b, base, end, grid, st);
}

cudaError_t persistent_mixed_fast(const Device &d, const BatchDev &b, int grid, cudaStream_t st) {
    return launch_mixed_mode<MODE_FAST, false>(d, b, grid, st);
}

int persistent_blocks_per_sm() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, k_persistent_same<true, true, 0, MODE_FAST, false, false>, FT, 0) != cudaSuccess)
        return 4;
    return nb > 0 ? nb : 1;
}

}  // namespace hbt
