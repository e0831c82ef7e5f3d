// Persistent kernels of the batched path for ordered cap admission
// (needed_number_of_pairs, src/HBT_correlation.cpp:400-406, :651-655): the
// COUNT pass (survivors per slot and row of the caller's list) and the
// ORDER pass (the rows before each slot's cut row).
#include "hbt_persist.cuh"

namespace hbt {

using namespace persist;

cudaError_t persistent_same_ordered(const Device &d, const BatchDev &b, unsigned base,
                                    unsigned end, int grid, cudaStream_t st, int mode) {
    if (mode == MODE_COUNT) return launch_same_mode<MODE_COUNT, false>(d, b, base, end, grid, st);
    if (mode == MODE_ORDER) return launch_same_mode<MODE_ORDER, false>(d, b, base, end, grid, st);
    return cudaErrorInvalidValue;
}

cudaError_t persistent_mixed_ordered(const Device &d, const BatchDev &b, int grid,
                                     cudaStream_t st, int mode) {
    if (mode == MODE_COUNT) return launch_mixed_mode<MODE_COUNT, false>(d, b, grid, st);
    if (mode == MODE_ORDER) return launch_mixed_mode<MODE_ORDER, false>(d, b, grid, st);
    return cudaErrorInvalidValue;
}

}  // namespace hbt
