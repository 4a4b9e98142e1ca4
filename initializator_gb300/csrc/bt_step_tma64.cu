// The FP32 fast path's kernels for 64-wide tiles (narrow grids), in their own
// translation unit so that they compile in parallel with the 128-wide ones.
#include "bt_step_tma.cuh"

namespace bt {

cudaError_t launch_step_tma64(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec, dim3 grid,
                              bool first, cudaStream_t s) {
    return launch_step_tma_w<64>(p, m, scheme, vel, prec, grid, first, s);
}

}  // namespace bt
