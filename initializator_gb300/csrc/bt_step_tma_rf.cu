// The FP32 fast path's pulse-step kernels (every pulse of the step
// fixed-angle, applied as one rotation before the step's sums), both tile
// widths, in their own translation unit so that they compile in parallel
// with the others.
#include "bt_step_tma.cuh"

namespace bt {

cudaError_t launch_step_tma_pulse(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec,
                                  dim3 grid, int tw, bool first, cudaStream_t s) {
    if (tw == 64) return launch_step_tma_rfw<64>(p, m, scheme, vel, prec, grid, first, s);
    return launch_step_tma_rfw<128>(p, m, scheme, vel, prec, grid, first, s);
}

}  // namespace bt
