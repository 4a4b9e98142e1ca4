// double instantiation of the fused step kernel and its helpers.
// Compiled with -fmad=false: no multiply-add contraction, so the FP64 field
// keeps the reference's rounding step for step.
#include "bt_step.cuh"
#include "bt_step_mac.cuh"

namespace bt {

template <>
cudaError_t launch_step<double>(const StepParams<double>& p, int scheme, int vel, int prec, dim3 grid, cudaStream_t s) {
    return launch_step_impl<double>(p, scheme, vel, prec, grid, s);
}

template <>
cudaError_t launch_sums<double>(const StepParams<double>& p, double* kvec_and_grid, cudaStream_t s) {
    // kvec_and_grid: {kx, ky, kz, nblocks}
    const int nblocks = (int)kvec_and_grid[3];
    sums_kernel<double><<<nblocks, NTHREADS, 0, s>>>(p, kvec_and_grid[0], kvec_and_grid[1], kvec_and_grid[2], p.partials);
    return cudaGetLastError();
}

template <>
cudaError_t launch_mac<double>(const StepParams<double>& p, double* const pred[3], int vel, int prec, dim3 grid, cudaStream_t s) {
    return launch_mac_impl<double>(p, pred, vel, prec, grid, s);
}

template <>
cudaError_t launch_phase_sums<double>(const StepParams<double>& p, const double* w1, const double* w2, double* part6, int nblocks,
                                double* mt6, long long cap, cudaStream_t s) {
    phase_sums_kernel<double><<<nblocks, NTHREADS, 0, s>>>(p, w1, w2, part6);
    phase_finish_kernel<<<1, NTHREADS, 0, s>>>(p.ctl, part6, nblocks, mt6, cap, &p.ctl->status);
    return cudaGetLastError();
}

template <>
cudaError_t launch_frame<double>(double* f[3], const uint8_t* code, int nx, int ny, int nz, int pitch, int cpitch,
                                double kx, double ky, double kz, double dx, double dy, double dz, int sign,
                                cudaStream_t s) {
    frame_kernel<double><<<1216, 256, 0, s>>>(f[0], f[1], code, nx, ny, nz, pitch, cpitch, kx, ky, kz, dx, dy, dz, sign);
    return cudaGetLastError();
}

}  // namespace bt
