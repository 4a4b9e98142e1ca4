// float instantiation of the fused step kernel and its helpers.
// Compiled with the default -fmad=true (FP32 production path).
#include "bt_step.cuh"

namespace bt {

template <>
cudaError_t launch_step<float>(const StepParams<float>& p, int scheme, int vel, int prec, dim3 grid, cudaStream_t s) {
    return launch_step_impl<float>(p, scheme, vel, prec, grid, s);
}

template <>
cudaError_t launch_sums<float>(const StepParams<float>& p, double* kvec_and_grid, cudaStream_t s) {
    // kvec_and_grid: {kx, ky, kz, nblocks}
    const int nblocks = (int)kvec_and_grid[3];
    sums_kernel<float><<<nblocks, NTHREADS, 0, s>>>(p, kvec_and_grid[0], kvec_and_grid[1], kvec_and_grid[2], p.partials);
    return cudaGetLastError();
}

template <>
cudaError_t launch_frame<float>(float* f[3], const uint8_t* code, int nx, int ny, int nz, double kx, double ky,
                                double kz, double dx, double dy, double dz, int sign, cudaStream_t s) {
    frame_kernel<float><<<1216, 256, 0, s>>>(f[0], f[1], code, nx, ny, nz, kx, ky, kz, dx, dy, dz, sign);
    return cudaGetLastError();
}

}  // namespace bt
