// float instantiation of the fused step kernel and its helpers.
// Compiled with the default -fmad=true (FP32 production path).
#include <cstdlib>

#include "bt_step_tma.cuh"
#include "bt_step_mac.cuh"

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
cudaError_t launch_mac<float>(const StepParams<float>& p, float* const pred[3], int vel, int prec, dim3 grid, cudaStream_t s) {
    return launch_mac_impl<float>(p, pred, vel, prec, grid, s);
}

template <>
cudaError_t launch_phase_sums<float>(const StepParams<float>& p, const float* w1, const float* w2, double* part6, int nblocks,
                                double* mt6, long long cap, cudaStream_t s) {
    phase_sums_kernel<float><<<nblocks, NTHREADS, 0, s>>>(p, w1, w2, part6);
    phase_finish_kernel<<<1, NTHREADS, 0, s>>>(p.ctl, part6, nblocks, mt6, cap, &p.ctl->status);
    return cudaGetLastError();
}

template <>
cudaError_t launch_frame<float>(float* f[3], const uint8_t* code, int nx, int ny, int nz, int pitch, int cpitch,
                                double kx, double ky, double kz, double dx, double dy, double dz, int sign,
                                cudaStream_t s) {
    frame_kernel<float><<<1216, 256, 0, s>>>(f[0], f[1], code, nx, ny, nz, pitch, cpitch, kx, ky, kz, dx, dy, dz, sign);
    return cudaGetLastError();
}


cudaError_t launch_cell_velocity(const StepParams<float>& p, float* u, long long comp, cudaStream_t s) {
    cell_velocity_kernel<<<1216, 256, 0, s>>>(p, u, comp);
    return cudaGetLastError();
}

cudaError_t launch_tma_finish(const StepParams<float>& p, dim3 grid, cudaStream_t s) {
    const unsigned nb = p.nbatch > 1 ? (unsigned)p.nbatch : 1u;
    const unsigned nb_per = (grid.x / nb) * grid.y * grid.z;
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = pdl_config(dim3(1), dim3(256), 0, s, attr);
    return cudaLaunchKernelEx(&cfg, step_finish_kernel<float>, p, nb_per);
}

cudaError_t launch_step_tma(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec, bool pal,
                            bool rf, dim3 grid, int tw, bool first, cudaStream_t s) {
    if (rf) return launch_step_tma_pulse(p, m, scheme, vel, prec, grid, tw, first, s);
    if (pal) return launch_step_tma_palette(p, m, scheme, vel, prec, grid, tw, first, s);
    if (tw == 64) return launch_step_tma64(p, m, scheme, vel, prec, grid, first, s);
    return launch_step_tma_w<128>(p, m, scheme, vel, prec, grid, first, s);
}

}  // namespace bt
