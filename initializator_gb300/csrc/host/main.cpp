// nmr_exe: the reference program's entry point (src/main.cpp of
// soleh00/Initializator) over the GB300 solver.
//   nmr_exe gx gy gz [deviceShift]
// gx gy gz select the gradient lines of data/Nmr_grad.dat (PulseNum); the
// device is deviceShift modulo the number of GPUs (one process, one GPU: the
// reference's MPI z-split is replaced by the whole z-extent on one device).
#include <cuda_runtime.h>

#include <cstdlib>
#include <iostream>

#include "NmrRelaxationSolve.h"

int main(int argc, char** argv) {
    int gradientNum[3] = {0, 0, 0};
    if (argc >= 4) {
        gradientNum[0] = std::atoi(argv[1]);
        gradientNum[1] = std::atoi(argv[2]);
        gradientNum[2] = std::atoi(argv[3]);
    } else {
        std::cout << "Caught exception number:  0 gradient pulse failer!" << std::endl;
    }
    std::cout << "Gradient pulses are:   X=" << gradientNum[0] << " Y=" << gradientNum[1] << " Z=" << gradientNum[2]
              << std::endl;
    int deviceShift = 0;
    if (argc >= 5) deviceShift = std::atoi(argv[4]);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        std::cout << "no CUDA device" << std::endl;
        return 1;
    }
    std::cout << "Cuda device " << deviceShift % ndev << std::endl;
    cudaSetDevice(deviceShift % ndev);
    NmrRelaxationSolve solver(1, 0, gradientNum);
    solver.init();
    if (std::getenv("BT_CPU_PATH")) solver.solve();  // results_cpu.csv semantics
    else solver.solve_gpu();
    return 0;
}
