// Drop-in replacement for the reference solver's driver class
// (headers/NmrRelaxationSolve.h:32-130 of soleh00/Initializator).
//
// Public interface kept exactly: the constructor (MPI size, rank, the three
// gradient line numbers), init(), solve(), solve_gpu() and the public fields
// MPI_size, MPI_rank, PulseNum. It reads the same data/*.dat files relative to
// the working directory and writes the same CSV outputs. Every step runs on
// the GPU through the C ABI of include/bt.h; there is no CPU stepper:
//   solve()     the reference's CPU path semantics (Sequence, cpp:2610-2679;
//               M(t) printed BEFORE each step into results_cpu.csv)
//   solve_gpu() the reference's GPU path semantics (Sequence_gpu,
//               cpp:2681-3146; M(t) printed AFTER each step into
//               results_gpu.csv, final line into
//               results_NMR/results_grad_<gx>_<gy>_<gz>.csv)
// Each steps with the update of its reference path: solve() with the explicit
// upwind update (ExplicitSimple, cpp:3148-3282), solve_gpu() with the
// predictor-corrector of the reference's kernels (NMR_predictor_upgrade /
// NMR_corrector_upgrade, cu:637-967); BT_SCHEME=explicit makes solve_gpu()
// use ExplicitSimple too. The whole z-extent lives on one GPU, so MPI_size
// must be 1. The arithmetic is FP64 (bit-identical fields) unless the
// environment sets BT_PRECISION=f32 (FP32 fields; ExplicitSimple steps then
// take the FP32 fast path).
#pragma once
#include <string>
#include <vector>

#include "../../../include/bt.h"
#include "nmr_io.h"

class NmrRelaxationSolve {
public:
    NmrRelaxationSolve(int size, int rank, int* num) {
        MPI_size = size;
        MPI_rank = rank;
        PulseNum[0] = num[0];
        PulseNum[1] = num[1];
        PulseNum[2] = num[2];
    }
    ~NmrRelaxationSolve();
    int MPI_size, MPI_rank, PulseNum[3];
    void solve();
    void init();
    void solve_gpu();

    // Not in the reference: the parameters init() derived, one "key value" per
    // line (time step, step count, equilibrium magnetization, field direction).
    std::string describe() const;

private:
    nmr::Data data_;
    int nx_ = 0, ny_ = 0, nz_ = 0;
    std::vector<uint8_t> mask_;
    std::vector<double> vx_, vy_, vz_;
    double gradientPulse_ = 0.0, multipleGradients_[3] = {0.0, 0.0, 0.0};
    double direction_[3] = {0.0, 0.0, 0.0};
    double pEq_ = 0.0, endTime_ = 0.0, dTime_ = 0.0;
    double dTimeVel_ = 1.0, dTimeDiff_ = 1.0, dTimeRel_ = 1.0, dTimeNoise_ = 0.0, dTimeGrad_ = 0.0;
    int nStep_ = 0;
    // per-voxel coefficients (SurfRel*.dat or NCOMP 2): T1, T2, D as
    // FillInDiffusinAndTime forms them, and the phase fractions c1, c2
    bool fields_ = false;
    std::vector<double> t1_, t2_, diff_, c1_, c2_;
    bool initialised_ = false;
    bt_handle* h_ = nullptr;

    bt_config make_config(bool gpu_path) const;
    void initial_field(std::vector<double>& mx, std::vector<double>& my, std::vector<double>& mz) const;
    void run(bool gpu_path);
    void check(int rc, const char* what) const;
};
