// Pinning harness, test infrastructure only: drives the reference solver's
// own CPU path (built unmodified from the reference sources against the
// single-rank MPI stub) and dumps what the oracle is checked against.
//
// It reproduces the body of NmrRelaxationSolve::solve() (reference
// src/NmrRelaxationSolve.cpp:35-66) step by step so that the fields can be read
// before ClearAll() frees them:
//   for i in [0, nsteps): currentTime = i*dTime; OutputX/Y/Z; ExplicitSimple();
//                         Sequence(); BoundaryConditionsForVectorField(&magnetization)
// followed by one more OutputX/Y/Z of the final field.
//
// usage: ref_harness <workdir> <nsteps> <dt or 0> <outdir> [state.bin|-] [pulses.txt]
//   workdir holds data/Nmr_start.dat, data/Nmr_data.dat, data/Nmr_grad.dat and
//   whatever else the data file switches on (Poro.dat, Vx/Vy/Vz.dat).
//   state.bin (optional): 3*nx*ny*nz doubles (x, y, z; [k][j][i]) replacing the
//   initial magnetization of the interior before the first step.
//   pulses.txt (optional): lines "step flag param ax ay az"; when given, these
//   AddImpulse calls replace Sequence() (so every pulse flag can be pinned).
// outputs in outdir: mt.bin ((nsteps+1)*3 doubles, sums before each step and
//   after the last), state.bin (3*N doubles), rates.bin (tau1 then tau2, N each),
//   times.bin (relTime.t1 then relTime.t2 as stored, N each), diff.bin (N),
//   info.txt; with NCOMP 2 also mt6.bin ((nsteps+1)*6 doubles: X1 Y1 Z1 X2 Y2 Z2)
//   and phases.bin (the concentrations, 2*N).

// standard headers first, so that the access override below only reaches the
// reference's class
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>
#include <math.h>
#include <memory.h>
#include <stdlib.h>
#include <omp.h>
#include <cuda_runtime.h>
#include <unistd.h>
#include "mpi.h"

#define private public
#include "NmrRelaxationSolve.h"
#undef private

static void dump(const std::string& path, const double* p, size_t n) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(3); }
    std::fwrite(p, sizeof(double), n, f);
    std::fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s workdir nsteps dt outdir [state.bin]\n", argv[0]);
        return 2;
    }
    std::string outdir = argv[4];
    if (outdir[0] != '/') {
        char cwd[4096];
        if (!getcwd(cwd, sizeof(cwd))) return 2;
        outdir = std::string(cwd) + "/" + outdir;
    }
    if (chdir(argv[1]) != 0) { std::perror("chdir"); return 2; }
    long nsteps = std::atol(argv[2]);
    double dt = std::atof(argv[3]);
    int num[3] = {1, 1, 1};
    NmrRelaxationSolve s(1, 0, num);
    s.init();
    const double dTime_init = s.dTime;  // what StepTime derived
    const int nStep_init = s.nStep;
    if (dt > 0) s.dTime = dt;
    const GridSize gs = s.gs;
    const size_t N = (size_t)gs.ik * gs.jk * gs.kk;
    auto interior = [&](int i, int j, int k) { return s.index(i + 1, j + 1, k + 1, gs); };
    struct Pulse { long step; int flag; double param, ax, ay, az; };
    std::vector<Pulse> pulses;
    bool explicit_pulses = false;
    if (argc >= 7) {
        explicit_pulses = true;
        FILE* pf = std::fopen(argv[6], "r");
        if (!pf) { std::perror(argv[6]); return 2; }
        Pulse p;
        while (std::fscanf(pf, "%ld %d %lf %lf %lf %lf", &p.step, &p.flag, &p.param, &p.ax, &p.ay, &p.az) == 6)
            pulses.push_back(p);
        std::fclose(pf);
    }
    if (argc >= 6 && std::strcmp(argv[5], "-") != 0) {
        std::vector<double> st(3 * N);
        FILE* f = std::fopen(argv[5], "rb");
        if (!f || std::fread(st.data(), sizeof(double), 3 * N, f) != 3 * N) { std::fprintf(stderr, "bad state\n"); return 2; }
        std::fclose(f);
        for (int k = 0; k < gs.kk; k++)
            for (int j = 0; j < gs.jk; j++)
                for (int i = 0; i < gs.ik; i++) {
                    size_t q = (size_t)i + (size_t)gs.ik * ((size_t)j + (size_t)gs.jk * k);
                    int c = interior(i, j, k);
                    s.magnetization.x[c] = st[q];
                    s.magnetization.y[c] = st[N + q];
                    s.magnetization.z[c] = st[2 * N + q];
                }
        s.BoundaryConditionsForVectorField(&s.magnetization);
    }
    std::vector<double> mt, mt6;
    auto push6 = [&]() {
        if (s.nComponents != 2) return;
        const double v6[6] = {s.resX1, s.resY1, s.resZ1, s.resX2, s.resY2, s.resZ2};
        mt6.insert(mt6.end(), v6, v6 + 6);
    };
    for (long i = 0; i < nsteps; i++) {
        s.currentTime = i * s.dTime;
        s.OutputX(&s.magnetization); s.OutputY(&s.magnetization); s.OutputZ(&s.magnetization);
        mt.push_back(s.resX); mt.push_back(s.resY); mt.push_back(s.resZ);
        push6();
        s.ExplicitSimple();
        if (explicit_pulses) {
            for (const Pulse& p : pulses)
                if (p.step == i) s.AddImpulse(p.flag, p.param, p.ax, p.ay, p.az, &s.magnetization);
        } else {
            s.Sequence();
        }
        s.BoundaryConditionsForVectorField(&s.magnetization);
    }
    s.OutputX(&s.magnetization); s.OutputY(&s.magnetization); s.OutputZ(&s.magnetization);
    mt.push_back(s.resX); mt.push_back(s.resY); mt.push_back(s.resZ);
    push6();

    std::vector<double> st(3 * N), rates(2 * N), times(2 * N), diff(N), phases(2 * N);
    for (int k = 0; k < gs.kk; k++)
        for (int j = 0; j < gs.jk; j++)
            for (int i = 0; i < gs.ik; i++) {
                size_t q = (size_t)i + (size_t)gs.ik * ((size_t)j + (size_t)gs.jk * k);
                int c = interior(i, j, k);
                st[q] = s.magnetization.x[c];
                st[N + q] = s.magnetization.y[c];
                st[2 * N + q] = s.magnetization.z[c];
                rates[q] = 1.0 / s.relTime.t1[c];
                rates[N + q] = 1.0 / s.relTime.t2[c];
                times[q] = s.relTime.t1[c];
                times[N + q] = s.relTime.t2[c];
                diff[q] = s.diffusion[c];
                phases[q] = s.concentration[0][c];
                phases[N + q] = s.concentration[1][c];
            }
    dump(outdir + "/mt.bin", mt.data(), mt.size());
    dump(outdir + "/state.bin", st.data(), st.size());
    dump(outdir + "/rates.bin", rates.data(), rates.size());
    dump(outdir + "/diff.bin", diff.data(), diff.size());
    dump(outdir + "/times.bin", times.data(), times.size());
    if (s.nComponents == 2) {
        dump(outdir + "/mt6.bin", mt6.data(), mt6.size());
        dump(outdir + "/phases.bin", phases.data(), phases.size());
    }
    FILE* f = std::fopen((outdir + "/info.txt").c_str(), "w");
    std::fprintf(f, "nx %d\nny %d\nnz %d\ndTime %.17g\npEq %.17g\nnStep %d\ndirection %.17g %.17g %.17g\n",
                 gs.ik, gs.jk, gs.kk, s.dTime, s.equilibriumMagnetization, s.nStep,
                 s.direction[0], s.direction[1], s.direction[2]);
    std::fprintf(f, "dTimeInit %.17g\nnStepInit %d\ngradientPulse %.17g\n", dTime_init, nStep_init,
                 s.gradientPulse);
    std::fclose(f);
    return 0;
}
