// Drop-in NmrRelaxationSolve over the GB300 solver (see NmrRelaxationSolve.h).
//
// init() reproduces the reference's set-up on the host (ReadAndFillInAll,
// src/NmrRelaxationSolve.cpp:2441-2454): grid, the 61 data keys, gradients,
// porosity, velocities, rates, field direction, equilibrium magnetization and
// the time step (StepTime, cpp:2519-2534). solve() / solve_gpu() upload that
// to one bt_handle and run the time loop on the GPU.
#include "NmrRelaxationSolve.h"

#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>

namespace {

const double kG = 4.78941714e+7;  // the reference's gyromagnetic constant (cpp:807)
const double kSmall = 1.0e-50;

double rmin(double a, double b) { return a <= b ? a : b; }  // NmrRelaxationSolve::min (cpp:3289-3293)

// the reference's choice of the smallest edge for the CFL limits (cpp:1578-1580, 1851-1855)
double cfl_edge_limit(double dx, double dy, double dz, double num_of_d, double den, bool squared) {
    double r = 0.0;
    auto f = [&](double d) { return squared ? num_of_d * d * d / den : num_of_d * d / den; };
    if ((dx <= dy) && (dx <= dz)) r = f(dx);
    if ((dy <= dy) && (dy <= dz)) r = f(dy);
    if ((dz <= dy) && (dz <= dz)) r = f(dz);
    return r;
}

[[noreturn]] void die(const std::string& msg) {
    std::cout << msg << std::endl;
    std::exit(1);
}

}  // namespace

NmrRelaxationSolve::~NmrRelaxationSolve() {
    if (h_) bt_destroy(h_);
}

void NmrRelaxationSolve::check(int rc, const char* what) const {
    if (rc != BT_OK) die(std::string("bt error in ") + what + ": " + (h_ ? bt_last_error(h_) : "") +
                         " (code " + std::to_string(rc) + ")");
}

void NmrRelaxationSolve::init() {
    std::string err;
    if (MPI_size != 1)
        die("This solver keeps the whole z-extent on one GPU: run it as a single process (MPI_size = 1)");
    if (!nmr::read_start("data/Nmr_start.dat", nx_, ny_, nz_, err)) die("Caught exception: " + err);
    if (!nmr::read_data("data/Nmr_data.dat", data_, err)) die("Caught exception: " + err);
    if (!nmr::read_grad("data/Nmr_grad.dat", PulseNum, gradientPulse_, multipleGradients_, err))
        die("Caught exception: " + err);
    const nmr::Data& d = data_;
    std::cout << "X grid size" << nx_ << std::endl << "Y grid size" << ny_ << std::endl
              << "Z grid size" << nz_ << std::endl;
    if (d.nComponents != 1 && d.nComponents != 2) die("NCOMP must be 1 or 2");
    if (d.noiseAmpl != 0.0 && d.nDirectionField != 0)
        die("AMPL_NOISE != 0 (an unseeded random noise field) is not supported");

    // ReadStart tail (cpp:780-816): end time, field direction, equilibrium magnetization
    const double b_total = std::sqrt(d.bsx * d.bsx + d.bsy * d.bsy + d.bsz * d.bsz);
    if (d.nSequence == 0 || d.nSequence == 1) endTime_ = 2 * d.t2Water;
    if (d.nSequence == 2) endTime_ = 4.0 * d.time1 + d.time2;
    if (d.nSequence == 5) endTime_ = d.time2 + 2.0 * d.time1;
    if (d.nSequence == 9 || d.nSequence == 99 || d.nSequence == 98) endTime_ = d.time2 + 2.0 * d.time1;
    const double bs[3] = {d.bsx, d.bsy, d.bsz};
    for (int i = 0; i < 3; ++i) {
        direction_[i] = 0.0;
        if (d.nDirectionField == i + 1) direction_[i] = 1.0;
        if (d.nDirectionField == 0) direction_[i] = bs[i] / b_total;
    }
    pEq_ = 1.0 / double((nx_ - 2 * d.bufferX) * (ny_ - 2 * d.bufferY) * (nz_ - 2 * d.bufferZ));

    // porosity (ReadActiveCells, cpp:819-878)
    if (d.nPoro == 1) {
        if (!nmr::read_poro("data/Poro.dat", nx_, ny_, nz_, mask_, err)) die("Caught exception: " + err);
    } else {
        mask_.assign((size_t)nx_ * ny_ * nz_, d.nPoro == 0 ? 1 : 0);
    }
    std::cout << "Poro read successfully!" << std::endl;

    // velocities and their CFL limit (ReadVelocity, cpp:1435-1583)
    dTimeVel_ = 1.0;
    if (d.nVelocity == 1) {
        double vmax = 0.0, vmin = 0.0;
        if (!nmr::read_velocity("data", nx_, ny_, nz_, d.velMult, vx_, vy_, vz_, vmax, vmin, err))
            die("Caught exception: " + err);
        const double vm = (vmax > std::fabs(vmin) ? vmax : std::fabs(vmin)) * d.velMult;
        dTimeVel_ = cfl_edge_limit(d.dx, d.dy, d.dz, d.cfl, vm + kSmall, false);
    }

    // phase fractions: FillInConcentration (cpp:935-1008), then for two
    // components the z1/z2 interpolation between the phase points (cpp:1780-1786)
    const size_t nvox = (size_t)nx_ * ny_ * nz_;
    c1_.assign(nvox, 0.0);
    c2_.assign(nvox, 0.0);
    if (d.nComponents == 2) {
        std::vector<double> n1;
        if (!nmr::read_n1("data/n1_init.dat", nx_, ny_, nz_, n1, err)) die("Caught exception: " + err);
        for (size_t q = 0; q < nvox; ++q) {
            const double a = n1[q], b = 1.0 - n1[q];
            const double z1 = std::sqrt((a - d.an1) * (a - d.an1) + (b - d.an2) * (b - d.an2));
            const double z2 = std::sqrt((a - d.bn1) * (a - d.bn1) + (b - d.bn2) * (b - d.bn2));
            c1_[q] = z2 / (z1 + z2);
            c2_[q] = z1 / (z1 + z2);
        }
    } else {
        for (size_t q = 0; q < nvox; ++q) {
            c1_[q] = d.nFluid == 1 ? 1.0 : 0.0;
            c2_[q] = d.nFluid == 2 ? 1.0 : 0.0;
        }
    }
    fields_ = d.nComponents == 2 || d.nSurfRelWater == 1 || d.nSurfRelOil == 1;

    // face relaxivities (ReadSurfRel, cpp:1012-1435): [1Water, 2Water, 1Oil, 2Oil][axis]
    std::vector<double> sr[4][3];
    {
        const char* keys[4] = {"1Water", "2Water", "1Oil", "2Oil"};
        const int flags[4] = {d.nSurfRelWater, d.nSurfRelWater, d.nSurfRelOil, d.nSurfRelOil};
        const double consts[4] = {d.r1Water, d.r2Water, d.r1Oil, d.r2Oil};
        const size_t nface[3] = {(size_t)(nx_ + 1) * ny_ * nz_, (size_t)nx_ * (ny_ + 1) * nz_,
                                 (size_t)nx_ * ny_ * (nz_ + 1)};
        for (int s = 0; s < 4; ++s) {
            if (flags[s] == 1) {
                if (!nmr::read_surfrel("data", keys[s], nx_, ny_, nz_, sr[s][0], sr[s][1], sr[s][2], err))
                    die("Caught exception: " + err);
            } else {
                for (int a = 0; a < 3; ++a) sr[s][a].assign(nface[a], consts[s]);
            }
        }
    }

    // rates, diffusivity and their limits (FillInDiffusinAndTime, cpp:1756-1863)
    double dMax = 0.0, tMin = 100.0;
    const long long plane = (long long)nx_ * ny_;
    const double dd[3] = {d.dx, d.dy, d.dz};
    if (fields_) {
        t1_.assign(nvox, 1.0e50);
        t2_.assign(nvox, 1.0e50);
        diff_.assign(nvox, kSmall);
    }
    for (int k = 0; k < nz_; ++k)
        for (int j = 0; j < ny_; ++j)
            for (int i = 0; i < nx_; ++i) {
                const long long q = i + (long long)nx_ * j + plane * k;
                if (!mask_[q]) continue;
                const double c1 = c1_[q], c2 = c2_[q];
                const double cd = (c1 * d.dWater + c2 * d.dOil);
                double Dv = cd * std::pow((1.0 - 2.0 * c1 * c2 / (c1 * c1 + c2 * c2)), 10.0);
                if (d.nDiffusion == 0) Dv = kSmall;
                double ct1 = c1 / d.t1Water + c2 / d.t1Oil;
                double ct2 = c1 / d.t2Water + c2 / d.t2Oil;
                // out-of-domain neighbours copy the voxel itself: never solid
                const bool solid[6] = {i > 0 && !mask_[q - 1], i < nx_ - 1 && !mask_[q + 1],
                                       j > 0 && !mask_[q - nx_], j < ny_ - 1 && !mask_[q + nx_],
                                       k > 0 && !mask_[q - plane], k < nz_ - 1 && !mask_[q + plane]};
                // the face of each neighbour in its axis' face array
                const size_t fidx[6] = {(size_t)i + (size_t)(nx_ + 1) * ((size_t)j + (size_t)ny_ * k),
                                        (size_t)(i + 1) + (size_t)(nx_ + 1) * ((size_t)j + (size_t)ny_ * k),
                                        (size_t)i + (size_t)nx_ * ((size_t)j + (size_t)(ny_ + 1) * k),
                                        (size_t)i + (size_t)nx_ * ((size_t)(j + 1) + (size_t)(ny_ + 1) * k),
                                        (size_t)i + (size_t)nx_ * ((size_t)j + (size_t)ny_ * k),
                                        (size_t)i + (size_t)nx_ * ((size_t)j + (size_t)ny_ * (k + 1))};
                for (int f = 0; f < 6; ++f)
                    if (solid[f]) {
                        const int a = f / 2;
                        const size_t fi = fidx[f];
                        ct1 += (c1 * sr[0][a][fi] + c2 * sr[2][a][fi]) / dd[a];
                        ct2 += (c1 * sr[1][a][fi] + c2 * sr[3][a][fi]) / dd[a];
                    }
                if (fields_) {
                    t1_[q] = 1.0 / ct1;
                    t2_[q] = 1.0 / ct2;
                    diff_[q] = Dv;
                }
                if (dMax <= Dv) dMax = Dv;
                if (tMin >= 1.0 / ct1) tMin = 1.0 / ct1;
                if (tMin >= 1.0 / ct2) tMin = 1.0 / ct2;
            }
    dTimeDiff_ = d.nDiffusion == 1 ? cfl_edge_limit(d.dx, d.dy, d.dz, 2.0 * d.cfl, dMax, true) : 1.0;
    dTimeRel_ = d.cfl1 * tMin;

    // gradient and noise limits (FillInMainField, cpp:1979-1988)
    double gradAmpl = 0.0;
    if (d.gradX != 0) gradAmpl = std::fabs(d.gradX * d.dx * nx_);
    if (d.gradY != 0) gradAmpl = std::fabs(d.gradY * d.dy * ny_);
    if (d.gradZ != 0) gradAmpl = std::fabs(d.gradZ * d.dz * nz_);
    if (d.gradX == 0 && d.gradY == 0 && d.gradZ == 0) gradAmpl = kSmall;
    dTimeNoise_ = d.cfl1 / (kG * d.noiseAmpl);
    dTimeGrad_ = d.cfl1 / (kG * gradAmpl);

    // StepTime (cpp:2519-2534)
    if (d.time1 != 0)
        dTime_ = rmin(rmin(rmin(dTimeNoise_, dTimeGrad_), rmin(dTimeVel_, dTimeDiff_)), rmin(dTimeRel_, d.time1 / 100.0));
    else
        dTime_ = rmin(rmin(rmin(dTimeNoise_, dTimeGrad_), rmin(dTimeVel_, dTimeDiff_)), rmin(dTimeRel_, d.time2 / 100.0));
    nStep_ = int(endTime_ / dTime_) + 1;
    std::cout << "dTime=" << std::scientific << dTime_ << std::endl << "nStep=" << nStep_ << std::endl;
    std::cout.unsetf(std::ios::floatfield);
    initialised_ = true;
}

std::string NmrRelaxationSolve::describe() const {
    std::ostringstream s;
    s.precision(17);
    s << "nx " << nx_ << "\nny " << ny_ << "\nnz " << nz_ << "\ndTime " << dTime_ << "\nnStep " << nStep_
      << "\npEq " << pEq_ << "\nendTime " << endTime_ << "\ndirection " << direction_[0] << " " << direction_[1] << " "
      << direction_[2] << "\ngradientPulse " << gradientPulse_ << "\ndTimeVel " << dTimeVel_ << "\ndTimeDiff "
      << dTimeDiff_ << "\ndTimeRel " << dTimeRel_ << "\n";
    return s.str();
}

bt_config NmrRelaxationSolve::make_config(bool gpu_path) const {
    const nmr::Data& d = data_;
    bt_config c{};
    c.nx = nx_;
    c.ny = ny_;
    c.nz = nz_;
    const char* p = std::getenv("BT_PRECISION");
    c.precision = (p && std::string(p) == "f32") ? BT_F32 : BT_F64;
    // solve() steps as the reference's CPU path (ExplicitSimple), solve_gpu() as
    // its GPU path (the MacCormack ExplicitMakUpgrade); BT_SCHEME=explicit
    // runs solve_gpu() with ExplicitSimple
    const char* sch = std::getenv("BT_SCHEME");
    c.scheme = (gpu_path && !(sch && std::string(sch) == "explicit")) ? BT_SCHEME_MACCORMACK : BT_SCHEME_REFERENCE;
    c.vector_mult = d.nVectorMult;
    c.velocity = d.nVelocity;
    c.diffusion = d.nDiffusion;
    c.buffer[0] = d.bufferX;
    c.buffer[1] = d.bufferY;
    c.buffer[2] = d.bufferZ;
    c.dx = d.dx;
    c.dy = d.dy;
    c.dz = d.dz;
    c.dt = dTime_;
    // FillInMainField (cpp:1944-1962)
    c.main_field[0] = (d.nDirectionField == 1 || d.nDirectionField == 0) ? d.bsx : 0.0;
    c.main_field[1] = (d.nDirectionField == 2 || d.nDirectionField == 0) ? d.bsy : 0.0;
    c.main_field[2] = (d.nDirectionField == 3 || d.nDirectionField == 0) ? d.bsz : 0.0;
    c.gamma = kG;
    c.grad[0] = d.gradX;
    c.grad[1] = d.gradY;
    c.grad[2] = d.gradZ;
    const bool water = d.nFluid == 1;
    c.d_pore = water ? d.dWater : d.dOil;
    c.t1 = water ? d.t1Water : d.t1Oil;
    c.t2 = water ? d.t2Water : d.t2Oil;
    c.rho1 = water ? d.r1Water : d.r1Oil;
    c.rho2 = water ? d.r2Water : d.r2Oil;
    c.p_eq = pEq_;
    // ghost layers: the CPU path (solve, ExplicitSimple) copies on every face
    // whatever Nmr_data.dat says (BoundaryConditionsForVectorField,
    // cpp:1664-1754); the GPU path dispatches on nBoundary1..6 (cu:1321-1396):
    // per pair (x: 1 and 3, y: 2 and 4, z: 5 and 6) copy when both are 1,
    // periodic when both are 3, and zero otherwise (BC_Advanced on x for a 2;
    // a pair that routine leaves alone keeps never-written, zero ghosts)
    for (int a = 0; a < 3; ++a) c.boundary[a] = BT_BC_COPY;
    if (gpu_path) {
        const int lo[3] = {d.nb[0], d.nb[1], d.nb[4]}, hi[3] = {d.nb[2], d.nb[3], d.nb[5]};
        for (int a = 0; a < 3; ++a)
            c.boundary[a] = (lo[a] == 1 && hi[a] == 1) ? BT_BC_COPY
                            : (lo[a] == 3 && hi[a] == 3) ? BT_BC_PERIODIC
                                                         : BT_BC_ZERO;
    }
    return c;
}

// FillInMagnetization (cpp:2472-2517): p_eq along the field axis in pores, 0 in solid
void NmrRelaxationSolve::initial_field(std::vector<double>& mx, std::vector<double>& my,
                                       std::vector<double>& mz) const {
    const nmr::Data& d = data_;
    const size_t n = mask_.size();
    mx.assign(n, 0.0);
    my.assign(n, 0.0);
    mz.assign(n, 0.0);
    double v[3] = {0.0, 0.0, 0.0};
    if (d.nDirectionField >= 1 && d.nDirectionField <= 3) v[d.nDirectionField - 1] = pEq_;
    if (d.nDirectionField == 0) {
        const double b_total = std::sqrt(d.bsx * d.bsx + d.bsy * d.bsy + d.bsz * d.bsz);
        v[0] = pEq_ * (d.bsx / b_total);
        v[1] = pEq_ * (d.bsy / b_total);
        v[2] = pEq_ * (d.bsz / b_total);
    }
    for (size_t q = 0; q < n; ++q)
        if (mask_[q]) {
            mx[q] = v[0];
            my[q] = v[1];
            mz[q] = v[2];
        }
}

void NmrRelaxationSolve::run(bool gpu_path) {
    if (!initialised_) die("init() must come before solve()");
    const nmr::Data& d = data_;
    const bt_config c = make_config(gpu_path);
    check(bt_create(&c, &h_), "bt_create");
    check(bt_upload_geometry(h_, mask_.data(), vx_.empty() ? nullptr : vx_.data(), vy_.empty() ? nullptr : vy_.data(),
                             vz_.empty() ? nullptr : vz_.data()),
          "bt_upload_geometry");
    const bool two = d.nComponents == 2;
    if (fields_) check(bt_upload_rates(h_, t1_.data(), t2_.data(), diff_.data()), "bt_upload_rates");
    if (two) check(bt_set_phase_weights(h_, c1_.data(), c2_.data()), "bt_set_phase_weights");
    std::vector<double> mx, my, mz;
    initial_field(mx, my, mz);
    check(bt_set_state(h_, mx.data(), my.data(), mz.data()), "bt_set_state");
    // the reference's own schedule over the loop's nStep + 1 iterations
    const long long iters = (long long)nStep_ + 1;
    bt_sequence_params sp{};
    sp.n_sequence = d.nSequence;
    sp.gpu_variant = gpu_path ? 1 : 0;
    sp.dt = dTime_;
    sp.time1 = d.time1;
    sp.time2 = d.time2;
    for (int a = 0; a < 3; ++a) sp.direction[a] = direction_[a];
    sp.gradient_pulse = gradientPulse_;
    for (int a = 0; a < 3; ++a) sp.multiple_gradients[a] = multipleGradients_[a];
    int npulses = 0;
    check(bt_sequence_schedule(&sp, iters, nullptr, 0, &npulses), "bt_sequence_schedule");
    std::vector<bt_pulse> pulses(std::max(npulses, 1));
    check(bt_sequence_schedule(&sp, iters, pulses.data(), npulses, &npulses), "bt_sequence_schedule");
    check(bt_set_schedule(h_, pulses.data(), npulses, nullptr, 0), "bt_set_schedule");

    // the sums of one output row: 3 (SumX, SumY, SumZ) or, with two
    // components, 6 (X1 Y1 Z1 X2 Y2 Z2; OutputX/Y/Z cpp:3324-3350)
    const int w = two ? 6 : 3;
    std::vector<double> m0(w, 0.0);
    if (two) {
        // the initial field's two-component sums, in the reference's order
        for (int k = d.bufferZ; k < nz_ - d.bufferZ; ++k)
            for (int j = d.bufferY; j < ny_ - d.bufferY; ++j)
                for (int i = d.bufferX; i < nx_ - d.bufferX; ++i) {
                    const size_t q = (size_t)i + (size_t)nx_ * ((size_t)j + (size_t)ny_ * k);
                    if (!mask_[q] || !(c1_[q] > 0.8 || c2_[q] > 0.8)) continue;
                    m0[0] += mx[q] * c1_[q];
                    m0[3] += mx[q] * c2_[q];
                    m0[1] += my[q] * c1_[q];
                    m0[4] += my[q] * c2_[q];
                    m0[2] += mz[q] * c1_[q];
                    m0[5] += mz[q] * c2_[q];
                }
    } else {
        check(bt_measure(h_, m0.data()), "bt_measure");
    }
    std::vector<double> mt((size_t)w * iters);
    std::vector<double> mt3(two ? 3 * std::min<long long>(iters, 65536) : 0);
    const long long chunk = 65536;
    for (long long s = 0; s < iters; s += chunk) {
        const long long n = std::min(chunk, iters - s);
        if (two) {
            check(bt_run(h_, n, mt3.data()), "bt_run");
            check(bt_read_mt_phases(h_, &mt[6 * s], n), "bt_read_mt_phases");
        } else {
            check(bt_run(h_, n, &mt[3 * s]), "bt_run");
        }
    }
    // sums printed at step i: after the step on the GPU path (cu:1187-1219),
    // before it on the CPU path (cpp:38-55)
    auto sums_at = [&](long long i) -> const double* {
        if (gpu_path) return &mt[(size_t)w * i];
        return i == 0 ? m0.data() : &mt[(size_t)w * (i - 1)];
    };
    auto row = [&](std::ostream& o, double t, const double* r) {
        o << std::scientific << t;
        for (int c = 0; c < w; ++c) o << "; " << std::scientific << r[c];
        o << std::endl;
    };
    std::ofstream res(gpu_path ? "results_gpu.csv" : "results_cpu.csv");
    res << "Time; SumX; SumY; SumZ" << std::endl;
    for (long long i = 0; i < iters; ++i) {
        if (i % d.ndPrint != 0) continue;
        const double t = i * dTime_;
        const double* r = sums_at(i);
        if (two)
            std::cout << " Time = " << t << " SumX1=" << r[0] << " SumY1=" << r[1] << " SumZ1=" << r[2]
                      << "\t SumX2=" << r[3] << " SumY2=" << r[4] << " SumZ2=" << r[5] << std::endl;
        else
            std::cout << " Time = " << t << " SumX=" << r[0] << " SumY=" << r[1] << " SumZ=" << r[2] << std::endl;
        row(res, t, r);
    }
    res.close();
    if (gpu_path) {
        // the final line (cu:1290-1314): last loop time and the final field's sums
        mkdir("results_NMR", 0755);
        char name[256];
        std::snprintf(name, sizeof(name), "results_NMR/results_grad_%d_%d_%d.csv", PulseNum[0], PulseNum[1],
                      PulseNum[2]);
        std::ofstream rg(name);
        const double* r = &mt[(size_t)w * (iters - 1)];
        std::cout << " SumX=" << r[0] << " SumY=" << r[1] << " SumZ=" << r[2] << std::endl;
        row(rg, (iters - 1) * dTime_, r);
    }
    bt_destroy(h_);
    h_ = nullptr;
}

void NmrRelaxationSolve::solve() { run(false); }

void NmrRelaxationSolve::solve_gpu() { run(true); }
