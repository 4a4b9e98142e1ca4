// Readers of the reference solver's input files (host only).
//
// Formats follow the reference (soleh00/Initializator, src/NmrRelaxationSolve.cpp):
//   Nmr_start.dat  three integers, each followed by the rest of its line (cpp:68-93)
//   Nmr_data.dat   exactly 61 lines "value<TAB>comment"; a parameter is the value
//                  of the first line whose comment contains its token (cpp:175-723)
//   Nmr_grad.dat   a count, then one gradient per line (cpp:727-778)
//   Poro.dat       header line, then '0'/'1' characters read with >>, k outer,
//                  j, i inner (cpp:859-872)
//   Vx/Vy/Vz.dat   header line, then (nx+1)*ny*nz / nx*(ny+1)*nz / nx*ny*(nz+1)
//                  doubles, i outer, j, k inner (cpp:1466-1536)
// Arrays returned here use this library's layouts: x fastest, [k][j][i].
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace nmr {

struct Data {
    int key = 1, iPrint = 1, jPrint = 1, kPrint = 1, ndPrint = 500, ndWrite = 1, ndVid = 1, ndAmpl = 1;
    int nPoro = 1, nComponents = 1, nFluid = 1, nSurfRelWater = 0, nSurfRelOil = 0;
    int nVectorMult = 0, nVelocity = 0, nDiffusion = 1, nDirectionField = 1, nSequence = 0;
    int nb[6] = {1, 1, 1, 1, 1, 1};
    double dx = 1e-6, dy = 1e-6, dz = 1e-6;
    double bsx = 1.0, bsy = 0.0, bsz = 0.0, bdx = 0.0, bdy = 0.0, bdz = 0.0;
    double time1 = 0.0, time2 = 0.0;
    double gradX = 0.0, gradY = 0.0, gradZ = 0.0, noiseAmpl = 0.0, velMult = 1.0;
    double dOil = 0.0, dWater = 0.0, r1Oil = 0.0, r1Water = 0.0, r2Oil = 0.0, r2Water = 0.0;
    double t1Oil = 0.0, t1Water = 0.0, t2Oil = 0.0, t2Water = 0.0;
    double temperature = 300.0, an1 = 1.0, an2 = 0.0, bn1 = 0.0, bn2 = 1.0, cfl = 0.002, cfl1 = 0.002, step0 = 0.0;
    int bufferX = 0, bufferY = 0, bufferZ = 0;
};

// Each reader returns false and fills `err` when the file is missing or short.
bool read_start(const std::string& path, int& nx, int& ny, int& nz, std::string& err);
bool read_data(const std::string& path, Data& d, std::string& err);
// gradientPulse and multipleGradients for the gradient line numbers PulseNum[0..2]
bool read_grad(const std::string& path, const int pulse_num[3], double& gradient_pulse, double multiple[3],
               std::string& err);
bool read_poro(const std::string& path, int nx, int ny, int nz, std::vector<uint8_t>& mask, std::string& err);
// face velocities times vel_mult; vmax_raw / vmin_raw are the extremes of the
// raw file values over all three files (ReadVelocity, cpp:1458-1583)
bool read_velocity(const std::string& dir, int nx, int ny, int nz, double vel_mult, std::vector<double>& vx,
                   std::vector<double>& vy, std::vector<double>& vz, double& vmax_raw, double& vmin_raw,
                   std::string& err);

// SurfRel<key>{X,Y,Z}.dat, key one of 1Water 2Water 1Oil 2Oil (ReadSurfRel,
// cpp:1035-1434): face arrays in the velocity layout, [k][j][i] with nx+1,
// ny+1, nz+1 faces along the array's own axis
bool read_surfrel(const std::string& dir, const std::string& key, int nx, int ny, int nz, std::vector<double>& fx,
                  std::vector<double>& fy, std::vector<double>& fz, std::string& err);
// n1_init.dat (cpp:974-1006): ik*jk*kk values read as float, i outer, k inner;
// out [k][j][i]
bool read_n1(const std::string& path, int nx, int ny, int nz, std::vector<double>& n1, std::string& err);

}  // namespace nmr
