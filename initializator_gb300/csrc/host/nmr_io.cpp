// Readers of the reference solver's input files (see nmr_io.h for the formats).
#include "nmr_io.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <utility>

namespace nmr {

bool read_start(const std::string& path, int& nx, int& ny, int& nz, std::string& err) {
    std::ifstream f(path);
    if (!f) {
        err = "No file " + path;
        return false;
    }
    std::string rest;
    f >> nx;
    std::getline(f, rest);
    f >> ny;
    std::getline(f, rest);
    f >> nz;
    if (!f || nx <= 0 || ny <= 0 || nz <= 0) {
        err = path + ": expected three positive grid sizes";
        return false;
    }
    return true;
}

bool read_data(const std::string& path, Data& d, std::string& err) {
    std::ifstream f(path);
    if (!f) {
        err = "No file " + path;
        return false;
    }
    // exactly 61 "value<TAB>comment" lines, as ReadStart reads them
    std::vector<std::pair<std::string, std::string>> lines;
    for (int i = 0; i < 61; ++i) {
        std::string v, c;
        if (!std::getline(f, v, '\t') || !std::getline(f, c, '\n')) {
            err = path + ": fewer than 61 value<TAB>comment lines";
            return false;
        }
        lines.emplace_back(v, c);
    }
    // first line whose comment contains the token wins
    auto find = [&](const char* token, const std::string** out) {
        for (const auto& kv : lines)
            if (kv.second.find(token) != std::string::npos) {
                *out = &kv.first;
                return true;
            }
        return false;
    };
    auto geti = [&](const char* token, int& dst) {
        const std::string* v;
        if (find(token, &v)) dst = std::atoi(v->c_str());
    };
    auto getd = [&](const char* token, double& dst) {
        const std::string* v;
        if (find(token, &v)) dst = std::atof(v->c_str());
    };
    geti("KEY", d.key);
    geti("IPRINT", d.iPrint);
    geti("JPRINT", d.jPrint);
    geti("KPRINT", d.kPrint);
    geti("Printing on", d.ndPrint);
    geti("NDWRIT", d.ndWrite);
    geti("NDVID", d.ndVid);
    geti("NDAMPL", d.ndAmpl);
    geti("NPOR", d.nPoro);
    geti("NCOMP", d.nComponents);
    geti("NFLUID", d.nFluid);
    geti("nSurfRelWater", d.nSurfRelWater);
    geti("nSurfRelOil", d.nSurfRelOil);
    geti("NVECTOR", d.nVectorMult);
    geti("NVELOC", d.nVelocity);
    geti("NDIFFUS", d.nDiffusion);
    geti("NDIRECT_FIELD", d.nDirectionField);
    geti("NSEQUENCE", d.nSequence);
    const char* nbk[6] = {"NB1", "NB2", "NB3", "NB4", "NB5", "NB6"};
    for (int b = 0; b < 6; ++b) geti(nbk[b], d.nb[b]);
    getd("DX", d.dx);
    getd("DY", d.dy);
    getd("DZ", d.dz);
    getd("BX0", d.bsx);
    getd("BY0", d.bsy);
    getd("BZ0", d.bsz);
    getd("TIME1", d.time1);
    getd("TIME2", d.time2);
    getd("GRAD_X", d.gradX);
    getd("GRAD_Y", d.gradY);
    getd("GRAD_Z", d.gradZ);
    getd("AMPL_NOISE", d.noiseAmpl);
    getd("VEL_MULT", d.velMult);
    getd("D_OIL", d.dOil);
    getd("D_WAT", d.dWater);
    getd("R1_OIL", d.r1Oil);
    getd("R1_WAT", d.r1Water);
    getd("R2_OIL", d.r2Oil);
    getd("R2_WAT", d.r2Water);
    getd("T1_OIL", d.t1Oil);
    getd("T1_WAT", d.t1Water);
    getd("T2_OIL", d.t2Oil);
    getd("T2_WAT", d.t2Water);
    getd("T0", d.temperature);
    getd("AN(1)", d.an1);
    getd("AN(2)", d.an2);
    getd("BN(1)", d.bn1);
    getd("BN(2)", d.bn2);
    getd("CFL", d.cfl);
    getd("CFL1", d.cfl1);
    getd("TIMEW", d.step0);
    geti("bufferX", d.bufferX);
    geti("bufferY", d.bufferY);
    geti("bufferZ", d.bufferZ);
    return true;
}

bool read_grad(const std::string& path, const int pulse_num[3], double& gradient_pulse, double multiple[3],
               std::string& err) {
    std::ifstream f(path);
    if (!f) {
        err = "No file " + path;
        return false;
    }
    std::vector<std::string> lines;
    std::string l;
    while (std::getline(f, l)) lines.push_back(l);
    if (lines.empty()) {
        err = path + ": empty";
        return false;
    }
    const int total = std::atoi(lines[0].c_str());
    if (total < pulse_num[0]) {
        err = path + ": gradient line " + std::to_string(pulse_num[0]) + " beyond the count " + std::to_string(total);
        return false;
    }
    // the value on line n (1-based, after the count line) is the n-th gradient
    auto value = [&](int n) -> double {
        if (n <= 0 || n >= (int)lines.size()) return 0.0;
        return std::atof(lines[n].c_str());
    };
    gradient_pulse = value(pulse_num[0] >= 1 ? pulse_num[0] : 1);
    for (int a = 0; a < 3; ++a) multiple[a] = pulse_num[a] != 0 ? value(pulse_num[a]) : 0.0;
    return true;
}

bool read_poro(const std::string& path, int nx, int ny, int nz, std::vector<uint8_t>& mask, std::string& err) {
    std::ifstream f(path);
    if (!f) {
        err = "No file " + path;
        return false;
    }
    std::string header;
    std::getline(f, header);
    const size_t n = (size_t)nx * ny * nz;
    mask.assign(n, 0);
    char c;
    for (size_t q = 0; q < n; ++q) {
        if (!(f >> c)) {
            err = path + ": expected " + std::to_string(n) + " cells, found " + std::to_string(q);
            return false;
        }
        mask[q] = (c == '1') ? 1 : 0;  // k outer, j, i inner == [k][j][i]
    }
    return true;
}

namespace {

bool read_faces(const std::string& path, int ni, int nj, int nk, double mult, std::vector<double>& out, int nx_,
                int ny_, double& vmax, double& vmin, std::string& err) {
    // file order: i outer, j, k inner; out: [k][j][i] with the given extents
    std::ifstream f(path);
    if (!f) {
        err = "No file " + path;
        return false;
    }
    std::string header;
    std::getline(f, header);
    out.assign((size_t)ni * nj * nk, 0.0);
    double v;
    for (int i = 0; i < ni; ++i)
        for (int j = 0; j < nj; ++j)
            for (int k = 0; k < nk; ++k) {
                if (!(f >> v)) {
                    err = path + ": too few values";
                    return false;
                }
                if (vmax < v) vmax = v;
                if (vmin > v) vmin = v;
                out[(size_t)i + (size_t)nx_ * ((size_t)j + (size_t)ny_ * k)] = mult * v;
            }
    return true;
}

}  // namespace

bool read_velocity(const std::string& dir, int nx, int ny, int nz, double vel_mult, std::vector<double>& vx,
                   std::vector<double>& vy, std::vector<double>& vz, double& vmax_raw, double& vmin_raw,
                   std::string& err) {
    vmax_raw = 0.0;
    vmin_raw = 0.0;
    if (!read_faces(dir + "/Vx.dat", nx + 1, ny, nz, vel_mult, vx, nx + 1, ny, vmax_raw, vmin_raw, err)) return false;
    if (!read_faces(dir + "/Vy.dat", nx, ny + 1, nz, vel_mult, vy, nx, ny + 1, vmax_raw, vmin_raw, err)) return false;
    if (!read_faces(dir + "/Vz.dat", nx, ny, nz + 1, vel_mult, vz, nx, ny, vmax_raw, vmin_raw, err)) return false;
    return true;
}

bool read_surfrel(const std::string& dir, const std::string& key, int nx, int ny, int nz, std::vector<double>& fx,
                  std::vector<double>& fy, std::vector<double>& fz, std::string& err) {
    double hi = 0.0, lo = 0.0;
    const std::string p = dir + "/SurfRel" + key;
    if (!read_faces(p + "X.dat", nx + 1, ny, nz, 1.0, fx, nx + 1, ny, hi, lo, err)) return false;
    if (!read_faces(p + "Y.dat", nx, ny + 1, nz, 1.0, fy, nx, ny + 1, hi, lo, err)) return false;
    if (!read_faces(p + "Z.dat", nx, ny, nz + 1, 1.0, fz, nx, ny, hi, lo, err)) return false;
    return true;
}

bool read_n1(const std::string& path, int nx, int ny, int nz, std::vector<double>& n1, std::string& err) {
    std::ifstream f(path);
    if (!f) {
        err = "No file " + path;
        return false;
    }
    std::string header;
    std::getline(f, header);
    n1.assign((size_t)nx * ny * nz, 0.0);
    float v;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                if (!(f >> v)) {
                    err = path + ": too few values";
                    return false;
                }
                n1[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)] = v;
            }
    return true;
}

}  // namespace nmr
