// Test driver: runs the drop-in NmrRelaxationSolve::init() in a case directory
// (no GPU needed) and prints what it derived.
//   describe_init <case dir> [--fields out.bin] [gx gy gz]
// --fields writes the per-voxel T1, T2, D, c1, c2 that init() formed (5 x N
// doubles, [k][j][i]; empty arrays when the case needs none).
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

// test access to the class's per-voxel arrays
#define private public
#include "NmrRelaxationSolve.h"
#undef private

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    std::string fields_out;
    int a = 2;
    if (argc >= 4 && std::strcmp(argv[2], "--fields") == 0) {
        fields_out = argv[3];
        if (fields_out[0] != '/') {
            char cwd[4096];
            if (!getcwd(cwd, sizeof(cwd))) return 2;
            fields_out = std::string(cwd) + "/" + fields_out;
        }
        a = 4;
    }
    if (chdir(argv[1]) != 0) return 2;
    int num[3] = {1, 1, 1};
    for (int q = 0; q < 3 && a + q < argc; ++q) num[q] = std::atoi(argv[a + q]);
    NmrRelaxationSolve s(1, 0, num);
    s.init();
    if (!fields_out.empty()) {
        FILE* f = std::fopen(fields_out.c_str(), "wb");
        if (!f) return 3;
        for (const std::vector<double>* v : {&s.t1_, &s.t2_, &s.diff_, &s.c1_, &s.c2_})
            if (!v->empty()) std::fwrite(v->data(), sizeof(double), v->size(), f);
        std::fclose(f);
    }
    std::cout << "BEGIN-DESCRIBE\n" << s.describe();
    return 0;
}
