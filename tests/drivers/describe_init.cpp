// Test driver: runs the drop-in NmrRelaxationSolve::init() in a case directory
// (no GPU needed) and prints what it derived.
//   describe_init <case dir> [gx gy gz]
#include <unistd.h>

#include <cstdlib>
#include <iostream>

#include "NmrRelaxationSolve.h"

int main(int argc, char** argv) {
    if (argc < 2 || chdir(argv[1]) != 0) return 2;
    int num[3] = {1, 1, 1};
    for (int a = 0; a < 3 && 2 + a < argc; ++a) num[a] = std::atoi(argv[2 + a]);
    NmrRelaxationSolve s(1, 0, num);
    s.init();
    std::cout << "BEGIN-DESCRIBE\n" << s.describe();
    return 0;
}
