// Runs the reference's own DCD writer (src/dcdio.cpp, compiled from the
// reference tree) on given coordinates: TEST INFRASTRUCTURE ONLY.
//   ref_dcd <out.dcd> <N> <nfile> <npriv> <nsavc> <delta> <frames.bin>
// frames.bin holds F frames of X[N], Y[N], Z[N] float32.  remark2 is replaced
// by a fixed string (the reference puts the date there).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "dcdio.h"

int main(int argc, char **argv) {
    if (argc != 8) return 2;
    const int N = std::atoi(argv[2]);
    DCD dcd;
    createDCD(&dcd, N, std::atoi(argv[3]), std::atoi(argv[4]), (float)std::atof(argv[6]), std::atoi(argv[5]), 0, 0, 0,
              0);
    std::memset(dcd.header.remark2, 0, sizeof dcd.header.remark2);
    std::snprintf(dcd.header.remark2, sizeof dcd.header.remark2, "REMARKS FIXED FOR COMPARISON");
    dcdOpenWrite(&dcd, argv[1]);
    dcdWriteHeader(dcd);
    dcdClose(dcd);
    FILE *in = std::fopen(argv[7], "rb");
    if (!in) return 3;
    std::vector<float> buf(3 * (size_t)N);
    while (std::fread(buf.data(), sizeof(float), buf.size(), in) == buf.size()) {
        std::memcpy(dcd.frame.X, buf.data(), sizeof(float) * N);
        std::memcpy(dcd.frame.Y, buf.data() + N, sizeof(float) * N);
        std::memcpy(dcd.frame.Z, buf.data() + 2 * N, sizeof(float) * N);
        dcdOpenAppend(&dcd, argv[1]);
        dcdWriteFrame(dcd);
        dcdClose(dcd);
    }
    std::fclose(in);
    return 0;
}
