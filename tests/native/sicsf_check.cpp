// The library's SetSiCSF builder (mulskips_gb300/csrc/sicsf.h) compiled for
// the host with a C ABI, so tests/test_shape_points.py can compare its
// LattCoo and lists with the oracle's.
#include <cstring>

#include "../../mulskips_gb300/csrc/sicsf.h"

extern "C" long long sicsf_build(int lx, int ly, int lz, int len, int vx, int vy, int vz, int *lattcoo, int *xyz,
                                 int *nn, int *kind, long long cap, char *msg, int msgcap)
{
    mks_sicsf::Result R;
    const int vsf[3] = {vx, vy, vz};
    const std::string e = mks_sicsf::build(lx, ly, lz, len, vsf, R);
    if (!e.empty()) {
        std::strncpy(msg, e.c_str(), (size_t)msgcap - 1);
        msg[msgcap - 1] = 0;
        return -1;
    }
    std::memcpy(lattcoo, R.lattcoo.data(), sizeof(int) * R.lattcoo.size());
    long long k = 0;
    for (int pass = 0; pass < 2; pass++)
        for (const auto &en : pass == 0 ? R.mc : R.bulk) {
            if (k < cap) {
                for (int c = 0; c < 3; c++) xyz[3 * k + c] = en.xyz[c];
                for (int j = 0; j < 4; j++)
                    for (int c = 0; c < 3; c++) nn[12 * k + 3 * j + c] = en.nn[j][c];
                kind[k] = pass + 1;
            }
            k++;
        }
    return k;
}
