// Test helper: builds an initial lattice twice, with the oracle's list-based
// restatement of the reference's initializer and with the one-byte
// initializers of mulskips_gb300/csrc/shapes.cuh compiled for the host, and
// compares every site byte.  POINTS is the point-list file of InitSt SH
// (mks_shapes::set_points), or @KIND followed by Len1..Len4 for the shaped
// initializers (mks_shapes::build_shape).  Prints "product: ok|<reason>",
// "oracle: ok|<reason>" and, when both built, "mismatch N".  Exit code 0
// when both built identical lattices or both refused the input.
// usage: shape_check START.DAT NUMBERS POINTS|@KIND LX LY LZ [L1 L2 L3 L4]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "../../oracle/mks_oracle.h"
#include "../../mulskips_gb300/csrc/shapes.cuh"

static int compare(mks_shapes::Grid &g, const char *e, const char *startdat, const char *numbers)
{
    printf("product: %s\n", e ? e : "ok");
    ora_t *o = ora_create(startdat, numbers, g.lx, g.ly, g.lz, 0);
    bool ook = o && ora_init(o) == 0;
    printf("oracle: %s\n", ook ? "ok" : ora_last_error());
    if (!e && ook) {
        std::vector<uint8_t> ref(g.st.size());
        if (ora_compact_state(o, ref.data()) != 0) {
            printf("oracle state has sites off the diamond grid\n");
            return 1;
        }
        long long mism = 0, first = -1;
        for (size_t i = 0; i < ref.size(); i++)
            if (ref[i] != g.st[i]) {
                if (first < 0) first = (long long)i;
                mism++;
            }
        printf("mismatch %lld", mism);
        if (first >= 0) printf(" first %lld oracle %02x product %02x", first, ref[first], g.st[first]);
        printf("\n");
        return mism ? 3 : 0;
    }
    return (!e) == ook ? 0 : 4;
}

int main(int argc, char **argv)
{
    if (argc < 7) return 2;
    const int lx = atoi(argv[4]), ly = atoi(argv[5]), lz = atoi(argv[6]);
    mks_shapes::Grid g(lx, ly, lz);
    const char *e = nullptr;
    char msg[160];
    if (argv[3][0] == '@') {
        int32_t lens[4] = {0, 0, 0, 0};
        for (int i = 0; i < 4 && 7 + i < argc; i++) lens[i] = atoi(argv[7 + i]);
        std::vector<int> temp;
        if (mks_shapes::build_shape(g, argv[3] + 1, lens, nullptr, temp, msg, sizeof msg)) e = msg;
        return compare(g, e, argv[1], argv[2]);
    }
    FILE *f = fopen(argv[3], "r");
    if (!f) return 2;
    long long n = 0;
    char line[512];
    if (!fgets(line, sizeof line, f) || sscanf(line, "%lld", &n) != 1 || !fgets(line, sizeof line, f)) return 2;
    std::vector<int32_t> xyz((size_t)n * 3);
    std::vector<int8_t> sp((size_t)n);
    for (long long i = 0; i < n; i++) {
        char sym[64];
        int x, y, z;
        if (!fgets(line, sizeof line, f) || sscanf(line, "%63s %d %d %d", sym, &x, &y, &z) != 4) return 2;
        std::string s(sym, strnlen(sym, 2));
        sp[i] = s == "Si" ? 1 : (s == "C" || s == "Ge") ? 2 : 0;
        xyz[3 * i] = x;
        xyz[3 * i + 1] = y;
        xyz[3 * i + 2] = z;
    }
    fclose(f);
    e = mks_shapes::set_points(g, xyz.data(), sp.data(), n);
    return compare(g, e, argv[1], argv[2]);
}
