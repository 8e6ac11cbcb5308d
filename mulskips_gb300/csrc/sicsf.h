// SetSiCSF (mulskips-source/initial/SetSiCSF.f:7-473, InitSt 'E',
// main.f:267-272): a 3C-SiC (001) slab holding a triangular triple stacking
// fault, built on the host as the reference's LattCoo and its three lists.
// The atoms of the fault sit off the diamond sub-grid, so the state goes to
// the explicit-neighbour engine through mks_load_lists, which rates every
// entry from the final state (Get_Prob with reciprocal bonds, the coor-1
// dummy at the init-time 1e-6): after SetSiCSF's repair passes every atom's
// coordination is its count of reciprocal bonds, so those rates are the ones
// SetSiCSF leaves.  Host code only; no CUDA.
//
// The lists are kept in the reference's order (AddMC / AddBulk append,
// EraseBulk moves the last entry into the hole): the order decides which
// bulk atoms the repair loop visits and which atom is an ad-void's first
// NextN, and NextN order is state (the first entry supports a coor-1 site,
// the last reciprocal one becomes NBuff on evaporation).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

namespace mks_sicsf {

// LattCoo bits (defsystem.f:87-91)
constexpr int POS_OCC = 23, POS_COOR = 24, POS_SI = 27, POS_C = 28;

struct Entry {
    int xyz[3];
    int nn[4][3];
};

struct Result {
    std::vector<int32_t> lattcoo;      // LattCoo(0:LenX-1, 0:LenY-1, 0:LenZ), x fastest
    std::vector<Entry> mc, bulk;       // ListAdAtom(1..), ListAtom(1..) in the reference's order
};

namespace detail {

// one rounding per operation: the stores keep a compiler from fusing a
// product into the following sum
inline double mul(double a, double b)
{
    volatile double r = a * b;
    return r;
}
inline double add(double a, double b)
{
    volatile double r = a + b;
    return r;
}

inline int isign(int a, int b) { return b >= 0 ? std::abs(a) : -std::abs(a); }

// FIND_NN (mulskips-source/lattice/FIND_NN.f:25-77): the two other bond
// partners of sitec given two, by rotating site2 - sitec by 120 and 240
// degrees about the axis sitec - site1; FP64 as the reference, NINT to the
// grid, periodic in x and y
inline void find_nn(const int site1[3], const int site2[3], const int sitec[3], int out[2][3], int lx, int ly)
{
    const double pi = (double)3.14159265358979323f;   // FIND_NN.f:37: a default-REAL literal
    int s11[3] = {site1[0], site1[1], site1[2]}, s22[3] = {site2[0], site2[1], site2[2]};
    if (std::abs(sitec[0] - s11[0]) > lx / 2) s11[0] += isign(lx, sitec[0] - s11[0]);
    if (std::abs(sitec[1] - s11[1]) > ly / 2) s11[1] += isign(ly, sitec[1] - s11[1]);
    if (std::abs(sitec[0] - s22[0]) > lx / 2) s22[0] += isign(lx, sitec[0] - s22[0]);
    if (std::abs(sitec[1] - s22[1]) > ly / 2) s22[1] += isign(ly, sitec[1] - s22[1]);
    double ax[3];
    for (int k = 0; k < 3; k++) ax[k] = (double)sitec[k] - (double)s11[k];
    const double snorm = std::sqrt(add(add(mul(ax[0], ax[0]), mul(ax[1], ax[1])), mul(ax[2], ax[2])));
    for (int k = 0; k < 3; k++) ax[k] = ax[k] / snorm;
    for (int irot = 1; irot <= 2; irot++) {
        const double cth = std::cos((double)(2 * irot) * pi / 3.0);
        const double sth = std::sin((double)(2 * irot) * pi / 3.0);
        const double omc = 1.0 - cth;
        double rot[3][3];   // rot[i][j] = Rot(i+1, j+1)
        for (int i = 0; i < 3; i++) rot[i][i] = add(mul(mul(ax[i], ax[i]), omc), cth);
        rot[1][0] = add(mul(mul(ax[0], ax[1]), omc), -mul(ax[2], sth));
        rot[0][1] = add(mul(mul(ax[0], ax[1]), omc), mul(ax[2], sth));
        rot[2][0] = add(mul(mul(ax[0], ax[2]), omc), mul(ax[1], sth));
        rot[0][2] = add(mul(mul(ax[0], ax[2]), omc), -mul(ax[1], sth));
        rot[2][1] = add(mul(mul(ax[1], ax[2]), omc), -mul(ax[0], sth));
        rot[1][2] = add(mul(mul(ax[1], ax[2]), omc), mul(ax[0], sth));
        for (int k = 0; k < 3; k++) {
            double r = 0.0;
            for (int l = 0; l < 3; l++) r = add(r, mul(rot[l][k], (double)s22[l] - (double)sitec[l]));
            out[irot - 1][k] = (int)std::lround(r) + sitec[k];
        }
        int *ns = out[irot - 1];
        if (ns[0] >= lx) ns[0] -= lx;
        if (ns[0] < 0) ns[0] += lx;
        if (ns[1] >= ly) ns[1] -= ly;
        if (ns[1] < 0) ns[1] += ly;
    }
}

// the sublattice of a diamond site: 1 where (x1+y1+z1) mod 4 = 0 (Si), 2
// where it is 3 (C), 0 off the sites
inline int dia_kind(int x, int y, int z)
{
    if (x % 3 || y % 3 || z % 3) return 0;
    const int x1 = x / 3, y1 = y / 3, z1 = z / 3;
    if ((x1 % 2) != (y1 % 2) || (x1 % 2) != (z1 % 2)) return 0;
    const int m = (x1 + y1 + z1) % 4;
    return m == 0 ? 1 : (m == 3 ? 2 : 0);
}

// JumpDia (defsystem.f:104-105): bonds of a mod-0 site (0..3), a mod-3 site (4..7)
constexpr int JUMP[8][3] = {{3, 3, 3}, {3, -3, -3}, {-3, -3, 3}, {-3, 3, -3},
                            {3, 3, -3}, {3, -3, 3}, {-3, -3, -3}, {-3, 3, 3}};

struct Builder {
    int lx, ly, lz;
    Result &R;
    std::vector<int32_t> ind;       // LattInd up to the layers the routine touches
    int zmax;

    int64_t at(int x, int y, int z) const { return (int64_t)x + (int64_t)lx * ((int64_t)y + (int64_t)ly * z); }
    int32_t &coo(const int p[3]) { return R.lattcoo[(size_t)at(p[0], p[1], p[2])]; }
    int32_t &li(const int p[3]) { return ind[(size_t)at(p[0], p[1], p[2])]; }
    static int bits(int32_t v, int pos, int len) { return (int)(((uint32_t)v >> pos) & ((1u << len) - 1u)); }
    static void setbits(int32_t &v, int val, int pos, int len)
    {
        const uint32_t m = ((1u << len) - 1u) << pos;
        v = (int32_t)(((uint32_t)v & ~m) | (((uint32_t)val << pos) & m));
    }
    void wrap(int p[3]) const
    {
        if (p[0] >= lx) p[0] -= lx;
        if (p[0] < 0) p[0] += lx;
        if (p[1] >= ly) p[1] -= ly;
        if (p[1] < 0) p[1] += ly;
    }
    void neighbours(const int s[3], int first, int nn[4][3]) const
    {
        for (int i = 0; i < 4; i++) {
            for (int k = 0; k < 3; k++) nn[i][k] = s[k] + JUMP[first + i][k];
            wrap(nn[i]);
        }
    }
    void add_mc(const int s[3], const int nn[4][3])
    {
        Entry e;
        for (int k = 0; k < 3; k++) e.xyz[k] = s[k];
        for (int i = 0; i < 4; i++)
            for (int k = 0; k < 3; k++) e.nn[i][k] = nn[i][k];
        R.mc.push_back(e);
        li(s) = (int32_t)R.mc.size();
    }
    void add_bulk(const int s[3], const int nn[4][3])
    {
        Entry e;
        for (int k = 0; k < 3; k++) e.xyz[k] = s[k];
        for (int i = 0; i < 4; i++)
            for (int k = 0; k < 3; k++) e.nn[i][k] = nn[i][k];
        R.bulk.push_back(e);
        li(s) = (int32_t)R.bulk.size();
    }
    // EraseBulk (Erase.f:82-127): the last entry fills the hole
    void erase_bulk(const int s[3])
    {
        const int i = li(s);
        const int last = (int)R.bulk.size();
        if (i != last) {
            R.bulk[(size_t)i - 1] = R.bulk[(size_t)last - 1];
            li(R.bulk[(size_t)i - 1].xyz) = i;
        }
        R.bulk.pop_back();
        li(s) = 0;
    }
    void set_atom(int x, int y, int z, int kind)
    {
        int32_t &v = R.lattcoo[(size_t)at(x, y, z)];
        v = (int32_t)((uint32_t)v | (1u << (kind == 1 ? POS_SI : POS_C)) | (1u << POS_OCC));
    }
};

}  // namespace detail

// Returns an empty string, or the reference's own stop message.
inline std::string build(int lx, int ly, int lz, int len, const int vsf[3], Result &R)
{
    using namespace detail;
    const int box_sf = len - vsf[2];
    int shell[32][3], ns = 0;                         // ListNN (:24-35): k outer, i inner
    for (int k = -6; k <= 6; k++)
        for (int j = -6; j <= 6; j++)
            for (int i = -6; i <= 6; i++)
                if (i * i + j * j + k * k == 27) {
                    shell[ns][0] = i;
                    shell[ns][1] = j;
                    shell[ns][2] = k;
                    ns++;
                }
    if (vsf[0] + box_sf > lx || vsf[1] + box_sf > ly || box_sf <= 0) return "error SF dimension is not correctly set";
    if (dia_kind(vsf[0], vsf[1], vsf[2]) != 1) return "SF Vertex position in wrong Site";
    if (len + 9 > lz) return "SetSiCSF reads up to z = Len + 9: LenZ too small";
    R.lattcoo.assign((size_t)lx * ly * (lz + 1), 0);
    R.mc.clear();
    R.bulk.clear();
    Builder B{lx, ly, lz, R, {}, len + 9};
    B.ind.assign((size_t)lx * ly * (B.zmax + 1), 0);
    int site[3], nextn[4][3];
    // :56-107: bulk 3C for z = 0..12
    for (int z = 0; z <= 12; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                const int k = dia_kind(x, y, z);
                if (!k) continue;
                B.set_atom(x, y, z, k);
                site[0] = x;
                site[1] = y;
                site[2] = z;
                Builder::setbits(B.coo(site), 4, POS_COOR, 3);
                B.neighbours(site, k == 1 ? 0 : 4, nextn);
                B.add_bulk(site, nextn);
            }
    // :109-163: z = 13..Len-1, the atoms of two {111} planes per sublattice
    // shifted by (+2, +2, +4) and (-2, -2, -4) inside the fault's region
    for (int z = 13; z <= len - 1; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                const int k = dia_kind(x, y, z);
                if (!k) continue;
                const bool inside = x >= vsf[0] && y >= vsf[1] && z >= vsf[2];
                const int d = (x - vsf[0]) + (y - vsf[1]) - (z - vsf[2]);
                const int p1 = inside ? d - (k == 1 ? 12 : 3) : -1;
                const int p2 = inside ? d - (k == 1 ? 24 : 15) : -1;
                if (p1 == 0) {
                    if (x + 2 < lx && y + 2 < ly && z + 4 < len) B.set_atom(x + 2, y + 2, z + 4, k);
                } else if (p2 == 0) {
                    if (x - 2 > 0 && y - 2 > 0 && z - 4 > 0) B.set_atom(x - 2, y - 2, z - 4, k);
                } else {
                    B.set_atom(x, y, z, k);
                }
            }
    // :166-332: two scans of z = 13..Len+6 -- the first empties atoms with
    // fewer than two neighbours, the second sets coordinations and lists
    int nd[32][3];
    for (int pass = 0; pass < 2; pass++)
        for (int z = 13; z <= len + 6; z++)
            for (int y = 0; y < ly; y++)
                for (int x = 0; x < lx; x++) {
                    int32_t &v = R.lattcoo[(size_t)B.at(x, y, z)];
                    if (!Builder::bits(v, POS_OCC, 1)) continue;
                    site[0] = x;
                    site[1] = y;
                    site[2] = z;
                    const int sic = ((x / 3 + y / 3 + z / 3) % 4 == 3) ? 4 : 0;
                    B.neighbours(site, sic, nextn);
                    int coor = 0, coord = 0, j = 0;
                    for (int i = 0; i < 4; i++)
                        if (Builder::bits(B.coo(nextn[i]), POS_OCC, 1)) coor++;
                    if (coor < 2) {
                        for (int i = 0; i < ns; i++) {
                            int q[3] = {x + shell[i][0], y + shell[i][1], z + shell[i][2]};
                            B.wrap(q);
                            if (Builder::bits(B.coo(q), POS_OCC, 1)) {
                                coord++;
                                for (int k = 0; k < 3; k++) nd[j][k] = q[k];
                                j++;
                            }
                        }
                        if (j > 4) return "SetSiCSF: an atom with more than four shell neighbours";
                    }
                    if (pass == 0) {
                        if (coord > coor) {
                            if (coord <= 1) v = 0;
                        } else if (coor <= 1) {
                            v = 0;
                        }
                        continue;
                    }
                    if (coord > coor) {
                        Builder::setbits(v, coord, POS_COOR, 3);
                        int nn4[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                        for (int i = 0; i < j && i < 4; i++)
                            for (int k = 0; k < 3; k++) nn4[i][k] = nd[i][k];
                        if (coord <= 3) {
                            int ns2[2][3];
                            find_nn(nn4[0], nn4[1], site, ns2, lx, ly);
                            for (int k = 0; k < 3; k++) {
                                nn4[2][k] = ns2[0][k];
                                nn4[3][k] = ns2[1][k];
                            }
                            B.add_mc(site, nn4);
                        } else {
                            B.add_bulk(site, nn4);
                        }
                    } else {
                        Builder::setbits(v, coor, POS_COOR, 3);
                        if (coor <= 3) B.add_mc(site, nextn);
                        else B.add_bulk(site, nextn);
                    }
                }
    // :336-427: coordinations cut to reciprocal bonds, MC atoms first, then
    // bulk atoms of z >= 13 (one that changes becomes MC); the bulk loop runs
    // over the count at its start, as the Fortran DO does
    for (int kind = 0; kind < 2; kind++) {
        const size_t n0 = kind == 0 ? R.mc.size() : R.bulk.size();
        for (size_t i = 0; i < n0; i++) {
            Entry e;
            if (kind == 0) {
                e = R.mc[i];
            } else {
                if (i >= R.bulk.size()) continue;     // an entry EraseBulk zeroed: z = 0
                e = R.bulk[i];
                if (e.xyz[2] < 13) continue;
            }
            int32_t &v = B.coo(e.xyz);
            int coor = Builder::bits(v, POS_COOR, 3);
            const int coor_old = coor;
            for (int jn = 0; jn < 4; jn++) {
                const int32_t w = B.coo(e.nn[jn]);
                if (!Builder::bits(w, POS_OCC, 1)) continue;
                const int ind_nn = B.li(e.nn[jn]);
                const bool in_bulk = Builder::bits(w, POS_COOR, 3) == 4;
                if (ind_nn <= 0 || (size_t)ind_nn > (in_bulk ? R.bulk.size() : R.mc.size()))
                    return "SetSiCSF: a bonded atom without a list entry";
                const Entry &b = in_bulk ? R.bulk[(size_t)ind_nn - 1] : R.mc[(size_t)ind_nn - 1];
                bool recip = false;
                for (int kk = 0; kk < 4; kk++)
                    recip |= b.nn[kk][0] == e.xyz[0] && b.nn[kk][1] == e.xyz[1] && b.nn[kk][2] == e.xyz[2];
                if (!recip) coor--;
            }
            if (coor == coor_old) continue;
            Builder::setbits(v, coor, POS_COOR, 3);
            if (kind == 1) {
                B.erase_bulk(e.xyz);
                B.add_mc(e.xyz, e.nn);
            }
        }
    }
    // :429-471: the ad-voids of every MC atom's NextN
    const size_t nmc_old = R.mc.size();
    for (size_t i = 0; i < nmc_old; i++) {
        const Entry a = R.mc[i];
        for (int jn = 0; jn < 4; jn++) {
            const int *s = a.nn[jn];
            int32_t &v = B.coo(s);
            if (Builder::bits(v, POS_OCC, 1)) continue;
            const int coor = Builder::bits(v, POS_COOR, 3) + 1;
            if (coor == 1) {
                int nn4[4][3] = {{a.xyz[0], a.xyz[1], a.xyz[2]}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                Builder::setbits(v, coor, POS_COOR, 3);
                B.add_mc(s, nn4);
            } else if (coor == 2) {
                Entry &m = R.mc[(size_t)B.li(s) - 1];
                for (int k = 0; k < 3; k++) m.nn[1][k] = a.xyz[k];
                int ns2[2][3];
                find_nn(m.nn[0], m.nn[1], s, ns2, lx, ly);
                for (int k = 0; k < 3; k++) {
                    m.nn[2][k] = ns2[0][k];
                    m.nn[3][k] = ns2[1][k];
                }
                Builder::setbits(v, coor, POS_COOR, 3);
            } else if (coor == 3) {
                Builder::setbits(v, coor, POS_COOR, 3);
            } else {
                return "Vacancy in the SF setting";
            }
        }
    }
    return "";
}

}  // namespace mks_sicsf
