// shapes.cuh — the reference's free-form initial lattices, built on the host
// directly in the compact one-byte-per-diamond-site layout (lattice.cuh):
// SetNC / SetNCSp (a 3C parallelepiped or ball), SetInvPOff (inverted
// pyramids in a 3C layer), SetSiFINFET (Si between walls), SetTrenchSi (a Si
// trench under a temperature gradient) and SetCAD (a geometry file).  Each
// writes occupancy, species, walls and the coordinations of its closing
// passes; the list heads and dummy flags of coor-1 sites follow from those
// (as Get_Prob_Ini finds them).  Only diamond sites exist here: the walls'
// off-grid points never neighbour a diamond site.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

#include "lattice.cuh"

namespace mks_shapes {

using mks::WALL;

struct Grid {
    int lx, ly, lz, NA, NB, NZ;
    std::vector<uint8_t> st;   // index (z1 * NB + b) * NA + a
    Grid(int lx_, int ly_, int lz_) : lx(lx_), ly(ly_), lz(lz_), NA(lx_ / 6), NB(ly_ / 6), NZ(lz_ / 3 + 1)
    {
        st.assign((size_t)NZ * NB * NA, 0);
    }
    // the byte of grid point (x, y, z), or nullptr if it is not a diamond site
    uint8_t *at(int x, int y, int z)
    {
        if (x < 0 || y < 0 || z < 0 || x >= lx || y >= ly || z > lz) return nullptr;
        if (x % 3 || y % 3 || z % 3) return nullptr;
        int x1 = x / 3, y1 = y / 3, z1 = z / 3;
        if ((x1 & 1) != (z1 & 1) || (y1 & 1) != (z1 & 1)) return nullptr;
        int a = x1 >> 1, b = y1 >> 1;
        if ((a + b + (z1 >> 1)) & 1) return nullptr;
        return &st[((size_t)z1 * NB + b) * NA + a];
    }
    // neighbour d of site (a, b, z1), periodic in a and b; nullptr outside z
    uint8_t *nb(int a, int b, int z1, int d)
    {
        int da, db, dz;
        mks::nb_off(z1 & 1, d, da, db, dz);
        int zz = z1 + dz;
        if (zz < 0 || zz >= NZ) return nullptr;
        int aa = (a + da + NA) % NA, bb = (b + db + NB) % NB;
        return &st[((size_t)zz * NB + bb) * NA + aa];
    }
};

// sublattice of a diamond grid point: 1 for (x1+y1+z1) mod 4 == 0, 2 for 3
inline int kind_of(int x, int y, int z) { return ((x / 3 + y / 3 + z / 3) % 4 == 0) ? 1 : 2; }

inline bool occupied(uint8_t v) { return v == WALL || (v & 3) != 0; }

// The coordination pass of the closing passes over grid points x in [xa, xb],
// y in [ya, yb], z in [za, zb] (z, y, x order, SetNC.f:62-134 and kin): a
// site's coordination is its occupied neighbours (with walls: an empty site
// does not count wall neighbours, SetSiFINFET.f:120-200); an occupied site
// with none is removed and its neighbours' counts drop by one (floored at 0).
inline void coor_pass(Grid &g, int xa, int xb, int ya, int yb, int za, int zb, bool walls)
{
    for (int z = za; z <= zb; z++) {
        if (z % 3) continue;
        int z1 = z / 3;
        if (z < 0 || z1 >= g.NZ) continue;
        for (int y = ya; y <= yb; y++)
            for (int x = xa; x <= xb; x++) {
                uint8_t *v = g.at((x % g.lx + g.lx) % g.lx, (y % g.ly + g.ly) % g.ly, z);
                if (!v || (x % 3) || (y % 3)) continue;
                if (walls && *v == WALL) continue;
                int a = (int)((v - g.st.data()) % g.NA);
                int b = (int)(((v - g.st.data()) / g.NA) % g.NB);
                bool occ = occupied(*v);
                int coor = 0;
                for (int d = 0; d < 4; d++) {
                    uint8_t *w = g.nb(a, b, z1, d);
                    if (!w || !occupied(*w)) continue;
                    if (occ || !walls || *w != WALL) coor++;
                }
                if (occ && *v != WALL && coor == 0) {
                    *v = 0;
                    for (int d = 0; d < 4; d++) {
                        uint8_t *w = g.nb(a, b, z1, d);
                        if (!w || *w == WALL) continue;
                        int c = mks::co_of(*w) - 1;
                        *w = mks::mk(mks::sp_of(*w), c < 0 ? 0 : c, mks::fd_of(*w), mks::dm_of(*w));
                    }
                } else if (*v != WALL) {
                    *v = mks::mk(mks::sp_of(*v), coor, mks::fd_of(*v), mks::dm_of(*v));
                }
            }
    }
}

inline void fill(Grid &g, int x, int y, int z, int sp)
{
    uint8_t *v = g.at(x, y, z);
    if (v && *v != WALL) *v = mks::mk(sp, mks::co_of(*v), 0, 0);
}

// SetNC (SetNC.f:24-235) or, with sphere, SetNCSp (SetNCSp.f:24-237); with
// all_si as well, SetNCSpSi (SetNCSpSi.f: the ball with Si on both sublattices)
inline void set_nc(Grid &g, int len1, int len2, int len3, bool sphere, bool all_si = false)
{
    int x0 = g.lx / 2 - len1 / 2, x1 = g.lx / 2 + len1 / 2 - 1;
    int y0 = g.ly / 2 - len2 / 2, y1 = g.ly / 2 + len2 / 2 - 1;
    int z0 = g.lz / 2 - len3 / 2, z1 = g.lz / 2 + len3 / 2 - 1;
    for (int z = z0; z <= z1; z++)
        for (int y = y0; y <= y1; y++)
            for (int x = x0; x <= x1; x++) {
                if (!g.at(x, y, z)) continue;
                if (sphere) {
                    long dx = x - g.lx / 2, dy = y - g.ly / 2, dz = z - g.lz / 2;
                    if (dx * dx + dy * dy + dz * dz > (long)len1 * len1 / 4) continue;
                }
                fill(g, x, y, z, all_si ? 1 : kind_of(x, y, z));
            }
    coor_pass(g, x0 - 10, x1 + 10, y0 - 10, y1 + 10, z0 - 10, z1 + 10, false);
}

// SetInvPOff (SetInvPOff.f:22-286), called with (Len1, Len2): pits where
// |x-xc| + |y-yc| - 1.10 (z - Len3) <= Len for the box centre or a corner,
// evaluated in single precision like the reference's default-REAL literal
// The species of the inverted-pyramid family at (x, y) on sublattice k:
// 'I' SetInvPOff (k itself), 'Z' SetInvPSi (Si), 'D' SetInvPC (C), and the
// antiphase domains of 'K' SetInvPwOnlySiorC (sublattices swapped outside
// the quadrants x < LenX/2 <= y and y < LenY/2 <= x), 'L' SetInvPwOnlyCorSi
// (swapped inside them) and 'J' SetInvPwAPB (swapped where x + y > LenY).
inline int invp_species(char mode, int k, int x, int y, int lx, int ly)
{
    if (mode == 'I') return k;
    if (mode == 'Z') return 1;
    if (mode == 'D') return 2;
    bool r = mode == 'J' ? x + y <= ly : ((x < lx / 2 && y >= ly / 2) || (x >= lx / 2 && y < ly / 2));
    if (mode == 'L') r = !r;
    return r ? k : 3 - k;
}

// With mode 'D', 'Z', 'J', 'K' or 'L' the pits have slope 1, tested in
// integers (SetInvPC.f, SetInvPSi.f, SetInvPwAPB.f, SetInvPwOnlySiorC.f,
// SetInvPwOnlyCorSi.f), and the species follow invp_species.
inline void set_invp(Grid &g, int len, int len3, char mode = 'I')
{
    int lenh = g.lx / 2 - 1;
    for (int z = 0; z <= 20; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++) {
                uint8_t *v = g.at(x, y, z);
                if (v) *v = mks::mk(invp_species(mode, kind_of(x, y, z), x, y, g.lx, g.ly), 4, 0, 0);
            }
    const int cx[5] = {lenh, 0, g.lx, 0, g.lx}, cy[5] = {lenh, 0, 0, g.ly, g.ly};
    for (int z = 21; z <= len3 - 1; z++) {
        float dz = 1.10f * (float)(z - len3);
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++) {
                if (!g.at(x, y, z)) continue;
                bool pit = false;
                for (int c = 0; c < 5 && !pit; c++) {
                    int d = std::abs(x - cx[c]) + std::abs(y - cy[c]);
                    pit = mode == 'I' ? (float)d - dz <= (float)len : d - (z - len3) <= len;
                }
                if (!pit) fill(g, x, y, z, invp_species(mode, kind_of(x, y, z), x, y, g.lx, g.ly));
            }
    }
    coor_pass(g, 0, g.lx - 1, 0, g.ly - 1, 21, len3 + 9, false);
}

// SetSiFINFET (SetSiFINFET.f:23-312): walls at z = 0..5 and LenZ-6..LenZ-1, a
// wall layer from Lenwwtop, side walls from Lenww leaving an aperture of
// Laperture around the centre in x; Si below Len
inline void set_finfet(Grid &g, int len, int lenww, int lenwwtop, int lap)
{
    int xl = (int)(0.5f * (float)(g.lx - lap)), xr = (int)(0.5f * (float)(g.lx + lap));
    auto wall = [&](int z, int xa, int xb) {
        for (int y = 0; y < g.ly; y++)
            for (int x = xa; x < xb; x++) {
                uint8_t *v = g.at(x, y, z);
                if (v) *v = WALL;
            }
    };
    for (int z = 0; z <= 5; z++) wall(z, 0, g.lx);
    for (int z = lenww; z <= g.lz - 7; z++) {
        wall(z, 0, xl);
        wall(z, xr, g.lx);
    }
    for (int z = lenwwtop; z <= g.lz - 7; z++) wall(z, 0, g.lx);
    for (int z = g.lz - 6; z <= g.lz - 1; z++) wall(z, 0, g.lx);
    for (int z = 6; z <= len - 1; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++) fill(g, x, y, z, 1);
    coor_pass(g, 0, g.lx - 1, 0, g.ly - 1, 6, lenwwtop + 9, true);
}

// SetTrenchSi (SetTrenchSi.f:22-338): walls at z = 0..3 and LenZ-4..LenZ-1, Si
// bulk at z = 4..20, Si at z = 21..Len3-1 except the trench |x - Lenh| <=
// Len - (Len3 - z) cot(angle), Len2 < z < Len3.  The reference's Pi is a
// REAL(8) set from a default-REAL literal (single precision).  temp[z] gets
// the temperature of layer z.
inline void set_trench(Grid &g, int len, int len2, int len3, double angle, double ttop, double tbottom,
                       std::vector<int> &temp)
{
    const double pi = (double)3.1415926535897932384626433832795028841971f;
    double arad = angle * pi / 180.0;
    int lenh = g.lx / 2 - 1;
    temp.assign((size_t)g.lz + 1, 0);
    for (int z = 0; z <= g.lz; z++)
        temp[z] = z < len3 ? (int)(tbottom + (ttop - tbottom) * z / (len3 - 1)) : (int)ttop;
    for (int z = 0; z <= 3; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++)
                if (uint8_t *v = g.at(x, y, z)) *v = WALL;
    for (int z = g.lz - 4; z <= g.lz - 1; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++)
                if (uint8_t *v = g.at(x, y, z)) *v = WALL;
    for (int z = 4; z <= 20; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++)
                if (uint8_t *v = g.at(x, y, z)) *v = mks::mk(1, 4, 0, 0);
    for (int z = 21; z <= len3 - 1; z++) {
        double half = (double)len - (double)(len3 - z) * std::cos(arad) / std::sin(arad);
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++) {
                if (!g.at(x, y, z)) continue;
                if ((double)std::abs(x - lenh) <= half && z > len2 && z < len3) continue;
                fill(g, x, y, z, 1);
            }
    }
    coor_pass(g, 0, g.lx - 1, 0, g.ly - 1, 21, len3 + 9, false);
}

// SetTrench (SetTrench.f:23-283, InitSt T): the 3C substrate from z = 0 (no
// walls, no temperatures) under a layer z = 21..Len3-1 with a trench of
// vertical sides, |x - Lenh| <= Len for Len2 < z < Len3
inline void set_trench_sic(Grid &g, int len, int len2, int len3)
{
    int lenh = g.lx / 2 - 1;
    for (int z = 0; z <= 20; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++)
                if (uint8_t *v = g.at(x, y, z)) *v = mks::mk(kind_of(x, y, z), 4, 0, 0);
    for (int z = 21; z <= len3 - 1; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++) {
                if (!g.at(x, y, z)) continue;
                if (std::abs(x - lenh) <= len && z > len2 && z < len3) continue;
                fill(g, x, y, z, kind_of(x, y, z));
            }
    coor_pass(g, 0, g.lx - 1, 0, g.ly - 1, 21, len3 + 9, false);
}

// SetSiC3Cww (SetSiC3Cww.f:25-230, InitSt Fw) or, with lap >= 0,
// SetSiC3Cwwaperture (SetSiC3Cwwaperture.f, Fa): the SetSiC3C slab of height
// Len over SetSi's walls (z = 0..5 and LenZ-6..LenZ-1, bulk from z = 6; 3C
// species, surface atoms at Len-3 and the empty layer at Len of coordination
// 2), then walls over z = Lenww..LenZ-7 (leaving x in [INT(0.5 (LenX - lap)),
// INT(0.5 (LenX + lap))) open) written without touching the counts.
inline void set_flat_ww(Grid &g, int len, int lenww, int lap)
{
    for (int z = 0; z <= g.lz; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++) {
                uint8_t *v = g.at(x, y, z);
                if (!v) continue;
                if (z <= 5 || (z >= g.lz - 6 && z <= g.lz - 1)) *v = WALL;
                else if (z <= len - 4) *v = mks::mk(kind_of(x, y, z), 4, 0, 0);
                else if (z <= len - 1) *v = mks::mk(kind_of(x, y, z), 2, 0, 0);
                else if (z == len) *v = mks::mk(0, 2, 0, 0);
            }
    const int xa = lap >= 0 ? (int)(0.5 * (g.lx - lap)) : g.lx, xb = lap >= 0 ? (int)(0.5 * (g.lx + lap)) : g.lx;
    for (int z = lenww; z <= g.lz - 7; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++) {
                if (lap >= 0 && x >= xa && x < xb) continue;
                if (uint8_t *v = g.at(x, y, z)) *v = WALL;
            }
}

// SetCAD for InitSt IN (SetCAD.f:80-341, fresh start): walls at z = 0..3 and
// LenZ-4..LenZ-1; from the geometry id of every grid point (geo[(z * LenY +
// y) * LenX + x], z = 4..LenZ-5): 10 a wall, 1 Si on both sublattices; then
// the coordination pass with the wall rules over the whole box.  The alloy
// draw of SetCAD.f:215-222 uses the compiler's RAND stream; here it is the
// seeded cad_draw (alloy fraction > 0, InitSt IN).
// With la, the Si sites of InitSt LA (SetCAD.f:166-212): kept below
// LenZ - INT((LenVac + LenNuc)/sf) when homogeneous, else outside the ball of
// radius LenNuc/sf around (LenX/2, LenY/2, LenZ - INT(LenVac/sf)).
struct CadLA {
    bool on = false, homogeneous = true;
    double len_vac = 0.0, len_nuc = 0.0, sf = 1.0;
};

// With alloy > 0 (InitSt IN only, SetCAD.f:215-222) each Si site of id 1
// takes species 2 when its draw u < alloy; u is the reference's RAND(), here
// a splitmix64 hash of (seed, grid point).
inline double cad_draw(uint64_t seed, uint64_t k)
{
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (k + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

inline void set_cad(Grid &g, const int8_t *geo, const CadLA &la = CadLA(), double alloy = 0.0, uint64_t seed = 0)
{
    const int zmax = g.lz - (int)((la.len_vac + la.len_nuc) / la.sf);
    const int x0 = g.lx / 2, y0 = g.ly / 2, z0 = g.lz - (int)(la.len_vac / la.sf);
    const long r2 = (long)((la.len_nuc / la.sf) * (la.len_nuc / la.sf));
    for (int z = 0; z < g.lz; z++)
        for (int y = 0; y < g.ly; y++)
            for (int x = 0; x < g.lx; x++) {
                uint8_t *v = g.at(x, y, z);
                if (!v) continue;
                if (z <= 3 || z >= g.lz - 4) {
                    *v = WALL;
                    continue;
                }
                int id = geo[((size_t)z * g.ly + y) * g.lx + x];
                if (id == 10) {
                    *v = WALL;
                } else if (id == 1) {
                    bool occ = true;
                    if (la.on && la.homogeneous) {
                        occ = z <= zmax;
                    } else if (la.on) {
                        long d2 = (long)(x - x0) * (x - x0) + (long)(y - y0) * (y - y0) + (long)(z - z0) * (z - z0);
                        occ = d2 > r2;
                    }
                    if (occ) {
                        int sp = 1;
                        if (alloy > 0.0 && cad_draw(seed, ((uint64_t)z * g.ly + y) * g.lx + x) < alloy) sp = 2;
                        *v = mks::mk(sp, 0, 0, 0);
                    }
                }
            }
    coor_pass(g, 0, g.lx - 1, 0, g.ly - 1, 0, g.lz - 1, true);
}

// The first list entry of every coor-1 empty site is its one occupied
// neighbour that is not a wall (Get_Prob_Ini keeps it as NextN(1)); the site
// is a dummy when that neighbour has coordination < 2, with the rate of
// Get_Prob_Ini.f:89-104 (ini) or of Get_Prob.f:156-184 for the initializers
// that rate their sites with Get_Prob.
inline void list_heads(Grid &g, bool ini)
{
    for (int z1 = 0; z1 < g.NZ; z1++)
        for (int b = 0; b < g.NB; b++)
            for (int a = 0; a < g.NA; a++) {
                if ((a + b + (z1 >> 1)) & 1) continue;
                uint8_t &v = g.st[((size_t)z1 * g.NB + b) * g.NA + a];
                if (v == WALL || (v & 3) || mks::co_of(v) != 1) continue;
                int found = -1;
                uint8_t ns = 0;
                for (int d = 0; d < 4; d++) {
                    uint8_t *w = g.nb(a, b, z1, d);
                    if (w && *w != WALL && (*w & 3)) {
                        found = d;
                        ns = *w;
                    }
                }
                if (found >= 0) v = mks::mk_c1(found, mks::co_of(ns), ini);
            }
}

// SetShape (SetShape.f:25-436, InitSt SH): grid points (x, y, z) with
// species 1 (Si) or 2 (C or Ge), n of them.  A point with z <= 3 or
// z >= LenZ-4 is a wall (:58-62), any other an atom, which must sit on a
// diamond site.  An atom's coordination counts its occupied neighbours,
// walls included, and its first list entry is the first of them in the
// reference's shell scan, dz then dy then dx ascending (:87-131); with
// coordination <= 3 it is an MC particle.  An empty site counts its MC
// neighbours only, and its first list entry is the first of those in z, y, x
// order, the order of the MC list (:378-431).  Returns nullptr, or what in
// the input the reference leaves undefined or this lattice cannot hold: an
// atom off the diamond sites or next to an off-site wall point, an atom with
// fewer than two neighbours, an MC particle next to a wall or a bulk atom
// above z = 12 next to one (the reference's reciprocity checks, :277-373,
// then read the list entry 0), an empty site with four MC neighbours.
inline const char *set_points(Grid &g, const int32_t *xyz, const int8_t *sp, int64_t n)
{
    std::vector<int64_t> offsite;
    for (int64_t i = 0; i < n; i++) {
        const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        if (x < 0 || x >= g.lx || y < 0 || y >= g.ly || z < 0 || z > g.lz) return "a point outside the box";
        uint8_t *v = g.at(x, y, z);
        if (z <= 3 || z >= g.lz - 4) {
            if (v) *v = WALL;
            else offsite.push_back(i);
            continue;
        }
        if (!v) return "an atom off the diamond sites";
        if (sp[i] != 1 && sp[i] != 2) return "an atom symbol other than Si, C or Ge";
        *v = mks::mk(mks::sp_of(*v) | sp[i], 0, 0, 0);
    }
    // an off-site wall point within an atom's |d|^2 = 27 shell (the 32
    // offsets of SetShape.f:87-99) would count as a neighbour the one-byte
    // lattice cannot list
    int shell[32][3], ns = 0;
    for (int k = -5; k <= 5; k++)
        for (int j = -5; j <= 5; j++)
            for (int l = -5; l <= 5; l++)
                if (l * l + j * j + k * k == 27) {
                    shell[ns][0] = l;
                    shell[ns][1] = j;
                    shell[ns][2] = k;
                    ns++;
                }
    for (int64_t i : offsite)
        for (int q = 0; q < ns; q++) {
            const int z = xyz[3 * i + 2] + shell[q][2];
            if (z < 4 || z > g.lz - 5) continue;
            uint8_t *v = g.at(((xyz[3 * i] + shell[q][0]) % g.lx + g.lx) % g.lx,
                              ((xyz[3 * i + 1] + shell[q][1]) % g.ly + g.ly) % g.ly, z);
            if (v && *v != WALL && occupied(*v)) return "an atom next to an off-site wall point";
        }
    auto is_atom = [](uint8_t v) { return v != WALL && (v & 3) != 0; };
    for (int z1 = 0; z1 < g.NZ; z1++)
        for (int b = 0; b < g.NB; b++)
            for (int a = 0; a < g.NA; a++) {
                if ((a + b + (z1 >> 1)) & 1) continue;
                uint8_t &v = g.st[((size_t)z1 * g.NB + b) * g.NA + a];
                if (!is_atom(v)) continue;
                int coor = 0, first = -1, best = 1 << 30;
                bool wall = false;
                for (int d = 0; d < 4; d++) {
                    uint8_t *w = g.nb(a, b, z1, d);
                    if (!w || !occupied(*w)) continue;
                    int da, db, dz;
                    mks::nb_off(z1 & 1, d, da, db, dz);
                    const int par = ((z1 + dz) & 1) - (z1 & 1);
                    const int ox = 3 * (2 * da + par), oy = 3 * (2 * db + par), oz = 3 * dz;
                    const int key = ((oz + 6) * 13 + oy + 6) * 13 + ox + 6;
                    if (key < best) {
                        best = key;
                        first = d;
                    }
                    coor++;
                    wall |= *w == WALL;
                }
                if (coor < 2) return "an atom with fewer than two neighbours";
                if (wall && (coor <= 3 || 3 * z1 >= 13)) return "a reciprocity check that meets a wall";
                v = mks::mk(mks::sp_of(v), coor, first, 0);
            }
    for (int z1 = 0; z1 < g.NZ; z1++)
        for (int b = 0; b < g.NB; b++)
            for (int a = 0; a < g.NA; a++) {
                if ((a + b + (z1 >> 1)) & 1) continue;
                const uint8_t v = g.st[((size_t)z1 * g.NB + b) * g.NA + a];
                if (!is_atom(v) || mks::co_of(v) > 3) continue;
                for (int d = 0; d < 4; d++) {
                    uint8_t *w = g.nb(a, b, z1, d);
                    if (!w || occupied(*w)) continue;
                    const int c = mks::co_of(*w);
                    if (c == 3) return "an empty site with four MC neighbours";
                    *w = mks::mk(0, c + 1, c == 0 ? mks::rev_dir(d) : mks::fd_of(*w), 0);
                }
            }
    list_heads(g, true);     // the ad-voids are rated by Get_Prob_Ini (SetShape.f:378-431)
    return nullptr;
}

// Does the shaped initializer rate its sites with Get_Prob_Ini (SetNC,
// SetNCSp(Si), SetInvP*, SetTrench(Si), SetSiFINFET) rather than Get_Prob
// (SetSiC3Cww, SetSiC3Cwwaperture)?
inline bool ini_rates(const std::string &kind) { return kind != "Fw" && kind != "Fa"; }

// The shaped initializers by InitSt (main.f:224-278): lens are Len1..Len4 as
// start.dat gives them, params the angle, Ttop and Tbottom of "ST" (whose
// temperatures per layer z go to temp).  Returns 0, or 1 for lengths that do
// not fit the box, 2 for an InitSt without a shape here or an input the
// reference would leave inconsistent, with the reason in msg.
inline int build_shape(Grid &g, const std::string &kind, const int32_t *lens, const double *params,
                       std::vector<int> &temp, char *msg, size_t cap)
{
    const int lx = g.lx, ly = g.ly, lz = g.lz;
    auto within = [&](int v, int lo, int hi) { return v >= lo && v <= hi; };
    auto err = [&](int code, const char *fmt, auto... a) {
        snprintf(msg, cap, fmt, a...);
        return code;
    };
    if (kind == "C") {                                        // main.f:261-262
        if (!within(lens[0], 1, lx - 24) || !within(lens[1], 1, ly - 24) || !within(lens[2], 1, lz - 24))
            return err(1, "SetNC lengths %d %d %d do not fit the box", lens[0], lens[1], lens[2]);
        set_nc(g, lens[0], lens[1], lens[2], false);
    } else if (kind == "S" || kind == "SS") {                 // main.f:257-260: SetNCSp, SetNCSpSi
        if (!within(lens[0], 1, std::min(std::min(lx, ly), lz) - 24)) return err(1, "SetNCSp length %d", lens[0]);
        set_nc(g, lens[0], lens[0], lens[0], true, kind == "SS");
    } else if (kind.size() == 1 && std::string("IDZJKL").find(kind[0]) != std::string::npos) {
        // main.f:245-256: SetInvPOff, SetInvPC, SetInvPSi, SetInvPwAPB,
        // SetInvPwOnlySiorC, SetInvPwOnlyCorSi, each called with (Len1, Len2)
        if (!within(lens[1], 24, lz - 12)) return err(1, "SetInvP Len3 %d outside the box", lens[1]);
        set_invp(g, lens[0], lens[1], kind[0]);
    } else if (kind == "T") {                                 // main.f:263-264: SetTrench(Len1, Len2, Len3)
        if (!within(lens[2], 22, lz - 14)) return err(1, "SetTrench Len3 %d outside the box", lens[2]);
        set_trench_sic(g, lens[0], lens[1], lens[2]);
    } else if (kind == "Fw" || kind == "Fa") {                // main.f:228-236, lengths rounded to 24
        int l[3];
        for (int i = 0; i < 3; i++) l[i] = lens[i] - lens[i] % 24;
        if (!within(l[0], 24, lz - 12)) return err(1, "SetSiC3Cww slab height %d", l[0]);
        // the wall block is written after the lists: over a listed site it
        // would leave the reference with a stale list entry
        if (l[1] <= l[0]) return err(2, "SetSiC3Cww wall height %d not above the slab %d", l[1], l[0]);
        if (kind == "Fa" && !within(l[2], 0, lx)) return err(1, "SetSiC3Cwwaperture aperture %d", l[2]);
        set_flat_ww(g, l[0], l[1], kind == "Fa" ? l[2] : -1);
    } else if (kind == "FF") {                                // main.f:273-278
        int l[4];
        for (int i = 0; i < 4; i++) l[i] = lens[i] - lens[i] % 24;
        if (!within(l[0], 6, lz - 7) || !within(l[2], 6, lz - 16)) return err(1, "SetSiFINFET lengths %d %d", l[0], l[2]);
        set_finfet(g, l[0], l[1], l[2], l[3]);
    } else if (kind == "ST") {                                // main.f:265-266
        if (!params) return err(1, "%s", "SetTrenchSi needs angle, Ttop, Tbottom");
        if (!within(lens[2], 22, lz - 14)) return err(1, "SetTrenchSi Len3 %d outside the box", lens[2]);
        set_trench(g, lens[0], lens[1], lens[2], params[0], params[1], params[2], temp);
    } else {
        return err(2, "InitSt %s has no shape initializer", kind.c_str());
    }
    list_heads(g, ini_rates(kind));
    return 0;
}

}  // namespace mks_shapes
