// lattice.cuh — compact diamond-site lattice: geometry, one-byte site state,
// event rules and rate classes of the MulSKIPS KMC, for GB300 kernels.
//
// The reference stores every point of an a/12 super-lattice as an int32 bit
// field (LattCoo, mulskips-source/modules/defsystem.f:49,87-91) plus, per
// listed site, four neighbour coordinates (NextNXYZ, defdertype.f:32-37).
// With cubic (zig-zag) stacking only — which is what the reference produces
// whenever PtransZig = 1 (IF_Arm_Choice.f:42-54: arm-chair wins only on a
// strictly larger coordination sum, and arm-chair sites are off the diamond
// sub-grid, so their coordination stays 0) — every site is a diamond site and
// every neighbour list is a permutation of the four bond directions.  The
// whole per-site state the dynamics reads then fits in one byte:
//
//   bits 0-1  species (0 empty, 1..3 = ListCrystal index)      LattCoo bits 27-29
//   bits 2-4  coordination 0..4                                LattCoo bits 24-26
//   bits 5-6  direction of the first NextNXYZ entry            NextNXYZ(:,1)
//   bit  7    dummy-rate flag of an unsupported coor-1 empty site
//             (Get_Prob.f:181-184); with species 0 and coordination 0 the
//             value 0x80 marks a wall site (CovInd 113, SetSi.f:38-46)
//
// Site (a, b, z1) sits at grid point x = 3(2a + (z1&1)), y = 3(2b + (z1&1)),
// z = 3 z1 and exists when (a + b + (z1 >> 1)) is even.  Even layers hold the
// (x1+y1+z1) mod 4 == 0 sublattice (JumpDia columns 1-4), odd layers the
// == 3 sublattice (columns 5-8), defsystem.f:104-105.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define MKS_HD __host__ __device__ __forceinline__
#else
#define MKS_HD static inline
#endif

namespace mks {

// ---- state byte ----
constexpr uint8_t WALL = 0x80;
MKS_HD int sp_of(uint8_t s) { return s & 3; }
MKS_HD int co_of(uint8_t s) { return (s >> 2) & 7; }
MKS_HD int fd_of(uint8_t s) { return (s >> 5) & 3; }
MKS_HD int dm_of(uint8_t s) { return (s >> 7) & 1; }
MKS_HD bool is_wall(uint8_t s) { return s == WALL; }
MKS_HD bool is_occ(uint8_t s) { return s == WALL || (s & 3) != 0; }
MKS_HD uint8_t mk(int sp, int co, int fd, int dm)
{
    return (uint8_t)((sp & 3) | ((co & 7) << 2) | ((fd & 3) << 5) | ((dm & 1) << 7));
}

// ---- geometry ----
// Neighbour offsets (da, db, dz1) of bond direction d for even / odd layers;
// direction d is JumpDia column d+1 (even) or d+5 (odd).  The reverse bond of
// direction d is direction (d + 2) & 3 on the other sublattice.
MKS_HD void nb_off(int zpar, int d, int &da, int &db, int &dz)
{
    // even layer: (0,0,+1) (0,-1,-1) (-1,-1,+1) (-1,0,-1)
    // odd  layer: (+1,+1,-1) (+1,0,+1) (0,0,-1) (0,+1,+1)
    const int8_t t[2][4][3] = {{{0, 0, 1}, {0, -1, -1}, {-1, -1, 1}, {-1, 0, -1}},
                               {{1, 1, -1}, {1, 0, 1}, {0, 0, -1}, {0, 1, 1}}};
    da = t[zpar][d][0];
    db = t[zpar][d][1];
    dz = t[zpar][d][2];
}
MKS_HD int rev_dir(int d) { return (d + 2) & 3; }

// ---- rate classes ----
// 0 none (bulk, void, wall, untracked empty), 1 empty coor-1, 2 empty coor-1
// dummy, 3 empty coor-2, 4 empty coor-3, 5 isolated atom, 6.. occupied
// species sp with reciprocal-neighbour census (nSi+nWall, nC, nB) summing to
// 1..3 (the PTransE key of Get_Prob.f:309-321 without coverage).
constexpr int CLS_NONE = 0, CLS_C1 = 1, CLS_C1D = 2, CLS_C2 = 3, CLS_C3 = 4, CLS_ISO = 5, CLS_OCC0 = 6;
constexpr int NCENSUS = 19;
constexpr int NCLASS = CLS_OCC0 + 3 * NCENSUS;   // 63

MKS_HD int census_index(int n1, int n2, int n3)
{
    // enumerate (n1,n2,n3), 1 <= n1+n2+n3 <= 3, ordered by total then n1 desc, n2 desc
    int t = n1 + n2 + n3;
    int base = (t == 1) ? 0 : (t == 2) ? 3 : 9;
    // index within the simplex of total t: position of (n1,n2) among pairs with n1+n2 <= t
    int k = 0;
    for (int a = t; a > n1; a--) k += (t - a) + 1;
    k += (t - n1) - n2;
    return base + k;
}

// Accessor concept: uint8_t get(int a, int b, int z) const; void put(int a, int b, int z, uint8_t v);
// with periodic wrap in a, b handled by the accessor and 0 outside the z range.

// Class of the site (a,b,z): Get_Prob's branch selection (Get_Prob.f:151-323)
// restated for the one-byte state.
template <class L>
MKS_HD int site_class(const L &lat, int a, int b, int z)
{
    uint8_t s = lat.get(a, b, z);
    if (s == 0 || s == WALL) return CLS_NONE;
    int sp = sp_of(s), co = co_of(s);
    if (sp == 0) {
        if (co == 1) return dm_of(s) ? CLS_C1D : CLS_C1;
        if (co == 2) return CLS_C2;
        if (co == 3) return CLS_C3;
        return CLS_NONE;
    }
    if (co >= 4) return CLS_NONE;
    int n[4] = {0, 0, 0, 0};
    int zp = z & 1;
    for (int d = 0; d < 4; d++) {
        int da, db, dz;
        nb_off(zp, d, da, db, dz);
        uint8_t t = lat.get(a + da, b + db, z + dz);
        if (t == WALL) n[1]++;
        else n[sp_of(t)]++;
    }
    int tot = n[1] + n[2] + n[3];
    if (tot == 0) return CLS_ISO;
    if (tot > 3) return CLS_NONE;
    return CLS_OCC0 + (sp - 1) * NCENSUS + census_index(n[1], n[2], n[3]);
}

// Direction of the unique occupied non-wall neighbour (the NBuff of
// Evaporation.f:87-104,238-253); -1 if there is none.
template <class L>
MKS_HD int occupied_dir(const L &lat, int a, int b, int z)
{
    int r = -1, zp = z & 1;
    for (int d = 0; d < 4; d++) {
        int da, db, dz;
        nb_off(zp, d, da, db, dz);
        uint8_t t = lat.get(a + da, b + db, z + dz);
        if (t != WALL && sp_of(t) != 0 && co_of(t) <= 3) r = d;
    }
    return r;
}

struct Touched {            // sites whose class may have changed
    int n;
    int a[5], b[5], z[5];
};

// Deposition of species sp on the empty site (a,b,z), deposition.f:24-251.
// Returns 0, or a nonzero code when the state contradicts the cubic model.
template <class L>
MKS_HD int apply_deposition(L &lat, int a, int b, int z, int sp, Touched &tc)
{
    uint8_t sx = lat.get(a, b, z);
    if (sp_of(sx) != 0 || sx == WALL) return 1;
    int c_old = co_of(sx), fdx = fd_of(sx);
    // occupancy and species are set first; the coordination bits keep the
    // empty-site value until the end (deposition.f:43-46,237)
    lat.put(a, b, z, mk(sp, c_old, fdx, 0));
    int walls = 0, zp = z & 1;
    tc.n = 1;
    tc.a[0] = a; tc.b[0] = b; tc.z[0] = z;
    for (int d = 0; d < 4; d++) {
        int da, db, dz;
        nb_off(zp, d, da, db, dz);
        int ya = a + da, yb = b + db, yz = z + dz;
        uint8_t sy = lat.get(ya, yb, yz);
        tc.a[tc.n] = ya; tc.b[tc.n] = yb; tc.z[tc.n] = yz; tc.n++;
        if (sy == WALL) { walls++; continue; }
        int cy = co_of(sy);
        if (sp_of(sy) != 0) {                  // occupied neighbour, :192-230
            if (cy <= 3) lat.put(ya, yb, yz, mk(sp_of(sy), cy + 1, fd_of(sy), 0));
        } else if (cy == 0) {                  // new coor-1 MC site, :86-99
            // Get_Prob checks the coordination bits of its single neighbour,
            // i.e. of this site before its own update (Get_Prob.f:156-158)
            lat.put(ya, yb, yz, mk(0, 1, rev_dir(d), c_old < 2 ? 1 : 0));
        } else if (cy == 1) {                  // coor 1 -> 2 with FIND_NN, :100-160
            int cnt = 0, yzp = yz & 1;
            for (int e = 0; e < 4; e++) {
                int ea, eb, ez;
                nb_off(yzp, e, ea, eb, ez);
                uint8_t t = lat.get(ya + ea, yb + eb, yz + ez);
                if (t != WALL && sp_of(t) != 0) cnt++;
            }
            if (cnt < 2) return 2;
            lat.put(ya, yb, yz, mk(0, cnt, fd_of(sy), 0));
        } else if (cy == 2 || cy == 3) {       // :161-191
            lat.put(ya, yb, yz, mk(0, cy + 1, fd_of(sy), 0));
        }
    }
    lat.put(a, b, z, mk(sp, c_old + walls, fdx, 0));
    return 0;
}

// Evaporation of the atom at (a,b,z), Evaporation.f:25-262.
template <class L>
MKS_HD int apply_evaporation(L &lat, int a, int b, int z, Touched &tc)
{
    uint8_t sx = lat.get(a, b, z);
    if (sp_of(sx) == 0 || sx == WALL) return 1;
    int c_atom = co_of(sx), fdx = fd_of(sx);
    // occupancy cleared first, coordination bits kept until the end (:40-44,218)
    lat.put(a, b, z, mk(0, c_atom, fdx, 0));
    int walls = 0, zp = z & 1;
    tc.n = 1;
    tc.a[0] = a; tc.b[0] = b; tc.z[0] = z;
    for (int d = 0; d < 4; d++) {
        int da, db, dz;
        nb_off(zp, d, da, db, dz);
        int ya = a + da, yb = b + db, yz = z + dz;
        uint8_t sy = lat.get(ya, yb, yz);
        tc.a[tc.n] = ya; tc.b[tc.n] = yb; tc.z[tc.n] = yz; tc.n++;
        if (sy == WALL) { walls++; continue; }
        int cy = co_of(sy);
        if (sp_of(sy) != 0) {                  // :166-210
            if (cy >= 1) lat.put(ya, yb, yz, mk(sp_of(sy), cy - 1, fd_of(sy), 0));
            else return 3;
        } else if (cy == 1) {                  // :51-68, reciprocal only
            if (fd_of(sy) == rev_dir(d)) lat.put(ya, yb, yz, 0);
        } else if (cy == 2) {                  // :69-123
            // the rate check reads the first entry of the list before pruning
            int f = fd_of(sy), fa, fb, fz;
            nb_off(yz & 1, f, fa, fb, fz);
            uint8_t sf = lat.get(ya + fa, yb + fb, yz + fz);
            int w = occupied_dir(lat, ya, yb, yz);
            if (w < 0) return 4;
            lat.put(ya, yb, yz, mk(0, 1, w, co_of(sf) < 2 ? 1 : 0));
        } else if (cy == 3) {                  // :124-141
            lat.put(ya, yb, yz, mk(0, 2, fd_of(sy), 0));
        } else if (cy == 4) {                  // void -> MC, :142-164
            lat.put(ya, yb, yz, mk(0, 3, fd_of(sy), 0));
        }
    }
    int c = c_atom - walls;                     // :216-261
    if (c <= 0) {
        lat.put(a, b, z, 0);
    } else if (c == 1) {
        int fa, fb, fz;
        nb_off(zp, fdx, fa, fb, fz);
        uint8_t sf = lat.get(a + fa, b + fb, z + fz);
        int w = occupied_dir(lat, a, b, z);
        if (w < 0) return 5;
        lat.put(a, b, z, mk(0, 1, w, co_of(sf) < 2 ? 1 : 0));
    } else {
        lat.put(a, b, z, mk(0, c, fdx, 0));
    }
    return 0;
}

// Initial state of SetSi ('FS', SetSi.f:25-221) and SetSiC3C ('F',
// SetSiC3C.f:25-199) for one diamond site; lz = LenZ, len = Len1 (multiple of 24).
MKS_HD uint8_t flat_init_state(int z1, int lz, int len, bool sic)
{
    int zg = 3 * z1;
    bool odd = z1 & 1;               // (x1+y1+z1) mod 4 == 3 sublattice
    int sp = (sic && odd) ? 2 : 1;
    if (!sic && (zg <= 5 || (zg >= lz - 6 && zg <= lz - 1))) return WALL;
    int zb = sic ? 0 : 6;
    if (zg >= zb && zg <= len - 4) return mk(sp, 4, 0, 0);
    if (zg >= len - 3 && zg <= len - 1) return mk(sp, 2, 0, 0);
    if (zg == len) return mk(0, 2, 0, 0);
    return 0;
}

}  // namespace mks
