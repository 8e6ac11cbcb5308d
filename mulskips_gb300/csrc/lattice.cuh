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
// A dummy coor-1 site written by an initializer carries the init-time rate
// 1e-6 of Get_Prob_Ini.f:102-104 instead of Get_Prob's 1e-8 until the site
// itself changes (nothing re-rates a coor-1 site before its one neighbour
// has an event, and that event changes the site): its coordination field
// holds 5 (bits 2-4 = 101).  co_of() reads it as coordination 1, so only the
// rate class tells the two dummies apart; every event writes a fresh byte
// and so drops the mark.
//
// Coverage mode (one coverage species with NCrystal <= 2, or two with
// NCrystal = 1): species value 3 marks an EMPTY site carrying a coverage
// species (LattCoo Occ = 0 with CovInd = ListCov(i), absorption.f:34-36);
// bit 7, the dummy flag of an uncovered empty site, says which: 0 ListCov(1),
// 1 ListCov(2) (a covered site has no dummy rate: Get_Prob takes its
// desorption branch first, Get_Prob.f:91-119).  A covered site keeps its
// coordination and list head; the reference clears the whole word when its
// last neighbour leaves (Evaporation.f:60-67), so a covered site always has
// coordination 1..4.
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
// coordination; the field value 5 of an init-time dummy site reads as 1
MKS_HD int co_of(uint8_t s) { return (s >> 2) & (7 ^ (s & 4)); }
MKS_HD bool ini_of(uint8_t s) { return (s & 0x1C) == 0x14; }
MKS_HD int fd_of(uint8_t s) { return (s >> 5) & 3; }
MKS_HD int dm_of(uint8_t s) { return (s >> 7) & 1; }
MKS_HD bool is_wall(uint8_t s) { return s == WALL; }
MKS_HD bool is_occ(uint8_t s) { return s == WALL || (s & 3) != 0; }
constexpr int COVSP = 3;                       // species value of a covered empty site
constexpr uint8_t COV2 = 0x80;                 // with COVSP: the second coverage species
// species of an atom, 0 for an empty (or covered) site; cov selects coverage mode
MKS_HD int atom_sp(uint8_t s, bool cov) { int sp = s & 3; return (cov && sp == COVSP) ? 0 : sp; }
MKS_HD bool is_cov(uint8_t s, bool cov) { return cov && (s & 3) == COVSP; }
MKS_HD uint8_t mk(int sp, int co, int fd, int dm)
{
    return (uint8_t)((sp & 3) | ((co & 7) << 2) | ((fd & 3) << 5) | ((dm & 1) << 7));
}
// an empty coor-1 site whose one occupied neighbour (direction fd) has
// coordination nco: Get_Prob's dummy when nco < 2; from an initializer
// (ini) the dummy keeps Get_Prob_Ini's rate
MKS_HD uint8_t mk_c1(int fd, int nco, bool ini)
{
    return nco >= 2 ? mk(0, 1, fd, 0) : (uint8_t)(mk(0, 1, fd, 1) | (ini ? 0x10 : 0));
}

// ---- geometry ----
// Neighbour offsets (da, db, dz1) of bond direction d for even / odd layers;
// direction d is JumpDia column d+1 (even) or d+5 (odd).  The reverse bond of
// direction d is direction (d + 2) & 3 on the other sublattice.
MKS_HD void nb_off(int zpar, int d, int &da, int &db, int &dz)
{
    // even layer: (0,0,+1) (0,-1,-1) (-1,-1,+1) (-1,0,-1)
    // odd  layer: (+1,+1,-1) (+1,0,+1) (0,0,-1) (0,+1,+1)
    da = zpar - (d >> 1);
    db = zpar - ((d ^ (d >> 1)) & 1);
    dz = ((d ^ zpar) & 1) ? -1 : 1;
}
MKS_HD int rev_dir(int d) { return (d + 2) & 3; }

// ---- rate classes ----
// 0 none (bulk, void, wall, untracked empty), 1 empty coor-1, 2 empty coor-1
// dummy, 3 empty coor-2, 4 empty coor-3, 5 isolated atom, 6.. occupied
// species sp with reciprocal-neighbour census (nSi+nWall, nC, nB) summing to
// 1..3 (the PTransE key of Get_Prob.f:309-321 without coverage); 63 the
// empty coor-1 dummy of an initializer (Get_Prob_Ini.f:102-104, rate 1e-6).
constexpr int CLS_NONE = 0, CLS_C1 = 1, CLS_C1D = 2, CLS_C2 = 3, CLS_C3 = 4, CLS_ISO = 5, CLS_OCC0 = 6;
constexpr int NCENSUS = 19;
constexpr int CLS_C1I = CLS_OCC0 + 3 * NCENSUS;  // 63
constexpr int NCLASS = CLS_C1I + 1;              // 64
// an empty site's deposition class (coordination 1..3, either dummy)
MKS_HD bool dep_class(int c) { return (c >= CLS_C1 && c <= CLS_C3) || c == CLS_C1I; }
MKS_HD bool dummy_class(int c) { return c == CLS_C1D || c == CLS_C1I; }
// Coverage mode: 6..8 covered site of coordination 1..3 (desorption,
// Get_Prob.f:93-118), 9.. atom of species sp (1..2) with census (nSi+nWall,
// nC) summing to 1..3 and c covered neighbours, c <= 4 - census (the PTransE
// key PE(NSiC, n1, n2, 0, c, 0, 0) of Get_Prob.f:309-312).  C1..C3 carry
// deposition + absorption (Get_Prob.f:155-204).
constexpr int CLS_D1 = 6, CLS_COV0 = 9;
constexpr int NCOVCENSUS = 25;
// Two coverage species (NCrystal = 1): 6..8 and 59..61 the sites covered by
// species 1 and 2 (desorption), 9..27 atoms with (nSi+nWall) = n1 and c1, c2
// covered neighbours of each species, c1 + c2 <= 4 - n1 (the PTransE key
// PE(1, n1, 0, 0, c1, c2, 0) of Get_Prob.f:309-312).
constexpr int CLS_D2 = 59;
constexpr int NCOV2CENSUS = 19;
MKS_HD int cov2_census_index(int n1, int c1, int c2)
{
    int m = 4 - n1;                                     // c1 + c2 <= m
    int base = n1 == 1 ? 0 : (n1 == 2 ? 10 : 16);
    return base + c1 * (m + 1) - c1 * (c1 - 1) / 2 + c2;
}

MKS_HD int cov_census_index(int n1, int n2, int c)
{
    // total t = n1 + n2 in 1..3, n1 descending, then c = 0..4-t
    int t = n1 + n2;
    int base = (t == 1) ? 0 : (t == 2) ? 8 : 17;
    return base + (t - n1) * (5 - t) + c;
}

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

// Does the site carry an event (site_class != CLS_NONE)?  Decided by its own
// byte: an empty site with 1..3 occupied neighbours, or an atom with <= 3
// (its census equals its coordination; census 4 is bulk).
MKS_HD bool event_byte(uint8_t s)
{
    if (s == 0 || s == WALL) return false;
    int co = co_of(s);
    return sp_of(s) ? co <= 3 : (co >= 1 && co <= 3);
}

// Accessor concept: uint8_t get(int a, int b, int z) const; void put(int a, int b, int z, uint8_t v);
// with periodic wrap in a, b handled by the accessor and 0 outside the z range.

// Class of the site (a,b,z): Get_Prob's branch selection (Get_Prob.f:151-323)
// restated for the one-byte state.
// single: the lattice holds species 1 only, so an atom's census is
// (coordination, 0, 0) — walls count with species 1 and reciprocity holds —
// and the neighbours need not be read.
// cov: coverage mode (then single is ignored: the census reads the neighbours);
// cov2: two coverage species.
template <class L>
MKS_HD int site_class(const L &lat, int a, int b, int z, bool single = false, bool cov = false, bool cov2 = false)
{
    uint8_t s = lat.get(a, b, z);
    if (s == 0 || s == WALL) return CLS_NONE;
    int sp = sp_of(s), co = co_of(s);
    if (cov) {
        if (sp == COVSP)
            return (co >= 1 && co <= 3) ? ((cov2 && (s & COV2)) ? CLS_D2 : CLS_D1) + co - 1 : CLS_NONE;
        if (sp != 0) {
            if (co >= 4) return CLS_NONE;
            int n1 = 0, n2 = 0, nc = 0, nc2 = 0;
            int zp = z & 1;
#pragma unroll
            for (int d = 0; d < 4; d++) {
                int da, db, dz;
                nb_off(zp, d, da, db, dz);
                uint8_t t = lat.get(a + da, b + db, z + dz);
                int st = sp_of(t);
                n1 += (t == WALL || st == 1) ? 1 : 0;
                n2 += st == 2 ? 1 : 0;
                nc += (st == COVSP && !(t & COV2)) ? 1 : 0;
                nc2 += (st == COVSP && (t & COV2)) ? 1 : 0;
            }
            int tot = n1 + n2;
            if (tot == 0) return CLS_ISO;
            if (tot > 3) return CLS_NONE;
            if (cov2) return CLS_COV0 + cov2_census_index(n1, nc, nc2);
            return CLS_COV0 + (sp - 1) * NCOVCENSUS + cov_census_index(n1, n2, nc);
        }
    }
    if (sp == 0) {
        if (co == 1) return dm_of(s) ? (ini_of(s) ? CLS_C1I : CLS_C1D) : CLS_C1;
        if (co == 2) return CLS_C2;
        if (co == 3) return CLS_C3;
        return CLS_NONE;
    }
    if (co >= 4) return CLS_NONE;
    if (single) return co == 0 ? CLS_ISO : CLS_OCC0 + census_index(co, 0, 0);
    int n1 = 0, n2 = 0, n3 = 0;
    int zp = z & 1;
#pragma unroll
    for (int d = 0; d < 4; d++) {
        int da, db, dz;
        nb_off(zp, d, da, db, dz);
        uint8_t t = lat.get(a + da, b + db, z + dz);
        int st = sp_of(t);
        n1 += (t == WALL || st == 1) ? 1 : 0;
        n2 += st == 2 ? 1 : 0;
        n3 += st == 3 ? 1 : 0;
    }
    int tot = n1 + n2 + n3;
    if (tot == 0) return CLS_ISO;
    if (tot > 3) return CLS_NONE;
    return CLS_OCC0 + (sp - 1) * NCENSUS + census_index(n1, n2, n3);
}

// Direction of the unique occupied non-wall neighbour (the NBuff of
// Evaporation.f:87-104,238-253); -1 if there is none.
template <class L>
MKS_HD int occupied_dir(const L &lat, int a, int b, int z, bool cov = false)
{
    int r = -1, zp = z & 1;
    for (int d = 0; d < 4; d++) {
        int da, db, dz;
        nb_off(zp, d, da, db, dz);
        uint8_t t = lat.get(a + da, b + db, z + dz);
        if (t != WALL && atom_sp(t, cov) != 0 && co_of(t) <= 3) r = d;
    }
    return r;
}

struct Touched {            // sites whose class may have changed
    int n;
    int a[5], b[5], z[5];
};

// One event split in three stages.  The four neighbour updates of stage 2
// are independent of one another -- two neighbours of a diamond site are
// never bonded, and each rule reads only its own site's bonds -- so they may
// run in any order or concurrently with the same result as the reference's
// loop over the four neighbours.
struct EvCtx {
    int a, b, z;
    int sp;        // deposited species, 0 for an evaporation
    int c0;        // coordination bits of the site before the event
    int fdx;       // first-list-entry direction of the site
    bool cov;      // coverage mode: species 3 is a covered empty site
};

// Stage 1: occupancy and species of the event site change first; its
// coordination bits keep their old value until stage 3 (deposition.f:43-46,
// 237; Evaporation.f:40-44,218).  ev_prepare only reads the site byte sx;
// ev_begin also writes the site.  Both return 0, or 1 if the event does not
// apply to the site.
MKS_HD int ev_prepare(uint8_t sx, int a, int b, int z, int sp, EvCtx &e, bool cov = false)
{
    if (sx == WALL) return 1;
    if (sp ? sp_of(sx) != 0 : atom_sp(sx, cov) == 0) return 1;
    e.a = a; e.b = b; e.z = z; e.sp = sp;
    e.c0 = co_of(sx);
    e.fdx = fd_of(sx);
    e.cov = cov;
    return 0;
}
MKS_HD uint8_t ev_begin_state(const EvCtx &e) { return mk(e.sp, e.c0, e.fdx, 0); }

template <class L>
MKS_HD int ev_begin(L &lat, int a, int b, int z, int sp, EvCtx &e, bool cov = false)
{
    if (ev_prepare(lat.get(a, b, z), a, b, z, sp, e, cov)) return 1;
    lat.put(a, b, z, ev_begin_state(e));
    return 0;
}

// Stage 2: update neighbour d.  Returns 1 if it is a wall, 0 otherwise, or a
// negative code when the state contradicts the cubic model.  A covered
// neighbour is an empty site whose coverage survives every change but the
// loss of its last neighbour (deposition.f:82-191 and Evaporation.f:51-164
// pass its CovInd on to Get_Prob).
template <class L>
MKS_HD int ev_neighbour(L &lat, const EvCtx &e, int d, int &ya, int &yb, int &yz)
{
    int da, db, dz;
    nb_off(e.z & 1, d, da, db, dz);
    ya = e.a + da; yb = e.b + db; yz = e.z + dz;
    uint8_t sy = lat.get(ya, yb, yz);
    if (sy == WALL) return 1;
    int cy = co_of(sy);
    int ay = atom_sp(sy, e.cov);               // species of an atom, 0 if empty
    int cv = sp_of(sy) - ay;                   // COVSP on a covered site, else 0
    const uint8_t hi = cv ? (uint8_t)(sy & COV2) : (uint8_t)0;   // which coverage species
    if (e.sp) {                                // deposition.f:78-235
        if (ay != 0) {                         // occupied neighbour, :192-230
            if (cy <= 3) lat.put(ya, yb, yz, mk(ay, cy + 1, fd_of(sy), 0));
        } else if (cy == 0) {                  // new coor-1 MC site, :86-99
            if (cv) return -6;
            // Get_Prob reads the coordination bits of its single neighbour,
            // i.e. of the event site before stage 3 (Get_Prob.f:156-158)
            lat.put(ya, yb, yz, mk(0, 1, rev_dir(d), e.c0 < 2 ? 1 : 0));
        } else if (cy == 1) {                  // coor 1 -> 2 with FIND_NN, :100-160
            int cnt = 0, yzp = yz & 1;
            for (int f = 0; f < 4; f++) {
                int ea, eb, ez;
                nb_off(yzp, f, ea, eb, ez);
                uint8_t t = lat.get(ya + ea, yb + eb, yz + ez);
                if (t != WALL && atom_sp(t, e.cov) != 0) cnt++;
            }
            if (cnt < 2) return -2;
            lat.put(ya, yb, yz, (uint8_t)(mk(cv, cnt, fd_of(sy), 0) | hi));
        } else if (cy == 2 || cy == 3) {       // :161-191
            lat.put(ya, yb, yz, (uint8_t)(mk(cv, cy + 1, fd_of(sy), 0) | hi));
        }
    } else {                                   // Evaporation.f:46-215
        if (ay != 0) {                         // :166-210
            if (cy >= 1) lat.put(ya, yb, yz, mk(ay, cy - 1, fd_of(sy), 0));
            else return -3;
        } else if (cy == 1) {                  // :51-68, reciprocal only
            if (fd_of(sy) == rev_dir(d)) lat.put(ya, yb, yz, 0);
        } else if (cy == 2) {                  // :69-123
            // the rate check reads the first entry of the list before pruning
            int f = fd_of(sy), fa, fb, fz;
            nb_off(yz & 1, f, fa, fb, fz);
            uint8_t sf = lat.get(ya + fa, yb + fb, yz + fz);
            int w = occupied_dir(lat, ya, yb, yz, e.cov);
            if (w < 0) return -4;
            lat.put(ya, yb, yz, (uint8_t)(mk(cv, 1, w, (!cv && co_of(sf) < 2) ? 1 : 0) | hi));
        } else if (cy == 3) {                  // :124-141
            lat.put(ya, yb, yz, (uint8_t)(mk(cv, 2, fd_of(sy), 0) | hi));
        } else if (cy == 4) {                  // void -> MC, :142-164
            lat.put(ya, yb, yz, (uint8_t)(mk(cv, 3, fd_of(sy), 0) | hi));
        }
    }
    return 0;
}

// Stage 3: final coordination and list head of the event site
// (deposition.f:236-250; Evaporation.f:216-261).  Returns 0 or -5.
template <class L>
MKS_HD int ev_finish(L &lat, const EvCtx &e, int walls)
{
    if (e.sp) {
        lat.put(e.a, e.b, e.z, mk(e.sp, e.c0 + walls, e.fdx, 0));
        return 0;
    }
    int c = e.c0 - walls;
    if (c <= 0) {
        lat.put(e.a, e.b, e.z, 0);
    } else if (c == 1) {
        int fa, fb, fz;
        nb_off(e.z & 1, e.fdx, fa, fb, fz);
        uint8_t sf = lat.get(e.a + fa, e.b + fb, e.z + fz);
        int w = occupied_dir(lat, e.a, e.b, e.z, e.cov);
        if (w < 0) return -5;
        lat.put(e.a, e.b, e.z, mk(0, 1, w, co_of(sf) < 2 ? 1 : 0));
    } else {
        lat.put(e.a, e.b, e.z, mk(0, c, e.fdx, 0));
    }
    return 0;
}

// Serial form: deposition of species sp on the empty site (a,b,z)
// (deposition.f:24-251) or, with sp = 0, evaporation of the atom there
// (Evaporation.f:25-262).  Returns 0 or a nonzero code.
template <class L>
MKS_HD int apply_event(L &lat, int a, int b, int z, int sp, Touched &tc, bool cov = false)
{
    EvCtx e;
    if (ev_begin(lat, a, b, z, sp, e, cov)) return 1;
    tc.n = 5;
    tc.a[0] = a; tc.b[0] = b; tc.z[0] = z;
    int walls = 0;
    for (int d = 0; d < 4; d++) {
        int r = ev_neighbour(lat, e, d, tc.a[d + 1], tc.b[d + 1], tc.z[d + 1]);
        if (r < 0) return -r;
        walls += r;
    }
    int r = ev_finish(lat, e, walls);
    return r < 0 ? -r : 0;
}

template <class L>
MKS_HD int apply_deposition(L &lat, int a, int b, int z, int sp, Touched &tc, bool cov = false)
{
    return sp >= 1 && sp <= (cov ? 2 : 3) ? apply_event(lat, a, b, z, sp, tc, cov) : 1;
}

template <class L>
MKS_HD int apply_evaporation(L &lat, int a, int b, int z, Touched &tc, bool cov = false)
{
    return apply_event(lat, a, b, z, 0, tc, cov);
}

// Coverage events: the new state of the event site, or -1 if the event does
// not apply.  Absorption (absorption.f:24-78) of coverage species `which`
// (1 or 2) covers an empty site of coordination 1..3 keeping its coordination
// and list; desorption (desorption.f:24-117) uncovers it, and Get_Prob then
// recomputes the dummy flag of a coor-1 site from its list head's
// coordination (Get_Prob.f:156-158).  Only the site byte changes; its four
// neighbours' classes follow from it.
template <class L>
MKS_HD int cov_event_state(const L &lat, int a, int b, int z, bool absorb, int which = 1)
{
    uint8_t s = lat.get(a, b, z);
    int co = co_of(s);
    if (s == WALL || co < 1 || co > 3) return -1;
    if (absorb) return sp_of(s) == 0 ? (int)(mk(COVSP, co, fd_of(s), 0) | (which == 2 ? COV2 : 0)) : -1;
    if (sp_of(s) != COVSP) return -1;
    int dm = 0;
    if (co == 1) {
        int fa, fb, fz;
        nb_off(z & 1, fd_of(s), fa, fb, fz);
        dm = co_of(lat.get(a + fa, b + fb, z + fz)) < 2 ? 1 : 0;
    }
    return mk(0, co, fd_of(s), dm);
}

template <class L>
MKS_HD int apply_coverage(L &lat, int a, int b, int z, bool absorb, Touched &tc, int which = 1)
{
    int v = cov_event_state(lat, a, b, z, absorb, which);
    if (v < 0) return 1;
    lat.put(a, b, z, (uint8_t)v);
    tc.n = 5;
    tc.a[0] = a; tc.b[0] = b; tc.z[0] = z;
    for (int d = 0; d < 4; d++) {
        int da, db, dz;
        nb_off(z & 1, d, da, db, dz);
        tc.a[d + 1] = a + da; tc.b[d + 1] = b + db; tc.z[d + 1] = z + dz;
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
