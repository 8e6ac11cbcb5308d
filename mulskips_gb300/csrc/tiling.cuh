// tiling.cuh — tilings of a replica's (a, b) plane for the synchronous
// sublattice method (host code, shared by the engine and its tests).
//
// Tiles of one colour advance together, so two of them must never touch
// each other's event neighbourhoods: an event reads two bonds and writes one,
// and a bond moves at most one column in a and in b, so tiles of one colour
// must be at least four columns apart (three columns between them) in the
// Chebyshev sense.  Two layouts satisfy it:
//
//   square grid  nqa x nqb tiles (both even), colour (qa & 1) + 2 (qb & 1):
//                4 colours, each tile waits on its 8 neighbours;
//   brick        rows of tiles as in the grid, the odd rows shifted by half a
//                tile, nqa a multiple of 3, colour (qa + 2 (qb & 1)) mod 3:
//                three tiles meet at a corner (as hexagons do), so 3 colours
//                and 6 neighbours suffice.  Tiles of one colour in adjacent
//                rows are the half shift apart, so every tile must be at
//                least 6 sites wide.
//
// A window of the sublattice method is one phase per colour: the brick
// layout runs 3 phases per window where the grid runs 4.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

namespace mks_tiling {

constexpr int QMAX = 8;       // largest tile side (sites); the staging buffers hold QMAX + 4 rows

struct Tile {
    int a0, a1, b0, b1;       // sites [a0, a1) x [b0, b1); a1 may exceed NA (the tile runs over the periodic edge)
    int qa, qb, colour;
    int nbr[8];               // tiles to wait on (the brick layout repeats its 6)
};

struct Layout {
    int nqa = 0, nqb = 0, shift = 0, ncol = 4;
    std::vector<Tile> tiles;  // index qb * nqa + qa
};

// tiles per side of n sites for a target width: even, each at most QMAX wide
inline int tiles_for(int n, int width)
{
    int t = 2 * (n / (2 * width));
    if (t < 2) t = 2;
    while ((n + t - 1) / t > QMAX) t += 2;
    return t;
}

// brick tiles per row (a multiple of 3) and the shift of the odd rows, if
// every tile of an n-site row can be at least 6 sites wide at this width
inline bool brick_fits(int n, int width, int &nqa, int &shift)
{
    int t = 3 * std::max(1, (int)std::lround((double)n / (3.0 * width)));
    while ((n + t - 1) / t > QMAX) t += 3;
    const int wmin = n / t;
    if (wmin < 6) return false;
    nqa = t;
    shift = wmin / 2;
    return true;
}

inline Layout layout(int NA, int NB, int width, bool allow_brick)
{
    Layout L;
    int bq = 0, bs = 0;
    const bool brick = allow_brick && brick_fits(NA, width, bq, bs);
    L.ncol = brick ? 3 : 4;
    L.nqa = brick ? bq : tiles_for(NA, width);
    L.nqb = tiles_for(NB, width);
    L.shift = brick ? bs : 0;
    auto id = [&](int a, int b) { return ((b + L.nqb) % L.nqb) * L.nqa + (a + L.nqa) % L.nqa; };
    for (int qb = 0; qb < L.nqb; qb++)
        for (int qa = 0; qa < L.nqa; qa++) {
            Tile q;
            const int sh = (qb & 1) ? L.shift : 0;
            q.a0 = (qa * NA) / L.nqa + sh;
            q.a1 = ((qa + 1) * NA) / L.nqa + sh;
            q.b0 = (qb * NB) / L.nqb;
            q.b1 = ((qb + 1) * NB) / L.nqb;
            q.qa = qa;
            q.qb = qb;
            if (brick) {
                q.colour = (qa + 2 * (qb & 1)) % 3;
                const int lo = (qb & 1) ? qa : qa - 1;   // first overlapping tile of the rows above and below
                const int nb6[6] = {id(qa - 1, qb), id(qa + 1, qb), id(lo, qb - 1), id(lo + 1, qb - 1), id(lo, qb + 1),
                                    id(lo + 1, qb + 1)};
                for (int k = 0; k < 8; k++) q.nbr[k] = nb6[k % 6];
            } else {
                q.colour = (qa & 1) + 2 * (qb & 1);
                int k = 0;
                for (int db = -1; db <= 1; db++)
                    for (int da = -1; da <= 1; da++)
                        if (da || db) q.nbr[k++] = id(qa + da, qb + db);
            }
            L.tiles.push_back(q);
        }
    return L;
}

#ifdef __CUDACC__
#define MKS_TILING_HD __host__ __device__ __forceinline__
#else
#define MKS_TILING_HD inline
#endif

// the tile holding site (a, b): the mapping of the engine's band scan
MKS_TILING_HD int tile_of(int NA, int NB, int nqa, int nqb, int shift, int a, int b)
{
    const int qb = ((b + 1) * nqb - 1) / NB;
    const int sh = (qb & 1) ? shift : 0;
    const int as = a - sh < 0 ? a - sh + NA : a - sh;
    const int qa = ((as + 1) * nqa - 1) / NA;
    return qb * nqa + qa;
}

}  // namespace mks_tiling
