// Test helper: checks the sublattice tilings of mulskips_gb300/csrc/tiling.cuh
// on every even plane size from 16 to MAXN sites per side and every tile
// width 4..8, both layouts:
//   * every site lies in exactly one tile, and tile_of (the band scan's
//     mapping) names that tile;
//   * no tile is wider or taller than QMAX;
//   * two tiles of one colour are at least 4 columns apart (Chebyshev, on the
//     torus): an event reads two bonds and writes one;
//   * two tiles closer than that are listed as each other's neighbours, and
//     neighbours have different colours;
//   * the brick layout is taken whenever every tile can be 6 sites wide.
// Prints "ok N" (layouts checked) or the first failure; exit code 0 on success.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "../../mulskips_gb300/csrc/tiling.cuh"
using namespace mks_tiling;

static int pdist(int lo0, int hi0, int lo1, int hi1, int n)
{   // columns between two periodic intervals [lo, hi) (0 when they touch or overlap), as a Chebyshev distance - 1
    int best = 1 << 30;
    for (int s = -1; s <= 1; s++) {
        int l1 = lo1 + s * n, h1 = hi1 + s * n;
        int d = l1 >= hi0 ? l1 - hi0 + 1 : (lo0 >= h1 ? lo0 - h1 + 1 : 0);
        best = d < best ? d : best;
    }
    return best;   // Chebyshev distance between the nearest sites (0: overlap)
}

int main(int argc, char **argv)
{
    const int maxn = argc > 1 ? atoi(argv[1]) : 96;
    long long checked = 0;
    for (int brick = 0; brick <= 1; brick++)
        for (int NA = 16; NA <= maxn; NA += 2)
            for (int NB = 16; NB <= maxn; NB += 2)
                for (int w = 4; w <= 8; w++) {
                    Layout L = layout(NA, NB, w, brick != 0);
                    int t, sh;
                    bool fits = brick_fits(NA, w, t, sh);
                    if (brick && fits != (L.ncol == 3)) {
                        printf("FAIL %d %d w%d: brick taken %d, fits %d\n", NA, NB, w, L.ncol == 3, fits);
                        return 1;
                    }
                    const int nt = (int)L.tiles.size();
                    std::vector<int> owner((size_t)NA * NB, -1);
                    for (int i = 0; i < nt; i++) {
                        const Tile &q = L.tiles[i];
                        if (q.a1 - q.a0 > QMAX || q.b1 - q.b0 > QMAX || q.a1 <= q.a0 || q.b1 <= q.b0) {
                            printf("FAIL %d %d w%d: tile %d size %dx%d\n", NA, NB, w, i, q.a1 - q.a0, q.b1 - q.b0);
                            return 1;
                        }
                        for (int b = q.b0; b < q.b1; b++)
                            for (int a = q.a0; a < q.a1; a++) {
                                int &o = owner[(size_t)b * NA + (a % NA)];
                                if (o >= 0) {
                                    printf("FAIL %d %d w%d: site %d %d in tiles %d and %d\n", NA, NB, w, a % NA, b, o, i);
                                    return 1;
                                }
                                o = i;
                            }
                    }
                    for (int b = 0; b < NB; b++)
                        for (int a = 0; a < NA; a++) {
                            int o = owner[(size_t)b * NA + a];
                            if (o < 0 || tile_of(NA, NB, L.nqa, L.nqb, L.shift, a, b) != o) {
                                printf("FAIL %d %d w%d: site %d %d owner %d tile_of %d\n", NA, NB, w, a, b, o,
                                       tile_of(NA, NB, L.nqa, L.nqb, L.shift, a, b));
                                return 1;
                            }
                        }
                    for (int i = 0; i < nt; i++)
                        for (int j = i + 1; j < nt; j++) {
                            const Tile &p = L.tiles[i], &q = L.tiles[j];
                            int d = std::max(pdist(p.a0, p.a1, q.a0, q.a1, NA), pdist(p.b0, p.b1, q.b0, q.b1, NB));
                            bool nb_ij = false, nb_ji = false;
                            for (int k = 0; k < 8; k++) {
                                nb_ij |= p.nbr[k] == j;
                                nb_ji |= q.nbr[k] == i;
                            }
                            if (p.colour == q.colour && d < 4) {
                                printf("FAIL %d %d w%d ncol %d: same-colour tiles %d %d at distance %d\n", NA, NB, w,
                                       L.ncol, i, j, d);
                                return 1;
                            }
                            if (d < 4 && !(nb_ij && nb_ji)) {
                                printf("FAIL %d %d w%d ncol %d: tiles %d %d at distance %d not neighbours\n", NA, NB, w,
                                       L.ncol, i, j, d);
                                return 1;
                            }
                            if ((nb_ij || nb_ji) && p.colour == q.colour) {
                                printf("FAIL %d %d w%d: neighbours %d %d share colour\n", NA, NB, w, i, j);
                                return 1;
                            }
                        }
                    checked++;
                }
    printf("ok %lld\n", checked);
    return 0;
}
