// stacking.cuh — interface between the C ABI (engine.cu) and the
// explicit-neighbour engine of stacking.cu, which runs the KMC with
// arm-chair (hexagonal) stacking: PtransZig < 1 (IF_Arm_Choice.f:21-56).
//
// With arm-chair stacking, atoms leave the diamond sub-grid: FIND_SN.f:67
// shifts a second neighbour by 8.6602254037 grid units along the bond axis
// (5 units per axis), and FIND_NN.f:25-77 rotates bonds of twinned atoms
// about axes that are no longer <111>, rounding to the grid.  Such a lattice
// has no fixed neighbour tables, so this engine keeps the reference's own
// data model on the device: one LattCoo word per grid point
// (defsystem.f:49,87-91), one index word per grid point (LattInd), and one
// record per listed site with its four NextN coordinates (the ListAdAtom /
// ListAtom / ListVoid entries of defdertype.f:25-45).
#pragma once
#include <stdint.h>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/mulskips_gpu.h"

namespace mks_stk {

struct State;

// A box lx x ly x lz (the handle's config) on `stream`.  Returns an MKS_ERR_*
// code with the message in err.
int create(State **out, const mks_config &cfg, cudaStream_t stream, std::string &err);
void destroy(State *s);
// PTransE (3*4096 doubles, the layout of mks_set_rates) and PTransD (3x3).
int set_rates(State *s, const double *ptransE, const double *ptransD, std::string &err);
// The compact lattice of an initializer (one byte per diamond site, rows of
// `pitch` bytes, layer-major [z1][b][a], device memory) into the explicit
// form: LattCoo words, LattInd and one record per listed site with the four
// bond directions as NextN, then the rates (Get_Prob_Ini: an init-time dummy
// keeps 1e-6).
int from_compact(State *s, const uint8_t *d_st, int NA, int NB, int NZ, int pitch, std::string &err);
// The full reference state: LattCoo(0:lx-1, 0:ly-1, 0:lz) (x fastest) and
// n list entries (grid point xyz[3i..], NextN nn[12i..]), rated by
// Get_Prob_Ini, or with the given event codes and rates (both non-NULL).
int load_lists(State *s, const int32_t *lattcoo, int64_t n, const int32_t *xyz, const int32_t *nn,
               const int32_t *event, const float *rate, std::string &err);
// Deposition.f / Evaporation.f applied to the events in order; a
// deposition of coordination 1 takes its stacking from IF_Arm_Choice, the
// trace's arm flag deciding a tie.  *done gets the events applied.
int replay(State *s, const mks_event *trace, int64_t n, int64_t *done, std::string &err);
// Synchronous-sublattice KMC (see stacking.cu); max_* <= 0 means no limit.
int run(State *s, double tau, int64_t max_windows, int64_t max_events, double max_time, int64_t *events,
        double *time, std::string &err);
int get_lattice(State *s, int32_t *lattcoo, std::string &err);
// List entries: kind 1 a site with an event (ListAdAtom), 2 a bulk atom
// (ListAtom), 3 a void (ListVoid), each with its grid point, NextN, event
// code (1 deposition, 2 dummy deposition, 4 evaporation, 5 isolated atom)
// and FP32 rate.  *n gets the count; arrays are written when cap >= *n.
int get_lists(State *s, int64_t cap, int32_t *xyz, int32_t *nn, int32_t *kind, int32_t *ev, float *rate,
              int64_t *n, std::string &err);
// Every listed site with its LattCoo word, for the host-side writers.
struct Site {
    int32_t x, y, z;
    int32_t nn[4][3];
    uint32_t word;
    int32_t ev;
    float rate;
};
int sites(State *s, std::vector<Site> &out, std::string &err);
// FP32 rates of the sites with a deposition or evaporation (dummies and
// isolated atoms left out), in no particular order.
int event_rates(State *s, std::vector<float> &out, std::string &err);
int observables(State *s, mks_observables *o, std::string &err);
int clock(State *s, double *time, int64_t *window, int64_t *events);
int status(State *s, mks_status *st);
bool loaded(const State *s);

}  // namespace mks_stk
