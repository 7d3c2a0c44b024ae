// Launch interface of the cost-only affine fill (pa_cost.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pa_core.cuh"

namespace pa {

// missing_distance value meaning "no all-gap rule" (per-call cost_affine_3)
constexpr int NOBT_NO_MISSING = -0x7fffffff;

struct NobtArgs {
    const uint8_t* seqs;
    const long long* offa;
    const int* lena;
    const long long* offb;
    const int* lenb;
    int npairs;
    const Tables* tables;
    const int* order;         // optional visiting order (longest first)
    int missing_distance;     // cost of pairs with an all-gap sequence
    int* next;                // work counters (one pair per warp; one per CTA), zero
    int* next_coop;           // before the launch
    int ncoop;                // the first ncoop pairs of the order go one per CTA
                              // (nobt_coop_kernel); the rest to nobt_kernel, which
                              // gives a CTA each to its leading pairs of at least
    long long long_cells;     // max(long_cells, *total / warps launched) cells
    const unsigned long long* total;  // cells of all pairs (null: long_cells alone)
    int4* bnd;                // per warp: block boundary column, bnd_stride rows
    int bnd_stride;           // >= the shorter length of every pair
    int4* coop_cols;          // per CTA of the cooperative kernel: one column per
    long long coop_stride;    // column block, bnd_stride rows each
    int* cost;
    int* status;              // 0 ok, -4 empty, -6 too long, -7 bad state
};

// nobt_kernel: no pair below this many cells runs one per CTA
constexpr long long NOBT_LONG_CELLS = 1LL << 16;

int nobt_warps_per_cta();
int nobt_blocks_per_sm();
// column blocks of a pair whose longer sequence has maxlen positions
int nobt_coop_columns(int maxlen);
// The cost-only launches; a.total (when set) is zero before them.
void launch_nobt(const NobtArgs& a, int grid, int coop_grid, cudaStream_t s);

}  // namespace pa
