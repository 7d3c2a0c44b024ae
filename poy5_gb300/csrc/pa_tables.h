// Host-side cost matrix of the library: the five tables of POY's `struct cm`
// (src/cm.h:33-76) for a bitset alphabet, plus the derived kernel view.
#pragma once
#include <stdint.h>
#include "pa_core.cuh"

namespace pa {

constexpr int CM_ENTRIES = 2 * NSTATE * NSTATE;  // 2 * (1 << lcm)^2 for lcm = 5

struct HostCM {
    int alph;          // symbols of the input matrix (gap last); 5 for DNA
    int lcm, gap, a_sz, combinations, cost_model, gap_open;
    int is_metric, is_identity;
    int mnz;           // smallest positive cost (cm_get_min_non0_cost)
    int cost[CM_ENTRIES];
    int worst[CM_ENTRIES];
    int tail[CM_ENTRIES];
    int prepend[CM_ENTRIES];
    uint8_t median[CM_ENTRIES];
};

// Build the tables POY derives in OCaml from an alph x alph transformation
// cost matrix (gap last) and a gap-opening cost (0 = linear model).
// Returns 0, or a negative code for unsupported input.
int build_cm(HostCM* cm, const int* tcm, int alph, int gap_open);

// Same tables taken verbatim from a caller (the drop-in path: POY built them).
int adopt_cm(HostCM* cm, int lcm, int gap, int a_sz, int combinations,
             int cost_model, int gap_open, const int* cost,
             const uint8_t* median, const int* worst, const int* tail,
             const int* prepend);

// The shared-memory view the kernels use.
void kernel_tables(const HostCM& cm, Tables* t);

}  // namespace pa
