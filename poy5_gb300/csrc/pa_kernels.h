// Launch interface between the C-ABI layer and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pa_core.cuh"

namespace pa {

// lastcls[k]: class of pair k's final fill, plus LASTCLS_LEAN when that fill
// wrote lean direction bytes (aff_lean_step) instead of aff_step words
constexpr int LASTCLS_LEAN = 0x100;
constexpr int LASTCLS_ROW = 0x200;  // lean fill on the row tile (row-major bytes)
constexpr int LASTCLS_MASK = 0xFF;

// Everything a batch launch needs, all device pointers.
struct BatchArgs {
    const uint8_t* seqs;       // concatenated input sequences
    const long long* offa;     // pair k: a = seqs[offa[k] .. + lena[k])
    const int* lena;
    const long long* offb;
    const int* lenb;
    int npairs;
    // the caller's declared shape: lena + lenb <= max_pair_len sizes every
    // direction slab, out_off[k] + lena + lenb + 2 <= out_bytes every output
    // slot and the affine row-0 shadow; prep fails a pair outside either
    int max_pair_len;
    long long out_bytes;
    int affine;
    int do_traceback;          // 0: keep the last fill in the slab (per-call stubs)
    int distance;              // DOS.distance: deltaw = max 8 |la - lb|, all-gap -> missing
    int missing_distance;
    Ladder lad;                // pipeline classes of this model
    int row_tile;              // lean affine classes up to 512 wide run on the row tile
    const Tables* tables;
    int* pfull;                // linear plane choice per pair
    int* shadow;               // affine: row-0 EB left by earlier iterations (n per pair)
    int* shadowEH0;            // affine: row-0 EH at column 0
    int2* qitems;              // NQUEUE queues of (pair, T) with capacity qcap
    int* qcount;
    int* qhead;
    int qcap;
    // a class's queues sorted longest pair first just before it runs (null:
    // the class kernels take qitems in push order)
    int2* qsorted;             // same layout as qitems
    int* qhist;                // NQUEUE x NBUCKET counts, zero before the batch
    int* qcur;                 // NQUEUE x NBUCKET scatter cursors, zero before the batch
    uint8_t* slab;             // per-CTA direction slabs, reused class after class
    long long slab_stride;     // bytes per CTA for the class being launched
    const long long* out_off;  // pair k writes its outputs at out_off[k]
    int* cost;
    int* maxcost;
    int* alen;
    int* mlen;
    int* wlen;
    int* status;               // 1 pending, 0 done, < 0 error
    int* passes;               // band iterations run
    int* lastcls;              // class of the final iteration (| LASTCLS_LEAN)
    int* slab_cta;             // pipeline whose slab holds the final fill
    const int* deltawh_override;  // per-call linear stub: caller's deltawh, no reordering
    const int* swap_override;     // per-call stubs: caller's tie preference
    const int* order;             // prep visits pairs in this order (longest first)
    uint8_t* ea;
    uint8_t* eb;
    uint8_t* med;
    uint8_t* mwg;
    // deferred tracebacks: each pair's fills in a class get their own arena
    // region, and the tracebacks run after all fills (dm_cap 0: in-kernel)
    uint8_t* dm_arena;
    long long dm_cap;
    long long dm_max_region;      // larger fills keep the pipeline's slab
    long long dm_max_region2;     // the same for the traced pass of the second sweep
    unsigned long long* dm_used;  // bump counter, zero before the batch
    long long* dm_off;            // per pair: arena offset of the final fill, -1 if none
    // Speculative band passes (small batches): the first spec_S passes of
    // every linear or lean affine pair run at once as independent items (a
    // pass depends on the earlier ones only through the stop decision and,
    // for the affine model, a row-0 value that is a function of the pass
    // index); spec_resolve_kernel then keeps the first pass that satisfies
    // the doubling test, as the sequential doubling would have stopped there.
    int spec;                     // this sweep's linear / lean items are speculative
    int spec_S;                   // passes per pair (0: no speculation in this batch)
    int* spec_T0;                 // per pair: T of pass 0 (0: not speculated)
    int* spec_n;                  // per pair: passes queued (| SPEC_NOCLASS)
    int4* spec_res;               // per pair x SPEC_STRIDE passes: cost, gap count, class flags, 1 = ran
    long long* spec_off;          // per pair x SPEC_STRIDE passes: arena region (-1: none)
    // Second speculative sweep (linear batches of long pairs): a pair's gap
    // count settles once its band holds the alignment, so the first resolve
    // predicts the pass that will end the doubling (the first whose p exceeds
    // the last gap count + 1) and queues every pass up to it at once; the
    // predicted final pass traces back in its class kernel when its own test
    // stops the doubling, and spec_resolve2_kernel keeps exactly the pass the
    // sequential doubling stops at (rerunning it when the prediction missed).
    int spec2;                    // the first resolve queues the second sweep
    int keep_fill;                // per-call simple_2: the final fill's region is
                                  // recorded for a later traceback (dm_off)
    int* spec_Tstar;              // per pair: T of the predicted final pass
    int2* spec_p2;                // per pair: first pass after the first sweep, predicted
                                  // final pass (-1: the sequential sweep resumes there)
};

// spec_res / spec_off hold every speculated pass of a pair at its pass index
constexpr int SPEC_STRIDE = 16;
// spec_res.z: the pass's traceback already ran (second sweep), with its
// status negated in bits 16..23
constexpr int SPEC_TRACED = 0x1000;

// spec_n: the pass after the queued ones has no class (the sequential
// doubling would fail the pair there with status -5)
constexpr int SPEC_NOCLASS = 1 << 30;

// Work queues: 2 per class (variant 1 = affine gap-free fast path).
constexpr int NQUEUE = 2 * NCLASS;
// Length buckets of the queue sort (8 per octave of m + n).
constexpr int NBUCKET = 256;
// Queue counters: counts, heads, and the sort's histograms and cursors.
constexpr int QCTR_INTS = 2 * NQUEUE * (1 + NBUCKET);
// Sort the class's two queues longest pair first (no-op without qsorted).
void launch_sort_queues(const BatchArgs& a, int cls, int grid, cudaStream_t s);
// After a speculative sweep: finish the pairs one of whose passes stopped,
// queue the others for the sequential sweep.
void launch_spec_resolve(const BatchArgs& a, cudaStream_t s);
// After the second speculative sweep: keep each pair's stopping pass or
// queue the sequential sweep where the doubling continues.
void launch_spec_resolve2(const BatchArgs& a, cudaStream_t s);
// Persistent CTAs per SM a class kernel can keep resident.
int class_blocks_per_sm(const Ladder& lad, int affine, int cls, int variant, int row_tile);
// The row tile width of a class's lean queue (0: lane pipeline).
int class_row_tile(const Ladder& lad, int affine, int cls, int variant, int row_tile);
// Bytes of direction slab one pipeline of a class needs for pairs up to
// maxmn = m + n.
long long class_slab_bytes(const Ladder& lad, int affine, int cls, int maxmn, int row_tile);

void launch_prep(const BatchArgs& a, cudaStream_t s);
// Longest-first order of the pairs (by len(a) * len(b)) into `order`.
// `scratch` must hold order_scratch_bytes(npairs) bytes.
size_t order_scratch_bytes(int npairs);
int launch_order(const int* lena, const int* lenb, int npairs, int* order, void* scratch,
                 cudaStream_t s);
void launch_class(const BatchArgs& a, int cls, int variant, int grid, cudaStream_t s);
// Traceback + medians of pairs whose fill was left in the slab (per-call
// path); d_strides[c] = slab bytes per pipeline of class c.
void launch_traceback(const BatchArgs& a, const long long* d_strides, cudaStream_t s);
// The per-call backtrace_2d of the kept linear fill of a one-pair batch (in
// its arena region, or in its pipeline's slab), one warp through the window.
void launch_call_traceback_lin(const BatchArgs& a, const long long* d_strides, cudaStream_t s);
// Tracebacks + medians of the pairs whose final fill sits in the arena: one
// thread per pair, or (small batches, latency-bound) one warp per pair
// through the shared-memory window for byte-coded fills. Returns the
// launches made.
int launch_deferred_traceback(const BatchArgs& a, bool warp_per_pair, cudaStream_t s);
// Pipelines per CTA of a class launch.
int class_pipes_per_cta(const Ladder& lad, int affine, int cls, int variant, int row_tile);
// Column-wise medians of already aligned pairs (ancestor_2 / with-gaps / worst).
void launch_aligned_medians(const Tables* t, const uint8_t* x, const uint8_t* y,
                            int len, uint8_t* anc, uint8_t* mwg, int* out3,
                            cudaStream_t s);
// out2 = {verify cost, no-gap median length}; nogap holds len + 1 bytes
void launch_aligned_extra(const Tables* t, const uint8_t* x, const uint8_t* y, int len,
                          uint8_t* nogap, int* out2, cudaStream_t s);

// backtrace_2d_limit from any start (lin_limit_walk) over the fill the
// per-call path kept in its slab: s1 = l1 rows, s2 = l2 columns, planned with
// the caller's deltawh. One thread; out2 = {walk status, length}; r1 / r2
// end at index cap - 1.
struct LimitWalk {
    const Tables* t;
    const uint8_t* slab;
    const long long* strides;  // slab bytes per pipeline of each class
    const int* lastcls;
    const int* slab_cta;
    const int* passes;
    const int* pfull;
    const long long* dm_off;   // the fill's arena region (-1: in the slab)
    const uint8_t* dm_arena;
    Ladder lad;
    const uint8_t* s1;
    const uint8_t* s2;
    int l1, l2, deltawh, st_s1, st_s2, algn_s1, algn_s2, swaped, cap;
    uint8_t* r1;
    uint8_t* r2;
    int* out2;
};
void launch_limit_walk(const LimitWalk& a, cudaStream_t s);

}  // namespace pa
