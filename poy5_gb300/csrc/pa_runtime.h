// Runtime internals shared by the C ABI units (pa_capi.cu, pa_driver.cu):
// error text, growable device buffers, the context and cost-matrix objects
// and the batch launcher.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/poyalgn.h"
#include "pa_kernels.h"
#include "pa_tables.h"

namespace pa {

// Format the calling thread's error text (poyalgn_last_error); returns code.
int set_err(int code, const char* fmt, ...);

#define CU(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return ::pa::set_err(POYALGN_ECUDA, "%s: %s (%s:%d)", #call,                \
                                 cudaGetErrorString(e_), __FILE__, __LINE__);           \
    } while (0)

// A device buffer that only grows.
struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
};

int reserve(DevBuf& b, size_t bytes);
void release(DevBuf& b);

template <class T>
T* as(DevBuf& b) { return reinterpret_cast<T*>(b.p); }

}  // namespace pa

struct poyalgn_cm {
    pa::HostCM h;
    pa::Tables t;
    pa::Tables* d = nullptr;
};

struct poyalgn_ctx {
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    pa::Ladder lad[2] = {pa::default_ladder(0), pa::default_ladder(1)};
    int bps[2][pa::NCLASS][2] = {};  // resident CTAs per SM: [affine][class][variant]
    int bps_rt[pa::NCLASS] = {};     // the same for the row tile (affine, lean)
    int row_tile_mode = 2;           // 0 lane pipeline, 1 row tile, 2 by batch size
    // host-pointer batches: staging of inputs and outputs
    pa::DevBuf seqs, offa, lena, offb, lenb, outoff, ints, bytes;
    // per-batch scratch
    pa::DevBuf pfull, eh0, lastcls, slabcta, passes, shadow, qitems, qctr, slab, strides;
    pa::DevBuf dwh, swp, order, order_scratch;
    // per-call staging: one device block (offsets, lengths, tie, sequences)
    // filled from one pinned host block, and a pinned block for the results
    pa::DevBuf callblk;
    bool skip_deferred = false;  // simple_2: the traceback waits for backtrace_2d
    unsigned char* h_in = nullptr;
    size_t h_in_n = 0;
    unsigned char* h_out = nullptr;
    size_t h_out_n = 0;
    unsigned char* h_q = nullptr;  // queue counts read back by small batches
    size_t h_q_n = 0;
    pa::DevBuf nobt_bnd, nobt_ctr, nobt_coop;  // cost-only affine fill scratch
    // Algn_Newkk (pa_newkk.cu): per-warp boundary rows and tile offsets, the
    // direction-code arena, counters, visiting order
    pa::DevBuf nk_bnd, nk_bndg, nk_tb, nk_arena, nk_ctr, nk_order;
    long long nk_arena_words = 0;  // 0: sized from the free device memory
    pa::DevBuf dmarena, dmoff, dmctr;          // deferred tracebacks
    int defer_traceback = 1;                   // 0: trace back inside the class kernels
    pa::DevBuf spec_t0, spec_n, spec_res, spec_off;  // speculative band passes
    pa::DevBuf spec_tstar, spec_p2;                  // the second speculative sweep
    int spec_mode = 2;     // 0 off, 1 every batch, 2 by batch size
    int spec_passes = 8;   // passes per pair run at once
    // the speculative sweep runs every class at once, one stream per class
    cudaStream_t spec_st[pa::NCLASS] = {};
    cudaEvent_t spec_fork = nullptr, spec_join[pa::NCLASS] = {};
    long long dm_fixed = 0;                    // > 0: arena reserved up front, never grown
    int last_launches = 0;
    // upper bound on the direction-slab arena of one batch (0: half the free
    // device memory, at most 64 GB)
    long long slab_budget = 0;
    // caller's caps (poyalgn_set_memory_budget; 0: the defaults below)
    long long slab_cap = 0, arena_cap = 0;
    long long last_budget = 1LL << 30;  // slab budget of the last uncaptured batch
    long long last_free = 0;            // free memory seen by it (arena included)
    // optional per-launch timing: one event before the prep launch and one
    // after each launch of a batch, for up to prof_cap batches
    std::vector<cudaEvent_t> prof_ev;
    int prof_cap = 0, prof_used = 0;
    // per-call stub state: the fill of the last simple_2 / align_affine_3
    bool call_valid = false;
    int call_affine = 0, call_l1 = 0, call_l2 = 0;
    int call_dwh = 0;  // deltawh of the kept linear fill (its plane choice)
    const poyalgn_cm* call_cm = nullptr;
    std::vector<uint8_t> call_s1, call_s2;
    long long call_strides[pa::NCLASS] = {0};
    // per-call Newkk stubs: the alignment of the last newkk_algn_affine
    bool nk_valid = false;
    int nk_l1 = 0, nk_l2 = 0, nk_swaped = 0, nk_k = 0;
    const poyalgn_cm* nk_cm = nullptr;
    std::vector<uint8_t> nk_s1, nk_s2, nk_r1, nk_r2;
    // three-sequence alignment (pa_ukk3.cu): triple workspaces and metadata,
    // the workspace budget (0: half the free memory, at most 192 GB), and the
    // kernel time and launch rounds of the last batch
    pa::DevBuf u3_work, u3_meta;
    long long u3_budget = 0;
    float u3_ms = 0.f;
    int u3_rounds = 0;
};

// Device-resident node sequences (poyalgn_store_*, pa_driver.cu).
struct poyalgn_store {
    poyalgn_ctx* ctx = nullptr;
    pa::DevBuf arena;             // node bytes, bump-allocated
    long long cap = 0, used = 0;
    std::vector<long long> off;   // per node: arena offset and length
    std::vector<int> len;
    // batch scratch: pair metadata, per-pair ints, ea/eb/mwg (and discarded
    // medians), plus pinned host mirrors
    pa::DevBuf meta, ints, bytes;
    std::vector<unsigned char> hmeta;
    std::vector<int> hints;
};

namespace pa {

int ensure_device(poyalgn_ctx* c);

// Enqueue one DOS.median batch on `st` (all pointers on the device); see
// pa_capi.cu.
int run_batch(poyalgn_ctx* c, const poyalgn_cm* cm, int affine, int npairs, int maxmn,
              long long out_total, const uint8_t* seqs, const long long* offa,
              const int* lena, const long long* offb, const int* lenb,
              const long long* out_off, int* cost, int* maxcost, int* alen, int* mlen,
              int* wlen, int* status, uint8_t* ea, uint8_t* eb, uint8_t* med, uint8_t* mwg,
              int* passes, const int* dwh, const int* swp, int do_traceback, cudaStream_t st,
              int distance = 0, int missing_distance = 0);

// Enqueue the cost-only affine fill (algn_CAML_cost_affine_3 semantics) of
// npairs pairs; max_pair_len bounds la + lb of every pair. missing:
// cost of pairs with an all-gap sequence (NOBT_NO_MISSING: no such rule).
int run_nobt(poyalgn_ctx* c, const poyalgn_cm* cm, int npairs, int max_pair_len,
             const uint8_t* seqs, const long long* offa, const int* lena,
             const long long* offb, const int* lenb, int missing, int* cost, int* status,
             cudaStream_t st);
// Reserve run_nobt's scratch for up to max_pairs pairs of lengths up to
// max_len.
int prereserve_nobt(poyalgn_ctx* c, int max_pairs, int max_len);

// Enqueue Algn_Newkk DOS.median (use_ukk, affine) for npairs pairs and wait
// for it (the direction arena may need a rerun of some pairs); max_len
// bounds every sequence length. swp (optional): pair k is already in
// internal order (lena <= lenb) and swp[k] is its swaped flag. kmax
// (optional): receives the last pass's band half-width of each pair.
int run_newkk(poyalgn_ctx* c, const poyalgn_cm* cm, int npairs, int max_len,
              const uint8_t* seqs, const long long* offa, const int* lena,
              const long long* offb, const int* lenb, const long long* out_off, int* cost,
              int* maxcost, int* alen, int* mlen, int* wlen, int* status, uint8_t* ea,
              uint8_t* eb, uint8_t* med, uint8_t* mwg, int* passes, const int* order,
              const int* swp, int* kmax, cudaStream_t st);

// Reserve the per-batch scratch of run_batch for batches of up to max_pairs
// pairs, out_total output bytes and a slab arena of slab_bytes, so that such
// batches allocate nothing.
int prereserve(poyalgn_ctx* c, int affine, int max_pairs, long long out_total,
               long long slab_bytes);

}  // namespace pa
