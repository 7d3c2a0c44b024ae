// C ABI of libpoyalgn.so (include/poyalgn.h): contexts, cost matrices, the
// batched DOS.median driver and the per-call stubs that replace POY's
// algn_CAML_* externals.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <vector>

#include "pa_cost.h"
#include "pa_runtime.h"

using namespace pa;

namespace {

thread_local char g_err[512];

}  // namespace

namespace pa {

int set_err(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int reserve(DevBuf& b, size_t bytes)
{
    if (bytes <= b.n && b.p) return 0;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
    size_t want = std::max<size_t>(bytes, 256);
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
        cudaGetLastError();
        return set_err(POYALGN_ENOMEM, "cudaMalloc of %zu bytes failed", want);
    }
    b.n = want;
    return 0;
}

void release(DevBuf& b)
{
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
}

int ensure_device(poyalgn_ctx* c)
{
    CU(cudaSetDevice(c->device));
    return 0;
}

constexpr int ROW_TILE_MAX_PAIRS = 2;  // per SM, for row_tile_mode 2
// spec_mode 2: batches of at most SPEC_FULL_PAIRS pairs per SM speculate
// spec_passes passes, up to SPEC_MAX_PAIRS two fewer (measured on GB300: the
// extra cells cost more than the latency saved beyond about 30 pairs per SM)
constexpr int SPEC_FULL_PAIRS = 8;
// batches of at most this many pairs per SM trace back a warp per pair
constexpr int WIN_TB_PAIRS = 8;
// batches of at most this many pairs launch only their non-empty classes
constexpr int HOST_PLAN_PAIRS = 4;
constexpr int SPEC_MAX_PAIRS = 32;
// Largest arena region one pair's fills in one class may take; wider fills
// (long pairs) keep the pipeline's slab and trace back in the class kernel.
constexpr long long DM_MAX_REGION = 64LL << 20;
// The second speculative sweep (linear batches with pairs of at least
// SPEC2_MIN_LEN positions together): the traced final pass of each pair
// takes a region of up to DM_MAX_REGION2, from an arena of up to
// ARENA_MAX_SPEC2 (64 GB otherwise).
constexpr int SPEC2_MIN_LEN = 8192;
constexpr long long DM_MAX_REGION2 = 512LL << 20;
constexpr long long ARENA_MAX = 64LL << 30;
constexpr long long ARENA_MAX_SPEC2 = 192LL << 30;

// A pinned host buffer that only grows.
int pinned(unsigned char** p, size_t* n, size_t want)
{
    if (*n >= want) return 0;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *n = 0;
    if (cudaHostAlloc((void**)p, want, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_err(POYALGN_ENOMEM, "pinned staging of %zu bytes", want);
    }
    *n = want;
    return 0;
}

// Enqueue one batch on `st`. All pointers are device pointers. `out_total`
// bounds out_off[k] + cap_k (sizes the affine row-0 scratch).
int run_batch(poyalgn_ctx* c, const poyalgn_cm* cm, int affine, int npairs,
              int maxmn, long long out_total, const uint8_t* seqs,
              const long long* offa, const int* lena, const long long* offb,
              const int* lenb, const long long* out_off, int* cost, int* maxcost,
              int* alen, int* mlen, int* wlen, int* status, uint8_t* ea,
              uint8_t* eb, uint8_t* med, uint8_t* mwg, int* passes,
              const int* dwh, const int* swp, int do_traceback, cudaStream_t st,
              int distance, int missing_distance)
{
    int rc;
    if (npairs <= 0) return 0;
    c->call_valid = false;  // the slabs and the arena are about to be reused
    // Batches too small to fill the GPU run their pairs' first band passes
    // at once (speculative sweep, then the sequential sweep for the pairs
    // that need more). The fills must outlive the sweep: the arena holds
    // them, or only the cost is wanted.
    const bool spec_ok = distance || (do_traceback && c->defer_traceback);
    int spec_S = 0;
    if (spec_ok && c->spec_mode == 1) spec_S = c->spec_passes;
    if (spec_ok && c->spec_mode == 2) {
        if (npairs <= SPEC_FULL_PAIRS * c->nsm) spec_S = c->spec_passes;
        else if (npairs <= SPEC_MAX_PAIRS * c->nsm) spec_S = std::max(1, c->spec_passes - 2);
    }
    // small batches take the row tile unless their passes run speculatively
    // on the lane pipeline (one long pair: the row tile's per-row scans cost
    // more per pass than a lane pipeline's anti-diagonal steps)
    const int row_tile = affine && !spec_S &&
                         (c->row_tile_mode == 1 ||
                          (c->row_tile_mode == 2 && npairs <= ROW_TILE_MAX_PAIRS * c->nsm));
    // long linear pairs: every pass after the first sweep up to the predicted
    // final one runs at once in a second speculative sweep
    const bool spec2 = spec_S > 0 && !affine && maxmn >= SPEC2_MIN_LEN;
    // queue capacity: a sweep queues at most spec_S passes of a pair, the
    // second one at most SPEC_STRIDE
    const int items = npairs * std::max(spec2 ? SPEC_STRIDE : 1, spec_S);
    if ((rc = reserve(c->pfull, (size_t)npairs * 4))) return rc;
    if ((rc = reserve(c->eh0, (size_t)npairs * 4))) return rc;
    if ((rc = reserve(c->lastcls, (size_t)npairs * 4))) return rc;
    if ((rc = reserve(c->slabcta, (size_t)npairs * 4))) return rc;
    if (!passes) {
        if ((rc = reserve(c->passes, (size_t)npairs * 4))) return rc;
        passes = as<int>(c->passes);
    }
    if ((rc = reserve(c->shadow, (size_t)(affine ? out_total : 1) * 4))) return rc;
    if ((rc = reserve(c->qitems, 2 * (size_t)NQUEUE * items * sizeof(int2)))) return rc;
    if ((rc = reserve(c->qctr, QCTR_INTS * sizeof(int)))) return rc;
    if ((rc = reserve(c->strides, NCLASS * sizeof(long long)))) return rc;
    const size_t spec_items = (size_t)npairs * SPEC_STRIDE;  // every pass by its index
    if (spec_S) {
        DevBuf* per_pair[] = {&c->spec_t0, &c->spec_n, &c->spec_tstar};
        for (DevBuf* b : per_pair)
            if ((rc = reserve(*b, (size_t)npairs * 4))) return rc;
        if ((rc = reserve(c->spec_p2, (size_t)npairs * sizeof(int2)))) return rc;
        if ((rc = reserve(c->spec_res, spec_items * sizeof(int4)))) return rc;
        if ((rc = reserve(c->spec_off, spec_items * 8))) return rc;
        CU(cudaMemsetAsync(c->spec_res.p, 0, spec_items * sizeof(int4), st));
    }

    // a capture (poyalgn_batch_graph_create) records the launches only: the
    // budget of the run before it, and no host-memory copies
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CU(cudaStreamIsCapturing(st, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    // persistent grid per class, bounded by a slab budget; with deferred
    // tracebacks the fills go to the direction arena and the slabs are only
    // the fallback when it is full
    const bool defer = do_traceback && c->defer_traceback;
    long long total_budget = c->last_budget;
    if (!capturing) {
        size_t free_b = 0, total_b = 0;
        CU(cudaMemGetInfo(&free_b, &total_b));
        // half of the free memory, at most 128 GB: the widest long-pair
        // classes (512 pairs of 50 kb on 256-lane pipelines) fit in one round
        total_budget = std::min<long long>((long long)(free_b / 2), 128LL << 30);
        if (c->slab_budget > 0) total_budget = std::min(total_budget, c->slab_budget);
        if (c->slab_cap > 0) total_budget = std::min(total_budget, c->slab_cap);
        c->last_budget = total_budget;
    }
    const long long budget = total_budget;
    int grid[NCLASS][2];
    long long strides[NCLASS];
    long long arena = 0;
    for (int k = 0; k < NCLASS; k++) {
        strides[k] = class_slab_bytes(c->lad[affine], affine, k, maxmn, row_tile);
        for (int v = 0; v < 2; v++) {
            const int pipes = class_pipes_per_cta(c->lad[affine], affine, k, v, row_tile);
            const int bps = class_row_tile(c->lad[affine], affine, k, v, row_tile)
                                ? c->bps_rt[k] : c->bps[affine][k][v];
            long long g = (long long)c->nsm * std::max(1, bps);
            g = std::min<long long>(g, (items + pipes - 1) / pipes);
            g = std::min<long long>(g, std::max<long long>(1, budget / (strides[k] * pipes)));
            grid[k][v] = (int)std::max<long long>(1, g);
            arena = std::max(arena, (long long)grid[k][v] * pipes * strides[k]);
        }
    }
    if ((rc = reserve(c->slab, (size_t)arena))) return rc;
    long long dm_cap = 0;
    if (defer) {
        // the arena takes what is free after the slabs (16 GB kept back), at
        // most 64 GB and DM_MAX_REGION per pair
        long long free_now = c->last_free;
        if (!capturing) {
            size_t fr = 0, tot = 0;
            CU(cudaMemGetInfo(&fr, &tot));
            free_now = (long long)fr + (long long)c->dmarena.n;  // the arena may be re-reserved
            c->last_free = free_now;
        }
        const long long want = (long long)items * DM_MAX_REGION +
                               (spec2 ? (long long)npairs * DM_MAX_REGION2 : 0);
        dm_cap = std::max<long long>(0, std::min({free_now - (16LL << 30),
                                                  spec2 ? ARENA_MAX_SPEC2 : ARENA_MAX, want}));
        if (capturing) dm_cap = std::min<long long>(dm_cap, (long long)c->dmarena.n);
        if (c->dm_fixed > 0) dm_cap = std::min(dm_cap, c->dm_fixed);
        if (c->arena_cap > 0) dm_cap = std::min(dm_cap, c->arena_cap);
        if ((rc = reserve(c->dmarena, (size_t)std::max<long long>(dm_cap, 256)))) return rc;
        if ((rc = reserve(c->dmoff, (size_t)npairs * 8))) return rc;
        if ((rc = reserve(c->dmctr, 8))) return rc;
        CU(cudaMemsetAsync(c->dmctr.p, 0, 8, st));
    }
    if (do_traceback && dm_cap <= 0) {
        // no arena: every fill stays in its slab (a later per-call traceback
        // reads "no region" here)
        if ((rc = reserve(c->dmoff, (size_t)npairs * 8))) return rc;
        CU(cudaMemsetAsync(c->dmoff.p, 0xFF, (size_t)npairs * 8, st));
    }
    if (!capturing)  // slab strides for the per-call traceback
        CU(cudaMemcpyAsync(c->strides.p, strides, sizeof(strides), cudaMemcpyHostToDevice, st));
    memcpy(c->call_strides, strides, sizeof(strides));
    CU(cudaMemsetAsync(c->qctr.p, 0, QCTR_INTS * sizeof(int), st));

    BatchArgs A;
    memset(&A, 0, sizeof(A));
    A.seqs = seqs;
    A.offa = offa;
    A.lena = lena;
    A.offb = offb;
    A.lenb = lenb;
    A.npairs = npairs;
    A.max_pair_len = maxmn;
    A.out_bytes = out_total;
    A.affine = affine;
    A.do_traceback = do_traceback;
    A.distance = distance;
    A.missing_distance = missing_distance;
    A.lad = c->lad[affine];
    A.row_tile = row_tile;
    A.tables = cm->d;
    A.pfull = as<int>(c->pfull);
    A.shadow = as<int>(c->shadow);
    A.shadowEH0 = as<int>(c->eh0);
    A.qitems = as<int2>(c->qitems);
    A.qcount = as<int>(c->qctr);
    A.qhead = as<int>(c->qctr) + NQUEUE;
    A.qcap = items;
    A.qsorted = as<int2>(c->qitems) + (size_t)NQUEUE * items;
    A.qhist = as<int>(c->qctr) + 2 * NQUEUE;
    A.qcur = A.qhist + NQUEUE * NBUCKET;
    A.slab = as<uint8_t>(c->slab);
    A.out_off = out_off;
    A.cost = cost;
    A.maxcost = maxcost;
    A.alen = alen;
    A.mlen = mlen;
    A.wlen = wlen;
    A.status = status;
    A.passes = passes;
    A.lastcls = as<int>(c->lastcls);
    A.slab_cta = as<int>(c->slabcta);
    A.deltawh_override = dwh;
    A.swap_override = swp;
    A.ea = ea;
    A.eb = eb;
    A.med = med;
    A.mwg = mwg;
    if (defer && dm_cap > 0) {
        A.dm_arena = as<uint8_t>(c->dmarena);
        A.dm_cap = dm_cap;
        A.dm_max_region = DM_MAX_REGION;
        A.dm_max_region2 = DM_MAX_REGION2;
        A.dm_used = as<unsigned long long>(c->dmctr);
        A.dm_off = as<long long>(c->dmoff);
    }

    // longest pairs enter the queues first so the persistent grid drains evenly
    if ((rc = reserve(c->order, (size_t)npairs * 4))) return rc;
    if ((rc = reserve(c->order_scratch, order_scratch_bytes(npairs)))) return rc;
    if (launch_order(lena, lenb, npairs, as<int>(c->order), c->order_scratch.p, st) != 0)
        return set_err(POYALGN_ECUDA, "ordering pairs failed");
    A.order = as<int>(c->order);

    if (spec_S) {
        A.spec_S = spec_S;
        A.spec_T0 = as<int>(c->spec_t0);
        A.spec_n = as<int>(c->spec_n);
        A.spec_res = as<int4>(c->spec_res);
        A.spec_off = as<long long>(c->spec_off);
        A.spec2 = spec2 ? 1 : 0;
        A.keep_fill = c->skip_deferred ? 1 : 0;
        A.spec_Tstar = as<int>(c->spec_tstar);
        A.spec_p2 = as<int2>(c->spec_p2);
    }

    int launches = 0;
    cudaEvent_t* ev = nullptr;
    if (!capturing && c->prof_used < c->prof_cap) {
        ev = &c->prof_ev[(size_t)c->prof_used * (NCLASS + 2)];
        c->prof_used++;
        CU(cudaEventRecord(ev[0], st));
    }
    launch_prep(A, st);
    launches++;
    // the prep slot of a speculative batch also holds its speculative sweep
    if (ev && !spec_S) CU(cudaEventRecord(ev[1], st));
    const int sort_grid = std::max(1, std::min(2 * c->nsm, (items + 255) / 256));
    // A batch of a few pairs (the per-call stubs) reads its queue counts
    // back before each sweep, so that a speculative sweep launches only its
    // non-empty classes and the sequential sweep starts at the lowest
    // non-empty class (items only move up the ladder) or is skipped: two
    // short synchronisations instead of dozens of empty launches.
    const bool host_plan = !capturing && !ev && npairs <= HOST_PLAN_PAIRS;
    int qcnt[NQUEUE];
    auto read_counts = [&]() -> int {
        if ((rc = pinned(&c->h_q, &c->h_q_n, NQUEUE * sizeof(int)))) return rc;
        CU(cudaMemcpyAsync(c->h_q, c->qctr.p, NQUEUE * sizeof(int), cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        memcpy(qcnt, c->h_q, sizeof(qcnt));
        return 0;
    };
    auto sweep = [&]() -> int {
        int k0 = 0;
        if (host_plan) {
            if ((rc = read_counts())) return rc;
            while (k0 < NCLASS && qcnt[2 * k0] == 0 && qcnt[2 * k0 + 1] == 0) k0++;
        }
        for (int k = k0; k < NCLASS; k++) {
            A.slab_stride = strides[k];
            launch_sort_queues(A, k, sort_grid, st);
            launches += 2;
            for (int v = 0; v < (affine ? 2 : 1); v++) {
                launch_class(A, k, v, grid[k][v], st);
                launches++;
            }
            if (ev) CU(cudaEventRecord(ev[k + 2], st));
        }
        return 0;
    };
    if (spec_S) {
        // speculative sweeps: only linear / lean items, which never move
        // between classes, so the classes run concurrently (fork / join)
        if (!c->spec_fork) {
            CU(cudaEventCreateWithFlags(&c->spec_fork, cudaEventDisableTiming));
            for (int k = 0; k < NCLASS; k++) {
                CU(cudaStreamCreateWithFlags(&c->spec_st[k], cudaStreamNonBlocking));
                CU(cudaEventCreateWithFlags(&c->spec_join[k], cudaEventDisableTiming));
            }
        }
        auto spec_sweep = [&](int phase) -> int {
            const int v = affine ? 1 : 0;
            if (host_plan && (rc = read_counts())) return rc;
            A.spec = phase;
            CU(cudaEventRecord(c->spec_fork, st));
            // the second sweep's passes are the wide ones: the widest class
            // goes first, so its long passes start at once and the narrower
            // classes fill the SMs it leaves
            for (int i = 0; i < NCLASS; i++) {
                const int k = phase == 2 ? NCLASS - 1 - i : i;
                if (host_plan && qcnt[2 * k + v] == 0) continue;
                cudaStream_t sk = c->spec_st[k];
                CU(cudaStreamWaitEvent(sk, c->spec_fork, 0));
                A.slab_stride = strides[k];
                launch_sort_queues(A, k, sort_grid, sk);
                launch_class(A, k, v, grid[k][v], sk);
                launches += 3;
                CU(cudaEventRecord(c->spec_join[k], sk));
                CU(cudaStreamWaitEvent(st, c->spec_join[k], 0));
            }
            // fresh queues for the next sweep, which the resolve fills
            CU(cudaMemsetAsync(c->qctr.p, 0, QCTR_INTS * sizeof(int), st));
            A.spec = 0;
            return 0;
        };
        if ((rc = spec_sweep(1))) return rc;
        launch_spec_resolve(A, st);
        launches++;
        if (spec2) {
            if ((rc = spec_sweep(2))) return rc;
            launch_spec_resolve2(A, st);
            launches++;
        }
        if (ev) CU(cudaEventRecord(ev[1], st));
    }
    if ((rc = sweep())) return rc;
    if (A.dm_cap > 0 && !c->skip_deferred) {
        // a warp per pair through the shared-memory window cuts a small
        // batch's latency; a large batch has the parallelism to hide one
        // thread per pair's dependent loads and less traffic that way
        launches += launch_deferred_traceback(A, npairs <= WIN_TB_PAIRS * c->nsm, st);
    }
    CU(cudaGetLastError());
    c->last_launches = launches;
    return 0;
}

int prereserve(poyalgn_ctx* c, int affine, int max_pairs, long long out_total,
               long long slab_bytes)
{
    int rc;
    const size_t n = (size_t)std::max(max_pairs, 1);
    DevBuf* per_pair[] = {&c->pfull, &c->eh0, &c->lastcls, &c->slabcta, &c->passes, &c->order};
    for (DevBuf* b : per_pair)
        if ((rc = reserve(*b, n * 4))) return rc;
    if ((rc = reserve(c->shadow, (size_t)(affine ? out_total : 1) * 4))) return rc;
    // speculative batches queue up to spec_passes items per pair, and linear
    // ones up to SPEC_STRIDE in the second sweep
    const size_t items =
        n * (size_t)(c->spec_mode ? std::max(affine ? 1 : SPEC_STRIDE, c->spec_passes) : 1);
    if ((rc = reserve(c->qitems, 2 * (size_t)NQUEUE * items * sizeof(int2)))) return rc;
    if ((rc = reserve(c->qctr, QCTR_INTS * sizeof(int)))) return rc;
    if ((rc = reserve(c->strides, NCLASS * sizeof(long long)))) return rc;
    if ((rc = reserve(c->order_scratch, order_scratch_bytes((int)n)))) return rc;
    if (c->spec_mode) {
        if ((rc = reserve(c->spec_t0, n * 4))) return rc;
        if ((rc = reserve(c->spec_n, n * 4))) return rc;
        if ((rc = reserve(c->spec_tstar, n * 4))) return rc;
        if ((rc = reserve(c->spec_p2, n * sizeof(int2)))) return rc;
        if ((rc = reserve(c->spec_res, n * SPEC_STRIDE * sizeof(int4)))) return rc;
        if ((rc = reserve(c->spec_off, n * SPEC_STRIDE * 8))) return rc;
    }
    if ((rc = reserve(c->slab, (size_t)slab_bytes))) return rc;
    if (c->dm_fixed > 0) {
        if ((rc = reserve(c->dmarena, (size_t)c->dm_fixed))) return rc;
        if ((rc = reserve(c->dmoff, n * 8))) return rc;
        if ((rc = reserve(c->dmctr, 8))) return rc;
    }
    return 0;
}

static int nobt_grid(const poyalgn_ctx* c, int npairs)
{
    const int per_sm = std::max(1, nobt_blocks_per_sm());
    return std::max(1, std::min(c->nsm * per_sm,
                                (npairs + nobt_warps_per_cta() - 1) / nobt_warps_per_cta()));
}

// Small batches run one pair per CTA (all its warps on one pair, lower
// latency); large ones one pair per warp.
static int nobt_ncoop(const poyalgn_ctx* c, int npairs) { return npairs <= 2 * c->nsm ? npairs : 0; }

static int nobt_reserve(poyalgn_ctx* c, int npairs, int max_pair_len, int* grid, int* cgrid,
                        int* stride, long long* cstride)
{
    int rc;
    *stride = std::max(max_pair_len / 2, 1);  // rows: the shorter length
    *grid = nobt_grid(c, npairs);
    const int ncoop = nobt_ncoop(c, npairs);
    *cgrid = std::max(1, std::min(ncoop, c->nsm));
    *cstride = (long long)nobt_coop_columns(max_pair_len) * *stride;
    const size_t warps = (size_t)*grid * nobt_warps_per_cta();
    if ((rc = reserve(c->nobt_bnd, warps * (size_t)*stride * sizeof(int4)))) return rc;
    if ((rc = reserve(c->nobt_coop, ncoop > 0 ? (size_t)*cgrid * (size_t)*cstride * sizeof(int4)
                                              : sizeof(int4))))
        return rc;
    // work counters (2 ints) and the batch's cell total (u64 at byte 8)
    if ((rc = reserve(c->nobt_ctr, 16))) return rc;
    if ((rc = reserve(c->order, (size_t)std::max(npairs, 1) * 4))) return rc;
    return reserve(c->order_scratch, order_scratch_bytes(std::max(npairs, 1)));
}

int prereserve_nobt(poyalgn_ctx* c, int max_pairs, int max_len)
{
    int g, cg, st;
    long long cs;
    // both kernels' scratch: the largest per-warp and per-CTA layouts
    int rc = nobt_reserve(c, max_pairs, 2 * max_len, &g, &cg, &st, &cs);
    if (rc) return rc;
    return nobt_reserve(c, std::min(max_pairs, 2 * c->nsm), 2 * max_len, &g, &cg, &st, &cs);
}

int run_nobt(poyalgn_ctx* c, const poyalgn_cm* cm, int npairs, int max_pair_len,
             const uint8_t* seqs, const long long* offa, const int* lena,
             const long long* offb, const int* lenb, int missing, int* cost, int* status,
             cudaStream_t st)
{
    int rc;
    if (npairs <= 0) return 0;
    int grid, cgrid, stride;
    long long cstride;
    if ((rc = nobt_reserve(c, npairs, max_pair_len, &grid, &cgrid, &stride, &cstride))) return rc;
    CU(cudaMemsetAsync(c->nobt_ctr.p, 0, 16, st));
    if (launch_order(lena, lenb, npairs, as<int>(c->order), c->order_scratch.p, st) != 0)
        return set_err(POYALGN_ECUDA, "ordering pairs failed");
    NobtArgs A;
    memset(&A, 0, sizeof(A));
    A.seqs = seqs;
    A.offa = offa;
    A.lena = lena;
    A.offb = offb;
    A.lenb = lenb;
    A.npairs = npairs;
    A.tables = cm->d;
    A.order = as<int>(c->order);
    A.missing_distance = missing;
    A.next = as<int>(c->nobt_ctr);
    A.next_coop = as<int>(c->nobt_ctr) + 1;
    A.ncoop = nobt_ncoop(c, npairs);
    A.long_cells = NOBT_LONG_CELLS;
    A.total = reinterpret_cast<const unsigned long long*>(as<uint8_t>(c->nobt_ctr) + 8);
    A.bnd = as<int4>(c->nobt_bnd);
    A.bnd_stride = stride;
    A.coop_cols = as<int4>(c->nobt_coop);
    A.coop_stride = cstride;
    A.cost = cost;
    A.status = status;
    launch_nobt(A, grid, cgrid, st);
    CU(cudaGetLastError());
    c->last_launches = 2 + (A.ncoop > 0 ? 1 : 0) + (A.ncoop < npairs ? 2 : 0);
    return 0;
}

}  // namespace pa

namespace {

int upload_cm(poyalgn_cm* m)
{
    kernel_tables(m->h, &m->t);
    CU(cudaMalloc(&m->d, sizeof(Tables)));
    CU(cudaMemcpy(m->d, &m->t, sizeof(Tables), cudaMemcpyHostToDevice));
    return 0;
}


// Per-call block layout: offa, offb, out_off (3 int64), lena, lenb, tie,
// deltawh (4 int32), then both sequences from byte CALL_SEQ.
constexpr size_t CALL_SEQ = 48;
constexpr size_t CALL_TIE = 32;

// One pair, its tie preference and deltawh staged with a single copy from
// pinned host memory; the device pointers of the block's fields.
struct CallPair {
    const uint8_t* seqs;
    const long long* offa;
    const int* lena;
    const int* tie;
    const int* dwh;
};
int stage_call(poyalgn_ctx* c, const uint8_t* a, int la, const uint8_t* b, int lb, int tie,
               int deltawh, CallPair* cp)
{
    int rc;
    const size_t n = CALL_SEQ + (size_t)la + lb;
    if ((rc = pinned(&c->h_in, &c->h_in_n, n))) return rc;
    if ((rc = reserve(c->callblk, n))) return rc;
    long long* o = reinterpret_cast<long long*>(c->h_in);
    o[0] = CALL_SEQ;
    o[1] = CALL_SEQ + la;
    o[2] = 0;
    int* l = reinterpret_cast<int*>(c->h_in + 24);
    l[0] = la;
    l[1] = lb;
    l[2] = tie;
    l[3] = deltawh;
    memcpy(c->h_in + CALL_SEQ, a, (size_t)la);
    memcpy(c->h_in + CALL_SEQ + la, b, (size_t)lb);
    CU(cudaMemcpyAsync(c->callblk.p, c->h_in, n, cudaMemcpyHostToDevice, c->stream));
    const uint8_t* d = as<uint8_t>(c->callblk);
    cp->seqs = d;  // offsets are from the block's start
    cp->offa = reinterpret_cast<const long long*>(d);
    cp->lena = reinterpret_cast<const int*>(d + 24);
    cp->tie = reinterpret_cast<const int*>(d + CALL_TIE);
    cp->dwh = reinterpret_cast<const int*>(d + CALL_TIE + 4);
    return 0;
}

// Results of a staged one-pair call: the seven result ints and nbytes of
// the output buffers, copied to the pinned result block with one
// synchronisation. Returns the host pointer of the ints (bytes follow at 32).
int fetch_call(poyalgn_ctx* c, size_t nbytes, const int** h)
{
    int rc;
    if ((rc = pinned(&c->h_out, &c->h_out_n, 32 + nbytes))) return rc;
    CU(cudaMemcpyAsync(c->h_out, c->ints.p, 7 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if (nbytes)
        CU(cudaMemcpyAsync(c->h_out + 32, c->bytes.p, nbytes, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    *h = reinterpret_cast<const int*>(c->h_out);
    return 0;
}

}  // namespace

extern "C" {

const char* poyalgn_last_error(void) { return g_err; }

const char* poyalgn_version(void) { return "poyalgn 0.1 sm_103a"; }

int poyalgn_init(int device, poyalgn_ctx** out)
{
    if (!out) return set_err(POYALGN_EINVAL, "null output");
    *out = nullptr;
    int n = 0;
    CU(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return set_err(POYALGN_EINVAL, "no CUDA device %d", device);
    poyalgn_ctx* c = new (std::nothrow) poyalgn_ctx;
    if (!c) return set_err(POYALGN_ENOMEM, "context allocation");
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return set_err(POYALGN_ECUDA, "device setup: %s", cudaGetErrorString(e));
    }
    for (int a = 0; a < 2; a++)
        for (int k = 0; k < NCLASS; k++)
            for (int v = 0; v < 2; v++) c->bps[a][k][v] = class_blocks_per_sm(c->lad[a], a, k, v, 0);
    for (int k = 0; k < NCLASS; k++) c->bps_rt[k] = class_blocks_per_sm(c->lad[1], 1, k, 1, 1);
    *out = c;
    return 0;
}

void poyalgn_free(poyalgn_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    DevBuf* bufs[] = {&c->seqs, &c->offa, &c->lena, &c->offb, &c->lenb, &c->outoff,
                      &c->ints, &c->bytes, &c->pfull, &c->eh0, &c->lastcls, &c->slabcta,
                      &c->passes, &c->shadow, &c->qitems, &c->qctr, &c->slab, &c->strides,
                      &c->dwh, &c->swp, &c->order, &c->order_scratch, &c->nobt_bnd,
                      &c->nobt_ctr, &c->nobt_coop, &c->dmarena, &c->dmoff, &c->dmctr,
                      &c->spec_t0, &c->spec_n, &c->spec_res, &c->spec_off,
                      &c->spec_tstar, &c->spec_p2, &c->callblk};
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    if (c->h_in) cudaFreeHost(c->h_in);
    if (c->h_out) cudaFreeHost(c->h_out);
    if (c->h_q) cudaFreeHost(c->h_q);
    for (cudaEvent_t e : c->prof_ev) cudaEventDestroy(e);
    for (int k = 0; k < NCLASS; k++) {
        if (c->spec_st[k]) cudaStreamDestroy(c->spec_st[k]);
        if (c->spec_join[k]) cudaEventDestroy(c->spec_join[k]);
    }
    if (c->spec_fork) cudaEventDestroy(c->spec_fork);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int poyalgn_cm_build(poyalgn_ctx* ctx, const int32_t* tcm, int alph, int gap_open,
                     poyalgn_cm** out)
{
    if (!ctx || !tcm || !out) return set_err(POYALGN_EINVAL, "null argument");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    poyalgn_cm* m = new (std::nothrow) poyalgn_cm;
    if (!m) return set_err(POYALGN_ENOMEM, "cost matrix allocation");
    rc = build_cm(&m->h, tcm, alph, gap_open);
    if (rc) {
        delete m;
        return set_err(rc == -1 ? POYALGN_EUNSUPPORTED : POYALGN_EINVAL,
                       "cost matrix rejected (alph %d, gap_open %d)", alph, gap_open);
    }
    if ((rc = upload_cm(m))) {
        delete m;
        return rc;
    }
    *out = m;
    return 0;
}

int poyalgn_cm_adopt(poyalgn_ctx* ctx, int lcm, int gap, int a_sz, int combinations,
                     int cost_model, int gap_open, const int32_t* cost,
                     const uint8_t* median, const int32_t* worst, const int32_t* tail,
                     const int32_t* prepend, poyalgn_cm** out)
{
    if (!ctx || !cost || !median || !worst || !tail || !prepend || !out)
        return set_err(POYALGN_EINVAL, "null argument");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    poyalgn_cm* m = new (std::nothrow) poyalgn_cm;
    if (!m) return set_err(POYALGN_ENOMEM, "cost matrix allocation");
    if (adopt_cm(&m->h, lcm, gap, a_sz, combinations, cost_model, gap_open, cost, median,
                 worst, tail, prepend)) {
        delete m;
        return set_err(POYALGN_EUNSUPPORTED, "only bitset alphabets with lcm <= 5");
    }
    if ((rc = upload_cm(m))) {
        delete m;
        return rc;
    }
    *out = m;
    return 0;
}

int poyalgn_cm_tables(const poyalgn_cm* m, int32_t* cost, uint8_t* median, int32_t* worst,
                      int32_t* tail, int32_t* prepend, int32_t* info)
{
    if (!m) return set_err(POYALGN_EINVAL, "null cost matrix");
    const int n = 2 * (1 << m->h.lcm) * (1 << m->h.lcm);
    if (cost) memcpy(cost, m->h.cost, (size_t)n * 4);
    if (worst) memcpy(worst, m->h.worst, (size_t)n * 4);
    if (tail) memcpy(tail, m->h.tail, (size_t)n * 4);
    if (prepend) memcpy(prepend, m->h.prepend, (size_t)n * 4);
    if (median) memcpy(median, m->h.median, (size_t)n);
    if (info) {
        info[0] = m->h.lcm;
        info[1] = m->h.gap;
        info[2] = m->h.a_sz;
        info[3] = m->h.combinations;
        info[4] = m->h.cost_model;
        info[5] = m->h.gap_open;
        info[6] = m->h.mnz;
    }
    return n;
}

void poyalgn_cm_free(poyalgn_cm* m)
{
    if (!m) return;
    if (m->d) cudaFree(m->d);
    delete m;
}

int poyalgn_simple_2(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* s1, int l1,
                     const uint8_t* s2, int l2, int deltawh, int32_t* cost)
{
    if (!ctx || !cm || !s1 || !s2 || !cost) return set_err(POYALGN_EINVAL, "null argument");
    if (l1 < 1 || l2 < 1) return set_err(POYALGN_EINVAL, "empty sequence");
    if (l1 > l2)  // the reference's assert (src/algn.c:1139) is compiled out there
        return set_err(POYALGN_EUNSUPPORTED,
                       "s1 (%d) longer than s2 (%d): the band arithmetic of algn_fill_plane_2 "
                       "assumes the shorter sequence first", l1, l2);
    int rc;
    ctx->call_valid = false;
    if ((rc = ensure_device(ctx))) return rc;
    // one pinned copy in; a one-pair batch with the caller's deltawh and no
    // reordering (its first band passes speculative); the final fill stays
    // in its arena region (or its pipeline's slab) for backtrace_2d, whose
    // tie preference is not known yet, so no traceback runs here
    CallPair cp;
    if ((rc = stage_call(ctx, s1, l1, s2, l2, 0, deltawh, &cp))) return rc;
    const int pcap = l1 + l2 + 2;
    if ((rc = reserve(ctx->ints, 16 * sizeof(int)))) return rc;
    if ((rc = reserve(ctx->bytes, (size_t)4 * pcap))) return rc;
    int* ints = as<int>(ctx->ints);
    uint8_t* bytes = as<uint8_t>(ctx->bytes);
    ctx->skip_deferred = true;
    rc = run_batch(ctx, cm, 0, 1, l1 + l2, pcap, cp.seqs, cp.offa, cp.lena, cp.offa + 1,
                   cp.lena + 1, cp.offa + 2, ints + 0, ints + 1, ints + 2, ints + 3, ints + 4,
                   ints + 5, bytes, bytes + pcap, bytes + 2 * pcap, bytes + 3 * pcap, ints + 6,
                   cp.dwh, cp.tie, 1, ctx->stream);
    ctx->skip_deferred = false;
    if (rc) return rc;
    const int* h;
    if ((rc = fetch_call(ctx, 0, &h))) return rc;
    if (h[5] != 0) return set_err(POYALGN_EUNSUPPORTED, "pair rejected (status %d)", h[5]);
    *cost = h[0];
    ctx->call_valid = true;
    ctx->call_affine = 0;
    ctx->call_dwh = deltawh;
    ctx->call_cm = cm;
    ctx->call_l1 = l1;
    ctx->call_l2 = l2;
    ctx->call_s1.assign(s1, s1 + l1);
    ctx->call_s2.assign(s2, s2 + l2);
    return 0;
}

int poyalgn_backtrace_2d(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* s1, int l1,
                         const uint8_t* s2, int l2, uint8_t* s1p, uint8_t* s2p, int cap,
                         int32_t* len, int swap)
{
    if (!ctx || !cm || !s1 || !s2 || !s1p || !s2p || !len)
        return set_err(POYALGN_EINVAL, "null argument");
    if (!ctx->call_valid || ctx->call_affine || ctx->call_l1 != l1 || ctx->call_l2 != l2 ||
        memcmp(ctx->call_s1.data(), s1, l1) || memcmp(ctx->call_s2.data(), s2, l2))
        return set_err(POYALGN_EINVAL, "backtrace_2d needs the fill of simple_2 on the same pair");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    // the kept fill of simple_2, walked by one warp through the shared-memory
    // window with this call's tie preference; one pinned copy of the results
    const int pcap = l1 + l2 + 2;
    *reinterpret_cast<int*>(ctx->h_in + CALL_TIE) = swap ? 1 : 0;
    CU(cudaMemcpyAsync(static_cast<uint8_t*>(ctx->callblk.p) + CALL_TIE, ctx->h_in + CALL_TIE,
                       sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    const uint8_t* blk = as<uint8_t>(ctx->callblk);
    int* ints = as<int>(ctx->ints);
    uint8_t* bytes = as<uint8_t>(ctx->bytes);
    BatchArgs A;
    memset(&A, 0, sizeof(A));
    A.seqs = blk;
    A.offa = reinterpret_cast<const long long*>(blk);
    A.lena = reinterpret_cast<const int*>(blk + 24);
    A.offb = A.offa + 1;
    A.lenb = A.lena + 1;
    A.out_off = A.offa + 2;
    A.npairs = 1;
    A.lad = ctx->lad[0];
    A.tables = cm->d;
    A.slab = as<uint8_t>(ctx->slab);
    A.dm_arena = as<uint8_t>(ctx->dmarena);
    A.dm_off = as<long long>(ctx->dmoff);
    A.cost = ints + 0;
    A.maxcost = ints + 1;
    A.alen = ints + 2;
    A.mlen = ints + 3;
    A.wlen = ints + 4;
    A.status = ints + 5;
    A.passes = ints + 6;
    A.lastcls = as<int>(ctx->lastcls);
    A.slab_cta = as<int>(ctx->slabcta);
    A.swap_override = reinterpret_cast<const int*>(blk + CALL_TIE);
    A.ea = bytes;
    A.eb = bytes + pcap;
    A.med = bytes + 2 * pcap;
    A.mwg = bytes + 3 * pcap;
    launch_call_traceback_lin(A, as<long long>(ctx->strides), ctx->stream);
    CU(cudaGetLastError());
    const int* h;
    if ((rc = fetch_call(ctx, (size_t)2 * pcap, &h))) return rc;
    if (h[5] != 0) return set_err(POYALGN_EINVAL, "traceback failed (status %d)", h[5]);
    const int L = h[2];
    if (L > cap) return set_err(POYALGN_EINVAL, "capacity %d < aligned length %d", cap, L);
    const uint8_t* hb = ctx->h_out + 32;
    const uint8_t* ea = hb + (pcap - L);
    const uint8_t* eb = hb + pcap + (pcap - L);
    // the traceback writes caller order; with swap the first sequence is y
    memcpy(s1p + cap - L, swap ? eb : ea, (size_t)L);
    memcpy(s2p + cap - L, swap ? ea : eb, (size_t)L);
    *len = L;
    return 0;
}

int poyalgn_align_2d(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* s1, int l1,
                     const uint8_t* s2, int l2, uint8_t* s1p, uint8_t* s2p, int cap,
                     int32_t* len, int deltawh, int swap, int32_t* cost)
{
    int rc = poyalgn_simple_2(ctx, cm, s1, l1, s2, l2, deltawh, cost);
    if (rc) return rc;
    return poyalgn_backtrace_2d(ctx, cm, s1, l1, s2, l2, s1p, s2p, cap, len, swap);
}

int poyalgn_align_affine_3(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* si, int li,
                           const uint8_t* sj, int lj, uint8_t* resi, uint8_t* resj,
                           uint8_t* median, uint8_t* medianwg, int cap, int32_t* lens,
                           int swaped, int32_t* cost)
{
    if (!ctx || !cm || !si || !sj || !resi || !resj || !median || !medianwg || !lens || !cost)
        return set_err(POYALGN_EINVAL, "null argument");
    if (lj < li) return set_err(POYALGN_EINVAL, "pass the shorter one as first");
    if (li < 1 || (li == 1 && lj == 1)) return set_err(POYALGN_EINVAL, "empty sequences");
    int rc;
    ctx->call_valid = false;
    if ((rc = ensure_device(ctx))) return rc;
    // one pinned copy in; the pair runs as a one-pair DOS.median batch with
    // the caller's tie preference (its first band passes speculative, the
    // traceback from its arena region); one pinned copy of the results out
    CallPair cp;
    if ((rc = stage_call(ctx, si, li, sj, lj, swaped ? 1 : 0, 0, &cp))) return rc;
    const int pcap = li + lj + 2;
    if ((rc = reserve(ctx->ints, 16 * sizeof(int)))) return rc;
    if ((rc = reserve(ctx->bytes, (size_t)4 * pcap))) return rc;
    int* ints = as<int>(ctx->ints);
    uint8_t* bytes = as<uint8_t>(ctx->bytes);
    if ((rc = run_batch(ctx, cm, 1, 1, li + lj, pcap, cp.seqs, cp.offa, cp.lena, cp.offa + 1,
                        cp.lena + 1, cp.offa + 2, ints + 0, ints + 1, ints + 2, ints + 3,
                        ints + 4, ints + 5, bytes, bytes + pcap, bytes + 2 * pcap,
                        bytes + 3 * pcap, ints + 6, nullptr, cp.tie, 1, ctx->stream)))
        return rc;
    const int* h;
    if ((rc = fetch_call(ctx, (size_t)4 * pcap, &h))) return rc;
    if (h[5] != 0) return set_err(POYALGN_EUNSUPPORTED, "pair rejected (status %d)", h[5]);
    const int L = h[2], ML = h[3], WL = h[4];
    if (L > cap || ML > cap || WL > cap) return set_err(POYALGN_EINVAL, "capacity %d too small", cap);
    const uint8_t* hb = ctx->h_out + 32;
    const uint8_t* ea = hb + (pcap - L);
    const uint8_t* eb = hb + pcap + (pcap - L);
    // the traceback writes caller order; with swaped the first sequence is sj's side
    memcpy(resi + cap - L, swaped ? eb : ea, (size_t)L);
    memcpy(resj + cap - L, swaped ? ea : eb, (size_t)L);
    memcpy(median + cap - ML, hb + 2 * pcap + (pcap - ML), (size_t)ML);
    memcpy(medianwg + cap - WL, hb + 3 * pcap + (pcap - WL), (size_t)WL);
    *cost = h[0];
    lens[0] = L;
    lens[1] = ML;
    lens[2] = WL;
    return 0;
}

// every state of an aligned pair indexes the cost matrix's tables
static int check_aligned_states(const poyalgn_cm* cm, const uint8_t* a, const uint8_t* b, int len)
{
    const int ns = 1 << cm->h.lcm;
    for (int i = 0; i < len; i++)
        if (a[i] >= ns || b[i] >= ns)
            return set_err(POYALGN_EINVAL, "state %d at position %d outside the alphabet",
                           a[i] >= ns ? a[i] : b[i], i);
    return 0;
}

int poyalgn_aligned_medians(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* a,
                            const uint8_t* b, int len, uint8_t* ancestor, int cap,
                            int32_t* anc_len, uint8_t* median_wg, int32_t* worst)
{
    if (!ctx || !cm || !a || !b || !ancestor || !anc_len || !median_wg || !worst)
        return set_err(POYALGN_EINVAL, "null argument");
    if (len < 1) return set_err(POYALGN_EINVAL, "empty alignment");
    int rc;
    if ((rc = check_aligned_states(cm, a, b, len))) return rc;
    if ((rc = ensure_device(ctx))) return rc;
    if ((rc = reserve(ctx->seqs, (size_t)2 * len))) return rc;
    if ((rc = reserve(ctx->bytes, (size_t)2 * len + 2))) return rc;
    if ((rc = reserve(ctx->ints, 16 * sizeof(int)))) return rc;
    uint8_t* d = as<uint8_t>(ctx->seqs);
    uint8_t* o = as<uint8_t>(ctx->bytes);
    CU(cudaMemcpyAsync(d, a, len, cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaMemcpyAsync(d + len, b, len, cudaMemcpyHostToDevice, ctx->stream));
    launch_aligned_medians(cm->d, d, d + len, len, o, o + len + 1, as<int>(ctx->ints), ctx->stream);
    CU(cudaGetLastError());
    int h[3];
    CU(cudaMemcpyAsync(h, ctx->ints.p, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    if (h[2] != 0) return set_err(POYALGN_EINVAL, "median should not be 0");
    if (h[0] > cap) return set_err(POYALGN_EINVAL, "ancestor capacity %d < %d", cap, h[0]);
    CU(cudaMemcpy(ancestor + cap - h[0], o, h[0], cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(median_wg, o + len + 1, len, cudaMemcpyDeviceToHost));
    *anc_len = h[0];
    *worst = h[1];
    return 0;
}

// algn_verify_2 / seq_get_median_2d_no_gaps of an aligned pair on the
// device: res = {verify cost, no-gap median length}; the median is left in
// ctx->bytes[0, res[1]).
static int aligned_extra(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* a,
                         const uint8_t* b, int len, int res[2])
{
    if (!ctx || !cm || !a || !b) return set_err(POYALGN_EINVAL, "null argument");
    if (len < 1) return set_err(POYALGN_EINVAL, "empty alignment");
    int rc;
    if ((rc = check_aligned_states(cm, a, b, len))) return rc;
    if ((rc = ensure_device(ctx))) return rc;
    if ((rc = reserve(ctx->seqs, (size_t)2 * len))) return rc;
    if ((rc = reserve(ctx->bytes, (size_t)len + 1))) return rc;
    if ((rc = reserve(ctx->ints, 16 * sizeof(int)))) return rc;
    uint8_t* d = as<uint8_t>(ctx->seqs);
    CU(cudaMemcpyAsync(d, a, len, cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaMemcpyAsync(d + len, b, len, cudaMemcpyHostToDevice, ctx->stream));
    launch_aligned_extra(cm->d, d, d + len, len, as<uint8_t>(ctx->bytes), as<int>(ctx->ints),
                         ctx->stream);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(res, ctx->ints.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int poyalgn_verify_2(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* a, const uint8_t* b,
                     int len, int32_t* cost)
{
    if (!cost) return set_err(POYALGN_EINVAL, "null argument");
    int res[2], rc;
    if ((rc = aligned_extra(ctx, cm, a, b, len, res))) return rc;
    *cost = res[0];
    return 0;
}

int poyalgn_median_2_no_gaps(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* a,
                             const uint8_t* b, int len, uint8_t* median, int cap,
                             int32_t* median_len)
{
    if (!median || !median_len) return set_err(POYALGN_EINVAL, "null argument");
    int res[2], rc;
    if ((rc = aligned_extra(ctx, cm, a, b, len, res))) return rc;
    if (res[1] > cap) return set_err(POYALGN_EINVAL, "median capacity %d < %d", cap, res[1]);
    CU(cudaMemcpy(median + cap - res[1], ctx->bytes.p, res[1], cudaMemcpyDeviceToHost));
    *median_len = res[1];
    return 0;
}

int poyalgn_limit_2(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* s1, int l1,
                    const uint8_t* s2, int l2, int w, int h, int s1_st, int s2_st, int s1_len,
                    int s2_len, int32_t* cost)
{
    (void)h;
    (void)s1_st;
    (void)s2_st;
    // algn_nw_limit fills the whole plane of (s1, s2); the window lengths
    // only replace the full lengths in the plane choice's height, which
    // simple_2 computes as (l1 - l2) + 50 + deltawh
    return poyalgn_simple_2(ctx, cm, s1, l1, s2, l2, w + (s1_len - s2_len) - (l1 - l2), cost);
}

int poyalgn_backtrace_2d_limit(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* s1, int l1,
                               const uint8_t* s2, int l2, uint8_t* s1p, uint8_t* s2p, int cap,
                               int32_t* len, int st_s1, int st_s2, int algn_s1, int algn_s2,
                               int swaped)
{
    if (st_s1 == 0 && st_s2 == 0 && algn_s1 == l1 && algn_s2 == l2)
        return poyalgn_backtrace_2d(ctx, cm, s1, l1, s2, l2, s1p, s2p, cap, len, swaped);
    if (!ctx || !cm || !s1 || !s2 || !s1p || !s2p || !len)
        return set_err(POYALGN_EINVAL, "null argument");
    if (!ctx->call_valid || ctx->call_affine || ctx->call_l1 != l1 || ctx->call_l2 != l2 ||
        memcmp(ctx->call_s1.data(), s1, l1) || memcmp(ctx->call_s2.data(), s2, l2))
        return set_err(POYALGN_EINVAL,
                       "backtrace_2d_limit needs the fill of simple_2 / limit_2 on the same pair");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    // the walk writes at most one column per counter step: l1 + l2 columns
    const int wcap = l1 + l2 + 2;
    uint8_t* bytes = as<uint8_t>(ctx->bytes);  // staged with 4 (l1 + l2 + 2) bytes
    int* out2 = as<int>(ctx->ints) + 8;
    LimitWalk w;
    w.t = cm->d;
    w.slab = as<uint8_t>(ctx->slab);
    w.strides = as<long long>(ctx->strides);
    w.lastcls = as<int>(ctx->lastcls);
    w.slab_cta = as<int>(ctx->slabcta);
    w.passes = as<int>(ctx->ints) + 6;  // written by the kept fill
    w.pfull = as<int>(ctx->pfull);
    w.dm_off = as<long long>(ctx->dmoff);
    w.dm_arena = as<uint8_t>(ctx->dmarena);
    w.lad = ctx->lad[0];
    w.s1 = as<uint8_t>(ctx->callblk) + CALL_SEQ;
    w.s2 = as<uint8_t>(ctx->callblk) + CALL_SEQ + l1;
    w.l1 = l1;
    w.l2 = l2;
    w.deltawh = ctx->call_dwh;
    w.st_s1 = st_s1;
    w.st_s2 = st_s2;
    w.algn_s1 = algn_s1;
    w.algn_s2 = algn_s2;
    w.swaped = swaped ? 1 : 0;
    w.cap = wcap;
    w.r1 = bytes;
    w.r2 = bytes + wcap;
    w.out2 = out2;
    launch_limit_walk(w, ctx->stream);
    CU(cudaGetLastError());
    int h[2];
    CU(cudaMemcpyAsync(h, out2, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    if (h[0] == -14)
        return set_err(POYALGN_EUNSUPPORTED,
                       "backtrace_2d_limit from (%d, %d, %d, %d) reaches a cell the last fill "
                       "never wrote (the reference reads what earlier alignments left there)",
                       st_s1, st_s2, algn_s1, algn_s2);
    if (h[0] == -15)
        return set_err(POYALGN_EINVAL, "backtrace_2d_limit start (%d, %d, %d, %d) leaves the "
                       "sequences", st_s1, st_s2, algn_s1, algn_s2);
    if (h[0] != 0) return set_err(POYALGN_EINVAL, "backtrace_2d_limit walk failed (%d)", h[0]);
    const int L = h[1];
    if (L > cap) return set_err(POYALGN_EINVAL, "capacity %d < aligned length %d", cap, L);
    CU(cudaMemcpy(s1p + cap - L, bytes + wcap - L, L, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(s2p + cap - L, bytes + 2 * wcap - L, L, cudaMemcpyDeviceToHost));
    *len = L;
    return 0;
}

int poyalgn_median_batch_device(poyalgn_ctx* ctx, const poyalgn_cm* cm, int npairs,
                                int max_pair_len, int64_t out_bytes, const uint8_t* seqs,
                                const int64_t* offa, const int32_t* lena, const int64_t* offb,
                                const int32_t* lenb, const int64_t* out_off, int32_t* cost,
                                int32_t* maxcost, int32_t* alen, int32_t* mlen, int32_t* wlen,
                                int32_t* status, uint8_t* ea, uint8_t* eb, uint8_t* med,
                                uint8_t* mwg, int32_t* passes, void* stream)
{
    if (!ctx || !cm) return set_err(POYALGN_EINVAL, "null argument");
    if (npairs < 0 || max_pair_len < 2 || out_bytes < 1) return set_err(POYALGN_EINVAL, "bad batch shape");
    if (npairs == 0) return 0;
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    return run_batch(ctx, cm, cm->h.cost_model == 1, npairs, max_pair_len, out_bytes, seqs,
                     reinterpret_cast<const long long*>(offa), lena,
                     reinterpret_cast<const long long*>(offb), lenb,
                     reinterpret_cast<const long long*>(out_off), cost, maxcost, alen, mlen,
                     wlen, status, ea, eb, med, mwg, passes, nullptr, nullptr, 1,
                     (cudaStream_t)stream);
}

int poyalgn_median_batch(poyalgn_ctx* ctx, const poyalgn_cm* cm, int npairs,
                         const uint8_t* seqs, const int64_t* offa, const int32_t* lena,
                         const int64_t* offb, const int32_t* lenb, const int64_t* out_off,
                         int32_t* cost, int32_t* maxcost, int32_t* alen, int32_t* mlen,
                         int32_t* wlen, int32_t* status, uint8_t* ea, uint8_t* eb,
                         uint8_t* med, uint8_t* mwg, int32_t* passes)
{
    if (!ctx || !cm || (npairs > 0 && (!seqs || !offa || !lena || !offb || !lenb || !out_off ||
                                       !cost || !maxcost || !alen || !mlen || !wlen || !status ||
                                       !ea || !eb || !med || !mwg)))
        return set_err(POYALGN_EINVAL, "null argument");
    if (npairs <= 0) return 0;
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    long long seq_bytes = 0, out_total = 0;
    int maxmn = 2;
    for (int k = 0; k < npairs; k++) {
        if (lena[k] < 1 || lenb[k] < 1) return set_err(POYALGN_EINVAL, "pair %d: empty sequence", k);
        seq_bytes = std::max<long long>(seq_bytes, std::max(offa[k] + lena[k], offb[k] + lenb[k]));
        out_total = std::max<long long>(out_total, out_off[k] + lena[k] + lenb[k] + 2);
        maxmn = std::max(maxmn, lena[k] + lenb[k]);
    }
    const size_t ni = (size_t)npairs;
    if ((rc = reserve(ctx->seqs, (size_t)seq_bytes))) return rc;
    if ((rc = reserve(ctx->offa, ni * 8))) return rc;
    if ((rc = reserve(ctx->offb, ni * 8))) return rc;
    if ((rc = reserve(ctx->lena, ni * 4))) return rc;
    if ((rc = reserve(ctx->lenb, ni * 4))) return rc;
    if ((rc = reserve(ctx->outoff, ni * 8))) return rc;
    if ((rc = reserve(ctx->ints, ni * 4 * 7))) return rc;
    if ((rc = reserve(ctx->bytes, (size_t)out_total * 4))) return rc;
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(ctx->seqs.p, seqs, (size_t)seq_bytes, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->offa.p, offa, ni * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->offb.p, offb, ni * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->lena.p, lena, ni * 4, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->lenb.p, lenb, ni * 4, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->outoff.p, out_off, ni * 8, cudaMemcpyHostToDevice, st));
    int* I = as<int>(ctx->ints);
    uint8_t* B = as<uint8_t>(ctx->bytes);
    const size_t ot = (size_t)out_total;
    if ((rc = run_batch(ctx, cm, cm->h.cost_model == 1, npairs, maxmn, out_total,
                        as<uint8_t>(ctx->seqs), as<long long>(ctx->offa), as<int>(ctx->lena),
                        as<long long>(ctx->offb), as<int>(ctx->lenb), as<long long>(ctx->outoff),
                        I, I + ni, I + 2 * ni, I + 3 * ni, I + 4 * ni, I + 5 * ni, B, B + ot,
                        B + 2 * ot, B + 3 * ot, I + 6 * ni, nullptr, nullptr, 1, st)))
        return rc;
    int32_t* outs[7] = {cost, maxcost, alen, mlen, wlen, status, passes};
    for (int j = 0; j < 7; j++)
        if (outs[j]) CU(cudaMemcpyAsync(outs[j], I + j * ni, ni * 4, cudaMemcpyDeviceToHost, st));
    uint8_t* bo[4] = {ea, eb, med, mwg};
    for (int j = 0; j < 4; j++)
        CU(cudaMemcpyAsync(bo[j], B + j * ot, ot, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    for (int k = 0; k < npairs; k++)
        if (status[k] != 0) return set_err(POYALGN_EPAIR, "pair %d failed with status %d", k, status[k]);
    return 0;
}

int poyalgn_last_launches(const poyalgn_ctx* ctx) { return ctx ? ctx->last_launches : 0; }

int poyalgn_profile_begin(poyalgn_ctx* ctx, int max_batches)
{
    if (!ctx || max_batches < 0) return set_err(POYALGN_EINVAL, "bad argument");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    for (cudaEvent_t e : ctx->prof_ev) cudaEventDestroy(e);
    ctx->prof_ev.assign((size_t)max_batches * (NCLASS + 2), nullptr);
    for (auto& e : ctx->prof_ev) CU(cudaEventCreate(&e));
    ctx->prof_cap = max_batches;
    ctx->prof_used = 0;
    return 0;
}

int poyalgn_profile_end(poyalgn_ctx* ctx, float* ms, int* batches)
{
    if (!ctx || !ms || !batches) return set_err(POYALGN_EINVAL, "bad argument");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    for (int k = 0; k < NCLASS + 1; k++) ms[k] = 0.f;
    for (int b = 0; b < ctx->prof_used; b++) {
        cudaEvent_t* ev = &ctx->prof_ev[(size_t)b * (NCLASS + 2)];
        CU(cudaEventSynchronize(ev[NCLASS + 1]));
        for (int k = 0; k < NCLASS + 1; k++) {
            float t = 0.f;
            CU(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            ms[k] += t;
        }
    }
    *batches = ctx->prof_used;
    for (cudaEvent_t e : ctx->prof_ev) cudaEventDestroy(e);
    ctx->prof_ev.clear();
    ctx->prof_cap = ctx->prof_used = 0;
    return 0;
}

int poyalgn_num_classes(void) { return NCLASS; }

int poyalgn_set_memory_budget(poyalgn_ctx* ctx, int64_t slab_bytes, int64_t arena_bytes)
{
    if (!ctx || slab_bytes < 0 || arena_bytes < 0) return set_err(POYALGN_EINVAL, "bad budget");
    ctx->slab_cap = slab_bytes;
    ctx->arena_cap = arena_bytes;
    return 0;
}

struct poyalgn_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int device = 0;
};

int poyalgn_batch_graph_create(poyalgn_ctx* ctx, const poyalgn_cm* cm, int npairs,
                               int max_pair_len, int64_t out_bytes, const uint8_t* seqs,
                               const int64_t* offa, const int32_t* lena, const int64_t* offb,
                               const int32_t* lenb, const int64_t* out_off, int32_t* cost,
                               int32_t* maxcost, int32_t* alen, int32_t* mlen, int32_t* wlen,
                               int32_t* status, uint8_t* ea, uint8_t* eb, uint8_t* med,
                               uint8_t* mwg, int32_t* passes, poyalgn_graph** out)
{
    if (!ctx || !cm || !out || npairs < 1 || max_pair_len < 2 || out_bytes < 1)
        return set_err(POYALGN_EINVAL, "bad graph arguments");
    *out = nullptr;
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    const int affine = cm->h.cost_model == 1;
    auto batch = [&](cudaStream_t st) {
        return run_batch(ctx, cm, affine, npairs, max_pair_len, out_bytes, seqs,
                         reinterpret_cast<const long long*>(offa), lena,
                         reinterpret_cast<const long long*>(offb), lenb,
                         reinterpret_cast<const long long*>(out_off), cost, maxcost, alen, mlen,
                         wlen, status, ea, eb, med, mwg, passes, nullptr, nullptr, 1, st);
    };
    // one plain run reserves every buffer the captured launches use
    if ((rc = batch(ctx->stream))) return rc;
    CU(cudaStreamSynchronize(ctx->stream));
    poyalgn_graph* g = new (std::nothrow) poyalgn_graph;
    if (!g) return set_err(POYALGN_ENOMEM, "graph allocation");
    g->device = ctx->device;
    CU(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    rc = batch(ctx->stream);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (rc || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        delete g;
        cudaGetLastError();
        return rc ? rc : set_err(POYALGN_ECUDA, "capture: %s", cudaGetErrorString(e));
    }
    g->graph = graph;
    if (cudaGraphInstantiate(&g->exec, graph, 0) != cudaSuccess) {
        cudaGraphDestroy(graph);
        delete g;
        cudaGetLastError();
        return set_err(POYALGN_ECUDA, "graph instantiation failed");
    }
    *out = g;
    return 0;
}

int poyalgn_batch_graph_launch(poyalgn_graph* g, void* stream)
{
    if (!g) return set_err(POYALGN_EINVAL, "null graph");
    CU(cudaSetDevice(g->device));
    CU(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    return 0;
}

void poyalgn_batch_graph_free(poyalgn_graph* g)
{
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
}

int poyalgn_set_row_tile(poyalgn_ctx* ctx, int mode)
{
    if (!ctx || mode < 0 || mode > 2) return set_err(POYALGN_EINVAL, "bad row tile mode");
    ctx->row_tile_mode = mode;
    ctx->call_valid = false;
    return 0;
}

int poyalgn_set_speculation(poyalgn_ctx* ctx, int mode, int passes)
{
    if (!ctx || mode < 0 || mode > 2 || passes < 1 || passes > POYALGN_SPEC_MAX_PASSES)
        return set_err(POYALGN_EINVAL, "bad speculation mode %d / passes %d", mode, passes);
    ctx->spec_mode = mode;
    ctx->spec_passes = passes;
    return 0;
}

int poyalgn_cost_affine_3(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* si, int li,
                          const uint8_t* sj, int lj, int32_t* cost)
{
    if (!ctx || !cm || !si || !sj || !cost || li < 1 || lj < 1)
        return set_err(POYALGN_EINVAL, "null argument");
    if (cm->h.cost_model != 1) return set_err(POYALGN_EINVAL, "cost matrix is not affine");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    CallPair cp;
    if ((rc = stage_call(ctx, si, li, sj, lj, 0, 0, &cp))) return rc;
    if ((rc = reserve(ctx->ints, 16 * sizeof(int)))) return rc;
    int* I = as<int>(ctx->ints);
    if ((rc = run_nobt(ctx, cm, 1, li + lj, cp.seqs, cp.offa, cp.lena, cp.offa + 1, cp.lena + 1,
                       NOBT_NO_MISSING, I, I + 1, ctx->stream)))
        return rc;
    const int* h;
    if ((rc = fetch_call(ctx, 0, &h))) return rc;
    if (h[1] != 0) return set_err(POYALGN_EUNSUPPORTED, "pair rejected (status %d)", h[1]);
    *cost = h[0];
    return 0;
}

int poyalgn_distance_batch_device(poyalgn_ctx* ctx, const poyalgn_cm* cm, int npairs,
                                  int max_pair_len, const uint8_t* seqs, const int64_t* offa,
                                  const int32_t* lena, const int64_t* offb, const int32_t* lenb,
                                  int32_t missing_distance, int32_t* cost, int32_t* status,
                                  void* stream)
{
    if (!ctx || !cm) return set_err(POYALGN_EINVAL, "null argument");
    if (npairs < 0 || max_pair_len < 2) return set_err(POYALGN_EINVAL, "bad batch shape");
    if (npairs == 0) return 0;
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    const long long* oa = reinterpret_cast<const long long*>(offa);
    const long long* ob = reinterpret_cast<const long long*>(offb);
    cudaStream_t st = (cudaStream_t)stream;
    if (cm->h.cost_model == 1)
        return run_nobt(ctx, cm, npairs, max_pair_len, seqs, oa, lena, ob, lenb,
                        missing_distance, cost, status, st);
    return run_batch(ctx, cm, 0, npairs, max_pair_len, 1, seqs, oa, lena, ob, lenb, nullptr,
                     cost, nullptr, nullptr, nullptr, nullptr, status, nullptr, nullptr, nullptr,
                     nullptr, nullptr, nullptr, nullptr, 0, st, 1, missing_distance);
}

int poyalgn_distance_batch(poyalgn_ctx* ctx, const poyalgn_cm* cm, int npairs,
                           const uint8_t* seqs, const int64_t* offa, const int32_t* lena,
                           const int64_t* offb, const int32_t* lenb, int32_t missing_distance,
                           int32_t* cost, int32_t* status)
{
    if (!ctx || !cm || (npairs > 0 && (!seqs || !offa || !lena || !offb || !lenb || !cost ||
                                       !status)))
        return set_err(POYALGN_EINVAL, "null argument");
    if (npairs <= 0) return 0;
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    long long seq_bytes = 0;
    int maxmn = 2;
    for (int k = 0; k < npairs; k++) {
        if (lena[k] < 1 || lenb[k] < 1) return set_err(POYALGN_EINVAL, "pair %d: empty sequence", k);
        seq_bytes = std::max<long long>(seq_bytes, std::max(offa[k] + lena[k], offb[k] + lenb[k]));
        maxmn = std::max(maxmn, lena[k] + lenb[k]);
    }
    const size_t ni = (size_t)npairs;
    if ((rc = reserve(ctx->seqs, (size_t)seq_bytes))) return rc;
    if ((rc = reserve(ctx->offa, ni * 8))) return rc;
    if ((rc = reserve(ctx->offb, ni * 8))) return rc;
    if ((rc = reserve(ctx->lena, ni * 4))) return rc;
    if ((rc = reserve(ctx->lenb, ni * 4))) return rc;
    if ((rc = reserve(ctx->ints, ni * 4 * 2))) return rc;
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(ctx->seqs.p, seqs, (size_t)seq_bytes, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->offa.p, offa, ni * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->offb.p, offb, ni * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->lena.p, lena, ni * 4, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->lenb.p, lenb, ni * 4, cudaMemcpyHostToDevice, st));
    int* I = as<int>(ctx->ints);
    if ((rc = poyalgn_distance_batch_device(
             ctx, cm, npairs, maxmn, as<uint8_t>(ctx->seqs), as<int64_t>(ctx->offa),
             as<int>(ctx->lena), as<int64_t>(ctx->offb), as<int>(ctx->lenb), missing_distance, I,
             I + ni, st)))
        return rc;
    CU(cudaMemcpyAsync(cost, I, ni * 4, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(status, I + ni, ni * 4, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    for (int k = 0; k < npairs; k++)
        if (status[k] != 0) return set_err(POYALGN_EPAIR, "pair %d failed with status %d", k, status[k]);
    return 0;
}

int poyalgn_set_ladder(poyalgn_ctx* ctx, int affine, const int32_t* P, const int32_t* R)
{
    if (!ctx || !P || !R || (affine != 0 && affine != 1)) return set_err(POYALGN_EINVAL, "null argument");
    Ladder L;
    for (int k = 0; k < NCLASS; k++) {
        L.P[k] = P[k];
        L.R[k] = R[k];
    }
    if (!ladder_valid(L, affine)) return set_err(POYALGN_EINVAL, "ladder not supported");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    ctx->lad[affine] = L;
    for (int k = 0; k < NCLASS; k++) {
        for (int v = 0; v < 2; v++) ctx->bps[affine][k][v] = class_blocks_per_sm(L, affine, k, v, 0);
        if (affine) ctx->bps_rt[k] = class_blocks_per_sm(L, 1, k, 1, 1);
    }
    CU(cudaGetLastError());
    ctx->call_valid = false;  // a kept per-call fill was laid out for the old ladder
    return 0;
}

int poyalgn_get_ladder(const poyalgn_ctx* ctx, int affine, int32_t* P, int32_t* R)
{
    if (!ctx || !P || !R || (affine != 0 && affine != 1)) return set_err(POYALGN_EINVAL, "null argument");
    for (int k = 0; k < NCLASS; k++) {
        P[k] = ctx->lad[affine].P[k];
        R[k] = ctx->lad[affine].R[k];
    }
    return 0;
}

int poyalgn_autotune(poyalgn_ctx* ctx, const poyalgn_cm* cm, int npairs, const uint8_t* seqs,
                     const int64_t* offa, const int32_t* lena, const int64_t* offb,
                     const int32_t* lenb, int ncand, const int32_t* cand_P,
                     const int32_t* cand_R, int reps, float* ms, int32_t* best)
{
    if (!ctx || !cm || npairs < 1 || !seqs || !offa || !lena || !offb || !lenb || ncand < 1 ||
        !cand_P || !cand_R || reps < 1 || !ms || !best)
        return set_err(POYALGN_EINVAL, "null argument");
    const int affine = cm->h.cost_model == 1;
    for (int q = 0; q < ncand; q++) {
        Ladder L;
        for (int k = 0; k < NCLASS; k++) {
            L.P[k] = cand_P[q * NCLASS + k];
            L.R[k] = cand_R[q * NCLASS + k];
        }
        if (!ladder_valid(L, affine)) return set_err(POYALGN_EINVAL, "candidate %d not supported", q);
    }
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    // stage the sample once
    long long seq_bytes = 0, out_total = 0;
    int maxmn = 2;
    std::vector<long long> oo(npairs);
    for (int k = 0; k < npairs; k++) {
        if (lena[k] < 1 || lenb[k] < 1) return set_err(POYALGN_EINVAL, "pair %d: empty sequence", k);
        seq_bytes = std::max<long long>(seq_bytes, std::max(offa[k] + lena[k], offb[k] + lenb[k]));
        oo[k] = out_total;
        out_total += lena[k] + lenb[k] + 2;
        maxmn = std::max(maxmn, lena[k] + lenb[k]);
    }
    const size_t ni = (size_t)npairs;
    if ((rc = reserve(ctx->seqs, (size_t)seq_bytes))) return rc;
    if ((rc = reserve(ctx->offa, ni * 8))) return rc;
    if ((rc = reserve(ctx->offb, ni * 8))) return rc;
    if ((rc = reserve(ctx->lena, ni * 4))) return rc;
    if ((rc = reserve(ctx->lenb, ni * 4))) return rc;
    if ((rc = reserve(ctx->outoff, ni * 8))) return rc;
    if ((rc = reserve(ctx->ints, ni * 4 * 7))) return rc;
    if ((rc = reserve(ctx->bytes, (size_t)out_total * 4))) return rc;
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(ctx->seqs.p, seqs, (size_t)seq_bytes, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->offa.p, offa, ni * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->offb.p, offb, ni * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->lena.p, lena, ni * 4, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->lenb.p, lenb, ni * 4, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->outoff.p, oo.data(), ni * 8, cudaMemcpyHostToDevice, st));
    int* I = as<int>(ctx->ints);
    uint8_t* B = as<uint8_t>(ctx->bytes);
    const size_t ot = (size_t)out_total;
    auto batch = [&]() {
        return run_batch(ctx, cm, affine, npairs, maxmn, out_total, as<uint8_t>(ctx->seqs),
                         as<long long>(ctx->offa), as<int>(ctx->lena), as<long long>(ctx->offb),
                         as<int>(ctx->lenb), as<long long>(ctx->outoff), I, I + ni, I + 2 * ni,
                         I + 3 * ni, I + 4 * ni, I + 5 * ni, B, B + ot, B + 2 * ot, B + 3 * ot,
                         I + 6 * ni, nullptr, nullptr, 1, st);
    };
    const Ladder saved = ctx->lad[affine];
    int saved_bps[NCLASS][2];
    memcpy(saved_bps, ctx->bps[affine], sizeof(saved_bps));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    std::vector<int> first(2 * ni), got(2 * ni);
    std::vector<float> t(reps);
    int bi = 0;
    rc = 0;
    for (int q = 0; q < ncand && !rc; q++) {
        Ladder L;
        for (int k = 0; k < NCLASS; k++) {
            L.P[k] = cand_P[q * NCLASS + k];
            L.R[k] = cand_R[q * NCLASS + k];
            for (int v = 0; v < 2; v++)
                ctx->bps[affine][k][v] = class_blocks_per_sm(L, affine, k, v, 0);
            if (affine) ctx->bps_rt[k] = class_blocks_per_sm(L, 1, k, 1, 1);
        }
        ctx->lad[affine] = L;
        if ((rc = batch())) break;
        for (int r = 0; r < reps && !rc; r++) {
            if (cudaEventRecord(e0, st) != cudaSuccess) rc = set_err(POYALGN_ECUDA, "event");
            if (!rc) rc = batch();
            if (!rc && cudaEventRecord(e1, st) != cudaSuccess) rc = set_err(POYALGN_ECUDA, "event");
            if (!rc && (cudaEventSynchronize(e1) != cudaSuccess ||
                        cudaEventElapsedTime(&t[r], e0, e1) != cudaSuccess))
                rc = set_err(POYALGN_ECUDA, "timing candidate %d", q);
        }
        if (rc) break;
        std::vector<float> sorted(t);
        std::sort(sorted.begin(), sorted.end());
        ms[q] = sorted[reps / 2];
        // cost and status of every pair must not depend on the ladder
        std::vector<int>& dst = q == 0 ? first : got;
        if (cudaMemcpy(dst.data(), I, ni * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(dst.data() + ni, I + 5 * ni, ni * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = set_err(POYALGN_ECUDA, "reading candidate %d", q);
            break;
        }
        if (q > 0 && got != first) {
            rc = set_err(POYALGN_EINVAL, "candidate %d changed a result", q);
            break;
        }
        if (ms[q] < ms[bi]) bi = q;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
        ctx->lad[affine] = saved;
        memcpy(ctx->bps[affine], saved_bps, sizeof(saved_bps));
        return rc;
    }
    *best = bi;
    return poyalgn_set_ladder(ctx, affine, cand_P + bi * NCLASS, cand_R + bi * NCLASS);
}

}  // extern "C"

// ---- poyalgn_median_batch_device_noalloc ----------------------------------
//
// The same launch sequence as run_batch (ordering, prep, one persistent
// launch per class and variant), with every scratch buffer carved out of one
// static device array instead of cudaMalloc'd context buffers.

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[POYALGN_NOALLOC_SCRATCH_BYTES];

constexpr int kNoAllocDevices = 64;

struct NoAllocDevice {
    bool ready = false;
    unsigned char* base = nullptr;
    int nsm = 0;
    int bps[2][NCLASS][2] = {};
};

NoAllocDevice g_noalloc[kNoAllocDevices];
std::mutex g_noalloc_mu;

// One-time setup for `dev` (the current device): the region's address, the
// SM count and the per-class occupancy that sizes the persistent grids.
int noalloc_device(int dev, const NoAllocDevice** out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice& d = g_noalloc[dev];
    if (!d.ready) {
        void* p = nullptr;
        CU(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        CU(cudaDeviceGetAttribute(&d.nsm, cudaDevAttrMultiProcessorCount, dev));
        for (int a = 0; a < 2; a++)
            for (int k = 0; k < NCLASS; k++)
                for (int v = 0; v < 2; v++)
                    d.bps[a][k][v] = class_blocks_per_sm(default_ladder(a), a, k, v, 0);
        CU(cudaGetLastError());
        d.base = static_cast<unsigned char*>(p);
        d.ready = true;
    }
    *out = &d;
    return 0;
}

// Bump carving of the region in 256-byte aligned pieces.
struct Carve {
    unsigned char* base;
    size_t used, cap;
    void* take(size_t bytes)
    {
        const size_t a = (std::max<size_t>(bytes, 1) + 255) & ~(size_t)255;
        if (used + a > cap) return nullptr;
        void* r = base + used;
        used += a;
        return r;
    }
};

}  // namespace

extern "C" int poyalgn_median_batch_device_noalloc(
    const poyalgn_cm* cm, int npairs, int max_pair_len, int64_t out_bytes, const uint8_t* seqs,
    const int64_t* offa, const int32_t* lena, const int64_t* offb, const int32_t* lenb,
    const int64_t* out_off, int32_t* cost, int32_t* maxcost, int32_t* alen, int32_t* mlen,
    int32_t* wlen, int32_t* status, uint8_t* ea, uint8_t* eb, uint8_t* med, uint8_t* mwg,
    int32_t* passes, void* stream)
{
    if (!cm || (npairs > 0 && (!seqs || !offa || !lena || !offb || !lenb || !out_off || !cost ||
                               !maxcost || !alen || !mlen || !wlen || !status || !ea || !eb ||
                               !med || !mwg)))
        return set_err(POYALGN_EINVAL, "null argument");
    if (npairs < 0 || max_pair_len < 2 || out_bytes < 1) return set_err(POYALGN_EINVAL, "bad batch shape");
    if (npairs > POYALGN_NOALLOC_MAX_PAIRS)
        return set_err(POYALGN_EINVAL, "npairs %d exceeds POYALGN_NOALLOC_MAX_PAIRS (%d)", npairs,
                       POYALGN_NOALLOC_MAX_PAIRS);
    if (max_pair_len > POYALGN_NOALLOC_MAX_PAIR_LEN)
        return set_err(POYALGN_EINVAL, "max_pair_len %d exceeds POYALGN_NOALLOC_MAX_PAIR_LEN (%d)",
                       max_pair_len, POYALGN_NOALLOC_MAX_PAIR_LEN);
    if (out_bytes > POYALGN_NOALLOC_MAX_OUT_BYTES)
        return set_err(POYALGN_EINVAL, "out_bytes %lld exceeds POYALGN_NOALLOC_MAX_OUT_BYTES (%d)",
                       (long long)out_bytes, POYALGN_NOALLOC_MAX_OUT_BYTES);
    if (npairs == 0) return 0;

    int dev = -1;
    CU(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocDevices)
        return set_err(POYALGN_EUNSUPPORTED, "device ordinal %d beyond %d", dev, kNoAllocDevices - 1);
    cudaPointerAttributes pa;
    CU(cudaPointerGetAttributes(&pa, cm->d));
    if (pa.device != dev)
        return set_err(POYALGN_EINVAL, "cost matrix lives on device %d, current device is %d",
                       pa.device, dev);
    const NoAllocDevice* d = nullptr;
    int rc;
    if ((rc = noalloc_device(dev, &d))) return rc;

    const int affine = cm->h.cost_model == 1;
    const Ladder lad = default_ladder(affine);
    const size_t ni = (size_t)npairs;
    Carve cv{d->base, 0, (size_t)POYALGN_NOALLOC_SCRATCH_BYTES};
    int* qctr = static_cast<int*>(cv.take(2 * NQUEUE * sizeof(int)));
    int* pfull = static_cast<int*>(cv.take(ni * 4));
    int* eh0 = static_cast<int*>(cv.take(ni * 4));
    int* lastcls = static_cast<int*>(cv.take(ni * 4));
    int* slabcta = static_cast<int*>(cv.take(ni * 4));
    int* pass_buf = static_cast<int*>(cv.take(ni * 4));
    int* order = static_cast<int*>(cv.take(ni * 4));
    void* order_scratch = cv.take(order_scratch_bytes(npairs));
    int2* qitems = static_cast<int2*>(cv.take((size_t)NQUEUE * ni * sizeof(int2)));
    int* shadow = static_cast<int*>(cv.take((size_t)(affine ? out_bytes : 1) * 4));
    if (!qctr || !pfull || !eh0 || !lastcls || !slabcta || !pass_buf || !order ||
        !order_scratch || !qitems || !shadow)
        return set_err(POYALGN_EINVAL, "batch state does not fit POYALGN_NOALLOC_SCRATCH_BYTES");
    // the direction slabs take what is left, at least one CTA per class
    const long long budget = (long long)(cv.cap - cv.used);
    int grid[NCLASS][2];
    long long strides[NCLASS];
    long long arena = 0;
    for (int k = 0; k < NCLASS; k++) {
        strides[k] = class_slab_bytes(lad, affine, k, max_pair_len, 0);
        for (int v = 0; v < 2; v++) {
            const int pipes = class_pipes_per_cta(lad, affine, k, v, 0);
            if (strides[k] * pipes > budget)
                return set_err(POYALGN_EINVAL,
                               "max_pair_len %d leaves no room for class %d in POYALGN_NOALLOC_SCRATCH_BYTES",
                               max_pair_len, k);
            long long g = (long long)d->nsm * std::max(1, d->bps[affine][k][v]);
            g = std::min<long long>(g, (npairs + pipes - 1) / pipes);
            g = std::min<long long>(g, budget / (strides[k] * pipes));
            grid[k][v] = (int)std::max<long long>(1, g);
            arena = std::max(arena, (long long)grid[k][v] * pipes * strides[k]);
        }
    }
    uint8_t* slab = static_cast<uint8_t*>(cv.take((size_t)arena));
    if (!slab) return set_err(POYALGN_EINVAL, "direction slabs do not fit POYALGN_NOALLOC_SCRATCH_BYTES");

    cudaStream_t st = (cudaStream_t)stream;
    CU(cudaMemsetAsync(qctr, 0, 2 * NQUEUE * sizeof(int), st));

    BatchArgs A;
    memset(&A, 0, sizeof(A));
    A.seqs = seqs;
    A.offa = reinterpret_cast<const long long*>(offa);
    A.lena = lena;
    A.offb = reinterpret_cast<const long long*>(offb);
    A.lenb = lenb;
    A.npairs = npairs;
    A.max_pair_len = max_pair_len;
    A.out_bytes = out_bytes;
    A.affine = affine;
    A.do_traceback = 1;
    A.lad = lad;
    A.tables = cm->d;
    A.pfull = pfull;
    A.shadow = shadow;
    A.shadowEH0 = eh0;
    A.qitems = qitems;
    A.qcount = qctr;
    A.qhead = qctr + NQUEUE;
    A.qcap = npairs;
    A.slab = slab;
    A.out_off = reinterpret_cast<const long long*>(out_off);
    A.cost = cost;
    A.maxcost = maxcost;
    A.alen = alen;
    A.mlen = mlen;
    A.wlen = wlen;
    A.status = status;
    A.passes = passes ? passes : pass_buf;
    A.lastcls = lastcls;
    A.slab_cta = slabcta;
    A.deltawh_override = nullptr;
    A.swap_override = nullptr;
    A.ea = ea;
    A.eb = eb;
    A.med = med;
    A.mwg = mwg;
    if (launch_order(lena, lenb, npairs, order, order_scratch, st) != 0)
        return set_err(POYALGN_ECUDA, "ordering pairs failed");
    A.order = order;
    launch_prep(A, st);
    for (int k = 0; k < NCLASS; k++) {
        A.slab_stride = strides[k];
        for (int v = 0; v < (affine ? 2 : 1); v++) launch_class(A, k, v, grid[k][v], st);
    }
    CU(cudaGetLastError());
    return 0;
}
