// Algn_Newkk (src/newkkonen.c), affine cost model, on the GPU: one warp per
// pair. Each band pass (ukktest, src/newkkonen.c:1077-1153) is filled on a
// rolling schedule: lane r takes rows r, r + 32, r + 64, ..., one column
// per step and one column behind lane r - 1, so the cells above and
// above-left come from lane r - 1 by shuffle; a lane moves on to its next
// row as soon as its row ends, and lane 0 reads the previous round's last
// row from a per-warp boundary row that lane 31 writes. A step's 32
// direction codes are one contiguous 64-byte store. After the last pass
// lane 0 walks the codes back (backtrace_affine) and derives DOS.median's
// ancestor, median with gaps and worst cost.
//
// C ABI (include/poyalgn.h): poyalgn_newkk_median_batch[_device] (DOS.median
// with use_ukk, src/seqCS.ml:1043-1051), and the per-call stubs
// poyalgn_newkk_algn_affine / poyalgn_newkk_backtrace_affine /
// poyalgn_newkk_get_k (newkkonen_CAML_algn_affine, src/newkkonen.c:1473;
// newkkonen_CAML_backtrace_affine, :1788; newkkonen_CAML_get_k, :247).
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "pa_newkk.cuh"
#include "pa_runtime.h"

namespace pa {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NK_WARPS = 4;  // warps per CTA

struct NewkkArgs {
    const uint8_t* seqs;
    const long long* offa;
    const int* lena;
    const long long* offb;
    const int* lenb;
    int npairs;
    const int* order;  // optional visiting order
    const int* swp;    // optional: pairs already in internal order, their swaped flag
    const Tables* tables;
    int* ctr;          // [0] next pair, [1] pairs to rerun (band too large for a slice)
    uint16_t* arena;
    long long slice_words;  // each warp's slice of the arena
    nk::Quad* bnd;     // per warp: P, Q, ED, CD of the tile's upper row
    uint32_t* bndg;    // per warp: gap counters of that row
    int bnd_stride;    // >= the longer length of every pair
    int* tb;           // per warp: the rounds table of its pass
    int tb_stride;     // >= rounds of every pair
    int rerun;         // 1: only pairs whose status is POYALGN_PAIR_RETRY
    const long long* out_off;
    int *cost, *maxcost, *alen, *mlen, *wlen, *status, *passes, *kmax;
    uint8_t *ea, *eb, *med, *mwg;
};

__device__ __forceinline__ void load_tables_nk(Tables& st, const Tables* g)
{
    const int n = (int)(sizeof(Tables) / sizeof(int));
    const int* src = reinterpret_cast<const int*>(g);
    int* dst = reinterpret_cast<int*>(&st);
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

__device__ __forceinline__ nk::State shfl_up_state(const nk::State& v)
{
    nk::State r;
    r.P = __shfl_up_sync(FULL, v.P, 1);
    r.Q = __shfl_up_sync(FULL, v.Q, 1);
    r.ED = __shfl_up_sync(FULL, v.ED, 1);
    r.CD = __shfl_up_sync(FULL, v.CD, 1);
    r.g = __shfl_up_sync(FULL, v.g, 1);
    return r;
}

struct ArenaDir {
    const uint16_t* a;  // the pass's first word
    const int* c0;
    __device__ int operator()(int i, int j) const { return a[nk::dir_word(c0, i, j)]; }
};

// The rounds table of a pass (C0 of every round, nk::rounds_table) built by
// the warp with a scan over 32 rounds at a time; returns the pass's steps.
__device__ long long build_rounds(const nk::Band& B, int* c0)
{
    const int lane = threadIdx.x & 31;
    const int Q = B.rounds();
    int carry = 0;
    for (int q0 = 0; q0 < Q; q0 += 32) {
        const int q = q0 + lane;
        const int dl = q < Q - 1 ? B.delta(q) : 0;
        int incl = dl;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += v;
        }
        if (q < Q) c0[q] = carry + incl - dl;
        carry += __shfl_sync(FULL, incl, 31);
    }
    __syncwarp();
    return B.steps(c0[Q - 1]);
}

// One band pass of the warp at half-width k on the rolling schedule into
// the arena words from `dm`; returns the last cell's cost (all lanes) and
// its gap counters.
__device__ int fill_pass(const Tables& t, const uint8_t* s1, int l1, const uint8_t* s2, int l2,
                         int k, int go, uint16_t* dm, long long steps, nk::Quad* bnd,
                         uint32_t* bndg, const int* c0, uint32_t& glast)
{
    const int lane = threadIdx.x & 31;
    const nk::Band B{l1, l2, k};
    nk::Lane L;
    nk::lane_start(L, B, s1, lane);
    for (long long st = 0; st < steps; st++) {
        int j = 0;
        const int dir = nk::lane_step(L, t, s1, s2, B, c0, lane, st, bnd, bndg, go, j);
        if (dir >= 0) {
            dm[st * 32 + lane] = (uint16_t)dir;
            if (lane == 31) {
                bnd[j] = {L.left.P, L.left.Q, L.left.ED, L.left.CD};
                bndg[j] = L.left.g;
            }
        }
        L.nu = shfl_up_state(L.left);
        __syncwarp();  // lane 31's boundary-row writes before lane 0's later reads
    }
    const int rl = (l1 - 1) & 31;
    glast = __shfl_sync(FULL, L.left.g, rl);
    return __shfl_sync(FULL, L.lcost, rl);
}

__global__ void __launch_bounds__(NK_WARPS * 32) newkk_kernel(NewkkArgs A)
{
    __shared__ Tables st;
    load_tables_nk(st, A.tables);
    __syncthreads();
    const Tables& t = st;
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    nk::Quad* bnd = A.bnd + gw * A.bnd_stride;
    uint32_t* bndg = A.bndg + gw * A.bnd_stride;
    int* tb = A.tb + gw * A.tb_stride;
    const int go = t.go > 0 ? t.go : 0;
    const long long slice = gw * A.slice_words;  // this warp's arena slice
    for (;;) {
        int idx = 0;
        if (lane == 0) idx = atomicAdd(A.ctr, 1);
        idx = __shfl_sync(FULL, idx, 0);
        if (idx >= A.npairs) break;
        const int k = A.order ? A.order[idx] : idx;
        if (A.rerun && A.status[k] != POYALGN_PAIR_RETRY) continue;
        const uint8_t* a = A.seqs + A.offa[k];
        const uint8_t* b = A.seqs + A.offb[k];
        const int la = A.lena[k], lb = A.lenb[k];
        const int swaped = A.swp ? A.swp[k] : (la <= lb ? 0 : 1);
        const bool flip = !A.swp && swaped;
        const uint8_t* s1 = flip ? b : a;
        const uint8_t* s2 = flip ? a : b;
        const int l1 = flip ? lb : la, l2 = flip ? la : lb;
        PairOut o;
        o.ea = A.ea + A.out_off[k];
        o.eb = A.eb + A.out_off[k];
        o.med = A.med + A.out_off[k];
        o.mwg = A.mwg + A.out_off[k];
        o.cap = la + lb + 2;
        // the boundary row and the rounds table hold max_len columns / rows;
        // the cost matrix covers states below 1 << lcm
        const bool shape = l1 < 1 || l1 > l2;
        const bool too_long = l2 > A.bnd_stride;
        bool bad = shape || too_long;
        for (int x = lane; x < l1 + l2 && !bad; x += 32)
            bad = (x < l1 ? s1[x] : s2[x - l1]) >= (1 << t.lcm);
        if (__any_sync(FULL, bad)) {
            if (lane == 0) {
                A.status[k] = shape ? POYALGN_PAIR_EMPTY
                              : too_long ? POYALGN_PAIR_TOO_LONG : POYALGN_PAIR_BAD_STATE;
                A.cost[k] = A.maxcost[k] = A.alen[k] = A.mlen[k] = A.wlen[k] = 0;
                if (A.passes) A.passes[k] = 0;
            }
            continue;
        }
        const bool trivial = (long long)l1 * nk::MUCH_LONGER < l2;
        int cost = 0, npass = 0, kk = 0, status = 0;
        if (trivial) {
            cost = nk::trivial_cost(t, s1, l1, s2, l2);
        } else {
            auto fill = [&](int kp, int& c, uint32_t& g) -> bool {
                const nk::Band B{l1, l2, kp};
                const long long steps = build_rounds(B, tb);
                if (steps * 32 > A.slice_words) {
                    status = POYALGN_PAIR_RETRY;  // rerun with fewer, larger slices
                    return false;
                }
                c = fill_pass(t, s1, l1, s2, l2, kp, go, A.arena + slice, steps, bnd, bndg, tb, g);
                return true;
            };
            cost = nk::drive(t, l1, l2, fill, kk, npass, status);
        }
        if (lane == 0) {
            PairRes r = {0, 0, 0, 0, status};
            if (status == 0) {
                ArenaDir dir{A.arena + slice, tb};
                r = nk::traceback(t, dir, trivial, kk, s1, l1, s2, l2, swaped, o);
            } else if (status == POYALGN_PAIR_RETRY) {
                atomicAdd(A.ctr + 1, 1);
            }
            A.cost[k] = cost;
            A.alen[k] = r.alen;
            A.mlen[k] = r.mlen;
            A.wlen[k] = r.wlen;
            A.maxcost[k] = r.maxcost;
            A.status[k] = r.status;
            if (A.passes) A.passes[k] = npass;
            if (A.kmax) A.kmax[k] = kk;
        }
        __syncwarp();
    }
}

}  // namespace

int run_newkk(poyalgn_ctx* c, const poyalgn_cm* cm, int npairs, int max_len,
              const uint8_t* seqs, const long long* offa, const int* lena,
              const long long* offb, const int* lenb, const long long* out_off, int* cost,
              int* maxcost, int* alen, int* mlen, int* wlen, int* status, uint8_t* ea,
              uint8_t* eb, uint8_t* med, uint8_t* mwg, int* passes, const int* order,
              const int* swp, int* kmax, cudaStream_t st)
{
    if (cm->h.cost_model != 1)
        return set_err(POYALGN_EUNSUPPORTED,
                       "Algn_Newkk is built for the affine cost model only (the reference's "
                       "linear variant does not produce an alignment)");
    if (npairs <= 0) return 0;
    int rc;
    int bps = 0;
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, newkk_kernel, NK_WARPS * 32, 0));
    bps = std::max(bps, 1);
    const int grid = (int)std::min<long long>((long long)c->nsm * bps,
                                              (npairs + NK_WARPS - 1) / NK_WARPS);
    const long long nwarps = (long long)grid * NK_WARPS;
    const int stride = std::max(max_len, 1);
    const int tstride = (stride + 31) / 32;
    if ((rc = reserve(c->nk_bnd, (size_t)nwarps * stride * sizeof(nk::Quad)))) return rc;
    if ((rc = reserve(c->nk_bndg, (size_t)nwarps * stride * sizeof(uint32_t)))) return rc;
    if ((rc = reserve(c->nk_tb, (size_t)nwarps * tstride * sizeof(int)))) return rc;
    if ((rc = reserve(c->nk_ctr, 16))) return rc;
    long long words = c->nk_arena_words;
    if (words <= 0) {
        size_t fr = 0, tot = 0;
        CU(cudaMemGetInfo(&fr, &tot));
        const long long have = (long long)(c->nk_arena.n / 2);
        words = std::max(have, std::min<long long>((long long)(fr / 3) / 2, 16LL << 30));
    }
    if ((rc = reserve(c->nk_arena, (size_t)words * 2))) return rc;
    NewkkArgs A;
    A.seqs = seqs;
    A.offa = offa;
    A.lena = lena;
    A.offb = offb;
    A.lenb = lenb;
    A.npairs = npairs;
    A.order = order;
    A.swp = swp;
    A.tables = cm->d;
    A.ctr = as<int>(c->nk_ctr);
    A.arena = as<uint16_t>(c->nk_arena);
    A.bnd = as<nk::Quad>(c->nk_bnd);
    A.bndg = as<uint32_t>(c->nk_bndg);
    A.bnd_stride = stride;
    A.tb = as<int>(c->nk_tb);
    A.tb_stride = tstride;
    A.out_off = out_off;
    A.cost = cost;
    A.maxcost = maxcost;
    A.alen = alen;
    A.mlen = mlen;
    A.wlen = wlen;
    A.status = status;
    A.passes = passes;
    A.kmax = kmax;
    A.ea = ea;
    A.eb = eb;
    A.med = med;
    A.mwg = mwg;
    // Every warp owns an equal slice of the arena. A pair whose band does
    // not fit its warp's slice is marked for a rerun, which launches fewer
    // warps (larger slices) over the marked pairs only, down to one warp
    // holding the whole arena.
    int w = (int)std::min<long long>(nwarps, npairs), launches = 0;
    for (A.rerun = 0;; A.rerun = 1) {
        const int threads = std::min(w, NK_WARPS) * 32;
        const int blocks = (w * 32 + threads - 1) / threads;
        const long long launched = (long long)blocks * threads / 32;
        A.slice_words = (words / launched) & ~31LL;
        CU(cudaMemsetAsync(c->nk_ctr.p, 0, 8, st));
        newkk_kernel<<<blocks, threads, 0, st>>>(A);
        CU(cudaGetLastError());
        launches++;
        int h = 0;
        CU(cudaMemcpyAsync(&h, A.ctr + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        if (h == 0) break;
        if (launched == 1)
            return set_err(POYALGN_ENOMEM, "Newkk: %d pairs have bands larger than the "
                           "direction arena (%lld words)", h, words);
        w = std::max(1, std::min(w / 2, h));
    }
    c->last_launches = launches;
    return 0;
}

}  // namespace pa

using namespace pa;

namespace {

int nk_max_len(int npairs, const int32_t* lena, const int32_t* lenb)
{
    int m = 1;
    for (int k = 0; k < npairs; k++) m = std::max(m, std::max(lena[k], lenb[k]));
    return m;
}

}  // namespace

extern "C" {

int poyalgn_newkk_median_batch_device(poyalgn_ctx* ctx, const poyalgn_cm* cm, int npairs,
                                      const uint8_t* seqs, const int64_t* offa,
                                      const int32_t* lena, const int64_t* offb,
                                      const int32_t* lenb, const int64_t* out_off, int max_len,
                                      int32_t* cost, int32_t* maxcost, int32_t* alen,
                                      int32_t* mlen, int32_t* wlen, int32_t* status, uint8_t* ea,
                                      uint8_t* eb, uint8_t* med, uint8_t* mwg, int32_t* passes,
                                      void* stream)
{
    if (!ctx || !cm || max_len < 1 ||
        (npairs > 0 && (!seqs || !offa || !lena || !offb || !lenb || !out_off || !cost ||
                        !maxcost || !alen || !mlen || !wlen || !status || !ea || !eb || !med ||
                        !mwg)))
        return set_err(POYALGN_EINVAL, "null argument");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    return run_newkk(ctx, cm, npairs, max_len, seqs, (const long long*)offa, lena,
                     (const long long*)offb, lenb, (const long long*)out_off, cost, maxcost,
                     alen, mlen, wlen, status, ea, eb, med, mwg, passes, nullptr, nullptr,
                     nullptr, (cudaStream_t)stream);
}

int poyalgn_newkk_median_batch(poyalgn_ctx* ctx, const poyalgn_cm* cm, int npairs,
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
    for (int k = 0; k < npairs; k++) {
        if (lena[k] < 1 || lenb[k] < 1) return set_err(POYALGN_EINVAL, "pair %d: empty sequence", k);
        seq_bytes = std::max<long long>(seq_bytes, std::max(offa[k] + lena[k], offb[k] + lenb[k]));
        out_total = std::max<long long>(out_total, out_off[k] + lena[k] + lenb[k] + 2);
    }
    // longest pairs first: the tail of the launch is then made of short ones
    std::vector<int> order((size_t)npairs);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return (long long)lena[x] * lenb[x] > (long long)lena[y] * lenb[y];
    });
    const size_t ni = (size_t)npairs;
    if ((rc = reserve(ctx->seqs, (size_t)seq_bytes))) return rc;
    if ((rc = reserve(ctx->offa, ni * 8))) return rc;
    if ((rc = reserve(ctx->offb, ni * 8))) return rc;
    if ((rc = reserve(ctx->lena, ni * 4))) return rc;
    if ((rc = reserve(ctx->lenb, ni * 4))) return rc;
    if ((rc = reserve(ctx->outoff, ni * 8))) return rc;
    if ((rc = reserve(ctx->nk_order, ni * 4))) return rc;
    if ((rc = reserve(ctx->ints, ni * 4 * 7))) return rc;
    if ((rc = reserve(ctx->bytes, (size_t)out_total * 4))) return rc;
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(ctx->seqs.p, seqs, (size_t)seq_bytes, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->offa.p, offa, ni * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->offb.p, offb, ni * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->lena.p, lena, ni * 4, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->lenb.p, lenb, ni * 4, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->outoff.p, out_off, ni * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->nk_order.p, order.data(), ni * 4, cudaMemcpyHostToDevice, st));
    int* I = as<int>(ctx->ints);
    uint8_t* B = as<uint8_t>(ctx->bytes);
    const size_t ot = (size_t)out_total;
    if ((rc = run_newkk(ctx, cm, npairs, nk_max_len(npairs, lena, lenb), as<uint8_t>(ctx->seqs),
                        as<long long>(ctx->offa), as<int>(ctx->lena), as<long long>(ctx->offb),
                        as<int>(ctx->lenb), as<long long>(ctx->outoff), I, I + ni, I + 2 * ni,
                        I + 3 * ni, I + 4 * ni, I + 5 * ni, B, B + ot, B + 2 * ot, B + 3 * ot,
                        I + 6 * ni, as<int>(ctx->nk_order), nullptr, nullptr, st)))
        return rc;
    int32_t* outs[7] = {cost, maxcost, alen, mlen, wlen, status, passes};
    for (int j = 0; j < 7; j++)
        if (outs[j]) CU(cudaMemcpyAsync(outs[j], I + j * ni, ni * 4, cudaMemcpyDeviceToHost, st));
    uint8_t* bo[4] = {ea, eb, med, mwg};
    for (int j = 0; j < 4; j++) CU(cudaMemcpyAsync(bo[j], B + j * ot, ot, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    for (int k = 0; k < npairs; k++)
        if (status[k] != 0) return set_err(POYALGN_EPAIR, "pair %d failed with status %d", k, status[k]);
    return 0;
}

int poyalgn_newkk_algn_affine(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* s1, int l1,
                              const uint8_t* s2, int l2, int swaped, int32_t* cost)
{
    if (!ctx || !cm || !s1 || !s2 || !cost || l1 < 1 || l2 < 1)
        return set_err(POYALGN_EINVAL, "bad argument");
    if (l1 > l2) return set_err(POYALGN_EINVAL, "ERROR: newkkonen.newk_algn, s1 len > s2 len");
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    ctx->nk_valid = false;
    const size_t cap = (size_t)l1 + l2 + 2;
    if ((rc = reserve(ctx->seqs, (size_t)l1 + l2))) return rc;
    if ((rc = reserve(ctx->offa, 16))) return rc;
    if ((rc = reserve(ctx->ints, 4 * 10))) return rc;
    if ((rc = reserve(ctx->bytes, cap * 4))) return rc;
    cudaStream_t st = ctx->stream;
    long long hoff[2] = {0, l1};
    int hlen[2] = {l1, l2}, hsw = swaped ? 1 : 0;
    long long* off = as<long long>(ctx->offa);
    int* I = as<int>(ctx->ints);
    uint8_t* B = as<uint8_t>(ctx->bytes);
    CU(cudaMemcpyAsync(ctx->seqs.p, s1, (size_t)l1, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(as<uint8_t>(ctx->seqs) + l1, s2, (size_t)l2, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(off, hoff, 16, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(I + 7, hlen, 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(I + 9, &hsw, 4, cudaMemcpyHostToDevice, st));
    // out_off = 0: reuse hoff[0] on the device
    if ((rc = run_newkk(ctx, cm, 1, l2, as<uint8_t>(ctx->seqs), off, I + 7, off + 1, I + 8, off, I,
                        I + 1, I + 2, I + 3, I + 4, I + 5, B, B + cap, B + 2 * cap, B + 3 * cap,
                        nullptr, nullptr, I + 9, I + 6, st)))
        return rc;
    int h[7];
    CU(cudaMemcpyAsync(h, I, sizeof(h), cudaMemcpyDeviceToHost, st));
    std::vector<uint8_t> r(2 * cap);
    CU(cudaMemcpyAsync(r.data(), B, 2 * cap, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (h[5] != 0) return set_err(POYALGN_EPAIR, "Newkk alignment failed with status %d", h[5]);
    const int L = h[2];
    // swaped: the traceback wrote s1's aligned states to the second slot
    const uint8_t* ea = r.data() + cap - L;
    const uint8_t* eb = r.data() + 2 * cap - L;
    ctx->nk_r1.assign(hsw ? eb : ea, (hsw ? eb : ea) + L);
    ctx->nk_r2.assign(hsw ? ea : eb, (hsw ? ea : eb) + L);
    ctx->nk_s1.assign(s1, s1 + l1);
    ctx->nk_s2.assign(s2, s2 + l2);
    ctx->nk_l1 = l1;
    ctx->nk_l2 = l2;
    ctx->nk_swaped = hsw;
    ctx->nk_k = h[6];
    ctx->nk_cm = cm;
    ctx->nk_valid = true;
    *cost = h[0];
    return 0;
}

int poyalgn_newkk_backtrace_affine(poyalgn_ctx* ctx, const poyalgn_cm* cm, const uint8_t* s1,
                                   int l1, const uint8_t* s2, int l2, uint8_t* s1p, uint8_t* s2p,
                                   int cap, int32_t* len, int swaped)
{
    if (!ctx || !cm || !s1 || !s2 || !s1p || !s2p || !len)
        return set_err(POYALGN_EINVAL, "bad argument");
    if (!ctx->nk_valid || ctx->nk_cm != cm || ctx->nk_l1 != l1 || ctx->nk_l2 != l2 ||
        ctx->nk_swaped != (swaped ? 1 : 0) ||
        !std::equal(s1, s1 + l1, ctx->nk_s1.begin()) || !std::equal(s2, s2 + l2, ctx->nk_s2.begin()))
        return set_err(POYALGN_EINVAL,
                       "newkk_backtrace_affine needs the pair of the last newkk_algn_affine call");
    const int L = (int)ctx->nk_r1.size();
    if (cap < L) return set_err(POYALGN_EINVAL, "output capacity %d < %d", cap, L);
    // like seq_prepend: the aligned states end at the last byte
    std::copy(ctx->nk_r1.begin(), ctx->nk_r1.end(), s1p + cap - L);
    std::copy(ctx->nk_r2.begin(), ctx->nk_r2.end(), s2p + cap - L);
    *len = L;
    return 0;
}

int poyalgn_newkk_set_arena_words(poyalgn_ctx* ctx, int64_t words)
{
    if (!ctx || words < 0) return set_err(POYALGN_EINVAL, "bad argument");
    ctx->nk_arena_words = words;
    if (words > 0 && ctx->nk_arena.n > (size_t)words * 2) release(ctx->nk_arena);
    return 0;
}

int poyalgn_newkk_get_k(const poyalgn_ctx* ctx, int32_t* k)
{
    if (!ctx || !k) return set_err(POYALGN_EINVAL, "bad argument");
    *k = ctx->nk_valid ? ctx->nk_k : 0;
    return 0;
}

}  // extern "C"
