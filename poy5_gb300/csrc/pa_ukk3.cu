// Three-sequence alignment on the GPU: Sequence.Align.align_3_powell ->
// powell_3D_align (src/ukkCommon.c:109-145, src/ukk.checkp.c), many triples
// per launch, one warp per triple replaying the reference recursion
// (pa_ukk3.cuh).
//
// C ABI (include/poyalgn.h): poyalgn_powell_3d (the per-call external
// `powell_3d`, src/sequence.ml:1309-1310) and poyalgn_powell_3d_batch.
//
// The replay is a chain of dependent loads and stores into the triple's own
// workspace, so it is bound by memory latency, not by issue: a whole warp
// runs each triple, its lanes loading a frame's candidate cells in one round
// (pa_ukk3.cuh), and the driver keeps as many triples resident as the
// workspace budget allows.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "pa_runtime.h"
#include "pa_ukk3.cuh"

namespace pa {
namespace {

constexpr int U3_BLOCK = 128;
static_assert(u3::RING == 32, "one ring tag per lane is cleared at launch");

struct U3Args {
    const uint8_t* seqs;
    const long long* off;   // 3 per triple
    const int* len;         // 3 per triple, POY lengths (leading gap included)
    const long long* out_off;
    const int* list;        // triples of this launch
    const long long* wofs;  // per list entry: its workspace offset
    const int* win;         // per list entry: window half-width
    int nlist;
    unsigned char* work;
    uint8_t *ra, *rb, *rc;
    int *rlen, *cost, *status;
    u3::Model model;
};

__global__ void __launch_bounds__(U3_BLOCK) powell_kernel(const U3Args A)
{
    __shared__ u3::Model sm;
    // each warp's stack top: frames popped from here do not wait on memory
    __shared__ u3::Frame ring[U3_BLOCK / 32][u3::RING];
    __shared__ int ring_tag[U3_BLOCK / 32][u3::RING];
    if (threadIdx.x == 0) sm = A.model;
    ring_tag[threadIdx.x >> 5][threadIdx.x & 31] = -1;
    __syncthreads();
    // one warp per triple: every lane holds the same machine state and the
    // lanes load a frame's candidate cells together
    const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= A.nlist) return;
    const int k = A.list[i];
    const int la = A.len[3 * k] - 1, lb = A.len[3 * k + 1] - 1, lc = A.len[3 * k + 2] - 1;
    const u3::Layout L = u3::layout(sm, la, lb, lc, A.win[i]);
    u3::Work w = u3::work_at(A.work + A.wofs[i], L);
    w.ring = ring[threadIdx.x >> 5];
    w.ring_tag = ring_tag[threadIdx.x >> 5];
    const int cap = la + lb + lc + 3;
    const long long end = A.out_off[k] + cap;
    u3::Machine mc(sm, w, A.seqs + A.off[3 * k], la, A.seqs + A.off[3 * k + 1], lb,
                   A.seqs + A.off[3 * k + 2], lc);
    int n = 0;
    const int d = mc.run(A.ra + end, A.rb + end, A.rc + end, cap, &n);
    A.status[k] = mc.status;
    A.cost[k] = d;
    A.rlen[k] = n;
}

// the two timing events of a batch, destroyed on every return path
struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    ~EventPair()
    {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

int status_code(int s)
{
    switch (s) {
    case u3::OK: return POYALGN_PAIR_OK;
    case u3::ERR_BASE: return POYALGN_PAIR_BAD_STATE;
    case u3::ERR_LEN: return POYALGN_PAIR_TOO_LONG;
    case u3::ERR_OUT: return POYALGN_PAIR_CAPACITY;
    default: return POYALGN_PAIR_INTERNAL;
    }
}

}  // namespace

// Host-pointer batch: validates, stages, and runs rounds of launches, each
// with as many triples as the workspace budget holds (longest first); a
// triple that outgrew its window is rerun with twice the width.
int run_powell(poyalgn_ctx* c, int n, const uint8_t* seqs, const int64_t* off,
               const int32_t* len, int mm, int go, int ge, const int64_t* out_off, uint8_t* ra,
               uint8_t* rb, uint8_t* rc, int32_t* rlen, int32_t* cost, int32_t* status)
{
    c->u3_ms = 0.f;
    if (n <= 0) return 0;
    if (mm < 1 || go < 0 || ge < 1 || mm > u3::MAXCOST || go > u3::MAXCOST || ge > u3::MAXCOST)
        return set_err(POYALGN_EINVAL,
                       "powell_3d: costs must be 1 <= mm, ge <= %d and 0 <= go <= %d",
                       u3::MAXCOST, u3::MAXCOST);
    u3::Model model;
    u3::model_init(model, mm, go, ge);
    long long seq_bytes = 0, out_total = 0;
    std::vector<int> win((size_t)n, 0);
    std::vector<int> pending;
    for (int k = 0; k < n; k++) {
        status[k] = POYALGN_PAIR_OK;
        rlen[k] = 0;
        cost[k] = -1;
        const int l[3] = {len[3 * k], len[3 * k + 1], len[3 * k + 2]};
        if (l[0] < 1 || l[1] < 1 || l[2] < 1) {
            status[k] = POYALGN_PAIR_EMPTY;
            continue;
        }
        if (l[0] - 1 > u3::MAXLEN || l[1] - 1 > u3::MAXLEN || l[2] - 1 > u3::MAXLEN ||
            u3::cost_bound(model.maxstep, l[0] - 1, l[1] - 1, l[2] - 1) > u3::MAX_COST_BOUND) {
            status[k] = POYALGN_PAIR_TOO_LONG;
            continue;
        }
        bool bad = false;
        for (int j = 0; j < 3 && !bad; j++) {
            const uint8_t* s = seqs + off[3 * k + j];
            for (int p = 1; p < l[j]; p++)
                if (!(s[p] & 15)) {
                    bad = true;
                    break;
                }
            seq_bytes = std::max<long long>(seq_bytes, off[3 * k + j] + l[j]);
        }
        if (bad) {
            status[k] = POYALGN_PAIR_BAD_STATE;  // "This is impossible!"
            continue;
        }
        out_total = std::max<long long>(out_total, out_off[k] + l[0] + l[1] + l[2]);
        win[k] = u3::first_window(l[0] - 1, l[1] - 1, l[2] - 1);
        if (!u3::window_fits(model, l[0] - 1, l[1] - 1, l[2] - 1, win[k])) {
            status[k] = POYALGN_PAIR_TOO_LONG;
            continue;
        }
        pending.push_back(k);
    }
    if (pending.empty()) goto done;
    {
        int rc_;
        const size_t ni = (size_t)n;
        if ((rc_ = reserve(c->seqs, (size_t)std::max<long long>(seq_bytes, 1)))) return rc_;
        // metadata block: each array at a 16-byte aligned offset
        size_t mo = 0;
        auto carve = [&](size_t bytes) {
            const size_t at = mo;
            mo += (bytes + 15) & ~(size_t)15;
            return at;
        };
        const size_t o_off = carve(ni * 24), o_len = carve(ni * 12), o_oo = carve(ni * 8);
        const size_t o_rlen = carve(ni * 4), o_cost = carve(ni * 4), o_st = carve(ni * 4);
        const size_t o_list = carve(ni * 4), o_wofs = carve(ni * 8), o_win = carve(ni * 4);
        if ((rc_ = reserve(c->u3_meta, mo))) return rc_;
        if ((rc_ = reserve(c->bytes, (size_t)out_total * 3))) return rc_;
        unsigned char* M = as<unsigned char>(c->u3_meta);
        long long* d_off = (long long*)(M + o_off);
        int* d_len = (int*)(M + o_len);
        long long* d_oo = (long long*)(M + o_oo);
        int* d_rlen = (int*)(M + o_rlen);
        int* d_cost = (int*)(M + o_cost);
        int* d_st = (int*)(M + o_st);
        int* d_list = (int*)(M + o_list);
        long long* d_wofs = (long long*)(M + o_wofs);
        int* d_win = (int*)(M + o_win);
        uint8_t* B = as<uint8_t>(c->bytes);
        const size_t ot = (size_t)out_total;
        cudaStream_t st = c->stream;
        CU(cudaMemcpyAsync(c->seqs.p, seqs, (size_t)seq_bytes, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(d_off, off, ni * 24, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(d_len, len, ni * 12, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(d_oo, out_off, ni * 8, cudaMemcpyHostToDevice, st));
        // workspace budget: the caller's, else half the free memory (at most
        // 192 GB). A launch lasts as long as its slowest triple, so a batch
        // that fits one round finishes in about that triple's time.
        long long budget = c->u3_budget;
        if (budget <= 0) {
            size_t fr = 0, tot = 0;
            CU(cudaMemGetInfo(&fr, &tot));
            budget = std::min<long long>((long long)(fr / 2), 192LL << 30);
        }
        EventPair ev;
        CU(cudaEventCreate(&ev.a));
        CU(cudaEventCreate(&ev.b));
        cudaEvent_t e0 = ev.a, e1 = ev.b;
        std::vector<int> list, hst((size_t)n);
        std::vector<long long> wofs;
        std::vector<int> lwin;
        float ms_total = 0.f;
        int rounds = 0;
        while (!pending.empty()) {
            auto bytes_of = [&](int k) {
                return u3::layout(model, len[3 * k] - 1, len[3 * k + 1] - 1, len[3 * k + 2] - 1,
                                  win[k]).bytes;
            };
            std::stable_sort(pending.begin(), pending.end(),
                             [&](int x, int y) { return bytes_of(x) > bytes_of(y); });
            list.clear(), wofs.clear(), lwin.clear();
            long long used = 0;
            std::vector<int> rest;
            for (int k : pending) {
                const long long b = bytes_of(k);
                if (list.empty() || used + b <= budget) {
                    list.push_back(k);
                    wofs.push_back(used);
                    lwin.push_back(win[k]);
                    used += b;
                } else {
                    rest.push_back(k);
                }
            }
            if ((rc_ = reserve(c->u3_work, (size_t)used))) return rc_;
            const size_t nl = list.size();
            CU(cudaMemcpyAsync(d_list, list.data(), nl * 4, cudaMemcpyHostToDevice, st));
            CU(cudaMemcpyAsync(d_wofs, wofs.data(), nl * 8, cudaMemcpyHostToDevice, st));
            CU(cudaMemcpyAsync(d_win, lwin.data(), nl * 4, cudaMemcpyHostToDevice, st));
            CU(cudaMemsetAsync(c->u3_work.p, 0, (size_t)used, st));
            U3Args A;
            A.seqs = as<uint8_t>(c->seqs);
            A.off = d_off;
            A.len = d_len;
            A.out_off = d_oo;
            A.list = d_list;
            A.wofs = d_wofs;
            A.win = d_win;
            A.nlist = (int)nl;
            A.work = as<unsigned char>(c->u3_work);
            A.ra = B, A.rb = B + ot, A.rc = B + 2 * ot;
            A.rlen = d_rlen, A.cost = d_cost, A.status = d_st;
            A.model = model;
            const long long threads = (long long)nl * 32;
            const unsigned blocks = (unsigned)((threads + U3_BLOCK - 1) / U3_BLOCK);
            CU(cudaEventRecord(e0, st));
            powell_kernel<<<blocks, U3_BLOCK, 0, st>>>(A);
            CU(cudaGetLastError());
            CU(cudaEventRecord(e1, st));
            CU(cudaMemcpyAsync(hst.data(), d_st, ni * 4, cudaMemcpyDeviceToHost, st));
            CU(cudaStreamSynchronize(st));
            float ms = 0.f;
            CU(cudaEventElapsedTime(&ms, e0, e1));
            ms_total += ms;
            rounds++;
            for (int k : list) {
                const int s = hst[(size_t)k];
                if (s == u3::ERR_WINDOW || s == u3::ERR_STACK || s == u3::ERR_STEPS) {
                    const int full = u3::full_window(len[3 * k] - 1, len[3 * k + 1] - 1,
                                                     len[3 * k + 2] - 1);
                    if (win[k] < full) {
                        const int wider = std::min(2 * win[k], full);
                        if (u3::window_fits(model, len[3 * k] - 1, len[3 * k + 1] - 1,
                                            len[3 * k + 2] - 1, wider)) {
                            win[k] = wider;
                            rest.push_back(k);
                            continue;
                        }
                        status[k] = POYALGN_PAIR_TOO_LONG;
                        continue;
                    }
                }
                status[k] = status_code(s);
            }
            pending.swap(rest);
        }
        c->u3_ms = ms_total;
        c->u3_rounds = rounds;
        CU(cudaMemcpyAsync(rlen, d_rlen, ni * 4, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(cost, d_cost, ni * 4, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(ra, B, ot, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(rb, B + ot, ot, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(rc, B + 2 * ot, ot, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
    }
done:
    for (int k = 0; k < n; k++)
        if (status[k] != POYALGN_PAIR_OK) {
            rlen[k] = 0;
            cost[k] = -1;
        }
    for (int k = 0; k < n; k++)
        if (status[k] != POYALGN_PAIR_OK)
            return set_err(POYALGN_EPAIR, "triple %d failed with status %d", k, status[k]);
    return 0;
}

}  // namespace pa

using namespace pa;

int poyalgn_powell_3d_batch(poyalgn_ctx* ctx, int ntriples, const uint8_t* seqs,
                            const int64_t* off, const int32_t* len, int mm, int go, int ge,
                            const int64_t* out_off, uint8_t* ra, uint8_t* rb, uint8_t* rc,
                            int32_t* rlen, int32_t* cost, int32_t* status)
{
    if (!ctx || ntriples < 0 ||
        (ntriples > 0 && (!seqs || !off || !len || !out_off || !ra || !rb || !rc || !rlen ||
                          !cost || !status)))
        return set_err(POYALGN_EINVAL, "null argument");
    int rc_;
    if ((rc_ = ensure_device(ctx))) return rc_;
    return run_powell(ctx, ntriples, seqs, off, len, mm, go, ge, out_off, ra, rb, rc, rlen, cost,
                      status);
}

int poyalgn_powell_3d(poyalgn_ctx* ctx, const uint8_t* a, int la, const uint8_t* b, int lb,
                      const uint8_t* c, int lc, int mm, int go, int ge, uint8_t* ra, uint8_t* rb,
                      uint8_t* rc, int cap, int32_t* rlen, int32_t* cost)
{
    if (!ctx || !a || !b || !c || !ra || !rb || !rc || !rlen || !cost)
        return set_err(POYALGN_EINVAL, "null argument");
    if (la < 1 || lb < 1 || lc < 1) return set_err(POYALGN_EINVAL, "empty sequence");
    if (cap < la + lb + lc) return set_err(POYALGN_EINVAL, "result capacity below la + lb + lc");
    std::vector<uint8_t> seqs((size_t)la + lb + lc);
    std::copy(a, a + la, seqs.begin());
    std::copy(b, b + lb, seqs.begin() + la);
    std::copy(c, c + lc, seqs.begin() + la + lb);
    const int64_t off[3] = {0, la, (int64_t)la + lb};
    const int32_t len[3] = {la, lb, lc};
    const int64_t oo = 0;
    const size_t cp = (size_t)la + lb + lc;
    std::vector<uint8_t> oa(cp), ob(cp), oc(cp);
    int32_t n = 0, d = 0, st = 0;
    int rc_ = poyalgn_powell_3d_batch(ctx, 1, seqs.data(), off, len, mm, go, ge, &oo, oa.data(),
                                      ob.data(), oc.data(), &n, &d, &st);
    if (rc_) return rc_;
    // back to front, ending at the end of the caller's buffers (seq_prepend)
    std::copy(oa.end() - n, oa.end(), ra + cap - n);
    std::copy(ob.end() - n, ob.end(), rb + cap - n);
    std::copy(oc.end() - n, oc.end(), rc + cap - n);
    *rlen = n;
    *cost = d;
    return 0;
}

int poyalgn_powell_3d_stats(poyalgn_ctx* ctx, float* kernel_ms, int32_t* rounds)
{
    if (!ctx) return set_err(POYALGN_EINVAL, "null argument");
    if (kernel_ms) *kernel_ms = ctx->u3_ms;
    if (rounds) *rounds = ctx->u3_rounds;
    return 0;
}

int poyalgn_powell_3d_set_budget(poyalgn_ctx* ctx, int64_t work_bytes)
{
    if (!ctx || work_bytes < 0) return set_err(POYALGN_EINVAL, "bad argument");
    ctx->u3_budget = work_bytes;
    return 0;
}
