// Serving: continuous batching of DOS.median requests over resident nodes.
//
// One scheduler thread owns nslots execution slots. A slot is a context (its
// own stream and batch scratch, reserved at creation) plus pinned host
// buffers for one batch's results. The thread completes finished slots
// (cudaEventQuery on the event recorded after the slot's result copies) and
// refills free slots from the oldest waiting requests, so batches overlap on
// the device and requests join the next batch as soon as a slot frees.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pa_runtime.h"

using namespace pa;
using Clock = std::chrono::steady_clock;

namespace {

constexpr long long kAlign = 16;
long long align_up(long long x) { return (x + kAlign - 1) & ~(kAlign - 1); }

struct Req {
    int64_t id = 0;
    int npairs = 0;
    long long out_bytes = 0;      // sum of aligned caps
    std::vector<int> na, nb;
    Clock::time_point t_arrive, t_done;
    bool done = false;
    int error = 0;
    std::vector<int> cost, status, mlen;
    std::vector<uint8_t> med;     // medians, concatenated
};

struct Slot {
    poyalgn_ctx* ctx = nullptr;
    DevBuf meta, ints, bytes;
    unsigned char* hmeta = nullptr;   // pinned: offa | offb | out_off | lena | lenb
    int* hints = nullptr;             // pinned: cost | maxcost | alen | mlen | wlen | status
    uint8_t* hmed = nullptr;          // pinned: the batch's median buffer
    cudaEvent_t done = nullptr;
    bool busy = false;
    std::vector<Req*> reqs;
    std::vector<long long> oo;        // per pair: output offset and cap
    std::vector<int> cap;
    long long total = 0;
};

}  // namespace

struct poyalgn_server {
    const poyalgn_cm* cm = nullptr;
    int affine = 0;
    int kind = POYALGN_SERVE_MEDIAN;
    int missing = 0;                  // DOS.distance's missing_distance
    int device = 0;
    const uint8_t* arena = nullptr;
    std::vector<long long> off;       // node table snapshot
    std::vector<int> len;
    int max_batch_pairs = 0;
    long long max_waiting_pairs = 0;
    long long out_cap = 0;            // bytes per output buffer of a slot
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req*> waiting;
    long long waiting_pairs = 0;
    // admission by device memory: the device bytes the waiting requests will
    // take in a slot, against the free device memory sampled at submission
    // (at most every kFreeSampleUs)
    long long waiting_bytes = 0;
    long long free_bytes = 0;
    Clock::time_point free_at;
    int64_t n_refused_hbm = 0;
    std::unordered_map<int64_t, Req*> reqs;
    int64_t next_id = 1;
    bool stop = false;
    int error = 0;                    // sticky scheduler error
    char errmsg[256] = {0};
    std::thread th;
    int64_t n_batches = 0, n_pairs = 0, n_refused = 0;
};

namespace {

void fail_all(poyalgn_server* s, int code, const char* msg)
{
    s->error = code;
    snprintf(s->errmsg, sizeof(s->errmsg), "%s", msg);
    for (auto& kv : s->reqs) {
        kv.second->done = true;
        kv.second->error = code;
    }
    s->waiting.clear();
    s->waiting_pairs = 0;
    s->waiting_bytes = 0;
    s->cv_done.notify_all();
}

// pairs per SM up to which a batch with no backlog speculates
constexpr int SERVE_SPEC_PAIRS = 2;
// the waiting requests may take at most this fraction of the free device
// memory; the free memory is sampled at most this often
constexpr double kAdmitFrac = 0.5;
constexpr int kFreeSampleUs = 1000;

// Device bytes a request occupies in a slot: its four output buffers, the
// per-pair metadata and result words.
long long request_device_bytes(long long out_bytes, int npairs)
{
    return 4 * out_bytes + 60LL * npairs;
}

// Build and enqueue one batch on slot `sl` from the requests in `batch`.
// Runs without the server lock; touches only the slot and the requests,
// which no other thread reads until they are marked done. Speculative band
// passes only for a small batch with nothing waiting behind it: with a
// backlog, or batches that with the other slots' fill the GPU, throughput
// matters more than one batch's latency.
int launch(poyalgn_server* s, Slot& sl, std::vector<Req*>& batch, bool backlog)
{
    int n = 0;
    for (Req* r : batch) n += r->npairs;
    sl.ctx->spec_mode = (backlog || n > SERVE_SPEC_PAIRS * sl.ctx->nsm) ? 0 : 2;
    const size_t ni = (size_t)n;
    long long* offa = reinterpret_cast<long long*>(sl.hmeta);
    long long* offb = offa + ni;
    long long* oo = offb + ni;
    int* lena = reinterpret_cast<int*>(oo + ni);
    int* lenb = lena + ni;
    sl.oo.resize(ni);
    sl.cap.resize(ni);
    long long total = 0;
    int maxmn = 2, k = 0;
    for (Req* r : batch)
        for (int p = 0; p < r->npairs; p++, k++) {
            offa[k] = s->off[r->na[p]];
            offb[k] = s->off[r->nb[p]];
            lena[k] = s->len[r->na[p]];
            lenb[k] = s->len[r->nb[p]];
            oo[k] = total;
            sl.oo[k] = total;
            sl.cap[k] = lena[k] + lenb[k] + 2;
            total += align_up(sl.cap[k]);
            maxmn = std::max(maxmn, lena[k] + lenb[k]);
        }
    sl.total = total;
    sl.reqs = batch;
    poyalgn_ctx* c = sl.ctx;
    cudaStream_t st = c->stream;
    CU(cudaMemcpyAsync(sl.meta.p, sl.hmeta, ni * 32, cudaMemcpyHostToDevice, st));
    const long long* d_offa = as<long long>(sl.meta);
    const int* d_lena = reinterpret_cast<const int*>(d_offa + 3 * ni);
    int* I = as<int>(sl.ints);
    uint8_t* B = as<uint8_t>(sl.bytes);
    const long long oc = s->out_cap;
    int rc;
    if (s->kind == POYALGN_SERVE_DISTANCE) {
        // cost at I, status at I + 5 ni, like the median layout; no medians
        CU(cudaMemsetAsync(I + 3 * ni, 0, ni * sizeof(int), st));
        if (s->affine)
            rc = run_nobt(c, s->cm, n, maxmn, s->arena, d_offa, d_lena, d_offa + ni,
                          d_lena + ni, s->missing, I, I + 5 * ni, st);
        else
            rc = run_batch(c, s->cm, 0, n, maxmn, 1, s->arena, d_offa, d_lena, d_offa + ni,
                           d_lena + ni, nullptr, I, nullptr, nullptr, nullptr, nullptr,
                           I + 5 * ni, nullptr, nullptr, nullptr, nullptr, I + 6 * ni, nullptr,
                           nullptr, 0, st, 1, s->missing);
        if (rc) return rc;
        CU(cudaMemcpyAsync(sl.hints, I, ni * 6 * sizeof(int), cudaMemcpyDeviceToHost, st));
    } else {
        rc = run_batch(c, s->cm, s->affine, n, maxmn, total, s->arena, d_offa, d_lena,
                       d_offa + ni, d_lena + ni, d_offa + 2 * ni, I, I + ni, I + 2 * ni,
                       I + 3 * ni, I + 4 * ni, I + 5 * ni, B, B + oc, B + 2 * oc, B + 3 * oc,
                       I + 6 * ni, nullptr, nullptr, 1, st);
        if (rc) return rc;
        CU(cudaMemcpyAsync(sl.hints, I, ni * 6 * sizeof(int), cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(sl.hmed, B + 2 * oc, (size_t)total, cudaMemcpyDeviceToHost, st));
    }
    CU(cudaEventRecord(sl.done, st));
    sl.busy = true;
    return 0;
}

// Copy a finished slot's results into its requests.
void complete(poyalgn_server* s, Slot& sl, Clock::time_point now)
{
    size_t ni = 0;
    for (Req* r : sl.reqs) ni += r->npairs;
    const int* h = sl.hints;
    size_t k = 0;
    for (Req* r : sl.reqs) {
        r->cost.resize(r->npairs);
        r->status.resize(r->npairs);
        r->mlen.resize(r->npairs);
        size_t mb = 0;
        for (int p = 0; p < r->npairs; p++) mb += std::max(0, h[3 * ni + k + p]);
        r->med.resize(mb);
        size_t at = 0;
        for (int p = 0; p < r->npairs; p++, k++) {
            r->cost[p] = h[k];
            r->status[p] = h[5 * ni + k];
            const int ml = std::max(0, h[3 * ni + k]);
            r->mlen[p] = ml;
            memcpy(r->med.data() + at, sl.hmed + sl.oo[k] + sl.cap[k] - ml, (size_t)ml);
            at += ml;
        }
        r->t_done = now;
        r->done = true;
    }
    s->n_batches++;
    s->n_pairs += (int64_t)ni;
    sl.reqs.clear();
    sl.busy = false;
}

void scheduler(poyalgn_server* s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    std::vector<Req*> batch;
    while (!s->stop) {
        bool progress = false;
        for (Slot& sl : s->slots) {
            if (!sl.busy) continue;
            const cudaError_t e = cudaEventQuery(sl.done);
            if (e == cudaErrorNotReady) continue;
            if (e != cudaSuccess) {
                fail_all(s, POYALGN_ECUDA, cudaGetErrorString(e));
                return;
            }
            complete(s, sl, Clock::now());
            progress = true;
        }
        if (progress) s->cv_done.notify_all();
        for (Slot& sl : s->slots) {
            if (sl.busy || s->waiting.empty()) continue;
            batch.clear();
            int n = 0;
            long long bytes = 0;
            while (!s->waiting.empty()) {
                Req* r = s->waiting.front();
                if (!batch.empty() &&
                    (n + r->npairs > s->max_batch_pairs || bytes + r->out_bytes > s->out_cap))
                    break;
                batch.push_back(r);
                n += r->npairs;
                bytes += r->out_bytes;
                s->waiting.pop_front();
            }
            s->waiting_pairs -= n;
            s->waiting_bytes -= request_device_bytes(bytes, n);
            const bool backlog = !s->waiting.empty();
            lk.unlock();
            const int rc = launch(s, sl, batch, backlog);
            lk.lock();
            if (rc) {
                fail_all(s, rc, poyalgn_last_error());
                return;
            }
            progress = true;
        }
        if (progress) continue;
        bool busy = false;
        for (Slot& sl : s->slots) busy |= sl.busy;
        if (busy) {
            // batches in flight: poll their events at a short interval
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        } else {
            s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
        }
    }
}

int submit_at(poyalgn_server* s, int npairs, const int32_t* na, const int32_t* nb,
              Clock::time_point t, int64_t* ticket)
{
    if (!s || npairs < 1 || !na || !nb || !ticket) return set_err(POYALGN_EINVAL, "bad request");
    const int nn = (int)s->len.size();
    long long bytes = 0;
    for (int p = 0; p < npairs; p++) {
        if (na[p] < 0 || na[p] >= nn || nb[p] < 0 || nb[p] >= nn)
            return set_err(POYALGN_EINVAL, "pair %d: unknown node (%d, %d)", p, na[p], nb[p]);
        bytes += align_up((long long)s->len[na[p]] + s->len[nb[p]] + 2);
    }
    if (npairs > s->max_batch_pairs || bytes > s->out_cap)
        return set_err(POYALGN_EINVAL, "request of %d pairs (%lld output bytes) exceeds one batch",
                       npairs, bytes);
    const long long dev_bytes = request_device_bytes(bytes, npairs);
    Req* r = new (std::nothrow) Req;
    if (!r) return set_err(POYALGN_ENOMEM, "request allocation");
    r->npairs = npairs;
    r->out_bytes = bytes;
    r->na.assign(na, na + npairs);
    r->nb.assign(nb, nb + npairs);
    r->t_arrive = t;
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->error) {
            delete r;
            return set_err(s->error, "server failed: %s", s->errmsg);
        }
        if (s->waiting_pairs + npairs > s->max_waiting_pairs) {
            s->n_refused++;
            delete r;
            return set_err(POYALGN_EBUSY, "admission refused: %lld pairs waiting",
                           s->waiting_pairs);
        }
        const Clock::time_point now = Clock::now();
        if (now - s->free_at > std::chrono::microseconds(kFreeSampleUs)) {
            size_t fr = 0, tot = 0;
            if (cudaSetDevice(s->device) == cudaSuccess &&
                cudaMemGetInfo(&fr, &tot) == cudaSuccess) {
                s->free_bytes = (long long)fr;
                s->free_at = now;
            }
        }
        if (s->waiting_bytes + dev_bytes > (long long)(kAdmitFrac * (double)s->free_bytes)) {
            s->n_refused++;
            s->n_refused_hbm++;
            delete r;
            return set_err(POYALGN_EBUSY,
                           "admission refused: waiting requests would take %lld of %lld free "
                           "device bytes", s->waiting_bytes + dev_bytes, s->free_bytes);
        }
        r->id = s->next_id++;
        s->reqs[r->id] = r;
        s->waiting.push_back(r);
        s->waiting_pairs += npairs;
        s->waiting_bytes += dev_bytes;
        *ticket = r->id;
    }
    s->cv_work.notify_one();
    return 0;
}

}  // namespace

extern "C" {

int poyalgn_server_create(poyalgn_store* store, const poyalgn_cm* cm, int kind,
                          int32_t missing_distance, int nslots, int max_batch_pairs,
                          int max_waiting_pairs, int64_t hbm_budget, poyalgn_server** out)
{
    if (!store || !cm || !out || nslots < 1 || nslots > 64 || max_batch_pairs < 1 ||
        max_waiting_pairs < max_batch_pairs || hbm_budget < 0 ||
        (kind != POYALGN_SERVE_MEDIAN && kind != POYALGN_SERVE_DISTANCE))
        return set_err(POYALGN_EINVAL, "bad server arguments");
    *out = nullptr;
    int rc;
    if ((rc = ensure_device(store->ctx))) return rc;
    if (hbm_budget == 0) {
        size_t fr = 0, tot = 0;
        CU(cudaMemGetInfo(&fr, &tot));
        hbm_budget = (int64_t)(fr / 2);
    }
    poyalgn_server* s = new (std::nothrow) poyalgn_server;
    if (!s) return set_err(POYALGN_ENOMEM, "server allocation");
    s->cm = cm;
    s->affine = cm->h.cost_model == 1;
    s->kind = kind;
    s->missing = missing_distance;
    s->device = store->ctx->device;
    s->arena = as<uint8_t>(store->arena);
    s->off = store->off;
    s->len = store->len;
    s->max_batch_pairs = max_batch_pairs;
    s->max_waiting_pairs = max_waiting_pairs;
    // per slot: half of its share for direction slabs (at most 8 GB), a
    // quarter for the deferred-traceback arena (at most 8 GB), the rest for
    // pair data (4 output buffers and the affine row-0 scratch)
    const long long share = hbm_budget / nslots;
    const long long slab = std::min<long long>(share / 2, 8LL << 30);
    const long long dm = std::min<long long>(share / 4, 8LL << 30);
    s->out_cap = std::min<long long>(share / 16, (long long)max_batch_pairs * 16384);
    s->out_cap &= ~(kAlign - 1);
    s->slots.resize(nslots);
    const size_t ni = (size_t)max_batch_pairs;
    int maxlen = 1;
    for (int L : s->len) maxlen = std::max(maxlen, L);
    for (Slot& sl : s->slots) {
        if ((rc = poyalgn_init(s->device, &sl.ctx))) break;
        sl.ctx->slab_budget = slab;
        sl.ctx->dm_fixed = dm;  // deferred tracebacks in an arena reserved here
        if ((rc = prereserve(sl.ctx, s->affine, max_batch_pairs, s->out_cap, slab))) break;
        if (kind == POYALGN_SERVE_DISTANCE && s->affine &&
            (rc = prereserve_nobt(sl.ctx, max_batch_pairs, maxlen))) break;
        if ((rc = reserve(sl.meta, ni * 32))) break;
        if ((rc = reserve(sl.ints, ni * 4 * 7))) break;
        if ((rc = reserve(sl.bytes, (size_t)s->out_cap * 4))) break;
        if (cudaHostAlloc((void**)&sl.hmeta, ni * 32, cudaHostAllocDefault) != cudaSuccess ||
            cudaHostAlloc((void**)&sl.hints, ni * 4 * 6, cudaHostAllocDefault) != cudaSuccess ||
            cudaHostAlloc((void**)&sl.hmed, (size_t)s->out_cap, cudaHostAllocDefault) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            rc = set_err(POYALGN_ENOMEM, "pinned host buffers or event");
            break;
        }
    }
    if (rc) {
        poyalgn_server_free(s);
        return rc;
    }
    s->th = std::thread(scheduler, s);
    *out = s;
    return 0;
}

void poyalgn_server_free(poyalgn_server* s)
{
    if (!s) return;
    if (s->th.joinable()) {
        {
            std::lock_guard<std::mutex> g(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        s->th.join();
    }
    cudaSetDevice(s->device);
    for (Slot& sl : s->slots) {
        if (sl.ctx) cudaStreamSynchronize(sl.ctx->stream);
        release(sl.meta);
        release(sl.ints);
        release(sl.bytes);
        if (sl.hmeta) cudaFreeHost(sl.hmeta);
        if (sl.hints) cudaFreeHost(sl.hints);
        if (sl.hmed) cudaFreeHost(sl.hmed);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.ctx) poyalgn_free(sl.ctx);
    }
    for (auto& kv : s->reqs) delete kv.second;
    delete s;
}

int poyalgn_server_submit(poyalgn_server* s, int npairs, const int32_t* node_a,
                          const int32_t* node_b, int64_t* ticket)
{
    return submit_at(s, npairs, node_a, node_b, Clock::now(), ticket);
}

int poyalgn_server_wait(poyalgn_server* s, int64_t ticket, int timeout_ms, int32_t* cost,
                        int32_t* status, int32_t* med_len, uint8_t* medians, int64_t med_cap,
                        double* latency_s)
{
    if (!s) return set_err(POYALGN_EINVAL, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_err(POYALGN_EINVAL, "unknown ticket %lld", (long long)ticket);
    Req* r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return set_err(POYALGN_EBUSY, "ticket %lld not done after %d ms", (long long)ticket,
                       timeout_ms);
    }
    s->reqs.erase(it);
    lk.unlock();
    int rc = 0;
    if (r->error) {
        rc = set_err(r->error, "server failed: %s", s->errmsg);
    } else {
        if (medians && (int64_t)r->med.size() > med_cap)
            rc = set_err(POYALGN_EINVAL, "median capacity %lld < %zu", (long long)med_cap,
                         r->med.size());
        for (int p = 0; p < r->npairs; p++) {
            if (cost) cost[p] = r->cost[p];
            if (status) status[p] = r->status[p];
            if (med_len) med_len[p] = r->mlen[p];
        }
        if (!rc && medians) memcpy(medians, r->med.data(), r->med.size());
        if (latency_s)
            *latency_s = std::chrono::duration<double>(r->t_done - r->t_arrive).count();
    }
    delete r;
    return rc;
}

int poyalgn_server_replay(poyalgn_server* s, int nreq, const double* arrival_s,
                          const int32_t* req_npairs, const int32_t* node_a,
                          const int32_t* node_b, int32_t* cost, int32_t* status,
                          double* latency_s, double* wall_s)
{
    if (!s || nreq < 0 || (nreq > 0 && (!arrival_s || !req_npairs || !node_a || !node_b ||
                                        !cost || !status || !latency_s)))
        return set_err(POYALGN_EINVAL, "null argument");
    std::vector<int64_t> tickets(nreq, 0);
    std::vector<long long> first(nreq, 0);
    long long at = 0;
    for (int r = 0; r < nreq; r++) {
        if (req_npairs[r] < 1 || (r > 0 && arrival_s[r] < arrival_s[r - 1]))
            return set_err(POYALGN_EINVAL, "request %d: bad size or arrival order", r);
        first[r] = at;
        at += req_npairs[r];
    }
    const Clock::time_point t0 = Clock::now() + std::chrono::milliseconds(1);
    auto when = [&](int r) {
        return t0 + std::chrono::duration_cast<Clock::duration>(
                        std::chrono::duration<double>(arrival_s[r]));
    };
    int rc = 0;
    for (int r = 0; r < nreq && !rc; r++) {
        const Clock::time_point t = when(r);
        for (;;) {
            const auto left = t - Clock::now();
            if (left <= Clock::duration::zero()) break;
            if (left > std::chrono::microseconds(200))
                std::this_thread::sleep_for(left - std::chrono::microseconds(100));
            else
                std::this_thread::yield();
        }
        const int q = submit_at(s, req_npairs[r], node_a + first[r], node_b + first[r], t,
                                &tickets[r]);
        if (q == POYALGN_EBUSY) {
            tickets[r] = 0;
        } else if (q) {
            rc = q;
        }
    }
    Clock::time_point last = t0;
    for (int r = 0; r < nreq; r++) {
        const long long f = first[r];
        if (!tickets[r]) {
            for (int p = 0; p < req_npairs[r]; p++) {
                cost[f + p] = 0;
                status[f + p] = 1;
            }
            latency_s[r] = -1.0;
            continue;
        }
        double lat = 0.0;
        const int w = poyalgn_server_wait(s, tickets[r], -1, cost + f, status + f, nullptr,
                                          nullptr, 0, &lat);
        if (w && !rc) rc = w;
        latency_s[r] = lat;
        const Clock::time_point done =
            when(r) + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(lat));
        last = std::max(last, done);
    }
    if (wall_s) *wall_s = nreq ? std::chrono::duration<double>(last - when(0)).count() : 0.0;
    return rc;
}

int poyalgn_server_stats(const poyalgn_server* s, int64_t* batches, int64_t* pairs,
                         int64_t* refused)
{
    if (!s) return set_err(POYALGN_EINVAL, "null server");
    poyalgn_server* m = const_cast<poyalgn_server*>(s);
    std::lock_guard<std::mutex> g(m->mu);
    if (batches) *batches = s->n_batches;
    if (pairs) *pairs = s->n_pairs;
    if (refused) *refused = s->n_refused;
    return 0;
}

}  // extern "C"
