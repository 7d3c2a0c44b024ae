// Device-resident node sequences (poyalgn_store) and the level-batched tree
// downpass built on them.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "pa_cost.h"
#include "pa_runtime.h"

using namespace pa;

namespace {

constexpr long long kAlign = 16;

long long align_up(long long x) { return (x + kAlign - 1) & ~(kAlign - 1); }

bool valid_node(const poyalgn_store* s, int node)
{
    return node >= 0 && node < (int)s->len.size();
}

// Enqueue DOS.median for n resident pairs and wait for the per-pair ints.
// Medians land in the arena after `used` (keep) or in scratch.
int store_batch(poyalgn_store* s, const poyalgn_cm* cm, int n, const int32_t* na,
                const int32_t* nb, int keep, int32_t* median_node, int32_t* cost,
                int32_t* maxcost, int32_t* status)
{
    poyalgn_ctx* c = s->ctx;
    int rc;
    if ((rc = ensure_device(c))) return rc;
    const size_t ni = (size_t)n;
    // metadata block: offa | offb | out_off (int64) | lena | lenb (int32)
    s->hmeta.resize(ni * 32);
    long long* offa = reinterpret_cast<long long*>(s->hmeta.data());
    long long* offb = offa + ni;
    long long* oo = offb + ni;
    int* lena = reinterpret_cast<int*>(oo + ni);
    int* lenb = lena + ni;
    long long total = 0;
    int maxmn = 2;
    for (int k = 0; k < n; k++) {
        if (!valid_node(s, na[k]) || !valid_node(s, nb[k]))
            return set_err(POYALGN_EINVAL, "pair %d: unknown node (%d, %d)", k, na[k], nb[k]);
        offa[k] = s->off[na[k]];
        offb[k] = s->off[nb[k]];
        lena[k] = s->len[na[k]];
        lenb[k] = s->len[nb[k]];
        oo[k] = total;
        total += align_up((long long)lena[k] + lenb[k] + 2);
        maxmn = std::max(maxmn, lena[k] + lenb[k]);
    }
    const long long base = align_up(s->used);
    if (keep && base + total > s->cap)
        return set_err(POYALGN_ENOMEM, "store full: %lld of %lld bytes used, batch needs %lld",
                       s->used, s->cap, total);
    if ((rc = reserve(s->meta, ni * 32))) return rc;
    if ((rc = reserve(s->ints, ni * 4 * 7))) return rc;
    if ((rc = reserve(s->bytes, (size_t)total * (keep ? 3 : 4)))) return rc;
    cudaStream_t st = c->stream;
    CU(cudaMemcpyAsync(s->meta.p, s->hmeta.data(), ni * 32, cudaMemcpyHostToDevice, st));
    const long long* d_offa = as<long long>(s->meta);
    const int* d_lena = reinterpret_cast<const int*>(d_offa + 3 * ni);
    int* I = as<int>(s->ints);
    uint8_t* B = as<uint8_t>(s->bytes);
    uint8_t* arena = as<uint8_t>(s->arena);
    uint8_t* med = keep ? arena + base : B + 3 * total;
    if ((rc = run_batch(c, cm, cm->h.cost_model == 1, n, maxmn, total, arena, d_offa, d_lena,
                        d_offa + ni, d_lena + ni, d_offa + 2 * ni, I, I + ni, I + 2 * ni,
                        I + 3 * ni, I + 4 * ni, I + 5 * ni, B, B + total, med, B + 2 * total,
                        I + 6 * ni, nullptr, nullptr, 1, st)))
        return rc;
    // cost | maxcost | alen | mlen | wlen | status
    s->hints.resize(ni * 6);
    CU(cudaMemcpyAsync(s->hints.data(), I, ni * 6 * sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    const int* h = s->hints.data();
    int failed = -1;
    for (int k = 0; k < n; k++) {
        if (cost) cost[k] = h[k];
        if (maxcost) maxcost[k] = h[ni + k];
        if (status) status[k] = h[5 * ni + k];
        if (h[5 * ni + k] != 0 && failed < 0) failed = k;
    }
    if (keep) {
        for (int k = 0; k < n; k++) {
            const int ml = h[3 * ni + k];
            const bool ok = h[5 * ni + k] == 0 && ml > 0;
            if (median_node) median_node[k] = ok ? (int)s->len.size() : -1;
            if (!ok) continue;
            s->off.push_back(base + oo[k] + lena[k] + lenb[k] + 2 - ml);
            s->len.push_back(ml);
        }
        s->used = base + total;
    }
    if (failed >= 0)
        return set_err(POYALGN_EPAIR, "pair %d failed with status %d", failed,
                       h[5 * ni + failed]);
    return 0;
}

// median_3_no_union's choice and median (src/seqCS.ml:1123-1147): of the
// alignments 2k (parent, child1) and 2k + 1 (parent, child2), keep the one
// of lower cost (the second on a tie) and write seq_get_median_2d_no_gaps
// (src/seq.c:259-272) of its aligned pair back to front into node k's
// region. res[4k..4k+3] = cost, worst cost, median length, status.
__global__ void median3_pick_kernel(const Tables* tg, int n, const long long* out_off,
                                    const int* lena, const int* lenb, const int* I,
                                    const uint8_t* ea, const uint8_t* eb, uint8_t* dst,
                                    const long long* dst_end, int* res)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const Tables& t = *tg;
    const int n2 = 2 * n, a = 2 * k, b = 2 * k + 1;
    const int *cost = I, *maxcost = I + n2, *alen = I + 2 * n2, *status = I + 5 * n2;
    const int st = status[a] != 0 ? status[a] : status[b];
    if (st != 0) {
        res[4 * k + 3] = st;
        return;
    }
    const int j = cost[a] < cost[b] ? a : b;
    const long long start = out_off[j] + lena[j] + lenb[j] + 2 - alen[j];
    const uint8_t* x = ea + start;  // aligned parent
    const uint8_t* y = eb + start;  // aligned child
    uint8_t* o = dst + dst_end[k];
    int w = 0;
    for (int i = alen[j] - 1; i >= 0; i--) {
        const int m = t.median[(x[i] << t.lcm) + y[i]];
        if (m != t.gap) o[-(++w)] = (uint8_t)m;
    }
    o[-(++w)] = (uint8_t)t.gap;
    res[4 * k] = cost[j];
    res[4 * k + 1] = maxcost[j];
    res[4 * k + 2] = w;
    res[4 * k + 3] = 0;
}

int store_median3(poyalgn_store* s, const poyalgn_cm* cm, int n, const int32_t* parent,
                  const int32_t* child1, const int32_t* child2, int32_t* node, int32_t* cost,
                  int32_t* maxcost, int32_t* status)
{
    poyalgn_ctx* c = s->ctx;
    int rc;
    if ((rc = ensure_device(c))) return rc;
    const size_t n2 = 2 * (size_t)n, ni = (size_t)n;
    // metadata: offa | offb | out_off (int64, 2n each) | lena | lenb (int32,
    // 2n each) | node region ends (int64, n)
    s->hmeta.resize(n2 * 32 + ni * 8);
    long long* offa = reinterpret_cast<long long*>(s->hmeta.data());
    long long* offb = offa + n2;
    long long* oo = offb + n2;
    int* lena = reinterpret_cast<int*>(oo + n2);
    int* lenb = lena + n2;
    long long* dend = reinterpret_cast<long long*>(lenb + n2);
    long long total = 0, ntotal = 0;
    int maxmn = 2;
    for (int k = 0; k < n; k++) {
        const int32_t nb2[2] = {child1[k], child2[k]};
        if (!valid_node(s, parent[k]) || !valid_node(s, child1[k]) || !valid_node(s, child2[k]))
            return set_err(POYALGN_EINVAL, "triple %d: unknown node (%d, %d, %d)", k, parent[k],
                           child1[k], child2[k]);
        for (int h = 0; h < 2; h++) {
            const size_t q = 2 * (size_t)k + h;
            offa[q] = s->off[parent[k]];
            offb[q] = s->off[nb2[h]];
            lena[q] = s->len[parent[k]];
            lenb[q] = s->len[nb2[h]];
            oo[q] = total;
            total += align_up((long long)lena[q] + lenb[q] + 2);
            maxmn = std::max(maxmn, lena[q] + lenb[q]);
        }
        // the median has at most one entry per aligned column plus the gap
        ntotal += align_up((long long)s->len[parent[k]] +
                           std::max(s->len[child1[k]], s->len[child2[k]]) + 2);
        dend[k] = ntotal;
    }
    const long long base = align_up(s->used);
    if (base + ntotal > s->cap)
        return set_err(POYALGN_ENOMEM, "store full: %lld of %lld bytes used, batch needs %lld",
                       s->used, s->cap, ntotal);
    if ((rc = reserve(s->meta, n2 * 32 + ni * 8))) return rc;
    if ((rc = reserve(s->ints, n2 * 4 * 7 + ni * 4 * 4))) return rc;
    if ((rc = reserve(s->bytes, (size_t)total * 4))) return rc;
    cudaStream_t st = c->stream;
    CU(cudaMemcpyAsync(s->meta.p, s->hmeta.data(), n2 * 32 + ni * 8, cudaMemcpyHostToDevice, st));
    const long long* d_offa = as<long long>(s->meta);
    const int* d_lena = reinterpret_cast<const int*>(d_offa + 3 * n2);
    const long long* d_dend = reinterpret_cast<const long long*>(d_lena + 2 * n2);
    int* I = as<int>(s->ints);
    int* res = I + 7 * n2;
    uint8_t* B = as<uint8_t>(s->bytes);
    uint8_t* arena = as<uint8_t>(s->arena);
    if ((rc = run_batch(c, cm, cm->h.cost_model == 1, (int)n2, maxmn, total, arena, d_offa,
                        d_lena, d_offa + n2, d_lena + n2, d_offa + 2 * n2, I, I + n2,
                        I + 2 * n2, I + 3 * n2, I + 4 * n2, I + 5 * n2, B, B + total,
                        B + 2 * total, B + 3 * total, I + 6 * n2, nullptr, nullptr, 1, st)))
        return rc;
    median3_pick_kernel<<<(n + 127) / 128, 128, 0, st>>>(cm->d, n, d_offa + 2 * n2, d_lena,
                                                         d_lena + n2, I, B, B + total,
                                                         arena + base, d_dend, res);
    CU(cudaGetLastError());
    s->hints.resize(ni * 4);
    CU(cudaMemcpyAsync(s->hints.data(), res, ni * 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    const int* h = s->hints.data();
    int failed = -1;
    for (int k = 0; k < n; k++) {
        const int ok = h[4 * k + 3] == 0;
        if (cost) cost[k] = h[4 * k];
        if (maxcost) maxcost[k] = h[4 * k + 1];
        if (status) status[k] = h[4 * k + 3];
        if (!ok && failed < 0) failed = k;
        if (node) node[k] = ok ? (int)s->len.size() : -1;
        if (!ok) continue;
        s->off.push_back(base + dend[k] - h[4 * k + 2]);
        s->len.push_back(h[4 * k + 2]);
    }
    s->used = base + ntotal;
    if (failed >= 0)
        return set_err(POYALGN_EPAIR, "triple %d failed with status %d", failed,
                       h[4 * failed + 3]);
    return 0;
}

// Cost_matrix.Two_D.get_closest (src/cost_matrix.ml:1387-1426) for a matrix
// with combinations and no levels: b without the gap bit unless a or b is
// the gap (both carrying it: the gap), then the first of its states
// (BitSet.Int.list_of_packed_max reversed: increasing codes) of lowest cost
// against a. 0 when b has no state (the reference fails there).
__device__ int closest_state(const Tables& t, int a, int b)
{
    const int gap = t.gap;
    const int bb = (a == gap || b == gap) ? b : ((a & gap) && (b & gap)) ? gap : (b & ~gap);
    int best = 0, bc = 0x7fffffff;
    for (int bit = 0; bit < t.lcm; bit++) {
        const int x = 1 << bit;
        if (!(bb & x)) continue;
        const int c = tcost(t, a, x);
        if (c < bc) {
            best = x;
            bc = c;
        }
    }
    return best;
}

// Align.closest's resolution of pair k (src/sequence.ml:1180-1237): node2
// all gaps -> itself (kind 0); equal sequences -> position by position with
// the gap bit cleared past position 0 (kind 1); otherwise the aligned pair of
// the batch (kind 2). The resolved sequence, gaps removed and the leading
// gap prepended (remove_gaps2), is written back to front into the node's
// region. res[3k..3k+2] = length, kind, status.
__global__ void closest_map_kernel(const Tables* tg, int n, const uint8_t* arena,
                                   const long long* offa, const int* lena, const long long* offb,
                                   const int* lenb, const long long* out_off, const int* I,
                                   const uint8_t* ea, const uint8_t* eb, uint8_t* dst,
                                   const long long* dst_end, int* res)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const Tables& t = *tg;
    const int gap = t.gap;
    const uint8_t* s1 = arena + offa[k];
    const uint8_t* s2 = arena + offb[k];
    const int l1 = lena[k], l2 = lenb[k];
    bool empty = true;
    for (int i = 0; i < l2 && empty; i++) empty = s2[i] == gap;
    if (empty) {
        res[3 * k] = l2;
        res[3 * k + 1] = 0;
        res[3 * k + 2] = 0;
        return;
    }
    bool equal = l1 == l2;
    for (int i = 0; i < l1 && equal; i++) equal = s1[i] == s2[i];
    const uint8_t *x = s1, *y = s2;
    int len = l1;
    if (!equal) {
        const int st = I[5 * n + k];
        if (st != 0) {
            res[3 * k + 2] = st;
            return;
        }
        len = I[2 * n + k];
        const long long start = out_off[k] + l1 + l2 + 2 - len;
        x = ea + start;
        y = eb + start;
    }
    uint8_t* o = dst + dst_end[k];
    int w = 0;
    for (int i = len - 1; i >= 0; i--) {
        int a = x[i], b = y[i];
        if (equal && i > 0) {
            a &= ~gap;
            b &= ~gap;
        }
        const int c = (a > 0 && b > 0) ? closest_state(t, a, b) : 0;
        if (c == 0) {
            res[3 * k + 2] = POYALGN_PAIR_EMPTY_STATE;
            return;
        }
        if (c != gap) o[-(++w)] = (uint8_t)c;
    }
    o[-(++w)] = (uint8_t)gap;
    res[3 * k] = w;
    res[3 * k + 1] = equal ? 1 : 2;
    res[3 * k + 2] = 0;
}

// Metadata of n resident pairs for a batch: offa | offb | out_off (int64) |
// lena | lenb (int32); returns the output bytes (cap la + lb + 2 per pair).
long long pair_meta(const poyalgn_store* s, int n, const int32_t* na, const int32_t* nb,
                    std::vector<uint8_t>& hmeta, int* maxmn)
{
    const size_t ni = (size_t)n;
    hmeta.resize(ni * 32);
    long long* offa = reinterpret_cast<long long*>(hmeta.data());
    long long* offb = offa + ni;
    long long* oo = offb + ni;
    int* lena = reinterpret_cast<int*>(oo + ni);
    int* lenb = lena + ni;
    long long total = 0;
    *maxmn = 2;
    for (int k = 0; k < n; k++) {
        offa[k] = s->off[na[k]];
        offb[k] = s->off[nb[k]];
        lena[k] = s->len[na[k]];
        lenb[k] = s->len[nb[k]];
        oo[k] = total;
        total += align_up((long long)lena[k] + lenb[k] + 2);
        *maxmn = std::max(*maxmn, lena[k] + lenb[k]);
    }
    return total;
}

// Align.cost_2 of n resident pairs (a first): the linear band doubling's
// cost (Align.cost_2 without deltaw) or algn_CAML_cost_affine_3.
int store_cost2(poyalgn_store* s, const poyalgn_cm* cm, int n, const int32_t* na,
                const int32_t* nb, int32_t* cost, int32_t* status)
{
    poyalgn_ctx* c = s->ctx;
    int rc, maxmn;
    const size_t ni = (size_t)n;
    const long long total = pair_meta(s, n, na, nb, s->hmeta, &maxmn);
    if ((rc = reserve(s->meta, ni * 32))) return rc;
    if ((rc = reserve(s->ints, ni * 4 * 7))) return rc;
    if ((rc = reserve(s->bytes, (size_t)total * 4))) return rc;
    cudaStream_t st = c->stream;
    CU(cudaMemcpyAsync(s->meta.p, s->hmeta.data(), ni * 32, cudaMemcpyHostToDevice, st));
    const long long* d_offa = as<long long>(s->meta);
    const int* d_lena = reinterpret_cast<const int*>(d_offa + 3 * ni);
    int* I = as<int>(s->ints);
    uint8_t* B = as<uint8_t>(s->bytes);
    uint8_t* arena = as<uint8_t>(s->arena);
    if (cm->h.cost_model == 1)
        rc = run_nobt(c, cm, n, maxmn, arena, d_offa, d_lena, d_offa + ni, d_lena + ni,
                      NOBT_NO_MISSING, I, I + 5 * ni, st);
    else
        rc = run_batch(c, cm, 0, n, maxmn, total, arena, d_offa, d_lena, d_offa + ni,
                       d_lena + ni, d_offa + 2 * ni, I, I + ni, I + 2 * ni, I + 3 * ni,
                       I + 4 * ni, I + 5 * ni, B, B + total, B + 2 * total, B + 3 * total,
                       I + 6 * ni, nullptr, nullptr, 0, st);
    if (rc) return rc;
    s->hints.resize(ni * 6);
    CU(cudaMemcpyAsync(s->hints.data(), I, ni * 6 * sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    for (int k = 0; k < n; k++) {
        cost[k] = s->hints[k];
        status[k] = s->hints[5 * ni + k];
    }
    return 0;
}

int store_closest(poyalgn_store* s, const poyalgn_cm* cm, int n, const int32_t* node1,
                  const int32_t* node2, int32_t* out_node, int32_t* cost, int32_t* status)
{
    poyalgn_ctx* c = s->ctx;
    int rc, maxmn;
    if ((rc = ensure_device(c))) return rc;
    if (!cm->t.comb) return set_err(POYALGN_EUNSUPPORTED, "closest needs a matrix with combinations");
    const size_t ni = (size_t)n;
    for (int k = 0; k < n; k++)
        if (!valid_node(s, node1[k]) || !valid_node(s, node2[k]))
            return set_err(POYALGN_EINVAL, "pair %d: unknown node (%d, %d)", k, node1[k], node2[k]);
    const long long total = pair_meta(s, n, node1, node2, s->hmeta, &maxmn);
    // node regions: at most one entry per aligned column plus the gap
    s->hmeta.resize(ni * 40);
    long long* dend = reinterpret_cast<long long*>(s->hmeta.data() + ni * 32);
    const int* lena = reinterpret_cast<const int*>(s->hmeta.data() + ni * 24);
    const int* lenb = lena + ni;
    long long ntotal = 0;
    for (int k = 0; k < n; k++) {
        ntotal += align_up((long long)lena[k] + lenb[k] + 2);
        dend[k] = ntotal;
    }
    const long long base = align_up(s->used);
    if (base + ntotal > s->cap)
        return set_err(POYALGN_ENOMEM, "store full: %lld of %lld bytes used, batch needs %lld",
                       s->used, s->cap, ntotal);
    if ((rc = reserve(s->meta, ni * 40))) return rc;
    if ((rc = reserve(s->ints, ni * 4 * 10))) return rc;
    if ((rc = reserve(s->bytes, (size_t)total * 4))) return rc;
    cudaStream_t st = c->stream;
    CU(cudaMemcpyAsync(s->meta.p, s->hmeta.data(), ni * 40, cudaMemcpyHostToDevice, st));
    const long long* d_offa = as<long long>(s->meta);
    const int* d_lena = reinterpret_cast<const int*>(d_offa + 3 * ni);
    const long long* d_dend = d_offa + 4 * ni;
    int* I = as<int>(s->ints);
    int* res = I + 7 * ni;
    uint8_t* B = as<uint8_t>(s->bytes);
    uint8_t* arena = as<uint8_t>(s->arena);
    if ((rc = run_batch(c, cm, cm->h.cost_model == 1, n, maxmn, total, arena, d_offa, d_lena,
                        d_offa + ni, d_lena + ni, d_offa + 2 * ni, I, I + ni, I + 2 * ni,
                        I + 3 * ni, I + 4 * ni, I + 5 * ni, B, B + total, B + 2 * total,
                        B + 3 * total, I + 6 * ni, nullptr, nullptr, 1, st)))
        return rc;
    closest_map_kernel<<<(n + 127) / 128, 128, 0, st>>>(cm->d, n, arena, d_offa, d_lena,
                                                        d_offa + ni, d_lena + ni, d_offa + 2 * ni,
                                                        I, B, B + total, arena + base, d_dend,
                                                        res);
    CU(cudaGetLastError());
    std::vector<int> h(ni * 3);
    CU(cudaMemcpyAsync(h.data(), res, ni * 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    std::vector<int32_t> ca, cb, cc(ni, 0), cs(ni, 0);
    std::vector<int> which;
    const long long dend_last = ntotal;
    int failed = -1;
    for (int k = 0; k < n; k++) {
        const int st_k = h[3 * k + 2], kind = h[3 * k + 1];
        status[k] = st_k;
        cost[k] = 0;
        out_node[k] = -1;
        if (st_k != 0) {
            if (failed < 0) failed = k;
            continue;
        }
        if (kind == 0) {
            out_node[k] = node2[k];
            continue;
        }
        out_node[k] = (int)s->len.size();
        s->off.push_back(base + dend[k] - h[3 * k]);
        s->len.push_back(h[3 * k]);
        if (kind == 2) {  // Align.cost_2 of node1 and the resolved sequence
            which.push_back(k);
            ca.push_back(node1[k]);
            cb.push_back(out_node[k]);
        }
    }
    s->used = base + dend_last;
    if (!which.empty()) {
        if ((rc = store_cost2(s, cm, (int)which.size(), ca.data(), cb.data(), cc.data(),
                              cs.data())))
            return rc;
        for (size_t q = 0; q < which.size(); q++) {
            cost[which[q]] = cc[q];
            if (cs[q] != 0) {
                status[which[q]] = cs[q];
                if (failed < 0 || which[q] < failed) failed = which[q];
            }
        }
    }
    if (failed >= 0)
        return set_err(POYALGN_EPAIR, "pair %d failed with status %d", failed, status[failed]);
    return 0;
}

// Sequence.readjust (src/sequence.ml:2097-2158) for n triples, in rounds of
// batches: algn = DOS.median's (cost, median) for both cost models.
int store_readjust(poyalgn_store* s, const poyalgn_cm* cm, int n, const int32_t* ca,
                   const int32_t* cb, const int32_t* cp, int32_t* node, int32_t* cost3,
                   int32_t* cost2, int32_t* status)
{
    const size_t ni = (size_t)n;
    for (size_t k = 0; k < ni; k++) {
        status[k] = 0;
        node[k] = -1;
        cost3[k] = cost2[k] = 0;
    }
    std::vector<int32_t> na(3 * ni), nb(3 * ni), med(3 * ni), cst(3 * ni), st(3 * ni);
    std::vector<char> bad(ni, 0);
    auto round = [&](int keep) -> int {  // 3 n alignments, per-triple failures recorded
        const int rc = store_batch(s, cm, (int)(3 * ni), na.data(), nb.data(), keep, med.data(),
                                   cst.data(), nullptr, st.data());
        if (rc && rc != POYALGN_EPAIR) return rc;
        for (size_t q = 0; q < 3 * ni; q++)
            if (st[q] != 0 && !bad[q / 3]) {
                bad[q / 3] = 1;
                status[q / 3] = st[q];
            }
        return 0;
    };
    int rc;
    // make_center a b c (c = parent): ab, bc, ac
    for (size_t k = 0; k < ni; k++) {
        na[3 * k] = ca[k], nb[3 * k] = cb[k];
        na[3 * k + 1] = cb[k], nb[3 * k + 1] = cp[k];
        na[3 * k + 2] = ca[k], nb[3 * k + 2] = cp[k];
    }
    if ((rc = round(1))) return rc;
    std::vector<int32_t> m1 = med, c1 = cst;
    // abc = algn ab c, bca = algn bc a, acb = algn ac b
    for (size_t k = 0; k < ni; k++) {
        const bool ok = !bad[k];
        na[3 * k] = ok ? m1[3 * k] : ca[k], nb[3 * k] = cp[k];
        na[3 * k + 1] = ok ? m1[3 * k + 1] : ca[k], nb[3 * k + 1] = ca[k];
        na[3 * k + 2] = ok ? m1[3 * k + 2] : ca[k], nb[3 * k + 2] = cb[k];
    }
    if ((rc = round(0))) return rc;
    // the cheapest route's centre, resolved with Align.closest
    std::vector<int32_t> x1(ni), x2(ni), cn(ni), cc(ni), cs(ni);
    for (size_t k = 0; k < ni; k++) {
        const long long cabc = (long long)cst[3 * k] + c1[3 * k];
        const long long cbca = (long long)cst[3 * k + 1] + c1[3 * k + 1];
        const long long cacb = (long long)cst[3 * k + 2] + c1[3 * k + 2];
        int32_t p, q;  // closest p q: q resolved towards p
        if (cabc <= cbca) {
            if (cabc <= cacb) p = cp[k], q = m1[3 * k];  // closest c ab
            else p = cb[k], q = m1[3 * k + 2];           // closest b ac
        } else if (cbca < cacb) {
            p = ca[k], q = m1[3 * k + 1];  // closest a bc
        } else {
            p = cb[k], q = m1[3 * k + 2];  // closest b ac
        }
        x1[k] = bad[k] ? ca[k] : p;
        x2[k] = bad[k] ? cb[k] : q;
    }
    rc = store_closest(s, cm, n, x1.data(), x2.data(), cn.data(), cc.data(), cs.data());
    if (rc && rc != POYALGN_EPAIR) return rc;
    for (size_t k = 0; k < ni; k++)
        if (cs[k] != 0 && !bad[k]) {
            bad[k] = 1;
            status[k] = cs[k];
        }
    // the centre against both children and the parent
    for (size_t k = 0; k < ni; k++) {
        const int32_t m = bad[k] ? ca[k] : cn[k];
        na[3 * k] = ca[k], nb[3 * k] = m;
        na[3 * k + 1] = cb[k], nb[3 * k + 1] = m;
        na[3 * k + 2] = cp[k], nb[3 * k + 2] = m;
    }
    if ((rc = round(0))) return rc;
    int failed = -1;
    for (size_t k = 0; k < ni; k++) {
        if (bad[k]) {
            if (failed < 0) failed = (int)k;
            continue;
        }
        node[k] = cn[k];
        cost2[k] = cst[3 * k] + cst[3 * k + 1];
        cost3[k] = cost2[k] + cst[3 * k + 2];
    }
    if (failed >= 0)
        return set_err(POYALGN_EPAIR, "triple %d failed with status %d", failed, status[failed]);
    return 0;
}

}  // namespace

extern "C" {

int poyalgn_store_create(poyalgn_ctx* ctx, int64_t capacity_bytes, poyalgn_store** out)
{
    if (!ctx || !out || capacity_bytes < 1) return set_err(POYALGN_EINVAL, "bad store arguments");
    *out = nullptr;
    int rc;
    if ((rc = ensure_device(ctx))) return rc;
    poyalgn_store* s = new (std::nothrow) poyalgn_store;
    if (!s) return set_err(POYALGN_ENOMEM, "store allocation");
    s->ctx = ctx;
    if ((rc = reserve(s->arena, (size_t)capacity_bytes))) {
        delete s;
        return rc;
    }
    s->cap = capacity_bytes;
    *out = s;
    return 0;
}

void poyalgn_store_free(poyalgn_store* s)
{
    if (!s) return;
    cudaSetDevice(s->ctx->device);
    release(s->arena);
    release(s->meta);
    release(s->ints);
    release(s->bytes);
    delete s;
}

int poyalgn_store_add(poyalgn_store* s, const uint8_t* seq, int len, int32_t* node)
{
    if (!s || !seq || !node || len < 1) return set_err(POYALGN_EINVAL, "bad sequence");
    const long long at = align_up(s->used);
    if (at + len > s->cap)
        return set_err(POYALGN_ENOMEM, "store full: %lld of %lld bytes used, sequence needs %d",
                       s->used, s->cap, len);
    int rc;
    if ((rc = ensure_device(s->ctx))) return rc;
    CU(cudaMemcpy(as<uint8_t>(s->arena) + at, seq, (size_t)len, cudaMemcpyHostToDevice));
    s->off.push_back(at);
    s->len.push_back(len);
    s->used = at + len;
    *node = (int32_t)(s->len.size() - 1);
    return 0;
}

int poyalgn_store_count(const poyalgn_store* s) { return s ? (int)s->len.size() : 0; }

int poyalgn_store_length(const poyalgn_store* s, int node)
{
    if (!s || !valid_node(s, node)) return set_err(POYALGN_EINVAL, "unknown node %d", node);
    return s->len[node];
}

int poyalgn_store_read(poyalgn_store* s, int node, uint8_t* out, int cap)
{
    if (!s || !out || !valid_node(s, node)) return set_err(POYALGN_EINVAL, "unknown node %d", node);
    if (cap < s->len[node]) return set_err(POYALGN_EINVAL, "capacity %d < %d", cap, s->len[node]);
    int rc;
    if ((rc = ensure_device(s->ctx))) return rc;
    CU(cudaStreamSynchronize(s->ctx->stream));
    CU(cudaMemcpy(out, as<uint8_t>(s->arena) + s->off[node], (size_t)s->len[node],
                  cudaMemcpyDeviceToHost));
    return 0;
}

int poyalgn_store_truncate(poyalgn_store* s, int nodes)
{
    if (!s || nodes < 0 || nodes > (int)s->len.size())
        return set_err(POYALGN_EINVAL, "bad node count %d", nodes);
    s->off.resize(nodes);
    s->len.resize(nodes);
    long long end = 0;
    for (int k = 0; k < nodes; k++) end = std::max(end, s->off[k] + s->len[k]);
    s->used = end;
    return 0;
}

int poyalgn_store_median_batch(poyalgn_store* s, const poyalgn_cm* cm, int npairs,
                               const int32_t* node_a, const int32_t* node_b, int keep,
                               int32_t* median_node, int32_t* cost, int32_t* maxcost,
                               int32_t* status)
{
    if (!s || !cm || npairs < 0 || (npairs > 0 && (!node_a || !node_b || !cost)))
        return set_err(POYALGN_EINVAL, "null argument");
    if (npairs == 0) return 0;
    return store_batch(s, cm, npairs, node_a, node_b, keep, median_node, cost, maxcost, status);
}

int poyalgn_downpass(poyalgn_store* s, const poyalgn_cm* cm, int nleaves,
                     const int32_t* leaf_node, int ninternal, const int32_t* left,
                     const int32_t* right, int32_t* internal_node, int32_t* internal_cost,
                     int64_t* total_cost, int32_t* levels)
{
    if (!s || !cm || nleaves < 1 || ninternal < 0 || !leaf_node ||
        (ninternal > 0 && (!left || !right || !internal_node || !internal_cost)) || !total_cost)
        return set_err(POYALGN_EINVAL, "null argument");
    // level of each internal node: 1 + the deeper child's level (leaves 0)
    std::vector<int> level(ninternal, 0);
    int depth = 0;
    for (int k = 0; k < ninternal; k++) {
        int lv = 0;
        for (int ch : {left[k], right[k]}) {
            if (ch < 0 || ch >= nleaves + k)
                return set_err(POYALGN_EINVAL, "internal node %d: child %d is not an earlier node",
                               k, ch);
            if (ch < nleaves) {
                if (!valid_node(s, leaf_node[ch]))
                    return set_err(POYALGN_EINVAL, "leaf %d: unknown node %d", ch, leaf_node[ch]);
            } else {
                lv = std::max(lv, level[ch - nleaves]);
            }
        }
        level[k] = lv + 1;
        depth = std::max(depth, level[k]);
    }
    auto node_of = [&](int ch) { return ch < nleaves ? leaf_node[ch] : internal_node[ch - nleaves]; };
    std::vector<int> idx, na, nb, med, cst;
    long long total = 0;
    for (int lv = 1; lv <= depth; lv++) {
        idx.clear();
        na.clear();
        nb.clear();
        for (int k = 0; k < ninternal; k++) {
            if (level[k] != lv) continue;
            idx.push_back(k);
            na.push_back(node_of(left[k]));
            nb.push_back(node_of(right[k]));
        }
        const int n = (int)idx.size();
        med.assign(n, -1);
        cst.assign(n, 0);
        int rc = store_batch(s, cm, n, na.data(), nb.data(), 1, med.data(), cst.data(), nullptr,
                             nullptr);
        if (rc) return rc;
        for (int t = 0; t < n; t++) {
            internal_node[idx[t]] = med[t];
            internal_cost[idx[t]] = cst[t];
            total += cst[t];
        }
    }
    *total_cost = total;
    if (levels) *levels = depth;
    return 0;
}

int poyalgn_store_median3_batch(poyalgn_store* s, const poyalgn_cm* cm, int n,
                                const int32_t* parent, const int32_t* child1,
                                const int32_t* child2, int32_t* node, int32_t* cost,
                                int32_t* maxcost, int32_t* status)
{
    if (!s || !cm || n < 0 || (n > 0 && (!parent || !child1 || !child2)))
        return set_err(POYALGN_EINVAL, "null argument");
    if (n == 0) return 0;
    return store_median3(s, cm, n, parent, child1, child2, node, cost, maxcost, status);
}

int poyalgn_store_closest_batch(poyalgn_store* s, const poyalgn_cm* cm, int n,
                                const int32_t* node1, const int32_t* node2, int32_t* out_node,
                                int32_t* cost, int32_t* status)
{
    if (!s || !cm || n < 0 || (n > 0 && (!node1 || !node2 || !out_node || !cost || !status)))
        return set_err(POYALGN_EINVAL, "null argument");
    if (n == 0) return 0;
    return store_closest(s, cm, n, node1, node2, out_node, cost, status);
}

int poyalgn_store_readjust_batch(poyalgn_store* s, const poyalgn_cm* cm, int n,
                                 const int32_t* child_a, const int32_t* child_b,
                                 const int32_t* parent, int32_t* node, int32_t* cost3,
                                 int32_t* cost2, int32_t* status)
{
    if (!s || !cm || n < 0 ||
        (n > 0 && (!child_a || !child_b || !parent || !node || !cost3 || !cost2 || !status)))
        return set_err(POYALGN_EINVAL, "null argument");
    if (n == 0) return 0;
    for (int k = 0; k < n; k++)
        if (!valid_node(s, child_a[k]) || !valid_node(s, child_b[k]) || !valid_node(s, parent[k]))
            return set_err(POYALGN_EINVAL, "triple %d: unknown node", k);
    return store_readjust(s, cm, n, child_a, child_b, parent, node, cost3, cost2, status);
}

int poyalgn_uppass(poyalgn_store* s, const poyalgn_cm* cm, int nleaves,
                   const int32_t* leaf_node, int ninternal, const int32_t* left,
                   const int32_t* right, const int32_t* internal_node, int32_t* final_node,
                   int32_t* final_cost, int32_t* levels)
{
    if (!s || !cm || nleaves < 1 || ninternal < 1 || !leaf_node || !left || !right ||
        !internal_node || !final_node || !final_cost)
        return set_err(POYALGN_EINVAL, "null argument");
    // parent of every internal node (children come before their parent)
    std::vector<int> up(ninternal, -1), depth(ninternal, 0);
    for (int k = 0; k < ninternal; k++)
        for (int ch : {left[k], right[k]}) {
            if (ch < 0 || ch >= nleaves + k)
                return set_err(POYALGN_EINVAL, "internal node %d: child %d is not an earlier node",
                               k, ch);
            if (ch >= nleaves) {
                if (up[ch - nleaves] >= 0)
                    return set_err(POYALGN_EINVAL, "internal node %d has two parents",
                                   ch - nleaves);
                up[ch - nleaves] = k;
            }
        }
    const int root = ninternal - 1;
    if (up[root] >= 0) return set_err(POYALGN_EINVAL, "the last internal node is not the root");
    int maxd = 0;
    for (int k = root - 1; k >= 0; k--) {  // parents come after their children
        if (up[k] < 0) return set_err(POYALGN_EINVAL, "internal node %d has no parent", k);
        depth[k] = depth[up[k]] + 1;
        maxd = std::max(maxd, depth[k]);
    }
    auto state = [&](int ch) { return ch < nleaves ? leaf_node[ch] : internal_node[ch - nleaves]; };
    final_node[root] = internal_node[root];
    final_cost[root] = 0;
    std::vector<int32_t> idx, pa, c1, c2, nd, cs;
    for (int d = 1; d <= maxd; d++) {
        idx.clear();
        pa.clear();
        c1.clear();
        c2.clear();
        for (int k = 0; k < ninternal; k++) {
            if (k == root || depth[k] != d) continue;
            idx.push_back(k);
            pa.push_back(final_node[up[k]]);
            c1.push_back(state(left[k]));
            c2.push_back(state(right[k]));
        }
        const int n = (int)idx.size();
        nd.assign(n, -1);
        cs.assign(n, 0);
        const int rc = store_median3(s, cm, n, pa.data(), c1.data(), c2.data(), nd.data(),
                                     cs.data(), nullptr, nullptr);
        if (rc) return rc;
        for (int t = 0; t < n; t++) {
            final_node[idx[t]] = nd[t];
            final_cost[idx[t]] = cs[t];
        }
    }
    if (levels) *levels = maxd + 1;
    return 0;
}

}  // extern "C"
