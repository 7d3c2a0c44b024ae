// CUDA kernels of the GB300 direct-optimization aligner (sm_103a).
//
// A batch runs as a fixed sequence of launches, so it can be captured in a
// CUDA graph:
//   prep_kernel          one warp per pair: argument order, plane choice,
//                        initial band, affine row-0 state; pushes the pair to
//                        the work queue of its first pipeline class.
//   *_class_kernel<R>    one persistent launch per class (K warps x R rows per
//                        lane). A pipeline (K warps) pops (pair, T) items, runs
//                        band iterations while the band fits the class, pushes
//                        the pair to a larger class when it outgrows it, and
//                        traces back + builds the medians when the doubling
//                        test passes. Classes only grow, so each queue is
//                        complete before its kernel starts.
// Single-warp classes run four independent pipelines per CTA so that the
// shared-memory tables are shared.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>

#include "pa_kernels.h"

namespace pa {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NARROW_WARPS = 4;  // pipelines per CTA for K = 1 classes
constexpr int MAX_PASSES = 40;   // band doublings before a pair is failed

__device__ __forceinline__ void load_tables(Tables& st, const Tables* g)
{
    const int n = (int)(sizeof(Tables) / sizeof(int));
    const int* src = reinterpret_cast<const int*>(g);
    int* dst = reinterpret_cast<int*>(&st);
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

template <int R>
__device__ __forceinline__ void store_u8(uint8_t* p, const int (&d)[R])
{
    if constexpr (R == 1) {
        p[0] = (uint8_t)d[0];
    } else if constexpr (R == 2) {
        *reinterpret_cast<uint16_t*>(p) = (uint16_t)(d[0] | (d[1] << 8));
    } else if constexpr (R == 4) {
        *reinterpret_cast<uint32_t*>(p) =
            (uint32_t)d[0] | ((uint32_t)d[1] << 8) | ((uint32_t)d[2] << 16) | ((uint32_t)d[3] << 24);
    } else {
        static_assert(R == 8, "rows per lane");
        uint32_t lo = (uint32_t)d[0] | ((uint32_t)d[1] << 8) | ((uint32_t)d[2] << 16) | ((uint32_t)d[3] << 24);
        uint32_t hi = (uint32_t)d[4] | ((uint32_t)d[5] << 8) | ((uint32_t)d[6] << 16) | ((uint32_t)d[7] << 24);
        *reinterpret_cast<uint2*>(p) = make_uint2(lo, hi);
    }
}

template <int R>
__device__ __forceinline__ void store_u16(uint16_t* p, const int (&d)[R])
{
    if constexpr (R == 1) {
        p[0] = (uint16_t)d[0];
    } else if constexpr (R == 2) {
        *reinterpret_cast<uint32_t*>(p) = (uint32_t)d[0] | ((uint32_t)d[1] << 16);
    } else {
        static_assert(R == 4, "rows per lane");
        *reinterpret_cast<uint2*>(p) = make_uint2((uint32_t)d[0] | ((uint32_t)d[1] << 16),
                                                  (uint32_t)d[2] | ((uint32_t)d[3] << 16));
    }
}

// Pipeline geometry of the calling thread.
struct Pipe {
    int K, P;       // warps and lanes per pipeline
    int g;          // lane index within the pipeline
    int lane, warp; // warp lane and warp index within the pipeline
    int slot;       // pipeline index within the grid (selects the slab)
};

__device__ __forceinline__ Pipe make_pipe(int K)
{
    Pipe p;
    p.K = K;
    p.P = 32 * K;
    p.lane = threadIdx.x & 31;
    if (K == 1) {
        p.g = p.lane;
        p.warp = 0;
        p.slot = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    } else {
        p.g = threadIdx.x;
        p.warp = threadIdx.x >> 5;
        p.slot = blockIdx.x;
    }
    return p;
}

__device__ __forceinline__ void pipe_sync(const Pipe& p)
{
    if (p.K == 1) __syncwarp();
    else __syncthreads();
}

// Pop the next work item of class `cls` for this pipeline (-1 when empty).
// Queue q = 2 * class + variant (variant 1: affine gap-free fast path).
__device__ __forceinline__ int pop_item(const BatchArgs& A, int q, const Pipe& p, int* sh)
{
    int it = 0;
    if (p.K == 1) {
        if (p.lane == 0) it = atomicAdd(&A.qhead[q], 1);
        it = __shfl_sync(FULL, it, 0);
    } else {
        __syncthreads();
        if (threadIdx.x == 0) *sh = atomicAdd(&A.qhead[q], 1);
        __syncthreads();
        it = *sh;
    }
    return it < A.qcount[q] ? it : -1;
}

__device__ __forceinline__ void push_item(const BatchArgs& A, int q, int pair, int T)
{
    int slot = atomicAdd(&A.qcount[q], 1);
    A.qitems[q * A.qcap + slot] = make_int2(pair, T);
}

__device__ __forceinline__ PairOut pair_out(const BatchArgs& A, int k)
{
    const long long o = A.out_off[k];
    PairOut po;
    po.ea = A.ea + o;
    po.eb = A.eb + o;
    po.med = A.med + o;
    po.mwg = A.mwg + o;
    po.cap = A.lena[k] + A.lenb[k] + 2;
    return po;
}

__device__ __forceinline__ void finish_pair(const BatchArgs& A, int k, int cost, const PairRes& r)
{
    A.cost[k] = cost;
    A.alen[k] = r.alen;
    A.mlen[k] = r.mlen;
    A.wlen[k] = r.wlen;
    A.maxcost[k] = r.maxcost;
    A.status[k] = r.status;
}

// ---------------------------------------------------------------------------
// linear

template <int R>
__device__ void lin_fill(const LinBand& b, const Tables& st, const uint8_t* x,
                         const uint8_t* y, uint8_t* dm, const Pipe& p,
                         int (*xv)[32], uint32_t (*xn)[32], int* res)
{
    LinLane<R> L;
    lin_lane_init(L, b, st, x, p.g, p.P);
    const int Tlast = (b.m - 1) + (b.n - 1);
    const int src = (p.lane + 31) & 31;
    for (int T = 1; T <= Tlast; T++) {
        const int sv = L.V[R - 1];
        const uint32_t sn = L.N[R - 1];
        int rv = __shfl_sync(FULL, sv, src);
        uint32_t rn = __shfl_sync(FULL, sn, src);
        if (p.K > 1) {
            if (p.lane == 31) {
                xv[T & 1][p.warp] = sv;
                xn[T & 1][p.warp] = sn;
            }
            __syncthreads();
            if (p.lane == 0) {
                const int w = (p.warp + p.K - 1) % p.K;
                rv = xv[T & 1][w];
                rn = xn[T & 1][w];
            }
        }
        int dc[R];
        lin_step<R>(L, b, st, x, y, p.P, T, rv, rn, dc);
        store_u8<R>(dm + (long long)T * (p.P * R) + p.g * R, dc);
    }
    // the lane that owns the corner row reports cost and gap count
    const int i = b.m - 1;
    const int blk = (i - 1) / R, g = blk % p.P, q = (i - 1) - blk * R;
    if (p.g == g) {
        int v = 0;
        uint32_t nn = 0;
#pragma unroll
        for (int r = 0; r < R; r++)
            if (r == q) { v = L.V[r]; nn = L.N[r]; }
        res[0] = v;
        res[1] = tmax((int)(nn & 0xFFFF), (int)(nn >> 16));
    }
    pipe_sync(p);
}

template <int R>
__global__ void __launch_bounds__(512) lin_class_kernel(BatchArgs A, int cls)
{
    constexpr int VARIANT = 0;
    __shared__ Tables st;
    __shared__ int xv[2][32];
    __shared__ uint32_t xn[2][32];
    __shared__ int sres[NARROW_WARPS][2];
    __shared__ int sitem;
    load_tables(st, A.tables);
    __syncthreads();
    const int K = class_K(0, cls);
    const Pipe p = make_pipe(K);
    int* res = sres[K == 1 ? (threadIdx.x >> 5) : 0];
    uint8_t* dm = A.slab + (long long)p.slot * A.slab_stride;
    for (;;) {
        const int it = pop_item(A, 2 * cls, p, &sitem);
        if (it < 0) break;
        const int2 w = A.qitems[2 * cls * A.qcap + it];
        const int k = w.x;
        int T = w.y;
        const int la = A.lena[k], lb = A.lenb[k];
        const int swaped = la <= lb ? 0 : 1;
        const uint8_t* x = A.seqs + (swaped ? A.offb[k] : A.offa[k]);
        const uint8_t* y = A.seqs + (swaped ? A.offa[k] : A.offb[k]);
        const int m = swaped ? lb : la, n = swaped ? la : lb;
        const int full = A.pfull[k];
        int cost = 0;
        int npass = A.passes[k];  // passes run by smaller classes (earlier launches)
        bool done = false, moved = false;
        while (!done) {
            const LinBand b = lin_band(m, n, full, full ? 0 : band_p(T, m, n));
            const int c = pick_class(0, lin_wu(b), n);
            if (c > cls || c < 0 || npass >= MAX_PASSES) {
                if (p.g == 0) {
                    if (c > cls && npass < MAX_PASSES) push_item(A, 2 * c + VARIANT, k, T);
                    else A.status[k] = c < 0 ? -5 : -8;
                }
                moved = true;
                break;
            }
            int gapnum;
            if (m == 1) {
                int s = 0;
                for (int j = 1; j < n; j++) s += st.prepend[y[j]];
                cost = s;
                gapnum = n - 1;
            } else {
                lin_fill<R>(b, st, x, y, dm, p, xv, xn, res);
                cost = res[0];
                gapnum = res[1];
                pipe_sync(p);
            }
            npass++;
            if (p.g == 0) A.passes[k] = npass;
            done = full || lin_done(T, m, n, gapnum);
            if (!done) T *= 2;
        }
        if (moved) continue;
        if (p.g == 0) {
            A.lastcls[k] = cls;
            A.slab_cta[k] = p.slot;
            if (A.do_traceback) {
                __threadfence_block();
                const PairRes r = lin_traceback(dm, p.P, R, st, x, m, y, n, swaped, pair_out(A, k));
                finish_pair(A, k, cost, r);
            } else {
                A.cost[k] = cost;
                A.status[k] = 0;
            }
        }
        pipe_sync(p);
    }
}

// ---------------------------------------------------------------------------
// affine

template <int R>
__device__ void aff_fill(const AffBand& b, const Tables& st, const uint8_t* x,
                         const uint8_t* y, uint16_t* dm, int* shadow, int shadowEH0,
                         const Pipe& p, AffCell (*xc)[32], int* res)
{
    AffLane<R> L;
    aff_lane_init(L, b, st, x, p.g, p.P);
    const int Tlast = (b.m - 1) + (b.n - 1);
    const int src = (p.lane + 31) & 31;
    for (int T = 1; T <= Tlast; T++) {
        const AffCell sv = L.V[R - 1];
        AffCell rc;
        rc.EH = __shfl_sync(FULL, sv.EH, src);
        rc.EV = __shfl_sync(FULL, sv.EV, src);
        rc.EB = __shfl_sync(FULL, sv.EB, src);
        rc.CB = __shfl_sync(FULL, sv.CB, src);
        rc.GM = __shfl_sync(FULL, sv.GM, src);
        if (p.K > 1) {
            if (p.lane == 31) xc[T & 1][p.warp] = sv;
            __syncthreads();
            if (p.lane == 0) rc = xc[T & 1][(p.warp + p.K - 1) % p.K];
        }
        int dc[R];
        aff_step<R>(L, b, st, x, y, p.P, T, rc, shadow, shadowEH0, shadow, dc);
        store_u16<R>(dm + (long long)T * (p.P * R) + p.g * R, dc);
        // order this step's shadow writes after the generator's read of the
        // same column one step earlier
        if (p.K == 1) __syncwarp();
    }
    const int i = b.m - 1;
    const int blk = (i - 1) / R, g = blk % p.P, q = (i - 1) - blk * R;
    if (p.g == g) {
        AffCell c = L.V[0];
#pragma unroll
        for (int r = 0; r < R; r++)
            if (r == q) c = L.V[r];
        res[0] = aff_final(c);
        res[1] = aff_gapnum(c);
    }
    pipe_sync(p);
}

template <int R>
__device__ void aff_fill_fast(const AffBand& b, const Tables& st, const uint8_t* x,
                         const uint8_t* y, uint16_t* dm, int* shadow, int shadowEH0,
                         const Pipe& p, AffCell (*xc)[32], int* res)
{
    AffFastLane<R> L;
    aff_fast_lane_init(L, b, st, x, p.g, p.P);
    const int Tlast = (b.m - 1) + (b.n - 1);
    const int src = (p.lane + 31) & 31;
    for (int T = 1; T <= Tlast; T++) {
        const AffCell sv = L.V[R - 1];
        AffCell rc;
        rc.EH = __shfl_sync(FULL, sv.EH, src);
        rc.EV = __shfl_sync(FULL, sv.EV, src);
        rc.EB = __shfl_sync(FULL, sv.EB, src);
        rc.CB = __shfl_sync(FULL, sv.CB, src);
        rc.GM = __shfl_sync(FULL, sv.GM, src);
        if (p.K > 1) {
            if (p.lane == 31) xc[T & 1][p.warp] = sv;
            __syncthreads();
            if (p.lane == 0) rc = xc[T & 1][(p.warp + p.K - 1) % p.K];
        }
        int dc[R];
        aff_fast_step<R>(L, b, st, x, y, p.P, T, rc, shadow, shadowEH0, dc);
        store_u16<R>(dm + (long long)T * (p.P * R) + p.g * R, dc);
        // order this step's shadow writes after the generator's read of the
        // same column one step earlier
        if (p.K == 1) __syncwarp();
    }
    const int i = b.m - 1;
    const int blk = (i - 1) / R, g = blk % p.P, q = (i - 1) - blk * R;
    if (p.g == g) {
        AffCell c = L.V[0];
#pragma unroll
        for (int r = 0; r < R; r++)
            if (r == q) c = L.V[r];
        res[0] = aff_final(c);
        res[1] = aff_gapnum(c);
    }
    pipe_sync(p);
}

template <int R, bool FAST>
__global__ void __launch_bounds__(512) aff_class_kernel(BatchArgs A, int cls)
{
    constexpr int VARIANT = FAST ? 1 : 0;
    __shared__ Tables st;
    __shared__ AffCell xc[2][32];
    __shared__ int sres[NARROW_WARPS][2];
    __shared__ int sitem;
    load_tables(st, A.tables);
    __syncthreads();
    const int K = class_K(1, cls);
    const Pipe p = make_pipe(K);
    int* res = sres[K == 1 ? (threadIdx.x >> 5) : 0];
    uint16_t* dm = reinterpret_cast<uint16_t*>(A.slab + (long long)p.slot * A.slab_stride);
    for (;;) {
        const int it = pop_item(A, 2 * cls + VARIANT, p, &sitem);
        if (it < 0) break;
        const int2 w = A.qitems[(2 * cls + VARIANT) * A.qcap + it];
        const int k = w.x;
        int T = w.y;
        const int la = A.lena[k], lb = A.lenb[k];
        const int swaped = la <= lb ? 0 : 1;
        const uint8_t* x = A.seqs + (swaped ? A.offb[k] : A.offa[k]);
        const uint8_t* y = A.seqs + (swaped ? A.offa[k] : A.offb[k]);
        const int m = swaped ? lb : la, n = swaped ? la : lb;
        int* shadow = A.shadow + A.out_off[k];
        int cost = 0;
        int npass = A.passes[k];  // passes run by smaller classes (earlier launches)
        bool done = false, moved = false;
        while (!done) {
            const AffBand b = aff_band(m, n, band_p(T, m, n));
            const int c = pick_class(1, aff_wu(b), n);
            if (c > cls || c < 0 || npass >= MAX_PASSES) {
                if (p.g == 0) {
                    if (c > cls && npass < MAX_PASSES) push_item(A, 2 * c + VARIANT, k, T);
                    else A.status[k] = c < 0 ? -5 : -8;
                }
                moved = true;
                break;
            }
            int gapnum;
            if (m == 1) {
                int s = st.go;
                for (int j = 1; j < n; j++) s += st.prepend[y[j]];
                cost = s;
                gapnum = 0xFFFF;
            } else {
                const int eh0 = A.shadowEH0[k];
                if constexpr (FAST) aff_fill_fast<R>(b, st, x, y, dm, shadow, eh0, p, xc, res);
                else aff_fill<R>(b, st, x, y, dm, shadow, eh0, p, xc, res);
                cost = res[0];
                gapnum = res[1];
                if (p.g == 0 && tmin(m - 1, b.newk) >= 2) A.shadowEH0[k] = HIGH;
                pipe_sync(p);
            }
            npass++;
            if (p.g == 0) A.passes[k] = npass;
            done = aff_done(T, m, n, gapnum);
            if (!done) T *= 2;
            pipe_sync(p);
        }
        if (moved) continue;
        if (p.g == 0) {
            A.lastcls[k] = cls;
            A.slab_cta[k] = p.slot;
            if (A.do_traceback) {
                __threadfence_block();
                const PairRes r = aff_traceback(dm, p.P, R, st, x, m, y, n, swaped, pair_out(A, k));
                finish_pair(A, k, cost, r);
            } else {
                A.cost[k] = cost;
                A.status[k] = 0;
            }
        }
        pipe_sync(p);
    }
}

// ---------------------------------------------------------------------------
// prep: one warp per pair

__global__ void prep_kernel(BatchArgs A)
{
    const int wk = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wk >= A.npairs) return;
    const int k = A.order ? A.order[wk] : wk;
    const Tables& t = *A.tables;
    const int la = A.lena[k], lb = A.lenb[k];
    const uint8_t* a = A.seqs + A.offa[k];
    const uint8_t* b = A.seqs + A.offb[k];
    // every state must index the 1 << lcm tables
    int bad = 0;
    const int ns = 1 << t.lcm;
    for (int i = lane; i < la; i += 32) bad |= (a[i] >= ns);
    for (int i = lane; i < lb; i += 32) bad |= (b[i] >= ns);
    bad = __any_sync(FULL, bad);
    // gap bit anywhere past the leading position -> generic affine cells
    int gapped = 0;
    for (int i = 1 + lane; i < la; i += 32) gapped |= (a[i] & TMPGAP);
    for (int i = 1 + lane; i < lb; i += 32) gapped |= (b[i] & TMPGAP);
    gapped = __any_sync(FULL, gapped);
    PairPlan pl;
    if (A.affine) {
        pl = plan_affine(t, la, lb);
        int* shadow = A.shadow + A.out_off[k];
        for (int j = lane; j < pl.n; j += 32) shadow[j] = HIGH;
        if (lane == 0) {
            A.shadowEH0[k] = t.go;
            A.pfull[k] = (!gapped && t.gap == TMPGAP) ? 2 : 0;
        }
    } else {
        int ga = 0, gb = 0;
        for (int i = lane; i < la; i += 32) ga += (a[i] >= t.gap && (a[i] & t.gap)) ? 1 : 0;
        for (int i = lane; i < lb; i += 32) gb += (b[i] >= t.gap && (b[i] & t.gap)) ? 1 : 0;
        for (int o = 16; o > 0; o >>= 1) {
            ga += __shfl_xor_sync(FULL, ga, o);
            gb += __shfl_xor_sync(FULL, gb, o);
        }
        if (A.deltawh_override) pl = plan_linear_deltawh(t, la, lb, A.deltawh_override[k]);
        else pl = plan_linear(t, ga, la, gb, lb);
        if (lane == 0) A.pfull[k] = pl.full;
    }
    if (lane != 0) return;
    A.passes[k] = 0;
    A.status[k] = 1;
    A.lastcls[k] = -1;
    if (la < 1 || lb < 1 || (A.affine && la == 1 && lb == 1)) {
        A.status[k] = -4;
        return;
    }
    if (bad) {
        A.status[k] = -7;
        return;
    }
    if (pl.n > 65535) {  // gap counts travel as packed 16-bit halves
        A.status[k] = -6;
        return;
    }
    int c;
    if (A.affine) c = pick_class(1, aff_wu(aff_band(pl.m, pl.n, band_p(pl.T0, pl.m, pl.n))), pl.n);
    else c = pick_class(0, lin_wu(lin_band(pl.m, pl.n, pl.full, pl.full ? 0 : band_p(pl.T0, pl.m, pl.n))), pl.n);
    if (c < 0) {
        A.status[k] = -5;
        return;
    }
    push_item(A, 2 * c + ((A.affine && (A.pfull[k] & 2)) ? 1 : 0), k, pl.T0);
}

// Traceback of fills kept in their slabs (per-call stub path); one thread
// per pair, slab chosen by the class and CTA recorded at the fill.
__global__ void traceback_kernel(BatchArgs A, const long long* strides)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.npairs || A.status[k] != 0) return;
    const Tables& t = *A.tables;
    const int la = A.lena[k], lb = A.lenb[k];
    const int swaped = la <= lb ? 0 : 1;
    const uint8_t* x = A.seqs + (swaped ? A.offb[k] : A.offa[k]);
    const uint8_t* y = A.seqs + (swaped ? A.offa[k] : A.offb[k]);
    const int m = swaped ? lb : la, n = swaped ? la : lb;
    const int tie = A.swap_override ? A.swap_override[k] : swaped;
    const int cls = A.lastcls[k];
    const int P = 32 * class_K(A.affine, cls), R = class_R(A.affine, cls);
    const uint8_t* base = A.slab + (long long)A.slab_cta[k] * strides[cls];
    PairRes r;
    if (A.affine) r = aff_traceback(reinterpret_cast<const uint16_t*>(base), P, R, t, x, m, y, n, tie, pair_out(A, k));
    else r = lin_traceback(base, P, R, t, x, m, y, n, tie, pair_out(A, k));
    finish_pair(A, k, A.cost[k], r);
}

// algn_ancestor_2 / seq_get_median_2d_with_gaps / algn_worst_2 on an aligned
// pair (single thread; the per-call stubs of those externals).
__global__ void aligned_medians_kernel(const Tables* tg, const uint8_t* x, const uint8_t* y,
                                       int len, uint8_t* anc, uint8_t* mwg, int* out3)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const Tables& t = *tg;
    const int gap = t.gap;
    const int drop = !t.comb || t.model != 1;
    int ka = len + 1, status = 0;
    for (int i = len - 1; i >= 0; i--) {
        const int med = t.median[(x[i] << t.lcm) + y[i]];
        mwg[i] = (uint8_t)med;
        if (med == 0) status = -3;
        if (!drop || med != gap) anc[--ka] = (uint8_t)med;
    }
    int n = len + 1 - ka;
    for (int i = 0; i < n; i++) anc[i] = anc[ka + i];
    if (!t.comb || (t.model != 1 && (n == 0 || anc[0] != gap))) {
        for (int i = n; i > 0; i--) anc[i] = anc[i - 1];
        anc[0] = (uint8_t)gap;
        n++;
    } else if (t.comb) {
        // algn_correct_blocks_affine + algn_remove_gaps (src/algn.c:3530-3600)
        int inside = 0, prev = 0, ext = 0;
        for (int i = 0; i < n; i++) {
            const int ab = x[i], bb = y[i];
            int sb = anc[i];
            if (!inside && (!(ab & gap) || !(bb & gap))) inside = 0;
            else if (inside && ((!(ab & gap)) || (!(bb & gap)))) inside = 0;
            else if (((ab & gap) || (bb & gap)) && ((ab != gap) || (bb != gap))) inside = 1;
            else inside = 0;
            if (((gap & ab) || (gap & bb)) && (!(sb & gap)) && !ext) {
                prev = inside;
                ext = 1;
            } else if ((gap & ab) && (gap & bb) && (sb & gap) && (sb != gap) && ext && inside && !prev) {
                sb = (~gap) & sb;
                prev = 0;
            } else if ((gap & ab) && (gap & bb) && (1 == ext)) {
                prev = inside;
                ext = 0;
            }
            anc[i] = (uint8_t)sb;
        }
        int w = 0;
        for (int i = 0; i < n; i++)
            if (anc[i] != gap) anc[w++] = anc[i];
        for (int i = w; i > 0; i--) anc[i] = anc[i - 1];
        anc[0] = (uint8_t)gap;
        n = w + 1;
    }
    int nga = 0, ngb = 0;
    for (int i = 0; i < len; i++) {
        nga |= x[i] != gap;
        ngb |= y[i] != gap;
    }
    out3[0] = n;
    out3[1] = (nga && ngb) ? worst_aligned(t, x, y, len) : 0;
    out3[2] = status;
}

}  // namespace

int class_blocks_per_sm(int affine, int cls, int variant)
{
    const int K = class_K(affine, cls), R = class_R(affine, cls);
    const int threads = K == 1 ? 32 * NARROW_WARPS : 32 * K;
    int n = 0;
    if (affine) {
        switch (R) {
            case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, variant ? aff_class_kernel<1, true> : aff_class_kernel<1, false>, threads, 0); break;
            case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, variant ? aff_class_kernel<2, true> : aff_class_kernel<2, false>, threads, 0); break;
            default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, variant ? aff_class_kernel<4, true> : aff_class_kernel<4, false>, threads, 0); break;
        }
    } else {
        switch (R) {
            case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lin_class_kernel<1>, threads, 0); break;
            case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lin_class_kernel<2>, threads, 0); break;
            case 4: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lin_class_kernel<4>, threads, 0); break;
            default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lin_class_kernel<8>, threads, 0); break;
        }
    }
    return n;
}

long long class_slab_bytes(int affine, int cls, int maxmn)
{
    const long long PR = 32LL * class_K(affine, cls) * class_R(affine, cls);
    long long b = (long long)(maxmn + 1) * PR * (affine ? 2 : 1);
    return (b + 255) & ~255LL;
}

__global__ void order_keys_kernel(const int* lena, const int* lenb, int n, unsigned* key,
                                  int* idx);

static size_t sort_temp_bytes(int n)
{
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, (const unsigned*)nullptr, (unsigned*)nullptr,
                                    (const int*)nullptr, (int*)nullptr, n);
    return tb;
}

size_t order_scratch_bytes(int npairs)
{
    const size_t a = ((size_t)npairs * 4 + 255) & ~(size_t)255;
    return 3 * a + sort_temp_bytes(npairs) + 256;
}

int launch_order(const int* lena, const int* lenb, int npairs, int* order, void* scratch,
                 cudaStream_t s)
{
    if (npairs <= 0) return 0;
    const size_t a = ((size_t)npairs * 4 + 255) & ~(size_t)255;
    char* p = static_cast<char*>(scratch);
    unsigned* key_in = reinterpret_cast<unsigned*>(p);
    unsigned* key_out = reinterpret_cast<unsigned*>(p + a);
    int* idx_in = reinterpret_cast<int*>(p + 2 * a);
    void* temp = p + 3 * a;
    size_t tb = sort_temp_bytes(npairs);
    order_keys_kernel<<<(npairs + 255) / 256, 256, 0, s>>>(lena, lenb, npairs, key_in, idx_in);
    return (int)cub::DeviceRadixSort::SortPairs(temp, tb, key_in, key_out, idx_in, order,
                                                npairs, 0, 32, s);
}

void launch_prep(const BatchArgs& a, cudaStream_t s)
{
    if (a.npairs <= 0) return;
    const int threads = 256;
    const long long warps = a.npairs;
    const int blocks = (int)((warps * 32 + threads - 1) / threads);
    prep_kernel<<<blocks, threads, 0, s>>>(a);
}

void launch_class(const BatchArgs& a, int cls, int variant, int grid, cudaStream_t s)
{
    const int K = class_K(a.affine, cls), R = class_R(a.affine, cls);
    const int threads = K == 1 ? 32 * NARROW_WARPS : 32 * K;
    if (a.affine) {
        switch (R) {
            case 1:
                if (variant) aff_class_kernel<1, true><<<grid, threads, 0, s>>>(a, cls);
                else aff_class_kernel<1, false><<<grid, threads, 0, s>>>(a, cls);
                break;
            case 2:
                if (variant) aff_class_kernel<2, true><<<grid, threads, 0, s>>>(a, cls);
                else aff_class_kernel<2, false><<<grid, threads, 0, s>>>(a, cls);
                break;
            default:
                if (variant) aff_class_kernel<4, true><<<grid, threads, 0, s>>>(a, cls);
                else aff_class_kernel<4, false><<<grid, threads, 0, s>>>(a, cls);
                break;
        }
    } else {
        switch (R) {
            case 1: lin_class_kernel<1><<<grid, threads, 0, s>>>(a, cls); break;
            case 2: lin_class_kernel<2><<<grid, threads, 0, s>>>(a, cls); break;
            case 4: lin_class_kernel<4><<<grid, threads, 0, s>>>(a, cls); break;
            default: lin_class_kernel<8><<<grid, threads, 0, s>>>(a, cls); break;
        }
    }
}

void launch_traceback(const BatchArgs& a, const long long* d_strides, cudaStream_t s)
{
    if (a.npairs <= 0) return;
    const int threads = 128;
    traceback_kernel<<<(a.npairs + threads - 1) / threads, threads, 0, s>>>(a, d_strides);
}

__global__ void order_keys_kernel(const int* lena, const int* lenb, int n, unsigned* key,
                                  int* idx)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned long long w = (unsigned long long)lena[k] * (unsigned long long)lenb[k];
    key[k] = ~(unsigned)(w > 0xffffffffull ? 0xffffffffull : w);  // descending work
    idx[k] = k;
}

int class_pipes_per_cta(int affine, int cls) { return class_K(affine, cls) == 1 ? NARROW_WARPS : 1; }

void launch_aligned_medians(const Tables* t, const uint8_t* x, const uint8_t* y,
                            int len, uint8_t* anc, uint8_t* mwg, int* out3,
                            cudaStream_t s)
{
    aligned_medians_kernel<<<1, 32, 0, s>>>(t, x, y, len, anc, mwg, out3);
}

}  // namespace pa
