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

#include <algorithm>

#include <cub/device/device_radix_sort.cuh>
#include <type_traits>

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
    } else if constexpr (R == 3) {  // 3 bytes at an odd offset for odd lanes
        p[0] = (uint8_t)d[0];
        p[1] = (uint8_t)d[1];
        p[2] = (uint8_t)d[2];
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
    } else if constexpr (R == 3) {
        p[0] = (uint16_t)d[0];
        p[1] = (uint16_t)d[1];
        p[2] = (uint16_t)d[2];
    } else {
        static_assert(R == 4, "rows per lane");
        *reinterpret_cast<uint2*>(p) = make_uint2((uint32_t)d[0] | ((uint32_t)d[1] << 16),
                                                  (uint32_t)d[2] | ((uint32_t)d[3] << 16));
    }
}

// Pipeline geometry of the calling thread. P < 32: 32/P pipelines share a
// warp, each aligning its own pair (shuffles of width P); P >= 32: one
// pipeline per warp (K = 1) or per CTA of K = P/32 warps.
struct Pipe {
    int P, K, G;     // lanes per pipeline, warps per pipeline, pipelines per warp
    int gl;          // lane index within the pipeline
    int grp;         // pipeline index within the warp (P < 32)
    int lane, warp;  // warp lane; warp index within a multi-warp pipeline
    int slot;        // pipeline index in the grid (selects the slab)
};

__device__ __forceinline__ Pipe make_pipe(int P)
{
    Pipe p;
    p.P = P;
    p.K = P >= 32 ? P / 32 : 1;
    p.G = P < 32 ? 32 / P : 1;
    p.lane = threadIdx.x & 31;
    if (p.K == 1) {
        p.gl = p.lane & (P - 1);
        p.grp = p.lane / P;
        p.warp = 0;
        p.slot = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * p.G + p.grp;
    } else {
        p.gl = threadIdx.x;
        p.grp = 0;
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

// True if any pipeline of the warp (or the CTA's one pipeline) is live.
__device__ __forceinline__ bool any_live(const Pipe& p, bool live)
{
    return p.K == 1 ? __any_sync(FULL, live) : live;
}

// Warp-wide max (pipelines of a warp run their steps in lockstep).
__device__ __forceinline__ int group_max(const Pipe& p, int v)
{
    return p.K == 1 ? __reduce_max_sync(FULL, v) : v;
}

// Rotate a value from lane g-1 of the pipeline (lane P-1 for lane 0).
template <class V>
__device__ __forceinline__ V rot_prev(const Pipe& p, V v)
{
    if (p.P < 32) return __shfl_sync(FULL, v, (p.gl + p.P - 1) & (p.P - 1), p.P);
    return __shfl_sync(FULL, v, (p.lane + 31) & 31);
}

// Value held by pipeline lane `src` (K = 1 pipelines only).
template <class V>
__device__ __forceinline__ V from_lane(const Pipe& p, V v, int src)
{
    return __shfl_sync(FULL, v, src, p.P < 32 ? p.P : 32);
}

// Queue q = 2 * class + variant (variant 1: affine gap-free fast path).
// A warp of small pipelines takes G consecutive items at once; returns the
// first index, or -1 when the queue is drained.
__device__ __forceinline__ int pop_items(const BatchArgs& A, int q, const Pipe& p, int* sh)
{
    int it = 0;
    if (p.K == 1) {
        if (p.lane == 0) it = atomicAdd(&A.qhead[q], p.G);
        it = __shfl_sync(FULL, it, 0);
    } else {
        __syncthreads();
        if (threadIdx.x == 0) *sh = atomicAdd(&A.qhead[q], 1);
        __syncthreads();
        it = *sh;
    }
    return it < A.qcount[q] ? it : -1;
}

// Pipelines that want an item take the next ones of queue q, one each (one
// atomic per warp, or per CTA for a multi-warp pipeline); `want` is uniform
// within a pipeline. Returns the item index, or -1 when the queue is drained
// (its count is fixed while the class kernel runs: items only move up).
__device__ __forceinline__ int take_item(const BatchArgs& A, int q, const Pipe& p, bool want,
                                         int* sh)
{
    int it = -1;
    if (p.K == 1) {
        const unsigned lead = __ballot_sync(FULL, want && p.gl == 0);
        int base = 0;
        if (p.lane == 0 && lead) base = atomicAdd(&A.qhead[q], __popc(lead));
        base = __shfl_sync(FULL, base, 0);
        const int leader = p.lane - p.gl;
        it = base + __popc(lead & ((1u << leader) - 1u));
    } else {
        __syncthreads();
        if (threadIdx.x == 0) *sh = want ? atomicAdd(&A.qhead[q], 1) : 0;
        __syncthreads();
        it = *sh;
    }
    return (want && it < A.qcount[q]) ? it : -1;
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

// Arena region of `bytes` for one pair's fills in one class; -1 when the
// arena is off or full (the fill then uses the pipeline's own slab and the
// traceback runs in the class kernel).
__device__ __forceinline__ long long arena_take(const BatchArgs& A, long long bytes)
{
    if (A.dm_cap <= 0 || bytes > (A.spec == 2 ? A.dm_max_region2 : A.dm_max_region)) return -1;
    const unsigned long long b = ((unsigned long long)bytes + 255ull) & ~255ull;
    const unsigned long long off = atomicAdd(A.dm_used, b);
    return off + b <= (unsigned long long)A.dm_cap ? (long long)off : -1;
}

// An arena region for the pipeline's item: its leader takes it, every lane of
// the pipeline gets it. Pipeline-uniform call (a CTA barrier when K > 1).
__device__ __forceinline__ long long pipe_take(const BatchArgs& A, const Pipe& p, bool want,
                                               long long bytes, long long* sh)
{
    long long off = -1;
    if (p.gl == 0 && want) off = arena_take(A, bytes);
    if (p.K == 1) {
        off = __shfl_sync(FULL, off, p.lane - p.gl);
    } else {
        __syncthreads();
        if (p.gl == 0) *sh = off;
        __syncthreads();
        off = *sh;
    }
    return off;
}

// Work item of one pipeline: the pair in internal order and its band state.
struct Item {
    int k, T, m, n, swaped, full, npass;
    int tie;  // traceback tie preference: swaped, or the per-call caller's
    const uint8_t* x;
    const uint8_t* y;
};

__device__ __forceinline__ Item load_item(const BatchArgs& A, int q, int it)
{
    Item w;
    const int2 e = (A.qsorted ? A.qsorted : A.qitems)[(long long)q * A.qcap + it];
    w.k = e.x;
    w.T = e.y;
    const int la = A.lena[w.k], lb = A.lenb[w.k];
    w.swaped = la <= lb ? 0 : 1;
    w.x = A.seqs + (w.swaped ? A.offb[w.k] : A.offa[w.k]);
    w.y = A.seqs + (w.swaped ? A.offa[w.k] : A.offb[w.k]);
    w.m = w.swaped ? lb : la;
    w.n = w.swaped ? la : lb;
    w.tie = A.swap_override ? A.swap_override[w.k] : w.swaped;
    w.full = A.pfull[w.k] & 1;
    w.npass = A.passes[w.k];  // passes run by smaller classes (earlier launches)
    return w;
}

__device__ __forceinline__ Item empty_item(const BatchArgs& A)
{
    Item w;
    w.k = 0;
    w.T = 1;
    w.m = 1;
    w.n = 1;
    w.swaped = 0;
    w.tie = 0;
    w.full = 0;
    w.npass = 0;
    w.x = A.seqs;
    w.y = A.seqs;
    return w;
}

// Pass index of a speculative item (T = T0 << j).
__device__ __forceinline__ int spec_pass(const BatchArgs& A, const Item& w)
{
    return __ffs(w.T / A.spec_T0[w.k]) - 1;
}

// Row-0 EH at column 0 for lean affine pass j: HIGH once an earlier pass had
// min(m - 1, newk) >= 2 (newk grows with T, so pass j - 1 decides), else the
// value prep left.
__device__ __forceinline__ int spec_eh0(const BatchArgs& A, const Item& w, int j)
{
    if (j == 0 || w.m - 1 < 2) return A.shadowEH0[w.k];
    const AffBand pb = aff_band(w.m, w.n, band_p(A.spec_T0[w.k] << (j - 1), w.m, w.n));
    return tmin(w.m - 1, pb.newk) >= 2 ? HIGH : A.shadowEH0[w.k];
}

__device__ __forceinline__ void spec_record(const BatchArgs& A, const Item& w, int j, int cost,
                                            int gapnum, int cls_flags, long long off)
{
    const long long si = (long long)w.k * SPEC_STRIDE + j;
    A.spec_res[si] = make_int4(cost, gapnum, cls_flags, 1);
    A.spec_off[si] = off;
}

// A pass of the second sweep that traced back at once: its outputs and
// results are written, the status waits for spec_resolve2_kernel.
__device__ __forceinline__ void spec_traced(const BatchArgs& A, const Item& w, int j, int cost,
                                            const PairRes& r)
{
    A.cost[w.k] = cost;
    A.alen[w.k] = r.alen;
    A.mlen[w.k] = r.mlen;
    A.wlen[w.k] = r.wlen;
    A.maxcost[w.k] = r.maxcost;
    const long long si = (long long)w.k * SPEC_STRIDE + j;
    A.spec_res[si].z |= SPEC_TRACED | ((-r.status & 0xFF) << 16);
}

// Items at least a third as long (m + n) as the longest item queued in this
// class run one pass per class launch (on the 65,536-pair batch: a third
// 83.0 ms, a half 83.7, two thirds 86.7, never 90.4): after a failed pass
// whose next band still fits here (or a narrower class), such an item moves
// on to the next class, as long as that one has single-warp pipelines. A pass runs the
// same band on any class it fits, so only the launch that runs it changes:
// no pipeline runs several passes of a long pair back to back while the
// rest of the GPU waits at the end of the launch. 0x7fffffff: never (no
// length-sorted queue, row tile, or no such next class).
__device__ __forceinline__ int promote_len(const BatchArgs& A, int q, int cls)
{
    if (!A.qsorted || A.row_tile || cls + 1 >= NCLASS || A.lad.P[cls + 1] > 32 ||
        A.qcount[q] == 0)
        return 0x7fffffff;
    const int k = A.qsorted[(long long)q * A.qcap].x;  // longest first
    return (A.lena[k] + A.lenb[k] + 2) / 3;
}

// ---------------------------------------------------------------------------
// linear

// One band iteration of every active pipeline of the warp/CTA, in lockstep
// over Tmax anti-diagonal steps; returns the corner cost and gap count of
// the calling lane's pipeline.
template <int R>
__device__ void lin_fill(const LinBand& b, const Tables& st, const uint8_t* x,
                         const uint8_t* y, uint8_t* dm, const Pipe& p, bool active,
                         int Tmax, int (*xv)[32], uint32_t (*xn)[32], int* sres,
                         int& cost, int& gapnum)
{
    LinLane<R> L;
    L.V0[R - 1] = L.V1[R - 1] = 0;
    L.N0[R - 1] = L.N1[R - 1] = 0;
    if (active) lin_lane_init(L, b, st, x, p.gl, p.P);
    const int Tlast = active ? (b.m - 1) + (b.n - 1) : 0;
    auto exchange = [&](int sv, uint32_t sn, int T, int& rv, uint32_t& rn) {
        rv = rot_prev(p, sv);
        rn = rot_prev(p, sn);
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
    };
    // two steps per iteration: set 0 -> 1 at odd T, set 1 -> 0 at even T
    auto steps = [&](auto gen, int T0, int T1) {
        constexpr bool GEN = decltype(gen)::value;
        for (int T = T0; T <= T1; T += 2) {
            {
                int rv;
                uint32_t rn;
                exchange(L.V0[R - 1], L.N0[R - 1], T, rv, rn);
                if (active && T <= Tlast) {
                    int dc[R];
                    lin_step<R, GEN>(L, L.V0, L.V1, L.N0, L.N1, L.R0, L.R1, L.RN0, L.RN1,
                                     L.G0, L.G1, b, st, x, y, p.P, T, rv, rn, dc);
                    store_u8<R>(dm + (long long)T * (p.P * R) + p.gl * R, dc);
                }
            }
            if (T + 1 <= Tmax) {
                int rv;
                uint32_t rn;
                exchange(L.V1[R - 1], L.N1[R - 1], T + 1, rv, rn);
                if (active && T + 1 <= Tlast) {
                    int dc[R];
                    lin_step<R, GEN>(L, L.V1, L.V0, L.N1, L.N0, L.R1, L.R0, L.RN1, L.RN0,
                                     L.G1, L.G0, b, st, x, y, p.P, T + 1, rv, rn, dc);
                    store_u8<R>(dm + (long long)(T + 1) * (p.P * R) + p.gl * R, dc);
                }
            }
        }
    };
    // lane 0 generates row 0 only while in its first block (both bounds even)
    const int tg = group_max(p, active ? lin_gen_steps(b, p.P, R) : 0);
    const int Tg = tmin((Tmax + 1) & ~1, tg);
    steps(std::true_type{}, 1, Tg - 1);
    steps(std::false_type{}, (Tg & ~1) + 1, Tmax);
    // the lane owning the corner row reports cost and gap count
    const int i = active ? b.m - 1 : 1;
    const int blk = (i - 1) / R, og = blk % p.P, oq = (i - 1) - blk * R;
    const bool odd = (Tlast & 1) != 0;  // odd last step wrote set 1
    int v = 0;
    uint32_t nn = 0;
#pragma unroll
    for (int r = 0; r < R; r++)
        if (r == oq) {
            v = odd ? L.V1[r] : L.V0[r];
            nn = odd ? L.N1[r] : L.N0[r];
        }
    if (p.K == 1) {
        v = from_lane(p, v, og);
        nn = from_lane(p, nn, og);
    } else {
        if (p.gl == og) {
            sres[0] = v;
            sres[1] = (int)nn;
        }
        __syncthreads();
        v = sres[0];
        nn = (uint32_t)sres[1];
        __syncthreads();
    }
    cost = v;
    gapnum = tmax((int)(nn & 0xFFFF), (int)(nn >> 16));
}

// Resident CTAs per SM the compiler must allow for the 128-thread (P <= 32)
// launches of each shape; the wide launches (up to 512 threads) keep 1.
constexpr int lin_narrow_minb(int R) { return R == 2 ? 6 : R == 4 ? 5 : 4; }
constexpr int aff_narrow_minb(int) { return 4; }  // higher counts spill more than they gain

template <int R, bool NARROW>
__global__ void __launch_bounds__(NARROW ? 128 : 512, NARROW ? lin_narrow_minb(R) : 1)
    lin_class_kernel(BatchArgs A, int cls)
{
    constexpr int VARIANT = 0;
    __shared__ Tables st;
    __shared__ int xv[2][32];
    __shared__ uint32_t xn[2][32];
    __shared__ int sres[2];
    __shared__ int sitem;
    __shared__ long long soff;
    load_tables(st, A.tables);
    __syncthreads();
    const Pipe p = make_pipe(A.lad.P[cls]);
    const int q = 2 * cls + VARIANT;
    uint8_t* const slot_dm = A.slab + (long long)p.slot * A.slab_stride;
    const bool spec = A.spec != 0;  // every linear item of a speculative sweep
    Item w = empty_item(A);
    bool live = false, drained = false;
    int cost = 0, sj = 0;
    long long off = -2;  // arena region of the item: not taken yet
    uint8_t* dm = slot_dm;
    const int plen = promote_len(A, q, cls);
    // the item's band for its next pass: stays here, moves up the ladder, or
    // fails (after a pass, a long item moves up whenever it fits)
    auto keep = [&](bool after) {
        const LinBand b = lin_band(w.m, w.n, w.full, w.full ? 0 : band_p(w.T, w.m, w.n));
        int c = pick_class(A.lad, lin_wu(b), w.n);
        if (after && c >= 0 && c <= cls && w.m + w.n >= plen) c = cls + 1;
        if (c > cls || c < 0 || w.npass >= MAX_PASSES) {
            if (p.gl == 0) {
                if (c > cls && w.npass < MAX_PASSES) push_item(A, 2 * c + VARIANT, w.k, w.T);
                else A.status[w.k] = c < 0 ? -5 : -8;
            }
            live = false;
        }
    };
    for (;;) {
        for (;;) {  // refill between passes (pipeline-uniform decisions)
            const bool want = !live && !drained;
            if (!any_live(p, want)) break;
            const int it = take_item(A, q, p, want, &sitem);
            if (want) {
                if (it < 0) {
                    drained = true;
                } else {
                    w = load_item(A, q, it);
                    live = true;
                    off = -2;
                    if (spec) sj = spec_pass(A, w);
                    keep(false);
                }
            }
        }
        if (!any_live(p, live)) break;
        const LinBand b = lin_band(w.m, w.n, w.full, w.full ? 0 : band_p(w.T, w.m, w.n));
        {  // first pass of an item in this class: its arena region (a warp-
           // or CTA-wide call: pipelines of one warp admit items at different times)
            const bool fresh = off == -2;
            // in the second sweep only the predicted final pass keeps its
            // fill (in a region of its own: the classes run concurrently and
            // share the slabs); the other passes are read for their gap counts
            const bool keepfill = A.spec != 2 || (live && w.T == A.spec_Tstar[w.k]);
            const long long o = pipe_take(A, p, fresh && live && A.do_traceback && keepfill,
                                          (long long)(w.m + w.n + 1) * p.P * R, &soff);
            if (fresh) {
                off = o;
                dm = off >= 0 ? A.dm_arena + off : slot_dm;
            }
        }
        const bool act = live && w.m > 1;
        const int Tmax = group_max(p, act ? (w.m - 1) + (w.n - 1) : 0);
        int fc = 0, fg = 0;
        if (Tmax > 0) lin_fill<R>(b, st, w.x, w.y, dm, p, act, Tmax, xv, xn, sres, fc, fg);
        bool finished = false;
        bool strace = false;  // second sweep: trace back the predicted final pass now
        if (live) {
            int gapnum = fg;
            cost = fc;
            if (w.m == 1) {  // no rows: row 0 is the whole alignment
                int s = 0;
                for (int j = 1; j < w.n; j++) s += st.prepend[w.y[j]];
                cost = s;
                gapnum = w.n - 1;
            }
            if (spec) {  // one pass; spec_resolve_kernel decides
                if (p.gl == 0) spec_record(A, w, sj, cost, gapnum, cls, off);
                // second sweep: the predicted final pass traces back at once
                // when its own test ends the doubling (kept by the resolve if
                // no earlier pass of the sweep stopped)
                strace = A.spec == 2 && A.do_traceback && off >= 0 &&
                         w.T == A.spec_Tstar[w.k] && (w.full || lin_done(w.T, w.m, w.n, gapnum));
                live = false;
            } else {
                w.npass++;
                if (p.gl == 0) A.passes[w.k] = w.npass;
                if (w.full || lin_done(w.T, w.m, w.n, gapnum)) {
                    live = false;
                    finished = true;
                } else {
                    w.T *= 2;
                    keep(true);
                }
            }
        }
        pipe_sync(p);
        if (finished && p.gl == 0) {
            A.lastcls[w.k] = cls;
            A.slab_cta[w.k] = p.slot;
        }
        if (finished && (!A.do_traceback || off >= 0)) {  // no traceback, or after all fills
            if (p.gl == 0) {
                if (off >= 0) A.dm_off[w.k] = off;
                A.cost[w.k] = cost;
                A.status[w.k] = 0;
            }
        } else if (finished || strace) {
            PairRes r;
            bool lead = false;
            if (lin_window_ok(p.P, R)) {
                // the pipeline's first warp walks the path through a shared
                // window of the slab (one round of loads per LW_DIAG steps)
                if (p.gl < 32) {
                    extern __shared__ uint32_t lin_win[];
                    LinDmWindow<> rd{dm, lin_win + (p.K == 1 ? (threadIdx.x >> 5) : 0) * LW_SMEM_WORDS,
                                   p.P * R, p.P * R / 4, p.lane, 32};
                    r = lin_traceback_dm(rd, st, w.x, w.m, w.y, w.n, w.tie, pair_out(A, w.k));
                    lead = p.gl == 0;
                }
            } else if (p.gl == 0) {
                r = lin_traceback(dm, p.P, R, st, w.x, w.m, w.y, w.n, w.tie, pair_out(A, w.k));
                lead = true;
            }
            if (lead && finished) finish_pair(A, w.k, cost, r);
            if (lead && strace) spec_traced(A, w, sj, cost, r);
        }
        pipe_sync(p);
    }
}

// Dynamic shared memory of a class launch: the traceback windows of linear
// pipelines of 32 lanes or more (one per pipeline of the CTA).
int class_dyn_smem(const Ladder& lad, int affine, int cls)
{
    if (affine || !lin_window_ok(lad.P[cls], lad.R[cls])) return 0;
    const int pipes = ladder_K(lad, cls) == 1 ? NARROW_WARPS : 1;
    return pipes * LW_SMEM_WORDS * (int)sizeof(uint32_t);
}

// ---------------------------------------------------------------------------
// affine

template <int R, bool FAST>
__device__ void aff_fill(const AffBand& b, const Tables& st, const uint8_t* x,
                         const uint8_t* y, uint16_t* dm, int* shadow, int shadowEH0,
                         const Pipe& p, bool active, int Tmax, AffCell (*xc)[32],
                         int* sres, int& cost, int& gapnum)
{
    using Lane = typename std::conditional<FAST, AffFastLane<R>, AffLane<R>>::type;
    Lane L;
    L.V[R - 1] = AffCell{0, 0, 0, 0, 0u};
    if (active) {
        if constexpr (FAST) aff_fast_lane_init(L, b, st, x, p.gl, p.P);
        else aff_lane_init(L, b, st, x, p.gl, p.P);
    }
    const int Tlast = active ? (b.m - 1) + (b.n - 1) : 0;
    for (int T = 1; T <= Tmax; T++) {
        const AffCell sv = L.V[R - 1];
        AffCell rc;
        rc.EH = rot_prev(p, sv.EH);
        rc.EV = rot_prev(p, sv.EV);
        rc.EB = rot_prev(p, sv.EB);
        rc.CB = rot_prev(p, sv.CB);
        rc.GM = rot_prev(p, sv.GM);
        if (p.K > 1) {
            if (p.lane == 31) xc[T & 1][p.warp] = sv;
            __syncthreads();
            if (p.lane == 0) rc = xc[T & 1][(p.warp + p.K - 1) % p.K];
        }
        if (active && T <= Tlast) {
            int dc[R];
            if constexpr (FAST) aff_fast_step<R>(L, b, st, x, y, p.P, T, rc, shadow, shadowEH0, dc);
            else aff_step<R>(L, b, st, x, y, p.P, T, rc, shadow, shadowEH0, shadow, dc);
            store_u16<R>(dm + (long long)T * (p.P * R) + p.gl * R, dc);
        }
        // order this step's shadow writes after the row-0 reads of one step
        // earlier (multi-warp pipelines are ordered by the exchange barrier)
        if (p.K == 1) __syncwarp();
    }
    const int i = active ? b.m - 1 : 1;
    const int blk = (i - 1) / R, og = blk % p.P, oq = (i - 1) - blk * R;
    AffCell c = L.V[0];
#pragma unroll
    for (int r = 0; r < R; r++)
        if (r == oq) c = L.V[r];
    int f = aff_final(c), g = aff_gapnum(c);
    if (p.K == 1) {
        f = from_lane(p, f, og);
        g = from_lane(p, g, og);
    } else {
        if (p.gl == og) {
            sres[0] = f;
            sres[1] = g;
        }
        __syncthreads();
        f = sres[0];
        g = sres[1];
        __syncthreads();
    }
    cost = f;
    gapnum = g;
}


// Lean affine fill (gap-free pairs within aff_lean_ok): one direction byte
// per cell, no block-diagonal state; the step loop is unrolled by two so the
// two register sets of AffLean swap roles statically.
template <int R>
__device__ void aff_fill_lean(const AffBand& b, const Tables& st, const uint8_t* x,
                              const uint8_t* y, uint8_t* dm, int shadowEH0, const Pipe& p,
                              bool active, int Tmax, LeanCell (*xc)[32], int* sres, int& cost,
                              int& gapnum)
{
    AffLean<R> L;
    L.V0[R - 1] = LeanCell{0, 0, 0, 0u};
    L.V1[R - 1] = LeanCell{0, 0, 0, 0u};
    if (active) aff_lean_init(L, b, st, x, p.gl, p.P);
    const int Tlast = active ? (b.m - 1) + (b.n - 1) : 0;
    // Pipelines that share a warp run their own pairs, and a lane's change
    // of block (aff_lean_enter) is a divergent branch for the whole warp.
    // Past its first rows a pipeline's lanes change blocks at steps 2 i - newk
    // (i = first row of the block), i.e. at steps = 2 - newk (mod 2 R); each
    // pipeline's item is delayed by `delta` steps so that these fall on
    // multiples of 2 R for every pipeline of the warp, and the warp takes
    // the branch once per 2 R steps instead of once per pipeline.
    const int delta = (active && p.P < 32) ? (((b.newk - 2) % (2 * R)) + 2 * R) % (2 * R) : 0;
    Tmax = group_max(p, active ? Tlast + delta : 0);
    auto exchange = [&](const LeanCell& sv, int T) {
        LeanCell rc;
        rc.EH = rot_prev(p, sv.EH);
        rc.EV = rot_prev(p, sv.EV);
        rc.CB = rot_prev(p, sv.CB);
        rc.GM = rot_prev(p, sv.GM);
        if (p.K > 1) {
            if (p.lane == 31) xc[T & 1][p.warp] = sv;
            __syncthreads();
            if (p.lane == 0) rc = xc[T & 1][(p.warp + p.K - 1) % p.K];
        }
        return rc;
    };
    // two step pairs per iteration: V0 -> V1 at odd T, V1 -> V0 at even T
    auto steps = [&](auto gen, int T0, int T1) {
        constexpr bool GEN = decltype(gen)::value;
        for (int T = T0; T <= T1; T += 2) {
            {
                const LeanCell rc = exchange(L.V0[R - 1], T);
                const int Ti = T - delta;  // the pipeline's own step
                if (active && Ti >= 1 && Ti <= Tlast) {
                    int dc[R];
                    aff_lean_step<R, GEN>(L, L.V0, L.V1, L.R0, L.R1, L.G0, L.G1, b, st, x, y,
                                          p.P, Ti, rc, shadowEH0, dc);
                    store_u8<R>(dm + (long long)Ti * (p.P * R) + p.gl * R, dc);
                }
            }
            if (T + 1 <= Tmax) {
                const LeanCell rc = exchange(L.V1[R - 1], T + 1);
                const int Ti = T + 1 - delta;
                if (active && Ti >= 1 && Ti <= Tlast) {
                    int dc[R];
                    aff_lean_step<R, GEN>(L, L.V1, L.V0, L.R1, L.R0, L.G1, L.G0, b, st, x, y,
                                          p.P, Ti, rc, shadowEH0, dc);
                    store_u8<R>(dm + (long long)Ti * (p.P * R) + p.gl * R, dc);
                }
            }
        }
    };
    // lane 0 generates row 0 only while in its first block (both bounds even;
    // the register sets alternate with every step, so a pipeline may start on
    // either of them: both hold the initial state)
    const int tg = group_max(p, active ? ((lean_gen_steps(b, p.P, R) + delta + 1) & ~1) : 0);
    const int Tg = tmin((Tmax + 1) & ~1, tg);
    steps(std::true_type{}, 1, Tg - 1);
    steps(std::false_type{}, (Tg & ~1) + 1, Tmax);
    const int i = active ? b.m - 1 : 1;
    const int blk = (i - 1) / R, og = blk % p.P, oq = (i - 1) - blk * R;
    LeanCell c = L.V0[0];
    const bool odd = ((Tlast + delta) & 1) != 0;  // an odd last warp step wrote V1
#pragma unroll
    for (int r = 0; r < R; r++)
        if (r == oq) c = odd ? L.V1[r] : L.V0[r];
    int f = lean_final(c), g = lean_gapnum(c);
    if (p.K == 1) {
        f = from_lane(p, f, og);
        g = from_lane(p, g, og);
    } else {
        if (p.gl == og) {
            sres[0] = f;
            sres[1] = g;
        }
        __syncthreads();
        f = sres[0];
        g = sres[1];
        __syncthreads();
    }
    cost = f;
    gapnum = g;
}

template <int R, bool FAST, bool NARROW>
__global__ void __launch_bounds__(NARROW ? 128 : 512, NARROW ? aff_narrow_minb(R) : 1)
    aff_class_kernel(BatchArgs A, int cls)
{
    constexpr int VARIANT = FAST ? 1 : 0;
    __shared__ Tables st;
    __shared__ AffCell xc[2][32];
    __shared__ LeanCell xl[2][32];
    __shared__ int sres[2];
    __shared__ int sitem;
    __shared__ long long soff;
    load_tables(st, A.tables);
    __syncthreads();
    const Pipe p = make_pipe(A.lad.P[cls]);
    const int q = 2 * cls + VARIANT;
    uint16_t* const slot_dm = reinterpret_cast<uint16_t*>(A.slab + (long long)p.slot * A.slab_stride);
    const bool spec = FAST && A.spec;  // lean items of a speculative sweep
    Item w = empty_item(A);
    bool live = false, drained = false;
    int cost = 0, sj = 0;
    long long off = -2;  // arena region of the item: not taken yet
    uint16_t* dm = slot_dm;
    // A pipeline that has no item (or whose item left this class) takes the
    // next one between passes, so the pipelines sharing a warp stay busy
    // whatever the number of passes each of their pairs runs in this class.
    auto admit = [&](int it) {
        w = load_item(A, q, it);
        live = true;
        off = -2;
        if (spec) sj = spec_pass(A, w);
    };
    const int plen = promote_len(A, q, cls);
    // the item's band for its next pass: stays here, moves up the ladder, or
    // fails (after a pass, a long item moves up whenever it fits)
    auto keep = [&](bool after) {
        const AffBand b = aff_band(w.m, w.n, band_p(w.T, w.m, w.n));
        int c = (FAST && A.row_tile) ? pick_class_lean(A.lad, aff_wu(b), w.n)
                                     : pick_class(A.lad, aff_wu(b), w.n);
        if (after && c >= 0 && c <= cls && w.m + w.n >= plen) c = cls + 1;
        if (c > cls || c < 0 || w.npass >= MAX_PASSES) {
            if (p.gl == 0) {
                if (c > cls && w.npass < MAX_PASSES) push_item(A, 2 * c + VARIANT, w.k, w.T);
                else A.status[w.k] = c < 0 ? -5 : -8;
            }
            live = false;
        }
    };
    for (;;) {
        for (;;) {  // refill (pipeline-uniform decisions)
            const bool want = !live && !drained;
            if (!any_live(p, want)) break;
            const int it = take_item(A, q, p, want, &sitem);
            if (want) {
                if (it < 0) {
                    drained = true;
                } else {
                    admit(it);
                    keep(false);
                }
            }
        }
        if (!any_live(p, live)) break;
        const AffBand b = aff_band(w.m, w.n, band_p(w.T, w.m, w.n));
        {  // first pass of an item in this class: its arena region (a warp-
           // or CTA-wide call: pipelines of one warp admit items at different times)
            const bool fresh = off == -2;
            const long long o =
                pipe_take(A, p, fresh && live && A.do_traceback,
                          (long long)(w.m + w.n + 1) * p.P * R * (FAST ? 1 : 2), &soff);
            if (fresh) {
                off = o;
                dm = off >= 0 ? reinterpret_cast<uint16_t*>(A.dm_arena + off) : slot_dm;
            }
        }
        int* shadow = A.shadow + (live ? A.out_off[w.k] : 0);
        const bool act = live && w.m > 1;
        const int Tmax = group_max(p, act ? (w.m - 1) + (w.n - 1) : 0);
        const int eh0 = !live ? 0 : spec ? spec_eh0(A, w, sj) : A.shadowEH0[w.k];
        int fc = 0, fg = 0;
        if (Tmax > 0) {
            if constexpr (FAST)
                aff_fill_lean<R>(b, st, w.x, w.y, reinterpret_cast<uint8_t*>(dm), eh0, p, act,
                                 Tmax, xl, sres, fc, fg);
            else
                aff_fill<R, false>(b, st, w.x, w.y, dm, shadow, eh0, p, act, Tmax, xc, sres, fc,
                                   fg);
        }
        bool finished = false;
        if (live) {
            int gapnum = fg;
            cost = fc;
            if (w.m == 1) {  // leni = 0: the initial row is the whole alignment
                int s = st.go;
                for (int j = 1; j < w.n; j++) s += st.prepend[w.y[j]];
                cost = s;
                gapnum = 0xFFFF;
            } else if (!spec && p.gl == 0 && tmin(w.m - 1, b.newk) >= 2) {
                A.shadowEH0[w.k] = HIGH;
            }
            if (spec) {  // one pass; spec_resolve_kernel decides
                if (p.gl == 0) spec_record(A, w, sj, cost, gapnum, cls | LASTCLS_LEAN, off);
                live = false;
            } else {
                w.npass++;
                if (p.gl == 0) A.passes[w.k] = w.npass;
                if (aff_done(w.T, w.m, w.n, gapnum)) {
                    live = false;
                    finished = true;
                } else {
                    w.T *= 2;
                    keep(true);
                }
            }
        }
        pipe_sync(p);
        if (finished) {
            if (p.gl == 0) {
                A.lastcls[w.k] = cls | (FAST ? LASTCLS_LEAN : 0);
                A.slab_cta[w.k] = p.slot;
            }
            if (!A.do_traceback || off >= 0) {  // no traceback, or after all fills
                if (p.gl == 0) {
                    if (off >= 0) A.dm_off[w.k] = off;
                    A.cost[w.k] = cost;
                    A.status[w.k] = 0;
                }
            } else if (p.gl == 0) {
                const PairRes r =
                    FAST ? aff_traceback_lean(reinterpret_cast<const uint8_t*>(dm), p.P, R, st,
                                              w.x, w.m, w.y, w.n, w.tie, pair_out(A, w.k))
                         : aff_traceback(dm, p.P, R, st, w.x, w.m, w.y, w.n, w.tie,
                                         pair_out(A, w.k));
                finish_pair(A, w.k, cost, r);
            }
        }
        pipe_sync(p);
    }
}

// ---------------------------------------------------------------------------
// Row tile for lean affine bands up to 32 K wide: one pair per warp, the
// band swept row by row (rk_* cell phases in pa_core.cuh). Direction bytes
// are stored row-major, 32 K per row.

template <int K>
__device__ __forceinline__ void store_codes(uint8_t* p, const int (&c)[K])
{
    if constexpr (K == 16) {
        uint32_t w[4];
#pragma unroll
        for (int h = 0; h < 4; h++)
            w[h] = (uint32_t)c[4 * h] | ((uint32_t)c[4 * h + 1] << 8) |
                   ((uint32_t)c[4 * h + 2] << 16) | ((uint32_t)c[4 * h + 3] << 24);
        *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
        store_u8<K>(p, c);
    }
}

template <int K>
__device__ void aff_rk_fill(const AffBand& b, const Tables& st, const uint8_t* x,
                            const uint8_t* y, uint8_t* dm, int shadowEH0, int lane, int& cost,
                            int& gapnum)
{
    constexpr int S = 32 * K;
    const int newk = b.newk, n = b.n, go = st.go;
    LeanCell P[K];
    int J[K], JG[K];
    {  // row 0: prefix sums of the prepend terms
        const int j0 = lane * K - newk;
        int pre[K], run = 0;
#pragma unroll
        for (int q = 0; q < K; q++) {
            const int j = j0 + q;
            run += (j >= 1 && j < n) ? rk_row0_term(st, y, j) : 0;
            pre[q] = run;
        }
        int incl = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += v;
        }
        const int base = incl - run;
#pragma unroll
        for (int q = 0; q < K; q++) P[q] = rk_row0(j0 + q, base + pre[q], shadowEH0);
    }
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = 1 + lane * K + q - newk;
        J[q] = (j >= 0 && j < n) ? y[j] : 0;
        JG[q] = st.prepend[J[q]];
    }
    for (int i = 1; i <= b.m - 1; i++) {
        if (i > 1) {  // row i's column at d is row i-1's at d + 1
            const int nj = __shfl_down_sync(FULL, J[0], 1);
            const int ng = __shfl_down_sync(FULL, JG[0], 1);
#pragma unroll
            for (int q = 0; q + 1 < K; q++) {
                J[q] = J[q + 1];
                JG[q] = JG[q + 1];
            }
            J[K - 1] = nj;
            JG[K - 1] = ng;
            if (lane == 31) {
                const int j = i + S - 1 - newk;
                J[K - 1] = (j >= 0 && j < n) ? y[j] : 0;
                JG[K - 1] = st.prepend[J[K - 1]];
            }
        }
        const RkRow r = rk_row(b, st, x, i);
        const int j0 = i + lane * K - newk;
        LeanCell upn;
        upn.EH = __shfl_down_sync(FULL, P[0].EH, 1);
        upn.EV = __shfl_down_sync(FULL, P[0].EV, 1);
        upn.CB = __shfl_down_sync(FULL, P[0].CB, 1);
        upn.GM = __shfl_down_sync(FULL, P[0].GM, 1);
        int EV[K], CB[K], EH[K], code[K], hv[K];
        uint32_t fl[K];
        rk_phase_a<K>(P, upn, J, r, st, j0, EV, CB, code);
        int cbl = __shfl_up_sync(FULL, CB[K - 1], 1);
        if (lane == 0) cbl = HIGH;
        // EH: exclusive scan of the lanes' min-plus maps
        MinPlus f = rk_eh_map<K>(JG, CB, r, go, j0, cbl);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int ps = __shfl_up_sync(FULL, f.s, o);
            const int pt = __shfl_up_sync(FULL, f.t, o);
            if (lane >= o) f = mp_then(MinPlus{ps, pt}, f);
        }
        const MinPlus ex{__shfl_up_sync(FULL, f.s, 1), __shfl_up_sync(FULL, f.t, 1)};
        const int xin = lane == 0 ? HIGH : mp_apply(ex, HIGH);
        GmMap g = rk_phase_b<K>(P, upn, JG, r, st, j0, xin, cbl, EV, CB, EH, code, hv, fl);
        // GM: a lane's composition is a constant unless every cell of it extends
        // horizontally; scan only when some lane's is not
        uint32_t yin;
        if (__any_sync(FULL, g.act)) {
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int pa = __shfl_up_sync(FULL, g.act, o);
                const uint32_t pd = __shfl_up_sync(FULL, g.add, o);
                const uint32_t pf = __shfl_up_sync(FULL, g.floor, o);
                if (lane >= o) g = gm_then(GmMap{pa, pd, pf}, g);
            }
            const GmMap ge{__shfl_up_sync(FULL, g.act, 1), __shfl_up_sync(FULL, g.add, 1),
                           __shfl_up_sync(FULL, g.floor, 1)};
            yin = lane == 0 ? 0u : gm_apply(ge, 0u);
        } else {
            yin = __shfl_up_sync(FULL, g.floor, 1);
            if (lane == 0) yin = 0u;
        }
        rk_phase_c<K>(P, r, j0, yin, EH, EV, CB, hv, fl, code);
        store_codes<K>(dm + (long long)i * S + lane * K, code);
    }
    const int dc = n - 1 - (b.m - 1) + newk;
    const int cl = dc / K, cq = dc % K;
    int f = 0, g = 0;
#pragma unroll
    for (int q = 0; q < K; q++)
        if (q == cq) {
            f = lean_final(P[q]);
            g = lean_gapnum(P[q]);
        }
    cost = __shfl_sync(FULL, f, cl);
    gapnum = __shfl_sync(FULL, g, cl);
}

// Class kernel of the row tile (lean queue of class cls, one pair per warp).
template <int K>
__global__ void __launch_bounds__(32 * NARROW_WARPS) aff_rk_kernel(BatchArgs A, int cls)
{
    __shared__ Tables st;
    __shared__ int sitem;
    load_tables(st, A.tables);
    __syncthreads();
    const Pipe p = make_pipe(32);
    const int q = 2 * cls + 1;
    uint8_t* const slot_dm = A.slab + (long long)p.slot * A.slab_stride;
    for (;;) {
        const int base = pop_items(A, q, p, &sitem);
        if (base < 0) break;
        const int it = base + p.grp;
        bool live = it < A.qcount[q];
        Item w = live ? load_item(A, q, it) : empty_item(A);
        bool finished = false;
        int cost = 0, newk = 0;
        long long off = -2;  // arena region: not taken yet
        uint8_t* dm = slot_dm;
        while (live) {  // uniform across the warp: one pair
            const AffBand b = aff_band(w.m, w.n, band_p(w.T, w.m, w.n));
            const int c = pick_class_lean(A.lad, aff_wu(b), w.n);
            if (c != cls || w.npass >= MAX_PASSES) {
                if (p.lane == 0) {
                    if (c > cls && w.npass < MAX_PASSES) push_item(A, 2 * c + 1, w.k, w.T);
                    else A.status[w.k] = c < 0 ? -5 : -8;
                }
                live = false;
                break;
            }
            if (off == -2) {  // first pass in this class: the arena region
                if (p.lane == 0) off = A.do_traceback ? arena_take(A, (long long)w.m * 32 * K) : -1;
                off = __shfl_sync(FULL, off, 0);
                dm = off >= 0 ? A.dm_arena + off : slot_dm;
            }
            int gapnum;
            if (w.m == 1) {  // leni = 0: the initial row is the whole alignment
                int s = st.go;
                for (int j = 1; j < w.n; j++) s += st.prepend[w.y[j]];
                cost = s;
                gapnum = 0xFFFF;
            } else {
                aff_rk_fill<K>(b, st, w.x, w.y, dm, A.shadowEH0[w.k], p.lane, cost, gapnum);
                if (p.lane == 0 && tmin(w.m - 1, b.newk) >= 2) A.shadowEH0[w.k] = HIGH;
            }
            newk = b.newk;
            w.npass++;
            if (p.lane == 0) A.passes[w.k] = w.npass;
            __syncwarp();
            if (aff_done(w.T, w.m, w.n, gapnum)) {
                finished = true;
                break;
            }
            w.T *= 2;
        }
        if (finished) {
            if (p.lane == 0) {
                A.lastcls[w.k] = cls | LASTCLS_LEAN | LASTCLS_ROW;
                A.slab_cta[w.k] = p.slot;
                if (!A.do_traceback || off >= 0) {  // no traceback, or after all fills
                    if (off >= 0) A.dm_off[w.k] = off;
                    A.cost[w.k] = cost;
                    A.status[w.k] = 0;
                } else {
                    const PairRes r = aff_traceback_rowtile(dm, 32 * K, newk, st, w.x, w.m, w.y,
                                                            w.n, w.tie, pair_out(A, w.k));
                    finish_pair(A, w.k, cost, r);
                }
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Queue sort: a counting sort of a class's two queues by the pairs' length
// m + n, longest first, so that the pipelines sharing a warp run pairs of
// similar length and the persistent grid ends on short pairs.

__device__ __forceinline__ int len_bucket(int x)
{
    x = x < 1 ? 1 : x;
    const int e = 31 - __clz(x);
    const int mant = e >= 3 ? (x >> (e - 3)) & 7 : (x << (3 - e)) & 7;
    return NBUCKET - 1 - (e * 8 + mant);
}

__global__ void __launch_bounds__(256) queue_hist_kernel(BatchArgs A, int cls)
{
    __shared__ int h[2 * NBUCKET];
    for (int i = threadIdx.x; i < 2 * NBUCKET; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int v = 0; v < 2; v++) {
        const int q = 2 * cls + v, n = A.qcount[q];
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            const int k = A.qitems[(long long)q * A.qcap + i].x;
            atomicAdd(&h[v * NBUCKET + len_bucket(A.lena[k] + A.lenb[k])], 1);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * NBUCKET; i += blockDim.x)
        if (h[i]) atomicAdd(&A.qhist[2 * cls * NBUCKET + i], h[i]);
}

__global__ void __launch_bounds__(256) queue_scatter_kernel(BatchArgs A, int cls)
{
    static_assert(NBUCKET == 256, "one bucket per thread");
    __shared__ int base[2 * NBUCKET];
    const int t = threadIdx.x;
    for (int v = 0; v < 2; v++) {  // exclusive prefix of each histogram (every block)
        const int h = A.qhist[(2 * cls + v) * NBUCKET + t];
        int* b = base + v * NBUCKET;
        b[t] = h;
        __syncthreads();
        for (int o = 1; o < NBUCKET; o <<= 1) {
            const int add = t >= o ? b[t - o] : 0;
            __syncthreads();
            b[t] += add;
            __syncthreads();
        }
        b[t] -= h;
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    const int wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (int v = 0; v < 2; v++) {
        const int q = 2 * cls + v, n = A.qcount[q];
        for (int w0 = wid * 32; w0 < n; w0 += warps * 32) {  // warp-uniform trips
            const int i = w0 + lane;
            const bool ok = i < n;
            const int2 e = ok ? A.qitems[(long long)q * A.qcap + i] : make_int2(0, 0);
            const int bk = ok ? len_bucket(A.lena[e.x] + A.lenb[e.x]) : -1;
            const unsigned peers = __match_any_sync(FULL, bk);
            const int leader = __ffs(peers) - 1;
            int at = 0;
            if (ok && lane == leader) at = atomicAdd(&A.qcur[q * NBUCKET + bk], __popc(peers));
            at = __shfl_sync(FULL, at, leader);
            if (ok) {
                const int pos = base[v * NBUCKET + bk] + at + __popc(peers & ((1u << lane) - 1u));
                A.qsorted[(long long)q * A.qcap + pos] = e;
            }
        }
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
    // a pair outside the caller's declared shape would overrun a direction
    // slab or its output slot: it fails before any read or write of its own
    const int oob = pair_bounds_status(la, lb, A.max_pair_len, A.out_off ? A.out_off[k] : 0,
                                       A.out_bytes, A.out_off != nullptr);
    if (oob) {
        if (lane == 0) {
            A.passes[k] = 0;
            A.lastcls[k] = -1;
            if (A.dm_off) A.dm_off[k] = -1;
            A.status[k] = oob;
        }
        return;
    }
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
            A.pfull[k] = (!gapped && t.gap == TMPGAP && aff_lean_ok(t, tmax(la, lb))) ? 2 : 0;
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
        else if (A.distance) pl = plan_linear_distance(t, ga, la, gb, lb);
        else pl = plan_linear(t, ga, la, gb, lb);
        if (lane == 0) A.pfull[k] = pl.full;
    }
    if (A.distance) {  // Sequence.is_empty: every position the gap
        int ea = 1, eb = 1;
        for (int i = lane; i < la; i += 32) ea &= a[i] == t.gap;
        for (int i = lane; i < lb; i += 32) eb &= b[i] == t.gap;
        const bool empty = __all_sync(FULL, ea) || __all_sync(FULL, eb);
        if (empty) {
            if (lane == 0) {
                A.passes[k] = 0;
                A.lastcls[k] = -1;
                A.cost[k] = A.missing_distance;
                A.status[k] = 0;
            }
            return;
        }
    }
    if (lane != 0) return;
    A.passes[k] = 0;
    A.status[k] = 1;
    A.lastcls[k] = -1;
    if (A.dm_off) A.dm_off[k] = -1;
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
    const bool lean = A.affine && (A.pfull[k] & 2);
    auto class_of = [&](int T) {
        if (A.affine) {
            const long long wu = aff_wu(aff_band(pl.m, pl.n, band_p(T, pl.m, pl.n)));
            return (lean && A.row_tile) ? pick_class_lean(A.lad, wu, pl.n)
                                        : pick_class(A.lad, wu, pl.n);
        }
        return pick_class(A.lad, lin_wu(lin_band(pl.m, pl.n, pl.full,
                                                 pl.full ? 0 : band_p(T, pl.m, pl.n))), pl.n);
    };
    // the doubling's first passes that cannot end it (unstoppable_passes)
    // are counted as run: linear pairs and lean affine ones, whose later
    // passes read nothing an earlier pass leaves but the row-0 value
    int s = 0;
    if ((lean || (!A.affine && !pl.full)) && pl.T0 > 0) {
        s = unstoppable_passes(pl.T0, pl.m, pl.n, A.affine != 0, MAX_PASSES - 1);
        A.passes[k] = s;
        if (s > 0 && lean && pl.m - 1 >= 2 &&
            tmin(pl.m - 1, aff_band(pl.m, pl.n, band_p(pl.T0 << (s - 1), pl.m, pl.n)).newk) >= 2)
            A.shadowEH0[k] = HIGH;
    }
    const int c = class_of(pl.T0 << s);
    if (c < 0) {
        A.status[k] = -5;
        return;
    }
    if (A.spec_S > 0 && (lean || !A.affine) && pl.T0 > 0) {
        // queue the next passes at once (the doubling's bands, up to the
        // one that covers the plane), each as its own item; pass s first
        const int S = (!A.affine && pl.full) ? 1 : A.spec_S;
        int T = pl.T0 << s, nq = 0;
        bool wide = false;
        for (;;) {
            if (s + nq >= SPEC_STRIDE) break;  // spec_res holds passes 0 .. SPEC_STRIDE - 1
            const int cj = class_of(T);
            if (cj < 0) {
                nq |= SPEC_NOCLASS;
                break;
            }
            // bands that need a multi-warp pipeline (a barrier per step) are
            // slow per step: at most the first of them is speculated, so that
            // the widest, slowest passes do not sit on every pair's
            // critical path; later ones go to the sequential sweep (or, with
            // a second sweep ahead, all of them go there: the gap count of
            // the single-warp passes predicts the final pass)
            if (A.lad.P[cj] > 32) {
                if ((wide || A.spec2) && nq > 0) break;
                wide = true;
            }
            push_item(A, 2 * cj + (lean ? 1 : 0), k, T);
            nq++;
            const bool last = A.affine ? aff_covers(T, pl.m, pl.n)
                                       : (pl.full || lin_covers(T, pl.m, pl.n));
            if (nq >= S || last) break;
            T *= 2;
        }
        A.spec_T0[k] = pl.T0;
        A.spec_n[k] = nq;
        return;
    }
    if (A.spec_S > 0) {  // speculative batch: sequential pairs wait for the second sweep
        A.spec_T0[k] = pl.T0;
        A.spec_n[k] = -1;
        return;
    }
    push_item(A, 2 * c + (lean ? 1 : 0), k, pl.T0 << s);
}

// The sequential doubling resumed at pass j (band T) on the second sweep.
__device__ void spec_requeue(const BatchArgs& A, int k, int m, int n, int j, int T, bool lean)
{
    A.passes[k] = j;
    int c;
    if (A.affine) {
        if (j > 0 && m - 1 >= 2 &&
            tmin(m - 1, aff_band(m, n, band_p(T / 2, m, n)).newk) >= 2)
            A.shadowEH0[k] = HIGH;
        c = pick_class(A.lad, aff_wu(aff_band(m, n, band_p(T, m, n))), n);
    } else {
        const int full = A.pfull[k] & 1;
        c = pick_class(A.lad, lin_wu(lin_band(m, n, full, full ? 0 : band_p(T, m, n))), n);
    }
    if (c < 0) {
        A.status[k] = -5;
        return;
    }
    push_item(A, 2 * c + (lean ? 1 : 0), k, T);
}

// The sequential sweep resumes a pair at pass j; with a second speculative
// sweep ahead, the first resolve only notes where (the queues then belong to
// that sweep).
__device__ void spec_resume(const BatchArgs& A, int k, int m, int n, int j, int T, bool lean)
{
    if (A.spec2) A.spec_p2[k] = make_int2(j, -1);
    else spec_requeue(A, k, m, n, j, T, lean);
}

// One thread per speculated pair: the first queued pass whose result
// satisfies the doubling test is the pair's final pass (the sequential
// doubling runs exactly the passes before it, in order, and stops there).
__global__ void spec_resolve_kernel(BatchArgs A)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.npairs || A.status[k] != 1) return;
    const int la = A.lena[k], lb = A.lenb[k];
    const int m = la <= lb ? la : lb, n = la <= lb ? lb : la;
    const bool lean = A.affine && (A.pfull[k] & 2);
    int T = A.spec_T0[k];
    if (A.spec_n[k] < 0) {  // not speculated (gap-bearing affine pair): sequential from pass 0
        spec_resume(A, k, m, n, 0, T, lean);
        return;
    }
    // passes j0 .. j0 + nq - 1 were queued (prep counted the j0 before them as run)
    const int j0 = A.passes[k];
    const int nq = A.spec_n[k] & ~SPEC_NOCLASS;
    const bool full = !A.affine && (A.pfull[k] & 1);
    T <<= j0;
    for (int j = j0; j < j0 + nq; j++, T *= 2) {
        const int4 r = A.spec_res[(long long)k * SPEC_STRIDE + j];
        if (r.w != 1) {  // a queued pass did not run
            A.status[k] = -9;
            return;
        }
        const bool done = A.affine ? aff_done(T, m, n, r.y) : (full || lin_done(T, m, n, r.y));
        if (!done) continue;
        const long long off = A.spec_off[(long long)k * SPEC_STRIDE + j];
        if (off >= 0 || !A.do_traceback) {
            A.cost[k] = r.x;
            A.passes[k] = j + 1;
            A.lastcls[k] = r.z;
            if (A.dm_off) A.dm_off[k] = off;
            A.status[k] = 0;
        } else {  // no arena region for its fill: the sequential sweep runs it again
            spec_resume(A, k, m, n, j, T, lean);
        }
        return;
    }
    if (A.spec_n[k] & SPEC_NOCLASS) {
        A.status[k] = -5;
        return;
    }
    if (A.spec2 && !A.affine && !full && nq > 0) {
        // the gap count of the last pass predicts the final one: the first
        // whose p exceeds it by more than one (or that covers the plane);
        // every pass up to it runs at once in the second sweep
        const int G = A.spec_res[(long long)k * SPEC_STRIDE + j0 + nq - 1].y;
        int last = -1;
        for (int j = j0 + nq; j < SPEC_STRIDE; j++, T *= 2) {
            const int c = pick_class(A.lad, lin_wu(lin_band(m, n, 0, band_p(T, m, n))), n);
            if (c < 0) break;
            push_item(A, 2 * c, k, T);
            last = j;
            if (band_p(T, m, n) > G + 1 || lin_covers(T, m, n)) break;
        }
        if (last >= 0) {
            A.spec_p2[k] = make_int2(j0 + nq, last);
            A.spec_Tstar[k] = A.spec_T0[k] << last;
            return;
        }
        T = A.spec_T0[k] << (j0 + nq);
    }
    spec_resume(A, k, m, n, j0 + nq, T, lean);
}

// One thread per pair still open after the first resolve, when the second
// speculative sweep ran (linear batches): the first of the sweep's passes
// whose result satisfies the doubling test ends the pair, exactly where the
// sequential doubling stops. The predicted final pass already traced back;
// any other stopping pass runs again in the sequential sweep with its
// traceback, and a pair none of whose passes stopped continues there.
__global__ void spec_resolve2_kernel(BatchArgs A)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.npairs || A.status[k] != 1) return;
    const int la = A.lena[k], lb = A.lenb[k];
    const int m = la <= lb ? la : lb, n = la <= lb ? lb : la;
    const int T0 = A.spec_T0[k];
    const int2 q = A.spec_p2[k];
    if (q.y < 0) {
        spec_requeue(A, k, m, n, q.x, T0 << q.x, false);
        return;
    }
    const bool full = A.pfull[k] & 1;
    for (int j = q.x; j <= q.y; j++) {
        const int T = T0 << j;
        const int4 r = A.spec_res[(long long)k * SPEC_STRIDE + j];
        if (r.w != 1) {
            A.status[k] = -9;
            return;
        }
        if (!(full || lin_done(T, m, n, r.y))) continue;
        if (j == q.y && (r.z & SPEC_TRACED)) {  // traced in the sweep: outputs are written
            A.passes[k] = j + 1;
            A.lastcls[k] = r.z & LASTCLS_MASK;
            if (A.keep_fill) A.dm_off[k] = A.spec_off[(long long)k * SPEC_STRIDE + j];
            A.status[k] = -((r.z >> 16) & 0xFF);
        } else if (!A.do_traceback) {
            A.cost[k] = r.x;
            A.passes[k] = j + 1;
            A.lastcls[k] = r.z & LASTCLS_MASK;
            A.status[k] = 0;
        } else {
            spec_requeue(A, k, m, n, j, T, false);
        }
        return;
    }
    spec_requeue(A, k, m, n, q.y + 1, T0 << (q.y + 1), false);
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
    const int cls = A.lastcls[k] & LASTCLS_MASK;
    const bool lean = (A.lastcls[k] & LASTCLS_LEAN) != 0;
    const bool row = (A.lastcls[k] & LASTCLS_ROW) != 0;
    const int P = A.lad.P[cls], R = A.lad.R[cls];
    const uint8_t* base = A.slab + (long long)A.slab_cta[k] * strides[cls];
    PairRes r;
    if (A.affine && row) {
        // the final pass's band: T doubled once per pass after the first
        const PairPlan pl = plan_affine(t, la, lb);
        const long long T = (long long)pl.T0 << tmax(A.passes[k] - 1, 0);
        const AffBand b = aff_band(m, n, band_p((int)T, m, n));
        r = aff_traceback_rowtile(base, 32 * rk_k_for(ladder_cap(A.lad, cls)), b.newk, t, x, m, y,
                                  n, tie, pair_out(A, k));
    } else if (A.affine && lean) r = aff_traceback_lean(base, P, R, t, x, m, y, n, tie, pair_out(A, k));
    else if (A.affine) r = aff_traceback(reinterpret_cast<const uint16_t*>(base), P, R, t, x, m, y, n, tie, pair_out(A, k));
    else r = lin_traceback(base, P, R, t, x, m, y, n, tie, pair_out(A, k));
    finish_pair(A, k, A.cost[k], r);
}

// Tracebacks of the pairs whose final fill sits in the arena, one thread per
// pair (after all class kernels, so no fill waits on a traceback).
__global__ void deferred_traceback_kernel(BatchArgs A, int skip_win)
{
    __shared__ Tables t;  // median and cost lookups from shared memory
    load_tables(t, A.tables);
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.npairs || A.dm_off[k] < 0 || A.status[k] != 0) return;
    // lean fills when deferred_traceback_win_kernel (lane pipeline) and
    // deferred_traceback_row_kernel (row tile) take them
    if (skip_win && A.affine && (A.lastcls[k] & LASTCLS_LEAN)) return;
    const int la = A.lena[k], lb = A.lenb[k];
    const int swaped = la <= lb ? 0 : 1;
    const uint8_t* x = A.seqs + (swaped ? A.offb[k] : A.offa[k]);
    const uint8_t* y = A.seqs + (swaped ? A.offa[k] : A.offb[k]);
    const int m = swaped ? lb : la, n = swaped ? la : lb;
    const int tie = A.swap_override ? A.swap_override[k] : swaped;
    const int cls = A.lastcls[k] & LASTCLS_MASK;
    const bool lean = (A.lastcls[k] & LASTCLS_LEAN) != 0;
    const bool row = (A.lastcls[k] & LASTCLS_ROW) != 0;
    const int P = A.lad.P[cls], R = A.lad.R[cls];
    const uint8_t* base = A.dm_arena + A.dm_off[k];
    PairRes r;
    if (A.affine && row) {
        const PairPlan pl = plan_affine(t, la, lb);
        const long long T = (long long)pl.T0 << tmax(A.passes[k] - 1, 0);
        const AffBand b = aff_band(m, n, band_p((int)T, m, n));
        r = aff_traceback_rowtile(base, 32 * rk_k_for(ladder_cap(A.lad, cls)), b.newk, t, x, m, y,
                                  n, tie, pair_out(A, k));
    } else if (A.affine && lean) {
        r = aff_traceback_lean(base, P, R, t, x, m, y, n, tie, pair_out(A, k));
    } else if (A.affine) {
        r = aff_traceback(reinterpret_cast<const uint16_t*>(base), P, R, t, x, m, y, n, tie,
                          pair_out(A, k));
    } else {
        r = lin_traceback(base, P, R, t, x, m, y, n, tie, pair_out(A, k));
    }
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
    int status = 0;
    for (int i = 0; i < len; i++)
        if ((mwg[i] = (uint8_t)t.median[(x[i] << t.lcm) + y[i]]) == 0) status = -3;
    const int n = ancestor_2(t, x, y, len, anc);
    int nga = 0, ngb = 0;
    for (int i = 0; i < len; i++) {
        nga |= x[i] != gap;
        ngb |= y[i] != gap;
    }
    out3[0] = n;
    out3[1] = (nga && ngb) ? worst_aligned(t, x, y, len) : 0;
    out3[2] = status;
}

// algn_verify_2 and seq_get_median_2d_no_gaps on an aligned pair (single
// thread; the per-call stubs of algn_CAML_verify_2 / seq_CAML_median_2_no_gaps).
__global__ void aligned_extra_kernel(const Tables* tg, const uint8_t* x, const uint8_t* y,
                                     int len, uint8_t* nogap, int* out2)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    out2[0] = verify_aligned(*tg, x, y, len);
    out2[1] = median_no_gaps(*tg, x, y, len, nogap);
}

}  // namespace

using ClassKernel = void (*)(BatchArgs, int);

// The compiled kernel for a class shape (narrow: a 128-thread CTA).
static ClassKernel class_kernel(int affine, int R, int variant, bool narrow)
{
    if (affine) {
        if (R == 2)
            return variant ? (narrow ? aff_class_kernel<2, true, true> : aff_class_kernel<2, true, false>)
                           : (narrow ? aff_class_kernel<2, false, true> : aff_class_kernel<2, false, false>);
        if (R == 3)
            return variant ? (narrow ? aff_class_kernel<3, true, true> : aff_class_kernel<3, true, false>)
                           : (narrow ? aff_class_kernel<3, false, true> : aff_class_kernel<3, false, false>);
        return variant ? (narrow ? aff_class_kernel<4, true, true> : aff_class_kernel<4, true, false>)
                       : (narrow ? aff_class_kernel<4, false, true> : aff_class_kernel<4, false, false>);
    }
    if (R == 2) return narrow ? lin_class_kernel<2, true> : lin_class_kernel<2, false>;
    if (R == 4) return narrow ? lin_class_kernel<4, true> : lin_class_kernel<4, false>;
    return narrow ? lin_class_kernel<8, true> : lin_class_kernel<8, false>;
}

int class_row_tile(const Ladder& lad, int affine, int cls, int variant, int row_tile)
{
    return (affine && variant == 1 && row_tile) ? rk_k_for(ladder_cap(lad, cls)) : 0;
}

static ClassKernel row_tile_kernel(int k)
{
    switch (k) {
        case 1: return aff_rk_kernel<1>;
        case 2: return aff_rk_kernel<2>;
        case 4: return aff_rk_kernel<4>;
        case 8: return aff_rk_kernel<8>;
        default: return aff_rk_kernel<16>;
    }
}

int class_blocks_per_sm(const Ladder& lad, int affine, int cls, int variant, int row_tile)
{
    int n = 0;
    const int rk = class_row_tile(lad, affine, cls, variant, row_tile);
    if (rk) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, row_tile_kernel(rk), 32 * NARROW_WARPS, 0);
        return n;
    }
    const int K = ladder_K(lad, cls), R = lad.R[cls];
    const int threads = K == 1 ? 32 * NARROW_WARPS : 32 * K;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, class_kernel(affine, R, variant, K == 1),
                                                  threads, class_dyn_smem(lad, affine, cls));
    return n;
}

long long class_slab_bytes(const Ladder& lad, int affine, int cls, int maxmn, int row_tile)
{
    const long long PR = (long long)lad.P[cls] * lad.R[cls];
    long long b = (long long)(maxmn + 1) * PR * (affine ? 2 : 1);
    const int rk = class_row_tile(lad, affine, cls, 1, row_tile);  // 32 K bytes per row
    b = std::max<long long>(b, (long long)(maxmn + 1) * 32 * rk);
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
    const int rk = class_row_tile(a.lad, a.affine, cls, variant, a.row_tile);
    if (rk) {
        row_tile_kernel(rk)<<<grid, 32 * NARROW_WARPS, 0, s>>>(a, cls);
        return;
    }
    const int K = ladder_K(a.lad, cls), R = a.lad.R[cls];
    const int threads = K == 1 ? 32 * NARROW_WARPS : 32 * K;
    class_kernel(a.affine, R, a.affine ? variant : 0, K == 1)<<<grid, threads,
                                                               class_dyn_smem(a.lad, a.affine, cls),
                                                               s>>>(a, cls);
}

void launch_sort_queues(const BatchArgs& a, int cls, int grid, cudaStream_t s)
{
    if (!a.qsorted) return;
    queue_hist_kernel<<<grid, 256, 0, s>>>(a, cls);
    queue_scatter_kernel<<<grid, 256, 0, s>>>(a, cls);
}

void launch_spec_resolve(const BatchArgs& a, cudaStream_t s)
{
    spec_resolve_kernel<<<(a.npairs + 127) / 128, 128, 0, s>>>(a);
}

void launch_spec_resolve2(const BatchArgs& a, cudaStream_t s)
{
    spec_resolve2_kernel<<<(a.npairs + 127) / 128, 128, 0, s>>>(a);
}

namespace {

constexpr int LWARP_WARPS = 4;  // warps (pairs) per CTA of the linear deferred traceback

// Deferred tracebacks of byte-coded lane-pipeline fills (every linear fill,
// lean affine ones), one warp per pair: every lane walks the same path
// through a shared-memory window of the pair's arena region (whole
// anti-diagonals for pipelines of fewer than 64 lane-rows: at any step a
// slot holds only the row of the band that owns it), refilled by all lanes
// at once every LW_DIAG anti-diagonals instead of one dependent load per
// step. Other affine fills are left to deferred_traceback_kernel.
__global__ void __launch_bounds__(32 * LWARP_WARPS)
    deferred_traceback_win_kernel(BatchArgs A)
{
    __shared__ Tables t;
    __shared__ uint32_t win[LWARP_WARPS][LW_SMEM_WORDS];
    load_tables(t, A.tables);
    __syncthreads();
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = blockIdx.x * LWARP_WARPS + wib;
    // warp-uniform exits
    if (k >= A.npairs || A.dm_off[k] < 0 || A.status[k] != 0) return;
    if (A.affine && (A.lastcls[k] & (LASTCLS_LEAN | LASTCLS_ROW)) != LASTCLS_LEAN) return;
    const int la = A.lena[k], lb = A.lenb[k];
    const int swaped = la <= lb ? 0 : 1;
    const uint8_t* x = A.seqs + (swaped ? A.offb[k] : A.offa[k]);
    const uint8_t* y = A.seqs + (swaped ? A.offa[k] : A.offb[k]);
    const int m = swaped ? lb : la, n = swaped ? la : lb;
    const int tie = A.swap_override ? A.swap_override[k] : swaped;
    const int cls = A.lastcls[k] & LASTCLS_MASK;
    const int PR = A.lad.P[cls] * A.lad.R[cls];
    const uint8_t* base = A.dm_arena + A.dm_off[k];
    PairRes r;
    if (!A.affine) {
        LinDmWindow<> w{base, win[wib], PR, PR / 4, lane, 32};
        r = lin_traceback_dm(w, t, x, m, y, n, tie, pair_out(A, k));
    } else if ((PR & (PR - 1)) == 0) {
        AffDmLeanWindow<true> rd{LinDmWindow<true>{base, win[wib], PR, PR / 4, lane, 32}};
        r = aff_traceback_dm(rd, t, x, m, y, n, tie, pair_out(A, k));
    } else {  // the R = 3 classes
        AffDmLeanWindow<false> rd{LinDmWindow<false>{base, win[wib], PR, PR / 4, lane, 32}};
        r = aff_traceback_dm(rd, t, x, m, y, n, tie, pair_out(A, k));
    }
    if (lane == 0) finish_pair(A, k, A.cost[k], r);
}

// The same for row-tile fills (lean affine, small batches): one warp per
// pair through a window of whole rows (AffDmRowWindow, RW_BYTES per warp).
constexpr int RWARP_WARPS = 4;
__global__ void __launch_bounds__(32 * RWARP_WARPS) deferred_traceback_row_kernel(BatchArgs A)
{
    __shared__ Tables t;
    __shared__ Word16 win[RWARP_WARPS][RW_BYTES / 16];
    load_tables(t, A.tables);
    __syncthreads();
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = blockIdx.x * RWARP_WARPS + wib;
    // warp-uniform exits
    if (k >= A.npairs || A.dm_off[k] < 0 || A.status[k] != 0) return;
    if ((A.lastcls[k] & (LASTCLS_LEAN | LASTCLS_ROW)) != (LASTCLS_LEAN | LASTCLS_ROW)) return;
    const int la = A.lena[k], lb = A.lenb[k];
    const int swaped = la <= lb ? 0 : 1;
    const uint8_t* x = A.seqs + (swaped ? A.offb[k] : A.offa[k]);
    const uint8_t* y = A.seqs + (swaped ? A.offa[k] : A.offb[k]);
    const int m = swaped ? lb : la, n = swaped ? la : lb;
    const int tie = A.swap_override ? A.swap_override[k] : swaped;
    const int cls = A.lastcls[k] & LASTCLS_MASK;
    // the final pass's band: T doubled once per pass after the first
    const PairPlan pl = plan_affine(t, la, lb);
    const long long T = (long long)pl.T0 << tmax(A.passes[k] - 1, 0);
    const AffBand b = aff_band(m, n, band_p((int)T, m, n));
    const int S = 32 * rk_k_for(ladder_cap(A.lad, cls));
    AffDmRowWindow rd{A.dm_arena + A.dm_off[k], win[wib], S, b.newk, RW_BYTES / S, lane, 32};
    const PairRes r = aff_traceback_dm(rd, t, x, m, y, n, tie, pair_out(A, k));
    if (lane == 0) finish_pair(A, k, A.cost[k], r);
}

}  // namespace

int launch_deferred_traceback(const BatchArgs& a, bool warp_per_pair, cudaStream_t s)
{
    if (a.npairs <= 0 || a.dm_cap <= 0) return 0;
    const int threads = 128;
    if (!warp_per_pair) {
        deferred_traceback_kernel<<<(a.npairs + threads - 1) / threads, threads, 0, s>>>(a, 0);
        return 1;
    }
    deferred_traceback_win_kernel<<<(a.npairs + LWARP_WARPS - 1) / LWARP_WARPS,
                                    32 * LWARP_WARPS, 0, s>>>(a);
    if (!a.affine) return 1;
    int n = 2;
    if (a.row_tile) {
        deferred_traceback_row_kernel<<<(a.npairs + RWARP_WARPS - 1) / RWARP_WARPS,
                                        32 * RWARP_WARPS, 0, s>>>(a);
        n++;
    }
    deferred_traceback_kernel<<<(a.npairs + threads - 1) / threads, threads, 0, s>>>(a, 1);
    return n;
}

namespace {

// The per-call backtrace_2d of a kept linear fill, one warp: the fill sits
// in the pair's arena region (dm_off[0] >= 0) or, when it had none, in the
// slab of the pipeline that ran it; every lane walks the path through the
// shared-memory window with the caller's tie preference.
__global__ void __launch_bounds__(32) call_traceback_lin_kernel(BatchArgs A,
                                                                 const long long* strides)
{
    __shared__ Tables t;
    __shared__ uint32_t win[LW_SMEM_WORDS];
    load_tables(t, A.tables);
    __syncthreads();
    if (A.status[0] != 0) return;
    const int la = A.lena[0], lb = A.lenb[0];
    const int swaped = la <= lb ? 0 : 1;
    const uint8_t* x = A.seqs + (swaped ? A.offb[0] : A.offa[0]);
    const uint8_t* y = A.seqs + (swaped ? A.offa[0] : A.offb[0]);
    const int m = swaped ? lb : la, n = swaped ? la : lb;
    const int tie = A.swap_override ? A.swap_override[0] : swaped;
    const int cls = A.lastcls[0] & LASTCLS_MASK;
    const int PR = A.lad.P[cls] * A.lad.R[cls];
    const uint8_t* base = A.dm_off[0] >= 0 ? A.dm_arena + A.dm_off[0]
                                           : A.slab + (long long)A.slab_cta[0] * strides[cls];
    LinDmWindow<> w{base, win, PR, PR / 4, (int)threadIdx.x, 32};
    const PairRes r = lin_traceback_dm(w, t, x, m, y, n, tie, pair_out(A, 0));
    if (threadIdx.x == 0) finish_pair(A, 0, A.cost[0], r);
}

}  // namespace

void launch_call_traceback_lin(const BatchArgs& a, const long long* d_strides, cudaStream_t s)
{
    call_traceback_lin_kernel<<<1, 32, 0, s>>>(a, d_strides);
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

int class_pipes_per_cta(const Ladder& lad, int affine, int cls, int variant, int row_tile)
{
    if (class_row_tile(lad, affine, cls, variant, row_tile)) return NARROW_WARPS;
    const int P = lad.P[cls];
    return P >= 64 ? 1 : NARROW_WARPS * (P < 32 ? 32 / P : 1);
}

void launch_aligned_medians(const Tables* t, const uint8_t* x, const uint8_t* y,
                            int len, uint8_t* anc, uint8_t* mwg, int* out3,
                            cudaStream_t s)
{
    aligned_medians_kernel<<<1, 32, 0, s>>>(t, x, y, len, anc, mwg, out3);
}

void launch_aligned_extra(const Tables* t, const uint8_t* x, const uint8_t* y, int len,
                          uint8_t* nogap, int* out2, cudaStream_t s)
{
    aligned_extra_kernel<<<1, 32, 0, s>>>(t, x, y, len, nogap, out2);
}

namespace {

__global__ void limit_walk_kernel(LimitWalk a)
{
    const Tables& t = *a.t;
    const int cls = a.lastcls[0] & LASTCLS_MASK;
    // the final pass's band: T doubled once per pass after the first
    const PairPlan pl = plan_linear_deltawh(t, a.l1, a.l2, a.deltawh);
    const int full = a.pfull[0] & 1;
    const long long T = (long long)pl.T0 << tmax(a.passes[0] - 1, 0);
    const LinBand b = lin_band(pl.m, pl.n, full, full ? 0 : band_p((int)T, pl.m, pl.n));
    const uint8_t* base = (a.dm_off && a.dm_off[0] >= 0)
                              ? a.dm_arena + a.dm_off[0]
                              : a.slab + (long long)a.slab_cta[0] * a.strides[cls];
    LinDmBytes rd{base, a.lad.P[cls], a.lad.R[cls]};
    int len = 0;
    a.out2[0] = lin_limit_walk(rd, b, a.s1, a.s2, t.gap, a.st_s1, a.st_s2, a.algn_s1,
                               a.algn_s2, a.swaped, a.r1, a.r2, a.cap, &len);
    a.out2[1] = len;
}

}  // namespace

void launch_limit_walk(const LimitWalk& a, cudaStream_t s)
{
    limit_walk_kernel<<<1, 1, 0, s>>>(a);
}

}  // namespace pa
