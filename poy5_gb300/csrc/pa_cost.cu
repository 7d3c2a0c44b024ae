// Cost-only affine alignment: algn_CAML_cost_affine_3 (src/algn.c:2456-2515)
// -> algn_fill_plane_3_aff_nobt (src/algn.c:1986-2110), the full unbanded
// four-state fill SeqCS.DOS.distance uses for affine cost models.
//
// One warp per pair. The columns are cut into blocks of 32 * K; each lane
// keeps the previous row of its K columns in registers, so a block sweeps
// all rows with no memory traffic but its left boundary column (one int4 per
// row, written by the previous block). Within a row, EV, EB and CB depend on
// the previous row only; the horizontal state EH[j] = min(EH[j-1] + x_j, t_j)
// is a min-plus recurrence, solved per row by composing each lane's K maps
// and an inclusive warp scan of the compositions.
//
// Long pairs take a whole CTA instead: its warps split the column blocks
// and advance one row per barrier, each a row behind the warp to its left.
// Small batches run every pair that way (nobt_coop_kernel); in large ones
// the leading pairs of the longest-first order with more cells than the
// batch has per launched warp do (nobt_kernel), so that no single warp is
// left with a long pair at the end.
//
// The reference keeps its rows in one buffer whose current and previous rows
// overlap by a few words (the previous row starts lenj + 2 ints after the
// current one, arrays of 2 * largest ints). For lenj >= 2 the only effect is
// that every even row writes HIGH into the previous row's EV[lenj] and
// CB[lenj] before reading them; sequences of at most 2 positions are replayed
// word for word instead.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pa_cost.h"

namespace pa {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int BIG = 1 << 29;  // "no path" inside a composed map; + HIGH stays < 2^31

__device__ __forceinline__ int gap_open_cost(int idx, int prev, int curr, int gap, int go)
{
    if (idx == 1 && (gap & curr)) return 0;
    if (idx > 1 && !(gap & prev) && (gap & curr)) return 0;
    return go;
}

// The reference's buffer, word for word, for sequences of at most 2 positions.
__device__ int nobt_tiny(const Tables& t, const uint8_t* si, int li, const uint8_t* sj, int lj)
{
    const int gap = t.gap, go = t.go;
    const int largest = lj;
    const int leni = li - 1, lenj = lj - 1;
    const int off = lenj + 2;
    int mat[12 * 2 + 4];
    for (int k = 0; k < 12 * largest + 4; k++) mat[k] = 0;
    int cb = 0, eb = 2 * largest, ev = 4 * largest, eh = 6 * largest;
    const int gopc = 10 * largest, shx = 11 * largest;
    mat[cb] = 0;
    mat[eb] = HIGH;
    mat[eh] = go;
    mat[ev] = go;
    for (int j = 1; j <= lenj; j++) {
        mat[eh + j] = mat[eh + j - 1] + t.prepend[sj[j]];
        mat[cb + j] = HIGH;
        mat[eb + j] = HIGH;
        mat[ev + j] = HIGH;
    }
    int peh = eh + off, pev = ev + off, peb = eb + off, pcb = cb + off;
    mat[shx] = 0;
    for (int j = 1; j <= lenj; j++) {
        mat[gopc + j] = gap_open_cost(j, sj[j - 1], sj[j], gap, go);
        mat[shx + j] = ((sj[j - 1] & gap) && !(sj[j] & gap)) ? mat[gopc + j] + t.prepend[sj[j]]
                                                               : t.prepend[sj[j]];
    }
    if (lenj >= 1) mat[shx + 1] = t.prepend[sj[1]];
    int ic = si[0];
    for (int i = 1; i <= leni; i++) {
        int x;
        x = peh; peh = eh; eh = x;
        x = pev; pev = ev; ev = x;
        x = peb; peb = eb; eb = x;
        x = pcb; pcb = cb; cb = x;
        mat[eh] = HIGH;
        const int ip = ic;
        ic = si[i];
        const int sgext = tcost(t, ic, gap);
        const int sgop = gap_open_cost(i, ip, ic, gap, go);
        const int sng = ic & NTMPGAP;
        const int svext = (i > 1 && (ip & gap) && !(ic & gap)) ? sgop + sgext : sgext;
        const int r = mat[pev] + svext;
        mat[eh] = HIGH;
        mat[cb] = r;
        mat[eb] = HIGH;
        mat[ev] = r;
        mat[cb] = HIGH;
        int jc = sj[0];
        for (int j = 1; j <= lenj; j++) {
            const int jp = jc;
            jc = sj[j];
            const int jng = jc & NTMPGAP;
            const int jgr = t.prepend[jc], jgo = mat[gopc + j];
            mat[eh + j] = tmin(mat[eh + j - 1] + mat[shx + j], mat[cb + j - 1] + jgo + jgr);
            mat[ev + j] = tmin(mat[pev + j] + svext, mat[pcb + j] + sgop + sgext);
            const bool flag = (TMPGAP & ic) && (TMPGAP & jc);
            const bool flag2 = !(TMPGAP & ip) && !(TMPGAP & jp);
            const int d = flag ? 0 : HIGH;
            const int od = flag ? (flag2 ? 0 : 2 * go) : HIGH;
            mat[eb + j] = tmin(mat[peb + j - 1] + d, mat[pcb + j - 1] + od);
            const int dg = tcost(t, sng, jng);
            const int xgo = tmax(jgo, sgop);
            const int a0 = mat[pcb + j - 1] + dg;
            const int a1 = (ic == sng) ? mat[pev + j - 1] + dg : mat[pev + j - 1] + dg + jgo;
            const int a2 = (jc == jng) ? mat[peh + j - 1] + dg : mat[peh + j - 1] + dg + sgop;
            const int a3 = mat[peb + j - 1] + dg + xgo;
            mat[cb + j] = tmin(tmin(a0, a1), tmin(a2, a3));
        }
    }
    return tmin(tmin(mat[eh + lenj], mat[ev + lenj]), tmin(mat[eb + lenj], mat[cb + lenj]));
}

// min(x + s, t) maps composed along a row: apply f then g
struct MinPlus {
    int s, t;
};
__device__ __forceinline__ MinPlus compose(MinPlus f, MinPlus g)
{
    return MinPlus{tmin(f.s + g.s, BIG), tmin(tmin(f.t + g.s, BIG), g.t)};
}
__device__ __forceinline__ int apply(MinPlus f, int x) { return tmin(x + f.s, f.t); }

// Inclusive scan over the warp: lane l gets f_l o ... o f_0 (f_0 first).
__device__ __forceinline__ MinPlus warp_scan(MinPlus f, int lane)
{
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int ps = __shfl_up_sync(FULL, f.s, d);
        const int pt = __shfl_up_sync(FULL, f.t, d);
        if (lane >= d) f = compose(MinPlus{ps, pt}, f);
    }
    return f;
}

// One lane's K columns of a column block: column constants (jc, gj = gop +
// prepend, gop, shx, jpgap, lastm = the bit of column lenj if this lane has
// it and lenj >= 2), the previous row of every state (pEH, pEV, pEB, pCB), the
// block geometry and, in lane 0, the previous row's value of column c0 - 1.
// Kept as separate arrays in the caller so that they stay in registers.
#define NOBT_LANE_PARAMS                                                                   \
    int (&jc)[K], int (&gj)[K], int (&gop)[K], int (&shx)[K], unsigned& jpgap, unsigned& lastm, \
        int (&pEH)[K], int (&pEV)[K], int (&pEB)[K], int (&pCB)[K], int &c0, int &last_lane, \
        int &last_q, int4 &dprev, int &ic_last
#define NOBT_LANE_DECL                                                                     \
    int jc[K], gj[K], gop[K], shx[K];                                                      \
    unsigned jpgap, lastm;                                                                 \
    int pEH[K], pEV[K], pEB[K], pCB[K];                                                    \
    int c0, last_lane, last_q;                                                             \
    int4 dprev;                                                                            \
    int ic_last
#define NOBT_LANE_ARGS jc, gj, gop, shx, jpgap, lastm, pEH, pEV, pEB, pCB, c0, last_lane, last_q, dprev, ic_last

// Start column block `blk`: constants and row 0. left: the previous block's
// last column (row 0 read here; unused for blk 0); out: this block's last
// column (row 0 written here). All 32 lanes call it.
template <int K>
__device__ __forceinline__ void nobt_block_begin(NOBT_LANE_PARAMS, const Tables& t,
                                                 const uint8_t* si, const uint8_t* sj, int lenj,
                                                 int blk, int lane, const int4* left, int4* out)
{
    const int gap = t.gap, go = t.go;
    constexpr int W = 32 * K;
    c0 = blk * W + lane * K;
    jpgap = 0;
    lastm = 0;
    int jgr[K];
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = c0 + q;
        const bool real = j <= lenj;
        const int c = real ? sj[j] : 0;
        const int cp = (real && j > 0) ? sj[j - 1] : 0;
        jc[q] = c;
        jgr[q] = t.prepend[c];
        gop[q] = (real && j > 0) ? gap_open_cost(j, cp, c, gap, go) : 0;
        gj[q] = gop[q] + jgr[q];
        shx[q] = (j > 1 && (cp & gap) && !(c & gap)) ? gop[q] + jgr[q] : jgr[q];
        jpgap |= (cp & TMPGAP) ? 1u << q : 0u;
        lastm |= (j == lenj && lenj >= 2) ? 1u << q : 0u;
    }
    MinPlus f{0, BIG};
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = c0 + q;
        f = compose(f, j == 0 ? MinPlus{BIG, go} : MinPlus{jgr[q], BIG});
    }
    const MinPlus pre = warp_scan(f, lane);
    const MinPlus ex{__shfl_up_sync(FULL, pre.s, 1), __shfl_up_sync(FULL, pre.t, 1)};
    const int4 l0 = blk > 0 ? left[0] : make_int4(HIGH, HIGH, HIGH, HIGH);
    int x = lane == 0 ? l0.x : apply(ex, l0.x);
    if (blk == 0) x = lane == 0 ? 0 : apply(ex, 0);
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = c0 + q;
        x = j == 0 ? go : x + jgr[q];
        pEH[q] = x;
        pEV[q] = j == 0 ? go : HIGH;
        pEB[q] = HIGH;
        pCB[q] = j == 0 ? 0 : HIGH;
    }
    const int last_col = tmin(lenj, blk * W + W - 1);
    last_lane = (last_col - blk * W) / K;
    last_q = (last_col - blk * W) % K;
    dprev = l0;
    ic_last = si[0];
    __syncwarp();
#pragma unroll
    for (int q = 0; q < K; q++)
        if (lane == last_lane && q == last_q)
            out[0] = make_int4(pEH[q], pEV[q], pEB[q], pCB[q]);
}

// The reference's even rows read HIGH for the previous row's EV and CB at
// column lenj (its overlapping row buffers). Applied to the lane state
// before the row's cells: the changed words feed no other column of the row
// (column lenj + 1 does not exist) and the row then overwrites them.
template <int K>
__device__ __forceinline__ void even_row_last_column(NOBT_LANE_PARAMS, int i)
{
    if ((i & 1) == 0 && lastm) {
#pragma unroll
        for (int q = 0; q < K; q++)
            if ((lastm >> q) & 1) {
                pEV[q] = HIGH;
                pCB[q] = HIGH;
            }
    }
}

// Row i >= 1 of the block: ic = si[i]; lbv = the block boundary of row i
// (the previous block's last column; used by lane 0 when blk > 0), read by
// the caller before this row writes out[i] (the last lane), so the boundary
// and out may be the same column.
template <int K>
__device__ __forceinline__ void nobt_block_row(NOBT_LANE_PARAMS, const Tables& t, int ic,
                                               int i, int lenj, int blk, int lane, int4 lbv,
                                               int4* out)
{
    const int gap = t.gap, go = t.go;
    const int ip = ic_last;
    ic_last = ic;
    const int sgext = tcost(t, ic, gap);
    const int sgop = gap_open_cost(i, ip, ic, gap, go);
    const int sng = ic & NTMPGAP;
    const int srow = t.rowoff[sng];
    const int svext = (i > 1 && (ip & gap) && !(ic & gap)) ? sgop + sgext : sgext;
    // left neighbour: previous row's last column of lane - 1 (lane 0: the
    // block boundary of row i - 1) and, for EH, the current row's
    int4 dg;
    dg.x = __shfl_up_sync(FULL, pEH[K - 1], 1);
    dg.y = __shfl_up_sync(FULL, pEV[K - 1], 1);
    dg.z = __shfl_up_sync(FULL, pEB[K - 1], 1);
    dg.w = __shfl_up_sync(FULL, pCB[K - 1], 1);
    int4 lb = make_int4(HIGH, HIGH, HIGH, HIGH);  // block boundary, row i
    if (lane == 0) {
        dg = dprev;
        if (blk > 0) lb = lbv;
        dprev = lb;
    }
    even_row_last_column(NOBT_LANE_ARGS, i);
    int nEV[K], nEB[K], nCB[K];
    int dEH = dg.x, dEV = dg.y, dEB = dg.z, dCB = dg.w;
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = c0 + q;
        const int c = jc[q];
        const int jng = c & NTMPGAP;
        if (j == 0) {
            nEV[q] = pEV[q] + svext;
            nEB[q] = HIGH;
            nCB[q] = HIGH;
        } else {
            nEV[q] = tmin(pEV[q] + svext, pCB[q] + sgop + sgext);
            const bool flag = (TMPGAP & ic) && (TMPGAP & c);
            const bool flag2 = !(TMPGAP & ip) && !((jpgap >> q) & 1);
            const int d = flag ? 0 : HIGH;
            const int od = flag ? (flag2 ? 0 : 2 * go) : HIGH;
            nEB[q] = tmin(dEB + d, dCB + od);
            const int dgc = t.csw[srow + jng];
            const int xgo = tmax(gop[q], sgop);
            const int a0 = dCB + dgc;
            const int a1 = dEV + dgc + (ic == sng ? 0 : gop[q]);
            const int a2 = dEH + dgc + (c == jng ? 0 : sgop);
            const int a3 = dEB + dgc + xgo;
            nCB[q] = tmin(tmin(a0, a1), tmin(a2, a3));
        }
        dEH = pEH[q];
        dEV = pEV[q];
        dEB = pEB[q];
        dCB = pCB[q];
    }
    // EH along the row: EH[j] = min(EH[j-1] + shx_j, CB[j-1] + gop_j + jgr_j)
    const int cbl = __shfl_up_sync(FULL, nCB[K - 1], 1);
    MinPlus f{0, BIG};
    int cprev = lane == 0 ? lb.w : cbl;
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = c0 + q;
        const MinPlus g = j == 0 ? MinPlus{BIG, HIGH}
                                 : MinPlus{shx[q], tmin(cprev + gj[q], BIG)};
        f = compose(f, g);
        cprev = nCB[q];
    }
    const MinPlus pre = warp_scan(f, lane);
    const MinPlus ex{__shfl_up_sync(FULL, pre.s, 1), __shfl_up_sync(FULL, pre.t, 1)};
    const int lbx = __shfl_sync(FULL, lb.x, 0);  // only lane 0 read the boundary
    int x = lane == 0 ? lbx : apply(ex, lbx);
    cprev = lane == 0 ? lb.w : cbl;
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = c0 + q;
        x = j == 0 ? HIGH : tmin(x + shx[q], cprev + gj[q]);
        pEH[q] = x;
        pEV[q] = nEV[q];
        pEB[q] = nEB[q];
        pCB[q] = nCB[q];
        cprev = nCB[q];
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < K; q++)
        if (lane == last_lane && q == last_q)
            out[i] = make_int4(pEH[q], pEV[q], pEB[q], pCB[q]);
}

// Composition without the BIG clamps, for rows whose values all stay below
// BIG: a "no path" term then only grows by the row's costs (far from 2^31),
// and apply() gives what the clamped maps give.
__device__ __forceinline__ MinPlus compose_nc(MinPlus f, MinPlus g)
{
    return MinPlus{f.s + g.s, __viaddmin_s32(f.t, g.s, g.t)};
}
__device__ __forceinline__ MinPlus warp_scan_nc(MinPlus f, int lane)
{
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int ps = __shfl_up_sync(FULL, f.s, d);
        const int pt = __shfl_up_sync(FULL, f.t, d);
        if (lane >= d) f = compose_nc(MinPlus{ps, pt}, f);
    }
    return f;
}

// Row i of the block when the row's base carries neither gap bit and the
// gap opening is not negative (the usual DNA row). Then the row's gap
// opening is go, the EB path from EB / CB is closed (+ HIGH), the diagonal
// gap-opening term is go, and CB's four terms share the substitution cost:
//   CB = min(min(CB', EV', EB' + go) + c(i, j), EH' + c(i, j) + go [j gapped])
// with tab[ic][jc] = {c(i, j), c(i, j) + (go if column j's base has the gap
// bit)}. Same values as nobt_block_row while every value is below BIG.
template <int K>
__device__ __forceinline__ void nobt_block_row_plain(NOBT_LANE_PARAMS, const Tables& t,
                                                     const int2* tab, int ic, int i, int blk,
                                                     int lane, int4 lbv, int4* out)
{
    const int gap = t.gap, go = t.go;
    const int ip = ic_last;
    ic_last = ic;
    const int sgext = tcost(t, ic, gap);
    const int svext = (i > 1 && (ip & gap)) ? go + sgext : sgext;
    const int sgoe = go + sgext;
    const int2* tr = tab + ic * 32;
    int4 dg;
    dg.x = __shfl_up_sync(FULL, pEH[K - 1], 1);
    dg.y = __shfl_up_sync(FULL, pEV[K - 1], 1);
    dg.z = __shfl_up_sync(FULL, pEB[K - 1], 1);
    dg.w = __shfl_up_sync(FULL, pCB[K - 1], 1);
    int4 lb = make_int4(HIGH, HIGH, HIGH, HIGH);
    if (lane == 0) {
        dg = dprev;
        if (blk > 0) lb = lbv;
        dprev = lb;
    }
    even_row_last_column(NOBT_LANE_ARGS, i);
    const bool z0 = c0 == 0;  // this lane holds column 0
    int nEV[K], nEB[K], nCB[K];
    int dEH = dg.x, dEV = dg.y, dEB = dg.z, dCB = dg.w;
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int2 cc = tr[jc[q]];
        nEV[q] = __viaddmin_s32(pEV[q], svext, pCB[q] + sgoe);
        nEB[q] = tmin(dEB, dCB) + HIGH;
        nCB[q] = __viaddmin_s32(__vimin3_s32(dCB, dEV, dEB + go), cc.x, dEH + cc.y);
        dEH = pEH[q];
        dEV = pEV[q];
        dEB = pEB[q];
        dCB = pCB[q];
    }
    if (z0) {
        nEV[0] = pEV[0] + svext;
        nEB[0] = HIGH;
        nCB[0] = HIGH;
    }
    const int cbl = __shfl_up_sync(FULL, nCB[K - 1], 1);
    const int cin = lane == 0 ? lb.w : cbl;
    int cprev = cin;
    MinPlus f = z0 ? MinPlus{BIG, HIGH} : MinPlus{shx[0], cprev + gj[0]};
    cprev = nCB[0];
#pragma unroll
    for (int q = 1; q < K; q++) {
        f = compose_nc(f, MinPlus{shx[q], cprev + gj[q]});
        cprev = nCB[q];
    }
    const MinPlus pre = warp_scan_nc(f, lane);
    const MinPlus ex{__shfl_up_sync(FULL, pre.s, 1), __shfl_up_sync(FULL, pre.t, 1)};
    const int lbx = __shfl_sync(FULL, lb.x, 0);
    int x = lane == 0 ? lbx : __viaddmin_s32(lbx, ex.s, ex.t);
    cprev = cin;
#pragma unroll
    for (int q = 0; q < K; q++) {
        x = __viaddmin_s32(x, shx[q], cprev + gj[q]);
        if (q == 0 && z0) x = HIGH;
        pEH[q] = x;
        pEV[q] = nEV[q];
        pEB[q] = nEB[q];
        pCB[q] = nCB[q];
        cprev = nCB[q];
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < K; q++)
        if (lane == last_lane && q == last_q)
            out[i] = make_int4(pEH[q], pEV[q], pEB[q], pCB[q]);
}

// Row i of the block, by its kind (tab null: every row the general way).
template <int K>
__device__ __forceinline__ void nobt_row(NOBT_LANE_PARAMS, const Tables& t, const int2* tab,
                                         int ic, int i, int lenj, int blk, int lane, int4 lbv,
                                         int4* out)
{
    if (tab && !(ic & (TMPGAP | t.gap)))
        nobt_block_row_plain<K>(NOBT_LANE_ARGS, t, tab, ic, i, blk, lane, lbv, out);
    else
        nobt_block_row<K>(NOBT_LANE_ARGS, t, ic, i, lenj, blk, lane, lbv, out);
}

// min of the four states of the block's last column (valid in every lane)
template <int K>
__device__ __forceinline__ int nobt_block_result(NOBT_LANE_PARAMS, int lane)
{
    int r = 0;
#pragma unroll
    for (int q = 0; q < K; q++)
        if (lane == last_lane && q == last_q)
            r = tmin(tmin(pEH[q], pEV[q]), tmin(pEB[q], pCB[q]));
    return __shfl_sync(FULL, r, last_lane);
}

// One warp, blocks in sequence; bnd: one column (the block boundary), read
// and rewritten row by row. The rows arrive in groups of 32: while a group
// runs from this warp's shared pfb / pfs (boundary words and row bases),
// each lane already holds one row of the next group in registers, so no row
// waits for its boundary word to come back from L2. A group's prefetch reads
// rows this block has not yet rewritten.
template <int K>
__device__ __forceinline__ int nobt_warp(const Tables& t, const int2* tab, const uint8_t* si, int li,
                                         const uint8_t* sj, int lj, int4* bnd, int lane,
                                         int4* pfb, uint8_t* pfs)
{
    const int leni = li - 1, lenj = lj - 1;
    const int nblk = (lenj + 1 + 32 * K - 1) / (32 * K);
    NOBT_LANE_DECL;
    int result = 0;
    for (int blk = 0; blk < nblk; blk++) {
        nobt_block_begin<K>(NOBT_LANE_ARGS, t, si, sj, lenj, blk, lane, bnd, bnd);
        int4 rb = make_int4(HIGH, HIGH, HIGH, HIGH);
        int rs = 0;
        if (1 + lane <= leni) {
            rs = si[1 + lane];
            if (blk > 0) rb = bnd[1 + lane];
        }
        for (int i0 = 1; i0 <= leni; i0 += 32) {
            __syncwarp();
            pfb[lane] = rb;
            pfs[lane] = (uint8_t)rs;
            __syncwarp();
            const int r = i0 + 32 + lane;
            if (r <= leni) {
                rs = si[r];
                if (blk > 0) rb = bnd[r];
            }
            const int n = tmin(32, leni - i0 + 1);
            for (int q = 0; q < n; q++)
                nobt_row<K>(NOBT_LANE_ARGS, t, tab, pfs[q], i0 + q, lenj, blk, lane, pfb[q], bnd);
        }
        __syncwarp();
        if (blk == nblk - 1) result = nobt_block_result<K>(NOBT_LANE_ARGS, lane);
    }
    return result;
}

// CTA barrier that the warps may reach from different loops (non-aligned
// barrier.sync): the cooperative schedule below has every warp execute the
// same number of them, from a stagger, its rows and a pad loop. It orders
// the warps' global writes before the other warps' later reads.
__device__ __forceinline__ void cta_barrier() { asm volatile("barrier.sync 0;" ::: "memory"); }

// All NW warps of the CTA on one pair: warp w takes blocks w, w + NW, ...
// and the warps advance one row per barrier, warp w a row behind warp w - 1,
// so block b + 1 reads block b's last column one row after it is written.
// cols: one column (rows 0..leni) per block; RING: one per warp instead,
// rewritten block after block. Warp w - 1 rewrites row i of its column
// rows - 1 barriers after warp w read it, and warp 0 reads warp NW - 1's
// column rows - NW + 1 barriers after it was written, so with li >= NW
// every read sees the previous block's row and no later one.
template <int K, int NW, bool RING = false>
__device__ __forceinline__ int nobt_coop(const Tables& t, const int2* tab, const uint8_t* si, int li,
                                         const uint8_t* sj, int lj, int4* cols, int col_stride,
                                         int warp, int lane, int* sres)
{
    const int leni = li - 1, lenj = lj - 1;
    const int nblk = (lenj + 1 + 32 * K - 1) / (32 * K);
    const int rows = leni + 1;
    // barriers of the schedule: the warp owning the last block finishes its
    // last row at step total - 1; every warp pads to total
    const long long total = (long long)((nblk - 1) / NW) * rows + rows + (nblk - 1) % NW;
    NOBT_LANE_DECL;
    long long it = 0;
    for (; it < warp; it++) cta_barrier();
    for (int blk = warp; blk < nblk; blk += NW) {
        const int4* left = RING ? cols + (long long)((warp + NW - 1) % NW) * col_stride
                                : cols + (long long)(blk > 0 ? blk - 1 : 0) * col_stride;
        int4* out = cols + (long long)(RING ? warp : blk) * col_stride;
        nobt_block_begin<K>(NOBT_LANE_ARGS, t, si, sj, lenj, blk, lane, left, out);
        cta_barrier();
        it++;
        for (int i = 1; i <= leni; i++) {
            nobt_row<K>(NOBT_LANE_ARGS, t, tab, si[i], i, lenj, blk, lane,
                        (lane == 0 && blk > 0) ? left[i] : make_int4(HIGH, HIGH, HIGH, HIGH), out);
            if (blk == nblk - 1 && i == leni) {
                const int r = nobt_block_result<K>(NOBT_LANE_ARGS, lane);
                if (lane == 0) *sres = r;
            }
            cta_barrier();
            it++;
        }
    }
    for (; it < total; it++) cta_barrier();
    return *sres;
}

// columns per lane: 16 for the large batches' one-warp-per-pair kernel (the
// row scan amortised over twice the cells beats the occupancy that 8 keeps:
// 8,192 serving pairs 31.0 vs 34.9 ms, 2 CTAs per SM against 3), 8 for the
// small batches' cooperative kernel (more column blocks for its warps)
constexpr int NOBT_K = 16;
constexpr int COOP_K = 8;
constexpr int NOBT_WARPS = 4;   // one pair per warp
constexpr int COOP_WARPS = 8;   // one pair per CTA

__device__ __forceinline__ void load_tables_smem(Tables& st, const Tables* g)
{
    for (int k = threadIdx.x; k < (int)(sizeof(Tables) / 4); k += blockDim.x)
        reinterpret_cast<int*>(&st)[k] = reinterpret_cast<const int*>(g)[k];
    __syncthreads();
}

// The plain rows' table (nobt_block_row_plain): tab[a * 32 + b] = {c(a, b &
// 15), c(a, b & 15) + (go if b has bits above the base's)} for row bases
// a < 16; null when go < 0 (every row then takes the general way).
__device__ __forceinline__ const int2* build_row_table(int2* tab, const Tables& st)
{
    for (int k = threadIdx.x; k < 16 * 32; k += blockDim.x) {
        const int a = k >> 5, b = k & 31;
        const int v = st.csw[st.rowoff[a] + (b & NTMPGAP)];
        tab[k] = make_int2(v, v + ((b & NTMPGAP) == b ? 0 : st.go));
    }
    __syncthreads();
    return st.go >= 0 ? tab : nullptr;
}

// Pair k's screening, as DOS.distance / cost_affine_3 need it (warp-uniform).
struct NobtPair {
    const uint8_t *si, *sj;
    int li, lj, k;
    int cost, status;
    bool run;  // the fill has to run
};

__device__ NobtPair nobt_screen(const NobtArgs& A, const Tables& st, int k, int lane)
{
    NobtPair q;
    q.k = k;
    const int la = A.lena[k], lb = A.lenb[k];
    const uint8_t* a = A.seqs + A.offa[k];
    const uint8_t* b = A.seqs + A.offb[k];
    // states must index the tables; distance: all-gap sequences are "missing"
    int bad = 0, ga = 1, gb = 1;
    const int ns = 1 << st.lcm;
    for (int i = lane; i < la; i += 32) {
        bad |= a[i] >= ns;
        ga &= a[i] == st.gap;
    }
    for (int i = lane; i < lb; i += 32) {
        bad |= b[i] >= ns;
        gb &= b[i] == st.gap;
    }
    bad = __any_sync(FULL, bad);
    ga = __all_sync(FULL, ga);
    gb = __all_sync(FULL, gb);
    q.cost = 0;
    q.status = 0;
    q.run = false;
    const bool sw = la > lb;  // the shorter sequence runs down the rows
    q.si = sw ? b : a;
    q.sj = sw ? a : b;
    q.li = sw ? lb : la;
    q.lj = sw ? la : lb;
    if (la < 1 || lb < 1) q.status = -4;
    else if (bad) q.status = -7;
    else if (A.missing_distance != NOBT_NO_MISSING && (ga || gb)) q.cost = A.missing_distance;
    else if (la > 65535 || lb > 65535 || q.li > A.bnd_stride) q.status = -6;
    else q.run = true;
    return q;
}

// Sum of la * lb over the batch into *A.total.
__global__ void nobt_total_kernel(NobtArgs A)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long c = k < A.npairs ? (unsigned long long)A.lena[k] * A.lenb[k] : 0ull;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) c += __shfl_down_sync(FULL, c, d);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(const_cast<unsigned long long*>(A.total), c);
}

// The first position of the order in [ncoop, npairs) whose pair has fewer
// cells than the CTA threshold (the order is by la * lb, largest first),
// minus ncoop. A pair above the batch's cells per launched warp would, on
// one warp, outlast the others' share of the batch.
__device__ int nobt_count_long(const NobtArgs& A)
{
    if (!A.order || A.long_cells <= 0) return 0;
    long long thr = A.long_cells;
    if (A.total) {
        const long long per_warp =
            (long long)(*A.total / ((unsigned long long)gridDim.x * NOBT_WARPS));
        thr = per_warp > thr ? per_warp : thr;
    }
    int lo = A.ncoop, hi = A.npairs;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int k = A.order[mid];
        if ((long long)A.lena[k] * A.lenb[k] >= thr) lo = mid + 1;
        else hi = mid;
    }
    return lo - A.ncoop;
}

// Pairs ncoop .. npairs - 1 of the visiting order. The leading ones with at
// least long_cells cells go one per CTA, the CTA's warps splitting the
// column blocks (nobt_coop over the warps' own boundary columns), so that no
// single warp is left with a long pair at the end of the launch; the rest go
// NOBT_WARPS neighbours of the order per fetch, one per warp.
__global__ void __launch_bounds__(32 * NOBT_WARPS, 2) nobt_kernel(NobtArgs A)
{
    __shared__ Tables st;
    __shared__ int4 pfb[NOBT_WARPS][32];
    __shared__ uint8_t pfs[NOBT_WARPS][32];
    __shared__ int s_item, s_nlong, sres;
    __shared__ int2 tabs[16 * 32];
    if (threadIdx.x == 0) s_nlong = nobt_count_long(A);
    load_tables_smem(st, A.tables);
    const int2* tab = build_row_table(tabs, st);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int4* cols = A.bnd + (long long)blockIdx.x * NOBT_WARPS * A.bnd_stride;
    int4* bnd = cols + (long long)warp * A.bnd_stride;
    const int nlong = s_nlong;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(A.next, 1);
        __syncthreads();
        const int item = s_item;
        if (item < nlong) {
            NobtPair q = nobt_screen(A, st, A.order[A.ncoop + item], lane);
            if (q.run && q.lj > 2 && q.li >= NOBT_WARPS) {
                q.cost = nobt_coop<NOBT_K, NOBT_WARPS, true>(st, tab, q.si, q.li, q.sj, q.lj, cols,
                                                              A.bnd_stride, warp, lane, &sres);
            } else if (q.run && warp == 0) {
                if (q.lj <= 2) {
                    if (lane == 0) q.cost = nobt_tiny(st, q.si, q.li, q.sj, q.lj);
                    q.cost = __shfl_sync(FULL, q.cost, 0);
                } else {
                    q.cost = nobt_warp<NOBT_K>(st, tab, q.si, q.li, q.sj, q.lj, bnd, lane, pfb[0],
                                               pfs[0]);
                }
            }
            if (threadIdx.x == 0) {
                A.cost[q.k] = q.cost;
                A.status[q.k] = q.status;
            }
            continue;
        }
        const int w0 = A.ncoop + nlong + (item - nlong) * NOBT_WARPS;
        if (w0 >= A.npairs) break;
        const int w = w0 + warp;
        if (w >= A.npairs) continue;
        NobtPair q = nobt_screen(A, st, A.order ? A.order[w] : w, lane);
        if (q.run) {
            if (q.lj <= 2) {
                if (lane == 0) q.cost = nobt_tiny(st, q.si, q.li, q.sj, q.lj);
                q.cost = __shfl_sync(FULL, q.cost, 0);
            } else {
                q.cost = nobt_warp<NOBT_K>(st, tab, q.si, q.li, q.sj, q.lj, bnd, lane, pfb[warp],
                                           pfs[warp]);
            }
        }
        if (lane == 0) {
            A.cost[q.k] = q.cost;
            A.status[q.k] = q.status;
        }
    }
}

// Pairs 0 .. ncoop - 1 of the visiting order (the longest), one CTA each:
// lower latency for small batches of long pairs.
__global__ void __launch_bounds__(32 * COOP_WARPS) nobt_coop_kernel(NobtArgs A)
{
    __shared__ Tables st;
    __shared__ int sw, sres;
    __shared__ int4 pfb[32];
    __shared__ uint8_t pfs[32];
    __shared__ int2 tabs[16 * 32];
    load_tables_smem(st, A.tables);
    const int2* tab = build_row_table(tabs, st);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int4* cols = A.coop_cols + (long long)blockIdx.x * A.coop_stride;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) sw = atomicAdd(A.next_coop, 1);
        __syncthreads();
        const int w = sw;
        if (w >= A.ncoop) break;
        NobtPair q = nobt_screen(A, st, A.order ? A.order[w] : w, lane);
        const int nblk = (q.lj + 32 * COOP_K - 1) / (32 * COOP_K);
        if (q.run && q.lj > 2 && q.li >= COOP_WARPS &&
            (long long)nblk * A.bnd_stride <= A.coop_stride) {
            q.cost = nobt_coop<COOP_K, COOP_WARPS>(st, tab, q.si, q.li, q.sj, q.lj, cols,
                                                    A.bnd_stride, warp, lane, &sres);
        } else if (q.run && warp == 0) {  // short or narrow pairs: warp 0 alone
            if (q.lj <= 2) {
                if (lane == 0) q.cost = nobt_tiny(st, q.si, q.li, q.sj, q.lj);
                q.cost = __shfl_sync(FULL, q.cost, 0);
            } else {
                q.cost = nobt_warp<COOP_K>(st, tab, q.si, q.li, q.sj, q.lj, cols, lane, pfb, pfs);
            }
        }
        if (threadIdx.x == 0) {
            A.cost[q.k] = q.cost;
            A.status[q.k] = q.status;
        }
    }
}

}  // namespace

int nobt_warps_per_cta() { return NOBT_WARPS; }

int nobt_blocks_per_sm()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, nobt_kernel, 32 * NOBT_WARPS, 0);
    return n;
}

int nobt_coop_columns(int maxlen) { return (maxlen + 32 * COOP_K - 1) / (32 * COOP_K); }

void launch_nobt(const NobtArgs& a, int grid, int coop_grid, cudaStream_t s)
{
    if (a.ncoop > 0) nobt_coop_kernel<<<coop_grid, 32 * COOP_WARPS, 0, s>>>(a);
    if (a.ncoop < a.npairs) {
        if (a.total) nobt_total_kernel<<<(a.npairs + 255) / 256, 256, 0, s>>>(a);
        nobt_kernel<<<grid, 32 * NOBT_WARPS, 0, s>>>(a);
    }
}

}  // namespace pa
