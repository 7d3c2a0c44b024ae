// Algn_Newkk (src/newkkonen.c), affine cost model: POY's own Ukkonen-style
// banded aligner behind Sequence.NewkkAlign.align_2 (src/sequence.ml:
// 1831-1901). Host/device code shared by the kernel (pa_newkk.cu) and its
// host replay: the cell rule, the first row, the traceback and the median
// of the aligned pair.
//
// The reference grows the band in place and re-evaluates only the cells
// whose neighbours changed (update_a_row, src/newkkonen.c:964-1074). A cell
// is a function of its left, upper and diagonal neighbours and of the band
// borders alone, so each pass here fills its band afresh with the same
// values.
#pragma once
#include <stdint.h>

#include "pa_core.cuh"

namespace pa {
namespace nk {

constexpr int INF = 0x7fffffff / 2;  // INT_MAX/2, the reference's sentinel
// direction flags, src/newkkonen.c:44-61
constexpr int START = 0, ALIGN = 1, DEL = 16, INS = 32, END_INS = 64, END_DEL = 128,
              END_DIAG = 256, DIAG = 512, INS_EQ_DEL = 1024;
constexpr int GAP = 16, NOGAP = 15;  // GAPCODE / NOGAP, src/newkkonen.c:37-41
constexpr int MUCH_LONGER = 100;     // src/newkkonen.c:34
constexpr int MAX_PASSES = 40;       // band doublings before a pair is failed

// The values a cell passes to its neighbours: the four affine states and the
// two gap counters (gapnumarr1 | gapnumarr2 << 16).
struct State {
    int P, Q, ED, CD;
    uint32_t g;
};

PA_HD int add(int a, int b)  // my_add, src/newkkonen.c:65-71
{
    return a >= INF ? INF : b >= INF ? INF : a + b;
}
PA_HD int go_of(int base, int prev, int idx, int go)  // get_go, :179-184
{
    if (idx == 1 && (base & GAP)) return 0;
    if (idx > 1 && !(prev & GAP) && (base & GAP)) return 0;
    return go;
}
PA_HD int extgo_of(int base, int prev, int go)  // get_extgo, :194-198
{
    return ((prev & GAP) && !(base & GAP)) ? go : 0;
}

// update_internal_cell + assign_best_cost_and_direction (src/newkkonen.c:
// 600-873) for cell (i, j); b1 = s1[i], p1 = s1[i-1], b2 = s2[j], p2 =
// s2[j-1]. lb / rb: the cell lies on the band's left (i - j == k) / right
// (j - i == lenY - lenX + k) border. L, U, D: cells (i, j-1), (i-1, j),
// (i-1, j-1), read only where the reference reads them. Returns the cost;
// dir receives the direction flags.
PA_HD int cell(const Tables& t, int b1, int p1, int b2, int p2, int i, int j, bool lb, bool rb,
               const State& L, const State& U, const State& D, int go, State& o, int& dir)
{
    const int gap = t.gap;
    const int go1 = go_of(b1, p1, i, go), go2 = go_of(b2, p2, j, go);
    int P = INF, Q = INF, ED = INF, CD = INF;
    int costL = INF, extL = INF, openL = INF;
    uint32_t gL = 0;
    if (!lb && j != 0) {
        const int a = tcost(t, b2, gap);
        extL = add(L.Q, a + extgo_of(b2, p2, go));
        openL = add(L.CD, a + go2);
        costL = Q = tmin(openL, extL);
        gL = L.g;
    }
    int costR = INF, extR = INF, openR = INF;
    uint32_t gR = 0;
    if (!rb && i != 0) {
        const int a = tcost(t, b1, gap);
        extR = add(U.P, a + extgo_of(b1, p1, go));
        openR = add(U.CD, a + go1);
        costR = P = tmin(openR, extR);
        gR = U.g;
    }
    int costM = INF, costD = INF, extD = INF, openD = INF;
    uint32_t gM = 0;
    if (i != 0 && j != 0) {
        const int n1 = b1 & NOGAP, n2 = b2 & NOGAP;
        const int a = tcost(t, n1, n2);
        CD = add(D.CD, a);
        CD = tmin(CD, D.P + tcost(t, n1, b2) + (n1 == b1 ? 0 : go));
        CD = tmin(CD, D.Q + tcost(t, b1, n2) + (n2 == b2 ? 0 : go));
        CD = tmin(CD, add(D.ED, go1 + go2 + a));
        openD = add(D.CD, go1 + go2);
        extD = add(D.ED, ((b1 & GAP) && (b2 & GAP)) ? 0 : INF);
        ED = tmin(extD, openD);
        costM = CD;
        costD = ED;
        gM = D.g;
    }
    int d = INS, best = costL;
    int g1 = (int)(gL & 0xffff) + 1, g2 = (int)(gL >> 16);
    if (costR <= best) {
        if (costR < best) {
            best = costR;
            d = DEL;
            g1 = (int)(gR & 0xffff);
            g2 = (int)(gR >> 16) + 1;
        } else {
            d |= DEL;
            g1 = tmax(g1, (int)(gR & 0xffff));
            g2 = tmax(g2, (int)(gR >> 16) + 1);
        }
    }
    const int m1 = (int)(gM & 0xffff), m2 = (int)(gM >> 16);
    if (costM <= best) {
        if (costM < best) {
            best = costM;
            d = ALIGN;
            g1 = m1;
            g2 = m2;
        } else {
            d |= ALIGN;
            g1 = tmax(g1, m1);
            g2 = tmax(g2, m2);
        }
    }
    if (costD <= best) {
        if (costD < best) {
            best = costD;
            d = DIAG;
            g1 = m1;
            g2 = m2;
        } else {
            d |= DIAG;
            g1 = tmax(g1, m1);
            g2 = tmax(g2, m2);
        }
    }
    if (extR >= openR) d |= END_DEL;
    if (extL >= openL) d |= END_INS;
    if (extD >= openD) d |= END_DIAG;
    if (extR == extL && extR == best) d |= INS_EQ_DEL;
    dir = d;
    o.P = P;
    o.Q = Q;
    o.ED = ED;
    o.CD = CD;
    o.g = (uint32_t)(g1 & 0xffff) | ((uint32_t)(g2 & 0xffff) << 16);
    return best;
}

// Cell (0, 0) and the first-row cells (0, 1 .. lenY-lenX) that newkk_algn
// sets before the passes (src/newkkonen.c:1380-1428). lcost: the cost of
// (0, j-1).
PA_HD int first_row(const Tables& t, int b2, int p2, int j, int lcost, const State& L, int go,
                    State& o, int& dir)
{
    if (j == 0) {
        o.P = o.Q = go;
        o.ED = INF;
        o.CD = 0;
        o.g = 0;
        dir = START;
        return 0;
    }
    const int gap = t.gap;
    const int a = tcost(t, b2, gap);
    const int flag = gap & p2, flag2 = gap & b2;
    const int gocost = (j == 1) ? (flag2 ? 0 : go) : ((!flag && flag2) ? 0 : go);
    const int ext = L.Q + a + ((flag && !flag2) ? go : 0);
    const int open = lcost + a + gocost;
    const int c = tmin(open, ext);
    o.P = o.ED = o.CD = INF;
    o.Q = c;
    o.g = (((L.g & 0xffff) + 1) & 0xffff) | (L.g & 0xffff0000u);
    dir = INS | END_INS | END_DEL | END_DIAG;
    return c;
}

// Band geometry of a pass at half-width k: row i holds columns js(i) ..
// je(i). The warp fills a pass on a rolling schedule: lane r takes rows r,
// r + 32, r + 64, ... (round q holds rows 32q .. 32q + 31), and cell (i, j)
// is computed at step j + C(i), C(32q + r) = C0(q) + r. Within a round,
// lane r is one column behind lane r - 1, so the cells above and above-left
// are lane r - 1's last two cells. Round q + 1 starts Delta(q) steps after
// round q: late enough for each lane to have finished its row, and at least
// 32 so that lane 0 trails lane 31's row (handed over through the boundary
// row). The direction codes of step t are 32 consecutive u16 words, lane
// r's at word 32t + r.
struct Band {
    int X, Y, k;
    PA_HDM int d() const { return Y - X; }
    PA_HDM int js(int i) const { return tmax(0, i - k); }
    PA_HDM int je(int i) const { return tmin(Y - 1, i + (Y - X) + k); }
    PA_HDM int rounds() const { return (X + 31) >> 5; }
    PA_HDM bool in_band(int i, int j) const
    {
        return i >= 0 && j >= 0 && i < X && j < Y && i - j <= k && j - i <= (Y - X) + k;
    }
    // Delta(q) = max(32, 1 + max over lanes r of je(32q + r) - js(32q + 32 + r))
    PA_HDM int delta(int q) const
    {
        int dl = 32;
        for (int r = 0; r < 32 && 32 * q + 32 + r < X; r++)
            dl = tmax(dl, je(32 * q + r) - js(32 * q + 32 + r) + 1);
        return dl;
    }
    // steps of a pass whose last round starts at c0last
    PA_HDM long long steps(int c0last) const
    {
        const int q = rounds() - 1;
        return (long long)c0last + (X - 1 - 32 * q) + (Y - 1) + 1;
    }
};

// C0 of every round of a pass, sequentially (the kernel builds the same
// table with a warp scan); returns the steps of the pass.
PA_HD long long rounds_table(const Band& b, int* c0)
{
    int c = 0;
    for (int q = 0; q < b.rounds(); q++) {
        c0[q] = c;
        c += b.delta(q);
    }
    return b.steps(c0[b.rounds() - 1]);
}

// One column of a round's last row (the states lane 31 leaves for lane 0
// of the next round); the gap counters travel in a separate u32 array.
struct alignas(16) Quad {
    int P, Q, ED, CD;
};

// A lane's registers during a pass: its current row i (C(i), its columns,
// s1[i], s1[i-1]), its last cell (left), the cells above and above-left of
// its next one, what lane r - 1 produced last step (nu), and the cost of
// its last cell.
struct Lane {
    State left, up, diag, nu;
    int lcost;
    int i, C, js, je, b1, p1;
};

PA_HD void lane_row(Lane& L, const Band& b, const uint8_t* s1, int i, int C)
{
    L.i = i;
    L.C = C;
    if (i < b.X) {
        L.js = b.js(i);
        L.je = b.je(i);
        L.b1 = s1[i];
        L.p1 = i > 0 ? s1[i - 1] : 0;
    } else {  // no row: the lane idles
        L.js = 1;
        L.je = 0;
        L.b1 = L.p1 = 0;
    }
}

PA_HD void lane_start(Lane& L, const Band& b, const uint8_t* s1, int lane)
{
    const State z = {0, 0, 0, 0, 0u};
    L.left = L.up = L.diag = L.nu = z;
    L.lcost = 0;
    lane_row(L, b, s1, lane, lane);
}

// Step `step` of a pass for lane `lane`: moves the lane to its next row
// when its row has ended (c0: the rounds table), takes the inputs (lane 0
// reads the previous round's last row from the boundary row, the others
// take lane - 1's last cells) and computes the cell. Returns its direction
// code with its column in jout, or -1 when the lane idles this step (its
// registers are then never read by a neighbour).
PA_HD int lane_step(Lane& L, const Tables& t, const uint8_t* s1, const uint8_t* s2,
                    const Band& b, const int* c0, int lane, long long step, const Quad* bnd,
                    const uint32_t* bndg, int go, int& jout)
{
    int j = (int)(step - L.C);
    if (j > L.je && L.i + 32 < b.X) {
        const int q = (L.i >> 5) + 1;
        lane_row(L, b, s1, L.i + 32, c0[q] + lane);
        j = (int)(step - L.C);
    }
    const bool valid = L.i < b.X && j >= L.js && j <= L.je;
    if (lane == 0) {
        if (valid && L.i > 0) {
            if (j == L.js) {
                if (j > 0) {
                    const Quad v = bnd[j - 1];
                    L.diag = {v.P, v.Q, v.ED, v.CD, bndg[j - 1]};
                }
            } else {
                L.diag = L.up;
            }
            const Quad v = bnd[j];
            L.up = {v.P, v.Q, v.ED, v.CD, bndg[j]};
        }
    } else {
        L.diag = L.up;
        L.up = L.nu;
    }
    if (!valid) return -1;
    const int i = L.i, d = b.d();
    const int b2 = s2[j], p2 = j > 0 ? s2[j - 1] : 0;
    State o;
    int dir;
    if (i == 0 && j <= d)
        L.lcost = first_row(t, b2, p2, j, L.lcost, L.left, go, o, dir);
    else
        L.lcost = cell(t, L.b1, L.p1, b2, p2, i, j, i - j == b.k, j - i == d + b.k, L.left, L.up,
                       L.diag, go, o, dir);
    L.left = o;
    jout = j;
    return dir;
}

// Word of cell (i, j) in its pass's direction codes.
PA_HD long long dir_word(const int* c0, int i, int j)
{
    const int r = i & 31;
    return ((long long)j + c0[i >> 5] + r) * 32 + r;
}

// trivial_algn (src/newkkonen.c:1334-1357)
PA_HD int trivial_cost(const Tables& t, const uint8_t* s1, int l1, const uint8_t* s2, int l2)
{
    int r = 0;
    for (int i = 0; i < l1; i++) r += tcost(t, s1[i] & NOGAP, t.gap);
    for (int j = 0; j < l2; j++) r += tcost(t, s2[j] & NOGAP, t.gap);
    return r;
}

// newkk_algn's pass loop (src/newkkonen.c:1155-1172, 1434-1436): T starts at
// (lenY - lenX + 1) * min_non0_cost; each pass runs at k = min(p, lenX - 1),
// p = (T - (lenY - lenX)) / 2, and the loop stops when p exceeds the larger
// gap counter of the last cell or (2T - (lenY - lenX)) / 2 >= lenY - 1;
// otherwise T doubles. fill(k, cost, g) runs one pass and returns false when
// it could not (status set by the caller). A pass at the k of the previous
// one is not rerun: it would repeat it. Returns the cost; k receives the
// last pass's half-width.
template <class FILL>
PA_HD int drive(const Tables& t, int l1, int l2, FILL& fill, int& k, int& npass, int& status,
                bool skip = true)
{
    const int d = l2 - l1;
    long long T = (long long)(d + 1) * t.mnz;
    int prevk = -1, cost = 0;
    uint32_t g = 0;
    npass = 0;
    // Passes that cannot end the loop are counted as run without a fill (skip;
    // off only in tests, to check the bound on every pass): the
    // gap counters are maxima over tied predecessors of path counts, so the
    // last cell's larger one is at least d, and p <= d cannot exceed it. A
    // skipped pass has k = p below lenX - 1 (k rises, every one would fill),
    // no cover, and the fill of each pass is a function of its k alone.
    while (skip && npass < MAX_PASSES - 1 && T > 0) {
        const int p = (int)((T - d) / 2);
        const long long newp = (T * 2 - d) / 2;
        if (p >= l1 - 1 || T >= 3LL * d + 2 || newp - l2 + 1 >= 0) break;
        prevk = p;
        npass++;
        T *= 2;
    }
    for (;;) {
        const int p = (int)((T - d) / 2);
        k = p < l1 - 1 ? p : l1 - 1;
        if (k < 0) {  // no positive cost in the matrix: T would not grow
            status = -8;
            return 0;
        }
        if (k != prevk) {
            if (!fill(k, cost, g)) return 0;
            npass++;
            prevk = k;
        }
        const int gn = tmax((int)(g & 0xffff), (int)(g >> 16));
        const long long newp = (T * 2 - d) / 2;
        if (p > gn || newp - l2 + 1 >= 0) return cost;
        if (npass >= MAX_PASSES) {
            status = -8;
            return cost;
        }
        T *= 2;
    }
}

// backtrace_affine (src/newkkonen.c:1666-1766; trivial_backtrace :1498-1520
// when `trivial`) on s1 (the shorter) and s2, then DOS.median's use_ukk
// tail (src/seqCS.ml:1043-1051): ancestor_2, median_2_with_gaps and
// max_cost_2 on the aligned pair in caller order (s1 is b when swaped).
// dir(i, j) returns the direction flags of the last pass at band
// half-width k. Every output ends at the last byte of its slot (cap).
template <class DIR>
PA_HD PairRes traceback(const Tables& t, const DIR& dir, bool trivial, int k, const uint8_t* s1,
                        int l1, const uint8_t* s2, int l2, int swaped, const PairOut& o)
{
    PairRes r = {0, 0, 0, 0, 0};
    uint8_t* r1 = swaped ? o.eb : o.ea;
    uint8_t* r2 = swaped ? o.ea : o.eb;
    const int gap = t.gap;
    int kr = o.cap;
#define NK_PUT(a, b)                            \
    do {                                        \
        if (kr <= 0) {                          \
            r.status = -2;                      \
            return r;                           \
        }                                       \
        kr--;                                   \
        r1[kr] = (uint8_t)(a);                  \
        r2[kr] = (uint8_t)(b);                  \
    } while (0)
    if (trivial) {
        for (int i = 0; i < l1; i++) NK_PUT(s1[i], gap);
        for (int j = 0; j < l2; j++) NK_PUT(gap, s2[j]);
    } else {
        const Band b{l1, l2, k};
        int mode = 0;  // 0 todo, 1 delete, 2 insert, 3 diagonal, 4 align
        int i = l1 - 1, j = l2 - 1;
        while (i >= 0 && j >= 0) {
            if (!b.in_band(i, j)) {  // the reference would read outside the band
                r.status = -13;
                return r;
            }
            const int d = dir(i, j);
            if (d == START) {
                if (i != 0 || j != 0) {
                    r.status = -13;
                    return r;
                }
                NK_PUT(gap, gap);
                i--;
                j--;
            } else if (mode == 0) {  // copy_dir_to_mode, :1645-1663
                const int ins = d & INS, del = d & DEL;
                mode = swaped ? (ins ? 2 : del ? 1 : 0) : (del ? 1 : ins ? 2 : 0);
                if (!mode) mode = (d & DIAG) ? 3 : (d & ALIGN) ? 4 : 0;
                if (!mode) {
                    r.status = -13;
                    return r;
                }
            } else if (mode == 1) {
                NK_PUT(s1[i], gap);
                i--;
                if ((d & END_DEL) || (d & INS_EQ_DEL)) mode = 0;
            } else if (mode == 2) {
                NK_PUT(gap, s2[j]);
                j--;
                if ((d & END_INS) || (d & INS_EQ_DEL)) mode = 0;
            } else if (mode == 3) {
                if (d & END_DIAG) mode = 0;
                NK_PUT(s1[i], s2[j]);
                i--;
                j--;
            } else {
                NK_PUT(s1[i] & NOGAP, s2[j] & NOGAP);
                i--;
                j--;
                mode = 0;
            }
        }
    }
#undef NK_PUT
    const int L = o.cap - kr;
    r.alen = L;
    const uint8_t* ea = o.ea + kr;
    const uint8_t* eb = o.eb + kr;
    int nga = 0, ngb = 0;
    for (int i = 0; i < L; i++) {
        const int m = t.median[(ea[i] << t.lcm) + eb[i]];
        if (m == 0) r.status = -3;  // "median should not be 0", src/algn.c:3619
        o.mwg[kr + i] = (uint8_t)m;
        nga |= ea[i] != gap;
        ngb |= eb[i] != gap;
    }
    r.wlen = L;
    if (L + 1 > o.cap) {
        r.status = -2;
        return r;
    }
    const int n = ancestor_2(t, ea, eb, L, o.med);
    for (int i = n - 1; i >= 0; i--) o.med[o.cap - n + i] = o.med[i];
    r.mlen = n;
    r.maxcost = (nga && ngb) ? worst_aligned(t, ea, eb, L) : 0;
    return r;
}

}  // namespace nk
}  // namespace pa
