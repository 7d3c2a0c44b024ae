// Powell's three-sequence alignment (POY's Sequence.Align.align_3_powell ->
// powell_3D_align, src/ukkCommon.c:109-145, src/ukk.checkp.c) as a resumable
// machine that one GPU thread runs per triple.
//
// The reference recursion is a memoised Ukkonen search over diagonals
// (ab = i - j, ac = i - k), edit cost d and 16 column states, with a
// check-point divide and conquer for the alignment. Its results depend on the
// order of evaluation: the memo keeps cost d in slot d mod 2*maxSingleStep,
// a cell whose slot was reused is recomputed, and `from` records are read
// from slots without a stamp check. So the machine replays the recursion call
// for call: an explicit stack of frames stands in for Ukk / calcUkk
// (src/ukk.checkp.c:576-782) and a second stack for the check-point passes
// (src/ukk.checkp.c:214-365), both in the triple's own workspace.
//
// Storage: a window of diagonals |ab|, |ac| <= D (clipped to the sequences)
// holds every cell a call can touch: a pass starting at cost c0 on diagonal
// (ab0, ac0) only computes cells with |ab - ab0| + ... bounded by
// (d - c0) / ge (withinMatrix, src/ukk.checkp.c:543-573), so with D >=
// finalCost / ge the first pass and every later pass stay inside. The host
// picks D per triple; a cell outside the window, a stack overflow or a step
// budget running out ends the triple with a status the host retries with a
// wider window. Layout per triple: U cells [2*maxstep][wab][wac][16] of 16
// bytes, check-point distances [maxstep][wab][wac][16], the frame stack and
// the pass stack.
#pragma once

#include <stdint.h>

#include "pa_core.cuh"

namespace pa {
namespace u3 {

constexpr int INF = 5000;      // INFINITY = MAXINT / 2 with MAXINT 10000
constexpr int NS = 16;         // states with a match and at most one insert
constexpr int SUB_CAP = 96;    // pending check-point passes
constexpr int MAXLEN = 32767;  // diagonals packed as int16 in `from`

enum Status : int {
    OK = 0,
    ERR_WINDOW = 1,  // a cell fell outside the window
    ERR_STACK = 2,   // frame or pass stack full
    ERR_STEPS = 3,   // step budget spent
    ERR_BASE = 4,    // a position with no A, C, G or T ("This is impossible!")
    ERR_LEN = 5,     // a sequence longer than MAXLEN or shorter than 1
    ERR_STAMP = 6,   // cost offsets past int32
    ERR_OUT = 7,     // output longer than its capacity
};

// Column-state model (src/ukkCommon.c:244-338): neighbour step bits, the cost
// of continuing a state, whether a second (mismatch) predecessor is tried,
// and the transition costs.
struct Model {
    int mm, go, ge, maxstep;
    int8_t neigh[NS], second[NS];
    int16_t cont[NS];
    int16_t trans[NS][NS];
};

PA_HDM void model_init(Model& m, int mm, int go, int ge)
{
    auto digit = [](int s, int i) { return i == 0 ? s % 3 : i == 1 ? (s / 3) % 3 : (s / 9) % 3; };
    auto count = [&](int s, int t) {
        int n = 0;
        for (int i = 0; i < 3; i++) n += digit(s, i) == t;
        return n;
    };
    // 0 = match, 1 = delete (gap in this sequence), 2 = insert (only this one advances)
    int code[NS];
    int ns = 0;
    for (int s = 0; s < 27 && ns < NS; s++) {
        if (count(s, 0) == 0 || count(s, 2) > 1) continue;
        code[ns] = s;
        const int want = count(s, 2) ? 2 : 0;
        int nb = 0;
        for (int i = 0; i < 3; i++)
            if (digit(s, i) == want) nb |= 1 << i;
        m.neigh[ns] = (int8_t)nb;
        if (count(s, 2)) {
            m.cont[ns] = (int16_t)ge, m.second[ns] = 0;
        } else if (count(s, 0) == 3) {
            m.cont[ns] = (int16_t)mm, m.second[ns] = 1;
        } else if (count(s, 1) == 1) {
            m.cont[ns] = (int16_t)ge, m.second[ns] = 1;
        } else {
            m.cont[ns] = (int16_t)(2 * ge), m.second[ns] = 0;
        }
        ns++;
    }
    int mx = 0;
    for (int f = 0; f < NS; f++)
        for (int t = 0; t < NS; t++) {
            int c = 0;
            for (int i = 0; i < 3; i++) {
                const int to = digit(code[t], i);
                if (to != 0 && to != digit(code[f], i)) c += go;
            }
            m.trans[f][t] = (int16_t)c;
            const int step = c + m.cont[t] + mm * (count(code[t], 0) - 1);
            mx = step > mx ? step : mx;
        }
    m.mm = mm, m.go = go, m.ge = ge, m.maxstep = mx;
}

struct Cell {
    int dist, stamp;
    int abac;   // from: (uint16)ab | (uint16)ac << 16
    int cs;     // from: cost * 32 + state (cost -1 for "no check point")
};

struct Frame {
    int ab, ac, d;
    int meta;   // to | phase << 5 | k << 8 | (fst + 1) << 13
    int best, fabac, fcs, ext;
};

struct Pass {
    int sab, sac, scost, sst, sdist, fab, fac, fcost, fst, fdist;
};

struct Work {
    Cell* U;
    int* CP;
    Frame* st;
    Pass* sub;
    int st_cap;
    int ab_lo, ac_lo, wab, wac;
    long long step_cap;
};

// A triple's workspace for window half-width D (la, lb, lc: sequence
// lengths without the leading gap). The frame stack holds 2 (C + 1) + 1
// frames for a final cost C (each frame's callee has a lower cost, or the
// same cost and a state other than 0 when the caller's is 0); C is at most
// maxstep per column and there are at most la + lb + lc columns.
struct Layout {
    int ab_lo, ac_lo, wab, wac, st_cap;
    long long u_off, cp_off, st_off, sub_off, bytes, step_cap;
};

PA_HDM Layout layout(const Model& m, int la, int lb, int lc, int D)
{
    Layout L;
    L.ab_lo = -(D < lb ? D : lb);
    L.ac_lo = -(D < lc ? D : lc);
    L.wab = (D < la ? D : la) - L.ab_lo + 1;
    L.wac = (D < la ? D : la) - L.ac_lo + 1;
    const long long ub = (long long)m.maxstep * (la + lb + lc + 1);
    L.st_cap = (int)(2 * ub + 8);
    const long long cells = (long long)L.wab * L.wac * NS;
    auto up16 = [](long long v) { return (v + 15) & ~15LL; };
    L.u_off = 0;
    L.cp_off = up16(cells * 2 * m.maxstep * (long long)sizeof(Cell));
    L.st_off = L.cp_off + up16(cells * m.maxstep * 4LL);
    L.sub_off = L.st_off + up16((long long)L.st_cap * sizeof(Frame));
    L.bytes = L.sub_off + up16((long long)SUB_CAP * sizeof(Pass));
    // a runaway guard only: far above the steps of any legitimate replay
    const double cap = 64.0 * (double)cells * (double)(ub + 1) * 2.0;
    L.step_cap = cap > 4.0e18 ? (long long)4.0e18 : (long long)cap;
    return L;
}

PA_HDM Work work_at(unsigned char* base, const Layout& L)
{
    Work w;
    w.U = (Cell*)(base + L.u_off);
    w.CP = (int*)(base + L.cp_off);
    w.st = (Frame*)(base + L.st_off);
    w.sub = (Pass*)(base + L.sub_off);
    w.st_cap = L.st_cap;
    w.ab_lo = L.ab_lo, w.ac_lo = L.ac_lo, w.wab = L.wab, w.wac = L.wac;
    w.step_cap = L.step_cap;
    return w;
}

// initial window half-width: the length spread plus a margin for the
// edit distance; a triple that leaves it is rerun with twice the width
PA_HDM int first_window(int la, int lb, int lc)
{
    auto ab = [](int x) { return x < 0 ? -x : x; };
    int spread = ab(la - lb);
    spread = ab(la - lc) > spread ? ab(la - lc) : spread;
    spread = ab(lb - lc) > spread ? ab(lb - lc) : spread;
    int mx = la > lb ? la : lb;
    mx = lc > mx ? lc : mx;
    return 16 + spread + mx / 16;
}

// the half-width at which the window covers every diagonal
PA_HDM int full_window(int la, int lb, int lc)
{
    int mx = la > lb ? la : lb;
    return lc > mx ? lc : mx;
}

PA_HD int pack_abac(int ab, int ac) { return (int)((uint32_t)(uint16_t)ab | ((uint32_t)(uint16_t)ac << 16)); }
PA_HD int unpack_ab(int v) { return (int)(int16_t)(v & 0xffff); }
PA_HD int unpack_ac(int v) { return (int)(int16_t)((uint32_t)v >> 16); }
PA_HD int iabs3(int v) { return v < 0 ? -v : v; }

// base of position i (0-based, after the leading gap): the lowest of A, C, G,
// T, as copySequence keeps it (src/ukkCommon.c:85-104)
PA_HD int base_at(const uint8_t* s, int i)
{
    const int v = s[i + 1] & 15;
    return v & -v;
}

PA_HD bool ok_index(int a, int da, int end) { return a >= 0 && (da ? a < end : a <= end); }

PA_HD int char_cost(int a, int b, int c)
{
    if (a == b && a == c) return 0;
    if (a == b || a == c || b == c) return 1;
    return 2;
}

enum Phase { PH_START = 0, PH_FS1 = 1, PH_FS2 = 2, PH_DM1 = 3, PH_EXT = 4 };

// One triple's replay. Sequences are POY sequences with the leading gap;
// output is written back to front so that it ends at out_end (the
// seq_prepend layout), leading gap included.
struct Machine {
    const Model& m;
    const Work& w;
    const uint8_t *A, *B, *C;
    int la, lb, lc;
    // globals of the reference recursion
    int off, final_cost, furthest, cp_cost, complete;
    int sab, sac, scost, sst, endA, endB, endC;
    long long steps;
    int status;
    int n;  // columns emitted

    PA_HDM Machine(const Model& m_, const Work& w_, const uint8_t* a, int la_, const uint8_t* b,
                   int lb_, const uint8_t* c, int lc_)
        : m(m_), w(w_), A(a), B(b), C(c), la(la_), lb(lb_), lc(lc_), off(1), final_cost(0),
          furthest(-1), cp_cost(INF), complete(0), sab(0), sac(0), scost(0), sst(0), endA(la_),
          endB(lb_), endC(lc_), steps(0), status(OK), n(0)
    {
    }

    PA_HDM int a_at(int i) const { return base_at(A, i); }
    PA_HDM int b_at(int i) const { return base_at(B, i); }
    PA_HDM int c_at(int i) const { return base_at(C, i); }

    PA_HDM bool in_window(int ab, int ac) const
    {
        return ab >= w.ab_lo && ab < w.ab_lo + w.wab && ac >= w.ac_lo && ac < w.ac_lo + w.wac;
    }
    PA_HDM long long slot(int ab, int ac, int plane, int s) const
    {
        return (((long long)plane * w.wab + (ab - w.ab_lo)) * w.wac + (ac - w.ac_lo)) * NS + s;
    }
    // U slot: caller has checked the window
    PA_HDM Cell* U(int ab, int ac, int d, int s) const
    {
        return w.U + slot(ab, ac, d % (2 * m.maxstep), s);
    }
    PA_HDM int* CP(int ab, int ac, int d, int s) const
    {
        return w.CP + slot(ab, ac, d % m.maxstep, s);
    }

    PA_HDM bool within(int ab, int ac, int d) const
    {
        if (d < 0) return false;
        int g = iabs3(sab - ab), h = iabs3(sac - ac), k = iabs3((sac - sab) - (ac - ab));
        // g, h = the two smallest
        if (h < g) { const int t = g; g = h; h = t; }
        if (k < h) h = k;
        if (h < g) { const int t = g; g = h; h = t; }
        const int cheapest = sst == 0 ? (g ? m.go + g * m.ge : 0) + (h ? m.go + h * m.ge : 0)
                                      : g * m.ge + h * m.ge;
        return cheapest + scost <= d;
    }

    PA_HDM void fail(int s)
    {
        if (status == OK) status = s;
    }

    // Ukk(ab, ac, d, s) (src/ukk.checkp.c:576-604) with the stack
    PA_HDM int ukk(int ab0, int ac0, int d0, int s0)
    {
        if (!within(ab0, ac0, d0)) return -INF;
        if (!in_window(ab0, ac0)) {
            fail(ERR_WINDOW);
            return -INF;
        }
        {
            const Cell* c = U(ab0, ac0, d0, s0);
            if (c->stamp == d0 + off) return c->dist;
        }
        int sp = 0;
        Frame* st = w.st;
        st[sp++] = Frame{ab0, ac0, d0, s0 | (PH_START << 5), 0, 0, 0, 0};
        int r = 0;
        while (sp > 0) {
            if (++steps > w.step_cap) {
                fail(ERR_STEPS);
                return -INF;
            }
            Frame& f = st[sp - 1];
            const int to = f.meta & 31;
            const int ph = (f.meta >> 5) & 7;
            int k = (f.meta >> 8) & 31;
            const int nb = m.neigh[to];
            const int da = nb & 1, db = (nb >> 1) & 1, dc = (nb >> 2) & 1;
            const int ab1 = f.ab - da + db, ac1 = f.ac - da + dc;
            const bool copy = f.d >= cp_cost + m.maxstep;
            // the callee of the next step: (cab, cac, cd, cs) with return phase nph
            int cab = 0, cac = 0, cd = 0, cst = 0, nph = -1;
            bool finish = false;
            switch (ph) {
            case PH_START: {
                f.best = -INF;
                if (f.d >= cp_cost && f.d < cp_cost + m.maxstep) {
                    f.fabac = pack_abac(f.ab, f.ac);
                    f.fcs = f.d * 32 + to;
                } else {
                    f.fabac = 0;
                    f.fcs = -32;
                }
                if (ab1 >= -endB && ab1 <= endA && ac1 >= -endC && ac1 <= endA) {
                    k = 0;
                    cab = ab1, cac = ac1, cd = f.d - m.trans[0][to] - m.cont[to], cst = 0;
                    nph = PH_FS1;
                } else {
                    cab = f.ab, cac = f.ac, cd = f.d - 1, cst = to, nph = PH_DM1;
                }
                break;
            }
            case PH_FS1:
            case PH_FS2: {
                const int cost = f.d - m.trans[k][to] - m.cont[to];
                const int a = r;
                int dist = -INF, fcost = 0;
                bool tried = true;
                if (ph == PH_FS1) {
                    if (ok_index(a, da, endA) && ok_index(a - ab1, db, endB) &&
                        ok_index(a - ac1, dc, endC) &&
                        char_cost(da ? a_at(a) : 16, db ? b_at(a - ab1) : 16,
                                  dc ? c_at(a - ac1) : 16) == 1) {
                        fcost = cost, dist = a + da;
                    } else if (m.second[to]) {
                        // try the mismatch predecessor next
                        cab = ab1, cac = ac1, cd = cost - m.mm, cst = k, nph = PH_FS2;
                        tried = false;
                    }
                } else if (ok_index(a, da, endA) && ok_index(a - ab1, db, endB) &&
                           ok_index(a - ac1, dc, endC)) {
                    fcost = cost - m.mm, dist = a + da;
                }
                if (!tried) break;
                if (f.best < dist) {
                    f.best = dist;
                    if (complete) {
                        f.fabac = pack_abac(ab1, ac1);
                        f.fcs = fcost * 32 + k;
                    } else if (copy) {
                        const Cell* c = U(ab1, ac1, fcost, k);
                        f.fabac = c->abac;
                        f.fcs = c->cs;
                    }
                }
                if (++k < NS) {
                    cab = ab1, cac = ac1, cd = f.d - m.trans[k][to] - m.cont[to], cst = k;
                    nph = PH_FS1;
                } else {
                    cab = f.ab, cac = f.ac, cd = f.d - 1, cst = to, nph = PH_DM1;
                }
                break;
            }
            case PH_DM1: {
                const int dist = r;
                if (ok_index(dist, 0, endA) && ok_index(dist - f.ab, 0, endB) &&
                    ok_index(dist - f.ac, 0, endC) && f.best < dist) {
                    f.best = dist;
                    if (complete) {
                        f.fabac = pack_abac(f.ab, f.ac);
                        f.fcs = (f.d - 1) * 32 + to;
                    } else if (copy) {
                        const Cell* c = U(f.ab, f.ac, f.d - 1, to);
                        f.fabac = c->abac;
                        f.fcs = c->cs;
                    }
                }
                if (to == 0) {
                    // furthest over the states at this cost, state 0 being
                    // the value just found (src/ukk.checkp.c:722-735)
                    if (f.best > -INF) {
                        f.ext = f.best;
                        f.meta = (f.meta & ~(31 << 13)) | (1 << 13);
                    } else {
                        f.ext = -INF;
                        f.meta &= ~(31 << 13);
                    }
                    k = 1;
                    cab = f.ab, cac = f.ac, cd = f.d, cst = 1, nph = PH_EXT;
                } else {
                    finish = true;
                }
                break;
            }
            case PH_EXT: {
                if (r > f.ext) {
                    f.ext = r;
                    f.meta = (f.meta & ~(31 << 13)) | ((k + 1) << 13);
                }
                if (++k < NS) {
                    cab = f.ab, cac = f.ac, cd = f.d, cst = k, nph = PH_EXT;
                } else {
                    int dist = f.ext;
                    const int fst = ((f.meta >> 13) & 31) - 1;
                    while (ok_index(dist, 1, endA) && ok_index(dist - f.ab, 1, endB) &&
                           ok_index(dist - f.ac, 1, endC) && a_at(dist) == b_at(dist - f.ab) &&
                           a_at(dist) == c_at(dist - f.ac))
                        dist++;
                    if (dist > f.best) {
                        f.best = dist;
                        if (fst != 0) {
                            if (complete) {
                                f.fabac = pack_abac(f.ab, f.ac);
                                f.fcs = f.d * 32 + fst;
                            } else if (copy) {
                                const Cell* c = U(f.ab, f.ac, f.d, fst);
                                f.fabac = c->abac;
                                f.fcs = c->cs;
                            }
                        }
                    }
                    finish = true;
                }
                break;
            }
            default:
                fail(ERR_STEPS);
                return -INF;
            }
            if (finish) {
                Cell* c = U(f.ab, f.ac, f.d, to);
                c->dist = f.best;
                c->stamp = f.d + off;
                c->abac = f.fabac;
                c->cs = f.fcs;
                if (f.d >= cp_cost && f.d < cp_cost + m.maxstep) *CP(f.ab, f.ac, f.d, to) = f.best;
                if (f.best > furthest) furthest = f.best;
                r = f.best;
                sp--;
                continue;
            }
            if (status != OK) return -INF;
            f.meta = (f.meta & ~((7 << 5) | (31 << 8))) | (nph << 5) | (k << 8);
            // the call: resolved here when outside the matrix or memoised
            if (!within(cab, cac, cd)) {
                r = -INF;
                continue;
            }
            if (!in_window(cab, cac)) {
                fail(ERR_WINDOW);
                return -INF;
            }
            const Cell* c = U(cab, cac, cd, cst);
            if (c->stamp == cd + off) {
                r = c->dist;
                continue;
            }
            if (sp >= w.st_cap) {
                fail(ERR_STACK);
                return -INF;
            }
            st[sp++] = Frame{cab, cac, cd, cst | (PH_START << 5), 0, 0, 0, 0};
        }
        return r;
    }

    // furthest distance (or its state) at (ab, ac, d) over the states
    PA_HDM int best_at(int ab, int ac, int d, bool want_state) const
    {
        int best = -INF, bs = -1;
        if (in_window(ab, ac))
            for (int s = 0; s < NS; s++) {
                const Cell* c = U(ab, ac, d, s);
                if (c->stamp == d + off && c->dist > best) best = c->dist, bs = s;
            }
        return want_state ? bs : best;
    }

    PA_HDM void emit(uint8_t* ea, uint8_t* eb, uint8_t* ec, int cap, int a, int b, int c)
    {
        if (n >= cap) {
            fail(ERR_OUT);
            return;
        }
        ea[-1 - n] = (uint8_t)a, eb[-1 - n] = (uint8_t)b, ec[-1 - n] = (uint8_t)c;
        n++;
    }

    // traceBack (src/ukk.checkp.c:368-443): columns back to front
    PA_HDM void traceback(const Pass& p, uint8_t* ea, uint8_t* eb, uint8_t* ec, int cap)
    {
        int ab = p.fab, ac = p.fac, d = p.fcost, s = p.fst;
        long long guard = 0;
        while ((ab != p.sab || ac != p.sac || d != p.scost || s != p.sst) && status == OK) {
            if (++guard > (long long)cap + 4) {
                fail(ERR_OUT);
                return;
            }
            if (!in_window(ab, ac) || d < 0) {
                fail(ERR_WINDOW);
                return;
            }
            const Cell* c = U(ab, ac, d, s);
            int a = c->dist;
            const int nab = unpack_ab(c->abac), nac = unpack_ac(c->abac);
            const int nd = c->cs >> 5, ns = c->cs & 31;
            if (!in_window(nab, nac) || nd < 0 || ns >= NS) {
                fail(ERR_WINDOW);
                return;
            }
            int b = a - ab, cc = a - ac;
            const int a1 = U(nab, nac, nd, ns)->dist;
            const int b1 = a1 - nab, c1 = a1 - nac;
            if (a1 < 0 || b1 < 0 || c1 < 0 || a > la || b > lb || cc > lc) {
                fail(ERR_OUT);
                return;
            }
            while (a > a1 && b > b1 && cc > c1) {
                a--, b--, cc--;
                emit(ea, eb, ec, cap, a_at(a), b_at(b), c_at(cc));
            }
            if (a != a1 || b != b1 || cc != c1) {
                int ca = 16, cb = 16, ccc = 16;
                if (a > a1) ca = a_at(--a);
                if (b > b1) cb = b_at(--b);
                if (cc > c1) ccc = c_at(--cc);
                emit(ea, eb, ec, cap, ca, cb, ccc);
            }
            ab = nab, ac = nac, d = nd, s = ns;
        }
    }

    // doUkk (src/ukk.checkp.c:111-212) with doUkkInLimits / getSplitRecurse
    // (:214-365) on the pass stack. ea/eb/ec point one past the end of the
    // outputs; returns the cost, *rlen the aligned length.
    PA_HDM int run(uint8_t* ea, uint8_t* eb, uint8_t* ec, int cap, int* rlen)
    {
        int start = 0;
        while (start < la && start < lb && start < lc && a_at(start) == b_at(start) &&
               a_at(start) == c_at(start))
            start++;
        if (!in_window(0, 0)) {
            fail(ERR_WINDOW);
            return -1;
        }
        {
            Cell* c0 = U(0, 0, 0, 0);
            c0->dist = start;
            c0->stamp = off;
        }
        const int fab = la - lb, fac = la - lc;
        bool cp_on_dist = true;
        // no alignment costs more than maxstep per column
        const long long ub = (long long)m.maxstep * (la + lb + lc + 1);
        int d = -1;
        do {
            d++;
            if (d > ub) {
                fail(ERR_STEPS);
                return -1;
            }
            ukk(fab, fac, d, 0);
            if (cp_on_dist && furthest >= la / 2) {
                cp_cost = d + 1;
                cp_on_dist = false;
            }
        } while (status == OK && best_at(fab, fac, d, false) < la);
        if (status != OK) return -1;
        final_cost = d;
        int nsub = 0;
        {
            const int fst = best_at(fab, fac, d, true);
            const Pass whole{0, 0, 0, 0, start, fab, fac, d, fst, la};
            if (U(fab, fac, d, fst)->cs >> 5 <= 0)
                w.sub[nsub++] = whole;
            else
                split(whole, nsub);
        }
        while (nsub > 0 && status == OK) {
            const Pass p = w.sub[--nsub];
            limits(p, nsub, ea, eb, ec, cap);
        }
        if (status != OK) return -1;
        // the leading run of matches, then the leading gap
        for (int i = start - 1; i >= 0; i--) emit(ea, eb, ec, cap, a_at(i), b_at(i), c_at(i));
        emit(ea, eb, ec, cap, 16, 16, 16);
        if (status != OK) return -1;
        *rlen = n;
        return d;
    }

    // getSplitRecurse: queue the two halves, second half on top
    PA_HDM void split(const Pass& p, int& nsub)
    {
        const Cell* c = U(p.fab, p.fac, p.fcost, p.fst);
        const int mab = unpack_ab(c->abac), mac = unpack_ac(c->abac);
        const int mcost = c->cs >> 5, mst = c->cs & 31;
        if (!in_window(mab, mac) || mcost < 0 || mst >= NS) {
            fail(ERR_WINDOW);
            return;
        }
        const int cpdist = *CP(mab, mac, mcost, mst);
        if (nsub + 2 > SUB_CAP) {
            fail(ERR_STACK);
            return;
        }
        w.sub[nsub++] = Pass{p.sab, p.sac, p.scost, p.sst, p.sdist, mab, mac, mcost, mst, cpdist};
        w.sub[nsub++] = Pass{mab, mac, mcost, mst, cpdist, p.fab, p.fac, p.fcost, p.fst, p.fdist};
    }

    // doUkkInLimits
    PA_HDM void limits(Pass p, int& nsub, uint8_t* ea, uint8_t* eb, uint8_t* ec, int cap)
    {
        sab = p.sab, sac = p.sac, scost = p.scost, sst = p.sst;
        endA = p.fdist, endB = p.fdist - p.fab, endC = p.fdist - p.fac;
        complete = 0;
        if ((long long)off + final_cost + 1 > 0x3fffffffLL) {
            fail(ERR_STAMP);
            return;
        }
        off += final_cost + 1;
        if (!in_window(p.sab, p.sac) || p.scost < 0 || p.sst < 0 || p.sst >= NS) {
            fail(ERR_WINDOW);
            return;
        }
        {
            Cell* c = U(p.sab, p.sac, p.scost, p.sst);
            c->dist = p.sdist;
            c->stamp = p.scost + off;
        }
        if (p.fcost - p.scost <= m.maxstep) {
            complete = 1;
            int i = p.scost - 1, dist;
            do {
                if (++i > final_cost) {
                    fail(ERR_STEPS);
                    return;
                }
                dist = ukk(p.fab, p.fac, i, p.fst);
            } while (dist < p.fdist && status == OK);
            if (status != OK) return;
            p.fcost = i;
            traceback(p, ea, eb, ec, cap);
            complete = 0;
            return;
        }
        cp_cost = (p.fcost + p.scost - m.maxstep + 1) / 2;
        int i = p.scost - 1, dist;
        do {
            if (++i > final_cost) {
                fail(ERR_STEPS);
                return;
            }
            ukk(p.fab, p.fac, i, 0);
            dist = ukk(p.fab, p.fac, i, p.fst);
        } while (dist < p.fdist && status == OK);
        if (status != OK) return;
        p.fcost = i;
        split(p, nsub);
    }
};

}  // namespace u3
}  // namespace pa
