// Powell's three-sequence alignment (POY's Sequence.Align.align_3_powell ->
// powell_3D_align, src/ukkCommon.c:109-145, src/ukk.checkp.c) as a resumable
// machine that one GPU warp runs per triple.
//
// The reference recursion is a memoised Ukkonen search over diagonals
// (ab = i - j, ac = i - k), edit cost d and 16 column states, with a
// check-point divide and conquer for the alignment. Its results depend on the
// order of evaluation: the memo keeps cost d in slot d mod 2*maxSingleStep,
// a cell whose slot was reused is recomputed, and `from` records are read
// from slots without a stamp check. So the machine replays the recursion call
// for call: an explicit stack of frames stands in for Ukk / calcUkk
// (src/ukk.checkp.c:576-782) and a second stack for the check-point passes
// (src/ukk.checkp.c:214-365), both in the triple's own workspace. Every lane
// of the warp holds the same machine state; the lanes read a frame's
// candidate cells together and judge one each.
//
// Storage: a window of diagonals |ab|, |ac| <= D (clipped to the sequences)
// holds every cell a call can touch: a pass starting at cost c0 on diagonal
// (ab0, ac0) only computes cells with |ab - ab0| + ... bounded by
// (d - c0) / ge (withinMatrix, src/ukk.checkp.c:543-573), so with D >=
// finalCost / ge the first pass and every later pass stay inside. The host
// picks D per triple; a cell outside the window, a stack overflow or a step
// budget running out ends the triple with a status the host retries with a
// wider window; a replay that passes TIME_LIMIT_NS of wall clock ends with a
// status of its own. Layout per triple: U cells [wab][wac][2*maxstep][16] of 16
// bytes, check-point distances [wab][wac][maxstep][16], the frame stack and
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
constexpr int MAXCOST = 10000;  // mm, go, ge: the state tables hold int16
// bound on a triple's alignment cost, maxstep (la + lb + lc + 1): costs are
// packed as cost * 32 + state in an int, and the frame stack holds twice it
constexpr long long MAX_COST_BOUND = 1LL << 26;

// the cost bound of a triple (la, lb, lc without the leading gap)
PA_HDM long long cost_bound(int maxstep, int la, int lb, int lc)
{
    return (long long)maxstep * ((long long)la + lb + lc + 1);
}

enum Status : int {
    OK = 0,
    ERR_WINDOW = 1,  // a cell fell outside the window
    ERR_STACK = 2,   // frame or pass stack full
    ERR_STEPS = 3,   // step budget spent
    ERR_BASE = 4,    // a position with no A, C, G or T ("This is impossible!")
    ERR_LEN = 5,     // a sequence longer than MAXLEN or shorter than 1
    ERR_STAMP = 6,   // cost offsets past int32
    ERR_OUT = 7,     // output longer than its capacity
    ERR_TIME = 8,    // the triple ran past TIME_LIMIT_NS (not retried)
};

// wall-clock bound of one triple's replay on the GPU: far above any triple
// of the workloads (about 2 s at most), it keeps a replay that went wrong
// from holding the device
constexpr unsigned long long TIME_LIMIT_NS = 120ull * 1000000000ull;

PA_HD unsigned long long now_ns()
{
#if defined(__CUDA_ARCH__)
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
#else
    return 0;  // the host replay has no time bound
#endif
}

// Column-state model (src/ukkCommon.c:244-338): neighbour step bits, the cost
// of continuing a state, whether a second (mismatch) predecessor is tried,
// and the transition costs.
struct Model {
    int mm, go, ge, maxstep;
    int8_t neigh[NS], second[NS];
    int16_t cont[NS];
    int16_t trans[NS][NS];  // [to][from]: a row per target state, read one entry per lane
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
            m.trans[t][f] = (int16_t)c;
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
    int meta;   // to | phase << 5 | k << 8 | sub << 13 | (fst + 1) << 14
    int best, fabac, fcs, ext;
    // fixed for the frame's life: the window index of its diagonal pair and
    // of the neighbour pair (-1 outside the window), both pairs' cost bound
    // from the pass start (withinMatrix), and the plane of d
    int diag0, diag1, ch0, ch1, pd;
};

struct Pass {
    int sab, sac, scost, sst, sdist, fab, fac, fcost, fst, fdist;
};

constexpr int RING = 32;  // frames of the stack top kept on chip

struct Work {
    Cell* U;
    int* CP;
    Frame* st;
    Pass* sub;
    Frame* ring;     // RING frames: slot j % RING holds frame j while ring_tag says so
    int* ring_tag;
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
    const long long ub = cost_bound(m.maxstep, la, lb, lc);  // <= MAX_COST_BOUND (host check)
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

// a window whose diagonal pairs are indexed in an int (diag_of)
PA_HDM bool window_fits(const Model& m, int la, int lb, int lc, int D)
{
    const Layout L = layout(m, la, lb, lc, D);
    return (long long)L.wab * L.wac < (1LL << 31);
}

PA_HDM Work work_at(unsigned char* base, const Layout& L)
{
    Work w;
    w.U = (Cell*)(base + L.u_off);
    w.CP = (int*)(base + L.cp_off);
    w.st = (Frame*)(base + L.st_off);
    w.sub = (Pass*)(base + L.sub_off);
    w.ring = nullptr;
    w.ring_tag = nullptr;
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

enum Phase { PH_FS = 0, PH_X = 1 };

// A frame's candidate cells, one per lane, loaded in one round: the tag is
// the memo value when the slot holds this cost, TAG_MISS when it must be
// computed, TAG_WINDOW when it lies outside the window and -INF outside the
// matrix; abac / cs are the slot's `from` record. Lanes take them from each
// other by index (a shuffle on the GPU; arrays when the machine runs on the
// host).
constexpr int TAG_MISS = -0x7fffffff;
constexpr int TAG_WINDOW = -0x7ffffffe;

struct Snap {
#if defined(__CUDA_ARCH__)
    int tag, abac, cs;
#else
    int tag[32], abac[32], cs[32];
#endif
};

PA_HD int tag_of(const Snap& S, int k)
{
#if defined(__CUDA_ARCH__)
    return __shfl_sync(0xffffffffu, S.tag, k);
#else
    return S.tag[k];
#endif
}
PA_HD int abac_of(const Snap& S, int k)
{
#if defined(__CUDA_ARCH__)
    return __shfl_sync(0xffffffffu, S.abac, k);
#else
    return S.abac[k];
#endif
}
PA_HD int cs_of(const Snap& S, int k)
{
#if defined(__CUDA_ARCH__)
    return __shfl_sync(0xffffffffu, S.cs, k);
#else
    return S.cs[k];
#endif
}

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
    unsigned long long t0;  // start of the replay (GPU global timer)
    int status;
    int n;  // columns emitted

    PA_HDM Machine(const Model& m_, const Work& w_, const uint8_t* a, int la_, const uint8_t* b,
                   int lb_, const uint8_t* c, int lc_)
        : m(m_), w(w_), A(a), B(b), C(c), la(la_), lb(lb_), lc(lc_), off(1), final_cost(0),
          furthest(-1), cp_cost(INF), complete(0), sab(0), sac(0), scost(0), sst(0), endA(la_),
          endB(lb_), endC(lc_), steps(0), status(OK), n(0)
    {
        t0 = now_ns();
    }

    PA_HDM int a_at(int i) const { return base_at(A, i); }
    PA_HDM int b_at(int i) const { return base_at(B, i); }
    PA_HDM int c_at(int i) const { return base_at(C, i); }

    PA_HDM bool in_window(int ab, int ac) const
    {
        return ab >= w.ab_lo && ab < w.ab_lo + w.wab && ac >= w.ac_lo && ac < w.ac_lo + w.wac;
    }
    // the planes of a diagonal pair are adjacent, so the cells a frame reads
    // (two diagonals, a few costs, 16 states) lie within a few kilobytes
    PA_HDM long long slot(int ab, int ac, int plane, int planes, int s) const
    {
        return ((((long long)(ab - w.ab_lo)) * w.wac + (ac - w.ac_lo)) * planes + plane) * NS + s;
    }
    // U slot: caller has checked the window
    PA_HDM Cell* U(int ab, int ac, int d, int s) const
    {
        return w.U + slot(ab, ac, d % (2 * m.maxstep), 2 * m.maxstep, s);
    }
    PA_HDM int* CP(int ab, int ac, int d, int s) const
    {
        return w.CP + slot(ab, ac, d % m.maxstep, m.maxstep, s);
    }

    // withinMatrix's lower bound on the cost of reaching (ab, ac) from the
    // pass's start (src/ukk.checkp.c:543-573)
    PA_HDM int cheapest(int ab, int ac) const
    {
        int g = iabs3(sab - ab), h = iabs3(sac - ac), k = iabs3((sac - sab) - (ac - ab));
        // g, h = the two smallest
        if (h < g) { const int t = g; g = h; h = t; }
        if (k < h) h = k;
        if (h < g) { const int t = g; g = h; h = t; }
        return sst == 0 ? (g ? m.go + g * m.ge : 0) + (h ? m.go + h * m.ge : 0)
                        : g * m.ge + h * m.ge;
    }
    PA_HDM bool within(int ab, int ac, int d) const
    {
        return d >= 0 && cheapest(ab, ac) + scost <= d;
    }
    PA_HDM int diag_of(int ab, int ac) const { return (ab - w.ab_lo) * w.wac + (ac - w.ac_lo); }
    // the plane of cost d - x from the plane of d (0 <= x < 2 maxstep)
    PA_HDM int plane_back(int pd, int x) const
    {
        const int p = pd - x;
        return p < 0 ? p + 2 * m.maxstep : p;
    }

    PA_HDM void fail(int s)
    {
        if (status == OK) status = s;
    }

    // one candidate on a diagonal pair of the frame (its window index diag,
    // -1 outside, and its cost bound ch): classify and load the slot of
    // cost d, plane pl, state s
    PA_HDM void load(int diag, int ch, int d, int pl, int s, int& tag, int& abac, int& cs) const
    {
        abac = 0, cs = 0;
        if (d < 0 || ch + scost > d) {
            tag = -INF;
            return;
        }
        if (diag < 0) {
            tag = TAG_WINDOW;
            return;
        }
        const Cell* c = w.U + ((long long)diag * (2 * m.maxstep) + pl) * NS + s;
#if defined(__CUDA_ARCH__)
        const int4 v = *reinterpret_cast<const int4*>(c);
        tag = v.y == d + off ? v.x : TAG_MISS;
        abac = v.z, cs = v.w;
#else
        tag = c->stamp == d + off ? c->dist : TAG_MISS;
        abac = c->abac, cs = c->cs;
#endif
    }

    // the predecessors on the neighbour diagonal: lanes 0-15 the cost of
    // state k's transition (k = lane), lanes 16-31 that cost less a mismatch
    PA_HDM void lane_fs(int l, const Frame& F, int to, int ab1, int ac1, int& tag, int& abac,
                        int& cs) const
    {
        const int k = l & 15;
        if (l >= 16 && !m.second[to]) {
            tag = -INF, abac = 0, cs = 0;
            return;
        }
        const int x = m.trans[to][k] + m.cont[to] + (l >= 16 ? m.mm : 0);
        load(F.diag1, F.ch1, F.d - x, plane_back(F.pd, x), k, tag, abac, cs);
    }
    // lane 0: the same state one cost lower; lanes 1-15 (state 0 only): the
    // other states at this cost
    PA_HDM void lane_x(int l, const Frame& F, int to, int& tag, int& abac, int& cs) const
    {
        if (l == 0)
            load(F.diag0, F.ch0, F.d - 1, plane_back(F.pd, 1), to, tag, abac, cs);
        else if (to == 0 && l < NS)
            load(F.diag0, F.ch0, F.d, F.pd, l, tag, abac, cs);
        else
            tag = -INF, abac = 0, cs = 0;
    }
    // both rounds of a frame in one go (the predecessor round only while
    // the frame is still in it): the two loads of a lane overlap
    PA_HDM void snap(Snap& Sf, Snap& Sx, const Frame& F, int to, int ph, int ab1, int ac1) const
    {
#if defined(__CUDA_ARCH__)
        const int l = (int)(threadIdx.x & 31);
        if (ph == PH_FS) lane_fs(l, F, to, ab1, ac1, Sf.tag, Sf.abac, Sf.cs);
        lane_x(l, F, to, Sx.tag, Sx.abac, Sx.cs);
#else
        for (int l = 0; l < 32; l++) {
            if (ph == PH_FS) lane_fs(l, F, to, ab1, ac1, Sf.tag[l], Sf.abac[l], Sf.cs[l]);
            lane_x(l, F, to, Sx.tag[l], Sx.abac[l], Sx.cs[l]);
        }
#endif
    }

    PA_HDM void push(int& sp, const Frame& F) const
    {
        w.st[sp] = F;
        if (w.ring) {
            w.ring[sp % RING] = F;
            w.ring_tag[sp % RING] = sp;
        }
        sp++;
    }
    PA_HDM void pop(int& sp, Frame& F) const
    {
        --sp;
        if (w.ring && w.ring_tag[sp % RING] == sp)
            F = w.ring[sp % RING];
        else
            F = w.st[sp];
    }

    // a frame for (ab, ac, d, to) on diagonal pair diag0 (cost bound ch0),
    // d in plane pd
    PA_HDM void start(Frame& F, int ab, int ac, int d, int to, int diag0, int ch0, int pd) const
    {
        F.ab = ab, F.ac = ac, F.d = d;
        F.diag0 = diag0, F.ch0 = ch0, F.pd = pd;
        F.best = -INF;
        F.ext = -INF;
        if (d >= cp_cost && d < cp_cost + m.maxstep) {
            F.fabac = pack_abac(ab, ac);
            F.fcs = d * 32 + to;
        } else {
            F.fabac = 0;
            F.fcs = -32;
        }
        const int nb = m.neigh[to];
        const int da = nb & 1, db = (nb >> 1) & 1, dc = (nb >> 2) & 1;
        const int ab1 = ab - da + db, ac1 = ac - da + dc;
        const bool diag = ab1 >= -endB && ab1 <= endA && ac1 >= -endC && ac1 <= endA;
        if (diag) {
            F.ch1 = cheapest(ab1, ac1);
            F.diag1 = in_window(ab1, ac1) ? diag_of(ab1, ac1) : -1;
        } else {
            F.ch1 = 0, F.diag1 = -1;
        }
        F.meta = to | ((diag ? PH_FS : PH_X) << 5);
    }

    // ---- a phase's candidates, evaluated one per lane ----------------------

    struct LaneRes {
        int code;  // 0 value (or none), 1 call the first candidate, 2 the second, 3 window
        int key;   // (dist + KEY_OFF) << 5 | (31 - k) for a value, 0 for none
        int abac, cs;
    };
    static constexpr int KEY_OFF = 8192;

    // predecessor k (src/ukk.checkp.c:644-691) from its two slots: the
    // transition cost (t1) and, for the states that try it, that cost less a
    // mismatch (t2). Candidates before k0 were taken already; at k0 with sub0
    // the first slot was, too.
    PA_HDM LaneRes fs_lane(int k, int k0, int sub0, const Frame& F, int to, int ab1, int ac1,
                           bool copy, int t1, int abac1, int cs1, int t2, int abac2,
                           int cs2) const
    {
        // written with predicates rather than early returns: the lanes of a
        // warp take different outcomes, and one straight path keeps them
        // together
        const bool live = k >= k0 && k < NS;
        const int kk = live ? k : 0;
        const int nb = m.neigh[to];
        const int da = nb & 1, db = (nb >> 1) & 1, dc = (nb >> 2) & 1;
        const int cost = F.d - m.trans[to][kk] - m.cont[to];
        const bool first = live && !(k == k0 && sub0);  // the first slot is still to judge
        const bool miss1 = first && t1 == TAG_MISS;
        const bool win1 = first && t1 == TAG_WINDOW;
        bool ok1 = first && !miss1 && !win1 && ok_index(t1, da, endA) &&
                   ok_index(t1 - ab1, db, endB) && ok_index(t1 - ac1, dc, endC);
        if (ok1)
            ok1 = char_cost(da ? a_at(t1) : 16, db ? b_at(t1 - ab1) : 16,
                            dc ? c_at(t1 - ac1) : 16) == 1;
        // the second slot: when the first failed on a state that tries it, or
        // when the first was taken already
        const bool second = live && !miss1 && !win1 && !ok1 && (!first || m.second[to]);
        const bool miss2 = second && t2 == TAG_MISS;
        const bool win2 = second && t2 == TAG_WINDOW;
        const bool ok2 = second && !miss2 && !win2 && ok_index(t2, da, endA) &&
                         ok_index(t2 - ab1, db, endB) && ok_index(t2 - ac1, dc, endC);
        LaneRes r;
        r.code = miss1 ? 1 : (win1 || win2) ? 3 : miss2 ? 2 : 0;
        const int t = ok1 ? t1 : t2;
        r.key = (ok1 || ok2) ? (((t + da + KEY_OFF) << 5) | (31 - kk)) : 0;
        r.abac = complete ? pack_abac(ab1, ac1) : copy ? (ok1 ? abac1 : abac2) : F.fabac;
        r.cs = complete ? (cost - (ok1 ? 0 : m.mm)) * 32 + kk : copy ? (ok1 ? cs1 : cs2) : F.fcs;
        return r;
    }

    // state l at this cost (src/ukk.checkp.c:722-735), from k0 on
    PA_HDM LaneRes x_lane(int l, int k0, int to, int t) const
    {
        LaneRes r{0, 0, 0, 0};
        if (to != 0 || l < k0 || l >= NS) return r;
        if (t == TAG_MISS) return r.code = 1, r;
        if (t == TAG_WINDOW) return r.code = 3, r;
        r.key = ((t + KEY_OFF) << 5) | (31 - l);
        return r;
    }

    // position p continues the run of matches on diagonal (ab, ac)
    PA_HDM bool run_at(int p, int ab, int ac) const
    {
        return ok_index(p, 1, endA) && ok_index(p - ab, 1, endB) && ok_index(p - ac, 1, endC) &&
               a_at(p) == b_at(p - ab) && a_at(p) == c_at(p - ac);
    }

    // the lanes' results of a round (each lane its own on the GPU)
    struct Lanes {
#if defined(__CUDA_ARCH__)
        LaneRes r;
#else
        LaneRes r[32];
#endif
    };
    // one lane's result, read by every lane (a warp-uniform index)
    PA_HDM int lane_abac(const Lanes& L, int k) const
    {
#if defined(__CUDA_ARCH__)
        return __shfl_sync(0xffffffffu, L.r.abac, k);
#else
        return L.r[k].abac;
#endif
    }
    PA_HDM int lane_cs(const Lanes& L, int k) const
    {
#if defined(__CUDA_ARCH__)
        return __shfl_sync(0xffffffffu, L.r.cs, k);
#else
        return L.r[k].cs;
#endif
    }
    PA_HDM int lane_code(const Lanes& L, int k) const
    {
#if defined(__CUDA_ARCH__)
        return __shfl_sync(0xffffffffu, L.r.code, k);
#else
        return L.r[k].code;
#endif
    }

    // the first lane asking for a call (32 if none), and the largest key of
    // the lanes before it (earliest lane among equals; 0 if none)
    struct Reduced {
        int first, key;
    };
    PA_HDM Reduced reduce(const Lanes& L) const
    {
        Reduced out;
#if defined(__CUDA_ARCH__)
        const unsigned full = 0xffffffffu;
        const int l = (int)(threadIdx.x & 31);
        const unsigned stop = __ballot_sync(full, L.r.code != 0);
        out.first = stop ? __ffs(stop) - 1 : 32;
        out.key = __reduce_max_sync(full, l < out.first ? L.r.key : 0);
#else
        out.first = 32, out.key = 0;
        for (int l = 0; l < 32; l++)
            if (L.r[l].code) {
                out.first = l;
                break;
            }
        for (int l = 0; l < out.first; l++)
            if (L.r[l].key > out.key) out.key = L.r[l].key;
#endif
        return out;
    }

    PA_HDM Reduced walk_fs(const Snap& S, int k0, int sub0, const Frame& F, int to, int ab1,
                           int ac1, bool copy, Lanes& L) const
    {
#if defined(__CUDA_ARCH__)
        const unsigned full = 0xffffffffu;
        const int l = (int)(threadIdx.x & 31);
        const int t2 = __shfl_down_sync(full, S.tag, 16);
        const int a2 = __shfl_down_sync(full, S.abac, 16);
        const int c2 = __shfl_down_sync(full, S.cs, 16);
        L.r = fs_lane(l < 16 ? l : NS, k0, sub0, F, to, ab1, ac1, copy, S.tag, S.abac, S.cs, t2,
                      a2, c2);
#else
        for (int l = 0; l < 32; l++)
            L.r[l] = l < 16 ? fs_lane(l, k0, sub0, F, to, ab1, ac1, copy, S.tag[l], S.abac[l],
                                      S.cs[l], S.tag[l + 16], S.abac[l + 16], S.cs[l + 16])
                            : fs_lane(NS, k0, sub0, F, to, ab1, ac1, copy, 0, 0, 0, 0, 0, 0);
#endif
        return reduce(L);
    }

    PA_HDM Reduced walk_x(const Snap& S, int k0, int to, Lanes& L) const
    {
#if defined(__CUDA_ARCH__)
        L.r = x_lane((int)(threadIdx.x & 31), k0, to, S.tag);
#else
        for (int l = 0; l < 32; l++) L.r[l] = x_lane(l, k0, to, S.tag[l]);
#endif
        return reduce(L);
    }

    // the end of the run of matches from `dist`, 32 positions a round
    PA_HDM int run_end(int dist, int ab, int ac) const
    {
        for (;;) {
#if defined(__CUDA_ARCH__)
            const unsigned mis =
                __ballot_sync(0xffffffffu, !run_at(dist + (int)(threadIdx.x & 31), ab, ac));
#else
            unsigned mis = 0;
            for (int l = 0; l < 32; l++)
                if (!run_at(dist + l, ab, ac)) mis |= 1u << l;
#endif
            if (mis) {
#if defined(__CUDA_ARCH__)
                return dist + __ffs(mis) - 1;
#else
                int l = 0;
                while (!(mis >> l & 1u)) l++;
                return dist + l;
#endif
            }
            dist += 32;
        }
    }

    // Ukk(ab, ac, d, s) (src/ukk.checkp.c:576-782), the whole warp running
    // one triple: the frame on top of the stack lives in registers, its
    // candidate cells are read in one round and evaluated one per lane, and
    // ballots and a max-reduction give what the reference's loops over them
    // give (the first candidate to compute, and the first strict maximum of
    // the ones before it). A round is read again after every callee returns,
    // since the callee may have written any slot; between reads nothing is
    // written, so each value is the one the reference reads at that point.
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
        Frame F;
        start(F, ab0, ac0, d0, s0, diag_of(ab0, ac0), cheapest(ab0, ac0), d0 % (2 * m.maxstep));
        Snap Sf, Sx;
        bool fresh = false;
        for (;;) {
            if (++steps > w.step_cap) {
                fail(ERR_STEPS);
                return -INF;
            }
            if ((steps & 4095) == 0 && now_ns() - t0 > TIME_LIMIT_NS) {
                fail(ERR_TIME);
                return -INF;
            }
            const int to = F.meta & 31;
            int ph = (F.meta >> 5) & 1;
            int k = (F.meta >> 8) & 31;
            int sub = (F.meta >> 13) & 1;
            int fst = ((F.meta >> 14) & 31) - 1;
            const int nb = m.neigh[to];
            const int da = nb & 1, db = (nb >> 1) & 1, dc = (nb >> 2) & 1;
            const int ab1 = F.ab - da + db, ac1 = F.ac - da + dc;
            const bool copy = F.d >= cp_cost + m.maxstep;
            if (!fresh) snap(Sf, Sx, F, to, ph, ab1, ac1);
            fresh = true;
            int cab = 0, cac = 0, cd = 0, cst = 0, cdiag = 0, cch = 0, cpl = 0;
            bool call = false;
            Lanes L;
            if (ph == PH_FS) {
                const Reduced R = walk_fs(Sf, k, sub, F, to, ab1, ac1, copy, L);
                if (R.key) {
                    const int dist = (R.key >> 5) - KEY_OFF;
                    if (F.best < dist) {
                        const int bl = 31 - (R.key & 31);
                        F.best = dist;
                        F.fabac = lane_abac(L, bl);
                        F.fcs = lane_cs(L, bl);
                    }
                }
                if (R.first < NS) {
                    const int code = lane_code(L, R.first);
                    if (code == 3) {
                        fail(ERR_WINDOW);
                        return -INF;
                    }
                    k = R.first;
                    sub = code == 2;
                    const int x = m.trans[to][k] + m.cont[to] + (sub ? m.mm : 0);
                    call = true, cab = ab1, cac = ac1, cst = k, cd = F.d - x;
                    cdiag = F.diag1, cch = F.ch1, cpl = plane_back(F.pd, x);
                } else {
                    // nothing was written since the round was read: the
                    // second round of the same read is current
                    ph = PH_X, k = 0, sub = 0;
                }
            }
            bool finish = false;
            if (!call) {
                if (k == 0) {
                    // the same state one cost lower (src/ukk.checkp.c:694-711)
                    const int t = tag_of(Sx, 0);
                    if (t == TAG_MISS) {
                        call = true, cab = F.ab, cac = F.ac, cd = F.d - 1, cst = to;
                        cdiag = F.diag0, cch = F.ch0, cpl = plane_back(F.pd, 1);
                    } else if (t == TAG_WINDOW) {
                        fail(ERR_WINDOW);
                        return -INF;
                    } else {
                        if (ok_index(t, 0, endA) && ok_index(t - F.ab, 0, endB) &&
                            ok_index(t - F.ac, 0, endC) && F.best < t) {
                            F.best = t;
                            if (complete) {
                                F.fabac = pack_abac(F.ab, F.ac);
                                F.fcs = (F.d - 1) * 32 + to;
                            } else if (copy) {
                                F.fabac = abac_of(Sx, 0);
                                F.fcs = cs_of(Sx, 0);
                            }
                        }
                        if (to != 0) {
                            finish = true;
                        } else {
                            F.ext = F.best > -INF ? F.best : -INF;
                            fst = F.best > -INF ? 0 : -1;
                            k = 1;
                        }
                    }
                }
                if (!call && !finish) {
                    // the other states at this cost, then the run of matches
                    // (src/ukk.checkp.c:712-759)
                    const Reduced R = walk_x(Sx, k, to, L);
                    if (R.key) {
                        const int t = (R.key >> 5) - KEY_OFF;
                        if (t > F.ext) {
                            F.ext = t;
                            fst = 31 - (R.key & 31);
                        }
                    }
                    if (R.first < NS) {
                        if (lane_code(L, R.first) == 3) {
                            fail(ERR_WINDOW);
                            return -INF;
                        }
                        k = R.first;
                        call = true, cab = F.ab, cac = F.ac, cd = F.d, cst = k;
                        cdiag = F.diag0, cch = F.ch0, cpl = F.pd;
                    } else {
                        const int dist = run_end(F.ext, F.ab, F.ac);
                        if (dist > F.best) {
                            F.best = dist;
                            if (fst != 0) {
                                if (complete) {
                                    F.fabac = pack_abac(F.ab, F.ac);
                                    F.fcs = F.d * 32 + fst;
                                } else if (copy) {
                                    F.fabac = abac_of(Sx, fst);
                                    F.fcs = cs_of(Sx, fst);
                                }
                            }
                        }
                        finish = true;
                    }
                }
            }
            if (finish) {
                Cell* c = w.U + ((long long)F.diag0 * (2 * m.maxstep) + F.pd) * NS + to;
                c->dist = F.best;
                c->stamp = F.d + off;
                c->abac = F.fabac;
                c->cs = F.fcs;
                if (F.d >= cp_cost && F.d < cp_cost + m.maxstep) {
                    const int cpl_ = F.pd >= m.maxstep ? F.pd - m.maxstep : F.pd;
                    w.CP[((long long)F.diag0 * m.maxstep + cpl_) * NS + to] = F.best;
                }
                if (F.best > furthest) furthest = F.best;
                if (sp == 0) return F.best;
                pop(sp, F);
                fresh = false;
                continue;
            }
            // the callee was a miss in the current round, so it lies in the
            // matrix and the window
            F.meta = to | (ph << 5) | (k << 8) | (sub << 13) | ((fst + 1) << 14);
            if (sp >= w.st_cap) {
                fail(ERR_STACK);
                return -INF;
            }
            push(sp, F);
            start(F, cab, cac, cd, cst, cdiag, cch, cpl);
            fresh = false;
        }
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
        const long long ub = cost_bound(m.maxstep, la, lb, lc);
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
