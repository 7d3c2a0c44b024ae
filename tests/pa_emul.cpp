// TEST-ONLY host replay of the GPU lane pipeline.
//
// Builds into libpa_emul.so, which only tests/ load. It runs the exact step
// functions of pa_core.cuh that the kernels run, lane by lane, with the
// rotating neighbour exchange done through an array, so the kernel algorithm
// can be checked against the oracle on a machine without a GPU. The product
// library never links this file.
#include <stdint.h>
#include <string.h>

#include <array>
#include <vector>

#include "pa_core.cuh"
#include "pa_newkk.cuh"
#include "pa_tables.h"

using namespace pa;

namespace {

template <int R>
void lin_pass(const LinBand& b, int P, const Tables& t, const uint8_t* x,
              const uint8_t* y, uint8_t* dm, int* cost, int* gapnum)
{
    std::vector<LinLane<R>> L(P);
    for (int g = 0; g < P; g++) lin_lane_init(L[g], b, t, x, g, P);
    std::vector<int> sv(P);
    std::vector<uint32_t> sn(P);
    const int Tlast = (b.m - 1) + (b.n - 1);
    // row 0 is generated only up to step Tg, as in the kernel
    const int Tg = tmin((Tlast + 1) & ~1, lin_gen_steps(b, P, R));
    for (int T = 1; T <= Tlast; T++) {
        const bool odd = T & 1;
        for (int g = 0; g < P; g++) {
            sv[g] = odd ? L[g].V0[R - 1] : L[g].V1[R - 1];
            sn[g] = odd ? L[g].N0[R - 1] : L[g].N1[R - 1];
        }
        for (int g = 0; g < P; g++) {
            const int src = (g + P - 1) % P;
            int dc[R];
            LinLane<R>& l = L[g];
            if (odd && T <= Tg)
                lin_step<R, true>(l, l.V0, l.V1, l.N0, l.N1, l.R0, l.R1, l.RN0, l.RN1, l.G0,
                                  l.G1, b, t, x, y, P, T, sv[src], sn[src], dc);
            else if (odd)
                lin_step<R, false>(l, l.V0, l.V1, l.N0, l.N1, l.R0, l.R1, l.RN0, l.RN1, l.G0,
                                   l.G1, b, t, x, y, P, T, sv[src], sn[src], dc);
            else if (T <= Tg)
                lin_step<R, true>(l, l.V1, l.V0, l.N1, l.N0, l.R1, l.R0, l.RN1, l.RN0, l.G1,
                                  l.G0, b, t, x, y, P, T, sv[src], sn[src], dc);
            else
                lin_step<R, false>(l, l.V1, l.V0, l.N1, l.N0, l.R1, l.R0, l.RN1, l.RN0, l.G1,
                                   l.G0, b, t, x, y, P, T, sv[src], sn[src], dc);
            for (int q = 0; q < R; q++) dm[(long long)T * P * R + g * R + q] = (uint8_t)dc[q];
        }
    }
    const int i = b.m - 1;
    const int blk = (i - 1) / R, g = blk % P, q = (i - 1) - blk * R;
    const bool odd = Tlast & 1;
    *cost = odd ? L[g].V1[q] : L[g].V0[q];
    const uint32_t N = odd ? L[g].N1[q] : L[g].N0[q];
    *gapnum = tmax((int)(N & 0xFFFF), (int)(N >> 16));
}

template <int R>
void aff_pass(const AffBand& b, int P, const Tables& t, const uint8_t* x,
              const uint8_t* y, uint16_t* dm, int* shadowEB, int shadowEH0,
              int* cost, int* gapnum)
{
    std::vector<AffLane<R>> L(P);
    for (int g = 0; g < P; g++) aff_lane_init(L[g], b, t, x, g, P);
    std::vector<AffCell> sv(P);
    const int Tlast = (b.m - 1) + (b.n - 1);
    for (int T = 1; T <= Tlast; T++) {
        for (int g = 0; g < P; g++) sv[g] = L[g].V[R - 1];
        for (int g = 0; g < P; g++) {
            int src = (g + P - 1) % P;
            int dc[R];
            aff_step<R>(L[g], b, t, x, y, P, T, sv[src], shadowEB, shadowEH0,
                        shadowEB, dc);
            for (int q = 0; q < R; q++) dm[(long long)T * P * R + g * R + q] = (uint16_t)dc[q];
        }
    }
    const int i = b.m - 1;
    const int blk = (i - 1) / R, g = blk % P, q = (i - 1) - blk * R;
    *cost = aff_final(L[g].V[q]);
    *gapnum = aff_gapnum(L[g].V[q]);
}

template <int R>
void aff_pass_fast(const AffBand& b, int P, const Tables& t, const uint8_t* x,
              const uint8_t* y, uint16_t* dm, int* shadowEB, int shadowEH0,
              int* cost, int* gapnum)
{
    std::vector<AffFastLane<R>> L(P);
    for (int g = 0; g < P; g++) aff_fast_lane_init(L[g], b, t, x, g, P);
    std::vector<AffCell> sv(P);
    const int Tlast = (b.m - 1) + (b.n - 1);
    for (int T = 1; T <= Tlast; T++) {
        for (int g = 0; g < P; g++) sv[g] = L[g].V[R - 1];
        for (int g = 0; g < P; g++) {
            int src = (g + P - 1) % P;
            int dc[R];
            aff_fast_step<R>(L[g], b, t, x, y, P, T, sv[src], shadowEB, shadowEH0, dc);
            for (int q = 0; q < R; q++) dm[(long long)T * P * R + g * R + q] = (uint16_t)dc[q];
        }
    }
    const int i = b.m - 1;
    const int blk = (i - 1) / R, g = blk % P, q = (i - 1) - blk * R;
    *cost = aff_final(L[g].V[q]);
    *gapnum = aff_gapnum(L[g].V[q]);
}

template <int R>
void aff_pass_lean(const AffBand& b, int P, const Tables& t, const uint8_t* x,
                   const uint8_t* y, uint8_t* dm, int shadowEH0, int* cost, int* gapnum)
{
    std::vector<AffLean<R>> L(P);
    for (int g = 0; g < P; g++) aff_lean_init(L[g], b, t, x, g, P);
    std::vector<LeanCell> sv(P);
    const int Tlast = (b.m - 1) + (b.n - 1);
    // row 0 is generated only up to step Tg, as in the kernel
    const int Tg = tmin((Tlast + 1) & ~1, lean_gen_steps(b, P, R));
    for (int T = 1; T <= Tlast; T++) {
        const bool odd = T & 1;
        for (int g = 0; g < P; g++) sv[g] = odd ? L[g].V0[R - 1] : L[g].V1[R - 1];
        for (int g = 0; g < P; g++) {
            const int src = (g + P - 1) % P;
            int dc[R];
            AffLean<R>& l = L[g];
            if (odd && T <= Tg)
                aff_lean_step<R, true>(l, l.V0, l.V1, l.R0, l.R1, l.G0, l.G1, b, t, x, y, P, T,
                                       sv[src], shadowEH0, dc);
            else if (odd)
                aff_lean_step<R, false>(l, l.V0, l.V1, l.R0, l.R1, l.G0, l.G1, b, t, x, y, P, T,
                                        sv[src], shadowEH0, dc);
            else if (T <= Tg)
                aff_lean_step<R, true>(l, l.V1, l.V0, l.R1, l.R0, l.G1, l.G0, b, t, x, y, P, T,
                                       sv[src], shadowEH0, dc);
            else
                aff_lean_step<R, false>(l, l.V1, l.V0, l.R1, l.R0, l.G1, l.G0, b, t, x, y, P, T,
                                        sv[src], shadowEH0, dc);
            for (int q = 0; q < R; q++) dm[(long long)T * P * R + g * R + q] = (uint8_t)dc[q];
        }
    }
    const int i = b.m - 1;
    const int blk = (i - 1) / R, g = blk % P, q = (i - 1) - blk * R;
    const LeanCell c = (Tlast & 1) ? L[g].V1[q] : L[g].V0[q];
    *cost = lean_final(c);
    *gapnum = lean_gapnum(c);
}

// The row tile, lane by lane: each cross-lane step of the kernel (shuffles,
// exclusive scans of the composed maps) is done over arrays of the 32 lanes.
template <int K>
void aff_pass_rk(const AffBand& b, const Tables& t, const uint8_t* x, const uint8_t* y,
                 uint8_t* dm, int shadowEH0, int* cost, int* gapnum)
{
    constexpr int S = 32 * K;
    const int newk = b.newk, n = b.n;
    std::vector<std::array<LeanCell, K>> P(32);
    std::vector<std::array<int, K>> J(32), JG(32);
    // row 0: prefix sums of the prepend terms
    {
        int run = 0;
        for (int l = 0; l < 32; l++)
            for (int q = 0; q < K; q++) {
                const int j = l * K + q - newk;
                run += (j >= 1 && j < n) ? rk_row0_term(t, y, j) : 0;
                P[l][q] = rk_row0(j, run, shadowEH0);
            }
    }
    for (int l = 0; l < 32; l++)
        for (int q = 0; q < K; q++) {
            const int j = 1 + l * K + q - newk;
            J[l][q] = (j >= 0 && j < n) ? y[j] : 0;
            JG[l][q] = t.prepend[J[l][q]];
        }
    for (int i = 1; i <= b.m - 1; i++) {
        if (i > 1) {
            for (int l = 0; l < 32; l++) {
                for (int q = 0; q + 1 < K; q++) {
                    J[l][q] = J[l][q + 1];
                    JG[l][q] = JG[l][q + 1];
                }
                if (l < 31) {
                    J[l][K - 1] = J[l + 1][0];
                    JG[l][K - 1] = JG[l + 1][0];
                } else {
                    const int j = i + S - 1 - newk;
                    J[l][K - 1] = (j >= 0 && j < n) ? y[j] : 0;
                    JG[l][K - 1] = t.prepend[J[l][K - 1]];
                }
            }
        }
        const RkRow r = rk_row(b, t, x, i);
        std::vector<std::array<int, K>> EV(32), CB(32), EH(32), code(32), hv(32);
        std::vector<std::array<uint32_t, K>> fl(32);
        std::vector<LeanCell> upn(32);
        std::vector<MinPlus> F(32);
        std::vector<GmMap> G(32);
        std::vector<int> cbl(32);
        for (int l = 0; l < 32; l++) upn[l] = l < 31 ? P[l + 1][0] : P[l][0];
        for (int l = 0; l < 32; l++) {
            LeanCell Pl[K];
            int Jl[K], EVl[K], CBl[K], codel[K];
            for (int q = 0; q < K; q++) {
                Pl[q] = P[l][q];
                Jl[q] = J[l][q];
            }
            rk_phase_a<K>(Pl, upn[l], Jl, r, t, i + l * K - newk, EVl, CBl, codel);
            for (int q = 0; q < K; q++) {
                EV[l][q] = EVl[q];
                CB[l][q] = CBl[q];
                code[l][q] = codel[q];
            }
        }
        for (int l = 0; l < 32; l++) {
            cbl[l] = l == 0 ? HIGH : CB[l - 1][K - 1];
            int JGl[K], CBl[K];
            for (int q = 0; q < K; q++) {
                JGl[q] = JG[l][q];
                CBl[q] = CB[l][q];
            }
            F[l] = rk_eh_map<K>(JGl, CBl, r, t.go, i + l * K - newk, cbl[l]);
        }
        MinPlus pre{0, MP_BIG};
        std::vector<int> xin(32);
        for (int l = 0; l < 32; l++) {
            xin[l] = l == 0 ? HIGH : mp_apply(pre, HIGH);
            pre = l == 0 ? F[0] : mp_then(pre, F[l]);
        }
        for (int l = 0; l < 32; l++) {
            LeanCell Pl[K];
            int JGl[K], EVl[K], CBl[K], EHl[K], codel[K], hvl[K];
            uint32_t fll[K];
            for (int q = 0; q < K; q++) {
                Pl[q] = P[l][q];
                JGl[q] = JG[l][q];
                EVl[q] = EV[l][q];
                CBl[q] = CB[l][q];
                codel[q] = code[l][q];
            }
            G[l] = rk_phase_b<K>(Pl, upn[l], JGl, r, t, i + l * K - newk, xin[l], cbl[l], EVl,
                                 CBl, EHl, codel, hvl, fll);
            for (int q = 0; q < K; q++) {
                EH[l][q] = EHl[q];
                code[l][q] = codel[q];
                hv[l][q] = hvl[q];
                fl[l][q] = fll[q];
            }
        }
        GmMap gpre{1, 0u, 0u};
        for (int l = 0; l < 32; l++) {
            const uint32_t yin = l == 0 ? 0u : gm_apply(gpre, 0u);
            LeanCell Pl[K];
            int EHl[K], EVl[K], CBl[K], hvl[K], codel[K];
            uint32_t fll[K];
            for (int q = 0; q < K; q++) {
                Pl[q] = P[l][q];
                EHl[q] = EH[l][q];
                EVl[q] = EV[l][q];
                CBl[q] = CB[l][q];
                hvl[q] = hv[l][q];
                fll[q] = fl[l][q];
                codel[q] = code[l][q];
            }
            rk_phase_c<K>(Pl, r, i + l * K - newk, yin, EHl, EVl, CBl, hvl, fll, codel);
            for (int q = 0; q < K; q++) {
                P[l][q] = Pl[q];
                dm[(long long)i * S + l * K + q] = (uint8_t)codel[q];
            }
            gpre = l == 0 ? G[0] : gm_then(gpre, G[l]);
        }
    }
    const int dc = b.n - 1 - (b.m - 1) + newk;
    const LeanCell c = P[dc / K][dc % K];
    *cost = lean_final(c);
    *gapnum = lean_gapnum(c);
}

struct Emul {
    HostCM cm;
    Tables t;
    Ladder lad[2] = {default_ladder(0), default_ladder(1)};
    int row_tile = 1;  // lean bands up to 512 wide on the row tile (0: lane pipeline)
    int window_all = 0;  // every linear traceback through the shared-memory window
    int skip = 1;        // start after the passes that cannot end the doubling, as prep does
    mutable std::vector<int> rec;  // affine passes run: T, gap count (pa_emul_aff_passes)
};

// The band doubling of plan pl (x = rows, y = columns), as the class
// kernels run it: the final fill stays in dm (P lanes x R rows) with band bd.
int lin_fill_doubling(const Emul& E, const PairPlan& pl, const uint8_t* x, const uint8_t* y,
                      std::vector<uint8_t>& dm, int& P, int& R, LinBand& bd, int* cost,
                      int* passes, int* last_class)
{
    const Tables& t = E.t;
    const int m = pl.m, n = pl.n;
    int T = pl.T0, g = 0;
    P = 32;
    R = 1;
    *passes = 0;
    *last_class = -1;
    if (E.skip && !pl.full) {
        const int s = unstoppable_passes(T, m, n, false, 39);
        T <<= s;
        *passes = s;
    }
    for (;;) {
        bd = lin_band(m, n, pl.full, pl.full ? 0 : band_p(T, m, n));
        int c = pick_class(E.lad[0], lin_wu(bd), n);
        if (c < 0) return -5;
        P = E.lad[0].P[c];
        R = E.lad[0].R[c];
        *last_class = c;
        dm.assign((size_t)(m + n + 1) * P * R, 0);
        (*passes)++;
        if (m == 1) {  // no rows: row 0 is the whole alignment
            int s = 0;
            for (int j = 1; j < n; j++) s += t.prepend[y[j]];
            *cost = s;
            g = n - 1;
        } else {
            switch (R) {
                case 1: lin_pass<1>(bd, P, t, x, y, dm.data(), cost, &g); break;
                case 2: lin_pass<2>(bd, P, t, x, y, dm.data(), cost, &g); break;
                case 4: lin_pass<4>(bd, P, t, x, y, dm.data(), cost, &g); break;
                default: lin_pass<8>(bd, P, t, x, y, dm.data(), cost, &g); break;
            }
        }
        if (pl.full || lin_done(T, m, n, g)) return 0;
        T *= 2;
    }
}

int run_linear(const Emul& E, const uint8_t* a, int la, const uint8_t* b, int lb,
               int* cost, uint8_t* ea, uint8_t* eb, uint8_t* med, uint8_t* mwg,
               int cap, int* res, int* passes, int* last_class)
{
    const Tables& t = E.t;
    PairPlan pl = plan_linear(t, count_gap_states(a, la, t.gap), la,
                              count_gap_states(b, lb, t.gap), lb);
    const uint8_t* x = pl.swaped ? b : a;
    const uint8_t* y = pl.swaped ? a : b;
    const int m = pl.m, n = pl.n;
    std::vector<uint8_t> dm;
    int P, R;
    LinBand bd;
    const int st = lin_fill_doubling(E, pl, x, y, dm, P, R, bd, cost, passes, last_class);
    if (st) return st;
    PairOut o = {ea, eb, med, mwg, cap};
    PairRes r;
    // as the kernels do: the class kernel's in-kernel traceback through the
    // window for pipelines of a warp or more; the deferred one (window_all)
    // through the window for every class
    if (lin_window_ok(P, R) || E.window_all) {
        std::vector<uint32_t> win(LW_SMEM_WORDS);
        LinDmWindow<> rd{dm.data(), win.data(), P * R, P * R / 4, 0, 1};
        r = lin_traceback_dm(rd, t, x, m, y, n, pl.swaped, o);
    } else {
        r = lin_traceback(dm.data(), P, R, t, x, m, y, n, pl.swaped, o);
    }
    res[0] = r.alen;
    res[1] = r.mlen;
    res[2] = r.wlen;
    res[3] = r.maxcost;
    return r.status;
}

int run_affine(const Emul& E, const uint8_t* a, int la, const uint8_t* b, int lb,
               int* cost, uint8_t* ea, uint8_t* eb, uint8_t* med, uint8_t* mwg,
               int cap, int* res, int* passes, int* last_class)
{
    const Tables& t = E.t;
    PairPlan pl = plan_affine(t, la, lb);
    const uint8_t* x = pl.swaped ? b : a;
    const uint8_t* y = pl.swaped ? a : b;
    const int m = pl.m, n = pl.n;
    if (m == 1 && n == 1) return -4;
    std::vector<uint16_t> dm;
    std::vector<uint8_t> dm8;  // lean passes
    bool lean_last = false;
    std::vector<int> shadow(n, HIGH);
    bool gapfree = t.gap == TMPGAP;
    for (int i = 1; i < la; i++) gapfree = gapfree && !(a[i] & TMPGAP);
    for (int i = 1; i < lb; i++) gapfree = gapfree && !(b[i] & TMPGAP);
    int shadowEH0 = t.go;
    int P = 32, R = 1, T = pl.T0, g = 0;
    *passes = 0;
    *last_class = -1;
    const bool lean = gapfree && aff_lean_ok(t, tmax(la, lb));
    int rk = 0, rk_newk = 0;
    if (E.skip && lean) {  // as prep: the row-0 value of the first pass run
        const int s = unstoppable_passes(T, m, n, true, 39);
        if (s > 0 && m - 1 >= 2 && tmin(m - 1, aff_band(m, n, band_p(T << (s - 1), m, n)).newk) >= 2)
            shadowEH0 = HIGH;
        T <<= s;
        *passes = s;
    }
    for (;;) {
        AffBand bd = aff_band(m, n, band_p(T, m, n));
        const bool rt = lean && E.row_tile;
        int c = rt ? pick_class_lean(E.lad[1], aff_wu(bd), n) : pick_class(E.lad[1], aff_wu(bd), n);
        if (c < 0) return -5;
        P = E.lad[1].P[c];
        R = E.lad[1].R[c];
        rk = rt ? rk_k_for(ladder_cap(E.lad[1], c)) : 0;
        rk_newk = bd.newk;
        *last_class = c;
        dm.assign((size_t)(m + n + 1) * P * R, 0);
        dm8.assign(std::max((size_t)(m + n + 1) * P * R, (size_t)m * 32 * (rk ? rk : 1)), 0);
        lean_last = false;
        (*passes)++;
        if (m == 1) {  // leni = 0: the initial row is the whole alignment
            int s = t.go;
            for (int j = 1; j < n; j++) s += t.prepend[y[j]];
            *cost = s;
            g = 0xFFFF;
        } else {
            if (lean && rk) {
                lean_last = true;
                switch (rk) {
                    case 1: aff_pass_rk<1>(bd, t, x, y, dm8.data(), shadowEH0, cost, &g); break;
                    case 2: aff_pass_rk<2>(bd, t, x, y, dm8.data(), shadowEH0, cost, &g); break;
                    case 4: aff_pass_rk<4>(bd, t, x, y, dm8.data(), shadowEH0, cost, &g); break;
                    case 8: aff_pass_rk<8>(bd, t, x, y, dm8.data(), shadowEH0, cost, &g); break;
                    default: aff_pass_rk<16>(bd, t, x, y, dm8.data(), shadowEH0, cost, &g); break;
                }
            } else if (lean) {
                lean_last = true;
                switch (R) {
                    case 1: aff_pass_lean<1>(bd, P, t, x, y, dm8.data(), shadowEH0, cost, &g); break;
                    case 2: aff_pass_lean<2>(bd, P, t, x, y, dm8.data(), shadowEH0, cost, &g); break;
                    case 3: aff_pass_lean<3>(bd, P, t, x, y, dm8.data(), shadowEH0, cost, &g); break;
                    default: aff_pass_lean<4>(bd, P, t, x, y, dm8.data(), shadowEH0, cost, &g); break;
                }
            } else if (gapfree) {
                switch (R) {
                    case 1: aff_pass_fast<1>(bd, P, t, x, y, dm.data(), shadow.data(), shadowEH0, cost, &g); break;
                    case 2: aff_pass_fast<2>(bd, P, t, x, y, dm.data(), shadow.data(), shadowEH0, cost, &g); break;
                    case 3: aff_pass_fast<3>(bd, P, t, x, y, dm.data(), shadow.data(), shadowEH0, cost, &g); break;
                    default: aff_pass_fast<4>(bd, P, t, x, y, dm.data(), shadow.data(), shadowEH0, cost, &g); break;
                }
            } else {
                switch (R) {
                    case 1: aff_pass<1>(bd, P, t, x, y, dm.data(), shadow.data(), shadowEH0, cost, &g); break;
                    case 2: aff_pass<2>(bd, P, t, x, y, dm.data(), shadow.data(), shadowEH0, cost, &g); break;
                    case 3: aff_pass<3>(bd, P, t, x, y, dm.data(), shadow.data(), shadowEH0, cost, &g); break;
                    default: aff_pass<4>(bd, P, t, x, y, dm.data(), shadow.data(), shadowEH0, cost, &g); break;
                }
            }
            if (tmin(m - 1, bd.newk) >= 2) shadowEH0 = HIGH;
        }
        E.rec.push_back(T);
        E.rec.push_back(g);
        if (aff_done(T, m, n, g)) break;
        T *= 2;
    }
    PairOut o = {ea, eb, med, mwg, cap};
    PairRes r;
    if (lean_last && !rk && E.window_all) {  // as the deferred lean traceback: the window
        std::vector<uint32_t> win(LW_SMEM_WORDS);
        const int PR = P * R;
        if ((PR & (PR - 1)) == 0) {
            AffDmLeanWindow<true> rd{LinDmWindow<true>{dm8.data(), win.data(), PR, PR / 4, 0, 1}};
            r = aff_traceback_dm(rd, t, x, m, y, n, pl.swaped, o);
        } else {
            AffDmLeanWindow<false> rd{LinDmWindow<false>{dm8.data(), win.data(), PR, PR / 4, 0, 1}};
            r = aff_traceback_dm(rd, t, x, m, y, n, pl.swaped, o);
        }
    } else if (lean_last && rk && E.window_all) {  // as the deferred row-tile traceback
        const int S = 32 * rk;
        std::vector<Word16> win(RW_BYTES / 16);
        AffDmRowWindow rd{dm8.data(), win.data(), S, rk_newk, RW_BYTES / S, 0, 1};
        r = aff_traceback_dm(rd, t, x, m, y, n, pl.swaped, o);
    } else {
        r = (lean_last && rk) ? aff_traceback_rowtile(dm8.data(), 32 * rk, rk_newk, t, x, m, y, n,
                                                      pl.swaped, o)
            : lean_last ? aff_traceback_lean(dm8.data(), P, R, t, x, m, y, n, pl.swaped, o)
                        : aff_traceback(dm.data(), P, R, t, x, m, y, n, pl.swaped, o);
    }
    res[0] = r.alen;
    res[1] = r.mlen;
    res[2] = r.wlen;
    res[3] = r.maxcost;
    return r.status;
}

// Algn_Newkk: the kernel's pass (pa_newkk.cu fill_pass) replayed with the
// 32 lanes of the warp in arrays: every step, lanes 0..31 run lane_step in
// turn (lane 0's boundary-row reads never meet lane 31's write of the same
// step: they are at least one column apart), then lane r receives lane
// r-1's last cell (shuffle up).
struct NkEmul {
    std::vector<uint16_t> arena;
    std::vector<nk::Quad> bnd;
    std::vector<uint32_t> bndg;
    std::vector<int> c0;
};

int nk_fill(NkEmul& E, const Tables& t, const uint8_t* s1, int l1, const uint8_t* s2, int l2,
            int k, int go, uint32_t& glast)
{
    const nk::Band B{l1, l2, k};
    E.c0.assign((size_t)B.rounds(), 0);
    const long long steps = nk::rounds_table(B, E.c0.data());
    E.arena.assign((size_t)steps * 32, 0xffff);
    E.bnd.assign((size_t)l2, nk::Quad{0, 0, 0, 0});
    E.bndg.assign((size_t)l2, 0u);
    nk::Lane L[32];
    for (int r = 0; r < 32; r++) nk::lane_start(L[r], B, s1, r);
    for (long long st = 0; st < steps; st++) {
        for (int r = 0; r < 32; r++) {
            int j = 0;
            const int dir = nk::lane_step(L[r], t, s1, s2, B, E.c0.data(), r, st, E.bnd.data(),
                                          E.bndg.data(), go, j);
            if (dir >= 0) {
                E.arena[(size_t)(st * 32 + r)] = (uint16_t)dir;
                if (r == 31) {
                    E.bnd[(size_t)j] = {L[r].left.P, L[r].left.Q, L[r].left.ED, L[r].left.CD};
                    E.bndg[(size_t)j] = L[r].left.g;
                }
            }
        }
        for (int r = 31; r >= 1; r--) L[r].nu = L[r - 1].left;
        L[0].nu = L[0].left;
    }
    const int rl = (l1 - 1) & 31;
    glast = L[rl].left.g;
    return L[rl].lcost;
}

struct NkDir {
    const NkEmul* E;
    int operator()(int i, int j) const
    {
        return E->arena[(size_t)nk::dir_word(E->c0.data(), i, j)];
    }
};

}  // namespace

extern "C" {

void* pa_emul_new(const int* tcm, int alph, int gap_open)
{
    Emul* e = new Emul;
    if (build_cm(&e->cm, tcm, alph, gap_open)) {
        delete e;
        return nullptr;
    }
    kernel_tables(e->cm, &e->t);
    return e;
}

void pa_emul_free(void* e) { delete (Emul*)e; }

// 0: lean affine passes on the lane pipeline only; 1: on the row tile up to
// 512 wide (the default, as in a context).
void pa_emul_set_row_tile(void* e, int mode) { ((Emul*)e)->row_tile = mode ? 1 : 0; }

// 1: every linear traceback and every lean affine one (lane pipeline) through
// the shared-memory window, as the deferred tracebacks run them (0: only
// linear pipelines of a warp or more).
void pa_emul_set_window(void* e, int all) { ((Emul*)e)->window_all = all ? 1 : 0; }

// 0: run every pass of the doubling from T0 (the reference's schedule)
void pa_emul_set_skip(void* e, int on) { ((Emul*)e)->skip = on ? 1 : 0; }

// unstoppable_passes (pa_core.cuh) for the host accounting's test
int pa_emul_unstoppable(int T0, int m, int n, int affine)
{
    return unstoppable_passes(T0, m, n, affine != 0, 39);
}

// Copies out the product's host tables for comparison with the oracle.
int pa_emul_tables(void* h, int* cost, uint8_t* median, int* worst, int* tail,
                   int* prepend, int* info)
{
    const HostCM& cm = ((Emul*)h)->cm;
    const int n = 2 * (1 << cm.lcm) * (1 << cm.lcm);
    memcpy(cost, cm.cost, (size_t)n * sizeof(int));
    memcpy(worst, cm.worst, (size_t)n * sizeof(int));
    memcpy(tail, cm.tail, (size_t)n * sizeof(int));
    memcpy(prepend, cm.prepend, (size_t)n * sizeof(int));
    memcpy(median, cm.median, (size_t)n);
    info[0] = cm.lcm;
    info[1] = cm.gap;
    info[2] = cm.a_sz;
    info[3] = cm.combinations;
    info[4] = cm.cost_model;
    info[5] = cm.gap_open;
    return n;
}

// DOS.median of one pair through the replayed pipeline. Outputs end at
// index cap-1 of each buffer; res = {alen, mlen, wlen, maxcost}.
int pa_emul_median(void* h, int affine, const uint8_t* a, int la,
                   const uint8_t* b, int lb, int* cost, uint8_t* ea,
                   uint8_t* eb, uint8_t* med, uint8_t* mwg, int cap, int* res,
                   int* passes, int* last_class)
{
    const Emul& E = *(Emul*)h;
    if (affine)
        return run_affine(E, a, la, b, lb, cost, ea, eb, med, mwg, cap, res, passes, last_class);
    return run_linear(E, a, la, b, lb, cost, ea, eb, med, mwg, cap, res, passes, last_class);
}

// The affine doubling of one pair (DOS.median) pass by pass: T and the gap
// count of every pass run, at most maxp; returns the number of passes run
// (or a negative status).
int pa_emul_aff_passes(void* h, const uint8_t* a, int la, const uint8_t* b, int lb, int* Ts,
                       int* gaps, int maxp)
{
    const Emul& E = *(Emul*)h;
    const int cap = la + lb + 2;
    std::vector<uint8_t> ea(cap), eb(cap), med(cap), mwg(cap);
    int cost = 0, res[4], passes = 0, lc = 0;
    E.rec.clear();
    const int rc = run_affine(E, a, la, b, lb, &cost, ea.data(), eb.data(), med.data(),
                              mwg.data(), cap, res, &passes, &lc);
    if (rc < 0 && rc != -4) return rc;
    const int np = (int)E.rec.size() / 2;
    for (int j = 0; j < np && j < maxp; j++) {
        Ts[j] = E.rec[2 * j];
        gaps[j] = E.rec[2 * j + 1];
    }
    return np;
}

// verify_aligned / median_no_gaps / worst_aligned (pa_core.cuh) on an
// aligned pair, as the per-call kernels run them; out holds len + 1 bytes.
int pa_emul_aligned_extra(void* h, const uint8_t* a, const uint8_t* b, int len, int* res,
                          uint8_t* out)
{
    const Tables& t = ((Emul*)h)->t;
    res[0] = verify_aligned(t, a, b, len);
    res[1] = median_no_gaps(t, a, b, len, out);
    res[2] = worst_aligned(t, a, b, len);
    return 0;
}

// DOS.median with use_ukk (affine) of one pair through the replayed Newkk
// warp, as newkk_kernel runs it. Outputs end at index cap-1 of each buffer
// (cap = la + lb + 2); res = {alen, mlen, wlen, maxcost}; returns the status.
int pa_emul_newkk_median(void* h, const uint8_t* a, int la, const uint8_t* b, int lb, int* cost,
                         uint8_t* ea, uint8_t* eb, uint8_t* med, uint8_t* mwg, int* res,
                         int* passes)
{
    const Emul& Em = *(Emul*)h;
    const Tables& t = Em.t;
    if (t.model != 1 || la < 1 || lb < 1) return -4;
    const int swaped = la <= lb ? 0 : 1;
    const uint8_t* s1 = swaped ? b : a;
    const uint8_t* s2 = swaped ? a : b;
    const int l1 = swaped ? lb : la, l2 = swaped ? la : lb;
    const int go = t.go > 0 ? t.go : 0;
    PairOut o{ea, eb, med, mwg, la + lb + 2};
    NkEmul E;
    const bool trivial = (long long)l1 * nk::MUCH_LONGER < l2;
    int kk = 0, npass = 0, status = 0;
    if (trivial) {
        *cost = nk::trivial_cost(t, s1, l1, s2, l2);
    } else {
        auto fill = [&](int kp, int& c, uint32_t& g) -> bool {
            c = nk_fill(E, t, s1, l1, s2, l2, kp, go, g);
            Em.rec.push_back(kp);
            Em.rec.push_back(tmax((int)(g & 0xffff), (int)(g >> 16)));
            return true;
        };
        Em.rec.clear();
        *cost = nk::drive(t, l1, l2, fill, kk, npass, status, Em.skip != 0);
    }
    *passes = npass;
    if (status) return status;
    NkDir dir{&E};
    PairRes r = nk::traceback(t, dir, trivial, kk, s1, l1, s2, l2, swaped, o);
    res[0] = r.alen;
    res[1] = r.mlen;
    res[2] = r.wlen;
    res[3] = r.maxcost;
    return r.status;
}

// The newkk pass loop of one pair: k and the larger gap counter of every
// fill run (at most maxp), the pass count in *npass; returns the fills run
// or a negative status.
int pa_emul_newkk_passes(void* h, const uint8_t* a, int la, const uint8_t* b, int lb, int* ks,
                         int* gns, int maxp, int* npass)
{
    const Emul& Em = *(Emul*)h;
    const int cap = la + lb + 2;
    std::vector<uint8_t> ea(cap), eb(cap), med(cap), mwg(cap);
    int cost = 0, res[4];
    const int rc = pa_emul_newkk_median(h, a, la, b, lb, &cost, ea.data(), eb.data(),
                                        med.data(), mwg.data(), res, npass);
    if (rc < 0 && rc != -4) return rc;
    const int nf = (int)Em.rec.size() / 2;
    for (int j = 0; j < nf && j < maxp; j++) {
        ks[j] = Em.rec[2 * j];
        gns[j] = Em.rec[2 * j + 1];
    }
    return nf;
}

// algn_CAML_simple_2 (caller's deltawh, s1 down the rows) followed by
// algn_CAML_backtrace_2d_limit from (st_s1, st_s2, algn_s1, algn_s2), as the
// per-call path runs them: the walk of lin_limit_walk over the kept fill.
// r1 / r2 end at index cap - 1; returns the walk's status.
int pa_emul_limit_walk(void* h, const uint8_t* s1, int l1, const uint8_t* s2, int l2,
                       int deltawh, int st_s1, int st_s2, int algn_s1, int algn_s2,
                       int swaped, uint8_t* r1, uint8_t* r2, int cap, int* len, int* cost)
{
    const Emul& E = *(Emul*)h;
    const PairPlan pl = plan_linear_deltawh(E.t, l1, l2, deltawh);
    std::vector<uint8_t> dm;
    int P, R, passes, cls;
    LinBand bd;
    const int st = lin_fill_doubling(E, pl, s1, s2, dm, P, R, bd, cost, &passes, &cls);
    if (st) return st;
    LinDmBytes rd{dm.data(), P, R};
    return lin_limit_walk(rd, bd, s1, s2, E.t.gap, st_s1, st_s2, algn_s1, algn_s2, swaped, r1,
                          r2, cap, len);
}

// The band doubling of one linear pair (DOS.median's plan) pass by pass:
// T, the gap count of the pass's fill and its pipeline class, for at most
// maxp passes; returns the number of passes (or a negative status).
int pa_emul_lin_passes(void* h, const uint8_t* a, int la, const uint8_t* b, int lb, int* Ts,
                       int* gaps, int* classes, int maxp)
{
    const Emul& E = *(Emul*)h;
    const Tables& t = E.t;
    PairPlan pl = plan_linear(t, count_gap_states(a, la, t.gap), la,
                              count_gap_states(b, lb, t.gap), lb);
    const uint8_t* x = pl.swaped ? b : a;
    const uint8_t* y = pl.swaped ? a : b;
    const int m = pl.m, n = pl.n;
    std::vector<uint8_t> dm;
    int T = pl.T0, np = 0;
    for (;;) {
        LinBand bd = lin_band(m, n, pl.full, pl.full ? 0 : band_p(T, m, n));
        int c = pick_class(E.lad[0], lin_wu(bd), n);
        if (c < 0) return -5;
        const int P = E.lad[0].P[c], R = E.lad[0].R[c];
        dm.assign((size_t)(m + n + 1) * P * R, 0);
        int cost = 0, g = 0;
        if (m == 1) {  // no rows: row 0 is the whole alignment (as the class kernels)
            g = n - 1;
        } else {
            switch (R) {
                case 2: lin_pass<2>(bd, P, t, x, y, dm.data(), &cost, &g); break;
                case 4: lin_pass<4>(bd, P, t, x, y, dm.data(), &cost, &g); break;
                default: lin_pass<8>(bd, P, t, x, y, dm.data(), &cost, &g); break;
            }
        }
        if (np < maxp) {
            Ts[np] = T;
            gaps[np] = g;
            classes[np] = c;
        }
        np++;
        if (pl.full || lin_done(T, m, n, g)) return np;
        T *= 2;
    }
}

// The per-pair bounds check prep_kernel runs before a pair touches any
// buffer (pair_bounds_status): 0, -6 or -2.
int pa_emul_pair_bounds(int la, int lb, int max_pair_len, long long out_off,
                        long long out_bytes, int has_out)
{
    return pair_bounds_status(la, lb, max_pair_len, out_off, out_bytes, has_out);
}

}  // extern "C"

// ---- three-sequence alignment (pa_ukk3.cuh), one triple on the host -------

#include "pa_ukk3.cuh"

extern "C" int pa_emul_powell_3d(const uint8_t* a, int la, const uint8_t* b, int lb,
                                 const uint8_t* c, int lc, int mm, int go, int ge, int D,
                                 uint8_t* ra, uint8_t* rb, uint8_t* rc, int cap, int* rlen,
                                 int* cost, long long* steps)
{
    u3::Model m;
    u3::model_init(m, mm, go, ge);
    const u3::Layout L = u3::layout(m, la - 1, lb - 1, lc - 1, D);
    std::vector<unsigned char> mem((size_t)L.bytes, 0);
    u3::Work w = u3::work_at(mem.data(), L);
    std::vector<u3::Frame> ring(u3::RING);
    std::vector<int> ring_tag(u3::RING, -1);
    w.ring = ring.data();
    w.ring_tag = ring_tag.data();
    u3::Machine mc(m, w, a, la - 1, b, lb - 1, c, lc - 1);
    int n = 0;
    const int d = mc.run(ra + cap, rb + cap, rc + cap, cap, &n);
    *rlen = n;
    *cost = d;
    *steps = mc.steps;
    return mc.status;
}

extern "C" long long pa_emul_powell_3d_bytes(int la, int lb, int lc, int mm, int go, int ge, int D)
{
    u3::Model m;
    u3::model_init(m, mm, go, ge);
    return u3::layout(m, la - 1, lb - 1, lc - 1, D).bytes;
}
