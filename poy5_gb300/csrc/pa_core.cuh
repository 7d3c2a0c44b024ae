// Core of the GB300 direct-optimization aligner: cell rules, band schedule,
// lane-pipeline step functions and tracebacks.
//
// Everything in this header is plain arithmetic on registers and pointers so
// that the same code is compiled into the CUDA kernels (pa_kernels.cu) and,
// for testing only, into a host build that replays the lane pipeline one lane
// at a time (tests/pa_emul.cpp).
//
// Fill layout ("lane pipeline"): a pipeline of P lanes (one CTA of P/32
// warps) aligns one pair. Lane g owns blocks of R consecutive rows; block b of
// the pair (rows 1 + bR .. bR + R) belongs to lane b mod P. All lanes step
// through anti-diagonals T = i + j together; at step T a lane computes cell
// (i, T - i) of each of its R rows that lies inside the band. Row q of a block
// reads its up/diagonal neighbours from row q-1 of the same lane (registers)
// and the top row reads them from the bottom row of lane g-1, which arrive by
// a rotating warp shuffle (shared memory across warp boundaries). Because the
// band shifts one column per row, a block of R rows is live for W + 2R - 2
// steps; the (P, R) pair is chosen so that the next block of the same lane
// (P*R rows further down) cannot start before the current one has drained
// (see band_fits).
//
// Direction codes are stored per step: dm[T * P*R + g*R + q], so every step of
// a warp is one contiguous store.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PA_HD __host__ __device__ __forceinline__
#define PA_HDM __host__ __device__ __forceinline__
#else
#define PA_HD static inline
#define PA_HDM inline
#endif

namespace pa {

constexpr int HIGH = 1000000;   // POY's "infinite" cost, src/algn.c:37
constexpr int NSTATE = 32;      // table rows: states < 1 << lcm, lcm <= 5
constexpr int CSW_STRIDE = 64;  // swizzled cost row: two copies of a row

// linear direction bits (src/matrices.h:22-27)
enum : int { L_ALIGN = 1, L_INSERT = 2, L_DELETE = 4 };

// affine direction flags (src/algn.c:1185-1199)
enum : int {
    A2A = 1, A2V = 2, A2H = 4, A2D = 8,
    BEG_B = 16, END_B = 32, BEG_V = 64, END_V = 128, BEG_H = 256, END_H = 512,
    DO_A = 1024, DO_V = 2048, DO_H = 4096, H_EQ_V = 8192, DO_D = 16384
};
constexpr int TMPGAP = 16;   // affine code hard-wires the DNA gap bit
constexpr int NTMPGAP = 15;

// Cost-matrix tables as the kernels see them (copied into shared memory).
// Costs are stored twice per row at a per-row rotation so that a warp whose
// lanes look up different (row, column) pairs of the DNA singletons hits 16
// different banks: cost(a, b) = csw[rowoff[a] + b].
struct Tables {
    int csw[NSTATE * CSW_STRIDE];
    int rowoff[NSTATE];
    int worst[NSTATE * NSTATE];
    int tail[NSTATE];
    int prepend[NSTATE];
    uint8_t median[NSTATE * NSTATE];
    int gap, lcm, go, mnz, comb, model, a_sz, pad;
};

PA_HD int tcost(const Tables& t, int a, int b) { return t.csw[t.rowoff[a] + b]; }
PA_HD int tmin(int a, int b) { return a < b ? a : b; }
PA_HD int tmax(int a, int b) { return a > b ? a : b; }

// per-halfword unsigned max of two packed u16 pairs
PA_HD uint32_t vmax2(uint32_t a, uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __vmaxu2(a, b);
#else
    uint32_t lo = tmax((int)(a & 0xFFFF), (int)(b & 0xFFFF));
    uint32_t hi = tmax((int)(a >> 16), (int)(b >> 16));
    return lo | (hi << 16);
#endif
}

// ---------------------------------------------------------------------------
// Pipeline shapes. A "class" is a (P lanes, R rows per lane) shape; a pair
// moves up its ladder as its band doubles. P < 32: 32/P pipelines share a
// warp (one pair each, shuffles of width P); P >= 32: P/32 warps of one CTA.
// Ladders are runtime data (a context may retune them; results do not
// depend on the ladder), drawn from the shapes the kernels are compiled for:
// P in {4, 8, ..., 512}, R in {2, 3, 4} (affine) or {2, 4, 8} (linear).
// Wider shapes are bounded by registers: a 512-thread CTA leaves 128
// registers per thread, enough for 8 linear or 4 affine rows per lane. A
// band of width w keeps w / (2 P R) of a class's lane-row slots busy, so
// the affine ladder interleaves R = 3 shapes between the powers of two.

constexpr int NCLASS = 12;

struct Ladder {
    int P[NCLASS];
    int R[NCLASS];
};

PA_HD Ladder default_ladder(int affine)
{
    Ladder L;
    const int lp[NCLASS] = {4, 8, 16, 32, 32, 32, 64, 128, 256, 512, 512, 512};
    const int lr[NCLASS] = {2, 2, 2, 2, 4, 8, 8, 8, 8, 8, 8, 8};
    const int ap[NCLASS] = {8, 8, 16, 16, 32, 32, 32, 64, 64, 128, 256, 512};
    const int ar[NCLASS] = {2, 3, 2, 3, 2, 3, 4, 3, 4, 4, 4, 4};
    for (int c = 0; c < NCLASS; c++) {
        L.P[c] = affine ? ap[c] : lp[c];
        L.R[c] = affine ? ar[c] : lr[c];
    }
    return L;
}

PA_HD int ladder_K(const Ladder& L, int c) { return L.P[c] >= 32 ? L.P[c] / 32 : 1; }

// A (P, R) pipeline processes a band of unclipped width wu over n columns
// without two blocks of one lane overlapping in time when either bound holds
// (next block start >= current block end + 2).
PA_HD bool band_fits(int P, int R, long long wu, int n)
{
    long long pr = (long long)(P - 1) * R;
    return (wu <= 2 * pr + 1) || (pr >= n);
}

// Band capacity of class c: 2 (P - 1) R + 1.
PA_HD long long ladder_cap(const Ladder& L, int c) { return 2LL * (L.P[c] - 1) * L.R[c] + 1; }

// Smallest class of the ladder for a band; -1 if none. wu < 0: full plane.
PA_HD int pick_class(const Ladder& L, long long wu, int n)
{
    for (int c = 0; c < NCLASS; c++)
        if (band_fits(L.P[c], L.R[c], wu < 0 ? (1LL << 40) : wu, n)) return c;
    return -1;
}

// Class of a lean affine band: classes up to 32 * RK_MAXK wide run on the
// row tile (band of unclipped width wu <= 32 K), wider ones on the lane
// pipeline.
constexpr int RK_MAXK = 16;  // widest row tile: 512 positions

// The tile width a class of capacity cap (2 (P - 1) R + 1) runs on, or 0
// for classes wider than RK_MAXK * 32 (lane pipeline).
PA_HD int rk_k_for(long long cap)
{
    for (int k = 1; k <= RK_MAXK; k <<= 1)
        if (32LL * k >= cap) return k;
    return 0;
}
PA_HD int pick_class_lean(const Ladder& L, long long wu, int n)
{
    for (int c = 0; c < NCLASS; c++) {
        const int k = rk_k_for(2LL * (L.P[c] - 1) * L.R[c] + 1);
        if (k > 0 ? wu <= 32LL * k : band_fits(L.P[c], L.R[c], wu, n)) return c;
    }
    return -1;
}

// A ladder the kernels can run: compiled shapes, and band capacity
// 2 (P - 1) R + 1 non-decreasing so that the last class is the widest.
PA_HD bool ladder_valid(const Ladder& L, int affine)
{
    long long prev = 0;
    for (int c = 0; c < NCLASS; c++) {
        const int P = L.P[c], R = L.R[c];
        if (P < 4 || P > 512 || (P & (P - 1))) return false;
        if (!(R == 2 || R == 4 || (affine ? R == 3 : R == 8))) return false;
        const long long cap = 2LL * (P - 1) * R + 1;
        if (cap < prev) return false;
        prev = cap;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Linear band (algn_newkk_test, src/algn.c:1063-1114; full plane :927-973)

struct LinBand {
    int m, n, D;    // rows (len of shorter incl. leading gap), cols, n - m
    int newk;       // band half-width (clipped to m - 1)
    int first;      // cells of row 0 that are filled
    int full;       // algn_fill_plane semantics
};

PA_HD LinBand lin_band(int m, int n, int full, int p)
{
    LinBand b;
    b.m = m;
    b.n = n;
    b.D = n - m;
    b.full = full;
    if (full) {
        b.newk = m - 1;
        b.first = n;
    } else {
        b.newk = p >= m ? m - 1 : p;
        int f = n - m + 1 + p;
        b.first = f > n ? n : f;
    }
    return b;
}
PA_HD int lin_hasL(const LinBand& b, int i) { return !b.full && (i - b.newk) > 0; }
PA_HD int lin_hasR(const LinBand& b, int i) { return !b.full && (i + b.D + b.newk) <= (b.n - 1); }
PA_HD int lin_s(const LinBand& b, int i) { return lin_hasL(b, i) ? i - b.newk : 0; }
PA_HD int lin_e(const LinBand& b, int i) { return lin_hasR(b, i) ? i + b.D + b.newk : b.n - 1; }
// unclipped width used to pick the pipeline class
PA_HD long long lin_wu(const LinBand& b) { return b.full ? -1 : (long long)b.D + 2LL * b.newk + 1; }

// Affine band (algn_newkk_test_aff, src/algn.c:2185-2306). Rows i = 1..m-1,
// columns 0..n-1 (the reference's leni = m-1, lenj = n-1).
struct AffBand {
    int m, n, D;
    int newk;       // clipped to leni - 1 = m - 2
};
PA_HD AffBand aff_band(int m, int n, int p)
{
    AffBand b;
    b.m = m;
    b.n = n;
    b.D = n - m;
    int lenX = m - 1;
    b.newk = p >= lenX ? lenX - 1 : p;
    return b;
}
PA_HD int aff_s(const AffBand& b, int i) { return (i - b.newk) > 0 ? i - b.newk : 0; }
PA_HD int aff_e(const AffBand& b, int i) { return tmin(b.n - 1, i + b.D + b.newk); }
PA_HD long long aff_wu(const AffBand& b) { return (long long)b.D + 2LL * b.newk + 1; }

// HAS_GAP_OPENING with gapstart <= 1 (src/algn.c:1236-1253)
PA_HD int gap_opening(int idx, int prev, int curr, int gap, int go)
{
    if (idx == 1 && (gap & curr)) return 0;
    if (idx > 1 && !(gap & prev) && (gap & curr)) return 0;
    return go;
}

// log2 of a power of two
PA_HD int log2_pow2(int x)
{
#if defined(__CUDA_ARCH__)
    return __ffs(x) - 1;
#else
    return __builtin_ctz((unsigned)x);
#endif
}

// Slab addressing shared by the fills and the tracebacks: row i >= 1 is row
// q of block b = (i - 1) / R, held by lane g = b mod P (P is a power of two
// in every ladder; R is 3 or a power of two).
PA_HD long long dm_index(int P, int R, int i, int j)
{
    const int b = R == 3 ? (i - 1) / 3 : (i - 1) >> log2_pow2(R);
    const int g = b & (P - 1);
    const int q = (i - 1) - b * R;
    return (long long)(i + j) * (P * R) + g * R + q;
}

// ---------------------------------------------------------------------------
// Linear lane state and step

template <int R>
struct LinLane {
    int V0[R], V1[R];       // cost of each row at two consecutive steps
    uint32_t N0[R], N1[R];  // forward gap counts (#ins | #del << 16), same steps
    int J[R], G[R];         // column symbol s2[j] and its insert cost
    int rb[R], dc[R], tl[R];// cost-row offset, delete and tail cost of the row symbol
    int Jn;                 // next step's column symbol of row 0 (loaded a step ahead)
    int Ts[R], Te[R];       // first / last step of each row (Ts > Te: no cell)
    int hr;                 // bit q: row q has a right border (no DELETE at Te)
    int R0, R1;             // neighbour's bottom row, two consecutive steps
    uint32_t RN0, RN1;
    int G0, G1;             // row 0 (lane 0 of the first block)
    int itop;               // first row of the current block
    int nstart;             // step at which the lane moves to its next block
};

PA_HD int block_start_step_lin(const LinBand& b, int itop)
{
    return itop <= b.m - 1 ? itop + lin_s(b, itop) : 0x7fffffff;
}

template <int R>
PA_HD void lin_enter_block(LinLane<R>& L, const LinBand& b, const Tables& t,
                           const uint8_t* s1, int itop, int P)
{
    L.itop = itop;
    L.hr = 0;
#pragma unroll
    for (int q = 0; q < R; q++) {
        const int i = itop + q;
        const bool real = i <= b.m - 1;
        const int c = real ? s1[i] : 0;
        L.rb[q] = t.rowoff[c];
        L.dc[q] = t.csw[t.rowoff[c] + t.gap];
        L.tl[q] = t.tail[c];
        L.Ts[q] = real ? i + lin_s(b, i) : 0x7fffffff;
        L.Te[q] = real ? i + lin_e(b, i) : -1;
        L.hr |= (real && lin_hasR(b, i)) ? 1 << q : 0;
    }
    L.nstart = block_start_step_lin(b, itop + P * R);
}

template <int R>
PA_HD void lin_lane_init(LinLane<R>& L, const LinBand& b, const Tables& t,
                         const uint8_t* s1, int g, int P)
{
#pragma unroll
    for (int q = 0; q < R; q++) {
        L.V0[q] = L.V1[q] = 0;
        L.N0[q] = L.N1[q] = 0;
        L.J[q] = 0;
        L.G[q] = 0;
    }
    L.R0 = L.R1 = L.G0 = L.G1 = 0;
    L.RN0 = L.RN1 = 0;
    lin_enter_block(L, b, t, s1, 1 + g * R, P);
    // step 1 reaches at most column 0 (lane 0), whose symbol no cell reads
    L.Jn = 0;
}

// Steps during which lane 0 still generates row 0 (its first block), rounded
// up to an even count so the step loop's register-set pairing is kept.
PA_HD int lin_gen_steps(const LinBand& b, int P, int R)
{
    const long long s = block_start_step_lin(b, 1 + P * R);
    const long long t = s > 0x7ffffff0LL ? 0x7ffffff0LL : s;
    return (int)((t + 1) & ~1LL);
}

// One anti-diagonal step of one lane (algn_fill_row and its border variants,
// src/algn.c:458-730). VC/NC/RC/RNC/GC hold step T-1, VP/NP/RP/RNP/GP step
// T-2; the step overwrites the latter, which become the caller's "T-1" set
// of the next step. recvV/recvN: bottom row of lane g-1 after step T-1.
// Each cell is the minimum of its candidates with the flags of every
// candidate equal to it (the reference's strict/equal comparison chains):
//  * column 0: DELETE only, costing the tail (band) or the gap cost (full);
//  * left border (j = s > 0): no INSERT; right border: no DELETE;
//  * last column without right border: the tail DELETE joins the DELETE
//    candidate (algn_fill_last_column).
// GEN = false promises that lane 0 has left its first block.
template <int R, bool GEN>
PA_HD void lin_step(LinLane<R>& L, int (&VC)[R], int (&VP)[R], uint32_t (&NC)[R],
                    uint32_t (&NP)[R], int& RC, int& RP, uint32_t& RNC, uint32_t& RNP,
                    int& GC, int& GP, const LinBand& b, const Tables& t, const uint8_t* s1,
                    const uint8_t* s2, int P, int T, int recvV, uint32_t recvN,
                    int (&dcode)[R])
{
    constexpr int BIG = 0x3fffffff;
    RP = recvV;
    RNP = recvN;
    const bool moved = (T >= L.nstart);
    if (moved) lin_enter_block(L, b, t, s1, L.itop + P * R, P);
    const bool gen = GEN && (L.itop == 1);
    if (gen) {  // row 0 at column T-1: prefix sums of the prepend costs
        const int j0 = T - 1;
        if (j0 == 0) GP = 0;
        else if (j0 < b.first) GP = GC + t.prepend[s2[j0]];
        else GP = GC;
    }
    if (moved) {  // a new block: every row needs its own column
#pragma unroll
        for (int q = 0; q < R; q++) {
            const int j = T - L.itop - q;
            const int c = (j >= 0 && j < b.n) ? s2[j] : 0;
            L.J[q] = c;
            L.G[q] = tcost(t, t.gap, c);
        }
    } else {  // row q takes row q-1's column of the previous step
#pragma unroll
        for (int q = R - 1; q > 0; q--) {
            L.J[q] = L.J[q - 1];
            L.G[q] = L.G[q - 1];
        }
        const int c = L.Jn;
        L.J[0] = c;
        L.G[0] = tcost(t, t.gap, c);
    }
    {  // the next step's row-0 column, loaded now so its latency overlaps this step
        const int jn = T + 1 - L.itop;
        L.Jn = (jn >= 0 && jn < b.n) ? s2[jn] : 0;
    }
#pragma unroll
    for (int q = R - 1; q >= 0; q--) {
        int upV, dgV;
        uint32_t upN, dgN;
        if (q > 0) {
            upV = VC[q - 1]; upN = NC[q - 1];
            dgV = VP[q - 1]; dgN = NP[q - 1];
        } else if (gen) {
            upV = GP; upN = (uint32_t)(T - 1);
            dgV = GC; dgN = (uint32_t)(T - 2);
        } else {
            upV = RP; upN = RNP;
            dgV = RC; dgN = RNC;
        }
        // Every row is computed every step, in its band or not: an in-band
        // cell reads an out-of-band neighbour only where the neighbour's
        // candidate is masked (left border: no INSERT; column 0: no ALIGN;
        // right border with a border bit: no DELETE), and no code outside
        // the band is ever read. All lookups stay in range for any row.
        const int i = L.itop + q;
        const bool c0 = (T == i);
        const bool hasR = (L.hr >> q) & 1;
        const bool lft = (T == L.Ts[q]) && !c0;
        const bool edge = (T == L.Te[q]);
        const int dlc = c0 ? (b.full ? L.dc[q] : L.tl[q]) : L.dc[q];
        const int aln = c0 ? BIG : dgV + t.csw[L.rb[q] + L.J[q]];
        const int ins = (c0 || lft) ? BIG : VC[q] + L.G[q];
        int del = (edge && hasR) ? BIG : upV + dlc;
        if (edge && !hasR && !c0) del = tmin(del, upV + L.tl[q]);
        const int v = tmin(tmin(aln, ins), del);
        const int d = (aln == v ? L_ALIGN : 0) | (ins == v ? L_INSERT : 0) |
                      (del == v ? L_DELETE : 0);
        // forward gap count along the path backtrace_2d_gaps follows
        NP[q] = (d & L_ALIGN) ? dgN : (d & L_INSERT) ? NC[q] + 1u : upN + 0x10000u;
        VP[q] = v;
        dcode[q] = d;
    }
}

// ---------------------------------------------------------------------------
// Affine lane state and step (algn_newkk_fill_a_row_aff, src/algn.c:2112-2180,
// cells :1220-1492, ASSIGN_MINIMUM :1935-1981, gap numbers :126-176)

struct AffCell {
    int EH, EV, EB, CB;
    uint32_t GM;  // gap numbers: gm1 | gm2 << 16
};

template <int R>
struct AffLane {
    AffCell V[R], Vp[R];
    int J[R], Jm[R];                 // sj[j], sj[j-1] for the row's column
    int sgext[R], sgop[R], svext[R]; // per-row constants
    int srb[R];                      // cost row of (row symbol & 15)
    int icf[R];                      // bit0: ic has gap, bit1: ip has gap, bit2: ic == ic & 15
    int itop, nstart;
    AffCell s, sp;                   // neighbour bottom row at T-1 / T-2
    AffCell g, gp;                   // row-0 generator (lane 0, first block)
    int gCB;                         // running CB of row 0
};

PA_HD int block_start_step_aff(const AffBand& b, int itop)
{
    return itop <= b.m - 1 ? itop + aff_s(b, itop) : 0x7fffffff;
}

template <int R>
PA_HD void aff_enter_block(AffLane<R>& L, const AffBand& b, const Tables& t,
                           const uint8_t* si, int itop, int P)
{
    L.itop = itop;
    const int gap = t.gap, go = t.go;
#pragma unroll
    for (int q = 0; q < R; q++) {
        int i = itop + q;
        int ic = 0, ip = 0;
        if (i <= b.m - 1) {
            ic = si[i];
            ip = si[i - 1];
        }
        int sg = tcost(t, ic, gap);
        int so = gap_opening(i, ip, ic, gap, go);
        L.sgext[q] = sg;
        L.sgop[q] = so;
        L.svext[q] = ((i > 1) && ((ip & gap) && !(ic & gap))) ? so + sg : sg;
        L.srb[q] = t.rowoff[NTMPGAP & ic];
        L.icf[q] = ((ic & TMPGAP) ? 1 : 0) | ((ip & TMPGAP) ? 2 : 0) | ((ic == (NTMPGAP & ic)) ? 4 : 0);
    }
    L.nstart = block_start_step_aff(b, itop + P * R);
}

template <int R>
PA_HD void aff_lane_init(AffLane<R>& L, const AffBand& b, const Tables& t,
                         const uint8_t* si, int g, int P)
{
    const AffCell z = {0, 0, 0, 0, 0u};
#pragma unroll
    for (int q = 0; q < R; q++) {
        L.V[q] = z;
        L.Vp[q] = z;
        L.J[q] = 0;
        L.Jm[q] = 0;
    }
    L.s = L.sp = L.g = L.gp = z;
    L.gCB = 0;
    aff_enter_block(L, b, t, si, 1 + g * R, P);
}

// shadow: EB of row 0 left in the base buffer by earlier doubling iterations
// (read at column j), and EH of row 0 column 0. The caller passes the state
// of the pair and receives the writes of this step through `shw_*`.
template <int R>
PA_HD void aff_step(AffLane<R>& L, const AffBand& b, const Tables& t,
                    const uint8_t* si, const uint8_t* sj, int P, int T,
                    const AffCell& recv, const int* shadowEB, int shadowEH0,
                    int* shadowEB_out, int (&dcode)[R])
{
    L.sp = L.s;
    L.s = recv;
    const bool moved = (T >= L.nstart);
    if (moved) aff_enter_block(L, b, t, si, L.itop + P * R, P);
    const int gap = t.gap, go = t.go;
    const bool gen = (L.itop == 1);
    if (gen) {  // row 0 at column T-1 (algn_newkk_test_aff init block)
        int j0 = T - 1;
        L.gp = L.g;
        if (j0 <= b.n - 1) {
            AffCell c;
            if (j0 == 0) {
                L.gCB = 0;
                c.EH = shadowEH0;
            } else {
                int cj = sj[j0], cm1 = sj[j0 - 1];
                int gr = t.prepend[cj];
                int gop = gap_opening(j0, cm1, cj, gap, go);
                int shx = ((cm1 & gap) && !(cj & gap)) ? gop + gr : gr;
                L.gCB += shx;
                c.EH = L.gCB;
            }
            c.CB = L.gCB;
            c.EV = HIGH;
            c.EB = shadowEB[j0];
            c.GM = (uint32_t)j0;
            L.g = c;
        }
    }
    if (moved) {
#pragma unroll
        for (int q = 0; q < R; q++) {
            int j = T - L.itop - q;
            L.J[q] = (j >= 0 && j < b.n) ? sj[j] : 0;
            L.Jm[q] = (j >= 1 && j - 1 < b.n) ? sj[j - 1] : 0;
        }
    } else {
#pragma unroll
        for (int q = R - 1; q > 0; q--) {
            L.J[q] = L.J[q - 1];
            L.Jm[q] = L.Jm[q - 1];
        }
        int j = T - L.itop;
        L.Jm[0] = L.J[0];
        L.J[0] = (j >= 0 && j < b.n) ? sj[j] : 0;
    }
    const int lenj = b.n - 1, leni = b.m - 1;
#pragma unroll
    for (int q = R - 1; q >= 0; q--) {
        const int i = L.itop + q;
        const int j = T - i;
        AffCell up, dg;
        if (q > 0) { up = L.V[q - 1]; dg = L.Vp[q - 1]; }
        else if (gen) { up = L.g; dg = L.gp; }
        else { up = L.s; dg = L.sp; }
        const AffCell lf = L.V[q];
        L.Vp[q] = L.V[q];
        dcode[q] = 0;
        if (i <= leni) {
            const int s = aff_s(b, i), e = aff_e(b, i);
            if (j >= s && j <= e) {
                const int right = (j == i + b.D + b.newk);
                const int left = (j == s);
                const int jc = L.J[q];
                const int jm = L.Jm[q];           // sj[j-1]
                const int jp = left ? jc : jm;    // fill_a_row_aff's jp quirk
                const int jgr = t.prepend[jc];
                const int jgop = j >= 1 ? gap_opening(j, jm, jc, gap, go) : 0;
                const int shx = (j == 1) ? jgr : (((jm & gap) && !(jc & gap)) ? jgop + jgr : jgr);
                const int f = L.icf[q];
                int dir = 0;
                AffCell c;
                if (!left) {
                    int ext = lf.EH + shx, open = lf.CB + jgop + jgr;
                    if (ext < open) { dir |= BEG_H; c.EH = ext; }
                    else { dir |= END_H; c.EH = open; }
                } else {
                    c.EH = HIGH;
                }
                if (!right) {
                    int ext = up.EV + L.svext[q], open = up.CB + L.sgop[q] + L.sgext[q];
                    if (ext < open) { dir |= BEG_V; c.EV = ext; }
                    else { dir |= END_V; c.EV = open; }
                } else {
                    c.EV = HIGH;
                }
                if (j > 0) {
                    const int flag = (f & 1) && (TMPGAP & jc);
                    const int flag2 = !(f & 2) && !(TMPGAP & jp);
                    const int diag = flag ? 0 : HIGH;
                    const int odiag = flag ? (flag2 ? 0 : 2 * go) : HIGH;
                    int ext = dg.EB + diag, open = dg.CB + odiag;
                    if (ext < open) { dir |= BEG_B; c.EB = ext; }
                    else { dir |= END_B; c.EB = open; }
                    const int dgc = t.csw[L.srb[q] + (NTMPGAP & jc)];
                    const int sgop = L.sgop[q];
                    const int xgo = (jgop < sgop) ? sgop : jgop;
                    const int algn = dg.CB + dgc;
                    const int fv = dg.EV + dgc + ((f & 4) ? 0 : jgop);
                    const int fh = dg.EH + dgc + ((jc == (NTMPGAP & jc)) ? 0 : sgop);
                    const int fd = dg.EB + dgc + xgo;
                    int v = algn, mask = A2A;
                    if (v >= fv) { if (v > fv) { v = fv; mask = A2V; } else mask |= A2V; }
                    if (v >= fh) { if (v > fh) { v = fh; mask = A2H; } else mask |= A2H; }
                    if (v >= fd) { if (v > fd) { v = fd; mask = A2D; } else mask |= A2D; }
                    c.CB = v;
                    dir |= mask;
                } else {
                    c.CB = HIGH;
                    c.EB = HIGH;
                }
                int fmin = c.EH, mask = DO_H;
                if (fmin >= c.EV) { if (fmin > c.EV) { fmin = c.EV; mask = DO_V; } else mask |= DO_V; }
                if (fmin >= c.EB) { if (fmin > c.EB) { fmin = c.EB; mask = DO_D; } else mask |= DO_D; }
                if (fmin >= c.CB) { if (fmin > c.CB) { fmin = c.CB; mask = DO_A; } else mask |= DO_A; }
                if (fmin == c.EH && c.EH == c.EV) mask |= H_EQ_V;
                dir |= mask;
                uint32_t gm = 0;
                if (dir & (DO_A | DO_D)) gm = dg.GM;
                if (dir & DO_H) gm = vmax2(gm, lf.GM + 1u);
                if (dir & DO_V) gm = vmax2(gm, up.GM + 0x10000u);
                c.GM = gm;
                L.V[q] = c;
                // EB left in row 0's buffer: the last even row >= 2 covering j
                if (shadowEB_out && (i & 1) == 0 && i >= 2 && i == (tmin(leni, j + b.newk) & ~1))
                    shadowEB_out[j] = c.EB;
                dcode[q] = dir;
                (void)fmin;
                (void)lenj;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Affine fast path for gap-free pairs: no state past position 0 of either
// sequence carries the gap bit (the usual DNA input). Under that condition
// the gap-dependent terms of the cell rules are exact constants:
// HAS_GAP_OPENING returns go for every row and column, sj_horizontal_extension
// is the prepend cost, si_vertical_extension the gap cost of the row symbol,
// FILL_CLOSE_BLOCK_DIAGONAL adds no opening to the vertical/horizontal
// predecessors and go to the diagonal one, and FILL_EXTEND_BLOCK_DIAGONAL
// adds HIGH to both of its candidates. Results are identical to aff_step;
// only the per-cell work is smaller.

template <int R>
struct AffFastLane {
    AffCell V[R], Vp[R];
    int J[R], JG[R];      // sj[j] and prepend[sj[j]] of the row's column
    int sgext[R];         // gap cost of the row symbol
    int srb[R];           // cost row of the row symbol
    int itop, nstart;
    AffCell s, sp;
    AffCell g, gp;
    int gCB;
};

template <int R>
PA_HD void aff_fast_enter_block(AffFastLane<R>& L, const AffBand& b, const Tables& t,
                                const uint8_t* si, int itop, int P)
{
    L.itop = itop;
#pragma unroll
    for (int q = 0; q < R; q++) {
        const int i = itop + q;
        const int ic = i <= b.m - 1 ? si[i] : 0;
        L.sgext[q] = tcost(t, ic, t.gap);
        L.srb[q] = t.rowoff[NTMPGAP & ic];
    }
    L.nstart = block_start_step_aff(b, itop + P * R);
}

template <int R>
PA_HD void aff_fast_lane_init(AffFastLane<R>& L, const AffBand& b, const Tables& t,
                              const uint8_t* si, int g, int P)
{
    const AffCell z = {0, 0, 0, 0, 0u};
#pragma unroll
    for (int q = 0; q < R; q++) {
        L.V[q] = z;
        L.Vp[q] = z;
        L.J[q] = 0;
        L.JG[q] = 0;
    }
    L.s = L.sp = L.g = L.gp = z;
    L.gCB = 0;
    aff_fast_enter_block(L, b, t, si, 1 + g * R, P);
}

template <int R>
PA_HD void aff_fast_step(AffFastLane<R>& L, const AffBand& b, const Tables& t,
                         const uint8_t* si, const uint8_t* sj, int P, int T,
                         const AffCell& recv, int* shadowEB, int shadowEH0,
                         int (&dcode)[R])
{
    L.sp = L.s;
    L.s = recv;
    const bool moved = (T >= L.nstart);
    if (moved) aff_fast_enter_block(L, b, t, si, L.itop + P * R, P);
    const int go = t.go;
    const bool gen = (L.itop == 1);
    if (gen) {  // row 0 at column T-1
        const int j0 = T - 1;
        L.gp = L.g;
        if (j0 <= b.n - 1) {
            AffCell c;
            if (j0 == 0) {
                L.gCB = 0;
                c.EH = shadowEH0;
            } else {
                // sj_horizontal_extension before its j = 1 override: the
                // leading gap followed by a base opens a gap at column 1
                const int cj = sj[j0];
                const int gr = t.prepend[cj];
                L.gCB += (j0 == 1 && (sj[0] & t.gap)) ? go + gr : gr;
                c.EH = L.gCB;
            }
            c.CB = L.gCB;
            c.EV = HIGH;
            c.EB = shadowEB[j0];
            c.GM = (uint32_t)j0;
            L.g = c;
        }
    }
    if (moved) {
#pragma unroll
        for (int q = 0; q < R; q++) {
            const int j = T - L.itop - q;
            const int c = (j >= 0 && j < b.n) ? sj[j] : 0;
            L.J[q] = c;
            L.JG[q] = t.prepend[c];
        }
    } else {
#pragma unroll
        for (int q = R - 1; q > 0; q--) {
            L.J[q] = L.J[q - 1];
            L.JG[q] = L.JG[q - 1];
        }
        const int j = T - L.itop;
        const int c = (j >= 0 && j < b.n) ? sj[j] : 0;
        L.J[0] = c;
        L.JG[0] = t.prepend[c];
    }
    const int leni = b.m - 1;
    const int kr = b.D + b.newk;  // right border: j == i + kr
#pragma unroll
    for (int q = R - 1; q >= 0; q--) {
        const int i = L.itop + q;
        const int j = T - i;
        AffCell up, dg;
        if (q > 0) { up = L.V[q - 1]; dg = L.Vp[q - 1]; }
        else if (gen) { up = L.g; dg = L.gp; }
        else { up = L.s; dg = L.sp; }
        const AffCell lf = L.V[q];
        L.Vp[q] = L.V[q];
        const int s = tmax(0, i - b.newk);
        const int e = tmin(b.n - 1, i + kr);
        dcode[q] = 0;
        if (i <= leni && j >= s && j <= e) {
            const int jgr = L.JG[q];
            int dir;
            AffCell c;
            // extend horizontal (left border: HIGH, no flag)
            {
                const int ext = lf.EH + jgr, open = lf.CB + go + jgr;
                const bool left = (j == s);
                c.EH = left ? HIGH : tmin(ext, open);
                dir = left ? 0 : (ext < open ? BEG_H : END_H);
            }
            // extend vertical (right border: HIGH, no flag)
            {
                const int sg = L.sgext[q];
                const int ext = up.EV + sg, open = up.CB + go + sg;
                const bool right = (j == i + kr);
                c.EV = right ? HIGH : tmin(ext, open);
                dir |= right ? 0 : (ext < open ? BEG_V : END_V);
            }
            if (j > 0) {
                const int ext = dg.EB + HIGH, open = dg.CB + HIGH;
                c.EB = tmin(ext, open);
                dir |= ext < open ? BEG_B : END_B;
                const int dgc = t.csw[L.srb[q] + (NTMPGAP & L.J[q])];
                const int algn = dg.CB + dgc, fv = dg.EV + dgc, fh = dg.EH + dgc;
                const int fd = dg.EB + dgc + go;
                int v = algn, mask = A2A;
                if (v >= fv) { if (v > fv) { v = fv; mask = A2V; } else mask |= A2V; }
                if (v >= fh) { if (v > fh) { v = fh; mask = A2H; } else mask |= A2H; }
                if (v >= fd) { if (v > fd) { v = fd; mask = A2D; } else mask |= A2D; }
                c.CB = v;
                dir |= mask;
            } else {
                c.CB = HIGH;
                c.EB = HIGH;
            }
            int f = c.EH, mask = DO_H;
            if (f >= c.EV) { if (f > c.EV) { f = c.EV; mask = DO_V; } else mask |= DO_V; }
            if (f >= c.EB) { if (f > c.EB) { f = c.EB; mask = DO_D; } else mask |= DO_D; }
            if (f >= c.CB) { if (f > c.CB) { f = c.CB; mask = DO_A; } else mask |= DO_A; }
            if (f == c.EH && c.EH == c.EV) mask |= H_EQ_V;
            dir |= mask;
            uint32_t gm = (dir & (DO_A | DO_D)) ? dg.GM : 0u;
            if (dir & DO_H) gm = vmax2(gm, lf.GM + 1u);
            if (dir & DO_V) gm = vmax2(gm, up.GM + 0x10000u);
            c.GM = gm;
            L.V[q] = c;
            if ((i & 1) == 0 && i >= 2 && i == (tmin(leni, j + b.newk) & ~1)) shadowEB[j] = c.EB;
            dcode[q] = dir;
        }
    }
}

// ---------------------------------------------------------------------------
// Affine fast path, register-lean form (gap-free pairs whose costs stay far
// below HIGH, see aff_lean_ok). Identical results to aff_step:
//  * every "keep the smaller, OR the flag on ties" chain of ASSIGN_MINIMUM
//    and FILL_CLOSE_BLOCK_DIAGONAL leaves exactly the flags of the candidates
//    equal to the final minimum, so the flags are equality tests against it;
//  * with no gap states the block-diagonal state only ever takes
//    min(EB, CB) + HIGH of its diagonal neighbour, so EB >= HIGH, while every
//    in-band cell (and row 0 and column 0) has EH, EV or CB below HIGH / 4:
//    EB never attains a minimum, DO_D and A2D are never set, and the
//    traceback never enters the block-diagonal mode. The lean cell drops EB
//    and stores only the direction bits the traceback then reads, one byte
//    per cell (LEAN_*);
//  * cell states ping-pong between two register sets (V0/V1, R0/R1, G0/G1)
//    and the caller alternates their roles on even and odd steps, so no
//    state is copied between steps.

struct LeanCell {
    int EH, EV, CB;
    uint32_t GM;  // gap numbers: gm1 | gm2 << 16
};

// direction byte of the lean path
enum : int {
    LEAN_A2V = 1, LEAN_A2H = 2, LEAN_END_V = 4, LEAN_END_H = 8,
    LEAN_DO_V = 16, LEAN_DO_H = 32, LEAN_H_EQ_V = 64
};

// the flags of a lean direction byte in the aff_step encoding (H_EQ_V: EH
// and EV both minimal, i.e. DO_H and DO_V)
PA_HD int lean_flags(int b)
{
    const bool hv = (b & (LEAN_DO_H | LEAN_DO_V)) == (LEAN_DO_H | LEAN_DO_V);
    return ((b & LEAN_A2V) ? A2V : 0) | ((b & LEAN_A2H) ? A2H : 0) |
           ((b & LEAN_END_V) ? END_V : 0) | ((b & LEAN_END_H) ? END_H : 0) |
           ((b & LEAN_DO_V) ? DO_V : 0) | ((b & LEAN_DO_H) ? DO_H : 0) |
           ((hv || (b & LEAN_H_EQ_V)) ? H_EQ_V : 0);
}

// min(a, b) and *le = (a <= b); min of three (DPX instructions on sm_90+)
PA_HD int bmin_le(int a, int b, bool* le)
{
#if defined(__CUDA_ARCH__)
    return __vibmin_s32(a, b, le);
#else
    *le = a <= b;
    return a <= b ? a : b;
#endif
}
PA_HD int min3(int a, int b, int c)
{
#if defined(__CUDA_ARCH__)
    return __vimin3_s32(a, b, c);
#else
    return tmin(tmin(a, b), c);
#endif
}
// per-halfword unsigned max of three packed u16 pairs
PA_HD uint32_t vmax3(uint32_t a, uint32_t b, uint32_t c)
{
#if defined(__CUDA_ARCH__)
    return __vimax3_u16x2(a, b, c);
#else
    return vmax2(vmax2(a, b), c);
#endif
}

template <int R>
struct AffLean {
    LeanCell V0[R], V1[R];  // row states of two consecutive steps
    LeanCell R0, R1;        // neighbour's bottom row, two consecutive steps
    LeanCell G0, G1;        // row 0 (lane 0 of the first block)
    int J[R], JG[R];        // column symbol and its prepend cost, per row
    int Ts[R], Te[R], Tr[R];// first / last / right-border step of each row
    int sg[R], sgo[R];      // gap cost of the row symbol (and + go)
    int srb[R];             // cost row of the row symbol
    int itop, nstart, gCB;
    int Jn;                 // next step's column symbol of row 0 (loaded a step ahead)
};

template <int R>
PA_HD void aff_lean_enter(AffLean<R>& L, const AffBand& b, const Tables& t,
                          const uint8_t* si, int itop, int P)
{
    L.itop = itop;
    const int kr = b.D + b.newk;
#pragma unroll
    for (int q = 0; q < R; q++) {
        const int i = itop + q;
        const bool real = i <= b.m - 1;
        const int ic = real ? si[i] : 0;
        const int sgv = tcost(t, ic, t.gap);
        L.sg[q] = sgv;
        L.sgo[q] = sgv + t.go;
        L.srb[q] = t.rowoff[ic];
        L.Ts[q] = real ? i + tmax(0, i - b.newk) : 0x7fffffff;
        L.Te[q] = real ? i + tmin(b.n - 1, i + kr) : -1;
        L.Tr[q] = 2 * i + kr;
    }
    L.nstart = block_start_step_aff(b, itop + P * R);
}

template <int R>
PA_HD void aff_lean_init(AffLean<R>& L, const AffBand& b, const Tables& t,
                         const uint8_t* si, int g, int P)
{
    const LeanCell z = {0, 0, 0, 0u};
#pragma unroll
    for (int q = 0; q < R; q++) {
        L.V0[q] = z;
        L.V1[q] = z;
        L.J[q] = 0;
        L.JG[q] = 0;
    }
    L.R0 = L.R1 = L.G0 = L.G1 = z;
    L.gCB = 0;
    aff_lean_enter(L, b, t, si, 1 + g * R, P);
    // step 1 reaches at most column 0 (lane 0), whose symbol no cell reads
    L.Jn = 0;
}

// The lean path needs every in-band cell to keep a state below HIGH / 4: a
// monotone path of at most n steps, each costing at most the largest
// substitution, insertion or deletion cost among gap-free states plus a gap
// opening, bounds the smallest state of every cell.
PA_HD bool aff_lean_ok(const Tables& t, int n)
{
    int mc = 0;
    for (int a = 0; a < 16; a++) {
        mc = tmax(mc, t.prepend[a]);
        mc = tmax(mc, tcost(t, a, t.gap));
        for (int c = 0; c < 16; c++) mc = tmax(mc, tcost(t, a, c));
    }
    if (t.go < 0 || mc < 0) return false;
    return (long long)n * (mc + t.go + 1) + t.go < HIGH / 4;
}

// One anti-diagonal step. VC/RC/GC hold step T-1 (up, left), VP/RP/GP hold
// step T-2 (diagonal); the step's results overwrite VP/RP/GP, which the
// caller then passes as VC/RC/GC of the next step. GEN = false promises that
// lane 0 has left its first block (T >= lean_gen_steps), so no lane
// generates row 0 any more.
template <int R, bool GEN>
PA_HD void aff_lean_step(AffLean<R>& L, LeanCell (&VC)[R], LeanCell (&VP)[R],
                         LeanCell& RC, LeanCell& RP, LeanCell& GC, LeanCell& GP,
                         const AffBand& b, const Tables& t, const uint8_t* si,
                         const uint8_t* sj, int P, int T, const LeanCell& recv,
                         int shadowEH0, int (&dcode)[R])
{
    RP = recv;  // neighbour bottom row at T-1 becomes this step's "up"
    const bool moved = (T >= L.nstart);
    if (moved) aff_lean_enter(L, b, t, si, L.itop + P * R, P);
    const int go = t.go;
    const bool gen = GEN && (L.itop == 1);
    if (gen) {  // row 0 at column T-1
        const int j0 = T - 1;
        if (j0 <= b.n - 1) {
            LeanCell c;
            if (j0 == 0) {
                L.gCB = 0;
                c.EH = shadowEH0;
            } else {
                const int gr = t.prepend[sj[j0]];
                L.gCB += (j0 == 1 && (sj[0] & t.gap)) ? go + gr : gr;
                c.EH = L.gCB;
            }
            c.CB = L.gCB;
            c.EV = HIGH;
            c.GM = (uint32_t)j0;
            GP = c;
        }
    }
    if (moved) {
#pragma unroll
        for (int q = 0; q < R; q++) {
            const int j = T - L.itop - q;
            const int c = (j >= 0 && j < b.n) ? sj[j] : 0;
            L.J[q] = c;
            L.JG[q] = t.prepend[c];
        }
    } else {
#pragma unroll
        for (int q = R - 1; q > 0; q--) {
            L.J[q] = L.J[q - 1];
            L.JG[q] = L.JG[q - 1];
        }
        const int c = L.Jn;
        L.J[0] = c;
        L.JG[0] = t.prepend[c];
    }
    {  // the next step's row-0 column, loaded now so its latency overlaps this step
        const int jn = T + 1 - L.itop;
        L.Jn = (jn >= 0 && jn < b.n) ? sj[jn] : 0;
    }
    // the "up" neighbours of row 0 are this step's received / generated
    // values (already in RP / GP); the diagonals are last step's (RC / GC)
#pragma unroll
    for (int q = R - 1; q >= 0; q--) {
        const LeanCell up = q > 0 ? VC[q - 1] : (gen ? GP : RP);
        const LeanCell dg = q > 0 ? VP[q - 1] : (gen ? GC : RC);
        const LeanCell& lf = VC[q];
        // Every row is computed every step, in its band or not. Outside its
        // band a row's state is never read by an in-band cell: a row's first
        // cell ignores its left neighbour (EH = HIGH, its H flags unread), an
        // up neighbour beyond the row above's band only occurs at the right
        // border (EV = HIGH), a diagonal one outside the band only at column
        // 0 (CB = HIGH), and the gap numbers take each neighbour only with
        // the state it decides; the codes of cells outside the band are
        // never read either. All lookups stay in range for any row.
        // Flags a traceback can never read are left unmasked: a row's first
        // cell is never in the H state, a right-border cell (EV = HIGH) never
        // in the V state, a column-0 cell (CB = HIGH) never in the D state;
        // H_EQ_V is DO_H and DO_V together (lean_flags).
        const int j = T - (L.itop + q);
        const int jgr = L.JG[q];
        LeanCell c;
        bool endh, endv;
        // EH: extend (left EH) vs open (left CB); END_H when open <= extend
        const int eh = bmin_le(lf.CB + go + jgr, lf.EH + jgr, &endh);
        const bool left = (T == L.Ts[q]);
        c.EH = left ? HIGH : eh;
        int code = endh ? LEAN_END_H : 0;
        const int ev = bmin_le(up.CB + L.sgo[q], up.EV + L.sg[q], &endv);
        const bool right = (T == L.Tr[q]);
        c.EV = right ? HIGH : ev;
        code |= endv ? LEAN_END_V : 0;
        // column 0 has no diagonal (CB = HIGH); J = sj[0] keeps the lookup
        // in range
        const int m3 = min3(dg.CB, dg.EV, dg.EH);
        const int dgc = t.csw[L.srb[q] + L.J[q]];
        c.CB = j > 0 ? m3 + dgc : HIGH;
        code |= (dg.EV == m3 ? LEAN_A2V : 0) | (dg.EH == m3 ? LEAN_A2H : 0);
        const int f = min3(c.EH, c.EV, c.CB);
        const bool hh = c.EH == f, vv = c.EV == f;
        code |= (hh ? LEAN_DO_H : 0) | (vv ? LEAN_DO_V : 0);
        c.GM = vmax3(c.CB == f ? dg.GM : 0u, hh ? lf.GM + 1u : 0u, vv ? up.GM + 0x10000u : 0u);
        VP[q] = c;
        dcode[q] = code;
    }
}

// Steps during which lane 0 still generates row 0 (its first block), rounded
// up to an even count so the step loop's register-set pairing is kept.
PA_HD int lean_gen_steps(const AffBand& b, int P, int R)
{
    const long long s = block_start_step_aff(b, 1 + P * R);
    const long long t = s > 0x7ffffff0LL ? 0x7ffffff0LL : s;
    return (int)((t + 1) & ~1LL);
}

// Final cost and gap count of the lean corner cell.
PA_HD int lean_final(const LeanCell& c) { return min3(c.EH, c.EV, c.CB); }
PA_HD int lean_gapnum(const LeanCell& c) { return tmax((int)(c.GM & 0xFFFF), (int)(c.GM >> 16)); }

// ---------------------------------------------------------------------------
// Row tile for the lean affine band ("row kernel"): one pair per warp, row
// after row. Lane l holds the band cells of skewed positions
// d = l * K + q (q < K), d = j - i + newk, so the band of every row lies in
// d in [0, 32 K) when its unclipped width wu = D + 2 newk + 1 <= 32 K. In
// skewed positions a cell's diagonal neighbour (i-1, j-1) sits at the same
// d and its up neighbour (i-1, j) at d + 1, both in the previous row, which
// the lanes keep in registers; the left neighbour (i, j-1) at d - 1 is in
// the same row: EH[j] = min(EH[j-1] + jgr, CB[j-1] + go + jgr) and the gap
// numbers GM[j] = max(a_j, hh_j ? GM[j-1] + 1 : 0) are solved per row by
// composing each lane's K maps and scanning the compositions across the
// warp (min-plus maps for EH, per-halfword max-plus maps for GM). Cells and
// flags are those of aff_lean_step; direction bytes are stored row-major,
// code(i, j) at dm[i * 32 K + d].

// x -> min(x + s, t), composed left to right
struct MinPlus {
    int s, t;
};
constexpr int MP_BIG = 1 << 29;  // "no path" inside a composed map; + HIGH stays < 2^31
PA_HD MinPlus mp_then(MinPlus f, MinPlus g)  // g after f
{
    return MinPlus{tmin(f.s + g.s, MP_BIG), tmin(tmin(f.t + g.s, MP_BIG), g.t)};
}
PA_HD int mp_apply(MinPlus f, int x) { return tmin(x + f.s, f.t); }

// x -> act ? vmax2(floor, x + add) : floor on packed u16 pairs (counts stay
// below 2^16, so max distributes over the addition)
struct GmMap {
    int act;
    uint32_t add, floor;
};
PA_HD GmMap gm_then(GmMap f, GmMap g)  // g after f
{
    if (!g.act) return g;
    if (!f.act) return GmMap{0, 0u, vmax2(g.floor, f.floor + g.add)};
    return GmMap{1, f.add + g.add, vmax2(g.floor, f.floor + g.add)};
}
PA_HD uint32_t gm_apply(GmMap g, uint32_t x) { return g.act ? vmax2(g.floor, x + g.add) : g.floor; }


// Row constants shared by the warp.
struct RkRow {
    int i, ic, sg, sgo, srow;
    int s, e, tr;  // band [s, e] of the row, right-border column tr
};
PA_HD RkRow rk_row(const AffBand& b, const Tables& t, const uint8_t* si, int i)
{
    RkRow r;
    r.i = i;
    r.ic = si[i];
    r.sg = tcost(t, r.ic, t.gap);
    r.sgo = r.sg + t.go;
    r.srow = t.rowoff[r.ic];
    r.s = tmax(0, i - b.newk);
    r.tr = i + b.D + b.newk;
    r.e = tmin(b.n - 1, r.tr);
    return r;
}

// Row 0 cell of position d (prefix sums of the prepend costs; CB and EH
// from the caller's scan). GM = j insertions.
PA_HD LeanCell rk_row0(int j, int cb, int shadowEH0)
{
    LeanCell c;
    c.CB = j == 0 ? 0 : cb;
    c.EH = j == 0 ? shadowEH0 : cb;
    c.EV = HIGH;
    c.GM = (uint32_t)tmax(j, 0);
    return c;
}
// prepend term of row 0's column j (j >= 1)
PA_HD int rk_row0_term(const Tables& t, const uint8_t* sj, int j)
{
    const int gr = t.prepend[sj[j]];
    return (j == 1 && (sj[0] & t.gap)) ? t.go + gr : gr;
}

// Phase A of one lane's K cells of row r (first column j0): EV and CB from
// the previous row (P: this lane's previous row, upn: the next lane's P[0]).
template <int K>
PA_HD void rk_phase_a(const LeanCell (&P)[K], const LeanCell& upn, const int (&J)[K],
                      const RkRow& r, const Tables& t, int j0, int (&EV)[K], int (&CB)[K],
                      int (&code)[K])
{
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = j0 + q;
        const LeanCell& up = q + 1 < K ? P[q + 1] : upn;
        const LeanCell& dg = P[q];
        bool endv;
        const int ev = bmin_le(up.CB + r.sgo, up.EV + r.sg, &endv);
        const bool right = j == r.tr;
        EV[q] = right ? HIGH : ev;
        const int m3 = min3(dg.CB, dg.EV, dg.EH);
        const int dgc = t.csw[r.srow + J[q]];
        CB[q] = j > 0 ? m3 + dgc : HIGH;
        code[q] = ((!right && endv) ? LEAN_END_V : 0) |
                  (j > 0 ? ((dg.EV == m3 ? LEAN_A2V : 0) | (dg.EH == m3 ? LEAN_A2H : 0)) : 0);
    }
}

// The lane's composed EH map (cbl: the current row's CB at this lane's
// d - 1, i.e. the previous lane's last CB).
template <int K>
PA_HD MinPlus rk_eh_map(const int (&JG)[K], const int (&CB)[K], const RkRow& r, int go, int j0,
                        int cbl)
{
    MinPlus f{0, MP_BIG};
    int cprev = cbl;
#pragma unroll
    for (int q = 0; q < K; q++) {
        const bool left = j0 + q == r.s;
        f = mp_then(f, left ? MinPlus{MP_BIG, HIGH}
                            : MinPlus{JG[q], tmin(cprev + go + JG[q], MP_BIG)});
        cprev = CB[q];
    }
    return f;
}

// Phase B: EH from the incoming EH[d-1] (x), the cell minima and flags, and
// the lane's composed gap-number map.
template <int K>
PA_HD GmMap rk_phase_b(const LeanCell (&P)[K], const LeanCell& upn, const int (&JG)[K],
                       const RkRow& r, const Tables& t, int j0, int x, int cbl,
                       const int (&EV)[K], const int (&CB)[K], int (&EH)[K], int (&code)[K],
                       int (&hv)[K], uint32_t (&fl)[K])
{
    const int go = t.go;
    GmMap g{1, 0u, 0u};
    int cprev = cbl;
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = j0 + q;
        const LeanCell& up = q + 1 < K ? P[q + 1] : upn;
        const LeanCell& dg = P[q];
        bool endh;
        const int eh = bmin_le(cprev + go + JG[q], x + JG[q], &endh);
        const bool left = j == r.s;
        EH[q] = left ? HIGH : eh;
        x = EH[q];
        cprev = CB[q];
        const int f = min3(EH[q], EV[q], CB[q]);
        const bool hh = EH[q] == f, vv = EV[q] == f;
        code[q] |= ((!left && endh) ? LEAN_END_H : 0) | (hh ? LEAN_DO_H : 0) |
                   (vv ? LEAN_DO_V : 0) | ((hh && vv) ? LEAN_H_EQ_V : 0);
        fl[q] = vmax2(CB[q] == f ? dg.GM : 0u, vv ? up.GM + 0x10000u : 0u);
        hv[q] = hh;
        g = gm_then(g, GmMap{hh ? 1 : 0, hh ? 1u : 0u, fl[q]});
    }
    return g;
}

// Phase C: gap numbers from the incoming GM[d-1] (y); the new row replaces P
// in band cells (cells outside the band keep their old state).
template <int K>
PA_HD void rk_phase_c(LeanCell (&P)[K], const RkRow& r, int j0, uint32_t y, const int (&EH)[K],
                      const int (&EV)[K], const int (&CB)[K], const int (&hv)[K],
                      const uint32_t (&fl)[K], int (&code)[K])
{
#pragma unroll
    for (int q = 0; q < K; q++) {
        const int j = j0 + q;
        y = hv[q] ? vmax2(fl[q], y + 1u) : fl[q];
        const bool in = j >= r.s && j <= r.e;
        if (in) {
            P[q].EH = EH[q];
            P[q].EV = EV[q];
            P[q].CB = CB[q];
            P[q].GM = y;
        } else {
            code[q] = 0;
        }
    }
}

// Final cost of the affine corner cell from its four states.
PA_HD int aff_final(const AffCell& c) { return tmin(tmin(c.EH, c.EV), tmin(c.EB, c.CB)); }
PA_HD int aff_gapnum(const AffCell& c) { return tmax((int)(c.GM & 0xFFFF), (int)(c.GM >> 16)); }

// ---------------------------------------------------------------------------
// Per-pair planning: the OCaml facade's argument order and plane choice, and
// the band-doubling schedule.

// count_gaps / seq_CAML_count (src/sequence.ml:854-865, src/seq.c:644-669)
PA_HD int count_gap_states(const uint8_t* s, int len, int gap)
{
    int n = 0;
    for (int i = 0; i < len; i++) n += (s[i] >= gap && (s[i] & gap)) ? 1 : 0;
    return n;
}

// Per-pair bounds of a batch, checked before a pair touches any buffer
// sized by the caller's declared shape: every direction slab holds a fill of
// m + n <= max_pair_len, and pair k's outputs and its affine row-0 shadow
// occupy [out_off, out_off + la + lb + 2) of buffers of out_bytes bytes
// (has_out = 0: the batch writes no per-pair outputs). Returns 0 when the
// pair fits, else the pair's status: -6 (longer than declared) or -2 (its
// output slot leaves the buffers).
PA_HD int pair_bounds_status(int la, int lb, int max_pair_len, long long out_off,
                             long long out_bytes, int has_out)
{
    if (la < 0 || lb < 0 || (long long)la + lb > (long long)max_pair_len) return -6;
    if (has_out && (out_off < 0 || out_off + la + lb + 2 > out_bytes)) return -2;
    return 0;
}

struct PairPlan {
    int swaped;  // caller's first sequence is the longer one
    int m, n;    // internal order: m = shorter length, n = longer
    int full;    // linear: algn_fill_plane instead of band doubling
    int T0;      // initial band parameter T
};

// Sequence.Align.cost_2 (src/sequence.ml:868-925, deltaw = None) feeding
// algn_nw_limit / algn_fill_plane_2 (src/algn.c:2954-2964, 1134-1177).
// int_of_float (0.1 * len) equals len / 10 for every int length, and the
// single-precision 1.5 test is exact for lengths below 2^24.
PA_HD PairPlan plan_linear(const Tables& t, int gaps_a, int la, int gaps_b, int lb)
{
    PairPlan p;
    p.swaped = la <= lb ? 0 : 1;
    p.m = p.swaped ? lb : la;
    p.n = p.swaped ? la : lb;
    const int gaps = tmax(gaps_a, gaps_b);
    const int lower = p.m / 10;
    const int dw = (p.m - p.n) < lower ? lower / 2 : 2;
    const int deltawh = gaps + dw;
    int height = (p.m - p.n) + 50 + deltawh;
    if (height > p.m) height = p.m;
    if (2LL * p.m >= 3LL * p.n) p.full = 1;
    else if (2 * height < p.m) p.full = 0;
    else p.full = (8 >= p.m - height) ? 1 : 0;
    p.T0 = (p.n - p.m + 1) * t.mnz;
    return p;
}

// SeqCS.DOS.distance (src/seqCS.ml:738-751) -> Sequence.Align.cost_2
// ~deltaw:(max 8 |la - lb|) (src/sequence.ml:868-925, the Some branch of
// deltaw_calc) feeding algn_nw_limit.
PA_HD PairPlan plan_linear_distance(const Tables& t, int gaps_a, int la, int gaps_b, int lb)
{
    PairPlan p;
    p.swaped = la <= lb ? 0 : 1;
    p.m = p.swaped ? lb : la;
    p.n = p.swaped ? la : lb;
    const int v = tmax(8, p.n - p.m);
    const int lower = p.m / 10;
    const int dw = (p.m - p.n) < lower ? lower : v;
    const int deltawh = tmax(gaps_a, gaps_b) + dw;
    int height = (p.m - p.n) + 50 + deltawh;
    if (height > p.m) height = p.m;
    if (2LL * p.m >= 3LL * p.n) p.full = 1;
    else if (2 * height < p.m) p.full = 0;
    else p.full = (8 >= p.m - height) ? 1 : 0;
    p.T0 = (p.n - p.m + 1) * t.mnz;
    return p;
}

// algn_nw called directly with s1 = a, s2 = b and the caller's deltawh
// (the algn_CAML_simple_2 external): no reordering.
PA_HD PairPlan plan_linear_deltawh(const Tables& t, int la, int lb, int deltawh)
{
    PairPlan p;
    p.swaped = 0;
    p.m = la;
    p.n = lb;
    int height = (p.m - p.n) + 50 + deltawh;
    if (height > p.m) height = p.m;
    if (2LL * p.m >= 3LL * p.n) p.full = 1;
    else if (2 * height < p.m) p.full = 0;
    else p.full = (8 >= p.m - height) ? 1 : 0;
    p.T0 = (p.n - p.m + 1) * t.mnz;
    return p;
}

// Sequence.Align.align_affine_3 (src/sequence.ml:633-649) + iniT of
// algn_fill_plane_3_aff (src/algn.c:2340-2354).
PA_HD PairPlan plan_affine(const Tables& t, int la, int lb)
{
    PairPlan p;
    p.swaped = la <= lb ? 0 : 1;
    p.m = p.swaped ? lb : la;
    p.n = p.swaped ? la : lb;
    p.full = 0;
    p.T0 = (p.n - p.m + 1) * t.mnz;
    return p;
}

PA_HD int band_p(int T, int m, int n) { return (T - (n - m)) / 2; }

// algn_newkk_increaseT stop rule (src/algn.c:1118-1130)
PA_HD bool lin_done(int T, int m, int n, int gapnum)
{
    const int p = band_p(T, m, n);
    const int newp = (2 * T - (n - m)) / 2;
    return (gapnum + 1) < p || newp - n + 1 >= 0;
}

// algn_newkk_increaseT_aff stop rule (src/algn.c:2310-2336); lenj = n - 1
PA_HD bool aff_done(int T, int m, int n, int gapnum)
{
    const int p = band_p(T, m, n);
    const int newp = (2 * T - (n - m)) / 2;
    return gapnum < p || newp - (n - 1) + 1 >= 0;
}

// The second clause of each stop rule alone: the doubling ends at band T
// whatever that pass's gap count is.
PA_HD bool lin_covers(int T, int m, int n) { return (2 * T - (n - m)) / 2 - n + 1 >= 0; }
PA_HD bool aff_covers(int T, int m, int n) { return (2 * T - (n - m)) / 2 - (n - 1) + 1 >= 0; }

// Leading passes of the doubling that cannot end it. Every path from (0, 0)
// to (m - 1, n - 1) takes n - m more horizontal steps than vertical ones,
// so the gap count a pass reports is at least n - m: the linear walk counts
// one path's insertions and deletions (backtrace_2d_gaps, src/algn.c:978-1005),
// and the affine counts are, per direction, the largest over the tied
// predecessors of path counts that start from row 0 / column 0
// (algn_fill_gapnum, src/algn.c:126-176). The gap test (gapnum + 1 < p
// linear, gapnum < p affine, p = (T - (n - m)) / 2) then needs
// T >= 3 (n - m) + 4 (linear) or 3 (n - m) + 2 (affine); a pass below that
// which does not cover the plane only fails its test. Such passes leave
// nothing a later pass reads in the linear model or on the lean affine
// cell (whose row-0 value is a function of the pass index), so those pairs
// start at T0 << s with s passes counted as run. At most maxp.
PA_HD int unstoppable_passes(int T0, int m, int n, bool affine, int maxp)
{
    const long long thr = 3LL * (n - m) + (affine ? 2 : 4);
    long long T = T0;
    int s = 0;
    while (s < maxp && T > 0 && T < thr &&
           !(affine ? aff_covers((int)T, m, n) : lin_covers((int)T, m, n))) {
        T *= 2;
        s++;
    }
    return s;
}

// ---------------------------------------------------------------------------
// Tracebacks and medians. Outputs are written back to front so that each
// sequence ends at index cap-1 of its buffer, as seq_prepend leaves them.

struct PairOut {
    uint8_t *ea, *eb, *med, *mwg;
    int cap;
};
struct PairRes {
    int alen, mlen, wlen, maxcost, status;
};

// Direction code of cell (i >= 1, j) of a linear slab.
struct LinDmBytes {
    const uint8_t* dm;
    int P, R;
    PA_HDM int operator()(int i, int j) const { return dm[dm_index(P, R, i, j)]; }
};

// backtrace_2d + algn_ancestor_2 + seq_get_median_2d_with_gaps + algn_worst_2
// (src/algn.c:3277-3327, 3602-3626, 3002-3105; src/seq.c:241-252), linear
// model. x = shorter (rows), y = longer; `swaped` = the caller passed y first.
// The traceback reads its codes through `rd`, which may be a shared-memory
// window that the calling warp refills together (every lane then runs the
// same traceback on the same data, so control flow stays uniform).
template <class DM>
PA_HD PairRes lin_traceback_dm(DM& rd, const Tables& t, const uint8_t* x, int m,
                               const uint8_t* y, int n, int swaped, const PairOut& o)
{
    PairRes r = {0, 0, 0, 0, 0};
    const int gap = t.gap, lcm = t.lcm;
    int i = m - 1, j = n - 1;
    int k = o.cap, ka = o.cap;
    int worst = 0, nga = 0, ngb = 0, wfirst = 0;
    int a = 0, bsym = 0;
    while (i >= 0) {
        if (k <= 0) { r.status = -2; return r; }
        const int d = i == 0 ? (j == 0 ? L_ALIGN : L_INSERT) : rd(i, j);
        int xs, ys;
        if (d & L_ALIGN) {
            xs = x[i--];
            ys = y[j--];
        } else {
            int ins = swaped ? (d & L_INSERT) != 0 : !(d & L_DELETE);
            if (ins) { xs = gap; ys = y[j--]; }
            else { xs = x[i--]; ys = gap; }
        }
        a = swaped ? ys : xs;
        bsym = swaped ? xs : ys;
        k--;
        o.ea[k] = (uint8_t)a;
        o.eb[k] = (uint8_t)bsym;
        int med = t.median[(a << lcm) + bsym];
        if (med == 0) { r.status = -3; return r; }
        o.mwg[k] = (uint8_t)med;
        if (med != gap) o.med[--ka] = (uint8_t)med;
        wfirst = t.worst[(a << lcm) + bsym];
        worst += wfirst;
        nga |= (a != gap);
        ngb |= (bsym != gap);
    }
    // the first aligned column is skipped when both carry the gap bit
    if ((gap & a) && (gap & bsym)) worst -= wfirst;
    o.med[--ka] = (uint8_t)gap;  // ancestor keeps a leading gap
    r.alen = o.cap - k;
    r.wlen = r.alen;
    r.mlen = o.cap - ka;
    r.maxcost = (nga && ngb) ? worst : 0;
    return r;
}

PA_HD PairRes lin_traceback(const uint8_t* dm, int P, int R, const Tables& t,
                            const uint8_t* x, int m, const uint8_t* y, int n,
                            int swaped, const PairOut& o)
{
    LinDmBytes rd{dm, P, R};
    return lin_traceback_dm(rd, t, x, m, y, n, swaped, o);
}

// A window of a linear slab for a traceback that one warp runs together
// (every lane walks the same path over the same data): the codes of rows
// [ilo, itop] on anti-diagonals (Ttop - LW_DIAG, Ttop], refilled by all
// lanes at once whenever the walk leaves it, so that a refill costs one
// round of independent loads instead of one dependent load per step. A path
// that enters at (itop, Ttop) stays inside for LW_DIAG - 1 anti-diagonals:
// each step lowers T by 1 or 2 and the row by at most 1. Row i of
// anti-diagonal T is byte (i - 1) mod (P R) of the step's P R bytes
// (dm_index), so the window's rows are LW_WORDS consecutive words (modulo
// the step) of every anti-diagonal. Needs P R a power of two (8 or more) and
// a 4-byte aligned slab. With P R < LW_ROWS the window holds whole
// anti-diagonals and rows alias modulo P R; the walk still reads the right
// byte because a path cell lies in the band, and at any step each of the
// P R slots holds the one band row that owns it (a band fits its class:
// fewer than P R rows cross one anti-diagonal).
constexpr int LW_DIAG = 64;
constexpr int LW_ROWS = 64;
constexpr int LW_WORDS = LW_ROWS / 4 + 1;
constexpr int LW_SMEM_WORDS = LW_DIAG * LW_WORDS;

template <bool POW2 = true>  // P R a power of two (every linear class)
struct LinDmWindow {
    const uint8_t* dm;
    uint32_t* win;   // LW_SMEM_WORDS words (shared memory on the device)
    int pr;          // P R, a multiple of 4 (a power of two on the linear ladder,
                     // 3 times one on the affine ladder's R = 3 classes)
    int prw;         // words per anti-diagonal, P R / 4
    int lane, nl;    // this lane, and the lanes that refill together
    int Ttop = -1, ilo = 0, itop = -1, w0 = 0;

    PA_HDM int slot(int i) const  // byte of row i >= 1 in its step
    {
        if constexpr (POW2) return (i - 1) & (pr - 1);
        else return (i - 1) % pr;
    }
    PA_HDM int wmod(int w) const  // w modulo the words of a step, w >= -prw
    {
        if constexpr (POW2) return w & (prw - 1);
        else return (w + prw) % prw;
    }
    PA_HDM void refill(int i, int T)
    {
#if defined(__CUDA_ARCH__)
        __syncwarp();  // every lane is done with the old window
#endif
        Ttop = T;
        itop = i;
        ilo = i - LW_ROWS + 1 > 1 ? i - LW_ROWS + 1 : 1;
        w0 = slot(ilo) >> 2;
        const uint32_t* d32 = reinterpret_cast<const uint32_t*>(dm);
        for (int e = lane; e < LW_SMEM_WORDS; e += nl) {
            const int dd = e / LW_WORDS, c = e - dd * LW_WORDS;
            const int t = Ttop - dd;
            win[e] = t >= 1 ? d32[(long long)t * prw + wmod(w0 + c - prw)] : 0u;
        }
#if defined(__CUDA_ARCH__)
        __syncwarp();
#endif
    }
    PA_HDM int operator()(int i, int j)
    {
        const int T = i + j;
        if (T > Ttop || T <= Ttop - LW_DIAG || i < ilo || i > itop) refill(i, T);
        const int off = slot(i);
        const int w = wmod((off >> 2) - w0);
        return (int)((win[(Ttop - T) * LW_WORDS + w] >> ((off & 3) * 8)) & 0xFFu);
    }
};

// Lean affine codes (one byte per cell, same slab layout) through the window.
template <bool POW2>
struct AffDmLeanWindow {
    LinDmWindow<POW2> w;
    PA_HDM int operator()(int i, int j) { return lean_flags(w(i, j)); }
};

// The class kernels' in-kernel traceback uses the window when the pipeline
// has a warp of its own (32 lanes or more).
PA_HD bool lin_window_ok(int P, int R) { return P * R >= LW_ROWS && P >= 32; }

// algn_CAML_backtrace_2d_limit from any start: backtrace_2d with st_s1,
// st_s2, algn_s1, algn_s2 (src/algn.c:3277-3327, 3448-3469) over the kept
// linear fill of s1 (m rows) against s2 (n columns) with band b. The walk
// keeps the reference's own arithmetic on a row-major matrix of row stride
// n: it starts at linear index st_s2 + n (algn_s1 - 1) + algn_s2 - 1, moves
// by -(n + 1) on ALIGN, -1 on an insertion and -n on a deletion (insertion
// before deletion when swaped, deletion first otherwise), takes s1 / s2 at
// counters that start at st_s1 + algn_s1 and st_s2 + algn_s2, and ends when
// the index drops below st_s2. Row 0 holds ALIGN at column 0 and INSERT up
// to its filled length. The pair is written back to front into
// r1 / r2[cap - len, cap). Returns 0; -2 when cap is exceeded; -14 when the
// walk reaches a cell the last fill never wrote (the reference reads what
// earlier alignments left in its workspace there); -15 when a counter
// leaves its sequence.
template <class DM>
PA_HD int lin_limit_walk(DM& rd, const LinBand& b, const uint8_t* s1, const uint8_t* s2,
                         int gap, int st_s1, int st_s2, int algn_s1, int algn_s2,
                         int swaped, uint8_t* r1, uint8_t* r2, int cap, int* len)
{
    const long long l = b.n;
    long long idx = (long long)st_s2 + l * (algn_s1 - 1) + algn_s2 - 1;
    long long a1 = (long long)algn_s1 + st_s1, a2 = (long long)algn_s2 + st_s2;
    int k = cap;
    *len = 0;
    while (idx >= st_s2) {
        if (idx < 0) return -14;
        const long long i = idx / l, j = idx - i * l;
        int d;
        if (i >= b.m) return -14;
        if (i == 0) {
            if (j >= b.first) return -14;
            d = j == 0 ? L_ALIGN : L_INSERT;
        } else {
            if (j < lin_s(b, (int)i) || j > lin_e(b, (int)i)) return -14;
            d = rd((int)i, (int)j);
        }
        if (k <= 0) return -2;
        int x, y;
        if (d & L_ALIGN) {
            if (a1 < 1 || a1 > b.m || a2 < 1 || a2 > b.n) return -15;
            x = s1[--a1];
            y = s2[--a2];
            idx -= l + 1;
        } else if (swaped ? (d & L_INSERT) != 0 : !(d & L_DELETE)) {
            if (a2 < 1 || a2 > b.n) return -15;
            x = gap;
            y = s2[--a2];
            idx -= 1;
        } else {
            if (a1 < 1 || a1 > b.m) return -15;
            x = s1[--a1];
            y = gap;
            idx -= l;
        }
        k--;
        r1[k] = (uint8_t)x;
        r2[k] = (uint8_t)y;
    }
    *len = cap - k;
    return 0;
}

// Direction flags of cell (i, j) from a slab of aff_step words or of lean
// bytes.
struct AffDmWords {
    const uint16_t* dm;
    int P, R;
    PA_HDM int operator()(int i, int j) const { return dm[dm_index(P, R, i, j)]; }
};
struct AffDmLean {
    const uint8_t* dm;
    int P, R;
    PA_HDM int operator()(int i, int j) const { return lean_flags(dm[dm_index(P, R, i, j)]); }
};
// row tile: code(i, j) at dm[i * S + j - i + newk]
struct AffDmRow {
    const uint8_t* dm;
    int S, newk;
    PA_HDM int operator()(int i, int j) const
    {
        return lean_flags(dm[(long long)i * S + (j - i + newk)]);
    }
};

// Row-tile codes through a window of whole rows that one warp walks
// together (every lane the same path): rows [ilo, itop] of the region (row
// i at i * S, contiguous), refilled by all lanes at once with 16-byte loads
// whenever the walk leaves them. A traceback only moves up or left, so a
// refill takes the current row and the `rows` - 1 above it. Needs a 16-byte
// aligned region of at least (i + 1) S bytes for every row i read.
struct alignas(16) Word16 {
    uint32_t v[4];
};
constexpr int RW_BYTES = 8192;  // row window of one warp
struct AffDmRowWindow {
    const uint8_t* dm;
    Word16* win;     // rows * S bytes (shared memory on the device)
    int S, newk, rows;
    int lane, nl;    // this lane, and the lanes that refill together
    int ilo = 1, itop = 0;  // empty

    PA_HDM void refill(int i)
    {
#if defined(__CUDA_ARCH__)
        __syncwarp();  // every lane is done with the old window
#endif
        itop = i;
        ilo = i - rows + 1 > 0 ? i - rows + 1 : 0;
        const Word16* src = reinterpret_cast<const Word16*>(dm + (long long)ilo * S);
        const int n16 = (itop - ilo + 1) * (S >> 4);
        for (int e = lane; e < n16; e += nl) win[e] = src[e];
#if defined(__CUDA_ARCH__)
        __syncwarp();
#endif
    }
    PA_HDM int operator()(int i, int j)
    {
        if (i < ilo || i > itop) refill(i);
        const uint8_t* w8 = reinterpret_cast<const uint8_t*>(win);
        return lean_flags(w8[(i - ilo) * S + (j - i + newk)]);
    }
};

// algn_calculate_from_2_aligned (src/algn.c:3003-3089), bitset alphabet:
// the cost of an aligned pair under table `cost` (a functor of two
// states), one gap opening per gap block of either sequence.
template <class COST>
PA_HD int aligned_cost_tbl(const Tables& t, const uint8_t* x, const uint8_t* y, int L,
                           const COST& cost)
{
    const int gap = t.gap, go = t.go;
    int i = ((gap & x[0]) && (gap & y[0])) ? 1 : 0, res = 0, st = 0;
    for (; i < L; i++) {
        int a = x[i], b = y[i];
        if (st == 0) {
            if ((a & gap) && !(b & gap)) { res += go; st = 1; }
            else if ((b & gap) && !(a & gap)) { res += go; st = 2; }
        } else if (st == 1) {
            if (!(a & gap)) {
                if ((b & gap) && !(a & gap)) { res += go; st = 2; }
                else st = 0;
            }
        } else {
            if (!(b & gap)) {
                if (a & gap) { res += go; st = 1; }
                else st = 0;
            }
        }
        res += cost(a, b);
    }
    return res;
}

struct WorstTbl {
    const Tables& t;
    PA_HDM int operator()(int a, int b) const { return t.worst[(a << t.lcm) + b]; }
};
struct CostTbl {
    const Tables& t;
    PA_HDM int operator()(int a, int b) const { return tcost(t, a, b); }
};

// algn_worst_2 (src/algn.c:3092-3097): the worst table
PA_HD int worst_aligned(const Tables& t, const uint8_t* x, const uint8_t* y, int L)
{
    return aligned_cost_tbl(t, x, y, L, WorstTbl{t});
}

// algn_verify_2 (src/algn.c:3099-3105): the cost table
PA_HD int verify_aligned(const Tables& t, const uint8_t* x, const uint8_t* y, int L)
{
    return aligned_cost_tbl(t, x, y, L, CostTbl{t});
}

// seq_get_median_2d_no_gaps (src/seq.c:259-272): the median of every
// column that is not the gap, after a leading gap; writes out[0, n) (out
// holds L + 1 bytes) and returns n.
PA_HD int median_no_gaps(const Tables& t, const uint8_t* x, const uint8_t* y, int L, uint8_t* out)
{
    int n = 0;
    out[n++] = (uint8_t)t.gap;
    for (int i = 0; i < L; i++) {
        const int m = t.median[(x[i] << t.lcm) + y[i]];
        if (m != t.gap) out[n++] = (uint8_t)m;
    }
    return n;
}

// algn_ancestor_2 (src/algn.c:3602-3626) on an aligned pair of length len:
// writes the ancestor to anc[0, n) (anc holds len + 1 bytes) and returns n.
// Linear models drop the gap columns and keep a leading gap; an affine
// model over a bitset alphabet keeps them for algn_correct_blocks_affine
// and algn_remove_gaps (src/algn.c:3530-3600).
PA_HD int ancestor_2(const Tables& t, const uint8_t* x, const uint8_t* y, int len, uint8_t* anc)
{
    const int gap = t.gap;
    const int drop = !t.comb || t.model != 1;
    int ka = len + 1;
    for (int i = len - 1; i >= 0; i--) {
        const int med = t.median[(x[i] << t.lcm) + y[i]];
        if (!drop || med != gap) anc[--ka] = (uint8_t)med;
    }
    int n = len + 1 - ka;
    for (int i = 0; i < n; i++) anc[i] = anc[ka + i];
    if (!t.comb || (t.model != 1 && (n == 0 || anc[0] != gap))) {
        for (int i = n; i > 0; i--) anc[i] = anc[i - 1];
        anc[0] = (uint8_t)gap;
        n++;
    } else if (t.comb) {
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
            } else if ((gap & ab) && (gap & bb) && (sb & gap) && (sb != gap) && ext && inside &&
                       !prev) {
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
    return n;
}

// backtrace_aff (src/algn.c:1714-1819) in internal order (x shorter), then
// the caller-order aligned pair and max_cost_2 on it.
template <class DM>
PA_HD PairRes aff_traceback_dm(DM& aff_dm, const Tables& t, const uint8_t* x, int m,
                               const uint8_t* y, int n, int swaped, const PairOut& o)
{
    PairRes r = {0, 0, 0, 0, 0};
    uint8_t* ri = swaped ? o.eb : o.ea;  // aligned x in caller order slot
    uint8_t* rj = swaped ? o.ea : o.eb;
    int i = m - 1, j = n - 1;
    int km = o.cap, kw = o.cap, kr = o.cap;
    int mode = 0;  // 0 todo, 1 vertical, 2 horizontal, 3 diagonal, 4 align
    int ic = x[i], jc = y[j];
    const int lcm = t.lcm;
#define PA_PUT(buf, k, v) do { if ((k) <= 0) { r.status = -2; return r; } (buf)[--(k)] = (uint8_t)(v); } while (0)
#define PA_PUTR(a, b) do { if (kr <= 0) { r.status = -2; return r; } kr--; ri[kr] = (uint8_t)(a); rj[kr] = (uint8_t)(b); } while (0)
    while (i != 0 && j != 0) {
        const int d = aff_dm(i, j);
        if (mode == 0) {
            int fv = d & DO_V, fh = d & DO_H, fd = d & DO_D;
            if (!swaped) mode = fv ? 1 : fh ? 2 : fd ? 3 : 4;
            else mode = fh ? 2 : fv ? 1 : fd ? 3 : 4;
        } else if (mode == 1) {
            if ((d & END_V) || (d & H_EQ_V)) mode = 0;
            if (!(ic & TMPGAP)) { PA_PUT(o.med, km, ic | TMPGAP); PA_PUT(o.mwg, kw, ic | TMPGAP); }
            else PA_PUT(o.mwg, kw, TMPGAP);
            PA_PUTR(ic, TMPGAP);
            i--;
            ic = x[i];
        } else if (mode == 2) {
            if ((d & END_H) || (d & H_EQ_V)) mode = 0;
            if (!(jc & TMPGAP)) { PA_PUT(o.med, km, jc | TMPGAP); PA_PUT(o.mwg, kw, jc | TMPGAP); }
            else PA_PUT(o.mwg, kw, TMPGAP);
            PA_PUTR(TMPGAP, jc);
            j--;
            jc = y[j];
        } else if (mode == 3) {
            if (d & END_B) mode = 0;
            PA_PUTR(ic, jc);
            PA_PUT(o.mwg, kw, TMPGAP);
            i--;
            j--;
            jc = y[j];
            ic = x[i];
        } else {
            int fd = d & A2D, fv = d & A2V, fh = d & A2H;
            if (!swaped) mode = fv ? 1 : fh ? 2 : fd ? 3 : 4;
            else mode = fh ? 2 : fv ? 1 : fd ? 3 : 4;
            int pm = t.median[((ic & NTMPGAP) << lcm) + (jc & NTMPGAP)];
            PA_PUT(o.med, km, pm);
            PA_PUT(o.mwg, kw, pm);
            PA_PUTR(ic, jc);
            i--;
            j--;
            jc = y[j];
            ic = x[i];
        }
    }
    while (i != 0) {
        if (!(ic & TMPGAP)) { PA_PUT(o.med, km, ic | TMPGAP); PA_PUT(o.mwg, kw, ic | TMPGAP); }
        else PA_PUT(o.mwg, kw, TMPGAP);
        PA_PUTR(ic, TMPGAP);
        i--;
        ic = x[i];
    }
    while (j != 0) {
        if (!(jc & TMPGAP)) { PA_PUT(o.med, km, jc | TMPGAP); PA_PUT(o.mwg, kw, jc | TMPGAP); }
        else PA_PUT(o.mwg, kw, TMPGAP);
        PA_PUTR(TMPGAP, jc);
        j--;
        jc = y[j];
    }
    PA_PUTR(TMPGAP, TMPGAP);
    PA_PUT(o.mwg, kw, TMPGAP);
    if (km == o.cap) { r.status = -4; return r; }  // empty median: undefined in POY
    if (TMPGAP != o.med[km]) PA_PUT(o.med, km, TMPGAP);
#undef PA_PUT
#undef PA_PUTR
    r.alen = o.cap - kr;
    r.mlen = o.cap - km;
    r.wlen = o.cap - kw;
    const uint8_t* ea = o.ea + kr;
    const uint8_t* eb = o.eb + kr;
    int nga = 0, ngb = 0;
    for (int k = 0; k < r.alen; k++) {
        nga |= ea[k] != t.gap;
        ngb |= eb[k] != t.gap;
    }
    r.maxcost = (nga && ngb) ? worst_aligned(t, ea, eb, r.alen) : 0;
    return r;
}

PA_HD PairRes aff_traceback(const uint16_t* dm, int P, int R, const Tables& t,
                            const uint8_t* x, int m, const uint8_t* y, int n, int swaped,
                            const PairOut& o)
{
    AffDmWords rd{dm, P, R};
    return aff_traceback_dm(rd, t, x, m, y, n, swaped, o);
}

PA_HD PairRes aff_traceback_lean(const uint8_t* dm, int P, int R, const Tables& t,
                                 const uint8_t* x, int m, const uint8_t* y, int n, int swaped,
                                 const PairOut& o)
{
    AffDmLean rd{dm, P, R};
    return aff_traceback_dm(rd, t, x, m, y, n, swaped, o);
}

PA_HD PairRes aff_traceback_rowtile(const uint8_t* dm, int S, int newk, const Tables& t,
                                    const uint8_t* x, int m, const uint8_t* y, int n, int swaped,
                                    const PairOut& o)
{
    AffDmRow rd{dm, S, newk};
    return aff_traceback_dm(rd, t, x, m, y, n, swaped, o);
}

}  // namespace pa
