/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- "the oracle".
 *
 * A C restatement of POY 5.1.1's direct-optimization pairwise alignment path
 * (linear and affine), written from the reference's behaviour for use as the
 * CPU checker of the CUDA library. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline arm load it; the product never links it.
 *
 * Parity pin: tests/test_oracle.py compares every function here with
 * the reference algn.c compiled unmodified (oracle/_ref), and the committed
 * golden fixtures in tests/golden/ were generated from that build.
 *
 * Reference behaviour followed (paths relative to the POY source tree):
 *   linear cell rules      src/algn.c:214-533 (algn_fill_row, asm = C twin)
 *   band edge cells        src/algn.c:543-730 (right / left / left-right /
 *                          last-column / first-row / first-cell)
 *   band row dispatch      src/algn.c:747-923, 1008-1031
 *   full plane             src/algn.c:927-973
 *   gap-count traceback    src/algn.c:978-1005
 *   band test / doubling   src/algn.c:1063-1130
 *   plane choice           src/algn.c:1134-1177, 2954-2975
 *   final traceback        src/algn.c:79-124, 3277-3327
 *   ancestor / medians     src/algn.c:3560-3626, src/seq.c:241-252
 *   worst cost             src/algn.c:3002-3105
 *   affine cells           src/algn.c:1220-1492, 1935-1981, 126-176
 *   affine init / band     src/algn.c:1866-1933, 2112-2354
 *   affine traceback       src/algn.c:1531-1619, 1714-1819
 *   affine entry           src/algn.c:2358-2447
 *   facade                 src/sequence.ml:633-649, 854-925, 1019-1082
 *   DOS.median             src/seqCS.ml:1053-1071
 *   Algn_Newkk (affine)    src/newkkonen.c:65-873 (cells), 1155-1172 and
 *                          1334-1446 (passes, trivial case), 1498-1766
 *                          (tracebacks); NewkkAlign.align_2 and DOS.median
 *                          with use_ukk, src/sequence.ml:1879-1901,
 *                          src/seqCS.ml:1043-1051
 */
#include <limits.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "poy_oracle.h"
#include "poy_tables.h"

#define HIGH 1000000 /* reference sentinel, src/algn.c:37 */

/* linear direction bits (src/matrices.h:22-27) */
enum { L_ALIGN = 1, L_INSERT = 2, L_DELETE = 4 };

/* affine direction flags (src/algn.c:1185-1199) */
enum {
    A2A = 1, A2V = 2, A2H = 4, A2D = 8,
    BEG_B = 16, END_B = 32, BEG_V = 64, END_V = 128, BEG_H = 256, END_H = 512,
    DO_A = 1024, DO_V = 2048, DO_H = 4096, H_EQ_V = 8192, DO_D = 16384
};
#define TMPGAP 16
#define NTMPGAP 15

static __thread char orc_err[256];
static int orc_check = 0;

void orc_set_check(int on) { orc_check = on; }
const char *orc_last_error(void) { return orc_err; }

static int fail(const char *msg)
{
    snprintf(orc_err, sizeof(orc_err), "%s", msg);
    return -1;
}

/* ------------------------------------------------------------------------ */
/* cost matrix                                                              */

typedef struct ocm {
    orc_tables t;
    int mnz; /* smallest positive cost (cm_get_min_non0_cost) */
} ocm;

void *orc_cm_new(const int *tcm, int alph, int gap_open)
{
    ocm *c = (ocm *)calloc(1, sizeof(ocm));
    if (!c) return NULL;
    if (orc_tables_build(&c->t, tcm, alph, gap_open)) {
        free(c);
        return NULL;
    }
    c->mnz = orc_min_non0_cost(&c->t);
    return c;
}

void orc_cm_free(void *cm) { free(cm); }

int orc_cm_tables(void *cm, int *cost, uint8_t *median, int *worst, int *tail,
                  int *prepend, int *info)
{
    ocm *c = (ocm *)cm;
    int n = 2 * (1 << c->t.lcm) * (1 << c->t.lcm);
    if (cost) memcpy(cost, c->t.cost, (size_t)n * sizeof(int));
    if (worst) memcpy(worst, c->t.worst, (size_t)n * sizeof(int));
    if (tail) memcpy(tail, c->t.tail, (size_t)n * sizeof(int));
    if (prepend) memcpy(prepend, c->t.prepend, (size_t)n * sizeof(int));
    if (median) memcpy(median, c->t.median, (size_t)n);
    if (info) {
        info[0] = c->t.lcm;
        info[1] = c->t.gap;
        info[2] = c->t.a_sz;
        info[3] = c->t.combinations;
        info[4] = c->t.cost_model;
        info[5] = c->t.gap_open;
    }
    return n;
}

static inline int C(const ocm *c, int a, int b) { return c->t.cost[(a << c->t.lcm) + b]; }

/* ------------------------------------------------------------------------ */
/* workspace                                                                */

typedef struct ows {
    /* linear: banded direction storage */
    uint8_t *ldm;
    size_t ldm_cap;
    int64_t *roff;
    int *rs, *re;
    int rows_cap;
    int *rowA, *rowB;
    int rowlen_cap;
    int lm, ln, lvalid; /* shape of the last linear fill */
    /* affine: same carve as the reference stub */
    int *abuf;
    size_t abuf_cap;
    uint16_t *adm;
    size_t adm_cap;
    uint16_t *gm[4];
    int gm_cap;
    int *abs_, *abe; /* band of each row in the last affine iteration */
    int arows_cap;
} ows;

void *orc_ws_new(void) { return calloc(1, sizeof(ows)); }

void orc_ws_free(void *p)
{
    ows *w = (ows *)p;
    if (!w) return;
    free(w->ldm);
    free(w->roff);
    free(w->rs);
    free(w->re);
    free(w->rowA);
    free(w->rowB);
    free(w->abuf);
    free(w->adm);
    for (int k = 0; k < 4; k++) free(w->gm[k]);
    free(w->abs_);
    free(w->abe);
    free(w);
}

#define GROW(ptr, cap, need, type)                                            \
    do {                                                                       \
        if ((size_t)(need) > (size_t)(cap)) {                                  \
            void *np_ = realloc((ptr), (size_t)(need) * sizeof(type));        \
            if (!np_) return fail("out of memory");                            \
            (ptr) = (type *)np_;                                               \
            (cap) = (need);                                                    \
        }                                                                      \
    } while (0)

/* ------------------------------------------------------------------------ */
/* linear fill: one band iteration (full = 0) or the whole plane (full = 1) */

static inline uint8_t *ldm_at(ows *w, int i, int j)
{
    if (j < w->rs[i] || j > w->re[i]) return NULL;
    return w->ldm + w->roff[i] + (j - w->rs[i]);
}

static int lin_fill(const ocm *c, ows *w, const uint8_t *s1, int m,
                    const uint8_t *s2, int n, int full, int p, int *cost_out)
{
    const int gap = c->t.gap, lcm = c->t.lcm;
    const int *tail = c->t.tail, *prep = c->t.prepend;
    int newk = full ? m - 1 : (p >= m ? m - 1 : p);
    int first = full ? n : n - m + 1 + p;
    if (first > n) first = n;

    if (m > w->rows_cap) {
        int *a = (int *)realloc(w->rs, (size_t)m * sizeof(int));
        if (!a) return fail("out of memory");
        w->rs = a;
        a = (int *)realloc(w->re, (size_t)m * sizeof(int));
        if (!a) return fail("out of memory");
        w->re = a;
        int64_t *o = (int64_t *)realloc(w->roff, (size_t)m * sizeof(int64_t));
        if (!o) return fail("out of memory");
        w->roff = o;
        w->rows_cap = m;
    }
    if (n > w->rowlen_cap) {
        int *a = (int *)realloc(w->rowA, (size_t)n * sizeof(int));
        if (!a) return fail("out of memory");
        w->rowA = a;
        a = (int *)realloc(w->rowB, (size_t)n * sizeof(int));
        if (!a) return fail("out of memory");
        w->rowB = a;
        w->rowlen_cap = n;
    }
    w->rs[0] = 0;
    w->re[0] = first - 1;
    int64_t tot = first;
    for (int i = 1; i < m; i++) {
        int s, e;
        if (full) {
            s = 0;
            e = n - 1;
        } else {
            s = (i - newk) > 0 ? i - newk : 0;
            e = (i + n - m + newk) <= (n - 1) ? i + n - m + newk : n - 1;
        }
        w->rs[i] = s;
        w->re[i] = e;
        w->roff[i] = tot;
        tot += e - s + 1;
    }
    w->roff[0] = 0;
    GROW(w->ldm, w->ldm_cap, tot, uint8_t);

    int *pm = w->rowA, *mm = w->rowB;
    pm[0] = 0;
    w->ldm[0] = L_ALIGN;
    for (int j = 1; j < first; j++) {
        pm[j] = pm[j - 1] + prep[s2[j]];
        w->ldm[j] = L_INSERT;
    }
    for (int i = 1; i < m; i++) {
        const int ic = s1[i];
        const int *crow = c->t.cost + (ic << lcm);
        const int *grow = c->t.cost + (gap << lcm);
        const int dcost = crow[gap]; /* s1[i] against a gap */
        const int tl = tail[ic];
        const int s = w->rs[i], e = w->re[i];
        /* border flags exactly as algn_newkk_test derives them */
        const int left = !full && (i - newk) > 0;
        const int right = !full && (i + n - m + newk) <= (n - 1);
        uint8_t *drow = w->ldm + w->roff[i] - s;
        for (int j = s; j <= e; j++) {
            int v, d;
            if (j == 0) {
                v = pm[0] + (full ? dcost : tl);
                d = L_DELETE;
            } else {
                const int aln = pm[j - 1] + crow[s2[j]];
                if (left && j == s) {
                    if (right && e == s) {
                        v = aln;
                        d = L_ALIGN;
                    } else {
                        const int del = pm[j] + dcost;
                        if (del < aln) { v = del; d = L_DELETE; }
                        else if (aln < del) { v = aln; d = L_ALIGN; }
                        else { v = del; d = L_ALIGN | L_DELETE; }
                    }
                } else if (right && j == e) {
                    const int ins = mm[j - 1] + grow[s2[j]];
                    if (ins < aln) { v = ins; d = L_INSERT; }
                    else if (aln < ins) { v = aln; d = L_ALIGN; }
                    else { v = aln; d = L_ALIGN | L_INSERT; }
                } else {
                    const int del = pm[j] + dcost;
                    const int ins = mm[j - 1] + grow[s2[j]];
                    v = aln < ins ? aln : ins;
                    if (del < v) v = del;
                    d = (aln == v ? L_ALIGN : 0) | (ins == v ? L_INSERT : 0) |
                        (del == v ? L_DELETE : 0);
                }
            }
            if (!right && j == n - 1 && j > 0) { /* last-column tail delete */
                const int cst = tl + pm[n - 1];
                if (cst < v) { v = cst; d = L_DELETE; }
                else if (cst == v) d |= L_DELETE;
            }
            mm[j] = v;
            drow[j] = (uint8_t)d;
        }
        int *t = pm;
        pm = mm;
        mm = t;
    }
    *cost_out = pm[n - 1];
    w->lm = m;
    w->ln = n;
    w->lvalid = 1;
    return 0;
}

/* backtrace_2d_gaps: preference ALIGN > INSERT > DELETE; max(#ins, #del) */
static int lin_gaps(ows *w, int *gap_num)
{
    int i = w->lm - 1, j = w->ln - 1, ni = 0, nd = 0;
    while (i >= 0) {
        uint8_t *d = ldm_at(w, i, j);
        if (!d) return fail("gap traceback left the band");
        if (*d & L_ALIGN) { i--; j--; }
        else if (*d & L_INSERT) { ni++; j--; }
        else { nd++; i--; }
    }
    *gap_num = nd > ni ? nd : ni;
    return 0;
}

/* algn_nw: s1 is the shorter sequence (m <= n). */
static int lin_cost(const ocm *c, ows *w, const uint8_t *s1, int m,
                    const uint8_t *s2, int n, int deltawh, int *cost)
{
    if (m > n) return fail("pass the shorter sequence first");
    if (m < 1) return fail("empty sequence");
    int height = (m - n) + 50 + deltawh;
    if (height > m) height = m;
    int full;
    if ((double)(float)m >= 1.5 * (double)(float)n) full = 1;
    else if (2 * height < m) full = 0;
    else full = (8 >= m - height);
    if (full) return lin_fill(c, w, s1, m, s2, n, 1, 0, cost);
    int T = (n - m + 1) * c->mnz;
    for (;;) {
        int p = (T - (n - m)) / 2, g;
        if (lin_fill(c, w, s1, m, s2, n, 0, p, cost)) return -1;
        if (lin_gaps(w, &g)) return -1;
        int newp = (2 * T - (n - m)) / 2;
        if ((g + 1) < p || newp - n + 1 >= 0) return 0;
        T *= 2;
    }
}

/* backtrace_2d on the last fill; output is written back to front into the
 * last `len` slots of r1/r2 (capacity cap), like seq_prepend. */
static int lin_backtrace(const ocm *c, ows *w, const uint8_t *s1,
                         const uint8_t *s2, int swap, uint8_t *r1, uint8_t *r2,
                         int cap, int *len)
{
    if (!w->lvalid) return fail("no alignment to trace back");
    const int gap = c->t.gap;
    int i = w->lm - 1, j = w->ln - 1, k = cap;
    while (i >= 0) {
        uint8_t *d = ldm_at(w, i, j);
        if (!d) return fail("traceback left the band");
        if (k <= 0) return fail("aligned sequence capacity exceeded");
        k--;
        if (*d & L_ALIGN) {
            r1[k] = s1[i--];
            r2[k] = s2[j--];
        } else {
            int ins = swap ? (*d & L_INSERT) != 0 : !(*d & L_DELETE);
            if (ins) {
                r1[k] = (uint8_t)gap;
                r2[k] = s2[j--];
            } else {
                r1[k] = s1[i--];
                r2[k] = (uint8_t)gap;
            }
        }
    }
    *len = cap - k;
    return 0;
}

int orc_simple_2(void *cm, void *ws, const uint8_t *s1, int l1,
                 const uint8_t *s2, int l2, int deltawh, int *cost)
{
    return lin_cost((ocm *)cm, (ows *)ws, s1, l1, s2, l2, deltawh, cost);
}

int orc_backtrace_2d(void *cm, void *ws, const uint8_t *s1, int l1,
                     const uint8_t *s2, int l2, int swap, uint8_t *r1,
                     uint8_t *r2, int cap, int *len)
{
    ows *w = (ows *)ws;
    if (w->lm != l1 || w->ln != l2) return fail("backtrace shape mismatch");
    uint8_t *t1 = (uint8_t *)malloc((size_t)cap), *t2 = (uint8_t *)malloc((size_t)cap);
    int rc = lin_backtrace((ocm *)cm, w, s1, s2, swap, t1, t2, cap, len);
    if (!rc) {
        memcpy(r1, t1 + cap - *len, (size_t)*len);
        memcpy(r2, t2 + cap - *len, (size_t)*len);
    }
    free(t1);
    free(t2);
    return rc;
}

/* count_gaps (src/sequence.ml:854-865 -> seq_CAML_count, src/seq.c:644-669) */
static int count_gaps(const uint8_t *s, int len, int gap)
{
    int n = 0;
    for (int i = 0; i < len; i++)
        if (s[i] >= gap && (s[i] & gap)) n++;
    return n;
}

/* Align.cost_2, linear: deltaw < 0 is the None branch */
static int facade_cost2(const ocm *c, ows *w, const uint8_t *a, int la,
                        const uint8_t *b, int lb, int deltaw, int *cost)
{
    int g1 = count_gaps(a, la, c->t.gap), g2 = count_gaps(b, lb, c->t.gap);
    int gaps = g1 > g2 ? g1 : g2;
    int sl = la <= lb ? la : lb, ll = la <= lb ? lb : la;
    int dif = sl - ll, lower = (int)((double)sl * 0.10), dw;
    if (deltaw < 0) dw = dif < lower ? lower / 2 : 2;
    else dw = dif < lower ? lower : deltaw;
    if (la <= lb) return lin_cost(c, w, a, la, b, lb, gaps + dw, cost);
    return lin_cost(c, w, b, lb, a, la, gaps + dw, cost);
}

int orc_cost_linear(void *cm, void *ws, const uint8_t *a, int la,
                    const uint8_t *b, int lb, int deltaw, int *cost)
{
    return facade_cost2((ocm *)cm, (ows *)ws, a, la, b, lb, deltaw, cost);
}

/* algn_calculate_from_2_aligned with the worst table, bitset alphabet */
static int worst_2(const ocm *c, const uint8_t *x, const uint8_t *y, int L)
{
    const int gap = c->t.gap, go = c->t.gap_open;
    int i = ((gap & x[0]) && (gap & y[0])) ? 1 : 0, res = 0, state = 0;
    for (; i < L; i++) {
        int a = x[i], b = y[i];
        if (state == 0) {
            if ((a & gap) && !(b & gap)) { res += go; state = 1; }
            else if ((b & gap) && !(a & gap)) { res += go; state = 2; }
        } else if (state == 1) {
            if (!(a & gap)) {
                if ((b & gap) && !(a & gap)) { res += go; state = 2; }
                else state = 0;
            }
        } else {
            if (!(b & gap)) {
                if (a & gap) { res += go; state = 1; }
                else state = 0;
            }
        }
        res += c->t.worst[(a << c->t.lcm) + b];
    }
    return res;
}

static int all_gaps(const uint8_t *s, int L, int gap)
{
    for (int i = 0; i < L; i++)
        if (s[i] != gap) return 0;
    return 1;
}

/* algn_remove_gaps + algn_correct_blocks_affine (src/algn.c:3530-3600),
 * applied by algn_ancestor_2 for combination alphabets under an affine
 * model. s holds n states; returns the new length (compacted in place). */
static int correct_blocks_affine(int gap, uint8_t *s, int n, const uint8_t *a,
                                 const uint8_t *b)
{
    int inside = 0, prev = 0, ext = 0;
    for (int i = 0; i < n; i++) {
        int ab = a[i], bb = b[i], sb = s[i];
        if (!inside && (!(ab & gap) || !(bb & gap))) inside = 0;
        else if (inside && ((!(ab & gap)) || (!(bb & gap)))) inside = 0;
        else if (((ab & gap) || (bb & gap)) && ((ab != gap) || (bb != gap))) inside = 1;
        else inside = 0;
        if (((gap & ab) || (gap & bb)) && (!(sb & gap)) && !ext) {
            prev = inside;
            ext = 1;
        } else if ((gap & ab) && (gap & bb) && (sb & gap) && (sb != gap) &&
                   ext && inside && !prev) {
            sb = (~gap) & sb;
            prev = 0;
        } else if ((gap & ab) && (gap & bb) && (1 == ext)) {
            prev = inside;
            ext = 0;
        }
        s[i] = (uint8_t)sb;
    }
    /* algn_remove_gaps: drop every `gap` entry, then restore a leading gap */
    int k = 0;
    for (int i = 0; i < n; i++)
        if (s[i] != gap) s[k++] = s[i];
    memmove(s + 1, s, (size_t)k);
    s[0] = (uint8_t)gap;
    return k + 1;
}

/* algn_ancestor_2: anc must hold L + 1 entries; returns the length. */
static int ancestor_2(const ocm *c, const uint8_t *x, const uint8_t *y, int L,
                      uint8_t *anc, int *len)
{
    const int gap = c->t.gap;
    const int drop = !c->t.combinations || c->t.cost_model != 1;
    int k = L + 1; /* prepend into [0, L+1) */
    for (int i = L - 1; i >= 0; i--) {
        int med = c->t.median[(x[i] << c->t.lcm) + y[i]];
        if (med == 0) return fail("median should not be 0");
        if (drop) {
            if (med != gap) anc[--k] = (uint8_t)med;
        } else {
            anc[--k] = (uint8_t)med;
        }
    }
    int n = L + 1 - k;
    memmove(anc, anc + k, (size_t)n);
    if (!c->t.combinations ||
        (c->t.cost_model != 1 && (n == 0 || anc[0] != gap))) {
        memmove(anc + 1, anc, (size_t)n);
        anc[0] = (uint8_t)gap;
        n++;
    } else if (c->t.combinations) {
        n = correct_blocks_affine(gap, anc, n, x, y);
    }
    *len = n;
    return 0;
}

int orc_median_linear(void *cm, void *ws, const uint8_t *a, int la,
                      const uint8_t *b, int lb, int *cost, uint8_t *ea,
                      uint8_t *eb, int *elen, uint8_t *anc, int *anclen,
                      uint8_t *mwg, int *mwglen, int *maxcost)
{
    ocm *c = (ocm *)cm;
    ows *w = (ows *)ws;
    if (facade_cost2(c, w, a, la, b, lb, -1, cost)) return -1;
    int cap = la + lb, L;
    uint8_t *t1 = (uint8_t *)malloc((size_t)cap), *t2 = (uint8_t *)malloc((size_t)cap);
    int rc;
    if (la <= lb) rc = lin_backtrace(c, w, a, b, 0, t1, t2, cap, &L);
    else rc = lin_backtrace(c, w, b, a, 1, t2, t1, cap, &L);
    if (!rc) {
        memcpy(ea, t1 + cap - L, (size_t)L);
        memcpy(eb, t2 + cap - L, (size_t)L);
        *elen = L;
        rc = ancestor_2(c, ea, eb, L, anc, anclen);
    }
    if (!rc) {
        for (int i = 0; i < L; i++) mwg[i] = c->t.median[(ea[i] << c->t.lcm) + eb[i]];
        *mwglen = L;
        int gap = c->t.gap;
        *maxcost = (all_gaps(ea, L, gap) || all_gaps(eb, L, gap)) ? 0 : worst_2(c, ea, eb, L);
    }
    free(t1);
    free(t2);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* affine                                                                   */

static inline int gap_opening(int idx, int prev, int curr, int gap, int go)
{
    /* HAS_GAP_OPENING with gapstart <= 1 (src/algn.c:1236-1253) */
    if (idx == 1 && (gap & curr)) return 0;
    if (idx > 1 && !(gap & prev) && (gap & curr)) return 0;
    return go;
}

/* one band iteration of algn_newkk_test_aff; leni/lenj are lengths - 1 */
static int aff_test(const ocm *c, ows *w, const uint8_t *si, int leni,
                    const uint8_t *sj, int lenj, int p, int *res_cost,
                    int *gap_num)
{
    const int gap = c->t.gap, go = c->t.gap_open, lcm = c->t.lcm;
    const int L = lenj + 2; /* row stride of every array */
    int *CB = w->abuf, *EB = w->abuf + 2 * L, *EV = w->abuf + 4 * L,
        *EH = w->abuf + 6 * L, *FIN = w->abuf + 8 * L,
        *GOP = w->abuf + 10 * L, *SHX = w->abuf + 11 * L;
    int *pCB = CB + L, *pEB = EB + L, *pEV = EV + L, *pEH = EH + L;
    uint16_t *g1 = w->gm[0], *ng1 = w->gm[1], *g2 = w->gm[2], *ng2 = w->gm[3];
    uint16_t *dm = w->adm;
    const int lenX = leni, lenY = lenj, D = lenY - lenX;
    const int newk = p >= lenX ? lenX - 1 : p;
    const int *gaprow = c->t.prepend; /* prec row 0 = prepend[sj[j]] */

    EV[0] = HIGH;
    CB[0] = 0;
    SHX[0] = 0;
    g1[0] = 0;
    g2[0] = 0;
    for (int j = 1; j <= lenj; j++) {
        GOP[j] = gap_opening(j, sj[j - 1], sj[j], gap, go);
        if ((sj[j - 1] & gap) && !(sj[j] & gap)) SHX[j] = GOP[j] + gaprow[sj[j]];
        else SHX[j] = gaprow[sj[j]];
        g1[j] = (uint16_t)j;
        g2[j] = 0;
        ng1[j] = 0xFFFF;
        ng2[j] = 0xFFFF;
        dm[j] = DO_H;
        EV[j] = HIGH;
        CB[j] = CB[j - 1] + SHX[j];
        EH[j] = CB[j];
    }
    if (lenj >= 1) SHX[1] = gaprow[sj[1]];

    int ic = si[0];
    for (int i = 1; i <= leni; i++) {
        uint16_t *cdm = dm + (size_t)i * L;
        const int s = (i - newk) > 0 ? i - newk : 0;
        const int e = (i + lenY - lenX + newk) <= (lenY - 1) ? i + D + newk : lenY;
        if (orc_check) {
            w->abs_[i] = s;
            w->abe[i] = e;
        }
        int *t;
        t = pEH; pEH = EH; EH = t;
        t = pEV; pEV = EV; EV = t;
        t = pEB; pEB = EB; EB = t;
        t = pCB; pCB = CB; CB = t;
        const int ip = ic;
        ic = si[i];
        const int sgext = C(c, ic, gap);
        const int sgop = gap_opening(i, ip, ic, gap, go);
        const int sng = NTMPGAP & ic;
        const int *srow = c->t.cost + (sng << lcm);
        const int svext = ((i > 1) && ((ip & gap) && !(ic & gap))) ? sgop + sgext : sgext;
        int jc = sj[s];
        for (int j = s; j <= e; j++) {
            const int right = (j - i - (lenY - lenX + 1) + 1 == newk);
            const int left = (j == s);
            const int jp = jc;
            jc = sj[j];
            int dir = 0;
            const int jng = NTMPGAP & jc;
            const int jgext = gaprow[jc], jgop = GOP[j];
            if (!left) {
                int ext = EH[j - 1] + SHX[j], open = CB[j - 1] + jgop + jgext;
                if (ext < open) { dir |= BEG_H; EH[j] = ext; }
                else { dir |= END_H; EH[j] = open; }
            } else {
                EH[j] = HIGH;
            }
            if (!right) {
                int ext = pEV[j] + svext, open = pCB[j] + sgop + sgext;
                if (ext < open) { dir |= BEG_V; EV[j] = ext; }
                else { dir |= END_V; EV[j] = open; }
            } else {
                EV[j] = HIGH;
            }
            if (j > 0) {
                const int flag = (TMPGAP & ic) && (TMPGAP & jc);
                const int flag2 = !(TMPGAP & ip) && !(TMPGAP & jp);
                const int diag = flag ? 0 : HIGH;
                const int odiag = flag ? (flag2 ? 0 : 2 * go) : HIGH;
                int ext = pEB[j - 1] + diag, open = pCB[j - 1] + odiag;
                if (ext < open) { dir |= BEG_B; EB[j] = ext; }
                else { dir |= END_B; EB[j] = open; }

                const int dg = srow[jng];
                const int xgo = (jgop < sgop) ? sgop : jgop;
                const int algn = pCB[j - 1] + dg;
                const int fv = pEV[j - 1] + dg + ((ic == sng) ? 0 : jgop);
                const int fh = pEH[j - 1] + dg + ((jc == jng) ? 0 : sgop);
                const int fd = pEB[j - 1] + dg + xgo;
                int v = algn, mask = A2A;
                if (v >= fv) { if (v > fv) { v = fv; mask = A2V; } else mask |= A2V; }
                if (v >= fh) { if (v > fh) { v = fh; mask = A2H; } else mask |= A2H; }
                if (v >= fd) { if (v > fd) { v = fd; mask = A2D; } else mask |= A2D; }
                CB[j] = v;
                dir |= mask;
            } else {
                CB[j] = HIGH;
                EB[j] = HIGH;
            }
            /* ASSIGN_MINIMUM + algn_fill_gapnum */
            const int eh = EH[j], ev = EV[j], eb = EB[j], cb = CB[j];
            int f = eh, mask = DO_H;
            if (f >= ev) { if (f > ev) { f = ev; mask = DO_V; } else mask |= DO_V; }
            if (f >= eb) { if (f > eb) { f = eb; mask = DO_D; } else mask |= DO_D; }
            if (f >= cb) { if (f > cb) { f = cb; mask = DO_A; } else mask |= DO_A; }
            if (f == eh && eh == ev) mask |= H_EQ_V;
            FIN[j] = f;
            dir |= mask;
            const int ha = (dir & (DO_A | DO_D)) != 0, hi = (dir & DO_H) != 0,
                      hd = (dir & DO_V) != 0;
            int n1, n2;
            if (ha) {
                if (hd && hi) {
                    int a = g1[j - 1], b = ng1[j - 1] + 1, cc = g1[j];
                    n1 = a > b ? a : b; if (cc > n1) n1 = cc;
                    a = g2[j - 1]; b = ng2[j - 1]; cc = g2[j] + 1;
                    n2 = a > b ? a : b; if (cc > n2) n2 = cc;
                } else if (hd) {
                    n1 = g1[j] > g1[j - 1] ? g1[j] : g1[j - 1];
                    n2 = g2[j - 1] > g2[j] + 1 ? g2[j - 1] : g2[j] + 1;
                } else if (hi) {
                    n1 = ng1[j - 1] + 1 > g1[j - 1] ? ng1[j - 1] + 1 : g1[j - 1];
                    n2 = g2[j - 1] > ng2[j - 1] ? g2[j - 1] : ng2[j - 1];
                } else {
                    n1 = g1[j - 1];
                    n2 = g2[j - 1];
                }
            } else if (hi) {
                if (hd) {
                    n1 = ng1[j - 1] + 1 > g1[j] ? ng1[j - 1] + 1 : g1[j];
                    n2 = g2[j] + 1 > ng2[j - 1] ? g2[j] + 1 : ng2[j - 1];
                } else {
                    n1 = ng1[j - 1] + 1;
                    n2 = ng2[j - 1];
                }
            } else {
                n1 = g1[j];
                n2 = g2[j] + 1;
            }
            ng1[j] = (uint16_t)n1;
            ng2[j] = (uint16_t)n2;
            cdm[j] = (uint16_t)dir;
        }
        if (i <= leni - 1) {
            uint16_t *t2;
            t2 = g1; g1 = ng1; ng1 = t2;
            t2 = g2; g2 = ng2; ng2 = t2;
        }
    }
    *res_cost = FIN[lenj];
    *gap_num = ng1[lenj] > ng2[lenj] ? ng1[lenj] : ng2[lenj];
    return 0;
}

static int aff_prepare(const ocm *c, ows *w, const uint8_t *sj, int leni,
                       int lenj)
{
    const int gap = c->t.gap;
    (void)gap;
    const int L = lenj + 2;
    GROW(w->abuf, w->abuf_cap, (size_t)12 * L, int);
    GROW(w->adm, w->adm_cap, (size_t)(leni + 1) * L, uint16_t);
    if (w->gm_cap < lenj + 1) {
        for (int k = 0; k < 4; k++) {
            void *np_ = realloc(w->gm[k], (size_t)(lenj + 1) * sizeof(uint16_t));
            if (!np_) return fail("out of memory");
            w->gm[k] = (uint16_t *)np_;
        }
        w->gm_cap = lenj + 1;
    }
    if (leni + 1 > w->arows_cap) {
        int *a = (int *)realloc(w->abs_, (size_t)(leni + 1) * sizeof(int));
        if (!a) return fail("out of memory");
        w->abs_ = a;
        a = (int *)realloc(w->abe, (size_t)(leni + 1) * sizeof(int));
        if (!a) return fail("out of memory");
        w->abe = a;
        w->arows_cap = leni + 1;
    }
    /* initialize_matrices_affine: row 0 of the base buffers */
    int *CB = w->abuf, *EB = w->abuf + 2 * L, *EV = w->abuf + 4 * L,
        *EH = w->abuf + 6 * L, *FIN = w->abuf + 8 * L;
    const int go = c->t.gap_open;
    CB[0] = 0;
    EB[0] = HIGH;
    EH[0] = go;
    EV[0] = go;
    FIN[0] = 0;
    w->adm[0] = 0xFFFF;
    for (int j = 1; j <= lenj; j++) {
        EH[j] = EH[j - 1] + c->t.prepend[sj[j]];
        CB[j] = HIGH;
        EB[j] = HIGH;
        EV[j] = HIGH;
        FIN[j] = EH[j];
        w->adm[j] = DO_H | END_H;
    }
    return 0;
}

static inline uint16_t adm_at(const ows *w, int i, int j, int L, int *bad)
{
    if (orc_check && i >= 1 && (j < w->abs_[i] || j > w->abe[i])) *bad = 1;
    return w->adm[(size_t)i * L + j];
}

/* backtrace_aff: internal order (si shorter). Outputs are written back to
 * front ending at index cap-1; lengths returned. */
static int aff_backtrace(const ocm *c, const ows *w, const uint8_t *si, int li,
                         const uint8_t *sj, int lj, int swaped, uint8_t *med,
                         uint8_t *mwg, uint8_t *ri, uint8_t *rj, int cap,
                         int *mlen, int *wlen, int *rlen)
{
    const int L = lj + 1;
    int i = li - 1, j = lj - 1;
    int km = cap, kw = cap, kr = cap, bad = 0;
    enum { M_TODO, M_V, M_H, M_D, M_A } mode = M_TODO;
    int ic = si[i], jc = sj[j];
#define PUT(buf, k, v) do { if ((k) <= 0) return fail("affine output capacity"); (buf)[--(k)] = (uint8_t)(v); } while (0)
#define PUTR(a, b) do { if (kr <= 0) return fail("affine output capacity"); kr--; ri[kr] = (uint8_t)(a); rj[kr] = (uint8_t)(b); } while (0)
    while (i != 0 && j != 0) {
        uint16_t d = adm_at(w, i, j, L, &bad);
        if (mode == M_TODO) {
            int fv = d & DO_V, fh = d & DO_H, fd = d & DO_D;
            if (!swaped) mode = fv ? M_V : fh ? M_H : fd ? M_D : M_A;
            else mode = fh ? M_H : fv ? M_V : fd ? M_D : M_A;
        } else if (mode == M_V || mode == M_H) {
            int vert = !swaped ? (mode == M_V) : !(mode == M_H);
            if (vert) {
                if ((d & END_V) || (d & H_EQ_V)) mode = M_TODO;
                if (!(ic & TMPGAP)) { PUT(med, km, ic | TMPGAP); PUT(mwg, kw, ic | TMPGAP); }
                else PUT(mwg, kw, TMPGAP);
                PUTR(ic, TMPGAP);
                i--;
                ic = si[i];
            } else {
                if ((d & END_H) || (d & H_EQ_V)) mode = M_TODO;
                if (!(jc & TMPGAP)) { PUT(med, km, jc | TMPGAP); PUT(mwg, kw, jc | TMPGAP); }
                else PUT(mwg, kw, TMPGAP);
                PUTR(TMPGAP, jc);
                j--;
                jc = sj[j];
            }
        } else if (mode == M_D) {
            if (d & END_B) mode = M_TODO;
            PUTR(ic, jc);
            PUT(mwg, kw, TMPGAP);
            i--;
            j--;
            jc = sj[j];
            ic = si[i];
        } else {
            int fd = d & A2D, fv = d & A2V, fh = d & A2H;
            if (!swaped) mode = fv ? M_V : fh ? M_H : fd ? M_D : M_A;
            else mode = fh ? M_H : fv ? M_V : fd ? M_D : M_A;
            int pm = c->t.median[((ic & NTMPGAP) << c->t.lcm) + (jc & NTMPGAP)];
            PUT(med, km, pm);
            PUT(mwg, kw, pm);
            PUTR(ic, jc);
            i--;
            j--;
            jc = sj[j];
            ic = si[i];
        }
    }
    if (bad) return fail("affine traceback left the band");
    while (i != 0) {
        if (!(ic & TMPGAP)) { PUT(med, km, ic | TMPGAP); PUT(mwg, kw, ic | TMPGAP); }
        else PUT(mwg, kw, TMPGAP);
        PUTR(ic, TMPGAP);
        i--;
        ic = si[i];
    }
    while (j != 0) {
        if (!(jc & TMPGAP)) { PUT(med, km, jc | TMPGAP); PUT(mwg, kw, jc | TMPGAP); }
        else PUT(mwg, kw, TMPGAP);
        PUTR(TMPGAP, jc);
        j--;
        jc = sj[j];
    }
    PUTR(TMPGAP, TMPGAP);
    PUT(mwg, kw, TMPGAP);
    if (km == cap) return fail("empty affine median");
    if (TMPGAP != med[km]) PUT(med, km, TMPGAP);
#undef PUT
#undef PUTR
    *mlen = cap - km;
    *wlen = cap - kw;
    *rlen = cap - kr;
    return 0;
}

/* algn_fill_plane_3_aff driver (internal order, li <= lj full lengths) */
static int aff_align(const ocm *c, ows *w, const uint8_t *si, int li,
                     const uint8_t *sj, int lj, int *cost)
{
    if (lj < li) return fail("pass the shorter one as first");
    if (li < 1) return fail("empty sequence");
    if (li == 1 && lj == 1) return fail("both sequences empty");
    const int leni = li - 1, lenj = lj - 1;
    if (aff_prepare(c, w, sj, leni, lenj)) return -1;
    int T = (lenj - leni + 1) * c->mnz;
    for (;;) {
        int p = (T - (lenj - leni)) / 2, g;
        if (aff_test(c, w, si, leni, sj, lenj, p, cost, &g)) return -1;
        int newp = (2 * T - (lenj - leni)) / 2;
        if (g < p || newp - lenj + 1 >= 0) return 0;
        T *= 2;
    }
}

int orc_median_affine(void *cm, void *ws, const uint8_t *a, int la,
                      const uint8_t *b, int lb, int *cost, uint8_t *med,
                      int *medlen, uint8_t *ea, uint8_t *eb, int *elen,
                      uint8_t *mwg, int *mwglen, int *maxcost)
{
    ocm *c = (ocm *)cm;
    ows *w = (ows *)ws;
    const int swaped = la <= lb ? 0 : 1;
    const uint8_t *si = swaped ? b : a, *sj = swaped ? a : b;
    const int li = swaped ? lb : la, lj = swaped ? la : lb;
    if (aff_align(c, w, si, li, sj, lj, cost)) return -1;
    const int cap = la + lb + 2;
    uint8_t *bufs = (uint8_t *)malloc((size_t)cap * 4);
    uint8_t *tm = bufs, *tw = bufs + cap, *ti = bufs + 2 * cap, *tj = bufs + 3 * cap;
    int ml, wl, rl;
    int rc = aff_backtrace(c, w, si, li, sj, lj, swaped, tm, tw, ti, tj, cap, &ml, &wl, &rl);
    if (!rc) {
        const uint8_t *pa = swaped ? tj : ti, *pb = swaped ? ti : tj;
        memcpy(ea, pa + cap - rl, (size_t)rl);
        memcpy(eb, pb + cap - rl, (size_t)rl);
        memcpy(med, tm + cap - ml, (size_t)ml);
        memcpy(mwg, tw + cap - wl, (size_t)wl);
        *elen = rl;
        *medlen = ml;
        *mwglen = wl;
        int gap = c->t.gap;
        *maxcost = (all_gaps(ea, rl, gap) || all_gaps(eb, rl, gap)) ? 0 : worst_2(c, ea, eb, rl);
    }
    free(bufs);
    return rc;
}

/* algn_CAML_cost_affine_3 -> algn_fill_plane_3_aff_nobt, replayed on the
 * reference's own buffer carve: with `largest` = the longer length the row
 * stride is largest + 1, so each state array's second row overlaps the first
 * entry of the next array (CB -> EB -> EV -> EH). The overlap is part of the
 * reference's observable behaviour and is kept here on purpose. */
static int aff_cost_nobt(const ocm *c, const uint8_t *si, int li,
                         const uint8_t *sj, int lj, int *cost)
{
    const int gap = c->t.gap, go = c->t.gap_open, lcm = c->t.lcm;
    const int largest = lj; /* li <= lj here */
    const int leni = li - 1, lenj = lj - 1;
    const int off = lenj + 2;
    int *mat = (int *)calloc((size_t)12 * largest + 4, sizeof(int));
    if (!mat) return fail("out of memory");
    int *CB = mat, *EB = mat + 2 * largest, *EV = mat + 4 * largest,
        *EH = mat + 6 * largest, *GOP = mat + 10 * largest,
        *SHX = mat + 11 * largest;
    const int *gaprow = c->t.prepend;
    /* initialize_matrices_affine_nobt */
    CB[0] = 0;
    EB[0] = HIGH;
    EH[0] = go;
    EV[0] = go;
    for (int j = 1; j <= lenj; j++) {
        EH[j] = EH[j - 1] + gaprow[sj[j]];
        CB[j] = HIGH;
        EB[j] = HIGH;
        EV[j] = HIGH;
    }
    int *pEH = EH + off, *pEV = EV + off, *pEB = EB + off, *pCB = CB + off;
    SHX[0] = 0;
    for (int j = 1; j <= lenj; j++) {
        GOP[j] = gap_opening(j, sj[j - 1], sj[j], gap, go);
        if ((sj[j - 1] & gap) && !(sj[j] & gap)) SHX[j] = GOP[j] + gaprow[sj[j]];
        else SHX[j] = gaprow[sj[j]];
    }
    if (lenj >= 1) SHX[1] = gaprow[sj[1]];
    int ic = si[0];
    for (int i = 1; i <= leni; i++) {
        int *t;
        t = pEH; pEH = EH; EH = t;
        t = pEV; pEV = EV; EV = t;
        t = pEB; pEB = EB; EB = t;
        t = pCB; pCB = CB; CB = t;
        EH[0] = HIGH;
        const int ip = ic;
        ic = si[i];
        const int sgext = C(c, ic, gap);
        const int sgop = gap_opening(i, ip, ic, gap, go);
        const int sng = NTMPGAP & ic;
        const int svext = ((i > 1) && ((ip & gap) && !(ic & gap))) ? sgop + sgext : sgext;
        const int r = pEV[0] + svext;
        EH[0] = HIGH;
        CB[0] = r;
        EB[0] = HIGH;
        EV[0] = r;
        int jc = sj[0];
        CB[0] = HIGH;
        const int *srow = c->t.cost + (sng << lcm);
        for (int j = 1; j <= lenj; j++) {
            const int jp = jc;
            jc = sj[j];
            const int jng = NTMPGAP & jc;
            const int jgext = gaprow[jc], jgop = GOP[j];
            int ext = EH[j - 1] + SHX[j], open = CB[j - 1] + jgop + jgext;
            EH[j] = ext < open ? ext : open;
            ext = pEV[j] + svext;
            open = pCB[j] + sgop + sgext;
            EV[j] = ext < open ? ext : open;
            const int flag = (TMPGAP & ic) && (TMPGAP & jc);
            const int flag2 = !(TMPGAP & ip) && !(TMPGAP & jp);
            const int diag = flag ? 0 : HIGH;
            const int odiag = flag ? (flag2 ? 0 : 2 * go) : HIGH;
            ext = pEB[j - 1] + diag;
            open = pCB[j - 1] + odiag;
            EB[j] = ext < open ? ext : open;
            const int dg = srow[jng];
            const int xgo = (jgop < sgop) ? sgop : jgop;
            const int algn = pCB[j - 1] + dg;
            const int fv = (ic == sng) ? pEV[j - 1] + dg : pEV[j - 1] + dg + jgop;
            const int fh = (jc == jng) ? pEH[j - 1] + dg : pEH[j - 1] + dg + sgop;
            const int fd = pEB[j - 1] + dg + xgo;
            int v = algn;
            if (v > fv) v = fv;
            if (v > fh) v = fh;
            if (v > fd) v = fd;
            CB[j] = v;
        }
    }
    int res = EH[lenj];
    if (res > EV[lenj]) res = EV[lenj];
    if (res > EB[lenj]) res = EB[lenj];
    if (res > CB[lenj]) res = CB[lenj];
    *cost = res;
    free(mat);
    return 0;
}

int orc_cost_affine(void *cm, void *ws, const uint8_t *a, int la,
                    const uint8_t *b, int lb, int *cost)
{
    (void)ws;
    ocm *c = (ocm *)cm;
    if (la <= lb) return aff_cost_nobt(c, a, la, b, lb, cost);
    return aff_cost_nobt(c, b, lb, a, la, cost);
}

/* ------------------------------------------------------------------------ */
/* batch + schedule helpers                                                 */

int orc_median_batch(void *cm, int affine, int npairs, const uint8_t *seqs,
                     const int64_t *offa, const int *lena, const int64_t *offb,
                     const int *lenb, const int64_t *out_off, int *cost,
                     int *maxcost, int *alen, int *mlen, int *wlen, uint8_t *ea,
                     uint8_t *eb, uint8_t *med, uint8_t *mwg, int *status,
                     int nthreads)
{
    int failures = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(+ : failures)
#endif
    {
        void *ws = orc_ws_new();
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int k = 0; k < npairs; k++) {
            const uint8_t *a = seqs + offa[k], *b = seqs + offb[k];
            int64_t o = out_off[k];
            int rc;
            if (affine)
                rc = orc_median_affine(cm, ws, a, lena[k], b, lenb[k], &cost[k],
                                       med + o, &mlen[k], ea + o, eb + o,
                                       &alen[k], mwg + o, &wlen[k], &maxcost[k]);
            else
                rc = orc_median_linear(cm, ws, a, lena[k], b, lenb[k], &cost[k],
                                       ea + o, eb + o, &alen[k], med + o,
                                       &mlen[k], mwg + o, &wlen[k], &maxcost[k]);
            status[k] = rc;
            if (rc) failures++;
        }
        orc_ws_free(ws);
    }
    return failures;
}

int orc_schedule(void *cm, int affine, const uint8_t *a, int la,
                 const uint8_t *b, int lb, int *iters, int64_t *cells)
{
    ocm *c = (ocm *)cm;
    const uint8_t *s1 = la <= lb ? a : b, *s2 = la <= lb ? b : a;
    int m = la <= lb ? la : lb, n = la <= lb ? lb : la;
    *iters = 0;
    *cells = 0;
    if (affine) {
        int leni = m - 1, lenj = n - 1;
        void *ws = orc_ws_new();
        ows *w = (ows *)ws;
        if (aff_prepare(c, w, s2, leni, lenj)) { orc_ws_free(ws); return -1; }
        int T = (lenj - leni + 1) * c->mnz;
        for (;;) {
            int p = (T - (lenj - leni)) / 2, g, cost;
            int newk = p >= leni ? leni - 1 : p;
            for (int i = 1; i <= leni; i++) {
                int s = (i - newk) > 0 ? i - newk : 0;
                int e = (i + lenj - leni + newk) <= (lenj - 1) ? i + lenj - leni + newk : lenj;
                *cells += e - s + 1;
            }
            aff_test(c, w, s1, leni, s2, lenj, p, &cost, &g);
            (*iters)++;
            int newp = (2 * T - (lenj - leni)) / 2;
            if (g < p || newp - lenj + 1 >= 0) break;
            T *= 2;
        }
        orc_ws_free(ws);
        return 0;
    }
    /* linear: replay lin_cost's plane choice and doubling */
    int g1 = count_gaps(a, la, c->t.gap), g2 = count_gaps(b, lb, c->t.gap);
    int gaps = g1 > g2 ? g1 : g2;
    int lower = (int)((double)m * 0.10);
    int dw = (m - n) < lower ? lower / 2 : 2;
    int deltawh = gaps + dw;
    int height = (m - n) + 50 + deltawh;
    if (height > m) height = m;
    int full;
    if ((double)(float)m >= 1.5 * (double)(float)n) full = 1;
    else if (2 * height < m) full = 0;
    else full = (8 >= m - height);
    void *ws = orc_ws_new();
    int cost;
    if (full) {
        lin_fill(c, (ows *)ws, s1, m, s2, n, 1, 0, &cost);
        *iters = 0;
        *cells = (int64_t)(m - 1) * n;
        orc_ws_free(ws);
        return 0;
    }
    int T = (n - m + 1) * c->mnz;
    for (;;) {
        int p = (T - (n - m)) / 2, g;
        lin_fill(c, (ows *)ws, s1, m, s2, n, 0, p, &cost);
        ows *w = (ows *)ws;
        for (int i = 1; i < m; i++) *cells += w->re[i] - w->rs[i] + 1;
        lin_gaps(w, &g);
        (*iters)++;
        int newp = (2 * T - (n - m)) / 2;
        if ((g + 1) < p || newp - n + 1 >= 0) break;
        T *= 2;
    }
    orc_ws_free(ws);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Algn_Newkk: POY's own Ukkonen-style banded aligner (src/newkkonen.c),    */
/* affine cost model (newkkonen_CAML_algn_affine / _backtrace_affine).      */
/*                                                                          */
/* The reference grows the band in place and re-evaluates only cells whose  */
/* neighbours changed (update_a_row, src/newkkonen.c:964-1074); every cell  */
/* is a function of its three neighbours and the band borders alone, so the */
/* band of each iteration is filled afresh here. tests/test_newkk.py checks */
/* costs and alignments against the reference compiled unmodified.          */

#define NK_INF (INT_MAX / 2)
/* direction flags, src/newkkonen.c:44-61 */
enum {
    NK_START = 0, NK_ALIGN = 1, NK_DEL = 16, NK_INS = 32, NK_END_INS = 64,
    NK_END_DEL = 128, NK_END_DIAG = 256, NK_DIAG = 512, NK_INS_EQ_DEL = 1024
};
#define NK_GAP 16  /* GAPCODE, src/newkkonen.c:37 */
#define NK_NOGAP 15 /* NOGAP, src/newkkonen.c:41 */
#define NK_MUCH_LONGER 100 /* src/newkkonen.c:34 */

typedef struct nkcell {
    int cost, P, Q, ED, CD;
    uint16_t dir, g1, g2;
} nkcell;

/* my_add, src/newkkonen.c:65-71 */
static inline int nk_add(int a, int b)
{
    if (a >= NK_INF) return NK_INF;
    if (b >= NK_INF) return NK_INF;
    return a + b;
}
/* get_go, src/newkkonen.c:179-184 */
static inline int nk_go(int base, int prev, int idx, int go)
{
    if (idx == 1 && (base & NK_GAP)) return 0;
    if (idx > 1 && !(prev & NK_GAP) && (base & NK_GAP)) return 0;
    return go;
}
/* get_extgo, src/newkkonen.c:194-198 */
static inline int nk_extgo(int base, int prev, int go)
{
    return ((prev & NK_GAP) && !(base & NK_GAP)) ? go : 0;
}
#define NK_MIN(a, b) ((a) < (b) ? (a) : (b))
#define NK_MAX(a, b) ((a) > (b) ? (a) : (b))

/* One band cell: update_internal_cell + assign_best_cost_and_direction
 * (src/newkkonen.c:600-873). lb / rb: the cell lies on the band's left
 * (i - j == k) / right (j - i == lenY - lenX + k) border. L, U, D: the
 * cells (i, j-1), (i-1, j), (i-1, j-1), read only where the reference
 * reads them. */
static void nk_cell(const ocm *c, const uint8_t *s1, const uint8_t *s2, int i,
                    int j, int lb, int rb, const nkcell *L, const nkcell *U,
                    const nkcell *D, int go, nkcell *out)
{
    const int gap = c->t.gap;
    const int b1 = s1[i], b2 = s2[j];
    /* seq_get(s, -1) is never needed: at i == 0 (j == 0) every candidate
     * that uses the previous base is out of the matrix */
    const int pb1 = i > 0 ? s1[i - 1] : 0, pb2 = j > 0 ? s2[j - 1] : 0;
    const int go1 = nk_go(b1, pb1, i, go), go2 = nk_go(b2, pb2, j, go);
    const int eg1 = nk_extgo(b1, pb1, go), eg2 = nk_extgo(b2, pb2, go);
    int thisP = NK_INF, thisQ = NK_INF, thisED = NK_INF, thisCD = NK_INF;
    int costL, extL, openL, gL1 = 0, gL2 = 0;
    if (lb || j == 0) {
        costL = extL = openL = NK_INF;
    } else {
        int add = C(c, b2, gap);
        extL = nk_add(L->Q, add + eg2);
        openL = nk_add(L->CD, add + go2);
        costL = thisQ = NK_MIN(openL, extL);
        gL1 = L->g1;
        gL2 = L->g2;
    }
    int costR, extR, openR, gR1 = 0, gR2 = 0;
    if (rb || i == 0) {
        costR = extR = openR = NK_INF;
    } else {
        int add = C(c, b1, gap);
        extR = nk_add(U->P, add + eg1);
        openR = nk_add(U->CD, add + go1);
        costR = thisP = NK_MIN(openR, extR);
        gR1 = U->g1;
        gR2 = U->g2;
    }
    int costM, costDiag, extD, openD, gM1 = 0, gM2 = 0;
    if (i == 0 || j == 0) {
        costM = costDiag = extD = openD = NK_INF;
    } else {
        const int n1 = b1 & NK_NOGAP, n2 = b2 & NK_NOGAP;
        const int add = C(c, n1, n2);
        thisCD = nk_add(D->CD, add);
        int fromR = D->P + C(c, n1, b2) + (n1 == b1 ? 0 : go);
        int fromL = D->Q + C(c, b1, n2) + (n2 == b2 ? 0 : go);
        thisCD = NK_MIN(thisCD, fromR);
        thisCD = NK_MIN(thisCD, fromL);
        thisCD = NK_MIN(thisCD, nk_add(D->ED, go1 + go2 + add));
        int diag = ((b1 & NK_GAP) && (b2 & NK_GAP)) ? 0 : NK_INF;
        openD = nk_add(D->CD, go1 + go2);
        extD = nk_add(D->ED, diag);
        thisED = NK_MIN(extD, openD);
        costM = thisCD;
        costDiag = thisED;
        gM1 = D->g1;
        gM2 = D->g2;
    }
    int dir = NK_INS, best = costL, g1 = gL1 + 1, g2 = gL2;
    if (costR <= best) {
        if (costR < best) { best = costR; dir = NK_DEL; g1 = gR1; g2 = gR2 + 1; }
        else { dir |= NK_DEL; g1 = NK_MAX(g1, gR1); g2 = NK_MAX(g2, gR2 + 1); }
    }
    if (costM <= best) {
        if (costM < best) { best = thisCD; dir = NK_ALIGN; g1 = gM1; g2 = gM2; }
        else { dir |= NK_ALIGN; g1 = NK_MAX(g1, gM1); g2 = NK_MAX(g2, gM2); }
    }
    if (costDiag <= best) {
        if (costDiag < best) { best = costDiag; dir = NK_DIAG; g1 = gM1; g2 = gM2; }
        else { dir |= NK_DIAG; g1 = NK_MAX(g1, gM1); g2 = NK_MAX(g2, gM2); }
    }
    if (extR >= openR) dir |= NK_END_DEL;
    if (extL >= openL) dir |= NK_END_INS;
    if (extD >= openD) dir |= NK_END_DIAG;
    if (extR == extL && extR == best) dir |= NK_INS_EQ_DEL;
    out->cost = best;
    out->dir = (uint16_t)dir;
    out->g1 = (uint16_t)g1;
    out->g2 = (uint16_t)g2;
    out->P = thisP;
    out->Q = thisQ;
    out->ED = thisED;
    out->CD = thisCD;
}

typedef struct nkband {
    nkcell *cell;
    size_t cap;
    int lenX, lenY, k, W; /* row i holds columns i-k .. i+lenY-lenX+k */
} nkband;

static inline nkcell *nk_at(nkband *b, int i, int j)
{
    return b->cell + (size_t)i * b->W + (j - (i - b->k));
}

/* Row 0 of the matrix, columns 0 .. lenY-lenX (newkk_algn's first row,
 * src/newkkonen.c:1380-1428). */
static void nk_first_row(const ocm *c, nkband *b, const uint8_t *s2, int go)
{
    const int gap = c->t.gap, bb = b->lenY - b->lenX + 1;
    nkcell *z = nk_at(b, 0, 0);
    z->cost = 0;
    z->dir = NK_START;
    z->g1 = z->g2 = 0;
    z->P = z->Q = go;
    z->ED = NK_INF;
    z->CD = 0;
    for (int j = 1; j < bb; j++) {
        const nkcell *l = nk_at(b, 0, j - 1);
        nkcell *o = nk_at(b, 0, j);
        int add = C(c, s2[j], gap);
        int flag = gap & s2[j - 1], flag2 = gap & s2[j], gocost;
        if (j == 1) gocost = flag2 ? 0 : go;
        else gocost = (!flag && flag2) ? 0 : go;
        int ext = l->Q + add + ((flag && !flag2) ? go : 0);
        int open = l->cost + add + gocost;
        o->cost = o->Q = NK_MIN(open, ext);
        o->dir = NK_INS | NK_END_INS | NK_END_DEL | NK_END_DIAG;
        o->g1 = (uint16_t)(l->g1 + 1);
        o->g2 = l->g2;
        o->P = o->ED = o->CD = NK_INF;
    }
}

/* One ukktest pass at band half-width k (src/newkkonen.c:1077-1153);
 * returns the last cell. */
static const nkcell *nk_fill(const ocm *c, nkband *b, const uint8_t *s1,
                             const uint8_t *s2, int k, int go)
{
    const int X = b->lenX, Y = b->lenY, d = Y - X;
    b->k = k;
    b->W = d + 2 * k + 1;
    size_t need = (size_t)X * b->W;
    if (need > b->cap) {
        free(b->cell);
        b->cell = (nkcell *)malloc(need * sizeof(nkcell));
        b->cap = need;
    }
    nk_first_row(c, b, s2, go);
    for (int i = 0; i < X; i++) {
        int js = i - k > 0 ? i - k : 0;
        int je = i + d + k < Y - 1 ? i + d + k : Y - 1;
        if (i == 0) js = d + 1; /* columns 0..d hold the first row */
        for (int j = js; j <= je; j++) {
            int lb = (i - j == k), rb = (j - i == d + k);
            nk_cell(c, s1, s2, i, j, lb, rb,
                    (!lb && j > 0) ? nk_at(b, i, j - 1) : NULL,
                    (!rb && i > 0) ? nk_at(b, i - 1, j) : NULL,
                    (i > 0 && j > 0) ? nk_at(b, i - 1, j - 1) : NULL, go,
                    nk_at(b, i, j));
        }
    }
    return nk_at(b, X - 1, Y - 1);
}

/* trivial_algn, src/newkkonen.c:1334-1357 */
static int nk_trivial_cost(const ocm *c, const uint8_t *s1, int l1,
                           const uint8_t *s2, int l2)
{
    int r = 0;
    for (int i = 0; i < l1; i++) r += C(c, s1[i] & NK_NOGAP, c->t.gap);
    for (int j = 0; j < l2; j++) r += C(c, s2[j] & NK_NOGAP, c->t.gap);
    return r;
}

/* newkk_algn + increaseT (src/newkkonen.c:1155-1172, 1361-1446) with the
 * affine gap opening `go`; s1 is the shorter. Leaves the last band in b
 * (b->lenX == 0 for the trivial case). */
static int nk_align_cost(const ocm *c, nkband *b, const uint8_t *s1, int l1,
                         const uint8_t *s2, int l2, int *iters, int64_t *cells)
{
    const int go = c->t.gap_open > 0 ? c->t.gap_open : 0;
    if (iters) *iters = 0;
    if ((int64_t)l1 * NK_MUCH_LONGER < l2) {
        b->lenX = 0;
        return nk_trivial_cost(c, s1, l1, s2, l2);
    }
    b->lenX = l1;
    b->lenY = l2;
    const int d = l2 - l1;
    int T = (d + 1) * c->mnz;
    for (;;) {
        int p = (T - d) / 2;
        int k = p < l1 - 1 ? p : l1 - 1;
        const nkcell *last = nk_fill(c, b, s1, s2, k, go);
        if (iters) (*iters)++;
        if (cells)
            for (int i = 0; i < l1; i++) {
                int js = i - k > 0 ? i - k : 0;
                int je = i + d + k < l2 - 1 ? i + d + k : l2 - 1;
                *cells += je - js + 1;
            }
        int gn = last->g1 > last->g2 ? last->g1 : last->g2;
        int newp = (T * 2 - d) / 2;
        if (p > gn || newp - l2 + 1 >= 0) return last->cost;
        T *= 2;
    }
}

/* backtrace_affine (src/newkkonen.c:1666-1766) and trivial_backtrace
 * (:1498-1520); writes back to front into r1/r2 of capacity l1 + l2 and
 * returns the aligned length. */
static int nk_backtrace(const ocm *c, nkband *b, const uint8_t *s1, int l1,
                        const uint8_t *s2, int l2, int swaped, uint8_t *r1,
                        uint8_t *r2)
{
    const int gap = c->t.gap, cap = l1 + l2;
    int n = 0;
#define NK_PUT(x, y)                                                        \
    do {                                                                    \
        if (n >= cap) return fail("newkk backtrace: output full");          \
        n++;                                                                \
        r1[cap - n] = (uint8_t)(x);                                         \
        r2[cap - n] = (uint8_t)(y);                                         \
    } while (0)
    if (b->lenX == 0) {
        for (int i = 0; i < l1; i++) NK_PUT(s1[i], gap);
        for (int j = 0; j < l2; j++) NK_PUT(gap, s2[j]);
        return n;
    }
    enum { M_TODO, M_DEL, M_INS, M_DIAG, M_ALIGN } mode = M_TODO;
    const int d = l2 - l1;
    int i = l1 - 1, j = l2 - 1;
    while (i >= 0 && j >= 0) {
        if (i - j > b->k || j - i > d + b->k)
            return fail("newkk backtrace left the band");
        int dir = nk_at(b, i, j)->dir;
        if (dir == NK_START) {
            if (i != 0 || j != 0) return fail("newkk backtrace: START off (0,0)");
            NK_PUT(gap, gap);
            i--;
            j--;
        } else if (mode == M_TODO) {
            int ins = dir & NK_INS, del = dir & NK_DEL;
            if (!swaped) mode = del ? M_DEL : ins ? M_INS : 0;
            else mode = ins ? M_INS : del ? M_DEL : 0;
            if (!mode) mode = (dir & NK_DIAG) ? M_DIAG : (dir & NK_ALIGN) ? M_ALIGN : 0;
            if (!mode) return fail("newkk backtrace: invalid direction");
        } else if (mode == M_DEL || mode == M_INS) {
            int same = dir & NK_INS_EQ_DEL;
            if (mode == M_DEL) {
                NK_PUT(s1[i], gap);
                i--;
                if ((dir & NK_END_DEL) || same) mode = M_TODO;
            } else {
                NK_PUT(gap, s2[j]);
                j--;
                if ((dir & NK_END_INS) || same) mode = M_TODO;
            }
        } else if (mode == M_DIAG) {
            if (dir & NK_END_DIAG) mode = M_TODO;
            NK_PUT(s1[i], s2[j]);
            i--;
            j--;
        } else {
            NK_PUT(s1[i] & NK_NOGAP, s2[j] & NK_NOGAP);
            i--;
            j--;
            mode = M_TODO;
        }
    }
#undef NK_PUT
    return n;
}

static int nk_check_affine(const ocm *c)
{
    if (c->t.cost_model != 1)
        return fail("Algn_Newkk is built for the affine cost model only");
    return 0;
}

/* newkkonen_CAML_algn_affine + newkkonen_CAML_backtrace_affine
 * (src/newkkonen.c:1473-1496, 1788-1805) on s1 (the shorter) and s2. The
 * aligned pair lands in r1/r2[0, *len); capacity l1 + l2 each. */
int orc_newkk_align(void *cm, const uint8_t *s1, int l1, const uint8_t *s2,
                    int l2, int swaped, int *cost, uint8_t *r1, uint8_t *r2,
                    int *len, int *iters, int64_t *cells)
{
    const ocm *c = (const ocm *)cm;
    if (nk_check_affine(c)) return -1;
    if (l1 > l2) return fail("ERROR: newkkonen.newkk_algn, s1 len > s2 len");
    if (l1 < 1) return fail("empty sequence");
    nkband b = {0};
    if (cells) *cells = 0;
    *cost = nk_align_cost(c, &b, s1, l1, s2, l2, iters, cells);
    int cap = l1 + l2, rc = 0;
    uint8_t *t1 = (uint8_t *)malloc((size_t)cap), *t2 = (uint8_t *)malloc((size_t)cap);
    int n = nk_backtrace(c, &b, s1, l1, s2, l2, swaped, t1, t2);
    if (n < 0) rc = -1;
    else {
        memcpy(r1, t1 + cap - n, (size_t)n);
        memcpy(r2, t2 + cap - n, (size_t)n);
        *len = n;
    }
    free(t1);
    free(t2);
    free(b.cell);
    return rc;
}

/* SeqCS.DOS.median with use_ukk under an affine model (src/seqCS.ml:
 * 1043-1051): NewkkAlign.align_2 (shorter first, src/sequence.ml:
 * 1879-1901), then Align.ancestor_2, median_2_with_gaps and max_cost_2 on
 * the aligned pair. Output capacities as orc_median_linear. */
int orc_newkk_median(void *cm, const uint8_t *a, int la, const uint8_t *b,
                     int lb, int *cost, uint8_t *ea, uint8_t *eb, int *elen,
                     uint8_t *anc, int *anclen, uint8_t *mwg, int *mwglen,
                     int *maxcost)
{
    const ocm *c = (const ocm *)cm;
    int L, rc;
    if (la <= lb) rc = orc_newkk_align(cm, a, la, b, lb, 0, cost, ea, eb, &L, NULL, NULL);
    else rc = orc_newkk_align(cm, b, lb, a, la, 1, cost, eb, ea, &L, NULL, NULL);
    if (rc) return rc;
    *elen = L;
    if (ancestor_2(c, ea, eb, L, anc, anclen)) return -1;
    for (int i = 0; i < L; i++) mwg[i] = c->t.median[(ea[i] << c->t.lcm) + eb[i]];
    *mwglen = L;
    int gap = c->t.gap;
    *maxcost = (all_gaps(ea, L, gap) || all_gaps(eb, L, gap)) ? 0 : worst_2(c, ea, eb, L);
    return 0;
}
