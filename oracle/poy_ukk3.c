/*
 * TEST INFRASTRUCTURE ONLY (the oracle): a CPU restatement of POY's
 * three-sequence alignment, Sequence.Align.align_3_powell (src/sequence.ml:
 * 1312-1321) -> powell_3D_align (src/ukkCommon.c:109-145) -> doUkk
 * (src/ukk.checkp.c:111-212). Only tests/, smoke() and the bench's CPU arms
 * call it; the product library never links it.
 *
 * The algorithm is Powell, Allison and Dix's generalisation of Ukkonen's
 * furthest-reaching-diagonal recursion to three sequences ("Fast, optimal
 * alignment of three sequences using linear gap costs", J. Theor. Biol. 207,
 * 2000), with a check-point divide and conquer that recovers the alignment.
 * What the results depend on, and what this file therefore keeps:
 *
 *  - the 16 column states and their neighbour steps, continuation costs and
 *    transition costs (src/ukkCommon.c:244-338);
 *  - the memo: U(ab, ac, d, s) lives in slot (ab, ac, d mod 2*maxSingleStep,
 *    s) and is valid when its stamp equals d + costOffset, costOffset growing
 *    by finalCost + 1 per check-point pass (src/ukkCommon.h getPtr with
 *    FIXED_NUM_PLANES; src/ukk.checkp.c:230-237). A cell whose slot was taken
 *    by another cost is recomputed, and the `from` records read without a
 *    stamp check see whatever the slot holds, so the evaluation order is
 *    part of the result and this restatement keeps it call for call;
 *  - the check-point store CP(ab, ac, d mod maxSingleStep, s)
 *    (src/ukk.checkp.c:586-589);
 *  - INFINITY = 10000/2 (src/ukk.checkp.c:31, src/ukkCommon.h), which is also
 *    the first pass's check-point cost until half of A has been reached;
 *  - the recursion order (second half first, src/ukk.checkp.c:351-358) and the
 *    emission order of the traceback (src/ukk.checkp.c:368-443, 454-501).
 *
 * The reference keeps all of this in globals; here it is one context per
 * call, so calls may run concurrently. Storage is lazily allocated blocks of
 * 16 x 16 diagonals per cost plane: the slot identity, not the layout, is
 * what the results depend on.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "poy_oracle.h"

#define U3_INF 5000     /* INFINITY of src/ukkCommon.h with MAXINT 10000 */
#define U3_BS 16
#define U3_MAXLEN 100000 /* MAX_STR */

enum { U3_M = 0, U3_D = 1, U3_I = 2 };

typedef struct { int ab, ac, cost, state; } u3_from;
typedef struct { int dist; long stamp; u3_from from; } u3_cell;
typedef struct { int dist, cost; } u3_cp;

typedef struct {
    size_t elem;
    int planes, ns;
    int ab_off, ac_off, nbab, nbac;
    void **blk;
} u3_store;

typedef struct {
    int mm, go, ge;
    int ns, neigh[27], cont[27], second[27], trans[27][27], maxstep;
    uint8_t *A, *B, *C;
    int la, lb, lc;
    u3_store U, CP;
    long off, final_cost;
    int furthest, cp_cost, cp_width, complete;
    int sab, sac, scost, sstate;
    int endA, endB, endC;
    uint8_t *ea, *eb, *ec;
    int n;
    int oom;
} u3_ctx;

/* ---- state machine (src/ukkCommon.c:206-338) ---------------------------- */

static int u3_digit(int s, int i) { return i == 0 ? s % 3 : i == 1 ? (s / 3) % 3 : (s / 9) % 3; }

static int u3_count(int s, int t)
{
    int n = 0;
    for (int i = 0; i < 3; i++) n += u3_digit(s, i) == t;
    return n;
}

static void u3_setup(u3_ctx *x)
{
    int code[27];
    int ns = 0;
    for (int s = 0; s < 27; s++) {
        if (u3_count(s, U3_M) == 0 || u3_count(s, U3_I) > 1) continue;
        code[ns] = s;
        int want = u3_count(s, U3_I) ? U3_I : U3_M;
        int nb = 0;
        for (int i = 0; i < 3; i++)
            if (u3_digit(s, i) == want) nb |= 1 << i;
        x->neigh[ns] = nb;
        if (u3_count(s, U3_I)) {
            x->cont[ns] = x->ge;
            x->second[ns] = 0;
        } else if (u3_count(s, U3_M) == 3) {
            x->cont[ns] = x->mm;
            x->second[ns] = 1;
        } else if (u3_count(s, U3_D) == 1) {
            x->cont[ns] = x->ge;
            x->second[ns] = 1;
        } else {
            x->cont[ns] = 2 * x->ge;
            x->second[ns] = 0;
        }
        ns++;
    }
    x->ns = ns;
    int mx = 0;
    for (int f = 0; f < ns; f++)
        for (int t = 0; t < ns; t++) {
            int c = 0;
            for (int i = 0; i < 3; i++) {
                int to = u3_digit(code[t], i);
                if (to != U3_M && to != u3_digit(code[f], i)) c += x->go;
            }
            x->trans[f][t] = c;
            int step = c + x->cont[t] + x->mm * (u3_count(code[t], U3_M) - 1);
            if (step > mx) mx = step;
        }
    x->maxstep = mx;
}

/* ---- memo slots (src/ukkCommon.h allocInit / getPtr) --------------------- */

static int u3_store_init(u3_store *st, size_t elem, int planes, int ns, int la, int lb, int lc)
{
    st->elem = elem;
    st->planes = planes;
    st->ns = ns;
    st->ab_off = lb;
    st->ac_off = lc;
    st->nbab = (la + lb + 1) / U3_BS + 1;
    st->nbac = (la + lc + 1) / U3_BS + 1;
    st->blk = calloc((size_t)planes * st->nbab * st->nbac, sizeof(void *));
    return st->blk != NULL;
}

static void u3_store_free(u3_store *st)
{
    if (!st->blk) return;
    size_t n = (size_t)st->planes * st->nbab * st->nbac;
    for (size_t i = 0; i < n; i++) free(st->blk[i]);
    free(st->blk);
    st->blk = NULL;
}

static void *u3_slot(u3_ctx *x, u3_store *st, int ab, int ac, int d, int s)
{
    static u3_cell dummy_cell;
    static u3_cp dummy_cp;
    int p = d % st->planes;
    int i = ab + st->ab_off, j = ac + st->ac_off;
    size_t bi = ((size_t)p * st->nbab + i / U3_BS) * st->nbac + j / U3_BS;
    if (!st->blk[bi]) {
        st->blk[bi] = calloc((size_t)U3_BS * U3_BS * st->ns, st->elem);
        if (!st->blk[bi]) {
            x->oom = 1;
            return st->elem == sizeof(u3_cell) ? (void *)&dummy_cell : (void *)&dummy_cp;
        }
    }
    size_t k = ((size_t)(i % U3_BS) * U3_BS + j % U3_BS) * st->ns + s;
    return (char *)st->blk[bi] + k * st->elem;
}

static u3_cell *u3_U(u3_ctx *x, int ab, int ac, int d, int s)
{
    return (u3_cell *)u3_slot(x, &x->U, ab, ac, d, s);
}

static u3_cp *u3_CP(u3_ctx *x, int ab, int ac, int d, int s)
{
    return (u3_cp *)u3_slot(x, &x->CP, ab, ac, d, s);
}

/* ---- the recursion (src/ukk.checkp.c:506-782) ---------------------------- */

static int u3_ok(int a, int da, int end)
{
    if (a < 0) return 0;
    return da ? a < end : a <= end;
}

static int u3_chars(int a, int b, int c)
{
    if (a == b && a == c) return 0;
    if (a == b || a == c || b == c) return 1;
    return 2;
}

static int u3_iabs(int v) { return v < 0 ? -v : v; }

/* lower bound on the cost from the pass's start (withinMatrix) */
static int u3_within(const u3_ctx *x, int ab, int ac, int d)
{
    if (d < 0) return 0;
    int v[3] = {u3_iabs(x->sab - ab), u3_iabs(x->sac - ac),
                u3_iabs((x->sac - x->sab) - (ac - ab))};
    for (int i = 0; i < 2; i++)
        for (int j = i + 1; j < 3; j++)
            if (v[j] < v[i]) { int t = v[i]; v[i] = v[j]; v[j] = t; }
    int g = v[0], h = v[1], cheapest;
    if (x->sstate == 0)
        cheapest = (g ? x->go + g * x->ge : 0) + (h ? x->go + h * x->ge : 0);
    else
        cheapest = g * x->ge + h * x->ge;
    return cheapest + x->scost <= d;
}

static int u3_ukk(u3_ctx *x, int ab, int ac, int d, int s);

static void u3_calc(u3_ctx *x, int ab, int ac, int d, int to)
{
    const int nb = x->neigh[to];
    const int da = nb & 1, db = (nb >> 1) & 1, dc = (nb >> 2) & 1;
    const int in_cp = d >= x->cp_cost && d < x->cp_cost + x->cp_width;
    const int copy = d >= x->cp_cost + x->cp_width;
    u3_from from = {0, 0, -1, 0};
    int best = -U3_INF;
    if (in_cp) from = (u3_from){ab, ac, d, to};
    const int ab1 = ab - da + db, ac1 = ac - da + dc;
    if (ab1 >= -x->endB && ab1 <= x->endA && ac1 >= -x->endC && ac1 <= x->endA) {
        for (int fs = 0; fs < x->ns; fs++) {
            int cost = d - x->trans[fs][to] - x->cont[to];
            int fcost = 0, dist = -U3_INF;
            int a1 = u3_ukk(x, ab1, ac1, cost, fs);
            if (u3_ok(a1, da, x->endA) && u3_ok(a1 - ab1, db, x->endB) &&
                u3_ok(a1 - ac1, dc, x->endC) &&
                u3_chars(da ? x->A[a1] : 16, db ? x->B[a1 - ab1] : 16,
                         dc ? x->C[a1 - ac1] : 16) == 1) {
                fcost = cost;
                dist = a1 + da;
            } else {
                if (!x->second[to]) continue;
                int a2 = u3_ukk(x, ab1, ac1, cost - x->mm, fs);
                if (u3_ok(a2, da, x->endA) && u3_ok(a2 - ab1, db, x->endB) &&
                    u3_ok(a2 - ac1, dc, x->endC)) {
                    fcost = cost - x->mm;
                    dist = a2 + da;
                }
            }
            if (best < dist) {
                best = dist;
                if (x->complete)
                    from = (u3_from){ab1, ac1, fcost, fs};
                else if (copy)
                    from = u3_U(x, ab1, ac1, fcost, fs)->from;
            }
        }
    }
    {
        int dist = u3_ukk(x, ab, ac, d - 1, to);
        if (u3_ok(dist, 0, x->endA) && u3_ok(dist - ab, 0, x->endB) &&
            u3_ok(dist - ac, 0, x->endC) && best < dist) {
            best = dist;
            if (x->complete)
                from = (u3_from){ab, ac, d - 1, to};
            else if (copy)
                from = u3_U(x, ab, ac, d - 1, to)->from;
        }
    }
    if (to == 0) {
        int dist = -U3_INF, fst = -1;
        for (int s = 0; s < x->ns; s++) {
            int t = s == 0 ? best : u3_ukk(x, ab, ac, d, s);
            if (t > dist) {
                dist = t;
                fst = s;
            }
        }
        while (u3_ok(dist, 1, x->endA) && u3_ok(dist - ab, 1, x->endB) &&
               u3_ok(dist - ac, 1, x->endC) && x->A[dist] == x->B[dist - ab] &&
               x->A[dist] == x->C[dist - ac])
            dist++;
        if (dist > best) {
            best = dist;
            if (fst != 0) {
                if (x->complete)
                    from = (u3_from){ab, ac, d, fst};
                else if (copy)
                    from = u3_U(x, ab, ac, d, fst)->from;
            }
        }
    }
    u3_cell *c = u3_U(x, ab, ac, d, to);
    c->dist = best;
    c->stamp = d + x->off;
    c->from = from;
}

static int u3_ukk(u3_ctx *x, int ab, int ac, int d, int s)
{
    if (!u3_within(x, ab, ac, d)) return -U3_INF;
    u3_cell *c = u3_U(x, ab, ac, d, s);
    if (c->stamp == d + x->off) return c->dist;
    u3_calc(x, ab, ac, d, s);
    c = u3_U(x, ab, ac, d, s);
    if (d >= x->cp_cost && d < x->cp_cost + x->cp_width) {
        u3_cp *p = u3_CP(x, ab, ac, d, s);
        p->dist = c->dist;
        p->cost = d + 1;
    }
    if (c->dist > x->furthest) x->furthest = c->dist;
    return c->dist;
}

/* furthest distance (or its state) over the states at (ab, ac, d) */
static int u3_best(u3_ctx *x, int ab, int ac, int d, int want_state)
{
    int best = -U3_INF, bs = -1;
    for (int s = 0; s < x->ns; s++) {
        u3_cell *c = u3_U(x, ab, ac, d, s);
        if (c->stamp == d + x->off && c->dist > best) {
            best = c->dist;
            bs = s;
        }
    }
    return want_state ? bs : best;
}

static void u3_emit(u3_ctx *x, int a, int b, int c)
{
    x->ea[x->n] = (uint8_t)a;
    x->eb[x->n] = (uint8_t)b;
    x->ec[x->n] = (uint8_t)c;
    x->n++;
}

/* base case: walk the `from` records back to the pass's start */
static void u3_traceback(u3_ctx *x, int sab, int sac, int scost, int sst,
                         int ab, int ac, int d, int s)
{
    while (ab != sab || ac != sac || d != scost || s != sst) {
        u3_cell *c = u3_U(x, ab, ac, d, s);
        int a = c->dist;
        u3_from f = c->from;
        int b = a - ab, cc = a - ac;
        int a1 = u3_U(x, f.ab, f.ac, f.cost, f.state)->dist;
        int b1 = a1 - f.ab, c1 = a1 - f.ac;
        while (a > a1 && b > b1 && cc > c1) {
            a--, b--, cc--;
            u3_emit(x, x->A[a], x->B[b], x->C[cc]);
        }
        if (a != a1 || b != b1 || cc != c1) {
            int ca = 16, cb = 16, ccc = 16;
            if (a > a1) ca = x->A[--a];
            if (b > b1) cb = x->B[--b];
            if (cc > c1) ccc = x->C[--cc];
            u3_emit(x, ca, cb, ccc);
        }
        ab = f.ab, ac = f.ac, d = f.cost, s = f.state;
    }
}

static void u3_split(u3_ctx *x, int sab, int sac, int scost, int sst, int sdist,
                     int fab, int fac, int fcost, int fst, int fdist);

static void u3_limits(u3_ctx *x, int sab, int sac, int scost, int sst, int sdist,
                      int fab, int fac, int fcost, int fst, int fdist)
{
    x->sab = sab, x->sac = sac, x->scost = scost, x->sstate = sst;
    x->endA = fdist, x->endB = fdist - fab, x->endC = fdist - fac;
    x->complete = 0;
    x->off += x->final_cost + 1;
    u3_cell *c = u3_U(x, sab, sac, scost, sst);
    c->dist = sdist;
    c->stamp = scost + x->off;
    if (fcost - scost <= x->cp_width) {
        x->complete = 1;
        int i = scost - 1, dist;
        do {
            i++;
            dist = u3_ukk(x, fab, fac, i, fst);
        } while (dist < fdist && !x->oom);
        fcost = i;
        u3_traceback(x, sab, sac, scost, sst, fab, fac, fcost, fst);
        x->complete = 0;
        return;
    }
    x->cp_cost = (fcost + scost - x->cp_width + 1) / 2;
    int i = scost - 1, dist;
    do {
        i++;
        u3_ukk(x, fab, fac, i, 0);
        dist = u3_ukk(x, fab, fac, i, fst);
    } while (dist < fdist && !x->oom);
    fcost = i;
    u3_split(x, sab, sac, scost, sst, sdist, fab, fac, fcost, fst, fdist);
}

static void u3_split(u3_ctx *x, int sab, int sac, int scost, int sst, int sdist,
                     int fab, int fac, int fcost, int fst, int fdist)
{
    u3_from f = u3_U(x, fab, fac, fcost, fst)->from;
    u3_cp *p = u3_CP(x, f.ab, f.ac, f.cost, f.state);
    if (p->cost == 0) p->cost = 1;
    int cpdist = p->dist;
    u3_limits(x, f.ab, f.ac, f.cost, f.state, cpdist, fab, fac, fcost, fst, fdist);
    u3_limits(x, sab, sac, scost, sst, sdist, f.ab, f.ac, f.cost, f.state, cpdist);
}

/* POY sequence (leading gap at 0) to the base string copySequence builds
 * (src/ukkCommon.c:85-104): the lowest of A, C, G, T in each position. */
static int u3_bases(const uint8_t *s, int len, uint8_t *out)
{
    for (int i = 1; i < len; i++) {
        uint8_t v = s[i];
        out[i - 1] = (v & 1) ? 1 : (v & 2) ? 2 : (v & 4) ? 4 : (v & 8) ? 8 : 0;
        if (!out[i - 1]) return -1;
    }
    return 0;
}

int orc_powell_3d(const uint8_t *a, int la, const uint8_t *b, int lb, const uint8_t *c,
                  int lc, int mm, int go, int ge, uint8_t *ra, uint8_t *rb, uint8_t *rc,
                  int *rlen, int *cost)
{
    if (la < 1 || lb < 1 || lc < 1 || la > U3_MAXLEN || lb > U3_MAXLEN || lc > U3_MAXLEN ||
        mm == 0 || go < 0 || ge <= 0)
        return -1;
    u3_ctx x;
    memset(&x, 0, sizeof(x));
    x.mm = mm, x.go = go, x.ge = ge;
    x.la = la - 1, x.lb = lb - 1, x.lc = lc - 1;
    int cap = la + lb + lc;
    x.A = malloc((size_t)la), x.B = malloc((size_t)lb), x.C = malloc((size_t)lc);
    x.ea = malloc((size_t)cap), x.eb = malloc((size_t)cap), x.ec = malloc((size_t)cap);
    int rcode = -1;
    if (!x.A || !x.B || !x.C || !x.ea || !x.eb || !x.ec) goto out;
    if (u3_bases(a, la, x.A) || u3_bases(b, lb, x.B) || u3_bases(c, lc, x.C)) {
        rcode = -2; /* failwith "This is impossible!" */
        goto out;
    }
    u3_setup(&x);
    x.cp_width = x.maxstep;
    if (!u3_store_init(&x.U, sizeof(u3_cell), 2 * x.maxstep, x.ns, x.la, x.lb, x.lc) ||
        !u3_store_init(&x.CP, sizeof(u3_cp), x.cp_width, x.ns, x.la, x.lb, x.lc))
        goto out;
    x.off = 1;
    x.furthest = -1;
    /* doUkk (src/ukk.checkp.c:111-212) */
    int start = 0;
    /* the reference reads B and C up to their terminating NUL, which no base
     * equals; the bounds below stop at the same place */
    while (start < x.la && start < x.lb && start < x.lc && x.A[start] == x.B[start] &&
           x.A[start] == x.C[start])
        start++;
    {
        u3_cell *c0 = u3_U(&x, 0, 0, 0, 0);
        c0->dist = start;
        c0->stamp = 0 + x.off;
    }
    const int fab = x.la - x.lb, fac = x.la - x.lc;
    x.endA = x.la, x.endB = x.lb, x.endC = x.lc;
    int cp_on_dist = 1;
    x.cp_cost = U3_INF;
    int d = -1;
    do {
        d++;
        u3_ukk(&x, fab, fac, d, 0);
        if (cp_on_dist && x.furthest >= x.la / 2) {
            x.cp_cost = d + 1;
            cp_on_dist = 0;
        }
    } while (u3_best(&x, fab, fac, d, 0) < x.la && !x.oom);
    x.final_cost = d;
    {
        int fst = u3_best(&x, fab, fac, d, 1);
        if (u3_U(&x, fab, fac, d, fst)->from.cost <= 0)
            u3_limits(&x, 0, 0, 0, 0, start, fab, fac, d, fst, x.la);
        else
            u3_split(&x, 0, 0, 0, 0, start, fab, fac, d, fst, x.la);
    }
    if (x.oom) goto out;
    /* printTraceBack (src/ukk.checkp.c:454-501): the leading run of matches,
     * then everything front to back behind the leading gap */
    for (int i = start - 1; i >= 0; i--) u3_emit(&x, x.A[i], x.B[i], x.C[i]);
    ra[0] = rb[0] = rc[0] = 16;
    for (int i = 0; i < x.n; i++) {
        ra[1 + i] = x.ea[x.n - 1 - i];
        rb[1 + i] = x.eb[x.n - 1 - i];
        rc[1 + i] = x.ec[x.n - 1 - i];
    }
    *rlen = x.n + 1;
    *cost = d;
    rcode = 0;
out:
    u3_store_free(&x.U);
    u3_store_free(&x.CP);
    free(x.A), free(x.B), free(x.C);
    free(x.ea), free(x.eb), free(x.ec);
    return rcode;
}

/* Many triples, OpenMP over triples (the CPU baseline's batch form): triple
 * k's sequences at seqs + off[3k + j], len[3k + j] bytes; its aligned
 * sequences end at ra/rb/rc + out_off[k] + len[3k] + len[3k+1] + len[3k+2]
 * (back to front, as seq_prepend leaves them). status[k]: 0, or the value
 * orc_powell_3d returned. */
int orc_powell_3d_batch(int n, const uint8_t *seqs, const int64_t *off, const int32_t *len,
                        int mm, int go, int ge, const int64_t *out_off, uint8_t *ra,
                        uint8_t *rb, uint8_t *rc, int32_t *rlen, int32_t *cost,
                        int32_t *status, int nthreads)
{
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1) reduction(+ : bad)
    for (int k = 0; k < n; k++) {
        const int la = len[3 * k], lb = len[3 * k + 1], lc = len[3 * k + 2];
        const int cap = la + lb + lc;
        uint8_t *ta = malloc((size_t)cap * 3);
        if (!ta) {
            status[k] = -1;
            bad++;
            continue;
        }
        uint8_t *tb = ta + cap, *tc = tb + cap;
        int m = 0, d = 0;
        int r = orc_powell_3d(seqs + off[3 * k], la, seqs + off[3 * k + 1], lb,
                              seqs + off[3 * k + 2], lc, mm, go, ge, ta, tb, tc, &m, &d);
        status[k] = r;
        if (r == 0) {
            const int64_t e = out_off[k] + cap;
            memcpy(ra + e - m, ta, (size_t)m);
            memcpy(rb + e - m, tb, (size_t)m);
            memcpy(rc + e - m, tc, (size_t)m);
            rlen[k] = m;
            cost[k] = d;
        } else {
            rlen[k] = 0;
            cost[k] = -1;
            bad++;
        }
        free(ta);
    }
    return bad;
}
