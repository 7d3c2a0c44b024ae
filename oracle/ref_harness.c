/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Harness around the reference POY alignment C code, compiled unmodified from
 * the POY source tree together with this file (see oracle/build_oracle.py).
 * It supplies the few OCaml runtime entry points the shim headers declare,
 * builds `struct cm` / `struct seq` / `struct matrices` blocks, and replays
 * the OCaml facade's call sequence around the reference stubs:
 *
 *   Sequence.Align.cost_2        src/sequence.ml:868-925 (deltaw, shorter first)
 *   Sequence.Align.create_edited_2  src/sequence.ml:1019-1033 (swap flag)
 *   Sequence.Align.align_2       src/sequence.ml:1061-1082
 *   Sequence.Align.align_affine_3   src/sequence.ml:633-649
 *   Sequence.Align.ancestor_2    src/sequence.ml:1114-1122
 *   Sequence.median_2_with_gaps  src/sequence.ml:473-481
 *   Sequence.Align.max_cost_2    src/sequence.ml:651-657
 *   SeqCS.DOS.median             src/seqCS.ml:1053-1071 (Algn_Normal branch)
 *
 * Nothing here is shipped; the product never links it.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <caml/mlvalues.h>
#include "seq.h"
#include "cm.h"
#include "matrices.h"
#include "poy_tables.h"

/* ---- OCaml runtime pieces used by the reference sources ---------------- */

static __thread jmp_buf *ref_jmp;
static __thread char ref_errmsg[256];

void caml_failwith(const char *msg)
{
    snprintf(ref_errmsg, sizeof(ref_errmsg), "%s", msg ? msg : "");
    if (ref_jmp) longjmp(*ref_jmp, 1);
    fprintf(stderr, "reference failwith outside a harness call: %s\n", msg);
    abort();
}
void caml_invalid_argument(const char *msg) { caml_failwith(msg); }

value caml_alloc_custom(struct custom_operations *ops, uintnat size,
                        mlsize_t mem, mlsize_t max)
{
    (void)mem;
    (void)max;
    value *blk = (value *)calloc(1, sizeof(value) + size);
    if (!blk) caml_failwith("out of memory");
    *(struct custom_operations **)blk = ops;
    return (value)blk;
}
void caml_register_custom_operations(struct custom_operations *ops) { (void)ops; }
value caml_alloc(mlsize_t wosize, tag_t tag)
{
    (void)tag;
    return (value)calloc(wosize + 1, sizeof(value));
}
value caml_alloc_tuple(mlsize_t wosize) { return caml_alloc(wosize, 0); }
value caml_copy_double(double d)
{
    double *p = (double *)malloc(sizeof(double));
    *p = d;
    return (value)p;
}
void caml_serialize_int_1(int i) { (void)i; }
void caml_serialize_int_2(int i) { (void)i; }
void caml_serialize_int_4(int32_t i) { (void)i; }
void caml_serialize_int_8(int64_t i) { (void)i; }
void caml_serialize_block_1(void *d, intnat l) { (void)d; (void)l; }
void caml_serialize_block_4(void *d, intnat l) { (void)d; (void)l; }
int caml_deserialize_sint_1(void) { return 0; }
int caml_deserialize_uint_1(void) { return 0; }
int caml_deserialize_sint_2(void) { return 0; }
int caml_deserialize_uint_2(void) { return 0; }
int32_t caml_deserialize_sint_4(void) { return 0; }
uint32_t caml_deserialize_uint_4(void) { return 0; }
int64_t caml_deserialize_sint_8(void) { return 0; }
void caml_deserialize_block_1(void *d, intnat l) { (void)d; (void)l; }
void caml_deserialize_block_4(void *d, intnat l) { (void)d; (void)l; }
value caml_ba_alloc(int flags, int nd, void *data, intnat *dim)
{
    (void)flags; (void)nd; (void)data; (void)dim;
    caml_failwith("bigarray not available in the oracle harness");
    return Val_unit;
}
value caml_ba_alloc_dims(int flags, int nd, void *data, ...)
{
    (void)flags; (void)nd; (void)data;
    caml_failwith("bigarray not available in the oracle harness");
    return Val_unit;
}

/* ---- reference entry points (defined in the reference algn.c unit) ---- */

value algn_CAML_simple_2(value, value, value, value, value);
value algn_CAML_backtrace_2d(value, value, value, value, value, value, value);
value algn_CAML_ancestor_2(value, value, value, value);
value algn_CAML_worst_2(value, value, value);
value algn_CAML_align_affine_3(value, value, value, value, value, value,
                               value, value, value);
value algn_CAML_cost_affine_3(value, value, value, value);
value seq_CAML_median_2_with_gaps(value, value, value, value);
value seq_CAML_count(value, value, value);
cmt cm_set_val(int, int, int, int, int, int, int, cmt, int, int, int, int);

/* ---- block helpers ------------------------------------------------------ */

static value mkseq(int cap, const uint8_t *data, int len)
{
    value v = caml_alloc_custom(NULL, sizeof(struct seq) + (size_t)cap, 0, 0);
    struct seq *s = (struct seq *)Data_custom_val(v);
    s->magic_number = POY_SEQ_MAGIC_NUMBER;
    s->cap = cap;
    s->len = len;
    s->head = (SEQT *)(s + 1);
    s->end = s->head + cap - 1;
    s->begin = s->end - len + 1;
    s->my_pool = NULL;
    if (len) memcpy(s->begin, data, (size_t)len);
    return v;
}

static int seqlen(value v)
{
    return ((struct seq *)Data_custom_val(v))->len;
}

static int getseq(value v, uint8_t *out, int cap)
{
    struct seq *s = (struct seq *)Data_custom_val(v);
    SEQT *head = (SEQT *)(s + 1);
    SEQT *begin = head + s->cap - s->len;
    int n = s->len < cap ? s->len : cap;
    memcpy(out, begin, (size_t)n);
    return s->len;
}

static void freeblk(value v) { free((void *)v); }

static int seq_is_empty(const uint8_t *s, int len, int gap)
{
    for (int i = 0; i < len; i++)
        if (s[i] != gap) return 0;
    return 1;
}

/* ---- cost matrix and workspace ------------------------------------------ */

typedef struct ref_cm {
    value blk;
    int gap;
} ref_cm;

void *ref_cm_new(const int *tcm, int alph, int gap_open)
{
    static orc_tables t; /* large; callers are single-threaded here */
    if (orc_tables_build(&t, tcm, alph, gap_open)) return NULL;
    ref_cm *r = (ref_cm *)calloc(1, sizeof(*r));
    jmp_buf jb;
    ref_jmp = &jb;
    if (setjmp(jb)) {
        ref_jmp = NULL;
        free(r);
        return NULL;
    }
    r->blk = caml_alloc_custom(NULL, sizeof(struct cm), 0, 0);
    cmt m = (cmt)Data_custom_val(r->blk);
    m->total_size = m->a_sz = m->lcm = m->gap = m->cost_model_type = m->gap_open =
        m->all_elements = m->ori_a_sz = m->map_sz = m->level = m->gap_startNO =
            m->tie_breaker = -1;
    /* fill_cost_matrix -> create: level 0 with combinations, num_comb = alph,
     * gap_start = num_comb - num_withgap + 1 (cost_matrix.ml:1145-1165) */
    cm_set_val(alph, 1, 0, 0, 0, 0, (1 << alph) - 1, m, 0, alph, alph + 1, 1);
    size_t n = (size_t)2 * (1u << m->lcm) * (1u << m->lcm);
    memcpy(m->cost, t.cost, n * sizeof(int));
    memcpy(m->worst, t.worst, n * sizeof(int));
    memcpy(m->tail_cost, t.tail, n * sizeof(int));
    memcpy(m->prepend_cost, t.prepend, n * sizeof(int));
    memcpy(m->median, t.median, n * sizeof(SEQT));
    m->is_metric = t.is_metric;
    m->is_identity = t.is_identity;
    if (gap_open > 0) {
        m->cost_model_type = 1; /* c_set_aff m 1 go */
        m->gap_open = gap_open;
    }
    r->gap = m->gap;
    ref_jmp = NULL;
    return r;
}

void ref_cm_free(void *p)
{
    ref_cm *r = (ref_cm *)p;
    if (!r) return;
    cmt m = (cmt)Data_custom_val(r->blk);
    free(m->combmap);
    free(m->comb2list);
    free(m->cost);
    free(m->worst);
    free(m->prepend_cost);
    free(m->tail_cost);
    free(m->median);
    freeblk(r->blk);
    free(r);
}

/* Copy out the tables the reference will use; returns the entry count. */
int ref_cm_tables(void *p, int *cost, uint8_t *median, int *worst, int *tail,
                  int *prepend, int *info)
{
    ref_cm *r = (ref_cm *)p;
    cmt m = (cmt)Data_custom_val(r->blk);
    int n = 2 * (1 << m->lcm) * (1 << m->lcm);
    if (cost) memcpy(cost, m->cost, (size_t)n * sizeof(int));
    if (worst) memcpy(worst, m->worst, (size_t)n * sizeof(int));
    if (tail) memcpy(tail, m->tail_cost, (size_t)n * sizeof(int));
    if (prepend) memcpy(prepend, m->prepend_cost, (size_t)n * sizeof(int));
    if (median) memcpy(median, m->median, (size_t)n);
    if (info) {
        info[0] = m->lcm;
        info[1] = m->gap;
        info[2] = m->a_sz;
        info[3] = m->combinations;
        info[4] = m->cost_model_type;
        info[5] = m->gap_open;
    }
    return n;
}

void *ref_ws_new(void)
{
    value v = caml_alloc_custom(NULL, sizeof(struct matrices), 0, 0);
    return (void *)v;
}

void ref_ws_free(void *p)
{
    value v = (value)p;
    struct matrices *m = (struct matrices *)Data_custom_val(v);
    free(m->matrix);
    free(m->matrix_d);
    free(m->precalc);
    free(m->gap_num1);
    free(m->gap_num2);
    free(m->gap_num3);
    free(m->gap_num4);
    free(m->pointers_3d);
    freeblk(v);
}

const char *ref_last_error(void) { return ref_errmsg; }

/* ---- the OCaml facade, replayed ----------------------------------------- */

static int count_gaps(value s, int gap)
{
    return Int_val(seq_CAML_count(Val_int(gap), Val_int(0), s));
}

/* Sequence.Align.cost_2 (linear). deltaw < 0 selects the None branch. */
static int cost_2(ref_cm *r, value ws, value s1, value s2, int deltaw)
{
    int ls1 = seqlen(s1), ls2 = seqlen(s2);
    int g1 = count_gaps(s1, r->gap), g2 = count_gaps(s2, r->gap);
    int gaps = g1 > g2 ? g1 : g2;
    int shortl = ls1 <= ls2 ? ls1 : ls2, longl = ls1 <= ls2 ? ls2 : ls1;
    int dif = shortl - longl;
    int lower = (int)((double)shortl * 0.10);
    int dw;
    if (deltaw < 0)
        dw = dif < lower ? lower / 2 : 2;
    else
        dw = dif < lower ? lower : deltaw;
    value res;
    if (ls1 <= ls2)
        res = algn_CAML_simple_2(s1, s2, r->blk, ws, Val_int(gaps + dw));
    else
        res = algn_CAML_simple_2(s2, s1, r->blk, ws, Val_int(gaps + dw));
    return Int_val(res);
}

int ref_cost_linear(void *cm, void *ws, const uint8_t *a, int la,
                    const uint8_t *b, int lb, int deltaw, int *cost)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    value sa = mkseq(la, a, la), sb = mkseq(lb, b, lb);
    int rc = 0;
    if (setjmp(jb)) {
        rc = -1;
    } else {
        *cost = cost_2(r, (value)ws, sa, sb, deltaw);
    }
    ref_jmp = NULL;
    freeblk(sa);
    freeblk(sb);
    return rc;
}

int ref_cost_affine(void *cm, void *ws, const uint8_t *a, int la,
                    const uint8_t *b, int lb, int *cost)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    value sa = mkseq(la, a, la), sb = mkseq(lb, b, lb);
    int rc = 0;
    if (setjmp(jb))
        rc = -1;
    else
        *cost = Int_val(algn_CAML_cost_affine_3(sa, sb, r->blk, (value)ws));
    ref_jmp = NULL;
    freeblk(sa);
    freeblk(sb);
    return rc;
}

/* algn_CAML_simple_2 as the OCaml external calls it (s1 = shorter). */
int ref_simple_2(void *cm, void *ws, const uint8_t *s1, int l1,
                 const uint8_t *s2, int l2, int deltawh, int *cost)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    value v1 = mkseq(l1, s1, l1), v2 = mkseq(l2, s2, l2);
    int rc = 0;
    if (setjmp(jb))
        rc = -1;
    else
        *cost = Int_val(algn_CAML_simple_2(v1, v2, r->blk, (value)ws, Val_int(deltawh)));
    ref_jmp = NULL;
    freeblk(v1);
    freeblk(v2);
    return rc;
}

/* algn_CAML_backtrace_2d on the workspace left by the last simple_2. */
int ref_backtrace_2d(void *cm, void *ws, const uint8_t *s1, int l1,
                     const uint8_t *s2, int l2, int swap, uint8_t *r1,
                     uint8_t *r2, int cap, int *len)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    value v1 = mkseq(l1, s1, l1), v2 = mkseq(l2, s2, l2);
    value p1 = mkseq(cap, NULL, 0), p2 = mkseq(cap, NULL, 0);
    int rc = 0;
    if (setjmp(jb)) {
        rc = -1;
    } else {
        algn_CAML_backtrace_2d(v1, v2, p1, p2, (value)ws, r->blk, Val_bool(swap));
        *len = getseq(p1, r1, cap);
        getseq(p2, r2, cap);
    }
    ref_jmp = NULL;
    freeblk(v1);
    freeblk(v2);
    freeblk(p1);
    freeblk(p2);
    return rc;
}

/* algn_CAML_backtrace_2d_limit (src/algn.c:3448) from (st_s1, st_s2,
 * algn_s1, algn_s2) on the workspace left by the last simple_2 / limit_2. */
value algn_CAML_backtrace_2d_limit(value, value, value, value, value, value, value,
                                   value, value, value, value);
int ref_backtrace_2d_limit(void *cm, void *ws, const uint8_t *s1, int l1,
                           const uint8_t *s2, int l2, int st_s1, int st_s2,
                           int algn_s1, int algn_s2, int swaped, uint8_t *r1,
                           uint8_t *r2, int cap, int *len)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    value v1 = mkseq(l1, s1, l1), v2 = mkseq(l2, s2, l2);
    value p1 = mkseq(cap, NULL, 0), p2 = mkseq(cap, NULL, 0);
    int rc = 0;
    if (setjmp(jb)) {
        rc = -1;
    } else {
        algn_CAML_backtrace_2d_limit(v1, v2, p1, p2, (value)ws, r->blk, Val_int(st_s1),
                                     Val_int(st_s2), Val_int(algn_s1), Val_int(algn_s2),
                                     Val_bool(swaped));
        *len = getseq(p1, r1, cap);
        getseq(p2, r2, cap);
    }
    ref_jmp = NULL;
    freeblk(v1);
    freeblk(v2);
    freeblk(p1);
    freeblk(p2);
    return rc;
}

/*
 * SeqCS.DOS.median, linear cost model, Algn_Normal (seqCS.ml:1059-1071):
 * align_2 (cost_2 + create_edited_2), ancestor_2, median_2_with_gaps and
 * max_cost_2, all in the caller's (a, b) order. Output capacities: ea, eb
 * and mwg la+lb; anc la+lb+1.
 */
int ref_median_linear(void *cm, void *ws, const uint8_t *a, int la,
                      const uint8_t *b, int lb, int *cost, uint8_t *ea,
                      uint8_t *eb, int *elen, uint8_t *anc, int *anclen,
                      uint8_t *mwg, int *mwglen, int *maxcost)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    value sa = mkseq(la, a, la), sb = mkseq(lb, b, lb);
    value pa = mkseq(la + lb, NULL, 0), pb = mkseq(la + lb, NULL, 0);
    value sm = 0, swg = 0;
    int rc = 0;
    if (setjmp(jb)) {
        rc = -1;
    } else {
        *cost = cost_2(r, (value)ws, sa, sb, -1);
        if (la <= lb)
            algn_CAML_backtrace_2d(sa, sb, pa, pb, (value)ws, r->blk, Val_bool(0));
        else
            algn_CAML_backtrace_2d(sb, sa, pb, pa, (value)ws, r->blk, Val_bool(1));
        int L = seqlen(pa);
        sm = mkseq(L + 1, NULL, 0);
        algn_CAML_ancestor_2(pa, pb, r->blk, sm);
        swg = mkseq(L, NULL, 0);
        seq_CAML_median_2_with_gaps(pa, pb, r->blk, swg);
        *elen = getseq(pa, ea, la + lb);
        getseq(pb, eb, la + lb);
        *anclen = getseq(sm, anc, la + lb + 1);
        *mwglen = getseq(swg, mwg, la + lb);
        if (seq_is_empty(ea, L, r->gap) || seq_is_empty(eb, L, r->gap))
            *maxcost = 0;
        else
            *maxcost = Int_val(algn_CAML_worst_2(pa, pb, r->blk));
    }
    ref_jmp = NULL;
    freeblk(sa);
    freeblk(sb);
    freeblk(pa);
    freeblk(pb);
    if (sm) freeblk(sm);
    if (swg) freeblk(swg);
    return rc;
}

/*
 * SeqCS.DOS.median, affine cost model (seqCS.ml:1053-1058): align_affine_3
 * then max_cost_2 on the aligned pair in caller order. Capacities: la+lb+2.
 */
int ref_median_affine(void *cm, void *ws, const uint8_t *a, int la,
                      const uint8_t *b, int lb, int *cost, uint8_t *med,
                      int *medlen, uint8_t *ea, uint8_t *eb, int *elen,
                      uint8_t *mwg, int *mwglen, int *maxcost)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    int swaped = la <= lb ? 0 : 1;
    const uint8_t *si = swaped ? b : a, *sj = swaped ? a : b;
    int li = swaped ? lb : la, lj = swaped ? la : lb;
    int cap = la + lb + 2;
    value vi = mkseq(li, si, li), vj = mkseq(lj, sj, lj);
    value ri = mkseq(cap, NULL, 0), rj = mkseq(cap, NULL, 0);
    value vm = mkseq(cap, NULL, 0), vwg = mkseq(cap, NULL, 0);
    int rc = 0;
    if (setjmp(jb)) {
        rc = -1;
    } else {
        *cost = Int_val(algn_CAML_align_affine_3(vi, vj, r->blk, (value)ws, ri, rj,
                                                 vm, vwg, Val_int(swaped)));
        value va = swaped ? rj : ri, vb = swaped ? ri : rj;
        *elen = getseq(va, ea, cap);
        getseq(vb, eb, cap);
        *medlen = getseq(vm, med, cap);
        *mwglen = getseq(vwg, mwg, cap);
        if (seq_is_empty(ea, *elen, r->gap) || seq_is_empty(eb, *elen, r->gap))
            *maxcost = 0;
        else
            *maxcost = Int_val(algn_CAML_worst_2(va, vb, r->blk));
    }
    ref_jmp = NULL;
    freeblk(vi);
    freeblk(vj);
    freeblk(ri);
    freeblk(rj);
    freeblk(vm);
    freeblk(vwg);
    return rc;
}

/* ---- Algn_Newkk (src/newkkonen.c, compiled unmodified alongside) --------- */

value newkkonen_CAML_create_general(value);
value newkkonen_CAML_algn_affine(value, value, value, value, value);
value newkkonen_CAML_backtrace_affine(value, value, value, value, value, value, value);
void newkkmat_CAML_free(value);

/*
 * Sequence.NewkkAlign.align_2 (sequence.ml:1879-1901) under an affine cm, on a
 * fresh newkk matrix: shorter sequence first (swaped = 1 when b is shorter),
 * newkkonen_CAML_algn_affine then newkkonen_CAML_backtrace_affine; the aligned
 * pair comes back in the caller's (a, b) order (capacity la + lb each).
 */
int ref_newkk_align2(void *cm, const uint8_t *a, int la, const uint8_t *b,
                     int lb, int *cost, uint8_t *ea, uint8_t *eb, int *elen)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    int swaped = la <= lb ? 0 : 1;
    value sa = mkseq(la, a, la), sb = mkseq(lb, b, lb);
    value pa = mkseq(la + lb, NULL, 0), pb = mkseq(la + lb, NULL, 0);
    value mat = newkkonen_CAML_create_general(Val_unit);
    int rc = 0;
    if (setjmp(jb)) {
        rc = -1;
    } else {
        value s1 = swaped ? sb : sa, s2 = swaped ? sa : sb;
        value p1 = swaped ? pb : pa, p2 = swaped ? pa : pb;
        *cost = Int_val(newkkonen_CAML_algn_affine(s1, s2, r->blk, mat, Val_int(swaped)));
        newkkonen_CAML_backtrace_affine(s1, s2, p1, p2, r->blk, mat, Val_int(swaped));
        *elen = getseq(pa, ea, la + lb);
        getseq(pb, eb, la + lb);
    }
    ref_jmp = NULL;
    newkkmat_CAML_free(mat);
    freeblk(mat);
    freeblk(sa);
    freeblk(sb);
    freeblk(pa);
    freeblk(pb);
    return rc;
}

/*
 * SeqCS.DOS.median with use_ukk, affine (seqCS.ml:1043-1051): align_2 as
 * above, then ancestor_2, median_2_with_gaps and max_cost_2 in caller order.
 * Capacities: ea, eb, mwg la+lb; anc la+lb+1.
 */
int ref_newkk_median(void *cm, const uint8_t *a, int la, const uint8_t *b,
                     int lb, int *cost, uint8_t *ea, uint8_t *eb, int *elen,
                     uint8_t *anc, int *anclen, uint8_t *mwg, int *mwglen,
                     int *maxcost)
{
    ref_cm *r = (ref_cm *)cm;
    if (ref_newkk_align2(cm, a, la, b, lb, cost, ea, eb, elen)) return -1;
    int L = *elen;
    jmp_buf jb;
    ref_jmp = &jb;
    value pa = mkseq(L, ea, L), pb = mkseq(L, eb, L);
    value sm = mkseq(L + 1, NULL, 0), swg = mkseq(L, NULL, 0);
    int rc = 0;
    if (setjmp(jb)) {
        rc = -1;
    } else {
        algn_CAML_ancestor_2(pa, pb, r->blk, sm);
        seq_CAML_median_2_with_gaps(pa, pb, r->blk, swg);
        *anclen = getseq(sm, anc, la + lb + 1);
        *mwglen = getseq(swg, mwg, la + lb);
        if (seq_is_empty(ea, L, r->gap) || seq_is_empty(eb, L, r->gap))
            *maxcost = 0;
        else
            *maxcost = Int_val(algn_CAML_worst_2(pa, pb, r->blk));
    }
    ref_jmp = NULL;
    freeblk(pa);
    freeblk(pb);
    freeblk(sm);
    freeblk(swg);
    return rc;
}

/* ---- the remaining per-call externals ------------------------------------ */

value algn_CAML_limit_2(value, value, value, value, value, value, value, value,
                        value, value);
value algn_CAML_verify_2(value, value, value);
value seq_CAML_median_2_no_gaps(value, value, value, value);

/* algn_CAML_limit_2 (src/algn.c:3160), the reference's argument order. */
int ref_limit_2(void *cm, void *ws, const uint8_t *s1, int l1, const uint8_t *s2,
                int l2, int w, int h, int s1_st, int s2_st, int s1_len,
                int s2_len, int *cost)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    value v1 = mkseq(l1, s1, l1), v2 = mkseq(l2, s2, l2);
    int rc = 0;
    if (setjmp(jb))
        rc = -1;
    else
        *cost = Int_val(algn_CAML_limit_2(v1, v2, r->blk, (value)ws, Val_int(w),
                                          Val_int(h), Val_int(s1_st), Val_int(s2_st),
                                          Val_int(s1_len), Val_int(s2_len)));
    ref_jmp = NULL;
    freeblk(v1);
    freeblk(v2);
    return rc;
}

/* algn_CAML_verify_2 and seq_CAML_median_2_no_gaps on an aligned pair;
 * out holds len + 1 bytes (front-aligned on return). */
int ref_verify_and_nogap(void *cm, const uint8_t *a, const uint8_t *b, int len,
                         int *cost, uint8_t *out, int *outlen)
{
    ref_cm *r = (ref_cm *)cm;
    jmp_buf jb;
    ref_jmp = &jb;
    value va = mkseq(len, a, len), vb = mkseq(len, b, len);
    value vm = mkseq(len + 1, NULL, 0);
    int rc = 0;
    if (setjmp(jb)) {
        rc = -1;
    } else {
        *cost = Int_val(algn_CAML_verify_2(va, vb, r->blk));
        seq_CAML_median_2_no_gaps(va, vb, r->blk, vm);
        *outlen = getseq(vm, out, len + 1);
    }
    ref_jmp = NULL;
    freeblk(va);
    freeblk(vb);
    freeblk(vm);
    return rc;
}

/* powell_3D_align (src/ukkCommon.c:109-145), as Sequence.Align.align_3_powell
 * (src/sequence.ml:1312-1321) calls it: three POY sequences with their
 * leading gap, result sequences of capacity la + lb + lc. The reference keeps
 * its state in globals, so calls must not overlap. */
value powell_3D_align(value, value, value, value, value, value, value, value, value);

int ref_powell_3d(const uint8_t *a, int la, const uint8_t *b, int lb,
                  const uint8_t *c, int lc, int mm, int go, int ge,
                  uint8_t *ra, uint8_t *rb, uint8_t *rc_, int *rlen, int *cost)
{
    jmp_buf jb;
    ref_jmp = &jb;
    int cap = la + lb + lc;
    value va = mkseq(la, a, la), vb = mkseq(lb, b, lb), vc = mkseq(lc, c, lc);
    value wa = mkseq(cap, NULL, 0), wb = mkseq(cap, NULL, 0), wc = mkseq(cap, NULL, 0);
    int rc = 0;
    if (setjmp(jb)) {
        rc = -1;
    } else {
        *cost = Int_val(powell_3D_align(va, vb, vc, wa, wb, wc, Val_int(mm),
                                        Val_int(go), Val_int(ge)));
        *rlen = getseq(wa, ra, cap);
        getseq(wb, rb, cap);
        getseq(wc, rc_, cap);
    }
    ref_jmp = NULL;
    freeblk(va);
    freeblk(vb);
    freeblk(vc);
    freeblk(wa);
    freeblk(wb);
    freeblk(wc);
    return rc;
}
