/*
 * POY-side stub library: the OCaml externals of POY's direct-optimization
 * alignment path, defined over libpoyalgn.so (include/poyalgn.h).
 *
 * A POY maintainer compiles this file against POY's own headers (seq.h,
 * cm.h and the OCaml runtime headers), links it in place of the
 * definitions in src/algn.c / src/seq.c / src/newkkonen.c / src/ukkCommon.c
 * that it replaces,
 * and links -lpoyalgn. No OCaml changes: every symbol keeps the name and
 * argument list of the external it replaces (file:line in the POY 5.1.1
 * source tree beside each one), including the bytecode twins (_bc) of the
 * stubs with more than five arguments.
 *
 * Conventions kept from POY: sequences are read from the struct seq custom
 * blocks (Seq_custom_val), outputs are prepended into the caller-allocated
 * blocks exactly as seq_prepend leaves them, and errors become failwith.
 * Every buffer a stub allocates is freed before it fails. One context per
 * process plays the role of POY's Matrix.default workspace (the matrices
 * argument is accepted and unused); the device copy of a cost matrix is
 * rebuilt when a stub sees a different struct cm.
 */
#include <assert.h>
#include <stdint.h>
#include <stdlib.h>

#include <caml/fail.h>
#include <caml/memory.h>
#include <caml/mlvalues.h>

#include "cm.h"
#include "poyalgn.h"
#include "seq.h"

static poyalgn_ctx *g_ctx; /* the process-wide workspace */

static poyalgn_ctx *ctx(void)
{
    if (!g_ctx && poyalgn_init(0, &g_ctx) != 0) failwith((char *)poyalgn_last_error());
    return g_ctx;
}

/* failwith with the library's message, after freeing up to two buffers */
static void fail_free(void *a, void *b)
{
    free(a);
    free(b);
    failwith((char *)poyalgn_last_error());
}

static void *alloc_or_fail(size_t n, void *held)
{
    void *p = malloc(n > 0 ? n : 1);
    if (!p) {
        free(held);
        failwith("poyalgn stubs: out of memory");
    }
    return p;
}

/* device tables of a struct cm, rebuilt when the matrix changes */
static const poyalgn_cm *gpu_cm(cmt c)
{
    static cmt last_c;
    static poyalgn_cm *last;
    if (c != last_c) {
        if (last) poyalgn_cm_free(last);
        last = NULL;
        last_c = NULL;
        if (poyalgn_cm_adopt(ctx(), c->lcm, c->gap, c->a_sz, c->combinations,
                             c->cost_model_type, c->gap_open, c->cost, c->median, c->worst,
                             c->tail_cost, c->prepend_cost, &last) != 0)
            failwith((char *)poyalgn_last_error());
        last_c = c;
    }
    return last;
}

/* prepend the n bytes that end at buf[cap - 1] to s, as seq_prepend does */
static void fill_seq(seqt s, const unsigned char *buf, int cap, int n)
{
    for (int i = n - 1; i >= 0; i--) seq_prepend(s, buf[cap - n + i]);
}

/* ---- linear model ------------------------------------------------------- */

/* algn_CAML_simple_2 (src/algn.c:3133) */
value algn_CAML_simple_2(value s1, value s2, value c, value a, value deltawh)
{
    CAMLparam5(s1, s2, c, a, deltawh);
    seqt p1, p2;
    int32_t cost;
    Seq_custom_val(p1, s1);
    Seq_custom_val(p2, s2);
    if (poyalgn_simple_2(ctx(), gpu_cm(Cost_matrix_struct(c)), p1->begin, p1->len, p2->begin,
                         p2->len, Int_val(deltawh), &cost) != 0)
        failwith((char *)poyalgn_last_error());
    CAMLreturn(Val_int(cost));
}

/* algn_CAML_backtrace_2d (src/algn.c:3423) */
value algn_CAML_backtrace_2d(value s1, value s2, value s1p, value s2p, value a, value c,
                             value swap)
{
    CAMLparam5(s1, s2, s1p, s2p, a);
    CAMLxparam2(c, swap);
    seqt p1, p2, r1, r2;
    int32_t len;
    Seq_custom_val(p1, s1);
    Seq_custom_val(p2, s2);
    Seq_custom_val(r1, s1p);
    Seq_custom_val(r2, s2p);
    const int cap = r1->cap - r1->len;
    unsigned char *b1 = alloc_or_fail(cap, NULL);
    unsigned char *b2 = alloc_or_fail(cap, b1);
    if (poyalgn_backtrace_2d(ctx(), gpu_cm(Cost_matrix_struct(c)), p1->begin, p1->len,
                             p2->begin, p2->len, b1, b2, cap, &len, Bool_val(swap)) != 0)
        fail_free(b1, b2);
    fill_seq(r1, b1, cap, len);
    fill_seq(r2, b2, cap, len);
    free(b1);
    free(b2);
    CAMLreturn(Val_unit);
}

/* algn_CAML_backtrace_2d_bc (src/algn.c:3442) */
value algn_CAML_backtrace_2d_bc(value *argv, int argn)
{
    (void)argn;
    return algn_CAML_backtrace_2d(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5],
                                  argv[6]);
}

/* algn_CAML_align_2d (src/algn.c:3502): simple_2, then backtrace_2d */
value algn_CAML_align_2d(value s1, value s2, value c, value a, value s1p, value s2p,
                         value deltawh, value swaped)
{
    CAMLparam5(s1, s2, c, a, s1p);
    CAMLxparam3(s2p, deltawh, swaped);
    seqt p1, p2, r1, r2;
    int32_t len, cost;
    Seq_custom_val(p1, s1);
    Seq_custom_val(p2, s2);
    Seq_custom_val(r1, s1p);
    Seq_custom_val(r2, s2p);
    const int cap = r1->cap - r1->len;
    unsigned char *b1 = alloc_or_fail(cap, NULL);
    unsigned char *b2 = alloc_or_fail(cap, b1);
    if (poyalgn_align_2d(ctx(), gpu_cm(Cost_matrix_struct(c)), p1->begin, p1->len, p2->begin,
                         p2->len, b1, b2, cap, &len, Int_val(deltawh), Bool_val(swaped),
                         &cost) != 0)
        fail_free(b1, b2);
    fill_seq(r1, b1, cap, len);
    fill_seq(r2, b2, cap, len);
    free(b1);
    free(b2);
    CAMLreturn(Val_int(cost));
}

/* algn_CAML_align_2d_bc (src/algn.c:3514) */
value algn_CAML_align_2d_bc(value *argv, int argn)
{
    (void)argn;
    return algn_CAML_align_2d(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6],
                              argv[7]);
}

/* algn_CAML_limit_2 (src/algn.c:3160) */
value algn_CAML_limit_2(value s1, value s2, value c, value a, value w, value h, value s1_st,
                        value s2_st, value s1_len, value s2_len)
{
    CAMLparam5(s1, s2, c, a, w);
    CAMLxparam5(h, s1_st, s2_st, s1_len, s2_len);
    seqt p1, p2;
    int32_t cost;
    Seq_custom_val(p1, s1);
    Seq_custom_val(p2, s2);
    if (poyalgn_limit_2(ctx(), gpu_cm(Cost_matrix_struct(c)), p1->begin, p1->len, p2->begin,
                        p2->len, Int_val(w), Int_val(h), Int_val(s1_st), Int_val(s2_st),
                        Int_val(s1_len), Int_val(s2_len), &cost) != 0)
        failwith((char *)poyalgn_last_error());
    CAMLreturn(Val_int(cost));
}

/* algn_CAML_limit_2_bc (src/algn.c:3187) */
value algn_CAML_limit_2_bc(value *argv, int argn)
{
    (void)argn;
    return algn_CAML_limit_2(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6],
                             argv[7], argv[8], argv[9]);
}

/* algn_CAML_backtrace_2d_limit (src/algn.c:3448) */
value algn_CAML_backtrace_2d_limit(value s1, value s2, value s1p, value s2p, value a, value c,
                                   value st_s1, value st_s2, value algn_s1, value algn_s2,
                                   value swaped)
{
    CAMLparam5(s1, s2, s1p, s2p, a);
    CAMLxparam5(c, st_s1, st_s2, algn_s1, algn_s2);
    CAMLxparam1(swaped);
    seqt p1, p2, r1, r2;
    int32_t len;
    Seq_custom_val(p1, s1);
    Seq_custom_val(p2, s2);
    Seq_custom_val(r1, s1p);
    Seq_custom_val(r2, s2p);
    const int cap = r1->cap - r1->len;
    unsigned char *b1 = alloc_or_fail(cap, NULL);
    unsigned char *b2 = alloc_or_fail(cap, b1);
    if (poyalgn_backtrace_2d_limit(ctx(), gpu_cm(Cost_matrix_struct(c)), p1->begin, p1->len,
                                   p2->begin, p2->len, b1, b2, cap, &len, Int_val(st_s1),
                                   Int_val(st_s2), Int_val(algn_s1), Int_val(algn_s2),
                                   Bool_val(swaped)) != 0)
        fail_free(b1, b2);
    fill_seq(r1, b1, cap, len);
    fill_seq(r2, b2, cap, len);
    free(b1);
    free(b2);
    CAMLreturn(Val_unit);
}

/* algn_CAML_backtrace_2d_limit_bc (src/algn.c:3471) */
value algn_CAML_backtrace_2d_limit_bc(value *argv, int argn)
{
    (void)argn;
    return algn_CAML_backtrace_2d_limit(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5],
                                        argv[6], argv[7], argv[8], argv[9], argv[10]);
}

/* ---- affine model ------------------------------------------------------- */

/* algn_CAML_align_affine_3 (src/algn.c:2358) */
value algn_CAML_align_affine_3(value si, value sj, value cm, value am, value resi, value resj,
                               value median, value medianwg, value swaped)
{
    CAMLparam4(si, sj, cm, am);
    CAMLxparam5(resi, resj, median, medianwg, swaped);
    seqt a, b, ri, rj, m, mw;
    int32_t lens[3], cost;
    Seq_custom_val(a, si);
    Seq_custom_val(b, sj);
    Seq_custom_val(ri, resi);
    Seq_custom_val(rj, resj);
    Seq_custom_val(m, median);
    Seq_custom_val(mw, medianwg);
    const int cap = ri->cap - ri->len;
    unsigned char *buf = alloc_or_fail(4 * (size_t)cap, NULL);
    if (poyalgn_align_affine_3(ctx(), gpu_cm(Cost_matrix_struct(cm)), a->begin, a->len,
                               b->begin, b->len, buf, buf + cap, buf + 2 * cap, buf + 3 * cap,
                               cap, lens, Int_val(swaped), &cost) != 0)
        fail_free(buf, NULL);
    fill_seq(ri, buf, cap, lens[0]);
    fill_seq(rj, buf + cap, cap, lens[0]);
    fill_seq(m, buf + 2 * cap, cap, lens[1]);
    fill_seq(mw, buf + 3 * cap, cap, lens[2]);
    free(buf);
    CAMLreturn(Val_int(cost));
}

/* algn_CAML_align_affine_3_bc (src/algn.c:2449) */
value algn_CAML_align_affine_3_bc(value *argv, int argn)
{
    (void)argn;
    return algn_CAML_align_affine_3(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5],
                                    argv[6], argv[7], argv[8]);
}

/* algn_CAML_cost_affine_3 (src/algn.c:2456) */
value algn_CAML_cost_affine_3(value si, value sj, value cm, value am)
{
    CAMLparam4(si, sj, cm, am);
    seqt a, b;
    int32_t cost;
    Seq_custom_val(a, si);
    Seq_custom_val(b, sj);
    if (poyalgn_cost_affine_3(ctx(), gpu_cm(Cost_matrix_struct(cm)), a->begin, a->len,
                              b->begin, b->len, &cost) != 0)
        failwith((char *)poyalgn_last_error());
    CAMLreturn(Val_int(cost));
}

/* ---- medians and costs of an aligned pair --------------------------------- */

/* algn_CAML_ancestor_2 (src/algn.c:3741): the ancestor of an aligned pair */
value algn_CAML_ancestor_2(value sa, value sb, value cm, value sab)
{
    CAMLparam4(sa, sb, cm, sab);
    seqt a, b, ab;
    int32_t n, worst;
    Seq_custom_val(a, sa);
    Seq_custom_val(b, sb);
    Seq_custom_val(ab, sab);
    const int cap = ab->cap - ab->len;
    unsigned char *anc = alloc_or_fail(cap, NULL);
    unsigned char *mwg = alloc_or_fail(a->len, anc);
    if (poyalgn_aligned_medians(ctx(), gpu_cm(Cost_matrix_struct(cm)), a->begin, b->begin,
                                a->len, anc, cap, &n, mwg, &worst) != 0)
        fail_free(anc, mwg);
    fill_seq(ab, anc, cap, n);
    free(anc);
    free(mwg);
    CAMLreturn(Val_unit);
}

/* algn_CAML_worst_2 (src/algn.c:3107): worst cost of an aligned pair */
value algn_CAML_worst_2(value s1, value s2, value c)
{
    CAMLparam3(s1, s2, c);
    seqt a, b;
    int32_t n, worst;
    Seq_custom_val(a, s1);
    Seq_custom_val(b, s2);
    const int cap = a->len + 1;
    unsigned char *anc = alloc_or_fail(cap, NULL);
    unsigned char *mwg = alloc_or_fail(a->len, anc);
    if (poyalgn_aligned_medians(ctx(), gpu_cm(Cost_matrix_struct(c)), a->begin, b->begin,
                                a->len, anc, cap, &n, mwg, &worst) != 0)
        fail_free(anc, mwg);
    free(anc);
    free(mwg);
    CAMLreturn(Val_int(worst));
}

/* algn_CAML_verify_2 (src/algn.c:3120) */
value algn_CAML_verify_2(value s1, value s2, value c)
{
    CAMLparam3(s1, s2, c);
    seqt a, b;
    int32_t cost;
    Seq_custom_val(a, s1);
    Seq_custom_val(b, s2);
    if (poyalgn_verify_2(ctx(), gpu_cm(Cost_matrix_struct(c)), a->begin, b->begin, a->len,
                         &cost) != 0)
        failwith((char *)poyalgn_last_error());
    CAMLreturn(Val_int(cost));
}

/* seq_CAML_median_2_no_gaps (src/seq.c:274) */
value seq_CAML_median_2_no_gaps(value s1, value s2, value m, value sm)
{
    CAMLparam4(s1, s2, m, sm);
    seqt a, b, out;
    int32_t n;
    Seq_custom_val(a, s1);
    Seq_custom_val(b, s2);
    Seq_custom_val(out, sm);
    const int cap = out->cap - out->len;
    unsigned char *buf = alloc_or_fail(cap, NULL);
    if (poyalgn_median_2_no_gaps(ctx(), gpu_cm(Cost_matrix_struct(m)), a->begin, b->begin,
                                 a->len, buf, cap, &n) != 0)
        fail_free(buf, NULL);
    fill_seq(out, buf, cap, n);
    free(buf);
    CAMLreturn(Val_unit);
}

/* seq_CAML_median_2_with_gaps (src/seq.c:287): one median per aligned column */
value seq_CAML_median_2_with_gaps(value s1, value s2, value m, value sm)
{
    CAMLparam4(s1, s2, m, sm);
    seqt a, b, out;
    int32_t n, worst;
    Seq_custom_val(a, s1);
    Seq_custom_val(b, s2);
    Seq_custom_val(out, sm);
    const int cap = a->len + 1;
    unsigned char *anc = alloc_or_fail(cap, NULL);
    unsigned char *mwg = alloc_or_fail(a->len, anc);
    if (poyalgn_aligned_medians(ctx(), gpu_cm(Cost_matrix_struct(m)), a->begin, b->begin,
                                a->len, anc, cap, &n, mwg, &worst) != 0)
        fail_free(anc, mwg);
    fill_seq(out, mwg, a->len, a->len);
    free(anc);
    free(mwg);
    CAMLreturn(Val_unit);
}

/* ---- Algn_Newkk, affine (Sequence.NewkkAlign) ---------------------------------
 * The ukkm block OCaml passes is accepted and unused: the context keeps the
 * alignment of the last newkk_cost2_affine call, as the reference keeps it
 * in that block. */

/* newkkonen_CAML_algn_affine (src/newkkonen.c:1473) */
value newkkonen_CAML_algn_affine(value s1, value s2, value c, value a, value swaped)
{
    CAMLparam5(s1, s2, c, a, swaped);
    seqt p1, p2;
    int32_t cost;
    Seq_custom_val(p1, s1);
    Seq_custom_val(p2, s2);
    if (poyalgn_newkk_algn_affine(ctx(), gpu_cm(Cost_matrix_struct(c)), p1->begin, p1->len,
                                  p2->begin, p2->len, Int_val(swaped), &cost) != 0)
        failwith((char *)poyalgn_last_error());
    CAMLreturn(Val_int(cost));
}

/* newkkonen_CAML_backtrace_affine (src/newkkonen.c:1788) */
value newkkonen_CAML_backtrace_affine(value s1, value s2, value s1p, value s2p, value c,
                                      value a, value swaped)
{
    CAMLparam5(s1, s2, s1p, s2p, c);
    CAMLxparam2(a, swaped);
    seqt p1, p2, r1, r2;
    int32_t len;
    Seq_custom_val(p1, s1);
    Seq_custom_val(p2, s2);
    Seq_custom_val(r1, s1p);
    Seq_custom_val(r2, s2p);
    const int cap = r1->cap - r1->len;
    unsigned char *b1 = alloc_or_fail(cap, NULL);
    unsigned char *b2 = alloc_or_fail(cap, b1);
    if (poyalgn_newkk_backtrace_affine(ctx(), gpu_cm(Cost_matrix_struct(c)), p1->begin,
                                       p1->len, p2->begin, p2->len, b1, b2, cap, &len,
                                       Int_val(swaped)) != 0)
        fail_free(b1, b2);
    fill_seq(r1, b1, cap, len);
    fill_seq(r2, b2, cap, len);
    free(b1);
    free(b2);
    CAMLreturn(Val_unit);
}

/* newkkonen_CAML_backtrace_affine_bc (src/newkkonen.c:1812). The reference's
 * twin calls the linear backtrace; this one forwards to the affine stub, the
 * function its name and argument list stand for. */
value newkkonen_CAML_backtrace_affine_bc(value *argv, int argn)
{
    (void)argn;
    return newkkonen_CAML_backtrace_affine(argv[0], argv[1], argv[2], argv[3], argv[4],
                                           argv[5], argv[6]);
}

/* newkkonen_CAML_get_k (src/newkkonen.c:247) */
value newkkonen_CAML_get_k(value m)
{
    CAMLparam1(m);
    int32_t k = 0;
    if (poyalgn_newkk_get_k(ctx(), &k) != 0) failwith((char *)poyalgn_last_error());
    CAMLreturn(Val_int(k));
}

/* ---- three-sequence alignment ------------------------------------------ */

/* powell_3D_align (src/ukkCommon.c:109), the external `powell_3d` of
 * Sequence.Align (src/sequence.ml:1309): the aligned sequences are
 * prepended into ra, rb, rc (created by align_3_powell with capacity
 * la + lb + lc) and the alignment cost returned. */
value powell_3D_align(value sa, value sb, value sc, value ra, value rb, value rc, value mm,
                      value go, value ge)
{
    CAMLparam5(sa, sb, sc, mm, go);
    CAMLxparam4(ge, ra, rb, rc);
    seqt a, b, c, wa, wb, wc;
    int32_t len = 0, cost = 0;
    Seq_custom_val(a, sa);
    Seq_custom_val(b, sb);
    Seq_custom_val(c, sc);
    Seq_custom_val(wa, ra);
    Seq_custom_val(wb, rb);
    Seq_custom_val(wc, rc);
    const int cap = a->len + b->len + c->len;
    unsigned char *buf = alloc_or_fail((size_t)cap * 3, NULL);
    if (poyalgn_powell_3d(ctx(), a->begin, a->len, b->begin, b->len, c->begin, c->len,
                          Int_val(mm), Int_val(go), Int_val(ge), buf, buf + cap, buf + 2 * cap,
                          cap, &len, &cost) != 0)
        fail_free(buf, NULL);
    fill_seq(wa, buf, cap, len);
    fill_seq(wb, buf + cap, cap, len);
    fill_seq(wc, buf + 2 * cap, cap, len);
    free(buf);
    CAMLreturn(Val_int(cost));
}

/* powell_3D_align_bc (src/ukkCommon.c:147) */
value powell_3D_align_bc(value *argv, int argn)
{
    (void)argn;
    return powell_3D_align(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6],
                           argv[7], argv[8]);
}
