/*
 * ORACLE / TEST INFRASTRUCTURE ONLY: C restatement of POY's direct-
 * optimization pairwise alignment path (poy_oracle.c). Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline arm may load it.
 */
#ifndef POY_ORACLE_H
#define POY_ORACLE_H 1
#include <stdint.h>

void *orc_cm_new(const int *tcm, int alph, int gap_open);
void orc_cm_free(void *cm);
int orc_cm_tables(void *cm, int *cost, uint8_t *median, int *worst, int *tail,
                  int *prepend, int *info);
void *orc_ws_new(void);
void orc_ws_free(void *ws);
void orc_set_check(int on);
const char *orc_last_error(void);

int orc_simple_2(void *cm, void *ws, const uint8_t *s1, int l1,
                 const uint8_t *s2, int l2, int deltawh, int *cost);
int orc_backtrace_2d(void *cm, void *ws, const uint8_t *s1, int l1,
                     const uint8_t *s2, int l2, int swap, uint8_t *r1,
                     uint8_t *r2, int cap, int *len);
int orc_cost_linear(void *cm, void *ws, const uint8_t *a, int la,
                    const uint8_t *b, int lb, int deltaw, int *cost);
int orc_cost_affine(void *cm, void *ws, const uint8_t *a, int la,
                    const uint8_t *b, int lb, int *cost);
int orc_median_linear(void *cm, void *ws, const uint8_t *a, int la,
                      const uint8_t *b, int lb, int *cost, uint8_t *ea,
                      uint8_t *eb, int *elen, uint8_t *anc, int *anclen,
                      uint8_t *mwg, int *mwglen, int *maxcost);
int orc_median_affine(void *cm, void *ws, const uint8_t *a, int la,
                      const uint8_t *b, int lb, int *cost, uint8_t *med,
                      int *medlen, uint8_t *ea, uint8_t *eb, int *elen,
                      uint8_t *mwg, int *mwglen, int *maxcost);

/* Batched DOS.median over many pairs, OpenMP across pairs. Pair k reads
 * a = seqs[offa[k] .. +lena[k]), b likewise; writes results into slot k of a
 * flat output with capacity cap[k] = lena[k] + lenb[k] + 2 at out_off[k].
 * Per-pair status lands in status[k] (0 ok). Returns the number of failures. */
int orc_median_batch(void *cm, int affine, int npairs, const uint8_t *seqs,
                     const int64_t *offa, const int *lena, const int64_t *offb,
                     const int *lenb, const int64_t *out_off, int *cost,
                     int *maxcost, int *alen, int *mlen, int *wlen, uint8_t *ea,
                     uint8_t *eb, uint8_t *med, uint8_t *mwg, int *status,
                     int nthreads);

/* Band schedule statistics of one linear / affine alignment (internal order
 * already applied): number of doubling iterations and cells filled. */
int orc_schedule(void *cm, int affine, const uint8_t *a, int la,
                 const uint8_t *b, int lb, int *iters, int64_t *cells);

/* Algn_Newkk, affine (src/newkkonen.c): newkkonen_CAML_algn_affine +
 * newkkonen_CAML_backtrace_affine on s1 (shorter, l1 <= l2) and s2; the
 * aligned pair in r1/r2[0, *len) (capacity l1 + l2). iters/cells (optional)
 * receive the band passes run and the cells they filled. */
int orc_newkk_align(void *cm, const uint8_t *s1, int l1, const uint8_t *s2,
                    int l2, int swaped, int *cost, uint8_t *r1, uint8_t *r2,
                    int *len, int *iters, int64_t *cells);
/* SeqCS.DOS.median with use_ukk (affine): capacities as orc_median_linear. */
int orc_newkk_median(void *cm, const uint8_t *a, int la, const uint8_t *b,
                     int lb, int *cost, uint8_t *ea, uint8_t *eb, int *elen,
                     uint8_t *anc, int *anclen, uint8_t *mwg, int *mwglen,
                     int *maxcost);

/* Sequence.Align.align_3_powell -> powell_3D_align (src/ukkCommon.c:109):
 * three POY sequences with their leading gap; ra/rb/rc hold la + lb + lc
 * bytes and receive the aligned sequences front to back (leading gap
 * first), *rlen bytes each. Returns -2 where the reference fails ("This is
 * impossible!": a position without A, C, G or T). */
int orc_powell_3d(const uint8_t *a, int la, const uint8_t *b, int lb, const uint8_t *c,
                  int lc, int mm, int go, int ge, uint8_t *ra, uint8_t *rb, uint8_t *rc,
                  int *rlen, int *cost);

/* orc_powell_3d over many triples, OpenMP over triples; outputs laid out as
 * poyalgn_powell_3d_batch lays them out. Returns the count of failures. */
int orc_powell_3d_batch(int n, const uint8_t *seqs, const int64_t *off, const int32_t *len,
                        int mm, int go, int ge, const int64_t *out_off, uint8_t *ra,
                        uint8_t *rb, uint8_t *rc, int32_t *rlen, int32_t *cost,
                        int32_t *status, int nthreads);

#endif
