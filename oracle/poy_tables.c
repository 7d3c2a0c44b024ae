/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * C restatement of POY's OCaml cost-table builder for bitset ("combinations")
 * alphabets, e.g. DNA with A=1 C=2 G=4 T=8 gap=16. POY computes these tables
 * in OCaml and only stores them in the C `struct cm`; there is no OCaml
 * toolchain here, so the oracle (both the compiled reference and the C port)
 * gets its tables from this file. The product library has its own builder;
 * the tests compare the two.
 *
 * Followed step by step (paths relative to the POY source tree):
 *   src/cost_matrix.ml:1140-1189  fill_cost_matrix (use_comb, level 0)
 *   src/cost_matrix.ml:363-397    store_input_list_in_cost_matrix (all combinations)
 *   src/cost_matrix.ml:1096-1135  input_is_metric (positive, symmetric, zero diagonal)
 *   src/cost_matrix.ml:862-897    fill_best_cost_and_median_for_all_combinations
 *   src/cost_matrix.ml:479-506    test_combinations / test_all_combinations
 *   src/cost_matrix.ml:721-805    fill_best_cost_and_median_for_all_combinations_bitwise
 *   src/cost_matrix.ml:994-1001   fill_default_prepend_tail
 *   src/cost_matrix.ml:1003-1017  set_cost_model (Affine go) -> bitwise refill
 *   src/cost_matrix.ml:1337-1348  of_transformations_and_gaps
 *   src/bitSet.ml:343-353         list_of_packed_max (bits, highest first)
 *   src/cm.c:548-657              cm_set_val (lcm, gap, a_sz, table sizes)
 */
#include <limits.h>
#include <string.h>
#include "poy_tables.h"

#define ORC_BIG (INT_MAX / 4)

/* BitSet.Int.list_of_packed_max: the set bits of n below bit `max`, as single
 * bit values, highest bit first (the OCaml builds the list by prepending). */
static int packed_list(int n, int max, int *out)
{
    int k = 0;
    for (int bit = max - 1; bit >= 0; bit--)
        if (n & (1 << bit)) out[k++] = 1 << bit;
    return k;
}

static int at(const orc_tables *t, int a, int b) { return (a << t->lcm) + b; }

/* test_all_combinations li lj (linear fill, cost_matrix.ml:479-506,682-688). */
static void test_all_combinations(const orc_tables *t, const int *li, int ni,
                                  const int *lj, int nj, int *best, int *c,
                                  int *w)
{
    for (int x = 0; x < ni; x++) {
        int a = li[x];
        for (int y = 0; y < nj; y++) {
            int b = lj[y];
            for (int iv = 0; iv < t->alph; iv++) {
                int v = 1 << iv;
                int goa = 0;
                if (t->cost_model == 1 && v == t->gap && (a & t->gap) &&
                    (b & t->gap))
                    goa = t->gap_open;
                int tc = t->cost[at(t, a, v)] + t->cost[at(t, v, b)] + goa;
                if (tc < *c) {
                    *c = tc;
                    *best = v;
                } else if (tc == *c) {
                    *best = v | *best;
                }
            }
            int cab = t->cost[at(t, a, b)];
            if (cab > *w) *w = cab;
        }
    }
}

static void fill_all_combinations(orc_tables *t)
{
    int li[8], lj[8];
    int ncomb = (1 << t->alph) - 1;
    for (int i = 1; i <= ncomb; i++) {
        int ni = packed_list(i, t->alph, li);
        for (int j = 1; j <= ncomb; j++) {
            int nj = packed_list(j, t->alph, lj);
            int best = 0, c = ORC_BIG, w = 0;
            test_all_combinations(t, li, ni, lj, nj, &best, &c, &w);
            if (ni == 1 && nj == 1) {
                t->median[at(t, i, j)] = (unsigned char)(i | j);
            } else {
                /* cleanup is the identity for a linear model */
                t->cost[at(t, i, j)] = c;
                t->median[at(t, i, j)] = (unsigned char)best;
            }
            t->worst[at(t, i, j)] = w;
        }
    }
}

/* fill_best_cost_and_median_for_all_combinations_bitwise, create_original =
 * false (cost_matrix.ml:721-805). Reads the singleton costs of a snapshot. */
static void fill_all_combinations_bitwise(orc_tables *t)
{
    static int old[ORC_TABLE_SIZE];
    memcpy(old, t->cost, sizeof(old));
#define OLD(a, b) old[at(t, (a), (b))]
    int li[8], lj[8];
    int ncomb = (1 << t->alph) - 1;
    for (int i = 1; i <= ncomb; i++) {
        int ni = packed_list(i, t->alph, li);
        for (int j = 1; j <= ncomb; j++) {
            int nj = packed_list(j, t->alph, lj);
            int median, best, worst;
            if (ni == 1 && nj == 1) {
                if (i == j) {
                    int cii = OLD(i, i) * 2;
                    median = i;
                    best = cii;
                    worst = cii;
                } else {
                    int cost1 = OLD(i, j) + OLD(j, j);
                    int cost2 = OLD(i, i) + OLD(i, j);
                    int cij, mij;
                    if (cost1 == cost2) {
                        cij = cost1;
                        mij = i | j;
                    } else if (cost1 > cost2) {
                        cij = cost2;
                        mij = i;
                    } else {
                        cij = cost1;
                        mij = j;
                    }
                    median = mij;
                    best = cij;
                    worst = cij;
                }
            } else {
                /* find_best_combination: process lj li first, then li lj */
                int bcost = ORC_BIG, bmed = 0, wcost = 0;
                for (int pass = 0; pass < 2; pass++) {
                    const int *l1 = pass == 0 ? lj : li;
                    const int *l2 = pass == 0 ? li : lj;
                    int n1 = pass == 0 ? nj : ni;
                    int n2 = pass == 0 ? ni : nj;
                    for (int x = 0; x < n1; x++) {
                        for (int y = 0; y < n2; y++) {
                            int a = l1[x], b = l2[y];
                            int cost1 = OLD(a, a) + OLD(a, b);
                            int cost2 = OLD(a, b) + OLD(b, b);
                            int cij, mij;
                            if (cost1 == cost2) {
                                cij = cost1;
                                mij = a | b;
                            } else if (cost1 > cost2) {
                                cij = cost2;
                                mij = b;
                            } else {
                                cij = cost1;
                                mij = a;
                            }
                            if (cij < bcost) {
                                bcost = cij;
                                bmed = mij;
                            } else if (cij == bcost) {
                                bmed = mij | bmed;
                            }
                            if (cij > wcost) wcost = cij;
                        }
                    }
                }
                median = bmed;
                best = bcost;
                worst = wcost;
            }
            t->median[at(t, i, j)] = (unsigned char)median;
            t->cost[at(t, i, j)] = best;
            t->worst[at(t, i, j)] = worst;
        }
    }
#undef OLD
}

int orc_tables_build(orc_tables *t, const int *tcm, int alph, int gap_open)
{
    if (alph < 2 || alph > 6) return -1; /* bitset alphabets only (size < 7) */
    memset(t, 0, sizeof(*t));
    t->alph = alph;
    t->lcm = alph;                 /* cm_set_val: lcm = a_sz */
    t->gap = 1 << (alph - 1);      /* cm_set_val: gap = 1 << (a_sz - 1) */
    t->a_sz = (1 << alph) - 1;     /* cm_combinations_of_alphabet */
    t->combinations = 1;
    t->cost_model = 0;
    t->gap_open = 0;
    /* store_input_list_in_cost_matrix_all_combinations */
    for (int i = 1; i <= alph; i++)
        for (int j = 1; j <= alph; j++)
            t->cost[at(t, 1 << (i - 1), 1 << (j - 1))] = tcm[(i - 1) * alph + (j - 1)];
    /* input_is_metric: positive (asserted by POY), symmetric, zero diagonal */
    int sym = 1, ide = 1;
    for (int i = 0; i < alph; i++) {
        if (tcm[i * alph + i] != 0) ide = 0;
        for (int j = 0; j < alph; j++) {
            if (tcm[i * alph + j] < 0) return -2;
            if (tcm[i * alph + j] != tcm[j * alph + i]) sym = 0;
        }
    }
    t->is_metric = sym && ide;
    t->is_identity = ide;
    if (t->is_metric)
        fill_all_combinations(t);
    else
        fill_all_combinations_bitwise(t);
    /* fill_default_prepend_tail over the full alphabet size */
    for (int i = 1; i <= t->a_sz; i++) {
        t->tail[i] = t->cost[at(t, i, t->gap)];
        t->prepend[i] = t->cost[at(t, t->gap, i)];
    }
    if (gap_open > 0) {
        /* Data: a non-zero gap opening calls set_cost_model (Affine go) on
         * the full matrix; tail/prepend are not refilled. */
        t->cost_model = 1;
        t->gap_open = gap_open;
        fill_all_combinations_bitwise(t);
    }
    return 0;
}

int orc_tables_dna(orc_tables *t, int subs, int indel, int gap_open)
{
    /* of_transformations_and_gaps true 5 subs indel: zero diagonal, indel on
     * the gap row/column, subs elsewhere (cost_matrix.ml:1337-1348). */
    int tcm[25];
    for (int r = 0; r < 5; r++)
        for (int c = 0; c < 5; c++)
            tcm[r * 5 + c] = (r == c) ? 0 : ((r == 4 || c == 4) ? indel : subs);
    return orc_tables_build(t, tcm, 5, gap_open);
}

int orc_min_non0_cost(const orc_tables *t)
{
    /* cm_get_min_non0_cost scans the whole 2*(1<<lcm)^2 cost array */
    int m = INT_MAX / 2;
    for (int i = 0; i < ORC_TABLE_SIZE; i++)
        if (t->cost[i] > 0 && t->cost[i] < m) m = t->cost[i];
    return m;
}
