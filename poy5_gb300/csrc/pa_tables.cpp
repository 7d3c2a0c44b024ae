// Cost tables for bitset alphabets, built the way POY's OCaml side builds
// them before handing them to C (src/cost_matrix.ml):
//   fill_cost_matrix                 :1140-1189  (metric -> all-combinations
//                                                 fill, else bitwise fill)
//   fill_best_cost_and_median_for_all_combinations          :862-897, 479-506
//   fill_best_cost_and_median_for_all_combinations_bitwise  :721-805
//   fill_default_prepend_tail        :994-1001
//   set_cost_model (Affine go)       :1003-1017  (bitwise refill, tables of
//                                                 tail/prepend kept)
// Table layout and sizes follow cm_set_val (src/cm.c:548-657): lcm = alph,
// gap = 1 << (alph - 1), a_sz = 2^alph - 1, index (a << lcm) + b.
#include "pa_tables.h"

#include <string.h>

namespace pa {

namespace {

struct Sym {
    int n;          // singletons in the set
    int bit[8];     // their codes
};

Sym split(int code, int alph)
{
    Sym s;
    s.n = 0;
    for (int k = alph - 1; k >= 0; k--)
        if (code & (1 << k)) s.bit[s.n++] = 1 << k;
    return s;
}

// singleton cost from the table being built (singletons are never rewritten)
inline int sc(const HostCM* cm, int a, int b) { return cm->cost[(a << cm->lcm) + b]; }

// Linear fill for a metric matrix: for every pair of sets, the cheapest
// path a -> v -> b over all members and all intermediate singletons v; the
// median is the union of all optimal v (singleton pairs keep a|b and their
// input cost); worst is the largest member-to-member cost.
void fill_metric(HostCM* cm)
{
    const int ncomb = (1 << cm->alph) - 1;
    for (int A = 1; A <= ncomb; A++) {
        const Sym sa = split(A, cm->alph);
        for (int B = 1; B <= ncomb; B++) {
            const Sym sb = split(B, cm->alph);
            int best = 0x3fffffff, med = 0, worst = 0;
            for (int x = 0; x < sa.n; x++)
                for (int y = 0; y < sb.n; y++) {
                    const int a = sa.bit[x], b = sb.bit[y];
                    for (int k = 0; k < cm->alph; k++) {
                        const int v = 1 << k;
                        const int c = sc(cm, a, v) + sc(cm, v, b);
                        if (c < best) { best = c; med = v; }
                        else if (c == best) med |= v;
                    }
                    if (sc(cm, a, b) > worst) worst = sc(cm, a, b);
                }
            const int at = (A << cm->lcm) + B;
            if (sa.n == 1 && sb.n == 1) {
                cm->median[at] = (uint8_t)(A | B);
            } else {
                cm->cost[at] = best;
                cm->median[at] = (uint8_t)med;
            }
            cm->worst[at] = worst;
        }
    }
}

// Bitwise fill: each member pair (x, y) contributes the cheaper of "x is the
// median" (c(x,x) + c(x,y)) and "y is the median" (c(x,y) + c(y,y)), ties
// giving x|y; the set cost is the cheapest contribution (medians of equal
// contributions are united), worst the largest. Singleton costs come from a
// snapshot so the fill does not read its own output.
void fill_bitwise(HostCM* cm)
{
    static thread_local int old[CM_ENTRIES];
    memcpy(old, cm->cost, sizeof(old));
    auto oc = [&](int a, int b) { return old[(a << cm->lcm) + b]; };
    const int ncomb = (1 << cm->alph) - 1;
    for (int A = 1; A <= ncomb; A++) {
        const Sym sa = split(A, cm->alph);
        for (int B = 1; B <= ncomb; B++) {
            const Sym sb = split(B, cm->alph);
            int best, med, worst;
            if (sa.n == 1 && sb.n == 1) {
                if (A == B) {
                    best = worst = 2 * oc(A, A);
                    med = A;
                } else {
                    const int c1 = oc(A, B) + oc(B, B);  // median B
                    const int c2 = oc(A, A) + oc(A, B);  // median A
                    if (c1 == c2) { best = c1; med = A | B; }
                    else if (c1 > c2) { best = c2; med = A; }
                    else { best = c1; med = B; }
                    worst = best;
                }
            } else {
                best = 0x3fffffff;
                med = 0;
                worst = 0;
                for (int dir = 0; dir < 2; dir++) {
                    const Sym& s1 = dir == 0 ? sb : sa;
                    const Sym& s2 = dir == 0 ? sa : sb;
                    for (int x = 0; x < s1.n; x++)
                        for (int y = 0; y < s2.n; y++) {
                            const int a = s1.bit[x], b = s2.bit[y];
                            const int c1 = oc(a, a) + oc(a, b);
                            const int c2 = oc(a, b) + oc(b, b);
                            int c, mm;
                            if (c1 == c2) { c = c1; mm = a | b; }
                            else if (c1 > c2) { c = c2; mm = b; }
                            else { c = c1; mm = a; }
                            if (c < best) { best = c; med = mm; }
                            else if (c == best) med |= mm;
                            if (c > worst) worst = c;
                        }
                }
            }
            const int at = (A << cm->lcm) + B;
            cm->median[at] = (uint8_t)med;
            cm->cost[at] = best;
            cm->worst[at] = worst;
        }
    }
}

int min_positive(const HostCM* cm)
{
    int m = 0x3fffffff;
    const int n = 2 * (1 << cm->lcm) * (1 << cm->lcm);
    for (int i = 0; i < n; i++)
        if (cm->cost[i] > 0 && cm->cost[i] < m) m = cm->cost[i];
    return m;
}

}  // namespace

int build_cm(HostCM* cm, const int* tcm, int alph, int gap_open)
{
    if (alph < 2 || alph > 5) return -1;  // GPU tables hold 5-bit states
    if (gap_open < 0) return -2;
    memset(cm, 0, sizeof(*cm));
    cm->alph = alph;
    cm->lcm = alph;
    cm->gap = 1 << (alph - 1);
    cm->a_sz = (1 << alph) - 1;
    cm->combinations = 1;
    int sym = 1, ide = 1;
    for (int r = 0; r < alph; r++) {
        if (tcm[r * alph + r] != 0) ide = 0;
        for (int c = 0; c < alph; c++) {
            if (tcm[r * alph + c] < 0) return -3;
            if (tcm[r * alph + c] != tcm[c * alph + r]) sym = 0;
            cm->cost[((1 << r) << cm->lcm) + (1 << c)] = tcm[r * alph + c];
        }
    }
    cm->is_metric = sym && ide;
    cm->is_identity = ide;
    if (cm->is_metric) fill_metric(cm);
    else fill_bitwise(cm);
    for (int i = 1; i <= cm->a_sz; i++) {
        cm->tail[i] = cm->cost[(i << cm->lcm) + cm->gap];
        cm->prepend[i] = cm->cost[(cm->gap << cm->lcm) + i];
    }
    if (gap_open > 0) {
        cm->cost_model = 1;
        cm->gap_open = gap_open;
        fill_bitwise(cm);
    }
    cm->mnz = min_positive(cm);
    return 0;
}

int adopt_cm(HostCM* cm, int lcm, int gap, int a_sz, int combinations,
             int cost_model, int gap_open, const int* cost,
             const uint8_t* median, const int* worst, const int* tail,
             const int* prepend)
{
    if (lcm < 1 || lcm > 5 || !combinations) return -1;
    if (gap != (1 << (lcm - 1))) return -1;
    memset(cm, 0, sizeof(*cm));
    cm->alph = lcm;
    cm->lcm = lcm;
    cm->gap = gap;
    cm->a_sz = a_sz;
    cm->combinations = combinations;
    cm->cost_model = cost_model;
    cm->gap_open = gap_open;
    const int n = 2 * (1 << lcm) * (1 << lcm);
    memcpy(cm->cost, cost, (size_t)n * sizeof(int));
    memcpy(cm->worst, worst, (size_t)n * sizeof(int));
    memcpy(cm->tail, tail, (size_t)n * sizeof(int));
    memcpy(cm->prepend, prepend, (size_t)n * sizeof(int));
    memcpy(cm->median, median, (size_t)n);
    cm->mnz = min_positive(cm);
    return 0;
}

void kernel_tables(const HostCM& cm, Tables* t)
{
    memset(t, 0, sizeof(*t));
    const int ns = 1 << cm.lcm;
    for (int a = 0; a < NSTATE; a++) {
        // rotate the rows of A, C, G, T onto disjoint bank octets
        int rot = (a == 1) ? 0 : (a == 2) ? 8 : (a == 4) ? 16 : (a == 8) ? 24 : 8 * (a & 3);
        t->rowoff[a] = a * CSW_STRIDE + rot;
        for (int b = 0; b < NSTATE; b++)
            t->csw[t->rowoff[a] + b] = (a < ns && b < ns) ? cm.cost[(a << cm.lcm) + b] : 0;
        t->tail[a] = a < ns ? cm.tail[a] : 0;
        t->prepend[a] = a < ns ? cm.prepend[a] : 0;
    }
    for (int i = 0; i < ns * ns; i++) {
        t->worst[i] = cm.worst[i];
        t->median[i] = cm.median[i];
    }
    t->gap = cm.gap;
    t->lcm = cm.lcm;
    t->go = cm.gap_open;
    t->mnz = cm.mnz;
    t->comb = cm.combinations;
    t->model = cm.cost_model;
    t->a_sz = cm.a_sz;
}

}  // namespace pa
