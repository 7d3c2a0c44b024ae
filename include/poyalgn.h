/*
 * poyalgn -- GB300 (sm_103a) direct-optimization pairwise alignment.
 *
 * C ABI of libpoyalgn.so. Plain pointers and sizes only; no CUDA or Python
 * types cross this boundary (streams are passed as void *).
 *
 * Sequences are POY bitset sequences: one byte per position, A=1 C=2 G=4
 * T=8 gap=16 (ambiguities are unions), position 0 holding the leading gap
 * (POY src/data.ml:618). Aligned outputs are written back to front so that
 * each sequence ENDS at the last byte of its buffer, as POY's seq_prepend
 * leaves a `struct seq` (src/seq.c:155-161); lengths are returned.
 *
 * Per-call entry points replace POY's OCaml externals one for one and keep
 * their argument meaning (paths relative to the POY 5.1.1 source tree). Like
 * POY's process-wide Matrix.default workspace, a context holds the fill of
 * the last simple_2 call for a following backtrace_2d; a context is not
 * reentrant. Batched entry points have no POY counterpart: they run many
 * SeqCS.DOS.median computations (src/seqCS.ml:985-1084) in one launch
 * sequence.
 *
 * Return values: 0 on success, a negative POYALGN_E* code otherwise;
 * poyalgn_last_error() describes the last failure of the calling thread.
 */
#ifndef POYALGN_H
#define POYALGN_H 1

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define POYALGN_EINVAL -1       /* bad argument (POY would failwith or assert) */
#define POYALGN_ENOMEM -2       /* device or host allocation failed */
#define POYALGN_ECUDA -3        /* CUDA runtime error */
#define POYALGN_EUNSUPPORTED -4 /* input outside what the GPU path handles */
#define POYALGN_EPAIR -5        /* one or more pairs of a batch failed (see status) */

/* Per-pair status codes written by the batched entry points. */
#define POYALGN_PAIR_OK 0
#define POYALGN_PAIR_CAPACITY -2   /* output capacity exceeded (a device batch pair
                                      whose slot ends past out_bytes) */
#define POYALGN_PAIR_ZERO_MEDIAN -3 /* "median should not be 0" (src/algn.c:3619) */
#define POYALGN_PAIR_EMPTY -4      /* empty sequence / empty median (POY UB) */
#define POYALGN_PAIR_TOO_WIDE -5   /* band wider than the largest pipeline */
#define POYALGN_PAIR_TOO_LONG -6   /* sequence longer than 65535, or a device batch
                                      pair with lena + lenb > max_pair_len */
#define POYALGN_PAIR_BAD_STATE -7  /* a state outside the cost matrix's alphabet */
#define POYALGN_PAIR_NO_CONVERGE -8 /* band doubling did not stop (e.g. all costs 0) */
#define POYALGN_PAIR_INTERNAL -9   /* a speculative band pass was queued but did not run */
#define POYALGN_PAIR_EMPTY_STATE -11 /* closest: a position with no state (POY asserts) */
#define POYALGN_PAIR_RETRY -12     /* internal: direction arena full, the pair is rerun */
#define POYALGN_PAIR_OFF_BAND -13  /* Newkk traceback leaves the band (POY reads
                                      memory outside it) */

typedef struct poyalgn_ctx poyalgn_ctx;
typedef struct poyalgn_cm poyalgn_cm;

/* ---- context ------------------------------------------------------------ */

/* Bind a context to CUDA device `device`. No POY counterpart. */
int poyalgn_init(int device, poyalgn_ctx **out);
void poyalgn_free(poyalgn_ctx *ctx);
const char *poyalgn_last_error(void);
/* Library version string, e.g. "poyalgn 0.1 sm_103a". */
const char *poyalgn_version(void);

/* ---- cost matrices -------------------------------------------------------- */

/*
 * Build the tables of a bitset alphabet from an alph x alph transformation
 * cost matrix (row-major, gap last) and a gap-opening cost (0 = linear).
 * Replaces Cost_matrix.Two_D.of_list / fill_cost_matrix
 * (src/cost_matrix.ml:1140-1189, 1300-1312) followed, when gap_open > 0, by
 * set_cost_model (Affine gap_open) (src/cost_matrix.ml:1003-1017). alph <= 5.
 */
int poyalgn_cm_build(poyalgn_ctx *ctx, const int32_t *tcm, int alph,
                     int gap_open, poyalgn_cm **out);

/*
 * Adopt tables POY already built: the arrays of `struct cm` (src/cm.h:33-76;
 * each 2 << (2*lcm) entries, index (a << lcm) + b). This is the conversion
 * the drop-in stub library performs on cm_CAML_create's block
 * (src/cm.c:2452-2469) before the first alignment.
 */
int poyalgn_cm_adopt(poyalgn_ctx *ctx, int lcm, int gap, int a_sz,
                     int combinations, int cost_model, int gap_open,
                     const int32_t *cost, const uint8_t *median,
                     const int32_t *worst, const int32_t *tail,
                     const int32_t *prepend, poyalgn_cm **out);

/* Copy the tables out (same layout as above). info = {lcm, gap, a_sz,
 * combinations, cost_model, gap_open, min_non0_cost}. Returns #entries. */
int poyalgn_cm_tables(const poyalgn_cm *cm, int32_t *cost, uint8_t *median,
                      int32_t *worst, int32_t *tail, int32_t *prepend,
                      int32_t *info);
void poyalgn_cm_free(poyalgn_cm *cm);

/* ---- per-call drop-in entry points ---------------------------------------- */

/*
 * algn_CAML_simple_2 (src/algn.c:3133-3158): cost of aligning s1 (the
 * shorter, l1 <= l2) with s2 under a linear cost matrix, band doubling seeded
 * with deltawh (algn_nw, src/algn.c:2954-2975). The fill stays in the
 * context for poyalgn_backtrace_2d. l1 > l2 returns POYALGN_EUNSUPPORTED: the
 * reference compiles out its assertion that s1 is the shorter
 * (src/algn.c:25, 1139) and runs its band arithmetic with a negative length
 * difference; Sequence.cost_2 never passes that order.
 */
int poyalgn_simple_2(poyalgn_ctx *ctx, const poyalgn_cm *cm, const uint8_t *s1,
                     int l1, const uint8_t *s2, int l2, int deltawh,
                     int32_t *cost);

/*
 * algn_CAML_backtrace_2d (src/algn.c:3423-3440): aligned s1p/s2p (capacity
 * cap each, results end at cap-1) from the fill of the last simple_2 call on
 * the same s1/s2. swap = 1 prefers insertions over deletions on ties.
 */
int poyalgn_backtrace_2d(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                         const uint8_t *s1, int l1, const uint8_t *s2, int l2,
                         uint8_t *s1p, uint8_t *s2p, int cap, int32_t *len,
                         int swap);

/* algn_CAML_align_2d (src/algn.c:3502-3512): simple_2 then backtrace_2d. */
int poyalgn_align_2d(poyalgn_ctx *ctx, const poyalgn_cm *cm, const uint8_t *s1,
                     int l1, const uint8_t *s2, int l2, uint8_t *s1p,
                     uint8_t *s2p, int cap, int32_t *len, int deltawh,
                     int swap, int32_t *cost);

/*
 * algn_CAML_align_affine_3 (src/algn.c:2358-2447): affine alignment of si
 * (the shorter, li <= lj, else POYALGN_EINVAL like "pass the shorter one as
 * first") with sj; writes resi, resj, median and medianwg (capacity cap
 * each; lens = {len resi/resj, len median, len medianwg}) and the cost.
 */
int poyalgn_align_affine_3(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                           const uint8_t *si, int li, const uint8_t *sj, int lj,
                           uint8_t *resi, uint8_t *resj, uint8_t *median,
                           uint8_t *medianwg, int cap, int32_t *lens,
                           int swaped, int32_t *cost);

/*
 * algn_CAML_ancestor_2 (src/algn.c:3741-3752) and
 * seq_CAML_median_2_with_gaps (src/seq.c:287-298) and algn_CAML_worst_2
 * (src/algn.c:3107-3118) on an aligned pair of length len: ancestor (cap
 * >= len + 1, ends at cap-1), with-gap median (len), worst cost.
 */
int poyalgn_aligned_medians(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                            const uint8_t *a, const uint8_t *b, int len,
                            uint8_t *ancestor, int cap, int32_t *anc_len,
                            uint8_t *median_wg, int32_t *worst);

/*
 * algn_CAML_verify_2 (src/algn.c:3120-3131 -> algn_verify_2, :3099-3105): the
 * cost of an aligned pair of length len under cm's cost table, one gap
 * opening per gap block (algn_calculate_from_2_aligned).
 */
int poyalgn_verify_2(poyalgn_ctx *ctx, const poyalgn_cm *cm, const uint8_t *a,
                     const uint8_t *b, int len, int32_t *cost);

/*
 * seq_CAML_median_2_no_gaps (src/seq.c:274-285 -> seq_get_median_2d_no_gaps,
 * :259-272): the median of every column of an aligned pair that is not the
 * gap, after a leading gap; written back to front into median[cap - n, cap).
 */
int poyalgn_median_2_no_gaps(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                             const uint8_t *a, const uint8_t *b, int len,
                             uint8_t *median, int cap, int32_t *median_len);

/*
 * algn_CAML_limit_2 (src/algn.c:3160-3185 -> algn_nw_limit, :2954-2964), same
 * argument order: the whole plane of (s1, s2) is filled; the window arguments
 * only enter the plane choice, whose height is (s1_len - s2_len) + 50 + w
 * (h, s1_st and s2_st are unused, as in the reference). The fill is kept for
 * poyalgn_backtrace_2d / poyalgn_backtrace_2d_limit.
 */
int poyalgn_limit_2(poyalgn_ctx *ctx, const poyalgn_cm *cm, const uint8_t *s1,
                    int l1, const uint8_t *s2, int l2, int w, int h, int s1_st,
                    int s2_st, int s1_len, int s2_len, int32_t *cost);

/*
 * algn_CAML_backtrace_2d_limit (src/algn.c:3448-3469): backtrace_2d from a
 * start given by (st_s1, st_s2, algn_s1, algn_s2), over the fill of the last
 * simple_2 / limit_2 call on the same pair, with the reference's arithmetic:
 * the walk starts at cell (algn_s1 - 1, st_s2 + algn_s2 - 1) of the row-major
 * matrix of row stride l2, takes s1 / s2 at counters that start at
 * st_s1 + algn_s1 and st_s2 + algn_s2, and ends when its linear index drops
 * below st_s2. From the last cell (0, 0, l1, l2) it is poyalgn_backtrace_2d.
 * A walk that reaches a cell the last fill never wrote returns
 * POYALGN_EUNSUPPORTED (the reference reads what earlier alignments left in
 * its workspace there); one whose counters leave the sequences POYALGN_EINVAL.
 */
int poyalgn_backtrace_2d_limit(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                               const uint8_t *s1, int l1, const uint8_t *s2,
                               int l2, uint8_t *s1p, uint8_t *s2p, int cap,
                               int32_t *len, int st_s1, int st_s2, int algn_s1,
                               int algn_s2, int swaped);

/* ---- batched SeqCS.DOS.median ---------------------------------------------- */

/*
 * Median of every pair k (a = seqs[offa[k]..+lena[k]), b likewise) under the
 * cost model of `cm` (linear or affine), exactly as DOS.median computes it
 * with Algn_Normal. Pair k writes its aligned a/b (ea, eb), its median
 * (ancestor_2 for linear, the backtrace median for affine; med) and its
 * median with gaps (mwg) into [out_off[k], out_off[k] + cap_k) of each
 * output buffer, cap_k = lena[k] + lenb[k] + 2, each ending at the last byte.
 * cost/maxcost/alen/mlen/wlen/status are per pair.
 *
 * poyalgn_median_batch takes host pointers (copies in and out inside the
 * call); poyalgn_median_batch_device takes device pointers and a cudaStream_t
 * (as void *) and only enqueues work; max_pair_len bounds lena + lenb and
 * out_bytes bounds out_off[k] + cap_k (the size of each output buffer).
 * Both size device scratch, so they are checked on the device per pair: a
 * pair with lena + lenb > max_pair_len gets POYALGN_PAIR_TOO_LONG, one whose
 * slot ends past out_bytes POYALGN_PAIR_CAPACITY; such a pair reads and
 * writes nothing, and the other pairs of the batch are unaffected.
 * passes (optional) receives the band iterations run per pair.
 */
int poyalgn_median_batch(poyalgn_ctx *ctx, const poyalgn_cm *cm, int npairs,
                         const uint8_t *seqs, const int64_t *offa,
                         const int32_t *lena, const int64_t *offb,
                         const int32_t *lenb, const int64_t *out_off,
                         int32_t *cost, int32_t *maxcost, int32_t *alen,
                         int32_t *mlen, int32_t *wlen, int32_t *status,
                         uint8_t *ea, uint8_t *eb, uint8_t *med, uint8_t *mwg,
                         int32_t *passes);

int poyalgn_median_batch_device(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                                int npairs, int max_pair_len,
                                int64_t out_bytes, const uint8_t *seqs,
                                const int64_t *offa,
                                const int32_t *lena, const int64_t *offb,
                                const int32_t *lenb, const int64_t *out_off,
                                int32_t *cost, int32_t *maxcost, int32_t *alen,
                                int32_t *mlen, int32_t *wlen, int32_t *status,
                                uint8_t *ea, uint8_t *eb, uint8_t *med,
                                uint8_t *mwg, int32_t *passes, void *stream);

/*
 * poyalgn_median_batch_device without any memory allocation. No counterpart
 * in the reference: it is for callers that must not allocate device memory
 * during the call (a serving loop with a fixed memory budget, code that runs
 * while an allocator is locked) but can accept a bounded batch.
 *
 * Arguments and results are those of poyalgn_median_batch_device, without
 * the context; the work runs on the current CUDA device, which must be the
 * device `cm` was built on. All scratch (work queues, direction slabs,
 * per-pair state, the pair ordering) lives in one fixed region of
 * POYALGN_NOALLOC_SCRATCH_BYTES of static device memory per device, which
 * exists from the moment the library's device code is loaded on that device.
 * Limits: npairs <= POYALGN_NOALLOC_MAX_PAIRS, max_pair_len (lena + lenb) <=
 * POYALGN_NOALLOC_MAX_PAIR_LEN, out_bytes <= POYALGN_NOALLOC_MAX_OUT_BYTES;
 * larger requests fail with POYALGN_EINVAL and a message naming the limit.
 * Fewer CTAs may run than in poyalgn_median_batch_device (the direction
 * slabs share the fixed region); results are identical.
 *
 * The first call on a device does one-time setup (looks up the region's
 * address, queries the SM count and kernel occupancy); make one call per
 * device before capturing a stream that uses this function. Each call
 * clears the queue counters at the start of the region on `stream` before
 * its first kernel; nothing else needs to start at zero, and the caller's
 * output buffers need no clearing.
 *
 * The region is shared by every call on the same device: two calls whose
 * work overlaps in time (different streams, or several host threads) race
 * on it and give wrong results. Serialise calls per device, e.g. by issuing
 * them all on one stream.
 */
#define POYALGN_NOALLOC_SCRATCH_BYTES (64u << 20)
#define POYALGN_NOALLOC_MAX_PAIRS 16384
#define POYALGN_NOALLOC_MAX_PAIR_LEN 4096
#define POYALGN_NOALLOC_MAX_OUT_BYTES (4 << 20)

int poyalgn_median_batch_device_noalloc(const poyalgn_cm *cm, int npairs,
                                        int max_pair_len, int64_t out_bytes,
                                        const uint8_t *seqs, const int64_t *offa,
                                        const int32_t *lena, const int64_t *offb,
                                        const int32_t *lenb, const int64_t *out_off,
                                        int32_t *cost, int32_t *maxcost,
                                        int32_t *alen, int32_t *mlen, int32_t *wlen,
                                        int32_t *status, uint8_t *ea, uint8_t *eb,
                                        uint8_t *med, uint8_t *mwg, int32_t *passes,
                                        void *stream);

/* ---- cost-only scoring (SeqCS.DOS.distance) ---------------------------------- */

/*
 * algn_CAML_cost_affine_3 (src/algn.c:2456-2515): cost of the full unbanded
 * affine fill without traceback (algn_fill_plane_3_aff_nobt,
 * src/algn.c:1986-2110), the shorter sequence down the rows. This is the
 * cost SeqCS.DOS.distance reports under affine gap costs; it can differ from
 * the banded poyalgn_align_affine_3 cost, as in POY.
 */
int poyalgn_cost_affine_3(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                          const uint8_t *si, int li, const uint8_t *sj, int lj,
                          int32_t *cost);

/*
 * SeqCS.DOS.distance (src/seqCS.ml:701-774, Algn_Normal) of many pairs:
 * pairs in which either sequence is all gaps (Sequence.is_empty) cost
 * missing_distance; otherwise the affine model runs algn_CAML_cost_affine_3
 * and the linear model Align.cost_2 ~deltaw:(max 8 |la - lb|)
 * (src/sequence.ml:868-925) -> algn_CAML_simple_2's band doubling, without
 * traceback. Layout as poyalgn_median_batch; per-pair cost and status.
 * The _device form takes device pointers and a stream and only enqueues; a
 * pair with lena + lenb > max_pair_len gets POYALGN_PAIR_TOO_LONG.
 */
int poyalgn_distance_batch(poyalgn_ctx *ctx, const poyalgn_cm *cm, int npairs,
                           const uint8_t *seqs, const int64_t *offa,
                           const int32_t *lena, const int64_t *offb,
                           const int32_t *lenb, int32_t missing_distance,
                           int32_t *cost, int32_t *status);
int poyalgn_distance_batch_device(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                                  int npairs, int max_pair_len,
                                  const uint8_t *seqs, const int64_t *offa,
                                  const int32_t *lena, const int64_t *offb,
                                  const int32_t *lenb, int32_t missing_distance,
                                  int32_t *cost, int32_t *status, void *stream);

/* ---- Algn_Newkk: POY's own banded aligner (src/newkkonen.c), affine ---------- */

/*
 * newkkonen_CAML_algn_affine (src/newkkonen.c:1473-1496, external
 * Sequence.NewkkAlign.newkk_cost2_affine, src/sequence.ml:1840): cost of
 * aligning s1 (the shorter, l1 <= l2) with s2 under the affine model of cm,
 * band passes doubled as newkk_algn does (src/newkkonen.c:1361-1446). The
 * context keeps the alignment for the following backtrace, as the reference
 * keeps it in its ukkm matrix. The linear variant (newkkonen_CAML_algn) is
 * not provided: in the reference it leaves a zero-cost diagonal candidate in
 * every inner cell and its backtrace fails an assertion
 * (src/newkkonen.c:796, 1554); cm must be affine.
 */
int poyalgn_newkk_algn_affine(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                              const uint8_t *s1, int l1, const uint8_t *s2,
                              int l2, int swaped, int32_t *cost);

/*
 * newkkonen_CAML_backtrace_affine (src/newkkonen.c:1788-1805, external
 * newkk_backtrace_affine, src/sequence.ml:1844): the aligned pair of the
 * last poyalgn_newkk_algn_affine call on the same (s1, s2, swaped), written
 * back to front like seq_prepend: s1p/s2p[cap - len, cap).
 */
int poyalgn_newkk_backtrace_affine(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                                   const uint8_t *s1, int l1, const uint8_t *s2,
                                   int l2, uint8_t *s1p, uint8_t *s2p, int cap,
                                   int32_t *len, int swaped);

/* Bound the Newkk direction-code arena to `words` u16 words (0: a third of
 * the free device memory, at most 16 G words). Pairs whose band does not fit
 * beside the others are finished in further launches. */
int poyalgn_newkk_set_arena_words(poyalgn_ctx *ctx, int64_t words);

/* newkkonen_CAML_get_k (src/newkkonen.c:247-252): band half-width of the
 * last pass of the last poyalgn_newkk_algn_affine call. */
int poyalgn_newkk_get_k(const poyalgn_ctx *ctx, int32_t *k);

/*
 * SeqCS.DOS.median with use_ukk under an affine model (src/seqCS.ml:
 * 1043-1051): Sequence.NewkkAlign.align_2 (shorter first, swaped when b is
 * the shorter, src/sequence.ml:1879-1901), then Align.ancestor_2,
 * median_2_with_gaps and max_cost_2 on the aligned pair. Inputs and output
 * layout as poyalgn_median_batch: ea/eb = the aligned pair, med = the
 * ancestor, mwg = the median with gaps, each ending at the last byte of the
 * pair's slot [out_off[k], out_off[k] + lena[k] + lenb[k] + 2). passes
 * (optional) receives the band passes run per pair.
 *
 * poyalgn_newkk_median_batch takes host pointers; the _device variant takes
 * device pointers, max_len >= every sequence length (a longer pair gets
 * POYALGN_PAIR_TOO_LONG) and a cudaStream_t (as
 * void *), and returns once the batch is done (a batch whose direction codes
 * do not fit the context's arena at once is finished in further launches).
 */
int poyalgn_newkk_median_batch(poyalgn_ctx *ctx, const poyalgn_cm *cm,
                               int npairs, const uint8_t *seqs,
                               const int64_t *offa, const int32_t *lena,
                               const int64_t *offb, const int32_t *lenb,
                               const int64_t *out_off, int32_t *cost,
                               int32_t *maxcost, int32_t *alen, int32_t *mlen,
                               int32_t *wlen, int32_t *status, uint8_t *ea,
                               uint8_t *eb, uint8_t *med, uint8_t *mwg,
                               int32_t *passes);
int poyalgn_newkk_median_batch_device(
    poyalgn_ctx *ctx, const poyalgn_cm *cm, int npairs, const uint8_t *seqs,
    const int64_t *offa, const int32_t *lena, const int64_t *offb,
    const int32_t *lenb, const int64_t *out_off, int max_len, int32_t *cost,
    int32_t *maxcost, int32_t *alen, int32_t *mlen, int32_t *wlen,
    int32_t *status, uint8_t *ea, uint8_t *eb, uint8_t *med, uint8_t *mwg,
    int32_t *passes, void *stream);

/* ---- device-resident sequences and the tree downpass ------------------------ */

/*
 * A store keeps node sequences (leaves and computed medians) in one device
 * arena of fixed capacity, so that a downpass or a stream of scoring
 * requests aligns them without copying sequences across the host boundary
 * again. Node ids are dense, in order of addition. No counterpart in the
 * reference, where each OCaml node holds its own `struct seq`; the batches
 * compute exactly SeqCS.DOS.median (src/seqCS.ml:985-1084) per pair.
 *
 * A store belongs to one context and uses its stream; calls on one store
 * must not run concurrently.
 */
typedef struct poyalgn_store poyalgn_store;

int poyalgn_store_create(poyalgn_ctx *ctx, int64_t capacity_bytes,
                         poyalgn_store **out);
void poyalgn_store_free(poyalgn_store *s);

/* Copy one sequence (leading gap included, len >= 1) to the device. */
int poyalgn_store_add(poyalgn_store *s, const uint8_t *seq, int len,
                      int32_t *node);
int poyalgn_store_count(const poyalgn_store *s);
int poyalgn_store_length(const poyalgn_store *s, int node);
/* Copy node's sequence to host memory (cap >= its length). */
int poyalgn_store_read(poyalgn_store *s, int node, uint8_t *out, int cap);
/* Forget every node >= nodes and the arena space after the last kept one. */
int poyalgn_store_truncate(poyalgn_store *s, int nodes);

/*
 * DOS.median of the resident pairs (node_a[k], node_b[k]) under `cm`. With
 * keep != 0 each median becomes a new node (median_node[k]); otherwise the
 * medians are discarded (cost-only use). cost, maxcost and status are per
 * pair (maxcost and median_node may be NULL). Returns POYALGN_EPAIR if any
 * pair failed (its status says why); other pairs' results are valid.
 */
int poyalgn_store_median_batch(poyalgn_store *s, const poyalgn_cm *cm,
                               int npairs, const int32_t *node_a,
                               const int32_t *node_b, int keep,
                               int32_t *median_node, int32_t *cost,
                               int32_t *maxcost, int32_t *status);

/*
 * Downpass of a rooted binary tree over resident leaves, one batched launch
 * sequence per tree level (AllDirChar.internal_downpass,
 * src/allDirChar.ml:1366, with Node.median reducing to DOS.median for one
 * dynamic character). Internal node k (0 <= k < ninternal) has children
 * left[k] and right[k], encoded as leaf index (< nleaves, stored as node
 * leaf_node[index]) or nleaves + internal index; children come before their
 * parent. Writes each internal node's store id and median cost, and the
 * total tree cost (the sum).
 */
int poyalgn_downpass(poyalgn_store *s, const poyalgn_cm *cm, int nleaves,
                     const int32_t *leaf_node, int ninternal,
                     const int32_t *left, const int32_t *right,
                     int32_t *internal_node, int32_t *internal_cost,
                     int64_t *total_cost, int32_t *levels);

/*
 * SeqCS.DOS.median_3_no_union (src/seqCS.ml:1123-1147) for n resident
 * triples: node k's parent state parent[k] is aligned with each child
 * (child1[k], child2[k]) by Sequence.Align.align_2 (parent first); the
 * alignment of lower cost is kept (the second child's on a tie) and the
 * no-gap median of its aligned pair (Sequence.median_2 ->
 * seq_get_median_2d_no_gaps, src/seq.c:259-272, leading gap included)
 * becomes a new node (node[k]). cost and maxcost are the kept alignment's
 * cost and worst cost (Align.max_cost_2), the cost2 and cost2_max fields of
 * the reference's result; status is per triple. Returns POYALGN_EPAIR if
 * any triple failed. The 2 n alignments run as one batch.
 */
int poyalgn_store_median3_batch(poyalgn_store *s, const poyalgn_cm *cm, int n,
                                const int32_t *parent, const int32_t *child1,
                                const int32_t *child2, int32_t *node,
                                int32_t *cost, int32_t *maxcost,
                                int32_t *status);

/*
 * Sequence.Align.closest (src/sequence.ml:1180-1237; cost matrices with
 * combinations, no levels) for n resident pairs: node2's sequence resolved
 * towards node1's. An all-gap node2 is returned as it is (cost 0). Equal
 * sequences are resolved position by position with the gap bit cleared past
 * the leading gap (cost 0); otherwise the pair is aligned (Align.align_2,
 * node1 first), each aligned position of node2 becomes
 * Cost_matrix.Two_D.get_closest of the two (src/cost_matrix.ml:1387-1426:
 * the cheapest state against node1's, the first on a tie), gaps are removed
 * (remove_gaps2) and the cost is Align.cost_2 of node1 and the result.
 * out_node[k] is a new node (node2 itself when it was all gaps); status is
 * per pair. Returns POYALGN_EPAIR if any pair failed, POYALGN_EUNSUPPORTED
 * for a matrix without combinations.
 */
int poyalgn_store_closest_batch(poyalgn_store *s, const poyalgn_cm *cm, int n,
                                const int32_t *node1, const int32_t *node2,
                                int32_t *out_node, int32_t *cost,
                                int32_t *status);

/*
 * Sequence.readjust (src/sequence.ml:2097-2158, without Ukkonen) for n
 * resident triples (child a, child b, parent): the three pairwise medians
 * (DOS.median's cost and median: Align.align_2 + median_2 for the linear
 * model, align_affine_3's median for the affine one), the three medians
 * of a median with the third sequence, the centre of the cheapest
 * two-step route resolved with Align.closest (the reference's choice and
 * tie order), and the costs of the centre against the two children (cost2)
 * and the parent (cost3 = cost2 + that cost). Writes the centre's node and
 * both costs; status is per triple. Four rounds of batches.
 */
int poyalgn_store_readjust_batch(poyalgn_store *s, const poyalgn_cm *cm, int n,
                                 const int32_t *child_a, const int32_t *child_b,
                                 const int32_t *parent, int32_t *node,
                                 int32_t *cost3, int32_t *cost2, int32_t *status);

/*
 * Uppass of the tree of poyalgn_downpass (same encoding): final states top
 * down, one batch per depth. The root keeps its downpass state
 * (root_final = internal_node[ninternal - 1]); every other internal node k
 * gets median_3_no_union(final state of its parent, states of its two
 * children), where a child's state is its leaf sequence or its downpass
 * median (internal_node). Writes final_node[k] and final_cost[k] (cost2 of
 * the kept alignment; 0 for the root) for every internal node.
 */
int poyalgn_uppass(poyalgn_store *s, const poyalgn_cm *cm, int nleaves,
                   const int32_t *leaf_node, int ninternal,
                   const int32_t *left, const int32_t *right,
                   const int32_t *internal_node, int32_t *final_node,
                   int32_t *final_cost, int32_t *levels);

/* ---- serving: continuous batching of scoring requests ------------------------ */

/*
 * A server takes requests of DOS.median pairs over resident store nodes (the
 * SPR/TBR join and downpass scoring that POY issues one call at a time) and
 * batches them continuously. No counterpart in the reference.
 *
 * A scheduler thread keeps nslots batches in flight, each on its own CUDA
 * stream with its own preallocated buffers, so the work of requests that
 * arrive while others run overlaps on the device. Whenever a slot frees it
 * forms the next batch from the oldest waiting requests, up to
 * max_batch_pairs pairs and the slot's share of the device-memory budget.
 * Slot memory is reserved once, at creation: hbm_budget bytes (0: half of
 * the free device memory) split across the slots. A request whose pairs
 * cannot fit one slot is refused at submission (POYALGN_EINVAL). Admission
 * control refuses a submission with POYALGN_EBUSY (nothing is queued) when
 * it would make more than max_waiting_pairs pairs wait, or when the device
 * memory the waiting requests will take in a slot (their four output
 * buffers and per-pair metadata) would exceed half of the device's free
 * memory, sampled at submission (at most once a millisecond).
 *
 * Nodes are those the store holds when the server is created (later
 * additions are not visible to it); the store must outlive the server, and
 * its arena must not be truncated below them meanwhile. Results are
 * identical to poyalgn_store_median_batch for the same pairs, whatever the
 * batch a request lands in.
 */
#define POYALGN_EBUSY -6 /* server admission refused: too many waiting pairs */

/* What a server computes per pair: DOS.median (cost, median) or
 * DOS.distance (cost only, as poyalgn_distance_batch; missing_distance for
 * pairs with an all-gap sequence). */
#define POYALGN_SERVE_MEDIAN 0
#define POYALGN_SERVE_DISTANCE 1

typedef struct poyalgn_server poyalgn_server;

int poyalgn_server_create(poyalgn_store *store, const poyalgn_cm *cm, int kind,
                          int32_t missing_distance, int nslots,
                          int max_batch_pairs, int max_waiting_pairs,
                          int64_t hbm_budget, poyalgn_server **out);
void poyalgn_server_free(poyalgn_server *s);

/* Queue a request of npairs pairs (node ids); non-blocking. */
int poyalgn_server_submit(poyalgn_server *s, int npairs, const int32_t *node_a,
                          const int32_t *node_b, int64_t *ticket);

/*
 * Wait up to timeout_ms (< 0: no limit; POYALGN_EBUSY on timeout) for a
 * ticket, then release it. Per pair: cost, status and the median's length
 * (0 for a distance server); the medians are concatenated into medians (NULL to skip;
 * POYALGN_EINVAL if med_cap is too small). latency_s: submission to
 * completion of the batch that carried the request.
 */
int poyalgn_server_wait(poyalgn_server *s, int64_t ticket, int timeout_ms,
                        int32_t *cost, int32_t *status, int32_t *med_len,
                        uint8_t *medians, int64_t med_cap, double *latency_s);

/*
 * Open-loop replay of a request trace (a load generator): request r is
 * submitted at arrival_s[r] seconds after the call starts (arrival_s
 * ascending) with the next req_npairs[r] pairs of node_a/node_b. Per pair it
 * writes cost and status (status 1: request refused by admission control);
 * per request the latency from its scheduled arrival to completion
 * (latency_s, -1 if refused). wall_s: first arrival to last completion.
 */
int poyalgn_server_replay(poyalgn_server *s, int nreq, const double *arrival_s,
                          const int32_t *req_npairs, const int32_t *node_a,
                          const int32_t *node_b, int32_t *cost,
                          int32_t *status, double *latency_s, double *wall_s);

/* Counters since creation: batches launched, pairs completed, requests refused. */
int poyalgn_server_stats(const poyalgn_server *s, int64_t *batches,
                         int64_t *pairs, int64_t *refused);

/* ---- pipeline ladders and the autotuner ------------------------------------- */

/*
 * No counterpart in the reference. A context aligns each band pass on a
 * pipeline class picked from a ladder of POYALGN_NCLASS shapes: class c has
 * P[c] lanes (a power of two, 4..512) and R[c] rows per lane (2, 3 or 4 for
 * the affine model, 2, 4 or 8 for the linear one) and takes bands up to
 * 2 (P[c] - 1) R[c] + 1 cells wide; capacities must not decrease along the
 * ladder. Results never depend on the ladder, only the speed does.
 */
#define POYALGN_NCLASS 12

int poyalgn_set_ladder(poyalgn_ctx *ctx, int affine, const int32_t *P,
                       const int32_t *R);
int poyalgn_get_ladder(const poyalgn_ctx *ctx, int affine, int32_t *P,
                       int32_t *R);

/*
 * Time ncand candidate ladders (cand_P, cand_R: ncand rows of
 * POYALGN_NCLASS) on a sample batch given as for poyalgn_median_batch (host
 * pointers; copied to the device once), each run reps times after one
 * warm-up run; keep the fastest for cm's cost model. ms[k] receives the
 * median batch time of candidate k and *best its index. Every candidate's
 * per-pair costs and statuses are checked against the first candidate's;
 * a difference is reported as POYALGN_EINVAL (and the ladder is left
 * unchanged).
 */
int poyalgn_autotune(poyalgn_ctx *ctx, const poyalgn_cm *cm, int npairs,
                     const uint8_t *seqs, const int64_t *offa,
                     const int32_t *lena, const int64_t *offb,
                     const int32_t *lenb, int ncand, const int32_t *cand_P,
                     const int32_t *cand_R, int reps, float *ms,
                     int32_t *best);

/*
 * Lean affine passes (gap-free pairs) with bands up to 512 cells wide run
 * either on the lane pipeline (throughput) or on a row tile, one pair per
 * warp swept row by row (latency). mode 0: lane pipeline; 1: row tile;
 * 2 (default): row tile for batches of at most 2 pairs per SM. Results are
 * identical. No counterpart in the reference.
 */
int poyalgn_set_row_tile(poyalgn_ctx *ctx, int mode);

/*
 * Speculative band passes, for batches too small to fill the GPU: the band
 * doubling of a pair runs its passes one after another, each a full sweep of
 * the pair's anti-diagonals, which bounds a small batch's latency. With
 * speculation the first `passes` bands of every linear or gap-free affine
 * pair run at once (each class of the ladder on its own stream), and the
 * pair keeps the first pass that satisfies the doubling test (the one the
 * sequential doubling stops at); pairs that need more, and gap-bearing
 * affine pairs, continue sequentially. Costs extra cells, never changes a result.
 * mode 0: off; 1: every batch; 2 (default): batches of at most 8 pairs per
 * SM with `passes`, of at most 32 pairs per SM with passes - 2, larger
 * batches without. passes: 1 .. POYALGN_SPEC_MAX_PASSES (default 8). Only batches whose
 * fills outlive the sweep speculate (tracebacks deferred to the arena, or
 * cost-only distances). No counterpart in the reference.
 */
#define POYALGN_SPEC_MAX_PASSES 16
int poyalgn_set_speculation(poyalgn_ctx *ctx, int mode, int passes);

/*
 * Caps on the device scratch a context's batches reserve (no counterpart in
 * the reference): slab_bytes bounds the direction slabs (default: half of
 * the free memory at the batch, at most 128 GB; a smaller cap runs a wide
 * class in more rounds), arena_bytes the deferred-traceback arena (default:
 * the free memory less 16 GB, at most 64 GB; fills that do not fit trace
 * back in their slab). 0 keeps a default. Results never depend on either.
 */
int poyalgn_set_memory_budget(poyalgn_ctx *ctx, int64_t slab_bytes,
                              int64_t arena_bytes);

/*
 * A CUDA graph of poyalgn_median_batch_device's launch sequence for fixed
 * buffers and shapes (no counterpart in the reference). Create runs the
 * batch once (reserving all scratch) and captures a second run; each
 * launch then replays the whole batch on `stream` with whatever the buffers
 * hold at that time (same pair count, max_pair_len and out_bytes).
 */
typedef struct poyalgn_graph poyalgn_graph;
int poyalgn_batch_graph_create(poyalgn_ctx *ctx, const poyalgn_cm *cm, int npairs,
                               int max_pair_len, int64_t out_bytes,
                               const uint8_t *seqs, const int64_t *offa,
                               const int32_t *lena, const int64_t *offb,
                               const int32_t *lenb, const int64_t *out_off,
                               int32_t *cost, int32_t *maxcost, int32_t *alen,
                               int32_t *mlen, int32_t *wlen, int32_t *status,
                               uint8_t *ea, uint8_t *eb, uint8_t *med, uint8_t *mwg,
                               int32_t *passes, poyalgn_graph **out);
int poyalgn_batch_graph_launch(poyalgn_graph *g, void *stream);
void poyalgn_batch_graph_free(poyalgn_graph *g);

/* Number of kernel launches the last batch enqueued (for accounting). */
int poyalgn_last_launches(const poyalgn_ctx *ctx);

/*
 * Launch timing (no POY counterpart). After poyalgn_profile_begin, each of
 * the next max_batches batches records CUDA events on its own stream around
 * its prep launch and each pipeline-class launch. poyalgn_profile_end waits
 * for them and writes, per launch slot (prep, class 0 .. class N-1, N =
 * poyalgn_num_classes()), the summed milliseconds into ms[N + 1]; the prep
 * slot of a batch that runs speculative band passes also holds that sweep.
 */
int poyalgn_profile_begin(poyalgn_ctx *ctx, int max_batches);
int poyalgn_profile_end(poyalgn_ctx *ctx, float *ms, int *batches);
int poyalgn_num_classes(void);

/*
 * Integer issue-rate microbenchmark (no POY counterpart): the measured peak
 * against which the fill kernels' int32 roofline is reported. Runs one
 * instruction kind back to back at full occupancy on `device` (iters loop
 * trips of 128 instructions per thread; 2048 threads per SM) and writes the
 * thread-instructions per second of the timed launch (CUDA events, after one
 * untimed launch), its duration and its instruction count. Kinds: 32-bit
 * add, two-way signed min, bitwise logic, DPX three-way signed min
 * (__vimin3_s32) and DPX packed u16 three-way max (__vimax3_u16x2).
 */
#define POYALGN_PEAK_ADD 0
#define POYALGN_PEAK_MIN 1
#define POYALGN_PEAK_LOGIC 2
#define POYALGN_PEAK_MIN3 3
#define POYALGN_PEAK_MAX3_U16X2 4
int poyalgn_int32_peak(int device, int kind, int iters, double *inst_per_s,
                       float *ms, int64_t *thread_inst);

/*
 * ---- Three-sequence alignment ------------------------------------------
 *
 * poyalgn_powell_3d replaces the external `powell_3d` of Sequence.Align
 * (src/sequence.ml:1309-1310, "powell_3D_align_bc" / "powell_3D_align",
 * src/ukkCommon.c:109-150), which align_3_powell (src/sequence.ml:1312-1321)
 * and so readjust_3d (:1373) call: Powell's optimal alignment of three
 * sequences under linear or affine gap costs, recovered by Ukkonen
 * check-pointing (src/ukk.checkp.c).
 *
 * a, b, c are POY sequences with their leading gap (la, lb, lc >= 1 bytes);
 * each later position is read as the lowest of A, C, G, T it holds (a
 * position with none: POYALGN_EPAIR / POYALGN_PAIR_BAD_STATE, where POY
 * fails with "This is impossible!"). mm, go, ge are the mismatch, gap
 * opening and gap extension costs as align_3_powell_inter passes them
 * (src/sequence.ml:1323-1337); 1 <= mm, ge <= 10,000 and 0 <= go <= 10,000
 * (else POYALGN_EINVAL). ra, rb, rc
 * receive the three aligned sequences, leading gap included, written back
 * to front so that they end at ra + cap (POY's seq_prepend into sequences
 * of capacity la + lb + lc: cap >= la + lb + lc); *rlen is their length and
 * *cost the alignment cost (the external's return value). Sequences longer
 * than 32,768 positions, or a triple whose cost bound (the largest single
 * column cost times la + lb + lc - 2) passes 2^26: POYALGN_PAIR_TOO_LONG.
 *
 * poyalgn_powell_3d_batch runs many triples at once: triple k's sequences
 * are seqs + off[3k + j], len[3k + j] bytes (j = 0, 1, 2 for a, b, c), and
 * its aligned sequences end at ra/rb/rc + out_off[k] + len[3k] + len[3k+1] +
 * len[3k+2]; rlen, cost and status have one entry per triple. Host pointers;
 * returns POYALGN_EPAIR when any status is not POYALGN_PAIR_OK.
 *
 * poyalgn_powell_3d_stats reports the summed kernel time and the number of
 * launch rounds of the last batch; poyalgn_powell_3d_set_budget caps the
 * device memory the triples' workspaces take at once (0: half the free
 * memory, at most 192 GB).
 */
int poyalgn_powell_3d(poyalgn_ctx *ctx, const uint8_t *a, int la, const uint8_t *b, int lb,
                      const uint8_t *c, int lc, int mm, int go, int ge, uint8_t *ra,
                      uint8_t *rb, uint8_t *rc, int cap, int32_t *rlen, int32_t *cost);
int poyalgn_powell_3d_batch(poyalgn_ctx *ctx, int ntriples, const uint8_t *seqs,
                            const int64_t *off, const int32_t *len, int mm, int go, int ge,
                            const int64_t *out_off, uint8_t *ra, uint8_t *rb, uint8_t *rc,
                            int32_t *rlen, int32_t *cost, int32_t *status);
int poyalgn_powell_3d_stats(poyalgn_ctx *ctx, float *kernel_ms, int32_t *rounds);
int poyalgn_powell_3d_set_budget(poyalgn_ctx *ctx, int64_t work_bytes);

#ifdef __cplusplus
}
#endif

#endif /* POYALGN_H */
