/*
 * spaghetty_gb300.h -- C ABI of the GB300 tensor-permutation library.
 *
 * Drop-in replacements for NWChem TCE's tensor sorts.  The input
 * `unsorted` with dims (d1..dr) is a flat FP64 buffer whose LAST index is
 * stride-1 (equivalently the Fortran array u(dr,...,d1)); for the 1-based
 * permutation (p1..pr) the output `sorted` has dims (d_{p1}..d_{pr}) and
 *     sort:    sorted[j_{p1},...,j_{pr}] = unsorted[j1,...,jr] * factor
 *     sortacc: sorted[j_{p1},...,j_{pr}] = sorted[...] + unsorted[j1,...,jr] * factor
 * with the product rounded once and the sum rounded once (no FMA), so results
 * are bit-identical to the reference's FP64 loop nests.
 *
 * Pointers may be device pointers (the kernel runs in place on the GPU) or
 * host pointers (staged through cached device buffers).  The Fortran-style
 * void entry points are synchronous: when they return, `sorted` holds the
 * result.  They never abort; an error is printed once per call to stderr,
 * `sorted` is left untouched where possible, and the code is kept for
 * spaghetty_last_error().  Dims and permutation are 4-byte integers passed
 * by reference, as the reference's default-integer Fortran callers do.
 */
#ifndef SPAGHETTY_GB300_H
#define SPAGHETTY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define SPAGHETTY_OK                0
#define SPAGHETTY_ERR_RANK          1  /* rank outside 1..8                       */
#define SPAGHETTY_ERR_PERM          2  /* permutation not a bijection of 1..r     */
#define SPAGHETTY_ERR_DIMS          3  /* a dimension <= 0                        */
#define SPAGHETTY_ERR_OVERFLOW      4  /* element count overflows int64           */
#define SPAGHETTY_ERR_NULL          5  /* null pointer with a non-empty tensor    */
#define SPAGHETTY_ERR_ALIAS         6  /* unsorted and sorted overlap             */
#define SPAGHETTY_ERR_CUDA          7  /* a CUDA runtime call failed              */
#define SPAGHETTY_ERR_MEMSPACE      8  /* pointer kinds not supported together    */
#define SPAGHETTY_ERR_CONFIG        9  /* invalid kernel configuration override   */
#define SPAGHETTY_ERR_BATCH        10  /* invalid batch entry                     */
#define SPAGHETTY_ERR_DEVICE       11  /* device-side status word reported error  */
#define SPAGHETTY_ERR_NOKERNEL     12  /* no compiled kernel variant fits         */
#define SPAGHETTY_ERR_TOO_LARGE    13  /* batch exceeds the fixed scratch limits  */

/* ---- NWChem drop-ins (trunk/tce_sort4_switch.F:1-8; the Hirata routines in
 *      branches/spaghetty3/python/tce_sort_hirata.F:62-63,143-144 and
 *      branches/spaghetty2/tce_sortacc_hirata.F:49,120).  Names without and
 *      with the trailing underscore, as GNU (-fno-underscoring) and
 *      underscoring Fortran compilers emit (trunk/generator2.py:768,
 *      trunk/tester_cutil.c:60-76). ---------------------------------------- */
void tce_sort_4(const double *unsorted, double *sorted,
                const int *a, const int *b, const int *c, const int *d,
                const int *i, const int *j, const int *k, const int *l,
                const double *factor);
void tce_sort_4_(const double *unsorted, double *sorted,
                 const int *a, const int *b, const int *c, const int *d,
                 const int *i, const int *j, const int *k, const int *l,
                 const double *factor);
void tce_sortacc_4(const double *unsorted, double *sorted,
                   const int *a, const int *b, const int *c, const int *d,
                   const int *i, const int *j, const int *k, const int *l,
                   const double *factor);
void tce_sortacc_4_(const double *unsorted, double *sorted,
                    const int *a, const int *b, const int *c, const int *d,
                    const int *i, const int *j, const int *k, const int *l,
                    const double *factor);
void tce_sort_6(const double *unsorted, double *sorted,
                const int *a, const int *b, const int *c, const int *d,
                const int *e, const int *f,
                const int *i, const int *j, const int *k, const int *l,
                const int *m, const int *n, const double *factor);
void tce_sort_6_(const double *unsorted, double *sorted,
                 const int *a, const int *b, const int *c, const int *d,
                 const int *e, const int *f,
                 const int *i, const int *j, const int *k, const int *l,
                 const int *m, const int *n, const double *factor);
void tce_sortacc_6(const double *unsorted, double *sorted,
                   const int *a, const int *b, const int *c, const int *d,
                   const int *e, const int *f,
                   const int *i, const int *j, const int *k, const int *l,
                   const int *m, const int *n, const double *factor);
void tce_sortacc_6_(const double *unsorted, double *sorted,
                    const int *a, const int *b, const int *c, const int *d,
                    const int *e, const int *f,
                    const int *i, const int *j, const int *k, const int *l,
                    const int *m, const int *n, const double *factor);

/* Rank 2 and rank 8 members of the family (trunk/old_sort.f:10-31,236-478,
 * 489-510,715-957; tce_sort_hirata.F:22-61,303). */
void tce_sort_2(const double *unsorted, double *sorted, const int *a, const int *b,
                const int *i, const int *j, const double *factor);
void tce_sort_2_(const double *unsorted, double *sorted, const int *a, const int *b,
                 const int *i, const int *j, const double *factor);
void tce_sortacc_2(const double *unsorted, double *sorted, const int *a, const int *b,
                   const int *i, const int *j, const double *factor);
void tce_sortacc_2_(const double *unsorted, double *sorted, const int *a, const int *b,
                    const int *i, const int *j, const double *factor);
void tce_sort_8(const double *unsorted, double *sorted,
                const int *a, const int *b, const int *c, const int *d,
                const int *e, const int *f, const int *g, const int *h,
                const int *i, const int *j, const int *k, const int *l,
                const int *m, const int *n, const int *o, const int *p,
                const double *factor);
void tce_sort_8_(const double *unsorted, double *sorted,
                 const int *a, const int *b, const int *c, const int *d,
                 const int *e, const int *f, const int *g, const int *h,
                 const int *i, const int *j, const int *k, const int *l,
                 const int *m, const int *n, const int *o, const int *p,
                 const double *factor);
void tce_sortacc_8(const double *unsorted, double *sorted,
                   const int *a, const int *b, const int *c, const int *d,
                   const int *e, const int *f, const int *g, const int *h,
                   const int *i, const int *j, const int *k, const int *l,
                   const int *m, const int *n, const int *o, const int *p,
                   const double *factor);
void tce_sortacc_8_(const double *unsorted, double *sorted,
                    const int *a, const int *b, const int *c, const int *d,
                    const int *e, const int *f, const int *g, const int *h,
                    const int *i, const int *j, const int *k, const int *l,
                    const int *m, const int *n, const int *o, const int *p,
                    const double *factor);

/* -i8 shims for NWChem built with 8-byte default integers: the same
 * drop-ins with dims and permutation as int64 (values must fit 32 bits).
 * Link them under the plain names with the linker's symbol renaming, or call
 * them through a Fortran bind(C) interface. */
void tce_sort_4_i8(const double *unsorted, double *sorted,
                   const int64_t *a, const int64_t *b, const int64_t *c, const int64_t *d,
                   const int64_t *i, const int64_t *j, const int64_t *k, const int64_t *l,
                   const double *factor);
void tce_sort_4_i8_(const double *unsorted, double *sorted,
                    const int64_t *a, const int64_t *b, const int64_t *c, const int64_t *d,
                    const int64_t *i, const int64_t *j, const int64_t *k, const int64_t *l,
                    const double *factor);
void tce_sortacc_4_i8(const double *unsorted, double *sorted,
                      const int64_t *a, const int64_t *b, const int64_t *c, const int64_t *d,
                      const int64_t *i, const int64_t *j, const int64_t *k, const int64_t *l,
                      const double *factor);
void tce_sortacc_4_i8_(const double *unsorted, double *sorted,
                       const int64_t *a, const int64_t *b, const int64_t *c, const int64_t *d,
                       const int64_t *i, const int64_t *j, const int64_t *k, const int64_t *l,
                       const double *factor);
void tce_sort_6_i8(const double *unsorted, double *sorted,
                   const int64_t *a, const int64_t *b, const int64_t *c, const int64_t *d,
                   const int64_t *e, const int64_t *f,
                   const int64_t *i, const int64_t *j, const int64_t *k, const int64_t *l,
                   const int64_t *m, const int64_t *n, const double *factor);
void tce_sort_6_i8_(const double *unsorted, double *sorted,
                    const int64_t *a, const int64_t *b, const int64_t *c, const int64_t *d,
                    const int64_t *e, const int64_t *f,
                    const int64_t *i, const int64_t *j, const int64_t *k, const int64_t *l,
                    const int64_t *m, const int64_t *n, const double *factor);
void tce_sortacc_6_i8(const double *unsorted, double *sorted,
                      const int64_t *a, const int64_t *b, const int64_t *c, const int64_t *d,
                      const int64_t *e, const int64_t *f,
                      const int64_t *i, const int64_t *j, const int64_t *k, const int64_t *l,
                      const int64_t *m, const int64_t *n, const double *factor);
void tce_sortacc_6_i8_(const double *unsorted, double *sorted,
                       const int64_t *a, const int64_t *b, const int64_t *c, const int64_t *d,
                       const int64_t *e, const int64_t *f,
                       const int64_t *i, const int64_t *j, const int64_t *k, const int64_t *l,
                       const int64_t *m, const int64_t *n, const double *factor);

/* Status-returning forms of the rank-4/6 drop-ins: same arguments, return a
 * SPAGHETTY_* code instead of printing (the reference's tce_sort4_switch.F
 * :58-60 can only print 'something is wrong...' and return). */
int tce_sort_4_status(const double *unsorted, double *sorted,
                      const int *a, const int *b, const int *c, const int *d,
                      const int *i, const int *j, const int *k, const int *l,
                      const double *factor);
int tce_sortacc_4_status(const double *unsorted, double *sorted,
                         const int *a, const int *b, const int *c, const int *d,
                         const int *i, const int *j, const int *k, const int *l,
                         const double *factor);
int tce_sort_6_status(const double *unsorted, double *sorted,
                      const int *a, const int *b, const int *c, const int *d,
                      const int *e, const int *f,
                      const int *i, const int *j, const int *k, const int *l,
                      const int *m, const int *n, const double *factor);
int tce_sortacc_6_status(const double *unsorted, double *sorted,
                         const int *a, const int *b, const int *c, const int *d,
                         const int *e, const int *f,
                         const int *i, const int *j, const int *k, const int *l,
                         const int *m, const int *n, const double *factor);

/* ---- generic entry points --------------------------------------------- */

/* The generated nests' two-factor form trans_<perm>_loop_<order>(unsorted,
 * sorted, dims..., factor, acc_factor) (trunk/generator2.py:57-130,
 * trunk/generator6.py:79-134) for any rank 1..8:
 *     acc_factor == 0:  sorted = factor*unsorted
 *     acc_factor == 1:  sorted = sorted + factor*unsorted
 *     otherwise:        sorted = acc_factor*sorted + factor*unsorted
 * `dims` and `perm` are host arrays of `rank` ints (perm 1-based).
 * Both tensor pointers must be device (or managed) memory of one device,
 * else SPAGHETTY_ERR_MEMSPACE; the work runs on that device whatever the
 * calling thread's current device is, and is enqueued on `stream` (a
 * cudaStream_t of that device, NULL = legacy default stream); the call
 * returns without waiting.  Returns a SPAGHETTY_* code. */
int spaghetty_sort_async(int rank, const double *unsorted, double *sorted,
                         const int *dims, const int *perm,
                         double factor, double acc_factor, void *stream);

/* Same, synchronous, accepting host or device pointers. */
int spaghetty_sort(int rank, const double *unsorted, double *sorted,
                   const int *dims, const int *perm,
                   double factor, double acc_factor);

/* Last error recorded by any call on this host thread (0 = none), and a
 * static description of a code. */
int spaghetty_last_error(void);

/* The CUDA error behind the last SPAGHETTY_ERR_CUDA in this process: a
 * cudaError_t value, or a negated CUresult when the tensor-map encoding was
 * rejected; 0 if none.  The string form names it. */
int spaghetty_last_cuda_error(void);
const char *spaghetty_last_cuda_error_string(void);
const char *spaghetty_error_string(int code);

/* Library options.  SPAGHETTY_OPT_HOST_ZERO_COPY (default 1): the
 * synchronous entry points run the kernels directly on PINNED host buffers
 * through their mapped device addresses (over NVLink-C2C on GB300) instead
 * of staging them through device copies; 0 stages every host buffer.
 * Pageable host buffers are always staged. */
#define SPAGHETTY_OPT_HOST_ZERO_COPY 1
/* SPAGHETTY_OPT_HOST_PIPELINE (default 0): when both buffers are pinned
 * host memory, move them in slabs through a three-stream upload / sort /
 * download pipeline on the copy engines instead (slabs of the output's
 * slowest index, or of the input's, whichever leaves one side contiguous
 * and the other in long rows; where neither does, the kernels work on the
 * pinned buffers in place as by default). */
#define SPAGHETTY_OPT_HOST_PIPELINE 2
/* SPAGHETTY_OPT_TMA_SKEW (default 1): TMA-staged plans may rotate the
 * permute step's slot map to spread its shared-memory accesses over the
 * banks (chosen per plan by simulating them); 0 plans without the rotation.
 * Changing it drops the cached plans. */
#define SPAGHETTY_OPT_TMA_SKEW 3
/* SPAGHETTY_OPT_WARP_TR (default 1): transposes whose two stride-1 extents
 * are at most 32 with a product of at most 128 move each such inner tile
 * through one warp's registers with warp shuffles (no shared memory) when
 * the tensor has at most 2^22 elements; 0 never, 2 at any size.  Changing it
 * drops the cached plans. */
#define SPAGHETTY_OPT_WARP_TR 4
/* SPAGHETTY_OPT_BATCH_OWN_MIN (default 16777216 = 2^24): batches created
 * afterwards run every sort of at least this many elements that
 * SPAGHETTY_OPT_BATCH_OWN_KINDS admits as its own launch (on streams forked
 * from the launch stream and joined before the persistent kernel) instead
 * of on the persistent kernel's work list; 0 keeps every sort on the work
 * list. */
#define SPAGHETTY_OPT_BATCH_OWN_MIN 5
/* SPAGHETTY_OPT_BATCH_OWN_KINDS (default 0): which of those large sorts
 * leave the work list: 0 = those whose single-sort plan is the TMA-staged
 * kernel, 1 = all of them. */
#define SPAGHETTY_OPT_BATCH_OWN_KINDS 6
int spaghetty_set_option(int option, int value);

/* Synchronise the current device and report (then clear) the kernels'
 * status word: SPAGHETTY_ERR_DEVICE if a kernel gave up a bounded wait (its
 * pipeline's transfers did not arrive in time), else SPAGHETTY_OK.  The
 * synchronous entry points check it themselves.  The word is process-wide:
 * one word for every device, stream and host thread, so a timed-out wait in
 * one stream's kernel is reported (and cleared) by whichever synchronous
 * call or spaghetty_device_status() reads it next. */
int spaghetty_device_status(void);

/* ---- plans (host only, no GPU needed) --------------------------------- */

typedef struct spaghetty_plan_info {
    int kind;           /* 0 = empty, 1 = flat (rank <= 1 after folding),
                           2 = direct (fastest index unchanged),
                           3 = tiled transpose through shared memory,
                           4 = tiled, boxes moved by TMA bulk tensor copies,
                           5 = small inner tiles transposed in one warp's
                               registers with warp shuffles */
    int rank;           /* rank after dropping unit dims and fusing indices */
    int64_t dims[8];    /* folded dims, input order, last is stride-1     */
    int perm[8];        /* folded permutation, 0-based, output position -> input dim */
    int box[8];         /* tile box length per folded dim                 */
    int threads;        /* CTA size                                       */
    int ept;            /* elements per thread per tile                   */
    int64_t ntiles;     /* number of boxes covering the tensor            */
    int run_in;         /* contiguous input elements per box row          */
    int run_out;        /* contiguous output elements per box row         */
    int pad_period;     /* shared-memory bank-conflict avoidance: kinds 2/3,
                           padding of one word every N; kind 4, the step of
                           the permute step's diagonal skew (0 = none) */
    int masked;         /* 1 when boundary boxes need element masks      */
    int grid;           /* CTAs launched                                  */
    int vec;            /* 2 when 16-byte vector accesses are used        */
    int stages;         /* tiled: 0 = register-staged, 2/3 = cp.async pipeline depth */
    int smem_bytes;     /* dynamic shared memory per CTA                  */
} spaghetty_plan_info;

/* Fold and plan without launching.  op: 0 = sort, 1 = sortacc, 2 = general
 * acc_factor.  Returns a SPAGHETTY_* code. */
int spaghetty_plan_query(int rank, const int *dims, const int *perm, int op,
                         spaghetty_plan_info *out);

/* Host-side index-safety check of a plan, needing no GPU: replays the exact
 * launch parameters through the kernels' own index functions, moving element
 * indices instead of values, and returns SPAGHETTY_OK only if every global
 * read and write lies inside the tensors, every shared-memory index inside
 * the staging tile, and every output element is written exactly once from
 * the input element the permutation maps to it.  stats (may be NULL)
 * receives {reads, writes, boxes, staging elements}.  Tensors up to 2^27
 * elements.  Returns SPAGHETTY_ERR_CONFIG on any violation. */
int spaghetty_plan_verify(int rank, const int *dims, const int *perm, int op, int num_sms,
                          int64_t *stats);

/* Autotuner hook: force the tile box / block shape for subsequent calls
 * with the same folded (dims, perm, op).  box[] is indexed by folded dim;
 * threads in {128,256,512}; ept in {1,2,4,8}; stages in {0,2,3} (tiled
 * kernel: 0 = register-staged, 2/3 = cp.async pipeline depth, needs
 * ept >= 2) or 12/13/14/16 (TMA-staged kernel with 2/3/4/6 load stages;
 * threads in {128,256}, ept in {8,16}) or 20 (the warp-shuffle transpose:
 * threads 256, ept = registers per lane, the problem fixes the box).  Pass box == NULL to clear every override.  Returns a
 * SPAGHETTY_* code. */
int spaghetty_tune_set(int rank, const int *dims, const int *perm, int op,
                       const int *box, int threads, int ept, int stages);

/* Load autotuner winners from a tune file (lines
 * `gpu_name|sm_count|folded dims|folded perm (0-based)|op class|box|threads|ept|stages`)
 * for the current device; returns how many were installed, or -1 if the
 * file cannot be read.  The library also loads, once, the file named by
 * $SPAGHETTY_GB300_TUNE_FILE (empty = none), else tune_cache.txt beside the
 * shared library -- the per-GPU table the reference shipped as makelib's
 * best-loop list (trunk/makelib.py:39-62). */
int spaghetty_tune_load(const char *path);

/* Host-side self checks of the planner's integer helpers (fast division by
 * invariant divisors).  Returns 0 when they pass.  Needs no GPU. */
int spaghetty_selftest(void);

/* ---- several sortaccs into one output, fused --------------------------- */

/* For k = 0..nsrc-1 in order: sorted = sorted + factors[k] *
 * permute_{perms[k]}(unsorted[k]), with each product and each sum rounded
 * as nsrc consecutive tce_sortacc calls round them (bit-identical), but
 * reading and writing `sorted` once -- the CCSD(T) triples pattern of nine
 * sortaccs per t3 tile (branches/spaghetty2/ccsd_t_tce_sort_list.txt).
 * dims: nsrc*rank source dims, as each tce_sortacc call would pass them;
 * perms: nsrc*rank, 1-based; every permuted shape must equal the output's.
 * rank <= 6, nsrc <= 16.  Device (or managed) memory of one device, else
 * SPAGHETTY_ERR_MEMSPACE; runs on that device, asynchronous on `stream`. */
int spaghetty_sortacc_fused(int rank, int nsrc, const double *const *unsorted,
                            const int *dims, const int *perms, const double *factors,
                            double *sorted, void *stream);

/* The same with the first term overwriting: sorted = factors[0] *
 * permute_{perms[0]}(unsorted[0]), then the sortaccs of k = 1..nsrc-1 --
 * bit-identical to one tce_sort call followed by nsrc-1 tce_sortacc calls
 * (trunk/old_sort.f:33-95 then :512-575; a zero-filled start would turn a
 * -0.0 first product into +0.0), without reading `sorted`.  Sources may
 * repeat (y = sum_k f_k * permute_k(x), the differentiable sort's forward
 * and backward).  Same arguments and limits as spaghetty_sortacc_fused. */
int spaghetty_sort_fused(int rank, int nsrc, const double *const *unsorted,
                         const int *dims, const int *perms, const double *factors,
                         double *sorted, void *stream);

/* ---- batched work lists (one persistent launch for many sorts) -------- */

/* One sort of a batch.  Device pointers on the current device.  perm is
 * 1-based; entries past `rank` are ignored.  acc_factor as in
 * spaghetty_sort (0 = sort, 1 = sortacc). */
typedef struct spaghetty_batch_entry {
    const double *unsorted;
    double *sorted;
    int rank;
    int dims[8];
    int perm[8];
    double factor;
    double acc_factor;
} spaghetty_batch_entry;

typedef struct spaghetty_batch spaghetty_batch;

/* Plan every entry, cut the work into units and upload the work list (the
 * only allocations: job records, unit map, a counter and a status word, and
 * three streams with their events when the batch has direct sorts).
 * Rejects invalid entries (SPAGHETTY_ERR_* of the first bad one; its index
 * from spaghetty_batch_bad_index()), host pointers, and any output that
 * overlaps another buffer of the batch (inputs may be shared). */
int spaghetty_batch_create(const spaghetty_batch_entry *entries, int n, spaghetty_batch **out);
int spaghetty_batch_bad_index(void);

/* Enqueue the whole batch on `stream`: the sorts of at least
 * SPAGHETTY_OPT_BATCH_OWN_MIN elements (2^24 by default) that the
 * single-sort planner puts on the TMA-staged kernel ("direct" sorts; the
 * options in force when the batch was created) one launch each, spread over three streams of the batch that are
 * forked from `stream` by an event and joined back into it; then, on
 * `stream`, a counter reset and ONE persistent kernel launch over the rest.
 * Work enqueued on `stream` afterwards sees every sort done.  Capturable in
 * a CUDA graph (the fork and the join become graph edges).  Launches of one
 * batch on different streams must not overlap (they share the counter and
 * the three streams). */
int spaghetty_batch_launch(spaghetty_batch *batch, void *stream);

/* The same sorts as one launch each through spaghetty_sort_async (the plain
 * path, for comparison). */
int spaghetty_batch_launch_plain(spaghetty_batch *batch, void *stream);

/* Synchronise `stream` and read (and clear) the device status word:
 * SPAGHETTY_OK, or SPAGHETTY_ERR_DEVICE if a job record failed the kernel's
 * validation and was skipped. */
int spaghetty_batch_status(spaghetty_batch *batch, void *stream);

/* {jobs on the work list, work units, algorithmic bytes per launch, shared
 * bytes per CTA}. */
int spaghetty_batch_info(const spaghetty_batch *batch, int64_t *info);

/* Kernel launches one spaghetty_batch_launch enqueues: the large
 * TMA-planned sorts run as their own launch, the rest as one persistent
 * launch. */
int spaghetty_batch_launches(const spaghetty_batch *batch);

/* Fault injection for tests, done by the host: overwrite job `index`'s kind
 * in device memory with an invalid value.  The kernel must flag it in the
 * status word and skip it without touching memory. */
int spaghetty_batch_poison(spaghetty_batch *batch, int index);

int spaghetty_batch_destroy(spaghetty_batch *batch);

/* Autotuner hook of the batched kernel (per-size-bucket tile shapes): sorts
 * of rank `rank` whose largest extent lies in [ext_lo, ext_hi] get boxes
 * grown until the input and output rows hold run_in / run_out contiguous
 * doubles, towards `volume` elements (at most 1024).  A bucket overlapping
 * an existing one replaces it; rank 0 clears every rule.  Applies to batches
 * created afterwards.  The tune file's `batch` lines install these rules.
 * Returns a SPAGHETTY_* code. */
int spaghetty_batch_tune_set(int rank, int ext_lo, int ext_hi, int run_in, int run_out, int volume);

/* Host replay of a batch's plan, needing no GPU: plans the entries as
 * spaghetty_batch_create puts sorts on the persistent kernel's work list
 * (every sort, as with SPAGHETTY_OPT_BATCH_OWN_MIN = 0; the entries'
 * pointers are not read), checks each job record as the kernel does and that
 * its work units cover its boxes once each, and replays every box through
 * the kernel's own index functions: every read, write and staging slot in
 * bounds, and every output element written once, from the input element the
 * permutation maps to it.  num_sms: the SM count the work-unit sizes follow
 * (0: 152).  stats (4 int64, may be NULL): jobs, work units, boxes,
 * elements.  Sorts up to 2^27 elements.  SPAGHETTY_ERR_CONFIG on a violation
 * (and above that size), with spaghetty_batch_bad_index() naming the entry. */
int spaghetty_batch_verify(const spaghetty_batch_entry *entries, int n, int num_sms, int64_t *stats);

/* ---- a contraction with its sorts fused --------------------------------- */

/* The TCE pattern sort -> DGEMM('T','N') -> sort in one kernel
 * (branches/old/python/macaroni/ccsd_t2_8_skeleton.F:174-184), rank-4
 * operands with two contracted indices.  With a_sort = a.permute(perm_a-1)
 * of dims (SA0,SA1,SA2,SA3) read as the matrix [M=SA0*SA1][K=SA2*SA3], and
 * b_sort = b.permute(perm_b-1) of dims (SB0,SB1,SA2,SA3) as [N][K]:
 *   c_sort[n][m] = Sum_k (alpha*a_sort[m][k]) * b_sort[n][k],  dims (SB0,SB1,SA0,SA1)
 *   c = factor * c_sort.permute(perm_c-1)             (acc_factor 0), or
 *   c = c + factor * c_sort.permute(perm_c-1)         (acc_factor 1), or
 *   c = acc_factor*c + factor*(...)                   (otherwise),
 * as tce_sort_4 / tce_sortacc_4 of c_sort round them.  mode 0: k ascending,
 * every product and sum rounded -- the bits of the skeleton's loop_dgemm
 * case 3 (ccsd_t2_8_skeleton.F:214-292) on a zeroed c_sort; mode 1: the
 * same order with fused multiply-adds (faster, not bit-identical); mode 2:
 * the products summed by FP64 matrix instructions (mma.sync .f64, within
 * rounding like mode 1).  Dims
 * and perms are 4 ints each (1-based perms); the operands must agree on the
 * contracted dims (else SPAGHETTY_ERR_DIMS).  Device (or managed) memory of
 * one device, else SPAGHETTY_ERR_MEMSPACE; asynchronous on `stream`. */
int spaghetty_contract_4x4(const double *a, const int *dims_a, const int *perm_a,
                           const double *b, const int *dims_b, const int *perm_b,
                           double *c, const int *perm_c, double alpha, double factor,
                           double acc_factor, int mode, void *stream);

/* The last SPAGHETTY_* code of the contraction entries on this thread. */
int spaghetty_contract_last_error(void);

/* Host replay of the contraction kernel's index arithmetic for one problem
 * (no GPU needed): every operand element is read for exactly the (m, k) or
 * (n, k) it holds and inside its tensor, and every result element is written
 * exactly once, under each of the kernel's three thread shapes.  stats (4
 * int64, may be NULL): M, N, K, tiles.  SPAGHETTY_ERR_CONFIG on a violation,
 * SPAGHETTY_ERR_TOO_LARGE above 2^28 elements per tensor. */
int spaghetty_contract_verify(const int *dims_a, const int *perm_a, const int *dims_b,
                              const int *perm_b, const int *perm_c, int64_t *stats);

/* The macaroni skeleton's subroutine, drop-in
 * (ccsd_t2_8_skeleton.F:174-184): i0(p3,p4,h1,h2) = Sum(p5,p6)
 * v(p3,p4,p5,p6) * t(p5,p6,h1,h2) with a_raw = t of dims (dim5,dim6,dim1,
 * dim2), b_raw = v of dims (dim3,dim4,dim5,dim6) and c_done of dims
 * (dim3,dim4,dim1,dim2), last index stride-1; c_done is overwritten.  The
 * sizes must hold those element counts.  Host or device memory, synchronous;
 * mode 0 arithmetic (bit-identical to the skeleton's loop_dgemm path).  The
 * void forms print 'something is wrong...' and a line naming the problem on
 * a bad argument; the _status form returns the code. */
void ccsd_t2_8(const double *a_raw, const int *size_a, const double *b_raw, const int *size_b,
               double *c_done, const int *size_c, const int *dim1, const int *dim2,
               const int *dim3, const int *dim4, const int *dim5, const int *dim6);
void ccsd_t2_8_(const double *a_raw, const int *size_a, const double *b_raw, const int *size_b,
                double *c_done, const int *size_c, const int *dim1, const int *dim2,
                const int *dim3, const int *dim4, const int *dim5, const int *dim6);
int ccsd_t2_8_status(const double *a_raw, const int *size_a, const double *b_raw,
                     const int *size_b, double *c_done, const int *size_c, const int *dim1,
                     const int *dim2, const int *dim3, const int *dim4, const int *dim5,
                     const int *dim6);

/* Batched sorts for callers that cannot allocate device memory -- an
 * application that has handed the whole device memory to its own pool
 * allocator (a library's cudaMalloc would then fail or escape its
 * accounting), or code that must not cause the device-wide synchronisation
 * cudaMalloc/cudaFree may trigger while other streams run.  No counterpart
 * in the reference (its sorts are host loops that need no scratch).  Runs
 * the same persistent batched kernel as
 * spaghetty_batch_launch, but the work list, unit counter and status word
 * live in a 4 MiB device array that is part of this library (every GPU that
 * loads it holds that array until exit); the caller passes only inputs and
 * outputs, and the call allocates nothing.  Limits: at most 1024 sorts, and
 * the work list must fit the 4 MiB: 896 bytes per sort plus 4 bytes per work
 * unit, a unit being up to 64 boxes and 4K to 64K elements of one sort (the
 * larger the batch, the longer its units; with 1024 sorts, about 819,000
 * units: some 53 G elements on 1024-element boxes, 13 G on 256-element
 * boxes); larger batches return SPAGHETTY_ERR_TOO_LARGE.  The first
 * call on a device looks up the array's device address (set-up); make that
 * first call before any stream capture.  Every call shares the one array,
 * which keeps the previous call's contents: the counter and status word are
 * cleared on each call, the rest is overwritten.  The call is synchronous on
 * `stream` (it returns after the sorts finish, with SPAGHETTY_ERR_DEVICE if
 * a job failed the kernel's checks).  Calls from several host threads are
 * serialised by a lock and each waits for its kernel, so one loaded copy of
 * the library does not run two at once; calls that did overlap on the GPU
 * (a caller that ignores an error return and calls again while the failed
 * call's kernel still runs) would race on the array. */
int spaghetty_sort_batch_noalloc(const spaghetty_batch_entry *entries, int n, void *stream);

/* Library version string. */
const char *spaghetty_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SPAGHETTY_GB300_H */
