// plan.h -- folded-permutation plans and the kernel parameter block.
//
// A call tce_sort_r(u, s, d1..dr, p1..pr, f) is reduced on the host to a
// "folded" problem: unit dims dropped and every run of input indices that
// stays adjacent and in order in the output fused into one index (the
// reference's generator2.py:158-193 fuses trailing pairs and the identity in
// the same spirit; generator3.py:182-210 turns matching trailing runs into
// memcpy).  The folded problem is then covered by "boxes": a box takes a
// length len[d] <= D[d] in every folded dim, chosen so that each box holds a
// contiguous run of >= 32 doubles on the input side AND on the output side.
// A CTA stages one box through shared memory: it reads the box in input
// order (coalesced), and writes it in output order (coalesced).
#pragma once
#include <stdint.h>
#include <nvtx3/nvToolsExt.h>

#define SPG_MAXR 8

// Unsigned division by an invariant divisor (Granlund & Montgomery,
// "Division by Invariant Integers using Multiplication", PLDI 1994, sec. 4):
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, q = (mulhi(m,n) + n) >> l.
// Exact for 1 <= d < 2^31 and 0 <= n < 2^31.
struct FastDiv {
    uint32_t d, m, l;
};

#if defined(__CUDACC__)
#define SPG_HD __host__ __device__ __forceinline__
#else
#define SPG_HD inline
#endif

SPG_HD uint32_t fd_div(uint32_t n, const FastDiv &f) {
#if defined(__CUDA_ARCH__)
    uint32_t hi = __umulhi(f.m, n);
#else
    uint32_t hi = (uint32_t)(((uint64_t)f.m * (uint64_t)n) >> 32);
#endif
    return (hi + n) >> f.l;
}

// One enumeration of the box's elements (fastest dim first).
struct BoxWalk {
    int n;                        // number of box dims with length > 1
    FastDiv len[SPG_MAXR];        // box length per listed dim
    int64_t gs_a[SPG_MAXR];       // primary global stride (elements)
    int64_t gs_b[SPG_MAXR];       // secondary global stride (direct kernels)
    int32_t bs[SPG_MAXR];         // box-local input-order linear stride
    int8_t  mpos[SPG_MAXR];       // 1 = partial dim A, 2 = partial dim B, 0 = none
};

// The grid of boxes (fastest output dim first).
struct BoxGrid {
    int n;                        // dims with more than one box
    FastDiv cnt[SPG_MAXR];        // boxes along the dim
    int64_t in_step[SPG_MAXR];    // len * input stride
    int64_t out_step[SPG_MAXR];   // len * output stride
    int8_t  mpos[SPG_MAXR];       // 1 = partial dim A, 2 = partial dim B
};

// The factors of one call.  f = +-2^k is applied by exponent arithmetic where
// that is exact (kshift = k << 52, sgn = sign bit of f); see spg_pow2.
struct SpgFactor {
    double f, g;
    int32_t k;          // f = +-2^k
    uint32_t sgn_hi;    // sign bit of f in the high 32-bit word
    // high words (sign bit cleared) of the x for which x and x*2^k are both
    // normal: elo <= hi(x) & 0x7FFFFFFF < elo + erange (erange 0: none)
    uint32_t elo, erange;
    // any other normal f, for the integer multiply (spg_mul_int): f's 53-bit
    // significand with its leading one as two 32-bit words (mhi holds the top
    // 21 bits), its biased exponent minus 1023, and its sign in the high
    // word; mul_ok = 0 (f zero, subnormal, inf or NaN) sends every element
    // to the rounded multiply
    uint32_t mhi, mlo;
    int32_t ebias;
    uint32_t mul_ok;
};

struct KParams {
    BoxWalk ld;                   // load phase: input order
    BoxWalk st;                   // store phase: output order
    BoxGrid grid;
    int64_t nelem;                // flat kernel: element count
    uint32_t ntiles;              // number of boxes
    int32_t vol;                  // elements per box
    int32_t pad;                  // shared-memory pad period (0 = none)
    int32_t stage;                // staging-tile stride in elements (pipelined kernel)
    int32_t lenA, extA;           // partial dim A: box length and extent (or 1,1)
    int32_t lenB, extB;
    SpgFactor fac;
};

// KIND_WARP: the warp-shuffle transpose (spg_warp_tr) of small inner tiles,
// both stride-1 extents at most 32 and their product at most 128.
enum SpgKind { KIND_EMPTY = 0, KIND_FLAT = 1, KIND_DIRECT = 2, KIND_TILED = 3, KIND_TMA = 4, KIND_WARP = 5 };

// TMA-staged kernel: how box t's tile coordinates map onto the two 5-D
// tensor maps (input map over the folded input dims in input order, output
// map over the folded dims in output order, adjacent dims merged where the
// box allows).  Grid dim k adds c_k * in_mul[k] to input-map coordinate
// in_mdim[k] (and likewise for the output map).
struct TmaParams {
    int8_t in_mdim[SPG_MAXR];
    int8_t out_mdim[SPG_MAXR];
    int32_t in_mul[SPG_MAXR];
    int32_t out_mul[SPG_MAXR];
    int32_t stage_bytes;          // one load stage: input tile [+ old-output tile]
    int32_t in_bytes;             // one tile, 1024-aligned (old-output tile offset)
    int32_t out_bytes;            // one output slot (two of them follow the stages)
    int32_t tx_bytes;             // bytes the loads of one box deliver
    int32_t same_order;           // 1: both maps list the dims in input order (identity permute)
    // diagonal skew of the permute step (spg_tma_slot): slot n's output-tile
    // coordinate y along one output dim (stride sk_stride in the output
    // tile, box length sk_len) is moved to (y + (n mod 16) * sk_mul) mod
    // sk_len; sk_mul = 0: no skew
    int32_t sk_stride, sk_len, sk_mul;
    int *status;                  // error word (bounded waits that timed out)
};

struct TmaLayout {
    int rank_in, rank_out;        // map ranks before padding to 5
    uint64_t in_dim[5], out_dim[5];
    uint64_t in_stride[5], out_stride[5];   // bytes, [0] = 8 (element)
    uint32_t in_box[5], out_box[5];
    TmaParams tp;
};

// Arithmetic applied per element: the reference generated nests' cases
// (trunk/generator2.py:57-130: copy, scale, add, scaled add, g*s + f*u),
// with the factor split by how it can be applied.  GB300 executes FP64 at a
// small fraction of its integer rate, so factors whose product is exact
// (f = 1, -1, +-2^k) are applied with integer operations on the bit pattern
// wherever that gives the same bits as the rounded multiply, and with the
// multiply otherwise (zero, subnormal, inf/NaN inputs, over/underflow).
enum SpgOp {
    OP_SORT_ONE = 0,   // s = u
    OP_SORT_NEG = 1,   // s = -u
    OP_SORT_POW2 = 2,  // s = u * (+-2^k)
    OP_SORT_ANY = 3,   // s = u * f
    OP_ACC_ONE = 4,    // s = s + u
    OP_ACC_NEG = 5,    // s = s + (-u)
    OP_ACC_POW2 = 6,   // s = s + u * (+-2^k)
    OP_ACC_ANY = 7,    // s = s + u * f
    OP_GEN = 8,        // s = g*s + f*u
    OP_COUNT = 9
};

// 0 = sort, 1 = sortacc, 2 = general acc_factor
inline int spg_op_class(int op) { return op < OP_ACC_ONE ? 0 : (op == OP_GEN ? 2 : 1); }

struct Folded {
    int rank;                 // folded rank (0 = single element or empty)
    int64_t D[SPG_MAXR];      // folded extents, input order, last is stride-1
    int P[SPG_MAXR];          // output position -> input dim (0-based)
    int64_t nelem;
    bool empty;
};

struct Plan {
    Folded fo;
    int kind;
    int op;
    int box[SPG_MAXR];
    int threads, ept;
    int stages;               // tiled: 0 = register-staged, 2/3 = cp.async pipeline depth
    int run_in, run_out;
    int masked;
    int grid;                 // filled at launch time
    int smem_bytes;
    int64_t wf_pad0, wf_ideal; // store-phase shared wavefronts: unpadded tile, conflict-free
    int sk_stride, sk_len, sk_mul;   // TMA kernel: permute-step skew (TmaParams)
    KParams kp;
};

// An NVTX range around one library entry (header-only NVTX 3: a few
// nanoseconds when no profiler is attached), so that timelines name the
// library's host calls: the synchronous sorts, the batched launches, the
// fused sortacc and the fused contraction.
struct SpgRange {
    explicit SpgRange(const char *name) { nvtxRangePushA(name); }
    ~SpgRange() { nvtxRangePop(); }
    SpgRange(const SpgRange &) = delete;
    SpgRange &operator=(const SpgRange &) = delete;
};

// Host-side planning (plan.cpp).  All return a SPAGHETTY_* status.
FastDiv spg_make_fastdiv(uint32_t d);
int spg_fold(int rank, const int *dims, const int *perm, Folded *out);
int spg_choose_op(double f, double g);
int spg_plan(const Folded &fo, int op, const int *box_override, int threads_override,
             int ept_override, int stages_override, int num_sms, Plan *out);
// Tile-shape rule of the batched kernel for one size bucket: sorts of rank
// `rank` whose largest extent lies in [ext_lo, ext_hi] get boxes grown until
// the input and output rows hold run_in / run_out doubles, towards `volume`
// elements.
// CTA shape of the persistent batched kernel (batch.cu); its boxes hold at
// most SPG_BATCH_NT * SPG_BATCH_EPT elements (spg_plan_batch).
#ifndef SPG_BATCH_NT
#define SPG_BATCH_NT 256
#endif
#ifndef SPG_BATCH_EPT
#define SPG_BATCH_EPT 4
#endif
struct SpgBatchRule {
    int rank, ext_lo, ext_hi, run_in, run_out, volume;
};
int spg_plan_batch(const Folded &fo, int op, const SpgBatchRule *rule, Plan *out);
// Installs the tune file beside the library once per process (api.cu).
void spg_autoload_tune();
// Tensor-map encoding (5 dims, FP64; swizzle128: 128-byte swizzle) and the
// device address of the kernels' status word (api.cu).
struct CUtensorMap_st;
int spg_encode_map(CUtensorMap_st *m, const double *ptr, const uint64_t *dim, const uint64_t *stride,
                   const uint32_t *box, int swizzle128);
int *spg_status_word();
// Whether the single-sort plan of a problem is the TMA-staged kernel (api.cu).
bool spg_plan_is_tma(int dev, int rank, const int *dims, const int *perm, double factor, double acc_factor,
                     const double *unsorted, const double *sorted);
// Host replay of one launch's index arithmetic (api.cu): in-bounds reads,
// writes and tile slots, and a bijection onto the permuted output.
int spg_replay_params(const KParams &kp, const Folded &fo, int kind, int64_t smem_elems, int64_t *stats);
// The batch options SPAGHETTY_OPT_BATCH_OWN_MIN / _OWN_KINDS (batch.cu).
int spg_batch_option(int option, int value);
// Asynchronous sort of device pointers of device `dev` (api.cu), no pointer checks.
int spg_sort_async_on(int dev, int rank, const double *unsorted, double *sorted, const int *dims,
                      const int *perm, double factor, double acc_factor, void *stream);
int spg_default_box_tma(const Folded &fo, int num_sms, int vmax, int *box);
int spg_box_greedy(const Folded &fo, int trun_in, int trun_out, int vtarget, int vmax, int *box);
int spg_build_params(Plan *pl, double f, double g);
SpgFactor spg_make_factor(double f, double g);
int spg_selftest_host(void);
// TMA layout of a tiled plan: SPAGHETTY_OK, or SPAGHETTY_ERR_NOKERNEL when
// the plan cannot be expressed as 5-D tensor maps (odd stride-1 extents,
// > 5 map dims, box > 256 along a map dim, ...).  stages: pipeline depth.
int spg_tma_layout(const Plan &pl, int stages, TmaLayout *out);

