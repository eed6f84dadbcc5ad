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
    double f, g;
};

enum SpgKind { KIND_EMPTY = 0, KIND_FLAT = 1, KIND_DIRECT = 2, KIND_TILED = 3 };

// Arithmetic applied per element (the reference generated nests' five cases,
// trunk/generator2.py:57-130, plus the accumulate with an exact factor).
enum SpgOp {
    OP_COPY = 0,    // s = u                       (factor == 1, sort)
    OP_SCALE = 1,   // s = u*f                     (sort)
    OP_ACC1 = 2,    // s = s + u                   (factor == 1, sortacc)
    OP_ACCF = 3,    // s = s + u*f                 (sortacc)
    OP_GEN = 4,     // s = g*s + f*u               (general acc_factor)
    OP_COUNT = 5
};

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
    KParams kp;
};

// Host-side planning (plan.cpp).  All return a SPAGHETTY_* status.
int spg_fold(int rank, const int *dims, const int *perm, Folded *out);
int spg_choose_op(double f, double g);
int spg_plan(const Folded &fo, int op, const int *box_override, int threads_override,
             int ept_override, int stages_override, int num_sms, Plan *out);
int spg_build_params(Plan *pl, double f, double g);
int spg_selftest_host(void);
