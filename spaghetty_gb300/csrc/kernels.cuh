// kernels.cuh -- sm_103a tensor-permutation kernels (FP64, bit-exact).
//
// Three kernel families cover every folded permutation:
//   spg_flat    rank <= 1 after folding: identity permutation, a streaming
//               copy/scale/axpy (the reference's f_memcpy path,
//               trunk/tester_cutil.c:51-76, trunk/generator3.py:182-210).
//   spg_direct  the stride-1 index is unchanged and its rows are long: every
//               element is read and written by the same thread, no staging.
//   spg_tiled   everything else: a persistent CTA walks the grid of boxes;
//               per box it loads the elements in input order (coalesced
//               runs), stages them in a padded shared-memory tile, and writes
//               them in output order (coalesced runs).
// Per-element box offsets are computed once per CTA (fast division) and kept
// in registers for all the boxes the CTA processes.
//
// Arithmetic is the reference's: one rounded product, then one rounded sum
// (trunk/old_sort.f:58,537: y(ib) = y(ib) + x(ia)*s); __dmul_rn/__dadd_rn
// forbid contraction into an FMA.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "plan.h"

// The rounded FP64 multiply of the rarely taken inexact cases, kept out of
// line: inlined, the compiler predicates it (or hoists it) into the common
// path, where a predicated-off FP64 instruction still occupies GB300's
// narrow FP64 pipe for every element.
static __device__ __noinline__ double spg_dmul_branch(double x, double f) {
    return __dmul_rn(x, f);
}

// x * f for f = +-2^k on the integer path: when x and x*f are both normal
// (the high word of x, sign bit cleared, in the window [elo, elo + erange)
// that the host derives from k), the product is exact and equals x with k
// added to its exponent field and f's sign applied; for x = +-0 only the
// sign changes.  Exponent and sign live in the high 32-bit word, so this is
// 32-bit integer work only (64-bit integer arithmetic on the bit pattern
// occupies GB300's scarce FP64 pipe).  `exact` is cleared for every other
// input (subnormal, inf, NaN) or result (overflow, underflow): those need the
// rounded multiply.
__device__ __forceinline__ double spg_pow2_fast(double x, const SpgFactor &F, bool &exact) {
    const uint32_t hi = (uint32_t)__double2hiint(x);
    const int lo = __double2loint(x);
    const uint32_t h = hi & 0x7FFFFFFFu;
    const bool inr = h - F.elo < F.erange;
    exact = exact && (inr || (h | (uint32_t)lo) == 0u);
    return __hiloint2double((int)((hi + (inr ? ((uint32_t)F.k << 20) : 0u)) ^ F.sgn_hi), lo);
}

// x * -1 is exact for every input: the sign bit flipped, in the integer pipe
// (for NaN the multiply would also give a NaN; NaN payloads are not part of
// the contract).
__device__ __forceinline__ double spg_neg(double x) {
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000u, __double2loint(x));
}

// The same for sortacc, with NaN inputs sent to the rounded multiply behind a
// warp vote.  Measured on GB300 against y - x (one rounded subtract, the same
// bits): the sweep's f = -1 sortaccs at 50^4 run 5% faster this way on their
// tuned plans (4263 vs 4052 GB/s); the fused kernel uses the subtract.
__device__ __forceinline__ double spg_neg_voted(double x, const SpgFactor &F) {
    const uint32_t hi = (uint32_t)__double2hiint(x);
    const int lo = __double2loint(x);
    const uint32_t mag = hi & 0x7FFFFFFFu;
    const bool exact = mag < 0x7FF00000u || (mag == 0x7FF00000u && lo == 0);
    double r = __hiloint2double((int)(hi ^ 0x80000000u), lo);
    if (__any_sync(__activemask(), !exact)) {
        if (!exact) r = spg_dmul_branch(x, F.f);
    }
    return r;
}

// x * f, rounded to nearest even, for any normal f, in 32-bit integer
// operations: the IEEE 754 binary64 product by the schoolbook method for
// software floating point (exact product of the two 53-bit significands,
// normalisation by one bit, round to nearest with ties to even from the round
// bit and the sticky bits, exponents added; IEEE 754-2008 sec. 4.3.1 and 5.4.1).
// The 106-bit significand product is built from four 32 x 32-bit products
// (x's significand as 21 + 32 bits, f's precomputed on the host the same way)
// with carry-chained 32-bit adds.  The packed result's rounding increment
// carries into the exponent field, which also gives the right infinity when
// rounding overflows.  `exact` is cleared where this path does not apply:
// x subnormal, inf or NaN, a product outside the normal range before
// rounding, or f itself not normal (F.mul_ok = 0); x = +-0 gives a signed
// zero.  GB300 issues FP64 multiplies at a small fraction of its 32-bit
// integer rate, but this costs about 40 integer instructions per element:
// measured on GB300 with f = 0.3, it is faster only in the flat streaming
// kernel (100^4 identity: sortacc 6683 against 5969 GB/s, sort 6283 against
// 6200), and slower in the staged kernels, whose permute threads are issue
// bound (100^4 perm 4321 on the TMA kernel: sort 4872 against 5730; the
// batched mix 2958 against 3470), which keep the rounded multiply.
__device__ __forceinline__ double spg_mul_int(double x, const SpgFactor &F, bool &exact) {
    const uint32_t hi = (uint32_t)__double2hiint(x);
    const uint32_t lo = (uint32_t)__double2loint(x);
    const uint32_t ex = (hi >> 20) & 0x7FFu;
    const uint32_t xh = (hi & 0xFFFFFu) | 0x100000u;
    // P = (xh 2^32 + lo)(mhi 2^32 + mlo) as the words w3:w2:w1:w0, P < 2^106
    const uint32_t a0 = lo * F.mlo, a1 = __umulhi(lo, F.mlo);
    const uint32_t b0 = xh * F.mlo, b1 = __umulhi(xh, F.mlo);
    const uint32_t c0 = lo * F.mhi, c1 = __umulhi(lo, F.mhi);
    const uint32_t d0 = xh * F.mhi, d1 = __umulhi(xh, F.mhi);
    uint32_t w1, w2, w3;
    asm("add.cc.u32 %0, %3, %4;\n\t"
        "addc.cc.u32 %1, %5, %6;\n\t"
        "addc.u32 %2, %7, 0;\n\t"
        "add.cc.u32 %0, %0, %8;\n\t"
        "addc.cc.u32 %1, %1, %9;\n\t"
        "addc.u32 %2, %2, 0;"
        : "=&r"(w1), "=&r"(w2), "=&r"(w3)
        : "r"(a1), "r"(b0), "r"(b1), "r"(d0), "r"(d1), "r"(c0), "r"(c1));
    // P in [2^104, 2^106): s = 1 when bit 105 (bit 9 of w3) is set; the
    // significand is P >> (52 + s), the round bit the one below it
    const uint32_t s = (w3 >> 9) & 1u;
    const uint32_t sh = 20u + s;
    const uint32_t sig_lo = __funnelshift_r(w1, w2, sh);
    const uint32_t sig_hi = __funnelshift_r(w2, w3, sh);      // 21 bits, leading one at bit 20
    const uint32_t rnd = (w1 >> (sh - 1u)) & 1u;
    const uint32_t sticky = (w1 & ((1u << (sh - 1u)) - 1u)) | a0;
    const uint32_t inc = rnd & ((sticky != 0u ? 1u : 0u) | (sig_lo & 1u));
    const uint32_t e = ex + (uint32_t)F.ebias + s;             // biased exponent of the result
    uint32_t rlo, rhi;
    asm("add.cc.u32 %0, %2, %3;\n\t"
        "addc.u32 %1, %4, 0;"
        : "=r"(rlo), "=r"(rhi)
        : "r"(sig_lo), "r"(inc), "r"((e << 20) + sig_hi - 0x100000u));
    const uint32_t sign = (hi ^ F.sgn_hi) & 0x80000000u;
    const bool zero = ((hi & 0x7FFFFFFFu) | lo) == 0u;
    const bool normal = ex - 1u < 2046u && e - 1u < 2046u;
    exact = exact && F.mul_ok != 0u && (normal || zero);
    // select on the 32-bit halves: a select of two doubles would be an FP64
    // pipe instruction on GB300
    return __hiloint2double((int)(zero ? sign : (rhi | sign)), (int)(zero ? 0u : rlo));
}

// The integer multiply's operand fields of a run-time factor f (the host
// builds them once per call with spg_make_factor; the fused contraction's
// products have a different factor every step).
__device__ __forceinline__ SpgFactor spg_mul_operand(double f) {
    SpgFactor F;
    const uint32_t hi = (uint32_t)__double2hiint(f);
    const uint32_t ef = (hi >> 20) & 0x7FFu;
    F.f = f;
    F.g = 0.0;
    F.k = 0;
    F.elo = 0;
    F.erange = 0;
    F.sgn_hi = hi & 0x80000000u;
    F.mhi = (hi & 0xFFFFFu) | 0x100000u;
    F.mlo = (uint32_t)__double2loint(f);
    F.ebias = (int32_t)ef - 1023;
    F.mul_ok = (ef - 1u < 2046u) ? 1u : 0u;
    return F;
}

__device__ __forceinline__ double spg_mul(double x, const SpgFactor &F) {
    bool exact = true;
    double r = spg_mul_int(x, F, exact);
    if (__any_sync(__activemask(), !exact)) {
        if (!exact) r = spg_dmul_branch(x, F.f);
    }
    return r;
}

// Per-element forms: the rare inexact cases take the rounded multiply behind
// a warp vote, so that it is a real branch and the bits always equal
// __dmul_rn(x, f).
__device__ __forceinline__ double spg_pow2(double x, const SpgFactor &F) {
    bool exact = true;
    double r = spg_pow2_fast(x, F, exact);
    if (__any_sync(__activemask(), !exact)) {
        if (!exact) r = spg_dmul_branch(x, F.f);
    }
    return r;
}

template <int OP>
__device__ __forceinline__ double spg_apply(double x, double y, const SpgFactor &F) {
    if (OP == OP_SORT_ONE) return x;
    if (OP == OP_SORT_NEG) return spg_neg(x);
    if (OP == OP_SORT_POW2) return spg_pow2(x, F);
    if (OP == OP_SORT_ANY) return __dmul_rn(x, F.f);
    if (OP == OP_ACC_ONE) return __dadd_rn(y, x);
    if (OP == OP_ACC_NEG) return __dadd_rn(y, spg_neg_voted(x, F));
    if (OP == OP_ACC_POW2) return __dadd_rn(y, spg_pow2(x, F));
    if (OP == OP_ACC_ANY) return __dadd_rn(y, __dmul_rn(x, F.f));
    return __dadd_rn(__dmul_rn(F.g, y), __dmul_rn(F.f, x));   // OP_GEN
}

template <int OP>
struct spg_reads_out { static constexpr bool value = (OP >= OP_ACC_ONE); };

// Two-phase form for the register-staged kernels, whose threads write EPT
// elements of a box straight to global memory: spg_apply_fast gives every
// element's integer-path result and clears `exact` where that is not the
// rounded product; after one warp vote over all of them, a warp with any
// such element recomputes its elements with spg_apply_mul, the rounded
// arithmetic for every input.  No vote or branch sits between the elements,
// so their shared-memory loads and global stores stay batched.  (The
// TMA-staged kernel keeps the per-element form: there it measured faster.)
template <int OP>
struct spg_has_fast {
    static constexpr bool value = OP == OP_SORT_POW2 || OP == OP_ACC_POW2;
};

template <int OP>
__device__ __forceinline__ double spg_apply_fast(double x, double y, const SpgFactor &F, bool &exact) {
    if (OP == OP_SORT_POW2) return spg_pow2_fast(x, F, exact);
    if (OP == OP_ACC_POW2) return __dadd_rn(y, spg_pow2_fast(x, F, exact));
    return spg_apply<OP>(x, y, F);
}

// (the multiply out of line: this runs only for a warp with an inexact
// element, and inlined the compiler predicates it into every box)
template <int OP>
__device__ __forceinline__ double spg_apply_mul(double x, double y, const SpgFactor &F) {
    if (OP == OP_SORT_POW2) return spg_dmul_branch(x, F.f);
    if (OP == OP_ACC_POW2) return __dadd_rn(y, spg_dmul_branch(x, F.f));
    return spg_apply<OP>(x, y, F);
}

// Every element is read once and written once: streaming (evict-first)
// accesses.  Measured on GB300 (100^4, perm 4321): with default write-back
// stores DRAM reads grew from 1.03 GB to 1.49 GB for 0.80 GB of input.
__device__ __forceinline__ double spg_ld_in(const double *p) { return __ldcs(p); }
__device__ __forceinline__ double spg_ld_out(const double *p) { return __ldcs(p); }
__device__ __forceinline__ void spg_st_out(double *p, double v) { __stcs(p, v); }

// Decompose a box-local element index along a walk.  Host-callable too, so
// that spaghetty_plan_verify can replay the exact index arithmetic on the CPU.
__host__ __device__ __forceinline__ void spg_walk(const BoxWalk &w, uint32_t e, int32_t &oa,
                                         int32_t &ob, int32_t &lin, uint32_t &pk) {
    oa = 0; ob = 0; lin = 0; pk = 0;
#pragma unroll
    for (int k = 0; k < SPG_MAXR; ++k) {
        if (k < w.n) {
            const uint32_t q = fd_div(e, w.len[k]);
            const uint32_t c = e - q * w.len[k].d;
            e = q;
            oa += (int32_t)c * (int32_t)w.gs_a[k];
            ob += (int32_t)c * (int32_t)w.gs_b[k];
            lin += (int32_t)c * w.bs[k];
            if (w.mpos[k] == 1) pk |= c << 16;
            if (w.mpos[k] == 2) pk |= c;
        }
    }
}

// Box t -> base offsets and the element limits of the (at most two) dims
// whose last box is partial.
__host__ __device__ __forceinline__ void spg_box(const KParams &p, uint32_t t, int64_t &ib,
                                        int64_t &ob, uint32_t &limA, uint32_t &limB) {
    ib = 0; ob = 0;
    limA = (uint32_t)p.lenA;
    limB = (uint32_t)p.lenB;
#pragma unroll
    for (int k = 0; k < SPG_MAXR; ++k) {
        if (k < p.grid.n) {
            const uint32_t q = fd_div(t, p.grid.cnt[k]);
            const uint32_t c = t - q * p.grid.cnt[k].d;
            t = q;
            ib += (int64_t)c * p.grid.in_step[k];
            ob += (int64_t)c * p.grid.out_step[k];
            if (p.grid.mpos[k] == 1) {
                const int r = p.extA - (int)c * p.lenA;
                limA = (uint32_t)(r < p.lenA ? r : p.lenA);
            }
            if (p.grid.mpos[k] == 2) {
                const int r = p.extB - (int)c * p.lenB;
                limB = (uint32_t)(r < p.lenB ? r : p.lenB);
            }
        }
    }
}

__host__ __device__ __forceinline__ bool spg_valid(uint32_t pk, uint32_t limA, uint32_t limB) {
    return (pk >> 16) < limA && (pk & 0xFFFFu) < limB;
}

#define SPG_INVALID 0xFFFFFFFFu

// ---------------------------------------------------------------------------
// Per-thread element tables of one box shape, built once per CTA (and again
// by the batched kernel whenever it switches to another sort).
//   tiled:  ioff/smw/pkl = load side (input offset, shared slot, mask coords)
//           ooff/smr/pks = store side (output offset, shared slot, mask coords)
//   direct: ioff/ooff/pkl only (input and output offset of the same element)
template <int NT, int EPT>
struct SpgTab {
    int32_t ioff[EPT], smw[EPT], ooff[EPT], smr[EPT];
    uint32_t pkl[EPT], pks[EPT];

    __device__ __forceinline__ void build_tiled(const KParams &p, uint32_t tid) {
#pragma unroll
        for (int k = 0; k < EPT; ++k) {
            const uint32_t e = tid + k * NT;
            if (e < (uint32_t)p.vol) {
                int32_t a, b, lin;
                uint32_t pk;
                spg_walk(p.ld, e, a, b, lin, pk);
                ioff[k] = a;
                smw[k] = (int32_t)e + (p.pad ? (int32_t)e / p.pad : 0);
                pkl[k] = pk;
                spg_walk(p.st, e, a, b, lin, pk);
                ooff[k] = a;
                smr[k] = lin + (p.pad ? lin / p.pad : 0);
                pks[k] = pk;
            } else {
                ioff[k] = 0; smw[k] = 0; pkl[k] = SPG_INVALID;
                ooff[k] = 0; smr[k] = 0; pks[k] = SPG_INVALID;
            }
        }
    }

    __device__ __forceinline__ void build_direct(const KParams &p, uint32_t tid) {
#pragma unroll
        for (int k = 0; k < EPT; ++k) {
            const uint32_t e = tid + k * NT;
            if (e < (uint32_t)p.vol) {
                int32_t a, b, lin;
                uint32_t pk;
                spg_walk(p.ld, e, a, b, lin, pk);
                ioff[k] = a; ooff[k] = b; pkl[k] = pk;
            } else {
                ioff[k] = 0; ooff[k] = 0; pkl[k] = SPG_INVALID;
            }
            smw[k] = 0; smr[k] = 0; pks[k] = SPG_INVALID;
        }
    }
};

// Output phase of a register-staged box: this thread's element k goes from
// staged-tile slot smr[k] to dst + ooff[k] (y[k]: the old output, sortacc).
template <int NT, int EPT, int OP>
__device__ __forceinline__ void spg_write_box(const SpgTab<NT, EPT> &tb, const double *tile,
                                              const double (&y)[EPT], double *dst,
                                              uint32_t limA, uint32_t limB, const SpgFactor &fac) {
    if (spg_has_fast<OP>::value) {
        double r[EPT];
        bool exact = true;
#pragma unroll
        for (int k = 0; k < EPT; ++k) {
            r[k] = 0.0;
            if (spg_valid(tb.pks[k], limA, limB))
                r[k] = spg_apply_fast<OP>(tile[tb.smr[k]], spg_reads_out<OP>::value ? y[k] : 0.0,
                                          fac, exact);
        }
        if (!__all_sync(__activemask(), exact)) {
#pragma unroll
            for (int k = 0; k < EPT; ++k)
                if (spg_valid(tb.pks[k], limA, limB))
                    r[k] = spg_apply_mul<OP>(tile[tb.smr[k]],
                                             spg_reads_out<OP>::value ? y[k] : 0.0, fac);
        }
#pragma unroll
        for (int k = 0; k < EPT; ++k)
            if (spg_valid(tb.pks[k], limA, limB)) spg_st_out(dst + tb.ooff[k], r[k]);
    } else {
#pragma unroll
        for (int k = 0; k < EPT; ++k) {
            if (spg_valid(tb.pks[k], limA, limB)) {
                const double x = tile[tb.smr[k]];
                spg_st_out(dst + tb.ooff[k],
                           spg_apply<OP>(x, spg_reads_out<OP>::value ? y[k] : 0.0, fac));
            }
        }
    }
}

// One box of the register-staged tiled kernel.  Contains two CTA barriers:
// every thread of the CTA must call it for the same box.
template <int NT, int EPT, int OP>
__device__ __forceinline__ void spg_tiled_box(const KParams &p, const SpgTab<NT, EPT> &tb,
                                              const double *__restrict__ in,
                                              double *__restrict__ out, uint32_t t, double *sm) {
    int64_t ib, ob;
    uint32_t limA, limB;
    spg_box(p, t, ib, ob, limA, limB);
    const double *src = in + ib;
    double *dst = out + ob;
    const SpgFactor fac = p.fac;
    double v[EPT];
#pragma unroll
    for (int k = 0; k < EPT; ++k) {
        v[k] = 0.0;
        if (spg_valid(tb.pkl[k], limA, limB)) v[k] = spg_ld_in(src + tb.ioff[k]);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < EPT; ++k)
        if (tb.pkl[k] != SPG_INVALID) sm[tb.smw[k]] = v[k];
    __syncthreads();
    double y[EPT];
    if (spg_reads_out<OP>::value) {
#pragma unroll
        for (int k = 0; k < EPT; ++k) {
            y[k] = 0.0;
            if (spg_valid(tb.pks[k], limA, limB)) y[k] = spg_ld_out(dst + tb.ooff[k]);
        }
    }
    spg_write_box<NT, EPT, OP>(tb, sm, y, dst, limA, limB, fac);
}

// One box of the direct kernel (no barrier).
template <int NT, int EPT, int OP>
__device__ __forceinline__ void spg_direct_box(const KParams &p, const SpgTab<NT, EPT> &tb,
                                               const double *__restrict__ in,
                                               double *__restrict__ out, uint32_t t) {
    int64_t ib, ob;
    uint32_t limA, limB;
    spg_box(p, t, ib, ob, limA, limB);
    const double *src = in + ib;
    double *dst = out + ob;
    const SpgFactor fac = p.fac;
    double v[EPT], y[EPT];
#pragma unroll
    for (int k = 0; k < EPT; ++k) {
        v[k] = 0.0; y[k] = 0.0;
        if (spg_valid(tb.pkl[k], limA, limB)) {
            v[k] = spg_ld_in(src + tb.ioff[k]);
            if (spg_reads_out<OP>::value) y[k] = spg_ld_out(dst + tb.ooff[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < EPT; ++k)
        if (spg_valid(tb.pkl[k], limA, limB))
            spg_st_out(dst + tb.ooff[k], spg_apply<OP>(v[k], y[k], fac));
}

// ---------------------------------------------------------------------------
template <int NT, int EPT, int OP>
__global__ void __launch_bounds__(NT)
spg_tiled(const double *__restrict__ in, double *__restrict__ out,
          const __grid_constant__ KParams p) {
    extern __shared__ double sm[];
    SpgTab<NT, EPT> tb;
    tb.build_tiled(p, threadIdx.x);
    for (uint32_t t = blockIdx.x; t < p.ntiles; t += gridDim.x)
        spg_tiled_box<NT, EPT, OP>(p, tb, in, out, t, sm);
}

// ---------------------------------------------------------------------------
// Pipelined tiled kernel: the load phase issues 8-byte cp.async copies
// straight from global memory into one of S shared-memory stages (masked
// elements are zero-filled without touching memory), so S-1 boxes are in
// flight per CTA while the current one is written out in output order.
__device__ __forceinline__ void spg_cp_async8(uint32_t saddr, const double *src, uint32_t bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(saddr), "l"(src),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void spg_cp_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void spg_cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <int NT, int EPT, int OP, int S>
__global__ void __launch_bounds__(NT)
spg_tiled_async(const double *__restrict__ in, double *__restrict__ out,
                const __grid_constant__ KParams p) {
    extern __shared__ __align__(128) double sm[];
    SpgTab<NT, EPT> tb;
    tb.build_tiled(p, threadIdx.x);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
    const uint32_t G = gridDim.x;
    const uint32_t stage_bytes = (uint32_t)p.stage * 8u;

    auto issue = [&](uint32_t t, int st) {
        if (t < p.ntiles) {
            int64_t ib, ob;
            uint32_t limA, limB;
            spg_box(p, t, ib, ob, limA, limB);
            const double *src = in + ib;
            const uint32_t sb = sbase + (uint32_t)st * stage_bytes;
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                if (tb.pkl[k] != SPG_INVALID) {
                    const bool v = spg_valid(tb.pkl[k], limA, limB);
                    spg_cp_async8(sb + (uint32_t)tb.smw[k] * 8u, v ? src + tb.ioff[k] : in,
                                  v ? 8u : 0u);
                }
            }
        }
        spg_cp_commit();
    };

    const SpgFactor fac = p.fac;
    uint32_t t = blockIdx.x;
#pragma unroll
    for (int q = 0; q < S - 1; ++q) issue(t + (uint32_t)q * G, q);
    // One block barrier per box: after it every thread's copies of box t
    // have landed and every thread has finished box t-1, whose stage is the
    // one refilled (with box t+S-1) right after it.  A sortacc's old-output
    // loads go out before the wait, which hides their latency (over the
    // host link, for host-mapped buffers, a few microseconds).
    for (int it = 0; t < p.ntiles; t += G, ++it) {
        const int st = it % S;
        int64_t ib, ob;
        uint32_t limA, limB;
        spg_box(p, t, ib, ob, limA, limB);
        double *dst = out + ob;
        double y[EPT];
        if (spg_reads_out<OP>::value) {
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                y[k] = 0.0;
                if (spg_valid(tb.pks[k], limA, limB)) y[k] = spg_ld_out(dst + tb.ooff[k]);
            }
        }
        spg_cp_wait<S - 2>();                  // this thread's copies for box t have landed
        __syncthreads();                       // ... everyone's, and box t-1 is done
        issue(t + (uint32_t)(S - 1) * G, (it + S - 1) % S);
        const double *tile = sm + st * p.stage;
        spg_write_box<NT, EPT, OP>(tb, tile, y, dst, limA, limB, fac);
    }
    spg_cp_wait<0>();
}

// ---------------------------------------------------------------------------
template <int NT, int EPT, int OP>
__global__ void __launch_bounds__(NT)
spg_direct(const double *__restrict__ in, double *__restrict__ out,
           const __grid_constant__ KParams p) {
    SpgTab<NT, EPT> tb;
    tb.build_direct(p, threadIdx.x);
    for (uint32_t t = blockIdx.x; t < p.ntiles; t += gridDim.x)
        spg_direct_box<NT, EPT, OP>(p, tb, in, out, t);
}

// The flat kernel's arithmetic: arbitrary factors on the integer multiply.
template <int OP>
__device__ __forceinline__ double spg_apply_flat(double x, double y, const SpgFactor &F) {
    if (OP == OP_SORT_ANY) return spg_mul(x, F);
    if (OP == OP_ACC_ANY) return __dadd_rn(y, spg_mul(x, F));
    return spg_apply<OP>(x, y, F);
}

// ---------------------------------------------------------------------------
// Flat: n contiguous elements, identity order.  VEC = 2 uses 16-byte
// accesses (both pointers 16-byte aligned); the odd tail element is handled
// by thread 0 of block 0.
template <int OP, int VEC>
__global__ void __launch_bounds__(256)
spg_flat(const double *__restrict__ in, double *__restrict__ out, int64_t n,
         const SpgFactor fac) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (VEC == 2) {
        const int64_t n2 = n >> 1;
        const double2 *in2 = reinterpret_cast<const double2 *>(in);
        double2 *out2 = reinterpret_cast<double2 *>(out);
        int64_t j = i0;
        for (; j + 3 * stride < n2; j += 4 * stride) {
            double2 x[4], y[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                x[u] = __ldcs(in2 + j + u * stride);
                if (spg_reads_out<OP>::value) y[u] = __ldcs(out2 + j + u * stride);
                else y[u] = make_double2(0.0, 0.0);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                double2 r;
                r.x = spg_apply_flat<OP>(x[u].x, y[u].x, fac);
                r.y = spg_apply_flat<OP>(x[u].y, y[u].y, fac);
                __stcs(out2 + j + u * stride, r);
            }
        }
        for (; j < n2; j += stride) {
            const double2 x = __ldcs(in2 + j);
            double2 y = make_double2(0.0, 0.0);
            if (spg_reads_out<OP>::value) y = __ldcs(out2 + j);
            double2 r;
            r.x = spg_apply_flat<OP>(x.x, y.x, fac);
            r.y = spg_apply_flat<OP>(x.y, y.y, fac);
            __stcs(out2 + j, r);
        }
        if ((n & 1) && i0 == 0) {
            const double x = in[n - 1];
            const double y = spg_reads_out<OP>::value ? out[n - 1] : 0.0;
            out[n - 1] = spg_apply_flat<OP>(x, y, fac);
        }
    } else {
        for (int64_t j = i0; j < n; j += stride) {
            const double x = __ldcs(in + j);
            const double y = spg_reads_out<OP>::value ? __ldcs(out + j) : 0.0;
            __stcs(out + j, spg_apply_flat<OP>(x, y, fac));
        }
    }
}

// ---------------------------------------------------------------------------
// Warp-shuffle transpose of small inner tiles.  When the input's stride-1
// dim a and the output's stride-1 dim b are different and short (A, B <= 32,
// A*B <= 32*K), one warp moves a whole A x B tile (every other dim is a
// single index of the tile grid) through its registers: it loads the tile
// in input order (lane l holds elements l, l+32, ... : rows of A contiguous
// doubles), and each lane fetches the elements of its output-order slots
// from the lanes that hold them with warp shuffles (K shuffles of 64 bits
// per slot, keeping the one from the right register), then stores them in
// output order (rows of B contiguous doubles).  No shared memory and no
// block barrier: a warp's tile is done after one round of loads, shuffles
// and stores, which is what small tensors (where a few microseconds of
// latency per staged box dominate) and batches of small tiles need.  The
// per-slot offsets come from the plan's two box walks (ld: a then b; st:
// b then a), whose lin index is the element's input-order place in the tile.
template <int OP, int K>
__global__ void __launch_bounds__(256)
spg_warp_tr(const double *__restrict__ in, double *__restrict__ out, const __grid_constant__ KParams p) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t V = (uint32_t)p.vol;
    int32_t ioff[K], ooff[K];
    uint32_t sl[K], sr[K];          // output slot m: source lane and register
    bool valid[K];                  // slot j of the lane holds an element (input and output order alike)
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const uint32_t e = lane + 32u * (uint32_t)j;
        int32_t a, b, lin;
        uint32_t pk;
        valid[j] = e < V;
        ioff[j] = 0;
        ooff[j] = 0;
        sl[j] = 0;
        sr[j] = 0;
        if (e < V) {
            spg_walk(p.ld, e, a, b, lin, pk);
            ioff[j] = a;
            spg_walk(p.st, e, a, b, lin, pk);
            ooff[j] = a;
            sl[j] = (uint32_t)lin & 31u;
            sr[j] = (uint32_t)lin >> 5;
        }
    }
    const SpgFactor fac = p.fac;
    for (uint32_t t = warp; t < p.ntiles; t += nwarps) {
        int64_t ib, ob;
        uint32_t limA, limB;
        spg_box(p, t, ib, ob, limA, limB);
        double v[K], y[K];
#pragma unroll
        for (int j = 0; j < K; ++j) {
            v[j] = valid[j] ? spg_ld_in(in + ib + ioff[j]) : 0.0;
            y[j] = (spg_reads_out<OP>::value && valid[j]) ? spg_ld_out(out + ob + ooff[j]) : 0.0;
        }
#pragma unroll
        for (int m = 0; m < K; ++m) {
            double r = 0.0;
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const double x = __shfl_sync(0xffffffffu, v[j], (int)sl[m]);
                if (sr[m] == (uint32_t)j) r = x;
            }
            if (valid[m]) spg_st_out(out + ob + ooff[m], spg_apply<OP>(r, y[m], fac));
        }
    }
}

// Table entry emitted by the generator for every compiled variant.
struct SpgKernelEntry {
    int kind;       // SpgKind
    int op;         // SpgOp
    int threads;
    int ept;        // elements per thread (flat: vector width)
    int stages;     // tiled: 0 = register-staged, 2/3 = cp.async pipeline depth
    const void *fn;
};
