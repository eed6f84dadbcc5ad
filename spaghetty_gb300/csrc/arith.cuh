// arith.cuh -- the IEEE round-to-nearest-even double addition in 32-bit
// integer arithmetic.
//
// GB300 issues about 1.2 FP64 additions per SM per clock, and the fused
// sortacc adds nine sources into every element of its output: it is bound
// by that pipe.  Computing part of the additions in the integer pipes,
// which are otherwise idle there, splits the load.  The algorithm is the
// textbook one of a hardware adder: order the operands by magnitude, align
// the smaller one's significand keeping a guard, a round and a sticky bit,
// add or subtract, normalise, and round to nearest even on those three
// bits.  Every step uses 32-bit words only (64-bit integer instructions
// would run on the FP64 pipe on this GPU).
//
// It covers normal operands with a normal result.  Everything else (a zero,
// subnormal, infinite or NaN operand, an exact cancellation to zero, a
// subnormal or overflowing result) reports !ok, and the caller takes the
// hardware addition, so the bits always equal __dadd_rn(a, b).  The same
// code compiles for the host, where the library's self-test compares it
// with the CPU's IEEE addition.
#pragma once
#include <stdint.h>
#include <string.h>
#include <cuda_runtime.h>

__host__ __device__ __forceinline__ uint32_t spg_fshr(uint32_t lo, uint32_t hi, uint32_t s) {
    // (hi:lo) >> s, low word, 0 <= s < 32
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, s);
#else
    return s ? (lo >> s) | (hi << (32 - s)) : lo;
#endif
}

__host__ __device__ __forceinline__ uint32_t spg_fshl(uint32_t lo, uint32_t hi, uint32_t s) {
    // (hi:lo) << s, high word, 0 <= s < 32
#ifdef __CUDA_ARCH__
    return __funnelshift_l(lo, hi, s);
#else
    return s ? (hi << s) | (lo >> (32 - s)) : hi;
#endif
}

__host__ __device__ __forceinline__ uint32_t spg_clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__clz((int)x);
#else
    return x ? (uint32_t)__builtin_clz(x) : 32u;
#endif
}

// a + b from the 32-bit halves of both operands; result halves in *rhi,
// *rlo.  Returns false (result unset) for the cases listed above.
__host__ __device__ __forceinline__ bool spg_add_words(uint32_t ahi, uint32_t alo, uint32_t bhi, uint32_t blo,
                                                       uint32_t *rhi, uint32_t *rlo) {
    uint32_t am = ahi & 0x7FFFFFFFu, bm = bhi & 0x7FFFFFFFu;
    if (am < bm || (am == bm && alo < blo)) {      // |a| >= |b| from here on
        uint32_t t = ahi; ahi = bhi; bhi = t;
        t = alo; alo = blo; blo = t;
        t = am; am = bm; bm = t;
    }
    const uint32_t ea = am >> 20, eb = bm >> 20;
    if (eb == 0u || ea == 0x7FFu) return false;   // zero, subnormal, inf, NaN
    // significands with the hidden bit, three extra low bits: 56 bits in
    // (hi: 24 bits, lo: 32 bits)
    uint32_t ah = (((am & 0xFFFFFu) | 0x100000u) << 3) | (alo >> 29), al = alo << 3;
    uint32_t bh = (((bm & 0xFFFFFu) | 0x100000u) << 3) | (blo >> 29), bl = blo << 3;
    const uint32_t d = ea - eb;
    if (d >= 56u) {
        bh = 0u;
        bl = 1u;                                   // only the sticky bit is left
    } else if (d >= 32u) {
        const uint32_t s = d - 32u;
        const uint32_t lost = bl | (bh & ((1u << s) - 1u));
        bl = (bh >> s) | (lost != 0u ? 1u : 0u);
        bh = 0u;
    } else if (d > 0u) {
        const uint32_t lost = bl & ((1u << d) - 1u);
        bl = spg_fshr(bl, bh, d) | (lost != 0u ? 1u : 0u);
        bh >>= d;
    }
    int32_t e = (int32_t)ea;
    uint32_t h, l;
    if (((ahi ^ bhi) & 0x80000000u) == 0u) {
        l = al + bl;
        h = ah + bh + (l < al ? 1u : 0u);
        if (h >> 24) {                             // carry out of bit 55
            const uint32_t st = l & 1u;
            l = spg_fshr(l, h, 1u) | st;
            h >>= 1;
            e += 1;
        }
    } else {
        l = al - bl;
        h = ah - bh - (al < bl ? 1u : 0u);
        if (h == 0u && l == 0u) return false;      // exact zero: its sign rules
        const uint32_t lz = h != 0u ? spg_clz32(h) - 8u : 24u + spg_clz32(l);
        if (lz >= 32u) {
            h = l << (lz - 32u);
            l = 0u;
        } else if (lz > 0u) {
            h = spg_fshl(l, h, lz);
            l <<= lz;
        }
        e -= (int32_t)lz;
        if (e <= 0) return false;                  // subnormal result
    }
    // round to nearest even on guard, round and sticky
    const uint32_t grs = l & 7u;
    l = spg_fshr(l, h, 3u);
    h >>= 3;
    if (grs > 4u || (grs == 4u && (l & 1u))) {
        l += 1u;
        if (l == 0u) h += 1u;
        if (h >> 21) {                             // rounded up to 2^53
            l = spg_fshr(l, h, 1u);
            h >>= 1;
            e += 1;
        }
    }
    if (e >= 0x7FF) return false;                  // overflow
    *rhi = (ahi & 0x80000000u) | ((uint32_t)e << 20) | (h & 0xFFFFFu);
    *rlo = l;
    return true;
}

#ifdef __CUDACC__
// a + b, bit-identical to __dadd_rn(a, b); the integer path for the common
// case, the FP64 pipe for the rest behind a warp vote (a real branch).
__device__ __forceinline__ double spg_dadd_int(double a, double b) {
    uint32_t rh = 0u, rl = 0u;
    const bool ok = spg_add_words((uint32_t)__double2hiint(a), (uint32_t)__double2loint(a),
                                  (uint32_t)__double2hiint(b), (uint32_t)__double2loint(b), &rh, &rl);
    double r = __hiloint2double((int)rh, (int)rl);
    if (__any_sync(__activemask(), !ok)) {
        if (!ok) r = __dadd_rn(a, b);
    }
    return r;
}
#endif

// Host form for the self-test: false where the integer path declines.
__host__ __forceinline__ bool spg_add_int_host(double a, double b, double *r) {
    uint64_t ua, ub;
    memcpy(&ua, &a, 8);
    memcpy(&ub, &b, 8);
    uint32_t rh, rl;
    if (!spg_add_words((uint32_t)(ua >> 32), (uint32_t)ua, (uint32_t)(ub >> 32), (uint32_t)ub, &rh, &rl))
        return false;
    const uint64_t ur = ((uint64_t)rh << 32) | rl;
    memcpy(r, &ur, 8);
    return true;
}
