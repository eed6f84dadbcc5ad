// contract.cu -- a TCE tensor contraction with its two operand sorts and its
// result sort fused into one kernel.
//
// The reference builds every TCE contraction as sort -> DGEMM -> sort; its
// macaroni skeleton for one CCSD term, i0(p3,p4,h1,h2) = Sum(p5,p6)
// v(p3,p4,p5,p6) * t(p5,p6,h1,h2), is
// (branches/old/python/macaroni/ccsd_t2_8_skeleton.F:174-184):
//   tce_sort_4(a_raw, a_sort, dim5,dim6,dim1,dim2, 4,3,2,1, 1.0)
//   tce_sort_4(b_raw, b_sort, dim3,dim4,dim5,dim6, 2,1,4,3, 1.0)
//   dgemm('T','N', dim1*dim2, dim3*dim4, dim5*dim6, 1.0, a_sort, dim5*dim6,
//         b_sort, dim5*dim6, 1.0, c_sort, dim1*dim2)      (c_sort zeroed)
//   tce_sort_4(c_sort, c_done, dim4,dim3,dim2,dim1, 2,1,4,3, 1.0)
// and the skeleton checks the dgemm against its own loop_dgemm, case 3
// ('T','N'; :214-292): c(i,j) = beta*c(i,j), then for k = 1..K in order
// c(i,j) = c(i,j) + alpha*a(k,i)*b(k,j).
//
// Here one kernel reads the unsorted operands through the sorts' index maps,
// keeps the GEMM tile in shared memory and registers, and writes each result
// element once, straight into its sorted (or sort-accumulated) position: the
// three sorted intermediates never exist.  Arithmetic, per output element:
//   exact mode: s = 0; for k ascending: s = s + (alpha*a)*b, every product
//               and sum rounded -- the bits of loop_dgemm case 3 on a zeroed
//               c_sort (alpha*a rounded first, as Fortran evaluates it);
//   fma mode:   the same order with a fused multiply-add per term (faster,
//               not bit-identical to the loop);
//   mma mode:   FP64 matrix instructions (spg_contract_mma below), within
//               rounding of the loop like fma mode.
// Exact mode cannot use a matrix instruction: the loop's bits need every
// product rounded, then added to the running sum in k order, while an MMA
// fuses each product into a sum of several terms.
// The result goes through the sorts' factor arithmetic: c_done = f*s (sort)
// or c_done + f*s (sortacc), exactly as tce_sort_4 / tce_sortacc_4 of c_sort.
//
// GB300 has a narrow FP64 pipe (about 1.5 operations per SM per clock): the
// kernel is bound by it, not by memory.  A 16x16 output tile per CTA keeps
// every SM busy even for the small tiles of CCSD (M = N = 256), and each
// operand element, once in shared memory, serves 16 products.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "kernels.cuh"
#include "plan.h"
#include "spaghetty_gb300.h"

#define SPG_CT_TM 16   // output tile: m
#define SPG_CT_TN 16   // output tile: n
#define SPG_CT_TK 32   // contracted indices staged per step

// Offset of a two-index group x = x0*e1 + x1 inside a raw tensor:
// x0*w0 + x1*w1.
struct SpgGroup2 {
    FastDiv e1;
    uint32_t e1v;
    int64_t w0, w1;
};

struct ContractParams {
    const double *a, *b;
    double *c;
    int32_t M, N, K;
    uint32_t ntiles;
    FastDiv mtiles;               // tiles along m
    double alpha;
    int32_t scale_a;              // alpha != 1: the loop's alpha*a(k,i)
    SpgGroup2 am, ak, bn, bk, cm, cn;
    SpgFactor fac;
};

// Host-callable too, so that spaghetty_contract_verify replays the kernel's
// own index arithmetic on the CPU.
SPG_HD int64_t spg_g2(const SpgGroup2 &g, uint32_t x) {
    const uint32_t x0 = fd_div(x, g.e1);
    return (int64_t)x0 * g.w0 + (int64_t)(x - x0 * g.e1v) * g.w1;
}

// RM x RN outputs per thread; (16/RM) x (16/RN) threads per CTA.
template <int OP, bool FMA, int RM, int RN>
__global__ void __launch_bounds__((SPG_CT_TM / RM) * (SPG_CT_TN / RN))
spg_contract(const __grid_constant__ ContractParams p) {
    constexpr int TMX = SPG_CT_TM / RM;             // threads along m
    constexpr int NT = TMX * (SPG_CT_TN / RN);
    constexpr int KROWS = NT / 16;                  // k rows one staging pass covers
    constexpr int LPT = SPG_CT_TK / KROWS;          // staged elements per thread and operand
    // two staging buffers: step s is computed from buffer s&1 while step
    // s+1's operands travel from memory into the other
    __shared__ __align__(16) double As[2][SPG_CT_TK][SPG_CT_TM];
    __shared__ __align__(16) double Bs[2][SPG_CT_TK][SPG_CT_TN];
    const uint32_t tid = threadIdx.x;
    const uint32_t tx = tid % TMX, ty = tid / TMX;
    // staging: this thread loads tile row (tid & 15) at k rows (tid >> 4) + KROWS*j
    const uint32_t lrow = tid & 15u, lk = tid >> 4;
    const SpgFactor fac = p.fac;
    for (uint32_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        const uint32_t tn = fd_div(t, p.mtiles);
        const uint32_t tm = t - tn * p.mtiles.d;
        const uint32_t m0 = tm * SPG_CT_TM, n0 = tn * SPG_CT_TN;
        const bool lm_ok = m0 + lrow < (uint32_t)p.M, ln_ok = n0 + lrow < (uint32_t)p.N;
        const int64_t offa = lm_ok ? spg_g2(p.am, m0 + lrow) : 0;
        const int64_t offb = ln_ok ? spg_g2(p.bn, n0 + lrow) : 0;
        // step k0's operands go straight from memory into buffer `buf` by
        // 8-byte cp.async copies (zero-filled outside the tensors), so no
        // registers hold them in flight
        auto fetch = [&](int32_t k0, int buf) {
#pragma unroll
            for (int j = 0; j < LPT; ++j) {
                const uint32_t kk = lk + (uint32_t)KROWS * j;
                const uint32_t k = (uint32_t)k0 + kk;
                const bool kin = k < (uint32_t)p.K;
                const bool a_ok = kin && lm_ok, b_ok = kin && ln_ok;
                spg_cp_async8((uint32_t)__cvta_generic_to_shared(&As[buf][kk][lrow]),
                              a_ok ? p.a + offa + spg_g2(p.ak, k) : p.a, a_ok ? 8u : 0u);
                spg_cp_async8((uint32_t)__cvta_generic_to_shared(&Bs[buf][kk][lrow]),
                              b_ok ? p.b + offb + spg_g2(p.bk, k) : p.b, b_ok ? 8u : 0u);
            }
            spg_cp_commit();
        };
        // the loop's alpha*a(k,i), rounded once per element: each thread
        // scales the elements it copied, after they landed
        auto scale = [&](int buf) {
            if (!p.scale_a) return;
#pragma unroll
            for (int j = 0; j < LPT; ++j) {
                double *q = &As[buf][lk + (uint32_t)KROWS * j][lrow];
                *q = __dmul_rn(p.alpha, *q);
            }
        };
        double acc[RM][RN];
#pragma unroll
        for (int i = 0; i < RM; ++i)
#pragma unroll
            for (int j = 0; j < RN; ++j) acc[i][j] = 0.0;
        __syncthreads();                    // the previous tile's last step is consumed
        fetch(0, 0);
        int buf = 0;
        for (int32_t k0 = 0; k0 < p.K; k0 += SPG_CT_TK, buf ^= 1) {
            if (k0 + SPG_CT_TK < p.K) {
                fetch(k0 + SPG_CT_TK, buf ^ 1);
                spg_cp_wait<1>();           // this thread's copies of step k0 landed
            } else {
                spg_cp_wait<0>();
            }
            scale(buf);
            __syncthreads();                // ... and everyone else's
            const int32_t kn = min(SPG_CT_TK, p.K - k0);
            // k strictly ascending: the loop's order of additions
            for (int32_t kk = 0; kk < kn; ++kk) {
                double av[RM], bv[RN];
#pragma unroll
                for (int i = 0; i < RM; ++i) av[i] = As[buf][kk][RM * tx + i];
#pragma unroll
                for (int j = 0; j < RN; ++j) bv[j] = Bs[buf][kk][RN * ty + j];
                if (FMA) {
#pragma unroll
                    for (int i = 0; i < RM; ++i)
#pragma unroll
                        for (int j = 0; j < RN; ++j) acc[i][j] = __fma_rn(av[i], bv[j], acc[i][j]);
                } else {
                    // exact mode: every product rounded, then added in k
                    // order.  The products take the integer multiply
                    // (spg_mul_int: the same bits as __dmul_rn wherever it
                    // applies), which leaves the FP64 pipe only the adds;
                    // one warp vote per k step sends a warp with any product
                    // it does not cover to the rounded multiply.
                    SpgFactor bf[RN];
#pragma unroll
                    for (int j = 0; j < RN; ++j) bf[j] = spg_mul_operand(bv[j]);
                    double pr[RM][RN];
                    bool exact = true;
#pragma unroll
                    for (int i = 0; i < RM; ++i)
#pragma unroll
                        for (int j = 0; j < RN; ++j) pr[i][j] = spg_mul_int(av[i], bf[j], exact);
                    if (!__all_sync(0xffffffffu, exact)) {
                        // out of line (spg_dmul_branch): inlined, the
                        // compiler predicates these multiplies into every
                        // step, where they occupy the FP64 pipe even when
                        // predicated off (0.85 ms against 0.49 ms at 24^6)
#pragma unroll
                        for (int i = 0; i < RM; ++i)
#pragma unroll
                            for (int j = 0; j < RN; ++j) pr[i][j] = spg_dmul_branch(av[i], bv[j]);
                    }
#pragma unroll
                    for (int i = 0; i < RM; ++i)
#pragma unroll
                        for (int j = 0; j < RN; ++j) acc[i][j] = __dadd_rn(acc[i][j], pr[i][j]);
                }
            }
            __syncthreads();                // buffer buf is refilled two steps on
        }
        // each result element written once, at its sorted position
#pragma unroll
        for (int i = 0; i < RM; ++i) {
            const uint32_t m = m0 + RM * tx + i;
            if (m >= (uint32_t)p.M) continue;
            const int64_t ocm = spg_g2(p.cm, m);
#pragma unroll
            for (int j = 0; j < RN; ++j) {
                const uint32_t n = n0 + RN * ty + j;
                if (n >= (uint32_t)p.N) continue;
                double *dst = p.c + ocm + spg_g2(p.cn, n);
                const double y = spg_reads_out<OP>::value ? *dst : 0.0;
                *dst = spg_apply<OP>(acc[i][j], y, fac);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// mma mode: the same fused sort -> GEMM -> sort with the products summed by
// FP64 matrix instructions (mma.sync m8n8k4, .f64): one instruction per warp
// multiplies an 8x4 slice of A by a 4x8 slice of B into an 8x8 accumulator.
// A CTA of four warps owns a 16x16 output tile; each staged block of 32
// contracted indices is split over the warps (warp w takes the 4-wide steps
// w, w+4, ...), every warp accumulating the whole tile (four 8x8
// sub-tiles), and the four partial tiles are added at the end.  Like fma
// mode it is within rounding of the loop, not bit-identical (the order of
// the additions differs).  Fragment layouts of m8n8k4 .f64 (PTX ISA): a0 =
// A[lane/4][lane%4], b0 = B[lane%4][lane/4], d = D[lane/4][2*(lane%4)+i].
// The staging rows are padded to 20 doubles: a half warp's fragment reads
// (4 k rows x 4 consecutive m) then fall in 16 different bank pairs.
#define SPG_CTM_NT 128
#define SPG_CTM_PITCH 20

__device__ __forceinline__ void spg_dmma(double &d0, double &d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

template <int OP>
__global__ void __launch_bounds__(SPG_CTM_NT)
spg_contract_mma(const __grid_constant__ ContractParams p) {
    constexpr int KROWS = SPG_CTM_NT / 16;          // k rows one staging pass covers
    constexpr int LPT = SPG_CT_TK / KROWS;          // staged elements per thread and operand
    __shared__ __align__(16) double As[2][SPG_CT_TK][SPG_CTM_PITCH];
    __shared__ __align__(16) double Bs[2][SPG_CT_TK][SPG_CTM_PITCH];
    __shared__ double part[4][SPG_CT_TM][SPG_CT_TN];   // per-warp partial tiles
    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u, warp = tid >> 5;
    const uint32_t g = lane >> 2, t4 = lane & 3u;
    const uint32_t lrow = tid & 15u, lk = tid >> 4;
    const SpgFactor fac = p.fac;
    for (uint32_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        const uint32_t tn = fd_div(t, p.mtiles);
        const uint32_t tm = t - tn * p.mtiles.d;
        const uint32_t m0 = tm * SPG_CT_TM, n0 = tn * SPG_CT_TN;
        const bool lm_ok = m0 + lrow < (uint32_t)p.M, ln_ok = n0 + lrow < (uint32_t)p.N;
        const int64_t offa = lm_ok ? spg_g2(p.am, m0 + lrow) : 0;
        const int64_t offb = ln_ok ? spg_g2(p.bn, n0 + lrow) : 0;
        auto fetch = [&](int32_t k0, int buf) {
#pragma unroll
            for (int j = 0; j < LPT; ++j) {
                const uint32_t kk = lk + (uint32_t)KROWS * j;
                const uint32_t k = (uint32_t)k0 + kk;
                const bool kin = k < (uint32_t)p.K;
                const bool a_ok = kin && lm_ok, b_ok = kin && ln_ok;
                spg_cp_async8((uint32_t)__cvta_generic_to_shared(&As[buf][kk][lrow]),
                              a_ok ? p.a + offa + spg_g2(p.ak, k) : p.a, a_ok ? 8u : 0u);
                spg_cp_async8((uint32_t)__cvta_generic_to_shared(&Bs[buf][kk][lrow]),
                              b_ok ? p.b + offb + spg_g2(p.bk, k) : p.b, b_ok ? 8u : 0u);
            }
            spg_cp_commit();
        };
        auto scale = [&](int buf) {
            if (!p.scale_a) return;
#pragma unroll
            for (int j = 0; j < LPT; ++j) {
                double *q = &As[buf][lk + (uint32_t)KROWS * j][lrow];
                *q = __dmul_rn(p.alpha, *q);
            }
        };
        // acc[i][j][0..1]: sub-tile (8i.., 8j..), elements (g, 2*t4 + 0..1)
        double acc[2][2][2];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
        __syncthreads();                    // the previous tile's partials are consumed
        fetch(0, 0);
        int buf = 0;
        for (int32_t k0 = 0; k0 < p.K; k0 += SPG_CT_TK, buf ^= 1) {
            if (k0 + SPG_CT_TK < p.K) {
                fetch(k0 + SPG_CT_TK, buf ^ 1);
                spg_cp_wait<1>();
            } else {
                spg_cp_wait<0>();
            }
            scale(buf);
            __syncthreads();
            // indices past K were zero-filled: whole 4-wide steps are safe
#pragma unroll
            for (int s = 0; s < SPG_CT_TK / 16; ++s) {
                const uint32_t kk = 4u * (warp + 4u * (uint32_t)s) + t4;
                const double a0 = As[buf][kk][g], a1 = As[buf][kk][8 + g];
                const double b0 = Bs[buf][kk][g], b1 = Bs[buf][kk][8 + g];
                spg_dmma(acc[0][0][0], acc[0][0][1], a0, b0);
                spg_dmma(acc[0][1][0], acc[0][1][1], a0, b1);
                spg_dmma(acc[1][0][0], acc[1][0][1], a1, b0);
                spg_dmma(acc[1][1][0], acc[1][1][1], a1, b1);
            }
            __syncthreads();                // buffer buf is refilled two steps on
        }
        // the four warps' partial tiles, added in warp order
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                part[warp][8 * i + g][8 * j + 2 * t4] = acc[i][j][0];
                part[warp][8 * i + g][8 * j + 2 * t4 + 1] = acc[i][j][1];
            }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const uint32_t idx = tid + (uint32_t)e * SPG_CTM_NT;
            const uint32_t mi = idx >> 4, ni = idx & 15u;
            const uint32_t m = m0 + mi, n = n0 + ni;
            if (m >= (uint32_t)p.M || n >= (uint32_t)p.N) continue;
            const double s = ((part[0][mi][ni] + part[1][mi][ni]) + part[2][mi][ni]) + part[3][mi][ni];
            double *dst = p.c + spg_g2(p.cm, m) + spg_g2(p.cn, n);
            const double y = spg_reads_out<OP>::value ? *dst : 0.0;
            *dst = spg_apply<OP>(s, y, fac);
        }
    }
}

namespace {

typedef void (*ContractFn)(ContractParams);

ContractFn contract_mma_kernel(int op) {
    switch (op) {
        case OP_SORT_ONE: return spg_contract_mma<OP_SORT_ONE>;
        case OP_SORT_NEG: return spg_contract_mma<OP_SORT_NEG>;
        case OP_SORT_POW2: return spg_contract_mma<OP_SORT_POW2>;
        case OP_SORT_ANY: return spg_contract_mma<OP_SORT_ANY>;
        case OP_ACC_ONE: return spg_contract_mma<OP_ACC_ONE>;
        case OP_ACC_NEG: return spg_contract_mma<OP_ACC_NEG>;
        case OP_ACC_POW2: return spg_contract_mma<OP_ACC_POW2>;
        case OP_ACC_ANY: return spg_contract_mma<OP_ACC_ANY>;
        default: return spg_contract_mma<OP_GEN>;
    }
}

template <bool FMA, int RM, int RN>
ContractFn contract_kernel(int op) {
    switch (op) {
        case OP_SORT_ONE: return spg_contract<OP_SORT_ONE, FMA, RM, RN>;
        case OP_SORT_NEG: return spg_contract<OP_SORT_NEG, FMA, RM, RN>;
        case OP_SORT_POW2: return spg_contract<OP_SORT_POW2, FMA, RM, RN>;
        case OP_SORT_ANY: return spg_contract<OP_SORT_ANY, FMA, RM, RN>;
        case OP_ACC_ONE: return spg_contract<OP_ACC_ONE, FMA, RM, RN>;
        case OP_ACC_NEG: return spg_contract<OP_ACC_NEG, FMA, RM, RN>;
        case OP_ACC_POW2: return spg_contract<OP_ACC_POW2, FMA, RM, RN>;
        case OP_ACC_ANY: return spg_contract<OP_ACC_ANY, FMA, RM, RN>;
        default: return spg_contract<OP_GEN, FMA, RM, RN>;
    }
}

// Threads per tile: GB300's FP64 units sit in the SM's four sub-partitions,
// each a warp's home, so an SM needs several warps to use them all.  The
// tile is fixed at 16 x 16 outputs; small problems (few tiles per SM) get
// more threads per tile, each with fewer outputs.
ContractFn pick_kernel(int op, bool fma, uint32_t ntiles, int sms, int *threads) {
    const uint64_t want_warps = (uint64_t)sms * 8;
    if ((uint64_t)ntiles * 2 >= want_warps) {
        *threads = 64;
        return fma ? contract_kernel<true, 2, 2>(op) : contract_kernel<false, 2, 2>(op);
    }
    if ((uint64_t)ntiles * 4 >= want_warps) {
        *threads = 128;
        return fma ? contract_kernel<true, 2, 1>(op) : contract_kernel<false, 2, 1>(op);
    }
    *threads = 256;
    return fma ? contract_kernel<true, 1, 1>(op) : contract_kernel<false, 1, 1>(op);
}

thread_local int g_contract_error = 0;

int crecord(int rc) {
    g_contract_error = rc;
    return rc;
}

SpgGroup2 group2(int64_t e1, int64_t w0, int64_t w1) {
    SpgGroup2 g;
    g.e1 = spg_make_fastdiv((uint32_t)e1);
    g.e1v = (uint32_t)e1;
    g.w0 = w0;
    g.w1 = w1;
    return g;
}

bool is_perm4(const int *p) {
    int seen = 0;
    for (int q = 0; q < 4; ++q) {
        if (p[q] < 1 || p[q] > 4 || (seen >> p[q]) & 1) return false;
        seen |= 1 << p[q];
    }
    return true;
}

// Shape checks and the six index maps; sizes in elements.
int contract_params(const int *dims_a, const int *perm_a, const int *dims_b, const int *perm_b,
                    const int *perm_c, ContractParams *P, int64_t *na, int64_t *nb, int64_t *nc) {
    if (!dims_a || !perm_a || !dims_b || !perm_b || !perm_c) return SPAGHETTY_ERR_NULL;
    if (!is_perm4(perm_a) || !is_perm4(perm_b) || !is_perm4(perm_c)) return SPAGHETTY_ERR_PERM;
    int64_t SA[4], SB[4], stA[4], stB[4];
    for (int q = 0; q < 4; ++q)
        if (dims_a[q] <= 0 || dims_b[q] <= 0) return SPAGHETTY_ERR_DIMS;
    stA[3] = stB[3] = 1;
    for (int q = 2; q >= 0; --q) {
        stA[q] = stA[q + 1] * dims_a[q + 1];
        stB[q] = stB[q + 1] * dims_b[q + 1];
    }
    for (int q = 0; q < 4; ++q) {
        SA[q] = dims_a[perm_a[q] - 1];
        SB[q] = dims_b[perm_b[q] - 1];
    }
    // the sorted operands share their two trailing (contracted) dims
    if (SA[2] != SB[2] || SA[3] != SB[3]) return SPAGHETTY_ERR_DIMS;
    const int64_t M = SA[0] * SA[1], N = SB[0] * SB[1], K = SA[2] * SA[3];
    if (M >= (int64_t(1) << 31) || N >= (int64_t(1) << 31) || K >= (int64_t(1) << 31))
        return SPAGHETTY_ERR_OVERFLOW;
    *na = M * K;
    *nb = N * K;
    *nc = M * N;
    // c_sort has dims (SB0, SB1, SA0, SA1); c_done = c_sort.permute(perm_c - 1)
    const int64_t CS[4] = {SB[0], SB[1], SA[0], SA[1]};
    int64_t CD[4], stD[4], w[4];
    for (int q = 0; q < 4; ++q) CD[q] = CS[perm_c[q] - 1];
    stD[3] = 1;
    for (int q = 2; q >= 0; --q) stD[q] = stD[q + 1] * CD[q + 1];
    for (int q = 0; q < 4; ++q) w[perm_c[q] - 1] = stD[q];
    P->M = (int32_t)M;
    P->N = (int32_t)N;
    P->K = (int32_t)K;
    P->am = group2(SA[1], stA[perm_a[0] - 1], stA[perm_a[1] - 1]);
    P->ak = group2(SA[3], stA[perm_a[2] - 1], stA[perm_a[3] - 1]);
    P->bn = group2(SB[1], stB[perm_b[0] - 1], stB[perm_b[1] - 1]);
    P->bk = group2(SB[3], stB[perm_b[2] - 1], stB[perm_b[3] - 1]);
    P->cn = group2(SB[1], w[0], w[1]);
    P->cm = group2(SA[1], w[2], w[3]);
    const uint32_t mt = (uint32_t)((M + SPG_CT_TM - 1) / SPG_CT_TM);
    const uint64_t nt = (uint64_t)mt * (uint64_t)((N + SPG_CT_TN - 1) / SPG_CT_TN);
    if (nt >= (uint64_t(1) << 31)) return SPAGHETTY_ERR_OVERFLOW;
    P->mtiles = spg_make_fastdiv(mt);
    P->ntiles = (uint32_t)nt;
    return SPAGHETTY_OK;
}

bool overlap(const void *x, int64_t nx, const void *y, int64_t ny) {
    const char *a = (const char *)x, *b = (const char *)y;
    return a < b + ny * 8 && b < a + nx * 8;
}

int launch_contract(ContractParams &P, int mode, double factor, double acc_factor, cudaStream_t st) {
    P.fac = spg_make_factor(factor, acc_factor);
    P.scale_a = P.alpha != 1.0;
    const int op = spg_choose_op(factor, acc_factor);
    int dev = 0, sms = 152, nb = 0, nt = 64;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return SPAGHETTY_ERR_CUDA; }
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 152;
    const ContractFn fn = mode == 2 ? contract_mma_kernel(op) : pick_kernel(op, mode != 0, P.ntiles, sms, &nt);
    if (mode == 2) nt = SPG_CTM_NT;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void *)fn, nt, 0) != cudaSuccess || nb < 1)
        nb = 1;
    cudaGetLastError();
    const int grid = (int)std::min<int64_t>((int64_t)sms * nb, (int64_t)P.ntiles);
    void *args[] = {(void *)&P};
    if (cudaLaunchKernel((const void *)fn, dim3(grid), dim3(nt), args, 0, st) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    return SPAGHETTY_OK;
}

// Device memory of one device (or managed memory): 1 and the device; host
// memory: 0; unknown: -1.
int where(const void *p, int *dev) {
    cudaPointerAttributes at;
    memset(&at, 0, sizeof(at));
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
        *dev = at.device;
        return 1;
    }
    return 0;
}

// Grow-only device staging for host-memory calls of the drop-in, per device.
struct CtStage {
    double *p[3] = {nullptr, nullptr, nullptr};
    size_t n[3] = {0, 0, 0};
};
std::map<int, CtStage> g_ct_stage;
std::mutex g_ct_mu;

int stage_buf(CtStage &s, int i, size_t n) {
    if (s.n[i] >= n) return SPAGHETTY_OK;
    if (s.p[i]) cudaFree(s.p[i]);
    s.p[i] = nullptr;
    s.n[i] = 0;
    if (cudaMalloc(&s.p[i], n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    s.n[i] = n;
    return SPAGHETTY_OK;
}

// Synchronous contraction on any mix of host and device memory: device
// operands are used in place, host ones go through staging buffers.
int contract_sync(const double *a, const int *dims_a, const int *perm_a, const double *b,
                  const int *dims_b, const int *perm_b, double *c, const int *perm_c, double alpha,
                  double factor, double acc_factor, int mode) {
    ContractParams P;
    memset(&P, 0, sizeof(P));
    int64_t na, nb, nc;
    int rc = contract_params(dims_a, perm_a, dims_b, perm_b, perm_c, &P, &na, &nb, &nc);
    if (rc) return rc;
    if (!a || !b || !c) return SPAGHETTY_ERR_NULL;
    if (overlap(a, na, c, nc) || overlap(b, nb, c, nc)) return SPAGHETTY_ERR_ALIAS;
    int da = -1, db = -1, dc = -1;
    const int ka = where(a, &da), kb = where(b, &db), kc = where(c, &dc);
    if (ka < 0 || kb < 0 || kc < 0) return SPAGHETTY_ERR_MEMSPACE;
    int dev = -1;
    for (int d : {ka ? da : -1, kb ? db : -1, kc ? dc : -1}) {
        if (d < 0) continue;
        if (dev >= 0 && d != dev) return SPAGHETTY_ERR_MEMSPACE;
        dev = d;
    }
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) { cudaGetLastError(); return SPAGHETTY_ERR_CUDA; }
    if (dev < 0) dev = cur;
    if (cudaSetDevice(dev) != cudaSuccess) { cudaGetLastError(); return SPAGHETTY_ERR_CUDA; }
    std::lock_guard<std::mutex> lk(g_ct_mu);
    CtStage &s = g_ct_stage[dev];
    const double *ga = a, *gb = b;
    double *gc = c;
    const bool reads_c = acc_factor != 0.0;
    cudaError_t e = cudaSuccess;
    if (!ka && !(rc = stage_buf(s, 0, (size_t)na))) {
        e = cudaMemcpy(s.p[0], a, (size_t)na * 8, cudaMemcpyHostToDevice);
        ga = s.p[0];
    }
    if (!rc && e == cudaSuccess && !kb && !(rc = stage_buf(s, 1, (size_t)nb))) {
        e = cudaMemcpy(s.p[1], b, (size_t)nb * 8, cudaMemcpyHostToDevice);
        gb = s.p[1];
    }
    if (!rc && e == cudaSuccess && !kc && !(rc = stage_buf(s, 2, (size_t)nc))) {
        if (reads_c) e = cudaMemcpy(s.p[2], c, (size_t)nc * 8, cudaMemcpyHostToDevice);
        gc = s.p[2];
    }
    if (!rc && e == cudaSuccess) {
        P.a = ga;
        P.b = gb;
        P.c = gc;
        P.alpha = alpha;
        rc = launch_contract(P, mode, factor, acc_factor, 0);
    }
    if (!rc && e == cudaSuccess) e = cudaDeviceSynchronize();
    if (!rc && e == cudaSuccess && !kc) e = cudaMemcpy(c, gc, (size_t)nc * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        cudaGetLastError();
        rc = SPAGHETTY_ERR_CUDA;
    }
    if (cur != dev) cudaSetDevice(cur);
    return rc;
}

// The skeleton's index maps (ccsd_t2_8_skeleton.F:174-184).
int t2_8(const double *a_raw, const int *size_a, const double *b_raw, const int *size_b,
         double *c_done, const int *size_c, const int *d1, const int *d2, const int *d3,
         const int *d4, const int *d5, const int *d6) {
    SpgRange range("ccsd_t2_8");
    if (!size_a || !size_b || !size_c || !d1 || !d2 || !d3 || !d4 || !d5 || !d6)
        return SPAGHETTY_ERR_NULL;
    const int dims_a[4] = {*d5, *d6, *d1, *d2}, perm_a[4] = {4, 3, 2, 1};
    const int dims_b[4] = {*d3, *d4, *d5, *d6}, perm_b[4] = {2, 1, 4, 3};
    const int perm_c[4] = {2, 1, 4, 3};
    for (int q = 0; q < 4; ++q)
        if (dims_a[q] <= 0 || dims_b[q] <= 0) return SPAGHETTY_ERR_DIMS;
    const int64_t na = (int64_t)*d1 * *d2 * *d5 * *d6, nb = (int64_t)*d3 * *d4 * *d5 * *d6,
                  nc = (int64_t)*d1 * *d2 * *d3 * *d4;
    if (*size_a < na || *size_b < nb || *size_c < nc) return SPAGHETTY_ERR_DIMS;
    return contract_sync(a_raw, dims_a, perm_a, b_raw, dims_b, perm_b, c_done, perm_c, 1.0, 1.0, 0.0, 0);
}

void t2_8_void(const double *a_raw, const int *size_a, const double *b_raw, const int *size_b,
               double *c_done, const int *size_c, const int *d1, const int *d2, const int *d3,
               const int *d4, const int *d5, const int *d6) {
    const int rc = crecord(t2_8(a_raw, size_a, b_raw, size_b, c_done, size_c, d1, d2, d3, d4, d5, d6));
    if (rc) {
        printf("something is wrong...\n");
        printf("ccsd_t2_8: %s (code %d)\n", spaghetty_error_string(rc), rc);
        fflush(stdout);
    }
}

// Replays, on the host, every address the kernel forms for one problem:
// the operand element (m, k) / (n, k) that each staging copy reads and the
// result element (m, n) that each thread writes, with the tile walk and the
// thread-to-output map of each of the three thread shapes.  Every operand
// element must be read for exactly the (m, k) it holds, inside the tensor;
// every result element written exactly once.
template <int RM, int RN>
bool verify_writes(const ContractParams &P, int64_t nc, std::vector<uint8_t> &seen) {
    constexpr int TMX = SPG_CT_TM / RM, NT = TMX * (SPG_CT_TN / RN);
    std::fill(seen.begin(), seen.end(), 0);
    for (uint32_t t = 0; t < P.ntiles; ++t) {
        const uint32_t tn = fd_div(t, P.mtiles);
        const uint32_t tm = t - tn * P.mtiles.d;
        const uint32_t m0 = tm * SPG_CT_TM, n0 = tn * SPG_CT_TN;
        for (uint32_t tid = 0; tid < (uint32_t)NT; ++tid) {
            const uint32_t tx = tid % TMX, ty = tid / TMX;
            for (int i = 0; i < RM; ++i)
                for (int j = 0; j < RN; ++j) {
                    const uint32_t m = m0 + RM * tx + i, n = n0 + RN * ty + j;
                    if (m >= (uint32_t)P.M || n >= (uint32_t)P.N) continue;
                    const int64_t o = spg_g2(P.cm, m) + spg_g2(P.cn, n);
                    if (o < 0 || o >= nc || seen[(size_t)o]++) return false;
                }
        }
    }
    for (int64_t o = 0; o < nc; ++o)
        if (seen[(size_t)o] != 1) return false;
    return true;
}

bool verify_operand(const SpgGroup2 &rows, const SpgGroup2 &ks, uint32_t R, uint32_t K, int64_t n,
                    std::vector<uint8_t> &seen) {
    seen.assign((size_t)n, 0);
    for (uint32_t r = 0; r < R; ++r)
        for (uint32_t k = 0; k < K; ++k) {
            const int64_t o = spg_g2(rows, r) + spg_g2(ks, k);
            if (o < 0 || o >= n || seen[(size_t)o]++) return false;
        }
    return true;
}

}  // namespace

extern "C" {

int spaghetty_contract_verify(const int *dims_a, const int *perm_a, const int *dims_b,
                              const int *perm_b, const int *perm_c, int64_t *stats) {
    ContractParams P;
    memset(&P, 0, sizeof(P));
    int64_t na, nb, nc;
    int rc = contract_params(dims_a, perm_a, dims_b, perm_b, perm_c, &P, &na, &nb, &nc);
    if (rc) return rc;
    if (na > (int64_t(1) << 28) || nb > (int64_t(1) << 28) || nc > (int64_t(1) << 28))
        return SPAGHETTY_ERR_TOO_LARGE;
    std::vector<uint8_t> seen;
    if (!verify_operand(P.am, P.ak, (uint32_t)P.M, (uint32_t)P.K, na, seen) ||
        !verify_operand(P.bn, P.bk, (uint32_t)P.N, (uint32_t)P.K, nb, seen))
        return SPAGHETTY_ERR_CONFIG;
    seen.assign((size_t)nc, 0);
    if (!verify_writes<2, 2>(P, nc, seen) || !verify_writes<2, 1>(P, nc, seen) ||
        !verify_writes<1, 1>(P, nc, seen))
        return SPAGHETTY_ERR_CONFIG;
    if (stats) {
        stats[0] = P.M;
        stats[1] = P.N;
        stats[2] = P.K;
        stats[3] = P.ntiles;
    }
    return SPAGHETTY_OK;
}


int spaghetty_contract_4x4(const double *a, const int *dims_a, const int *perm_a, const double *b,
                           const int *dims_b, const int *perm_b, double *c, const int *perm_c,
                           double alpha, double factor, double acc_factor, int mode, void *stream) {
    SpgRange range("spaghetty_contract_4x4");
    if (mode < 0 || mode > 2) return crecord(SPAGHETTY_ERR_CONFIG);
    ContractParams P;
    memset(&P, 0, sizeof(P));
    int64_t na, nb, nc;
    int rc = contract_params(dims_a, perm_a, dims_b, perm_b, perm_c, &P, &na, &nb, &nc);
    if (rc) return crecord(rc);
    if (!a || !b || !c) return crecord(SPAGHETTY_ERR_NULL);
    if (overlap(a, na, c, nc) || overlap(b, nb, c, nc)) return crecord(SPAGHETTY_ERR_ALIAS);
    // device (or managed) memory of one device; the work runs there
    int da = -1, db = -1, dc = -1;
    if (where(a, &da) != 1 || where(b, &db) != 1 || where(c, &dc) != 1 || da != db || db != dc)
        return crecord(SPAGHETTY_ERR_MEMSPACE);
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) cudaGetLastError();
    if (cudaSetDevice(da) != cudaSuccess) {
        cudaGetLastError();
        return crecord(SPAGHETTY_ERR_CUDA);
    }
    P.a = a;
    P.b = b;
    P.c = c;
    P.alpha = alpha;
    rc = launch_contract(P, mode, factor, acc_factor, (cudaStream_t)stream);
    if (cur >= 0 && cur != da) cudaSetDevice(cur);
    return crecord(rc);
}

int spaghetty_contract_last_error(void) { return g_contract_error; }

int ccsd_t2_8_status(const double *a_raw, const int *size_a, const double *b_raw, const int *size_b,
                     double *c_done, const int *size_c, const int *dim1, const int *dim2,
                     const int *dim3, const int *dim4, const int *dim5, const int *dim6) {
    return crecord(t2_8(a_raw, size_a, b_raw, size_b, c_done, size_c, dim1, dim2, dim3, dim4, dim5, dim6));
}

void ccsd_t2_8(const double *a_raw, const int *size_a, const double *b_raw, const int *size_b,
               double *c_done, const int *size_c, const int *dim1, const int *dim2, const int *dim3,
               const int *dim4, const int *dim5, const int *dim6) {
    t2_8_void(a_raw, size_a, b_raw, size_b, c_done, size_c, dim1, dim2, dim3, dim4, dim5, dim6);
}

void ccsd_t2_8_(const double *a_raw, const int *size_a, const double *b_raw, const int *size_b,
                double *c_done, const int *size_c, const int *dim1, const int *dim2, const int *dim3,
                const int *dim4, const int *dim5, const int *dim6) {
    t2_8_void(a_raw, size_a, b_raw, size_b, c_done, size_c, dim1, dim2, dim3, dim4, dim5, dim6);
}

}  // extern "C"
