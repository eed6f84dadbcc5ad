// tma.cuh -- the TMA-staged tiled kernel (sm_90+ bulk tensor copies; built
// for sm_103a).
//
// Each box is moved global -> shared by ONE cp.async.bulk.tensor load
// described by a tensor map over the (folded) input, and shared -> global by
// ONE bulk tensor store described by a tensor map over the output.  The
// hardware clips partial boxes at the tensor edges (loads zero-fill, stores
// drop), so the kernel carries no element masks and no global address
// arithmetic.  Threads only permute inside shared memory: element e of the
// output-ordered tile takes element smr[e] of the input-ordered tile, with
// the factor arithmetic applied; for sortacc the old output box is loaded
// into the output tile by the same bulk load.
//
// Pipeline (warp-specialised): S load stages, each an input tile,
// (sortacc) an old-output tile, a "full" mbarrier (the loads landed) and an
// "empty" mbarrier (every permute warp has read it), and two output slots,
// each with a "done" mbarrier (the permute warps wrote it) and a "free"
// mbarrier (the store has read it).  One load thread keeps every stage
// busy, one store thread issues the stores and waits for them to read their
// slot, so a store never delays a refill; the permute threads never meet at a
// block barrier inside the loop.  Every wait is bounded: on timeout a thread
// records an error in the status word and leaves, and the load and store
// threads wait (bounded) for their own transfers in flight before the CTA
// retires.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include "kernels.cuh"
#include "plan.h"

#define SPG_TMA_WAIT_LIMIT (1u << 22)

__device__ __forceinline__ void spg_mbar_init(uint32_t addr, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(addr), "r"(count) : "memory");
}
__device__ __forceinline__ void spg_mbar_expect_tx(uint32_t addr, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(addr), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool spg_mbar_try_wait(uint32_t addr, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false after SPG_TMA_WAIT_LIMIT polls.
__device__ __forceinline__ bool spg_mbar_wait(uint32_t addr, uint32_t parity) {
    for (uint32_t i = 0; i < SPG_TMA_WAIT_LIMIT; ++i)
        if (spg_mbar_try_wait(addr, parity)) return true;
    return false;
}
__device__ __forceinline__ void spg_tma_load5(uint32_t dst, const void *tmap, const int32_t *c,
                                              uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];\n" ::"r"(dst),
        "l"(tmap), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(mbar)
        : "memory");
}
__device__ __forceinline__ void spg_tma_store5(const void *tmap, const int32_t *c, uint32_t src) {
    asm volatile(
        "cp.async.bulk.tensor.5d.global.shared::cta.tile.bulk_group"
        " [%0, {%2, %3, %4, %5, %6}], [%1];\n" ::"l"(tmap),
        "r"(src), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4])
        : "memory");
}
__device__ __forceinline__ void spg_bulk_commit() {
    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void spg_bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void spg_bulk_wait0() {
    asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
}
__device__ __forceinline__ void spg_fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ void spg_fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Box t -> start coordinates of the box in both tensor maps.
__host__ __device__ __forceinline__ void spg_tma_coords(const KParams &p, const TmaParams &tp,
                                                       uint32_t t, int32_t *ci, int32_t *co) {
#pragma unroll
    for (int q = 0; q < 5; ++q) { ci[q] = 0; co[q] = 0; }
#pragma unroll
    for (int k = 0; k < SPG_MAXR; ++k) {
        if (k < p.grid.n) {
            const uint32_t q = fd_div(t, p.grid.cnt[k]);
            const uint32_t c = t - q * p.grid.cnt[k].d;
            t = q;
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                if (tp.in_mdim[k] == m) ci[m] += (int32_t)c * tp.in_mul[k];
                if (tp.out_mdim[k] == m) co[m] += (int32_t)c * tp.out_mul[k];
            }
        }
    }
}

// Permute-step slot n -> the output-tile element e it writes and the
// input-tile element lin it reads.  Without skew e = n, so 16 consecutive
// slots (a half warp's 8-byte accesses) write 16 consecutive words; but when
// the input's stride-1 index lies along a slower output dim they read 16
// words one input-tile row apart, and rows of 16, 32, 64... doubles put them
// all in one bank pair (a 16-way conflict).  The skew moves the slot's
// coordinate y along one output dim (stride sk_stride in the output tile,
// box length sk_len) to (y + (lo mod 16) * sk_mul) mod sk_len, where lo =
// n mod sk_stride holds the coordinates of the faster output dims: the shift
// does not depend on y, so for each value of the other coordinates this is a
// rotation of y and the slots still cover every element exactly once.  With
// sk_stride a multiple of 16, lo mod 16 is the slot's lane in its half warp,
// and the half warp's reads step along the input's stride-1 index into
// different bank pairs (the host picks the dim and step by simulating the
// banks).
__host__ __device__ __forceinline__ void spg_tma_slot(const KParams &p, const TmaParams &tp, uint32_t n,
                                                     uint32_t &e, int32_t &lin) {
    e = n;
    if (tp.sk_mul) {
        const uint32_t lo = n % (uint32_t)tp.sk_stride;
        const int32_t y = (int32_t)((n / (uint32_t)tp.sk_stride) % (uint32_t)tp.sk_len);
        const int32_t y2 = (int32_t)((uint32_t)(y + (int32_t)(lo & 15u) * tp.sk_mul) % (uint32_t)tp.sk_len);
        e = (uint32_t)((int32_t)n + (y2 - y) * tp.sk_stride);
    }
    if (tp.same_order) {
        lin = (int32_t)e;
        return;
    }
    int32_t a, b;
    uint32_t pk;
    spg_walk(p.st, e, a, b, lin, pk);
}

// Fetch a tensor map (kernel-parameter space) into the TMA unit's cache
// ahead of its first use.
__device__ __forceinline__ void spg_prefetch_tmap(const void *tmap) {
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(tmap) : "memory");
}

__device__ __forceinline__ void spg_mbar_arrive(uint32_t addr) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(addr) : "memory");
}

// Threads in one CTA of spg_tiled_tma: NT permute threads, one load warp and
// one store warp (one active thread each).
#define SPG_TMA_BLOCK(NT) ((NT) + 64)

template <int NT, int EPT, int OP, int S>
__global__ void __launch_bounds__(SPG_TMA_BLOCK(NT), 1)
spg_tiled_tma(const __grid_constant__ CUtensorMap tmap_in,
              const __grid_constant__ CUtensorMap tmap_out,
              const __grid_constant__ KParams p, const __grid_constant__ TmaParams tp) {
    extern __shared__ __align__(1024) unsigned char smem_raw0[];
    // load stage s at s*stage_bytes (input tile, then the old-output tile
    // for sortacc at +in_bytes); output slot o at S*stage_bytes +
    // o*out_bytes; then the mbarriers: full[S], empty[S], done[2], free[2].
    // The base is rounded up to 1024 bytes (the launch adds 1 KB).
    const uint32_t raw = (uint32_t)__cvta_generic_to_shared(smem_raw0);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char *smem_raw = smem_raw0 + (base - raw);
    const uint32_t sb = (uint32_t)tp.stage_bytes;
    const uint32_t in_bytes = (uint32_t)tp.in_bytes;     // old-output tile offset
    const uint32_t ob = (uint32_t)tp.out_bytes;
    const uint32_t out0 = (uint32_t)S * sb;
    const uint32_t full0 = base + out0 + 2u * ob;        // loads of a stage landed
    const uint32_t empty0 = full0 + 8u * S;              // permute threads read a stage
    const uint32_t done0 = empty0 + 8u * S;              // permute threads wrote a slot
    const uint32_t free0 = done0 + 16u;                  // the store has read a slot
    const uint32_t tid = threadIdx.x;
    const uint32_t G = gridDim.x;
    const uint32_t load_tid = NT, store_tid = NT + 32;

    auto issue = [&](uint32_t t, int s) {
        int32_t ci[5], co[5];
        spg_tma_coords(p, tp, t, ci, co);
        const uint32_t mb = full0 + 8u * (uint32_t)s;
        spg_mbar_expect_tx(mb, (uint32_t)tp.tx_bytes);
        spg_tma_load5(base + (uint32_t)s * sb, &tmap_in, ci, mb);
        if (spg_reads_out<OP>::value) spg_tma_load5(base + (uint32_t)s * sb + in_bytes, &tmap_out, co, mb);
        (void)co;
    };
    // the load thread sets up the barriers and fills every stage before the
    // permute threads build their tables, so DRAM latency overlaps the
    // prologue
    int issued = 0;                         // load thread: boxes whose loads were issued
    if (tid == store_tid) spg_prefetch_tmap(&tmap_out);
    if (tid == load_tid) {
        spg_prefetch_tmap(&tmap_in);
        if (spg_reads_out<OP>::value) spg_prefetch_tmap(&tmap_out);
#pragma unroll
        for (int s = 0; s < S; ++s) {
            spg_mbar_init(full0 + 8u * s, 1u);
            spg_mbar_init(empty0 + 8u * s, (uint32_t)(NT / 32));
        }
#pragma unroll
        for (int o = 0; o < 2; ++o) {
            spg_mbar_init(done0 + 8u * o, (uint32_t)(NT / 32));
            spg_mbar_init(free0 + 8u * o, 1u);
        }
        spg_fence_mbar_init();
        for (int q = 0; q < S; ++q) {
            const uint32_t t = blockIdx.x + (uint32_t)q * G;
            if (t < p.ntiles) { issue(t, q); ++issued; }
        }
    }
    // permute-thread tables: slot n = tid + k*NT writes output-tile element
    // e and reads input-tile element lin (spg_tma_slot).  Without skew e = n
    // and tab[k] = lin; with skew tab[k] = e << 16 | lin (tiles hold at most
    // 2^16 elements).  Unused slots hold SPG_INVALID.
    const bool skew = tp.sk_mul != 0;
    uint32_t tab[EPT];
#pragma unroll
    for (int k = 0; k < EPT; ++k) {
        const uint32_t n = tid + k * NT;
        tab[k] = SPG_INVALID;
        if (tid < NT && n < (uint32_t)p.vol) {
            uint32_t e;
            int32_t lin;
            spg_tma_slot(p, tp, n, e, lin);
            tab[k] = skew ? (e << 16) | (uint32_t)lin : (uint32_t)lin;
        }
    }
    __syncthreads();                        // barriers initialised before anyone waits

    if (tid == load_tid) {
        // ---- loads: refill stage s with box it+S once box it has been read ----
        bool ok = true;
        int it = 0;
        for (uint32_t t = blockIdx.x + (uint32_t)S * G; t < p.ntiles; t += G, ++it) {
            const int s = it % S;
            ok = spg_mbar_wait(empty0 + 8u * (uint32_t)s, (uint32_t)((it / S) & 1));
            if (!ok) break;
            issue(t, s);
            ++issued;
        }
        if (!ok && tp.status) *(volatile int *)tp.status = 1;
        // the CTA must not retire with a load in flight: wait (bounded) for
        // the last S issued, which on the normal path have already landed
        for (int j = issued > S ? issued - S : 0; j < issued; ++j)
            spg_mbar_wait(full0 + 8u * (uint32_t)(j % S), (uint32_t)((j / S) & 1));
        return;
    }
    if (tid == store_tid) {
        // ---- stores: box it from slot it&1 once the permute threads wrote it ----
        bool ok = true;
        int it = 0;
        for (uint32_t t = blockIdx.x; t < p.ntiles; t += G, ++it) {
            const int o = it & 1;
            ok = spg_mbar_wait(done0 + 8u * (uint32_t)o, (uint32_t)((it >> 1) & 1));
            if (!ok) break;
            int32_t ci[5], co[5];
            spg_tma_coords(p, tp, t, ci, co);
            spg_tma_store5(&tmap_out, co, base + out0 + (uint32_t)o * ob);
            spg_bulk_commit();
            // slot o is free again once this store has read it
            spg_bulk_wait_read<0>();
            spg_mbar_arrive(free0 + 8u * (uint32_t)o);
        }
        if (!ok && tp.status) *(volatile int *)tp.status = 1;
        spg_bulk_wait0();                   // stores complete before the CTA retires
        return;
    }
    if (tid >= NT) return;                  // idle lanes of the load and store warps

    // ---- permute threads ----
    const SpgFactor fac = p.fac;
    const uint32_t lane = tid & 31u;
    int it = 0;
    for (uint32_t t = blockIdx.x; t < p.ntiles; t += G, ++it) {
        const int s = it % S;
        const int o = it & 1;
        // box it's loads have landed, and the store two boxes back has
        // finished reading slot o (a fresh barrier passes parity 1)
        bool ok = spg_mbar_wait(full0 + 8u * (uint32_t)s, (uint32_t)((it / S) & 1)) &&
                  spg_mbar_wait(free0 + 8u * (uint32_t)o, (uint32_t)(((it >> 1) & 1) ^ 1));
        ok = __all_sync(0xffffffffu, ok);   // a warp leaves as a whole
        if (!ok) {
            if (tp.status) *(volatile int *)tp.status = 1;
            break;
        }
        const double *tin = reinterpret_cast<const double *>(smem_raw + (size_t)s * sb);
        const double *told = reinterpret_cast<const double *>(smem_raw + (size_t)s * sb + in_bytes);
        double *tout = reinterpret_cast<double *>(smem_raw + out0 + (size_t)o * ob);
        if (skew) {
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                if (tab[k] != SPG_INVALID) {
                    const uint32_t e = tab[k] >> 16;
                    const double y = spg_reads_out<OP>::value ? told[e] : 0.0;
                    tout[e] = spg_apply<OP>(tin[tab[k] & 0xFFFFu], y, fac);
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                if (tab[k] != SPG_INVALID) {
                    const uint32_t e = tid + k * NT;
                    const double y = spg_reads_out<OP>::value ? told[e] : 0.0;
                    tout[e] = spg_apply<OP>(tin[tab[k]], y, fac);
                }
            }
        }
        spg_fence_async_smem();             // generic-proxy writes -> visible to the bulk store
        __syncwarp();
        if (lane == 0) {
            spg_mbar_arrive(empty0 + 8u * (uint32_t)s);
            spg_mbar_arrive(done0 + 8u * (uint32_t)o);
        }
    }
}
