// fused.cu -- several sortaccs into one output, with ONE read and ONE write
// of the output.
//
// The CCSD(T) triples code applies nine tce_sortacc_6 calls, with different
// permutations and sources, to every t3 tile (the 27 permutations of
// branches/spaghetty2/ccsd_t_tce_sort_list.txt, three groups of nine).  Run
// one by one, each call reads and writes the whole t3 tile: 9 x 24 bytes per
// element.  Fused, t3 is read once and written once and each source is read
// once: 16 + 8*S bytes per element.
//
// Per element the sum is formed in the call order, t = ((t3 + f0*x0) + f1*x1)
// + ..., each product and each sum rounded exactly as the sequential calls
// round them, so the result is bit-identical.
//
// Two kernels.  spg_fused_tma (below, first choice): a warp-specialised
// TMA pipeline over three-dim output boxes, every source tile loaded by one
// bulk tensor copy.  spg_fused_sortacc (shapes the bulk copies cannot
// take): a persistent CTA walks boxes of the OUTPUT index space (box
// lengths divide the extents, so no element masks).  For each box it loads
// its t3 elements into registers (output order), then for every source in
// turn stages that source's elements through shared memory -- loaded in the
// source's own memory order (coalesced), placed at their output-order slot
// -- and adds them.  Sources are double-buffered with cp.async: source k+1
// is in flight while source k is added.  Each source's box walk (offset and
// slot of every element) is a shared-memory table built once per CTA.
#include "../../include/spaghetty_gb300.h"
#include "kernels.cuh"
#include "plan.h"
#include "tma.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#define SPG_FUSED_MAXS 16
#define SPG_FUSED_MAXR 6
#define SPG_FUSED_NT 256
#define SPG_FUSED_EPT 4
#define SPG_FUSED_VMAX (SPG_FUSED_NT * SPG_FUSED_EPT)

struct FusedParams {
    int32_t nsrc, vol, pad, tile;          // tile = staging slots per buffer
    uint32_t ntiles;
    // output-order box walk (fastest first)
    int32_t no;
    FastDiv olen[SPG_FUSED_MAXR];
    int32_t ostr[SPG_FUSED_MAXR];          // global output stride (box-local offsets < 2^31)
    // per source: box walk in the source's memory order (fastest first)
    int32_t ns[SPG_FUSED_MAXS];
    FastDiv slen[SPG_FUSED_MAXS][SPG_FUSED_MAXR];
    int32_t sstr[SPG_FUSED_MAXS][SPG_FUSED_MAXR];   // global source stride
    int32_t scan[SPG_FUSED_MAXS][SPG_FUSED_MAXR];   // output-order (canonical) stride in the box
    // grid of boxes (fastest first)
    int32_t ng;
    FastDiv gcnt[SPG_FUSED_MAXR];
    int64_t gout[SPG_FUSED_MAXR];
    int64_t gsrc[SPG_FUSED_MAXS][SPG_FUSED_MAXR];
    const double *src[SPG_FUSED_MAXS];
    SpgFactor fac[SPG_FUSED_MAXS];
    int32_t op[SPG_FUSED_MAXS];            // OP_ACC_* per source (OP_SORT_* for source 0 when first_sets)
    int32_t first_sets;                    // 1: source 0's product starts the sum, the output is not read
};

template <int OPA>
__device__ __forceinline__ double spg_fused_add(double acc, double x, const SpgFactor &F) {
    return spg_apply<OPA>(x, acc, F);
}

__device__ __forceinline__ double spg_fused_apply(int op, double acc, double x, const SpgFactor &F) {
    switch (op) {
        // the first term of a fused sort (first_sets): the rounded product
        // alone, as tce_sort computes it
        case OP_SORT_ONE: return spg_apply<OP_SORT_ONE>(x, 0.0, F);
        case OP_SORT_NEG: return spg_apply<OP_SORT_NEG>(x, 0.0, F);
        case OP_SORT_POW2: return spg_apply<OP_SORT_POW2>(x, 0.0, F);
        case OP_SORT_ANY: return spg_apply<OP_SORT_ANY>(x, 0.0, F);
        case OP_ACC_ONE: return spg_fused_add<OP_ACC_ONE>(acc, x, F);
        case OP_ACC_NEG: return __dsub_rn(acc, x);   // acc + x*(-1): one rounding
        case OP_ACC_POW2: return spg_fused_add<OP_ACC_POW2>(acc, x, F);
        default: return spg_fused_add<OP_ACC_ANY>(acc, x, F);
    }
}

__global__ void __launch_bounds__(SPG_FUSED_NT, 1)
spg_fused_sortacc(double *__restrict__ out, const __grid_constant__ FusedParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    // layout: int32 off[nsrc][vol] | uint16 slot[nsrc][vol] | double buf[2][tile]
    int32_t *toff = reinterpret_cast<int32_t *>(smem);
    uint16_t *tslot = reinterpret_cast<uint16_t *>(smem + (size_t)p.nsrc * p.vol * 4);
    size_t boff = (size_t)p.nsrc * p.vol * 6;
    boff = (boff + 15) & ~(size_t)15;
    double *buf = reinterpret_cast<double *>(smem + boff);
    const uint32_t bufsh = (uint32_t)__cvta_generic_to_shared(buf);
    const uint32_t tid = threadIdx.x;

    // source tables (once per CTA)
    for (int k = 0; k < p.nsrc; ++k) {
        for (uint32_t j = tid; j < (uint32_t)p.vol; j += SPG_FUSED_NT) {
            uint32_t rem = j;
            int32_t off = 0, can = 0;
            for (int d = 0; d < SPG_FUSED_MAXR; ++d) {
                if (d < p.ns[k]) {
                    const uint32_t q = fd_div(rem, p.slen[k][d]);
                    const uint32_t c = rem - q * p.slen[k][d].d;
                    rem = q;
                    off += (int32_t)c * p.sstr[k][d];
                    can += (int32_t)c * p.scan[k][d];
                }
            }
            toff[k * p.vol + j] = off;
            tslot[k * p.vol + j] = (uint16_t)(can + (p.pad ? can / p.pad : 0));
        }
    }
    // this thread's output elements: canonical e = tid + m*NT
    int32_t ooff[SPG_FUSED_EPT], oslot[SPG_FUSED_EPT];
#pragma unroll
    for (int m = 0; m < SPG_FUSED_EPT; ++m) {
        const uint32_t e = tid + m * SPG_FUSED_NT;
        ooff[m] = -1;
        oslot[m] = 0;
        if (e < (uint32_t)p.vol) {
            uint32_t rem = e;
            int32_t off = 0;
            for (int d = 0; d < SPG_FUSED_MAXR; ++d) {
                if (d < p.no) {
                    const uint32_t q = fd_div(rem, p.olen[d]);
                    const uint32_t c = rem - q * p.olen[d].d;
                    rem = q;
                    off += (int32_t)c * p.ostr[d];
                }
            }
            ooff[m] = off;
            oslot[m] = (int32_t)e + (p.pad ? (int32_t)e / p.pad : 0);
        }
    }
    __syncthreads();

    for (uint32_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        // box t: output base and the bases of every source
        uint32_t c[SPG_FUSED_MAXR];
        {
            uint32_t rem = t;
            for (int d = 0; d < SPG_FUSED_MAXR; ++d) {
                c[d] = 0;
                if (d < p.ng) {
                    const uint32_t q = fd_div(rem, p.gcnt[d]);
                    c[d] = rem - q * p.gcnt[d].d;
                    rem = q;
                }
            }
        }
        int64_t obase = 0;
        for (int d = 0; d < p.ng; ++d) obase += (int64_t)c[d] * p.gout[d];

        auto issue = [&](int k, int b) {
            int64_t sbase = 0;
            for (int d = 0; d < p.ng; ++d) sbase += (int64_t)c[d] * p.gsrc[k][d];
            const double *src = p.src[k] + sbase;
            const uint32_t dst = bufsh + (uint32_t)(b * p.tile) * 8u;
            for (uint32_t j = tid; j < (uint32_t)p.vol; j += SPG_FUSED_NT)
                spg_cp_async8(dst + (uint32_t)tslot[k * p.vol + j] * 8u, src + toff[k * p.vol + j], 8u);
            spg_cp_commit();
        };

        issue(0, 0);
        double acc[SPG_FUSED_EPT];
#pragma unroll
        for (int m = 0; m < SPG_FUSED_EPT; ++m)
            acc[m] = (ooff[m] >= 0 && !p.first_sets) ? spg_ld_out(out + obase + ooff[m]) : 0.0;
        for (int k = 0; k < p.nsrc; ++k) {
            if (k + 1 < p.nsrc) issue(k + 1, (k + 1) & 1);
            else spg_cp_commit();
            spg_cp_wait<1>();                   // source k has landed (this thread's copies)
            __syncthreads();                    // ... everyone's
            const double *tb = buf + (size_t)(k & 1) * p.tile;
            const SpgFactor F = p.fac[k];
            const int op = p.op[k];
#pragma unroll
            for (int m = 0; m < SPG_FUSED_EPT; ++m)
                if (ooff[m] >= 0) acc[m] = spg_fused_apply(op, acc[m], tb[oslot[m]], F);
            __syncthreads();                    // buffer k&1 free for source k+2
        }
#pragma unroll
        for (int m = 0; m < SPG_FUSED_EPT; ++m)
            if (ooff[m] >= 0) spg_st_out(out + obase + ooff[m], acc[m]);
    }
    spg_cp_wait<0>();
}

// ===========================================================================
// TMA-staged form of one pass.  The box spans three output dims: the one
// the pass's sources hold stride-1 (p, 16 elements), the output's stride-1
// dim (q, lq elements) and one more (r, lr elements); every other dim has
// box length 1.  Every source tile then has the layout [p fastest (16
// doubles = one 128-byte row), then q and r in the source's order], so two
// precomputed indices per element (q before r, or r before q) serve every
// source; the tiles are loaded with the 128-byte swizzle, which spreads the
// row-strided reads of a warp over the banks.  The old output tile and the
// result are in output order, [q fastest, then p and r].
//
// Warp-specialised like spg_tiled_tma: a load thread streams the items of
// each box (old output tile, then source 0..nsrc-1) through a ring of S
// slots ("full" / "empty" mbarriers); NT permute threads add the items in
// order into registers and write the result to one of two output slots
// ("done" / "free"); a store thread stores it.  Every wait is bounded.
#define SPG_FT_MAXS 16
#define SPG_FT_BLOCK(NT) ((NT) + 64)

struct FusedTmaParams {
    uint32_t ntiles;
    int32_t ng;                                    // grid dims, fastest first
    FastDiv gcnt[SPG_FUSED_MAXR];
    int8_t mdim[SPG_FT_MAXS + 1][SPG_FUSED_MAXR];  // per map (0 = output) and grid dim
    int32_t mul[SPG_FT_MAXS + 1][SPG_FUSED_MAXR];  // map coordinate step per box
    int32_t nsrc, vol, lq, lr, lp;                 // output box: lp along p, lq along q, lr along r
    int32_t pw;                                    // source tile row: pw doubles along p
    int32_t swz;                                   // 1: 128-byte swizzled source rows (pw == 16)
    int32_t out_r_first;                           // output order lists r before p
    int32_t src_r_first[SPG_FT_MAXS];              // source k lists r before q
    uint32_t tile_bytes;                           // one slot, 1024-aligned
    uint32_t tx_out, tx_src;                       // bytes one load delivers
    SpgFactor fac[SPG_FT_MAXS];
    int32_t op[SPG_FT_MAXS];
    int32_t first_sets;                            // 1: no old-output item; source 0 starts the sum
    int *status;
};

struct FusedTmaMaps {
    CUtensorMap m[SPG_FT_MAXS + 1];                // 0 = output, 1.. = sources
};

__device__ __forceinline__ void spg_ft_coords(const FusedTmaParams &p, int map, uint32_t t, int32_t *c) {
#pragma unroll
    for (int m = 0; m < 5; ++m) c[m] = 0;
#pragma unroll
    for (int k = 0; k < SPG_FUSED_MAXR; ++k) {
        if (k < p.ng) {
            const uint32_t q = fd_div(t, p.gcnt[k]);
            const uint32_t x = t - q * p.gcnt[k].d;
            t = q;
#pragma unroll
            for (int m = 0; m < 5; ++m)
                if (p.mdim[map][k] == m) c[m] += (int32_t)x * p.mul[map][k];
        }
    }
}

template <int NT, int EPT, int S>
__global__ void __launch_bounds__(SPG_FT_BLOCK(NT), 1)
spg_fused_tma(const __grid_constant__ FusedTmaMaps maps, const __grid_constant__ FusedTmaParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw0[];
    const uint32_t raw = (uint32_t)__cvta_generic_to_shared(smem_raw0);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char *smem = smem_raw0 + (base - raw);
    const uint32_t tb = p.tile_bytes;
    const uint32_t out0 = (uint32_t)S * tb;
    const uint32_t full0 = base + out0 + 2u * tb;
    const uint32_t empty0 = full0 + 8u * S;
    const uint32_t done0 = empty0 + 8u * S;
    const uint32_t free0 = done0 + 16u;
    const uint32_t tid = threadIdx.x;
    const uint32_t G = gridDim.x;
    // items per box: the old output tile (unless first_sets), then the sources
    const int lead = p.first_sets ? 0 : 1;
    const int items = p.nsrc + lead;
    const uint32_t load_tid = NT, store_tid = NT + 32;

    if (tid == load_tid) {
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
    }
    // permute threads: output-order element e = tid + m*NT of the box is
    // (xq, xp) = (e % lq, e / lq); its byte offset in a (swizzled) source
    // tile is ((xp + 16*xq) * 8) with the 16-byte chunk index XOR row % 8
    uint32_t soff[EPT], soff_r[EPT];       // q-before-r and r-before-q sources
#pragma unroll
    for (int m = 0; m < EPT; ++m) {
        const uint32_t e = tid + (uint32_t)m * NT;
        soff[m] = 0xFFFFFFFFu;
        soff_r[m] = 0xFFFFFFFFu;
        if (tid < NT && e < (uint32_t)p.vol) {
            const uint32_t lq = (uint32_t)p.lq, lr = (uint32_t)p.lr, lp = (uint32_t)p.lp;
            const uint32_t pw = (uint32_t)p.pw;
            const uint32_t xq = e % lq, rest = e / lq;
            const uint32_t xp = p.out_r_first ? rest / lr : rest % lp;
            const uint32_t xr = p.out_r_first ? rest % lr : rest / lp;
            const uint32_t row_a = xq + lq * xr, row_b = xr + lr * xq;   // source tile rows
            soff[m] = (xp + pw * row_a) * 8u;
            soff_r[m] = (xp + pw * row_b) * 8u;
            if (p.swz) {                    // 16-byte chunk index XOR row % 8
                soff[m] ^= (row_a & 7u) << 4;
                soff_r[m] ^= (row_b & 7u) << 4;
            }
        }
    }
    __syncthreads();                        // barriers initialised before anyone waits

    if (tid == load_tid) {
        // ---- loads: item i of box it goes to slot j % S, j = it*items + i ----
        bool ok = true;
        int64_t j = 0;
        int it = 0;
        for (uint32_t t = blockIdx.x; t < p.ntiles && ok; t += G, ++it) {
            for (int i = 0; i < items; ++i, ++j) {
                const int s = (int)(j % S);
                if (j >= S) {
                    ok = spg_mbar_wait(empty0 + 8u * (uint32_t)s, (uint32_t)(((j / S) - 1) & 1));
                    if (!ok) break;
                }
                const int map = i + 1 - lead;       // 0 = output, 1.. = sources
                int32_t c[5];
                spg_ft_coords(p, map, t, c);
                const uint32_t mb = full0 + 8u * (uint32_t)s;
                spg_mbar_expect_tx(mb, map == 0 ? p.tx_out : p.tx_src);
                spg_tma_load5(base + (uint32_t)s * tb, &maps.m[map], c, mb);
            }
        }
        if (!ok && p.status) *(volatile int *)p.status = 1;
        // the CTA must not retire with a load in flight
        for (int64_t q = j > S ? j - S : 0; q < j; ++q)
            spg_mbar_wait(full0 + 8u * (uint32_t)(q % S), (uint32_t)((q / S) & 1));
        return;
    }
    if (tid == store_tid) {
        bool ok = true;
        int it = 0;
        for (uint32_t t = blockIdx.x; t < p.ntiles; t += G, ++it) {
            const int o = it & 1;
            ok = spg_mbar_wait(done0 + 8u * (uint32_t)o, (uint32_t)((it >> 1) & 1));
            if (!ok) break;
            int32_t c[5];
            spg_ft_coords(p, 0, t, c);
            spg_tma_store5(&maps.m[0], c, base + out0 + (uint32_t)o * tb);
            spg_bulk_commit();
            spg_bulk_wait_read<0>();
            spg_mbar_arrive(free0 + 8u * (uint32_t)o);
        }
        if (!ok && p.status) *(volatile int *)p.status = 1;
        spg_bulk_wait0();
        return;
    }
    if (tid >= NT) return;

    // ---- permute threads ----
    const uint32_t lane = tid & 31u;
    int64_t j = 0;
    int it = 0;
    bool ok = true;
    for (uint32_t t = blockIdx.x; t < p.ntiles && ok; t += G, ++it) {
        double acc[EPT];
#pragma unroll
        for (int m = 0; m < EPT; ++m) acc[m] = 0.0;
        for (int i = 0; i < items; ++i, ++j) {
            const int s = (int)(j % S);
            ok = __all_sync(0xffffffffu, spg_mbar_wait(full0 + 8u * (uint32_t)s, (uint32_t)((j / S) & 1)));
            if (!ok) break;
            const unsigned char *slot = smem + (size_t)s * tb;
            if (i < lead) {
                const double *told = reinterpret_cast<const double *>(slot);
#pragma unroll
                for (int m = 0; m < EPT; ++m) {
                    acc[m] = 0.0;
                    if (soff[m] == 0xFFFFFFFFu) break;   // the rest of this thread's slots are empty
                    acc[m] = told[tid + (uint32_t)m * NT];
                }
            } else {
                const int k = i - lead;
                const SpgFactor F = p.fac[k];
                const int op = p.op[k];
                const bool rf = p.src_r_first[k] != 0;
#pragma unroll
                for (int m = 0; m < EPT; ++m) {
                    if (soff[m] == 0xFFFFFFFFu) break;
                    acc[m] = spg_fused_apply(op, acc[m],
                                             *reinterpret_cast<const double *>(slot + (rf ? soff_r[m] : soff[m])), F);
                }
            }
            __syncwarp();
            if (lane == 0) spg_mbar_arrive(empty0 + 8u * (uint32_t)s);
        }
        if (!ok) break;
        const int o = it & 1;
        ok = __all_sync(0xffffffffu, spg_mbar_wait(free0 + 8u * (uint32_t)o, (uint32_t)(((it >> 1) & 1) ^ 1)));
        if (!ok) break;
        double *tout = reinterpret_cast<double *>(smem + out0 + (size_t)o * tb);
#pragma unroll
        for (int m = 0; m < EPT; ++m) {
            if (soff[m] == 0xFFFFFFFFu) break;
            tout[tid + (uint32_t)m * NT] = acc[m];
        }
        spg_fence_async_smem();
        __syncwarp();
        if (lane == 0) spg_mbar_arrive(done0 + 8u * (uint32_t)o);
    }
    if (!ok && p.status) *(volatile int *)p.status = 1;
}

// Four load slots of 8 KB (about 48 KB per CTA, four CTAs per SM):
// measured on GB300 on the triples groups at 16^6, 0.343-0.387 ms against
// 0.394-0.456 ms with eight slots (two CTAs per SM); two or three slots,
// 512 x 2 and 128 x 8 threads x elements were slower.  A t3 element's adds
// form one dependent chain of rounded FP64 adds, so more resident warps
// hide more of the FP64 pipe's latency.
#define SPG_FT_NT 256
#define SPG_FT_EPT 4
#define SPG_FT_S 4

// ===========================================================================
namespace {

// Grow box lengths over the output dims (divisors of the extents) until the
// output and every source read contiguous runs of >= 16 doubles where the
// extents allow, with at most SPG_FUSED_VMAX elements per box.
void fused_box(int R, const int64_t *O, int nl, const int (*order)[SPG_FUSED_MAXR], int64_t *L) {
    for (int q = 0; q < R; ++q) L[q] = 1;
    const int64_t T = 16;
    auto run = [&](int l) {
        int64_t r = 1;
        for (int i = 0; i < R; ++i) {
            const int q = order[l][i];
            r *= L[q];
            if (L[q] < O[q]) break;
        }
        return r;
    };
    auto frontier = [&](int l) {
        for (int i = 0; i < R; ++i)
            if (L[order[l][i]] < O[order[l][i]]) return order[l][i];
        return -1;
    };
    auto vol = [&]() {
        int64_t v = 1;
        for (int q = 0; q < R; ++q) v *= L[q];
        return v;
    };
    bool stuck[SPG_FUSED_MAXS + 1] = {false};
    for (int it = 0; it < 64; ++it) {
        int best = -1;
        int64_t br = 0;
        for (int l = 0; l < nl; ++l) {
            if (stuck[l]) continue;
            const int64_t r = run(l);
            if (r >= T || frontier(l) < 0) continue;
            if (best < 0 || r < br) { best = l; br = r; }
        }
        if (best < 0) break;
        const int q = frontier(best);
        const int64_t need = (T * L[q] + br - 1) / br;
        int64_t nl_len = O[q];
        for (int64_t x = L[q] + 1; x <= O[q]; ++x)
            if (O[q] % x == 0 && x >= need) { nl_len = x; break; }
        // respect the volume cap: the largest divisor that fits
        const int64_t v = vol() / L[q];
        while (nl_len > L[q] && v * nl_len > SPG_FUSED_VMAX) {
            int64_t x = nl_len - 1;
            while (x > L[q] && O[q] % x) --x;
            nl_len = x;
        }
        if (nl_len <= L[q]) { stuck[best] = true; continue; }
        L[q] = nl_len;
    }
    // grow towards half the cap along the output frontier for fewer boxes
    for (int it = 0; it < 16 && vol() * 2 <= SPG_FUSED_VMAX; ++it) {
        const int q = frontier(0);
        if (q < 0) break;
        int64_t x = L[q] + 1;
        while (x <= O[q] && O[q] % x) ++x;
        if (x > O[q] || vol() / L[q] * x > SPG_FUSED_VMAX) break;
        L[q] = x;
    }
}

}  // namespace

// One tensor map for the TMA-staged pass: dims in memory order (fastest
// first: index into the kept output dims), their extents, element strides
// and box lengths.  Consecutive dims merge into one map dim when they
// continue its memory range and the map dim so far is covered in full or
// has box length 1 (never into map dim 0 when `lone_inner`, which the
// swizzled source tiles need).  Fills per-kept-dim map dim and coordinate
// weight; returns false when the bulk copy's rules are not met.
static bool ft_map(int R, const int *order, const int64_t *ext, const int64_t *str, const int64_t *L,
                   bool lone_inner, uint64_t *dim, uint64_t *stride, uint32_t *box, int8_t *mdim,
                   int64_t *weight) {
    int m = -1;
    bool full = false, unit = false;
    for (int q = 0; q < R; ++q) {
        const int d = order[q];
        bool merge = m >= 0 && !(lone_inner && m == 0) && (uint64_t)str[d] * 8u == stride[m] * dim[m] &&
                     (full || (unit && L[d] == 1));
        if (merge) {
            weight[d] = (int64_t)dim[m];
            dim[m] *= (uint64_t)ext[d];
            box[m] = (uint32_t)((int64_t)box[m] * L[d]);
            full = full && L[d] == ext[d];
            unit = unit && L[d] == 1;
        } else {
            if (++m >= 5) return false;
            dim[m] = (uint64_t)ext[d];
            box[m] = (uint32_t)L[d];
            stride[m] = (uint64_t)str[d] * 8u;
            weight[d] = 1;
            full = L[d] == ext[d];
            unit = L[d] == 1;
        }
        mdim[d] = (int8_t)m;
    }
    const int n = m + 1;
    for (int k = 0; k < n; ++k) {
        if (box[k] < 1 || box[k] > 256 || dim[k] > ((uint64_t)1 << 31)) return false;
        if (k > 0 && (stride[k] % 16 != 0 || stride[k] >= ((uint64_t)1 << 40))) return false;
    }
    if (stride[0] != 8 || (box[0] * 8u) % 16u != 0) return false;
    for (int k = n; k < 5; ++k) {
        dim[k] = 1;
        box[k] = 1;
        stride[k] = stride[k - 1] * dim[k - 1];
        if (stride[k] >= ((uint64_t)1 << 40)) return false;
    }
    return true;
}

static int fused_tma_try(int R, const int64_t *O, const int64_t *ostr, int64_t (*sstr)[SPG_FUSED_MAXR],
                         int nsrc, const double *const *unsorted, const double *factors, double *sorted,
                         void *stream, int p, int q, int r, const int64_t *L, int64_t pw,
                         FusedTmaParams *PP, FusedTmaMaps *MM, bool launch, bool first_sets);
static int fused_tma_mode(int R, const int64_t *O, const int64_t *ostr, int64_t (*sstr)[SPG_FUSED_MAXR],
                          int nsrc, const double *const *unsorted, const double *factors, double *sorted,
                          void *stream, int p, int q, int64_t lq, int64_t lp, int64_t pw, bool first_sets);

// The TMA-staged pass, or SPAGHETTY_ERR_NOKERNEL when the shapes or the
// buffers do not allow it (the caller then runs the cp.async kernel).
// O, ostr: kept output dims (output order) and their element strides;
// sstr[k]: each kept dim's element stride in source k.
static int fused_tma_pass(int R, const int64_t *O, const int64_t *ostr, int64_t (*sstr)[SPG_FUSED_MAXR],
                          int nsrc, const double *const *unsorted, const double *factors, double *sorted,
                          void *stream, bool first_sets) {
    if (R < 2 || nsrc < 1 || nsrc > SPG_FT_MAXS) return SPAGHETTY_ERR_NOKERNEL;
    if (((uintptr_t)sorted & 15u) != 0) return SPAGHETTY_ERR_NOKERNEL;
    for (int k = 0; k < nsrc; ++k)
        if (((uintptr_t)unsorted[k] & 15u) != 0) return SPAGHETTY_ERR_NOKERNEL;
    const int q = R - 1;                    // output stride-1 dim
    int p = -1;                             // the sources' stride-1 dim
    for (int i = 0; i < R && p < 0; ++i) {
        bool all = true;
        for (int k = 0; k < nsrc; ++k) all = all && sstr[k][i] == 1;
        if (all) p = i;
    }
    if (p < 0 || p == q || O[p] < 16 || O[q] < 8) return SPAGHETTY_ERR_NOKERNEL;
    int64_t lq = std::min<int64_t>(O[q], 64);
    lq &= ~(int64_t)1;
    // source tiles: rows of 16 doubles along p with the 128-byte swizzle,
    // or the whole of a short p in one row of pw doubles, pw the smallest
    // even width >= O[p] with pw/2 odd (rows of an odd number of 16-byte
    // chunks spread a warp's row-strided reads over the banks; the columns
    // past O[p] are out of the tensor, zero-filled, never read from memory)
    // extents that 16 divides keep whole swizzled rows; other short ones
    // are loaded whole into padded rows
    for (int mode = (O[p] <= 64 && O[p] % 16 != 0) ? 0 : 1; mode < 2; ++mode) {
        int64_t lp = 16, pw = 16;
        if (mode == 0) {
            lp = O[p];
            pw = (O[p] + 1) & ~(int64_t)1;
            if ((pw / 2) % 2 == 0) pw += 2;
        }
        const int rc = fused_tma_mode(R, O, ostr, sstr, nsrc, unsorted, factors, sorted, stream, p, q, lq,
                                      lp, pw, first_sets);
        if (rc != SPAGHETTY_ERR_NOKERNEL) return rc;
    }
    return SPAGHETTY_ERR_NOKERNEL;
}

// The TMA-staged pass with source rows of pw doubles along p (lp of them
// in the output box): the third box dim r that gives the largest box whose
// maps fit, then the launch.
static int fused_tma_mode(int R, const int64_t *O, const int64_t *ostr, int64_t (*sstr)[SPG_FUSED_MAXR],
                          int nsrc, const double *const *unsorted, const double *factors, double *sorted,
                          void *stream, int p, int q, int64_t lq, int64_t lp, int64_t pw, bool first_sets) {
    static thread_local FusedTmaParams P;
    static thread_local FusedTmaMaps M;
    // the third box dim r: the one giving the largest box whose maps stay
    // within five dims; its length fills the CTA's elements
    const int64_t cap = SPG_FT_NT * SPG_FT_EPT;
    int best_r = -2;
    int64_t best_vol = 0, bestL[SPG_FUSED_MAXR];
    for (int r = -1; r < R; ++r) {          // -1: a two-dim box
        if (r == p || r == q) continue;
        int64_t L[SPG_FUSED_MAXR];
        for (int i = 0; i < R; ++i) L[i] = 1;
        L[p] = lp;
        L[q] = lq;
        if (r >= 0) {
            L[r] = std::min<int64_t>(O[r], cap / (std::max(lp, pw) * lq));
            if (L[r] < 2) continue;
        }
        const int64_t vol = lp * lq * (r >= 0 ? L[r] : 1);
        if (vol <= best_vol) continue;
        if (fused_tma_try(R, O, ostr, sstr, nsrc, unsorted, factors, sorted, stream, p, q, r < 0 ? p : r, L,
                          pw, &P, &M, false, first_sets) != SPAGHETTY_OK)
            continue;
        best_r = r;
        best_vol = vol;
        std::memcpy(bestL, L, sizeof(L));
    }
    if (best_r == -2) return SPAGHETTY_ERR_NOKERNEL;
    return fused_tma_try(R, O, ostr, sstr, nsrc, unsorted, factors, sorted, stream, p, q,
                         best_r < 0 ? p : best_r, bestL, pw, &P, &M, true, first_sets);
}

// One attempt at the TMA-staged pass with box L (16 along p, lq along q,
// lr along r; r == p for a two-dim box).
static int fused_tma_try(int R, const int64_t *O, const int64_t *ostr, int64_t (*sstr)[SPG_FUSED_MAXR],
                         int nsrc, const double *const *unsorted, const double *factors, double *sorted,
                         void *stream, int p, int q, int r, const int64_t *L, int64_t pw,
                         FusedTmaParams *PP, FusedTmaMaps *MM, bool launch, bool first_sets) {
    FusedTmaParams &P = *PP;
    FusedTmaMaps &M = *MM;
    const int64_t lq = L[q], lr = r == p ? 1 : L[r], lp = L[p];
    const int64_t vol = lp * lq * lr, vol_src = pw * lq * lr;
    const bool swz = pw == 16 && lp == 16;
    if (vol > SPG_FT_NT * SPG_FT_EPT || pw < lp || pw > 256) return SPAGHETTY_ERR_NOKERNEL;
    // the source maps' box: pw along p (the rest as the output's)
    int64_t Ls[SPG_FUSED_MAXR];
    for (int i = 0; i < R; ++i) Ls[i] = L[i];
    Ls[p] = pw;
    std::memset(&P, 0, sizeof(P));
    // grid: kept dims with more than one box, output order fastest first
    int gd[SPG_FUSED_MAXR];
    int ng = 0;
    int64_t ntiles = 1;
    for (int i = R - 1; i >= 0; --i) {
        const int64_t c = (O[i] + L[i] - 1) / L[i];
        if (c <= 1) continue;
        gd[ng] = i;
        P.gcnt[ng] = spg_make_fastdiv((uint32_t)c);
        ++ng;
        ntiles *= c;
        if (ntiles > INT32_MAX) return SPAGHETTY_ERR_NOKERNEL;
    }
    P.ng = ng;
    P.ntiles = (uint32_t)ntiles;
    // maps: 0 = output (output order), 1.. = sources (their memory order)
    for (int mi = 0; mi <= nsrc; ++mi) {
        int order[SPG_FUSED_MAXR];
        const int64_t *str = mi == 0 ? ostr : sstr[mi - 1];
        for (int i = 0; i < R; ++i) order[i] = i;
        std::sort(order, order + R, [&](int a, int b) { return str[a] < str[b]; });
        uint64_t dim[5], stride[5];
        uint32_t box[5];
        int8_t mdim[SPG_FUSED_MAXR];
        int64_t w[SPG_FUSED_MAXR];
        if (!ft_map(R, order, O, str, mi > 0 ? Ls : L, mi > 0, dim, stride, box, mdim, w))
            return SPAGHETTY_ERR_NOKERNEL;
        if (mi > 0 && box[0] != (uint32_t)pw) return SPAGHETTY_ERR_NOKERNEL;   // one source row
        for (int g = 0; g < ng; ++g) {
            const int i = gd[g];
            const int64_t mul = L[i] * w[i];
            if (mul * ((O[i] + L[i] - 1) / L[i]) > INT32_MAX) return SPAGHETTY_ERR_NOKERNEL;
            P.mdim[mi][g] = mdim[i];
            P.mul[mi][g] = (int32_t)mul;
        }
        const double *ptr = mi == 0 ? sorted : unsorted[mi - 1];
        if (spg_encode_map(&M.m[mi], ptr, dim, stride, box, mi > 0 && swz) != SPAGHETTY_OK)
            return SPAGHETTY_ERR_NOKERNEL;
    }
    P.nsrc = nsrc;
    P.vol = (int32_t)vol;
    P.lq = (int32_t)lq;
    P.lr = (int32_t)lr;
    P.lp = (int32_t)lp;
    P.pw = (int32_t)pw;
    P.swz = swz ? 1 : 0;
    // output order (fastest first) is q, then p and r as their strides say;
    // a source lists q before r when q's stride there is the smaller
    P.out_r_first = (r != p && ostr[r] < ostr[p]) ? 1 : 0;
    for (int k = 0; k < nsrc; ++k) P.src_r_first[k] = (r != p && sstr[k][r] < sstr[k][q]) ? 1 : 0;
    P.tile_bytes = (uint32_t)(((std::max(vol, vol_src) * 8) + 1023) & ~(int64_t)1023);
    P.tx_out = (uint32_t)(vol * 8);
    P.tx_src = (uint32_t)(vol_src * 8);
    for (int k = 0; k < nsrc; ++k) {
        const double g = (first_sets && k == 0) ? 0.0 : 1.0;
        P.fac[k] = spg_make_factor(factors[k], g);
        P.op[k] = spg_choose_op(factors[k], g);
    }
    P.first_sets = first_sets ? 1 : 0;
    P.status = spg_status_word();
    if (!launch) return SPAGHETTY_OK;
    const size_t smem = (size_t)(SPG_FT_S + 2) * P.tile_bytes + (2 * SPG_FT_S + 4) * 8 + 1024;
    const void *fn = (const void *)spg_fused_tma<SPG_FT_NT, SPG_FT_EPT, SPG_FT_S>;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    int dev = 0, sms = 152, nb = 1;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return SPAGHETTY_ERR_CUDA; }
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 152;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, SPG_FT_BLOCK(SPG_FT_NT), smem) != cudaSuccess || nb < 1)
        nb = 1;
    cudaGetLastError();
    const int grid = (int)std::min<int64_t>((int64_t)sms * nb, ntiles);
    void *args[] = {(void *)&M, (void *)&P};
    if (cudaLaunchKernel(fn, dim3(grid), dim3(SPG_FT_BLOCK(SPG_FT_NT)), args, smem, (cudaStream_t)stream) !=
        cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    return SPAGHETTY_OK;
}

static int fused_pass(int rank, int nsrc, const double *const *unsorted, const int *dims,
                      const int *perms, const double *factors, double *sorted, void *stream,
                      bool first_sets, bool allow_tma) {
    if (rank < 1 || rank > SPG_FUSED_MAXR) return SPAGHETTY_ERR_RANK;
    if (nsrc < 1 || nsrc > SPG_FUSED_MAXS) return SPAGHETTY_ERR_CONFIG;
    if (!unsorted || !dims || !perms || !factors) return SPAGHETTY_ERR_NULL;
    // output shape from source 0; every source must agree
    int64_t out_dims[SPG_FUSED_MAXR];
    for (int k = 0; k < nsrc; ++k) {
        bool seen[SPG_FUSED_MAXR] = {false};
        for (int q = 0; q < rank; ++q) {
            const int p = perms[k * rank + q];
            if (p < 1 || p > rank || seen[p - 1]) return SPAGHETTY_ERR_PERM;
            seen[p - 1] = true;
            if (dims[k * rank + p - 1] < 0) return SPAGHETTY_ERR_DIMS;
            const int64_t e = dims[k * rank + p - 1];
            if (k == 0) out_dims[q] = e;
            else if (out_dims[q] != e) return SPAGHETTY_ERR_DIMS;
        }
    }
    int64_t n = 1;
    for (int q = 0; q < rank; ++q) n *= out_dims[q];
    if (n == 0) return SPAGHETTY_OK;
    if (!sorted) return SPAGHETTY_ERR_NULL;
    for (int k = 0; k < nsrc; ++k) {
        if (!unsorted[k]) return SPAGHETTY_ERR_NULL;
        const uintptr_t a0 = (uintptr_t)unsorted[k], a1 = a0 + (uintptr_t)n * 8;
        const uintptr_t b0 = (uintptr_t)sorted, b1 = b0 + (uintptr_t)n * 8;
        if (a0 < b1 && b0 < a1) return SPAGHETTY_ERR_ALIAS;
    }
    // drop unit output dims
    int keep[SPG_FUSED_MAXR], R = 0;
    for (int q = 0; q < rank; ++q)
        if (out_dims[q] > 1) keep[R++] = q;
    if (R == 0) { keep[0] = rank - 1; R = 1; }
    int64_t O[SPG_FUSED_MAXR], ostride_full[SPG_FUSED_MAXR];
    {
        int64_t s = 1;
        for (int q = rank - 1; q >= 0; --q) { ostride_full[q] = s; s *= out_dims[q]; }
    }
    for (int i = 0; i < R; ++i) O[i] = out_dims[keep[i]];
    // per source: global stride of each kept output dim
    static thread_local FusedParams P;
    std::memset(&P, 0, sizeof(P));
    int64_t sstride[SPG_FUSED_MAXS][SPG_FUSED_MAXR];
    for (int k = 0; k < nsrc; ++k) {
        int64_t sst[SPG_FUSED_MAXR];
        int64_t s = 1;
        for (int i = rank - 1; i >= 0; --i) { sst[i] = s; s *= dims[k * rank + i]; }
        for (int i = 0; i < R; ++i) sstride[k][i] = sst[perms[k * rank + keep[i]] - 1];
    }
    int64_t ostr[SPG_FUSED_MAXR];
    for (int i = 0; i < R; ++i) ostr[i] = ostride_full[keep[i]];
    if (allow_tma) {
        const int rc = fused_tma_pass(R, O, ostr, sstride, nsrc, unsorted, factors, sorted, stream, first_sets);
        if (rc != SPAGHETTY_ERR_NOKERNEL) return rc;
    }
    // layouts: 0 = output, 1.. = sources; each lists the kept dims fastest first
    int order[SPG_FUSED_MAXS + 1][SPG_FUSED_MAXR];
    for (int i = 0; i < R; ++i) order[0][i] = R - 1 - i;
    for (int k = 0; k < nsrc; ++k) {
        for (int i = 0; i < R; ++i) order[k + 1][i] = i;
        std::sort(order[k + 1], order[k + 1] + R,
                  [&](int a, int b) { return sstride[k][a] < sstride[k][b]; });
    }
    int64_t L[SPG_FUSED_MAXR];
    fused_box(R, O, nsrc + 1, order, L);
    int64_t vol = 1;
    for (int i = 0; i < R; ++i) vol *= L[i];
    if (vol > SPG_FUSED_VMAX) return SPAGHETTY_ERR_CONFIG;
    // canonical (output-order) box strides
    int64_t can[SPG_FUSED_MAXR];
    {
        int64_t s = 1;
        for (int i = R - 1; i >= 0; --i) { can[i] = s; s *= L[i]; }
    }
    P.nsrc = nsrc;
    P.vol = (int32_t)vol;
    P.pad = 0;
    // output walk
    int64_t maxoff = 0;
    for (int i = R - 1; i >= 0; --i) {
        if (L[i] <= 1) continue;
        const int d = P.no++;
        P.olen[d] = spg_make_fastdiv((uint32_t)L[i]);
        P.ostr[d] = (int32_t)ostr[i];
        maxoff += (L[i] - 1) * ostr[i];
    }
    for (int k = 0; k < nsrc; ++k) {
        int64_t smax = 0;
        for (int j = 0; j < R; ++j) {
            const int i = order[k + 1][j];
            if (L[i] <= 1) continue;
            const int d = P.ns[k]++;
            P.slen[k][d] = spg_make_fastdiv((uint32_t)L[i]);
            P.sstr[k][d] = (int32_t)sstride[k][i];
            P.scan[k][d] = (int32_t)can[i];
            smax += (L[i] - 1) * sstride[k][i];
        }
        if (smax > INT32_MAX) return SPAGHETTY_ERR_NOKERNEL;
        P.src[k] = unsorted[k];
        const double g = (first_sets && k == 0) ? 0.0 : 1.0;
        P.fac[k] = spg_make_factor(factors[k], g);
        P.op[k] = spg_choose_op(factors[k], g);
    }
    P.first_sets = first_sets ? 1 : 0;
    if (maxoff > INT32_MAX) return SPAGHETTY_ERR_NOKERNEL;
    // pad: one slot every `pad` canonical elements, picked to spread the
    // scattered source writes over the banks (fewest simulated conflicts)
    {
        int64_t best = -1;
        int cands[SPG_FUSED_MAXR + 1];
        int nc = 0;
        cands[nc++] = 0;
        for (int i = 0; i < R; ++i)
            if (can[i] > 1 && can[i] < vol) cands[nc++] = (int)can[i];
        for (int ci = 0; ci < nc; ++ci) {
            const int pad = cands[ci];
            int64_t cost = 0;
            for (int k = 0; k < nsrc; ++k) {
                // the first two warps of the source's write pattern
                for (int w = 0; w < 2; ++w)
                    for (int h = 0; h < 2; ++h) {
                        int cnt[16] = {0}, worst = 0;
                        for (int tt = 0; tt < 16; ++tt) {
                            int64_t j = w * 32 + h * 16 + tt;
                            if (j >= vol) break;
                            int64_t rem = j, cidx = 0;
                            for (int d = 0; d < P.ns[k]; ++d) {
                                const int64_t len = P.slen[k][d].d;
                                cidx += (rem % len) * P.scan[k][d];
                                rem /= len;
                            }
                            const int64_t slot = cidx + (pad ? cidx / pad : 0);
                            worst = std::max(worst, ++cnt[slot & 15]);
                        }
                        cost += worst;
                    }
            }
            if (best < 0 || cost < best) { best = cost; P.pad = pad; }
        }
    }
    P.tile = (int32_t)((vol + (P.pad ? vol / P.pad + 1 : 0) + 1) & ~1);
    if (P.tile > 65535) return SPAGHETTY_ERR_CONFIG;
    // grid over the kept dims, output-fastest first
    int64_t ntiles = 1;
    for (int i = R - 1; i >= 0; --i) {
        const int64_t cnt = O[i] / L[i];
        if (cnt <= 1) continue;
        const int d = P.ng++;
        P.gcnt[d] = spg_make_fastdiv((uint32_t)cnt);
        P.gout[d] = L[i] * ostr[i];
        for (int k = 0; k < nsrc; ++k) P.gsrc[k][d] = L[i] * sstride[k][i];
        ntiles *= cnt;
        if (ntiles > INT32_MAX) return SPAGHETTY_ERR_NOKERNEL;
    }
    P.ntiles = (uint32_t)ntiles;
    const size_t smem = (((size_t)nsrc * vol * 6 + 15) & ~(size_t)15) + (size_t)2 * P.tile * 8;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(spg_fused_sortacc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    int dev = 0, sms = 152, nb = 1;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return SPAGHETTY_ERR_CUDA; }
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 152;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spg_fused_sortacc, SPG_FUSED_NT, smem) != cudaSuccess || nb < 1)
        nb = 1;
    cudaGetLastError();
    const int grid = (int)std::min<int64_t>((int64_t)sms * nb, ntiles);
    void *args[] = {(void *)&sorted, (void *)&P};
    if (cudaLaunchKernel((const void *)spg_fused_sortacc, dim3(grid), dim3(SPG_FUSED_NT), args, smem,
                         (cudaStream_t)stream) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    return SPAGHETTY_OK;
}

// The sources are split into passes of consecutive sortaccs (so every
// element still receives its additions in call order) whose sources share
// their stride-1 index: one box then gives every source and the output
// long contiguous runs.  The nine triples sortaccs of one group touch one to
// three such indices, i.e. one to three passes over t3 instead of nine.
// Outputs of at most SPG_FUSED_ONE_PASS elements (L2-resident, where a
// launch costs more than the shorter runs) take all the sources in one pass
// of the cp.async kernel instead.  first_sets: the first source's product
// starts the sum (a sort followed by sortaccs); the first pass then does not
// read the output.
#ifndef SPG_FUSED_ONE_PASS
#define SPG_FUSED_ONE_PASS (int64_t(1) << 22)
#endif

static int fused_entry(const char *name, int rank, int nsrc, const double *const *unsorted,
                       const int *dims, const int *perms, const double *factors, double *sorted,
                       void *stream, bool first_sets) {
    SpgRange range(name);
    if (rank < 1 || rank > SPG_FUSED_MAXR) return SPAGHETTY_ERR_RANK;
    if (nsrc < 1 || nsrc > SPG_FUSED_MAXS) return SPAGHETTY_ERR_CONFIG;
    if (!unsorted || !dims || !perms || !factors) return SPAGHETTY_ERR_NULL;
    // output position holding each source's stride-1 index (source dim rank)
    int fast[SPG_FUSED_MAXS];
    for (int k = 0; k < nsrc; ++k) {
        fast[k] = -1;
        for (int q = 0; q < rank; ++q) {
            const int p = perms[k * rank + q];
            if (p < 1 || p > rank) return SPAGHETTY_ERR_PERM;
            // unit source dims do not count: take the fastest non-unit one
        }
        for (int i = rank - 1; i >= 0 && fast[k] < 0; --i) {
            if (dims[k * rank + i] == 1 && i > 0) continue;
            for (int q = 0; q < rank; ++q)
                if (perms[k * rank + q] == i + 1) fast[k] = q;
        }
    }
    int64_t n0 = 1;
    for (int q = 0; q < rank; ++q) n0 *= dims[q] > 0 ? dims[q] : 0;
    if (n0 == 0) return SPAGHETTY_OK;   // empty tensors: nothing to do
    // device (or managed) memory of one device only: the kernel reads and
    // writes these pointers directly; the work runs on that device
    int dev = -1;
    for (int k = -1; k < nsrc; ++k) {
        const void *ptr = k < 0 ? (const void *)sorted : (const void *)unsorted[k];
        if (!ptr) return SPAGHETTY_ERR_NULL;
        cudaPointerAttributes at;
        std::memset(&at, 0, sizeof(at));
        if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
            cudaGetLastError();
            return SPAGHETTY_ERR_MEMSPACE;
        }
        if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) || (dev >= 0 && at.device != dev))
            return SPAGHETTY_ERR_MEMSPACE;
        dev = at.device;
    }
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) cudaGetLastError();
    if (cudaSetDevice(dev) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    int passes = 1;
    for (int k = 1; k < nsrc; ++k) passes += fast[k] != fast[k - 1];
    int rc = SPAGHETTY_OK;
    if (passes > 1 && n0 <= SPG_FUSED_ONE_PASS) {
        rc = fused_pass(rank, nsrc, unsorted, dims, perms, factors, sorted, stream, first_sets, false);
    } else {
        int k0 = 0;
        while (k0 < nsrc && rc == SPAGHETTY_OK) {
            int k1 = k0 + 1;
            while (k1 < nsrc && fast[k1] == fast[k0]) ++k1;
            rc = fused_pass(rank, k1 - k0, unsorted + k0, dims + k0 * rank, perms + k0 * rank,
                            factors + k0, sorted, stream, first_sets && k0 == 0, true);
            k0 = k1;
        }
    }
    if (cur >= 0 && cur != dev) cudaSetDevice(cur);
    return rc;
}

extern "C" int spaghetty_sortacc_fused(int rank, int nsrc, const double *const *unsorted,
                                       const int *dims, const int *perms, const double *factors,
                                       double *sorted, void *stream) {
    return fused_entry("spaghetty_sortacc_fused", rank, nsrc, unsorted, dims, perms, factors, sorted,
                       stream, false);
}

extern "C" int spaghetty_sort_fused(int rank, int nsrc, const double *const *unsorted, const int *dims,
                                    const int *perms, const double *factors, double *sorted, void *stream) {
    return fused_entry("spaghetty_sort_fused", rank, nsrc, unsorted, dims, perms, factors, sorted, stream,
                       true);
}
