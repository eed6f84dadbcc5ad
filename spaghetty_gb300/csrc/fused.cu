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
// Kernel: a persistent CTA walks boxes of the OUTPUT index space (box lengths
// divide the extents, so no element masks).  For each box it loads its t3
// elements into registers (output order), then for every source in turn
// stages that source's elements through shared memory -- loaded in the
// source's own memory order (coalesced), placed at their output-order slot --
// and adds them.  Sources are double-buffered with cp.async: source k+1 is in
// flight while source k is added.  Each source's box walk (offset and slot of
// every element) is a shared-memory table built once per CTA.
#include "../../include/spaghetty_gb300.h"
#include "kernels.cuh"
#include "plan.h"

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
    int32_t op[SPG_FUSED_MAXS];            // OP_ACC_* per source
};

template <int OPA>
__device__ __forceinline__ double spg_fused_add(double acc, double x, const SpgFactor &F) {
    return spg_apply<OPA>(x, acc, F);
}

__device__ __forceinline__ double spg_fused_apply(int op, double acc, double x, const SpgFactor &F) {
    switch (op) {
        case OP_ACC_ONE: return spg_fused_add<OP_ACC_ONE>(acc, x, F);
        case OP_ACC_NEG: return spg_fused_add<OP_ACC_NEG>(acc, x, F);
        case OP_ACC_POW2: return spg_fused_add<OP_ACC_POW2>(acc, x, F);
        default: return spg_fused_add<OP_ACC_ANY>(acc, x, F);
    }
}

__global__ void __launch_bounds__(SPG_FUSED_NT)
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
            acc[m] = ooff[m] >= 0 ? spg_ld_out(out + obase + ooff[m]) : 0.0;
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

static int fused_pass(int rank, int nsrc, const double *const *unsorted, const int *dims,
                      const int *perms, const double *factors, double *sorted, void *stream) {
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
        const double g = 1.0;
        P.fac[k] = spg_make_factor(factors[k], g);
        P.op[k] = spg_choose_op(factors[k], g);
    }
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
extern "C" int spaghetty_sortacc_fused(int rank, int nsrc, const double *const *unsorted,
                                       const int *dims, const int *perms, const double *factors,
                                       double *sorted, void *stream) {
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
    {
        int64_t n0 = 1;
        for (int q = 0; q < rank; ++q) n0 *= dims[q] > 0 ? dims[q] : 0;
        if (n0 == 0) return SPAGHETTY_OK;   // empty tensors: nothing to do
    }
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
    int rc = SPAGHETTY_OK;
    int k0 = 0;
    while (k0 < nsrc && rc == SPAGHETTY_OK) {
        int k1 = k0 + 1;
        while (k1 < nsrc && fast[k1] == fast[k0]) ++k1;
        rc = fused_pass(rank, k1 - k0, unsorted + k0, dims + k0 * rank, perms + k0 * rank,
                        factors + k0, sorted, stream);
        k0 = k1;
    }
    if (cur >= 0 && cur != dev) cudaSetDevice(cur);
    return rc;
}
