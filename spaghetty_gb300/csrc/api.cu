// api.cu -- the C ABI: NWChem drop-ins, generic entry points, dispatch.
//
// The reference's boundary is trunk/tce_sort4_switch.F:1-62 (tce_sort_4 maps
// the permutation to the tuned loop nest; an unknown permutation prints
// 'something is wrong...' and returns).  Here every entry point validates,
// folds and plans on the host (plan.cpp), then launches one of the compiled
// kernel variants (kernels.cuh, instantiated by generator.py).
#include "../../include/spaghetty_gb300.h"
#include "kernels.cuh"
#include "plan.h"
#include "tma.cuh"

#include <cuda.h>
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iterator>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

const SpgKernelEntry *spg_kernels_op0(int *n);
const SpgKernelEntry *spg_kernels_op1(int *n);
const SpgKernelEntry *spg_kernels_op2(int *n);
const SpgKernelEntry *spg_kernels_op3(int *n);
const SpgKernelEntry *spg_kernels_op4(int *n);
const SpgKernelEntry *spg_kernels_op5(int *n);
const SpgKernelEntry *spg_kernels_op6(int *n);
const SpgKernelEntry *spg_kernels_op7(int *n);
const SpgKernelEntry *spg_kernels_op8(int *n);

namespace {

thread_local int g_last_error = 0;

// Dynamic shared memory one CTA may opt into on sm_100-class GPUs (227 KB).
const int kMaxSmemPerBlock = 232448;

int record(int rc) {
    g_last_error = rc;
    return rc;
}

// The CUDA error behind the last SPAGHETTY_ERR_CUDA (a cudaError_t, or the
// negated CUresult of a failed tensor-map encoding); process-wide.
std::atomic<int> g_last_cuda{0};

int cuda_fail(cudaError_t e) {
    g_last_cuda.store((int)e);
    cudaGetLastError();
    return SPAGHETTY_ERR_CUDA;
}

std::mutex g_mu;

struct TuneOverride {
    int box[SPG_MAXR];
    int threads, ept, stages;
};
std::map<std::string, TuneOverride> g_tune;

// Plain sorts on tuned TMA plans from this many elements (256 MiB per
// array, twice GB300's L2) run on the power-of-two path (make_plan_uncached).
#define SPG_TUNED_ONE_AS_POW2 (int64_t(1) << 25)
std::map<int, int> g_sms;
std::map<std::pair<const void *, int>, int> g_occ;

const SpgKernelEntry *find_kernel(int kind, int op, int nt, int ept, int stages) {
    static const SpgKernelEntry *tabs[OP_COUNT];
    static int counts[OP_COUNT];
    static std::once_flag once;
    std::call_once(once, [] {
        tabs[0] = spg_kernels_op0(&counts[0]);
        tabs[1] = spg_kernels_op1(&counts[1]);
        tabs[2] = spg_kernels_op2(&counts[2]);
        tabs[3] = spg_kernels_op3(&counts[3]);
        tabs[4] = spg_kernels_op4(&counts[4]);
        tabs[5] = spg_kernels_op5(&counts[5]);
        tabs[6] = spg_kernels_op6(&counts[6]);
        tabs[7] = spg_kernels_op7(&counts[7]);
        tabs[8] = spg_kernels_op8(&counts[8]);
    });
    if (op < 0 || op >= OP_COUNT) return nullptr;
    for (int i = 0; i < counts[op]; ++i) {
        const SpgKernelEntry &e = tabs[op][i];
        if (e.kind == kind && e.threads == nt && e.ept == ept && e.stages == stages) return &e;
    }
    return nullptr;
}

int device_sms(int dev) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_sms.find(dev);
    if (it != g_sms.end()) return it->second;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        sms = 152;
    }
    g_sms[dev] = sms;
    return sms;
}

// Threads per CTA of a table entry: the TMA-staged kernel adds a load warp
// and a store warp to its permute threads.
int block_threads(const SpgKernelEntry *k) {
    return k->kind == KIND_TMA ? SPG_TMA_BLOCK(k->threads) : k->threads;
}

int occupancy(const SpgKernelEntry *k, int smem) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_pair(k->fn, smem);
    auto it = g_occ.find(key);
    if (it != g_occ.end()) return it->second;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k->fn, block_threads(k), smem) != cudaSuccess) {
        cudaGetLastError();
        nb = 1;
    }
    if (nb < 1) nb = 1;
    g_occ[key] = nb;
    return nb;
}

std::string tune_key(const Folded &fo, int op) {
    const int cls = spg_op_class(op);
    std::string k = std::to_string(fo.rank) + ":";
    for (int d = 0; d < fo.rank; ++d) k += std::to_string(fo.D[d]) + ",";
    k += ":";
    for (int d = 0; d < fo.rank; ++d) k += std::to_string(fo.P[d]) + ",";
    k += ":" + std::to_string(cls);
    return k;
}

void autoload_tune_file();

// Plans are cached by (rank, dims, perm, op, SM count): NWChem repeats the
// same few shapes thousands of times, and planning (box search, bank
// simulations) costs up to a few hundred microseconds.  Cleared whenever an
// override changes; past kPlanCacheMax entries half of them are dropped.
std::unordered_map<std::string, Plan> g_plans;
std::mutex g_plans_mu;
const size_t kPlanCacheMax = 16384;   // about 1.3 KB per entry

std::string plan_key(int rank, const int *dims, const int *perm, int op, int sms) {
    std::string k;
    k.reserve(96);
    k += std::to_string(rank) + ":" + std::to_string(op) + ":" + std::to_string(sms) + ":";
    for (int q = 0; q < rank; ++q) k += std::to_string(dims[q]) + ",";
    k += ":";
    for (int q = 0; q < rank; ++q) k += std::to_string(perm[q]) + ",";
    return k;
}

int make_plan_uncached(int rank, const int *dims, const int *perm, double f, double g, int sms,
                       bool allow_tma, bool host_link, Plan *pl);
int tma_smem_bytes(const TmaLayout &tl, int stages);

// allow_tma: both tensors 16-byte aligned device memory (the bulk tensor
// copies' rule); host_link: a tensor is pinned host memory that the kernel
// reads or writes in place over the host link
int make_plan(int rank, const int *dims, const int *perm, double f, double g, int sms, Plan *pl,
              bool allow_tma = true, bool host_link = false) {
    autoload_tune_file();
    if (rank < 1 || rank > SPG_MAXR || !dims || !perm)
        return make_plan_uncached(rank, dims, perm, f, g, sms, allow_tma, host_link, pl);
    const int op = spg_choose_op(f, g);
    const std::string key = plan_key(rank, dims, perm, op, sms) + (allow_tma ? "t" : "n") + (host_link ? "h" : "");
    {
        std::lock_guard<std::mutex> lk(g_plans_mu);
        auto it = g_plans.find(key);
        if (it != g_plans.end()) {
            *pl = it->second;
            pl->kp.fac = spg_make_factor(f, g);
            return SPAGHETTY_OK;
        }
    }
    int rc = make_plan_uncached(rank, dims, perm, f, g, sms, allow_tma, host_link, pl);
    if (rc == SPAGHETTY_OK) {
        std::lock_guard<std::mutex> lk(g_plans_mu);
        if (g_plans.size() >= kPlanCacheMax) {
            // drop every other entry rather than all: a working set just
            // above the limit then re-plans a part of its shapes, not all
            bool drop = true;
            for (auto it = g_plans.begin(); it != g_plans.end(); drop = !drop)
                it = drop ? g_plans.erase(it) : std::next(it);
        }
        g_plans[key] = *pl;
    }
    return rc;
}

int choose_skew(Plan *pl);
// SPAGHETTY_OPT_TMA_SKEW: 1 (default) lets choose_skew rotate the permute
// step's slot map where the bank simulation favours it, 0 plans every TMA
// kernel without skew.
int g_tma_skew = 1;

// Switch a built tiled plan to the TMA-staged kernel with the given shape.
int to_tma(Plan *pl, int threads, int ept, int stages, bool strict) {
    TmaLayout tl;
    pl->sk_stride = pl->sk_len = pl->sk_mul = 0;
    if ((pl->kind != KIND_TILED && pl->kind != KIND_DIRECT) || threads * ept < pl->kp.vol ||
        spg_tma_layout(*pl, stages, &tl) != SPAGHETTY_OK ||
        tma_smem_bytes(tl, stages) > kMaxSmemPerBlock)
        return strict ? SPAGHETTY_ERR_CONFIG : SPAGHETTY_ERR_NOKERNEL;
    pl->threads = threads;
    pl->ept = ept;
    pl->stages = stages;
    pl->kind = KIND_TMA;
    pl->smem_bytes = tma_smem_bytes(tl, stages);
    choose_skew(pl);
    return SPAGHETTY_OK;
}

// Shared-memory wavefronts of the TMA kernel's permute step under one slot
// mapping: per half warp (16 consecutive slots of one element index k), the
// 8-byte reads of the input tile at lin and the writes of the output tile at
// e (a sortacc's reads of the old output use the same words as the writes).
// A half warp's accesses take one wavefront per access of the busiest bank
// pair.  Slot -> e and e -> lin are bijections, so a half warp's 16 words
// are distinct and the count needs no de-duplication.  lin0[e]: the
// input-tile element of output-tile element e (spg_walk, computed once).
static int64_t tma_permute_wavefronts(const Plan &pl, const TmaParams &tp, const std::vector<int32_t> &lin0) {
    const int NT = pl.threads, V = pl.kp.vol;
    int64_t total = 0;
    for (int k = 0; k < pl.ept; ++k)
        for (int h = 0; h < NT / 16; ++h) {
            int cr[16] = {0}, cw[16] = {0}, wr = 0, ww = 0;
            for (int t = 0; t < 16; ++t) {
                const uint32_t n = (uint32_t)(k * NT + h * 16 + t);
                if (n >= (uint32_t)V) break;
                uint32_t e = n;
                if (tp.sk_mul) {
                    const uint32_t lo = n % (uint32_t)tp.sk_stride;
                    const int32_t y = (int32_t)((n / (uint32_t)tp.sk_stride) % (uint32_t)tp.sk_len);
                    const int32_t y2 =
                        (int32_t)((uint32_t)(y + (int32_t)(lo & 15u) * tp.sk_mul) % (uint32_t)tp.sk_len);
                    e = (uint32_t)((int32_t)n + (y2 - y) * tp.sk_stride);
                }
                wr = std::max(wr, ++cr[(uint32_t)lin0[e] & 15u]);
                ww = std::max(ww, ++cw[e & 15u]);
            }
            total += wr + ww;
        }
    return total;
}

// Pick the permute-step skew of a TMA plan: no skew, or a rotation of one
// output dim's coordinate by (slot mod 16) * m for m in 1..3, whichever
// takes the fewest simulated wavefronts (ties keep the simpler mapping).
// The rotation formula is the kernel's (spg_tma_slot), written out here
// over the precomputed table.
int choose_skew(Plan *pl) {
    pl->sk_stride = pl->sk_len = pl->sk_mul = 0;
    if (!g_tma_skew || pl->kind != KIND_TMA || pl->kp.vol >= 65535 || pl->fo.P[pl->fo.rank - 1] == pl->fo.rank - 1)
        return SPAGHETTY_OK;   // same-order tiles: the permute step is the identity
    TmaParams tp;
    std::memset(&tp, 0, sizeof(tp));
    std::vector<int32_t> lin0((size_t)pl->kp.vol);
    for (uint32_t e = 0; e < (uint32_t)pl->kp.vol; ++e) {
        int32_t a, b;
        uint32_t pk;
        spg_walk(pl->kp.st, e, a, b, lin0[e], pk);
    }
    int64_t best = tma_permute_wavefronts(*pl, tp, lin0);
    const int64_t ideal = 2 * (int64_t)((pl->kp.vol + 15) / 16);
    const BoxWalk &w = pl->kp.st;
    int32_t stride = 1;
    for (int d = 0; d < w.n && best > ideal; ++d) {
        const int32_t len = (int32_t)w.len[d].d;
        for (int m = 1; m <= 3 && len > 1; ++m) {
            tp.sk_stride = stride;
            tp.sk_len = len;
            tp.sk_mul = m;
            const int64_t wf = tma_permute_wavefronts(*pl, tp, lin0);
            if (wf < best) {
                best = wf;
                pl->sk_stride = stride;
                pl->sk_len = len;
                pl->sk_mul = m;
            }
        }
        stride *= len;
    }
    return SPAGHETTY_OK;
}

// SPAGHETTY_OPT_WARP_TR: 1 (default) plans the warp-shuffle transpose
// where its rule picks it, 0 never, 2 wherever its inner tile qualifies.
int g_warp_tr = 1;
const int64_t kWarpMaxElems = (int64_t)1 << 22;

// The warp-shuffle transpose plan (spg_warp_tr) of a folded problem: the
// tile covers the input's and the output's stride-1 dims whole (A x B
// elements, A, B <= 32, A*B <= 128: K = ceil(A*B/32) registers per lane),
// one index of every other dim.  SPAGHETTY_ERR_NOKERNEL when the problem
// does not qualify.
int make_warp_plan(const Folded &fo, int op, double f, double g, int sms, Plan *pl) {
    const int R = fo.rank;
    if (fo.empty || R < 2) return SPAGHETTY_ERR_NOKERNEL;
    const int a = R - 1, b = fo.P[R - 1];
    if (a == b || fo.D[a] > 32 || fo.D[b] > 32 || fo.D[a] * fo.D[b] > 128) return SPAGHETTY_ERR_NOKERNEL;
    const int V = (int)(fo.D[a] * fo.D[b]);
    const int K = (V + 31) / 32;
    int box[SPG_MAXR];
    for (int d = 0; d < R; ++d) box[d] = 1;
    box[a] = (int)fo.D[a];
    box[b] = (int)fo.D[b];
    Plan tp;
    int rc = spg_plan(fo, op, box, 256, K, 0, sms, &tp);
    if (!rc) rc = spg_build_params(&tp, f, g);
    if (rc) return rc == SPAGHETTY_ERR_NOKERNEL ? rc : SPAGHETTY_ERR_NOKERNEL;
    if (tp.kp.ld.n != 2 || tp.kp.st.n != 2 || tp.masked) return SPAGHETTY_ERR_NOKERNEL;
    tp.kind = KIND_WARP;
    tp.threads = 256;
    tp.ept = K;
    tp.stages = 0;
    tp.smem_bytes = 0;
    tp.kp.pad = 0;
    tp.sk_stride = tp.sk_len = tp.sk_mul = 0;
    *pl = tp;
    return SPAGHETTY_OK;
}

int make_plan_uncached(int rank, const int *dims, const int *perm, double f, double g, int sms,
                       bool allow_tma, bool host_link, Plan *pl) {
    Folded fo;
    int rc = spg_fold(rank, dims, perm, &fo);
    if (rc) return rc;
    const int op = spg_choose_op(f, g);
    if (host_link && !fo.empty && fo.rank >= 2) {
        // over the host link long output rows matter most (measured on
        // GB300, pinned buffers at 100^4: up to 15% over the device plan):
        // the greedy box with 32-double input and 128-double output rows
        // grown towards 4096 elements on the cp.async kernel (the smallest
        // of 128/256/512 threads x 8 that holds it), 3 stages; the
        // device-memory tune table does not apply
        int box[SPG_MAXR];
        Plan tp;
        if (spg_box_greedy(fo, 32, 128, 4096, 4096, box) == SPAGHETTY_OK) {
            int vol = 1;
            for (int d = 0; d < fo.rank; ++d) vol *= box[d];
            const int nt = vol <= 1024 ? 128 : (vol <= 2048 ? 256 : 512);
            if (spg_plan(fo, op, box, nt, 8, 3, sms, &tp) == SPAGHETTY_OK &&
                spg_build_params(&tp, f, g) == SPAGHETTY_OK && tp.kind == KIND_TILED) {
                *pl = tp;
                return SPAGHETTY_OK;
            }
        }
    }
    TuneOverride ov;
    bool have = false;
    if (!fo.empty && fo.rank >= 2) {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_tune.find(tune_key(fo, op));
        if (it != g_tune.end()) { ov = it->second; have = true; }
    }
    // an override with stages 12/13/14/16 asks for the TMA kernel (2/3/4/6
    // load stages);
    // it is ignored where the TMA kernel cannot run (misaligned or host
    // buffers), which then get the default plan
    if (have && ov.stages == 20) {
        // a forced warp-shuffle transpose
        if (make_warp_plan(fo, op, f, g, sms, pl) == SPAGHETTY_OK) return SPAGHETTY_OK;
        have = false;
    }
    if (have && ov.stages >= 12 && !allow_tma) have = false;
    const bool want_tma = have && ov.stages >= 12;
    if (have) {
        rc = want_tma ? spg_plan(fo, op, ov.box, 256, 16, 0, sms, pl)
                      : spg_plan(fo, op, ov.box, ov.threads, ov.ept, ov.stages, sms, pl);
        if (rc) return rc;
        rc = spg_build_params(pl, f, g);
        if (rc) return rc;
        if (want_tma) {
            // The tuner times with f = 0.5, so a sort with f = 1 or -1 (and
            // a sortacc with f = -1) of a large array on a tuned TMA plan
            // runs that same kernel, as f = +-2^0 on the power-of-two path
            // (the same bits for every input but NaN, whose payload is not
            // part of the contract).  Measured on GB300: the bare
            // shared-memory copy of f = 1 is 15-20% slower on the plans
            // tuned at 100^4 (f = 1 sorts 5729 -> 6222 GB/s on the sweep),
            // but 2-4% faster on those tuned at 30^4 and 50^4, whose arrays
            // fit twice in L2; on untuned default plans neither is faster
            // overall (0.93-1.08 across 50^4..100^4 and 12^6..20^6).
            if (fo.nelem >= SPG_TUNED_ONE_AS_POW2) {
                if (pl->op == OP_SORT_ONE || pl->op == OP_SORT_NEG) pl->op = OP_SORT_POW2;
                if (pl->op == OP_ACC_NEG) pl->op = OP_ACC_POW2;
            }
            return to_tma(pl, ov.threads, ov.ept, ov.stages - 10, true);
        }
        return SPAGHETTY_OK;
    }
    // small inner tiles: the warp-shuffle transpose (rule: kWarpMaxElems)
    if (g_warp_tr) {
        Plan wp;
        if (make_warp_plan(fo, op, f, g, sms, &wp) == SPAGHETTY_OK &&
            (g_warp_tr == 2 || fo.nelem <= kWarpMaxElems)) {
            *pl = wp;
            return SPAGHETTY_OK;
        }
    }
    rc = spg_plan(fo, op, nullptr, 0, 0, 0, sms, pl);
    if (rc) return rc;
    rc = spg_build_params(pl, f, g);
    if (rc) return rc;
    // Default plans, chosen from the GB300 autotuner's timings of every
    // candidate over the sort4 sweep, the sort6 sample and random shapes:
    //  - transposes: the TMA-staged kernel on the greedy box with 32-double
    //    rows on both sides grown towards 1024 elements, the smallest CTA
    //    (128x8, 256x8, 256x16) that holds it, 3 load stages (2 when 3 do
    //    not fit); otherwise the register-staged tiled kernel on the greedy
    //    box with 16/32-double rows towards 512 elements.  (Of the rules
    //    (input rows, output rows, volume, stages) timed on 184 problems,
    //    ranks 4 and 6, this one came within 6% of each problem's best
    //    candidate on average; towards 4096 elements, one CTA per SM, was
    //    15% off: 4.7 against 5.6 TB/s at 16^6.)
    //  - the stride-1 index unchanged: the same-order TMA plan on a box of
    //    at most 1K elements, 128 threads x 8, 3 load stages (else 2).
    // Host-mapped (zero-copy) and misaligned buffers cannot use the bulk
    // copies: they keep the planner's own plan (the cp.async pipeline with
    // its larger boxes keeps the most bytes in flight over the host link).
    if (pl->kind == KIND_TILED && allow_tma) {
        int box[SPG_MAXR];
        Plan tp;
        bool done = false;
        if (spg_box_greedy(fo, 32, 32, 1024, 4096, box) == SPAGHETTY_OK) {
            // the bulk copies move whole 16-byte units along both stride-1
            // dims: round an odd partial box length there up to even
            for (const int d : {fo.rank - 1, fo.P[fo.rank - 1]})
                if (box[d] % 2 && box[d] < fo.D[d]) box[d] += 1;
            int vol = 1;
            for (int d = 0; d < fo.rank; ++d) vol *= box[d];
            const int nt = vol <= 1024 ? 128 : 256, ept = vol <= 2048 ? 8 : 16;
            if (spg_plan(fo, op, box, nt, ept, 0, sms, &tp) == SPAGHETTY_OK &&
                spg_build_params(&tp, f, g) == SPAGHETTY_OK &&
                (tp.kind == KIND_TILED || tp.kind == KIND_DIRECT)) {
                const Plan keep = tp;
                for (int S = 3; S >= 2 && !done; --S) {
                    tp = keep;
                    done = to_tma(&tp, nt, ept, S, false) == SPAGHETTY_OK;
                }
            }
        }
        if (!done && spg_box_greedy(fo, 16, 32, 512, 4096, box) == SPAGHETTY_OK) {
            // no TMA plan fits (strides or box rows not multiples of 16 bytes)
            int vol = 1;
            for (int d = 0; d < fo.rank; ++d) vol *= box[d];
            const int nt = vol <= 512 ? 128 : (vol <= 1024 ? 256 : 512), ept = vol <= 2048 ? 4 : 8;
            done = spg_plan(fo, op, box, nt, ept, 0, sms, &tp) == SPAGHETTY_OK &&
                   spg_build_params(&tp, f, g) == SPAGHETTY_OK && tp.kind == KIND_TILED;
        }
        if (done) *pl = tp;
    } else if (pl->kind == KIND_DIRECT && allow_tma) {
        int box[SPG_MAXR];
        Plan tp;
        if (spg_default_box_tma(fo, sms, 1024, box) == SPAGHETTY_OK &&
            spg_plan(fo, op, box, 128, 8, 0, sms, &tp) == SPAGHETTY_OK &&
            spg_build_params(&tp, f, g) == SPAGHETTY_OK && tp.kind == KIND_DIRECT) {
            const Plan keep = tp;
            bool done = false;
            for (int S = 3; S >= 2 && !done; --S) {
                tp = keep;
                done = to_tma(&tp, 128, 8, S, false) == SPAGHETTY_OK;
            }
            if (done) *pl = tp;
        }
    }
    return SPAGHETTY_OK;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// ---- TMA support ----------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        cudaGetLastError();
    });
    return fn;
}

// Error word for the kernels' bounded waits: pinned, mapped host memory, so
// the host reads it after a synchronisation without a copy.
int *g_status_host = nullptr;
int *g_status_dev = nullptr;
std::once_flag g_status_once;

int *status_word_dev() {
    std::call_once(g_status_once, [] {
        void *h = nullptr;
        if (cudaHostAlloc(&h, 256, cudaHostAllocMapped | cudaHostAllocPortable) == cudaSuccess) {
            void *d = nullptr;
            if (cudaHostGetDevicePointer(&d, h, 0) == cudaSuccess) {
                g_status_host = (int *)h;
                *g_status_host = 0;
                g_status_dev = (int *)d;
            }
        }
        cudaGetLastError();
    });
    return g_status_dev;
}

// L2 promotion of the bulk copies' requests: 128-byte measured 0.5% faster
// on the sweep than 256-byte (TMA sorts at 100^4: 5875-5890 vs 5810 GB/s).
#define SPG_L2_PROMOTION CU_TENSOR_MAP_L2_PROMOTION_L2_128B
int encode_map(CUtensorMap *m, const double *ptr, const uint64_t *dim, const uint64_t *stride,
               const uint32_t *box, bool swizzle128 = false) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return SPAGHETTY_ERR_CUDA;
    cuuint64_t gd[5], gs[4];
    cuuint32_t bd[5], es[5];
    for (int k = 0; k < 5; ++k) { gd[k] = dim[k]; bd[k] = box[k]; es[k] = 1; }
    for (int k = 0; k < 4; ++k) gs[k] = stride[k + 1];
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5, (void *)ptr, gd, gs, bd, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE,
                    swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                    SPG_L2_PROMOTION, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        g_last_cuda.store(-(int)r);
        return SPAGHETTY_ERR_CUDA;
    }
    return SPAGHETTY_OK;
}

// SPAGHETTY_ERR_DEVICE (and clear) if a kernel reported a timed-out wait.
int take_device_status() {
    if (g_status_host && *(volatile int *)g_status_host) {
        *(volatile int *)g_status_host = 0;
        return SPAGHETTY_ERR_DEVICE;
    }
    return SPAGHETTY_OK;
}

int tma_smem_bytes(const TmaLayout &tl, int stages) {
    // stages, two output slots, the mbarriers (full[stages], empty[stages],
    // done[2], free[2]) and 1 KB for aligning the base
    return stages * tl.tp.stage_bytes + 2 * tl.tp.out_bytes + (2 * stages + 4) * 8 + 1024;
}

int launch_plan(Plan &pl, const double *u, double *s, cudaStream_t st, int dev) {
    if (pl.kind == KIND_EMPTY) return SPAGHETTY_OK;
    const int sms = device_sms(dev);
    cudaError_t err;
    if (pl.kind == KIND_FLAT) {
        const int vec = (aligned16(u) && aligned16(s)) ? 2 : 1;
        const SpgKernelEntry *k = find_kernel(KIND_FLAT, pl.op, 256, vec, 0);
        if (!k) return SPAGHETTY_ERR_NOKERNEL;
        int64_t n = pl.fo.nelem;
        int64_t work = (n / vec + 255) / 256;
        int grid = (int)std::min<int64_t>(std::max<int64_t>(work, 1), (int64_t)sms * 8);
        SpgFactor fac = pl.kp.fac;
        void *args[] = {(void *)&u, (void *)&s, (void *)&n, (void *)&fac};
        pl.grid = grid;
        err = cudaLaunchKernel(k->fn, dim3(grid), dim3(256), args, 0, st);
    } else if (pl.kind == KIND_TMA) {
        const SpgKernelEntry *k = find_kernel(KIND_TMA, pl.op, pl.threads, pl.ept, pl.stages);
        if (!k) return SPAGHETTY_ERR_NOKERNEL;
        TmaLayout tl;
        int rc = spg_tma_layout(pl, pl.stages, &tl);
        if (rc) return rc;
        tl.tp.status = status_word_dev();
        alignas(64) CUtensorMap mi, mo;
        if ((rc = encode_map(&mi, u, tl.in_dim, tl.in_stride, tl.in_box))) return rc;
        if ((rc = encode_map(&mo, s, tl.out_dim, tl.out_stride, tl.out_box))) return rc;
        const int smem = tma_smem_bytes(tl, pl.stages);
        if (smem > 48 * 1024) {
            const cudaError_t e = cudaFuncSetAttribute(k->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return cuda_fail(e);
        }
        const int occ = occupancy(k, smem);
        int64_t grid = std::min<int64_t>((int64_t)pl.kp.ntiles, (int64_t)sms * occ);
        if (grid < 1) grid = 1;
        pl.grid = (int)grid;
        void *args[] = {(void *)&mi, (void *)&mo, (void *)&pl.kp, (void *)&tl.tp};
        err = cudaLaunchKernel(k->fn, dim3((unsigned)grid), dim3(block_threads(k)), args, (size_t)smem, st);
    } else if (pl.kind == KIND_WARP) {
        // one tile per warp at a time, eight warps per CTA
        const SpgKernelEntry *k = find_kernel(KIND_WARP, pl.op, 256, pl.ept, 0);
        if (!k) return SPAGHETTY_ERR_NOKERNEL;
        const int occ = occupancy(k, 0);
        int64_t grid = std::min<int64_t>(((int64_t)pl.kp.ntiles + 7) / 8, (int64_t)sms * occ);
        if (grid < 1) grid = 1;
        pl.grid = (int)grid;
        void *args[] = {(void *)&u, (void *)&s, (void *)&pl.kp};
        err = cudaLaunchKernel(k->fn, dim3((unsigned)grid), dim3(256), args, 0, st);
    } else {
        const SpgKernelEntry *k = find_kernel(pl.kind, pl.op, pl.threads, pl.ept, pl.stages);
        if (!k) return SPAGHETTY_ERR_NOKERNEL;
        if (pl.smem_bytes > 48 * 1024) {
            const cudaError_t e =
                cudaFuncSetAttribute(k->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, pl.smem_bytes);
            if (e != cudaSuccess) return cuda_fail(e);
        }
        const int occ = occupancy(k, pl.smem_bytes);
        int64_t grid = std::min<int64_t>((int64_t)pl.kp.ntiles, (int64_t)sms * occ);
        if (grid < 1) grid = 1;
        pl.grid = (int)grid;
        void *args[] = {(void *)&u, (void *)&s, (void *)&pl.kp};
        err = cudaLaunchKernel(k->fn, dim3((unsigned)grid), dim3(pl.threads), args,
                               (size_t)pl.smem_bytes, st);
    }
    if (err != cudaSuccess) return cuda_fail(err);
    return SPAGHETTY_OK;
}

bool overlaps(const double *a, const double *b, int64_t n) {
    const uintptr_t a0 = (uintptr_t)a, a1 = a0 + (uintptr_t)n * sizeof(double);
    const uintptr_t b0 = (uintptr_t)b, b1 = b0 + (uintptr_t)n * sizeof(double);
    return a0 < b1 && b0 < a1;
}

// Host buffers that are pinned (page-locked, registered with CUDA) are read
// and written by the kernels in place through their mapped device address --
// over NVLink-C2C on GB300, both directions at once -- instead of being
// staged with copies.  spaghetty_set_option(SPAGHETTY_OPT_HOST_ZERO_COPY, 0)
// turns that off (staging for every host buffer).
std::atomic<int> g_zero_copy{1};
// Pinned host buffers on both sides may instead be moved in slabs through a
// three-stream copy/sort/copy pipeline (SPAGHETTY_OPT_HOST_PIPELINE).  Both
// flags are read by calls on any thread, hence atomic.
std::atomic<int> g_pipeline{0};

// Where a pointer lives.  0 = pageable host memory, 1 = memory a kernel on
// `dev` may access (device or managed), 2 = pinned host memory (its mapped
// device address in *mapped).
int classify(const void *p, int *dev, const void **mapped) {
    cudaPointerAttributes at;
    std::memset(&at, 0, sizeof(at));
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
        *dev = at.device;
        if (mapped) *mapped = p;
        return 1;
    }
    if (at.type == cudaMemoryTypeHost && at.devicePointer && g_zero_copy) {
        if (mapped) *mapped = at.devicePointer;
        return 2;
    }
    return 0;
}

// Cached staging buffers for host-pointer calls, per device (grow-only).
struct Staging {
    double *u = nullptr, *s = nullptr;
    size_t nu = 0, ns = 0;
};
std::map<int, Staging> g_stage;
std::mutex g_stage_mu;

int grow(double **p, size_t *cap, size_t n) {
    if (*cap >= n) return SPAGHETTY_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    if (cudaMalloc((void **)p, n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return SPAGHETTY_ERR_CUDA;
    }
    *cap = n;
    return SPAGHETTY_OK;
}

struct DeviceGuard {
    int old = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&old) != cudaSuccess) { cudaGetLastError(); old = -1; }
        if (dev >= 0 && dev != old) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (old >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != old) cudaSetDevice(old);
    }
};

// Library streams and slab buffer pairs per device for the pipeline.
#define SPG_PIPE_N 3
struct PipeRes {
    cudaStream_t st[SPG_PIPE_N] = {};
    double *in[SPG_PIPE_N] = {}, *out[SPG_PIPE_N] = {};
    size_t cap = 0;
};
std::map<int, PipeRes> g_pipe;

// Host buffers moved in slabs along one index c: slab [c0, c0 + cn) of
// index c is, in the input, `outer_in` rows of cn * inner_in contiguous
// elements (pitch d_c * inner_in) and, in the output, `outer_out` rows of
// cn * inner_out (pitch d_c * inner_out).  Each slab is gathered by a
// pitched 2-D copy into a packed device buffer, sorted there as a smaller
// sort of the same permutation (d_c -> cn), and scattered back by a pitched
// 2-D copy (a sortacc's old output is gathered the same way first).  Slabs
// rotate over SPG_PIPE_N streams, so the upload of one slab, the sort of
// another and the download of a third overlap (the two copy directions run
// on separate copy engines).  The index is the output's slowest (the
// download is contiguous) when its upload rows hold 32 KB, else the input's
// slowest (the upload is contiguous) when its download rows do: measured on
// GB300 at 100^4, pitched copies on both sides, or rows of a few KB, ran at
// 200-250 GB/s against 310 with one side contiguous.  SPAGHETTY_ERR_CONFIG
// when neither qualifies.
int sort_host_pipelined(int rank, const double *u, double *s, const int *dims, const int *perm,
                        double f, double g, int dev, int sms) {
    int64_t n = 1;
    for (int q = 0; q < rank; ++q) n *= dims[q];
    int qpos[SPG_MAXR];                                 // output position of each input index
    for (int q = 0; q < rank; ++q) qpos[perm[q] - 1] = q;
    // slabs of ~32 MB of output, widened until the pitched side's rows hold
    // 32 KB, at most 256 MB, and at least ~4 of them
    const int64_t slab_target = (int64_t)32 << 20, slab_max = (int64_t)256 << 20;
    const int64_t row_min = 4096;                       // elements: 32 KB
    auto slab_of = [&](int k, int64_t row_unit, int64_t *cs_out) {
        const int64_t slice = n / dims[k];
        int64_t cs = std::max<int64_t>(slab_target / (slice * 8), (row_min + row_unit - 1) / row_unit);
        cs = std::min<int64_t>(cs, std::max<int64_t>(1, slab_max / (slice * 8)));
        cs = std::max<int64_t>(1, std::min<int64_t>(cs, dims[k] / 4));
        *cs_out = cs;
        return cs * row_unit;
    };
    int c = -1;
    int64_t best_cs = 0;
    const int a = perm[0] - 1;                          // the output's slowest index
    if (a != rank - 1 && dims[a] >= 4) {
        int64_t inner_in = 1, cs = 0;
        for (int q = a + 1; q < rank; ++q) inner_in *= dims[q];
        if (slab_of(a, inner_in, &cs) >= row_min) {
            c = a;
            best_cs = cs;
        }
    }
    if (c < 0 && qpos[0] != rank - 1 && dims[0] >= 4) {
        int64_t inner_out = 1, cs = 0;
        for (int q = qpos[0] + 1; q < rank; ++q) inner_out *= dims[perm[q] - 1];
        if (slab_of(0, inner_out, &cs) >= row_min) {
            c = 0;
            best_cs = cs;
        }
    }
    if (c < 0) return SPAGHETTY_ERR_CONFIG;
    const int64_t E = dims[c], cs = best_cs;
    int64_t outer_in = 1, inner_in = 1, outer_out = 1, inner_out = 1;
    for (int q = 0; q < c; ++q) outer_in *= dims[q];
    for (int q = c + 1; q < rank; ++q) inner_in *= dims[q];
    for (int q = 0; q < qpos[c]; ++q) outer_out *= dims[perm[q] - 1];
    for (int q = qpos[c] + 1; q < rank; ++q) inner_out *= dims[perm[q] - 1];
    if (E * inner_in * 8 > ((int64_t)1 << 31) || E * inner_out * 8 > ((int64_t)1 << 31))
        return SPAGHETTY_ERR_CONFIG;                  // pitches beyond what 2-D copies take
    const bool acc = g != 0.0;
    PipeRes &pr = g_pipe[dev];
    const size_t need = (size_t)(cs * (n / E));
    if (!pr.st[0]) {
        for (int b = 0; b < SPG_PIPE_N; ++b)
            if (cudaStreamCreateWithFlags(&pr.st[b], cudaStreamNonBlocking) != cudaSuccess) {
                cudaGetLastError();
                return SPAGHETTY_ERR_CUDA;
            }
    }
    if (pr.cap < need) {
        for (int b = 0; b < SPG_PIPE_N; ++b) {
            if (pr.in[b]) cudaFree(pr.in[b]);
            if (pr.out[b]) cudaFree(pr.out[b]);
            pr.in[b] = pr.out[b] = nullptr;
        }
        pr.cap = 0;
        for (int b = 0; b < SPG_PIPE_N; ++b)
            if (cudaMalloc((void **)&pr.in[b], need * 8) != cudaSuccess ||
                cudaMalloc((void **)&pr.out[b], need * 8) != cudaSuccess) {
                cudaGetLastError();
                return SPAGHETTY_ERR_CUDA;
            }
        pr.cap = need;
    }
    int sub[SPG_MAXR];
    for (int q = 0; q < rank; ++q) sub[q] = dims[q];
    int rc = SPAGHETTY_OK;
    int k = 0;
    for (int64_t c0 = 0; c0 < E && rc == SPAGHETTY_OK; c0 += cs, ++k) {
        const int64_t cn = std::min<int64_t>(cs, E - c0);
        const int b = k % SPG_PIPE_N;
        cudaStream_t st = pr.st[b];
        const size_t wi = (size_t)(cn * inner_in * 8), wo = (size_t)(cn * inner_out * 8);
        const size_t pi = (size_t)(E * inner_in * 8), po = (size_t)(E * inner_out * 8);
        if (cudaMemcpy2DAsync(pr.in[b], wi, u + c0 * inner_in, pi, wi, (size_t)outer_in,
                              cudaMemcpyHostToDevice, st) != cudaSuccess) { rc = SPAGHETTY_ERR_CUDA; break; }
        if (acc && cudaMemcpy2DAsync(pr.out[b], wo, s + c0 * inner_out, po, wo, (size_t)outer_out,
                                     cudaMemcpyHostToDevice, st) != cudaSuccess) { rc = SPAGHETTY_ERR_CUDA; break; }
        sub[c] = (int)cn;
        Plan pl;
        rc = make_plan(rank, sub, perm, f, g, sms, &pl, true);
        if (rc) break;
        rc = launch_plan(pl, pr.in[b], pr.out[b], st, dev);
        if (rc) break;
        if (cudaMemcpy2DAsync(s + c0 * inner_out, po, pr.out[b], wo, wo, (size_t)outer_out,
                              cudaMemcpyDeviceToHost, st) != cudaSuccess) { rc = SPAGHETTY_ERR_CUDA; break; }
    }
    for (int b = 0; b < SPG_PIPE_N; ++b)
        if (cudaStreamSynchronize(pr.st[b]) != cudaSuccess) rc = SPAGHETTY_ERR_CUDA;
    if (rc == SPAGHETTY_ERR_CUDA) cudaGetLastError();
    return rc ? rc : take_device_status();
}

int sort_sync(int rank, const double *u, double *s, const int *dims, const int *perm,
              double f, double g) {
    SpgRange range(g == 0.0 ? "tce_sort" : "tce_sortacc");
    Folded fo;
    int rc = spg_fold(rank, dims, perm, &fo);
    if (rc) return rc;
    if (fo.empty) return SPAGHETTY_OK;
    if (!u || !s) return SPAGHETTY_ERR_NULL;
    if (overlaps(u, s, fo.nelem)) return SPAGHETTY_ERR_ALIAS;
    int du = -1, ds = -1;
    const void *mu = nullptr, *ms = nullptr;
    int ku = classify(u, &du, &mu), ks = classify(s, &ds, &ms);
    if (ku < 0 || ks < 0) return SPAGHETTY_ERR_CUDA;
    int dev = ku == 1 ? du : (ks == 1 ? ds : -1);
    if (ku == 1 && ks == 1 && du != ds) return SPAGHETTY_ERR_MEMSPACE;
    DeviceGuard guard(dev);
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return SPAGHETTY_ERR_CUDA; }
    Plan pl;
    // staged sides use cudaMalloc'd buffers (aligned); device sides are the
    // caller's pointers; pinned host sides are used in place, where the bulk
    // tensor copies are not used
    const bool allow_tma = ku != 2 && ks != 2 && (ku == 1 ? aligned16(u) : true) &&
                           (ks == 1 ? aligned16(s) : true);
    rc = make_plan(rank, dims, perm, f, g, device_sms(dev), &pl, allow_tma, ku == 2 || ks == 2);
    if (rc) return rc;
    cudaStream_t st = 0;  // legacy default stream: ordered after prior blocking-stream work
    const size_t n = (size_t)fo.nelem;
    const size_t bytes = n * sizeof(double);
    if (g_pipeline && ku == 2 && ks == 2) {
        std::lock_guard<std::mutex> lk(g_stage_mu);
        if (cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return SPAGHETTY_ERR_CUDA; }
        rc = sort_host_pipelined(rank, u, s, dims, perm, f, g, dev, device_sms(dev));
        if (rc != SPAGHETTY_ERR_CONFIG) return rc;
    }
    if (ku != 0 && ks != 0) {
        rc = launch_plan(pl, (const double *)mu, (double *)ms, st, dev);
        if (rc) return rc;
        if (cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return SPAGHETTY_ERR_CUDA; }
        return take_device_status();
    }
    std::lock_guard<std::mutex> lk(g_stage_mu);
    Staging &sg = g_stage[dev];
    const double *du_ptr = ku == 2 ? (const double *)mu : u;
    double *ds_ptr = ks == 2 ? (double *)ms : s;
    if (ku == 0) {
        if ((rc = grow(&sg.u, &sg.nu, n))) return rc;
        if (cudaMemcpyAsync(sg.u, u, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) goto cuda_fail;
        du_ptr = sg.u;
    }
    if (ks == 0) {
        if ((rc = grow(&sg.s, &sg.ns, n))) return rc;
        if (spg_op_class(pl.op) != 0)
            if (cudaMemcpyAsync(sg.s, s, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) goto cuda_fail;
        ds_ptr = sg.s;
    }
    rc = launch_plan(pl, du_ptr, ds_ptr, st, dev);
    if (rc) {
        cudaStreamSynchronize(st);
        return rc;
    }
    if (ks == 0)
        if (cudaMemcpyAsync(s, sg.s, bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess) goto cuda_fail;
    if (cudaStreamSynchronize(st) != cudaSuccess) goto cuda_fail;
    return take_device_status();
cuda_fail:
    cudaGetLastError();
    cudaStreamSynchronize(st);
    cudaGetLastError();
    return SPAGHETTY_ERR_CUDA;
}

void report(const char *who, int rc, int rank, const int *perm) {
    if (rc == SPAGHETTY_OK) return;
    if (rc == SPAGHETTY_ERR_PERM) {
        // the reference's only diagnostic (trunk/tce_sort4_switch.F:58-60)
        std::fprintf(stderr, " something is wrong...\n");
    }
    std::fprintf(stderr, "spaghetty_gb300: %s: %s (permutation", who, spaghetty_error_string(rc));
    for (int q = 0; q < rank; ++q) std::fprintf(stderr, " %d", perm[q]);
    std::fprintf(stderr, ")\n");
}

int call_r(const char *who, bool print, int rank, const double *u, double *s, const int *dims,
           const int *perm, double f, double g) {
    int rc = sort_sync(rank, u, s, dims, perm, f, g);
    record(rc);
    if (print) report(who, rc, rank, perm);
    return rc;
}

// Tune file: one winner per line,
//   gpu_name|sm_count|D0,D1,..|P0,P1,..|op_class|box0,box1,..|threads|ept|stages
// (folded dims and 0-based folded permutation, as the autotuner writes them),
// and one line per size bucket of the batched kernel,
//   gpu_name|sm_count|batch|rank|ext_lo|ext_hi|run_in|run_out|volume
int load_tune_file(const char *path, bool only_this_gpu) {
    FILE *fh = std::fopen(path, "r");
    if (!fh) return -1;
    char name[256] = {0};
    int sms = 0, have_dev = 0;
    if (only_this_gpu) {
        int dev = 0;
        cudaDeviceProp prop;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
            std::snprintf(name, sizeof(name), "%s", prop.name);
            sms = prop.multiProcessorCount;
            have_dev = 1;
        } else {
            cudaGetLastError();
        }
    }
    int installed = 0;
    char line[1024];
    while (std::fgets(line, sizeof(line), fh)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        char *fields[9];
        int nf = 0;
        char *save = nullptr;
        for (char *tok = strtok_r(line, "|\n", &save); tok && nf < 9; tok = strtok_r(nullptr, "|\n", &save))
            fields[nf++] = tok;
        if (nf != 9) continue;
        if (only_this_gpu && (!have_dev || std::strcmp(fields[0], name) != 0 || std::atoi(fields[1]) != sms))
            continue;
        if (std::strcmp(fields[2], "batch") == 0) {
            if (spaghetty_batch_tune_set(std::atoi(fields[3]), std::atoi(fields[4]), std::atoi(fields[5]),
                                         std::atoi(fields[6]), std::atoi(fields[7]),
                                         std::atoi(fields[8])) == SPAGHETTY_OK)
                ++installed;
            continue;
        }
        int D[SPG_MAXR], P[SPG_MAXR], B[SPG_MAXR];
        auto parse = [](char *txt, int *out) {
            int n = 0;
            char *sv = nullptr;
            for (char *t = strtok_r(txt, ",", &sv); t && n < SPG_MAXR; t = strtok_r(nullptr, ",", &sv))
                out[n++] = std::atoi(t);
            return n;
        };
        const int r = parse(fields[2], D);
        if (parse(fields[3], P) != r || parse(fields[5], B) != r || r < 2) continue;
        for (int q = 0; q < r; ++q) P[q] += 1;   // the drop-in convention is 1-based
        const int cls = std::atoi(fields[4]);
        if (spaghetty_tune_set(r, D, P, cls, B, std::atoi(fields[6]), std::atoi(fields[7]),
                               std::atoi(fields[8])) == SPAGHETTY_OK)
            ++installed;
    }
    std::fclose(fh);
    return installed;
}

void autoload_tune_file() {
    static std::once_flag once;
    std::call_once(once, [] {
        const char *env = std::getenv("SPAGHETTY_GB300_TUNE_FILE");
        if (env && !*env) return;             // explicitly disabled
        std::string path;
        if (env) {
            path = env;
        } else {
            Dl_info info;
            if (!dladdr((void *)&autoload_tune_file, &info) || !info.dli_fname) return;
            path = info.dli_fname;
            const size_t slash = path.rfind('/');
            path = (slash == std::string::npos ? std::string(".") : path.substr(0, slash)) +
                   "/tune_cache.txt";
        }
        load_tune_file(path.c_str(), true);
    });
}

}  // namespace

// Installs the tune file beside the library once per process (batch.cu calls
// it before planning a batch, so that its size-bucket rules apply).
void spg_autoload_tune() { autoload_tune_file(); }

// Tensor-map encoding and the kernels' status word, for fused.cu.
int spg_encode_map(CUtensorMap *m, const double *ptr, const uint64_t *dim, const uint64_t *stride,
                   const uint32_t *box, int swizzle128) {
    return encode_map(m, ptr, dim, stride, box, swizzle128 != 0);
}
int *spg_status_word() { return status_word_dev(); }

// The asynchronous sort for pointers already known to be device memory of
// device `dev`, the current device of the calling thread (the batched
// plain path, which validated them when the batch was created).
// Whether the single-sort plan of this problem on these buffers is the
// TMA-staged kernel (batch.cu runs such large sorts as their own launch).
bool spg_plan_is_tma(int dev, int rank, const int *dims, const int *perm, double factor, double acc_factor,
                     const double *unsorted, const double *sorted) {
    Plan pl;
    return make_plan(rank, dims, perm, factor, acc_factor, device_sms(dev), &pl,
                     aligned16(unsorted) && aligned16(sorted)) == SPAGHETTY_OK &&
           pl.kind == KIND_TMA;
}

int spg_sort_async_on(int dev, int rank, const double *unsorted, double *sorted, const int *dims,
                      const int *perm, double factor, double acc_factor, void *stream) {
    Folded fo;
    int rc = spg_fold(rank, dims, perm, &fo);
    if (rc) return rc;
    if (fo.empty) return SPAGHETTY_OK;
    Plan pl;
    rc = make_plan(rank, dims, perm, factor, acc_factor, device_sms(dev), &pl,
                   aligned16(unsorted) && aligned16(sorted));
    if (rc) return rc;
    return launch_plan(pl, unsorted, sorted, (cudaStream_t)stream, dev);
}

// ===========================================================================
// Host replay of one launch's index arithmetic (the kernels' own spg_box /
// spg_walk), moving element indices instead of values: every global read
// and write inside the tensors, every staging-tile slot inside smem_elems,
// and every output element written exactly once, from the input element the
// permutation maps to it.  Kinds: direct (each element read and written by
// one thread), tiled and warp (staged through a tile in input order, read
// back in output order).  stats (may be NULL): reads, writes, boxes, tile
// elements.  Tensors up to 2^27 elements; SPAGHETTY_ERR_CONFIG on any
// violation (and above that size).
int spg_replay_params(const KParams &kp, const Folded &fo, int kind, int64_t smem_elems, int64_t *stats) {
    const int64_t n = fo.nelem;
    if (n > ((int64_t)1 << 27)) return SPAGHETTY_ERR_CONFIG;
    const int R = fo.rank;
    int64_t istr[SPG_MAXR];
    {
        int64_t s = 1;
        for (int d = R - 1; d >= 0; --d) { istr[d] = s; s *= fo.D[d]; }
    }
    std::vector<int64_t> got((size_t)n, -1);
    std::vector<int64_t> sm((size_t)std::max<int64_t>(smem_elems, 1), -2);
    int64_t reads = 0, writes = 0;
    for (uint32_t t = 0; t < kp.ntiles; ++t) {
        int64_t ib, ob;
        uint32_t limA, limB;
        spg_box(kp, t, ib, ob, limA, limB);
        for (uint32_t e = 0; e < (uint32_t)kp.vol; ++e) {
            int32_t a, b, lin;
            uint32_t pk;
            spg_walk(kp.ld, e, a, b, lin, pk);
            const bool v = spg_valid(pk, limA, limB);
            if (kind == KIND_DIRECT) {
                if (!v) continue;
                const int64_t src = ib + a, dst = ob + b;
                if (src < 0 || src >= n || dst < 0 || dst >= n) return SPAGHETTY_ERR_CONFIG;
                if (got[(size_t)dst] != -1) return SPAGHETTY_ERR_CONFIG;
                got[(size_t)dst] = src;
                ++reads; ++writes;
            } else {
                const int64_t w = (int64_t)e + (kp.pad ? (int64_t)e / kp.pad : 0);
                if (w < 0 || w >= smem_elems) return SPAGHETTY_ERR_CONFIG;
                if (v) {
                    const int64_t src = ib + a;
                    if (src < 0 || src >= n) return SPAGHETTY_ERR_CONFIG;
                    sm[(size_t)w] = src;
                    ++reads;
                } else {
                    sm[(size_t)w] = -3;
                }
            }
        }
        if (kind == KIND_TILED || kind == KIND_WARP) {
            for (uint32_t e = 0; e < (uint32_t)kp.vol; ++e) {
                int32_t a, b, lin;
                uint32_t pk;
                spg_walk(kp.st, e, a, b, lin, pk);
                if (!spg_valid(pk, limA, limB)) continue;
                const int64_t r = (int64_t)lin + (kp.pad ? (int64_t)lin / kp.pad : 0);
                if (r < 0 || r >= smem_elems) return SPAGHETTY_ERR_CONFIG;
                const int64_t dst = ob + a;
                if (dst < 0 || dst >= n) return SPAGHETTY_ERR_CONFIG;
                if (got[(size_t)dst] != -1 || sm[(size_t)r] < 0) return SPAGHETTY_ERR_CONFIG;
                got[(size_t)dst] = sm[(size_t)r];
                ++writes;
            }
        }
    }
    // every output element written once, from the input element the
    // permutation maps to it
    for (int64_t o = 0; o < n; ++o) {
        int64_t rem = o, src = 0;
        for (int q = R - 1; q >= 0; --q) {
            const int64_t ext = fo.D[fo.P[q]];
            src += (rem % ext) * istr[fo.P[q]];
            rem /= ext;
        }
        if (got[(size_t)o] != src) return SPAGHETTY_ERR_CONFIG;
    }
    if (stats) {
        stats[0] = reads;
        stats[1] = writes;
        stats[2] = kp.ntiles;
        stats[3] = smem_elems;
    }
    return SPAGHETTY_OK;
}

extern "C" {

int spaghetty_tune_load(const char *path) {
    if (!path) return -SPAGHETTY_ERR_NULL;
    return load_tune_file(path, true);
}

const char *spaghetty_error_string(int code) {
    switch (code) {
        case SPAGHETTY_OK: return "ok";
        case SPAGHETTY_ERR_RANK: return "rank outside 1..8";
        case SPAGHETTY_ERR_PERM: return "permutation is not a bijection of 1..rank";
        case SPAGHETTY_ERR_DIMS: return "negative dimension";
        case SPAGHETTY_ERR_OVERFLOW: return "element count overflows int64";
        case SPAGHETTY_ERR_NULL: return "null pointer";
        case SPAGHETTY_ERR_ALIAS: return "unsorted and sorted overlap";
        case SPAGHETTY_ERR_CUDA: return "CUDA runtime error";
        case SPAGHETTY_ERR_MEMSPACE: return "pointers on different devices";
        case SPAGHETTY_ERR_CONFIG: return "invalid kernel configuration";
        case SPAGHETTY_ERR_BATCH: return "invalid batch entry";
        case SPAGHETTY_ERR_DEVICE: return "device status word reported an error";
        case SPAGHETTY_ERR_NOKERNEL: return "no compiled kernel variant fits";
        case SPAGHETTY_ERR_TOO_LARGE: return "batch exceeds the fixed scratch limits of the no-allocation entry";
        default: return "unknown error";
    }
}

int spaghetty_last_error(void) { return g_last_error; }

int spaghetty_last_cuda_error(void) { return g_last_cuda.load(); }

const char *spaghetty_last_cuda_error_string(void) {
    const int e = g_last_cuda.load();
    if (e < 0) return "tensor-map encoding rejected its arguments";
    return cudaGetErrorString((cudaError_t)e);
}

int spaghetty_set_option(int option, int value) {
    if (option == SPAGHETTY_OPT_HOST_ZERO_COPY) {
        g_zero_copy = value ? 1 : 0;
        return SPAGHETTY_OK;
    }
    if (option == SPAGHETTY_OPT_HOST_PIPELINE) {
        g_pipeline = value ? 1 : 0;
        return SPAGHETTY_OK;
    }
    if (option == SPAGHETTY_OPT_WARP_TR) {
        if (value < 0 || value > 2) return SPAGHETTY_ERR_CONFIG;
        std::lock_guard<std::mutex> lk(g_plans_mu);
        g_warp_tr = value;
        g_plans.clear();
        return SPAGHETTY_OK;
    }
    if (option == SPAGHETTY_OPT_TMA_SKEW) {
        std::lock_guard<std::mutex> lk(g_plans_mu);
        g_tma_skew = value ? 1 : 0;
        g_plans.clear();
        return SPAGHETTY_OK;
    }
    if (option == SPAGHETTY_OPT_BATCH_OWN_MIN || option == SPAGHETTY_OPT_BATCH_OWN_KINDS)
        return spg_batch_option(option, value);
    return SPAGHETTY_ERR_CONFIG;
}

int spaghetty_device_status(void) {
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    return take_device_status();
}

const char *spaghetty_version(void) { return "spaghetty_gb300 0.1 (sm_103a)"; }

int spaghetty_selftest(void) { return spg_selftest_host(); }

int spaghetty_sort_async(int rank, const double *unsorted, double *sorted, const int *dims,
                         const int *perm, double factor, double acc_factor, void *stream) {
    SpgRange range("spaghetty_sort_async");
    Folded fo;
    int rc = spg_fold(rank, dims, perm, &fo);
    if (rc) return record(rc);
    if (fo.empty) return record(SPAGHETTY_OK);
    if (!unsorted || !sorted) return record(SPAGHETTY_ERR_NULL);
    if (overlaps(unsorted, sorted, fo.nelem)) return record(SPAGHETTY_ERR_ALIAS);
    // the asynchronous form works on device (or managed) memory of one
    // device, and runs on that device whatever the calling thread's current
    // device is: setting it also binds its context to a thread that has
    // none yet (a worker thread of the caller), which the tensor-map
    // encoding needs
    int du = -1, ds = -1;
    if (classify(unsorted, &du, nullptr) != 1 || classify(sorted, &ds, nullptr) != 1 || du != ds)
        return record(SPAGHETTY_ERR_MEMSPACE);
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) cudaGetLastError();
    cudaError_t e = cudaSetDevice(du);
    if (e != cudaSuccess) return record(cuda_fail(e));
    Plan pl;
    rc = make_plan(rank, dims, perm, factor, acc_factor, device_sms(du), &pl,
                   aligned16(unsorted) && aligned16(sorted));
    if (!rc) rc = launch_plan(pl, unsorted, sorted, (cudaStream_t)stream, du);
    if (cur >= 0 && cur != du) cudaSetDevice(cur);
    return record(rc);
}

int spaghetty_sort(int rank, const double *unsorted, double *sorted, const int *dims,
                   const int *perm, double factor, double acc_factor) {
    return record(sort_sync(rank, unsorted, sorted, dims, perm, factor, acc_factor));
}

int spaghetty_plan_query(int rank, const int *dims, const int *perm, int op,
                         spaghetty_plan_info *out) {
    if (!out) return SPAGHETTY_ERR_NULL;
    std::memset(out, 0, sizeof(*out));
    const double f = 0.5, g = op == 0 ? 0.0 : (op == 1 ? 1.0 : 2.0);
    Plan pl;
    int rc = make_plan(rank, dims, perm, f, g, 152, &pl);
    if (rc) return rc;
    out->kind = pl.kind;
    out->rank = pl.fo.rank;
    for (int d = 0; d < pl.fo.rank; ++d) {
        out->dims[d] = pl.fo.D[d];
        out->perm[d] = pl.fo.P[d];
        out->box[d] = pl.box[d];
    }
    out->threads = pl.threads;
    out->ept = pl.ept;
    out->ntiles = pl.kp.ntiles;
    out->run_in = pl.run_in;
    out->run_out = pl.run_out;
    out->pad_period = pl.kind == KIND_TMA ? pl.sk_mul : pl.kp.pad;
    out->masked = pl.masked;
    out->grid = 0;
    out->vec = 0;
    out->stages = pl.stages;
    out->smem_bytes = pl.smem_bytes;
    return SPAGHETTY_OK;
}

// Replays the TMA kernel's data movement on the host: box coordinates from
// spg_tma_coords, element positions inside the two tensor maps' boxes
// (clipped exactly as the hardware clips: out-of-range loads read zero,
// out-of-range stores are dropped), and the permute step's table.
static int verify_tma(const Plan &pl, int64_t *stats) {
    TmaLayout tl;
    if (spg_tma_layout(pl, pl.stages, &tl)) return SPAGHETTY_ERR_CONFIG;
    const KParams &kp = pl.kp;
    const Folded &fo = pl.fo;
    const int64_t n = fo.nelem;
    if (n > ((int64_t)1 << 27)) return SPAGHETTY_ERR_CONFIG;
    if ((int64_t)kp.vol * 8 > tl.tp.in_bytes || pl.threads * pl.ept < kp.vol) return SPAGHETTY_ERR_CONFIG;
    const int R = fo.rank;
    int64_t istr[SPG_MAXR];
    {
        int64_t s = 1;
        for (int d = R - 1; d >= 0; --d) { istr[d] = s; s *= fo.D[d]; }
    }
    // the permute step's slots (spg_tma_slot, skew included) must cover
    // every tile element exactly once; slot_in[e] = the input-tile element
    // read for output-tile element e
    std::vector<int32_t> slot_in((size_t)kp.vol, -1);
    for (uint32_t s = 0; s < (uint32_t)kp.vol; ++s) {
        uint32_t e;
        int32_t lin;
        spg_tma_slot(kp, tl.tp, s, e, lin);
        if (e >= (uint32_t)kp.vol || slot_in[e] != -1) return SPAGHETTY_ERR_CONFIG;
        if (tl.tp.sk_mul && (e > 0xFFFFu || lin < 0 || lin > 0xFFFF)) return SPAGHETTY_ERR_CONFIG;
        slot_in[e] = lin;
    }
    std::vector<int64_t> got((size_t)n, -1);
    int64_t writes = 0;
    for (uint32_t t = 0; t < kp.ntiles; ++t) {
        int32_t ci[5], co[5];
        spg_tma_coords(kp, tl.tp, t, ci, co);
        for (int m = 0; m < 5; ++m)
            if (ci[m] < 0 || co[m] < 0 || (uint64_t)ci[m] >= tl.in_dim[m] || (uint64_t)co[m] >= tl.out_dim[m])
                return SPAGHETTY_ERR_CONFIG;   // every box starts inside both tensors
        if ((ci[0] * 8) % 16 || (co[0] * 8) % 16) return SPAGHETTY_ERR_CONFIG;
        for (uint32_t e = 0; e < (uint32_t)kp.vol; ++e) {
            // output position of tile element e (dense over the output box)
            int64_t rem = e, og = 0;
            bool oin = true;
            for (int m = 0; m < 5; ++m) {
                const int64_t c = rem % tl.out_box[m];
                rem /= tl.out_box[m];
                const int64_t x = co[m] + c;
                if ((uint64_t)x >= tl.out_dim[m]) oin = false;
                og += x * (int64_t)(tl.out_stride[m] / 8);
            }
            // input position of the element the permute step reads
            const int32_t lin = slot_in[e];
            if (lin < 0 || lin >= kp.vol) return SPAGHETTY_ERR_CONFIG;
            int64_t remi = lin, ig = 0;
            bool iin = true;
            for (int m = 0; m < 5; ++m) {
                const int64_t c = remi % tl.in_box[m];
                remi /= tl.in_box[m];
                const int64_t x = ci[m] + c;
                if ((uint64_t)x >= tl.in_dim[m]) iin = false;
                ig += x * (int64_t)(tl.in_stride[m] / 8);
            }
            if (!oin) continue;
            if (!iin || og < 0 || og >= n || ig < 0 || ig >= n) return SPAGHETTY_ERR_CONFIG;
            if (got[(size_t)og] != -1) return SPAGHETTY_ERR_CONFIG;
            got[(size_t)og] = ig;
            ++writes;
        }
    }
    for (int64_t o = 0; o < n; ++o) {
        int64_t rem = o, src = 0;
        for (int q = R - 1; q >= 0; --q) {
            const int64_t ext = fo.D[fo.P[q]];
            src += (rem % ext) * istr[fo.P[q]];
            rem /= ext;
        }
        if (got[(size_t)o] != src) return SPAGHETTY_ERR_CONFIG;
    }
    if (stats) {
        stats[0] = writes;
        stats[1] = writes;
        stats[2] = kp.ntiles;
        stats[3] = tl.tp.stage_bytes / 8;
    }
    return SPAGHETTY_OK;
}

int spaghetty_plan_verify(int rank, const int *dims, const int *perm, int op, int num_sms,
                          int64_t *stats) {
    // Replays, on the host, the index arithmetic of the exact KParams a
    // launch would receive (spg_box / spg_walk are the kernels' own
    // functions), moving element INDICES instead of values.
    const double f = 0.5, g = op == 0 ? 0.0 : (op == 1 ? 1.0 : 2.0);
    Plan pl;
    int rc = make_plan(rank, dims, perm, f, g, num_sms > 0 ? num_sms : 152, &pl);
    if (rc) return rc;
    if (stats) for (int q = 0; q < 4; ++q) stats[q] = 0;
    if (pl.kind == KIND_EMPTY || pl.kind == KIND_FLAT) return SPAGHETTY_OK;
    if (pl.kind == KIND_TMA) return verify_tma(pl, stats);
    // one staging tile: the whole buffer of the register-staged kernel, one
    // stage of the pipelined kernel
    // (the warp-shuffle transpose's "tile" is the warp's registers, vol
    // elements in input order, with no padding)
    const int64_t smem_elems = pl.kind == KIND_WARP ? (int64_t)pl.kp.vol
                               : pl.stages ? (int64_t)pl.kp.stage
                                           : pl.smem_bytes / (int64_t)sizeof(double);
    if (pl.stages && (int64_t)pl.stages * pl.kp.stage * 8 > pl.smem_bytes) return SPAGHETTY_ERR_CONFIG;
    return spg_replay_params(pl.kp, pl.fo, pl.kind, smem_elems, stats);
}

int spaghetty_tune_set(int rank, const int *dims, const int *perm, int op, const int *box,
                       int threads, int ept, int stages) {
    if (!box) {
        {
            std::lock_guard<std::mutex> lk(g_mu);
            g_tune.clear();
        }
        std::lock_guard<std::mutex> lk2(g_plans_mu);
        g_plans.clear();
        return SPAGHETTY_OK;
    }
    Folded fo;
    int rc = spg_fold(rank, dims, perm, &fo);
    if (rc) return rc;
    if (fo.empty || fo.rank < 2) return SPAGHETTY_ERR_CONFIG;
    const bool tma = stages == 12 || stages == 13 || stages == 14 || stages == 16;
    if (stages == 20) {
        // the warp-shuffle transpose: its box is fixed by the problem
        Plan wp;
        const int opw = op == 0 ? OP_SORT_ANY : (op == 1 ? OP_ACC_ANY : OP_GEN);
        if (threads != 256 || make_warp_plan(fo, opw, 0.5, 1.0, 152, &wp) != SPAGHETTY_OK || wp.ept != ept)
            return SPAGHETTY_ERR_CONFIG;
        TuneOverride ov;
        for (int d = 0; d < SPG_MAXR; ++d) ov.box[d] = d < fo.rank ? wp.box[d] : 1;
        ov.threads = 256;
        ov.ept = ept;
        ov.stages = 20;
        {
            std::lock_guard<std::mutex> lk(g_mu);
            g_tune[tune_key(fo, opw)] = ov;
        }
        std::lock_guard<std::mutex> lk2(g_plans_mu);
        g_plans.clear();
        return SPAGHETTY_OK;
    }
    if (tma) {
        if ((threads != 128 && threads != 256) || (ept != 8 && ept != 16)) return SPAGHETTY_ERR_CONFIG;
    } else {
        if (threads != 128 && threads != 256 && threads != 512) return SPAGHETTY_ERR_CONFIG;
        if (ept != 1 && ept != 2 && ept != 4 && ept != 8) return SPAGHETTY_ERR_CONFIG;
        if (stages != 0 && stages != 2 && stages != 3) return SPAGHETTY_ERR_CONFIG;
        if (stages && ept < 2) return SPAGHETTY_ERR_CONFIG;
    }
    const int opc = op == 0 ? OP_SORT_ANY : (op == 1 ? OP_ACC_ANY : OP_GEN);
    Plan pl;
    rc = spg_plan(fo, opc, box, tma ? 256 : threads, tma ? 16 : ept, tma ? 0 : stages, 152, &pl);
    if (rc) return rc;
    rc = spg_build_params(&pl, 0.5, 1.0);
    if (rc) return rc;
    if (tma) {
        TmaLayout tl;
        if ((pl.kind != KIND_TILED && pl.kind != KIND_DIRECT) || threads * ept < pl.kp.vol ||
            spg_tma_layout(pl, stages - 10, &tl) ||
            tma_smem_bytes(tl, stages - 10) > kMaxSmemPerBlock)
            return SPAGHETTY_ERR_CONFIG;
    }
    TuneOverride ov;
    for (int d = 0; d < SPG_MAXR; ++d) ov.box[d] = d < fo.rank ? box[d] : 1;
    ov.threads = threads;
    ov.ept = ept;
    ov.stages = stages;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_tune[tune_key(fo, opc)] = ov;
    }
    std::lock_guard<std::mutex> lk2(g_plans_mu);
    g_plans.clear();
    return SPAGHETTY_OK;
}

// ---- NWChem drop-ins ------------------------------------------------------
#define SPG_R4_ARGS                                                                        \
    const double *unsorted, double *sorted, const int *a, const int *b, const int *c,       \
        const int *d, const int *i, const int *j, const int *k, const int *l,               \
        const double *factor
#define SPG_R6_ARGS                                                                        \
    const double *unsorted, double *sorted, const int *a, const int *b, const int *c,       \
        const int *d, const int *e, const int *f, const int *i, const int *j, const int *k, \
        const int *l, const int *m, const int *n, const double *factor
#define SPG_R8_ARGS                                                                        \
    const double *unsorted, double *sorted, const int *a, const int *b, const int *c,       \
        const int *d, const int *e, const int *f, const int *g, const int *h, const int *i, \
        const int *j, const int *k, const int *l, const int *m, const int *n, const int *o, \
        const int *p, const double *factor

static int r2(const char *w, bool pr, const double *u, double *s, const int *a, const int *b,
              const int *i, const int *j, const double *fac, double g) {
    const int dm[2] = {*a, *b}, pm[2] = {*i, *j};
    return call_r(w, pr, 2, u, s, dm, pm, *fac, g);
}
static int r4(const char *w, bool pr, SPG_R4_ARGS, double g) {
    const int dm[4] = {*a, *b, *c, *d}, pm[4] = {*i, *j, *k, *l};
    return call_r(w, pr, 4, unsorted, sorted, dm, pm, *factor, g);
}
static int r6(const char *w, bool pr, SPG_R6_ARGS, double g) {
    const int dm[6] = {*a, *b, *c, *d, *e, *f}, pm[6] = {*i, *j, *k, *l, *m, *n};
    return call_r(w, pr, 6, unsorted, sorted, dm, pm, *factor, g);
}
static int r8(const char *w, bool pr, SPG_R8_ARGS, double gg) {
    const int dm[8] = {*a, *b, *c, *d, *e, *f, *g, *h}, pm[8] = {*i, *j, *k, *l, *m, *n, *o, *p};
    return call_r(w, pr, 8, unsorted, sorted, dm, pm, *factor, gg);
}

void tce_sort_2(const double *u, double *s, const int *a, const int *b, const int *i, const int *j, const double *f) { r2("tce_sort_2", true, u, s, a, b, i, j, f, 0.0); }
void tce_sort_2_(const double *u, double *s, const int *a, const int *b, const int *i, const int *j, const double *f) { r2("tce_sort_2", true, u, s, a, b, i, j, f, 0.0); }
void tce_sortacc_2(const double *u, double *s, const int *a, const int *b, const int *i, const int *j, const double *f) { r2("tce_sortacc_2", true, u, s, a, b, i, j, f, 1.0); }
void tce_sortacc_2_(const double *u, double *s, const int *a, const int *b, const int *i, const int *j, const double *f) { r2("tce_sortacc_2", true, u, s, a, b, i, j, f, 1.0); }

void tce_sort_4(SPG_R4_ARGS) { r4("tce_sort_4", true, unsorted, sorted, a, b, c, d, i, j, k, l, factor, 0.0); }
void tce_sort_4_(SPG_R4_ARGS) { r4("tce_sort_4", true, unsorted, sorted, a, b, c, d, i, j, k, l, factor, 0.0); }
void tce_sortacc_4(SPG_R4_ARGS) { r4("tce_sortacc_4", true, unsorted, sorted, a, b, c, d, i, j, k, l, factor, 1.0); }
void tce_sortacc_4_(SPG_R4_ARGS) { r4("tce_sortacc_4", true, unsorted, sorted, a, b, c, d, i, j, k, l, factor, 1.0); }
int tce_sort_4_status(SPG_R4_ARGS) { return r4("tce_sort_4", false, unsorted, sorted, a, b, c, d, i, j, k, l, factor, 0.0); }
int tce_sortacc_4_status(SPG_R4_ARGS) { return r4("tce_sortacc_4", false, unsorted, sorted, a, b, c, d, i, j, k, l, factor, 1.0); }

void tce_sort_6(SPG_R6_ARGS) { r6("tce_sort_6", true, unsorted, sorted, a, b, c, d, e, f, i, j, k, l, m, n, factor, 0.0); }
void tce_sort_6_(SPG_R6_ARGS) { r6("tce_sort_6", true, unsorted, sorted, a, b, c, d, e, f, i, j, k, l, m, n, factor, 0.0); }
void tce_sortacc_6(SPG_R6_ARGS) { r6("tce_sortacc_6", true, unsorted, sorted, a, b, c, d, e, f, i, j, k, l, m, n, factor, 1.0); }
void tce_sortacc_6_(SPG_R6_ARGS) { r6("tce_sortacc_6", true, unsorted, sorted, a, b, c, d, e, f, i, j, k, l, m, n, factor, 1.0); }
int tce_sort_6_status(SPG_R6_ARGS) { return r6("tce_sort_6", false, unsorted, sorted, a, b, c, d, e, f, i, j, k, l, m, n, factor, 0.0); }
int tce_sortacc_6_status(SPG_R6_ARGS) { return r6("tce_sortacc_6", false, unsorted, sorted, a, b, c, d, e, f, i, j, k, l, m, n, factor, 1.0); }

void tce_sort_8(SPG_R8_ARGS) { r8("tce_sort_8", true, unsorted, sorted, a, b, c, d, e, f, g, h, i, j, k, l, m, n, o, p, factor, 0.0); }
void tce_sort_8_(SPG_R8_ARGS) { r8("tce_sort_8", true, unsorted, sorted, a, b, c, d, e, f, g, h, i, j, k, l, m, n, o, p, factor, 0.0); }
void tce_sortacc_8(SPG_R8_ARGS) { r8("tce_sortacc_8", true, unsorted, sorted, a, b, c, d, e, f, g, h, i, j, k, l, m, n, o, p, factor, 1.0); }
void tce_sortacc_8_(SPG_R8_ARGS) { r8("tce_sortacc_8", true, unsorted, sorted, a, b, c, d, e, f, g, h, i, j, k, l, m, n, o, p, factor, 1.0); }

// ---- -i8 shims: NWChem built with 8-byte default integers passes dims and
// permutation as int64 (trunk/generator2.py:926-932 lists the reference's
// compiler flag tables; the Fortran callers are unchanged).  Values must fit
// 32 bits; anything larger is rejected as bad dims.
static bool narrow(const int64_t *const *src, int n, int *dst) {
    for (int q = 0; q < n; ++q) {
        if (!src[q]) return false;
        const int64_t v = *src[q];
        if (v < INT32_MIN || v > INT32_MAX) return false;
        dst[q] = (int)v;
    }
    return true;
}
static int r4_i8(const char *w, bool pr, const double *u, double *s, const int64_t *a, const int64_t *b,
                 const int64_t *c, const int64_t *d, const int64_t *i, const int64_t *j, const int64_t *k,
                 const int64_t *l, const double *f, double g) {
    const int64_t *src[8] = {a, b, c, d, i, j, k, l};
    int v[8];
    if (!narrow(src, 8, v)) {
        record(SPAGHETTY_ERR_DIMS);
        if (pr) std::fprintf(stderr, "spaghetty_gb300: %s: dims or permutation out of range\n", w);
        return SPAGHETTY_ERR_DIMS;
    }
    return call_r(w, pr, 4, u, s, v, v + 4, *f, g);
}
static int r6_i8(const char *w, bool pr, const double *u, double *s, const int64_t *a, const int64_t *b,
                 const int64_t *c, const int64_t *d, const int64_t *e, const int64_t *ff, const int64_t *i,
                 const int64_t *j, const int64_t *k, const int64_t *l, const int64_t *m, const int64_t *n,
                 const double *f, double g) {
    const int64_t *src[12] = {a, b, c, d, e, ff, i, j, k, l, m, n};
    int v[12];
    if (!narrow(src, 12, v)) {
        record(SPAGHETTY_ERR_DIMS);
        if (pr) std::fprintf(stderr, "spaghetty_gb300: %s: dims or permutation out of range\n", w);
        return SPAGHETTY_ERR_DIMS;
    }
    return call_r(w, pr, 6, u, s, v, v + 6, *f, g);
}
#define SPG_I8_R4 const double *u, double *s, const int64_t *a, const int64_t *b, const int64_t *c, \
    const int64_t *d, const int64_t *i, const int64_t *j, const int64_t *k, const int64_t *l, const double *f
#define SPG_I8_R6 const double *u, double *s, const int64_t *a, const int64_t *b, const int64_t *c, \
    const int64_t *d, const int64_t *e, const int64_t *ff, const int64_t *i, const int64_t *j, \
    const int64_t *k, const int64_t *l, const int64_t *m, const int64_t *n, const double *f
void tce_sort_4_i8(SPG_I8_R4) { r4_i8("tce_sort_4", true, u, s, a, b, c, d, i, j, k, l, f, 0.0); }
void tce_sort_4_i8_(SPG_I8_R4) { r4_i8("tce_sort_4", true, u, s, a, b, c, d, i, j, k, l, f, 0.0); }
void tce_sortacc_4_i8(SPG_I8_R4) { r4_i8("tce_sortacc_4", true, u, s, a, b, c, d, i, j, k, l, f, 1.0); }
void tce_sortacc_4_i8_(SPG_I8_R4) { r4_i8("tce_sortacc_4", true, u, s, a, b, c, d, i, j, k, l, f, 1.0); }
void tce_sort_6_i8(SPG_I8_R6) { r6_i8("tce_sort_6", true, u, s, a, b, c, d, e, ff, i, j, k, l, m, n, f, 0.0); }
void tce_sort_6_i8_(SPG_I8_R6) { r6_i8("tce_sort_6", true, u, s, a, b, c, d, e, ff, i, j, k, l, m, n, f, 0.0); }
void tce_sortacc_6_i8(SPG_I8_R6) { r6_i8("tce_sortacc_6", true, u, s, a, b, c, d, e, ff, i, j, k, l, m, n, f, 1.0); }
void tce_sortacc_6_i8_(SPG_I8_R6) { r6_i8("tce_sortacc_6", true, u, s, a, b, c, d, e, ff, i, j, k, l, m, n, f, 1.0); }

}  // extern "C"
