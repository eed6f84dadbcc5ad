// batch.cu -- many independent sorts in ONE persistent kernel launch.
//
// A CCSD/CCSD(T) sweep issues thousands of uneven tce_sort_4/6 calls (the
// triples code applies nine sortaccs to every t3 tile,
// branches/spaghetty2/ccsd_t_tce_sort_list.txt).  One launch per call pays the
// launch gap and a grid tail every time.  Here the host plans every sort once
// (spg_plan_batch: one CTA shape for all), cuts each sort's boxes into work
// units of 4K-64K elements (longer in larger batches), and uploads the job
// records plus a unit -> job map.
// The persistent kernel's CTAs take units from an atomic counter; a CTA
// rebuilds its per-element tables only when it moves to another sort.  The
// launch (a counter reset and one kernel) is capturable in a CUDA graph.
//
// Faults are never raised on the device: a job record that fails validation
// (kind, op, box volume, null pointers, unit range) sets a bit in a device
// status word and is skipped; spaghetty_batch_status() reports it.  There is
// no inter-CTA waiting of any kind.
#include "../../include/spaghetty_gb300.h"
#include "kernels.cuh"
#include "plan.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#define SPG_BATCH_VMAX (SPG_BATCH_NT * SPG_BATCH_EPT)
// Elements per work unit (consecutive boxes of one sort, at most
// SPG_BATCH_MAXB of them), a power of two from SPG_BATCH_UNIT_MIN to
// SPG_BATCH_UNIT_ELEMS chosen per batch: the largest that still gives every
// CTA SPG_BATCH_UNITS_PER_CTA units.  Each unit starts and drains its own
// cp.async pipeline, so long units leave fewer bubbles (on the batched
// configuration's mix 16K -> 64K elements went from 4070 to 4235 GB/s, all
// sorts on the work list; 48K and 96K measured 4218 and 4133); but one CTA
// moves a unit alone, at a few GB/s, so in a small batch the last long
// units are its tail (the small-tile mix, 22M elements: 24.4M tiles/s with
// 16K-element units, 20.8M with 64K).
#ifndef SPG_BATCH_UNIT_ELEMS
#define SPG_BATCH_UNIT_ELEMS 65536
#endif
#ifndef SPG_BATCH_UNIT_MIN
#define SPG_BATCH_UNIT_MIN 4096
#endif
#ifndef SPG_BATCH_UNITS_PER_CTA
#define SPG_BATCH_UNITS_PER_CTA 4
#endif
// Boxes per work unit at most: a unit's box offsets and edge limits are
// computed once, one box per thread, into shared memory, so that the box
// loop reads three words instead of walking the job's box grid (tens of
// shared-memory reads of the job record per thread and box).
#ifndef SPG_BATCH_MAXB
#define SPG_BATCH_MAXB 64
#endif
// Sorts of at least this many elements whose single-sort plan is the
// TMA-staged kernel fill the GPU by themselves at a higher rate than the
// persistent kernel: a batch launch runs each of them as its own launch,
// then the persistent kernel over the rest.  Both are enqueued on the same
// stream, so a captured graph holds them all.  On the batched
// configuration's mix (random 6-D shapes, random factors) the persistent
// kernel moves the sorts of 2^22..2^24 elements as fast as their own
// launches do, and the threshold 2^24 measured best (GB/s with 64K-element
// units: 2^22 4193, 2^23 4256, 2^24 4269, none 4235).
// SPAGHETTY_OPT_BATCH_OWN_MIN and SPAGHETTY_OPT_BATCH_OWN_KINDS change the
// size and the plan kinds.
#define SPG_BATCH_DIRECT_ELEMS (1 << 24)
// Those direct launches are spread over this many streams beside the launch
// stream: independent sorts (disjoint outputs), so one launch's last wave of
// CTAs overlaps the next ones instead of leaving SMs idle.
#define SPG_BATCH_AUX 3
#ifndef SPG_BATCH_S
#define SPG_BATCH_S 3          // cp.async stages of the tiled path
#endif
#ifndef SPG_BATCH_MINB
#define SPG_BATCH_MINB 4       // CTAs per SM the register allocation must allow
#endif

struct BatchJob {
    KParams kp;
    const double *in;
    double *out;
    int32_t kind;
    int32_t op;
    uint32_t ubeg;     // first work unit of this job
    uint32_t chunk;    // boxes per work unit
};

// Dynamic shared memory of one launch: SPG_BATCH_S stages of the largest
// stage size (elements) among the batch's tiled sorts.
static inline size_t batch_smem_bytes(int stage_elems) {
    return (size_t)SPG_BATCH_S * (size_t)stage_elems * sizeof(double);
}
// The kernel also holds the current job record in static shared memory, and
// the 48 KB default limit counts static plus dynamic bytes: above this many
// dynamic bytes the launch needs the opt-in attribute.
#define SPG_BATCH_SMEM_OPTIN (40 * 1024)

// Elements of a thread's SPG_BATCH_EPT per box whose arbitrary-factor
// product takes the 32-bit integer multiply (spg_mul: the same bits as the
// rounded multiply) instead of the FP64 pipe, the busiest unit of this
// kernel on random factors.  Measured on the batched configuration's mix
// (GB/s): 0 4268, 1 4278, 2 4224, 4 3805 -- the kernel is bound by latency
// (its block barrier per box, global and shared memory), not by the FP64
// pipe, and the integer multiply's 40 instructions and registers cost more
// than the FP64 cycles they free; so 0.
#ifndef SPG_BATCH_INT_ELEMS
#define SPG_BATCH_INT_ELEMS 0
#endif

template <int OP>
__device__ __forceinline__ double spg_batch_apply(int k, double x, double y, const SpgFactor &F) {
    if ((OP == OP_SORT_ANY || OP == OP_ACC_ANY) && k >= SPG_BATCH_EPT - SPG_BATCH_INT_ELEMS)
        return spg_apply_flat<OP>(x, y, F);
    return spg_apply<OP>(x, y, F);
}

// The kernel's check of a job record before it runs any of its units (a
// record that fails it is skipped and flagged in the status word);
// spaghetty_batch_verify runs the same check on the host.
__host__ __device__ __forceinline__ bool spg_batch_job_ok(const BatchJob &j, int smem_elems) {
    const KParams &p = j.kp;
    const int tile = p.vol + (p.pad > 0 ? p.vol / p.pad + 1 : 0);
    // the stages: SPG_BATCH_S of the sort's stage size fit the dynamic
    // shared memory (smem_elems per stage)
    return (j.kind == KIND_TILED || j.kind == KIND_DIRECT) && j.op >= 0 && j.op < OP_COUNT &&
           p.vol >= 1 && p.vol <= SPG_BATCH_VMAX && p.pad >= 0 && j.in != nullptr && j.out != nullptr &&
           j.chunk >= 1 && j.chunk <= SPG_BATCH_MAXB && p.lenA <= 0xFFFF && p.lenB <= 0xFFFF &&
           p.ntiles >= 1 && p.ld.n >= 0 && p.ld.n <= SPG_MAXR && p.st.n >= 0 && p.st.n <= SPG_MAXR &&
           p.grid.n >= 0 && p.grid.n <= SPG_MAXR &&
           (j.kind != KIND_TILED || (tile <= p.stage && p.stage <= smem_elems));
}

// Status word bits.
#define SPG_ST_BAD_JOB 1
#define SPG_ST_BAD_UNIT 2

// Boxes [b0, b1) of one tiled sort, pipelined: 8-byte cp.async copies put
// box t+S-1 in flight (SPG_BATCH_S stages of the sort's stage size) while
// box t is written out in output order.  Every thread of the CTA calls it
// with the same arguments; nothing is left in flight when it returns.
// The unit's box table (shared memory, one entry per box of [b0, b1)):
// input and output element offsets and the two edge limits.
struct SpgBoxTab {
    int64_t ib[SPG_BATCH_MAXB];
    int64_t ob[SPG_BATCH_MAXB];
    uint32_t lim[SPG_BATCH_MAXB];     // limA << 16 | limB
};

// The unit's box table, one box per thread (kept out of line: its 64-bit
// box walk would otherwise add to the register pressure of the box loop).
static __device__ __noinline__ void spg_batch_fill_boxes(const KParams &p, uint32_t b0, uint32_t b1,
                                                         SpgBoxTab &bt) {
    for (uint32_t i = threadIdx.x; b0 + i < b1; i += SPG_BATCH_NT) {
        int64_t ib, ob;
        uint32_t limA, limB;
        spg_box(p, b0 + i, ib, ob, limA, limB);
        bt.ib[i] = ib;
        bt.ob[i] = ob;
        bt.lim[i] = limA << 16 | limB;
    }
}

template <int OP>
__device__ __forceinline__ void spg_batch_tiled(const BatchJob &j, const SpgTab<SPG_BATCH_NT, SPG_BATCH_EPT> &tb,
                                                uint32_t b0, uint32_t b1, double *sm, const SpgBoxTab &bt) {
    const KParams &p = j.kp;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
    const uint32_t stage_bytes = (uint32_t)p.stage * 8u;
    const double *in = j.in;
    auto issue = [&](uint32_t t, int st) {
        if (t < b1) {
            const uint32_t lim = bt.lim[t - b0];
            const uint32_t limA = lim >> 16, limB = lim & 0xFFFFu;
            const double *src = in + bt.ib[t - b0];
            const uint32_t sb = sbase + (uint32_t)st * stage_bytes;
#pragma unroll
            for (int k = 0; k < SPG_BATCH_EPT; ++k) {
                if (tb.pkl[k] != SPG_INVALID) {
                    const bool v = spg_valid(tb.pkl[k], limA, limB);
                    spg_cp_async8(sb + (uint32_t)tb.smw[k] * 8u, v ? src + tb.ioff[k] : in, v ? 8u : 0u);
                }
            }
        }
        spg_cp_commit();
    };
    const SpgFactor fac = p.fac;
#pragma unroll
    for (int q = 0; q < SPG_BATCH_S - 1; ++q) issue(b0 + (uint32_t)q, q);
    // One block barrier per box: after it every thread's copies of box t
    // have landed and every thread has finished box t-1, whose stage is the
    // one refilled (with box t+S-1) right after it.
    int it = 0;
    for (uint32_t t = b0; t < b1; ++t, ++it) {
        const int st = it % SPG_BATCH_S;
        const uint32_t lim = bt.lim[t - b0];
        const uint32_t limA = lim >> 16, limB = lim & 0xFFFFu;
        double *dst = j.out + bt.ob[t - b0];
        // a sortacc's old output: loads issued before the wait, which
        // hides their latency
        double y[SPG_BATCH_EPT];
        if (spg_reads_out<OP>::value) {
#pragma unroll
            for (int k = 0; k < SPG_BATCH_EPT; ++k) {
                y[k] = 0.0;
                if (spg_valid(tb.pks[k], limA, limB)) y[k] = spg_ld_out(dst + tb.ooff[k]);
            }
        }
        spg_cp_wait<SPG_BATCH_S - 2>();        // this thread's copies for box t have landed
        __syncthreads();                       // ... everyone's, and box t-1 is done
        issue(t + SPG_BATCH_S - 1, (it + SPG_BATCH_S - 1) % SPG_BATCH_S);
        const double *tile = sm + (size_t)st * p.stage;
#pragma unroll
        for (int k = 0; k < SPG_BATCH_EPT; ++k) {
            if (spg_valid(tb.pks[k], limA, limB)) {
                const double x = tile[tb.smr[k]];
                spg_st_out(dst + tb.ooff[k], spg_batch_apply<OP>(k, x, spg_reads_out<OP>::value ? y[k] : 0.0, fac));
            }
        }
    }
    spg_cp_wait<0>();
}

// A direct sort's box from the unit's box table: every element read and
// written by the same thread (the stride-1 index is unchanged).
template <int OP>
__device__ __forceinline__ void spg_batch_direct_box(const BatchJob &j, const SpgTab<SPG_BATCH_NT, SPG_BATCH_EPT> &tb,
                                                     const SpgBoxTab &bt, uint32_t i) {
    const uint32_t lim = bt.lim[i];
    const uint32_t limA = lim >> 16, limB = lim & 0xFFFFu;
    const double *src = j.in + bt.ib[i];
    double *dst = j.out + bt.ob[i];
    const SpgFactor fac = j.kp.fac;
    double v[SPG_BATCH_EPT], y[SPG_BATCH_EPT];
#pragma unroll
    for (int k = 0; k < SPG_BATCH_EPT; ++k) {
        v[k] = 0.0;
        y[k] = 0.0;
        if (spg_valid(tb.pkl[k], limA, limB)) {
            v[k] = spg_ld_in(src + tb.ioff[k]);
            if (spg_reads_out<OP>::value) y[k] = spg_ld_out(dst + tb.ooff[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < SPG_BATCH_EPT; ++k)
        if (spg_valid(tb.pkl[k], limA, limB)) spg_st_out(dst + tb.ooff[k], spg_batch_apply<OP>(k, v[k], y[k], fac));
}

template <int OP>
__device__ __forceinline__ void spg_batch_units(const BatchJob &j, const SpgTab<SPG_BATCH_NT, SPG_BATCH_EPT> &tb,
                                                uint32_t b0, uint32_t b1, double *sm, const SpgBoxTab &bt) {
    if (j.kind == KIND_TILED) spg_batch_tiled<OP>(j, tb, b0, b1, sm, bt);
    else
        for (uint32_t t = b0; t < b1; ++t) spg_batch_direct_box<OP>(j, tb, bt, t - b0);
}

__global__ void __launch_bounds__(SPG_BATCH_NT, SPG_BATCH_MINB)
spg_batched(const BatchJob *__restrict__ jobs, uint32_t njobs,
            const uint32_t *__restrict__ unit_job, uint32_t total_units,
            uint32_t *counter, int *status, int smem_elems) {
    extern __shared__ __align__(16) double sm[];
    __shared__ BatchJob sj;
    __shared__ SpgBoxTab sbt;
    __shared__ uint32_t s_next;
    __shared__ int s_ok;
    const uint32_t tid = threadIdx.x;
    SpgTab<SPG_BATCH_NT, SPG_BATCH_EPT> tb;
    uint32_t cur = 0xFFFFFFFFu;
    if (tid == 0) s_next = atomicAdd(counter, 1u);
    __syncthreads();
    for (;;) {
        const uint32_t u = s_next;
        if (u >= total_units) break;
        const uint32_t j = unit_job[u];
        __syncthreads();                      // everyone has read s_next
        if (tid == 0) s_next = atomicAdd(counter, 1u);   // next unit, fetched early
        if (j >= njobs) {
            if (tid == 0) atomicOr(status, SPG_ST_BAD_UNIT);
            __syncthreads();
            continue;
        }
        if (j != cur) {
            const uint32_t *src = reinterpret_cast<const uint32_t *>(jobs + j);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&sj);
            for (uint32_t i = tid; i < sizeof(BatchJob) / 4; i += SPG_BATCH_NT) dst[i] = src[i];
            __syncthreads();
            if (tid == 0) {
                const bool ok = spg_batch_job_ok(sj, smem_elems) && u >= sj.ubeg;
                s_ok = ok ? 1 : 0;
                if (!ok) atomicOr(status, SPG_ST_BAD_JOB);
            }
            __syncthreads();
            if (s_ok) {
                if (sj.kind == KIND_TILED) tb.build_tiled(sj.kp, tid);
                else tb.build_direct(sj.kp, tid);
            }
            cur = j;
        }
        if (s_ok) {
            const uint32_t b0 = (u - sj.ubeg) * sj.chunk;
            const uint32_t b1 = min(b0 + sj.chunk, sj.kp.ntiles);
            spg_batch_fill_boxes(sj.kp, b0, b1, sbt);
            __syncthreads();
            switch (sj.op) {
                case OP_SORT_ONE: spg_batch_units<OP_SORT_ONE>(sj, tb, b0, b1, sm, sbt); break;
                case OP_SORT_NEG: spg_batch_units<OP_SORT_NEG>(sj, tb, b0, b1, sm, sbt); break;
                case OP_SORT_POW2: spg_batch_units<OP_SORT_POW2>(sj, tb, b0, b1, sm, sbt); break;
                case OP_SORT_ANY: spg_batch_units<OP_SORT_ANY>(sj, tb, b0, b1, sm, sbt); break;
                case OP_ACC_ONE: spg_batch_units<OP_ACC_ONE>(sj, tb, b0, b1, sm, sbt); break;
                case OP_ACC_NEG: spg_batch_units<OP_ACC_NEG>(sj, tb, b0, b1, sm, sbt); break;
                case OP_ACC_POW2: spg_batch_units<OP_ACC_POW2>(sj, tb, b0, b1, sm, sbt); break;
                case OP_ACC_ANY: spg_batch_units<OP_ACC_ANY>(sj, tb, b0, b1, sm, sbt); break;
                default: spg_batch_units<OP_GEN>(sj, tb, b0, b1, sm, sbt); break;
            }
        }
        __syncthreads();                      // unit done: sj and the tile may be replaced
    }
}

// ===========================================================================
struct spaghetty_batch {
    int dev = 0;
    int n = 0;
    uint32_t njobs = 0;
    uint32_t total_units = 0;
    int smem_elems = 0;               // stage size (elements) of the largest tiled sort
    BatchJob *d_jobs = nullptr;
    uint32_t *d_unit_job = nullptr;
    uint32_t *d_words = nullptr;      // [0] = unit counter, [1] = status word
    std::vector<spaghetty_batch_entry> entries;
    std::vector<BatchJob> jobs;       // host copy of the job records
    std::vector<int> direct;          // entries large enough to run as their own launch
    int64_t bytes = 0;                // algorithmic bytes of one launch
    // streams that run the direct sorts beside the persistent kernel (forked
    // from and joined back into the launch stream by events)
    int naux = 0;
    cudaStream_t aux[SPG_BATCH_AUX] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[SPG_BATCH_AUX] = {};
};

namespace {
thread_local int g_batch_bad_index = -1;

// Which sorts leave the work list for their own launches (read when a batch
// is created): at least g_own_min elements (0: none), and, unless
// g_own_any, only those whose single-sort plan is the TMA-staged kernel.
std::atomic<int64_t> g_own_min{SPG_BATCH_DIRECT_ELEMS};
std::atomic<int> g_own_any{0};

// Tuned tile-shape rules, one per size bucket (spaghetty_batch_tune_set).
std::mutex g_rules_mu;
std::vector<SpgBatchRule> g_rules;

// The rule for one sort: its rank and its largest extent pick the bucket.
bool find_rule(int rank, const int *dims, SpgBatchRule *out) {
    int emax = 0;
    for (int q = 0; q < rank; ++q) emax = std::max(emax, dims[q]);
    std::lock_guard<std::mutex> lk(g_rules_mu);
    for (const SpgBatchRule &r : g_rules)
        if (r.rank == rank && emax >= r.ext_lo && emax <= r.ext_hi) {
            *out = r;
            return true;
        }
    return false;
}

// The work-unit size for a work list of `elems` elements on `sms` SMs.
int64_t batch_unit_elems_sms(int64_t elems, int sms) {
    const int64_t per = elems / ((int64_t)std::max(sms, 1) * SPG_BATCH_MINB * SPG_BATCH_UNITS_PER_CTA);
    int64_t u = SPG_BATCH_UNIT_MIN;
    while (u < SPG_BATCH_UNIT_ELEMS && 2 * u <= per) u *= 2;
    return u;
}

// ... on device `dev`.
int64_t batch_unit_elems(int64_t elems, int dev) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
        cudaGetLastError();
        sms = 152;
    }
    return batch_unit_elems_sms(elems, sms);
}

// Boxes per work unit of a job whose boxes hold `vol` elements.
uint32_t batch_chunk(int64_t unit_elems, int32_t vol) {
    return (uint32_t)std::min<int64_t>(SPG_BATCH_MAXB, std::max<int64_t>(1, unit_elems / std::max(1, (int)vol)));
}

// One sort of a batch planned as a work-list job: every field of the record
// but chunk and ubeg, which depend on the whole work list.  *pfo (may be
// NULL) receives the folded problem the job's parameters describe.
int batch_plan_job(const spaghetty_batch_entry &e, const Folded &fo, BatchJob *j, Folded *pfo) {
    Plan pl;
    const int op = spg_choose_op(e.factor, e.acc_factor);
    SpgBatchRule rule;
    const bool have_rule = find_rule(e.rank, e.dims, &rule);
    int rc = spg_plan_batch(fo, op, have_rule ? &rule : nullptr, &pl);
    if (!rc) rc = spg_build_params(&pl, e.factor, e.acc_factor);
    if (rc) return rc;
    std::memset(j, 0, sizeof(*j));
    j->kp = pl.kp;
    j->in = e.unsorted;
    j->out = e.sorted;
    j->kind = pl.kind;
    j->op = op;
    if (pfo) *pfo = pl.fo;
    return SPAGHETTY_OK;
}

bool is_device_ptr(const void *p, int *dev) {
    cudaPointerAttributes at;
    std::memset(&at, 0, sizeof(at));
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
        *dev = at.device;
        return true;
    }
    return false;
}

int grid_for(spaghetty_batch *b) {
    int sms = 0, nb = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->dev) != cudaSuccess) sms = 152;
    const size_t smem = batch_smem_bytes(b->smem_elems);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spg_batched, SPG_BATCH_NT, smem) != cudaSuccess ||
        nb < 1)
        nb = 1;
    cudaGetLastError();
    int64_t g = (int64_t)sms * nb;
    g = std::min<int64_t>(g, std::max<uint32_t>(b->total_units, 1));
    return (int)g;
}
}  // namespace

int spg_batch_option(int option, int value) {
    if (option == SPAGHETTY_OPT_BATCH_OWN_MIN) {
        if (value < 0) return SPAGHETTY_ERR_CONFIG;
        g_own_min.store(value);
        return SPAGHETTY_OK;
    }
    if (option == SPAGHETTY_OPT_BATCH_OWN_KINDS) {
        if (value < 0 || value > 1) return SPAGHETTY_ERR_CONFIG;
        g_own_any.store(value);
        return SPAGHETTY_OK;
    }
    return SPAGHETTY_ERR_CONFIG;
}

extern "C" {

int spaghetty_batch_create(const spaghetty_batch_entry *entries, int n, spaghetty_batch **out) {
    g_batch_bad_index = -1;
    if (!out) return SPAGHETTY_ERR_NULL;
    *out = nullptr;
    if (n < 0 || (n > 0 && !entries)) return SPAGHETTY_ERR_NULL;
    spaghetty_batch *b = new spaghetty_batch();
    b->n = n;
    b->entries.assign(entries, entries + n);
    if (cudaGetDevice(&b->dev) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return SPAGHETTY_ERR_CUDA;
    }
    spg_autoload_tune();                      // size-bucket rules from the tune file
    std::vector<uint32_t> unit_job;
    struct Range { uintptr_t lo, hi; int idx; bool out; };
    std::vector<Range> ranges;
    int64_t list_elems = 0;                   // elements of the sorts on the work list
    int rc = SPAGHETTY_OK;
    for (int i = 0; i < n && rc == SPAGHETTY_OK; ++i) {
        const spaghetty_batch_entry &e = entries[i];
        Folded fo;
        rc = spg_fold(e.rank, e.dims, e.perm, &fo);
        if (rc) { g_batch_bad_index = i; break; }
        if (fo.empty) continue;
        if (!e.unsorted || !e.sorted) { rc = SPAGHETTY_ERR_NULL; g_batch_bad_index = i; break; }
        int du = -1, ds = -1;
        if (!is_device_ptr(e.unsorted, &du) || !is_device_ptr(e.sorted, &ds) || du != b->dev ||
            ds != b->dev) {
            rc = SPAGHETTY_ERR_MEMSPACE;
            g_batch_bad_index = i;
            break;
        }
        const uintptr_t nb = (uintptr_t)fo.nelem * sizeof(double);
        ranges.push_back({(uintptr_t)e.unsorted, (uintptr_t)e.unsorted + nb, i, false});
        ranges.push_back({(uintptr_t)e.sorted, (uintptr_t)e.sorted + nb, i, true});
        const int64_t own_min = g_own_min.load();
        if (own_min > 0 && fo.nelem >= own_min &&
            (g_own_any.load() ||
             spg_plan_is_tma(b->dev, e.rank, e.dims, e.perm, e.factor, e.acc_factor, e.unsorted, e.sorted))) {
            const int op = spg_choose_op(e.factor, e.acc_factor);
            b->direct.push_back(i);
            b->bytes += fo.nelem * (spg_op_class(op) == 0 ? 16 : 24);
            continue;
        }
        BatchJob j;
        rc = batch_plan_job(e, fo, &j, nullptr);
        if (rc) { g_batch_bad_index = i; break; }
        if (j.kind == KIND_TILED)
            b->smem_elems = std::max(b->smem_elems, (int)j.kp.stage);
        b->bytes += fo.nelem * (spg_op_class(j.op) == 0 ? 16 : 24);
        list_elems += fo.nelem;
        b->jobs.push_back(j);
    }
    // the work units, once the work list's size is known
    const int64_t unit_elems = batch_unit_elems(list_elems, b->dev);
    for (size_t q = 0; q < b->jobs.size() && rc == SPAGHETTY_OK; ++q) {
        BatchJob &j = b->jobs[q];
        j.chunk = batch_chunk(unit_elems, j.kp.vol);
        j.ubeg = (uint32_t)unit_job.size();
        const uint32_t units = (j.kp.ntiles + j.chunk - 1) / j.chunk;
        if ((uint64_t)unit_job.size() + units > 0xFFFFFFF0ull) { rc = SPAGHETTY_ERR_OVERFLOW; break; }
        for (uint32_t u = 0; u < units; ++u) unit_job.push_back((uint32_t)q);
    }
    if (rc == SPAGHETTY_OK) {
        // No output may overlap any other buffer of the batch (inputs may be
        // shared between sorts): outputs pairwise disjoint, then every input
        // checked against the sorted outputs.
        std::vector<Range> outs, ins;
        for (const Range &r : ranges) (r.out ? outs : ins).push_back(r);
        std::sort(outs.begin(), outs.end(), [](const Range &a, const Range &c) { return a.lo < c.lo; });
        for (size_t q = 1; q < outs.size() && rc == SPAGHETTY_OK; ++q)
            if (outs[q].lo < outs[q - 1].hi) { rc = SPAGHETTY_ERR_ALIAS; g_batch_bad_index = outs[q].idx; }
        for (size_t q = 0; q < ins.size() && rc == SPAGHETTY_OK; ++q) {
            // first output whose end lies beyond this input's start
            auto it = std::upper_bound(outs.begin(), outs.end(), ins[q].lo,
                                       [](uintptr_t v, const Range &r) { return v < r.hi; });
            if (it != outs.end() && it->lo < ins[q].hi) { rc = SPAGHETTY_ERR_ALIAS; g_batch_bad_index = ins[q].idx; }
        }
    }
    if (rc != SPAGHETTY_OK) {
        delete b;
        return rc;
    }
    b->njobs = (uint32_t)b->jobs.size();
    b->total_units = (uint32_t)unit_job.size();
    b->smem_elems = std::max(b->smem_elems, 2);
    bool ok = cudaMalloc((void **)&b->d_words, 2 * sizeof(uint32_t)) == cudaSuccess &&
              cudaMemset(b->d_words, 0, 2 * sizeof(uint32_t)) == cudaSuccess;
    if (ok && b->njobs) {
        ok = cudaMalloc((void **)&b->d_jobs, b->jobs.size() * sizeof(BatchJob)) == cudaSuccess &&
             cudaMalloc((void **)&b->d_unit_job, unit_job.size() * sizeof(uint32_t)) == cudaSuccess &&
             cudaMemcpy(b->d_jobs, b->jobs.data(), b->jobs.size() * sizeof(BatchJob),
                        cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(b->d_unit_job, unit_job.data(), unit_job.size() * sizeof(uint32_t),
                        cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        spaghetty_batch_destroy(b);
        return SPAGHETTY_ERR_CUDA;
    }
    if (!b->direct.empty()) {
        // streams and events for the direct sorts; without them (creation
        // failed) the direct sorts run in order on the launch stream
        bool ok2 = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
        for (int a = 0; a < SPG_BATCH_AUX && ok2; ++a) {
            ok2 = cudaStreamCreateWithFlags(&b->aux[a], cudaStreamNonBlocking) == cudaSuccess &&
                  cudaEventCreateWithFlags(&b->join[a], cudaEventDisableTiming) == cudaSuccess;
            if (ok2) b->naux = a + 1;
        }
        if (!ok2) b->naux = 0;
        cudaGetLastError();
    }
    if (batch_smem_bytes(b->smem_elems) > SPG_BATCH_SMEM_OPTIN) {
        if (cudaFuncSetAttribute(spg_batched, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)batch_smem_bytes(b->smem_elems)) != cudaSuccess) {
            cudaGetLastError();
            spaghetty_batch_destroy(b);
            return SPAGHETTY_ERR_CUDA;
        }
    }
    *out = b;
    return SPAGHETTY_OK;
}

int spaghetty_batch_bad_index(void) { return g_batch_bad_index; }

int spaghetty_batch_tune_set(int rank, int ext_lo, int ext_hi, int run_in, int run_out, int volume) {
    std::lock_guard<std::mutex> lk(g_rules_mu);
    if (rank == 0) {
        g_rules.clear();
        return SPAGHETTY_OK;
    }
    if (rank < 1 || rank > SPG_MAXR || ext_lo < 1 || ext_hi < ext_lo || run_in < 1 || run_out < 1 ||
        volume < 1 || volume > SPG_BATCH_VMAX)
        return SPAGHETTY_ERR_CONFIG;
    // a bucket overlapping an existing one replaces it
    for (size_t q = 0; q < g_rules.size();) {
        const SpgBatchRule &r = g_rules[q];
        if (r.rank == rank && !(ext_hi < r.ext_lo || r.ext_hi < ext_lo)) g_rules.erase(g_rules.begin() + q);
        else ++q;
    }
    g_rules.push_back({rank, ext_lo, ext_hi, run_in, run_out, volume});
    return SPAGHETTY_OK;
}

int spaghetty_batch_launch(spaghetty_batch *b, void *stream) {
    SpgRange range("spaghetty_batch_launch");
    if (!b) return SPAGHETTY_ERR_NULL;
    cudaStream_t st = (cudaStream_t)stream;
    // direct sorts: forked onto the aux streams (round robin) and joined
    // back into the launch stream before the persistent kernel
    const bool forked = !b->direct.empty() && b->naux > 0;
    int rc = SPAGHETTY_OK;
    if (!b->direct.empty()) {
        int cur = -1;
        if (cudaGetDevice(&cur) != cudaSuccess) cudaGetLastError();
        if (cudaSetDevice(b->dev) != cudaSuccess) {
            cudaGetLastError();
            return SPAGHETTY_ERR_CUDA;
        }
        if (forked) {
            if (cudaEventRecord(b->fork, st) != cudaSuccess) rc = SPAGHETTY_ERR_CUDA;
            for (int a = 0; a < b->naux && !rc; ++a)
                if (cudaStreamWaitEvent(b->aux[a], b->fork, 0) != cudaSuccess) rc = SPAGHETTY_ERR_CUDA;
        }
        for (size_t q = 0; q < b->direct.size() && !rc; ++q) {
            const spaghetty_batch_entry &e = b->entries[(size_t)b->direct[q]];
            rc = spg_sort_async_on(b->dev, e.rank, e.unsorted, e.sorted, e.dims, e.perm, e.factor,
                                   e.acc_factor, forked ? (void *)b->aux[q % (size_t)b->naux] : stream);
        }
        if (cur >= 0 && cur != b->dev) cudaSetDevice(cur);
    }
    // the join: every aux stream's work before anything later on the launch stream
    auto join = [&]() {
        if (!forked) return;
        for (int a = 0; a < b->naux; ++a)
            if (cudaEventRecord(b->join[a], b->aux[a]) != cudaSuccess ||
                cudaStreamWaitEvent(st, b->join[a], 0) != cudaSuccess)
                rc = rc ? rc : SPAGHETTY_ERR_CUDA;
    };
    // joined before the persistent kernel: running beside the direct sorts
    // it was slower on the configuration mix (3587 against 3779 GB/s)
    join();
    if (rc || b->total_units == 0) {
        cudaGetLastError();
        return rc;
    }
    if (cudaMemsetAsync(b->d_words, 0, sizeof(uint32_t), st) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    const int grid = grid_for(b);
    uint32_t *counter = b->d_words;
    int *status = (int *)(b->d_words + 1);
    const BatchJob *jobs = b->d_jobs;
    const uint32_t *uj = b->d_unit_job;
    uint32_t nj = b->njobs, tu = b->total_units;
    int se = b->smem_elems;
    void *args[] = {(void *)&jobs, (void *)&nj, (void *)&uj, (void *)&tu,
                    (void *)&counter, (void *)&status, (void *)&se};
    if (cudaLaunchKernel((const void *)spg_batched, dim3(grid), dim3(SPG_BATCH_NT), args,
                         batch_smem_bytes(b->smem_elems), st) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    return SPAGHETTY_OK;
}

int spaghetty_batch_launch_plain(spaghetty_batch *b, void *stream) {
    SpgRange range("spaghetty_batch_launch_plain");
    if (!b) return SPAGHETTY_ERR_NULL;
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) cudaGetLastError();
    if (cudaSetDevice(b->dev) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    int rc = SPAGHETTY_OK;
    for (const spaghetty_batch_entry &e : b->entries) {
        rc = spg_sort_async_on(b->dev, e.rank, e.unsorted, e.sorted, e.dims, e.perm, e.factor,
                               e.acc_factor, stream);
        if (rc) break;
    }
    if (cur >= 0 && cur != b->dev) cudaSetDevice(cur);
    return rc;
}

int spaghetty_batch_status(spaghetty_batch *b, void *stream) {
    if (!b) return SPAGHETTY_ERR_NULL;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    int st = 0;
    if (cudaMemcpy(&st, b->d_words + 1, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    if (cudaMemset(b->d_words + 1, 0, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    return st ? SPAGHETTY_ERR_DEVICE : SPAGHETTY_OK;
}

int spaghetty_batch_launches(const spaghetty_batch *b) {
    if (!b) return -SPAGHETTY_ERR_NULL;
    return (int)b->direct.size() + (b->total_units > 0 ? 1 : 0);
}

int spaghetty_batch_info(const spaghetty_batch *b, int64_t *info) {
    if (!b || !info) return SPAGHETTY_ERR_NULL;
    info[0] = b->njobs;
    info[1] = b->total_units;
    info[2] = b->bytes;
    info[3] = (int64_t)batch_smem_bytes(b->smem_elems);
    return SPAGHETTY_OK;
}

int spaghetty_batch_poison(spaghetty_batch *b, int index) {
    // Host-side fault injection for tests: overwrite one job record's kind
    // with an invalid value in device memory (the kernel must flag and skip
    // it without touching memory).
    if (!b) return SPAGHETTY_ERR_NULL;
    if (index < 0 || (uint32_t)index >= b->njobs) return SPAGHETTY_ERR_BATCH;
    BatchJob j = b->jobs[index];
    j.kind = 99;
    if (cudaMemcpy(b->d_jobs + index, &j, sizeof(BatchJob), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    return SPAGHETTY_OK;
}

int spaghetty_batch_destroy(spaghetty_batch *b) {
    if (!b) return SPAGHETTY_OK;
    if (b->d_jobs) cudaFree(b->d_jobs);
    if (b->d_unit_job) cudaFree(b->d_unit_job);
    if (b->d_words) cudaFree(b->d_words);
    for (int a = 0; a < SPG_BATCH_AUX; ++a) {
        if (b->aux[a]) cudaStreamDestroy(b->aux[a]);
        if (b->join[a]) cudaEventDestroy(b->join[a]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    cudaGetLastError();
    delete b;
    return SPAGHETTY_OK;
}

}  // extern "C"

// ===========================================================================
// Batched sorts without any allocation.
//
// Some callers cannot call cudaMalloc: an application that has handed the
// whole device memory to its own pool allocator at start-up (a library's
// cudaMalloc then fails, or escapes the application's accounting), and code
// that must not trigger the device-wide synchronisation that cudaMalloc and
// cudaFree may cause while other streams are running.
// spaghetty_sort_batch_noalloc() runs the same persistent
// batched kernel as spaghetty_batch_create()/spaghetty_batch_launch(), but
// its work list, unit counter and status word live in the file-scope device
// array below, which every GPU that loads this library holds until exit.
// The caller passes only its input and output tensors.
#define SPG_NOALLOC_BYTES (4u << 20)          // 4 MiB of device scratch
#define SPG_NOALLOC_MAX_SORTS 1024
#define SPG_NOALLOC_MAX_DEVICES 64
#define SPG_NOALLOC_JOBS_OFFSET 256u

static __device__ __align__(256) unsigned char g_spg_noalloc_scratch[SPG_NOALLOC_BYTES];

namespace {
std::mutex g_na_mu;
// Device address of g_spg_noalloc_scratch per device: in host code the
// array's name is only a host-side stand-in, so the address is looked up once
// per device with cudaGetSymbolAddress (with that device current).
unsigned char *g_na_dev[SPG_NOALLOC_MAX_DEVICES];
// Host image of the work list (static: the entry point allocates nothing).
alignas(256) unsigned char g_na_host[SPG_NOALLOC_BYTES];
struct NaRange { uintptr_t lo, hi; int idx; };
NaRange g_na_outs[SPG_NOALLOC_MAX_SORTS];
NaRange g_na_ins[SPG_NOALLOC_MAX_SORTS];
int g_na_status;
}  // namespace

extern "C" int spaghetty_sort_batch_noalloc(const spaghetty_batch_entry *entries, int n,
                                            void *stream) {
    if (n < 0 || (n > 0 && !entries)) return SPAGHETTY_ERR_NULL;
    if (n > SPG_NOALLOC_MAX_SORTS) return SPAGHETTY_ERR_TOO_LARGE;
    // the shipped size-bucket rules, as spaghetty_batch_create loads them,
    // so that plans do not depend on which batched entry ran first
    spg_autoload_tune();
    std::lock_guard<std::mutex> lk(g_na_mu);
    g_batch_bad_index = -1;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= SPG_NOALLOC_MAX_DEVICES) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    if (!g_na_dev[dev]) {
        // first call on this device: set-up (do it before any stream capture)
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_spg_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return SPAGHETTY_ERR_CUDA;
        }
        g_na_dev[dev] = (unsigned char *)p;
    }
    unsigned char *dbase = g_na_dev[dev];
    BatchJob *hjobs = reinterpret_cast<BatchJob *>(g_na_host + SPG_NOALLOC_JOBS_OFFSET);
    uint32_t njobs = 0, nunits = 0, nouts = 0;
    int64_t list_elems = 0;
    int smem_elems = 2;
    // pass 1: validate and plan every sort into the host image
    for (int i = 0; i < n; ++i) {
        const spaghetty_batch_entry &e = entries[i];
        Folded fo;
        int rc = spg_fold(e.rank, e.dims, e.perm, &fo);
        if (rc) { g_batch_bad_index = i; return rc; }
        if (fo.empty) continue;
        if (!e.unsorted || !e.sorted) { g_batch_bad_index = i; return SPAGHETTY_ERR_NULL; }
        int du = -1, ds = -1;
        if (!is_device_ptr(e.unsorted, &du) || !is_device_ptr(e.sorted, &ds) || du != dev || ds != dev) {
            g_batch_bad_index = i;
            return SPAGHETTY_ERR_MEMSPACE;
        }
        BatchJob &j = hjobs[njobs];
        rc = batch_plan_job(e, fo, &j, nullptr);
        if (rc) { g_batch_bad_index = i; return rc; }
        const uintptr_t nb = (uintptr_t)fo.nelem * sizeof(double);
        g_na_outs[nouts] = {(uintptr_t)e.sorted, (uintptr_t)e.sorted + nb, i};
        g_na_ins[nouts] = {(uintptr_t)e.unsorted, (uintptr_t)e.unsorted + nb, i};
        ++nouts;
        if (j.kind == KIND_TILED)
            smem_elems = std::max(smem_elems, (int)j.kp.stage);
        list_elems += fo.nelem;
        ++njobs;
    }
    // the work units, once the work list's size is known
    const int64_t unit_elems = batch_unit_elems(list_elems, dev);
    uint64_t units_all = 0;
    for (uint32_t q = 0; q < njobs; ++q) {
        BatchJob &j = hjobs[q];
        j.chunk = batch_chunk(unit_elems, j.kp.vol);
        j.ubeg = (uint32_t)units_all;
        units_all += (j.kp.ntiles + j.chunk - 1) / j.chunk;
        if (units_all > SPG_NOALLOC_BYTES / sizeof(uint32_t)) return SPAGHETTY_ERR_TOO_LARGE;
    }
    nunits = (uint32_t)units_all;
    // the unit map follows the job records
    const size_t units_off = (SPG_NOALLOC_JOBS_OFFSET + (size_t)njobs * sizeof(BatchJob) + 255) & ~(size_t)255;
    const size_t used = units_off + (size_t)nunits * sizeof(uint32_t);
    if (used > SPG_NOALLOC_BYTES) return SPAGHETTY_ERR_TOO_LARGE;
    uint32_t *hunits = reinterpret_cast<uint32_t *>(g_na_host + units_off);
    for (uint32_t q = 0; q < njobs; ++q) {
        const uint32_t units = (hjobs[q].kp.ntiles + hjobs[q].chunk - 1) / hjobs[q].chunk;
        for (uint32_t u = 0; u < units; ++u) hunits[hjobs[q].ubeg + u] = q;
    }
    // outputs pairwise disjoint and disjoint from every input (in-place sort)
    std::sort(g_na_outs, g_na_outs + nouts, [](const NaRange &a, const NaRange &b) { return a.lo < b.lo; });
    for (uint32_t q = 1; q < nouts; ++q)
        if (g_na_outs[q].lo < g_na_outs[q - 1].hi) { g_batch_bad_index = g_na_outs[q].idx; return SPAGHETTY_ERR_ALIAS; }
    for (uint32_t q = 0; q < nouts; ++q) {
        const NaRange *it = std::upper_bound(g_na_outs, g_na_outs + nouts, g_na_ins[q].lo,
                                             [](uintptr_t v, const NaRange &r) { return v < r.hi; });
        if (it != g_na_outs + nouts && it->lo < g_na_ins[q].hi) {
            g_batch_bad_index = g_na_ins[q].idx;
            return SPAGHETTY_ERR_ALIAS;
        }
    }
    if (nunits == 0) return SPAGHETTY_OK;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t *counter = reinterpret_cast<uint32_t *>(dbase);
    int *status = reinterpret_cast<int *>(dbase + sizeof(uint32_t));
    const BatchJob *djobs = reinterpret_cast<const BatchJob *>(dbase + SPG_NOALLOC_JOBS_OFFSET);
    const uint32_t *dunits = reinterpret_cast<const uint32_t *>(dbase + units_off);
    // the counter and the status word must start at zero; the rest of the
    // scratch still holds the previous call's work list and is overwritten
    if (cudaMemsetAsync(dbase, 0, 2 * sizeof(uint32_t), st) != cudaSuccess ||
        cudaMemcpyAsync(dbase + SPG_NOALLOC_JOBS_OFFSET, g_na_host + SPG_NOALLOC_JOBS_OFFSET,
                        used - SPG_NOALLOC_JOBS_OFFSET, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    const size_t smem = batch_smem_bytes(smem_elems);
    if (smem > SPG_BATCH_SMEM_OPTIN &&
        cudaFuncSetAttribute(spg_batched, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    int sms = 0, nb = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 152;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spg_batched, SPG_BATCH_NT, smem) != cudaSuccess || nb < 1)
        nb = 1;
    cudaGetLastError();
    const int grid = (int)std::min<int64_t>((int64_t)sms * nb, nunits);
    void *args[] = {(void *)&djobs, (void *)&njobs, (void *)&dunits, (void *)&nunits,
                    (void *)&counter, (void *)&status, (void *)&smem_elems};
    if (cudaLaunchKernel((const void *)spg_batched, dim3(grid), dim3(SPG_BATCH_NT), args, smem, st) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    // synchronous: the status word is read back before the scratch can be reused
    if (cudaMemcpyAsync(&g_na_status, status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return SPAGHETTY_ERR_CUDA;
    }
    return g_na_status ? SPAGHETTY_ERR_DEVICE : SPAGHETTY_OK;
}

// ===========================================================================
// Host replay of a batch's plan (no GPU needed).
extern "C" int spaghetty_batch_verify(const spaghetty_batch_entry *entries, int n, int num_sms,
                                      int64_t *stats) {
    g_batch_bad_index = -1;
    if (stats) for (int q = 0; q < 4; ++q) stats[q] = 0;
    if (n < 0 || (n > 0 && !entries)) return SPAGHETTY_ERR_NULL;
    spg_autoload_tune();                      // the same size-bucket rules as a launch
    std::vector<BatchJob> jobs;
    std::vector<Folded> fos;
    std::vector<int> idx;
    int64_t list_elems = 0;
    int smem_elems = 2;
    for (int i = 0; i < n; ++i) {
        const spaghetty_batch_entry &e = entries[i];
        Folded fo;
        int rc = spg_fold(e.rank, e.dims, e.perm, &fo);
        if (rc) { g_batch_bad_index = i; return rc; }
        if (fo.empty) continue;
        // the records are replayed, not run: stand-in buffer addresses
        spaghetty_batch_entry ev = e;
        ev.unsorted = reinterpret_cast<const double *>(uintptr_t(256));
        ev.sorted = reinterpret_cast<double *>(uintptr_t(512));
        BatchJob j;
        Folded pfo;
        rc = batch_plan_job(ev, fo, &j, &pfo);
        if (rc) { g_batch_bad_index = i; return rc; }
        if (j.kind == KIND_TILED) smem_elems = std::max(smem_elems, (int)j.kp.stage);
        list_elems += fo.nelem;
        jobs.push_back(j);
        fos.push_back(pfo);
        idx.push_back(i);
    }
    const int64_t unit_elems = batch_unit_elems_sms(list_elems, num_sms > 0 ? num_sms : 152);
    int64_t units = 0, boxes = 0, elems = 0;
    for (size_t q = 0; q < jobs.size(); ++q) {
        BatchJob &j = jobs[q];
        j.chunk = batch_chunk(unit_elems, j.kp.vol);
        j.ubeg = (uint32_t)units;
        const int64_t cnt = ((int64_t)j.kp.ntiles + j.chunk - 1) / j.chunk;
        // the units [ubeg, ubeg + cnt) cover boxes [0, ntiles) once each:
        // unit u runs boxes [(u - ubeg) * chunk, min(+chunk, ntiles))
        const bool cover = cnt >= 1 && cnt * (int64_t)j.chunk >= (int64_t)j.kp.ntiles &&
                           (cnt - 1) * (int64_t)j.chunk < (int64_t)j.kp.ntiles;
        if (!cover || !spg_batch_job_ok(j, smem_elems) || units + cnt > 0xFFFFFFF0ll) {
            g_batch_bad_index = idx[q];
            return SPAGHETTY_ERR_CONFIG;
        }
        // the boxes, through the kernels' own index functions: the tiled
        // path stages each box in one stage of kp.stage elements
        const int rc = spg_replay_params(j.kp, fos[q], j.kind, j.kind == KIND_TILED ? (int64_t)j.kp.stage : 1,
                                         nullptr);
        if (rc) {
            g_batch_bad_index = idx[q];
            return rc;
        }
        units += cnt;
        boxes += j.kp.ntiles;
        elems += fos[q].nelem;
    }
    if (stats) {
        stats[0] = (int64_t)jobs.size();
        stats[1] = units;
        stats[2] = boxes;
        stats[3] = elems;
    }
    return SPAGHETTY_OK;
}
