// plan.cpp -- host-side folding and box planning (no CUDA calls).
#include "plan.h"
#include "../../include/spaghetty_gb300.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>

static FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d ? d : 1;
    uint32_t l = 0;
    while (l < 32 && (1ull << l) < f.d) ++l;
    f.l = l;
    uint64_t num = ((uint64_t)1 << 32) * (((uint64_t)1 << l) - f.d);
    f.m = (uint32_t)(num / f.d + 1);
    return f;
}

FastDiv spg_make_fastdiv(uint32_t d) { return make_fastdiv(d); }

// ---------------------------------------------------------------------------
// Folding.  perm is 1-based (reference convention, trunk/old_sort.f:44-56).
int spg_fold(int rank, const int *dims, const int *perm, Folded *out) {
    std::memset(out, 0, sizeof(*out));
    if (rank < 1 || rank > SPG_MAXR) return SPAGHETTY_ERR_RANK;
    if (!dims || !perm) return SPAGHETTY_ERR_NULL;
    bool seen[SPG_MAXR] = {false};
    for (int q = 0; q < rank; ++q) {
        int p = perm[q];
        if (p < 1 || p > rank || seen[p - 1]) return SPAGHETTY_ERR_PERM;
        seen[p - 1] = true;
    }
    int64_t n = 1;
    bool empty = false;
    for (int q = 0; q < rank; ++q) {
        if (dims[q] < 0) return SPAGHETTY_ERR_DIMS;
        if (dims[q] == 0) empty = true;
    }
    if (!empty) {
        for (int q = 0; q < rank; ++q) {
            if (n > INT64_MAX / dims[q]) return SPAGHETTY_ERR_OVERFLOW;
            n *= dims[q];
        }
    }
    out->nelem = empty ? 0 : n;
    out->empty = empty;
    if (empty) return SPAGHETTY_OK;

    // 1. drop unit dims
    int newidx[SPG_MAXR];
    int64_t D1[SPG_MAXR];
    int r1 = 0;
    for (int d = 0; d < rank; ++d) {
        if (dims[d] > 1) { newidx[d] = r1; D1[r1++] = dims[d]; }
        else newidx[d] = -1;
    }
    int P1[SPG_MAXR];
    int np = 0;
    for (int q = 0; q < rank; ++q) {
        int d = perm[q] - 1;
        if (newidx[d] >= 0) P1[np++] = newidx[d];
    }
    // 2. fuse runs that are adjacent and ordered in both input and output
    //    group g (output order) = consecutive output positions whose input
    //    dims are consecutive increasing
    int gstart[SPG_MAXR], glen[SPG_MAXR], ng = 0;
    for (int q = 0; q < r1; ++q) {
        if (q > 0 && P1[q] == P1[q - 1] + 1) { glen[ng - 1]++; }
        else { gstart[ng] = q; glen[ng] = 1; ++ng; }
    }
    // groups sorted by their first input dim give the folded input order
    int order[SPG_MAXR];
    for (int g = 0; g < ng; ++g) order[g] = g;
    std::sort(order, order + ng, [&](int a, int b) { return P1[gstart[a]] < P1[gstart[b]]; });
    int pos_in[SPG_MAXR];
    for (int k = 0; k < ng; ++k) pos_in[order[k]] = k;
    out->rank = ng;
    for (int k = 0; k < ng; ++k) {
        int g = order[k];
        int64_t e = 1;
        for (int t = 0; t < glen[g]; ++t) e *= D1[P1[gstart[g]] + t];
        out->D[k] = e;
    }
    for (int g = 0; g < ng; ++g) out->P[g] = pos_in[g];
    return SPAGHETTY_OK;
}

// Factor class: 0 = one, 1 = minus one, 2 = +-2^k, 3 = any other value.
static int factor_class(double f, int *kout) {
    *kout = 0;
    if (f == 1.0) return 0;
    if (f == -1.0) return 1;
    if (!std::isfinite(f) || f == 0.0) return 3;
    int e = 0;
    const double m = std::frexp(f, &e);     // f = m * 2^e, |m| in [0.5, 1)
    if (std::fabs(m) == 0.5 && e - 1 >= -1100 && e - 1 <= 1100) {
        *kout = e - 1;
        return 2;
    }
    return 3;
}

int spg_choose_op(double f, double g) {
    int k;
    const int fc = factor_class(f, &k);
    if (g == 0.0) return OP_SORT_ONE + fc;
    if (g == 1.0) return OP_ACC_ONE + fc;
    return OP_GEN;
}

SpgFactor spg_make_factor(double f, double g) {
    SpgFactor F;
    std::memset(&F, 0, sizeof(F));
    F.f = f;
    F.g = g;
    int k = 0;
    const int fc = factor_class(f, &k);
    // f = 1 and f = -1 get the fields of +-2^0 too: tuned TMA-staged plans
    // of large arrays run them on the power-of-two path
    if (fc <= 2) {
        F.k = k;
        F.sgn_hi = std::signbit(f) ? 0x80000000u : 0u;
        // biased exponents e of x with 1 <= e <= 2046 and 1 <= e + k <= 2046
        const int elo = std::max(1, 1 - k), ehi = std::min(2046, 2046 - k);
        if (elo <= ehi) {
            F.elo = (uint32_t)elo << 20;
            F.erange = (uint32_t)(ehi - elo + 1) << 20;
        }
    }
    // the integer multiply's operand: f normal (biased exponent 1..2046)
    uint64_t bits;
    std::memcpy(&bits, &f, sizeof(bits));
    const int ef = (int)((bits >> 52) & 0x7FF);
    if (ef >= 1 && ef <= 2046) {
        const uint64_t m = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        F.mhi = (uint32_t)(m >> 32);
        F.mlo = (uint32_t)m;
        F.ebias = ef - 1023;
        F.mul_ok = 1;
        if (fc > 2) F.sgn_hi = std::signbit(f) ? 0x80000000u : 0u;
    }
    return F;
}

// ---------------------------------------------------------------------------
// Box selection.
namespace {

struct Shape {
    int R;
    int64_t D[SPG_MAXR];
    int in_order[SPG_MAXR];   // input dims, fastest first
    int out_order[SPG_MAXR];  // input dims in output order, fastest first
};

int64_t run_len(const Shape &s, const int64_t *L, const int *order) {
    int64_t r = 1;
    for (int q = 0; q < s.R; ++q) {
        int d = order[q];
        r *= L[d];
        if (L[d] < s.D[d]) break;
    }
    return r;
}

int frontier(const Shape &s, const int64_t *L, const int *order) {
    for (int q = 0; q < s.R; ++q)
        if (L[order[q]] < s.D[order[q]]) return order[q];
    return -1;
}

int64_t volume(const Shape &s, const int64_t *L) {
    int64_t v = 1;
    for (int d = 0; d < s.R; ++d) v *= L[d];
    return v;
}

// smallest even split of D into boxes of length >= want
int64_t split_len(int64_t D, int64_t want) {
    if (want >= D) return D;
    if (want < 1) want = 1;
    int64_t nt = std::max<int64_t>(1, D / want);
    return (D + nt - 1) / nt;
}

int64_t largest_divisor_le(int64_t D, int64_t v) {
    for (int64_t x = std::min(D, v); x > 1; --x)
        if (D % x == 0) return x;
    return 1;
}

}  // namespace

static const int kTRun = 32;      // minimum contiguous doubles per box row
static const int kDirectRun = 16;  // shortest shared stride-1 row of the direct kernel
static const int kVMax = 4096;    // largest box (512 threads x 8)
static const int kDefaultStages = 3;
static const int kBatchThreads = SPG_BATCH_NT;
static const int kBatchEpt = SPG_BATCH_EPT;

// Greedy box: grow the box until the input rows hold trun_in and the output
// rows trun_out contiguous doubles (or the whole extent of that side), then
// towards a target volume: vtarget when positive, else one that still leaves
// a few boxes per SM.
static void choose_box_t(const Shape &s, int64_t nelem, int num_sms, int64_t *L, int vmax,
                         int trun_in, int trun_out, int vtarget) {
    for (int d = 0; d < s.R; ++d) L[d] = 1;
    // phase 1: both runs long enough
    for (int it = 0; it < 64; ++it) {
        int64_t vol = volume(s, L);
        int64_t ri = run_len(s, L, s.in_order), ro = run_len(s, L, s.out_order);
        int d = -1;
        int64_t need = 0;
        if (ri < trun_in && (d = frontier(s, L, s.in_order)) >= 0) {
            need = (trun_in * L[d] + ri - 1) / ri;
        } else if (ro < trun_out && (d = frontier(s, L, s.out_order)) >= 0) {
            need = (trun_out * L[d] + ro - 1) / ro;
        } else {
            break;
        }
        int64_t nl = split_len(s.D[d], need);
        if (vol / L[d] * nl > vmax) nl = std::max<int64_t>(L[d], vmax * L[d] / vol);
        if (nl <= L[d]) break;
        L[d] = nl;
    }
    // phase 2: grow the box towards a target volume that still leaves
    // enough boxes to fill every SM a few times
    int64_t target = nelem / (4 * (int64_t)std::max(1, num_sms));
    target = std::max<int64_t>(256, std::min<int64_t>(2048, target));
    if (vtarget > 0) target = vtarget;
    for (int it = 0; it < 64; ++it) {
        int64_t vol = volume(s, L);
        if (vol >= target) break;
        int64_t ri = run_len(s, L, s.in_order), ro = run_len(s, L, s.out_order);
        int fi = frontier(s, L, s.in_order), fo = frontier(s, L, s.out_order);
        int d = -1;
        if (fi >= 0 && fo >= 0) d = (ro <= ri) ? fo : fi;
        else if (fo >= 0) d = fo;
        else if (fi >= 0) d = fi;
        if (d < 0) break;
        int64_t want = std::min<int64_t>(L[d] * 2, L[d] * std::max<int64_t>(2, target / vol));
        int64_t nl = split_len(s.D[d], want);
        if (vol / L[d] * nl > vmax) {
            if (vtarget > 0) break;      // explicit targets stop at the cap (the autotuner's greedy)
            nl = largest_divisor_le(s.D[d], vmax * L[d] / vol);
        }
        if (nl <= L[d]) break;
        L[d] = nl;
    }
    // at most two dims may end in a partial box (they carry element masks):
    // keep the two frontier dims, round any other partial dim down to a divisor
    const int fi = frontier(s, L, s.in_order), fo = frontier(s, L, s.out_order);
    for (int d = 0; d < s.R; ++d)
        if (L[d] < s.D[d] && s.D[d] % L[d] != 0 && d != fi && d != fo)
            L[d] = largest_divisor_le(s.D[d], L[d]);
}

static void choose_box(const Shape &s, int64_t nelem, int num_sms, int64_t *L, int vmax) {
    choose_box_t(s, nelem, num_sms, L, vmax, kTRun, kTRun, 0);
}

static int pick_block(int vol, int *threads, int *ept) {
    static const int nts[3] = {256, 512, 128};
    static const int epts[4] = {1, 2, 4, 8};
    int best = INT_MAX, bt = 0, be = 0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 4; ++b) {
            int cap = nts[a] * epts[b];
            if (cap < vol) continue;
            if (cap < best) { best = cap; bt = nts[a]; be = epts[b]; }
        }
    if (!bt) return SPAGHETTY_ERR_NOKERNEL;
    *threads = bt;
    *ept = be;
    return SPAGHETTY_OK;
}

// Count shared-memory wavefronts of the store phase (8-byte words: a half
// warp is served per wavefront when its 16 words fall in distinct bank
// pairs) for one pad choice.
static int64_t smem_wavefronts(const Plan &pl, int pad, const int *e_in_of_out, int V) {
    int64_t total = 0;
    const int NT = pl.threads;
    const int nwarps = std::min(NT / 32, 8);
    for (int k = 0; k < pl.ept; ++k)
        for (int w = 0; w < nwarps; ++w)
            for (int h = 0; h < 2; ++h) {
                int64_t words[16];
                int nw = 0;
                for (int t = 0; t < 16; ++t) {
                    int e = k * NT + w * 32 + h * 16 + t;
                    if (e >= V) continue;
                    int64_t idx = e_in_of_out[e];
                    if (pad) idx += idx / pad;
                    words[nw++] = idx;
                }
                // the words are distinct (slot -> element and the padded
                // index are both one-to-one): count banks directly
                int cnt[16] = {0};
                int worst = 0;
                for (int a = 0; a < nw; ++a) worst = std::max(worst, ++cnt[(int)(words[a] & 15)]);
                total += worst;
            }
    return total;
}

int spg_plan(const Folded &fo, int op, const int *box_override, int threads_override,
             int ept_override, int stages_override, int num_sms, Plan *pl) {
    std::memset(pl, 0, sizeof(*pl));
    pl->fo = fo;
    pl->op = op;
    if (fo.empty) { pl->kind = KIND_EMPTY; return SPAGHETTY_OK; }
    const int R = fo.rank;
    if (R <= 1 && !box_override) {
        pl->kind = KIND_FLAT;
        pl->threads = 256;
        pl->ept = 8;
        pl->run_in = pl->run_out = (int)std::min<int64_t>(fo.nelem, INT_MAX);
        return SPAGHETTY_OK;
    }
    Shape s;
    s.R = R;
    for (int d = 0; d < R; ++d) { s.D[d] = fo.D[d]; s.in_order[d] = R - 1 - d; }
    for (int q = 0; q < R; ++q) s.out_order[q] = fo.P[R - 1 - q];
    int64_t L[SPG_MAXR];
    if (box_override) {
        for (int d = 0; d < R; ++d) {
            if (box_override[d] < 1 || box_override[d] > s.D[d]) return SPAGHETTY_ERR_CONFIG;
            L[d] = box_override[d];
        }
        int np = 0;
        for (int d = 0; d < R; ++d) if (s.D[d] % L[d]) ++np;
        if (np > 2) return SPAGHETTY_ERR_CONFIG;
    } else {
        choose_box(s, fo.nelem, num_sms, L, kVMax);
    }
    int64_t vol = volume(s, L);
    if (vol > kVMax) return SPAGHETTY_ERR_CONFIG;
    for (int d = 0; d < R; ++d) pl->box[d] = (int)L[d];
    pl->run_in = (int)run_len(s, L, s.in_order);
    pl->run_out = (int)run_len(s, L, s.out_order);
    // direct (no staging) only when the shared stride-1 dim alone gives
    // coalesced rows on both sides: at least 16 doubles, one full 128-byte
    // line per half warp (measured on GB300 over the 44 rank-6 perms of
    // 16^6 that keep the stride-1 index and take no bulk tensor copy: 5815
    // against 5403 GB/s staged through shared memory; non-cubic 5299
    // against 4693)
    const bool same_fastest = (fo.P[R - 1] == R - 1);
    pl->kind = (same_fastest && L[R - 1] >= kDirectRun) ? KIND_DIRECT : KIND_TILED;
    if (threads_override) {
        pl->threads = threads_override;
        pl->ept = ept_override;
        if (pl->threads * pl->ept < vol) return SPAGHETTY_ERR_CONFIG;
        pl->stages = stages_override;
    } else {
        int rc = pick_block((int)vol, &pl->threads, &pl->ept);
        if (rc) return rc;
        pl->stages = kDefaultStages;
    }
    if (pl->kind != KIND_TILED) pl->stages = 0;
    if (pl->stages != 0 && pl->stages != 2 && pl->stages != 3) return SPAGHETTY_ERR_CONFIG;
    if (pl->stages && pl->ept < 2) pl->stages = 0;
    return SPAGHETTY_OK;
}

// Default box for the TMA-staged kernel: smaller than the register-staged
// kernels' (boxes of ~1-2K elements keep 3-4 CTAs and their pipelines
// resident per SM), with the same >= 32-double runs on both sides.
int spg_default_box_tma(const Folded &fo, int num_sms, int vmax, int *box) {
    if (fo.empty || fo.rank < 2) return SPAGHETTY_ERR_CONFIG;
    const int R = fo.rank;
    Shape s;
    s.R = R;
    for (int d = 0; d < R; ++d) { s.D[d] = fo.D[d]; s.in_order[d] = R - 1 - d; }
    for (int q = 0; q < R; ++q) s.out_order[q] = fo.P[R - 1 - q];
    int64_t L[SPG_MAXR];
    choose_box(s, std::min<int64_t>(fo.nelem, (int64_t)1024 * 4 * std::max(1, num_sms)), num_sms, L, vmax);
    // the bulk copy's innermost box row must be a multiple of 16 bytes
    if (L[R - 1] % 2 && L[R - 1] < s.D[R - 1]) L[R - 1] += 1;
    const int ob = fo.P[R - 1];
    if (L[ob] % 2 && L[ob] < s.D[ob]) L[ob] += 1;
    int64_t vol = 1;
    for (int d = 0; d < R; ++d) vol *= L[d];
    if (vol > vmax) return SPAGHETTY_ERR_CONFIG;
    for (int d = 0; d < R; ++d) box[d] = (int)L[d];
    return SPAGHETTY_OK;
}

// The greedy box with explicit run and volume targets (the autotuner's box
// family), for the default plans of api.cu.
int spg_box_greedy(const Folded &fo, int trun_in, int trun_out, int vtarget, int vmax, int *box) {
    if (fo.empty || fo.rank < 2) return SPAGHETTY_ERR_CONFIG;
    const int R = fo.rank;
    Shape s;
    s.R = R;
    for (int d = 0; d < R; ++d) { s.D[d] = fo.D[d]; s.in_order[d] = R - 1 - d; }
    for (int q = 0; q < R; ++q) s.out_order[q] = fo.P[R - 1 - q];
    int64_t L[SPG_MAXR];
    choose_box_t(s, fo.nelem, 1, L, vmax, trun_in, trun_out, vtarget);
    if (volume(s, L) > vmax) return SPAGHETTY_ERR_CONFIG;
    for (int d = 0; d < R; ++d) box[d] = (int)L[d];
    return SPAGHETTY_OK;
}

// Plan for one sort of a batch: the persistent batched kernel runs every
// sort with one CTA shape (256 threads x 8 elements), so boxes are capped at
// 2048 elements, and a rank <= 1 problem becomes a 1-D direct box.
int spg_plan_batch(const Folded &fo, int op, const SpgBatchRule *rule, Plan *pl) {
    std::memset(pl, 0, sizeof(*pl));
    pl->fo = fo;
    pl->op = op;
    if (fo.empty) { pl->kind = KIND_EMPTY; return SPAGHETTY_OK; }
    pl->threads = kBatchThreads;
    pl->ept = kBatchEpt;
    pl->stages = 0;
    const int vmax = kBatchThreads * kBatchEpt;
    if (fo.rank <= 1) {
        pl->fo.rank = 1;
        pl->fo.D[0] = fo.nelem;
        pl->fo.P[0] = 0;
        pl->box[0] = (int)std::min<int64_t>(fo.nelem, vmax);
        pl->kind = KIND_DIRECT;
        pl->run_in = pl->run_out = pl->box[0];
        return SPAGHETTY_OK;
    }
    const int R = fo.rank;
    Shape s;
    s.R = R;
    for (int d = 0; d < R; ++d) { s.D[d] = fo.D[d]; s.in_order[d] = R - 1 - d; }
    for (int q = 0; q < R; ++q) s.out_order[q] = fo.P[R - 1 - q];
    int64_t L[SPG_MAXR];
    // many sorts share the GPU, so aim for full-size boxes, unless a tuned
    // rule for this size bucket says otherwise
    if (rule)
        choose_box_t(s, (int64_t)1 << 40, 1, L, vmax, rule->run_in, rule->run_out,
                     std::min(rule->volume, vmax));
    else
        choose_box(s, (int64_t)1 << 40, 1, L, vmax);
    for (int d = 0; d < R; ++d) pl->box[d] = (int)L[d];
    pl->run_in = (int)run_len(s, L, s.in_order);
    pl->run_out = (int)run_len(s, L, s.out_order);
    const bool same_fastest = (fo.P[R - 1] == R - 1);
    pl->kind = (same_fastest && L[R - 1] >= kTRun) ? KIND_DIRECT : KIND_TILED;
    return volume(s, L) <= vmax ? SPAGHETTY_OK : SPAGHETTY_ERR_CONFIG;
}

// Order of the box grid's dims, fastest-varying first.  Dims that the box
// covers partially (1 < L < D) come first: two boxes that are neighbours
// along such a dim share the cache lines at their common edge, and giving
// them consecutive box indices keeps both in flight at the same time, so the
// shared lines are fetched from DRAM once.  The remaining dims (L == 1)
// follow, all in output order.  Returns the number of dims listed.
static int grid_order(const Plan &pl, int *dims_out) {
    const Folded &fo = pl.fo;
    const int R = fo.rank;
    int n = 0;
    for (int pass = 0; pass < 2; ++pass)
        for (int q = R - 1; q >= 0; --q) {
            const int d = fo.P[q];
            const int64_t c = (fo.D[d] + pl.box[d] - 1) / pl.box[d];
            if (c <= 1) continue;
            const bool partial = pl.box[d] > 1;
            if ((pass == 0) == partial) dims_out[n++] = d;
        }
    return n;
}

// ---------------------------------------------------------------------------
// Kernel parameter block.
int spg_build_params(Plan *pl, double f, double g) {
    KParams &kp = pl->kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.fac = spg_make_factor(f, g);
    if (pl->kind == KIND_EMPTY) return SPAGHETTY_OK;
    if (pl->kind == KIND_FLAT) { kp.nelem = pl->fo.nelem; return SPAGHETTY_OK; }
    const Folded &fo = pl->fo;
    const int R = fo.rank;
    int64_t istr[SPG_MAXR], ostr[SPG_MAXR];   // per input dim
    int pinv[SPG_MAXR];
    for (int q = 0; q < R; ++q) pinv[fo.P[q]] = q;
    {
        int64_t s = 1;
        for (int d = R - 1; d >= 0; --d) { istr[d] = s; s *= fo.D[d]; }
        int64_t so = 1;
        int64_t ostr_pos[SPG_MAXR];
        for (int q = R - 1; q >= 0; --q) { ostr_pos[q] = so; so *= fo.D[fo.P[q]]; }
        for (int d = 0; d < R; ++d) ostr[d] = ostr_pos[pinv[d]];
    }
    // partial (masked) dims
    int pA = -1, pB = -1;
    for (int d = 0; d < R; ++d)
        if (fo.D[d] % pl->box[d]) {
            if (pA < 0) pA = d;
            else if (pB < 0) pB = d;
            else return SPAGHETTY_ERR_CONFIG;
        }
    pl->masked = (pA >= 0);
    // the per-box limit arithmetic of masked dims is 32-bit
    if ((pA >= 0 && fo.D[pA] > INT32_MAX / 2) || (pB >= 0 && fo.D[pB] > INT32_MAX / 2))
        return SPAGHETTY_ERR_NOKERNEL;
    kp.lenA = pA >= 0 ? pl->box[pA] : 1;
    kp.extA = pA >= 0 ? (int32_t)fo.D[pA] : 1;
    kp.lenB = pB >= 0 ? pl->box[pB] : 1;
    kp.extB = pB >= 0 ? (int32_t)fo.D[pB] : 1;
    auto mp = [&](int d) -> int8_t { return d == pA ? 1 : (d == pB ? 2 : 0); };
    // box-local input-order strides
    int32_t bs[SPG_MAXR];
    {
        int32_t s = 1;
        for (int d = R - 1; d >= 0; --d) { bs[d] = s; s *= pl->box[d]; }
        kp.vol = s;
    }
    int64_t maxoff_in = 0, maxoff_out = 0;
    // load walk: input order, fastest first
    kp.ld.n = 0;
    for (int d = R - 1; d >= 0; --d) {
        if (pl->box[d] <= 1) continue;
        int k = kp.ld.n++;
        kp.ld.len[k] = make_fastdiv((uint32_t)pl->box[d]);
        kp.ld.gs_a[k] = istr[d];
        kp.ld.gs_b[k] = ostr[d];
        kp.ld.bs[k] = bs[d];
        kp.ld.mpos[k] = mp(d);
        maxoff_in += (int64_t)(pl->box[d] - 1) * istr[d];
        maxoff_out += (int64_t)(pl->box[d] - 1) * ostr[d];
    }
    // store walk: output order, fastest first
    kp.st.n = 0;
    for (int q = R - 1; q >= 0; --q) {
        int d = fo.P[q];
        if (pl->box[d] <= 1) continue;
        int k = kp.st.n++;
        kp.st.len[k] = make_fastdiv((uint32_t)pl->box[d]);
        kp.st.gs_a[k] = ostr[d];
        kp.st.gs_b[k] = istr[d];
        kp.st.bs[k] = bs[d];
        kp.st.mpos[k] = mp(d);
    }
    if (maxoff_in > INT32_MAX || maxoff_out > INT32_MAX) return SPAGHETTY_ERR_NOKERNEL;
    // grid of boxes (grid_order)
    int64_t ntiles = 1;
    kp.grid.n = 0;
    int gdims[SPG_MAXR];
    const int ng = grid_order(*pl, gdims);
    for (int gi = 0; gi < ng; ++gi) {
        const int d = gdims[gi];
        const int64_t c = (fo.D[d] + pl->box[d] - 1) / pl->box[d];
        int k = kp.grid.n++;
        kp.grid.cnt[k] = make_fastdiv((uint32_t)c);
        kp.grid.in_step[k] = (int64_t)pl->box[d] * istr[d];
        kp.grid.out_step[k] = (int64_t)pl->box[d] * ostr[d];
        kp.grid.mpos[k] = mp(d);
        ntiles *= c;
        if (c > INT32_MAX || ntiles > INT32_MAX) return SPAGHETTY_ERR_NOKERNEL;
    }
    kp.ntiles = (uint32_t)ntiles;
    // shared-memory padding for the tiled kernel: pick the pad period with the
    // fewest store-phase wavefronts among {none, stride of the output-fastest
    // box dim in the input-ordered tile}
    kp.pad = 0;
    if (pl->kind == KIND_TILED && kp.st.n > 0) {
        int e_in[kVMax];   // on the stack: planning never touches the heap
        for (int e = 0; e < kp.vol; ++e) {
            int rem = e, lin = 0;
            for (int k = 0; k < kp.st.n; ++k) {
                int len = (int)kp.st.len[k].d;
                lin += (rem % len) * kp.st.bs[k];
                rem /= len;
            }
            e_in[e] = lin;
        }
        int cands[3] = {0, (int)kp.st.bs[0], (int)kp.st.bs[0] * 2};
        int64_t best = -1;
        for (int c : cands) {
            if (c < 0 || (c && c >= kp.vol)) continue;
            int64_t w = smem_wavefronts(*pl, c, e_in, kp.vol);
            if (c == 0) pl->wf_pad0 = w;
            if (best < 0 || w < best) { best = w; kp.pad = c; }
        }
        // conflict-free: one wavefront per half warp of live elements
        {
            const int nwarps = std::min(pl->threads / 32, 8);
            int64_t ideal = 0;
            for (int k = 0; k < pl->ept; ++k)
                for (int w = 0; w < nwarps; ++w)
                    for (int h = 0; h < 2; ++h)
                        if (k * pl->threads + w * 32 + h * 16 < kp.vol) ++ideal;
            pl->wf_ideal = ideal;
        }
    }
    const int tile = kp.vol + (kp.pad ? kp.vol / kp.pad + 1 : 0);
    kp.stage = (tile + 15) & ~15;   // 128-byte aligned stages
    if (pl->kind != KIND_TILED) pl->smem_bytes = 0;
    else if (pl->stages) pl->smem_bytes = pl->stages * kp.stage * (int)sizeof(double);
    else pl->smem_bytes = tile * (int)sizeof(double);
    return SPAGHETTY_OK;
}

// ---------------------------------------------------------------------------
int spg_selftest_host(void) {
    // fast division against plain division
    uint32_t ds[] = {1, 2, 3, 5, 6, 7, 10, 12, 16, 17, 20, 29, 30, 31, 33, 100, 255,
                     1000, 4096, 65537, 1000003, 0x7fffffffu};
    uint32_t ns[] = {0, 1, 2, 3, 31, 32, 33, 999, 1000, 65535, 65536, 1u << 20,
                     123456789, 0x7ffffffeu, 0x7fffffffu};
    for (uint32_t d : ds) {
        FastDiv f = make_fastdiv(d);
        for (uint32_t n : ns)
            if (fd_div(n, f) != n / d) return 1;
        uint64_t x = 88172645463325252ull;
        for (int t = 0; t < 20000; ++t) {
            x ^= x << 13; x ^= x >> 7; x ^= x << 17;
            uint32_t n = (uint32_t)(x & 0x7fffffffu);
            if (fd_div(n, f) != n / d) return 1;
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// TMA layout.  Folded dims are grouped, fastest first, into at most five
// tensor-map dims: a slower dim joins the current group when every dim
// already in it is covered by the box in full (the group is then one
// contiguous range), or when it and every dim already in the group have
// box length 1, and in both cases only when its stride continues the
// group's memory range.  A dim whose box is longer than 256 elements is
// split into two map dims.  Box lengths along a map dim are at most 256, the
// innermost box row is a multiple of 16 bytes, and every stride a multiple
// of 16 bytes (the bulk tensor copy's rules); otherwise the plan is not
// TMA-eligible.
static int tma_map(const Plan &pl, const int *order, const int64_t *gstride, int *nmap,
                   uint64_t *dim, uint64_t *stride, uint32_t *box, int8_t *mdim_of,
                   int64_t *weight_of) {
    const Folded &fo = pl.fo;
    const int R = fo.rank;
    int m = -1;
    bool group_full = false, group_unit = false;
    for (int q = 0; q < R; ++q) {
        const int d = order[q];
        const int64_t D = fo.D[d];
        const int64_t L = pl.box[d];
        bool merge = false;
        // a dim joins the group only where it continues the group's memory
        // range (its stride is the group's stride times the group's extent)
        // and the group's box stays within the bulk copy's 256 per dim (a
        // longer one would be rejected below; unmerged, the dims keep the
        // same element order in the tile)
        if (m >= 0 && (uint64_t)gstride[d] * 8u == stride[m] * dim[m]) {
            if (group_full && (int64_t)box[m] * L <= 256) merge = true;
            else if (group_unit && L == 1) merge = true;
        }
        if (merge) {
            weight_of[d] = (int64_t)dim[m];
            dim[m] *= (uint64_t)D;
            box[m] = (uint32_t)((int64_t)box[m] * L);
            group_full = group_full && (L == D);
            group_unit = group_unit && (L == 1);
        } else if (L > 256) {
            // a box row longer than the bulk copy allows: split the dim into
            // an inner map dim of w elements (whole box rows of w) and an
            // outer one, w dividing both the box length and the extent; the
            // outer coordinate is the element offset / w (weight -w)
            int64_t w = 256;
            const bool inner = (m < 0);
            for (; w > 1; --w)
                if (L % w == 0 && D % w == 0 && (!inner || (w * 8) % 16 == 0)) break;
            if (w <= 1 || m + 2 >= 5) return SPAGHETTY_ERR_NOKERNEL;
            ++m;
            dim[m] = (uint64_t)w;
            box[m] = (uint32_t)w;
            stride[m] = (uint64_t)gstride[d] * 8u;
            ++m;
            dim[m] = (uint64_t)(D / w);
            box[m] = (uint32_t)(L / w);
            stride[m] = (uint64_t)gstride[d] * 8u * (uint64_t)w;
            weight_of[d] = -w;
            group_full = (L == D);
            group_unit = false;
        } else {
            if (++m >= 5) return SPAGHETTY_ERR_NOKERNEL;
            dim[m] = (uint64_t)D;
            box[m] = (uint32_t)L;
            stride[m] = (uint64_t)gstride[d] * 8u;
            weight_of[d] = 1;
            group_full = (L == D);
            group_unit = (L == 1);
        }
        mdim_of[d] = (int8_t)m;
    }
    *nmap = m + 1;
    for (int k = 0; k < *nmap; ++k) {
        if (box[k] < 1 || box[k] > 256) return SPAGHETTY_ERR_NOKERNEL;
        if (dim[k] > ((uint64_t)1 << 31)) return SPAGHETTY_ERR_NOKERNEL;
        if (k > 0 && (stride[k] % 16 != 0 || stride[k] >= ((uint64_t)1 << 40))) return SPAGHETTY_ERR_NOKERNEL;
    }
    if (stride[0] != 8 || (box[0] * 8u) % 16u != 0) return SPAGHETTY_ERR_NOKERNEL;
    // pad to five dims with unit dims
    for (int k = *nmap; k < 5; ++k) {
        dim[k] = 1;
        box[k] = 1;
        stride[k] = stride[k - 1] * dim[k - 1];
        if (stride[k] >= ((uint64_t)1 << 40)) return SPAGHETTY_ERR_NOKERNEL;
    }
    return SPAGHETTY_OK;
}

int spg_tma_layout(const Plan &pl, int stages, TmaLayout *out) {
    std::memset(out, 0, sizeof(*out));
    if (pl.kind != KIND_TILED && pl.kind != KIND_TMA && pl.kind != KIND_DIRECT) return SPAGHETTY_ERR_NOKERNEL;
    const Folded &fo = pl.fo;
    const int R = fo.rank;
    if (R < 1) return SPAGHETTY_ERR_NOKERNEL;
    int64_t istr[SPG_MAXR], ostr[SPG_MAXR];
    {
        int pinv[SPG_MAXR];
        for (int q = 0; q < R; ++q) pinv[fo.P[q]] = q;
        int64_t s = 1;
        for (int d = R - 1; d >= 0; --d) { istr[d] = s; s *= fo.D[d]; }
        int64_t so = 1, op[SPG_MAXR];
        for (int q = R - 1; q >= 0; --q) { op[q] = so; so *= fo.D[fo.P[q]]; }
        for (int d = 0; d < R; ++d) ostr[d] = op[pinv[d]];
    }
    // When the stride-1 index is the same on both sides, the output map
    // lists its dims in INPUT order (each with its output stride): the tile
    // is then laid out identically for the load and the store, and the
    // permute step is the identity.
    const bool same_order = fo.P[R - 1] == R - 1;
    int in_order[SPG_MAXR], out_order[SPG_MAXR];
    for (int q = 0; q < R; ++q) {
        in_order[q] = R - 1 - q;
        out_order[q] = same_order ? R - 1 - q : fo.P[R - 1 - q];
    }
    int8_t mi[SPG_MAXR], mo[SPG_MAXR];
    int64_t wi[SPG_MAXR], wo[SPG_MAXR];
    int rc = tma_map(pl, in_order, istr, &out->rank_in, out->in_dim, out->in_stride, out->in_box, mi, wi);
    if (rc) return rc;
    rc = tma_map(pl, out_order, ostr, &out->rank_out, out->out_dim, out->out_stride, out->out_box, mo, wo);
    if (rc) return rc;
    // grid dims in the order spg_build_params lists them (grid_order)
    const KParams &kp = pl.kp;
    int k = 0;
    int gdims[SPG_MAXR];
    const int ng = grid_order(pl, gdims);
    for (int gi = 0; gi < ng; ++gi) {
        const int d = gdims[gi];
        const int64_t c = (fo.D[d] + pl.box[d] - 1) / pl.box[d];
        if (k >= kp.grid.n) return SPAGHETTY_ERR_CONFIG;
        // coordinate step of one box along d (a split dim moves its outer
        // map dim by box / w)
        const int64_t mul_in = wi[d] > 0 ? (int64_t)pl.box[d] * wi[d] : (int64_t)pl.box[d] / -wi[d];
        const int64_t mul_out = wo[d] > 0 ? (int64_t)pl.box[d] * wo[d] : (int64_t)pl.box[d] / -wo[d];
        if (mul_in * c > INT32_MAX || mul_out * c > INT32_MAX) return SPAGHETTY_ERR_NOKERNEL;
        out->tp.in_mdim[k] = mi[d];
        out->tp.out_mdim[k] = mo[d];
        out->tp.in_mul[k] = (int32_t)mul_in;
        out->tp.out_mul[k] = (int32_t)mul_out;
        ++k;
    }
    if (k != kp.grid.n) return SPAGHETTY_ERR_CONFIG;
    // each bulk load delivers exactly one box: the mbarrier's transaction
    // count must equal it
    int64_t pin = 1, pout = 1;
    for (int m = 0; m < 5; ++m) { pin *= out->in_box[m]; pout *= out->out_box[m]; }
    if (pin != kp.vol || pout != kp.vol) return SPAGHETTY_ERR_NOKERNEL;
    const int64_t tile = (int64_t)kp.vol * 8;
    const int64_t tile_al = (tile + 1023) & ~(int64_t)1023;
    const bool reads_out = spg_op_class(pl.op) != 0;
    // load stage = input tile [+ old-output tile (sortacc)]; two output
    // slots follow the stages
    out->tp.in_bytes = (int32_t)tile_al;
    out->tp.out_bytes = (int32_t)tile_al;
    out->tp.stage_bytes = (int32_t)(tile_al * (reads_out ? 2 : 1));
    out->tp.tx_bytes = (int32_t)(tile * (reads_out ? 2 : 1));
    out->tp.same_order = same_order ? 1 : 0;
    out->tp.sk_stride = pl.sk_stride;
    out->tp.sk_len = pl.sk_len;
    out->tp.sk_mul = pl.sk_mul;
    (void)stages;
    return SPAGHETTY_OK;
}
