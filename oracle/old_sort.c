/*
 * oracle/old_sort.c -- TEST INFRASTRUCTURE ONLY (the parity oracle).
 *
 * A plain-C restatement of NWChem's reference tensor sorts, used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
 * Nothing in the product library links or calls this file.
 *
 * Follows trunk/old_sort.f of jeffhammond/spaghetty:
 *   old_sort_0     :1-8      y = x * s
 *   old_sort_2     :10-31    y(ib) = x(ia) * s
 *   old_sort_4     :33-95    three loop orders chosen by the last index l
 *   old_sort_6     :97-234   five loop orders chosen by the last index n
 *   old_sort_8     :236-478  seven loop orders chosen by the last index p
 *   old_sortacc_0  :480-487  y = y + x * s
 *   old_sortacc_2  :489-510
 *   old_sortacc_4  :512-575
 *   old_sortacc_6  :576-714
 *   old_sortacc_8  :715-957
 *
 * Argument convention is the Fortran one: every argument by pointer, dims
 * and permutation as 4-byte integers, permutation 1-based.  The input x has
 * dims (d1..dr) with the LAST index stride-1; the output y has dims
 * (d_{p1}..d_{pr}) with index j_{pr} stride-1.
 *
 * Arithmetic: IEEE binary64, the product x*s rounded once, then (sortacc)
 * y + product rounded once.  Build with -ffp-contract=off so that the
 * compiler never fuses the two into an FMA (the Fortran source has none).
 *
 * The loop order does not change any result (each output element is written
 * exactly once), but it is restated as in the reference: the loops run over
 * the natural order with the output's fastest input index q = p_r moved to
 * just outside the innermost (input-fastest) loop, unless q is already one
 * of the two innermost indices.
 */
#include <stdint.h>
#include <stddef.h>

#define ORACLE_MAXR 8

/* Walk every element of x in the given loop order, computing the 1-based
 * Fortran offsets ia (input) and ib (output) exactly as old_sort.f does:
 *   ia = id(r) + jd(r)*(id(r-1)-1 + jd(r-1)*( ... ))
 *   ib = id(p_r) + jd(p_r)*(id(p_{r-1})-1 + jd(p_{r-1})*( ... ))
 * and apply y(ib) = x(ia)*s (acc = 0) or y(ib) = y(ib) + x(ia)*s (acc = 1). */
static void visit(int r, const int *jd, const int *p, const int *order,
                  const double *x, double *y, double s, int acc)
{
    int64_t id[ORACLE_MAXR + 1];
    int64_t total = 1;
    for (int q = 1; q <= r; ++q) {
        if (jd[q] <= 0) return;
        id[q] = 1;
        total *= jd[q];
    }
    for (int64_t it = 0; it < total; ++it) {
        /* ia = id(r) + jd(r)*(id(r-1)-1 + jd(r-1)*(... + jd(2)*(id(1)-1))) */
        int64_t ia;
        {
            int64_t acc_i = id[1] - 1;
            for (int q = 2; q <= r - 1; ++q) acc_i = id[q] - 1 + jd[q] * acc_i;
            ia = (r == 1) ? id[1] : id[r] + jd[r] * acc_i;
        }
        int64_t ib;
        {
            int64_t acc_o = id[p[1]] - 1;
            for (int q = 2; q <= r - 1; ++q) acc_o = id[p[q]] - 1 + jd[p[q]] * acc_o;
            ib = (r == 1) ? id[p[1]] : id[p[r]] + jd[p[r]] * acc_o;
        }
        const double prod = x[ia - 1] * s;
        if (acc) y[ib - 1] = y[ib - 1] + prod;
        else     y[ib - 1] = prod;
        /* advance the odometer: order[r] is the innermost loop */
        for (int q = r; q >= 1; --q) {
            const int dim = order[q];
            if (++id[dim] <= jd[dim]) break;
            id[dim] = 1;
        }
    }
}

/* The reference's loop-order rule (old_sort.f :45/:61/:77 for rank 4,
 * :112/:136/:160/:184/:208 for rank 6, :252-:444 for rank 8): keep the natural
 * order when the last permutation index q is r or r-1; otherwise loop over
 * the natural order without q, with q inserted just before the innermost r. */
static void loop_order(int r, int q, int *order)
{
    if (q == r || q == r - 1 || r <= 2) {
        for (int t = 1; t <= r; ++t) order[t] = t;
        return;
    }
    int n = 1;
    for (int t = 1; t <= r - 1; ++t)
        if (t != q) order[n++] = t;
    order[n++] = q;
    order[n] = r;
}

static int run(int r, const double *x, double *y, const int *dims,
               const int *perm, double s, int acc)
{
    int jd[ORACLE_MAXR + 1], p[ORACLE_MAXR + 1], order[ORACLE_MAXR + 1];
    for (int t = 1; t <= r; ++t) {
        jd[t] = dims[t - 1];
        p[t] = perm[t - 1];
        if (p[t] < 1 || p[t] > r) return -1;
    }
    loop_order(r, p[r], order);
    visit(r, jd, p, order, x, y, s, acc);
    return 0;
}

/* old_sort_0 / old_sortacc_0 (old_sort.f:1-8, :480-487) */
void oracle_old_sort_0(const double *x, double *y, const double *s) { *y = *x * *s; }
void oracle_old_sortacc_0(const double *x, double *y, const double *s) { *y = *y + *x * *s; }

/* old_sort_2 (old_sort.f:10-31): ib = id(j)+jd(j)*(id(i)-1) */
void oracle_old_sort_2(const double *x, double *y, const int *a, const int *b,
                       const int *i, const int *j, const double *s)
{
    const int d[2] = {*a, *b}, p[2] = {*i, *j};
    run(2, x, y, d, p, *s, 0);
}
void oracle_old_sortacc_2(const double *x, double *y, const int *a, const int *b,
                          const int *i, const int *j, const double *s)
{
    const int d[2] = {*a, *b}, p[2] = {*i, *j};
    run(2, x, y, d, p, *s, 1);
}

/* old_sort_4 (old_sort.f:33-95) and old_sortacc_4 (:512-575) */
void oracle_old_sort_4(const double *x, double *y, const int *a, const int *b,
                       const int *c, const int *d, const int *i, const int *j,
                       const int *k, const int *l, const double *s)
{
    const int dm[4] = {*a, *b, *c, *d}, p[4] = {*i, *j, *k, *l};
    run(4, x, y, dm, p, *s, 0);
}
void oracle_old_sortacc_4(const double *x, double *y, const int *a, const int *b,
                          const int *c, const int *d, const int *i, const int *j,
                          const int *k, const int *l, const double *s)
{
    const int dm[4] = {*a, *b, *c, *d}, p[4] = {*i, *j, *k, *l};
    run(4, x, y, dm, p, *s, 1);
}

/* old_sort_6 (old_sort.f:97-234) and old_sortacc_6 (:576-714) */
void oracle_old_sort_6(const double *x, double *y, const int *a, const int *b,
                       const int *c, const int *d, const int *e, const int *f,
                       const int *i, const int *j, const int *k, const int *l,
                       const int *m, const int *n, const double *s)
{
    const int dm[6] = {*a, *b, *c, *d, *e, *f}, p[6] = {*i, *j, *k, *l, *m, *n};
    run(6, x, y, dm, p, *s, 0);
}
void oracle_old_sortacc_6(const double *x, double *y, const int *a, const int *b,
                          const int *c, const int *d, const int *e, const int *f,
                          const int *i, const int *j, const int *k, const int *l,
                          const int *m, const int *n, const double *s)
{
    const int dm[6] = {*a, *b, *c, *d, *e, *f}, p[6] = {*i, *j, *k, *l, *m, *n};
    run(6, x, y, dm, p, *s, 1);
}

/* old_sort_8 (old_sort.f:236-478) and old_sortacc_8 (:715-957): dims and
 * permutation passed as arrays here, since eighteen scalar pointers add
 * nothing to a checker. */
void oracle_old_sort_8(const double *x, double *y, const int *dims,
                       const int *perm, const double *s)
{
    run(8, x, y, dims, perm, *s, 0);
}
void oracle_old_sortacc_8(const double *x, double *y, const int *dims,
                          const int *perm, const double *s)
{
    run(8, x, y, dims, perm, *s, 1);
}

/* Generic entry used by the Python side: any rank 1..8, with the general
 * two-factor update of the generated nests (trunk/generator2.py:48-130,
 * trunk/generator6.py:61-134) built from the same roundings:
 *   g == 0: y = x*f            (old_sort)
 *   g == 1: y = y + x*f        (old_sortacc)
 *   else:   y = g*y + f*x      (each product rounded, then the sum)      */
int oracle_sort_generic(int r, const double *x, double *y, const int *dims,
                        const int *perm, double f, double g)
{
    if (r < 1 || r > ORACLE_MAXR) return -1;
    if (g == 0.0) return run(r, x, y, dims, perm, f, 0);
    if (g == 1.0) return run(r, x, y, dims, perm, f, 1);
    /* general g: scale y in place in output order, then accumulate */
    int64_t n = 1;
    for (int t = 0; t < r; ++t) n *= dims[t];
    for (int64_t t = 0; t < n; ++t) y[t] = g * y[t];
    return run(r, x, y, dims, perm, f, 1);
}
