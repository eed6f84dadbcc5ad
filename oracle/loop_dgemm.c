/* loop_dgemm.c -- TEST INFRASTRUCTURE ONLY (the oracle of the fused
 * contraction; the product library never calls it).
 *
 * A C restatement of the macaroni skeleton's reference DGEMM,
 * loop_dgemm(alpha, beta, a_in, b_in, c_out, row_a, col_a, row_b, col_b,
 * row_c, col_c, case) in branches/old/python/macaroni/ccsd_t2_8_skeleton.F
 * :214-292, which the skeleton uses to check its BLAS dgemm call (:142-158).
 * Column-major matrices (Fortran), every element visited in the reference's
 * i, j, k loop order, and the update written as Fortran evaluates it:
 *   c = beta*c;  then for k in order:  c = c + (alpha*a)*b
 * Each operation rounds on its own: this file is compiled with
 * -ffp-contract=off, so no FMA is formed.
 *
 *   case 1: C(i,j) += A(i,k) * B(k,j)   ('N','N')   :226-243
 *   case 2: C(i,j) += A(i,k) * B(j,k)   ('N','T')   :244-261
 *   case 3: C(i,j) += A(k,i) * B(k,j)   ('T','N')   :262-279
 *   case 4: C(i,j) += A(k,i) * B(j,k)   ('T','T')   :280-291
 */
#include <stdint.h>

int oracle_loop_dgemm(double alpha, double beta, const double *a, const double *b, double *c,
                      int row_a, int col_a, int row_b, int col_b, int row_c, int col_c,
                      int mcase)
{
    /* the reference prints 'moron' on a shape mismatch and carries on; the
     * checker refuses instead */
    const int kmax = (mcase == 1 || mcase == 2) ? col_a : row_a;
    switch (mcase) {
    case 1: if (row_a != row_c || col_b != col_c || col_a != row_b) return -1; break;
    case 2: if (row_a != row_c || row_b != col_c || col_a != col_b) return -1; break;
    case 3: if (col_a != row_c || col_b != col_c || row_a != row_b) return -1; break;
    case 4: if (row_c != col_a || col_c != row_b || row_a != col_b) return -1; break;
    default: return -1;
    }
    for (int64_t i = 0; i < row_c; ++i) {
        for (int64_t j = 0; j < col_c; ++j) {
            const int64_t co = i + j * row_c;
            double t = beta * c[co];
            for (int64_t k = 0; k < kmax; ++k) {
                int64_t ao, bo;
                switch (mcase) {
                case 1: ao = i + k * row_a; bo = k + j * row_b; break;
                case 2: ao = i + k * row_a; bo = j + k * row_b; break;
                case 3: ao = k + i * row_a; bo = k + j * row_b; break;
                default: ao = k + i * row_a; bo = j + k * row_b; break;
                }
                const double aa = alpha * a[ao];
                t = t + aa * b[bo];
            }
            c[co] = t;
        }
    }
    return 0;
}
