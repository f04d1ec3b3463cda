/* femtc CPU oracle: test infrastructure only.
 *
 * This is the checker for the GPU operator library, never part of it.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * Everything here is FP64 and restates the reference's per-cell algorithm
 * (IgorBaratta/femtc src/mass.hpp, src/stiffness.hpp, src/linalg.hpp,
 * src/tmm.hpp) with general quadrature size Q.
 *
 * Layouts (the reference's):
 *   u, y      : [cell][i0][i1][i2], N^3 per cell, i0 slowest (src/mass.hpp:25-29)
 *   D (mass)  : [cell][q0][q1][q2], Q^3 per cell           (src/mass.hpp:27)
 *   G (stiff) : [cell][q][6], components [zz,yz,xz,yy,xy,xx] (src/stiffness.hpp:20-27)
 *   tables    : Phi(q,i) = tables[q + i*Q] (column-major QxN, src/linalg.hpp:49),
 *               Gamma(q,i) = tables[Q*N + q + i*Q]        (src/stiffness.hpp:45)
 *
 * Semantics:
 *   ORACLE_EXACT     : the true operators y = B^T D B u and
 *                      y = sum_d D_d^T (G grad u)_d, with B^T applied as the
 *                      transposed table (src/tmm.hpp:65-85, Tr=false).
 *   ORACLE_REFERENCE : what the reference code computes (Q == N only):
 *                      mass reuses Phi (not Phi^T) backward (src/mass.hpp:21);
 *                      stiffness keeps only the last backward chain
 *                      (src/stiffness.hpp:85,91,97), with Wz missing its
 *                      derivative (src/stiffness.hpp:76-77).
 */
#ifndef FEMTC_ORACLE_H
#define FEMTC_ORACLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_EXACT = 0, ORACLE_REFERENCE = 1 };

/* linalg::gemm_blocked restated (src/linalg.hpp:101-182): C = A.B (assign),
 * A column-major (m x k), B row-major (k x n), C column-major (m x n). */
void oracle_gemm_blocked(int k, int m, int n, const double* a, const double* b,
                         double* c);

/* linalg::gemm_micro restated (src/linalg.hpp:45-94): c += a.b with a
 * column-major (m x k, leading dimension lda), b row-major (k x nc, ldb), c
 * row-major (m x nc, ldc); products added in increasing p (kij order). */
void oracle_gemm_micro(int k, int m, int nc, int lda, int ldb, int ldc,
                       const double* a, const double* b, double* c);

/* One cell-batched axis contraction as used by the operators: for each cell
 * c, C_c[i + j*m] = sum_p A[i + p*m] * B_c[p*n + j]. */
void oracle_gemm_blocked_batched(int k, int m, int n, const double* a,
                                 const double* b, double* c, size_t ncells);

/* tmm apply_contractions restated (src/tmm.hpp:91-126) batched over cells:
 * A[a0,a1,a2] = sum I0(a0,b0) I1(a1,b1) I2(a2,b2) B[b0,b1,b2];
 * tr != 0: I(a,b) = I[a*Nb + b]; tr == 0: I(a,b) = I[b*Na + a]. */
void oracle_apply_contractions(int na, int nb, int tr, const double* i0,
                               const double* i1, const double* i2,
                               const double* b, double* a, size_t ncells);

int oracle_mass(int sem, int n, int q, const double* tables, const double* u,
                const double* d, double* y, size_t ncells, int nthreads);
int oracle_stiffness(int sem, int n, int q, const double* tables,
                     const double* u, const double* g, double* y,
                     size_t ncells, int nthreads);

/* y = alpha*M u + beta*K u for the exact operators (the CG system matrix
 * M + sigma K of the solve service; alpha=1, beta=sigma). */
int oracle_helmholtz(int n, int q, const double* tables, const double* u,
                     const double* d, const double* g, double alpha,
                     double beta, double* y, size_t ncells, int nthreads);

/* Diagonal of alpha*M + beta*K per cell (Jacobi preconditioner), exact
 * semantics, computed column by column from the operator definition. */
int oracle_helmholtz_diagonal(int n, int q, const double* tables,
                              const double* d, const double* g, double alpha,
                              double beta, double* diag, size_t ncells);

/* Plain FP64 Jacobi-preconditioned CG on the cell-local (block-diagonal)
 * system (alpha M + beta K) x = b; returns the iteration count, or -1 when
 * maxit is reached first.  Textbook algorithm (Saad, Iterative Methods for
 * Sparse Linear Systems, Alg. 9.1). */
int oracle_cg(int n, int q, const double* tables, const double* d,
              const double* g, double alpha, double beta, const double* b,
              double* x, size_t ncells, double rtol, int maxit,
              double* final_relres);

#ifdef __cplusplus
}
#endif
#endif
