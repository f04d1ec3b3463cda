/* femtc CPU oracle (FP64): test infrastructure only -- the checker for the
 * GPU operator library.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it; nothing in the product calls it.
 *
 * Restates, in plain C, the per-cell algorithm of IgorBaratta/femtc:
 *   linalg::gemm_micro         src/linalg.hpp:45-94
 *   linalg::gemm_blocked       src/linalg.hpp:101-182
 *   operators::mass_operator   src/mass.hpp:10-49
 *   transform                  src/stiffness.hpp:14-29
 *   operators::stiffness_operator src/stiffness.hpp:34-99
 *   apply_contractions         src/tmm.hpp:91-126
 * generalised to Q != N quadrature points per axis (the reference supports
 * Q == N only; tmm.hpp shows the general Q contraction with the exact
 * transpose through its Tr flag).
 *
 * Parity pin: tests compare this file against the reference's own templates
 * compiled from the reference sources (oracle/Makefile -> oracle/_ref) and
 * against the committed golden vectors made from them (tests/golden/).
 */
#include "femtc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FORCE_INLINE static inline __attribute__((always_inline))

/* out = contraction of the 3-tensor `in` (dims d0 x d1 x d2, row-major, axis
 * 0 slowest) along `axis` with the matrix A(m,k) = A[m*sm + k*sk]; the
 * contracted axis gets size M.  Sums run k = 0..K-1 from zero, the order of
 * gemm_micro's kij loop (src/linalg.hpp:73-79). */
FORCE_INLINE void contract_axis(int axis, int d0, int d1, int d2, int M,
                                const double* A, int sm, int sk,
                                const double* in, double* out)
{
  if (axis == 0)
  {
    const int L = d1 * d2;
    for (int m = 0; m < M; ++m)
    {
      double* o = out + m * L;
      for (int j = 0; j < L; ++j)
        o[j] = 0.0;
      for (int k = 0; k < d0; ++k)
      {
        const double a = A[m * sm + k * sk];
        const double* x = in + k * L;
        for (int j = 0; j < L; ++j)
          o[j] += a * x[j];
      }
    }
  }
  else if (axis == 1)
  {
    for (int a0 = 0; a0 < d0; ++a0)
      for (int m = 0; m < M; ++m)
      {
        double* o = out + (a0 * M + m) * d2;
        for (int j = 0; j < d2; ++j)
          o[j] = 0.0;
        for (int k = 0; k < d1; ++k)
        {
          const double a = A[m * sm + k * sk];
          const double* x = in + (a0 * d1 + k) * d2;
          for (int j = 0; j < d2; ++j)
            o[j] += a * x[j];
        }
      }
  }
  else
  {
    for (int r = 0; r < d0 * d1; ++r)
      for (int m = 0; m < M; ++m)
      {
        double s = 0.0;
        for (int k = 0; k < d2; ++k)
          s += A[m * sm + k * sk] * in[r * d2 + k];
        out[r * M + m] = s;
      }
  }
}

/* One axis contraction in the reference's rotating form (src/linalg.hpp:
 * 101-182, as the operators chain it, src/mass.hpp:36-47): `in` is K x L
 * row-major (the contracted axis slowest, L = the other two axes), `out`
 * is L x M row-major, out[j*M + m] = sum_p A(m,p) in[p*L + j] with
 * A(m,p) = A[m*sm + p*sk].  The contracted axis becomes the fastest, so
 * three contractions return a tensor to its axis order.  Products are added
 * from zero in increasing p (gemm_micro's kij order, :73-79), into a row
 * of L values that is then written with stride M (gemm_blocked's copy of
 * its Ctemp block, :128-136). */
FORCE_INLINE void rot_contract(int K, int L, int M, const double* A, int sm,
                               int sk, const double* in, double* out)
{
  double row[4096];
  for (int m = 0; m < M; ++m)
  {
    for (int j = 0; j < L; ++j)
      row[j] = 0.0;
    for (int p = 0; p < K; ++p)
    {
      const double a = A[m * sm + p * sk];
      const double* x = in + p * L;
      for (int j = 0; j < L; ++j)
        row[j] += a * x[j];
    }
    for (int j = 0; j < L; ++j)
      out[j * M + m] = row[j];
  }
}

/* ------------------------------------------------------------------------ */
void oracle_gemm_blocked(int k, int m, int n, const double* a, const double* b,
                         double* c)
{
  /* src/linalg.hpp:101-182: C[i + j*m] = sum_p a[i + p*m] * b[p*n + j];
   * assigns (the reference zeroes its Ctemp block, :123). */
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i)
    {
      double s = 0.0;
      for (int p = 0; p < k; ++p)
        s += a[i + p * m] * b[p * n + j];
      c[i + j * m] = s;
    }
}

void oracle_gemm_micro(int k, int m, int nc, int lda, int ldb, int ldc,
                       const double* a, const double* b, double* c)
{
  /* src/linalg.hpp:45-94: c(i,j) += sum_p a[i + p*lda] * b[p*ldb + j], c
   * row-major with leading dimension ldc; the kij order (:73-79) adds the
   * products into c in increasing p. */
  for (int p = 0; p < k; ++p)
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < nc; ++j)
        c[i * ldc + j] += a[i + p * lda] * b[p * ldb + j];
}

void oracle_gemm_blocked_batched(int k, int m, int n, const double* a,
                                 const double* b, double* c, size_t ncells)
{
  for (size_t cell = 0; cell < ncells; ++cell)
    oracle_gemm_blocked(k, m, n, a, b + cell * (size_t)k * n,
                        c + cell * (size_t)m * n);
}

void oracle_apply_contractions(int na, int nb, int tr, const double* i0,
                               const double* i1, const double* i2,
                               const double* b, double* a, size_t ncells)
{
  /* src/tmm.hpp:65-85: Tr=true reads I[a*Nk + k] (row-major Na x Nb),
   * Tr=false reads I[k*Na + a] (the stored Nb x Na table, transposed). */
  const int sm = tr ? nb : 1, sk = tr ? 1 : na;
  const size_t bsz = (size_t)nb * nb * nb, asz = (size_t)na * na * na;
  int big = na > nb ? na : nb;
  double* w1 = (double*)malloc(sizeof(double) * big * big * big);
  double* w2 = (double*)malloc(sizeof(double) * big * big * big);
  for (size_t cell = 0; cell < ncells; ++cell)
  {
    contract_axis(0, nb, nb, nb, na, i0, sm, sk, b + cell * bsz, w1);
    contract_axis(1, na, nb, nb, na, i1, sm, sk, w1, w2);
    contract_axis(2, na, na, nb, na, i2, sm, sk, w2, a + cell * asz);
  }
  free(w1);
  free(w2);
}

/* ------------------------------------------------------------------------ */
/* Mass, one cell.  Forward: src/mass.hpp:36-38; scaling :40-41; backward
 * :45-47.  Exact semantics applies Phi^T backward (A(i,q) = phi[q + i*Q]);
 * reference semantics reuses Phi (phi[i + q*N], Q == N) as :21 does. */
FORCE_INLINE void mass_cell(int sem, int N, int Q, const double* phi,
                            const double* u, const double* D, double* y,
                            double* w1, double* w2, double* w3)
{
  rot_contract(N, N * N, Q, phi, 1, Q, u, w1);
  rot_contract(N, N * Q, Q, phi, 1, Q, w1, w2);
  rot_contract(N, Q * Q, Q, phi, 1, Q, w2, w3);
  const int nq = Q * Q * Q;
  for (int i = 0; i < nq; ++i)
    w3[i] *= D[i];
  const int bsm = (sem == ORACLE_EXACT) ? Q : 1;
  const int bsk = (sem == ORACLE_EXACT) ? 1 : Q;
  rot_contract(Q, Q * Q, N, phi, bsm, bsk, w3, w1);
  rot_contract(Q, Q * N, N, phi, bsm, bsk, w1, w2);
  rot_contract(Q, N * N, N, phi, bsm, bsk, w2, y);
}

/* src/stiffness.hpp:14-29, G components [zz,yz,xz,yy,xy,xx] per point. */
FORCE_INLINE void transform(int nq, const double* G, double* f0, double* f1,
                            double* f2)
{
  for (int q = 0; q < nq; ++q)
  {
    const double* g = G + 6 * q;
    const double w0 = f0[q], w1 = f1[q], w2 = f2[q];
    f0[q] = g[5] * w0 + g[4] * w1 + g[2] * w2;
    f1[q] = g[4] * w0 + g[3] * w1 + g[1] * w2;
    f2[q] = g[2] * w0 + g[1] * w1 + g[0] * w2;
  }
}

/* Forward 3-contraction chain with per-axis tables (forward tables
 * A(q,i) = t[q + i*Q]), axis 0 first. */
FORCE_INLINE void chain_fwd(int N, int Q, const double* t0, const double* t1,
                            const double* t2, const double* u, double* out,
                            double* w1, double* w2)
{
  rot_contract(N, N * N, Q, t0, 1, Q, u, w1);
  rot_contract(N, N * Q, Q, t1, 1, Q, w1, w2);
  rot_contract(N, Q * Q, Q, t2, 1, Q, w2, out);
}

/* Backward chain: transposed tables (exact) or the forward tables again
 * (reference semantics, Q == N), axis 0 first. */
FORCE_INLINE void chain_bwd(int N, int Q, int sm, int sk, const double* t0,
                            const double* t1, const double* t2,
                            const double* f, double* out, double* w1,
                            double* w2)
{
  rot_contract(Q, Q * Q, N, t0, sm, sk, f, w1);
  rot_contract(Q, Q * N, N, t1, sm, sk, w1, w2);
  rot_contract(Q, N * N, N, t2, sm, sk, w2, out);
}

/* Stiffness, one cell.  Exact: y = sum_d D_d^T (G D u)_d with
 * D_x = Gamma x Phi x Phi (axis 0 = x, slowest), evaluated with shared
 * partial contractions: forward Phi_0 u and Gamma_0 u feed the three
 * gradients (2 + 3 + 3 contractions), backward the x and y chains meet
 * before their common last table (3 + 3 + 2), 16 contractions per cell
 * against the reference's 17
 * (src/stiffness.hpp:68-97).  Reference semantics (src/stiffness.hpp:68-97):
 * Wx = (Gamma,Phi,Phi)u, Wy = (Phi,Gamma,Phi)u, Wz = (Phi,Phi,Phi)u (no
 * derivative, :76-77), transform, and only the last backward chain
 * (Phi,Phi,Gamma) survives because each chain assigns W (:85,91,97). */
FORCE_INLINE void stiffness_cell(int sem, int N, int Q, const double* tab,
                                 const double* u, const double* G, double* y,
                                 double* gx, double* gy, double* gz,
                                 double* w1, double* w2, double* tmp)
{
  const double* P = tab;
  const double* D = tab + Q * N;
  const int nq = Q * Q * Q, nd = N * N * N, nh = Q * N * N;
  if (sem == ORACLE_EXACT)
  {
    /* forward: axis 0, then 1, then 2 (each contraction rotates the axes) */
    rot_contract(N, N * N, Q, P, 1, Q, u, w1);    /* Phi_0 u   */
    rot_contract(N, N * N, Q, D, 1, Q, u, w2);    /* Gamma_0 u */
    rot_contract(N, N * Q, Q, P, 1, Q, w2, tmp);
    rot_contract(N, Q * Q, Q, P, 1, Q, tmp, gx); /* d/dx */
    rot_contract(N, N * Q, Q, D, 1, Q, w1, tmp);
    rot_contract(N, Q * Q, Q, P, 1, Q, tmp, gy); /* d/dy */
    rot_contract(N, N * Q, Q, P, 1, Q, w1, tmp);
    rot_contract(N, Q * Q, Q, D, 1, Q, tmp, gz); /* d/dz */
    transform(nq, G, gx, gy, gz);
    /* backward: axis 0, then 1, then 2; the x and y chains share the last
     * table (Phi_2^T), so they are summed before it */
    rot_contract(Q, Q * Q, N, D, Q, 1, gx, w1);  /* Gamma_0^T fx */
    rot_contract(Q, Q * Q, N, P, Q, 1, gy, w2);  /* Phi_0^T fy   */
    rot_contract(Q, Q * Q, N, P, Q, 1, gz, gx);  /* Phi_0^T fz   */
    rot_contract(Q, Q * N, N, P, Q, 1, w1, tmp); /* x: Phi_1^T   */
    rot_contract(Q, Q * N, N, D, Q, 1, w2, gy);  /* y: Gamma_1^T */
    rot_contract(Q, Q * N, N, P, Q, 1, gx, w1);  /* z: Phi_1^T   */
    for (int i = 0; i < nh; ++i)
      tmp[i] += gy[i];
    rot_contract(Q, N * N, N, P, Q, 1, tmp, y);  /* x + y: Phi_2^T */
    rot_contract(Q, N * N, N, D, Q, 1, w1, w2);  /* z: Gamma_2^T   */
    for (int i = 0; i < nd; ++i)
      y[i] += w2[i];
  }
  else
  {
    chain_fwd(N, Q, D, P, P, u, gx, w1, w2);
    chain_fwd(N, Q, P, D, P, u, gy, w1, w2);
    chain_fwd(N, Q, P, P, P, u, gz, w1, w2);
    transform(nq, G, gx, gy, gz);
    chain_bwd(N, Q, 1, Q, P, P, D, gz, y, w1, w2);
  }
}

typedef struct
{
  double* b[7];
} work_t;

static int work_alloc(work_t* w, int N, int Q)
{
  int big = N > Q ? N : Q;
  size_t sz = (size_t)big * big * big;
  for (int i = 0; i < 7; ++i)
  {
    w->b[i] = (double*)malloc(sizeof(double) * sz);
    if (!w->b[i])
      return -1;
  }
  return 0;
}

static void work_free(work_t* w)
{
  for (int i = 0; i < 7; ++i)
    free(w->b[i]);
}

/* Compile-time (N,Q) specialisations: the same inline bodies with constant
 * sizes, so gcc unrolls them the way the reference's templates are unrolled.
 * Used only to make the CPU baseline a fair one; results are identical. */
#define SPEC(NN, QQ)                                                           \
  static void mass_##NN##_##QQ(int sem, int N, int Q, const double* t,         \
                               const double* u, const double* d, double* y,   \
                               work_t* w)                                     \
  {                                                                            \
    (void)N;                                                                   \
    (void)Q;                                                                   \
    mass_cell(sem, NN, QQ, t, u, d, y, w->b[0], w->b[1], w->b[2]);             \
  }                                                                            \
  static void stiff_##NN##_##QQ(int sem, int N, int Q, const double* t,        \
                                const double* u, const double* g, double* y,  \
                                work_t* w)                                    \
  {                                                                            \
    (void)N;                                                                   \
    (void)Q;                                                                   \
    stiffness_cell(sem, NN, QQ, t, u, g, y, w->b[0], w->b[1], w->b[2],         \
                   w->b[3], w->b[4], w->b[5]);                                 \
  }
SPEC(2, 2) SPEC(2, 3) SPEC(3, 3) SPEC(3, 4) SPEC(4, 4) SPEC(4, 5) SPEC(5, 5)
SPEC(5, 6) SPEC(6, 6) SPEC(6, 7) SPEC(7, 7) SPEC(7, 8) SPEC(8, 8) SPEC(8, 9)
#undef SPEC

typedef void (*cell_fn)(int, int, int, const double*, const double*,
                        const double*, double*, work_t*);

/* Runtime-size path for (N,Q) pairs without a specialisation. */
static void mass_generic(int sem, int N, int Q, const double* t,
                         const double* u, const double* d, double* y,
                         work_t* w)
{
  mass_cell(sem, N, Q, t, u, d, y, w->b[0], w->b[1], w->b[2]);
}

static void stiff_generic(int sem, int N, int Q, const double* t,
                          const double* u, const double* g, double* y,
                          work_t* w)
{
  stiffness_cell(sem, N, Q, t, u, g, y, w->b[0], w->b[1], w->b[2], w->b[3],
                 w->b[4], w->b[5]);
}

static cell_fn pick(int stiff, int N, int Q)
{
#define CASE(NN, QQ)                                                           \
  if (N == NN && Q == QQ)                                                      \
    return stiff ? stiff_##NN##_##QQ : mass_##NN##_##QQ;
  CASE(2, 2) CASE(2, 3) CASE(3, 3) CASE(3, 4) CASE(4, 4) CASE(4, 5) CASE(5, 5)
  CASE(5, 6) CASE(6, 6) CASE(6, 7) CASE(7, 7) CASE(7, 8) CASE(8, 8) CASE(8, 9)
#undef CASE
  return 0;
}

static int run_cells(int stiff, int sem, int N, int Q, const double* tables,
                     const double* u, const double* dg, double* y,
                     size_t ncells, int nthreads)
{
  if (N < 1 || Q < 1 || (sem == ORACLE_REFERENCE && Q != N))
    return -1;
  cell_fn fn = pick(stiff, N, Q);
  if (!fn)
    fn = stiff ? stiff_generic : mass_generic;
  const size_t nd = (size_t)N * N * N;
  const size_t nqd = (size_t)Q * Q * Q * (stiff ? 6 : 1);
  int err = 0;
#ifdef _OPENMP
  if (nthreads < 1)
    nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    work_t w;
    if (work_alloc(&w, N, Q) != 0)
      err |= 1;
    else
    {
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
      for (long long c = 0; c < (long long)ncells; ++c)
        fn(sem, N, Q, tables, u + c * nd, dg + c * nqd, y + c * nd, &w);
    }
    work_free(&w);
  }
  (void)nthreads;
  return err ? -2 : 0;
}

int oracle_mass(int sem, int n, int q, const double* tables, const double* u,
                const double* d, double* y, size_t ncells, int nthreads)
{
  return run_cells(0, sem, n, q, tables, u, d, y, ncells, nthreads);
}

int oracle_stiffness(int sem, int n, int q, const double* tables,
                     const double* u, const double* g, double* y,
                     size_t ncells, int nthreads)
{
  return run_cells(1, sem, n, q, tables, u, g, y, ncells, nthreads);
}

/* ------------------------------------------------------------------------ */
/* Helmholtz-type operator and CG (no reference counterpart: the reference
 * has no solver).  Exact semantics only. */
int oracle_helmholtz(int n, int q, const double* tables, const double* u,
                     const double* d, const double* g, double alpha,
                     double beta, double* y, size_t ncells, int nthreads)
{
  const size_t nd = (size_t)n * n * n * ncells;
  double* tmp = (double*)malloc(sizeof(double) * nd);
  if (!tmp)
    return -2;
  int rc = oracle_mass(ORACLE_EXACT, n, q, tables, u, d, y, ncells, nthreads);
  if (rc == 0)
    rc = oracle_stiffness(ORACLE_EXACT, n, q, tables, u, g, tmp, ncells,
                          nthreads);
  for (size_t i = 0; i < nd && rc == 0; ++i)
    y[i] = alpha * y[i] + beta * tmp[i];
  free(tmp);
  return rc;
}

int oracle_helmholtz_diagonal(int n, int q, const double* tables,
                              const double* d, const double* g, double alpha,
                              double beta, double* diag, size_t ncells)
{
  const double* P = tables;
  const double* D = tables + q * n;
  const int nq = q * q * q, nd = n * n * n;
  for (size_t c = 0; c < ncells; ++c)
  {
    const double* dc = d + c * nq;
    const double* gc = g + c * nq * 6;
    for (int i = 0; i < nd; ++i)
    {
      const int i0 = i / (n * n), i1 = (i / n) % n, i2 = i % n;
      double m = 0.0, k = 0.0;
      for (int p = 0; p < nq; ++p)
      {
        const int p0 = p / (q * q), p1 = (p / q) % q, p2 = p % q;
        const double f0 = P[p0 + i0 * q], f1 = P[p1 + i1 * q],
                     f2 = P[p2 + i2 * q];
        const double g0 = D[p0 + i0 * q], g1 = D[p1 + i1 * q],
                     g2 = D[p2 + i2 * q];
        const double v = f0 * f1 * f2;
        m += dc[p] * v * v;
        const double gx = g0 * f1 * f2, gy = f0 * g1 * f2, gz = f0 * f1 * g2;
        const double* G = gc + 6 * p;
        k += G[5] * gx * gx + G[3] * gy * gy + G[0] * gz * gz +
             2.0 * (G[4] * gx * gy + G[2] * gx * gz + G[1] * gy * gz);
      }
      diag[c * nd + i] = alpha * m + beta * k;
    }
  }
  return 0;
}

static double dot(const double* a, const double* b, size_t n)
{
  double s = 0.0;
  for (size_t i = 0; i < n; ++i)
    s += a[i] * b[i];
  return s;
}

int oracle_cg(int n, int q, const double* tables, const double* d,
              const double* g, double alpha, double beta, const double* b,
              double* x, size_t ncells, double rtol, int maxit,
              double* final_relres)
{
  const size_t nd = (size_t)n * n * n * ncells;
  double* r = (double*)malloc(sizeof(double) * nd);
  double* z = (double*)malloc(sizeof(double) * nd);
  double* p = (double*)malloc(sizeof(double) * nd);
  double* ap = (double*)malloc(sizeof(double) * nd);
  double* dg = (double*)malloc(sizeof(double) * nd);
  int it = -1;
  double rn = 0.0, bnorm = 0.0;
  if (!r || !z || !p || !ap || !dg)
    goto done;
  oracle_helmholtz_diagonal(n, q, tables, d, g, alpha, beta, dg, ncells);
  for (size_t i = 0; i < nd; ++i)
  {
    x[i] = 0.0;
    r[i] = b[i];
    z[i] = r[i] / dg[i];
    p[i] = z[i];
  }
  bnorm = sqrt(dot(b, b, nd));
  double rz = dot(r, z, nd);
  rn = bnorm;
  if (bnorm == 0.0)
  {
    it = 0;
    rn = 0.0;
    goto done;
  }
  for (int k = 0; k < maxit; ++k)
  {
    oracle_helmholtz(n, q, tables, p, d, g, alpha, beta, ap, ncells, 0);
    const double a = rz / dot(p, ap, nd);
    for (size_t i = 0; i < nd; ++i)
    {
      x[i] += a * p[i];
      r[i] -= a * ap[i];
    }
    rn = sqrt(dot(r, r, nd));
    if (rn <= rtol * bnorm)
    {
      it = k + 1;
      break;
    }
    for (size_t i = 0; i < nd; ++i)
      z[i] = r[i] / dg[i];
    const double rz1 = dot(r, z, nd);
    const double be = rz1 / rz;
    rz = rz1;
    for (size_t i = 0; i < nd; ++i)
      p[i] = z[i] + be * p[i];
  }
done:
  if (final_relres)
    *final_relres = rn / (bnorm > 0 ? bnorm : 1.0);
  free(r);
  free(z);
  free(p);
  free(ap);
  free(dg);
  return it;
}
