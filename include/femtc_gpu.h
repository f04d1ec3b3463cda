/* femtc_gpu.h -- C ABI of the GB300 (sm_103a) matrix-free hexahedral
 * operator library.
 *
 * This is the drop-in boundary for the hot path of IgorBaratta/femtc: the
 * per-cell, sum-factorized mass and stiffness action.  Every entry point
 * names the reference interface it replaces.  All functions return
 * FEMTC_OK (0) or a negative status; femtc_last_error() then describes the
 * failure (per calling thread).  No function allocates memory that outlives
 * the call except the library context (a cached stream and grow-only device
 * staging buffers used by the *_host entry points).
 *
 * Layouts (the reference's):
 *   u, y   : [ncells][N][N][N], N = degree+1, axis 0 slowest
 *            (src/mass.hpp:25-29)
 *   dw     : mass quadrature weights detJ*w, [ncells][Q][Q][Q]
 *            (src/mass.hpp:27, where the reference has Q == N)
 *   G      : stiffness geometry, [ncells][Q^3][6], components
 *            [zz, yz, xz, yy, xy, xx] (src/stiffness.hpp:20-27)
 *   tables : Phi(q,i) = tables[q + i*Q] (column-major Q x N,
 *            src/linalg.hpp:49), followed by Gamma(q,i) = tables[Q*N + q + i*Q]
 *            (src/stiffness.hpp:44-48).  Mass reads only Phi.  Tables are
 *            HOST memory: they are copied into the launch's parameter block.
 *
 * Element types: FEMTC_F64 and FEMTC_F64E -> double storage of u, y, dw/G
 * and the tables; FEMTC_F32 and the mixed forms -> float storage.
 */
#ifndef FEMTC_GPU_H
#define FEMTC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FEMTC_OK 0
#define FEMTC_ERR_INVALID (-1)     /* bad argument: size, pointer, alignment */
#define FEMTC_ERR_UNSUPPORTED (-2) /* (degree, Q, dtype, semantics) not built */
#define FEMTC_ERR_CUDA (-3)        /* a CUDA runtime call failed */
#define FEMTC_ERR_NOMEM (-4)       /* device or pinned allocation failed */
#define FEMTC_ERR_DEVICE (-5)      /* a kernel's bounded wait gave up */
#define FEMTC_ERR_NOT_CONVERGED (-6) /* a solve stopped at its iteration cap */
#define FEMTC_ERR_TIMEOUT (-7)     /* a wait ran out of time */

typedef enum
{
  FEMTC_F64 = 0,   /* FP64 storage and arithmetic */
  FEMTC_F32 = 1,   /* FP32 storage and arithmetic (CUDA cores) */
  FEMTC_F16X2 = 2, /* FP32 storage; tensor-core FP16 hi/lo split, FP32 acc. */
  FEMTC_BF16X3 = 3, /* FP32 storage; tensor-core BF16 3-term split, FP32 acc. */
  FEMTC_F64E = 4    /* FP64 storage and tables; double-float (FP32-pair)
                       arithmetic on the FP32 pipes, FP64-accurate */
} femtc_dtype;

typedef enum
{
  FEMTC_EXACT = 0,    /* the true operators, any supported Q */
  FEMTC_REFERENCE = 1 /* the reference's literal arithmetic, Q == N only */
} femtc_semantics;

typedef enum
{
  FEMTC_OP_MASS = 0,
  FEMTC_OP_STIFFNESS = 1,
  FEMTC_OP_HELMHOLTZ = 2, /* alpha M + beta K in one pass (femtc_helmholtz_apply) */
  FEMTC_OP_MASS_AFFINE = 3,     /* mass, one detJ per cell (femtc_affine_apply) */
  FEMTC_OP_STIFFNESS_AFFINE = 4 /* stiffness, one G per cell (femtc_affine_apply) */
} femtc_op;

/* Library version (major*10000 + minor*100 + patch). */
int femtc_version(void);

/* Number of operator kernels (mass / stiffness, every form) this library
 * has launched in this process (a monotonic counter). */
long long femtc_operator_launches(void);

/* Description of the last failure on the calling thread ("" if none). */
const char* femtc_last_error(void);

/* Reads and clears the device fault word of every kernel unit (bits set by
 * bounded waits that gave up: 1 = an mbarrier wait timed out, 2 = a batched
 * work item named an unknown variant).  Synchronises the device.  Returns
 * the OR of the words, 0 when clean, or a negative status. */
int femtc_device_status(void);

/* Diagnostic, no reference counterpart (the reference has no device code):
 * launches one CTA on `stream` whose mbarrier wait cannot complete (armed
 * for transaction bytes that no copy delivers) and that waits through the
 * library's bounded wait with a limit of `polls` polls (1..2^22; the
 * library's kernels use 2^22).  The wait gives up, the kernel sets
 * FAULT bit 1 (mbarrier wait timed out) in its fault word and returns:
 * femtc_device_status() then reports 1.  No copy is issued and no memory is
 * touched, so the GPU stays usable; this shows that a stalled copy in any
 * kernel of the library ends as a status word, not a hang. */
int femtc_bounded_wait_check(int polls, void* stream);

/* Whether (op, dtype, semantics, degree, nquad) has a compiled kernel:
 * 1 yes, 0 no. */
int femtc_supported(int op, int dtype, int semantics, int degree, int nquad);

/* Mass action y = B^T D B u on device-resident buffers, asynchronous on
 * `stream` (a cudaStream_t; NULL = legacy default stream).
 * Replaces operators::mass_operator<T,P,Order,Mb,Nb>(phi, U, W, detJ,
 * num_cells) (src/mass.hpp:10-12) and its runtime dispatcher
 * operators::mass_operator<T>(phi, U, W, detJ, num_cells, degree, order,
 * Mb, Nb) (src/mass.hpp:196-219); the loop order and register blocks of
 * the CPU code have no GPU meaning and are not arguments here.
 * u, y, dw: device pointers, 16-byte aligned.  tables: host pointer. */
int femtc_mass_apply(int dtype, int semantics, int degree, int nquad,
                     const void* tables, const void* u, void* y,
                     const void* dw, size_t ncells, void* stream);

/* Stiffness action y = sum_d D_d^T (G D u)_d, device-resident buffers.
 * Replaces operators::stiffness_operator<T,P,Order,Mb,Nb>(phi, U, W, G,
 * num_cells) (src/stiffness.hpp:34-36) and its dispatcher
 * (src/stiffness.hpp:245-268). */
int femtc_stiffness_apply(int dtype, int semantics, int degree, int nquad,
                          const void* tables, const void* u, void* y,
                          const void* G, size_t ncells, void* stream);

/* Helmholtz action y = alpha M u + beta K u in one pass over the cells,
 * device-resident buffers, exact semantics, FEMTC_F32 only.  No reference
 * counterpart: the reference applies mass and stiffness separately; this
 * is the operator of the matrix-free solver (femtc_solve) exposed as an
 * entry point.  One read of u and one write of y instead of two each; the
 * stiffness passes already hold the values the mass term needs.
 * geo8: [ncells][Q^3][8] per quadrature point: beta*G as
 * [zz,yz,xz,yy,xy,xx], then alpha*detJ*w, then 0 (the caller folds alpha and
 * beta in; femtc_helmholtz_geometry builds it from dw and G).
 * tables: Phi then Gamma, as for femtc_stiffness_apply. */
int femtc_helmholtz_apply(int dtype, int degree, int nquad, const void* tables,
                          const void* u, void* y, const void* geo8,
                          size_t ncells, void* stream);

/* geo8 = [beta*G, alpha*dw, 0] per quadrature point from dw [ncells][Q^3]
 * and G [ncells][Q^3][6], all FP32 device buffers (16-byte aligned geo8),
 * asynchronous on `stream`. */
int femtc_helmholtz_geometry(int nquad, double alpha, const void* dw,
                             double beta, const void* G, void* geo8,
                             size_t ncells, void* stream);

/* Affine cells (parallelepipeds): J is constant over a cell, so the
 * geometry is one set of factors per cell instead of Q^3 per point.
 * op FEMTC_OP_MASS_AFFINE: cgeo [ncells] = detJ; FEMTC_OP_STIFFNESS_AFFINE:
 * cgeo [ncells][6] = detJ J^-1 J^-T as [zz,yz,xz,yy,xy,xx].  tables (host):
 * Phi (Q x N), Gamma (Q x N), then the Q 1D quadrature weights w, in the
 * dtype's table type (FP64 or FP32).  The result equals femtc_mass_apply /
 * femtc_stiffness_apply (exact semantics) with the per-point factors
 * dw[c][q0][q1][q2] = w(q0) w(q1) w(q2) detJ[c] and
 * G[c][q0][q1][q2][k] = w(q0) w(q1) w(q2) cgeo[c][k], up to rounding: the
 * weights are folded into the backward contractions' tables.  The geometry
 * stream shrinks from 8*6Q^3 to 48 bytes per cell (stiffness, FP64).
 * femtc_geometry(dtype, 1, &one, J, 0, detJ, G, ncells, stream) with
 * one = 1.0 computes cgeo from per-cell Jacobians.  FEMTC_F64 and
 * FEMTC_F32, degree 1..7, and FEMTC_F64E (FP64-accurate double-float),
 * degree 1..4; nquad in degree+1..degree+3.  No reference
 * counterpart: the reference takes per-point factors (src/mass.hpp:10-12,
 * src/stiffness.hpp:34-36).  u, y, cgeo: device pointers, 16-byte aligned. */
int femtc_affine_apply(int op, int dtype, int degree, int nquad, const void* tables,
                       const void* u, void* y, const void* cgeo, size_t ncells,
                       void* stream);
/* The same with host buffers (as femtc_mass_apply_host). */
int femtc_affine_apply_host(int op, int dtype, int degree, int nquad, const void* tables,
                            const void* u, void* y, const void* cgeo, size_t ncells);

/* Assembled (global-DOF) action y = sum_c P_c^T A_c P_c x for mass or
 * stiffness (op FEMTC_OP_MASS / FEMTC_OP_STIFFNESS), any dtype and
 * semantics of the cell operators.  dofmap: device [ncells][N^3] int32,
 * the global index of each local DOF (the cell-local order of u, y);
 * offsets [ndofs+1], entries [ncells*N^3]: its transpose in CSR form
 * (device copies of femtc_dofmap_transpose's output).  x, y: device
 * [ndofs] in the dtype's storage type (FP64 for F64/F64E, else FP32);
 * geo as for the cell operators; work: device scratch of
 * femtc_assembled_work_bytes() bytes, 256-byte aligned.  y is written in a
 * fixed summation order (no atomics).  Map entries outside [0, ndofs) (or a
 * transpose that does not match) are not dereferenced: they give NaN.  No reference counterpart: the
 * reference is cell-local only (src/mass.hpp:10-49). */
int femtc_assembled_apply(int op, int dtype, int semantics, int degree, int nquad,
                          const void* tables, const int32_t* dofmap, const int32_t* offsets,
                          const int32_t* entries, size_t ndofs, const void* x, void* y,
                          const void* geo, size_t ncells, void* work, void* stream);
size_t femtc_assembled_work_bytes(int dtype, int degree, size_t ncells);
/* Host: transpose a DOF map (ncells x n3 int32, values in [0, ndofs)) into
 * CSR form: offsets[ndofs+1], entries[ncells*n3] = local positions c*n3+i
 * in increasing order per global DOF. */
int femtc_dofmap_transpose(const int32_t* dofmap, size_t ncells, int n3, size_t ndofs,
                           int32_t* offsets, int32_t* entries);

/* Host-buffer forms of mass and stiffness: every pointer is host memory
 * (pinned memory copies fastest).  Copies u and dw/G to the device, applies
 * the operator, copies y back and returns when y is written -- the drop-in
 * path behind the templated C++ header femtc_gpu/operators.hpp. */
int femtc_mass_apply_host(int dtype, int semantics, int degree, int nquad,
                          const void* tables, const void* u, void* y,
                          const void* dw, size_t ncells);
int femtc_stiffness_apply_host(int dtype, int semantics, int degree,
                               int nquad, const void* tables, const void* u,
                               void* y, const void* G, size_t ncells);

/* Even-odd contractions (default on).  FP64, FP32 and double-float (F64E)
 * launches with exact semantics and one lane per slab
 * whose tables have the symmetry of Lagrange bases on symmetric nodes at
 * symmetric points -- Phi(Q-1-q, N-1-i) = Phi(q,i) and
 * Gamma(Q-1-q, N-1-i) = -Gamma(q,i) to 1e-12 of the largest entry, as
 * femtc_tabulate's tables have -- run kernels that split every 1D
 * contraction into even and odd halves (about 30-45% fewer arithmetic
 * operations).  Other tables run the plain kernels.  0 forces the plain
 * kernels.  No reference counterpart. */
int femtc_set_even_odd(int enable);
/* 1 when a launch of (op, dtype, semantics, degree, nquad) with these host
 * tables would run the even-odd kernels, 0 the plain ones; negative status
 * on bad arguments. */
int femtc_even_odd_used(int op, int dtype, int semantics, int degree, int nquad,
                        const void* tables);

/* How the host-buffer entry points move data.  0 (default): when u, y and
 * the geometry are all pinned host memory (cudaHostAlloc /
 * cudaHostRegister), the kernel reads u and the geometry and writes y
 * directly over the coherent Grace-Blackwell host link, with no staging
 * copies -- unless femtc_autotune_host found the staging pipeline faster
 * for this variant; other buffers are copied through device staging
 * buffers in a pipeline of whole-wave chunks (host-to-device copy, kernel
 * and device-to-host copy of neighbouring chunks overlap).
 * 1: always the staging pipeline.  2: zero-copy only (pageable buffers are
 * an error). */
int femtc_set_host_path(int mode);

/* Tile shape of a variant: cells per tile cb (multiple of 4), how the
 * per-point geometry is read (geo_staged: 0 in the quadrature-point pass,
 * each thread asking L2 for its next pencil's geometry; 1 staged through
 * shared memory by TMA with the DOF slab; 2 in the quadrature-point pass,
 * the tile's geometry asked of L2 when the tile starts), threads per CTA
 * (multiple of 32, at most 256; <= 0 means 256) and, for the FP32 CUDA-core
 * kernels, lanes per slab (1 or 2; <= 0 means the built-in choice).
 * cb <= 0 restores the built-in heuristic.  The autotuner writes these. */
int femtc_set_tile_config(int op, int dtype, int semantics, int degree,
                          int nquad, int cb, int geo_staged, int threads,
                          int lanes);
int femtc_get_tile_config(int op, int dtype, int semantics, int degree,
                          int nquad, int* cb, int* geo_staged, int* threads,
                          int* lanes);

/* Autotuner: times candidate tile shapes of one variant on the caller's
 * device buffers (as for femtc_*_apply; y is overwritten), keeps the fastest
 * as the variant's tile configuration and returns it (any output pointer may
 * be NULL).  Synchronises `stream`.  No reference counterpart (the reference
 * picks CPU register blocks Mb/Nb by hand, src/mass.hpp:176-218). */
int femtc_autotune(int op, int dtype, int semantics, int degree, int nquad,
                   const void* tables, const void* u, void* y,
                   const void* geo, size_t ncells, void* stream, int* cb,
                   int* geo_staged, int* threads, float* best_ms);

/* The same for the host-buffer path: u, y and geo are pinned host buffers.
 * Tile shapes are timed with the kernels reading and writing them over the
 * host link (zero-copy); then whole calls of the zero-copy path and of the
 * staging-copy pipeline are timed (alternating, best call of each), and
 * host-path mode 0 (auto) uses the faster of the two from then on for this
 * variant and calls of a similar size (cell counts within the same power
 * of four). */
int femtc_autotune_host(int op, int dtype, int semantics, int degree,
                        int nquad, const void* tables, const void* u, void* y,
                        const void* geo, size_t ncells, int* cb,
                        int* geo_staged, int* threads, float* best_ms);

/* Save / load every explicitly set or tuned tile configuration as text
 * ("op dtype semantics n q cb geo_staged threads" per line).  Load returns
 * the number of entries applied, or a negative status. */
int femtc_tile_db_save(const char* path);
int femtc_tile_db_load(const char* path);

/* linalg::gemm_micro (src/linalg.hpp:45-94), batched over `batch` items:
 * C_b += A_b B_b with A column-major m x k (element (i,p) at a[i + p*lda]),
 * B row-major k x nc (b[p*ldb + j]) and C row-major m x nc (c[i*ldc + j]);
 * C is accumulated into, as the reference's micro-kernel does, with the
 * products added in increasing p (one FMA each).  Item b's matrices start
 * stride_a, stride_b, stride_c elements after item b-1's (0 shares A or B
 * between items; C blocks must not overlap).  dtype FEMTC_F64 or
 * FEMTC_F32; a, b, c are device pointers.  The reference's test of it is
 * tests/test_micro.cpp:12-53 (k = 26, m = 4, nc = 16, lda = 4,
 * ldb = ldc = 16). */
int femtc_gemm_micro(int dtype, int k, int m, int nc, int lda, int ldb, int ldc,
                     const void* a, const void* b, void* c, size_t batch,
                     size_t stride_a, size_t stride_b, size_t stride_c,
                     void* stream);

/* One batched axis contraction, as linalg::gemm_blocked
 * (src/linalg.hpp:101-182) for every cell c: C_c = A B_c with A column-major
 * m x k (HOST memory, k, m <= 32), B_c row-major k x n and C_c column-major
 * m x n (device, cell-contiguous; C is assigned, not accumulated).
 * dtype FEMTC_F64 or FEMTC_F32.  The reference's own unit test exercises
 * this at k = m = P+1, n = (P+1)^2 (tests/test_gemm.cpp:10-60). */
int femtc_gemm_blocked(int dtype, int k, int m, int n, const void* a,
                       const void* b, void* c, size_t batch, void* stream);

/* apply_contractions (src/tmm.hpp:91-126) for every cell:
 * A[a0,a1,a2] = sum I0(a0,b0) I1(a1,b1) I2(a2,b2) B[b0,b1,b2], with
 * I(a,b) = I[a*Nb + b] when tr != 0 and I[b*Na + a] otherwise (the
 * transpose the reference's Tr flag selects).  Tables are HOST memory,
 * Na, Nb <= 16; B (Nb^3 per cell) and A (Na^3 per cell) on the device. */
int femtc_apply_contractions(int dtype, int na, int nb, int tr,
                             const void* i0, const void* i1, const void* i2,
                             const void* b, void* a, size_t ncells,
                             void* stream);

/* Quadrature factors from Jacobians, computed in FP64 on the device:
 * J row-major 3x3 per cell (per_point = 0, affine cells) or per point
 * (per_point = 1, [ncells][Q^3][9]); weights: the Q 1D Gauss weights (host).
 * Writes dw = detJ*w (mass, [ncells][Q^3]) and/or G = detJ w J^-1 J^-T
 * ([ncells][Q^3][6], [zz,yz,xz,yy,xy,xx]) as FP64 or cast to FP32
 * (out_dtype); either output may be NULL.  The reference has no geometry
 * (bench_mass.cpp:86-88 draws detJ and G at random). */
int femtc_geometry(int out_dtype, int nquad, const double* weights,
                   const double* J, int per_point, void* dw, void* G,
                   size_t ncells, void* stream);

/* ----------------------------------------------------------------------
 * Batched persistent launch: many meshes of mixed degree (1..7, Q = P+2)
 * and operator in one kernel, captured once in a CUDA graph and replayed.
 * No reference counterpart: the reference applies one operator of one
 * degree per call (src/mass.hpp:196-219).
 * Items with the same degree must share their tables.  Device pointers
 * must stay valid, with unchanged contents' shapes, for the batch's life;
 * their contents may change between launches.
 * dtype: FEMTC_F32 (CUDA cores), FEMTC_F16X2 or FEMTC_BF16X3 (tensor
 * cores); FP32 storage and tables.
 * flags: FEMTC_BATCH_TUNE measures tile shapes per (degree, op) on the
 * batch's own buffers at creation (the y buffers are overwritten), and
 * the split plan (femtc_batch_plan); the single-mesh tile shapes it tunes
 * stay in the process's tile table, as femtc_autotune's do.
 * ---------------------------------------------------------------------- */
#define FEMTC_BATCH_TUNE 1
/* Take the tuner's split plan (see femtc_batch_plan) even when the one-kernel
 * plan measured faster. */
#define FEMTC_BATCH_SPLIT 2

typedef struct
{
  int op;             /* femtc_op */
  int degree;         /* 1..7 */
  int nquad;          /* degree + 2 */
  const void* tables; /* host, 2*Q*(degree+1) floats (Phi then Gamma) */
  const void* u;      /* device, [ncells][N^3] */
  void* y;            /* device, [ncells][N^3] */
  const void* geo;    /* device, detJ*w or G as for the single-mesh calls */
  size_t ncells;
} femtc_batch_item;

typedef struct femtc_batch femtc_batch;

int femtc_batch_create(int dtype, const femtc_batch_item* items, int nitems,
                       int flags, femtc_batch** out);
/* Replays the captured graph on `stream` (asynchronous). */
int femtc_batch_launch(femtc_batch* b, void* stream);
/* The same kernel launched without the graph (for comparison). */
int femtc_batch_launch_eager(femtc_batch* b, void* stream);
int femtc_batch_info(const femtc_batch* b, long long* ntiles, int* ctas,
                     int* smem_bytes, long long* ndofs);
int femtc_batch_layout(const femtc_batch* b, int op, int degree, int* cb,
                       int* geo_staged);
/* Threads per CTA of the batch's launch (built-in or chosen by the tuner;
 * split plan: of its batch kernel with the most tiles, 0 when it has none). */
int femtc_batch_threads(const femtc_batch* b);
/* The batch's plan.  Without FEMTC_BATCH_TUNE: one persistent kernel over
 * every mesh (kernels = 1, single_launches = 0).  With it the tuner may
 * split the graph: one persistent kernel per (degree, operator) whose
 * meshes run faster batched, and single-mesh operator launches for the
 * variants whose meshes run faster alone (large meshes, where a launch's
 * overhead is negligible) -- whichever whole plan measured faster.  The
 * graph is still one femtc_batch_launch.  femtc_batch_layout reports 0
 * cells for variants run by single-mesh launches. */
int femtc_batch_plan(const femtc_batch* b, int* kernels, int* single_launches);
void femtc_batch_destroy(femtc_batch* b);

/* The batched launch for callers that cannot allocate device memory (code
 * running while another thread captures a CUDA graph in global mode, apps
 * whose memory manager owns the device memory, loops that must not take
 * cudaMalloc's device synchronisation).  No counterpart in the reference.
 * Same items and kernel as femtc_batch_create + femtc_batch_launch, launched
 * directly on `stream`; the tile schedule and mesh table go to a fixed 8 MiB
 * device array of the library (held on every GPU that loads it), so the
 * call allocates nothing.  Limits: at most 4096 meshes and as many tiles as
 * fit in 8 MiB (about 349,000); larger batches are rejected with
 * FEMTC_ERR_INVALID.  The first call on a device sets up the array's address
 * (cudaGetSymbolAddress): make it before any stream capture.  The schedule
 * is copied from host memory that the call frees on return, so a call on a
 * stream that is capturing is rejected with FEMTC_ERR_UNSUPPORTED before it
 * does any work.  Every call reuses the array, so calls whose work overlaps
 * on the GPU (different streams or threads) race; calls on one stream are
 * ordered. */
int femtc_batch_apply_static(int dtype, const femtc_batch_item* items,
                             int nitems, void* stream);

/* ----------------------------------------------------------------------
 * Matrix-free solve of (alpha M + beta K) x = b on a cell-local hexahedral
 * mesh (affine cells): Jacobi-preconditioned CG with a mixed-precision
 * operator (inner_dtype) inside FP64 iterative refinement; the residual,
 * the dot products and x are FP64.  No reference counterpart (the
 * reference has no solver): this is the caller the serving workload needs.
 * ---------------------------------------------------------------------- */
typedef struct
{
  int degree, nquad;   /* degree 1..7, nquad in degree+1..degree+3 */
  size_t ncells;
  double alpha, beta;  /* A = alpha M + beta K; alpha > 0, beta >= 0 */
  const double* J;     /* host [ncells][9] row-major affine Jacobians */
  const double* b;     /* host [ncells][N^3] */
  double* x;           /* host [ncells][N^3], written on completion */
  double rtol;         /* ||b - A x|| <= rtol ||b|| (FP64 residual) */
  double inner_rtol;   /* inner CG tolerance (<= 0: 1e-4) */
  int max_outer;       /* <= 0: 20 */
  int max_inner;       /* per outer iteration, <= 0: 2000 */
  int inner_dtype;     /* FEMTC_F32, FEMTC_F16X2 or FEMTC_BF16X3 */
} femtc_solve_request;

typedef struct
{
  int status;          /* FEMTC_OK, FEMTC_ERR_NOT_CONVERGED, ... */
  int outer_iters, inner_iters;
  double relres;       /* final ||b - A x|| / ||b|| in FP64 */
  double bnorm;
  double ms_total;     /* wall time of the solve itself */
  double t_submit_ms, t_admit_ms, t_done_ms; /* server clock (server only) */
} femtc_solve_result;

/* Device bytes one solve allocates (one stream-ordered allocation). */
size_t femtc_solve_bytes(int degree, int nquad, size_t ncells);

/* Synchronous solve on `stream` (NULL: a private stream). */
int femtc_solve(const femtc_solve_request* rq, femtc_solve_result* res,
                void* stream);

/* Serving loop with continuous batching: up to max_active requests (solves
 * and operator applications) run at once, each on its own stream and host
 * worker, so their kernels overlap on the device; queued requests are
 * admitted as slots and HBM budget free up
 * (a request larger than the whole budget is rejected at submit with
 * FEMTC_ERR_NOMEM).  Request memory (J, b, x) must stay valid until the
 * request's result has been collected. */
typedef struct femtc_server femtc_server;

/* Admission order (femtc_server_set_policy).  SHORTEST_FIRST (default): the
 * queued request with the least estimated work (cells x N^4) less the time
 * it has waited, so small requests pass large ones but a request's wait is
 * bounded by the work admitted ahead of it; the chosen request waits for
 * HBM rather than being passed.  FIFO: arrival order. */
#define FEMTC_SERVE_FIFO 0
#define FEMTC_SERVE_SHORTEST_FIRST 1

typedef struct
{
  long long submitted, completed, rejected, queued, active;
  size_t in_use_bytes, peak_in_use_bytes;
  int max_concurrent;  /* most solves seen running at once */
} femtc_server_stats;

/* An operator application served beside the solves: y = A u on host
 * buffers, as femtc_mass_apply_host / femtc_stiffness_apply_host with the
 * same arguments.  The worker that admits it allocates device copies of u,
 * the geometry and y on its stream, copies in, applies the operator and
 * copies y back; those device bytes count against the HBM budget.  The
 * tables are copied at submit; u, geo and y must stay valid until the
 * result has been collected. */
typedef struct
{
  int op;              /* FEMTC_OP_MASS or FEMTC_OP_STIFFNESS */
  int dtype;           /* any dtype of femtc_*_apply */
  int semantics;       /* FEMTC_EXACT or FEMTC_REFERENCE */
  int degree, nquad;
  size_t ncells;
  const void* tables;  /* host, as femtc_*_apply */
  const void* u;       /* host [ncells][N^3] (FP64 for F64/F64E, else FP32) */
  const void* geo;     /* host geometry, as femtc_*_apply */
  void* y;             /* host [ncells][N^3], written on completion */
} femtc_apply_request;

int femtc_server_create(size_t hbm_budget_bytes, int max_active,
                        femtc_server** out);
int femtc_server_submit(femtc_server* s, const femtc_solve_request* rq,
                        long long* ticket);
/* Queues an operator application (result through femtc_server_wait: status,
 * ms_total and the timestamps; the iteration counts are 0).  No reference
 * counterpart: the reference applies operators in its own benchmark loop. */
int femtc_server_submit_apply(femtc_server* s, const femtc_apply_request* rq,
                              long long* ticket);
/* Waits up to timeout_s seconds for the ticket's result (FEMTC_ERR_TIMEOUT
 * otherwise); returns the solve's status and fills *res. */
int femtc_server_wait(femtc_server* s, long long ticket, double timeout_s,
                      femtc_solve_result* res);
int femtc_server_get_stats(femtc_server* s, femtc_server_stats* st);
int femtc_server_set_policy(femtc_server* s, int policy);
/* Stops admitting, lets running solves finish, drops queued ones. */
void femtc_server_destroy(femtc_server* s);

/* 1D basis tables for degree P with Q Gauss-Legendre points on [0,1]:
 * Lagrange basis on the P+1 Gauss-Lobatto-Legendre nodes (tabulated in
 * FP64 on the host).  tables: 2*Q*(P+1) doubles in the layout above;
 * any of points (Q), weights (Q), nodes (P+1) may be NULL.
 * The reference has no tabulation (bench_mass.cpp:72-76 fills phi with
 * random numbers). */
int femtc_tabulate(int degree, int nquad, double* tables, double* points,
                   double* weights, double* nodes);

#ifdef __cplusplus
}
#endif

#endif /* FEMTC_GPU_H */
