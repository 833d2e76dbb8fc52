/*
 * magreete_gb300 -- C ABI of the GB300 coupled-dipole engine.
 *
 * Every entry point takes DEVICE pointers owned by the caller (torch tensors
 * in the Python host layer), plain sizes and leading dimensions in elements,
 * and a cudaStream_t (passed as void*) on which all work is enqueued.  No
 * entry point allocates device memory: scratch space is a caller-provided
 * workspace whose size the matching *_workspace_bytes function reports.
 * Return value: MGT_OK (0) or a negative MGT_ERR_* code for errors found on
 * the host (bad arguments, CUDA launch errors).  Errors found on the device
 * (zero pivot, a bounded wait that ran out) are written into the workspace's
 * status words and read back with mgt_workspace_status().
 *
 * Complex data is interleaved (re, im): complex128 = two doubles, complex64 =
 * two floats, exactly torch's layout.  Matrices are row-major.  The system
 * index of component a of scatterer i is d*i + a (d = 1, 2 or 3), as in the
 * reference's G0 reshape (Transmission2D.py:279, Transmission3D.py:267).
 */
#ifndef MAGREETE_GB300_H
#define MAGREETE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MGT_OK 0
#define MGT_ERR_ARG (-1)          /* invalid argument (shape, pointer, kind) */
#define MGT_ERR_CUDA (-2)         /* a CUDA runtime call failed */
#define MGT_ERR_SINGULAR (-3)     /* exact zero pivot (torch.linalg.solve raises) */
#define MGT_ERR_TIMEOUT (-4)      /* a bounded device-side wait ran out */
#define MGT_ERR_WORKSPACE (-5)    /* workspace smaller than required */
#define MGT_ERR_UNSUPPORTED (-6)  /* size or mode not supported by this build */
#define MGT_ERR_NOT_CONVERGED (-7)/* iterative refinement missed its tolerance */

/* Green's-function kinds, one per reference solver class */
#define MGT_2D_VECTOR 0   /* Transmission2D_vector (TE, 2x2 dyadic) */
#define MGT_2D_SCALAR 1   /* Transmission2D_scalar (TM) */
#define MGT_3D_VECTOR 2   /* Transmission3D_vector (3x3 dyadic) */
#define MGT_3D_SCALAR 3   /* Transmission3D_scalar */

/* element types */
#define MGT_C128 0   /* complex128: 2 x double */
#define MGT_C64 1    /* complex64: 2 x float */
#define MGT_CDF 2    /* double-float complex: 4 x float (re_hi, re_lo, im_hi,
                        im_lo), re = re_hi + re_lo exactly; ~2^-48 relative */

/* what the propagator kernel writes where the reference's G is NaN */
#define MGT_NAN_KEEP 0    /* NaN (propagate(): rows fixed up by the host) */
#define MGT_NAN_FILL 1    /* every entry of the block = fill value
                             (mean_DOS_measurements: S/V or 0) */

int mgt_abi_version(void);
const char* mgt_status_string(int status);

/*
 * System matrix M = I - coef * G(r_i - r_j) with diagonal 1 - shift.
 * Replaces G0_vector(None) / G0(None) + `-alpha*k0*k0*G` + fill_diagonal_(1)
 * + the self-term eye subtraction inside solve():
 *   Transmission2D.py:222-228 (TE), :733-739 (TM),
 *   Transmission3D.py:197-203 (vector), :709-715 (scalar).
 * points: (N, dim) float64 device array.  coef = k0^2 * alpha.  shift is
 * k0^2 alpha S/V (0 without self-interaction), already rounded as the
 * reference rounds it.  Entries are evaluated in FP64 and written, in one
 * pass, to up to two (dN x dN) outputs of element types dtype1 / dtype2
 * (MGT_C128, MGT_C64 or MGT_CDF); out2 may be NULL.
 */
int mgt_assemble_system(int kind, const double* points, int64_t n_points, double k0,
                        double coef_re, double coef_im, double shift_re, double shift_im,
                        void* out1, int64_t ld1, int dtype1, void* out2, int64_t ld2, int dtype2,
                        void* stream);

/*
 * Propagator block matrix coef * G(t_m - s_j) between n_targets targets and
 * n_sources scatterers: the dense G0(points) of G0_vector / G0
 * (Transmission2D.py:263-280, :777-785; Transmission3D.py:240-268, :751-777)
 * with `regularize` / `radius` semantics per kind (the 2D TE class compares
 * k*R with radius, Transmission2D.py:86-89; the others compare R).
 * nan_policy: MGT_NAN_KEEP or MGT_NAN_FILL (fill = fill_re + i fill_im, not
 * multiplied by coef).  transpose = 0 writes (d*n_targets x d*n_sources),
 * transpose = 1 writes its transpose (used as right-hand sides).
 */
int mgt_assemble_propagator(int kind, const double* targets, int64_t n_targets,
                            const double* sources, int64_t n_sources, double k0,
                            double coef_re, double coef_im, int regularize, double radius,
                            int nan_policy, double fill_re, double fill_im, int transpose,
                            void* out_c128, int64_t ld, void* stream);

/*
 * Blocked right-looking LU with partial pivoting (row interchanges), in
 * place: the `torch.linalg.solve` -> LAPACK ?gesv factorisation step of
 * solve() (Transmission2D.py:230, :742; Transmission3D.py:205, :717).
 * dtype MGT_C128 (the plain FP64 method) or MGT_C64 (the mixed-precision
 * method, refined afterwards).  perm (n int32, device) receives the row
 * permutation: row i of P*A is row perm[i] of A.  Pivots are chosen by
 * |re|+|im| like LAPACK.  A zero pivot is recorded in the workspace status
 * (info, 1-based column like LAPACK) and the factorisation continues.
 */
int mgt_lu_workspace_bytes(int dtype, int64_t n, size_t* bytes);
int mgt_lu_factor(int dtype, void* A, int64_t n, int64_t lda, int32_t* perm,
                  void* work, size_t work_bytes, void* stream);

/*
 * Options of one factorisation (no counterpart in the reference, whose LU is
 * LAPACK's): the choices the process-wide MGT_TUNE_* keys set, per call, so
 * that concurrent callers (a server and a batched sweep in one process) do
 * not change each other's factorisations.  Zero / negative fields take the
 * process-wide value (mgt_set_tuning).
 *   pivoting  MGT_PIVOT_PARTIAL: LAPACK's partial pivoting (largest |re|+|im|
 *             of the column, lowest row on ties; the reference's pivot
 *             sequence).  MGT_PIVOT_TILE (complex64 only): each 64-column
 *             panel chooses its pivots among the 64 rows of its diagonal
 *             tile; the rows below are solved against the tile's U
 *             (L21 = A21 U11^-1), so no panel needs any exchange between
 *             CTAs.  P A = L U still holds; the growth of the factors is not
 *             bounded like partial pivoting's, so it is meant for the mixed
 *             method, whose refinement certifies the solution (callers fall
 *             back to partial pivoting when it does not converge).  An exact
 *             zero tile pivot sets info as a zero pivot does.
 *   panel_rows, panel_max_ctas, cooperative, lookahead, outer_block: as the
 *             MGT_TUNE_* keys of the same names (cooperative / lookahead: -1 =
 *             process value; outer_block 64 or 128)
 */
#define MGT_PIVOT_PARTIAL 0
#define MGT_PIVOT_TILE 1
typedef struct mgt_lu_options {
  int32_t size;            /* sizeof(mgt_lu_options) */
  int32_t pivoting;
  int32_t panel_rows;
  int32_t panel_max_ctas;
  int32_t cooperative;
  int32_t lookahead;
  int32_t outer_block;
} mgt_lu_options;
int mgt_lu_factor_ex(int dtype, void* A, int64_t n, int64_t lda, int32_t* perm, void* work, size_t work_bytes,
                     const mgt_lu_options* options, void* stream);

/*
 * mgt_lu_factor without a workspace argument; no counterpart in the
 * reference (whose solve is a single torch.linalg.solve call on the CPU).
 * For callers that cannot obtain device memory at call time -- a C or
 * Fortran host binding only this library, with no allocator to ask for the
 * LU workspace and a policy against cudaMalloc after start-up, or a process
 * whose device memory is already reserved by its own pool.  The scratch is a
 * 1 MiB device array inside the library, held on every GPU that loads it
 * until the process exits; n is limited to 65536 (larger: MGT_ERR_UNSUPPORTED).
 * All calls share that array: calls whose GPU work overlaps race on it, so
 * serialise them.  The first call on a device looks up the array's device
 * address (and sets the kernels' shared-memory limits on that device); make
 * it before any stream capture.  The address is kept for the life of the
 * process, so the library does not survive a cudaDeviceReset.  info (device,
 * 2 x int32, may be NULL) receives the status words: [0] device error, [1]
 * first zero pivot (1-based, 0 if none).  They are copied into info on
 * `stream`, in stream order, from the shared array: read them only after
 * synchronising the stream, and only under the same rule as the scratch (a
 * later call whose work overlaps can overwrite the words before the copy).
 * Allocates no device memory.
 */
int mgt_lu_factor_static(int dtype, void* A, int64_t n, int64_t lda, int32_t* perm, int32_t* info,
                         void* stream);

/*
 * Solve A X = B with the factors of mgt_lu_factor (the ?getrs half of
 * ?gesv): X = U^-1 L^-1 P B for nrhs columns.  B is not modified.  With a
 * workspace of mgt_lu_solve_workspace_bytes(dtype, n, nrhs) bytes each
 * triangle is two launches (inverse of the 64 x 64 diagonal blocks, then one
 * persistent flag-ordered solve over block rows and 16-column groups); with
 * work == NULL the solve launches two kernels per 64-row block instead.
 */
int mgt_lu_solve_workspace_bytes(int dtype, int64_t n, int64_t nrhs, size_t* bytes);
int mgt_lu_solve(int dtype, const void* LU, int64_t n, int64_t lda, const int32_t* perm,
                 const void* B, int64_t ldb, void* X, int64_t ldx, int64_t nrhs,
                 void* work, size_t work_bytes, void* stream);

/*
 * Complex GEMM update C (M x N) -= A (M x K) * B (K x N), row-major: the LU
 * trailing update A22 -= L21 U12 (inside ?getrf of torch.linalg.solve,
 * Transmission2D.py:230 / Transmission3D.py:205), exposed on its own.
 * MGT_C128: FP64 SIMT.  MGT_C64 with use_tensor_cores = 0: FP32 SIMT;
 * use_tensor_cores = 1: tcgen05 tensor cores with hi/lo split operands
 * (FP32-level accuracy; the scheme is MGT_TUNE_TC_PRECISION: F16x2 with
 * kind::f16 by default, or TF32x3 with kind::tf32), K <= 256, ldc even;
 * needs mgt_cgemm_workspace_bytes(max(M, N)) bytes of workspace.
 */
int mgt_cgemm_workspace_bytes(int64_t nmax, size_t* bytes);
int mgt_cgemm_sub(int dtype, int use_tensor_cores, int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                  const void* B, int64_t ldb, void* C, int64_t ldc, void* work, size_t work_bytes, void* stream);

/*
 * Read back the device status words of a workspace (synchronises `stream`):
 * out[0] = MGT_OK or a device error (MGT_ERR_TIMEOUT), out[1] = info (first
 * zero pivot, 1-based; 0 if none).  Also clears them.
 */
int mgt_workspace_status(void* work, int32_t out[2], void* stream);

/*
 * Residual R = B - M X with M (n x n) in MGT_CDF form, X, B, R complex128
 * (n x nrhs).  With a workspace of mgt_residual_workspace_bytes(n, nrhs)
 * bytes it runs on the tensor cores: M and X are split into seven 8-bit
 * digits per entry (row / column power-of-two scales), digit pairs of equal
 * weight accumulate exactly in FP32 on tcgen05 and exactly in 64-bit
 * integers across K (error ~1e-14 of ||B|| on system matrices; within
 * n 2^-48 of |M||X| entry-wise).  The workspace holds M's digits (14 bytes
 * per entry, rows padded to 128, columns to 32), made by a pass over M in
 * each call; mgt_solve_refined makes them once per solve and reuses them in
 * every correction.  A workspace of exactly n * nrhs * 16
 * bytes (the double-float copy of X) selects double-float arithmetic on the
 * FP32 pipes (products exact via fma, sums compensated), unsplit.  Used by
 * iterative refinement.
 */
int mgt_residual_workspace_bytes(int64_t n, int64_t nrhs, size_t* bytes);
int mgt_residual(const void* M, int64_t n, int64_t ldm, const void* X, int64_t ldx,
                 const void* B, int64_t ldb, void* R, int64_t ldr, int64_t nrhs,
                 void* work, size_t work_bytes, void* stream);

/*
 * The two halves of mgt_residual on its workspace (mgt_residual_workspace_bytes
 * for the largest nrhs to be applied): mgt_residual_prepare makes M's row
 * exponents and digits there; mgt_residual_apply then computes R = B - M X
 * from them, for any number of X while M is unchanged.  Stream-ordered: an
 * apply sees the prepare enqueued before it on the same stream.
 * MGT_ERR_UNSUPPORTED where the tensor-core residual is unavailable.
 */
int mgt_residual_prepare(const void* M, int64_t n, int64_t ldm, void* work, size_t work_bytes, void* stream);
int mgt_residual_apply(int64_t n, const void* X, int64_t ldx, const void* B, int64_t ldb, void* R, int64_t ldr,
                       int64_t nrhs, void* work, size_t work_bytes, void* stream);

/*
 * Mixed-precision solve of M X = B: complex64 LU factors of M (from
 * mgt_lu_factor with MGT_C64), M in MGT_CDF form for the residual,
 * refinement until ||B - M X||_F / ||B||_F <= tol or max_iter corrections.
 * X (complex128) receives the solution.  iters / rel_res (host pointers,
 * may be NULL) receive the number of corrections and the final relative
 * residual.  Returns MGT_ERR_NOT_CONVERGED if tol was not met.
 *
 * mgt_refine_prepare makes M's digits (the tensor-core residual's operand)
 * in a refinement workspace of mgt_refine_workspace_bytes(n, nrhs) bytes, so
 * that M itself may be freed: mgt_solve_refined, mgt_refine_correct and
 * mgt_refine_norms then take M = NULL and use the prepared digits, for any
 * nrhs up to the one prepared for (stream-ordered, like every call here).
 * MGT_ERR_UNSUPPORTED where the tensor-core residual is unavailable; M = NULL
 * without tensor cores is MGT_ERR_ARG.
 */
int mgt_refine_workspace_bytes(int64_t n, int64_t nrhs, size_t* bytes);
int mgt_refine_prepare(const void* M, int64_t ldm, int64_t n, int64_t nrhs, void* work, size_t work_bytes,
                       void* stream);
int mgt_solve_refined(const void* M, int64_t ldm, const void* LU, int64_t ldlu,
                      const int32_t* perm, int64_t n, const void* B, int64_t ldb,
                      void* X, int64_t ldx, int64_t nrhs, double tol, int max_iter,
                      void* work, size_t work_bytes, int* iters, double* rel_res,
                      void* stream);

/*
 * The refinement of mgt_solve_refined as stream-ordered steps that never
 * synchronise with the host, so a whole refined solve can be captured into a
 * CUDA graph (the batched sweep does).  Same workspace as mgt_solve_refined.
 *   mgt_refine_start:   X = LU^-1 B (complex64 solve, widened to complex128)
 *   mgt_refine_correct: X += LU^-1 (B - M X), residual as in mgt_residual
 *                       (M's digits are made again in each call)
 *   mgt_refine_norms:   norms_dev[0] = ||B||_F^2, norms_dev[1] = ||B - M X||_F^2
 *                       (device doubles; the caller reads them when it syncs)
 */
int mgt_refine_start(const void* LU, int64_t ldlu, const int32_t* perm, int64_t n, const void* B, int64_t ldb,
                     void* X, int64_t ldx, int64_t nrhs, void* work, size_t work_bytes, void* stream);
int mgt_refine_correct(const void* M, int64_t ldm, const void* LU, int64_t ldlu, const int32_t* perm, int64_t n,
                       const void* B, int64_t ldb, void* X, int64_t ldx, int64_t nrhs, void* work,
                       size_t work_bytes, void* stream);
int mgt_refine_norms(const void* M, int64_t ldm, int64_t n, const void* B, int64_t ldb, const void* X, int64_t ldx,
                     int64_t nrhs, void* work, size_t work_bytes, double* norms_dev, void* stream);

/*
 * Propagation to detectors:
 *   out[m*d + a, r] = coef * sum_{j,b} G_ab(t_m - s_j) Ek[j*d + b, r] + E0[m*d + a, r]
 * dtype MGT_C128 (the plain method): matrix-free, G is recomputed on the fly
 * in FP64 and contracted in FP64, never stored.  MGT_CDF (the mixed method):
 * the rows -coef G are evaluated in FP64, stored double-float in chunks of at
 * most 1 GiB of the workspace and contracted with Ek by the tensor-core
 * residual kernel (out = E0 - (-coef G) Ek; see mgt_residual), or in
 * double-float on the FP32 pipes where the tensor cores are unavailable.
 * Ek, E0 and out are complex128 in both cases.  Replaces the dense
 * G0(points) + matmul of propagate() (Transmission2D.py:190, :701;
 * Transmission3D.py:163, :675) and propagate_ss().  Rows where the
 * reference's G is NaN come out NaN; the host applies the reference's
 * row fix-up.  E0 may be NULL (treated as zero).
 */
int mgt_propagate_workspace_bytes(int kind, int64_t n_targets, int64_t n_sources, int64_t nrhs,
                                  size_t* bytes);
int mgt_propagate(int kind, int dtype, const double* targets, int64_t n_targets,
                  const double* sources, int64_t n_sources, double k0, double coef_re,
                  double coef_im, int regularize, double radius, const void* Ek,
                  int64_t ld_ek, const void* E0, int64_t ld_e0, void* out, int64_t ld_out,
                  int64_t nrhs, void* work, size_t work_bytes, void* stream);

/*
 * Column dots for the DOS: out[i] = sum_k A[k, i] * B[k, i] (no conjugate),
 * complex128, A and B (n x ncols) row-major.  With A = Gm^T and
 * B = M^-1 Gm^T, sum_i out[i] = sum((Gm^T Gm) * W) of
 * mean_DOS_measurements (Transmission2D.py:327) and out[i] is the
 * diag(Gm W Gm^T) entry of LDOS_measurements (Transmission2D.py:379).
 */
int mgt_column_dots(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t n,
                    int64_t ncols, void* out, void* stream);

/*
 * Tuning knobs of the LU (no counterpart in the reference), process-wide:
 *   MGT_TUNE_PANEL_ROWS  rows of the panel each CTA of the panel kernel aims
 *                        for (32..4096, default 256; the shared-memory limit
 *                        can raise the CTA count further)
 *   MGT_TUNE_OUTER_BLOCK outer block width of the complex64 tensor-core LU,
 *                        64 or 128 (default 128: two inner panels per block)
 *   MGT_TUNE_PANEL_MAX_CTAS  upper bound on the panel kernel's CTAs (0: one per SM)
 *   MGT_TUNE_COOPERATIVE  1 (default): the panel kernel is a cooperative
 *                        launch; 0: a plain launch (for CUDA-graph capture),
 *                        where the caller keeps the CTAs of all panels that may
 *                        run at once within the SM count (every panel CTA
 *                        then finds an SM and no panel waits on another)
 *   MGT_TUNE_PANEL_REGISTERS  panels with at most 256 rows per CTA keep one row
 *                        per thread in registers: 1 (default) for complex64,
 *                        2 for both types, 0 never (rows in shared memory)
 *   MGT_TUNE_TC_PRECISION  split-product scheme of the complex64 tensor-core
 *                        update: MGT_TC_F16X2 (default; operands scaled by
 *                        powers of two, split into two fp16, kind::f16) or
 *                        MGT_TC_TF32X3 (split into two tf32, kind::tf32); both
 *                        give ~22 significant bits per operand
 *   MGT_TUNE_LOOKAHEAD   1 (default): the complex64 tensor-core LU factors the
 *                        next block's panels on a side stream's spare SMs while
 *                        the rest of the trailing update runs (cooperative
 *                        panels, not under stream capture); 0: strictly in order
 *   MGT_TUNE_FUSED_RIGHT 1 (default): the complex64 tensor-core LU treats the
 *                        columns right of each 128-wide block in one pass (both
 *                        panels' interchanges, solves with the inverted 64 x 64
 *                        diagonal blocks); 0: two swap passes and a pre-update
 *                        pass with substitution
 *   MGT_TUNE_PANEL_CLUSTER 1 (default): complex64 register panels of at most 16
 *                        CTAs (8 where the device schedules no larger cluster)
 *                        run as one thread-block cluster and exchange pivots
 *                        through distributed shared memory; 0: through L2
 *   MGT_TUNE_SYM_ASSEMBLY 1 (default): mgt_assemble_system evaluates each pair
 *                        of points once and writes both mirror-image blocks
 *                        (bitwise the same matrix); 0: every block evaluated
 *   MGT_TUNE_WIDE_UPDATE smallest trailing order at which the complex64
 *                        tensor-core LU with tile pivoting pairs two 128-wide
 *                        blocks, so that the columns right of the pair take
 *                        one trailing update with K = 256 (default 8192;
 *                        0: never)
 * Set by the batched sweep and its autotuner; mgt_get_tuning returns the value.
 */
#define MGT_TUNE_PANEL_ROWS 1
#define MGT_TUNE_OUTER_BLOCK 2
#define MGT_TUNE_PANEL_MAX_CTAS 3
#define MGT_TUNE_COOPERATIVE 4
#define MGT_TUNE_PANEL_REGISTERS 5
#define MGT_TUNE_TC_PRECISION 6
#define MGT_TUNE_LOOKAHEAD 7
#define MGT_TUNE_FUSED_RIGHT 8
#define MGT_TUNE_PANEL_CLUSTER 9
#define MGT_TUNE_SYM_ASSEMBLY 10
#define MGT_TUNE_WIDE_UPDATE 11
#define MGT_TC_TF32X3 0
#define MGT_TC_F16X2 1
int mgt_set_tuning(int key, int value);
int mgt_get_tuning(int key);

/*
 * Diagnostics (no counterpart in the reference, which has no GPU path):
 * a counter of this library's kernel launches and optional CUDA-event timing
 * of every launch of the dominant kernel (the LU trailing update), with its
 * algorithmic flops and DRAM bytes.  mgt_diag_reset zeroes the counters and
 * turns the timing on or off; mgt_diag_read synchronises on the recorded
 * events and returns the totals (any pointer may be NULL).
 */
int mgt_diag_reset(int enable_timing);
int mgt_diag_read(uint64_t* launches, uint64_t* dom_launches, double* dom_ms, double* dom_flops,
                  double* dom_bytes);

#ifdef __cplusplus
}
#endif

#endif /* MAGREETE_GB300_H */
