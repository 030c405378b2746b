/*
 * miepy_gb300 -- C ABI of the GB300 (sm_103a) sphere-cluster aggregate T-matrix path.
 *
 * Every entry point takes plain device/host pointers and sizes, is ordered on the
 * CUDA stream it is given (NULL = legacy default stream), never throws, and returns
 * an int status (GB_OK = 0).  gb_last_error() returns the message of the last
 * failure on the calling thread.  All buffers are owned by the caller; entry points
 * that need scratch memory take a workspace pointer whose size is reported by the
 * matching *_workspace_size query.  The library itself holds only the per-lmax
 * coefficient tables (built on first use on each device) and small pinned host
 * staging buffers.
 *
 * Layout conventions (identical to the reference's C++ module):
 *   mode index      r = n(n+2) - n + m - 1,  n = 1..lmax, m = -n..n,  rmax = lmax(lmax+2)
 *   particle index  row = i*(2*rmax) + a*rmax + r   (a = 0 electric, 1 magnetic),
 *                   D = 2*rmax*N
 *   mie             [N, 2, lmax] complex128 (a_n then b_n), i.e. the reference's
 *                   mie_scat array, interleaved (re, im) doubles
 *   positions       [N, 3] float64
 *   dense matrices  [D, D] row-major complex128
 *
 * Packed pair-block format ("packed"): for the P = N(N-1)/2 pairs i < j in
 * i-major order, the block A_ij of the translation matrix WITHOUT the Mie
 * factors, B x B row-major (B = 2*rmax), one block after the other.  The full
 * aggregate matrix follows as  T[i,j] = A_ij diag(t_j)  and
 * T[j,i] = S A_ij S diag(t_i),  S = diag((-1)^(n+a)),  t_j = mie of particle j
 * expanded per row.  Half the storage of the dense matrix, no per-element Mie
 * product.
 */
#ifndef MIEPY_GB300_H
#define MIEPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GB_OK 0
#define GB_NOT_CONVERGED 1   /* maxiter reached before the tolerance */
#define GB_BREAKDOWN 2       /* Krylov breakdown that a restart did not cure */
#define GB_NAN 3             /* non-finite value in the iteration */
#define GB_OVER_BUDGET 4     /* workspace smaller than required */
#define GB_TIMEOUT 5         /* host-side wait limit reached */
#define GB_BAD_ARG 6
#define GB_CUDA_ERROR 7
#define GB_UNSUPPORTED 8

/* precision of a solve */
#define GB_PREC_FP64 0           /* complex128 matrix, complex128 Krylov vectors, FP64 arithmetic */
#define GB_PREC_MIXED 1          /* complex64 BiCGSTAB on the hi matrix; refinement residuals with the
                                    double-float (hi + lo) matrix, ~1e-14 relative accuracy, FP32 pipes;
                                    once |r| <= 2.5e4 tol |b| the residual is updated as r -= (I+T) d
                                    with the complex64 matrix */
#define GB_PREC_FP32 2           /* complex64 matrix + complex64 BiCGSTAB, no refinement */
#define GB_PREC_MIXED_FP64RES 3  /* as MIXED, refinement residuals in FP64 arithmetic on the complex128 matrix */

int gb_version(void);
size_t gb_last_error(char* buf, size_t cap);
int gb_device_sm_count(void);
/* Number of kernels this library has launched in the process so far (graph
 * replays count every kernel node they run). */
long long gb_launch_count(void);

/* ---------------------------------------------------------------- tables --
 * Per-lmax translation coefficient table (replaces create_vsh_cache_map,
 * cpp/src/vsh_translation.cpp:36-51, with gaunt_batch / wigner_3j_batch,
 * cpp/src/special.cpp:298-440).  Built on the device on first use.
 * gb_tables_export copies it to the host for tests: M tuples, nmvu [M,4],
 * qAB [M,2], cA [M, lmax+1], cB [M, lmax+1], elem_map [(2rmax)^2]. */
int gb_tables_prepare(int lmax, void* stream);
int gb_tables_count(int lmax, int* M_out);
int gb_tables_export(int lmax, int* nmvu, int* qab, double* cA, double* cB, int* elem_map);

/* -------------------------------------------------------------- assembly --
 * Dense aggregate T-matrix in the reference layout (zero diagonal blocks):
 * replaces sphere_aggregate_tmatrix, cpp/src/interactions.cpp:370-415, with
 * vsh_translation_insert_pair (Mie overload), cpp/src/vsh_translation.cpp:161-237.
 * pos [N,3] f64, mie [N,2,lmax] c128, out [D,D] c128 (all device). */
int gb_assemble_sphere_dense(int N, int lmax, const double* pos, const double* mie, double k,
                             double* out, void* stream);

/* Reflection matrix of a planar interface at height z, in the reference layout:
 * replaces reflection_matrix_nia, cpp/src/interactions.cpp:464-512.  Block (i, j)
 * for every particle pair, the particle itself included: the outgoing translation
 * from particle j to the mirror image of particle i, times -r (-1)^(m+n+a+1) and the
 * Mie coefficient of particle j; r = r_re + i r_im is the normal-incidence
 * reflection coefficient.  The reference subtracts it from the aggregate T-matrix
 * (sphere_cluster.py:704-710).  pos [N,3] f64, mie [N,2,lmax] c128, out [D,D] c128. */
int gb_reflection_matrix_dense(int N, int lmax, const double* pos, const double* mie, double k, double r_re,
                               double r_im, double z, double* out, void* stream);

/* Aggregate T-matrix of a periodic cluster, in the reference layout: replaces
 * sphere_aggregate_tmatrix_periodic, src/miepy/interactions.py:153-186.  The
 * aggregate of gb_assemble_sphere_dense plus, for every ordered particle pair (i, j)
 * (the particle itself included), the lattice sum over the cells c of
 * e^{-i k khat.c} times the outgoing translation from pos_j + c to pos_i, times the
 * Mie coefficient of particle j.  cells [ncell,3] f64 (device; the lattice vectors
 * of miepy.symmetry's generators, the origin cell excluded), khat = (kx, ky, kz) the
 * source's unit wave vector.  pos [N,3] f64, mie [N,2,lmax] c128, out [D,D] c128. */
int gb_aggregate_periodic_dense(int N, int lmax, const double* pos, const double* mie, double k, const double* cells,
                                int ncell, double kx, double ky, double kz, double* out, void* stream);

/* Packed pair-block translation matrix of one cluster (see above).  Any
 * output may be NULL: out128 [P*B*B] c128; out64 [P*B*B] c64 = fl32(a);
 * out64lo [P*B*B] c64 = fl32(a - fl32(a)) (hi + lo carries ~48 bits).  Without
 * out128 the complex64 outputs are built in double-float by two launches, and the
 * first 2(2 lmax + 2)^2 words of each pair's block (in out64lo, else out64) hold
 * that pair's special-function table until its block is written. */
int gb_assemble_sphere_packed(int N, int lmax, const double* pos, double k, double* out128, float* out64,
                              float* out64lo, void* stream);

/* ------------------------------------------------------ batched clusters --
 * A batch describes independent clusters (ragged N and lmax) that share one
 * launch sequence.  Offsets are in elements of the respective device arrays. */
typedef struct {
    int32_t N;          /* particles */
    int32_t lmax;       /* expansion order: 1..10 for assembly (at 10 an assembly writing
                         * complex128 and complex64 outputs in one call needs more than a
                         * CTA's 227 KB of shared memory: GB_UNSUPPORTED), 1..8 for the
                         * packed solvers (larger orders solve on the dense operator) */
    double k;           /* medium wavenumber */
    int64_t pos_off;    /* into pos (doubles): first of 3*N */
    int64_t mat_off;    /* into the packed matrices (complex elements): first of P*B*B */
    int64_t vec_off;    /* into the [D][R] vectors (complex elements): first of D*R */
    int64_t t_off;      /* into the per-row Mie factor vector (complex128): first of D */
} gb_system;

/* Assemble the packed matrices of every cluster in the batch (one launch per
 * lmax, preceded by the special-function launch without mat128); outputs as for
 * gb_assemble_sphere_packed, any may be NULL. */
int gb_assemble_batch(int nsys, const gb_system* sys, const double* pos, double* mat128, float* mat64,
                      float* mat64lo, void* stream);

/* Expand Mie coefficients [N,2,lmax] into the per-row factor t (D entries) for
 * every cluster; mie_off[s] is the complex offset of cluster s in mie. */
int gb_expand_mie_batch(int nsys, const gb_system* sys, const int64_t* mie_off, const double* mie, double* tvec,
                        void* stream);

/* Solve (I + T) x = b for every cluster and right-hand side (replaces
 * solve_linear_system, cpp/src/interactions.cpp:347-368, BiCGSTAB branch; the
 * iteration is the one Eigen's BiCGSTAB runs: x0 = 0, restart when rho becomes
 * tiny, stop when |r| <= tol |b|).  R right-hand sides per cluster share every
 * matrix pass.  b and x are [D][R] complex128 per cluster at vec_off.
 * prec: GB_PREC_FP64 uses mat128; GB_PREC_FP32 uses mat64; GB_PREC_MIXED runs
 * FP32 BiCGSTAB on mat64 to inner_tol and refines x with residuals computed
 * from mat64 + mat64lo until |b - (I+T)x| <= tol |b| (at most max_refine
 * refinement passes; once every running cluster has |r| <= 2.5e4 tol |b|, the
 * next residual is updated from the correction d with mat64, whose ~2e-6
 * relative product error then stays below tol |b| / 20);
 * GB_PREC_MIXED_FP64RES takes its residuals from mat128.
 * status/iters/resid: host arrays of nsys*R entries (may be NULL); iters are
 * BiCGSTAB iterations (FP64/FP32) or refinement passes (mixed).
 * R is 1, 2, 4 or 8, with B * R <= 384 for every cluster (B = 2 lmax (lmax + 2));
 * with R = 4 or 8 the CUDA-core matrix passes run once per pair of right-hand
 * sides. */
size_t gb_solve_workspace_size(int nsys, const gb_system* sys, int R, int prec);
int gb_solve_batch(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter, double inner_tol,
                   int max_refine, const double* mat128, const float* mat64, const float* mat64lo,
                   const double* tvec, const double* b, double* x, void* workspace, size_t ws_bytes, int* status,
                   int* iters, double* resid, void* stream);

/* gb_solve_batch with two options, each off when its pointer is NULL (both NULL
 * gives gb_solve_batch).
 *
 * mat_tc: multi-RHS blocks on the tensor cores (no counterpart in the reference,
 * whose solve_linear_system, cpp/src/interactions.cpp:347-368, takes one right-hand
 * side per call and multiplies with an Eigen/OpenMP GEMV, :70-92).  For R = 4 or 8
 * right-hand sides (polarisations x incidence directions or sources) of clusters
 * with lmax <= 5, the matrix passes of the FP32 solves (GB_PREC_FP32, and the inner
 * solves of GB_PREC_MIXED) run as tcgen05 split-BF16x3 GEMMs with FP32
 * accumulation on mat_tc, the bf16 hi/lo tiles of mat64 made by
 * gb_tc_matrix_build: one pass serves all R right-hand sides.  The product is
 * about 5e-6 accurate relative to its largest term (complex64 arithmetic: 4e-7);
 * the mixed method's refinement residuals stay on the CUDA-core passes, so its
 * result meets tol as with gb_solve_batch.
 *
 * pdiag: a diagonal right preconditioner M, complex128 [row] at each cluster's
 * t_off like tvec (replaces solve_linear_system_preconditioned,
 * cpp/src/interactions.cpp:321-345, with the sphere preconditioner of
 * build_block_preconditioner_sphere, src/miepy/interactions.py:9-39: M =
 * diag(1 / (1 + a_n)) of the Mie coefficients, 1 where |1 + a_n| < 1e-12; see
 * gb_sphere_preconditioner).  Every BiCGSTAB of the solve is Eigen's
 * right-preconditioned iteration (p^ = M p, v = (I + T) p^, x += alpha p^ + omega
 * s^); the residual that decides convergence is the unpreconditioned one, so tol
 * means the same as without M, and the mixed method's refinement residuals are the
 * unpreconditioned b - (I + T) x.
 *
 * The workspace is gb_solve_workspace_size's. */
int gb_solve_batch_ex(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter, double inner_tol,
                      int max_refine, const double* mat128, const float* mat64, const float* mat64lo,
                      const void* mat_tc, const double* pdiag, const double* tvec, const double* b, double* x,
                      void* workspace, size_t ws_bytes, int* status, int* iters, double* resid, void* stream);

/* The sphere preconditioner of gb_solve_batch_ex: pdiag[e] = 1 / (1 + tvec[e]) over
 * n entries of the Mie-factor arena (tvec from gb_expand_mie_batch), 1 where
 * |1 + tvec[e]| < 1e-12 (build_block_preconditioner_sphere,
 * src/miepy/interactions.py:9-39, whose blocks are diagonal: this is their
 * diagonal, row by row). */
int gb_sphere_preconditioner(long long n, const double* tvec, double* pdiag, void* stream);

/* Block-diagonal right preconditioning of the dense solve (replaces
 * solve_linear_system_preconditioned, cpp/src/interactions.cpp:321-345, with any
 * M_inv_blocks, e.g. build_block_preconditioner_particle's inv(I + T_i),
 * src/miepy/interactions.py:42-68).  Eigen's preconditioned BiCGSTAB on (I + T) is
 * BiCGSTAB on (I + T) M for u, with x = M u and the same residuals; so
 *   gb_dense_precondition_matrix: Tp = (I + T) M - I   (T, Tp [D][D] c128, Tp != T),
 *   gb_solve_dense on Tp gives u,
 *   gb_block_diag_apply: x = M u                      (u, x [D][R] c128, x != u),
 * with Minv = M_inv_blocks [D][bs] c128 (block j in rows j bs .. j bs + bs - 1) and
 * bs dividing D. */
int gb_dense_precondition_matrix(int D, int bs, const double* T, const double* Minv, double* Tp, void* stream);
int gb_block_diag_apply(int D, int R, int bs, const double* Minv, const double* u, double* x, void* stream);

/* Bytes of the bf16 tile arena for a batch: per pair block 2 planes of Bp x Kp bf16
 * (Bp = B rounded up to 8, Kp = 2B rounded up to 16), clusters in batch order. */
size_t gb_tc_matrix_bytes(int nsys, const gb_system* sys);
/* mat_tc = the bf16 hi/lo tiles of the packed complex64 matrix mat64 (hi = bf16(a),
 * lo = bf16(a - hi) per real component), in the core-matrix layout the tensor-core
 * pass streams into shared memory; one launch, to be repeated after every
 * assembly.  Both pointers 16-byte aligned. */
int gb_tc_matrix_build(int nsys, const gb_system* sys, const float* mat64, void* mat_tc, void* stream);

/* Dense solve of (I + T) x = b for a caller-supplied dense aggregate matrix
 * T [D,D] c128 (the plugin path, where the caller already holds T).  BiCGSTAB as
 * above in FP64, R right-hand sides stored [D][R]. */
size_t gb_solve_dense_workspace_size(int D, int R);
int gb_solve_dense(int D, int R, const double* T, const double* b, double* x, double tol, int maxiter,
                   void* workspace, size_t ws_bytes, int* status, int* iters, double* resid, void* stream);

/* gb_solve_dense without any allocation, for callers that cannot allocate device
 * memory: a server whose HBM is reserved up front, or a loop in which cudaMalloc /
 * cudaFree would synchronise the device.  It has no counterpart in the reference.
 * The solve (same arguments and results as gb_solve_dense) runs in a fixed scratch
 * array of 1.25 MiB that the library carries in device memory; D * R may be at most
 * 8192, larger sizes return GB_OVER_BUDGET.  No cudaMalloc, cudaFree or pinned host
 * buffer is used.  Every call looks up the array's address in the current device's
 * context; the first call on a device may load the library's module there, so make
 * it before any stream capture begins.  All calls on a device
 * share the one array and it keeps the previous call's contents: calls whose work
 * overlaps on the GPU (other streams, other host threads) race on it. */
int gb_solve_dense_noalloc(int D, int R, const double* T, const double* b, double* x, double tol, int maxiter,
                           int* status, int* iters, double* resid, void* stream);

/* One application y = (I + T) x of the packed operator, for tests and
 * benchmarks: FP64 arithmetic on mat128 (GB_PREC_FP64), FP32 on mat64
 * (GB_PREC_FP32) or double-float on mat64 + mat64lo (GB_PREC_MIXED).
 * x, y: [D][R] complex128. */
size_t gb_apply_workspace_size(int nsys, const gb_system* sys, int R, int prec);
int gb_apply_batch(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                   const float* mat64lo, const double* tvec, const double* x, double* y, void* workspace,
                   size_t ws_bytes, void* stream);

/* GEMV tile-shape autotuner (no counterpart in the reference, whose matvec is an
 * Eigen/OpenMP row-block product, cpp/src/interactions.cpp:27-92).  For every
 * block-size group of the batch, times each lane shape covering the block on the
 * batch's own plan and matrix (reps passes per shape, CUDA events on stream) and
 * keeps the fastest for that block size, precision class (GB_PREC_FP64: the
 * complex128 pass; any other: the complex64 pass) and R, in a process-wide table
 * that later solves use.  x [total_vec * R] is any vector (it feeds the y vectors),
 * y receives one product; the workspace is gb_apply_workspace_size's for
 * GB_PREC_FP64 or GB_PREC_FP32.  Call it outside stream capture. */
int gb_autotune_gemv(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                     const double* tvec, const double* x, double* y, void* workspace, size_t ws_bytes, int reps,
                     void* stream);

/* The lane shape (lanes per matrix row, columns per lane) the GEMV uses for block
 * size B, precision class and R: the autotuned one, else the model's. */
int gb_gemv_shape(int B, int prec, int R, int* lanes_per_row, int* cols_per_lane);

/* The operator product of gb_apply_batch launched reps times back to back on
 * one prepared plan (no host work between launches), for kernel timing with
 * events on the stream.  gemv_only != 0 repeats only the matrix pass (the
 * partial-sum kernel) after the first full product. */
int gb_apply_repeat(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                    const float* mat64lo, const double* tvec, const double* x, double* y, void* workspace,
                    size_t ws_bytes, int reps, int gemv_only, void* stream);

/* gb_apply_repeat with the tensor-core pass (R = 4 or 8): y = (I + T) x from the
 * bf16 tiles mat_tc, x rounded to complex64, y widened to FP64; reps = 1 is one
 * product.  The workspace is gb_apply_workspace_size's for GB_PREC_FP32. */
int gb_apply_repeat_tc(int nsys, const gb_system* sys, int R, const void* mat_tc, const double* tvec, const double* x,
                       double* y, void* workspace, size_t ws_bytes, int reps, int gemv_only, void* stream);

/* Wait limit of the GEMV's consumer waits on its matrix copies, in SM clock cycles
 * (no counterpart in the reference, whose matvec has no asynchronous copies).  A
 * wait that expires sets the launch's error flag and the call returns GB_TIMEOUT;
 * the warp first drains its own copies in flight with the default limit.  cycles = 0
 * makes every consumer wait expire at once (a test of that path); cycles < 0
 * restores the default (4e8 cycles, about 0.2 s).  The limit is per device (the
 * current one), read by every later launch, graph replays included.  previous, if
 * not null, receives the limit before the call. */
int gb_set_gemv_wait_limit(long long cycles, long long* previous);

/* -------------------------------------------------------------- epilogue --
 * Per cluster and right-hand side, from p_inc [D][R] (c128), p_src [D][R],
 * mie_scat / mie_int [N,2,lmax] c128:
 *   p_scat = t o p_inc,  p_int = p_inc * mie_int[:, ::-1, n-1]   (sphere_cluster.py:715-717)
 *   xs[N][R][3][2*Lx] per-multipole (Cscat, Cabs, Cext)          (cpp/src/flux.cpp:5-30)
 *      with Lx the largest lmax of the batch (a cluster of smaller lmax fills
 *      the first 2*lmax entries of each row and leaves the rest untouched)
 *   force, torque [N][R][3]                                       (cpp/src/forces.cpp:7-137)
 * with the incident coefficients p_inc (source != 0) or p_inc - p_src
 * (source == 0) in the force/torque sums (sphere_cluster.py:521-559).
 * eps_b: medium permittivity (real part used, as the reference's double eps_b).
 * p_scat/p_int are written at vec_off; xs/force/torque at obs_off[s] particles.
 * mie_off[s]: complex offset of cluster s in mie_scat/mie_int.  Any output
 * pointer may be NULL. */
int gb_epilogue_batch(int nsys, const gb_system* sys, int R, const int64_t* mie_off, const int64_t* obs_off,
                      const double* mie_scat, const double* mie_int, const double* p_inc, const double* p_src,
                      double eps_b, int source, double* p_scat, double* p_int, double* xs, double* force,
                      double* torque, void* stream);

/* ---------------------------------------------------- general particles --
 * Clusters of particles given by their T-matrices: the reference's
 * particle_aggregate_tmatrix (cpp/src/interactions.cpp:416-462) with the T-matrix
 * overload of vsh_translation_insert_pair (cpp/src/vsh_translation.cpp:53-159),
 * whose block (i, j) is A_ij T_j, and cluster._solve_interactions
 * (cluster.py:652-657).  The packed translation blocks A come from
 * gb_assemble_batch (they do not depend on the particles); each particle's T-matrix
 * [B][B] (B = 2 rmax, row-major, the reference's mode order) is applied to the
 * vector before every matrix pass.  tmat128 / tmat64: complex128 / complex64
 * T-matrices of all particles of all clusters, cluster s starting at complex
 * offset tm_off[s]; GB_PREC_FP64 needs tmat128, GB_PREC_FP32 tmat64, the mixed
 * methods both.  lmax <= 8.  Other arguments and results as gb_solve_batch (tvec
 * is not used); the workspace is gb_solve_workspace_size's. */
int gb_solve_batch_tmatrix(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter,
                           double inner_tol, int max_refine, const double* mat128, const float* mat64,
                           const float* mat64lo, const double* tmat128, const float* tmat64, const int64_t* tm_off,
                           const double* b, double* x, void* workspace, size_t ws_bytes, int* status, int* iters,
                           double* resid, void* stream);

/* Dense aggregate T-matrix of N general particles in the reference layout (replaces
 * particle_aggregate_tmatrix, cpp/src/interactions.cpp:417-462, with the T-matrix
 * overload of vsh_translation_insert_pair, cpp/src/vsh_translation.cpp:53-159):
 * block (i, j) = A_ij T_j for i != j, zero for i = j, with A_ij the translation
 * blocks of gb_assemble_sphere_dense at unit Mie coefficients.  pos [N,3] f64,
 * tmat [N][B][B] c128 (B = 2 rmax: each particle's [2, rmax, 2, rmax] T-matrix
 * row-major), out [D,D] c128; the workspace (gb_particle_aggregate_workspace_size
 * bytes) holds A and the unit coefficients. */
size_t gb_particle_aggregate_workspace_size(int N, int lmax);
int gb_particle_aggregate_dense(int N, int lmax, const double* pos, const double* tmat, double k, void* workspace,
                                size_t ws_bytes, double* out, void* stream);

/* Epilogue of T-matrix clusters: p_scat = T p_inc per particle (required output),
 * then the cross-sections per (a, n), forces and torques of gb_epilogue_batch from
 * p_scat, p_inc and p_src (flux.cpp:5-30, forces.cpp:7-171). */
int gb_tmatrix_epilogue_batch(int nsys, const gb_system* sys, int R, const double* tmat128, const int64_t* tm_off,
                              const int64_t* obs_off, const double* p_inc, const double* p_src, double eps_b,
                              int source, double* p_scat, double* xs, double* force, double* torque, void* stream);

/* Cross-sections of particles from given coefficients (replaces
 * flux.particle_cross_sections, cpp/src/flux.cpp:5-30, and the plugin function
 * particle_cross_sections_jax, backends/jax/flux.py:14-44): p_* [N,2,rmax] c128
 * -> out [N][3][2*lmax] (Cscat, Cabs, Cext), all device. */
int gb_particle_cross_sections(int N, int lmax, const double* p_scat, const double* p_inc, const double* p_src,
                               double k, double* out, void* stream);

/* ---------------------------------------------------------------- fields --
 * Near field of one cluster at Npts points, following sphere_cluster.E_field /
 * H_field (sphere_cluster.py:244-391) with expand_E / expand_H
 * (vsh/expansion.py:13-108) and the VSH of cpp/src/vsh_functions.cpp:60-98:
 *   outside every sphere: sum over particles of the outgoing expansion of p_scat
 *     about the particle (h_n(k r)), factor i E_mn;
 *   inside sphere i (when interior != 0): the interior expansion of p_int[i] with
 *     j_n(k_int,i r) (complex k_int, upward recurrence), factor -i E_mn; the
 *     scattered sum is not added there (the reference overwrites those points).
 * magnetic != 0 evaluates H: expand_E of the polarisation-swapped coefficients
 * times -i sqrt(eps/mu) (medium values outside, hfac_int[i] inside).
 * pos [N,3], radius [N], p_scat / p_int [N,2,rmax] c128, k (medium),
 * k_int [N] c128, hfac (re, im) and hfac_int [N] c128 (only for magnetic),
 * pts [Npts,3] f64 -> out [Npts,3] c128 (Cartesian).  The source field is not
 * included. */
int gb_near_field(int N, int lmax, const double* pos, const double* radius, const double* p_scat,
                  const double* p_int, double k, const double* k_int, int Npts, const double* pts, int interior,
                  int magnetic, double hfac_re, double hfac_im, const double* hfac_int, double* out, void* stream);

/* gb_near_field with the exterior sums (outgoing expansions of p_scat about every
 * particle) in FP32, for large maps; points inside a sphere take the FP64 interior
 * expansion.  Same arguments and output layout.  About 1e-6 relative accuracy
 * against gb_near_field (no counterpart in the reference, whose field evaluation
 * is the Python of sphere_cluster.py:244-391). */
int gb_near_field32(int N, int lmax, const double* pos, const double* radius, const double* p_scat,
                    const double* p_int, double k, const double* k_int, int Npts, const double* pts, int interior,
                    int magnetic, double hfac_re, double hfac_im, const double* hfac_int, double* out, void* stream);

/* Far-field form of the scattered field (replaces sphere_cluster.E_field /
 * H_field with far=True, src/miepy/sphere_cluster.py:244-391, whose per-particle
 * expand_E_far / expand_H_far are src/miepy/vsh/expansion.py:45-77,96-108): at each
 * point the sum over particles of e^{ikr}/(kr) (-i)^n E_mn (tau, pi) terms of p_scat
 * about the particle, no radial component and no interior expansions.  magnetic
 * swaps the coefficients and multiplies by hfac (-i sqrt(eps_b / mu_b)).
 * pos [N,3], p_scat [N,2,rmax] c128, pts [Npts,3] f64 (device), out [Npts][3] c128. */
int gb_far_field_expansions(int N, int lmax, const double* pos, const double* p_scat, double k, int Npts,
                            const double* pts, int magnetic, double hfac_re, double hfac_im, double* out,
                            void* stream);

/* ------------------------------------------------------------ beam source --
 * Beam expansion coefficients at N particles from the beam's far-field
 * projection: replaces integrate_phase, cpp/src/decomposition.cpp:29-66, as
 * applied per particle by beam.structure, sources/beams.py:168-200.
 *   pos [N,3] f64 (positions relative to the beam centre), rhat [G,3] f64 far-field
 *   directions, w [G][ncol] c128 the projected angular spectrum times the
 *   trapezoid weights of the (theta, phi) grid, ncol = 2*rmax columns (a*rmax + r);
 *   out[(i*ncol + c) * out_stride] = sum_g w[g][c] exp(-i k rhat_g . pos_i)  (c128). */
int gb_beam_project(int N, int ncol, int G, const double* pos, const double* rhat, const double* w, double k,
                    double* out, int out_stride, void* stream);

/* ------------------------------------------- cluster coefficients / far field --
 * Cluster expansion about one origin: replaces cluster_coefficients,
 * vsh/cluster_coefficients.py:14-53, with the incident-mode vsh_translation of
 * cpp/src/vsh_translation.cpp:428-470.  pos [N,3] f64, p_scat [N,2,rmax(lmax)] c128
 * (device); origin [3] f64 (host); p_cluster [2,rmax(lmax_cluster)] c128 (device).
 * Scratch: gb_cluster_coefficients_workspace_size(N, lmax_cluster) bytes. */
size_t gb_cluster_coefficients_workspace_size(int N, int lmax_cluster);
int gb_cluster_coefficients(int N, int lmax, const double* pos, const double* p_scat, double k, const double* origin,
                            int lmax_cluster, double* p_cluster, void* workspace, size_t ws_bytes, void* stream);

/* Far-field E (or H) of the cluster in spherical components at points (R, theta,
 * phi) about the origin: replaces E_angular / H_angular, sphere_cluster.py:393-426,
 * through expand_E_far / expand_H_far, vsh/expansion.py:45-108.  radius, theta, phi
 * [Npts] f64 (device); out [Npts][2] c128 (E_theta, E_phi); magnetic: swapped
 * coefficients times hfac.  Scattered field only (no source). */
int gb_far_field(int N, int lmax, const double* pos, const double* p_scat, double k, const double* origin, int Npts,
                 const double* radius, const double* theta, const double* phi, int magnetic, double hfac_re,
                 double hfac_im, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MIEPY_GB300_H */
