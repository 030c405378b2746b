// Plan records of the packed-operator solve, shared by the BiCGSTAB driver and its
// CUDA-core matrix pass (solve.cu) and the tensor-core matrix pass (gemv_tc.cu).
#pragma once

#include <cuda_runtime.h>

#include "gb_internal.h"

namespace gb {

struct Strip {          // GEMV work: blocks (i, j0 .. j0+nb-1) of cluster sys
    int sys, i, nb, pad;
    long long p0;       // first pair index (cluster-local)
};
struct Item {           // rows [r0, r0+nr) of cluster sys
    int sys, r0, nr, pad;
};
struct SysPlan {
    long long strip_row_base;   // index into row_strip (first block row of this cluster)
    long long strip_base;       // global index of the first strip of this cluster
    long long cw_off;           // element offset of this cluster's per-pair column partials
    long long cu_off;           // element offset of this cluster's per-strip row partials
    int vbeg, vend;             // vector items
    int rbeg, rend;             // reduce items
};

struct KState {         // per (cluster, rhs) BiCGSTAB scalars
    double2 rho, alpha, omega, beta;   // FP64 solver
    double r0sq, bsq, rsq, tol2;       // (bsq, rsq also mirrored from the FP32 solver, for the host)
    float2 rho_f, alpha_f, omega_f, beta_f;   // FP32 solver
    float r0sq_f, bsq_f, rsq_f, tol2_f;
    int iters, restarts, done, status;
    int need_restart, maxiter, pad0, pad1;
};

// mask_mode: -1 all, 0 running clusters, 1 restarting clusters
template <int R>
__device__ __forceinline__ bool active_rhs(const KState* st, int sys, int rr, int mask_mode) {
    if (mask_mode < 0) return true;
    const KState& k = st[sys * R + rr];
    return (mask_mode == 0) ? (!k.done && !k.need_restart) : (k.need_restart != 0);
}
template <int R>
__device__ __forceinline__ bool any_active(const KState* st, int sys, int mask_mode) {
    bool a = false;
#pragma unroll
    for (int rr = 0; rr < R; rr++) a |= active_rhs<R>(st, sys, rr, mask_mode);
    return a;
}

// Tensor-core matrix pass (gemv_tc.cu) over strips [sbeg, send) of one block size
// B: the same column partials (CW, per pair by destination block row) and row
// partials (CU, per strip) as the CUDA-core pass with complex64 arithmetic, as
// float2 [B][R] per term, from the bf16 hi/lo tiles of the matrix (mat_tc) and the
// y vectors Yu, Yw (float2 [D][R]).  R is 4 or 8.
int launch_pgemv_tc(int R, const SysDev* sys, const Strip* strips, long long sbeg, long long send, const KState* st,
                    int mask, const void* mat_tc, const void* Yu, const void* Yw, void* CU, void* CW,
                    const SysPlan* plan, int B, int* err, cudaStream_t stream);

// The R = 4 and 8 solves, applies and wait limit, compiled in their own unit
// (solve_multi.cu, which includes solve.cu with GB_SOLVE_MULTI_RHS defined) so that
// the two halves of the solver compile in parallel.
int solve_entry_multi(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter, double inner_tol,
                      int max_refine, const double* mat128, const float* mat64, const float* mat64lo,
                      const void* mat_tc, const double* pdiag, const double* tvec, const double* b, double* x,
                      void* workspace, size_t ws_bytes, int* status, int* iters, double* resid, cudaStream_t stream);
int apply_entry_multi(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                      const float* mat64lo, const void* mat_tc, const double* tvec, const double* x, double* y,
                      void* workspace, size_t ws_bytes, int reps, int repeat, cudaStream_t stream);
int set_wait_limit_multi(long long cycles);

}   // namespace gb
