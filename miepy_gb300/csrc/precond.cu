// Block-diagonal right preconditioners of the BiCGSTAB solves
// (cpp/src/interactions.cpp:211-345, builders src/miepy/interactions.py:9-68).
//
// The reference applies M = blockdiag(M_0 .. M_{N-1}) inside Eigen's BiCGSTAB:
// p^ = M p, v = A p^, s^ = M s, t = A s^, x += alpha p^ + omega s^.  That is
// BiCGSTAB on A M for u with x = M u: the residuals b - A M u = b - A x and every
// scalar of the two forms agree.  The packed sphere solver takes M's diagonal
// (the sphere builder's diag(1 / (1 + a_n))) and folds it into its products;
// the dense solver runs on (I + T) M - I, formed here, and maps u back to x.

#include <algorithm>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace {

// d = 1 / (1 + t) per row of the Mie-factor arena, 1 where |1 + t| < 1e-12
// (build_block_preconditioner_sphere, src/miepy/interactions.py:29-37).
__global__ void k_sphere_precond(const double2* __restrict__ t, double2* __restrict__ d, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const double2 v = make_double2(1.0 + t[e].x, t[e].y);
        const double m2 = v.x * v.x + v.y * v.y;
        d[e] = (sqrt(m2) < 1e-12) ? make_double2(1.0, 0.0) : make_double2(v.x / m2, -v.y / m2);
    }
}

// Tp = (I + T) M - I for a dense T [D][D] and M_inv_blocks [D][bs] (block j in rows
// j bs .. j bs + bs - 1).  Thread per output element, lanes along a row: the T
// segment of a block is shared by the lanes of that block, the M rows are read
// contiguously.
__global__ void k_dense_precond(int D, int bs, const double2* __restrict__ T, const double2* __restrict__ Minv,
                                double2* __restrict__ Tp) {
    const long long total = (long long)D * D;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / D), c = (int)(e % D);
        const int j0 = (c / bs) * bs, cc = c - j0;
        const double2* Tr = T + (long long)r * D + j0;
        const double2* Mj = Minv + (long long)j0 * bs + cc;
        double2 acc = make_double2(0.0, 0.0);
        for (int k = 0; k < bs; k++) cfma(acc, Tr[k], Mj[(long long)k * bs]);
        if (r >= j0 && r < j0 + bs) {   // the identity's share: M_j[r - j0, cc]
            const double2 m = Mj[(long long)(r - j0) * bs];
            acc.x += m.x;
            acc.y += m.y;
        }
        if (r == c) acc.x -= 1.0;
        Tp[e] = acc;
    }
}

// x = M u for R right-hand sides ([D][R] both).
__global__ void k_block_apply(int D, int R, int bs, const double2* __restrict__ Minv, const double2* __restrict__ u,
                              double2* __restrict__ x) {
    const long long total = (long long)D * R;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int row = (int)(e / R), rr = (int)(e % R);
        const int j0 = (row / bs) * bs;
        const double2* Mr = Minv + (long long)row * bs;
        double2 acc = make_double2(0.0, 0.0);
        for (int k = 0; k < bs; k++) cfma(acc, Mr[k], u[(long long)(j0 + k) * R + rr]);
        x[e] = acc;
    }
}

unsigned grid_for(long long n) {
    return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)gb::sm_count() * 16));
}

}   // namespace

extern "C" {

int gb_sphere_preconditioner(long long n, const double* tvec, double* pdiag, void* stream) {
    if (n < 0 || (n > 0 && (!tvec || !pdiag))) return gb_set_error(GB_BAD_ARG, "null argument");
    if (n == 0) return GB_OK;
    gb::note_launch();
    k_sphere_precond<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const double2*>(tvec),
                                                                     reinterpret_cast<double2*>(pdiag), n);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

int gb_dense_precondition_matrix(int D, int bs, const double* T, const double* Minv, double* Tp, void* stream) {
    if (D < 1 || bs < 1 || !T || !Minv || !Tp) return gb_set_error(GB_BAD_ARG, "null argument or empty system");
    if (D % bs) return gb_set_error(GB_BAD_ARG, "block size %d does not divide D = %d", bs, D);
    if (Tp == T) return gb_set_error(GB_BAD_ARG, "Tp must not alias T");
    gb::note_launch();
    k_dense_precond<<<grid_for((long long)D * D), 256, 0, (cudaStream_t)stream>>>(
        D, bs, reinterpret_cast<const double2*>(T), reinterpret_cast<const double2*>(Minv),
        reinterpret_cast<double2*>(Tp));
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

int gb_block_diag_apply(int D, int R, int bs, const double* Minv, const double* u, double* x, void* stream) {
    if (D < 1 || R < 1 || bs < 1 || !Minv || !u || !x) return gb_set_error(GB_BAD_ARG, "null argument or empty system");
    if (D % bs) return gb_set_error(GB_BAD_ARG, "block size %d does not divide D = %d", bs, D);
    if (u == x) return gb_set_error(GB_BAD_ARG, "x must not alias u");
    gb::note_launch();
    k_block_apply<<<grid_for((long long)D * R), 256, 0, (cudaStream_t)stream>>>(
        D, R, bs, reinterpret_cast<const double2*>(Minv), reinterpret_cast<const double2*>(u),
        reinterpret_cast<double2*>(x));
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

}   // extern "C"
