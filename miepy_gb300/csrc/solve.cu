// K3/K4: interaction-matrix products and the BiCGSTAB solve.
//
// Replaces solve_linear_system (cpp/src/interactions.cpp:347-368) with its
// OpenMP GEMV (ParallelDenseMatrix::scaleAndAddTo, :70-92) and Eigen's
// BiCGSTAB<IdentityPreconditioner>.
//
// Operator.  For a cluster, (I + T) x with T[i,j] = A_ij diag(t_j) (i < j, stored)
// and T[j,i] = S A_ij S diag(t_i).  Only the packed blocks A_ij are read, once
// per product, serving both block rows.  The translation blocks obey
// A[rho(s)][rho(r)] = eps(r) eps(s) A[r][s]  (rho: m -> -m, eps = (-1)^(m+a)),
// the placement symmetry of the reference's insertion loop, so both products of a
// block are computed as COLUMN sums  c[s] = sum_r A[r][s] y[r]  with
//   y_u[r] = eps(r) t_j[rho(r)] x_j[rho(r)]             (for block row i)
//   y_w[r] = eps(r) sig(r) t_i[rho(r)] x_i[rho(r)]      (for block row j)
// and (A_ij z_j)[r] = eps(r) c_u[rho(r)],  (S A_ij S z_i)[r] = sig(r) eps(r) c_w[rho(r)].
// Column sums let a warp stream a block row by row with every lane owning fixed
// columns: 128-bit coalesced loads, per-lane accumulators, no cross-lane traffic.
//
// K3a (k_pgemv): warp per strip of consecutive blocks (i, j0..j0+J-1) of one block
//   row.  c_u accumulates across the strip (written once per strip), c_w is
//   written per block.  Deterministic: no atomics.
// K3b (k_reduce): thread per row; sums the strip / block partials in a fixed order,
//   adds the identity term and emits per-item partial dot products.
// K4: BiCGSTAB vector updates fused with the dot-product partials, and one-thread-
//   per-(cluster, rhs) scalar kernels; all scalars stay on the device.  The host
//   launches fixed chunks of iterations and reads back one flag array per chunk;
//   kernels of finished clusters return immediately.
//
// The iteration is Eigen's: x0 = 0, r0 = r = b, rho = alpha = omega = 1, restart
// with r = b - A x when |rho| < eps^2 |r0|^2, stop when |r|^2 <= tol^2 |b|^2.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace {

constexpr int kItemRows = 128;      // rows per vector/reduce work item (= threads per CTA)
constexpr int kGemvThreads = 256;   // 8 warps
constexpr int kChunk = 4;           // iterations per host check

// ------------------------------------------------------------ type helpers --
template <typename T> struct Cplx;
template <> struct Cplx<double> { using t = double2; };
template <> struct Cplx<float> { using t = float2; };

__device__ __forceinline__ double2 to_d2(double2 v) { return v; }
__device__ __forceinline__ double2 to_d2(float2 v) { return make_double2(v.x, v.y); }
template <typename VT> __device__ __forceinline__ VT from_d2(double2 v);
template <> __device__ __forceinline__ double2 from_d2<double2>(double2 v) { return v; }
template <> __device__ __forceinline__ float2 from_d2<float2>(double2 v) {
    return make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
}

__device__ __forceinline__ void acc_fma(double2& a, double2 m, double2 y) { cfma(a, m, y); }
__device__ __forceinline__ void acc_fma(float2& a, float2 m, float2 y) { cfmaf(a, m, y); }

// ----------------------------------------------------------- plan structs --
struct Strip {          // GEMV work: blocks (i, j0 .. j0+nb-1) of cluster sys
    int sys, i, nb, pad;
    long long p0;       // first pair index (cluster-local)
};
struct Item {           // vector / reduce work: rows [r0, r0+nr) of cluster sys
    int sys, r0, nr, pad;
};
struct SysPlan {        // per-cluster plan data (device)
    long long strip_row_base;   // index into row_strip (first block row of this cluster)
    long long strip_base;       // global index of the first strip of this cluster
    long long cw_off;           // element offset of this cluster's per-pair column partials
    long long cu_off;           // element offset of this cluster's per-strip row partials
    int item_begin, item_end;
};

struct KState {         // per (cluster, rhs) BiCGSTAB scalars
    double2 rho, alpha, omega, beta;
    double r0sq, bsq, rsq, tol2;
    int iters, restarts, done, status;
    int need_restart, maxiter, pad0, pad1;
};

enum { ST_RUNNING = -1 };

// ------------------------------------------------------------ y vectors --
// Yu[k][r][rr] = eps(r) t_k[rho(r)] x_k[rho(r)][rr],  Yw = sig(r) Yu, for all
// particles k of all clusters (thread per row).
template <typename VT, int R>
__global__ void k_yprep(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems,
                        const KState* __restrict__ st, int mask_mode, const double2* __restrict__ tvec,
                        const VT* __restrict__ x, VT* __restrict__ Yu, VT* __restrict__ Yw) {
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    if (mask_mode >= 0) {   // skip clusters whose every rhs is finished (or not restarting)
        bool any = false;
        for (int rr = 0; rr < R; rr++) {
            const KState& k = st[I.sys * R + rr];
            any |= (mask_mode == 0) ? (!k.done && !k.need_restart) : (k.need_restart != 0);
        }
        if (!any) return;
    }
    const int lr = threadIdx.x;
    if (lr >= I.nr) return;
    const int row = I.r0 + lr;
    const int part = row / S.B, R_ = row % S.B;
    const int info = __ldg(S.rowinfo + R_);
    const int rho = info & ((1 << 29) - 1);
    const unsigned eneg = (info >> 29) & 1, sneg = (info >> 30) & 1;
    const long long src = (long long)part * S.B + rho;
    const double2 t = tvec[S.t_off + src];
    for (int rr = 0; rr < R; rr++) {
        double2 xv = to_d2(x[(S.vec_off + src * R) + rr]);
        double2 z = cmul(t, xv);
        double2 yu = make_double2(flipd(z.x, eneg), flipd(z.y, eneg));
        double2 yw = make_double2(flipd(yu.x, sneg), flipd(yu.y, sneg));
        Yu[(S.vec_off + (long long)row * R) + rr] = from_d2<VT>(yu);
        Yw[(S.vec_off + (long long)row * R) + rr] = from_d2<VT>(yw);
    }
}

// --------------------------------------------------------------- K3a GEMV --
// MT: matrix element (double2 | float2), AT: accumulator scalar (double | float).
// CPG: complex elements per 16-byte load (1 for c128, 2 for c64). NG: column
// groups per lane.
template <typename MT, typename AT, int R, int NG>
__global__ void __launch_bounds__(kGemvThreads)
k_pgemv(const gb::SysDev* __restrict__ sys, const Strip* __restrict__ strips, long long nstrips,
        const KState* __restrict__ st, int mask_mode, const MT* __restrict__ mat,
        const typename Cplx<AT>::t* __restrict__ Yu, const typename Cplx<AT>::t* __restrict__ Yw,
        typename Cplx<AT>::t* __restrict__ CU, typename Cplx<AT>::t* __restrict__ CW,
        const SysPlan* __restrict__ plan) {
    using AC = typename Cplx<AT>::t;
    constexpr int CPG = 16 / sizeof(MT);
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * kGemvThreads + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * kGemvThreads) >> 5;
    for (long long w = warp; w < nstrips; w += nwarps) {
        const Strip sp = strips[w];
        const gb::SysDev S = sys[sp.sys];
        if (mask_mode >= 0) {
            bool any = false;
            for (int rr = 0; rr < R; rr++) {
                const KState& k = st[sp.sys * R + rr];
                any |= (mask_mode == 0) ? (!k.done && !k.need_restart) : (k.need_restart != 0);
            }
            if (!any) continue;
        }
        const int B = S.B;
        const int ncg = B / CPG;     // column groups in a row
        AC cu[NG][CPG][R];
#pragma unroll
        for (int g = 0; g < NG; g++)
#pragma unroll
            for (int c = 0; c < CPG; c++)
#pragma unroll
                for (int rr = 0; rr < R; rr++) cu[g][c][rr] = AC{0, 0};
        const AC* yw_i = Yw + S.vec_off + (long long)sp.i * B * R;
        for (int b = 0; b < sp.nb; b++) {
            const long long p = sp.p0 + b;
            const int j = sp.i + 1 + (int)(p - pair_start(sp.i, S.N));
            const AC* yu_j = Yu + S.vec_off + (long long)j * B * R;
            const MT* blk = mat + S.mat_off + p * (long long)B * B;
            AC cw[NG][CPG][R];
#pragma unroll
            for (int g = 0; g < NG; g++)
#pragma unroll
                for (int c = 0; c < CPG; c++)
#pragma unroll
                    for (int rr = 0; rr < R; rr++) cw[g][c][rr] = AC{0, 0};
            constexpr int RU = 4;   // rows in flight per lane
            int r = 0;
            for (; r + RU <= B; r += RU) {
                uint4 q[RU][NG];
#pragma unroll
                for (int u = 0; u < RU; u++)
#pragma unroll
                    for (int g = 0; g < NG; g++) {
                        const int cg = lane + 32 * g;
                        q[u][g] = (cg < ncg) ? __ldg(reinterpret_cast<const uint4*>(blk + (long long)(r + u) * B) + cg)
                                             : make_uint4(0, 0, 0, 0);
                    }
#pragma unroll
                for (int u = 0; u < RU; u++) {
                    AC yu[R], yw[R];
#pragma unroll
                    for (int rr = 0; rr < R; rr++) {
                        yu[rr] = yu_j[(r + u) * R + rr];
                        yw[rr] = yw_i[(r + u) * R + rr];
                    }
#pragma unroll
                    for (int g = 0; g < NG; g++) {
                        const MT* m = reinterpret_cast<const MT*>(&q[u][g]);
#pragma unroll
                        for (int c = 0; c < CPG; c++) {
                            AC mv = AC{(AT)m[c].x, (AT)m[c].y};
#pragma unroll
                            for (int rr = 0; rr < R; rr++) {
                                acc_fma(cu[g][c][rr], mv, yu[rr]);
                                acc_fma(cw[g][c][rr], mv, yw[rr]);
                            }
                        }
                    }
                }
            }
            for (; r < B; r++) {
                AC yu[R], yw[R];
#pragma unroll
                for (int rr = 0; rr < R; rr++) {
                    yu[rr] = yu_j[r * R + rr];
                    yw[rr] = yw_i[r * R + rr];
                }
#pragma unroll
                for (int g = 0; g < NG; g++) {
                    const int cg = lane + 32 * g;
                    if (cg >= ncg) continue;
                    uint4 qq = __ldg(reinterpret_cast<const uint4*>(blk + (long long)r * B) + cg);
                    const MT* m = reinterpret_cast<const MT*>(&qq);
#pragma unroll
                    for (int c = 0; c < CPG; c++) {
                        AC mv = AC{(AT)m[c].x, (AT)m[c].y};
#pragma unroll
                        for (int rr = 0; rr < R; rr++) {
                            acc_fma(cu[g][c][rr], mv, yu[rr]);
                            acc_fma(cw[g][c][rr], mv, yw[rr]);
                        }
                    }
                }
            }
            // column partial of this block for block row j: CW[pair][col][rr]
            AC* cwp = CW + plan[sp.sys].cw_off + p * (long long)B * R;
#pragma unroll
            for (int g = 0; g < NG; g++) {
                const int cg = lane + 32 * g;
                if (cg >= ncg) continue;
#pragma unroll
                for (int c = 0; c < CPG; c++)
#pragma unroll
                    for (int rr = 0; rr < R; rr++) cwp[(cg * CPG + c) * R + rr] = cw[g][c][rr];
            }
        }
        AC* cup = CU + plan[sp.sys].cu_off + (w - plan[sp.sys].strip_base) * (long long)B * R;
#pragma unroll
        for (int g = 0; g < NG; g++) {
            const int cg = lane + 32 * g;
            if (cg >= ncg) continue;
#pragma unroll
            for (int c = 0; c < CPG; c++)
#pragma unroll
                for (int rr = 0; rr < R; rr++) cup[(cg * CPG + c) * R + rr] = cu[g][c][rr];
        }
    }
}

// ----------------------------------------------------- dense GEMV (plugin) --
// Tx = T x for a caller-supplied dense D x D complex128 matrix; warp per row.
template <int R>
__global__ void __launch_bounds__(256)
k_dense_gemv(int D, const double2* __restrict__ T, const double2* __restrict__ x, double2* __restrict__ Tx,
             const KState* __restrict__ st) {
    bool any = false;
    for (int rr = 0; rr < R; rr++) any |= (!st[rr].done && !st[rr].need_restart) || st[rr].need_restart;
    if (!any) return;
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long row = warp; row < D; row += nw) {
        double2 acc[R];
#pragma unroll
        for (int rr = 0; rr < R; rr++) acc[rr] = make_double2(0, 0);
        const double2* Tr = T + row * (long long)D;
        for (int c = lane; c < D; c += 32) {
            const double2 m = __ldg(Tr + c);
#pragma unroll
            for (int rr = 0; rr < R; rr++) cfma(acc[rr], m, x[(long long)c * R + rr]);
        }
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            for (int o = 16; o > 0; o >>= 1) {
                acc[rr].x += __shfl_xor_sync(0xffffffffu, acc[rr].x, o);
                acc[rr].y += __shfl_xor_sync(0xffffffffu, acc[rr].y, o);
            }
            if (lane == 0) Tx[row * R + rr] = acc[rr];
        }
    }
}

// --------------------------------------------------------------- K3b reduce --
// y = x + T x (row-wise from the partials, or from a dense Tx), plus per-item dot
// partials: mode 1 -> d0 = <r0, y>;  mode 2 -> d0 = |y|^2, d1 = <y, s>;
// mode 3 -> d0 = |b - y|^2 with y := b - y (restart residual).
template <typename AT, typename VT, int R, bool DENSE>
__global__ void __launch_bounds__(kItemRows)
k_reduce(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems,
         const SysPlan* __restrict__ plan, const long long* __restrict__ row_strip,
         const KState* __restrict__ st, int mask_mode,
         const typename Cplx<AT>::t* __restrict__ CU, const typename Cplx<AT>::t* __restrict__ CW,
         const double2* __restrict__ Tx_dense, const VT* __restrict__ x, VT* __restrict__ y, int mode,
         const VT* __restrict__ aux, const double2* __restrict__ b128, double2* __restrict__ dots) {
    using AC = typename Cplx<AT>::t;
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    bool act[R];
    bool any = false;
    for (int rr = 0; rr < R; rr++) {
        const KState& k = st[I.sys * R + rr];
        act[rr] = (mask_mode == 0) ? (!k.done && !k.need_restart) : (k.need_restart != 0);
        if (mask_mode < 0) act[rr] = true;
        any |= act[rr];
    }
    if (!any) return;
    __shared__ double2 red[kItemRows / 32][R][2];
    const int lr = threadIdx.x;
    double2 d0[R], d1[R];
    for (int rr = 0; rr < R; rr++) d0[rr] = d1[rr] = make_double2(0, 0);
    if (lr < I.nr) {
        const int row = I.r0 + lr;
        const int B = S.B;
        const int k = row / B, R_ = row % B;
        double2 tx[R];
        if (DENSE) {
            for (int rr = 0; rr < R; rr++) tx[rr] = Tx_dense[(long long)row * R + rr];
        } else {
            const int info = __ldg(S.rowinfo + R_);
            const int rho = info & ((1 << 29) - 1);
            const unsigned eneg = (info >> 29) & 1, sneg = (info >> 30) & 1;
            AC su[R], sw[R];
            for (int rr = 0; rr < R; rr++) su[rr] = sw[rr] = AC{0, 0};
            const SysPlan pl = plan[I.sys];
            const long long s0 = row_strip[pl.strip_row_base + k], s1 = row_strip[pl.strip_row_base + k + 1];
            for (long long q = s0; q < s1; q++)
                for (int rr = 0; rr < R; rr++) {
                    AC v = CU[pl.cu_off + ((q - pl.strip_base) * B + rho) * R + rr];
                    su[rr].x += v.x;
                    su[rr].y += v.y;
                }
            for (int i = 0; i < k; i++) {
                const long long pr = pair_start(i, S.N) + (k - i - 1);
                for (int rr = 0; rr < R; rr++) {
                    AC v = CW[pl.cw_off + (pr * B + rho) * R + rr];
                    sw[rr].x += v.x;
                    sw[rr].y += v.y;
                }
            }
            for (int rr = 0; rr < R; rr++) {
                double2 a = make_double2((double)su[rr].x, (double)su[rr].y);
                double2 c = make_double2((double)sw[rr].x, (double)sw[rr].y);
                a = make_double2(flipd(a.x, eneg), flipd(a.y, eneg));
                c = make_double2(flipd(c.x, eneg ^ sneg), flipd(c.y, eneg ^ sneg));
                tx[rr] = make_double2(a.x + c.x, a.y + c.y);
            }
        }
        const long long vo = S.vec_off + (long long)row * R;
        for (int rr = 0; rr < R; rr++) {
            if (!act[rr]) continue;
            const double2 xv = to_d2(x[vo + rr]);
            double2 yv = make_double2(xv.x + tx[rr].x, xv.y + tx[rr].y);
            if (mode == 3) {
                const double2 bv = b128 ? b128[vo + rr] : to_d2(aux[vo + rr]);
                yv = make_double2(bv.x - yv.x, bv.y - yv.y);
                d0[rr].x += yv.x * yv.x + yv.y * yv.y;
            }
            const VT yo = from_d2<VT>(yv);
            y[vo + rr] = yo;
            const double2 yq = to_d2(yo);   // dots of the stored (rounded) vector
            if (mode == 1) {
                const double2 r0 = to_d2(aux[vo + rr]);
                cfma_conj(d0[rr], r0, yq);
            } else if (mode == 2) {
                const double2 sv = to_d2(aux[vo + rr]);
                d0[rr].x += yq.x * yq.x + yq.y * yq.y;
                cfma_conj(d1[rr], yq, sv);
            }
        }
    }
    if (mode == 0) return;
    // block reduction in a fixed order
    const int lane = lr & 31, wid = lr >> 5;
    for (int rr = 0; rr < R; rr++) {
        for (int o = 16; o > 0; o >>= 1) {
            d0[rr].x += __shfl_xor_sync(0xffffffffu, d0[rr].x, o);
            d0[rr].y += __shfl_xor_sync(0xffffffffu, d0[rr].y, o);
            d1[rr].x += __shfl_xor_sync(0xffffffffu, d1[rr].x, o);
            d1[rr].y += __shfl_xor_sync(0xffffffffu, d1[rr].y, o);
        }
        if (lane == 0) {
            red[wid][rr][0] = d0[rr];
            red[wid][rr][1] = d1[rr];
        }
    }
    __syncthreads();
    if (lr < R * 2) {
        const int rr = lr >> 1, which = lr & 1;
        double2 s = make_double2(0, 0);
        for (int w = 0; w < kItemRows / 32; w++) {
            s.x += red[w][rr][which].x;
            s.y += red[w][rr][which].y;
        }
        dots[((long long)it * R + rr) * 2 + which] = s;
    }
}

// ------------------------------------------------------- K4 vector updates --
// kind 0: init      x = 0, r = r0 = b, p = v = 0;     dots: |b|^2
// kind 1: p-update  p = r + beta (p - omega v)
// kind 2: s-update  s = r - alpha v
// kind 3: x/r       x += alpha p + omega s; r = s - omega t;  dots: |r|^2, <r0, r>
// kind 4: restart   r0 = r (r already b - A x);  dots: none (|r|^2 from reduce)
template <typename VT, int R>
__global__ void __launch_bounds__(kItemRows)
k_vec(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems, const KState* __restrict__ st,
      int kind, const double2* __restrict__ b, VT* __restrict__ bx, VT* __restrict__ x, VT* __restrict__ r,
      VT* __restrict__ r0, VT* __restrict__ p, VT* __restrict__ v, VT* __restrict__ s, const VT* __restrict__ t,
      double2* __restrict__ dots) {
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    bool act[R];
    bool any = false;
    for (int rr = 0; rr < R; rr++) {
        const KState& k = st[I.sys * R + rr];
        act[rr] = (kind == 0) ? true : (kind == 4 ? (k.need_restart != 0) : (!k.done && !k.need_restart));
        any |= act[rr];
    }
    if (!any) return;
    __shared__ double2 red[kItemRows / 32][R][2];
    const int lr = threadIdx.x;
    double2 d0[R], d1[R];
    for (int rr = 0; rr < R; rr++) d0[rr] = d1[rr] = make_double2(0, 0);
    if (lr < I.nr) {
        const long long vo = S.vec_off + (long long)(I.r0 + lr) * R;
        for (int rr = 0; rr < R; rr++) {
            if (!act[rr]) continue;
            const long long e = vo + rr;
            const KState& k = st[I.sys * R + rr];
            if (kind == 0) {
                const double2 bv = b ? b[e] : to_d2(bx[e]);
                const VT bq = from_d2<VT>(bv);
                const VT z = from_d2<VT>(make_double2(0, 0));
                x[e] = z; p[e] = z; v[e] = z;
                r[e] = bq; r0[e] = bq;
                if (bx && b) bx[e] = bq;
                const double2 bd = to_d2(bq);
                d0[rr].x += bd.x * bd.x + bd.y * bd.y;
            } else if (kind == 1) {
                const double2 rv = to_d2(r[e]), pv = to_d2(p[e]), vv = to_d2(v[e]);
                const double2 tmp = make_double2(pv.x - (k.omega.x * vv.x - k.omega.y * vv.y),
                                                 pv.y - (k.omega.x * vv.y + k.omega.y * vv.x));
                const double2 bt = cmul(k.beta, tmp);
                p[e] = from_d2<VT>(make_double2(rv.x + bt.x, rv.y + bt.y));
            } else if (kind == 2) {
                const double2 rv = to_d2(r[e]), vv = to_d2(v[e]);
                const double2 av = cmul(k.alpha, vv);
                s[e] = from_d2<VT>(make_double2(rv.x - av.x, rv.y - av.y));
            } else if (kind == 3) {
                const double2 pv = to_d2(p[e]), sv = to_d2(s[e]), tv = to_d2(t[e]), xv = to_d2(x[e]);
                const double2 ap = cmul(k.alpha, pv), ws = cmul(k.omega, sv), wt = cmul(k.omega, tv);
                x[e] = from_d2<VT>(make_double2(xv.x + ap.x + ws.x, xv.y + ap.y + ws.y));
                const VT rq = from_d2<VT>(make_double2(sv.x - wt.x, sv.y - wt.y));
                r[e] = rq;
                const double2 rd = to_d2(rq), r0v = to_d2(r0[e]);
                d0[rr].x += rd.x * rd.x + rd.y * rd.y;
                cfma_conj(d1[rr], r0v, rd);
            } else if (kind == 4) {
                r0[e] = r[e];
            }
        }
    }
    if (kind == 1 || kind == 2 || kind == 4) return;
    const int lane = lr & 31, wid = lr >> 5;
    for (int rr = 0; rr < R; rr++) {
        for (int o = 16; o > 0; o >>= 1) {
            d0[rr].x += __shfl_xor_sync(0xffffffffu, d0[rr].x, o);
            d0[rr].y += __shfl_xor_sync(0xffffffffu, d0[rr].y, o);
            d1[rr].x += __shfl_xor_sync(0xffffffffu, d1[rr].x, o);
            d1[rr].y += __shfl_xor_sync(0xffffffffu, d1[rr].y, o);
        }
        if (lane == 0) {
            red[wid][rr][0] = d0[rr];
            red[wid][rr][1] = d1[rr];
        }
    }
    __syncthreads();
    if (lr < R * 2) {
        const int rr = lr >> 1, which = lr & 1;
        double2 sm = make_double2(0, 0);
        for (int w = 0; w < kItemRows / 32; w++) {
            sm.x += red[w][rr][which].x;
            sm.y += red[w][rr][which].y;
        }
        dots[((long long)it * R + rr) * 2 + which] = sm;
    }
}

// ------------------------------------------------------------ K4 scalars --
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    const double den = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}
__device__ __forceinline__ bool finite2(double2 a) { return isfinite(a.x) && isfinite(a.y); }

// phase 0: init (bsq from dots d0; tol); 1: alpha = rho/<r0,v>; 2: omega = <t,s>/|t|^2;
// 3: end of iteration (convergence, restart test, beta); 4: restart finished
// (dots d0 = |r|^2 of the new residual).
template <int R>
__global__ void k_scalar(const SysPlan* __restrict__ plan, int nsys, KState* __restrict__ st, int phase,
                         const double2* __restrict__ dots, double tol, int maxiter) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nsys * R) return;
    const int sidx = id / R, rr = id % R;
    KState& k = st[id];
    const SysPlan pl = plan[sidx];
    double2 d0 = make_double2(0, 0), d1 = make_double2(0, 0);
    for (int it = pl.item_begin; it < pl.item_end; it++) {
        const double2 a = dots[((long long)it * R + rr) * 2 + 0];
        const double2 c = dots[((long long)it * R + rr) * 2 + 1];
        d0.x += a.x; d0.y += a.y;
        d1.x += c.x; d1.y += c.y;
    }
    const double eps = 2.220446049250313e-16;
    if (phase == 0) {
        k.bsq = d0.x;
        k.r0sq = d0.x;
        k.rsq = d0.x;
        k.tol2 = tol * tol * d0.x;
        k.rho = k.alpha = k.omega = make_double2(1, 0);
        k.iters = 0;
        k.restarts = 0;
        k.need_restart = 0;
        k.maxiter = maxiter;
        if (d0.x == 0.0 || !(k.rsq > k.tol2) || maxiter <= 0) {
            k.done = 1;
            k.status = GB_OK;
        } else {
            k.done = 0;
            k.status = ST_RUNNING;
            // loop top of the first iteration: rho = <r0, r> = |b|^2
            const double2 rho_old = k.rho;
            k.rho = make_double2(d0.x, 0.0);
            k.beta = cmul(cdiv(k.rho, rho_old), cdiv(k.alpha, k.omega));
        }
        return;
    }
    if (phase == 4) {
        if (!k.need_restart) return;
        // Eigen: r = b - A x; r0 = r; rho = r0_sqnorm = |r|^2; first restart resets i
        k.need_restart = 0;
        k.rsq = d0.x;
        k.r0sq = d0.x;
        const double2 rho_old = k.rho;
        k.rho = make_double2(d0.x, 0.0);
        if (k.restarts++ == 0) k.iters = 0;
        if (!(k.rsq > k.tol2)) {   // converged exactly at the restart point
            k.done = 1;
            k.status = GB_OK;
            return;
        }
        k.beta = cmul(cdiv(k.rho, rho_old), cdiv(k.alpha, k.omega));
        if (!finite2(k.beta)) { k.done = 1; k.status = GB_BREAKDOWN; }
        return;
    }
    if (k.done || k.need_restart) return;
    if (phase == 1) {
        k.alpha = cdiv(k.rho, d0);
        if (!finite2(k.alpha)) { k.done = 1; k.status = (d0.x == 0 && d0.y == 0) ? GB_BREAKDOWN : GB_NAN; }
    } else if (phase == 2) {
        const double tt = d0.x;
        k.omega = (tt > 0.0) ? make_double2(d1.x / tt, d1.y / tt) : make_double2(0, 0);
        if (!finite2(k.omega)) { k.done = 1; k.status = GB_NAN; }
    } else if (phase == 3) {
        k.iters += 1;
        k.rsq = d0.x;
        if (!isfinite(k.rsq)) { k.done = 1; k.status = GB_NAN; return; }
        if (!(k.rsq > k.tol2)) { k.done = 1; k.status = GB_OK; return; }
        if (k.iters >= k.maxiter) { k.done = 1; k.status = GB_NOT_CONVERGED; return; }
        const double2 rho_old = k.rho;
        k.rho = d1;   // <r0, r>
        if (sqrt(k.rho.x * k.rho.x + k.rho.y * k.rho.y) < eps * eps * k.r0sq) {
            if (k.restarts > 8) { k.done = 1; k.status = GB_BREAKDOWN; return; }
            k.rho = rho_old;   // phase 4 recomputes rho from the fresh residual
            k.need_restart = 1;
            return;
        }
        k.beta = cmul(cdiv(k.rho, rho_old), cdiv(k.alpha, k.omega));
        if (!finite2(k.beta)) { k.done = 1; k.status = GB_NAN; }
    }
}

// ------------------------------------------------------ refinement helpers --
// x128 += d (FP32 correction); r32 = rounded FP64 residual
template <int R>
__global__ void k_refine_axpy(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems,
                              const KState* __restrict__ ost, double2* __restrict__ x128, const float2* __restrict__ d) {
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    const int lr = threadIdx.x;
    if (lr >= I.nr) return;
    const long long vo = S.vec_off + (long long)(I.r0 + lr) * R;
    for (int rr = 0; rr < R; rr++) {
        if (ost[I.sys * R + rr].done) continue;
        const float2 dv = d[vo + rr];
        double2 xv = x128[vo + rr];
        xv.x += (double)dv.x;
        xv.y += (double)dv.y;
        x128[vo + rr] = xv;
    }
}

// outer (refinement) state update from |r|^2 partials: done when |r|^2 <= tol^2 |b|^2
template <int R>
__global__ void k_refine_check(const SysPlan* __restrict__ plan, int nsys, KState* __restrict__ ost,
                               const double2* __restrict__ dots, int pass, int max_refine) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nsys * R) return;
    const int sidx = id / R, rr = id % R;
    KState& k = ost[id];
    if (k.done) return;
    const SysPlan pl = plan[sidx];
    double s = 0;
    for (int it = pl.item_begin; it < pl.item_end; it++) s += dots[((long long)it * R + rr) * 2].x;
    k.rsq = s;
    k.iters = pass;
    if (!isfinite(s)) { k.done = 1; k.status = GB_NAN; return; }
    if (!(s > k.tol2)) { k.done = 1; k.status = GB_OK; return; }
    if (pass > max_refine) { k.done = 1; k.status = GB_NOT_CONVERGED; }
}

// |b|^2 per (cluster, rhs) for the outer state
template <int R>
__global__ void k_outer_init(const SysPlan* __restrict__ plan, int nsys, KState* __restrict__ ost,
                             const double2* __restrict__ dots, double tol) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nsys * R) return;
    const int sidx = id / R, rr = id % R;
    const SysPlan pl = plan[sidx];
    double s = 0;
    for (int it = pl.item_begin; it < pl.item_end; it++) s += dots[((long long)it * R + rr) * 2].x;
    KState& k = ost[id];
    memset(&k, 0, sizeof(KState));
    k.bsq = s;
    k.tol2 = tol * tol * s;
    k.rsq = s;
    k.done = (s == 0.0) ? 1 : 0;
    k.status = k.done ? GB_OK : ST_RUNNING;
}

// r (FP64) = b;  x (FP64) = 0;  |b|^2 partials
template <int R>
__global__ void k_outer_start(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems,
                              const double2* __restrict__ b, double2* __restrict__ x, double2* __restrict__ dots) {
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    __shared__ double red[kItemRows / 32][R];
    const int lr = threadIdx.x;
    double d[R];
    for (int rr = 0; rr < R; rr++) d[rr] = 0;
    if (lr < I.nr) {
        const long long vo = S.vec_off + (long long)(I.r0 + lr) * R;
        for (int rr = 0; rr < R; rr++) {
            const double2 bv = b[vo + rr];
            x[vo + rr] = make_double2(0, 0);
            d[rr] = bv.x * bv.x + bv.y * bv.y;
        }
    }
    const int lane = lr & 31, wid = lr >> 5;
    for (int rr = 0; rr < R; rr++) {
        for (int o = 16; o > 0; o >>= 1) d[rr] += __shfl_xor_sync(0xffffffffu, d[rr], o);
        if (lane == 0) red[wid][rr] = d[rr];
    }
    __syncthreads();
    if (lr < R) {
        double s = 0;
        for (int w = 0; w < kItemRows / 32; w++) s += red[w][lr];
        dots[((long long)it * R + lr) * 2] = make_double2(s, 0);
        dots[((long long)it * R + lr) * 2 + 1] = make_double2(0, 0);
    }
}

// ================================================================== host ==
struct Plan {
    int nsys = 0, R = 1, nitems = 0;
    long long nstrips = 0, total_pairs = 0, total_rows = 0, total_vec = 0, max_B = 0;
    long long cw_elems = 0, cu_elems = 0;
    std::vector<gb::SysDev> sd;
    std::vector<Strip> strips;
    std::vector<Item> items;
    std::vector<SysPlan> sp;
    std::vector<long long> row_strip;
    int ng128 = 1, ng64 = 1;
};

int build_plan(int nsys, const gb_system* sys, int R, cudaStream_t stream, Plan& P) {
    P.nsys = nsys;
    P.R = R;
    int st = gb::make_sysdev(nsys, sys, stream, P.sd);
    if (st) return st;
    long long pairs = 0;
    for (auto& d : P.sd) pairs += d.P;
    P.total_pairs = pairs;
    const long long warps = (long long)gb::sm_count() * 32;
    const long long J = std::max<long long>(1, std::min<long long>(16, pairs / std::max<long long>(1, 4 * warps)));
    P.sp.resize(nsys);
    long long cw_off = 0, cu_off = 0;
    for (int s = 0; s < nsys; s++) {
        const gb::SysDev& d = P.sd[s];
        SysPlan& pl = P.sp[s];
        pl.strip_row_base = (long long)P.row_strip.size();
        pl.strip_base = (long long)P.strips.size();
        pl.cw_off = cw_off;
        pl.cu_off = cu_off;
        for (int i = 0; i < d.N; i++) {
            P.row_strip.push_back((long long)P.strips.size());
            const long long p0 = pair_start(i, d.N);
            const long long nb = d.N - 1 - i;
            for (long long b = 0; b < nb; b += J) {
                Strip sp_;
                sp_.sys = s;
                sp_.i = i;
                sp_.nb = (int)std::min<long long>(J, nb - b);
                sp_.pad = 0;
                sp_.p0 = p0 + b;
                P.strips.push_back(sp_);
            }
        }
        P.row_strip.push_back((long long)P.strips.size());
        cw_off += d.P * d.B * R;
        cu_off += ((long long)P.strips.size() - pl.strip_base) * d.B * R;
        pl.item_begin = (int)P.items.size();
        for (int r0 = 0; r0 < d.D; r0 += kItemRows) P.items.push_back(Item{s, r0, std::min(kItemRows, d.D - r0), 0});
        pl.item_end = (int)P.items.size();
        P.total_rows += d.D;
        P.total_vec = std::max<long long>(P.total_vec, d.vec_off + (long long)d.D * R);
        P.max_B = std::max<long long>(P.max_B, d.B);
    }
    P.nstrips = (long long)P.strips.size();
    P.nitems = (int)P.items.size();
    P.cw_elems = cw_off;
    P.cu_elems = cu_off;
    P.ng128 = (int)((P.max_B + 31) / 32);
    P.ng64 = (int)((P.max_B / 2 + 31) / 32);
    return GB_OK;
}

// workspace layout
struct WS {
    size_t off_state, off_ostate, off_dots, off_cu, off_cw, off_yu, off_yw, off_vec, off_tx, off_x128r, off_blob, total;
    int nvec;
};

WS ws_layout(const Plan& P, int prec, bool dense) {
    WS w;
    const int R = P.R;
    const size_t vsz = (prec == GB_PREC_FP64) ? sizeof(double2) : sizeof(float2);
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t r = o; o += (bytes + 255) & ~size_t(255); return r; };
    w.off_state = take(sizeof(KState) * P.nsys * R);
    w.off_ostate = take(sizeof(KState) * P.nsys * R);
    w.off_dots = take(sizeof(double2) * 2 * (size_t)std::max(P.nitems, 1) * R);
    if (!dense) {
        // partials in the accumulator type of the matrix pass (FP64 refinement passes need double)
        const size_t asz = sizeof(double2);
        w.off_cu = take(asz * (size_t)std::max<long long>(P.cu_elems, 1));
        w.off_cw = take(asz * (size_t)std::max<long long>(P.cw_elems, 1));
        w.off_yu = take(sizeof(double2) * (size_t)P.total_vec);
        w.off_yw = take(sizeof(double2) * (size_t)P.total_vec);
        w.off_tx = take(0);
    } else {
        w.off_cu = w.off_cw = w.off_yu = w.off_yw = take(0);
        w.off_tx = take(sizeof(double2) * (size_t)P.total_vec);
    }
    // Krylov vectors: r, r0, p, v, s, t (+ x, b copies in reduced precision)
    w.nvec = 8;
    w.off_vec = take(vsz * (size_t)P.total_vec * w.nvec);
    // FP64 residual for refinement
    w.off_x128r = take(prec == GB_PREC_MIXED ? sizeof(double2) * (size_t)P.total_vec : 0);
    // device copies of the plan
    w.off_blob = take(sizeof(gb::SysDev) * P.nsys + sizeof(Strip) * P.nstrips + sizeof(Item) * P.nitems +
                      sizeof(SysPlan) * P.nsys + sizeof(long long) * P.row_strip.size() + 64);
    w.total = o;
    return w;
}

struct DevPlan {
    const gb::SysDev* sys;
    const Strip* strips;
    const Item* items;
    const SysPlan* sp;
    const long long* row_strip;
};

int upload_plan(const Plan& P, unsigned char* base, const WS& w, cudaStream_t stream, DevPlan& D) {
    std::vector<unsigned char> blob;
    auto put = [&](const void* src, size_t bytes) {
        size_t off = blob.size();
        blob.resize(off + ((bytes + 15) & ~size_t(15)));
        if (bytes) memcpy(blob.data() + off, src, bytes);
        return off;
    };
    size_t o_sys = put(P.sd.data(), sizeof(gb::SysDev) * P.nsys);
    size_t o_str = put(P.strips.data(), sizeof(Strip) * P.nstrips);
    size_t o_it = put(P.items.data(), sizeof(Item) * P.nitems);
    size_t o_sp = put(P.sp.data(), sizeof(SysPlan) * P.nsys);
    size_t o_rs = put(P.row_strip.data(), sizeof(long long) * P.row_strip.size());
    unsigned char* dst = base + w.off_blob;
    GB_CUDA_TRY(cudaMemcpyAsync(dst, blob.data(), blob.size(), cudaMemcpyHostToDevice, stream));
    // the host blob dies at return: wait for the (pageable) copy
    GB_CUDA_TRY(cudaStreamSynchronize(stream));
    D.sys = reinterpret_cast<const gb::SysDev*>(dst + o_sys);
    D.strips = reinterpret_cast<const Strip*>(dst + o_str);
    D.items = reinterpret_cast<const Item*>(dst + o_it);
    D.sp = reinterpret_cast<const SysPlan*>(dst + o_sp);
    D.row_strip = reinterpret_cast<const long long*>(dst + o_rs);
    return GB_OK;
}

// launch the packed product partials + reduce for vector xin -> yout
template <typename MT, typename AT, typename VT, int R>
int launch_apply(const Plan& P, const DevPlan& D, const WS& w, unsigned char* base, const KState* st, int mask_mode,
                 const MT* mat, const double2* tvec, const VT* xin, VT* yout, int mode, const VT* aux,
                 const double2* b128, double2* dots, cudaStream_t stream) {
    using AC = typename Cplx<AT>::t;
    AC* Yu = reinterpret_cast<AC*>(base + w.off_yu);
    AC* Yw = reinterpret_cast<AC*>(base + w.off_yw);
    AC* CU = reinterpret_cast<AC*>(base + w.off_cu);
    AC* CW = reinterpret_cast<AC*>(base + w.off_cw);
    k_yprep<AC, R><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, st, mask_mode, tvec,
                                                       reinterpret_cast<const AC*>(xin), Yu, Yw);
    // Yu/Yw must be in the accumulator type: when VT differs (FP32 vectors with a c128
    // pass do not occur), xin is already AC.
    if (P.nstrips > 0) {
        constexpr int CPG = 16 / sizeof(MT);
        const int ng = (int)((P.max_B / CPG + 31) / 32);
        const long long warps_needed = P.nstrips;
        int per_sm = 2;
        long long grid = std::min<long long>((warps_needed * 32 + kGemvThreads - 1) / kGemvThreads,
                                             (long long)gb::sm_count() * 8);
        (void)per_sm;
        if (grid < 1) grid = 1;
        switch (ng) {
#define GB_NG_CASE(NGV)                                                                                         \
    case NGV:                                                                                                   \
        k_pgemv<MT, AT, R, NGV><<<(unsigned)grid, kGemvThreads, 0, stream>>>(D.sys, D.strips, P.nstrips, st,   \
                                                                              mask_mode, mat, Yu, Yw, CU, CW, D.sp); \
        break;
            GB_NG_CASE(1) GB_NG_CASE(2) GB_NG_CASE(3) GB_NG_CASE(4) GB_NG_CASE(5) GB_NG_CASE(6) GB_NG_CASE(7)
            GB_NG_CASE(8)
#undef GB_NG_CASE
            default: return gb_set_error(GB_UNSUPPORTED, "block size %lld too large", P.max_B);
        }
        GB_CUDA_TRY(cudaGetLastError());
    }
    k_reduce<AT, VT, R, false><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, D.sp, D.row_strip, st,
                                                                   mask_mode, CU, CW, nullptr, xin, yout, mode, aux,
                                                                   b128, dots);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

// ------------------------------------------------------------- BiCGSTAB run --
// Runs BiCGSTAB on vectors of type VT with the packed matrix of type MT until
// every (cluster, rhs) is done.  bsrc: right-hand side (FP64, or VT when b128 is
// null and bvt given).  The solution lands in the x vector of the workspace.
template <typename MT, typename AT, typename VT, int R, bool DENSE>
int run_bicgstab(const Plan& P, const DevPlan& D, const WS& w, unsigned char* base, const MT* mat,
                 const double2* tvec, const double2* b128, VT* bvt, double tol, int maxiter, KState* st,
                 int dense_D, cudaStream_t stream, int* host_status_buf) {
    const size_t TV = (size_t)P.total_vec;
    VT* V = reinterpret_cast<VT*>(base + w.off_vec);
    VT *x = V, *r = V + TV, *r0 = V + 2 * TV, *p = V + 3 * TV, *v = V + 4 * TV, *s = V + 5 * TV, *t = V + 6 * TV,
       *bx = V + 7 * TV;
    double2* dots = reinterpret_cast<double2*>(base + w.off_dots);
    double2* Tx = reinterpret_cast<double2*>(base + w.off_tx);
    const int nsr = P.nsys * R;
    const int sblocks = (nsr + 127) / 128;

    auto apply = [&](const VT* xin, VT* yout, int mode, const VT* aux, int mask, const double2* bb) -> int {
        if (DENSE) {
            const long long grid = std::min<long long>(((long long)dense_D * 32 + 255) / 256, (long long)gb::sm_count() * 8);
            k_dense_gemv<R><<<(unsigned)std::max<long long>(grid, 1), 256, 0, stream>>>(
                dense_D, reinterpret_cast<const double2*>(mat), reinterpret_cast<const double2*>(xin), Tx, st);
            GB_CUDA_TRY(cudaGetLastError());
            k_reduce<double, VT, R, true><<<P.nitems, kItemRows, 0, stream>>>(
                D.sys, D.items, P.nitems, D.sp, D.row_strip, st, mask, nullptr, nullptr, Tx, xin, yout, mode, aux, bb,
                dots);
            GB_CUDA_TRY(cudaGetLastError());
            return GB_OK;
        }
        return launch_apply<MT, AT, VT, R>(P, D, w, base, st, mask, mat, tvec, xin, yout, mode, aux, bb, dots, stream);
    };

    // init
    k_vec<VT, R><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, st, 0, b128, bvt ? bvt : bx, x, r, r0,
                                                     p, v, s, t, dots);
    GB_CUDA_TRY(cudaGetLastError());
    k_scalar<R><<<sblocks, 128, 0, stream>>>(D.sp, P.nsys, st, 0, dots, tol, maxiter);
    GB_CUDA_TRY(cudaGetLastError());
    const VT* bsrc_vt = bvt ? bvt : bx;

    KState* hst = nullptr;
    std::vector<KState> hbuf(nsr);
    (void)host_status_buf;
    const int max_chunks = maxiter / kChunk + 64;
    for (int chunk = 0; chunk < max_chunks; chunk++) {
        for (int itn = 0; itn < kChunk; itn++) {
            k_vec<VT, R><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, st, 1, nullptr, nullptr, x, r,
                                                             r0, p, v, s, t, dots);
            int e = apply(p, v, 1, r0, 0, nullptr);
            if (e) return e;
            k_scalar<R><<<sblocks, 128, 0, stream>>>(D.sp, P.nsys, st, 1, dots, tol, maxiter);
            k_vec<VT, R><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, st, 2, nullptr, nullptr, x, r,
                                                             r0, p, v, s, t, dots);
            e = apply(s, t, 2, s, 0, nullptr);
            if (e) return e;
            k_scalar<R><<<sblocks, 128, 0, stream>>>(D.sp, P.nsys, st, 2, dots, tol, maxiter);
            k_vec<VT, R><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, st, 3, nullptr, nullptr, x, r,
                                                             r0, p, v, s, t, dots);
            k_scalar<R><<<sblocks, 128, 0, stream>>>(D.sp, P.nsys, st, 3, dots, tol, maxiter);
            GB_CUDA_TRY(cudaGetLastError());
        }
        GB_CUDA_TRY(cudaMemcpyAsync(hbuf.data(), st, sizeof(KState) * nsr, cudaMemcpyDeviceToHost, stream));
        GB_CUDA_TRY(cudaStreamSynchronize(stream));
        bool all_done = true, restart = false;
        for (int q = 0; q < nsr; q++) {
            if (!hbuf[q].done) all_done = false;
            if (hbuf[q].need_restart) restart = true;
        }
        if (restart) {
            // r = b - A x for the restarting clusters, r0 = r, rho = |r|^2
            int e = apply(x, r, 3, bsrc_vt, 1, b128);
            if (e) return e;
            k_vec<VT, R><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, st, 4, nullptr, nullptr, x, r,
                                                             r0, p, v, s, t, dots);
            k_scalar<R><<<sblocks, 128, 0, stream>>>(D.sp, P.nsys, st, 4, dots, tol, maxiter);
            GB_CUDA_TRY(cudaGetLastError());
            continue;
        }
        if (all_done) return GB_OK;
    }
    (void)hst;
    return gb_set_error(GB_TIMEOUT, "BiCGSTAB driver exceeded its chunk limit");
}

template <typename VT>
__global__ void k_copy_out(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems, int R,
                           const VT* __restrict__ src, double2* __restrict__ dst) {
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    const int lr = threadIdx.x;
    if (lr >= I.nr) return;
    const long long vo = S.vec_off + (long long)(I.r0 + lr) * R;
    for (int rr = 0; rr < R; rr++) dst[vo + rr] = to_d2(src[vo + rr]);
}

__global__ void k_cast_f(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems, int R,
                         const double2* __restrict__ src, float2* __restrict__ dst, const KState* __restrict__ mask) {
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    const int lr = threadIdx.x;
    if (lr >= I.nr) return;
    const long long vo = S.vec_off + (long long)(I.r0 + lr) * R;
    for (int rr = 0; rr < R; rr++) {
        const double2 v = src[vo + rr];
        const bool off = mask && mask[I.sys * R + rr].done;   // finished clusters get b = 0
        dst[vo + rr] = off ? make_float2(0.f, 0.f) : make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
    }
}

int finish_status(const Plan& P, KState* st_dev, int* status, int* iters, double* resid, cudaStream_t stream) {
    const int nsr = P.nsys * P.R;
    std::vector<KState> h(nsr);
    GB_CUDA_TRY(cudaMemcpyAsync(h.data(), st_dev, sizeof(KState) * nsr, cudaMemcpyDeviceToHost, stream));
    GB_CUDA_TRY(cudaStreamSynchronize(stream));
    int worst = GB_OK;
    for (int q = 0; q < nsr; q++) {
        if (status) status[q] = h[q].status;
        if (iters) iters[q] = h[q].iters;
        if (resid) resid[q] = h[q].bsq > 0 ? std::sqrt(h[q].rsq / h[q].bsq) : 0.0;
        if (h[q].status != GB_OK && worst == GB_OK) worst = h[q].status;
    }
    return worst;
}

template <int R>
int solve_impl(const Plan& P, int prec, double tol, int maxiter, double inner_tol, int max_refine,
               const double* mat128, const float* mat64, const double* tvec, const double* b, double* x,
               unsigned char* base, const WS& w, int* status, int* iters, double* resid, cudaStream_t stream) {
    DevPlan D;
    int e = upload_plan(P, base, w, stream, D);
    if (e) return e;
    KState* st = reinterpret_cast<KState*>(base + w.off_state);
    KState* ost = reinterpret_cast<KState*>(base + w.off_ostate);
    const double2* t2 = reinterpret_cast<const double2*>(tvec);
    const double2* b2 = reinterpret_cast<const double2*>(b);
    double2* x2 = reinterpret_cast<double2*>(x);
    const size_t TV = (size_t)P.total_vec;
    if (prec == GB_PREC_FP64) {
        e = run_bicgstab<double2, double, double2, R, false>(P, D, w, base, reinterpret_cast<const double2*>(mat128),
                                                             t2, b2, nullptr, tol, maxiter, st, 0, stream, nullptr);
        if (e) return e;
        double2* xv = reinterpret_cast<double2*>(base + w.off_vec);
        k_copy_out<double2><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, R, xv, x2);
        GB_CUDA_TRY(cudaGetLastError());
        return finish_status(P, st, status, iters, resid, stream);
    }
    float2* V = reinterpret_cast<float2*>(base + w.off_vec);
    float2* bx = V + 7 * TV;
    if (prec == GB_PREC_FP32) {
        e = run_bicgstab<float2, float, float2, R, false>(P, D, w, base, reinterpret_cast<const float2*>(mat64), t2, b2,
                                                          nullptr, tol, maxiter, st, 0, stream, nullptr);
        if (e) return e;
        k_copy_out<float2><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, R, V, x2);
        GB_CUDA_TRY(cudaGetLastError());
        return finish_status(P, st, status, iters, resid, stream);
    }
    // mixed: x = 0, r = b (FP64); repeat { FP32 BiCGSTAB on (I+T) d = r; x += d; r = b - (I+T) x (FP64) }
    double2* r128 = reinterpret_cast<double2*>(base + w.off_x128r);
    double2* dots = reinterpret_cast<double2*>(base + w.off_dots);
    const int nsr = P.nsys * R;
    k_outer_start<R><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, b2, x2, dots);
    k_outer_init<R><<<(nsr + 127) / 128, 128, 0, stream>>>(D.sp, P.nsys, ost, dots, tol);
    GB_CUDA_TRY(cudaGetLastError());
    GB_CUDA_TRY(cudaMemcpyAsync(r128, b2, sizeof(double2) * TV, cudaMemcpyDeviceToDevice, stream));
    int total_inner = 0;
    std::vector<KState> hst(nsr), hin(nsr);
    for (int pass = 1; pass <= max_refine + 1; pass++) {
        // inner FP32 solve of the current residual (clusters already done are masked by ost)
        k_cast_f<<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, R, r128, bx, ost);
        GB_CUDA_TRY(cudaGetLastError());
        e = run_bicgstab<float2, float, float2, R, false>(P, D, w, base, reinterpret_cast<const float2*>(mat64), t2,
                                                          nullptr, bx, inner_tol, maxiter, st, 0, stream, nullptr);
        if (e) return e;
        GB_CUDA_TRY(cudaMemcpyAsync(hin.data(), st, sizeof(KState) * nsr, cudaMemcpyDeviceToHost, stream));
        k_refine_axpy<R><<<P.nitems, kItemRows, 0, stream>>>(D.sys, D.items, P.nitems, ost, x2, V);
        GB_CUDA_TRY(cudaGetLastError());
        // FP64 residual r = b - (I + T) x on the complex128 matrix
        e = launch_apply<double2, double, double2, R>(P, D, w, base, ost, -1, reinterpret_cast<const double2*>(mat128),
                                                      t2, x2, r128, 3, nullptr, b2, dots, stream);
        if (e) return e;
        k_refine_check<R><<<(nsr + 127) / 128, 128, 0, stream>>>(D.sp, P.nsys, ost, dots, pass, max_refine);
        GB_CUDA_TRY(cudaGetLastError());
        GB_CUDA_TRY(cudaMemcpyAsync(hst.data(), ost, sizeof(KState) * nsr, cudaMemcpyDeviceToHost, stream));
        GB_CUDA_TRY(cudaStreamSynchronize(stream));
        for (int q = 0; q < nsr; q++) total_inner = std::max(total_inner, hin[q].iters);
        bool all = true;
        for (int q = 0; q < nsr; q++) all &= (hst[q].done != 0);
        if (all) break;
    }
    int worst = GB_OK;
    for (int q = 0; q < nsr; q++) {
        if (status) status[q] = hst[q].status;
        if (iters) iters[q] = hst[q].iters;   // refinement passes
        if (resid) resid[q] = hst[q].bsq > 0 ? std::sqrt(hst[q].rsq / hst[q].bsq) : 0.0;
        if (hst[q].status != GB_OK && worst == GB_OK) worst = hst[q].status;
    }
    (void)total_inner;
    return worst;
}

}   // namespace

extern "C" {

size_t gb_solve_workspace_size(int nsys, const gb_system* sys, int R, int prec) {
    Plan P;
    if (build_plan(nsys, sys, R, 0, P)) return 0;
    return ws_layout(P, prec, false).total;
}

int gb_solve_batch(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter, double inner_tol,
                   int max_refine, const double* mat128, const float* mat64, const double* tvec, const double* b,
                   double* x, void* workspace, size_t ws_bytes, int* status, int* iters, double* resid,
                   void* stream) {
    if (nsys < 1 || !sys || !tvec || !b || !x || !workspace) return gb_set_error(GB_BAD_ARG, "null argument");
    if (R != 1 && R != 2) return gb_set_error(GB_UNSUPPORTED, "R must be 1 or 2 (got %d)", R);
    if (prec == GB_PREC_FP64 && !mat128) return gb_set_error(GB_BAD_ARG, "FP64 solve needs the complex128 matrix");
    if (prec == GB_PREC_FP32 && !mat64) return gb_set_error(GB_BAD_ARG, "FP32 solve needs the complex64 matrix");
    if (prec == GB_PREC_MIXED && (!mat64 || !mat128)) return gb_set_error(GB_BAD_ARG, "mixed solve needs both matrices");
    if (!(tol > 0) || maxiter < 1) return gb_set_error(GB_BAD_ARG, "tol must be > 0 and maxiter >= 1");
    cudaStream_t s = (cudaStream_t)stream;
    Plan P;
    int e = build_plan(nsys, sys, R, s, P);
    if (e) return e;
    WS w = ws_layout(P, prec, false);
    if (ws_bytes < w.total) return gb_set_error(GB_OVER_BUDGET, "workspace %zu B < required %zu B", ws_bytes, w.total);
    unsigned char* base = static_cast<unsigned char*>(workspace);
    if (inner_tol <= 0) inner_tol = 1e-6;
    if (R == 1)
        return solve_impl<1>(P, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, tvec, b, x, base, w, status,
                             iters, resid, s);
    return solve_impl<2>(P, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, tvec, b, x, base, w, status,
                         iters, resid, s);
}

size_t gb_apply_workspace_size(int nsys, const gb_system* sys, int R, int prec) {
    return gb_solve_workspace_size(nsys, sys, R, prec == GB_PREC_FP64 ? GB_PREC_FP64 : GB_PREC_FP32);
}

int gb_apply_batch(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                   const double* tvec, const double* x, double* y, void* workspace, size_t ws_bytes, void* stream) {
    if (nsys < 1 || !sys || !tvec || !x || !y || !workspace) return gb_set_error(GB_BAD_ARG, "null argument");
    if (R != 1 && R != 2) return gb_set_error(GB_UNSUPPORTED, "R must be 1 or 2 (got %d)", R);
    cudaStream_t s = (cudaStream_t)stream;
    Plan P;
    int e = build_plan(nsys, sys, R, s, P);
    if (e) return e;
    const int pw = (prec == GB_PREC_FP64) ? GB_PREC_FP64 : GB_PREC_FP32;
    WS w = ws_layout(P, pw, false);
    if (ws_bytes < w.total) return gb_set_error(GB_OVER_BUDGET, "workspace %zu B < required %zu B", ws_bytes, w.total);
    unsigned char* base = static_cast<unsigned char*>(workspace);
    DevPlan D;
    e = upload_plan(P, base, w, s, D);
    if (e) return e;
    KState* st = reinterpret_cast<KState*>(base + w.off_state);
    const double2* x2 = reinterpret_cast<const double2*>(x);
    double2* y2 = reinterpret_cast<double2*>(y);
    double2* dots = reinterpret_cast<double2*>(base + w.off_dots);
    const double2* t2 = reinterpret_cast<const double2*>(tvec);
    if (prec == GB_PREC_FP64) {
        if (!mat128) return gb_set_error(GB_BAD_ARG, "complex128 matrix missing");
        if (R == 1)
            return launch_apply<double2, double, double2, 1>(P, D, w, base, st, -1, reinterpret_cast<const double2*>(mat128),
                                                             t2, x2, y2, 0, nullptr, nullptr, dots, s);
        return launch_apply<double2, double, double2, 2>(P, D, w, base, st, -1, reinterpret_cast<const double2*>(mat128),
                                                         t2, x2, y2, 0, nullptr, nullptr, dots, s);
    }
    if (!mat64) return gb_set_error(GB_BAD_ARG, "complex64 matrix missing");
    // FP32 product on a rounded copy of x, result widened to FP64
    const size_t TV = (size_t)P.total_vec;
    float2* V = reinterpret_cast<float2*>(base + w.off_vec);
    float2 *xf = V, *yf = V + TV;
    k_cast_f<<<P.nitems, kItemRows, 0, s>>>(D.sys, D.items, P.nitems, R, x2, xf, nullptr);
    if (R == 1)
        e = launch_apply<float2, float, float2, 1>(P, D, w, base, st, -1, reinterpret_cast<const float2*>(mat64), t2, xf,
                                                   yf, 0, nullptr, nullptr, dots, s);
    else
        e = launch_apply<float2, float, float2, 2>(P, D, w, base, st, -1, reinterpret_cast<const float2*>(mat64), t2, xf,
                                                   yf, 0, nullptr, nullptr, dots, s);
    if (e) return e;
    k_copy_out<float2><<<P.nitems, kItemRows, 0, s>>>(D.sys, D.items, P.nitems, R, yf, y2);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

size_t gb_solve_dense_workspace_size(int D, int R) {
    // one pseudo-cluster of D rows (B = D handled by items only)
    Plan P;
    P.nsys = 1;
    P.R = R;
    gb::SysDev sd{};
    sd.D = D;
    sd.B = D;
    sd.N = 1;
    P.sd.push_back(sd);
    SysPlan sp{};
    sp.item_begin = 0;
    for (int r0 = 0; r0 < D; r0 += kItemRows) P.items.push_back(Item{0, r0, std::min(kItemRows, D - r0), 0});
    sp.item_end = (int)P.items.size();
    P.sp.push_back(sp);
    P.row_strip = {0, 0};
    P.nitems = (int)P.items.size();
    P.total_vec = (long long)D * R;
    return ws_layout(P, GB_PREC_FP64, true).total;
}

int gb_solve_dense(int D, int R, const double* T, const double* b, double* x, double tol, int maxiter,
                   void* workspace, size_t ws_bytes, int* status, int* iters, double* resid, void* stream) {
    if (D < 1 || !T || !b || !x || !workspace) return gb_set_error(GB_BAD_ARG, "null argument");
    if (R != 1 && R != 2) return gb_set_error(GB_UNSUPPORTED, "R must be 1 or 2 (got %d)", R);
    if (!(tol > 0) || maxiter < 1) return gb_set_error(GB_BAD_ARG, "tol must be > 0 and maxiter >= 1");
    cudaStream_t s = (cudaStream_t)stream;
    Plan P;
    P.nsys = 1;
    P.R = R;
    gb::SysDev sd{};
    sd.D = D;
    sd.B = D;
    sd.N = 1;
    sd.vec_off = 0;
    P.sd.push_back(sd);
    SysPlan sp{};
    sp.item_begin = 0;
    for (int r0 = 0; r0 < D; r0 += kItemRows) P.items.push_back(Item{0, r0, std::min(kItemRows, D - r0), 0});
    sp.item_end = (int)P.items.size();
    P.sp.push_back(sp);
    P.row_strip = {0, 0};
    P.nitems = (int)P.items.size();
    P.total_vec = (long long)D * R;
    WS w = ws_layout(P, GB_PREC_FP64, true);
    if (ws_bytes < w.total) return gb_set_error(GB_OVER_BUDGET, "workspace %zu B < required %zu B", ws_bytes, w.total);
    unsigned char* base = static_cast<unsigned char*>(workspace);
    DevPlan Dp;
    int e = upload_plan(P, base, w, s, Dp);
    if (e) return e;
    KState* st = reinterpret_cast<KState*>(base + w.off_state);
    if (R == 1)
        e = run_bicgstab<double2, double, double2, 1, true>(P, Dp, w, base, reinterpret_cast<const double2*>(T), nullptr,
                                                            reinterpret_cast<const double2*>(b), nullptr, tol, maxiter,
                                                            st, D, s, nullptr);
    else
        e = run_bicgstab<double2, double, double2, 2, true>(P, Dp, w, base, reinterpret_cast<const double2*>(T), nullptr,
                                                            reinterpret_cast<const double2*>(b), nullptr, tol, maxiter,
                                                            st, D, s, nullptr);
    if (e) return e;
    double2* xv = reinterpret_cast<double2*>(base + w.off_vec);
    k_copy_out<double2><<<P.nitems, kItemRows, 0, s>>>(Dp.sys, Dp.items, P.nitems, R, xv, reinterpret_cast<double2*>(x));
    GB_CUDA_TRY(cudaGetLastError());
    return finish_status(P, st, status, iters, resid, s);
}

}   // extern "C"
