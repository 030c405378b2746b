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
// columns: 128-bit coalesced loads, per-lane accumulators, no per-row cross-lane
// reduction.  A lane owns NS "slots" (row offset, column group) so that RPS rows
// are covered per step by all 32 lanes; slot sums of one column are combined in
// shared memory once per block.
//
// Three arithmetic policies share the kernel:
//   Pol64  complex128 matrix, FP64 FMAs (the plain method);
//   Pol32  complex64 matrix, FP32 FMAs (inner solves of the mixed method);
//   PolDF  double-float: the complex128 matrix stored as complex64 hi + lo
//          (hi = fl32(a), lo = fl32(a - hi)), x split the same way, every hi*hi
//          product formed exactly (FMA two-product) and accumulated with TwoSum;
//          the residual of the mixed method at about 1e-14 relative accuracy,
//          on the FP32 pipes (GB300's FP64 rate is 1/58 of its FP32 rate).
//
// K3a (k_pgemv): warp per strip of consecutive blocks (i, j0..j0+J-1) of one block
//   row; c_u accumulates across the strip, c_w is written per block.
// K3b (k_reduce): 8 warps x 32 rows; warps split the partial terms of a row, a
//   fixed-order shared-memory sum combines them (deterministic, no atomics),
//   adds the identity term and emits per-item partial dot products.
// K4: BiCGSTAB vector updates fused with the dot-product partials, and one-thread-
//   per-(cluster, rhs) scalar kernels; all scalars stay on the device.  Chunks of
//   iterations are captured once into a CUDA graph and replayed; the host reads one
//   flag array per chunk and finished clusters' kernels return immediately.
//
// The iteration is Eigen's: x0 = 0, r0 = r = b, rho = alpha = omega = 1, restart
// with r = b - A x when |rho| < eps^2 |r0|^2, stop when |r|^2 <= tol^2 |b|^2.

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"
#include "solve_plan.cuh"

namespace {

constexpr int kVRows = 128;        // rows per vector work item (= threads per CTA)
constexpr int kRBThreads = 384;    // threads of the block reduce and T-matrix y kernels (>= B*R for lmax <= 8, R <= 2)
constexpr int kRRows = 32;         // rows per reduce work item
constexpr int kGemvThreads = 128;  // 4 warps
constexpr int kGemvWarps = kGemvThreads / 32;
constexpr int kChunk = 4;          // iterations per host check
constexpr int kMaxRestarts = 8;
// Mixed refinement: once |r| <= kIncrTheta * tol * |b| for every running cluster,
// the next residual is updated as r -= (I + T) d with the complex64 matrix (the
// correction d is ~|r|, so the complex64 product's ~2e-6 relative error stays below
// tol |b| / 20) instead of recomputed as b - (I + T) x in double-float.
constexpr double kIncrTheta = 2.5e4;

// ------------------------------------------------------------ type helpers --
__device__ __forceinline__ double2 to_d2(double2 v) { return v; }
__device__ __forceinline__ double2 to_d2(float2 v) { return make_double2(v.x, v.y); }
template <typename VT> __device__ __forceinline__ VT from_d2(double2 v);
template <> __device__ __forceinline__ double2 from_d2<double2>(double2 v) { return v; }
template <> __device__ __forceinline__ float2 from_d2<float2>(double2 v) {
    return make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
}

// Arithmetic of the vector kernels, their dot products and the BiCGSTAB scalar
// step: FP32 for the FP32 solver (float2 vectors), FP64 otherwise.  GB300 issues an
// FP64 warp instruction about once per 64 cycles per SM sub-partition, so the FP32
// solver's small latency-bound kernels (reduce, vector update, scalar step) keep
// off the FP64 pipe entirely.
template <typename VT> struct Arith { using T = double; using C = double2; };
template <> struct Arith<float2> { using T = float; using C = float2; };
template <typename T> struct CplxT { using t = double2; };   // complex type of real type T
template <> struct CplxT<float> { using t = float2; };

template <typename C> __device__ __forceinline__ C to_c(float2 v);
template <typename C> __device__ __forceinline__ C to_c(double2 v);
template <> __device__ __forceinline__ float2 to_c<float2>(float2 v) { return v; }
template <> __device__ __forceinline__ float2 to_c<float2>(double2 v) { return from_d2<float2>(v); }
template <> __device__ __forceinline__ double2 to_c<double2>(double2 v) { return v; }
template <typename VT> __device__ __forceinline__ VT from_c(float2 v);
template <typename VT> __device__ __forceinline__ VT from_c(double2 v);
template <> __device__ __forceinline__ float2 from_c<float2>(float2 v) { return v; }
template <> __device__ __forceinline__ double2 from_c<double2>(double2 v) { return v; }

__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return cmulf(a, b); }
__device__ __forceinline__ void cfma_conj(float2& acc, float2 a, float2 b) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(-a.y, b.x, acc.y);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cflip(double2 a, unsigned neg) { return make_double2(flipd(a.x, neg), flipd(a.y, neg)); }
__device__ __forceinline__ float2 cflip(float2 a, unsigned neg) { return make_float2(flipf(a.x, neg), flipf(a.y, neg)); }
__device__ __forceinline__ double2 shfl_xor(double2 a, int o) {
    return make_double2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
}
__device__ __forceinline__ float2 shfl_xor(float2 a, int o) {
    return make_float2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
}
template <typename C> __device__ __forceinline__ C czero() { C z; z.x = 0; z.y = 0; return z; }

// ---------------------------------------------- programmatic dependent launch --
// The kernels of a BiCGSTAB iteration are launched with programmatic stream
// serialisation: a kernel may start while its predecessor drains, runs its
// prologue on plan data (constant during a solve), then waits for the predecessor
// (griddepcontrol.wait: its grid complete, its memory visible) before any access to
// data the predecessor produces or consumes.  Every CTA waits before it can exit,
// so a grid's completion implies its predecessors' completion.  Without the launch
// attribute the wait returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream, Args... args) {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// ----------------------------------------------------------- plan structs --
using gb::Strip;
using gb::Item;
using gb::SysPlan;
using gb::KState;
using gb::active_rhs;
using gb::any_active;

// The scalars of a KState in the solver's arithmetic T (read-only views for the
// vector kernels' alpha, omega, beta).
#define GB_KS_FIELD(name)                                                                            \
    __device__ __forceinline__ auto& ks_##name(KState& k, double) { return k.name; }                  \
    __device__ __forceinline__ auto& ks_##name(KState& k, float) { return k.name##_f; }
#define GB_KS_CFIELD(name)                                                                           \
    __device__ __forceinline__ const auto& ks_##name(const KState& k, double) { return k.name; }      \
    __device__ __forceinline__ const auto& ks_##name(const KState& k, float) { return k.name##_f; }
GB_KS_FIELD(rho)
GB_KS_FIELD(alpha)
GB_KS_FIELD(omega)
GB_KS_FIELD(beta)
GB_KS_FIELD(r0sq)
GB_KS_FIELD(bsq)
GB_KS_FIELD(rsq)
GB_KS_FIELD(tol2)
GB_KS_CFIELD(alpha)
GB_KS_CFIELD(omega)
GB_KS_CFIELD(beta)
#undef GB_KS_FIELD
#undef GB_KS_CFIELD

enum { ST_RUNNING = -1 };

// --------------------------------------------------------------- policies --
// Arithmetic of the GEMV.  A lane multiplies one matrix element m by the y
// values of its row; complex products use packed f32x2 FMAs where the policy is
// FP32-based: with m = (re, im) as loaded,
//   a += m * y.re,  b += m * y.im,  and m y = (a.x - b.y, a.y + b.x),
// so no shuffling of m is needed and each complex multiply-add is two FFMA2.
__device__ __forceinline__ float2 bc(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }

// (h, l) += p exactly (TwoSum on both components), error into l
__device__ __forceinline__ void two_sum2(float2& h, float2& l, float2 p) {
    const float2 s = __fadd2_rn(h, p);
    const float2 bb = fsub2(s, h);
    const float2 err = __fadd2_rn(fsub2(h, fsub2(s, bb)), fsub2(p, bb));
    h = s;
    l = __fadd2_rn(l, err);
}
// scalar double-float helpers: (h, l) normalised sum of two double-floats
__device__ __forceinline__ void df_add(float& h, float& l, float h2, float l2) {
    const float s = h + h2;
    const float bb = s - h;
    const float err = (h - (s - bb)) + (h2 - bb);
    const float t = err + l + l2;
    h = s + t;
    l = t - (h - s);
}

struct Pol64 {                 // complex128 matrix, FP64 FMAs
    static constexpr int ID = 0;
    static constexpr int MB = 16;
    static constexpr bool DF = false;
    using YT = double2;
    using OutT = double2;
    using Acc = double2;
    struct M { double2 h; };
    __device__ static M load(const unsigned char* hi, const unsigned char*, unsigned off) {
        return M{*reinterpret_cast<const double2*>(hi + off)};
    }
    __device__ static void zero(Acc& a) { a = make_double2(0, 0); }
    __device__ static void prep(M&) {}
    __device__ static void mac(Acc& a, const M& m, const YT& y) { cfma(a, m.h, y); }
    __device__ static OutT out(const Acc& a) { return a; }
    __device__ static OutT add(OutT u, OutT v) { return make_double2(u.x + v.x, u.y + v.y); }
    __device__ static OutT shfl(OutT v, int off) {
        return make_double2(__shfl_xor_sync(0xffffffffu, v.x, off), __shfl_xor_sync(0xffffffffu, v.y, off));
    }
};

struct Pol32 {                 // complex64 matrix, packed FP32 FMAs
    static constexpr int ID = 1;
    static constexpr int MB = 8;
    static constexpr bool DF = false;
    using YT = float4;         // (re, re, im, im)
    using OutT = float2;
    struct Acc { float2 a, b; };
    struct M { float2 h; };
    __device__ static M load(const unsigned char* hi, const unsigned char*, unsigned off) {
        return M{*reinterpret_cast<const float2*>(hi + off)};
    }
    __device__ static void zero(Acc& s) { s.a = s.b = make_float2(0, 0); }
    __device__ static void prep(M&) {}
    __device__ static void mac(Acc& s, const M& m, const YT& y) {
        s.a = __ffma2_rn(m.h, make_float2(y.x, y.y), s.a);
        s.b = __ffma2_rn(m.h, make_float2(y.z, y.w), s.b);
    }
    __device__ static OutT out(const Acc& s) { return make_float2(s.a.x - s.b.y, s.a.y + s.b.x); }
    __device__ static OutT add(OutT u, OutT v) { return make_float2(u.x + v.x, u.y + v.y); }
    __device__ static OutT shfl(OutT v, int off) {
        return make_float2(__shfl_xor_sync(0xffffffffu, v.x, off), __shfl_xor_sync(0xffffffffu, v.y, off));
    }
};

// Double-float: the complex128 matrix as complex64 hi + lo, y as (hi.re, hi.im,
// lo.re, lo.im).  Every hi*hi real product is formed exactly (p = fl(m y),
// e = fma(m, y, -p)) and summed with TwoSum; e, the TwoSum errors and the
// hi*lo + lo*hi corrections accumulate in the low word.  Partial results leave as
// a double-float complex float4 (re.h, im.h, re.l, im.l), about 1e-14 relative.
struct DFAcc { float2 ha, la, hb, lb; };
struct PolDF {
    static constexpr int ID = 2;
    static constexpr int MB = 8;
    static constexpr bool DF = true;
    using YT = float4;
    using OutT = float4;
    using Acc = DFAcc;
    struct M { float2 h, l, nh; };
    __device__ static M load(const unsigned char* hi, const unsigned char* lo, unsigned off) {
        M m;
        m.h = *reinterpret_cast<const float2*>(hi + off);
        m.l = *reinterpret_cast<const float2*>(lo + off);
        return m;
    }
    __device__ static void zero(Acc& s) { s.ha = s.la = s.hb = s.lb = make_float2(0, 0); }
    __device__ static void prep(M& m) { m.nh = neg2(m.h); }
    __device__ static void mac(Acc& s, const M& m, const YT& y) {
        const float2 yr = bc(y.x), yi = bc(y.y);
        float2 p = __fmul2_rn(m.h, yr);
        float2 en = __ffma2_rn(m.nh, yr, p);                 // p - m y = -(rounding error)
        two_sum2(s.ha, s.la, p);
        s.la = fsub2(s.la, en);
        s.la = __ffma2_rn(m.l, yr, s.la);
        s.la = __ffma2_rn(m.h, bc(y.z), s.la);
        p = __fmul2_rn(m.h, yi);
        en = __ffma2_rn(m.nh, yi, p);
        two_sum2(s.hb, s.lb, p);
        s.lb = fsub2(s.lb, en);
        s.lb = __ffma2_rn(m.l, yi, s.lb);
        s.lb = __ffma2_rn(m.h, bc(y.w), s.lb);
    }
    __device__ static OutT out(const Acc& s) {
        // re = a.x - b.y, im = a.y + b.x, each as a normalised double-float
        float rh = s.ha.x, rl = s.la.x, ih = s.ha.y, il = s.la.y;
        df_add(rh, rl, -s.hb.y, -s.lb.y);
        df_add(ih, il, s.hb.x, s.lb.x);
        return make_float4(rh, ih, rl, il);
    }
    __device__ static OutT add(OutT u, OutT v) {
        df_add(u.x, u.z, v.x, v.z);
        df_add(u.y, u.w, v.y, v.w);
        return u;
    }
    __device__ static OutT shfl(OutT v, int off) {
        return make_float4(__shfl_xor_sync(0xffffffffu, v.x, off), __shfl_xor_sync(0xffffffffu, v.y, off),
                           __shfl_xor_sync(0xffffffffu, v.z, off), __shfl_xor_sync(0xffffffffu, v.w, off));
    }
};

// Optional BiCGSTAB vector update folded into the y-vector preparation of the
// next product (kind 1: p-update into out = p; kind 2: s-update into out = s).
template <typename VT> struct YUpd {
    int kind = 0;
    const VT* r = nullptr;
    const VT* v = nullptr;
    VT* out = nullptr;
};

// ------------------------------------------------------------ y vectors --
// For every row (particle k, local row r) of every cluster:
//   z = eps(r) t_k[rho(r)] x_k[rho(r)],   Yu = z,  Yw = sig(r) z
// stored as double2 (YK 0), float4 (re, re, im, im) (YK 1) or the float4 hi/lo
// split (YK 2).
template <int YK> struct YType;
template <> struct YType<0> { using t = double2; };
template <> struct YType<1> { using t = float4; };   // (re, re, im, im): broadcast pairs for f32x2 FMAs
template <> struct YType<2> { using t = float4; };
template <> struct YType<3> { using t = float2; };   // (re, im): the tensor-core pass builds its own operands

template <int YK> __device__ __forceinline__ typename YType<YK>::t make_y(double2 z);
template <int YK> __device__ __forceinline__ typename YType<YK>::t make_y(float2 z);
template <> __device__ __forceinline__ double2 make_y<0>(double2 z) { return z; }
template <> __device__ __forceinline__ double2 make_y<0>(float2 z) { return to_d2(z); }
template <> __device__ __forceinline__ float4 make_y<1>(float2 z) { return make_float4(z.x, z.x, z.y, z.y); }
template <> __device__ __forceinline__ float4 make_y<1>(double2 z) { return make_y<1>(from_d2<float2>(z)); }
template <> __device__ __forceinline__ float4 make_y<2>(float2 z) { return make_float4(z.x, z.y, 0.f, 0.f); }
template <> __device__ __forceinline__ float2 make_y<3>(float2 z) { return z; }
template <> __device__ __forceinline__ float2 make_y<3>(double2 z) { return from_d2<float2>(z); }
template <> __device__ __forceinline__ float4 make_y<2>(double2 z) {
    const float hx = __double2float_rn(z.x), hy = __double2float_rn(z.y);
    return make_float4(hx, hy, __double2float_rn(z.x - (double)hx), __double2float_rn(z.y - (double)hy));
}

// Layout: [D][R] interleaved (element (row, rr) at vec_off + row*R + rr).
template <int YK, typename VT, int R>
__global__ void __launch_bounds__(kVRows)
k_yprep(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems, const KState* __restrict__ st,
        int mask_mode, const double2* __restrict__ tvec, const VT* __restrict__ x, typename YType<YK>::t* __restrict__ Yu,
        typename YType<YK>::t* __restrict__ Yw, YUpd<VT> up) {
    const int it = blockIdx.x;
    if (it >= nitems) {
        pdl_wait();
        return;
    }
    // prologue on plan data and the Mie vector (constant during a solve)
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    const int lr = threadIdx.x;
    const bool row_ok = lr < I.nr;
    const int row = I.r0 + (row_ok ? lr : 0);
    const int part = row / S.B, Rr = row % S.B;
    const int info = __ldg(S.rowinfo + Rr);
    const int rho = info & ((1 << 29) - 1);
    const unsigned eneg = (info >> 29) & 1, sneg = (info >> 30) & 1;
    const long long src = (long long)part * S.B + rho;
    using C = typename Arith<VT>::C;
    using T = typename Arith<VT>::T;
    const T tg{};
    const C t = to_c<C>(tvec[S.t_off + src]);
    pdl_wait();
    pdl_trigger();
    if (!row_ok || !any_active<R>(st, I.sys, mask_mode)) return;
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        const long long es = S.vec_off + src * R + rr;
        C xv;
        if (up.kind != 0 && active_rhs<R>(st, I.sys, rr, 0)) {
            // the BiCGSTAB vector update this product's input needs, on the source row
            // this thread alone reads: p = r + beta (p - omega v) or s = r - alpha v
            const KState& k = st[I.sys * R + rr];
            const C rv = to_c<C>(up.r[es]), vv = to_c<C>(up.v[es]);
            C nv;
            if (up.kind == 1) {
                const C pv = to_c<C>(up.out[es]);
                nv = cadd(rv, cmul(ks_beta(k, tg), csub(pv, cmul(ks_omega(k, tg), vv))));
            } else {
                nv = csub(rv, cmul(ks_alpha(k, tg), vv));
            }
            const VT q = from_c<VT>(nv);
            up.out[es] = q;
            xv = to_c<C>(q);
        } else {
            xv = to_c<C>(x[es]);
        }
        const C yu = cflip(cmul(t, xv), eneg);
        const C yw = cflip(yu, sneg);
        const long long o = S.vec_off + (long long)row * R + rr;
        Yu[o] = make_y<YK>(yu);
        Yw[o] = make_y<YK>(yw);
    }
}

// y vectors of clusters of general particles (the T-matrix overload of the
// reference's aggregate, vsh_translation.cpp:53-159: block (i, j) = A_ij T_j, so
// (I + T_agg) x = x + A (T x) with the packed translation blocks A).  One CTA per
// particle (an item of the reduce plan): it applies the BiCGSTAB vector update of
// the particle's rows, keeps the updated vector in shared memory, then forms
// z = eps(r) (T x)[rho(r)] for every row r with the particle's T-matrix: complex64
// in FP32 arithmetic for the FP32 solver, complex128 in FP64 otherwise.
template <int YK, typename VT, int R>
__global__ void __launch_bounds__(kRBThreads)
k_yprep_tmat(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems,
             const KState* __restrict__ st, int mask_mode, const VT* __restrict__ x,
             typename YType<YK>::t* __restrict__ Yu, typename YType<YK>::t* __restrict__ Yw, YUpd<VT> up) {
    const int it = blockIdx.x;
    if (it >= nitems) {
        pdl_wait();
        return;
    }
    const Item I = items[it];   // prologue on plan data
    const gb::SysDev S = sys[I.sys];
    using C = typename Arith<VT>::C;
    using T = typename Arith<VT>::T;
    const T tg{};
    const int B = S.B, part = I.r0 / B, tid = threadIdx.x;
    __shared__ C xs[kRBThreads];   // [B][R], B R <= kRBThreads
    pdl_wait();
    pdl_trigger();
    if (!any_active<R>(st, I.sys, mask_mode)) return;   // the same for the whole CTA
    if (tid < B * R) {
        const int e = tid / R, rr = tid - e * R;
        const long long es = S.vec_off + ((long long)part * B + e) * R + rr;
        C xv;
        if (up.kind != 0 && active_rhs<R>(st, I.sys, rr, 0)) {   // p = r + beta (p - omega v) or s = r - alpha v
            const KState& k = st[I.sys * R + rr];
            const C rv = to_c<C>(up.r[es]), vv = to_c<C>(up.v[es]);
            C nv;
            if (up.kind == 1) {
                const C pv = to_c<C>(up.out[es]);
                nv = cadd(rv, cmul(ks_beta(k, tg), csub(pv, cmul(ks_omega(k, tg), vv))));
            } else {
                nv = csub(rv, cmul(ks_alpha(k, tg), vv));
            }
            const VT q = from_c<VT>(nv);
            up.out[es] = q;
            xv = to_c<C>(q);
        } else {
            xv = to_c<C>(x[es]);
        }
        xs[tid] = xv;
    }
    __syncthreads();
    if (tid < B * R) {
        const int r = tid / R, rr = tid - r * R;
        const int info = __ldg(S.rowinfo + r);
        const int rho = info & ((1 << 29) - 1);
        const unsigned eneg = (info >> 29) & 1, sneg = (info >> 30) & 1;
        C z = czero<C>();
        if constexpr (std::is_same<C, float2>::value) {
            const float2* Tr = S.tmat64 + ((long long)part * B + rho) * B;
            for (int c = 0; c < B; c++) cfmaf(z, __ldg(Tr + c), xs[c * R + rr]);
        } else {
            const double2* Tr = S.tmat128 + ((long long)part * B + rho) * B;
            for (int c = 0; c < B; c++) cfma(z, __ldg(Tr + c), xs[c * R + rr]);
        }
        const C yu = cflip(z, eneg);
        const C yw = cflip(yu, sneg);
        const long long o = S.vec_off + ((long long)part * B + r) * R + rr;
        Yu[o] = make_y<YK>(yu);
        Yw[o] = make_y<YK>(yw);
    }
}

// --------------------------------------------------------------- K3a GEMV --
// The matrix stream is moved by TMA bulk copies (cp.async.bulk, 1-D): a strip of
// blocks is contiguous in memory, so lane 0 of a warp copies whole chunks of rows
// (and, with the first chunk of each block, the block's y vector) into a ring of S
// shared-memory stages, each completed through its own mbarrier.  The other lanes
// only wait on the mbarrier and read their slots from shared memory.  Every wait is
// bounded in time; a wait that expires sets the error flag and the warp stops.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_1d(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// The same copy with an L2 cache policy (the matrix stream is read once per pass and
// marked evict-first, so that it does not push the GEMV's partials and the solver's
// vectors out of L2 before the kernels that read them next).
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ void tma_1d_hint(void* dst, const void* src, unsigned bytes, uint64_t* bar, uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: at most lim cycles of clock (about 0.2 s by default); lim <= 0
// expires at once without waiting
constexpr long long kWaitCycles = 400000000LL;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, long long lim = kWaitCycles) {
    if (lim <= 0) return false;
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > lim) return false;
    return true;
}

}   // namespace

// Limit of the GEMV's consumer waits (the waits for a matrix chunk to land), read by
// every launch; gb_set_gemv_wait_limit changes it.  The waits that drain a warp's
// copies in flight after a failure always use kWaitCycles, so that no bulk copy is
// still landing in shared memory when its CTA exits.
static __device__ long long g_gemv_wait_cycles = kWaitCycles;

namespace {

struct GemvLayout {
    int chunk_cap, y_bytes, nys, warp_bytes;
};
// Per warp: S mbarriers | nys y-vector slots (y_u of the blocks in flight) | y_w of
// the strip's particle | S matrix stages (hi, then lo for double-float).  The
// producer runs S-1 chunks ahead of the consumer, so with cpb chunks per block the
// y_u of at most 1 + ceil((S-1)/cpb) blocks are live: the first chunk of block
// b + nys is issued only once every chunk of block b has been consumed.  (All
// blocks of one launch have the block size Bmax.)
__host__ __device__ inline GemvLayout gemv_layout(int Bmax, int rows_per_chunk, int RT, int S, int mat_bytes, bool df,
                                                  int y_bytes) {
    GemvLayout g;
    g.chunk_cap = ((rows_per_chunk * Bmax * mat_bytes) + 127) & ~127;
    g.y_bytes = (Bmax * RT * y_bytes + 127) & ~127;
    const int cpb = (Bmax + rows_per_chunk - 1) / rows_per_chunk;
    const int live = 1 + (S - 1 + cpb - 1) / cpb;
    g.nys = live < S ? live : S;
    // + 256 B of padding (kGemvPad): lanes whose columns lie past the block's end
    // read (and discard) the elements after the last stage (shape_fits bounds it)
    g.warp_bytes = 128 + (g.nys + 1) * g.y_bytes + S * g.chunk_cap * (df ? 2 : 1) + 256;
    return g;
}

// Row-lane mapping: LPR lanes share a matrix row, RPW = 32/LPR rows per step;
// lane (ro, cl) owns the columns cl + LPR*k (k < CPL) of its row, so one y load
// serves CPL elements and the smem reads of a row are contiguous across lanes.
// Column sums of the RPW rows are combined by shuffles once per block.  A chunk
// is G steps (G*RPW rows, the last chunk of a block may be shorter).
// RR right-hand sides per launch (rr0 .. rr0+RR-1), RT the row stride of y and
// of the partials.
template <class Pol, int RR, int RT, int LPR, int CPL, int G, int S>
__global__ void __launch_bounds__(kGemvThreads)
k_pgemv(const gb::SysDev* __restrict__ sys, const Strip* __restrict__ strips, long long sbeg, long long send,
        const KState* __restrict__ st, int mask_mode, const void* __restrict__ mat_hi, const void* __restrict__ mat_lo,
        const typename Pol::YT* __restrict__ Yu, const typename Pol::YT* __restrict__ Yw,
        typename Pol::OutT* __restrict__ CU, typename Pol::OutT* __restrict__ CW, const SysPlan* __restrict__ plan,
        int rr0_rt, int Bmax, int* __restrict__ err) {
    using Acc = typename Pol::Acc;
    using OutT = typename Pol::OutT;
    using YT = typename Pol::YT;
    constexpr int MB = Pol::MB;
    constexpr bool DF = Pol::DF;
    constexpr int RPW = 32 / LPR;
    constexpr int RC = G * RPW;   // rows per full chunk
    const int rr0 = (RR == RT) ? 0 : rr0_rt;
    extern __shared__ __align__(128) unsigned char gemv_smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int ro = lane / LPR, cl = lane % LPR;
    const GemvLayout lay = gemv_layout(Bmax, RC, RT, S, MB, DF, sizeof(YT));
    unsigned char* wbase = gemv_smem + (size_t)wid * lay.warp_bytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(wbase);
    unsigned char* yring = wbase + 128;
    YT* syw = reinterpret_cast<YT*>(yring + lay.nys * lay.y_bytes);
    unsigned char* stages = yring + (lay.nys + 1) * lay.y_bytes;
    const unsigned stage_stride = lay.chunk_cap * (DF ? 2 : 1);
    const unsigned char* mh = reinterpret_cast<const unsigned char*>(mat_hi);
    const unsigned char* ml = reinterpret_cast<const unsigned char*>(mat_lo);
    if (lane == 0)
        for (int k = 0; k < S; k++) mbar_init(bars + k, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    __syncwarp();
    // ring position: chunk number gc of this warp lives in stage gc % S, phase gc / S
    unsigned cstage = 0, cphase = 0;      // consumer
    unsigned pstage = 0;                  // producer (lane 0)
    const long long warp = ((long long)blockIdx.x * kGemvThreads + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * kGemvThreads) >> 5;
    bool failed = false;
    int in_flight = 0;                    // chunks issued and not yet consumed
    const uint64_t stream_pol = l2_evict_first_policy();
    // a volatile read: only the host writes the limit, which the compiler cannot see
    const long long wait_lim = *reinterpret_cast<volatile long long*>(&g_gemv_wait_cycles);
    pdl_wait();                           // y vectors and scalars of the predecessors
    pdl_trigger();
    for (long long w = sbeg + warp; w < send && !failed; w += nwarps) {
        const Strip sp = strips[w];
        bool act = false;
#pragma unroll
        for (int q = 0; q < RR; q++) act |= active_rhs<RT>(st, sp.sys, rr0 + q, mask_mode);
        if (!act) continue;
        const gb::SysDev& Sd = sys[sp.sys];
        const int B = Sd.B;
        const long long vec_off = Sd.vec_off;
        const SysPlan& pl = plan[sp.sys];
        const int cpb = (B + RC - 1) / RC;            // chunks per block
        const int total = sp.nb * cpb;
        const unsigned ybytes = (unsigned)(B * RT * sizeof(YT));
        const unsigned row_bytes = (unsigned)(B * MB);
        // first block of the strip: pair p0 = (i, j0), j0 = i + 1 + (p0 - pair_start(i))
        const int j0 = sp.i + 1 + (int)(sp.p0 - pair_start(sp.i, Sd.N));
        const unsigned char* mstrip_h = mh + (Sd.mat_off + sp.p0 * (long long)B * B) * MB;
        const unsigned char* mstrip_l = DF ? ml + (Sd.mat_off + sp.p0 * (long long)B * B) * MB : nullptr;
        int pb = 0, pc = 0;                           // producer cursor: block, chunk within block
        auto issue = [&]() {                          // lane 0: next chunk (+ its block's y_u with the first)
            const int r0 = pc * RC;
            const int nrows = min(RC, B - r0);
            const unsigned bytes = (unsigned)nrows * row_bytes;
            uint64_t* bar = bars + pstage;
            unsigned char* dst = stages + (size_t)pstage * stage_stride;
            const long long src = (long long)pb * B * row_bytes + (long long)r0 * row_bytes;
            mbar_expect_tx(bar, bytes * (DF ? 2u : 1u) + (pc == 0 ? ybytes : 0u));
            tma_1d_hint(dst, mstrip_h + src, bytes, bar, stream_pol);
            if (DF) tma_1d_hint(dst + lay.chunk_cap, mstrip_l + src, bytes, bar, stream_pol);
            if (pc == 0)
                tma_1d(yring + (size_t)(pb % lay.nys) * lay.y_bytes, Yu + vec_off + (long long)(j0 + pb) * B * RT,
                       ybytes, bar);
            pstage = (pstage + 1 == S) ? 0 : pstage + 1;
            if (++pc == cpb) { pc = 0; ++pb; }
        };
        {   // y_w of particle i: the same for every block of the strip
            const YT* src = Yw + vec_off + (long long)sp.i * B * RT;
            for (int e = lane; e < B * RT; e += 32) syw[e] = src[e];
        }
        Acc cu[CPL][RR], cw[CPL][RR];
#pragma unroll
        for (int k = 0; k < CPL; k++)
#pragma unroll
            for (int q = 0; q < RR; q++) Pol::zero(cu[k][q]);
        __syncwarp();   // syw written; every stage of the previous strip consumed
        if (lane == 0) asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        int npre = min(S - 1, total);
        if (lane == 0)
            for (int t = 0; t < npre; t++) issue();
        in_flight = npre;
        int issued = npre;
        for (int b = 0; b < sp.nb && !failed; b++) {
#pragma unroll
            for (int k = 0; k < CPL; k++)
#pragma unroll
                for (int q = 0; q < RR; q++) Pol::zero(cw[k][q]);
            const YT* syu = reinterpret_cast<const YT*>(yring + (size_t)(b % lay.nys) * lay.y_bytes);
            for (int c = 0; c < cpb; c++) {
                if (issued < total) {   // into the stage freed by the previous chunk
                    if (lane == 0) issue();
                    issued++;
                    in_flight++;
                }
                const bool ok = mbar_wait_bounded(bars + cstage, cphase, wait_lim);
                if (!__all_sync(0xffffffffu, ok)) {   // warp-uniform decision
                    if (lane == 0) atomicExch(err, 1);
                    failed = true;
                    break;
                }
                const unsigned char* stg = stages + (size_t)cstage * stage_stride;
                const int row0 = c * RC;
                const int nrows = min(RC, B - row0);
                // One step: rows lr of the chunk.  Columns cl + LPR*k >= B (when LPR*CPL
                // exceeds the block size) accumulate whatever follows the row in shared
                // memory; those sums are never stored.
                auto step = [&](int lr) {
                    const int row = row0 + lr;
                    YT yu[RR], yw[RR];
#pragma unroll
                    for (int q = 0; q < RR; q++) {
                        yu[q] = syu[row * RT + rr0 + q];
                        yw[q] = syw[row * RT + rr0 + q];
                    }
                    const unsigned rbase = (unsigned)lr * row_bytes + (unsigned)cl * MB;
#pragma unroll
                    for (int k = 0; k < CPL; k++) {
                        typename Pol::M m = Pol::load(stg, stg + lay.chunk_cap, rbase + LPR * k * MB);
                        Pol::prep(m);
#pragma unroll
                        for (int q = 0; q < RR; q++) {
                            Pol::mac(cu[k][q], m, yu[q]);
                            Pol::mac(cw[k][q], m, yw[q]);
                        }
                    }
                };
                if (nrows == RC) {   // full chunk: every lane has a row in every step
#pragma unroll
                    for (int g = 0; g < G; g++) step(g * RPW + ro);
                } else {
#pragma unroll
                    for (int g = 0; g < G; g++)
                        if (g * RPW + ro < nrows) step(g * RPW + ro);
                }
                __syncwarp();   // every lane is done with this stage (and, at the block's end, its y slot)
                if (lane == 0) asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                in_flight--;
                cstage = (cstage + 1 == S) ? 0 : cstage + 1;
                if (cstage == 0) cphase ^= 1u;
            }
            if (failed) break;
            // block done: column partial of block row j
            // column partials by destination: block row j's partials from i < j are
            // contiguous (index j(j-1)/2 + i), so the reduction streams them
            const long long jb = j0 + b;
            OutT* cwp = CW + pl.cw_off + (jb * (jb - 1) / 2 + sp.i) * (long long)B * RT;
#pragma unroll
            for (int k = 0; k < CPL; k++)
#pragma unroll
                for (int q = 0; q < RR; q++) {
                    OutT v = Pol::out(cw[k][q]);
#pragma unroll
                    for (int off = LPR; off < 32; off <<= 1) v = Pol::add(v, Pol::shfl(v, off));
                    const int col = cl + LPR * k;
                    if (ro == 0 && col < B) cwp[col * RT + rr0 + q] = v;
                }
        }
        if (failed) break;
        OutT* cup = CU + pl.cu_off + (w - pl.strip_base) * (long long)B * RT;
#pragma unroll
        for (int k = 0; k < CPL; k++)
#pragma unroll
            for (int q = 0; q < RR; q++) {
                OutT v = Pol::out(cu[k][q]);
#pragma unroll
                for (int off = LPR; off < 32; off <<= 1) v = Pol::add(v, Pol::shfl(v, off));
                const int col = cl + LPR * k;
                if (ro == 0 && col < B) cup[col * RT + rr0 + q] = v;
            }
    }
    if (failed) {   // drain: wait (bounded) for every copy this warp still has in flight
        for (int k = 0; k < in_flight; k++) {
            (void)mbar_wait_bounded(bars + cstage, cphase);
            cstage = (cstage + 1 == S) ? 0 : cstage + 1;
            if (cstage == 0) cphase ^= 1u;
        }
    }
}

// ----------------------------------------------------- dense GEMV (plugin) --
// Tx = T x for a caller-supplied dense D x D complex128 matrix; warp per row.
template <int R>
__global__ void __launch_bounds__(256)
k_dense_gemv(int D, const double2* __restrict__ T, const double2* __restrict__ x, double2* __restrict__ Tx) {
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

// ------------------------------------------------------------ K4 scalars --
// Partial dot products of the vector kernels.  The FP64 solver sums double2 values.
// The FP32 solver sums double-float complex values: every product exact (FMA
// error term), TwoSum accumulation, all on the FP32 pipe.  BiCGSTAB's inner
// products cancel heavily as it converges (rho = <r0, r> falls far below
// |r0| |r|), which a plain FP32 sum cannot follow on ill-conditioned clusters.
// Stored per (item, rhs, which) in the 16-byte slots of the dots buffer: double2,
// or float4 (re.h, im.h, re.l, im.l).
__device__ __forceinline__ void df_acc_prod(float& h, float& l, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float s = h + p;
    const float bb = s - h;
    const float err = (h - (s - bb)) + (p - bb);
    h = s;
    l += err + e;
}
template <typename T> struct DotAcc;
template <> struct DotAcc<double> {
    double2 s;
    __device__ void zero() { s = make_double2(0, 0); }
    __device__ void fma_conj(double2 a, double2 b) { cfma_conj(s, a, b); }
    __device__ void add_norm2(double2 y) { s.x += y.x * y.x + y.y * y.y; }
    __device__ void add(const DotAcc& o) { s = cadd(s, o.s); }
    __device__ DotAcc shuffled(int off) const {
        DotAcc r;
        r.s = shfl_xor(s, off);
        return r;
    }
    __device__ void store(double2* p) const { *p = s; }
    __device__ void load_cg(const double2* p) { s = __ldcg(p); }
    __device__ double2 value() const { return s; }
};
template <> struct DotAcc<float> {
    float2 h, l;
    __device__ void zero() { h = l = make_float2(0.f, 0.f); }
    __device__ void fma_conj(float2 a, float2 b) {   // += conj(a) b
        df_acc_prod(h.x, l.x, a.x, b.x);
        df_acc_prod(h.x, l.x, a.y, b.y);
        df_acc_prod(h.y, l.y, a.x, b.y);
        df_acc_prod(h.y, l.y, -a.y, b.x);
    }
    __device__ void add_norm2(float2 y) {
        df_acc_prod(h.x, l.x, y.x, y.x);
        df_acc_prod(h.x, l.x, y.y, y.y);
    }
    __device__ void add(const DotAcc& o) {
        df_add(h.x, l.x, o.h.x, o.l.x);
        df_add(h.y, l.y, o.h.y, o.l.y);
    }
    __device__ DotAcc shuffled(int off) const {
        DotAcc r;
        r.h = shfl_xor(h, off);
        r.l = shfl_xor(l, off);
        return r;
    }
    __device__ void store(double2* p) const { *reinterpret_cast<float4*>(p) = make_float4(h.x, h.y, l.x, l.y); }
    __device__ void load_cg(const double2* p) {
        const float4 v = __ldcg(reinterpret_cast<const float4*>(p));
        h = make_float2(v.x, v.y);
        l = make_float2(v.z, v.w);
    }
    __device__ float2 value() const { return make_float2(h.x + l.x, h.y + l.y); }
};

__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    const double den = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}
// FP32 complex division by Smith's method: no square of b's components, so the
// FP32 scalars of large right-hand sides (|b|^2 beyond ~1e19) do not overflow.
__device__ __forceinline__ float2 cdiv(float2 a, float2 b) {
    if (fabsf(b.x) >= fabsf(b.y)) {
        const float r = b.y / b.x, d = b.x + b.y * r;
        return make_float2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    const float r = b.x / b.y, d = b.y + b.x * r;
    return make_float2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
__device__ __forceinline__ bool finite2(double2 a) { return isfinite(a.x) && isfinite(a.y); }
__device__ __forceinline__ bool finite2(float2 a) { return isfinite(a.x) && isfinite(a.y); }
__device__ __forceinline__ double cabs_t(double2 v) { return sqrt(v.x * v.x + v.y * v.y); }
__device__ __forceinline__ float cabs_t(float2 v) { return hypotf(v.x, v.y); }   // no overflow of the squares
template <typename C> __device__ __forceinline__ C cmake(double re, double im) {
    C z;
    z.x = re;
    z.y = im;
    return z;
}

// Phases: 0 init (vector dots: |b|^2); 1 alpha = rho/<r0,v> (reduce dots);
// 2 omega = <t,s>/|t|^2 (reduce dots); 3 end of iteration (vector dots |r|^2,
// <r0,r>: convergence, restart test, beta); 4 restart done (reduce dots |r|^2).
// Scalar update of one (cluster, rhs) from its summed dots d0, d1 (one thread), in
// the solver's arithmetic T; the FP32 solver mirrors bsq and rsq into the FP64
// fields that the host reads.
template <typename T>
__device__ void scalar_apply_t(KState& k, int phase, typename CplxT<T>::t d0, typename CplxT<T>::t d1, double tol,
                               int maxiter) {
    using C = typename CplxT<T>::t;
    const T tg{};
    const T eps = (T)2.220446049250313e-16;
    auto& rho = ks_rho(k, tg);
    auto& alpha = ks_alpha(k, tg);
    auto& omega = ks_omega(k, tg);
    auto& beta = ks_beta(k, tg);
    auto& r0sq = ks_r0sq(k, tg);
    auto& bsq = ks_bsq(k, tg);
    auto& rsq = ks_rsq(k, tg);
    auto& tol2 = ks_tol2(k, tg);
    if (phase == 0) {
        bsq = r0sq = rsq = d0.x;
        tol2 = (T)tol * (T)tol * d0.x;
        rho = alpha = omega = cmake<C>(1, 0);
        k.iters = k.restarts = k.need_restart = 0;
        k.maxiter = maxiter;
        if (!isfinite(d0.x)) {   // a non-finite right-hand side: no comparison below may call it converged
            k.done = 1;
            k.status = GB_NAN;
            return;
        }
        if (d0.x == (T)0 || !(rsq > tol2) || maxiter <= 0) {
            k.done = 1;
            k.status = GB_OK;
        } else {
            k.done = 0;
            k.status = ST_RUNNING;
            const C rho_old = rho;          // loop top of the first iteration
            rho = cmake<C>(d0.x, 0.0);      // <r0, r> = |b|^2
            beta = cmul(cdiv(rho, rho_old), cdiv(alpha, omega));
        }
        return;
    }
    if (phase == 4) {   // Eigen: r = b - A x; r0 = r; rho = r0_sqnorm = |r|^2; the first restart resets i
        k.need_restart = 0;
        rsq = r0sq = d0.x;
        const C rho_old = rho;
        rho = cmake<C>(d0.x, 0.0);
        if (k.restarts++ == 0) k.iters = 0;
        if (!isfinite(rsq)) { k.done = 1; k.status = GB_NAN; return; }
        if (!(rsq > tol2)) { k.done = 1; k.status = GB_OK; return; }
        beta = cmul(cdiv(rho, rho_old), cdiv(alpha, omega));
        if (!finite2(beta)) { k.done = 1; k.status = GB_BREAKDOWN; }
        return;
    }
    if (phase == 1) {
        alpha = cdiv(rho, d0);
        if (!finite2(alpha)) { k.done = 1; k.status = (d0.x == 0 && d0.y == 0) ? GB_BREAKDOWN : GB_NAN; }
    } else if (phase == 2) {
        const T tt = d0.x;
        omega = (tt > (T)0) ? cmake<C>(d1.x / tt, d1.y / tt) : cmake<C>(0, 0);
        if (!finite2(omega)) { k.done = 1; k.status = GB_NAN; }
    } else if (phase == 3) {
        k.iters += 1;
        rsq = d0.x;
        if (!isfinite(rsq)) { k.done = 1; k.status = GB_NAN; return; }
        if (!(rsq > tol2)) { k.done = 1; k.status = GB_OK; return; }
        if (k.iters >= k.maxiter) { k.done = 1; k.status = GB_NOT_CONVERGED; return; }
        const C rho_old = rho;
        rho = d1;   // <r0, r>
        if (cabs_t(rho) < eps * eps * r0sq) {
            if (k.restarts >= kMaxRestarts) { k.done = 1; k.status = GB_BREAKDOWN; return; }
            rho = rho_old;   // phase 4 recomputes rho from the fresh residual
            k.need_restart = 1;
            return;
        }
        beta = cmul(cdiv(rho, rho_old), cdiv(alpha, omega));
        if (!finite2(beta)) { k.done = 1; k.status = GB_NAN; }
    }
}
template <typename T, typename C>
__device__ void scalar_apply(KState& k, int phase, C d0, C d1, double tol, int maxiter) {
    scalar_apply_t<T>(k, phase, d0, d1, tol, maxiter);
    if (std::is_same<T, float>::value) {
        k.bsq = (double)k.bsq_f;
        k.rsq = (double)k.rsq_f;
    }
}

__device__ __forceinline__ bool scalar_skips(const KState& k, int phase) {
    return (phase != 0 && phase != 4 && (k.done || k.need_restart)) || (phase == 4 && !k.need_restart);
}

// Per-item partial dots: [item][rhs][2] complex values in the solver's arithmetic
// (float2 for the FP32 solver, double2 otherwise) in the dots buffer.
// One warp per (cluster, rhs): lanes stride over the item partials, a fixed
// butterfly combines them (deterministic), lane 0 updates the scalars.
template <int R, typename T>
__device__ void scalar_step(const SysPlan* __restrict__ plan, KState* __restrict__ st, int phase,
                            const double2* __restrict__ dots_raw, double tol, int maxiter, int sidx, int rr, int lane) {
    const double2* dots = dots_raw;
    KState& k = st[sidx * R + rr];
    if (scalar_skips(k, phase)) return;
    const SysPlan pl = plan[sidx];
    const bool vec = (phase == 0 || phase == 3);
    const int b0 = vec ? pl.vbeg : pl.rbeg, b1 = vec ? pl.vend : pl.rend;
    DotAcc<T> d0, d1, t;
    d0.zero();
    d1.zero();
    for (int it = b0 + lane; it < b1; it += 32) {
        t.load_cg(dots + ((long long)it * R + rr) * 2 + 0);
        d0.add(t);
        t.load_cg(dots + ((long long)it * R + rr) * 2 + 1);
        d1.add(t);
    }
    for (int o = 16; o > 0; o >>= 1) {
        d0.add(d0.shuffled(o));
        d1.add(d1.shuffled(o));
    }
    if (lane == 0) scalar_apply<T>(k, phase, d0.value(), d1.value(), tol, maxiter);
}

template <int R, typename T>
__global__ void k_scalar(const SysPlan* __restrict__ plan, int nsys, KState* __restrict__ st, int phase,
                         const double2* __restrict__ dots, double tol, int maxiter) {
    const int id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (id >= nsys * R) return;
    scalar_step<R, T>(plan, st, phase, dots, tol, maxiter, id / R, id % R, lane);
}

// Scalar update fused into the kernel that produces its partial dots: each CTA
// of a cluster counts itself in after writing its partials; the last one (all of
// the cluster's partials are then visible) runs the scalar update for every rhs
// and resets the counter for the next launch.
struct ScalarFuse {
    KState* st = nullptr;   // null: no fused update
    int* cnt = nullptr;     // [nsys] arrivals, zero between launches
    int phase = 0;
    double tol = 0;
    int maxiter = 0;
};

// Called by every thread of a CTA of cluster sys once its partial dots are
// written and fenced.  The last CTA of the cluster sums the cluster's partials
// with all its NT threads (strided per thread, then warp butterflies, then the
// warps in order: a fixed order, deterministic) and updates the scalars.
template <int R, int NT, typename T>
__device__ void fused_scalar_cta(const ScalarFuse& fz, const SysPlan* __restrict__ plan,
                                 const double2* __restrict__ dots_raw, int sys, int nitems_sys) {
    const double2* dots = dots_raw;
    __shared__ int s_last;
    __shared__ DotAcc<T> s_red[NT / 32][R][2];
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const int old = atomicAdd(fz.cnt + sys, 1);
        s_last = (old == nitems_sys - 1);
        if (s_last) {
            fz.cnt[sys] = 0;
            __threadfence();
        }
    }
    __syncthreads();
    if (!s_last) return;
    const SysPlan pl = plan[sys];
    const bool vec = (fz.phase == 0 || fz.phase == 3);
    const int b0 = vec ? pl.vbeg : pl.rbeg, b1 = vec ? pl.vend : pl.rend;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        DotAcc<T> d0, d1, t;
        d0.zero();
        d1.zero();
        for (int it = b0 + (int)threadIdx.x; it < b1; it += NT) {
            t.load_cg(dots + ((long long)it * R + rr) * 2 + 0);   // written by other CTAs
            d0.add(t);
            t.load_cg(dots + ((long long)it * R + rr) * 2 + 1);
            d1.add(t);
        }
        for (int o = 16; o > 0; o >>= 1) {
            d0.add(d0.shuffled(o));
            d1.add(d1.shuffled(o));
        }
        if (lane == 0) {
            s_red[wid][rr][0] = d0;
            s_red[wid][rr][1] = d1;
        }
    }
    __syncthreads();
    if (threadIdx.x < R) {
        const int rr = threadIdx.x;
        KState& k = fz.st[sys * R + rr];
        if (scalar_skips(k, fz.phase)) return;
        DotAcc<T> d0, d1;
        d0.zero();
        d1.zero();
        for (int w = 0; w < NT / 32; w++) {
            d0.add(s_red[w][rr][0]);
            d1.add(s_red[w][rr][1]);
        }
        scalar_apply<T>(k, fz.phase, d0.value(), d1.value(), fz.tol, fz.maxiter);
    }
}

// --------------------------------------------------------------- K3b reduce --
// Per-lane sum of partials: plain sums for float2 / double2 partials, a
// double-float sum for the double-float complex partials (re.h, im.h, re.l, im.l).
template <typename OutT> struct RAcc {
    OutT s;
    __device__ void zero() { s.x = s.y = 0; }
    __device__ void add(const OutT& v) { s.x += v.x; s.y += v.y; }
    __device__ double2 get() const { return make_double2((double)s.x, (double)s.y); }
    template <typename C> __device__ C as() const {   // in the arithmetic C of the consumer
        if constexpr (std::is_same<C, OutT>::value) return s;
        else return to_c<C>(get());
    }
};
template <> struct RAcc<float4> {
    float rh, ih, rl, il;
    __device__ void zero() { rh = ih = rl = il = 0.f; }
    __device__ void add(const float4& v) {
        df_add(rh, rl, v.x, v.z);
        df_add(ih, il, v.y, v.w);
    }
    __device__ double2 get() const { return make_double2((double)rh + (double)rl, (double)ih + (double)il); }
    template <typename C> __device__ C as() const { return to_c<C>(get()); }
};

// y = x + T x (from the partials, or from a dense Tx), and per-item partial dots:
//   mode 1: d0 = <r0, y>;  mode 2: d0 = |y|^2, d1 = <y, s>;
//   mode 3: y := b - (x + T x), d0 = |y|^2  (residual).

// Partials are read as 16-byte words: two float2 elements, or one float4 / double2.
template <typename OutT> struct PWord {
    static constexpr int E = 1;
    __device__ static void load(const OutT* p, OutT (&v)[1]) { v[0] = __ldg(p); }
};
template <> struct PWord<float2> {
    static constexpr int E = 2;
    __device__ static void load(const float2* p, float2 (&v)[2]) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(p));
        v[0] = make_float2(q.x, q.y);
        v[1] = make_float2(q.z, q.w);
    }
};

// a[e] += term t's word element e for t = t0, t0 + G, ... < n (terms stride elements
// apart), in order; the loads of 8 terms are issued before their sums so that each
// thread keeps 8 words in flight.
template <typename OutT, int E>
__device__ __forceinline__ void sum_terms(const OutT* __restrict__ p, long long t0, long long n, int G, long long stride,
                                          RAcc<OutT> (&a)[E]) {
    constexpr int U = 8;
    long long t = t0;
    for (; t + (U - 1) * (long long)G < n; t += U * (long long)G) {
        OutT v[U][E];
#pragma unroll
        for (int u = 0; u < U; u++) PWord<OutT>::load(p + (t + u * (long long)G) * stride, v[u]);
#pragma unroll
        for (int u = 0; u < U; u++)
#pragma unroll
            for (int e = 0; e < E; e++) a[e].add(v[u][e]);
    }
    for (; t < n; t += G) {
        OutT v[E];
        PWord<OutT>::load(p + t * stride, v);
#pragma unroll
        for (int e = 0; e < E; e++) a[e].add(v[e]);
    }
}

// K3b (packed path): one CTA per particle block k of a cluster.  Its rows' products
// are the sum of the strip partials of block row k (contiguous in CU) and the
// column partials of the blocks (i, k), i < k (contiguous in CW by destination).
// A term (B R elements, element = column * R + rhs) is W 16-byte words; the CTA's
// threads form G = kRBThreads / W groups that split the terms, thread (g, w) streaming
// word w of its terms, so every term is one coalesced read.  The groups are combined
// in order (deterministic),
// then thread (row, rhs) applies the sign/permutation of its row, adds the identity
// term, stores y and contributes to the CTA's partial dot products (modes as k_reduce).
template <typename OutT, typename VT, int R>
__global__ void __launch_bounds__(kRBThreads)
k_reduce_blk(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems,
             const SysPlan* __restrict__ plan, const long long* __restrict__ row_strip, const KState* __restrict__ st,
             int mask_mode, const OutT* __restrict__ CU, const OutT* __restrict__ CW, const VT* __restrict__ x,
             VT* __restrict__ y, int mode, const VT* __restrict__ aux, const double2* __restrict__ b128,
             double2* __restrict__ dots, ScalarFuse fz, const double2* __restrict__ xscale) {
    const int it = blockIdx.x;
    if (it >= nitems) {
        pdl_wait();
        return;
    }
    const Item I = items[it];   // prologue on plan data
    const gb::SysDev S = sys[I.sys];
    const SysPlan pl = plan[I.sys];
    const int k = I.r0 / S.B;   // particle (block row) of this item
    const long long s0 = row_strip[pl.strip_row_base + k], s1 = row_strip[pl.strip_row_base + k + 1];
    constexpr int E = PWord<OutT>::E;
    const int B = S.B, BR = B * R;
    // The combine's inputs (row map, x, aux, b, the identity's scale, the solver
    // state) were written before the preceding matrix pass began, which waited for
    // them: loaded ahead of the wait for that pass, while it still runs.  Only its
    // partial sums need the wait.
    const bool act = any_active<R>(st, I.sys, mask_mode);
    int info_p = 0;
    VT x_p{}, aux_p{};
    double2 b_p = make_double2(0.0, 0.0), xs_p = make_double2(1.0, 0.0);
    if (act && threadIdx.x < BR) {
        const int r = threadIdx.x / R, rr = threadIdx.x - r * R;
        const long long e = S.vec_off + (long long)(I.r0 + r) * R + rr;
        info_p = __ldg(S.rowinfo + r);
        x_p = x[e];
        if (mode == 1 || mode == 2 || (mode == 3 && !b128)) aux_p = aux[e];
        if (mode == 3 && b128) b_p = b128[e];
        if (xscale) xs_p = xscale[S.t_off + I.r0 + r];
    }
    pdl_wait();
    pdl_trigger();
    if (!act) return;
    const int W = BR / E;   // 16-byte words per term (B R is even)
    const int G = kRBThreads / W;
    const int tid = threadIdx.x, g = tid / W, w = tid - g * W;
    using C = typename Arith<VT>::C;
    using T = typename Arith<VT>::T;
    __shared__ C partU[2 * kRBThreads], partW[2 * kRBThreads];
    __shared__ DotAcc<T> red[kRBThreads / 32][R][2];
    if (g < G) {
        const long long ns = s1 - s0;
        const OutT* cu = CU + pl.cu_off + (s0 - pl.strip_base) * (long long)BR + w * E;
        const OutT* cw = CW + pl.cw_off + ((long long)k * (k - 1) / 2) * BR + w * E;
        RAcc<OutT> au[E], aw[E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            au[e].zero();
            aw[e].zero();
        }
        sum_terms<OutT, E>(cu, g, ns, G, BR, au);
        sum_terms<OutT, E>(cw, g, k, G, BR, aw);
#pragma unroll
        for (int e = 0; e < E; e++) {
            partU[g * BR + w * E + e] = au[e].template as<C>();
            partW[g * BR + w * E + e] = aw[e].template as<C>();
        }
    }
    __syncthreads();
    DotAcc<T> d0, d1;
    d0.zero();
    d1.zero();
    if (tid < BR) {
        const int r = tid / R, rr = tid - r * R;
        const int info = info_p;
        const int rho = info & ((1 << 29) - 1);
        const unsigned eneg = (info >> 29) & 1, sneg = (info >> 30) & 1;
        C a = czero<C>(), c = czero<C>();
        for (int q = 0; q < G; q++) {
            a = cadd(a, partU[q * BR + rho * R + rr]);
            c = cadd(c, partW[q * BR + rho * R + rr]);
        }
        const C tx = cadd(cflip(a, eneg), cflip(c, eneg ^ sneg));
        if (active_rhs<R>(st, I.sys, rr, mask_mode)) {
            const long long e = S.vec_off + (long long)(I.r0 + r) * R + rr;
            C xe = to_c<C>(x_p);
            if (xscale) xe = cmul(xe, to_c<C>(xs_p));   // the identity's share of (I + T) D x
            C yv = cadd(xe, tx);
            if (mode == 3) yv = csub(b128 ? to_c<C>(b_p) : to_c<C>(aux_p), yv);
            const VT yo = from_c<VT>(yv);
            y[e] = yo;
            const C yq = to_c<C>(yo);   // dots of the stored (rounded) vector
            if (mode == 1) {
                d0.fma_conj(to_c<C>(aux_p), yq);
            } else if (mode == 2) {
                d0.add_norm2(yq);
                d1.fma_conj(yq, to_c<C>(aux_p));
            } else if (mode == 3) {
                d0.add_norm2(yq);
            }
        }
    }
    if (mode == 0) return;
    // CTA dots per rhs: rows of one rhs are R lanes apart, so butterflies over the
    // lanes of equal rhs leave each warp's sums in lanes 0..R-1; the warps holding
    // rows are then added in order (a fixed tree: deterministic)
    const int lane = tid & 31, wid = tid >> 5, nw = (BR + 31) / 32;
#pragma unroll
    for (int o = 16; o >= R; o >>= 1) {
        d0.add(d0.shuffled(o));
        d1.add(d1.shuffled(o));
    }
    if (lane < R && wid < nw) {
        red[wid][lane][0] = d0;
        red[wid][lane][1] = d1;
    }
    __syncthreads();
    if (tid < R) {
        DotAcc<T> s0, s1;
        s0.zero();
        s1.zero();
        for (int q = 0; q < nw; q++) {
            s0.add(red[q][tid][0]);
            s1.add(red[q][tid][1]);
        }
        s0.store(dots + ((long long)it * R + tid) * 2 + 0);
        s1.store(dots + ((long long)it * R + tid) * 2 + 1);
        __threadfence();
    }
    if (fz.st) fused_scalar_cta<R, kRBThreads, T>(fz, plan, dots, I.sys, pl.rend - pl.rbeg);
}

// Dense path (FP64 vectors): y = x + T x for the 32 rows of one item (one warp),
// with the partial dots of the modes of k_reduce_blk and the fused scalar update.
template <int R>
__global__ void __launch_bounds__(kRRows)
k_reduce_dense(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems,
               const SysPlan* __restrict__ plan, const KState* __restrict__ st, int mask_mode,
               const double2* __restrict__ Tx, const double2* __restrict__ x, double2* __restrict__ y, int mode,
               const double2* __restrict__ aux, const double2* __restrict__ b128, double2* __restrict__ dots,
               ScalarFuse fz) {
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    if (!any_active<R>(st, I.sys, mask_mode)) return;
    const gb::SysDev S = sys[I.sys];
    const int lane = threadIdx.x;
    const int row = I.r0 + lane;
    double2 d0[R], d1[R];
#pragma unroll
    for (int rr = 0; rr < R; rr++) d0[rr] = d1[rr] = make_double2(0, 0);
    if (lane < I.nr) {
        const long long vo = S.vec_off + (long long)row * R;
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            if (!active_rhs<R>(st, I.sys, rr, mask_mode)) continue;
            double2 yv = cadd(x[vo + rr], Tx[(long long)row * R + rr]);
            if (mode == 3) yv = csub(b128 ? b128[vo + rr] : aux[vo + rr], yv);
            y[vo + rr] = yv;
            if (mode == 1) {
                cfma_conj(d0[rr], aux[vo + rr], yv);
            } else if (mode == 2) {
                d0[rr].x += yv.x * yv.x + yv.y * yv.y;
                cfma_conj(d1[rr], yv, aux[vo + rr]);
            } else if (mode == 3) {
                d0[rr].x += yv.x * yv.x + yv.y * yv.y;
            }
        }
    }
    if (mode == 0) return;
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        for (int o = 16; o > 0; o >>= 1) {
            d0[rr] = cadd(d0[rr], shfl_xor(d0[rr], o));
            d1[rr] = cadd(d1[rr], shfl_xor(d1[rr], o));
        }
        if (lane == 0) {
            dots[((long long)it * R + rr) * 2 + 0] = d0[rr];
            dots[((long long)it * R + rr) * 2 + 1] = d1[rr];
            __threadfence();
        }
    }
    if (fz.st) {
        const SysPlan pl = plan[I.sys];
        fused_scalar_cta<R, kRRows, double>(fz, plan, dots, I.sys, pl.rend - pl.rbeg);
    }
}

// ------------------------------------------------------- K4 vector updates --
// kind 0: init      x = 0, r = r0 = b, p = v = 0;     dots: |b|^2
// kind 1: p-update  p = r + beta (p - omega v)
// kind 2: s-update  s = r - alpha v
// kind 3: x/r       x += alpha p + omega s (times pdiag, when given); r = s - omega t;  dots: |r|^2, <r0, r>
// kind 4: restart   r0 = r (r already b - A x)
template <typename VT, int R>
__global__ void __launch_bounds__(kVRows)
k_vec(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems, const KState* __restrict__ st,
      int kind, const double2* __restrict__ b, VT* __restrict__ bx, VT* __restrict__ x, VT* __restrict__ r,
      VT* __restrict__ r0, VT* __restrict__ p, VT* __restrict__ v, VT* __restrict__ s, const VT* __restrict__ t,
      double2* __restrict__ dots, const SysPlan* __restrict__ plan = nullptr, ScalarFuse fz = ScalarFuse(),
      const double2* __restrict__ pdiag = nullptr) {
    const int it = blockIdx.x;
    if (it >= nitems) {
        pdl_wait();
        return;
    }
    const Item I = items[it];   // prologue on plan data
    const gb::SysDev S = sys[I.sys];
    pdl_wait();
    pdl_trigger();
    const int mask = (kind == 0) ? -1 : (kind == 4 ? 1 : 0);
    if (!any_active<R>(st, I.sys, mask)) return;
    using C = typename Arith<VT>::C;
    using T = typename Arith<VT>::T;
    const T tg{};
    __shared__ DotAcc<T> red[kVRows / 32][R][2];
    const int lr = threadIdx.x;
    DotAcc<T> d0[R], d1[R];
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        d0[rr].zero();
        d1[rr].zero();
    }
    if (lr < I.nr) {
        const long long vo = S.vec_off + (long long)(I.r0 + lr) * R;
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            if (!active_rhs<R>(st, I.sys, rr, mask)) continue;
            const long long e = vo + rr;
            const KState& k = st[I.sys * R + rr];
            if (kind == 0) {
                const VT bq = b ? from_d2<VT>(b[e]) : bx[e];
                const VT z = from_c<VT>(czero<C>());
                x[e] = z; p[e] = z; v[e] = z;
                r[e] = bq; r0[e] = bq;
                if (bx && b) bx[e] = bq;
                d0[rr].add_norm2(to_c<C>(bq));
            } else if (kind == 1) {
                const C rv = to_c<C>(r[e]), pv = to_c<C>(p[e]), vv = to_c<C>(v[e]);
                const C bt = cmul(ks_beta(k, tg), csub(pv, cmul(ks_omega(k, tg), vv)));
                p[e] = from_c<VT>(cadd(rv, bt));
            } else if (kind == 2) {
                const C rv = to_c<C>(r[e]), vv = to_c<C>(v[e]);
                s[e] = from_c<VT>(csub(rv, cmul(ks_alpha(k, tg), vv)));
            } else if (kind == 3) {
                const C pv = to_c<C>(p[e]), sv = to_c<C>(s[e]), tv = to_c<C>(t[e]), xv = to_c<C>(x[e]);
                const C ap = cmul(ks_alpha(k, tg), pv), ws = cmul(ks_omega(k, tg), sv), wt = cmul(ks_omega(k, tg), tv);
                C dx = cadd(ap, ws);
                if (pdiag) dx = cmul(dx, to_c<C>(pdiag[S.t_off + I.r0 + lr]));   // x += D (alpha p + omega s)
                x[e] = from_c<VT>(cadd(xv, dx));
                const VT rq = from_c<VT>(csub(sv, wt));
                r[e] = rq;
                const C rd = to_c<C>(rq), r0v = to_c<C>(r0[e]);
                d0[rr].add_norm2(rd);
                d1[rr].fma_conj(r0v, rd);
            } else if (kind == 4) {
                r0[e] = r[e];
            }
        }
    }
    if (kind == 1 || kind == 2 || kind == 4) return;
    const int lane = lr & 31, wid = lr >> 5;
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        for (int o = 16; o > 0; o >>= 1) {
            d0[rr].add(d0[rr].shuffled(o));
            d1[rr].add(d1[rr].shuffled(o));
        }
        if (lane == 0) {
            red[wid][rr][0] = d0[rr];
            red[wid][rr][1] = d1[rr];
        }
    }
    __syncthreads();
    if (lr < R * 2) {
        const int rr = lr >> 1, which = lr & 1;
        DotAcc<T> sm;
        sm.zero();
        for (int w = 0; w < kVRows / 32; w++) sm.add(red[w][rr][which]);
        sm.store(dots + ((long long)it * R + rr) * 2 + which);
    }
    if (fz.st) {
        if (lr < R * 2) __threadfence();   // this thread's partial before the arrival count
        const SysPlan pl = plan[I.sys];
        fused_scalar_cta<R, kVRows, T>(fz, plan, dots, I.sys, pl.vend - pl.vbeg);
    }
}

// ------------------------------------------------------ refinement helpers --
template <int R>
__global__ void k_refine_axpy(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems,
                              const KState* __restrict__ ost, double2* __restrict__ x128, const float2* __restrict__ d,
                              double2* __restrict__ dout) {
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    const int lr = threadIdx.x;
    if (lr >= I.nr) return;
    const long long vo = S.vec_off + (long long)(I.r0 + lr) * R;
    for (int rr = 0; rr < R; rr++) {
        const KState& k = ost[I.sys * R + rr];
        if (k.done) {
            if (dout) dout[vo + rr] = make_double2(0, 0);
            continue;
        }
        const double sc = sqrt(k.rsq);   // the inner solve ran on r / |r| (k_cast_f)
        const float2 dv = d[vo + rr];
        const double2 dd = make_double2(sc * (double)dv.x, sc * (double)dv.y);
        double2 xv = x128[vo + rr];
        xv.x += dd.x;
        xv.y += dd.y;
        x128[vo + rr] = xv;
        if (dout) dout[vo + rr] = dd;   // the correction, for an incremental residual update
    }
}

// outer (refinement) state from the residual's |r|^2 (reduce dots)
template <int R>
__global__ void k_refine_check(const SysPlan* __restrict__ plan, int nsys, KState* __restrict__ ost,
                               const double2* __restrict__ dots, int pass, int max_refine) {
    const int id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (id >= nsys * R) return;
    const int sidx = id / R, rr = id % R;
    KState& k = ost[id];
    if (k.done) return;
    const SysPlan pl = plan[sidx];
    double s = 0;
    for (int it = pl.rbeg + lane; it < pl.rend; it += 32) s += dots[((long long)it * R + rr) * 2].x;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane != 0) return;
    k.rsq = s;
    k.iters = pass;
    if (!isfinite(s)) { k.done = 1; k.status = GB_NAN; return; }
    if (!(s > k.tol2)) { k.done = 1; k.status = GB_OK; return; }
    if (pass > max_refine) { k.done = 1; k.status = GB_NOT_CONVERGED; }
}

// outer state init from |b|^2 (vector dots of k_outer_start)
template <int R>
__global__ void k_outer_init(const SysPlan* __restrict__ plan, int nsys, KState* __restrict__ ost,
                             const double2* __restrict__ dots, double tol) {
    const int id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (id >= nsys * R) return;
    const int sidx = id / R, rr = id % R;
    const SysPlan pl = plan[sidx];
    double s = 0;
    for (int it = pl.vbeg + lane; it < pl.vend; it += 32) s += dots[((long long)it * R + rr) * 2].x;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane != 0) return;
    KState& k = ost[id];
    memset(&k, 0, sizeof(KState));
    k.bsq = s;
    k.tol2 = tol * tol * s;
    k.rsq = s;
    if (!isfinite(s)) {   // non-finite right-hand side
        k.done = 1;
        k.status = GB_NAN;
        return;
    }
    k.done = (s == 0.0) ? 1 : 0;
    k.status = k.done ? GB_OK : ST_RUNNING;
}

// x (FP64) = 0 and |b|^2 partials (vector items)
template <int R>
__global__ void __launch_bounds__(kVRows)
k_outer_start(const gb::SysDev* __restrict__ sys, const Item* __restrict__ items, int nitems,
              const double2* __restrict__ b, double2* __restrict__ x, double2* __restrict__ dots) {
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const Item I = items[it];
    const gb::SysDev S = sys[I.sys];
    __shared__ double red[kVRows / 32][R];
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
        for (int w = 0; w < kVRows / 32; w++) s += red[w][lr];
        dots[((long long)it * R + lr) * 2] = make_double2(s, 0);
        dots[((long long)it * R + lr) * 2 + 1] = make_double2(0, 0);
    }
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

// dst (FP32) = src (FP64), zero for clusters the mask marks done.  With the outer
// (refinement) state as mask, src is the residual r and dst = r / |r|: each inner
// FP32 solve sees a unit right-hand side, whatever the source amplitude, and
// k_refine_axpy scales its correction back by |r|.
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
        const bool off = mask && mask[I.sys * R + rr].done;
        const double sc = mask ? 1.0 / sqrt(mask[I.sys * R + rr].rsq) : 1.0;
        dst[vo + rr] = off ? make_float2(0.f, 0.f) : make_float2(__double2float_rn(v.x * sc), __double2float_rn(v.y * sc));
    }
}

// ================================================================== host ==
struct StripGroup {     // strips [beg, end) of clusters with block size B (one GEMV launch each)
    int B;
    long long beg, end;
};

struct Plan {
    int nsys = 0, R = 1, nv = 0, nr = 0;
    long long nstrips = 0, total_pairs = 0, total_vec = 0, total_t = 0, max_B = 0, cw_elems = 0, cu_elems = 0;
    bool tmat = false;   // general particles: y vectors from per-particle T-matrices (k_yprep_tmat)
    std::vector<StripGroup> groups;
    std::vector<gb::SysDev> sd;
    std::vector<Strip> strips;
    std::vector<Item> vitems, ritems;
    std::vector<SysPlan> sp;
    std::vector<long long> row_strip;
};

void add_items(std::vector<Item>& v, int s, int D, int rows, int& beg, int& end) {
    beg = (int)v.size();
    for (int r0 = 0; r0 < D; r0 += rows) v.push_back(Item{s, r0, std::min(rows, D - r0), 0});
    end = (int)v.size();
}

int build_plan(int nsys, const gb_system* sys, int R, cudaStream_t stream, Plan& P) {
    P.nsys = nsys;
    P.R = R;
    int st = gb::make_sysdev(nsys, sys, stream, P.sd);
    if (st) return st;
    long long pairs = 0;
    for (auto& d : P.sd) {
        pairs += d.P;
        // the block reduce holds one particle block's B x R terms, a thread each
        if (d.B * R > kRBThreads)
            return gb_set_error(GB_UNSUPPORTED, "R = %d right-hand sides need block size B <= %d (lmax %d gives %d)", R,
                                kRBThreads / R, d.lmax, d.B);
    }
    P.total_pairs = pairs;
    const long long warps = (long long)gb::sm_count() * 32;
    const long long J = std::max<long long>(1, std::min<long long>(8, pairs / std::max<long long>(1, 2 * warps)));
    P.sp.resize(nsys);
    long long cw_off = 0, cu_off = 0;
    // clusters in order of block size, so that the strips of one block size are
    // contiguous and each size gets a GEMV launch with its own lane shape
    std::vector<int> order(nsys);
    for (int s = 0; s < nsys; s++) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return P.sd[a].B < P.sd[b].B; });
    for (int s : order) {
        const gb::SysDev& d = P.sd[s];
        if (P.groups.empty() || P.groups.back().B != d.B)
            P.groups.push_back(StripGroup{d.B, (long long)P.strips.size(), (long long)P.strips.size()});
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
        P.groups.back().end = (long long)P.strips.size();
        cw_off += d.P * d.B * R;
        cu_off += ((long long)P.strips.size() - pl.strip_base) * d.B * R;
        add_items(P.vitems, s, d.D, kVRows, pl.vbeg, pl.vend);
        add_items(P.ritems, s, d.D, d.B, pl.rbeg, pl.rend);   // one item per particle block
        P.total_vec = std::max<long long>(P.total_vec, d.vec_off + (long long)d.D * R);
        P.total_t = std::max<long long>(P.total_t, d.t_off + (long long)d.D);
        P.max_B = std::max<long long>(P.max_B, d.B);
    }
    P.nstrips = (long long)P.strips.size();
    P.nv = (int)P.vitems.size();
    P.nr = (int)P.ritems.size();
    P.cw_elems = cw_off;
    P.cu_elems = cu_off;
    return GB_OK;
}

// dense pseudo-cluster (plugin path): one cluster of D rows, no strips
void dense_plan(int D, int R, Plan& P) {
    P.nsys = 1;
    P.R = R;
    gb::SysDev sd{};
    sd.D = D;
    sd.B = D;
    sd.N = 1;
    P.sd.push_back(sd);
    SysPlan sp{};
    add_items(P.vitems, 0, D, kVRows, sp.vbeg, sp.vend);
    add_items(P.ritems, 0, D, kRRows, sp.rbeg, sp.rend);
    P.sp.push_back(sp);
    P.row_strip = {0, 0};
    P.nv = (int)P.vitems.size();
    P.nr = (int)P.ritems.size();
    P.total_vec = (long long)D * R;
    P.max_B = 0;
}

struct WS {
    size_t off_state, off_ostate, off_dots, off_cu, off_cw, off_yu, off_yw, off_vec, off_tx, off_r128, off_r128b,
        off_d128, off_tp, off_blob, total;
};

WS ws_layout(const Plan& P, int prec, bool dense) {
    WS w;
    const int R = P.R;
    const size_t vsz = (prec == GB_PREC_FP64) ? sizeof(double2) : sizeof(float2);
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t r = o; o += (bytes + 255) & ~size_t(255); return r; };
    w.off_state = take(sizeof(KState) * P.nsys * R);
    w.off_ostate = take(sizeof(KState) * P.nsys * R);
    w.off_dots = take(sizeof(double2) * 2 * (size_t)std::max(std::max(P.nv, P.nr), 1) * R);
    if (!dense) {
        w.off_cu = take(sizeof(double2) * (size_t)std::max<long long>(P.cu_elems, 1));
        w.off_cw = take(sizeof(double2) * (size_t)std::max<long long>(P.cw_elems, 1));
        w.off_yu = take(16 * (size_t)P.total_vec);
        w.off_yw = take(16 * (size_t)P.total_vec);
        w.off_tx = take(0);
    } else {
        w.off_cu = w.off_cw = w.off_yu = w.off_yw = take(0);
        w.off_tx = take(sizeof(double2) * (size_t)P.total_vec);
    }
    w.off_vec = take(vsz * (size_t)P.total_vec * 8);   // x r r0 p v s t b
    w.off_r128 = take((prec == GB_PREC_MIXED || prec == GB_PREC_MIXED_FP64RES) ? sizeof(double2) * (size_t)P.total_vec : 0);
    // mixed: the second residual buffer and the correction of the incremental update
    w.off_r128b = take(prec == GB_PREC_MIXED ? sizeof(double2) * (size_t)P.total_vec : 0);
    w.off_d128 = take(prec == GB_PREC_MIXED ? sizeof(double2) * (size_t)P.total_vec : 0);
    w.off_tp = take(dense ? 0 : sizeof(double2) * (size_t)std::max<long long>(P.total_t, 1));   // t D (preconditioned)
    w.off_blob = take(sizeof(gb::SysDev) * P.nsys + sizeof(Strip) * P.nstrips + sizeof(Item) * (P.nv + P.nr) +
                      sizeof(SysPlan) * P.nsys + sizeof(long long) * P.row_strip.size() + sizeof(int) * P.nsys + 256);
    w.total = o;
    return w;
}

struct DevPlan {
    const gb::SysDev* sys;
    const Strip* strips;
    const Item* vitems;
    const Item* ritems;
    const SysPlan* sp;
    const long long* row_strip;
    int* err;   // set by a GEMV whose bounded wait on a copy expired
    int* cnt;   // [nsys] arrival counters of the fused scalar updates (zero between launches)
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
    size_t o_vi = put(P.vitems.data(), sizeof(Item) * P.nv);
    size_t o_ri = put(P.ritems.data(), sizeof(Item) * P.nr);
    size_t o_sp = put(P.sp.data(), sizeof(SysPlan) * P.nsys);
    size_t o_rs = put(P.row_strip.data(), sizeof(long long) * P.row_strip.size());
    const int zeros[4] = {0, 0, 0, 0};
    size_t o_err = put(zeros, sizeof(zeros));
    const std::vector<int> counters(P.nsys, 0);
    size_t o_cnt = put(counters.data(), sizeof(int) * P.nsys);
    unsigned char* dst = base + w.off_blob;
    void* dblob = nullptr;
    int slot = 0;
    int e = gb::stage_acquire(blob.data(), blob.size(), stream, &dblob, &slot);
    if (e) return e;
    GB_CUDA_TRY(cudaMemcpyAsync(dst, dblob, blob.size(), cudaMemcpyDeviceToDevice, stream));
    e = gb::stage_release(slot, stream);
    if (e) return e;
    D.sys = reinterpret_cast<const gb::SysDev*>(dst + o_sys);
    D.strips = reinterpret_cast<const Strip*>(dst + o_str);
    D.vitems = reinterpret_cast<const Item*>(dst + o_vi);
    D.ritems = reinterpret_cast<const Item*>(dst + o_ri);
    D.sp = reinterpret_cast<const SysPlan*>(dst + o_sp);
    D.row_strip = reinterpret_cast<const long long*>(dst + o_rs);
    D.err = reinterpret_cast<int*>(dst + o_err);
    D.cnt = reinterpret_cast<int*>(dst + o_cnt);
    return GB_OK;
}

// Readbacks of solver state go through the thread's pinned buffer, except while
// the no-allocation solve runs on this thread (it must not allocate one).
thread_local bool t_pageable_readback = false;
struct PageableReadback {
    bool prev;
    PageableReadback() : prev(t_pageable_readback) { t_pageable_readback = true; }
    ~PageableReadback() { t_pageable_readback = prev; }
};

int read_state(const DevPlan& D, const KState* dev, int nsr, std::vector<KState>& h, cudaStream_t stream);

// Reads the GEMV error flag back (synchronises the stream).
int check_device_error(const DevPlan& D, cudaStream_t stream) {
    if (t_pageable_readback) {
        int h = 0;
        GB_CUDA_TRY(cudaMemcpyAsync(&h, D.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
        GB_CUDA_TRY(cudaStreamSynchronize(stream));
        if (h) return gb_set_error(GB_TIMEOUT, "a GEMV copy did not complete within its wait limit");
        return GB_OK;
    }
    int* h = static_cast<int*>(gb::host_readback(sizeof(int)));
    if (!h) return gb_set_error(GB_CUDA_ERROR, "no pinned readback buffer");
    GB_CUDA_TRY(cudaMemcpyAsync(h, D.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    GB_CUDA_TRY(cudaStreamSynchronize(stream));
    if (*h) return gb_set_error(GB_TIMEOUT, "a GEMV copy did not complete within its wait limit");
    return GB_OK;
}

// --------------------------------------------------- GEMV launch selection --
struct Shape { int lpr, cpl; };

// Lanes per row and columns per lane for a block size: the fewest idle lanes
// (LPR*CPL >= Bmax), ties to more columns per lane.
constexpr Shape kShapes[] = {{8, 1}, {8, 2}, {8, 4}, {16, 3}, {16, 5}, {32, 3}, {32, 4}, {32, 5}};

Shape pick_shape(int Bmax) {
    Shape best{0, 0};
    double beff = -1;
    for (const Shape& c : kShapes) {
        if (c.lpr * c.cpl < Bmax) continue;
        const double eff = double(Bmax) / (c.lpr * c.cpl);
        if (eff > beff + 1e-9 || (std::fabs(eff - beff) < 1e-9 && c.cpl > best.cpl)) { beff = eff; best = c; }
    }
    return best;
}

// A lane reads columns up to LPR*CPL - 1 of every row; past a block's last column
// those reads land in the next row, the next stage or, after a warp's last stage,
// the kGemvPad bytes of padding that gemv_layout adds.  A shape may overshoot the
// block by no more than that padding (the model's shapes overshoot by at most
// 10 elements of 16 B).
constexpr int kGemvPad = 256;
inline bool shape_fits(const Shape& c, int B, int elem_bytes) {
    return c.lpr * c.cpl >= B && (c.lpr * c.cpl - B) * elem_bytes <= kGemvPad;
}

// Shapes measured by gb_autotune_gemv, per (block size, policy, RR, RT); the model
// above where none was measured.
std::mutex g_tune_mu;
std::map<std::array<int, 4>, Shape> g_tuned;

Shape tuned_shape(int B, int pol, int RR, int RT) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto f = g_tuned.find({B, pol, RR, RT});
    return f != g_tuned.end() ? f->second : pick_shape(B);
}

// Steps per chunk for a shape: chunks of about 6 KB of matrix for the block size
// the shape is made for (LPR*CPL columns); with three stages and two y slots per
// warp, two 4-warp CTAs share an SM.  (3 KB chunks with three CTAs per SM, and a
// fourth stage, measured no faster for the complex64 pass and 7 % slower for the
// compute-bound double-float pass, whose longer unrolled steps help.)
constexpr int gemv_steps(int lpr, int cpl, int elem_bytes) {
    return (6144 / ((32 / lpr) * lpr * cpl * elem_bytes)) < 1 ? 1
           : (6144 / ((32 / lpr) * lpr * cpl * elem_bytes)) > 8 ? 8
                                                                : 6144 / ((32 / lpr) * lpr * cpl * elem_bytes);
}

template <class Pol, int RR, int RT>
int launch_pgemv_group(const Plan& P, const DevPlan& D, const StripGroup& grp, const KState* st, int mask,
                       const void* mat_hi, const void* mat_lo, const void* Yu, const void* Yw, void* CU, void* CW,
                       int rr0, int* err, cudaStream_t stream, const Shape* force = nullptr) {
    using YT = typename Pol::YT;
    using OutT = typename Pol::OutT;
    constexpr int S = 3;   // stages per warp: one being read, two in flight
    const int Bmax = grp.B;
    // the double-float pass keeps the model's shape: launch_df splits the right-hand
    // sides by that shape's width
    const Shape sh = force ? *force : (Pol::DF ? pick_shape(Bmax) : tuned_shape(Bmax, Pol::ID, RR, RT));
    if (sh.lpr == 0) return gb_set_error(GB_UNSUPPORTED, "no GEMV shape for block size %d", Bmax);
    if (!shape_fits(sh, Bmax, Pol::MB))
        return gb_set_error(GB_UNSUPPORTED, "GEMV shape %dx%d overruns the %d-column block's padding", sh.lpr, sh.cpl,
                            Bmax);
    const int rpw = 32 / sh.lpr;
    const int G = gemv_steps(sh.lpr, sh.cpl, Pol::MB * (Pol::DF ? 2 : 1));
    const GemvLayout g = gemv_layout(Bmax, G * rpw, RT, S, Pol::MB, Pol::DF, sizeof(YT));
    const size_t smem = (size_t)kGemvWarps * g.warp_bytes;
    if (smem > 227 * 1024) return gb_set_error(GB_UNSUPPORTED, "GEMV needs %zu B of shared memory", smem);
    const long long n = grp.end - grp.beg;
    // one strip per warp (no persistent loop): CTAs retire after their strips, so
    // kernels of higher-priority streams are dispatched between them
    const long long grid = std::max<long long>(1, std::min<long long>((n * 32 + kGemvThreads - 1) / kGemvThreads,
                                                                      0x7fffffffLL));
#define GB_PG(LPRV, CPLV)                                                                                        \
    if (sh.lpr == LPRV && sh.cpl == CPLV) {                                                                      \
        constexpr int GV = gemv_steps(LPRV, CPLV, Pol::MB * (Pol::DF ? 2 : 1));                                  \
        auto kfn = k_pgemv<Pol, RR, RT, LPRV, CPLV, GV, S>;                                                      \
        if (smem > 48 * 1024)                                                                                    \
            GB_CUDA_TRY(gb::ensure_dynamic_smem(reinterpret_cast<const void*>(kfn), smem));      \
        gb::note_launch();                                                                                       \
        GB_CUDA_TRY(launch_pdl(kfn, dim3((unsigned)grid), dim3(kGemvThreads), smem, stream, D.sys, D.strips,    \
                               grp.beg, grp.end, st, mask, mat_hi, mat_lo, reinterpret_cast<const YT*>(Yu),        \
                               reinterpret_cast<const YT*>(Yw), reinterpret_cast<OutT*>(CU),                      \
                               reinterpret_cast<OutT*>(CW), D.sp, rr0, Bmax, err));                               \
        return GB_OK;                                                                                            \
    }
    GB_PG(8, 1) GB_PG(8, 2) GB_PG(8, 4) GB_PG(16, 3) GB_PG(16, 5) GB_PG(32, 3) GB_PG(32, 4) GB_PG(32, 5)
#undef GB_PG
    return gb_set_error(GB_UNSUPPORTED, "no GEMV shape for block size %d", Bmax);
}

// The matrix pass: one launch per block-size group of the batch, each with the
// lane shape of its block size.
template <class Pol, int RR, int RT>
int launch_pgemv(const Plan& P, const DevPlan& D, const KState* st, int mask, const void* mat_hi, const void* mat_lo,
                 const void* Yu, const void* Yw, void* CU, void* CW, int rr0, int* err, cudaStream_t stream) {
    // bulk copies need 16-byte aligned sources (block sizes are even, so offsets keep it)
    if ((reinterpret_cast<uintptr_t>(mat_hi) | reinterpret_cast<uintptr_t>(mat_lo) | reinterpret_cast<uintptr_t>(Yu) |
         reinterpret_cast<uintptr_t>(Yw)) & 15)
        return gb_set_error(GB_BAD_ARG, "matrix and workspace pointers must be 16-byte aligned");
    for (const StripGroup& grp : P.groups) {
        if (grp.end == grp.beg) continue;
        const int e = launch_pgemv_group<Pol, RR, RT>(P, D, grp, st, mask, mat_hi, mat_lo, Yu, Yw, CU, CW, rr0, err,
                                                      stream);
        if (e) return e;
    }
    return GB_OK;
}

// CUDA-core pass for R right-hand sides: one launch for R <= 2; for R = 4 or 8 one
// launch per pair of right-hand sides (the accumulators of more would not stay in
// registers), each a full matrix pass.
template <class Pol, int R>
int launch_pgemv_all(const Plan& P, const DevPlan& D, const KState* st, int mask, const void* mat_hi,
                     const void* Yu, const void* Yw, void* CU, void* CW, cudaStream_t stream) {
    if constexpr (R <= 2) {
        return launch_pgemv<Pol, R, R>(P, D, st, mask, mat_hi, nullptr, Yu, Yw, CU, CW, 0, D.err, stream);
    } else {
        for (int rr = 0; rr < R; rr += 2) {
            const int e = launch_pgemv<Pol, 2, R>(P, D, st, mask, mat_hi, nullptr, Yu, Yw, CU, CW, rr, D.err, stream);
            if (e) return e;
        }
        return GB_OK;
    }
}

// Double-float pass for R right-hand sides: one launch for both of R = 2, or one per
// right-hand side where the wide shapes (5 columns per lane) would not keep two
// sets of double-float accumulators in registers, and one per pair or per
// right-hand side for R = 4 or 8.
template <int R>
int launch_df(const Plan& P, const DevPlan& D, const KState* st, int mask, const void* hi, const void* lo,
              const void* Yu, const void* Yw, void* CU, void* CW, cudaStream_t stream) {
    if constexpr (R == 1) {
        return launch_pgemv<PolDF, 1, 1>(P, D, st, mask, hi, lo, Yu, Yw, CU, CW, 0, D.err, stream);
    } else {
        bool wide = false;
        for (const StripGroup& grp : P.groups) wide |= pick_shape(grp.B).cpl >= 5;
        if (!wide) {
            if constexpr (R == 2)
                return launch_pgemv<PolDF, 2, 2>(P, D, st, mask, hi, lo, Yu, Yw, CU, CW, 0, D.err, stream);
            for (int rr = 0; rr < R; rr += 2) {
                const int e = launch_pgemv<PolDF, 2, R>(P, D, st, mask, hi, lo, Yu, Yw, CU, CW, rr, D.err, stream);
                if (e) return e;
            }
            return GB_OK;
        }
        for (int rr = 0; rr < R; rr++) {
            const int e = launch_pgemv<PolDF, 1, R>(P, D, st, mask, hi, lo, Yu, Yw, CU, CW, rr, D.err, stream);
            if (e) return e;
        }
        return GB_OK;
    }
}

// Tensor-core pass (gemv_tc.cu): one launch per block-size group.
int launch_pgemv_tcore(const Plan& P, const DevPlan& D, int R, const KState* st, int mask, const void* mat_tc,
                       const void* Yu, const void* Yw, void* CU, void* CW, cudaStream_t stream) {
    for (const StripGroup& grp : P.groups) {
        if (grp.end == grp.beg) continue;
        const int e = gb::launch_pgemv_tc(R, D.sys, D.strips, grp.beg, grp.end, st, mask, mat_tc, Yu, Yw, CU, CW, D.sp,
                                          grp.B, D.err, stream);
        if (e) return e;
    }
    return GB_OK;
}

// One product y = (I + T) x (mode 0), or the BiCGSTAB variants (modes 1-3), on the
// packed matrices with arithmetic policy pol: 0 Pol64, 1 Pol32, 2 PolDF, 3 the
// tensor-core pass (mat_hi = the bf16 tiles).  xscale (optional) scales the
// identity's term per row: with tvec = t d and xscale = d the product is (I + T) D x.
template <typename VT, int R>
int launch_apply(const Plan& P, const DevPlan& D, const WS& w, unsigned char* base, const KState* st, int mask,
                 int pol, const void* mat_hi, const void* mat_lo, const double2* tvec, const VT* xin, VT* yout,
                 int mode, const VT* aux, const double2* b128, double2* dots, cudaStream_t stream,
                 ScalarFuse fz = ScalarFuse(), YUpd<VT> up = YUpd<VT>(), const double2* xscale = nullptr) {
    void* Yu = base + w.off_yu;
    void* Yw = base + w.off_yw;
    void* CU = base + w.off_cu;
    void* CW = base + w.off_cw;
    const unsigned vb = (unsigned)P.nv;
    int e = GB_OK;
    if (pol == 0) {
        gb::note_launch();
        if (P.tmat)
            GB_CUDA_TRY(launch_pdl(k_yprep_tmat<0, VT, R>, dim3((unsigned)P.nr), dim3(kRBThreads), 0, stream, D.sys,
                                   D.ritems, P.nr, st, mask, xin, reinterpret_cast<double2*>(Yu),
                                   reinterpret_cast<double2*>(Yw), up));
        else
            GB_CUDA_TRY(launch_pdl(k_yprep<0, VT, R>, dim3(vb), dim3(kVRows), 0, stream, D.sys, D.vitems, P.nv, st,
                                   mask, tvec, xin, reinterpret_cast<double2*>(Yu), reinterpret_cast<double2*>(Yw), up));
        if (P.nstrips) e = launch_pgemv_all<Pol64, R>(P, D, st, mask, mat_hi, Yu, Yw, CU, CW, stream);
        if (e) return e;
        gb::note_launch();
        GB_CUDA_TRY(launch_pdl(k_reduce_blk<double2, VT, R>, dim3((unsigned)P.nr), dim3(kRBThreads), 0, stream, D.sys,
                               D.ritems, P.nr, D.sp, D.row_strip, st, mask, reinterpret_cast<const double2*>(CU),
                               reinterpret_cast<const double2*>(CW), xin, yout, mode, aux, b128, dots, fz, xscale));
    } else if (pol == 1) {
        gb::note_launch();
        if (P.tmat)
            GB_CUDA_TRY(launch_pdl(k_yprep_tmat<1, VT, R>, dim3((unsigned)P.nr), dim3(kRBThreads), 0, stream, D.sys,
                                   D.ritems, P.nr, st, mask, xin, reinterpret_cast<float4*>(Yu),
                                   reinterpret_cast<float4*>(Yw), up));
        else
            GB_CUDA_TRY(launch_pdl(k_yprep<1, VT, R>, dim3(vb), dim3(kVRows), 0, stream, D.sys, D.vitems, P.nv, st,
                                   mask, tvec, xin, reinterpret_cast<float4*>(Yu), reinterpret_cast<float4*>(Yw), up));
        if (P.nstrips) e = launch_pgemv_all<Pol32, R>(P, D, st, mask, mat_hi, Yu, Yw, CU, CW, stream);
        if (e) return e;
        gb::note_launch();
        GB_CUDA_TRY(launch_pdl(k_reduce_blk<float2, VT, R>, dim3((unsigned)P.nr), dim3(kRBThreads), 0, stream, D.sys,
                               D.ritems, P.nr, D.sp, D.row_strip, st, mask, reinterpret_cast<const float2*>(CU),
                               reinterpret_cast<const float2*>(CW), xin, yout, mode, aux, b128, dots, fz, xscale));
    } else if (pol == 3) {   // tensor-core pass on the bf16 tiles (mat_hi): float2 y vectors and partials
        if constexpr (R == 4 || R == 8) {
            if (P.tmat) return gb_set_error(GB_UNSUPPORTED, "the tensor-core pass serves sphere clusters");
            gb::note_launch();
            GB_CUDA_TRY(launch_pdl(k_yprep<3, VT, R>, dim3(vb), dim3(kVRows), 0, stream, D.sys, D.vitems, P.nv, st,
                                   mask, tvec, xin, reinterpret_cast<float2*>(Yu), reinterpret_cast<float2*>(Yw), up));
            if (P.nstrips) e = launch_pgemv_tcore(P, D, R, st, mask, mat_hi, Yu, Yw, CU, CW, stream);
            if (e) return e;
            gb::note_launch();
            GB_CUDA_TRY(launch_pdl(k_reduce_blk<float2, VT, R>, dim3((unsigned)P.nr), dim3(kRBThreads), 0, stream,
                                   D.sys, D.ritems, P.nr, D.sp, D.row_strip, st, mask,
                                   reinterpret_cast<const float2*>(CU), reinterpret_cast<const float2*>(CW), xin, yout,
                                   mode, aux, b128, dots, fz, xscale));
        } else {
            return gb_set_error(GB_UNSUPPORTED, "the tensor-core pass needs R = 4 or 8 (got %d)", R);
        }
    } else {
        gb::note_launch();
        if (P.tmat)
            GB_CUDA_TRY(launch_pdl(k_yprep_tmat<2, VT, R>, dim3((unsigned)P.nr), dim3(kRBThreads), 0, stream, D.sys,
                                   D.ritems, P.nr, st, mask, xin, reinterpret_cast<float4*>(Yu),
                                   reinterpret_cast<float4*>(Yw), up));
        else
            GB_CUDA_TRY(launch_pdl(k_yprep<2, VT, R>, dim3(vb), dim3(kVRows), 0, stream, D.sys, D.vitems, P.nv, st,
                                   mask, tvec, xin, reinterpret_cast<float4*>(Yu), reinterpret_cast<float4*>(Yw), up));
        if (P.nstrips) e = launch_df<R>(P, D, st, mask, mat_hi, mat_lo, Yu, Yw, CU, CW, stream);
        if (e) return e;
        gb::note_launch();
        GB_CUDA_TRY(launch_pdl(k_reduce_blk<float4, VT, R>, dim3((unsigned)P.nr), dim3(kRBThreads), 0, stream, D.sys,
                               D.ritems, P.nr, D.sp, D.row_strip, st, mask, reinterpret_cast<const float4*>(CU),
                               reinterpret_cast<const float4*>(CW), xin, yout, mode, aux, b128, dots, fz, xscale));
    }
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

// ----------------------------------------------------------- graph cache --
struct GraphKey {
    const void* a[12];
    long long n[10];
    bool operator==(const GraphKey& o) const { return memcmp(this, &o, sizeof(GraphKey)) == 0; }
};
struct GraphKeyHash {
    size_t operator()(const GraphKey& k) const {
        const unsigned char* p = reinterpret_cast<const unsigned char*>(&k);
        size_t h = 1469598103934665603ull;
        for (size_t i = 0; i < sizeof(GraphKey); i++) h = (h ^ p[i]) * 1099511628211ull;
        return h;
    }
};
struct GraphEntry {
    cudaGraphExec_t exec;
    long long kernels;        // kernel nodes per replay
    int inuse;                // solves replaying it right now (other host threads included)
    unsigned long long last;  // use stamp, for eviction of the least recently used
};
struct GraphCache {
    std::mutex mu;
    std::unordered_map<GraphKey, GraphEntry, GraphKeyHash> map;
    unsigned long long clock = 0;
    // drop least recently used graphs that no solve is replaying, down to keep entries
    void evict(size_t keep) {
        while (map.size() > keep) {
            auto victim = map.end();
            for (auto it = map.begin(); it != map.end(); ++it)
                if (it->second.inuse == 0 && (victim == map.end() || it->second.last < victim->second.last)) victim = it;
            if (victim == map.end()) return;
            cudaGraphExecDestroy(victim->second.exec);
            map.erase(victim);
        }
    }
};
GraphCache g_graphs;

// Marks a cached graph in use for the lifetime of one solve.
struct GraphUse {
    GraphKey key{};
    bool held = false;
    ~GraphUse() {
        if (!held) return;
        std::lock_guard<std::mutex> lk(g_graphs.mu);
        auto f = g_graphs.map.find(key);
        if (f != g_graphs.map.end()) f->second.inuse--;
    }
};

// FNV-1a over the block-size groups of a plan (each group is one GEMV launch in a graph)
long long groups_hash(const Plan& P) {
    unsigned long long h = 1469598103934665603ull;
    for (const StripGroup& g : P.groups) {
        const long long v[3] = {g.B, g.beg, g.end};
        const unsigned char* b = reinterpret_cast<const unsigned char*>(v);
        for (size_t i = 0; i < sizeof(v); i++) h = (h ^ b[i]) * 1099511628211ull;
    }
    return (long long)h;
}

// Capture stream of the calling host thread on the current device: concurrent
// solves on different host threads capture on different streams.
cudaStream_t capture_stream() {
    thread_local cudaStream_t cap[64] = {nullptr};
    int dev = 0;
    cudaGetDevice(&dev);
    if (!cap[dev & 63]) cudaStreamCreateWithFlags(&cap[dev & 63], cudaStreamNonBlocking);
    return cap[dev & 63];
}

// ------------------------------------------------------------- BiCGSTAB run --
// Runs BiCGSTAB on vectors of type VT (double2 with pol 0 or dense, float2 with
// pol 1) until every (cluster, rhs) is done.  The right-hand side is b128 (FP64) or,
// when null, bvt.  The solution stays in the x vector of the workspace.
// pdiag (packed path, optional): a diagonal right preconditioner D (one complex
// factor per row, at t_off like tvec), and tvec_p = tvec * D: the iteration's
// products are (I + T) D p = D p + A diag(t D) p, x is updated by D (alpha p + omega
// s) (Eigen's BiCGSTAB with a preconditioner); restart residuals use (I + T) itself.
template <typename VT, int R, bool DENSE>
int run_bicgstab(const Plan& P, const DevPlan& D, const WS& w, unsigned char* base, int pol, const void* mat,
                 const double2* tvec, const double2* b128, VT* bvt, double tol, int maxiter, KState* st, int dense_D,
                 cudaStream_t stream, bool use_graph, const double2* pdiag = nullptr,
                 const double2* tvec_p = nullptr) {
    static_assert(!DENSE || std::is_same<VT, double2>::value, "the dense path runs FP64 vectors");
    const size_t TV = (size_t)P.total_vec;
    VT* V = reinterpret_cast<VT*>(base + w.off_vec);
    VT *x = V, *r = V + TV, *r0 = V + 2 * TV, *p = V + 3 * TV, *v = V + 4 * TV, *s = V + 5 * TV, *t = V + 6 * TV,
       *bx = V + 7 * TV;
    double2* dots = reinterpret_cast<double2*>(base + w.off_dots);
    double2* Tx = reinterpret_cast<double2*>(base + w.off_tx);
    const int nsr = P.nsys * R;
    const unsigned sblocks = (unsigned)((nsr * 32 + 127) / 128);
    const unsigned vb = (unsigned)P.nv;

    auto fuse = [&](int phase) {
        ScalarFuse f;
        f.st = st;
        f.cnt = D.cnt;
        f.phase = phase;
        f.tol = tol;
        f.maxiter = maxiter;
        return f;
    };
    auto apply = [&](const VT* xin, VT* yout, int mode, const VT* aux, int mask, const double2* bb,
                     cudaStream_t sm, ScalarFuse fz = ScalarFuse(), YUpd<VT> up = YUpd<VT>()) -> int {
        if constexpr (DENSE) {
            const long long grid = std::min<long long>(((long long)dense_D * 32 + 255) / 256, (long long)gb::sm_count() * 8);
            gb::note_launch();
            k_dense_gemv<R><<<(unsigned)std::max<long long>(grid, 1), 256, 0, sm>>>(
                dense_D, reinterpret_cast<const double2*>(mat), reinterpret_cast<const double2*>(xin), Tx);
            GB_CUDA_TRY(cudaGetLastError());
            gb::note_launch();
            k_reduce_dense<R><<<(unsigned)P.nr, kRRows, 0, sm>>>(D.sys, D.ritems, P.nr, D.sp, st, mask, Tx, xin, yout,
                                                               mode, aux, bb, dots, fz);
            GB_CUDA_TRY(cudaGetLastError());
            return GB_OK;
        }
        const bool pre = pdiag && mode != 3;   // the restart residual is b - (I + T) x
        return launch_apply<VT, R>(P, D, w, base, st, mask, pol, mat, nullptr, pre ? tvec_p : tvec, xin, yout, mode,
                                   aux, bb, dots, sm, fz, up, pre ? pdiag : nullptr);
    };
    // One iteration: p-update + v = A p (+ alpha), s-update + t = A s (+ omega),
    // x/r update (+ convergence, beta).  On the packed path the vector updates run
    // inside the y-vector preparation of the product that reads them, and each
    // scalar update inside the kernel that produces its dots (last CTA per cluster):
    // 7 launches per iteration.  The dense path keeps the p- and s-update kernels.
    auto iteration = [&](cudaStream_t sm) -> int {
        int e;
        if (DENSE) {
            gb::note_launch();
            k_vec<VT, R><<<vb, kVRows, 0, sm>>>(D.sys, D.vitems, P.nv, st, 1, nullptr, nullptr, x, r, r0, p, v, s, t,
                                                dots);
            e = apply(p, v, 1, r0, 0, nullptr, sm, fuse(1));
            if (e) return e;
            gb::note_launch();
            k_vec<VT, R><<<vb, kVRows, 0, sm>>>(D.sys, D.vitems, P.nv, st, 2, nullptr, nullptr, x, r, r0, p, v, s, t,
                                                dots);
            e = apply(s, t, 2, s, 0, nullptr, sm, fuse(2));
            if (e) return e;
        } else {
            YUpd<VT> up1;
            up1.kind = 1; up1.r = r; up1.v = v; up1.out = p;
            e = apply(p, v, 1, r0, 0, nullptr, sm, fuse(1), up1);
            if (e) return e;
            YUpd<VT> up2;
            up2.kind = 2; up2.r = r; up2.v = v; up2.out = s;
            e = apply(s, t, 2, s, 0, nullptr, sm, fuse(2), up2);
            if (e) return e;
        }
        gb::note_launch();
        GB_CUDA_TRY(launch_pdl(k_vec<VT, R>, dim3(vb), dim3(kVRows), 0, sm, D.sys, D.vitems, P.nv, st, 3, nullptr,
                               nullptr, x, r, r0, p, v, s, t, dots, D.sp, fuse(3), pdiag));
        GB_CUDA_TRY(cudaGetLastError());
        return GB_OK;
    };

    // init: x = 0, r = r0 = b, scalars
    gb::note_launch();
    k_vec<VT, R><<<vb, kVRows, 0, stream>>>(D.sys, D.vitems, P.nv, st, 0, b128, bvt ? bvt : bx, x, r, r0, p, v, s, t,
                                            dots, D.sp, fuse(0));
    GB_CUDA_TRY(cudaGetLastError());
    const VT* bsrc_vt = bvt ? bvt : bx;

    // chunks of nit iterations (kChunk, and single iterations for the tail of a
    // solve), captured once per argument set and replayed
    auto acquire = [&](int nit, GraphUse& use, cudaGraphExec_t& exec, long long& exec_kernels) -> int {
        GraphKey key{};
        const void* a[12] = {base, mat, tvec, D.sys, D.strips, D.vitems, D.ritems, D.sp, st, pdiag, tvec_p, nullptr};
        memcpy(key.a, a, sizeof(a));
        key.n[0] = P.nsys;
        key.n[1] = R | (pol << 8) | ((DENSE ? 1 : 0) << 16) | ((long long)sizeof(VT) << 24) | ((long long)P.tmat << 40);
        key.n[2] = P.nstrips;
        key.n[3] = P.nv | ((long long)P.nr << 32);
        memcpy(&key.n[4], &tol, sizeof(double));
        key.n[5] = maxiter | ((long long)dense_D << 32);
        key.n[6] = P.max_B;
        key.n[7] = P.total_vec;
        key.n[8] = groups_hash(P);
        key.n[9] = nit;
        use.key = key;
        {
            std::lock_guard<std::mutex> lk(g_graphs.mu);
            auto f = g_graphs.map.find(key);
            if (f != g_graphs.map.end()) {
                exec = f->second.exec;
                exec_kernels = f->second.kernels;
                f->second.inuse++;
                f->second.last = ++g_graphs.clock;
                use.held = true;
                return GB_OK;
            }
        }
        cudaStream_t cs = capture_stream();
        GB_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        gb::capture_begin();
        int e = GB_OK;
        for (int itn = 0; itn < nit && e == GB_OK; itn++) e = iteration(cs);
        exec_kernels = gb::capture_end();
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(cs, &g);
        if (e) {
            if (g) cudaGraphDestroy(g);
            return e;
        }
        if (ce != cudaSuccess) return gb_set_cuda_error(ce, "capture of BiCGSTAB chunk", __FILE__, __LINE__);
        ce = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return gb_set_cuda_error(ce, "instantiate BiCGSTAB graph", __FILE__, __LINE__);
        std::lock_guard<std::mutex> lk(g_graphs.mu);
        g_graphs.evict(255);   // bounded cache
        auto f = g_graphs.map.find(key);
        if (f != g_graphs.map.end()) {   // another thread built the same graph meanwhile
            cudaGraphExecDestroy(exec);
            exec = f->second.exec;
            exec_kernels = f->second.kernels;
            f->second.inuse++;
            f->second.last = ++g_graphs.clock;
        } else {
            g_graphs.map[key] = GraphEntry{exec, exec_kernels, 1, ++g_graphs.clock};
        }
        use.held = true;
        return GB_OK;
    };
    cudaGraphExec_t exec = nullptr, exec1 = nullptr;
    long long exec_kernels = 0, exec1_kernels = 0;
    GraphUse use, use1;
    if (use_graph) {
        const int e = acquire(kChunk, use, exec, exec_kernels);
        if (e) return e;
    }
    // iterations still needed by the slowest running cluster, from its mean
    // per-iteration residual reduction so far (kChunk when there is no estimate)
    auto predict = [&](const std::vector<KState>& h) -> int {
        int need = 1;
        for (int q = 0; q < nsr; q++) {
            const KState& k = h[q];
            if (k.done) continue;
            const bool f32 = std::is_same<VT, float2>::value;
            const double rs = f32 ? (double)k.rsq_f : k.rsq, r0 = f32 ? (double)k.r0sq_f : k.r0sq;
            const double t2 = tol * tol * (f32 ? (double)k.bsq_f : k.bsq);
            if (k.restarts > 0 || k.iters < 1 || !(rs > 0) || !(r0 > rs) || !(t2 > 0)) return kChunk;
            const double rate = std::log(rs / r0) / k.iters;   // log reduction of |r|^2 per iteration (< 0)
            const double n = std::ceil(std::log(t2 / rs) / rate);
            if (!(n < kChunk)) return kChunk;
            need = std::max(need, (int)std::max(1.0, n));
        }
        return need;
    };
    std::vector<KState> hst(nsr);
    // every restart may reset the count once, and a chunk holds at least one
    // iteration; bound the chunks accordingly
    const long long max_chunks = ((long long)maxiter + 2) * (kMaxRestarts + 2) + 16;
    int next = kChunk;   // iterations before the next host check
    for (long long chunk = 0; chunk < max_chunks; chunk++) {
        if (exec && next == kChunk) {
            GB_CUDA_TRY(cudaGraphLaunch(exec, stream));
            gb::note_launches(exec_kernels);
        } else if (exec) {
            if (!exec1) {
                const int e = acquire(1, use1, exec1, exec1_kernels);
                if (e) return e;
            }
            for (int itn = 0; itn < next; itn++) {
                GB_CUDA_TRY(cudaGraphLaunch(exec1, stream));
                gb::note_launches(exec1_kernels);
            }
        } else {
            for (int itn = 0; itn < next; itn++) {
                int e = iteration(stream);
                if (e) return e;
            }
        }
        {
            const int e = read_state(D, st, nsr, hst, stream);
            if (e) return e;
        }
        bool all_done = true, restart = false;
        for (int q = 0; q < nsr; q++) {
            if (!hst[q].done) all_done = false;
            if (hst[q].need_restart) restart = true;
        }
        if (restart) {   // r = b - A x for the restarting clusters, r0 = r, rho = |r|^2
            int e = apply(x, r, 3, bsrc_vt, 1, b128, stream);
            if (e) return e;
            gb::note_launch();
            k_vec<VT, R><<<vb, kVRows, 0, stream>>>(D.sys, D.vitems, P.nv, st, 4, nullptr, nullptr, x, r, r0, p, v, s,
                                                    t, dots);
            gb::note_launch();
            k_scalar<R, typename Arith<VT>::T><<<sblocks, 128, 0, stream>>>(D.sp, P.nsys, st, 4, dots, tol, maxiter);
            GB_CUDA_TRY(cudaGetLastError());
            next = kChunk;
            continue;
        }
        if (all_done) return GB_OK;
        next = predict(hst);
    }
    return gb_set_error(GB_TIMEOUT, "BiCGSTAB driver exceeded its iteration bound");
}

int finish_status(const KState* h, int nsr, int* status, int* iters, double* resid) {
    int worst = GB_OK;
    for (int q = 0; q < nsr; q++) {
        if (status) status[q] = h[q].status;
        if (iters) iters[q] = h[q].iters;
        if (resid) resid[q] = h[q].bsq > 0 ? std::sqrt(h[q].rsq / h[q].bsq) : 0.0;
        if (h[q].status != GB_OK && worst == GB_OK) worst = h[q].status;
    }
    return worst;
}

// The scalars of every (cluster, rhs) and the GEMV error flag, through this thread's
// pinned readback buffer (synchronises the stream).
int read_state(const DevPlan& D, const KState* dev, int nsr, std::vector<KState>& h, cudaStream_t stream) {
    h.resize(nsr);
    const size_t kb = sizeof(KState) * (size_t)nsr;
    if (t_pageable_readback) {
        int herr = 0;
        GB_CUDA_TRY(cudaMemcpyAsync(h.data(), dev, kb, cudaMemcpyDeviceToHost, stream));
        GB_CUDA_TRY(cudaMemcpyAsync(&herr, D.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
        GB_CUDA_TRY(cudaStreamSynchronize(stream));
        if (herr) return gb_set_error(GB_TIMEOUT, "a GEMV copy did not complete within its wait limit");
        return GB_OK;
    }
    unsigned char* pin = static_cast<unsigned char*>(gb::host_readback(kb + 16));
    if (!pin) return gb_set_error(GB_CUDA_ERROR, "no pinned readback buffer");
    int* herr = reinterpret_cast<int*>(pin + kb);
    GB_CUDA_TRY(cudaMemcpyAsync(pin, dev, kb, cudaMemcpyDeviceToHost, stream));
    GB_CUDA_TRY(cudaMemcpyAsync(herr, D.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    GB_CUDA_TRY(cudaStreamSynchronize(stream));
    if (*herr) return gb_set_error(GB_TIMEOUT, "a GEMV copy did not complete within its wait limit");
    memcpy(h.data(), pin, kb);
    return GB_OK;
}

// out[e] = t[e] d[e] over the Mie-factor arena (the preconditioned products' factors)
__global__ void k_scale_t(const double2* __restrict__ t, const double2* __restrict__ d, double2* __restrict__ out,
                          long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        out[e] = cmul(t[e], d[e]);
}

// pdiag (optional): the diagonal right preconditioner of run_bicgstab for every
// BiCGSTAB of the solve (the mixed method's refinement residuals stay unpreconditioned).
// mat_tc (optional, R = 4 or 8): the bf16 tiles of the tensor-core pass, used for
// the products of the FP32 solves (the FP32 method, and the inner solves of the
// mixed method); the refinement residuals keep the CUDA-core passes.
template <int R>
int solve_impl(const Plan& P, int prec, double tol, int maxiter, double inner_tol, int max_refine,
               const double* mat128, const float* mat64, const float* mat64lo, const double* tvec, const double* b,
               double* x, unsigned char* base, const WS& w, int* status, int* iters, double* resid,
               cudaStream_t stream, const void* mat_tc = nullptr, const double* pdiag = nullptr) {
    const int pol32 = mat_tc ? 3 : 1;
    const void* m32 = mat_tc ? mat_tc : static_cast<const void*>(mat64);
    DevPlan D;
    int e = upload_plan(P, base, w, stream, D);
    if (e) return e;
    const double2* pd = reinterpret_cast<const double2*>(pdiag);
    double2* tp = nullptr;
    if (pd) {
        tp = reinterpret_cast<double2*>(base + w.off_tp);
        gb::note_launch();
        k_scale_t<<<(unsigned)std::min<long long>((P.total_t + 255) / 256, 4096), 256, 0, stream>>>(
            reinterpret_cast<const double2*>(tvec), pd, tp, P.total_t);
        GB_CUDA_TRY(cudaGetLastError());
    }
    KState* st = reinterpret_cast<KState*>(base + w.off_state);
    KState* ost = reinterpret_cast<KState*>(base + w.off_ostate);
    const double2* t2 = reinterpret_cast<const double2*>(tvec);
    const double2* b2 = reinterpret_cast<const double2*>(b);
    double2* x2 = reinterpret_cast<double2*>(x);
    const size_t TV = (size_t)P.total_vec;
    const int nsr = P.nsys * R;
    const unsigned vb = (unsigned)P.nv;
    std::vector<KState> h;
    if (prec == GB_PREC_FP64) {
        e = run_bicgstab<double2, R, false>(P, D, w, base, 0, mat128, t2, b2, nullptr, tol, maxiter, st, 0, stream, true,
                                            pd, tp);
        if (e) return e;
        gb::note_launch();
        k_copy_out<double2><<<vb, kVRows, 0, stream>>>(D.sys, D.vitems, P.nv, R,
                                                       reinterpret_cast<double2*>(base + w.off_vec), x2);
        GB_CUDA_TRY(cudaGetLastError());
        e = read_state(D, st, nsr, h, stream);
        if (e) return e;
        return finish_status(h.data(), nsr, status, iters, resid);
    }
    float2* V = reinterpret_cast<float2*>(base + w.off_vec);
    float2* bx = V + 7 * TV;
    if (prec == GB_PREC_FP32) {
        e = run_bicgstab<float2, R, false>(P, D, w, base, pol32, m32, t2, b2, nullptr, tol, maxiter, st, 0, stream,
                                           true, pd, tp);
        if (e) return e;
        gb::note_launch();
        k_copy_out<float2><<<vb, kVRows, 0, stream>>>(D.sys, D.vitems, P.nv, R, V, x2);
        GB_CUDA_TRY(cudaGetLastError());
        e = read_state(D, st, nsr, h, stream);
        if (e) return e;
        return finish_status(h.data(), nsr, status, iters, resid);
    }
    // mixed: x = 0, r = b (FP64); repeat { FP32 BiCGSTAB on (I + T) d = r; x += d;
    // r = b - (I + T) x in double-float (or FP64), or r -= (I + T) d with the
    // complex64 matrix once |r| is small enough (kIncrTheta) }
    double2* r128 = reinterpret_cast<double2*>(base + w.off_r128);
    double2* r_nxt = prec == GB_PREC_MIXED ? reinterpret_cast<double2*>(base + w.off_r128b) : nullptr;
    double2* d128 = prec == GB_PREC_MIXED ? reinterpret_cast<double2*>(base + w.off_d128) : nullptr;
    double2* dots = reinterpret_cast<double2*>(base + w.off_dots);
    bool incr = prec == GB_PREC_MIXED && kIncrTheta * tol >= 1.0;   // first pass: |r| = |b|
    gb::note_launch();
    k_outer_start<R><<<vb, kVRows, 0, stream>>>(D.sys, D.vitems, P.nv, b2, x2, dots);
    gb::note_launch();
    k_outer_init<R><<<(nsr * 32 + 127) / 128, 128, 0, stream>>>(D.sp, P.nsys, ost, dots, tol);
    GB_CUDA_TRY(cudaGetLastError());
    GB_CUDA_TRY(cudaMemcpyAsync(r128, b2, sizeof(double2) * TV, cudaMemcpyDeviceToDevice, stream));
    for (int pass = 1; pass <= max_refine + 1; pass++) {
        gb::note_launch();
        k_cast_f<<<vb, kVRows, 0, stream>>>(D.sys, D.vitems, P.nv, R, r128, bx, ost);
        GB_CUDA_TRY(cudaGetLastError());
        e = run_bicgstab<float2, R, false>(P, D, w, base, pol32, m32, t2, nullptr, bx, inner_tol, maxiter, st, 0,
                                           stream, true, pd, tp);
        if (e) return e;
        gb::note_launch();
        k_refine_axpy<R><<<vb, kVRows, 0, stream>>>(D.sys, D.vitems, P.nv, ost, x2, V, incr ? d128 : nullptr);
        GB_CUDA_TRY(cudaGetLastError());
        if (incr) {   // r_nxt = r - (d + T d), complex64 matrix, FP64 vectors
            e = launch_apply<double2, R>(P, D, w, base, ost, -1, 1, mat64, nullptr, t2, d128, r_nxt, 3, nullptr, r128,
                                         dots, stream);
            std::swap(r128, r_nxt);
        } else if (prec == GB_PREC_MIXED)
            e = launch_apply<double2, R>(P, D, w, base, ost, -1, 2, mat64, mat64lo, t2, x2, r128, 3, nullptr, b2, dots,
                                         stream);
        else
            e = launch_apply<double2, R>(P, D, w, base, ost, -1, 0, mat128, nullptr, t2, x2, r128, 3, nullptr, b2,
                                         dots, stream);
        if (e) return e;
        gb::note_launch();
        k_refine_check<R><<<(nsr * 32 + 127) / 128, 128, 0, stream>>>(D.sp, P.nsys, ost, dots, pass, max_refine);
        GB_CUDA_TRY(cudaGetLastError());
        e = read_state(D, ost, nsr, h, stream);
        if (e) return e;
        bool all = true;
        for (int q = 0; q < nsr; q++) all &= (h[q].done != 0);
        if (all) break;
        if (prec == GB_PREC_MIXED) {   // the next update may be incremental if every running |r| is small
            incr = true;
            for (int q = 0; q < nsr; q++)
                if (!h[q].done && !(h[q].rsq <= kIncrTheta * kIncrTheta * h[q].tol2)) incr = false;
        }
    }
    return finish_status(h.data(), nsr, status, iters, resid);
}

bool prec_ok(int prec, const double* m128, const float* m64, const float* m64lo) {
    switch (prec) {
        case GB_PREC_FP64: return m128 != nullptr;
        case GB_PREC_FP32: return m64 != nullptr;
        case GB_PREC_MIXED: return m64 && m64lo;
        case GB_PREC_MIXED_FP64RES: return m64 && m128;
        default: return false;
    }
}

#ifndef GB_SOLVE_MULTI_RHS   // (the R = 4 / 8 unit carries no scratch array)
// ------------------------------------------- dense solve without allocation --
// Scratch of gb_solve_dense_noalloc: a fixed device array that the library's module
// brings with it, so that callers that must not allocate device memory (a server
// whose HBM is fully reserved up front, a real-time loop where cudaMalloc/cudaFree
// would synchronise the device) can still solve.  Enough for D * R <= 8192.
constexpr size_t kNoAllocScratchBytes = 1280u * 1024u;
constexpr long long kNoAllocMaxDR = 8192;

}   // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

// Device address of the scratch array in the current device's context.  Looked up
// on every call (a host-side table lookup once the module is loaded; the first
// call on a device may load the module there), so that an address never outlives
// the context it belongs to (cudaDeviceReset, a context torn down and recreated).
int noalloc_scratch(unsigned char** out) {
    void* p = nullptr;
    GB_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    *out = static_cast<unsigned char*>(p);
    return GB_OK;
}

// Plan upload for the scratch array: the same blob as upload_plan, copied straight
// from ordinary host memory (no pinned staging buffer, which would be allocated on
// first use).  The blob carries the zeroed GEMV error flag.
int upload_plan_pageable(const Plan& P, unsigned char* base, const WS& w, cudaStream_t stream, DevPlan& D) {
    std::vector<unsigned char> blob;
    auto put = [&](const void* src, size_t bytes) {
        size_t off = blob.size();
        blob.resize(off + ((bytes + 15) & ~size_t(15)));
        if (bytes) memcpy(blob.data() + off, src, bytes);
        return off;
    };
    size_t o_sys = put(P.sd.data(), sizeof(gb::SysDev) * P.nsys);
    size_t o_str = put(P.strips.data(), sizeof(Strip) * P.nstrips);
    size_t o_vi = put(P.vitems.data(), sizeof(Item) * P.nv);
    size_t o_ri = put(P.ritems.data(), sizeof(Item) * P.nr);
    size_t o_sp = put(P.sp.data(), sizeof(SysPlan) * P.nsys);
    size_t o_rs = put(P.row_strip.data(), sizeof(long long) * P.row_strip.size());
    const int zeros[4] = {0, 0, 0, 0};
    size_t o_err = put(zeros, sizeof(zeros));
    const std::vector<int> counters(P.nsys, 0);
    size_t o_cnt = put(counters.data(), sizeof(int) * P.nsys);
    unsigned char* dst = base + w.off_blob;
    // from pageable memory: returns once the blob has been taken, so it may go out of scope
    GB_CUDA_TRY(cudaMemcpyAsync(dst, blob.data(), blob.size(), cudaMemcpyHostToDevice, stream));
    D.sys = reinterpret_cast<const gb::SysDev*>(dst + o_sys);
    D.strips = reinterpret_cast<const Strip*>(dst + o_str);
    D.vitems = reinterpret_cast<const Item*>(dst + o_vi);
    D.ritems = reinterpret_cast<const Item*>(dst + o_ri);
    D.sp = reinterpret_cast<const SysPlan*>(dst + o_sp);
    D.row_strip = reinterpret_cast<const long long*>(dst + o_rs);
    D.err = reinterpret_cast<int*>(dst + o_err);
    D.cnt = reinterpret_cast<int*>(dst + o_cnt);
    return GB_OK;
}
#endif

// y = (I + T) x for FP64 vectors x, y.  prec: GB_PREC_FP64 (complex128 pass),
// GB_PREC_MIXED (double-float pass), GB_PREC_FP32 (complex64 pass, or the
// tensor-core pass when mat_tc is given, on a rounded copy of x, widened to FP64).
// repeat 0: one product; 1: reps products back to back; 2: one product, then the
// matrix pass alone reps - 1 more times (kernel timing).
template <int R>
int apply_impl(const Plan& P, int prec, const double* mat128, const float* mat64, const float* mat64lo,
               const void* mat_tc, const double* tvec, const double* x, double* y, unsigned char* base, const WS& w,
               int reps, int repeat, cudaStream_t s) {
    DevPlan D;
    int e = upload_plan(P, base, w, s, D);
    if (e) return e;
    KState* st = reinterpret_cast<KState*>(base + w.off_state);
    const double2* x2 = reinterpret_cast<const double2*>(x);
    double2* y2 = reinterpret_cast<double2*>(y);
    double2* dots = reinterpret_cast<double2*>(base + w.off_dots);
    const double2* t2 = reinterpret_cast<const double2*>(tvec);
    const unsigned vb = (unsigned)P.nv;
    const int pol = mat_tc ? 3 : (prec == GB_PREC_FP64 ? 0 : (prec == GB_PREC_MIXED ? 2 : 1));
    const void* hi = pol == 3 ? mat_tc : (pol == 0 ? (const void*)mat128 : (const void*)mat64);
    const void* lo = pol == 2 ? (const void*)mat64lo : nullptr;
    void* Yu = base + w.off_yu;
    void* Yw = base + w.off_yw;
    void* CU = base + w.off_cu;
    void* CW = base + w.off_cw;
    auto pass = [&]() -> int {   // the matrix pass alone, on the y vectors of the first product
        switch (pol) {
            case 0: return launch_pgemv_all<Pol64, R>(P, D, st, -1, hi, Yu, Yw, CU, CW, s);
            case 1: return launch_pgemv_all<Pol32, R>(P, D, st, -1, hi, Yu, Yw, CU, CW, s);
            case 2: return launch_df<R>(P, D, st, -1, hi, lo, Yu, Yw, CU, CW, s);
            default: return launch_pgemv_tcore(P, D, R, st, -1, hi, Yu, Yw, CU, CW, s);
        }
    };
    const int n = repeat == 0 ? 1 : reps;
    if (pol == 0 || pol == 2) {
        for (int k = 0; k < n; k++) {
            e = (k > 0 && repeat == 2) ? pass()
                                       : launch_apply<double2, R>(P, D, w, base, st, -1, pol, hi, lo, t2, x2, y2, 0,
                                                                  nullptr, nullptr, dots, s);
            if (e) return e;
        }
        return check_device_error(D, s);
    }
    // FP32 product on a rounded copy of x, widened to FP64
    const size_t TV = (size_t)P.total_vec;
    float2* V = reinterpret_cast<float2*>(base + w.off_vec);
    float2 *xf = V, *yf = V + TV;
    gb::note_launch();
    k_cast_f<<<vb, kVRows, 0, s>>>(D.sys, D.vitems, P.nv, R, x2, xf, nullptr);
    GB_CUDA_TRY(cudaGetLastError());
    for (int k = 0; k < n; k++) {
        e = (k > 0 && repeat == 2) ? pass()
                                   : launch_apply<float2, R>(P, D, w, base, st, -1, pol, hi, nullptr, t2, xf, yf, 0,
                                                             nullptr, nullptr, dots, s);
        if (e) return e;
    }
    gb::note_launch();
    k_copy_out<float2><<<vb, kVRows, 0, s>>>(D.sys, D.vitems, P.nv, R, yf, y2);
    GB_CUDA_TRY(cudaGetLastError());
    return check_device_error(D, s);
}

int apply_entry(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                const float* mat64lo, const void* mat_tc, const double* tvec, const double* x, double* y,
                void* workspace, size_t ws_bytes, int reps, int repeat, cudaStream_t s) {
    if (R != 1 && R != 2 && R != 4 && R != 8) return gb_set_error(GB_UNSUPPORTED, "R must be 1, 2, 4 or 8 (got %d)", R);
#ifndef GB_SOLVE_MULTI_RHS
    if (R > 2)
        return gb::apply_entry_multi(nsys, sys, R, prec, mat128, mat64, mat64lo, mat_tc, tvec, x, y, workspace, ws_bytes,
                                     reps, repeat, s);
#endif
    if (prec == GB_PREC_MIXED_FP64RES) prec = GB_PREC_FP64;
    Plan P;
    int e = build_plan(nsys, sys, R, s, P);
    if (e) return e;
    WS w = ws_layout(P, prec, false);
    if (ws_bytes < w.total) return gb_set_error(GB_OVER_BUDGET, "workspace %zu B < required %zu B", ws_bytes, w.total);
    unsigned char* base = static_cast<unsigned char*>(workspace);
#ifndef GB_SOLVE_MULTI_RHS
    if (R == 1) return apply_impl<1>(P, prec, mat128, mat64, mat64lo, nullptr, tvec, x, y, base, w, reps, repeat, s);
    return apply_impl<2>(P, prec, mat128, mat64, mat64lo, nullptr, tvec, x, y, base, w, reps, repeat, s);
#else
    if (R == 4) return apply_impl<4>(P, prec, mat128, mat64, mat64lo, mat_tc, tvec, x, y, base, w, reps, repeat, s);
    return apply_impl<8>(P, prec, mat128, mat64, mat64lo, mat_tc, tvec, x, y, base, w, reps, repeat, s);
#endif
}

// Validation, plan and dispatch of a packed-operator solve (gb_solve_batch_ex).
int solve_entry(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter, double inner_tol,
                int max_refine, const double* mat128, const float* mat64, const float* mat64lo, const void* mat_tc,
                const double* pdiag, const double* tvec, const double* b, double* x, void* workspace, size_t ws_bytes,
                int* status, int* iters, double* resid, cudaStream_t s) {
    if (nsys < 1 || !sys || !tvec || !b || !x || !workspace) return gb_set_error(GB_BAD_ARG, "null argument");
    if (R != 1 && R != 2 && R != 4 && R != 8) return gb_set_error(GB_UNSUPPORTED, "R must be 1, 2, 4 or 8 (got %d)", R);
    if (!prec_ok(prec, mat128, mat64, mat64lo))
        return gb_set_error(GB_BAD_ARG, "precision %d is missing one of its matrices", prec);
    if (mat_tc && (R < 4 || (prec != GB_PREC_FP32 && prec != GB_PREC_MIXED)))
        return gb_set_error(GB_UNSUPPORTED, "the tensor-core pass serves the FP32 and mixed methods with R = 4 or 8");
    if (!(tol > 0) || maxiter < 1) return gb_set_error(GB_BAD_ARG, "tol must be > 0 and maxiter >= 1");
#ifndef GB_SOLVE_MULTI_RHS
    if (R > 2)
        return gb::solve_entry_multi(nsys, sys, R, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo,
                                     mat_tc, pdiag, tvec, b, x, workspace, ws_bytes, status, iters, resid, s);
#endif
    Plan P;
    int e = build_plan(nsys, sys, R, s, P);
    if (e) return e;
    WS w = ws_layout(P, prec, false);
    if (ws_bytes < w.total) return gb_set_error(GB_OVER_BUDGET, "workspace %zu B < required %zu B", ws_bytes, w.total);
    unsigned char* base = static_cast<unsigned char*>(workspace);
    if (inner_tol <= 0) inner_tol = 1e-6;
#ifndef GB_SOLVE_MULTI_RHS
    if (R == 1)
        return solve_impl<1>(P, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo, tvec, b, x, base, w,
                             status, iters, resid, s, nullptr, pdiag);
    return solve_impl<2>(P, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo, tvec, b, x, base, w,
                         status, iters, resid, s, nullptr, pdiag);
#else
    if (R == 4)
        return solve_impl<4>(P, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo, tvec, b, x, base, w,
                             status, iters, resid, s, mat_tc, pdiag);
    return solve_impl<8>(P, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo, tvec, b, x, base, w,
                         status, iters, resid, s, mat_tc, pdiag);
#endif
}

}   // namespace

#ifndef GB_SOLVE_MULTI_RHS
extern "C" {

size_t gb_solve_workspace_size(int nsys, const gb_system* sys, int R, int prec) {
    Plan P;
    if (build_plan(nsys, sys, R, 0, P)) return 0;
    return ws_layout(P, prec, false).total;
}

int gb_solve_batch(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter, double inner_tol,
                   int max_refine, const double* mat128, const float* mat64, const float* mat64lo, const double* tvec,
                   const double* b, double* x, void* workspace, size_t ws_bytes, int* status, int* iters,
                   double* resid, void* stream) {
    return gb_solve_batch_ex(nsys, sys, R, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo, nullptr,
                             nullptr, tvec, b, x, workspace, ws_bytes, status, iters, resid, stream);
}

int gb_solve_batch_ex(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter, double inner_tol,
                      int max_refine, const double* mat128, const float* mat64, const float* mat64lo,
                      const void* mat_tc, const double* pdiag, const double* tvec, const double* b, double* x,
                      void* workspace, size_t ws_bytes, int* status, int* iters, double* resid, void* stream) {
    return solve_entry(nsys, sys, R, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo, mat_tc, pdiag,
                       tvec, b, x, workspace, ws_bytes, status, iters, resid, (cudaStream_t)stream);
}

int gb_solve_batch_tmatrix(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter,
                           double inner_tol, int max_refine, const double* mat128, const float* mat64,
                           const float* mat64lo, const double* tmat128, const float* tmat64, const int64_t* tm_off,
                           const double* b, double* x, void* workspace, size_t ws_bytes, int* status, int* iters,
                           double* resid, void* stream) {
    if (nsys < 1 || !sys || !tm_off || !b || !x || !workspace) return gb_set_error(GB_BAD_ARG, "null argument");
    if (R != 1 && R != 2) return gb_set_error(GB_UNSUPPORTED, "R must be 1 or 2 (got %d)", R);
    if (!prec_ok(prec, mat128, mat64, mat64lo))
        return gb_set_error(GB_BAD_ARG, "precision %d is missing one of its matrices", prec);
    const bool need128 = prec != GB_PREC_FP32, need64 = prec != GB_PREC_FP64;
    if ((need128 && !tmat128) || (need64 && !tmat64))
        return gb_set_error(GB_BAD_ARG, "precision %d needs the %s T-matrices", prec, need128 ? "complex128" : "complex64");
    if (!(tol > 0) || maxiter < 1) return gb_set_error(GB_BAD_ARG, "tol must be > 0 and maxiter >= 1");
    cudaStream_t s = (cudaStream_t)stream;
    Plan P;
    int e = build_plan(nsys, sys, R, s, P);
    if (e) return e;
    for (int q = 0; q < nsys; q++) {
        if (P.sd[q].B * R > kRBThreads) return gb_set_error(GB_UNSUPPORTED, "T-matrix clusters need lmax <= 8");
        if (tmat128) P.sd[q].tmat128 = reinterpret_cast<const double2*>(tmat128) + tm_off[q];
        if (tmat64) P.sd[q].tmat64 = reinterpret_cast<const float2*>(tmat64) + tm_off[q];
    }
    P.tmat = true;
    WS w = ws_layout(P, prec, false);
    if (ws_bytes < w.total) return gb_set_error(GB_OVER_BUDGET, "workspace %zu B < required %zu B", ws_bytes, w.total);
    unsigned char* base = static_cast<unsigned char*>(workspace);
    if (inner_tol <= 0) inner_tol = 1e-6;
    if (R == 1)
        return solve_impl<1>(P, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo, nullptr, b, x, base, w,
                             status, iters, resid, s);
    return solve_impl<2>(P, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo, nullptr, b, x, base, w,
                         status, iters, resid, s);
}

// Measured GEMV shapes: for every block-size group of the batch, each lane shape
// that covers the block (LPR * CPL >= B) runs reps matrix passes on the batch's own
// plan and matrices, timed with events; the fastest is kept for that (block size,
// policy, R) in a process-wide table that later launches read.  Run outside stream
// capture (the graphs of a solve keep the shapes they were captured with).
int gb_autotune_gemv(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                     const double* tvec, const double* x, double* y, void* workspace, size_t ws_bytes, int reps,
                     void* stream) {
    if (nsys < 1 || !sys || !tvec || !x || !y || !workspace || reps < 1) return gb_set_error(GB_BAD_ARG, "bad argument");
    if (R != 1 && R != 2) return gb_set_error(GB_UNSUPPORTED, "R must be 1 or 2 (got %d)", R);
    const bool f64 = prec == GB_PREC_FP64;
    if ((f64 && !mat128) || (!f64 && !mat64)) return gb_set_error(GB_BAD_ARG, "matrix missing for precision %d", prec);
    const int aprec = f64 ? GB_PREC_FP64 : GB_PREC_FP32;
    cudaStream_t s = (cudaStream_t)stream;
    Plan P;
    int e = build_plan(nsys, sys, R, s, P);
    if (e) return e;
    WS w = ws_layout(P, aprec, false);
    if (ws_bytes < w.total) return gb_set_error(GB_OVER_BUDGET, "workspace %zu B < required %zu B", ws_bytes, w.total);
    unsigned char* base = static_cast<unsigned char*>(workspace);
    DevPlan D;
    e = upload_plan(P, base, w, s, D);
    if (e) return e;
    KState* st = reinterpret_cast<KState*>(base + w.off_state);
    double2* dots = reinterpret_cast<double2*>(base + w.off_dots);
    const int pol = f64 ? 0 : 1;
    const void* hi = f64 ? (const void*)mat128 : (const void*)mat64;
    // one product prepares the y vectors the passes read
    e = R == 1 ? launch_apply<double2, 1>(P, D, w, base, st, -1, pol, hi, nullptr, reinterpret_cast<const double2*>(tvec),
                                          reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(y), 0,
                                          nullptr, nullptr, dots, s)
               : launch_apply<double2, 2>(P, D, w, base, st, -1, pol, hi, nullptr, reinterpret_cast<const double2*>(tvec),
                                          reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(y), 0,
                                          nullptr, nullptr, dots, s);
    if (e) return e;
    void* Yu = base + w.off_yu;
    void* Yw = base + w.off_yw;
    void* CU = base + w.off_cu;
    void* CW = base + w.off_cw;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    GB_CUDA_TRY(cudaEventCreate(&e0));
    GB_CUDA_TRY(cudaEventCreate(&e1));
    auto pass = [&](const StripGroup& grp, const Shape& c) -> int {
        if (f64)
            return R == 1 ? launch_pgemv_group<Pol64, 1, 1>(P, D, grp, st, -1, hi, nullptr, Yu, Yw, CU, CW, 0, D.err, s, &c)
                          : launch_pgemv_group<Pol64, 2, 2>(P, D, grp, st, -1, hi, nullptr, Yu, Yw, CU, CW, 0, D.err, s, &c);
        return R == 1 ? launch_pgemv_group<Pol32, 1, 1>(P, D, grp, st, -1, hi, nullptr, Yu, Yw, CU, CW, 0, D.err, s, &c)
                      : launch_pgemv_group<Pol32, 2, 2>(P, D, grp, st, -1, hi, nullptr, Yu, Yw, CU, CW, 0, D.err, s, &c);
    };
    for (const StripGroup& grp : P.groups) {
        if (grp.end == grp.beg) continue;
        Shape best{0, 0};
        float tbest = 0;
        for (const Shape& c : kShapes) {
            if (!shape_fits(c, grp.B, f64 ? Pol64::MB : Pol32::MB)) continue;
            e = pass(grp, c);   // warm-up (also rejects a shape whose shared memory does not fit)
            if (e == GB_UNSUPPORTED) continue;
            if (e) break;
            GB_CUDA_TRY(cudaEventRecord(e0, s));
            for (int k = 0; k < reps && !e; k++) e = pass(grp, c);
            if (e) break;
            GB_CUDA_TRY(cudaEventRecord(e1, s));
            GB_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0;
            GB_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            if (best.lpr == 0 || ms < tbest) { best = c; tbest = ms; }
        }
        if (e) break;
        if (best.lpr) {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tuned[{grp.B, pol, R, R}] = best;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e) return e;
    return check_device_error(D, s);
}

// The shape GEMV launches use for block size B, policy (0 complex128, 1 complex64)
// and R right-hand sides: the measured one, or the model's.
int gb_gemv_shape(int B, int prec, int R, int* lanes_per_row, int* cols_per_lane) {
    if (!lanes_per_row || !cols_per_lane || B < 1) return gb_set_error(GB_BAD_ARG, "bad argument");
    const Shape sh = tuned_shape(B, prec == GB_PREC_FP64 ? 0 : 1, R, R);
    *lanes_per_row = sh.lpr;
    *cols_per_lane = sh.cpl;
    return sh.lpr ? GB_OK : gb_set_error(GB_UNSUPPORTED, "no GEMV shape for block size %d", B);
}

size_t gb_apply_workspace_size(int nsys, const gb_system* sys, int R, int prec) {
    return gb_solve_workspace_size(nsys, sys, R, prec);
}

int gb_apply_batch(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                   const float* mat64lo, const double* tvec, const double* x, double* y, void* workspace,
                   size_t ws_bytes, void* stream) {
    if (nsys < 1 || !sys || !tvec || !x || !y || !workspace) return gb_set_error(GB_BAD_ARG, "null argument");
    if (!prec_ok(prec, mat128, mat64, mat64lo)) return gb_set_error(GB_BAD_ARG, "matrix missing for precision %d", prec);
    return apply_entry(nsys, sys, R, prec, mat128, mat64, mat64lo, nullptr, tvec, x, y, workspace, ws_bytes, 1, 0,
                       (cudaStream_t)stream);
}

int gb_apply_repeat(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                    const float* mat64lo, const double* tvec, const double* x, double* y, void* workspace,
                    size_t ws_bytes, int reps, int gemv_only, void* stream) {
    if (nsys < 1 || !sys || !tvec || !x || !y || !workspace || reps < 1) return gb_set_error(GB_BAD_ARG, "bad argument");
    if (!prec_ok(prec, mat128, mat64, mat64lo)) return gb_set_error(GB_BAD_ARG, "matrix missing for precision %d", prec);
    return apply_entry(nsys, sys, R, prec, mat128, mat64, mat64lo, nullptr, tvec, x, y, workspace, ws_bytes, reps,
                       gemv_only ? 2 : 1, (cudaStream_t)stream);
}

int gb_apply_repeat_tc(int nsys, const gb_system* sys, int R, const void* mat_tc, const double* tvec, const double* x,
                       double* y, void* workspace, size_t ws_bytes, int reps, int gemv_only, void* stream) {
    if (nsys < 1 || !sys || !mat_tc || !tvec || !x || !y || !workspace || reps < 1)
        return gb_set_error(GB_BAD_ARG, "bad argument");
    if (R != 4 && R != 8) return gb_set_error(GB_UNSUPPORTED, "the tensor-core pass needs R = 4 or 8 (got %d)", R);
    return apply_entry(nsys, sys, R, GB_PREC_FP32, nullptr, nullptr, nullptr, mat_tc, tvec, x, y, workspace, ws_bytes,
                       reps, gemv_only ? 2 : 1, (cudaStream_t)stream);
}

int gb_set_gemv_wait_limit(long long cycles, long long* previous) {
    long long old = 0;
    GB_CUDA_TRY(cudaMemcpyFromSymbol(&old, g_gemv_wait_cycles, sizeof(old)));
    const long long v = cycles < 0 ? kWaitCycles : cycles;
    GB_CUDA_TRY(cudaMemcpyToSymbol(g_gemv_wait_cycles, &v, sizeof(v)));
    const int e = gb::set_wait_limit_multi(v);   // the copy of the R = 4 / 8 unit
    if (e) return e;
    if (previous) *previous = old;
    return GB_OK;
}

size_t gb_solve_dense_workspace_size(int D, int R) {
    Plan P;
    dense_plan(D, R, P);
    return ws_layout(P, GB_PREC_FP64, true).total;
}

int gb_solve_dense(int D, int R, const double* T, const double* b, double* x, double tol, int maxiter,
                   void* workspace, size_t ws_bytes, int* status, int* iters, double* resid, void* stream) {
    if (D < 1 || !T || !b || !x || !workspace) return gb_set_error(GB_BAD_ARG, "null argument");
    if (R != 1 && R != 2) return gb_set_error(GB_UNSUPPORTED, "R must be 1 or 2 (got %d)", R);
    if (!(tol > 0) || maxiter < 1) return gb_set_error(GB_BAD_ARG, "tol must be > 0 and maxiter >= 1");
    cudaStream_t s = (cudaStream_t)stream;
    Plan P;
    dense_plan(D, R, P);
    WS w = ws_layout(P, GB_PREC_FP64, true);
    if (ws_bytes < w.total) return gb_set_error(GB_OVER_BUDGET, "workspace %zu B < required %zu B", ws_bytes, w.total);
    unsigned char* base = static_cast<unsigned char*>(workspace);
    DevPlan Dp;
    int e = upload_plan(P, base, w, s, Dp);
    if (e) return e;
    KState* st = reinterpret_cast<KState*>(base + w.off_state);
    if (R == 1)
        e = run_bicgstab<double2, 1, true>(P, Dp, w, base, 0, T, nullptr, reinterpret_cast<const double2*>(b), nullptr,
                                           tol, maxiter, st, D, s, false);
    else
        e = run_bicgstab<double2, 2, true>(P, Dp, w, base, 0, T, nullptr, reinterpret_cast<const double2*>(b), nullptr,
                                           tol, maxiter, st, D, s, false);
    if (e) return e;
    gb::note_launch();
    k_copy_out<double2><<<(unsigned)P.nv, kVRows, 0, s>>>(Dp.sys, Dp.vitems, P.nv, R,
                                                          reinterpret_cast<double2*>(base + w.off_vec),
                                                          reinterpret_cast<double2*>(x));
    GB_CUDA_TRY(cudaGetLastError());
    std::vector<KState> h;
    e = read_state(Dp, st, P.nsys * R, h, s);
    if (e) return e;
    return finish_status(h.data(), P.nsys * R, status, iters, resid);
}

int gb_solve_dense_noalloc(int D, int R, const double* T, const double* b, double* x, double tol, int maxiter,
                           int* status, int* iters, double* resid, void* stream) {
    if (D < 1 || !T || !b || !x) return gb_set_error(GB_BAD_ARG, "null argument");
    if (R != 1 && R != 2) return gb_set_error(GB_UNSUPPORTED, "R must be 1 or 2 (got %d)", R);
    if (!(tol > 0) || maxiter < 1) return gb_set_error(GB_BAD_ARG, "tol must be > 0 and maxiter >= 1");
    if ((long long)D * R > kNoAllocMaxDR)
        return gb_set_error(GB_OVER_BUDGET, "D * R = %lld exceeds the no-allocation solve's limit of %lld",
                            (long long)D * R, kNoAllocMaxDR);
    cudaStream_t s = (cudaStream_t)stream;
    const PageableReadback pageable;   // no pinned readback buffer either
    Plan P;
    dense_plan(D, R, P);
    WS w = ws_layout(P, GB_PREC_FP64, true);
    if (w.total > kNoAllocScratchBytes)
        return gb_set_error(GB_OVER_BUDGET, "D = %d, R = %d needs %zu B of scratch; the fixed array holds %zu B", D, R,
                            w.total, kNoAllocScratchBytes);
    unsigned char* base = nullptr;
    int e = noalloc_scratch(&base);
    if (e) return e;
    DevPlan Dp;
    e = upload_plan_pageable(P, base, w, s, Dp);
    if (e) return e;
    // every other scratch region is written before it is read (x0 = 0, r = b and
    // the iteration scalars are set by the first kernels of the solve)
    KState* st = reinterpret_cast<KState*>(base + w.off_state);
    if (R == 1)
        e = run_bicgstab<double2, 1, true>(P, Dp, w, base, 0, T, nullptr, reinterpret_cast<const double2*>(b), nullptr,
                                           tol, maxiter, st, D, s, false);
    else
        e = run_bicgstab<double2, 2, true>(P, Dp, w, base, 0, T, nullptr, reinterpret_cast<const double2*>(b), nullptr,
                                           tol, maxiter, st, D, s, false);
    if (e) return e;
    gb::note_launch();
    k_copy_out<double2><<<(unsigned)P.nv, kVRows, 0, s>>>(Dp.sys, Dp.vitems, P.nv, R,
                                                          reinterpret_cast<double2*>(base + w.off_vec),
                                                          reinterpret_cast<double2*>(x));
    GB_CUDA_TRY(cudaGetLastError());
    std::vector<KState> h;
    e = read_state(Dp, st, P.nsys * R, h, s);
    if (e) return e;
    return finish_status(h.data(), P.nsys * R, status, iters, resid);
}

}   // extern "C"
#else   // GB_SOLVE_MULTI_RHS: the R = 4 and 8 instantiations, reached from the main unit

namespace gb {

int solve_entry_multi(int nsys, const gb_system* sys, int R, int prec, double tol, int maxiter, double inner_tol,
                      int max_refine, const double* mat128, const float* mat64, const float* mat64lo,
                      const void* mat_tc, const double* pdiag, const double* tvec, const double* b, double* x,
                      void* workspace, size_t ws_bytes, int* status, int* iters, double* resid, cudaStream_t stream) {
    return solve_entry(nsys, sys, R, prec, tol, maxiter, inner_tol, max_refine, mat128, mat64, mat64lo, mat_tc, pdiag,
                       tvec, b, x, workspace, ws_bytes, status, iters, resid, stream);
}

int apply_entry_multi(int nsys, const gb_system* sys, int R, int prec, const double* mat128, const float* mat64,
                      const float* mat64lo, const void* mat_tc, const double* tvec, const double* x, double* y,
                      void* workspace, size_t ws_bytes, int reps, int repeat, cudaStream_t stream) {
    return apply_entry(nsys, sys, R, prec, mat128, mat64, mat64lo, mat_tc, tvec, x, y, workspace, ws_bytes, reps,
                       repeat, stream);
}

int set_wait_limit_multi(long long cycles) {
    GB_CUDA_TRY(cudaMemcpyToSymbol(g_gemv_wait_cycles, &cycles, sizeof(cycles)));
    return GB_OK;
}

}   // namespace gb
#endif
