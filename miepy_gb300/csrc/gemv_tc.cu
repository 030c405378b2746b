// Tensor-core (tcgen05) matrix pass of the packed operator, for blocks of R = 4 or
// 8 right-hand sides (polarisations x sources) of the FP32 inner solves.
//
// Replaces, for multi-RHS blocks, the row-block GEMV of the reference's
// solve_linear_system (cpp/src/interactions.cpp:70-92, ParallelDenseMatrix::
// scaleAndAddTo): with R right-hand sides a pass streams each matrix block once and
// multiplies it by 2R vectors (the block serves both block rows, see solve.cu), so
// the CUDA-core FP32 pipe runs out before HBM does; the tensor cores do not.
//
// Arithmetic: split-BF16x3.  Each complex64 matrix element a is held as two bf16
// planes, hi = bf16(a) and lo = bf16(a - hi) per real component (k_tc_tiles, once
// per assembly), and each vector element z likewise; the product is
// A_hi z_hi + A_hi z_lo + A_lo z_hi, accumulated in FP32 in tensor memory: about
// 5e-6 relative to the largest term, against 4e-7 for complex64 arithmetic.  The
// mixed method's FP32 inner solves (to 1e-4) use it; its refinement residuals keep
// the CUDA-core complex64 and double-float passes.
//
// A complex block product as one real GEMM: A is [B rows][2B real columns] (re, im
// interleaved along K); a complex vector z becomes two real B-operand rows,
// (re z, -im z) giving re(A z) and (im z, re z) giving im(A z).  One MMA per K-step
// multiplies A_hi by N = 8R rows [U_h | W_h | U_l | W_l] and a second A_lo by the
// first 4R, into one accumulator of N FP32 columns:
//   U = A z_j (row product of block (i, j), summed along the strip),
//   W = A w_i (column product, one partial per block), w_i = S z_i,
// with z[s] = eps(s) y[rho(s)] formed from the solver's y vectors, and the results
// stored as the CUDA-core pass stores its column sums, C[rho(r)] = eps(r) (A z)[r],
// so the block reduce that follows is shared.
//
// Pipeline per CTA (160 threads, two CTAs per SM, persistent over strips): a
// producer warp walks the CTA's strips ahead of the others and, per block, writes a
// job record and streams the block's two planes with its y_w (and the strip's y_u
// with its first block) by bulk copies (TMA) into a ring of 3 stages, reusing a stage
// once the MMAs that read it have committed to its empty barrier; the 4 consumer
// warps build the block's B operand (bf16, core-matrix layout) in one of two buffers;
// thread 0 issues the block's MMAs (M = 128: the block's rows, padding rows read and
// discarded) into one of two TMEM accumulators and commits them to mbarriers;
// meanwhile the consumer warps read the previous block's accumulator rows
// (tcgen05.ld), write its column partials and keep the strip's row sums.  Every wait
// is bounded; an expired wait sets the error flag, the consumers decide to stop
// together through a reduction barrier, and the CTA waits (again bounded) for its
// copies and MMAs in flight before it frees its TMEM and exits.

#include <cuda_bf16.h>

#include "gb_common.cuh"
#include "gb_internal.h"
#include "solve_plan.cuh"

namespace {

constexpr int kTcThreads = 160;   // 4 consumer warps + 1 producer warp
constexpr int kTcStages = 3;
constexpr long long kTcWaitCycles = 400000000LL;   // about 0.2 s of SM clock

__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void pdl_wait_tc() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger_tc() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// ----------------------------------------------------------------- mbarrier --
__device__ __forceinline__ void bar_init(uint64_t* b, unsigned n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(su32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_expect_tx(uint64_t* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t* b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool bar_wait(uint64_t* b, unsigned parity) {
    if (bar_try(b, parity)) return true;
    const long long t0 = clock64();
    while (!bar_try(b, parity))
        if (clock64() - t0 > kTcWaitCycles) return false;
    return true;
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes, uint64_t* b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     su32(dst)),
                 "l"(src), "r"(bytes), "r"(su32(b))
                 : "memory");
}
__device__ __forceinline__ void bulk_copy_hint(void* dst, const void* src, unsigned bytes, uint64_t* b, uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;\n" ::"r"(
            su32(dst)),
        "l"(src), "r"(bytes), "r"(su32(b)), "l"(pol)
        : "memory");
}
__device__ __forceinline__ uint64_t evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(pol));
    return pol;
}

// ------------------------------------------------------------------ tcgen05 --
__device__ __forceinline__ void tmem_alloc(unsigned* slot, unsigned ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(slot)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, bf16 inputs, FP32 accumulation (kind::f16)
__device__ __forceinline__ void mma_bf16(unsigned d, uint64_t a, uint64_t b, unsigned idesc, unsigned accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on the mbarrier once every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(su32(b))
                 : "memory");
}
// Shared-memory matrix descriptor, K-major, no swizzle: core matrices of 8 rows x
// 16 bytes; lbo = byte step between core matrices along K, sbo = along M (or N).
__device__ __forceinline__ uint64_t smem_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator, bf16 A and B, both K-major.
__host__ __device__ constexpr unsigned idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ unsigned bf2(float lo_half, float hi_half) {   // (first, second) in memory order
    __nv_bfloat162 v = __floats2bfloat162_rn(lo_half, hi_half);
    return *reinterpret_cast<unsigned*>(&v);
}
__device__ __forceinline__ float bf_round(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// ------------------------------------------------------------ shared layout --
// Header: S full barriers, 2 MMA barriers, the TMEM address, the abort flag, then S
// job records; the row map at off_row; the two B-operand buffers; S stages, each
// the block's two bf16 planes, its y_u (particle j) and y_w (particle i).
struct TcJob {
    long long cw;    // element offset of the block's column partials in CW
    long long cu;    // element offset of the strip's row partials in CU (last block of a strip), else -1
    int valid;       // 0: no more blocks for this CTA
    int pad;
};
struct TcLayout {
    unsigned sbo, plane, tile, ybytes, stage, bbytes;
    unsigned off_jobs, off_row, off_b, off_stage, total;
};
__host__ __device__ inline TcLayout tc_layout(int B, int R) {
    TcLayout L;
    const int Kp = gb::tc_cols(B), Bp = gb::tc_rows(B);
    L.sbo = (unsigned)Kp * 16u;
    L.plane = (unsigned)(Bp / 8) * L.sbo;
    L.tile = 2u * L.plane;
    L.ybytes = (unsigned)(B * R * 8);
    L.stage = (L.tile + 2u * L.ybytes + 127u) & ~127u;
    L.bbytes = (unsigned)(8 * R) * (unsigned)Kp * 2u;
    L.off_jobs = 128;   // after 2S + 2 barriers, the TMEM slot, the abort flag, the consumed count
    L.off_row = 256;
    L.off_b = 1024;
    L.off_stage = L.off_b + 2u * L.bbytes;
    unsigned end = L.off_stage + (unsigned)kTcStages * L.stage;
    // an M = 128 MMA reads 16 row groups of each plane: the lo plane of the last
    // stage reads up to plane + 16 sbo past that stage's start
    const unsigned reach = L.off_stage + (unsigned)(kTcStages - 1) * L.stage + L.plane + 16u * L.sbo;
    L.total = end > reach ? end : reach;
    return L;
}

// ------------------------------------------------------------- tile builder --
// mat64 [pairs][B][B] complex64 (the assembler's hi plane) -> bf16 hi/lo tiles.
// blockIdx.y = cluster; CTAs stride over its pairs; one thread per (row, 4 complex
// columns): two 16-byte loads, a 16-byte store into each plane.
__global__ void __launch_bounds__(256)
k_tc_tiles(const gb::SysDev* __restrict__ sys, const float2* __restrict__ mat64, unsigned char* __restrict__ out) {
    const gb::SysDev S = sys[blockIdx.y];
    const int B = S.B, Bp = gb::tc_rows(B), Kp = gb::tc_cols(B), KG = Kp / 8;
    const long long plane = gb::tc_plane_bytes(B), blk = gb::tc_block_bytes(B);
    const unsigned sbo = (unsigned)Kp * 16u;
    const int items = Bp * KG;
    for (long long p = blockIdx.x; p < S.P; p += gridDim.x) {
        const float2* src = mat64 + S.mat_off + p * (long long)B * B;
        unsigned char* dst = out + S.tc_off + p * blk;
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
            const int m8 = it & 7, rest = it >> 3, g = rest % KG, m = (rest / KG) * 8 + m8;
            float2 a[4];
            if (m < B && 4 * g + 3 < B) {
                const float4* q = reinterpret_cast<const float4*>(src + (long long)m * B + 4 * g);
                const float4 u = __ldg(q), v = __ldg(q + 1);
                a[0] = make_float2(u.x, u.y);
                a[1] = make_float2(u.z, u.w);
                a[2] = make_float2(v.x, v.y);
                a[3] = make_float2(v.z, v.w);
            } else {
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int c = 4 * g + e;
                    a[e] = (m < B && c < B) ? __ldg(src + (long long)m * B + c) : make_float2(0.f, 0.f);
                }
            }
            uint4 h, l;
            unsigned* hp = &h.x;
            unsigned* lp = &l.x;
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float hr = bf_round(a[e].x), hi = bf_round(a[e].y);
                hp[e] = bf2(hr, hi);
                lp[e] = bf2(a[e].x - hr, a[e].y - hi);
            }
            const size_t off = (size_t)(m >> 3) * sbo + (size_t)g * 128 + (size_t)m8 * 16;
            *reinterpret_cast<uint4*>(dst + off) = h;
            *reinterpret_cast<uint4*>(dst + plane + off) = l;
        }
    }
}

// ------------------------------------------------------------- matrix pass --
// NC consecutive TMEM columns (NC = 32 or 64) of the warp's 32 lanes, loaded in
// x16 pieces and waited for once, in one statement.
template <int NC> __device__ __forceinline__ void tmem_ld_cols(unsigned taddr, float* v);
template <> __device__ __forceinline__ void tmem_ld_cols<32>(unsigned taddr, float* v) {
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%32];\n"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%33];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr), "r"(taddr + 16u)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}
template <> __device__ __forceinline__ void tmem_ld_cols<64>(unsigned taddr, float* v) {
    tmem_ld_cols<32>(taddr, v);
    tmem_ld_cols<32>(taddr + 32u, v + 32);
}

// The pass over strips [sbeg, send) of one block size B.  Warps 0-3 consume, warp 4
// produces.  The producer (its lane 0) walks this CTA's strips (every gridDim.x-th,
// skipping clusters with no active right-hand side); for each block it waits until
// the block that last used the stage has finished its MMAs (the stage's empty
// barrier, committed with them), writes the block's job record (its partials'
// offsets) into the stage's slot and streams the block's bf16 planes, y_u of
// particle j and y_w of particle i into the stage; after the last block it arrives
// on the next stage's full barrier with an invalid job.  The consumers build each
// block's B operand, meet at a named barrier, and thread 0 issues the MMAs,
// committing them to the accumulator's barrier and the stage's empty barrier; then
// every consumer reads the previous block's accumulator rows.  Each consumer keeps
// the jobs of the block it builds and of the block it reads out in registers.
constexpr int kTcConsumers = 128;   // warps 0-3
template <int R>
__global__ void __launch_bounds__(kTcThreads, 1)
k_pgemv_tc(const gb::SysDev* __restrict__ sys, const gb::Strip* __restrict__ strips, long long sbeg, long long send,
           const gb::KState* __restrict__ st, int mask, const unsigned char* __restrict__ mat_tc,
           const float2* __restrict__ Yu, const float2* __restrict__ Yw, float2* __restrict__ CU,
           float2* __restrict__ CW, const gb::SysPlan* __restrict__ plan, int B, int* __restrict__ err) {
    constexpr int N = 8 * R;             // B-operand rows: [U_h | W_h | U_l | W_l], 2R each
    constexpr int S = kTcStages;
    constexpr unsigned NCOL = 2 * N;     // two accumulators of N FP32 columns (64 or 128: a power of 2 >= 32)
    constexpr unsigned IDESC_FULL = idesc_bf16(128, N);
    constexpr unsigned IDESC_HALF = idesc_bf16(128, N / 2);
    const TcLayout L = tc_layout(B, R);
    const int Kp = gb::tc_cols(B);
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t* full = reinterpret_cast<uint64_t*>(sm);
    uint64_t* empty = full + S;
    uint64_t* mdone = empty + S;
    unsigned* tslot = reinterpret_cast<unsigned*>(mdone + 2);
    volatile int* sabort = reinterpret_cast<volatile int*>(tslot + 1);
    long long* sconsumed = reinterpret_cast<long long*>(tslot + 2);
    TcJob* jobs = reinterpret_cast<TcJob*>(sm + L.off_jobs);
    int* srow = reinterpret_cast<int*>(sm + L.off_row);
    unsigned char* bbuf = sm + L.off_b;
    unsigned char* stages = sm + L.off_stage;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long G = gridDim.x;

    if (tid == 0) {
        for (int q = 0; q < S; q++) {
            bar_init(full + q, 1);
            bar_init(empty + q, 1);
        }
        bar_init(mdone, 1);
        bar_init(mdone + 1, 1);
        *sabort = 0;
        *sconsumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    {   // both B-operand buffers start at zero: their K padding is never written again
        uint4* z = reinterpret_cast<uint4*>(bbuf);
        for (unsigned e = tid; e < 2u * L.bbytes / 16u; e += kTcThreads) z[e] = make_uint4(0, 0, 0, 0);
    }
    const int* rowinfo = sys[strips[sbeg].sys].rowinfo;   // every cluster of the launch has block size B
    for (int r = tid; r < B; r += kTcThreads) srow[r] = __ldg(rowinfo + r);
    if (warp == 0) {
        tmem_alloc(tslot, NCOL);
        tmem_relinquish();
    }
    proxy_fence();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const unsigned tmem = *tslot;
    pdl_wait_tc();   // y vectors and solver state come from the preceding kernels
    pdl_trigger_tc();

    if (warp == kTcConsumers / 32) {
        // ------------------------------------------------------------ producer
        long long k = 0;   // stages written (blocks and the final invalid job)
        if (lane == 0) {
            long long pw = sbeg + blockIdx.x;
            int pb = 0;
            const uint64_t pol = evict_first_policy();
            auto seek = [&]() {
                while (pw < send && !gb::any_active<R>(st, strips[pw].sys, mask)) pw += G;
            };
            seek();
            for (;; k++) {
                const int s = (int)(k % S);
                if (k >= S && !bar_wait(empty + s, (unsigned)((k / S - 1) & 1))) {   // the stage's last MMAs
                    *sabort = 1;
                    atomicExch(err, 1);
                    break;
                }
                if (*sabort) break;
                if (pw >= send) {   // the end: an invalid job, with a plain arrive
                    jobs[s].valid = 0;
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(su32(full + s)) : "memory");
                    k++;
                    break;
                }
                const gb::Strip sp = strips[pw];
                const gb::SysDev& Sd = sys[sp.sys];
                const gb::SysPlan& pl = plan[sp.sys];
                const int j = sp.i + 1 + (int)(sp.p0 - pair_start(sp.i, Sd.N)) + pb;
                TcJob J;
                J.cw = pl.cw_off + ((long long)j * (j - 1) / 2 + sp.i) * (long long)B * R;
                J.cu = (pb == sp.nb - 1) ? pl.cu_off + (pw - pl.strip_base) * (long long)B * R : -1;
                J.valid = 1;
                J.pad = 0;
                jobs[s] = J;
                unsigned char* dst = stages + (size_t)s * L.stage;
                bar_expect_tx(full + s, L.tile + 2u * L.ybytes);   // arrive (release): the job record goes with it
                bulk_copy_hint(dst, mat_tc + Sd.tc_off + (sp.p0 + pb) * (long long)L.tile, L.tile, full + s, pol);
                bulk_copy(dst + L.tile, Yu + Sd.vec_off + (long long)j * B * R, L.ybytes, full + s);
                bulk_copy(dst + L.tile + L.ybytes, Yw + Sd.vec_off + (long long)sp.i * B * R, L.ybytes, full + s);
                if (++pb >= sp.nb) {
                    pb = 0;
                    pw += G;
                    seek();
                }
            }
        }
        __syncthreads();   // every thread of the CTA meets here once the consumers are done
        if (lane == 0)     // drain: every stage written and not consumed (bounded waits)
            for (long long q = *sconsumed; q < k; q++) (void)bar_wait(full + (q % S), (unsigned)((q / S) & 1));
    } else {
        // ------------------------------------------------------------ consumers
        float u[2 * R];
#pragma unroll
        for (int q = 0; q < 2 * R; q++) u[q] = 0.f;
        const int m = warp * 32 + lane;   // accumulator row (TMEM lane) of this thread
        const bool warp_rows = warp * 32 < B;
        int rho_m = 0;
        unsigned eneg_m = 0;
        if (m < B) {
            rho_m = srow[m] & ((1 << 29) - 1);
            eneg_m = (srow[m] >> 29) & 1;
        }
        // block e's accumulator: its column partials out, its row partial into u; at the
        // strip's end the row partials out
        auto epilogue = [&](long long e, const TcJob& J) -> bool {
            const int x = (int)(e & 1);
            bool ok = bar_wait(mdone + x, (unsigned)((e >> 1) & 1));
            ok = __all_sync(0xffffffffu, ok);
            tc_after_sync();
            if (ok && warp_rows) {
                float v[N];
                tmem_ld_cols<N>(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(x * N), v);
                if (m < B) {
                    float2 w[R];
#pragma unroll
                    for (int q = 0; q < R; q++) {
                        u[2 * q] += v[2 * q] + v[4 * R + 2 * q];
                        u[2 * q + 1] += v[2 * q + 1] + v[4 * R + 2 * q + 1];
                        w[q] = make_float2(flipf(v[2 * R + 2 * q] + v[6 * R + 2 * q], eneg_m),
                                           flipf(v[2 * R + 2 * q + 1] + v[6 * R + 2 * q + 1], eneg_m));
                    }
                    float4* cwp = reinterpret_cast<float4*>(CW + J.cw + (long long)rho_m * R);
#pragma unroll
                    for (int q = 0; q < R; q += 2) cwp[q / 2] = make_float4(w[q].x, w[q].y, w[q + 1].x, w[q + 1].y);
                }
            }
            tc_before_sync();
            if (!ok && lane == 0) {
                *sabort = 1;
                atomicExch(err, 1);
            }
            if (J.cu >= 0) {   // the strip's row partial
                if (ok && m < B) {
                    float4* cup = reinterpret_cast<float4*>(CU + J.cu + (long long)rho_m * R);
#pragma unroll
                    for (int q = 0; q < R; q += 2)
                        cup[q / 2] = make_float4(flipf(u[2 * q], eneg_m), flipf(u[2 * q + 1], eneg_m),
                                                 flipf(u[2 * q + 2], eneg_m), flipf(u[2 * q + 3], eneg_m));
                }
#pragma unroll
                for (int q = 0; q < 2 * R; q++) u[q] = 0.f;
            }
            return ok;
        };

        long long g = 0;   // blocks whose MMAs were issued
        bool aborted = false;
        TcJob prev;
        prev.valid = 0;
        while (true) {
            const int s = (int)(g % S), x = (int)(g & 1);
            unsigned char* stg = stages + (size_t)s * L.stage;
            bool ok = false;
            TcJob J;
            J.valid = 0;
            if (!*sabort) {
                ok = bar_wait(full + s, (unsigned)((g / S) & 1));
                if (!ok) {
                    *sabort = 1;
                    atomicExch(err, 1);
                } else {
                    J = jobs[s];
                }
            }
            // B operand of block g into buffer x (last read by the MMAs of block g - 2,
            // which completed before this thread's epilogue of g - 2)
            if (ok && J.valid) {
                const float2* yu = reinterpret_cast<const float2*>(stg + L.tile);
                const float2* yw = reinterpret_cast<const float2*>(stg + L.tile + L.ybytes);
                unsigned char* bb = bbuf + (size_t)x * L.bbytes;
                for (int it = tid; it < B * R; it += kTcConsumers) {
                    const int sc = it / R, q = it - sc * R;
                    const int info = srow[sc];
                    const int rs = info & ((1 << 29) - 1);
                    const unsigned en = (info >> 29) & 1;
                    const float2 zu = yu[rs * R + q], zw = yw[rs * R + q];
                    const float zr[2] = {flipf(zu.x, en), flipf(zw.x, en)};
                    const float zi[2] = {flipf(zu.y, en), flipf(zw.y, en)};
                    const unsigned col = (unsigned)(sc >> 2) * 128u + (unsigned)(sc & 3) * 4u;
#pragma unroll
                    for (int h = 0; h < 2; h++) {   // h 0: U rows (z_j), 1: W rows (w_i)
                        const float hr = bf_round(zr[h]), hi = bf_round(zi[h]);
                        const float lr = zr[h] - hr, li = zi[h] - hi;
                        const int n0 = h * 2 * R + 2 * q, n1 = n0 + 4 * R;   // hi rows, lo rows (n0 even)
                        unsigned char* r0 = bb + (n0 >> 3) * L.sbo + col + (n0 & 7) * 16;
                        unsigned char* r1 = bb + (n1 >> 3) * L.sbo + col + (n1 & 7) * 16;
                        *reinterpret_cast<unsigned*>(r0) = bf2(hr, -hi);        // row n0:     re(A z)
                        *reinterpret_cast<unsigned*>(r0 + 16) = bf2(hi, hr);    // row n0 + 1: im(A z)
                        *reinterpret_cast<unsigned*>(r1) = bf2(lr, -li);
                        *reinterpret_cast<unsigned*>(r1 + 16) = bf2(li, lr);
                    }
                }
            }
            proxy_fence();   // generic writes of the B operand -> the tensor core's reads
            tc_before_sync();
            // the consumer warps' barrier, with the OR of every consumer's view of the
            // abort flag (the producer may set it at any time): one decision for all
            unsigned stop = (!ok || *sabort) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, %2, p;\n"
                " selp.u32 %0, 1, 0, q;\n}\n"
                : "=r"(stop)
                : "r"(stop), "n"(kTcConsumers)
                : "memory");
            tc_after_sync();
            if (stop) {
                aborted = true;
                break;
            }
            if (!J.valid) break;   // the same record for every consumer: the end of this CTA's blocks
            if (tid == 0) {
                const unsigned a_hi = su32(stg), a_lo = a_hi + L.plane, bsm = su32(bbuf + (size_t)x * L.bbytes);
                const unsigned d = tmem + (unsigned)(x * N);
                for (int ks = 0; ks < Kp / 16; ks++) {
                    const uint64_t bd = smem_desc(bsm + ks * 256, 128, L.sbo);
                    mma_bf16(d, smem_desc(a_hi + ks * 256, 128, L.sbo), bd, IDESC_FULL, ks > 0);
                    mma_bf16(d, smem_desc(a_lo + ks * 256, 128, L.sbo), bd, IDESC_HALF, 1);
                }
                mma_commit(mdone + x);
                mma_commit(empty + s);   // the stage is free once these MMAs have read it
            }
            g++;
            if (g >= 2) epilogue(g - 2, prev);   // the previous block's accumulator out
            prev = J;
        }
        if (!aborted && g >= 1 && !epilogue(g - 1, prev)) aborted = true;
        if (tid == 0) {
            *sconsumed = g;
            if (aborted)   // bounded waits for the MMAs still in flight
                for (long long e = (g >= 2 ? g - 2 : 0); e < g; e++)
                    (void)bar_wait(mdone + (e & 1), (unsigned)((e >> 1) & 1));
        }
        tc_before_sync();
        __syncthreads();
    }
    // every thread has passed the CTA barrier above (the producer then drained its copies)
    tc_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc_after_sync();
        tmem_dealloc(tmem, NCOL);
    }
}

}   // namespace

namespace gb {

int launch_pgemv_tc(int R, const SysDev* sys, const Strip* strips, long long sbeg, long long send, const KState* st,
                    int mask, const void* mat_tc, const void* Yu, const void* Yw, void* CU, void* CW,
                    const SysPlan* plan, int B, int* err, cudaStream_t stream) {
    if (send <= sbeg) return GB_OK;
    if (R != 4 && R != 8) return gb_set_error(GB_UNSUPPORTED, "tensor-core pass: R must be 4 or 8 (got %d)", R);
    if (tc_rows(B) > 128) return gb_set_error(GB_UNSUPPORTED, "tensor-core pass: block size %d > 128 rows", B);
    if ((reinterpret_cast<uintptr_t>(mat_tc) | reinterpret_cast<uintptr_t>(Yu)) & 15)
        return gb_set_error(GB_BAD_ARG, "tensor-core pass: matrix and y vectors must be 16-byte aligned");
    const TcLayout L = tc_layout(B, R);
    if (L.total > 227u * 1024u)
        return gb_set_error(GB_UNSUPPORTED, "tensor-core pass: block size %d needs %u B of shared memory", B, L.total);
    const void* kfn = R == 4 ? reinterpret_cast<const void*>(k_pgemv_tc<4>) : reinterpret_cast<const void*>(k_pgemv_tc<8>);
    GB_CUDA_TRY(ensure_dynamic_smem(kfn, L.total));
    // two CTAs per SM where their shared memory fits (228 KB per SM, 1 KB reserved per CTA)
    const int per_sm = 2u * (L.total + 1024u) <= 228u * 1024u ? 2 : 1;
    const long long n = send - sbeg;
    const long long grid = n < (long long)sm_count() * per_sm ? n : (long long)sm_count() * per_sm;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kTcThreads);
    cfg.dynamicSmemBytes = L.total;
    cfg.stream = stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    note_launch();
    const unsigned char* m = static_cast<const unsigned char*>(mat_tc);
    const float2* yu = static_cast<const float2*>(Yu);
    const float2* yw = static_cast<const float2*>(Yw);
    float2* cu = static_cast<float2*>(CU);
    float2* cw = static_cast<float2*>(CW);
    if (R == 4)
        GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_pgemv_tc<4>, sys, strips, sbeg, send, st, mask, m, yu, yw, cu, cw, plan, B,
                                       err));
    else
        GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_pgemv_tc<8>, sys, strips, sbeg, send, st, mask, m, yu, yw, cu, cw, plan, B,
                                       err));
    return GB_OK;
}

}   // namespace gb

extern "C" {

size_t gb_tc_matrix_bytes(int nsys, const gb_system* sys) {
    if (nsys < 1 || !sys) return 0;
    std::vector<gb::SysDev> sd;
    if (gb::make_sysdev(nsys, sys, 0, sd)) return 0;
    const gb::SysDev& last = sd.back();
    return (size_t)(last.tc_off + last.P * gb::tc_block_bytes(last.B));
}

int gb_tc_matrix_build(int nsys, const gb_system* sys, const float* mat64, void* mat_tc, void* stream) {
    if (nsys < 1 || !sys || !mat64 || !mat_tc) return gb_set_error(GB_BAD_ARG, "null argument");
    if (reinterpret_cast<uintptr_t>(mat64) & 15 || reinterpret_cast<uintptr_t>(mat_tc) & 15)
        return gb_set_error(GB_BAD_ARG, "matrices must be 16-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<gb::SysDev> sd;
    int e = gb::make_sysdev(nsys, sys, s, sd);
    if (e) return e;
    if (nsys > 65535) return gb_set_error(GB_UNSUPPORTED, "more than 65535 clusters in one batch");
    long long maxP = 0;
    for (const gb::SysDev& d : sd) maxP = d.P > maxP ? d.P : maxP;
    if (maxP == 0) return GB_OK;
    void* dsys = nullptr;
    int slot = 0;
    e = gb::stage_acquire(sd.data(), sizeof(gb::SysDev) * sd.size(), s, &dsys, &slot);
    if (e) return e;
    const unsigned gx = (unsigned)(maxP < 4096 ? maxP : 4096);
    gb::note_launch();
    k_tc_tiles<<<dim3(gx, (unsigned)nsys), 256, 0, s>>>(static_cast<const gb::SysDev*>(dsys),
                                                         reinterpret_cast<const float2*>(mat64),
                                                         static_cast<unsigned char*>(mat_tc));
    GB_CUDA_TRY(cudaGetLastError());
    return gb::stage_release(slot, s);
}

}   // extern "C"
