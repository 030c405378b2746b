// Internal host-side declarations shared by the translation units of the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>

#include "../../include/miepy_gb300.h"

namespace gb {

// Per-lmax device tables (see tables.cu).
struct Tables {
    int lmax = 0, M = 0, rmax = 0, B = 0;
    int4* nmvu = nullptr;      // [M] canonical tuples (n, m, v, u)
    int2* qab = nullptr;       // [M] (qmax_A, qmax_B)
    double* cA = nullptr;      // [M][lmax+1]
    double* cB = nullptr;      // [M][lmax+1]
    float2* cA2 = nullptr;     // [M][lmax+1] (hi, lo) split of cA
    float2* cB2 = nullptr;     // [M][lmax+1] (hi, lo) split of cB
    // the tuples in order of (qmax_A, qmax_B) descending, so that the lanes of a warp
    // run sums of equal length: (t, n + v, u - m, qmax_A | qmax_B << 8) and the (hi,
    // lo) coefficients in that order
    int4* tinfo = nullptr;     // [M]
    float2* cA2s = nullptr;    // [M][lmax+1]
    float2* cB2s = nullptr;    // [M][lmax+1]
    int* elem_map = nullptr;   // [B*B] (tuple << 2) | (is_B << 1) | negate
    double* neg_ratio = nullptr;   // [(2L+2)^2] (-1)^mu (p-mu)!/(p+mu)!
    float4* neg_ratio2 = nullptr;  // the same as (m.hi, m.lo, e, s): ratio = (m.hi + m.lo) 2^e, m in [0.5, 1), s = 2^e if normal else 0
    int* rowinfo = nullptr;    // [B] rho(row) | eps_neg << 29 | sig_neg << 30
    int* miecol = nullptr;     // [B] a*lmax + n - 1
};

int get_tables(int lmax, cudaStream_t stream, const Tables** out);

// Translation tables between orders Lc (outgoing about an origin) and Lin (about a
// particle): every (n <= Lc, m, v <= Lin, u), tuple t = r(n, m) * rmax(Lin) + r(v, u).
struct CrossTables {
    int Lc = 0, Lin = 0, M = 0, Q = 0, PM = 0;
    int4* nmvu = nullptr;
    int2* qab = nullptr;
    double* cA = nullptr;        // [M][Q]
    double* cB = nullptr;        // [M][Q]
    double* neg_ratio = nullptr; // [PM][PM]
};
int get_cross_tables(int Lc, int Lin, cudaStream_t stream, const CrossTables** out);
int host_tuples(int L, std::vector<int4>& nmvu);

int sm_count();

// Kernel-launch accounting (gb_launch_count): direct launches call note_launch;
// launches recorded into a CUDA graph are counted once per graph replay.
// Raises (never lowers) a kernel's dynamic shared-memory limit, thread-safely.
cudaError_t ensure_dynamic_smem(const void* func, size_t bytes);

void note_launch();
void note_launches(long long n);
void capture_begin();
long long capture_end();

// Device-side description of one cluster of a batch (expanded from gb_system).
struct SysDev {
    int N, lmax, rmax, B, D;
    int M;                  // tuples of this lmax
    long long P;            // pairs
    double k;
    long long pos_off, mat_off, vec_off, t_off;
    // table pointers for this lmax
    const int4* nmvu;
    const int2* qab;
    const double* cA;
    const double* cB;
    const float2* cA2;
    const float2* cB2;
    const int4* tinfo;
    const float2* cA2s;
    const float2* cB2s;
    const int* elem_map;
    const double* neg_ratio;
    const float4* neg_ratio2;
    const int* rowinfo;
    const int* miecol;
    // general particles: per-particle T-matrices [N][B][B] (row-major, mode order of
    // the reference), complex128 and a complex64 copy; null for spheres (t vector)
    const double2* tmat128 = nullptr;
    const float2* tmat64 = nullptr;
    // byte offset of this cluster's blocks in the bf16 tile arena of the tensor-core
    // matrix pass (tc_block_bytes(B) per pair, clusters in batch order)
    long long tc_off = 0;
};

// bf16 tiles of one B x B complex64 block for the tensor-core matrix pass: the hi
// and lo planes (hi = bf16(a), lo = bf16(a - hi), per real component), each
// Bp x Kp bf16 (Bp = B rounded up to 8 rows, Kp = 2B real columns rounded up to 16)
// in the K-major core-matrix layout of tcgen05 operands: element (m, k) at
// (m / 8) * (Kp * 16) + (k / 8) * 128 + (m % 8) * 16 + (k % 8) * 2 bytes; padding
// rows and columns hold zeros.
__host__ __device__ inline int tc_rows(int B) { return (B + 7) & ~7; }
__host__ __device__ inline int tc_cols(int B) { return (2 * B + 15) & ~15; }
__host__ __device__ inline long long tc_plane_bytes(int B) { return 2LL * tc_rows(B) * tc_cols(B); }
__host__ __device__ inline long long tc_block_bytes(int B) { return 2 * tc_plane_bytes(B); }

// Pinned staging ring for per-call descriptor uploads (assemble.cu).
int stage_acquire(const void* src, size_t bytes, cudaStream_t stream, void** dev_out, int* slot_out);
int stage_release(int slot, cudaStream_t stream);

// This host thread's pinned buffer of at least bytes for device->host readbacks of
// solver state (assemble.cu).  Valid until the thread's next call; a copy into it
// waits only for its own stream, where one into pageable memory also holds the
// driver's shared staging path until the stream's earlier work is done.
void* host_readback(size_t bytes);

int make_sysdev(int nsys, const gb_system* sys, cudaStream_t stream, std::vector<SysDev>& out);

}   // namespace gb
