// Shared definitions for the sm_103a sphere-cluster kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/miepy_gb300.h"

#define GB_LMAX_MAX 10            // largest supported expansion order
#define GB_PMAX_MAX (2 * GB_LMAX_MAX + 1)
#define GB_Q_MAX (GB_LMAX_MAX + 1)  // q-terms per translation sum

// ------------------------------------------------------------- complex ops --
struct cdbl { double x, y; };
struct cflt { float x, y; };

__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// acc += a * b
// a - b on packed f32x2 (sub.rn.f32x2): the packed add takes no negated operand,
// so a - b written as a + (-b) costs a sign flip per component on the integer pipe
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
    unsigned long long ra, rb, rd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    float2 d;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(rd));
    return d;
}
__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ void cfmaf(float2& acc, float2 a, float2 b) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(-a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(a.y, b.x, acc.y);
}
// acc += conj(a) * b
__device__ __forceinline__ void cfma_conj(double2& acc, double2 a, double2 b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
}

// Sign flips by XOR of the sign bit (keeps the FP64 pipe free).
__device__ __forceinline__ double flipd(double v, unsigned neg) {
    return __longlong_as_double(__double_as_longlong(v) ^ ((unsigned long long)neg << 63));
}
__device__ __forceinline__ float flipf(float v, unsigned neg) {
    return __int_as_float(__float_as_int(v) ^ (neg << 31));
}

// --------------------------------------------------------------- indexing --
// mode index r = n(n+2) - n + m - 1 (n >= 1, |m| <= n); D = 2 * rmax * N.
__host__ __device__ __forceinline__ int lmax_to_rmax(int l) { return l * (l + 2); }

// Pair p (0-based, i-major order over i < j) -> (i, j); inverse of
// p = i*N - i*(i+1)/2 + (j - i - 1).
__host__ __device__ __forceinline__ long long pair_start(long long i, long long N) {
    return i * N - i * (i + 1) / 2;
}
__device__ __forceinline__ void pair_ij(long long p, int N, int& i, int& j) {
    double Nn = N;
    double disc = (2.0 * Nn - 1.0) * (2.0 * Nn - 1.0) - 8.0 * (double)p;
    int ii = (int)floor(((2.0 * Nn - 1.0) - sqrt(disc > 0 ? disc : 0.0)) * 0.5);
    if (ii < 0) ii = 0;
    if (ii > N - 2) ii = N - 2;
    while (ii > 0 && pair_start(ii, N) > p) ii--;
    while (ii < N - 2 && pair_start(ii + 1, N) <= p) ii++;
    i = ii;
    j = (int)(p - pair_start(ii, N)) + ii + 1;
}

// ------------------------------------------------------------ error state --
#define GB_CUDA_TRY(expr)                                                   \
    do {                                                                    \
        cudaError_t _e = (expr);                                            \
        if (_e != cudaSuccess) return gb_set_cuda_error(_e, #expr, __FILE__, __LINE__); \
    } while (0)

int gb_set_error(int code, const char* fmt, ...);
int gb_set_cuda_error(cudaError_t e, const char* what, const char* file, int line);
