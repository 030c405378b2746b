// Beam source decomposition at the particles (replaces integrate_phase,
// cpp/src/decomposition.cpp:29-66, which beam.structure, sources/beams.py:168-200,
// calls once per particle through the p_src function of
// integral_project_source_far, vsh/decomposition.py:284-325).
//
// For particle i at position x_i (relative to the beam centre) and mode column c
// (a*rmax + r):
//   p_src[i][c] = sum_g w[g][c] exp(-i k rhat_g . x_i)
// where g runs over the far-field (theta, phi) grid and w already holds the
// trapezoid weights of both 1-D rules times the far-field projection p0.  One CTA
// per particle: the phases of all grid points go to shared memory (FP64 sincos,
// one per grid point), then each thread sums one or more columns over the grid
// (FP64 complex FMAs, reads of w coalesced across threads).

#include <algorithm>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace {

constexpr int kBeamThreads = 128;

__global__ void __launch_bounds__(kBeamThreads)
k_beam_project(int N, int ncol, int G, const double* __restrict__ pos, const double* __restrict__ rhat,
               const double2* __restrict__ w, double k, double2* __restrict__ out, int es) {
    extern __shared__ double2 ph[];
    for (int i = blockIdx.x; i < N; i += gridDim.x) {
        const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        for (int g = threadIdx.x; g < G; g += kBeamThreads) {
            const double a = -k * (rhat[3 * g] * x + rhat[3 * g + 1] * y + rhat[3 * g + 2] * z);
            double s, c;
            sincos(a, &s, &c);
            ph[g] = make_double2(c, s);
        }
        __syncthreads();
        for (int col = threadIdx.x; col < ncol; col += kBeamThreads) {
            double2 acc = make_double2(0.0, 0.0);
            for (int g = 0; g < G; g++) cfma(acc, __ldg(w + (long long)g * ncol + col), ph[g]);
            out[((long long)i * ncol + col) * es] = acc;
        }
        __syncthreads();
    }
}

}   // namespace

extern "C" int gb_beam_project(int N, int ncol, int G, const double* pos, const double* rhat, const double* w,
                               double k, double* out, int out_stride, void* stream) {
    if (N < 0 || ncol < 1 || G < 1 || out_stride < 1) return gb_set_error(GB_BAD_ARG, "bad beam projection sizes");
    if (N == 0) return GB_OK;
    if (!pos || !rhat || !w || !out) return gb_set_error(GB_BAD_ARG, "null argument");
    const size_t smem = sizeof(double2) * (size_t)G;
    if (smem > 200 * 1024) return gb_set_error(GB_UNSUPPORTED, "far-field grid of %d points is too large", G);
    if (smem > 48 * 1024)
        GB_CUDA_TRY(gb::ensure_dynamic_smem(reinterpret_cast<const void*>(k_beam_project), smem));
    const int grid = std::min(N, gb::sm_count() * 8);
    gb::note_launch();
    k_beam_project<<<grid, kBeamThreads, smem, (cudaStream_t)stream>>>(
        N, ncol, G, pos, rhat, reinterpret_cast<const double2*>(w), k, reinterpret_cast<double2*>(out), out_stride);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}
