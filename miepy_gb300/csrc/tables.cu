// Per-lmax translation coefficient tables, built on the device.
//
// The reference builds, per call, a std::map from every (n, m, v<=n, u) to the
// Gaunt-weighted coefficients A(q), B(q) of the addition theorem
// (vsh_cache, cpp/src/vsh_translation.cpp:12-51; gaunt_batch and
// wigner_3j_batch, cpp/src/special.cpp:298-440).  Here the canonical tuples of
// the pair-insertion loop (cpp/src/vsh_translation.cpp:171-176, including its
// `n == v && u < -m` skip) are enumerated once per lmax, and one device thread
// per tuple evaluates the two Wigner-3j sequences with the Schulten-Gordon
// recurrence seeded by Racah's closed form.  The coefficients are folded so that
// the assembler needs only real x complex FMAs:
//
//   A_t = i^(n+v)   * sum_q cA[t][q] * G[n+v-2q][mu]
//   B_t = i^(n+v+1) * sum_q cB[t][q] * G[n+v-2q+1][mu],   mu = u - m,
//   G[p][mu] = P_p^mu(cos theta) h_p(k r) e^{i mu phi}    (per pair),
//
// cA = factor * a_q (-1)^q (n(n+1) + v(v+1) - p(p+1)),
// cB = -factor * b_q (-1)^q sqrt(((p+1)^2 - (n-v)^2)((n+v+1)^2 - (p+1)^2)),
// which is the reference's A(q) = a_q i^p (...), B(q) = b_q i^(p+1) sqrt(...)
// with i^p = i^(n+v) (-1)^q.
//
// The element map records, for every entry of the B x B block of pair (i, j),
// which tuple and which of (A, B) lands there and with which sign, by replaying
// the reference's placement rules (cpp/src/vsh_translation.cpp:211-232) for the
// (i, j) block.

#include <array>
#include <map>
#include <mutex>
#include <algorithm>
#include <vector>
#include <cmath>
#include <cstdio>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace {

__device__ double dfact(int n) { return tgamma((double)n + 1.0); }
__device__ double dsgn(int p) { return (p & 1) ? -1.0 : 1.0; }

// Racah's single-sum formula for the Wigner 3j symbol.
__device__ double w3j_racah(int j1, int j2, int j3, int m1, int m2, int m3) {
    if (m1 + m2 + m3 != 0) return 0.0;
    if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0.0;
    int t1 = j1 + j2 - j3, t2 = j1 - j2 + j3, t3 = -j1 + j2 + j3;
    if (t1 < 0 || t2 < 0 || t3 < 0) return 0.0;
    double delta = dfact(t1) * dfact(t2) * dfact(t3) / dfact(j1 + j2 + j3 + 1);
    double pre = dfact(j1 + m1) * dfact(j1 - m1) * dfact(j2 + m2) * dfact(j2 - m2) * dfact(j3 + m3) * dfact(j3 - m3);
    int tmin = max(0, max(j2 - j3 - m1, j1 - j3 + m2));
    int tmax = min(j1 + j2 - j3, min(j1 - m1, j2 + m2));
    double s = 0.0;
    for (int t = tmin; t <= tmax; t++) {
        double den = dfact(t) * dfact(j1 + j2 - j3 - t) * dfact(j1 - m1 - t) * dfact(j2 + m2 - t) *
                     dfact(j3 - j2 + m1 + t) * dfact(j3 - j1 - m2 + t);
        s += dsgn(t) / den;
    }
    return dsgn(j1 - j2 - m3) * sqrt(delta * pre) * s;
}

// All 3j(j, j2, j3; m1, m2, m3) for j = jmin..j2+j3, jmin = max(|j2-j3|, |m1|):
// two Racah seeds, then the Schulten-Gordon three-term recurrence in j.
__device__ int w3j_sequence(int j2, int j3, int m1, int m2, int m3, int* jmin_out, double* val, int cap) {
    *jmin_out = 0;
    if (m1 + m2 + m3 != 0) return 0;
    int jmin = max(abs(j2 - j3), abs(m1));
    int jmax = j2 + j3;
    int size = jmax - jmin + 1;
    *jmin_out = jmin;
    if (size <= 0) return 0;
    if (size > cap) size = cap;
    if (size <= 2) {
        for (int i = 0; i < size; i++) val[i] = w3j_racah(jmin + i, j2, j3, m1, m2, m3);
        return size;
    }
    val[0] = w3j_racah(jmin, j2, j3, m1, m2, m3);
    val[1] = w3j_racah(jmin + 1, j2, j3, m1, m2, m3);
    const double d = j2 - j3, s = j2 + j3 + 1;
    const double jj = (double)j2 * (j2 + 1) - (double)j3 * (j3 + 1);
    const double md = m3 - m2;
    for (int i = 1; i < size - 1; i++) {
        double j = jmin + i, jp = j + 1.0;
        double sj = sqrt(fmax(0.0, (j * j - d * d) * (s * s - j * j) * (j * j - (double)m1 * m1)));
        double sjp = sqrt(fmax(0.0, (jp * jp - d * d) * (s * s - jp * jp) * (jp * jp - (double)m1 * m1)));
        double A = jp * sj;
        double Bc = (2.0 * j + 1.0) * (-(double)m1 * jj + md * j * jp);
        double C = j * sjp;
        if (fabs(C) < 1e-30) val[i + 1] = w3j_racah((int)j + 1, j2, j3, m1, m2, m3);
        else val[i + 1] = (-A * val[i - 1] - Bc * val[i]) / C;
    }
    return size;
}

__global__ void k_tuple_table(int L, int M, const int4* __restrict__ nmvu, int2* __restrict__ qab,
                              double* __restrict__ cA, double* __restrict__ cB) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= M) return;
    const int Q = L + 1;
    int4 e = nmvu[t];
    const int n = e.x, v = e.z, u = e.w;
    const int m = -e.y;   // the insertion loop looks up the cache at (n, -m, v, u)
    double factor = 0.5 * dsgn(m) *
                    sqrt((2.0 * v + 1) * (2.0 * n + 1) * dfact(v - u) * dfact(n - m) /
                         ((double)v * (v + 1) * n * (n + 1) * dfact(v + u) * dfact(n + m)));
    int qA = min(min(n, v), (n + v - abs(m + u)) / 2);
    int qB = min(min(n, v), (n + v + 1 - abs(m + u)) / 2);
    qab[t] = make_int2(qA, qB);
    double w0[2 * GB_LMAX_MAX + 4], wm[2 * GB_LMAX_MAX + 4];
    int j0 = 0, jm = 0;
    w3j_sequence(n, v, 0, 0, 0, &j0, w0, 2 * GB_LMAX_MAX + 4);
    w3j_sequence(n, v, -(m + u), m, u, &jm, wm, 2 * GB_LMAX_MAX + 4);
    const double fnm = dfact(n + m), fn_m = dfact(n - m), fvu = dfact(v + u), fv_u = dfact(v - u);
    const double sign = dsgn(m + u);
    for (int q = 0; q < Q; q++) {
        cA[(size_t)t * Q + q] = 0.0;
        cB[(size_t)t * Q + q] = 0.0;
    }
    for (int q = 0; q <= qA; q++) {
        int p = n + v - 2 * q;
        double ratio = fnm * fvu * dfact(p - m - u) / (fn_m * fv_u * dfact(p + m + u));
        double aq = sign * (2 * p + 1) * sqrt(ratio) * w0[p - j0] * wm[p - jm];
        cA[(size_t)t * Q + q] = factor * aq * dsgn(q) * (double)(n * (n + 1) + v * (v + 1) - p * (p + 1));
    }
    for (int q = 1; q <= qB; q++) {
        int p = n + v - 2 * q;
        double ratio = fnm * fvu * dfact(p - m - u + 1) / (fn_m * fv_u * dfact(p + m + u + 1));
        double bq = sign * (2 * p + 3) * sqrt(ratio) * w0[p - j0] * wm[(p + 1) - jm];
        double g = sqrt(((double)(p + 1) * (p + 1) - (double)(n - v) * (n - v)) *
                        ((double)(n + v + 1) * (n + v + 1) - (double)(p + 1) * (p + 1)));
        cB[(size_t)t * Q + q] = -factor * bq * dsgn(q) * g;
    }
}

int rn(int n, int m) { return n * (n + 2) - n + m - 1; }

struct TableCache {
    std::mutex mu;
    // [device][lmax]
    std::vector<std::vector<gb::Tables*>> t;
};
TableCache g_cache;

// Double-float split of the coefficient tables: c = hi + lo, hi = fl32(c),
// lo = fl32(c - hi), for the FP32-pipe tuple sums of the assembler.
__global__ void k_split_coeffs(int n, const double* __restrict__ cA, const double* __restrict__ cB,
                               float2* __restrict__ cA2, float2* __restrict__ cB2) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float ah = __double2float_rn(cA[e]), bh = __double2float_rn(cB[e]);
    cA2[e] = make_float2(ah, __double2float_rn(cA[e] - (double)ah));
    cB2[e] = make_float2(bh, __double2float_rn(cB[e] - (double)bh));
}

// The coefficient tables in the sorted tuple order of tinfo; the sum lengths of tinfo
// are set from the device's own qab (the host's copy only orders the tuples).
__global__ void k_perm_coeffs(int M, int Q, int* __restrict__ tinfo, const int2* __restrict__ qab,
                              const float2* __restrict__ cA2, const float2* __restrict__ cB2,
                              float2* __restrict__ cA2s, float2* __restrict__ cB2s) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M * Q) return;
    const int i = e / Q, q = e - i * Q, t = tinfo[4 * i];   // word 0 of the int4: the tuple
    cA2s[e] = cA2[(size_t)t * Q + q];
    cB2s[e] = cB2[(size_t)t * Q + q];
    if (q == 0) tinfo[4 * i + 3] = qab[t].x | (qab[t].y << 8);   // word 3: the sum lengths
}

}   // namespace

namespace gb {

int host_tuples(int L, std::vector<int4>& nmvu) {
    nmvu.clear();
    for (int n = 1; n <= L; n++)
        for (int m = -n; m <= n; m++)
            for (int v = 1; v <= n; v++)
                for (int u = -v; u <= v; u++) {
                    if (n == v && u < -m) continue;
                    nmvu.push_back(make_int4(n, m, v, u));
                }
    return (int)nmvu.size();
}

// Replays the placement rules of the reference for block (i, j).
int host_elem_map(int L, const std::vector<int4>& nmvu, std::vector<int>& map) {
    const int rmax = lmax_to_rmax(L), B = 2 * rmax;
    map.assign((size_t)B * B, -1);
    for (size_t t = 0; t < nmvu.size(); t++) {
        const int n = nmvu[t].x, m = nmvu[t].y, v = nmvu[t].z, u = nmvu[t].w;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++) {
                const int comp = (a + b) & 1;
                int row = a * rmax + rn(n, m), col = b * rmax + rn(v, u);
                map[(size_t)row * B + col] = (int)(t << 2) | (comp << 1);
                if ((n == v && u != -m) || n != v) {
                    int row2 = b * rmax + rn(v, -u), col2 = a * rmax + rn(n, -m);
                    int neg = ((m + u - a - b) % 2 != 0) ? 1 : 0;
                    map[(size_t)row2 * B + col2] = (int)(t << 2) | (comp << 1) | neg;
                }
            }
    }
    for (int e : map)
        if (e < 0) return gb_set_error(GB_UNSUPPORTED, "element map incomplete for lmax %d", L);
    return GB_OK;
}

int get_tables(int lmax, cudaStream_t stream, const Tables** out) {
    if (lmax < 1 || lmax > GB_LMAX_MAX) return gb_set_error(GB_BAD_ARG, "lmax %d outside 1..%d", lmax, GB_LMAX_MAX);
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_cache.mu);
    if ((int)g_cache.t.size() <= dev) g_cache.t.resize(dev + 1);
    auto& per = g_cache.t[dev];
    if ((int)per.size() <= lmax) per.resize(lmax + 1, nullptr);
    if (per[lmax]) {
        *out = per[lmax];
        return GB_OK;
    }
    const int L = lmax, rmax = lmax_to_rmax(L), B = 2 * rmax, Q = L + 1, PM = 2 * L + 2;
    std::vector<int4> nmvu;
    const int M = host_tuples(L, nmvu);
    std::vector<int> map;
    int st = host_elem_map(L, nmvu, map);
    if (st) return st;
    // negative-order Legendre factor (-1)^mu (p-mu)!/(p+mu)! and GEMV row tables
    std::vector<double> negr((size_t)PM * PM, 0.0);
    for (int p = 0; p < PM; p++)
        for (int mu = 0; mu <= p; mu++)
            negr[(size_t)p * PM + mu] = ((mu & 1) ? -1.0 : 1.0) * std::tgamma(p - mu + 1.0) / std::tgamma(p + mu + 1.0);
    std::vector<int> rowinfo(B), miecol(B);
    for (int a = 0; a < 2; a++)
        for (int n = 1; n <= L; n++)
            for (int m = -n; m <= n; m++) {
                int R = a * rmax + rn(n, m);
                int rho = a * rmax + rn(n, -m);
                int eps_neg = ((m + a) & 1) ? 1 : 0;
                int sig_neg = ((n + a) & 1) ? 1 : 0;
                rowinfo[R] = rho | (eps_neg << 29) | (sig_neg << 30);
                miecol[R] = a * L + n - 1;
            }
    // sorted tuple order: the sum lengths of k_tuple_table, longest first
    std::vector<int4> tinfo(M);
    for (int t = 0; t < M; t++) {
        const int n = nmvu[t].x, m = -nmvu[t].y, v = nmvu[t].z, u = nmvu[t].w;
        const int qA = std::min(std::min(n, v), (n + v - std::abs(m + u)) / 2);
        const int qB = std::min(std::min(n, v), (n + v + 1 - std::abs(m + u)) / 2);
        tinfo[t] = make_int4(t, n + v, nmvu[t].w - nmvu[t].y, qA | (qB << 8));
    }
    std::stable_sort(tinfo.begin(), tinfo.end(), [](const int4& a, const int4& b) {
        const int la = a.w & 255, lb = b.w & 255;
        return la != lb ? la > lb : (a.w >> 8) > (b.w >> 8);
    });
    Tables* T = new Tables();
    T->lmax = L;
    T->M = M;
    T->rmax = rmax;
    T->B = B;
    cudaError_t e = cudaSuccess;
    e = cudaMalloc(&T->nmvu, sizeof(int4) * M);
    if (e == cudaSuccess) e = cudaMalloc(&T->qab, sizeof(int2) * M);
    if (e == cudaSuccess) e = cudaMalloc(&T->cA, sizeof(double) * M * Q);
    if (e == cudaSuccess) e = cudaMalloc(&T->cB, sizeof(double) * M * Q);
    if (e == cudaSuccess) e = cudaMalloc(&T->cA2, sizeof(float2) * M * Q);
    if (e == cudaSuccess) e = cudaMalloc(&T->cB2, sizeof(float2) * M * Q);
    if (e == cudaSuccess) e = cudaMalloc(&T->tinfo, sizeof(int4) * M);
    if (e == cudaSuccess) e = cudaMalloc(&T->cA2s, sizeof(float2) * M * Q);
    if (e == cudaSuccess) e = cudaMalloc(&T->cB2s, sizeof(float2) * M * Q);
    if (e == cudaSuccess) e = cudaMalloc(&T->elem_map, sizeof(int) * B * B);
    if (e == cudaSuccess) e = cudaMalloc(&T->neg_ratio, sizeof(double) * PM * PM);
    if (e == cudaSuccess) e = cudaMalloc(&T->neg_ratio2, sizeof(float4) * PM * PM);
    if (e == cudaSuccess) e = cudaMalloc(&T->rowinfo, sizeof(int) * B);
    if (e == cudaSuccess) e = cudaMalloc(&T->miecol, sizeof(int) * B);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->nmvu, nmvu.data(), sizeof(int4) * M, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->elem_map, map.data(), sizeof(int) * B * B, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->tinfo, tinfo.data(), sizeof(int4) * M, cudaMemcpyHostToDevice, stream);
    // double-float mantissa and binary exponent: the ratios reach 1/(2p)!, below the
    // FP32 range, while ratio * P_p^mu stays moderate
    std::vector<float4> negr2(negr.size());
    for (size_t q = 0; q < negr.size(); q++) {
        int ex = 0;
        const double m = std::frexp(negr[q], &ex);
        const float hi = (float)m;
        // .w: 2^e when it is a normal float (e >= -126), else 0 (the kernel then scales
        // with ldexpf)
        negr2[q] = make_float4(hi, (float)(m - (double)hi), (float)ex, ex >= -126 ? std::ldexp(1.0f, ex) : 0.f);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->neg_ratio, negr.data(), sizeof(double) * PM * PM, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->neg_ratio2, negr2.data(), sizeof(float4) * PM * PM, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->rowinfo, rowinfo.data(), sizeof(int) * B, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->miecol, miecol.data(), sizeof(int) * B, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) {
        gb::note_launch();
        k_tuple_table<<<(M + 127) / 128, 128, 0, stream>>>(L, M, T->nmvu, T->qab, T->cA, T->cB);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        gb::note_launch();
        k_split_coeffs<<<(M * Q + 255) / 256, 256, 0, stream>>>(M * Q, T->cA, T->cB, T->cA2, T->cB2);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        gb::note_launch();
        k_perm_coeffs<<<(M * Q + 255) / 256, 256, 0, stream>>>(M, Q, reinterpret_cast<int*>(T->tinfo), T->qab, T->cA2,
                                                                T->cB2, T->cA2s, T->cB2s);
        e = cudaGetLastError();
    }
    // the host vectors above go out of scope: make the copies complete first
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        cudaFree(T->nmvu); cudaFree(T->qab); cudaFree(T->cA); cudaFree(T->cB); cudaFree(T->cA2); cudaFree(T->cB2);
        cudaFree(T->tinfo); cudaFree(T->cA2s); cudaFree(T->cB2s);
        cudaFree(T->elem_map); cudaFree(T->neg_ratio); cudaFree(T->neg_ratio2); cudaFree(T->rowinfo); cudaFree(T->miecol);
        delete T;
        return gb_set_cuda_error(e, "building translation tables", __FILE__, __LINE__);
    }
    per[lmax] = T;
    *out = T;
    return GB_OK;
}

// Cross tables for translations between expansions of different orders (cluster
// coefficients: outgoing order n <= Lc about the origin, incoming v <= Lin about a
// particle), every (n, m, v, u) in mode order, t = r(n, m) * rmax(Lin) + r(v, u),
// with the argument convention of vsh_translation (cpp/src/vsh_translation.cpp:
// 428-470: the cache is evaluated at (n, -m, v, u)).  Same folded coefficients as
// the pair tables; coefficient stride Q = max(Lc, Lin) + 1; the negative-order
// Legendre ratio for orders p < Lc + Lin + 2.
int get_cross_tables(int Lc, int Lin, cudaStream_t stream, const CrossTables** out) {
    if (Lc < 1 || Lc > GB_LMAX_MAX || Lin < 1 || Lin > GB_LMAX_MAX)
        return gb_set_error(GB_BAD_ARG, "cross table orders %d, %d outside 1..%d", Lc, Lin, GB_LMAX_MAX);
    static std::mutex mu;
    static std::map<std::array<int, 3>, CrossTables*> cache;
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    const std::array<int, 3> key{dev, Lc, Lin};
    auto f = cache.find(key);
    if (f != cache.end()) {
        *out = f->second;
        return GB_OK;
    }
    const int rc = lmax_to_rmax(Lc), ri = lmax_to_rmax(Lin), M = rc * ri, L = std::max(Lc, Lin), Q = L + 1;
    const int PM = Lc + Lin + 2;
    std::vector<int4> nmvu;
    nmvu.reserve(M);
    for (int n = 1; n <= Lc; n++)
        for (int m = -n; m <= n; m++)
            for (int v = 1; v <= Lin; v++)
                for (int u = -v; u <= v; u++) nmvu.push_back(make_int4(n, m, v, u));
    std::vector<double> negr((size_t)PM * PM, 0.0);
    for (int p = 0; p < PM; p++)
        for (int mu2 = 0; mu2 <= p; mu2++)
            negr[(size_t)p * PM + mu2] = ((mu2 & 1) ? -1.0 : 1.0) * std::tgamma(p - mu2 + 1.0) / std::tgamma(p + mu2 + 1.0);
    CrossTables* T = new CrossTables();
    T->Lc = Lc;
    T->Lin = Lin;
    T->M = M;
    T->Q = Q;
    T->PM = PM;
    cudaError_t e = cudaMalloc(&T->nmvu, sizeof(int4) * M);
    if (e == cudaSuccess) e = cudaMalloc(&T->qab, sizeof(int2) * M);
    if (e == cudaSuccess) e = cudaMalloc(&T->cA, sizeof(double) * M * Q);
    if (e == cudaSuccess) e = cudaMalloc(&T->cB, sizeof(double) * M * Q);
    if (e == cudaSuccess) e = cudaMalloc(&T->neg_ratio, sizeof(double) * PM * PM);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->nmvu, nmvu.data(), sizeof(int4) * M, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->neg_ratio, negr.data(), sizeof(double) * PM * PM, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) {
        gb::note_launch();
        k_tuple_table<<<(M + 127) / 128, 128, 0, stream>>>(L, M, T->nmvu, T->qab, T->cA, T->cB);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);   // host vectors go out of scope
    if (e != cudaSuccess) {
        cudaFree(T->nmvu); cudaFree(T->qab); cudaFree(T->cA); cudaFree(T->cB); cudaFree(T->neg_ratio);
        delete T;
        return gb_set_cuda_error(e, "building cross translation tables", __FILE__, __LINE__);
    }
    cache[key] = T;
    *out = T;
    return GB_OK;
}

}   // namespace gb

extern "C" {

int gb_tables_prepare(int lmax, void* stream) {
    const gb::Tables* T = nullptr;
    return gb::get_tables(lmax, (cudaStream_t)stream, &T);
}

int gb_tables_count(int lmax, int* M_out) {
    if (lmax < 1 || lmax > GB_LMAX_MAX) return gb_set_error(GB_BAD_ARG, "lmax %d outside 1..%d", lmax, GB_LMAX_MAX);
    std::vector<int4> nmvu;
    *M_out = gb::host_tuples(lmax, nmvu);
    return GB_OK;
}

int gb_tables_export(int lmax, int* nmvu, int* qab, double* cA, double* cB, int* elem_map) {
    const gb::Tables* T = nullptr;
    int st = gb::get_tables(lmax, 0, &T);
    if (st) return st;
    const int M = T->M, Q = lmax + 1, B = T->B;
    if (nmvu) GB_CUDA_TRY(cudaMemcpy(nmvu, T->nmvu, sizeof(int4) * M, cudaMemcpyDeviceToHost));
    if (qab) GB_CUDA_TRY(cudaMemcpy(qab, T->qab, sizeof(int2) * M, cudaMemcpyDeviceToHost));
    if (cA) GB_CUDA_TRY(cudaMemcpy(cA, T->cA, sizeof(double) * M * Q, cudaMemcpyDeviceToHost));
    if (cB) GB_CUDA_TRY(cudaMemcpy(cB, T->cB, sizeof(double) * M * Q, cudaMemcpyDeviceToHost));
    if (elem_map) GB_CUDA_TRY(cudaMemcpy(elem_map, T->elem_map, sizeof(int) * B * B, cudaMemcpyDeviceToHost));
    return GB_OK;
}

}   // extern "C"
