// K7: fused epilogue of a solve.  One warp per (particle, right-hand side):
//   p_scat = t o p_inc, p_int = p_inc * mie_int[:, ::-1, n-1]  (sphere_cluster.py:715-717),
//   per-multipole cross-sections                             (cpp/src/flux.cpp:5-30),
//   force and torque (Barton-type coefficient sums)          (cpp/src/forces.cpp:7-137),
// all in FP64, reading each coefficient once.

#include <algorithm>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEps0 = 8.854187817e-12;   // the GSL MKSA vacuum permittivity the reference uses

__device__ __forceinline__ double2 cj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }

// 2 a conj(b) - a conj(bi) - ai conj(b)
__device__ __forceinline__ double2 tri(double2 a, double2 b, double2 ai, double2 bi) {
    double2 t = cscale(2.0, cmul(a, cj(b)));
    t = csub(t, cmul(a, cj(bi)));
    return csub(t, cmul(ai, cj(b)));
}

struct EpiArgs {
    const gb::SysDev* sys;
    const long long* base;      // prefix sums of N*R per cluster
    const long long* mie_off;
    const long long* obs_off;
    int nsys, R, source;
    int xs_L;                   // lmax stride of the xs rows (largest lmax of the batch)
    const double2* mie_scat;
    const double2* mie_int;
    const double2* p_inc;
    const double2* p_src;
    double eps_b;
    double2* p_scat;
    double2* p_int;
    const double2* pscat_in;    // given p_scat (general particles: T p_inc); null: t o p_inc
    double* xs;
    double* force;
    double* torque;
};

// One warp per (particle, rhs).  Lanes stride over the rows for p_scat / p_int,
// over the (a, n) multipoles for the cross-sections, and over the modes r for
// the force / torque sums; butterfly shuffles combine lane partials in a fixed
// order, so results do not depend on scheduling.
__global__ void __launch_bounds__(128) k_epilogue(EpiArgs a, long long total) {
    const long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (g >= total) return;
    int s = 0, hi = a.nsys - 1;   // last cluster whose base is <= g
    while (s < hi) {
        const int mid = (s + hi + 1) >> 1;
        if (a.base[mid] <= g) s = mid;
        else hi = mid - 1;
    }
    const gb::SysDev S = a.sys[s];
    const int R = a.R;
    const long long loc = g - a.base[s];
    const int i = (int)(loc / R), rr = (int)(loc % R);
    const int L = S.lmax, rmax = S.rmax, B = S.B;
    const double2* ms = a.mie_scat + a.mie_off[s] + (long long)i * 2 * L;
    const double2* mi = a.mie_int + a.mie_off[s] + (long long)i * 2 * L;
    const long long vb = S.vec_off + (long long)i * B * R + rr;   // row e at vb + e*R
    const double k = S.k;
    auto pin = [&](int e) { return a.p_inc[vb + (long long)e * R]; };
    auto psrc = [&](int e) { return a.p_src[vb + (long long)e * R]; };
    auto pscat = [&](int e) {
        return a.pscat_in ? a.pscat_in[vb + (long long)e * R] : cmul(pin(e), ms[__ldg(S.miecol + e)]);
    };
    // ---- p_scat, p_int (polarisation-swapped interior coefficients)
    for (int e = lane; e < B && !a.pscat_in; e += 32) {
        const double2 pi_ = pin(e);
        const int col = __ldg(S.miecol + e);   // a*L + n - 1
        if (a.p_scat) a.p_scat[vb + (long long)e * R] = cmul(pi_, ms[col]);
        if (a.p_int) {
            const int aa = col / L, n1 = col % L;
            a.p_int[vb + (long long)e * R] = cmul(pi_, mi[(1 - aa) * L + n1]);
        }
    }
    // ---- per-multipole cross-sections: lane per (a, n)
    if (a.xs) {
        const double f = 4.0 * kPi / (k * k);
        const int XL = a.xs_L;
        const long long xo = ((a.obs_off[s] + i) * R + rr) * 3LL * 2 * XL;
        for (int idx = lane; idx < 2 * L; idx += 32) {
            const int aa = idx / L, n = idx % L + 1;
            double cabs = 0.0, cext = 0.0;
            for (int m = -n; m <= n; m++) {
                const int e = aa * rmax + n * n + n + m - 1;
                const double2 pi_ = pin(e), pr = psrc(e);
                const double2 ps = a.pscat_in ? pscat(e) : cmul(pi_, ms[aa * L + n - 1]);
                cabs += f * ((pi_.x * ps.x + pi_.y * ps.y) - (ps.x * ps.x + ps.y * ps.y));
                cext += f * (pr.x * ps.x + pr.y * ps.y);
            }
            a.xs[xo + 0 * 2 * XL + idx] = cext - cabs;   // scattering
            a.xs[xo + 1 * 2 * XL + idx] = cabs;          // absorption
            a.xs[xo + 2 * 2 * XL + idx] = cext;          // extinction
        }
    }
    if (!a.force && !a.torque) return;
    // ---- force / torque: p, q = scattered electric / magnetic; pi, qi = incident
    auto P = [&](int r) { return pscat(r); };
    auto Qs = [&](int r) { return pscat(rmax + r); };
    auto PI = [&](int r) { return a.source ? pin(r) : csub(pin(r), psrc(r)); };
    auto QI = [&](int r) { return a.source ? pin(rmax + r) : csub(pin(rmax + r), psrc(rmax + r)); };
    const double eb = a.eps_b;
    const double Axy = kPi / (k * k) * kEps0 * eb;
    const double Az = -2 * Axy;
    const double At = -2 * kPi / (k * k * k) * kEps0 * eb;
    double2 Fxy = make_double2(0, 0), Fz = make_double2(0, 0);
    double T0 = 0, T1 = 0, T2 = 0;
    for (int r = lane; r < rmax; r += 32) {
        int n = (int)sqrt((double)(r + 1));
        while (n * n > r + 1) n--;
        while ((n + 1) * (n + 1) <= r + 1) n++;
        const int m = r + 1 - n * n - n;
        const double2 p = P(r), q = Qs(r), pi_ = PI(r), qi = QI(r);
        if (a.force) {
            if (m != n) {
                const double fc = Axy * sqrt((double)((n + m + 1) * (n - m))) / (double)(n * (n + 1));
                const int r1 = r + 1;
                const double2 p1 = P(r1), q1 = Qs(r1), pi1 = PI(r1), qi1 = QI(r1);
                Fxy = cadd(Fxy, cscale(fc, cadd(tri(p, q1, pi_, qi1), tri(q, p1, qi, pi1))));
            }
            const double fz = Az * m / (double)(n * (n + 1));
            Fz = cadd(Fz, cscale(fz, tri(p, q, pi_, qi)));
            if (n < L) {
                double fc = -Axy * sqrt((double)((n + m + 2) * (n + m + 1) * n * (n + 2)) /
                                        (double)((2 * n + 3) * (2 * n + 1))) / (n + 1);
                int r1 = (n + 1) * (n + 1) + (n + 1) + m;
                double2 p1 = P(r1), q1 = Qs(r1), pi1 = PI(r1), qi1 = QI(r1);
                Fxy = cadd(Fxy, cscale(fc, cadd(tri(p, p1, pi_, pi1), tri(q, q1, qi, qi1))));
                fc = Axy * sqrt((double)((n - m + 1) * (n - m + 2) * n * (n + 2)) /
                                (double)((2 * n + 3) * (2 * n + 1))) / (n + 1);
                r1 = (n + 1) * (n + 1) + (n + 1) + m - 2;
                p1 = P(r1); q1 = Qs(r1); pi1 = PI(r1); qi1 = QI(r1);
                Fxy = cadd(Fxy, cscale(fc, cadd(tri(p1, p, pi1, pi_), tri(q1, q, qi1, qi))));
                fc = Az * sqrt((double)((n - m + 1) * (n + m + 1) * n * (n + 2)) /
                               (double)((2 * n + 3) * (2 * n + 1))) / (n + 1);
                r1 = (n + 1) * (n + 1) + (n + 1) + m - 1;
                p1 = P(r1); q1 = Qs(r1); pi1 = PI(r1); qi1 = QI(r1);
                Fz = cadd(Fz, cscale(fc, cadd(tri(p1, p, pi1, pi_), tri(q1, q, qi1, qi))));
            }
        }
        if (a.torque) {
            if (m != n) {
                const double fc = -At * sqrt((double)((n - m) * (n + m + 1)));
                const int r1 = r + 1;
                const double2 p1 = P(r1), q1 = Qs(r1), pi1 = PI(r1), qi1 = QI(r1);
                const double2 base = cadd(cmul(p, cj(p1)), cmul(q, cj(q1)));
                const double2 sx = cadd(cadd(cmul(p1, cj(pi_)), cmul(p, cj(pi1))), cadd(cmul(q1, cj(qi)), cmul(q, cj(qi1))));
                const double2 sy = cadd(csub(cmul(p1, cj(pi_)), cmul(p, cj(pi1))), csub(cmul(q1, cj(qi)), cmul(q, cj(qi1))));
                T0 += fc * (base.x - 0.5 * sx.x);
                T1 += fc * (base.y + 0.5 * sy.y);
            }
            const double2 c = cadd(cmul(p, cj(pi_)), cmul(q, cj(qi)));
            T2 += At * m * ((p.x * p.x + p.y * p.y) + (q.x * q.x + q.y * q.y) - c.x);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        Fxy.x += __shfl_xor_sync(0xffffffffu, Fxy.x, o);
        Fxy.y += __shfl_xor_sync(0xffffffffu, Fxy.y, o);
        Fz.x += __shfl_xor_sync(0xffffffffu, Fz.x, o);
        T0 += __shfl_xor_sync(0xffffffffu, T0, o);
        T1 += __shfl_xor_sync(0xffffffffu, T1, o);
        T2 += __shfl_xor_sync(0xffffffffu, T2, o);
    }
    if (lane == 0) {
        const long long fo = ((a.obs_off[s] + i) * R + rr) * 3LL;
        if (a.force) {
            a.force[fo + 0] = Fxy.x;
            a.force[fo + 1] = Fxy.y;
            a.force[fo + 2] = Fz.x;
        }
        if (a.torque) {
            a.torque[fo + 0] = T0;
            a.torque[fo + 1] = T1;
            a.torque[fo + 2] = T2;
        }
    }
}

}   // namespace

extern "C" int gb_epilogue_batch(int nsys, const gb_system* sys, int R, const int64_t* mie_off,
                                 const int64_t* obs_off, const double* mie_scat, const double* mie_int,
                                 const double* p_inc, const double* p_src, double eps_b, int source, double* p_scat,
                                 double* p_int, double* xs, double* force, double* torque, void* stream) {
    if (nsys < 1 || !sys || !mie_off || !obs_off || !mie_scat || !p_inc || R < 1)
        return gb_set_error(GB_BAD_ARG, "bad epilogue arguments");
    if ((xs || !source) && !p_src) return gb_set_error(GB_BAD_ARG, "p_src required");
    if (p_int && !mie_int) return gb_set_error(GB_BAD_ARG, "mie_int required for p_int");
    cudaStream_t st_ = (cudaStream_t)stream;
    std::vector<gb::SysDev> sd;
    int st = gb::make_sysdev(nsys, sys, st_, sd);
    if (st) return st;
    std::vector<long long> base(nsys + 1, 0);
    for (int s = 0; s < nsys; s++) base[s + 1] = base[s] + (long long)sd[s].N * R;
    std::vector<unsigned char> blob(sizeof(gb::SysDev) * nsys + sizeof(long long) * (3 * nsys + 1));
    unsigned char* w = blob.data();
    memcpy(w, sd.data(), sizeof(gb::SysDev) * nsys);
    w += sizeof(gb::SysDev) * nsys;
    memcpy(w, base.data(), sizeof(long long) * (nsys + 1));
    w += sizeof(long long) * (nsys + 1);
    memcpy(w, mie_off, sizeof(long long) * nsys);
    w += sizeof(long long) * nsys;
    memcpy(w, obs_off, sizeof(long long) * nsys);
    void* dblob = nullptr;
    int slot = 0;
    st = gb::stage_acquire(blob.data(), blob.size(), st_, &dblob, &slot);
    if (st) return st;
    unsigned char* d = static_cast<unsigned char*>(dblob);
    EpiArgs a;
    a.sys = reinterpret_cast<const gb::SysDev*>(d);
    a.base = reinterpret_cast<const long long*>(d + sizeof(gb::SysDev) * nsys);
    a.mie_off = a.base + (nsys + 1);
    a.obs_off = a.mie_off + nsys;
    a.nsys = nsys;
    a.R = R;
    a.source = source;
    a.xs_L = 0;
    for (int s = 0; s < nsys; s++) a.xs_L = std::max(a.xs_L, sd[s].lmax);
    a.mie_scat = reinterpret_cast<const double2*>(mie_scat);
    a.mie_int = reinterpret_cast<const double2*>(mie_int);
    a.p_inc = reinterpret_cast<const double2*>(p_inc);
    a.p_src = reinterpret_cast<const double2*>(p_src);
    a.eps_b = eps_b;
    a.p_scat = reinterpret_cast<double2*>(p_scat);
    a.p_int = reinterpret_cast<double2*>(p_int);
    a.xs = xs;
    a.force = force;
    a.torque = torque;
    a.pscat_in = nullptr;
    const long long total = base[nsys];
    gb::note_launch();
    k_epilogue<<<(unsigned)((total * 32 + 127) / 128), 128, 0, st_>>>(a, total);
    GB_CUDA_TRY(cudaGetLastError());
    return gb::stage_release(slot, st_);
}

// p_scat = T p_inc for clusters of general particles (cluster.py:652-657): one
// thread per (cluster, row, rhs), B-term dot product with the particle's T-matrix row.
namespace {
__global__ void k_apply_tmat(const gb::SysDev* __restrict__ sys, const long long* __restrict__ base, int nsys, int R,
                             const double2* __restrict__ p_inc, double2* __restrict__ p_scat, long long total) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x) {
        int s = 0, hi = nsys - 1;
        while (s < hi) {
            const int mid = (s + hi + 1) >> 1;
            if (base[mid] <= g) s = mid;
            else hi = mid - 1;
        }
        const gb::SysDev S = sys[s];
        const long long loc = g - base[s];   // (row, rhs) within the cluster
        const int rr = (int)(loc % R);
        const long long row = loc / R;
        const int B = S.B, part = (int)(row / B), e = (int)(row % B);
        const double2* Tr = S.tmat128 + ((long long)part * B + e) * B;
        const double2* xin = p_inc + S.vec_off + (long long)part * B * R + rr;
        double2 acc = make_double2(0, 0);
        for (int c = 0; c < B; c++) cfma(acc, __ldg(Tr + c), xin[(long long)c * R]);
        p_scat[S.vec_off + row * R + rr] = acc;
    }
}
}   // namespace

extern "C" int gb_tmatrix_epilogue_batch(int nsys, const gb_system* sys, int R, const double* tmat128,
                                         const int64_t* tm_off, const int64_t* obs_off, const double* p_inc,
                                         const double* p_src, double eps_b, int source, double* p_scat, double* xs,
                                         double* force, double* torque, void* stream) {
    if (nsys < 1 || !sys || !tmat128 || !tm_off || !obs_off || !p_inc || !p_scat || R < 1)
        return gb_set_error(GB_BAD_ARG, "bad epilogue arguments");
    if ((xs || !source) && !p_src) return gb_set_error(GB_BAD_ARG, "p_src required");
    cudaStream_t st_ = (cudaStream_t)stream;
    std::vector<gb::SysDev> sd;
    int st = gb::make_sysdev(nsys, sys, st_, sd);
    if (st) return st;
    std::vector<long long> rows(nsys + 1, 0), base(nsys + 1, 0), zeros(nsys, 0);
    for (int s = 0; s < nsys; s++) {
        sd[s].tmat128 = reinterpret_cast<const double2*>(tmat128) + tm_off[s];
        rows[s + 1] = rows[s] + (long long)sd[s].D * R;
        base[s + 1] = base[s] + (long long)sd[s].N * R;
    }
    std::vector<unsigned char> blob(sizeof(gb::SysDev) * nsys + sizeof(long long) * (4 * nsys + 2));
    unsigned char* w = blob.data();
    memcpy(w, sd.data(), sizeof(gb::SysDev) * nsys);
    w += sizeof(gb::SysDev) * nsys;
    memcpy(w, base.data(), sizeof(long long) * (nsys + 1));
    w += sizeof(long long) * (nsys + 1);
    memcpy(w, zeros.data(), sizeof(long long) * nsys);
    w += sizeof(long long) * nsys;
    memcpy(w, obs_off, sizeof(long long) * nsys);
    w += sizeof(long long) * nsys;
    memcpy(w, rows.data(), sizeof(long long) * (nsys + 1));
    void* dblob = nullptr;
    int slot = 0;
    st = gb::stage_acquire(blob.data(), blob.size(), st_, &dblob, &slot);
    if (st) return st;
    unsigned char* d = static_cast<unsigned char*>(dblob);
    const gb::SysDev* dsys = reinterpret_cast<const gb::SysDev*>(d);
    const long long* dbase = reinterpret_cast<const long long*>(d + sizeof(gb::SysDev) * nsys);
    const long long* drows = dbase + (nsys + 1) + 2 * nsys;
    const long long total_rows = rows[nsys];
    gb::note_launch();
    k_apply_tmat<<<(unsigned)std::min<long long>((total_rows + 255) / 256, 65535), 256, 0, st_>>>(
        dsys, drows, nsys, R, reinterpret_cast<const double2*>(p_inc), reinterpret_cast<double2*>(p_scat), total_rows);
    GB_CUDA_TRY(cudaGetLastError());
    EpiArgs a;
    a.sys = dsys;
    a.base = dbase;
    a.mie_off = dbase + (nsys + 1);
    a.obs_off = a.mie_off + nsys;
    a.nsys = nsys;
    a.R = R;
    a.source = source;
    a.xs_L = 0;
    for (int s = 0; s < nsys; s++) a.xs_L = std::max(a.xs_L, sd[s].lmax);
    a.mie_scat = nullptr;
    a.mie_int = nullptr;
    a.p_inc = reinterpret_cast<const double2*>(p_inc);
    a.p_src = reinterpret_cast<const double2*>(p_src);
    a.eps_b = eps_b;
    a.p_scat = nullptr;
    a.p_int = nullptr;
    a.pscat_in = reinterpret_cast<const double2*>(p_scat);
    a.xs = xs;
    a.force = force;
    a.torque = torque;
    const long long total = base[nsys];
    gb::note_launch();
    k_epilogue<<<(unsigned)((total * 32 + 127) / 128), 128, 0, st_>>>(a, total);
    GB_CUDA_TRY(cudaGetLastError());
    return gb::stage_release(slot, st_);
}

// Per-particle cross-sections from given coefficients (flux.particle_cross_sections,
// cpp/src/flux.cpp:5-30): one thread per (particle, a, n).
namespace {
__global__ void k_particle_xs(int N, int lmax, const double2* __restrict__ ps, const double2* __restrict__ pi,
                              const double2* __restrict__ pr, double k, double* __restrict__ out) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= N * 2 * lmax) return;
    const int i = g / (2 * lmax), idx = g % (2 * lmax), a = idx / lmax, n = idx % lmax + 1;
    const int rmax = lmax * (lmax + 2);
    const double f = 4.0 * 3.14159265358979323846 / (k * k);
    double cabs = 0.0, cext = 0.0;
    for (int m = -n; m <= n; m++) {
        const long long e = (long long)i * 2 * rmax + a * rmax + n * n + n + m - 1;
        const double2 s = ps[e], c = pi[e], r = pr[e];
        cabs += f * ((c.x * s.x + c.y * s.y) - (s.x * s.x + s.y * s.y));
        cext += f * (r.x * s.x + r.y * s.y);
    }
    double* o = out + (long long)i * 6 * lmax;
    o[idx] = cext - cabs;
    o[2 * lmax + idx] = cabs;
    o[4 * lmax + idx] = cext;
}
}   // namespace

extern "C" int gb_particle_cross_sections(int N, int lmax, const double* p_scat, const double* p_inc,
                                          const double* p_src, double k, double* out, void* stream) {
    if (N < 1 || lmax < 1 || !p_scat || !p_inc || !p_src || !out) return gb_set_error(GB_BAD_ARG, "bad arguments");
    const int total = N * 2 * lmax;
    gb::note_launch();
    k_particle_xs<<<(total + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
        N, lmax, reinterpret_cast<const double2*>(p_scat), reinterpret_cast<const double2*>(p_inc),
        reinterpret_cast<const double2*>(p_src), k, out);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

// --------------------------------------------- general-particle aggregate --
// The dense aggregate of clusters of general particles (particle_aggregate_tmatrix,
// cpp/src/interactions.cpp:417-462, with the T-matrix overload of
// vsh_translation_insert_pair, cpp/src/vsh_translation.cpp:53-159): block (i, j)
// is A_ij T_j for i != j, zero for i = j, where A is the translation matrix with
// unit Mie coefficients (the sphere assembler's dense output) and T_j the particle's
// B x B T-matrix.  A batched complex128 block product on the FP64 pipe: one CTA per
// (i, j, 32 x 32 output tile), K staged through shared memory in steps of 16, each
// thread 2 x 2 outputs.
namespace {
constexpr int kBT = 32, kBK = 16;

__global__ void k_unit_mie(double2* __restrict__ u, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        u[e] = make_double2(1.0, 0.0);
}

__global__ void __launch_bounds__(256)
k_block_tmat_product(int N, int B, const double2* __restrict__ A, const double2* __restrict__ T,
                     double2* __restrict__ out) {
    const int tiles = (B + kBT - 1) / kBT;
    const int tr = blockIdx.x / tiles, tc = blockIdx.x - tr * tiles;
    const int j = blockIdx.y, i = blockIdx.z;
    const long long D = (long long)N * B;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int r0 = tr * kBT + 2 * ty, c0 = tc * kBT + 2 * tx;
    double2* ob = out + (long long)i * B * D + (long long)j * B;
    if (i == j) {   // diagonal blocks stay zero
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
            for (int b = 0; b < 2; b++)
                if (r0 + a < B && c0 + b < B) ob[(long long)(r0 + a) * D + c0 + b] = make_double2(0, 0);
        return;
    }
    __shared__ double2 As[kBT][kBK + 1], Ts[kBK][kBT + 1];
    const double2* ab = A + (long long)i * B * D + (long long)j * B;
    const double2* tb = T + (long long)j * B * B;
    double2 acc[2][2];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) acc[a][b] = make_double2(0, 0);
    for (int k0 = 0; k0 < B; k0 += kBK) {
        for (int e = tid; e < kBT * kBK; e += 256) {
            const int rr = e / kBK, kk = e - rr * kBK;   // A tile: rows of block i, columns k0..
            const int r = tr * kBT + rr, k = k0 + kk;
            As[rr][kk] = (r < B && k < B) ? __ldg(ab + (long long)r * D + k) : make_double2(0, 0);
            const int kr = e / kBT, cc = e - kr * kBT;   // T tile: rows k0.., columns of the output tile
            const int kt = k0 + kr, c = tc * kBT + cc;
            Ts[kr][cc] = (kt < B && c < B) ? __ldg(tb + (long long)kt * B + c) : make_double2(0, 0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; kk++) {
            const double2 a0 = As[2 * ty][kk], a1 = As[2 * ty + 1][kk];
            const double2 t0 = Ts[kk][2 * tx], t1 = Ts[kk][2 * tx + 1];
            cfma(acc[0][0], a0, t0);
            cfma(acc[0][1], a0, t1);
            cfma(acc[1][0], a1, t0);
            cfma(acc[1][1], a1, t1);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
            if (r0 + a < B && c0 + b < B) ob[(long long)(r0 + a) * D + c0 + b] = acc[a][b];
}
}   // namespace

extern "C" size_t gb_particle_aggregate_workspace_size(int N, int lmax) {
    if (N < 1 || lmax < 1 || lmax > GB_LMAX_MAX) return 0;
    const long long D = 2LL * lmax_to_rmax(lmax) * N;
    return sizeof(double2) * (size_t)(D * D + 2LL * N * lmax);
}

extern "C" int gb_particle_aggregate_dense(int N, int lmax, const double* pos, const double* tmat, double k,
                                           void* workspace, size_t ws_bytes, double* out, void* stream) {
    if (!pos || !tmat || !workspace || !out) return gb_set_error(GB_BAD_ARG, "null pointer");
    if (N < 1 || lmax < 1 || lmax > GB_LMAX_MAX) return gb_set_error(GB_BAD_ARG, "N=%d lmax=%d invalid", N, lmax);
    if (N > 65535) return gb_set_error(GB_UNSUPPORTED, "more than 65535 particles");
    const size_t need = gb_particle_aggregate_workspace_size(N, lmax);
    if (ws_bytes < need) return gb_set_error(GB_OVER_BUDGET, "workspace %zu B < required %zu B", ws_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    const int B = 2 * lmax_to_rmax(lmax);
    const long long D = (long long)B * N;
    double2* A = static_cast<double2*>(workspace);
    double2* unit = A + D * D;
    gb::note_launch();
    k_unit_mie<<<(unsigned)((2LL * N * lmax + 255) / 256), 256, 0, st>>>(unit, 2LL * N * lmax);
    GB_CUDA_TRY(cudaGetLastError());
    const int e = gb_assemble_sphere_dense(N, lmax, pos, reinterpret_cast<const double*>(unit), k,
                                           reinterpret_cast<double*>(A), stream);
    if (e) return e;
    const int tiles = (B + kBT - 1) / kBT;
    gb::note_launch();
    k_block_tmat_product<<<dim3((unsigned)(tiles * tiles), (unsigned)N, (unsigned)N), 256, 0, st>>>(
        N, B, A, reinterpret_cast<const double2*>(tmat), reinterpret_cast<double2*>(out));
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}
