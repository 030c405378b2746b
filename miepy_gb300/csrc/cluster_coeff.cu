// Cluster expansion coefficients and far fields.
//
// p_cluster: the scattered field of every particle re-expanded about one origin
// (cluster_coefficients, vsh/cluster_coefficients.py:14-53): for particle i at
// x_i != origin, with (r, theta, phi) of origin - x_i,
//   p_cluster[0][n,m] += sum_{v,u} a_i(v,u) A + b_i(v,u) B
//   p_cluster[1][n,m] += sum_{v,u} a_i(v,u) B + b_i(v,u) A,
// A, B = vsh_translation(m, n, u, v, r, theta, phi, k, incident)
// (cpp/src/vsh_translation.cpp:428-470): the folded Gaunt coefficients of the cross
// tables times G[p][mu] = P_p^mu(cos theta) j_p(k r) e^{i mu phi}.  j_p follows the
// reference's upward recurrence (cpp/src/special.cpp:20-45), which loses digits for
// p > k r, as the reference's own values do.  A particle at the origin adds its own
// coefficients.  One CTA per particle writes its contribution; a second kernel sums
// the particles in index order (deterministic).
//
// Far field: E_angular / H_angular (sphere_cluster.py:393-426): the far-field
// expansion expand_E_far (vsh/expansion.py:45-77) of every particle's p_scat about
// its own centre, evaluated at points (R, theta, phi) about the origin, summed in
// Cartesian components and returned as (E_theta, E_phi) at the point.  H uses the
// swapped coefficients times hfac = -i sqrt(eps_b / mu_b) (expand_H_far, :96-108).

#include <algorithm>
#include <cstring>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace {

constexpr int kCCThreads = 256;
constexpr int kLFF = GB_LMAX_MAX;                // largest order of the far-field kernel
constexpr int kPMax = 2 * GB_LMAX_MAX + 2;      // orders p <= Lc + Lin + 1
constexpr int kMUMax = 4 * GB_LMAX_MAX + 1;     // |mu| <= Lc + Lin

__device__ __forceinline__ double2 mul_ipow_cc(double2 z, int k) {
    switch (k & 3) {
        case 0: return z;
        case 1: return make_double2(-z.y, z.x);
        case 2: return make_double2(-z.x, -z.y);
        default: return make_double2(z.y, -z.x);
    }
}

__global__ void __launch_bounds__(kCCThreads)
k_cluster_contrib(int N, int Lin, int Lc, const double* __restrict__ pos, const double2* __restrict__ p_scat,
                  double k, double ox, double oy, double oz, const int4* __restrict__ nmvu,
                  const int2* __restrict__ qab, const double* __restrict__ cA, const double* __restrict__ cB,
                  int Q, const double* __restrict__ neg_ratio, double2* __restrict__ contrib) {
    __shared__ double jp[kPMax];
    __shared__ double Pl[kPMax][kPMax];
    __shared__ double2 eph[kMUMax];
    __shared__ double2 G[kPMax][kMUMax];
    __shared__ double geo[6];
    const int ri = Lin * (Lin + 2), rc = Lc * (Lc + 2);
    const int PM = Lc + Lin + 1;            // orders p = 0 .. Lc + Lin
    const int MO = Lc + Lin;                // |mu| <= MO
    const int MU = 2 * MO + 1;
    const int PMn = Lc + Lin + 2;           // stride of neg_ratio
    const int tid = threadIdx.x;
    for (int i = blockIdx.x; i < N; i += gridDim.x) {
        const double2* ps = p_scat + (long long)i * 2 * ri;
        double2* out = contrib + (long long)i * 2 * rc;
        const double dx = ox - pos[3 * i], dy = oy - pos[3 * i + 1], dz = oz - pos[3 * i + 2];
        if (dx == 0.0 && dy == 0.0 && dz == 0.0) {   // particle at the origin: its own coefficients
            for (int e = tid; e < 2 * rc; e += kCCThreads) {
                const int a = e / rc, r = e % rc;
                out[e] = (r < ri) ? ps[a * ri + r] : make_double2(0.0, 0.0);
            }
            __syncthreads();
            continue;
        }
        if (tid == 0) {
            const double rho2 = dx * dx + dy * dy;
            const double rad = sqrt(rho2 + dz * dz);
            const double rho = sqrt(rho2);
            geo[0] = dz / rad;                           // cos(theta)
            geo[1] = rho / rad;                          // sin(theta)
            geo[2] = rho2 > 0.0 ? dx / rho : 1.0;        // cos(phi); phi = 0 on the z axis
            geo[3] = rho2 > 0.0 ? dy / rho : 0.0;        // sin(phi)
            // j_p(k r) by the reference's upward recurrence
            const double z = k * rad;
            double sz, cz;
            sincos(z, &sz, &cz);
            double j2p = sz / z;
            jp[0] = j2p;
            if (PM > 1) {
                double j1 = j2p / z - cz / z;
                jp[1] = j1;
                for (int p = 2; p < PM; p++) {
                    const double jn = (2.0 * p - 1.0) / z * j1 - j2p;
                    j2p = j1;
                    j1 = jn;
                    jp[p] = jn;
                }
            }
        }
        __syncthreads();
        // Legendre P_p^mu (no Condon-Shortley phase), one thread per mu; e^{i mu phi}
        if (tid < PM) {
            const int mu = tid;
            const double x = geo[0], u = geo[1];
            double pmm = 1.0;
            for (int kk = 1; kk <= mu; kk++) pmm *= (2 * kk - 1) * u;
            Pl[mu][mu] = pmm;
            if (mu + 1 < PM) {
                double pa = pmm, pb = x * (2 * mu + 1) * pmm;
                Pl[mu + 1][mu] = pb;
                for (int q = mu + 2; q < PM; q++) {
                    const double pc = ((2 * q - 1) * x * pb - (q + mu - 1) * pa) / (double)(q - mu);
                    Pl[q][mu] = pc;
                    pa = pb;
                    pb = pc;
                }
            }
        } else if (tid >= 64 && tid < 64 + MO + 1) {
            const int mu = tid - 64;
            int e = mu;
            double2 acc = make_double2(1.0, 0.0), base = make_double2(geo[2], geo[3]);
            while (e) {
                if (e & 1) acc = cmul(acc, base);
                base = cmul(base, base);
                e >>= 1;
            }
            eph[MO + mu] = acc;
            eph[MO - mu] = make_double2(acc.x, -acc.y);
        }
        __syncthreads();
        for (int e = tid; e < PM * MU; e += kCCThreads) {
            const int q = e / MU, mi = e % MU, mu = mi - MO, am = mu < 0 ? -mu : mu;
            double2 g = make_double2(0.0, 0.0);
            if (am <= q) {
                double P = Pl[q][am];
                if (mu < 0) P *= neg_ratio[q * PMn + am];
                const double f = P * jp[q];
                g = make_double2(f * eph[mi].x, f * eph[mi].y);
            }
            G[q][mi] = g;
        }
        __syncthreads();
        // one thread per outgoing mode (n, m): sum over the particle's modes (v, u)
        for (int r = tid; r < rc; r += kCCThreads) {
            double2 acc0 = make_double2(0.0, 0.0), acc1 = make_double2(0.0, 0.0);
            for (int s = 0; s < ri; s++) {
                const int t = r * ri + s;
                const int4 e4 = nmvu[t];
                const int2 qq = qab[t];
                const int mi = (e4.w - e4.y) + MO;
                const int nv = e4.x + e4.z;
                double2 sa = make_double2(0.0, 0.0), sb = make_double2(0.0, 0.0);
                for (int q = 0; q <= qq.x; q++) {
                    const double c = cA[(size_t)t * Q + q];
                    const double2 gv = G[nv - 2 * q][mi];
                    sa.x = fma(c, gv.x, sa.x);
                    sa.y = fma(c, gv.y, sa.y);
                }
                for (int q = 1; q <= qq.y; q++) {
                    const double c = cB[(size_t)t * Q + q];
                    const double2 gv = G[nv - 2 * q + 1][mi];
                    sb.x = fma(c, gv.x, sb.x);
                    sb.y = fma(c, gv.y, sb.y);
                }
                const double2 A = mul_ipow_cc(sa, nv), Bt = mul_ipow_cc(sb, nv + 1);
                const double2 a = ps[s], b = ps[ri + s];
                cfma(acc0, a, A);
                cfma(acc0, b, Bt);
                cfma(acc1, a, Bt);
                cfma(acc1, b, A);
            }
            out[r] = acc0;
            out[rc + r] = acc1;
        }
        __syncthreads();
    }
}

__global__ void k_cluster_sum(int N, int n2rc, const double2* __restrict__ contrib, double2* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n2rc) return;
    double2 s = make_double2(0.0, 0.0);
    for (int i = 0; i < N; i++) {
        const double2 v = contrib[(long long)i * n2rc + e];
        s.x += v.x;
        s.y += v.y;
    }
    out[e] = s;
}

// ---------------------------------------------------------------- far field --
constexpr int kFFThreads = 128;

__device__ double2 emn_cc(int m, int n) {
    const double mag = sqrt((2.0 * n + 1) * tgamma((double)(n - m) + 1.0) /
                            ((double)n * (n + 1) * tgamma((double)(n + m) + 1.0)));
    switch (n & 3) {
        case 0: return make_double2(mag, 0);
        case 1: return make_double2(0, mag);
        case 2: return make_double2(-mag, 0);
        default: return make_double2(0, -mag);
    }
}

__global__ void __launch_bounds__(kFFThreads)
k_far_field(int N, int L, const double* __restrict__ pos, const double2* __restrict__ p_scat, double k,
            double ox, double oy, double oz, int Npts, const double* __restrict__ R, const double* __restrict__ th,
            const double* __restrict__ ph, int magnetic, double2 hfac, double2* __restrict__ out) {
    const int rmax = L * (L + 2);
    __shared__ double2 w[kLFF * (kLFF + 2)];       // E_mn (-i)^n
    __shared__ double negf[kLFF * (kLFF + 2)];
    for (int r = threadIdx.x; r < rmax; r += blockDim.x) {
        int n = (int)floor(sqrt((double)r + 1.0));
        while (n * n > r + 1) n--;
        while ((n + 1) * (n + 1) <= r + 1) n++;
        const int m = r + 1 - n * n - n;
        w[r] = mul_ipow_cc(emn_cc(m, n), 3 * n);   // (-i)^n = i^(3n)
        const int am = m < 0 ? -m : m;
        negf[r] = (m < 0) ? (((am & 1) ? -1.0 : 1.0) * tgamma((double)(n - am) + 1.0) / tgamma((double)(n + am) + 1.0)) : 1.0;
    }
    __syncthreads();
    const int pt = blockIdx.x * blockDim.x + threadIdx.x;
    if (pt >= Npts) return;
    double st0, ct0, sp0, cp0;
    sincos(th[pt], &st0, &ct0);
    sincos(ph[pt], &sp0, &cp0);
    const double X = ox + R[pt] * st0 * cp0, Y = oy + R[pt] * st0 * sp0, Z = oz + R[pt] * ct0;
    double2 E[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
    for (int i = 0; i < N; i++) {
        const double dx = X - pos[3 * i], dy = Y - pos[3 * i + 1], dz = Z - pos[3 * i + 2];
        const double rho2 = dx * dx + dy * dy;
        const double rad = sqrt(rho2 + dz * dz);
        const double rho = sqrt(rho2);
        const double ct = dz / rad, st = rho / rad;
        const double cph = rho2 > 0 ? dx / rho : 1.0, sph = rho2 > 0 ? dy / rho : 0.0;
        double s, c;
        sincos(k * rad, &s, &c);
        const double2 fac = make_double2(c / (k * rad), s / (k * rad));   // e^{ikr} / (kr)
        // Legendre P_n^m(ct), m >= 0, n <= L + 1
        double P[kLFF + 2][kLFF + 2];
        P[0][0] = 1.0;
        for (int m = 1; m <= L + 1; m++) P[m][m] = (2 * m - 1) * st * P[m - 1][m - 1];
        for (int m = 0; m <= L; m++) P[m + 1][m] = ct * (2 * m + 1) * P[m][m];
        for (int m = 0; m <= L + 1; m++)
            for (int n = m + 2; n <= L + 1; n++)
                P[n][m] = ((2 * n - 1) * ct * P[n - 1][m] - (n + m - 1) * P[n - 2][m]) / (double)(n - m);
        const bool axis = !(st > 0.0);
        const double2* c0 = p_scat + (long long)i * 2 * rmax + (magnetic ? rmax : 0);
        const double2* c1 = p_scat + (long long)i * 2 * rmax + (magnetic ? 0 : rmax);
        double2 Et = make_double2(0, 0), Ep = make_double2(0, 0);
        for (int n = 1; n <= L; n++) {
            for (int m = -n; m <= n; m++) {
                const int am = m < 0 ? -m : m;
                const int r = n * n + n + m - 1;
                double pi_v, tau_v;
                if (axis) {
                    const bool atpi = ct < 0;
                    const double sgn = atpi ? (((n + 1) & 1) ? -1.0 : 1.0) : 1.0;
                    const double sgt = atpi ? ((n & 1) ? -1.0 : 1.0) : 1.0;
                    if (m == 1) { pi_v = sgn * n * (n + 1) / 2.0; tau_v = sgt * n * (n + 1) / 2.0; }
                    else if (m == -1) { pi_v = sgn * 0.5; tau_v = -sgt * 0.5; }
                    else { pi_v = 0.0; tau_v = 0.0; }
                } else {
                    pi_v = m / st * negf[r] * P[n][am];
                    const double pm1 = (am >= 1) ? P[n][am - 1] : -P[n][1] / (double)(n * (n + 1));
                    const double pp1 = (am + 1 <= n) ? P[n][am + 1] : 0.0;
                    tau_v = negf[r] * 0.5 * ((n + am) * (n - am + 1) * pm1 - pp1);
                }
                // e^{i m phi}
                double2 e = make_double2(1.0, 0.0), base = make_double2(cph, am == m ? sph : -sph);
                for (int q = 0; q < am; q++) e = cmul(e, base);
                const double2 f = cmul(cmul(fac, w[r]), e);
                const double2 a = c0[r], b = c1[r];
                const double2 u1 = make_double2(a.x * tau_v + b.x * pi_v, a.y * tau_v + b.y * pi_v);
                const double2 u2 = make_double2(a.x * pi_v + b.x * tau_v, a.y * pi_v + b.y * tau_v);
                const double2 t1 = cmul(f, u1);   // E_theta += i f (a tau + b pi)
                Et.x += -t1.y;
                Et.y += t1.x;
                const double2 t2 = cmul(f, u2);   // E_phi -= f (a pi + b tau)
                Ep.x -= t2.x;
                Ep.y -= t2.y;
            }
        }
        // (0, E_theta, E_phi) at the particle's angles -> Cartesian
        const double th_[3] = {ct * cph, ct * sph, -st}, ph_[3] = {-sph, cph, 0.0};
        for (int d = 0; d < 3; d++) {
            E[d].x += Et.x * th_[d] + Ep.x * ph_[d];
            E[d].y += Et.y * th_[d] + Ep.y * ph_[d];
        }
    }
    // Cartesian -> (theta, phi) components at the point
    const double tt[3] = {ct0 * cp0, ct0 * sp0, -st0}, pp[3] = {-sp0, cp0, 0.0};
    double2 Eth = make_double2(0, 0), Eph = make_double2(0, 0);
    for (int d = 0; d < 3; d++) {
        Eth.x += E[d].x * tt[d]; Eth.y += E[d].y * tt[d];
        Eph.x += E[d].x * pp[d]; Eph.y += E[d].y * pp[d];
    }
    if (magnetic) {
        Eth = cmul(hfac, Eth);
        Eph = cmul(hfac, Eph);
    }
    out[2LL * pt] = Eth;
    out[2LL * pt + 1] = Eph;
}

}   // namespace

extern "C" {

size_t gb_cluster_coefficients_workspace_size(int N, int lmax_cluster) {
    if (N < 1 || lmax_cluster < 1) return 0;
    return sizeof(double2) * 2 * (size_t)lmax_to_rmax(lmax_cluster) * N;
}

int gb_cluster_coefficients(int N, int lmax, const double* pos, const double* p_scat, double k, const double* origin,
                            int lmax_cluster, double* p_cluster, void* workspace, size_t ws_bytes, void* stream) {
    if (N < 1 || !pos || !p_scat || !origin || !p_cluster || !workspace)
        return gb_set_error(GB_BAD_ARG, "bad cluster-coefficient arguments");
    if (lmax < 1 || lmax > GB_LMAX_MAX || lmax_cluster < 1 || lmax_cluster > GB_LMAX_MAX)
        return gb_set_error(GB_UNSUPPORTED, "orders must be in 1..%d (got %d, %d)", GB_LMAX_MAX, lmax, lmax_cluster);
    if (ws_bytes < gb_cluster_coefficients_workspace_size(N, lmax_cluster))
        return gb_set_error(GB_OVER_BUDGET, "workspace too small for %d particles", N);
    if (lmax_to_rmax(lmax_cluster) > kCCThreads * 64) return gb_set_error(GB_UNSUPPORTED, "lmax_cluster too large");
    cudaStream_t s = (cudaStream_t)stream;
    const gb::CrossTables* T = nullptr;
    int e = gb::get_cross_tables(lmax_cluster, lmax, s, &T);
    if (e) return e;
    double o[3];
    memcpy(o, origin, sizeof(o));   // host array
    const int grid = std::min(N, gb::sm_count() * 8);
    double2* contrib = static_cast<double2*>(workspace);
    gb::note_launch();
    k_cluster_contrib<<<grid, kCCThreads, 0, s>>>(N, lmax, lmax_cluster, pos, reinterpret_cast<const double2*>(p_scat),
                                                  k, o[0], o[1], o[2], T->nmvu, T->qab, T->cA, T->cB, T->Q,
                                                  T->neg_ratio, contrib);
    GB_CUDA_TRY(cudaGetLastError());
    const int n2rc = 2 * lmax_to_rmax(lmax_cluster);
    gb::note_launch();
    k_cluster_sum<<<(n2rc + 127) / 128, 128, 0, s>>>(N, n2rc, contrib, reinterpret_cast<double2*>(p_cluster));
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

int gb_far_field(int N, int lmax, const double* pos, const double* p_scat, double k, const double* origin, int Npts,
                 const double* radius, const double* theta, const double* phi, int magnetic, double hfac_re,
                 double hfac_im, double* out, void* stream) {
    if (N < 1 || Npts < 0 || !pos || !p_scat || !origin || !out) return gb_set_error(GB_BAD_ARG, "bad far-field arguments");
    if (lmax < 1 || lmax > kLFF) return gb_set_error(GB_UNSUPPORTED, "far field supports lmax 1..%d", kLFF);
    if (Npts == 0) return GB_OK;
    if (!radius || !theta || !phi) return gb_set_error(GB_BAD_ARG, "null point arrays");
    double o[3];
    memcpy(o, origin, sizeof(o));
    gb::note_launch();
    k_far_field<<<(Npts + kFFThreads - 1) / kFFThreads, kFFThreads, 0, (cudaStream_t)stream>>>(
        N, lmax, pos, reinterpret_cast<const double2*>(p_scat), k, o[0], o[1], o[2], Npts, radius, theta, phi,
        magnetic, make_double2(hfac_re, hfac_im), reinterpret_cast<double2*>(out));
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

}   // extern "C"
