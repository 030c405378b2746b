// K8: near field of a cluster on a set of points.
//
// Follows sphere_cluster.E_field / H_field (sphere_cluster.py:244-391): outside
// the spheres the outgoing expansions of p_scat about every particle are summed
// (expand_E, vsh/expansion.py:13-42, VSH N/M of vsh/vsh_functions.py:40-78 /
// cpp/src/vsh_functions.cpp:60-98, converted with vec_sph_to_cart); a point
// inside sphere i instead takes the interior expansion of p_int[i] with
// j_n(k_int r) (complex argument, the upward recurrence of
// cpp/src/special.cpp:20-45).  H fields use expand_H: the polarisation-swapped
// coefficients times -i sqrt(eps/mu).
//
// One thread per point; particles are streamed through shared memory in tiles of
// 16 with their coefficients; E_mn and the negative-order Legendre factors are
// tabulated once per CTA.

#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace {

constexpr int kFieldThreads = 128;

__device__ __forceinline__ double2 cdivd(double2 a, double2 b) {
    const double den = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}
__device__ __forceinline__ double2 cadd2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csin(double2 z) {
    double s, c;
    sincos(z.x, &s, &c);
    return make_double2(s * cosh(z.y), c * sinh(z.y));
}
__device__ __forceinline__ double2 ccos(double2 z) {
    double s, c;
    sincos(z.x, &s, &c);
    return make_double2(c * cosh(z.y), -s * sinh(z.y));
}

// E_mn = i^n sqrt((2n+1)(n-m)!/(n(n+1)(n+m)!))  (cpp/src/vsh_functions.cpp:56-58)
__device__ double2 Emn(int m, int n) {
    double mag = sqrt((2.0 * n + 1) * tgamma((double)(n - m) + 1.0) / ((double)n * (n + 1) * tgamma((double)(n + m) + 1.0)));
    switch (n & 3) {
        case 0: return make_double2(mag, 0);
        case 1: return make_double2(0, mag);
        case 2: return make_double2(-mag, 0);
        default: return make_double2(0, -mag);
    }
}

// Adds the expansion of coefficients c [2][rmax] about a particle to E (spherical
// components, then Cartesian).  outgoing: h_n of real kr, factor i;
// otherwise j_n of complex kr, factor -i.
constexpr int kLF = 8;   // largest expansion order of the field kernel

// far: the outgoing expansion's far-field form instead (expand_E_far,
// vsh/expansion.py:45-77): no radial component, h_n(kr) -> (-i)^n e^{ikr} / (kr) with
// E_theta = i f E_mn (-i)^n (c0 tau + c1 pi) e^{im phi},
// E_phi = -f E_mn (-i)^n (c0 pi + c1 tau) e^{im phi}, f = e^{ikr} / (kr).
__device__ void add_expansion(int L, const double2* __restrict__ c, int rmax, bool outgoing, double2 k, double rad,
                              double theta, double phi, bool swap, double2 pref, const double2* __restrict__ emn,
                              const double* __restrict__ negf_tab, double2 E[3], bool far = false) {
    const int NP = L + 2;
    // radial functions z_n and derivatives for n = 0..L (the reference's recurrences)
    double2 z[kLF + 2], zp[kLF + 2];
    const double2 kr = make_double2(k.x * rad, k.y * rad);
    double2 ffar = make_double2(0, 0);
    if (far) {
        double s, co;
        sincos(kr.x, &s, &co);
        ffar = make_double2(co / kr.x, s / kr.x);
    } else if (outgoing) {
        const double x = kr.x;
        double s, co;
        sincos(x, &s, &co);
        double j0 = s / x, y0 = -co / x;
        z[0] = make_double2(j0, y0);
        double j1 = j0 / x - co / x, y1 = y0 / x - j0;
        if (NP > 1) z[1] = make_double2(j1, y1);
        double ja = j0, jb = j1, ya = y0, yb = y1;
#pragma unroll 1
        for (int n = 2; n < NP; n++) {
            double jn = (2 * n - 1) / x * jb - ja, yn = (2 * n - 1) / x * yb - ya;
            ja = jb; jb = jn; ya = yb; yb = yn;
            z[n] = make_double2(jn, yn);
        }
    } else {
        // j_n of complex argument.  The upward recurrence (the reference's,
        // cpp/src/special.cpp:20-45) multiplies its rounding errors by about
        // |y_n / j_n| ~ ((2n-1)!!)^2 / |kr|^(2n+1) once n > |kr|, so it serves only
        // |kr| >= NP; below that the values come from Miller's downward recurrence
        // j_{n-1} = (2n+1)/kr j_n - j_{n+1}, started at n = NP + 24 from (j, j+1) =
        // (1, 0) and normalised by j_0 = sin(kr)/kr or j_1 = j_0/kr - cos(kr)/kr,
        // whichever is larger in modulus (they have no common zero).
        const double2 sz = csin(kr), cz = ccos(kr);
        const double2 e0 = cdivd(sz, kr);
        const double2 t1 = cdivd(e0, kr), u1 = cdivd(cz, kr);
        const double2 e1 = make_double2(t1.x - u1.x, t1.y - u1.y);
        if (hypot(kr.x, kr.y) >= (double)NP) {
            z[0] = e0;
            if (NP > 1) z[1] = e1;
#pragma unroll 1
            for (int n = 2; n < NP; n++) {
                double2 f = cdivd(make_double2(2.0 * n - 1, 0), kr);
                double2 a = cmul(f, z[n - 1]);
                z[n] = make_double2(a.x - z[n - 2].x, a.y - z[n - 2].y);
            }
        } else {
            double2 hi = make_double2(0.0, 0.0), cur = make_double2(1.0, 0.0);   // j_{n+1}, j_n (unscaled)
#pragma unroll 1
            for (int n = NP + 24; n >= 1; n--) {
                const double2 f = cdivd(make_double2(2.0 * n + 1, 0), kr);
                const double2 a = cmul(f, cur);
                const double2 lo = make_double2(a.x - hi.x, a.y - hi.y);   // j_{n-1}
                hi = cur;
                cur = lo;
                if (n - 1 < NP) z[n - 1] = lo;
                if (fabs(cur.x) + fabs(cur.y) > 1e150) {   // keep the unnormalised values finite
                    hi = make_double2(hi.x * 1e-150, hi.y * 1e-150);
                    cur = make_double2(cur.x * 1e-150, cur.y * 1e-150);
#pragma unroll 1
                    for (int q = n - 1; q < NP; q++) z[q] = make_double2(z[q].x * 1e-150, z[q].y * 1e-150);
                }
            }
            const bool use0 = !(NP > 1) || hypot(e0.x, e0.y) >= hypot(e1.x, e1.y);
            const double2 s = use0 ? cdivd(e0, z[0]) : cdivd(e1, z[1]);
#pragma unroll 1
            for (int n = 0; n < NP; n++) z[n] = cmul(s, z[n]);
        }
    }
    // derivative z_n' = z_{n-1} - (n+1)/kr z_n, n >= 1
#pragma unroll 1
    for (int n = 1; n <= L && !far; n++) {
        double2 f = cdivd(make_double2((double)(n + 1), 0), kr);
        double2 a = cmul(f, z[n]);
        zp[n] = make_double2(z[n - 1].x - a.x, z[n - 1].y - a.y);
    }
    // Legendre P_n^m (m >= 0, no Condon-Shortley phase) for n <= L+1
    const double x = cos(theta);
    const double u = sqrt(fmax(0.0, (1.0 - x) * (1.0 + x)));
    double P[kLF + 2][kLF + 3];
#pragma unroll 1
    for (int a = 0; a < L + 2; a++)
#pragma unroll 1
        for (int b = 0; b < L + 3; b++) P[a][b] = 0.0;
    P[0][0] = 1.0;
#pragma unroll 1
    for (int m = 1; m <= L + 1; m++) P[m][m] = (2 * m - 1) * u * P[m - 1][m - 1];
#pragma unroll 1
    for (int m = 0; m <= L; m++) P[m + 1][m] = x * (2 * m + 1) * P[m][m];
#pragma unroll 1
    for (int m = 0; m <= L + 1; m++)
#pragma unroll 1
        for (int n = m + 2; n <= L + 1; n++)
            P[n][m] = ((2 * n - 1) * x * P[n - 1][m] - (n + m - 1) * P[n - 2][m]) / (double)(n - m);
    const bool at0 = (theta == 0.0), atpi = (theta == 3.14159265358979323846);
    const double st = sin(theta), ct = x;
    double sp, cp;
    sincos(phi, &sp, &cp);
    const double2 fac = outgoing ? make_double2(0, 1) : make_double2(0, -1);
    double2 Es[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
#pragma unroll 1
    for (int n = 1; n <= L; n++) {
#pragma unroll 1
        for (int m = -n; m <= n; m++) {
            const int am = m < 0 ? -m : m;
            const int r = n * n + n + m - 1;
            const double negf = negf_tab[r];
            const double Pnm = negf * P[n][am];
            double pi_v, tau_v;
            if (at0 || atpi) {
                const double sgn = atpi ? (((n + 1) & 1) ? -1.0 : 1.0) : 1.0;    // (-1)^(n+1) at pi
                const double sgt = atpi ? ((n & 1) ? -1.0 : 1.0) : 1.0;          // (-1)^n at pi
                if (m == 1) { pi_v = sgn * n * (n + 1) / 2.0; tau_v = sgt * n * (n + 1) / 2.0; }
                else if (m == -1) { pi_v = sgn * 0.5; tau_v = -sgt * 0.5; }
                else { pi_v = 0.0; tau_v = 0.0; }
            } else {
                pi_v = m / st * Pnm;
                const double pm1 = (am >= 1) ? P[n][am - 1] : -P[n][1] / (double)(n * (n + 1));
                const double pp1 = (am + 1 <= n) ? P[n][am + 1] : 0.0;
                tau_v = negf * 0.5 * ((n + am) * (n - am + 1) * pm1 - pp1);
            }
            double sm, cm;
            sincos((double)m * phi, &sm, &cm);
            const double2 eph = make_double2(cm, sm);
            if (far) {
                const double2 c0 = swap ? c[rmax + r] : c[r];
                const double2 c1 = swap ? c[r] : c[rmax + r];
                // i f E_mn (-i)^n e^{im phi}
                const double2 mi_n = (n & 3) == 0 ? make_double2(1, 0)
                                   : (n & 3) == 1 ? make_double2(0, -1)
                                   : (n & 3) == 2 ? make_double2(-1, 0) : make_double2(0, 1);
                const double2 w = cmul(cmul(make_double2(0, 1), ffar), cmul(cmul(emn[r], mi_n), eph));
                const double2 a = make_double2(c0.x * tau_v + c1.x * pi_v, c0.y * tau_v + c1.y * pi_v);
                const double2 b = make_double2(c0.x * pi_v + c1.x * tau_v, c0.y * pi_v + c1.y * tau_v);
                const double2 t1 = cmul(w, a), t2 = cmul(make_double2(0, 1), cmul(w, b));
                Es[1].x += t1.x; Es[1].y += t1.y;
                Es[2].x += t2.x; Es[2].y += t2.y;
                continue;
            }
            const double2 H = z[n], Hp = zp[n];
            // N: (n(n+1) P H/kr e, (H + kr H') e/kr tau, i (H + kr H') e/kr pi)
            const double2 hk = cdivd(cmul(H, eph), kr);
            const double2 g = cdivd(cmul(make_double2(H.x + (kr.x * Hp.x - kr.y * Hp.y), H.y + (kr.x * Hp.y + kr.y * Hp.x)), eph), kr);
            const double2 N0 = make_double2(n * (n + 1) * Pnm * hk.x, n * (n + 1) * Pnm * hk.y);
            const double2 N1 = make_double2(g.x * tau_v, g.y * tau_v);
            const double2 N2 = make_double2(-g.y * pi_v, g.x * pi_v);
            // M: (0, i pi H e, -tau H e)
            const double2 he = cmul(H, eph);
            const double2 M1 = make_double2(-he.y * pi_v, he.x * pi_v);
            const double2 M2 = make_double2(-he.x * tau_v, -he.y * tau_v);
            const double2 c0 = swap ? c[rmax + r] : c[r];
            const double2 c1 = swap ? c[r] : c[rmax + r];
            const double2 w = cmul(fac, emn[r]);
            const double2 w0 = cmul(w, c0), w1 = cmul(w, c1);
            double2 t;
            t = cmul(w0, N0); Es[0].x += t.x; Es[0].y += t.y;
            t = cadd2(cmul(w0, N1), cmul(w1, M1)); Es[1].x += t.x; Es[1].y += t.y;
            t = cadd2(cmul(w0, N2), cmul(w1, M2)); Es[2].x += t.x; Es[2].y += t.y;
        }
    }
    // spherical -> Cartesian (vec_sph_to_cart), times the prefactor
    const double rh[3] = {st * cp, st * sp, ct}, th[3] = {ct * cp, ct * sp, -st}, ph[3] = {-sp, cp, 0.0};
    for (int d = 0; d < 3; d++) {
        double2 v = make_double2(Es[0].x * rh[d] + Es[1].x * th[d] + Es[2].x * ph[d],
                                 Es[0].y * rh[d] + Es[1].y * th[d] + Es[2].y * ph[d]);
        v = cmul(pref, v);
        E[d].x += v.x;
        E[d].y += v.y;
    }
}

__global__ void __launch_bounds__(kFieldThreads)
k_field(int L, int N, const double* __restrict__ pos, const double* __restrict__ radius, const double2* __restrict__ p_scat,
        const double2* __restrict__ p_int, double k, const double2* __restrict__ k_int, int Npts,
        const double* __restrict__ pts, int interior, int magnetic, double2 hfac, const double2* __restrict__ hfac_int,
        double2* __restrict__ out, int far) {
    const int rmax = L * (L + 2);
    constexpr int kTile = 16;
    __shared__ double sp_pos[kTile][3];
    __shared__ double2 sp_c[kTile * 2 * kLF * (kLF + 2)];
    __shared__ double2 emn[kLF * (kLF + 2)];
    __shared__ double negf_tab[kLF * (kLF + 2)];
    for (int r = threadIdx.x; r < rmax; r += blockDim.x) {
        int n = (int)floor(sqrt((double)r + 1.0));
        while (n * n > r + 1) n--;
        while ((n + 1) * (n + 1) <= r + 1) n++;
        const int m = r + 1 - n * n - n;
        emn[r] = Emn(m, n);
        const int am = m < 0 ? -m : m;
        negf_tab[r] = (m < 0) ? (((am & 1) ? -1.0 : 1.0) * tgamma((double)(n - am) + 1.0) / tgamma((double)(n + am) + 1.0)) : 1.0;
    }
    const int pt = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = pt < Npts;
    double X = 0, Y = 0, Z = 0;
    if (valid) {
        X = pts[3LL * pt];
        Y = pts[3LL * pt + 1];
        Z = pts[3LL * pt + 2];
    }
    // interior test first (the reference overwrites interior points)
    int inside = -1;
    if (interior && valid) {
        for (int i = 0; i < N; i++) {
            const double dx = X - pos[3 * i], dy = Y - pos[3 * i + 1], dz = Z - pos[3 * i + 2];
            if (dx * dx + dy * dy + dz * dz < radius[i] * radius[i]) inside = i;   // last match wins, as in the reference loop
        }
    }
    double2 E[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
    const double2 pref_out = magnetic ? hfac : make_double2(1, 0);
    for (int t0 = 0; t0 < N; t0 += kTile) {
        const int cnt = min(kTile, N - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt * 3; e += blockDim.x) sp_pos[e / 3][e % 3] = pos[3LL * t0 + e];
        for (int e = threadIdx.x; e < cnt * 2 * rmax; e += blockDim.x)
            sp_c[e] = p_scat[(long long)t0 * 2 * rmax + e];
        __syncthreads();
        if (!valid || inside >= 0) continue;
        for (int q = 0; q < cnt; q++) {
            const double dx = X - sp_pos[q][0], dy = Y - sp_pos[q][1], dz = Z - sp_pos[q][2];
            const double rad = sqrt(dx * dx + dy * dy + dz * dz);
            const double theta = acos(dz / rad);
            const double phi = atan2(dy, dx);
            add_expansion(L, sp_c + q * 2 * rmax, rmax, true, make_double2(k, 0), rad, theta, phi, magnetic != 0,
                          pref_out, emn, negf_tab, E, far != 0);
        }
    }
    if (!valid) return;
    if (inside >= 0) {
        const int i = inside;
        const double dx = X - pos[3 * i], dy = Y - pos[3 * i + 1], dz = Z - pos[3 * i + 2];
        const double rad = sqrt(dx * dx + dy * dy + dz * dz);
        const double theta = acos(dz / rad);
        const double phi = atan2(dy, dx);
        const double2 pref = magnetic ? hfac_int[i] : make_double2(1, 0);
        add_expansion(L, p_int + (long long)i * 2 * rmax, rmax, false, k_int[i], rad, theta, phi, magnetic != 0, pref,
                      emn, negf_tab, E);
    }
    for (int d = 0; d < 3; d++) out[3LL * pt + d] = E[d];
}

// ------------------------------------------------------------ FP32 field --
// The same exterior sum in FP32 for large maps (a 512 x 512 plane around
// thousands of spheres is ~1e9 point-particle terms): no trigonometry per term
// beyond one sincosf of k r; angles enter through r-hat components, e^{i m phi}
// by powering (x + i y)/rho.  Coefficients are pre-multiplied by i E_mn in shared
// memory (tiles of 32 particles); separations are formed in FP64.  Points inside a
// sphere take the FP64 interior expansion, as in k_field.
constexpr int kTile32 = 32;

template <int LT>
__global__ void __launch_bounds__(kFieldThreads)
k_field32(int Lrun, int N, const double* __restrict__ pos, const double* __restrict__ radius,
          const double2* __restrict__ p_scat, const double2* __restrict__ p_int, double k,
          const double2* __restrict__ k_int, int Npts, const double* __restrict__ pts, int interior, int magnetic,
          double2 hfac, const double2* __restrict__ hfac_int, double2* __restrict__ out) {
    // LT > 0: lmax known at compile time, every per-term loop unrolled (arrays in
    // registers); LT == 0: any lmax up to kLF
    const int L = LT > 0 ? LT : Lrun;
    const int rmax = L * (L + 2);
    __shared__ double sp_pos[kTile32][3];
    __shared__ float2 sw0[kTile32 * kLF * (kLF + 2)];
    __shared__ float2 sw1[kTile32 * kLF * (kLF + 2)];
    __shared__ double2 emn[kLF * (kLF + 2)];
    __shared__ double negf_tab[kLF * (kLF + 2)];
    __shared__ float negf32[kLF * (kLF + 2)];
    for (int r = threadIdx.x; r < rmax; r += blockDim.x) {
        int n = (int)floor(sqrt((double)r + 1.0));
        while (n * n > r + 1) n--;
        while ((n + 1) * (n + 1) <= r + 1) n++;
        const int m = r + 1 - n * n - n;
        emn[r] = Emn(m, n);
        const int am = m < 0 ? -m : m;
        negf_tab[r] = (m < 0) ? (((am & 1) ? -1.0 : 1.0) * tgamma((double)(n - am) + 1.0) / tgamma((double)(n + am) + 1.0)) : 1.0;
        negf32[r] = (float)negf_tab[r];
    }
    const int pt = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = pt < Npts;
    double X = 0, Y = 0, Z = 0;
    if (valid) {
        X = pts[3LL * pt];
        Y = pts[3LL * pt + 1];
        Z = pts[3LL * pt + 2];
    }
    int inside = -1;
    if (interior && valid) {
        for (int i = 0; i < N; i++) {
            const double dx = X - pos[3 * i], dy = Y - pos[3 * i + 1], dz = Z - pos[3 * i + 2];
            if (dx * dx + dy * dy + dz * dz < radius[i] * radius[i]) inside = i;
        }
    }
    const float kf = (float)k;
    float Ex[2] = {0.f, 0.f}, Ey[2] = {0.f, 0.f}, Ez[2] = {0.f, 0.f};
    for (int t0 = 0; t0 < N; t0 += kTile32) {
        const int cnt = min(kTile32, N - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt * 3; e += blockDim.x) sp_pos[e / 3][e % 3] = pos[3LL * t0 + e];
        for (int e = threadIdx.x; e < cnt * rmax; e += blockDim.x) {
            const int q = e / rmax, r = e % rmax;
            const double2* c = p_scat + (long long)(t0 + q) * 2 * rmax;
            const double2 c0 = magnetic ? c[rmax + r] : c[r];
            const double2 c1 = magnetic ? c[r] : c[rmax + r];
            const double2 w = cmul(make_double2(0, 1), emn[r]);   // outgoing: factor i
            const double2 a = cmul(w, c0), b = cmul(w, c1);
            sw0[e] = make_float2((float)a.x, (float)a.y);
            sw1[e] = make_float2((float)b.x, (float)b.y);
        }
        __syncthreads();
        if (!valid || inside >= 0) continue;
        for (int q = 0; q < cnt; q++) {
            const float dx = (float)(X - sp_pos[q][0]), dy = (float)(Y - sp_pos[q][1]), dz = (float)(Z - sp_pos[q][2]);
            const float rho2 = dx * dx + dy * dy;
            const float r = sqrtf(rho2 + dz * dz);
            const float inv_r = 1.f / r;
            const float rho = sqrtf(rho2);
            const float ct = dz * inv_r, st = rho * inv_r;
            float cphi = 1.f, sphi = 0.f;
            if (rho > 0.f) {
                const float ir = 1.f / rho;
                cphi = dx * ir;
                sphi = dy * ir;
            }
            // h_n(x) = j_n + i y_n, n = 0..L, by the upward recurrences
            const float x = kf * r, ix = 1.f / x;
            float sx, cx;
            sincosf(x, &sx, &cx);
            float hr[kLF + 1], hi[kLF + 1];
            hr[0] = sx * ix;
            hi[0] = -cx * ix;
            hr[1] = hr[0] * ix - cx * ix;
            hi[1] = hi[0] * ix - hr[0];
#pragma unroll
            for (int n = 2; n <= L; n++) {
                const float f = (2 * n - 1) * ix;
                hr[n] = f * hr[n - 1] - hr[n - 2];
                hi[n] = f * hi[n - 1] - hi[n - 2];
            }
            // Legendre P_n^m(ct), m >= 0, no Condon-Shortley phase
            float P[kLF + 1][kLF + 2];
            P[0][0] = 1.f;
#pragma unroll
            for (int m = 1; m <= L; m++) P[m][m] = (2 * m - 1) * st * P[m - 1][m - 1];
#pragma unroll
            for (int m = 0; m < L; m++) P[m + 1][m] = ct * (2 * m + 1) * P[m][m];
#pragma unroll
            for (int m = 0; m <= L; m++)
#pragma unroll
                for (int n = m + 2; n <= L; n++)
                    P[n][m] = ((2 * n - 1) * ct * P[n - 1][m] - (n + m - 1) * P[n - 2][m]) / (float)(n - m);
            const bool axis = !(st > 0.f);
            const float2* w0 = sw0 + q * rmax;
            const float2* w1 = sw1 + q * rmax;
            float Er[2] = {0.f, 0.f}, Et[2] = {0.f, 0.f}, Ep[2] = {0.f, 0.f};
#pragma unroll
            for (int n = 1; n <= L; n++) {
                // radial parts: h_n / x and (x h_n)'/x = h_{n-1} - n h_n / x
                const float hx_r = hr[n] * ix, hx_i = hi[n] * ix;
                const float dr = hr[n - 1] - n * hx_r, di = hi[n - 1] - n * hx_i;
                // e^{i m phi} for m = -n: conj((cphi + i sphi)^n)
                float er = 1.f, ei = 0.f;
                #pragma unroll
                for (int s = 0; s < n; s++) {
                    const float t = er * cphi + ei * sphi;   // multiply by e^{-i phi}
                    ei = ei * cphi - er * sphi;
                    er = t;
                }
#pragma unroll
                for (int m = -n; m <= n; m++) {
                    const int am = m < 0 ? -m : m;
                    const int rr = n * n + n + m - 1;
                    const float nf = negf32[rr];
                    const float Pnm = nf * P[n][am];
                    float pi_v, tau_v;
                    if (axis) {
                        const bool atpi = ct < 0.f;
                        const float sgn = atpi ? (((n + 1) & 1) ? -1.f : 1.f) : 1.f;
                        const float sgt = atpi ? ((n & 1) ? -1.f : 1.f) : 1.f;
                        if (m == 1) { pi_v = sgn * n * (n + 1) * 0.5f; tau_v = sgt * n * (n + 1) * 0.5f; }
                        else if (m == -1) { pi_v = sgn * 0.5f; tau_v = -sgt * 0.5f; }
                        else { pi_v = 0.f; tau_v = 0.f; }
                    } else {
                        pi_v = m / st * Pnm;
                        const float pm1 = (am >= 1) ? P[n][am - 1] : -P[n][1] / (float)(n * (n + 1));
                        const float pp1 = (am + 1 <= n) ? P[n][am + 1] : 0.f;
                        tau_v = nf * 0.5f * ((n + am) * (n - am + 1) * pm1 - pp1);
                    }
                    const float2 a = w0[rr], b = w1[rr];
                    // u = a e, v = b e
                    const float ur = a.x * er - a.y * ei, ui = a.x * ei + a.y * er;
                    const float vr = b.x * er - b.y * ei, vi = b.x * ei + b.y * er;
                    // N = (n(n+1) P h/x, d tau, i d pi) e ;  M = (0, i pi h, -tau h) e
                    const float c0 = n * (n + 1) * Pnm;
                    Er[0] += c0 * (ur * hx_r - ui * hx_i);
                    Er[1] += c0 * (ur * hx_i + ui * hx_r);
                    const float udr = ur * dr - ui * di, udi = ur * di + ui * dr;   // u d
                    const float vhr = vr * hr[n] - vi * hi[n], vhi = vr * hi[n] + vi * hr[n];   // v h
                    Et[0] += tau_v * udr - pi_v * vhi;
                    Et[1] += tau_v * udi + pi_v * vhr;
                    Ep[0] += -pi_v * udi - tau_v * vhr;
                    Ep[1] += pi_v * udr - tau_v * vhi;
                    const float t = er * cphi - ei * sphi;   // e <- e e^{i phi}
                    ei = er * sphi + ei * cphi;
                    er = t;
                }
            }
            // spherical -> Cartesian
            const float rh0 = st * cphi, rh1 = st * sphi, rh2 = ct;
            const float th0 = ct * cphi, th1 = ct * sphi, th2 = -st;
            const float ph0 = -sphi, ph1 = cphi;
            for (int c = 0; c < 2; c++) {
                Ex[c] += Er[c] * rh0 + Et[c] * th0 + Ep[c] * ph0;
                Ey[c] += Er[c] * rh1 + Et[c] * th1 + Ep[c] * ph1;
                Ez[c] += Er[c] * rh2 + Et[c] * th2;
            }
        }
    }
    if (!valid) return;
    double2 E[3];
    if (inside >= 0) {
        E[0] = E[1] = E[2] = make_double2(0, 0);
        const int i = inside;
        const double dx = X - pos[3 * i], dy = Y - pos[3 * i + 1], dz = Z - pos[3 * i + 2];
        const double rad = sqrt(dx * dx + dy * dy + dz * dz);
        const double theta = acos(dz / rad);
        const double phi = atan2(dy, dx);
        const double2 pref = magnetic ? hfac_int[i] : make_double2(1, 0);
        add_expansion(L, p_int + (long long)i * 2 * rmax, rmax, false, k_int[i], rad, theta, phi, magnetic != 0, pref,
                      emn, negf_tab, E);
    } else {
        const double2 pref = magnetic ? hfac : make_double2(1, 0);
        E[0] = cmul(pref, make_double2(Ex[0], Ex[1]));
        E[1] = cmul(pref, make_double2(Ey[0], Ey[1]));
        E[2] = cmul(pref, make_double2(Ez[0], Ez[1]));
    }
    for (int d = 0; d < 3; d++) out[3LL * pt + d] = E[d];
}

}   // namespace

extern "C" int gb_near_field(int N, int lmax, const double* pos, const double* radius, const double* p_scat,
                             const double* p_int, double k, const double* k_int, int Npts, const double* pts,
                             int interior, int magnetic, double hfac_re, double hfac_im, const double* hfac_int,
                             double* out, void* stream) {
    if (N < 1 || Npts < 0 || !pos || !p_scat || !pts || !out) return gb_set_error(GB_BAD_ARG, "bad field arguments");
    if (interior && (!radius || !p_int || !k_int)) return gb_set_error(GB_BAD_ARG, "interior fields need radius, p_int, k_int");
    if (magnetic && interior && !hfac_int) return gb_set_error(GB_BAD_ARG, "interior H fields need hfac_int");
    if (Npts == 0) return GB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((Npts + kFieldThreads - 1) / kFieldThreads);
    const double2 hf = make_double2(hfac_re, hfac_im);
    const double2* pi2 = reinterpret_cast<const double2*>(p_int);
    const double2* ps2 = reinterpret_cast<const double2*>(p_scat);
    const double2* ki2 = reinterpret_cast<const double2*>(k_int);
    const double2* hi2 = reinterpret_cast<const double2*>(hfac_int);
    double2* o2 = reinterpret_cast<double2*>(out);
    if (lmax < 1 || lmax > kLF) return gb_set_error(GB_UNSUPPORTED, "near field supports lmax 1..%d (got %d)", kLF, lmax);
    gb::note_launch();
    k_field<<<grid, kFieldThreads, 0, s>>>(lmax, N, pos, radius, ps2, pi2, k, ki2, Npts, pts, interior, magnetic, hf,
                                           hi2, o2, 0);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

// The far-field form of every particle's outgoing expansion, summed at the points
// (sphere_cluster.E_field / H_field with far=True, sphere_cluster.py:244-391, with
// expand_E_far / expand_H_far, vsh/expansion.py:45-77,96-108): no interior
// expansions; H fields swap the coefficients and take the prefactor hfac.
extern "C" int gb_far_field_expansions(int N, int lmax, const double* pos, const double* p_scat, double k, int Npts,
                                       const double* pts, int magnetic, double hfac_re, double hfac_im, double* out,
                                       void* stream) {
    if (N < 1 || Npts < 0 || !pos || !p_scat || !pts || !out) return gb_set_error(GB_BAD_ARG, "bad field arguments");
    if (lmax < 1 || lmax > kLF) return gb_set_error(GB_UNSUPPORTED, "far field supports lmax 1..%d (got %d)", kLF, lmax);
    if (Npts == 0) return GB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((Npts + kFieldThreads - 1) / kFieldThreads);
    gb::note_launch();
    k_field<<<grid, kFieldThreads, 0, s>>>(lmax, N, pos, nullptr, reinterpret_cast<const double2*>(p_scat), nullptr, k,
                                           nullptr, Npts, pts, 0, magnetic, make_double2(hfac_re, hfac_im), nullptr,
                                           reinterpret_cast<double2*>(out), 1);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

// Same arguments and result as gb_near_field, with the exterior sums in FP32.
extern "C" int gb_near_field32(int N, int lmax, const double* pos, const double* radius, const double* p_scat,
                               const double* p_int, double k, const double* k_int, int Npts, const double* pts,
                               int interior, int magnetic, double hfac_re, double hfac_im, const double* hfac_int,
                               double* out, void* stream) {
    if (N < 1 || Npts < 0 || !pos || !p_scat || !pts || !out) return gb_set_error(GB_BAD_ARG, "bad field arguments");
    if (interior && (!radius || !p_int || !k_int)) return gb_set_error(GB_BAD_ARG, "interior fields need radius, p_int, k_int");
    if (magnetic && interior && !hfac_int) return gb_set_error(GB_BAD_ARG, "interior H fields need hfac_int");
    if (Npts == 0) return GB_OK;
    if (lmax < 1 || lmax > kLF) return gb_set_error(GB_UNSUPPORTED, "near field supports lmax 1..%d (got %d)", kLF, lmax);
    const unsigned grid = (unsigned)((Npts + kFieldThreads - 1) / kFieldThreads);
    auto kfn = lmax == 1 ? k_field32<1> : lmax == 2 ? k_field32<2> : lmax == 3 ? k_field32<3>
             : lmax == 4 ? k_field32<4> : k_field32<0>;
    gb::note_launch();
    kfn<<<grid, kFieldThreads, 0, (cudaStream_t)stream>>>(
        lmax, N, pos, radius, reinterpret_cast<const double2*>(p_scat), reinterpret_cast<const double2*>(p_int), k,
        reinterpret_cast<const double2*>(k_int), Npts, pts, interior, magnetic, make_double2(hfac_re, hfac_im),
        reinterpret_cast<const double2*>(hfac_int), reinterpret_cast<double2*>(out));
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}
