// CPU ORACLE -- TEST INFRASTRUCTURE ONLY.
//
// A plain C++17 restatement of the native module of johnaparker/miepy
// (cpp/src/*.cpp), written for this project so that the sphere-cluster hot path
// can be checked and timed on the host.  Only the parity tests, the smoke check
// and the CPU-baseline leg of the benchmark may load this library; the product
// (miepy_gb300) never does.
//
// Third-party arithmetic that the reference takes from libraries absent here is
// restated from its published algorithm:
//   * GSL gsl_sf_legendre_array(GSL_SF_LEGENDRE_NONE)  -> unnormalised associated
//     Legendre upward recurrence in degree (no Condon-Shortley phase).
//   * GSL gsl_sf_coupling_3j                           -> Racah's closed formula.
//   * GSL gsl_sf_bessel_jl / gsl_sf_bessel_yl (real)   -> Miller backward recurrence
//     for j_l, upward recurrence for y_l.
//   * GSL_CONST_MKSA_VACUUM_PERMITTIVITY               -> 8.854187817e-12 F/m.
//   * Eigen BiCGSTAB<IdentityPreconditioner>           -> van der Vorst BiCGSTAB with
//     x0 = 0, relative-residual stop and Eigen's restart rule.
//   * Eigen partialPivLu                               -> LU with partial pivoting.
// Every exported function names the reference function (file:line) it follows.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using cd = std::complex<double>;

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEps0Gsl = 8.854187817e-12;   // GSL MKSA vacuum permittivity

double fact(double n) { return std::tgamma(n + 1.0); }   // cpp/src/special.cpp:15-17

// i^p exactly (the reference evaluates pow(1i, p) by repeated multiplication).
cd ipow(int p) {
    switch (((p % 4) + 4) % 4) {
        case 0: return cd(1, 0);
        case 1: return cd(0, 1);
        case 2: return cd(-1, 0);
        default: return cd(0, -1);
    }
}

double sgnpow(int p) { return (p % 2 == 0) ? 1.0 : -1.0; }   // pow(-1, p)

int lmax_to_rmax(int lmax) { return lmax * (lmax + 2); }
int rmax_to_lmax(int rmax) { return -1 + int(std::sqrt(1.0 + rmax)); }

// ---------------------------------------------------------------- Bessel --
// spherical_jn for complex z by upward recurrence: cpp/src/special.cpp:20-45.
cd sph_jn_c(int n, cd z) {
    cd s = std::sin(z), c = std::cos(z);
    cd j2 = s / z;
    cd jn = j2;
    if (n > 0) {
        cd j1 = j2 / z - c / z;
        jn = j1;
        for (int i = 2; i <= n; i++) {
            jn = double(2 * i - 1) / z * j1 - j2;
            j2 = j1;
            j1 = jn;
        }
    }
    return jn;
}

cd sph_jn_c_d(int n, cd z, bool deriv) {
    if (!deriv) return sph_jn_c(n, z);
    return sph_jn_c(n - 1, z) - double(n + 1) / z * sph_jn_c(n, z);
}

// spherical_hn for real z, upward recurrence of j and y: cpp/src/special.cpp:54-88.
cd sph_hn(int n, double z) {
    double s = std::sin(z), c = std::cos(z);
    double j2 = s / z, jn = j2;
    double y2 = -c / z, yn = y2;
    if (n > 0) {
        double j1 = j2 / z - c / z;
        double y1 = y2 / z - j2;
        jn = j1;
        yn = y1;
        for (int i = 2; i <= n; i++) {
            jn = (2 * i - 1) / z * j1 - j2;
            j2 = j1;
            j1 = jn;
            yn = (2 * i - 1) / z * y1 - y2;
            y2 = y1;
            y1 = yn;
        }
    }
    return cd(jn, yn);
}

cd sph_hn_d(int n, double z, bool deriv) {
    if (!deriv) return sph_hn(n, z);
    return sph_hn(n - 1, z) - double(n + 1) / z * sph_hn(n, z);
}

// spherical_hn_recursion: cpp/src/special.cpp:90-111 (all orders 0..nmax).
void sph_hn_all(int nmax, double z, cd* out) {
    double s = std::sin(z), c = std::cos(z);
    std::vector<double> j(nmax + 2), y(nmax + 2);
    j[0] = s / z;
    y[0] = -c / z;
    j[1] = j[0] / z + y[0];
    y[1] = y[0] / z - j[0];
    for (int i = 2; i <= nmax; i++) {
        j[i] = (2 * i - 1) / z * j[i - 1] - j[i - 2];
        y[i] = (2 * i - 1) / z * y[i - 1] - y[i - 2];
    }
    for (int i = 0; i <= nmax; i++) out[i] = cd(j[i], y[i]);
}

// Real spherical j_l (stands in for gsl_sf_bessel_jl): Miller's backward recurrence
// normalised by j_0 (or j_1 when j_0 is tiny); upward recurrence when x > l.
double sph_jl_real(int l, double x) {
    if (l < 0) return 0.0;
    if (x == 0.0) return l == 0 ? 1.0 : 0.0;
    double j0 = std::sin(x) / x;
    if (l == 0) return j0;
    double j1 = std::sin(x) / (x * x) - std::cos(x) / x;
    if (l == 1) return j1;
    if (x > double(l)) {
        double a = j0, b = j1, c = 0;
        for (int i = 1; i < l; i++) {
            c = (2 * i + 1) / x * b - a;
            a = b;
            b = c;
        }
        return b;
    }
    const int start = l + 30 + int(std::sqrt(40.0 * l));
    std::vector<double> f(start + 2, 0.0);
    f[start + 1] = 0.0;
    f[start] = 1e-280;
    for (int i = start; i >= 1; i--) {   // f_{i-1} = (2i+1)/x f_i - f_{i+1}
        f[i - 1] = (2 * i + 1) / x * f[i] - f[i + 1];
        if (std::fabs(f[i - 1]) > 1e250)
            for (int e = i - 1; e <= start; e++) f[e] *= 1e-250;
    }
    if (std::fabs(j0) > std::fabs(j1)) return f[l] * (j0 / f[0]);
    return f[l] * (j1 / f[1]);
}

// Real spherical y_l (stands in for gsl_sf_bessel_yl): upward recurrence.
double sph_yl_real(int l, double x) {
    double y0 = -std::cos(x) / x;
    if (l == 0) return y0;
    double y1 = -std::cos(x) / (x * x) - std::sin(x) / x;
    double a = y0, b = y1;
    for (int i = 1; i < l; i++) {
        double c = (2 * i + 1) / x * b - a;
        a = b;
        b = c;
    }
    return b;
}

// -------------------------------------------------------------- Legendre --
// Unnormalised P_n^m(x), m >= 0, no Condon-Shortley phase, for n <= nmax;
// stored at tab[n*(nmax+1) + m].
void legendre_pos(int nmax, double x, double* tab) {
    const int W = nmax + 1;
    for (int i = 0; i < W * W; i++) tab[i] = 0.0;
    double u = std::sqrt(std::max(0.0, (1.0 - x) * (1.0 + x)));
    tab[0] = 1.0;
    for (int m = 1; m <= nmax; m++) tab[m * W + m] = (2 * m - 1) * u * tab[(m - 1) * W + m - 1];
    for (int m = 0; m < nmax; m++) tab[(m + 1) * W + m] = x * (2 * m + 1) * tab[m * W + m];
    for (int m = 0; m <= nmax; m++)
        for (int n = m + 2; n <= nmax; n++)
            tab[n * W + m] = ((2 * n - 1) * x * tab[(n - 1) * W + m] - (n + m - 1) * tab[(n - 2) * W + m]) /
                             double(n - m);
}

// associated_legendre: cpp/src/special.cpp:148-178 (GSL replaced).
double assoc_legendre(int n, int m, double z) {
    if (n == 1) {
        if (m == 0) return z;
        if (m == 1) return std::sqrt(1 - z * z);
        if (m == -1) return -std::sqrt(1 - z * z) / 2;
    }
    int am = std::abs(m);
    if (am > n || n < 0) return 0.0;
    std::vector<double> tab((n + 1) * (n + 1));
    legendre_pos(n, z, tab.data());
    double leg = tab[n * (n + 1) + am];
    if (m < 0) leg *= sgnpow(m) * fact(n + m) / fact(n - m);
    return leg;
}

// associated_legendre_recursion: cpp/src/special.cpp:180-204, packed n(n+2)-n+m.
void assoc_legendre_all(int nmax, double z, double* out) {
    std::vector<double> tab((nmax + 1) * (nmax + 1));
    legendre_pos(nmax, z, tab.data());
    for (int n = 0; n <= nmax; n++)
        for (int m = -n; m <= n; m++) {
            double leg = tab[n * (nmax + 1) + std::abs(m)];
            if (m < 0) leg *= sgnpow(m) * fact(n + m) / fact(n - m);
            out[n * (n + 2) - n + m] = leg;
        }
}

// pi_func: cpp/src/special.cpp:209-231.
double pi_fn(int n, int m, double theta) {
    if (theta == 0) {
        if (m == 1) return n * (n + 1) / 2.0;
        if (m == -1) return 1 / 2.0;
        return 0;
    }
    if (theta == kPi) {
        if (m == 1) return sgnpow(n + 1) * n * (n + 1) / 2.0;
        if (m == -1) return sgnpow(n + 1) / 2.0;
        return 0;
    }
    return m / std::sin(theta) * assoc_legendre(n, m, std::cos(theta));
}

// tau_func: cpp/src/special.cpp:233-270.  dP_n^|m|/dtheta from the division-free
// identity dP_n^m/dtheta = [(n+m)(n-m+1) P_n^{m-1} - P_n^{m+1}] / 2.
double tau_fn(int n, int m, double theta) {
    if (theta == 0) {
        if (m == 1) return n * (n + 1) / 2.0;
        if (m == -1) return -1 / 2.0;
        return 0;
    }
    if (theta == kPi) {
        if (m == 1) return sgnpow(n) * n * (n + 1) / 2.0;
        if (m == -1) return -sgnpow(n) / 2.0;
        return 0;
    }
    int am = std::abs(m);
    if (am > n) return 0.0;
    double x = std::cos(theta);
    std::vector<double> tab((n + 2) * (n + 2));
    legendre_pos(n + 1, x, tab.data());
    const int W = n + 2;
    double pp1 = (am + 1 <= n) ? tab[n * W + am + 1] : 0.0;
    double pm1;
    if (am >= 1) pm1 = tab[n * W + am - 1];
    else pm1 = (n >= 1) ? -tab[n * W + 1] / double(n * (n + 1)) : 0.0;   // P_n^{-1}
    double dtheta = 0.5 * ((n + am) * (n - am + 1) * pm1 - pp1);
    if (m < 0) dtheta *= sgnpow(m) * fact(n + m) / fact(n - m);
    return dtheta;
}

// -------------------------------------------------------------- Wigner 3j --
// Racah's formula (stands in for gsl_sf_coupling_3j): cpp/src/special.cpp:272-274.
double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
    if (m1 + m2 + m3 != 0) return 0.0;
    if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
    if (j3 < std::abs(j1 - j2) || j3 > j1 + j2) return 0.0;
    int t1 = j1 + j2 - j3, t2 = j1 - j2 + j3, t3 = -j1 + j2 + j3;
    if (t1 < 0 || t2 < 0 || t3 < 0) return 0.0;
    double delta = fact(t1) * fact(t2) * fact(t3) / fact(j1 + j2 + j3 + 1);
    double pre = fact(j1 + m1) * fact(j1 - m1) * fact(j2 + m2) * fact(j2 - m2) * fact(j3 + m3) * fact(j3 - m3);
    int tmin = std::max({0, j2 - j3 - m1, j1 - j3 + m2});
    int tmax = std::min({j1 + j2 - j3, j1 - m1, j2 + m2});
    double s = 0.0;
    for (int t = tmin; t <= tmax; t++) {
        double den = fact(t) * fact(j1 + j2 - j3 - t) * fact(j1 - m1 - t) * fact(j2 + m2 - t) *
                     fact(j3 - j2 + m1 + t) * fact(j3 - j1 - m2 + t);
        s += sgnpow(t) / den;
    }
    return sgnpow(j1 - j2 - m3) * std::sqrt(delta * pre) * s;
}

// a_func / b_func: cpp/src/special.cpp:276-296.
double a_fn(int m, int n, int u, int v, int p) {
    double num = fact(n + m) * fact(v + u) * fact(p - m - u);
    double den = fact(n - m) * fact(v - u) * fact(p + m + u);
    double f = sgnpow(m + u) * (2 * p + 1) * std::sqrt(num / den);
    return f * wigner3j(n, v, p, 0, 0, 0) * wigner3j(n, v, p, m, u, -m - u);
}

double b_fn(int m, int n, int u, int v, int p) {
    double num = fact(n + m) * fact(v + u) * fact(p - m - u + 1);
    double den = fact(n - m) * fact(v - u) * fact(p + m + u + 1);
    double f = sgnpow(m + u) * (2 * p + 3) * std::sqrt(num / den);
    return f * wigner3j(n, v, p, 0, 0, 0) * wigner3j(n, v, p + 1, m, u, -m - u);
}

// wigner_3j_batch (Schulten-Gordon recurrence seeded by two closed-form values):
// cpp/src/special.cpp:298-363.
struct W3Batch {
    int jmin = 0, jmax = -1;
    std::vector<double> val;
};

W3Batch wigner3j_batch(int j2, int j3, int m1, int m2, int m3) {
    W3Batch r;
    if (m1 + m2 + m3 != 0) return r;
    r.jmin = std::max(std::abs(j2 - j3), std::abs(m1));
    r.jmax = j2 + j3;
    int size = r.jmax - r.jmin + 1;
    if (size <= 0) return r;
    r.val.assign(size, 0.0);
    if (size <= 2) {
        for (int i = 0; i < size; i++) r.val[i] = wigner3j(r.jmin + i, j2, j3, m1, m2, m3);
        return r;
    }
    r.val[0] = wigner3j(r.jmin, j2, j3, m1, m2, m3);
    r.val[1] = wigner3j(r.jmin + 1, j2, j3, m1, m2, m3);
    const double d23 = j2 - j3, s23 = j2 + j3 + 1;
    const double jj = double(j2) * (j2 + 1) - double(j3) * (j3 + 1);
    const double md = m3 - m2;
    for (int i = 1; i < size - 1; i++) {
        double j = r.jmin + i, jp = j + 1.0;
        double sj = std::sqrt(std::max(0.0, (j * j - d23 * d23) * (s23 * s23 - j * j) * (j * j - double(m1) * m1)));
        double sjp = std::sqrt(std::max(0.0, (jp * jp - d23 * d23) * (s23 * s23 - jp * jp) * (jp * jp - double(m1) * m1)));
        double A = jp * sj;
        double B = (2.0 * j + 1) * (-double(m1) * jj + md * j * jp);
        double C = j * sjp;
        if (std::fabs(C) < 1e-30) r.val[i + 1] = wigner3j(int(j) + 1, j2, j3, m1, m2, m3);
        else r.val[i + 1] = (-A * r.val[i - 1] - B * r.val[i]) / C;
    }
    return r;
}

// gaunt_batch: cpp/src/special.cpp:365-440.
void gaunt_batch(int m, int n, int u, int v, std::vector<double>& a, std::vector<double>& b) {
    int qA = std::min({n, v, (n + v - std::abs(m + u)) / 2});
    int qB = std::min({n, v, (n + v + 1 - std::abs(m + u)) / 2});
    a.assign(std::max(qA + 1, 0), 0.0);
    b.assign(std::max(qB + 1, 0), 0.0);
    W3Batch w0 = wigner3j_batch(n, v, 0, 0, 0);
    W3Batch wm = wigner3j_batch(n, v, -(m + u), m, u);
    double fnm = fact(n + m), fn_m = fact(n - m), fvu = fact(v + u), fv_u = fact(v - u);
    double sign = sgnpow(m + u);
    for (int q = 0; q <= qA; q++) {
        int p = n + v - 2 * q;
        double ratio = fnm * fvu * fact(p - m - u) / (fn_m * fv_u * fact(p + m + u));
        a[q] = sign * (2 * p + 1) * std::sqrt(ratio) * w0.val[p - w0.jmin] * wm.val[p - wm.jmin];
    }
    for (int q = 1; q <= qB; q++) {
        int p = n + v - 2 * q;
        double ratio = fnm * fvu * fact(p - m - u + 1) / (fn_m * fv_u * fact(p + m + u + 1));
        b[q] = sign * (2 * p + 3) * std::sqrt(ratio) * w0.val[p - w0.jmin] * wm.val[(p + 1) - wm.jmin];
    }
}

// ---------------------------------------------------- translation cache --
// vsh_cache: cpp/src/vsh_translation.cpp:12-34.  Held in a dense array keyed by
// (n, m, v, u) instead of a std::map.
struct TupleCache {
    cd factor;
    int qA = -1, qB = -1;
    cd A[32];
    cd B[32];
};

struct TranslationCache {
    int L = 0;
    std::vector<TupleCache> t;
    size_t key(int n, int m, int v, int u) const {
        const int W = 2 * L + 1;
        return ((size_t(n) * W + (m + L)) * (L + 1) + v) * W + (u + L);
    }
    const TupleCache& at(int n, int m, int v, int u) const { return t[key(n, m, v, u)]; }
};

TupleCache make_tuple_cache(int n, int m, int v, int u) {
    TupleCache c;
    c.factor = 0.5 * sgnpow(m) *
               std::sqrt((2 * v + 1) * (2 * n + 1) * fact(v - u) * fact(n - m) /
                         (v * (v + 1) * n * (n + 1) * fact(v + u) * fact(n + m)));
    c.qA = std::min({n, v, (n + v - std::abs(m + u)) / 2});
    c.qB = std::min({n, v, (n + v + 1 - std::abs(m + u)) / 2});
    std::vector<double> ga, gb;
    gaunt_batch(m, n, u, v, ga, gb);
    for (int q = 0; q <= c.qA; q++) {
        int p = n + v - 2 * q;
        c.A[q] = ga[q] * ipow(p) * double(n * (n + 1) + v * (v + 1) - p * (p + 1));
    }
    c.B[0] = 0;
    for (int q = 1; q <= c.qB; q++) {
        int p = n + v - 2 * q;
        c.B[q] = gb[q] * ipow(p + 1) *
                 std::sqrt((double(p + 1) * (p + 1) - double(n - v) * (n - v)) *
                           (double(n + v + 1) * (n + v + 1) - double(p + 1) * (p + 1)));
    }
    return c;
}

// create_vsh_cache_map: cpp/src/vsh_translation.cpp:36-51.
TranslationCache make_cache(int lmax) {
    TranslationCache C;
    C.L = lmax;
    const int W = 2 * lmax + 1;
    C.t.resize(size_t(lmax + 1) * W * (lmax + 1) * W);
    for (int n = 1; n <= lmax; n++)
        for (int m = -n; m <= n; m++)
            for (int v = 1; v <= n; v++)
                for (int u = -v; u <= v; u++) C.t[C.key(n, m, v, u)] = make_tuple_cache(n, m, v, u);
    return C;
}

// vsh_translation_insert_pair (Mie overload): cpp/src/vsh_translation.cpp:161-237.
// agg is a D x D row-major complex matrix; mie is [N, 2*lmax].
void insert_pair(cd* agg, int D, const cd* mie, int lmax, int i, int j, double rad, double theta, double phi,
                 double k, const TranslationCache& C) {
    const int rmax = lmax_to_rmax(lmax);
    const int pmax = 2 * lmax + 1;
    std::vector<cd> zn(pmax + 1);
    sph_hn_all(pmax, k * rad, zn.data());
    std::vector<double> Pnm(pmax * (pmax + 2) + 1);
    assoc_legendre_all(pmax, std::cos(theta), Pnm.data());
    auto M = [&](int p, int col) { return mie[size_t(p) * 2 * lmax + col]; };
    auto at = [&](int r, int c) -> cd& { return agg[size_t(r) * D + c]; };

    for (int n = 1; n <= lmax; n++)
        for (int m = -n; m <= n; m++)
            for (int v = 1; v <= n; v++)
                for (int u = -v; u <= v; u++) {
                    if (n == v && u < -m) continue;
                    const int mm = -m;
                    const TupleCache& c = C.at(n, mm, v, u);
                    cd eph = std::exp(cd(0, 1) * double(u + mm) * phi);
                    cd s = 0;
                    for (int q = 0; q <= c.qA; q++) {
                        int p = n + v - 2 * q;
                        s += c.A[q] * Pnm[p * (p + 2) - p + (u + mm)] * zn[p];
                    }
                    cd At = c.factor * eph * s;
                    s = 0;
                    for (int q = 1; q <= c.qB; q++) {
                        int p = n + v - 2 * q;
                        s += c.B[q] * Pnm[(p + 1) * (p + 3) - (p + 1) + (u + mm)] * zn[p + 1];
                    }
                    cd Bt = -c.factor * eph * s;
                    const cd tr[2] = {At, Bt};
                    for (int a = 0; a < 2; a++)
                        for (int b = 0; b < 2; b++) {
                            cd val = tr[(a + b) % 2];
                            int rn = n * (n + 2) - n + m - 1, rv = v * (v + 2) - v + u - 1;
                            at(i * 2 * rmax + a * rmax + rn, j * 2 * rmax + b * rmax + rv) = val * M(j, b * lmax + v - 1);
                            at(j * 2 * rmax + a * rmax + rn, i * 2 * rmax + b * rmax + rv) =
                                sgnpow(n + v + a + b) * val * M(i, b * lmax + v - 1);
                            if ((n == v && u != -m) || n != v) {
                                int rv2 = v * (v + 2) - v - u - 1, rn2 = n * (n + 2) - n - m - 1;
                                at(i * 2 * rmax + b * rmax + rv2, j * 2 * rmax + a * rmax + rn2) =
                                    sgnpow(m + u - a - b) * val * M(j, a * lmax + n - 1);
                                at(j * 2 * rmax + b * rmax + rv2, i * 2 * rmax + a * rmax + rn2) =
                                    sgnpow(m + u + n + v) * val * M(i, a * lmax + n - 1);
                            }
                        }
                }
}

// ----------------------------------------------------------- linear algebra --
// Row-block parallel GEMV y = A x (ParallelDenseMatrix::scaleAndAddTo,
// cpp/src/interactions.cpp:70-92, whose blocks run Eigen's vectorised GEMV kernel).
// Like Eigen's kernel, each thread works on a block of 4 rows that share every x
// load, and keeps independent partial sums (4 rows x 2 column phases x re/im), so
// that the product streams the matrix at memory speed rather than waiting on one
// dependent FMA chain per row.
void gemv(const cd* A, int D, const cd* x, cd* y) {
    const double* X = reinterpret_cast<const double*>(x);
    const int nb = (D + 3) / 4;
#pragma omp parallel for schedule(static)
    for (int blk = 0; blk < nb; blk++) {
        const int r0 = 4 * blk, nr = std::min(4, D - r0);
        double sr[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}}, si[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
        const double* row[4];
        for (int q = 0; q < 4; q++) row[q] = reinterpret_cast<const double*>(A + size_t(r0 + std::min(q, nr - 1)) * D);
        int c = 0;
        for (; c + 1 < D; c += 2) {
            for (int h = 0; h < 2; h++) {
                const double xr = X[2 * (c + h)], xi = X[2 * (c + h) + 1];
                for (int q = 0; q < 4; q++) {
                    const double ar = row[q][2 * (c + h)], ai = row[q][2 * (c + h) + 1];
                    sr[q][h] += ar * xr - ai * xi;
                    si[q][h] += ar * xi + ai * xr;
                }
            }
        }
        for (; c < D; c++) {
            const double xr = X[2 * c], xi = X[2 * c + 1];
            for (int q = 0; q < 4; q++) {
                const double ar = row[q][2 * c], ai = row[q][2 * c + 1];
                sr[q][0] += ar * xr - ai * xi;
                si[q][0] += ar * xi + ai * xr;
            }
        }
        for (int q = 0; q < nr; q++) y[r0 + q] = cd(sr[q][0] + sr[q][1], si[q][0] + si[q][1]);
    }
}

cd dotc(const std::vector<cd>& a, const std::vector<cd>& b) {   // sum conj(a) b
    double sr = 0, si = 0;
    for (size_t i = 0; i < a.size(); i++) {
        sr += a[i].real() * b[i].real() + a[i].imag() * b[i].imag();
        si += a[i].real() * b[i].imag() - a[i].imag() * b[i].real();
    }
    return cd(sr, si);
}

double sqnorm(const std::vector<cd>& a) {
    double s = 0;
    for (auto& z : a) s += std::norm(z);
    return s;
}

// y = M x for a block-diagonal M given as M_inv_blocks [D][bs]
// (apply_block_preconditioner, cpp/src/interactions.cpp:211-228).
void block_apply(const cd* M, int bs, int D, const std::vector<cd>& x, std::vector<cd>& y) {
    for (int j0 = 0; j0 < D; j0 += bs)
        for (int r = 0; r < bs; r++) {
            cd acc = 0;
            for (int k = 0; k < bs; k++) acc += M[size_t(j0 + r) * bs + k] * x[j0 + k];
            y[j0 + r] = acc;
        }
}

// Eigen-style BiCGSTAB (called from cpp/src/interactions.cpp:359-366 with the
// identity preconditioner, and from :335-341 with the block-diagonal one, M given):
// x0 = 0, stop when |r|^2 <= tol^2 |b|^2; with M the products are A (M p) and
// A (M s) and x moves by alpha M p + omega M s.
int bicgstab_eigen(const cd* A, int D, const cd* b, cd* xout, double tol, int maxit, double* err_out,
                   const cd* M = nullptr, int bs = 0) {
    std::vector<cd> x(D, 0.0), r(b, b + D), r0(r), v(D, 0.0), p(D, 0.0), s(D), t(D), y(D), z(D);
    double r0sq = sqnorm(r0), bsq = sqnorm(r);
    if (bsq == 0) {
        std::fill(xout, xout + D, cd(0));
        if (err_out) *err_out = 0;
        return 0;
    }
    cd rho = 1, alpha = 1, w = 1;
    const double tol2 = tol * tol * bsq;
    const double eps = 2.220446049250313e-16, eps2 = eps * eps;
    int i = 0, restarts = 0;
    while (sqnorm(r) > tol2 && i < maxit) {
        cd rho_old = rho;
        rho = dotc(r0, r);
        if (std::abs(rho) < eps2 * r0sq) {
            gemv(A, D, x.data(), t.data());
            for (int e = 0; e < D; e++) r[e] = b[e] - t[e];
            r0 = r;
            rho = r0sq = sqnorm(r);
            if (restarts++ == 0) i = 0;
        }
        cd beta = (rho / rho_old) * (alpha / w);
        for (int e = 0; e < D; e++) p[e] = r[e] + beta * (p[e] - w * v[e]);
        if (M) block_apply(M, bs, D, p, y); else y = p;
        gemv(A, D, y.data(), v.data());
        alpha = rho / dotc(r0, v);
        for (int e = 0; e < D; e++) s[e] = r[e] - alpha * v[e];
        if (M) block_apply(M, bs, D, s, z); else z = s;
        gemv(A, D, z.data(), t.data());
        double tmp = sqnorm(t);
        w = tmp > 0 ? dotc(t, s) / tmp : cd(0);
        for (int e = 0; e < D; e++) {
            x[e] += alpha * y[e] + w * z[e];
            r[e] = s[e] - w * t[e];
        }
        ++i;
    }
    if (err_out) *err_out = std::sqrt(sqnorm(r) / bsq);
    std::copy(x.begin(), x.end(), xout);
    return i;
}

// LU with partial pivoting, in place on a D x D row-major matrix; solves A x = b.
int lu_solve(cd* A, int D, const cd* b, cd* x) {
    std::vector<int> piv(D);
    for (int k = 0; k < D; k++) {
        int pr = k;
        double best = std::abs(A[size_t(k) * D + k]);
        for (int r = k + 1; r < D; r++) {
            double v = std::abs(A[size_t(r) * D + k]);
            if (v > best) { best = v; pr = r; }
        }
        piv[k] = pr;
        if (best == 0.0) return -1;
        if (pr != k)
            for (int c = 0; c < D; c++) std::swap(A[size_t(k) * D + c], A[size_t(pr) * D + c]);
        cd inv = 1.0 / A[size_t(k) * D + k];
#pragma omp parallel for schedule(static)
        for (int r = k + 1; r < D; r++) {
            cd f = A[size_t(r) * D + k] * inv;
            A[size_t(r) * D + k] = f;
            cd* rr = A + size_t(r) * D;
            const cd* kr = A + size_t(k) * D;
            for (int c = k + 1; c < D; c++) rr[c] -= f * kr[c];
        }
    }
    std::vector<cd> y(b, b + D);
    for (int k = 0; k < D; k++)
        if (piv[k] != k) std::swap(y[k], y[piv[k]]);
    for (int r = 0; r < D; r++) {
        cd s = y[r];
        for (int c = 0; c < r; c++) s -= A[size_t(r) * D + c] * y[c];
        y[r] = s;
    }
    for (int r = D - 1; r >= 0; r--) {
        cd s = y[r];
        for (int c = r + 1; c < D; c++) s -= A[size_t(r) * D + c] * y[c];
        y[r] = s / A[size_t(r) * D + r];
    }
    std::copy(y.begin(), y.end(), x);
    return 0;
}

// ------------------------------------------------------------------- VSH --
cd Emn_fn(int m, int n) {   // cpp/src/vsh_functions.cpp:56-58
    return ipow(n) * std::sqrt((2 * n + 1) * fact(n - m) / (n * (n + 1) * fact(n + m)));
}

// zn(mode): outgoing -> h_n, ingoing -> conj(h_n), incident/interior -> j_n
// (cpp/src/vsh_functions.cpp:42-54).
cd zn_mode(int mode, int n, double z, bool deriv) {
    switch (mode) {
        case 0: return sph_hn_d(n, z, deriv);
        case 2:
        case 3: return sph_jn_c_d(n, cd(z, 0), deriv);
        default: return std::conj(sph_hn_d(n, z, deriv));
    }
}

void vsh_electric(int n, int m, int mode, double rad, double theta, double phi, double k, cd* E) {
    double kr = k * rad;
    cd eph = std::exp(cd(0, 1) * double(m) * phi);
    cd H = zn_mode(mode, n, kr, false), Hp = zn_mode(mode, n, kr, true);
    double P = assoc_legendre(n, m, std::cos(theta));
    cd f = (H + kr * Hp) * eph / kr;
    E[0] = double(n * (n + 1)) * P * H / kr * eph;
    E[1] = f * tau_fn(n, m, theta);
    E[2] = cd(0, 1) * f * pi_fn(n, m, theta);
}

void vsh_magnetic(int n, int m, int mode, double rad, double theta, double phi, double k, cd* E) {
    double kr = k * rad;
    cd eph = std::exp(cd(0, 1) * double(m) * phi);
    cd H = zn_mode(mode, n, kr, false);
    cd f = H * eph;
    E[0] = 0;
    E[1] = cd(0, 1) * f * pi_fn(n, m, theta);
    E[2] = -f * tau_fn(n, m, theta);
}

void sph_to_cart_vec(const cd* v, double th, double ph, cd* out) {   // vec_sph_to_cart
    double st = std::sin(th), ct = std::cos(th), sp = std::sin(ph), cp = std::cos(ph);
    out[0] = v[0] * st * cp + v[1] * ct * cp + v[2] * (-sp);
    out[1] = v[0] * st * sp + v[1] * ct * sp + v[2] * cp;
    out[2] = v[0] * ct + v[1] * (-st);
}

}   // namespace

// =========================================================================
// C ABI
// =========================================================================
extern "C" {

int orc_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

double orc_factorial(double n) { return fact(n); }

// special.spherical_jn (complex argument): cpp/src/special.cpp:20-45
void orc_spherical_jn(int cnt, const int* n, const double* z /*cnt x 2*/, int deriv, double* out /*cnt x 2*/) {
    for (int i = 0; i < cnt; i++) {
        cd r = sph_jn_c_d(n[i], cd(z[2 * i], z[2 * i + 1]), deriv != 0);
        out[2 * i] = r.real();
        out[2 * i + 1] = r.imag();
    }
}

// special.spherical_yn: cpp/src/special.cpp:47-52
void orc_spherical_yn(int cnt, const int* n, const double* z, int deriv, double* out) {
    for (int i = 0; i < cnt; i++) {
        int l = n[i];
        double x = z[i];
        if (!deriv) out[i] = sph_yl_real(l, x);
        else out[i] = sph_yl_real(l - 1, x) - (l + 1) / x * sph_yl_real(l, x);
    }
}

// special.spherical_hn / spherical_hn_2: cpp/src/special.cpp:54-88, 114-116
void orc_spherical_hn(int cnt, const int* n, const double* z, int deriv, int second_kind, double* out) {
    for (int i = 0; i < cnt; i++) {
        cd r = sph_hn_d(n[i], z[i], deriv != 0);
        if (second_kind) r = std::conj(r);
        out[2 * i] = r.real();
        out[2 * i + 1] = r.imag();
    }
}

// special.spherical_hn_recursion: cpp/src/special.cpp:90-111
void orc_spherical_hn_recursion(int nmax, double z, double* out) {
    std::vector<cd> h(nmax + 1);
    sph_hn_all(nmax, z, h.data());
    std::memcpy(out, h.data(), sizeof(cd) * (nmax + 1));
}

// special.riccati_1/2/3: cpp/src/special.cpp:118-142
void orc_riccati(int kind, int cnt, const int* n, const double* z, int deriv, double* out) {
    for (int i = 0; i < cnt; i++) {
        int l = n[i];
        double x = z[i];
        double r1, r2;
        double jn = sph_jl_real(l, x);
        r1 = !deriv ? x * jn : x * (sph_jl_real(l - 1, x) - (l + 1) / x * jn) + jn;
        double yn = sph_yl_real(l, x);
        r2 = !deriv ? -x * yn : -x * (sph_yl_real(l - 1, x) - (l + 1) / x * yn) - yn;
        out[i] = kind == 1 ? r1 : (kind == 2 ? r2 : r2 - r1);
    }
}

// special.associated_legendre: cpp/src/special.cpp:148-178
void orc_associated_legendre(int cnt, const int* n, const int* m, const double* z, double* out) {
    for (int i = 0; i < cnt; i++) out[i] = assoc_legendre(n[i], m[i], z[i]);
}

// special.associated_legendre_recursion: cpp/src/special.cpp:180-204
void orc_associated_legendre_recursion(int nmax, double z, double* out) { assoc_legendre_all(nmax, z, out); }

// special.pi_func / tau_func: cpp/src/special.cpp:209-270
void orc_pi_func(int cnt, const int* n, const int* m, const double* th, double* out) {
    for (int i = 0; i < cnt; i++) out[i] = pi_fn(n[i], m[i], th[i]);
}
void orc_tau_func(int cnt, const int* n, const int* m, const double* th, double* out) {
    for (int i = 0; i < cnt; i++) out[i] = tau_fn(n[i], m[i], th[i]);
}

// special.wigner_3j / a_func / b_func: cpp/src/special.cpp:272-296
double orc_wigner_3j(int j1, int j2, int j3, int m1, int m2, int m3) { return wigner3j(j1, j2, j3, m1, m2, m3); }
double orc_a_func(int m, int n, int u, int v, int p) { return a_fn(m, n, u, v, p); }
double orc_b_func(int m, int n, int u, int v, int p) { return b_fn(m, n, u, v, p); }

// wigner_3j_batch: cpp/src/special.cpp:298-363.  Returns the count written.
int orc_wigner_3j_batch(int j2, int j3, int m1, int m2, int m3, int* jmin, double* out, int cap) {
    W3Batch w = wigner3j_batch(j2, j3, m1, m2, m3);
    *jmin = w.jmin;
    int c = int(w.val.size());
    for (int i = 0; i < c && i < cap; i++) out[i] = w.val[i];
    return c;
}

// gaunt_batch: cpp/src/special.cpp:365-440.  a_out/b_out need n+1 entries.
void orc_gaunt_batch(int m, int n, int u, int v, double* a_out, int* na, double* b_out, int* nb) {
    std::vector<double> a, b;
    gaunt_batch(m, n, u, v, a, b);
    *na = int(a.size());
    *nb = int(b.size());
    for (size_t i = 0; i < a.size(); i++) a_out[i] = a[i];
    for (size_t i = 0; i < b.size(); i++) b_out[i] = b[i];
}

// vsh_translation (scalar): cpp/src/vsh_translation.cpp:428-470.  out = {A, B}.
void orc_vsh_translation(int cnt, int m, int n, int u, int v, const double* rad, const double* theta,
                         const double* phi, double k, int mode, double* out /* cnt x {A.re,A.im,B.re,B.im} */) {
    m *= -1;
    double base = 0.5 * sgnpow(m) *
                  std::sqrt((2 * v + 1) * (2 * n + 1) * fact(v - u) * fact(n - m) /
                            (v * (v + 1) * n * (n + 1) * fact(v + u) * fact(n + m)));
    std::vector<double> ga, gb;
    gaunt_batch(m, n, u, v, ga, gb);
    int qA = std::min({n, v, (n + v - std::abs(m + u)) / 2});
    int qB = std::min({n, v, (n + v + 1 - std::abs(m + u)) / 2});
    for (int i = 0; i < cnt; i++) {
        cd factor = base * std::exp(cd(0, 1) * double(u + m) * phi[i]);
        double ct = std::cos(theta[i]);
        cd s = 0;
        for (int q = 0; q <= qA; q++) {
            int p = n + v - 2 * q;
            cd Aq = ga[q] * ipow(p) * double(n * (n + 1) + v * (v + 1) - p * (p + 1));
            s += Aq * assoc_legendre(p, u + m, ct) * zn_mode(mode, p, k * rad[i], false);
        }
        cd At = factor * s;
        s = 0;
        for (int q = 1; q <= qB; q++) {
            int p = n + v - 2 * q;
            cd Bq = gb[q] * ipow(p + 1) *
                    std::sqrt((double(p + 1) * (p + 1) - double(n - v) * (n - v)) *
                              (double(n + v + 1) * (n + v + 1) - double(p + 1) * (p + 1)));
            s += Bq * assoc_legendre(p + 1, u + m, ct) * zn_mode(mode, p + 1, k * rad[i], false);
        }
        cd Bt = -factor * s;
        out[4 * i] = At.real();
        out[4 * i + 1] = At.imag();
        out[4 * i + 2] = Bt.real();
        out[4 * i + 3] = Bt.imag();
    }
}

// Translation-cache entry (vsh_cache, cpp/src/vsh_translation.cpp:12-34):
// factor, qmax_A, qmax_B, A[q], B[q] as interleaved complex.
void orc_vsh_cache_entry(int n, int m, int v, int u, double* factor, int* qA, int* qB, double* A, double* B) {
    TupleCache c = make_tuple_cache(n, m, v, u);
    factor[0] = c.factor.real();
    factor[1] = c.factor.imag();
    *qA = c.qA;
    *qB = c.qB;
    for (int q = 0; q <= c.qA; q++) { A[2 * q] = c.A[q].real(); A[2 * q + 1] = c.A[q].imag(); }
    for (int q = 0; q <= c.qB; q++) { B[2 * q] = c.B[q].real(); B[2 * q + 1] = c.B[q].imag(); }
}

// interactions.sphere_aggregate_tmatrix: cpp/src/interactions.cpp:370-415.
// positions [N,3] f64, mie [N, 2*lmax] c128, out [D,D] c128 (D = 2*rmax*N).
void orc_sphere_aggregate_tmatrix(int N, int lmax, const double* pos, const double* mie, double k, double* out) {
    const int rmax = lmax_to_rmax(lmax);
    const int D = 2 * rmax * N;
    cd* agg = reinterpret_cast<cd*>(out);
    const cd* M = reinterpret_cast<const cd*>(mie);
#pragma omp parallel for schedule(static)
    for (long e = 0; e < long(D) * D; e++) agg[e] = 0.0;
    if (N == 1) return;
    const int P = N * (N - 1) / 2;
    std::vector<int> iv(P), jv(P);
    int c = 0;
    for (int i = 0; i < N; i++)
        for (int j = i + 1; j < N; j++) { iv[c] = i; jv[c] = j; c++; }
    TranslationCache C = make_cache(lmax);
#pragma omp parallel for schedule(dynamic, 4)
    for (int ij = 0; ij < P; ij++) {
        int i = iv[ij], j = jv[ij];
        double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1], dz = pos[3 * i + 2] - pos[3 * j + 2];
        double rad = std::sqrt(dx * dx + dy * dy + dz * dz);
        double theta = std::acos(dz / rad);
        double phi = std::atan2(dy, dx);
        insert_pair(agg, D, M, lmax, i, j, rad, theta, phi, k, C);
    }
}

// interactions.particle_aggregate_tmatrix: cpp/src/interactions.cpp:416-462 with
// vsh_translation_insert_pair (T-matrix overload), cpp/src/vsh_translation.cpp:53-159:
// the translation blocks of the pair (the Mie overload's placements with unit Mie
// coefficients), then agg(i, j) = A(i, j) T_j and agg(j, i) = A(j, i) T_i.
// positions [N,3] f64, tmatrix [N, 2*rmax, 2*rmax] c128 (row-major), out [D,D] c128.
void orc_particle_aggregate_tmatrix(int N, int rmax, const double* pos, const double* tmat, double k, double* out) {
    const int lmax = int(std::lround(std::sqrt(1.0 + rmax) - 1.0));
    const int B = 2 * rmax, D = B * N;
    cd* agg = reinterpret_cast<cd*>(out);
    const cd* T = reinterpret_cast<const cd*>(tmat);
    for (long e = 0; e < long(D) * D; e++) agg[e] = 0.0;
    if (N == 1) return;
    std::vector<cd> A(size_t(D) * D, cd(0.0));
    std::vector<cd> ones(size_t(N) * 2 * lmax, cd(1.0));
    const int P = N * (N - 1) / 2;
    std::vector<int> iv(P), jv(P);
    int c = 0;
    for (int i = 0; i < N; i++)
        for (int j = i + 1; j < N; j++) { iv[c] = i; jv[c] = j; c++; }
    TranslationCache C = make_cache(lmax);
#pragma omp parallel for schedule(dynamic, 4)
    for (int ij = 0; ij < P; ij++) {
        const int i = iv[ij], j = jv[ij];
        double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1], dz = pos[3 * i + 2] - pos[3 * j + 2];
        double rad = std::sqrt(dx * dx + dy * dy + dz * dz);
        insert_pair(A.data(), D, ones.data(), lmax, i, j, rad, std::acos(dz / rad), std::atan2(dy, dx), k, C);
        for (int r = 0; r < B; r++)
            for (int col = 0; col < B; col++) {
                cd sij = 0, sji = 0;
                for (int q = 0; q < B; q++) {
                    sij += A[size_t(i * B + r) * D + j * B + q] * T[(size_t(j) * B + q) * B + col];
                    sji += A[size_t(j * B + r) * D + i * B + q] * T[(size_t(i) * B + q) * B + col];
                }
                agg[size_t(i * B + r) * D + j * B + col] = sij;
                agg[size_t(j * B + r) * D + i * B + col] = sji;
            }
    }
}

// interactions.reflection_matrix_nia: cpp/src/interactions.cpp:464-512.  Every
// (i, j) block, i and j over all particles: the outgoing translation from particle
// j to the mirror image of particle i in the plane z (its z replaced by 2 z - z_i),
// times -reflection (-1)^(m+n+a+1) and the Mie coefficient of the column particle.
// positions [N,3] f64, mie [N, 2*lmax] c128, out [D,D] c128.
void orc_reflection_matrix_nia(int N, int lmax, const double* pos, const double* mie, double k, double r_re,
                               double r_im, double z, double* out) {
    const int rmax = lmax_to_rmax(lmax);
    const int D = 2 * rmax * N;
    cd* R = reinterpret_cast<cd*>(out);
    const cd* M = reinterpret_cast<const cd*>(mie);
    const cd refl(r_re, r_im);
    for (long e = 0; e < long(D) * D; e++) R[e] = 0.0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < N; i++) {
        const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2] - 2 * (pos[3 * i + 2] - z);
        for (int j = 0; j < N; j++) {
            const double dx = xi - pos[3 * j], dy = yi - pos[3 * j + 1], dz = zi - pos[3 * j + 2];
            double rad = std::sqrt(dx * dx + dy * dy + dz * dz);
            double theta = std::acos(dz / rad);
            double phi = std::atan2(dy, dx);
            for (int n = 1; n <= lmax; n++)
                for (int m = -n; m <= n; m++)
                    for (int v = 1; v <= lmax; v++)
                        for (int u = -v; u <= v; u++) {
                            double tr[4];
                            orc_vsh_translation(1, m, n, u, v, &rad, &theta, &phi, k, 0, tr);
                            const cd transfer[2] = {cd(tr[0], tr[1]), cd(tr[2], tr[3])};
                            for (int a = 0; a < 2; a++)
                                for (int b = 0; b < 2; b++) {
                                    const cd factor = -refl * double(sgnpow(m + n + a + 1));
                                    const long idx = long(i) * 2 * rmax + a * rmax + n * (n + 2) - n + m - 1;
                                    const long idy = long(j) * 2 * rmax + b * rmax + v * (v + 2) - v + u - 1;
                                    R[idx * D + idy] = factor * transfer[(a + b) % 2] * M[long(j) * 2 * lmax + b * lmax + v - 1];
                                }
                        }
        }
    }
}

// interactions.sphere_aggregate_tmatrix_periodic: src/miepy/interactions.py:153-186.
// The aggregate of orc_sphere_aggregate_tmatrix, then for every ordered pair (i, j)
// and every mode pair the lattice sum over the cells c of the outgoing translation
// (orc_vsh_translation) from pos_j + c to pos_i, times e^{-i k khat.c}, times
// mie(j, b, v).  cells [ncell,3], khat [3].
void orc_sphere_aggregate_tmatrix_periodic(int N, int lmax, const double* pos, const double* mie, double k, int ncell,
                                           const double* cells, const double* khat, double* out) {
    orc_sphere_aggregate_tmatrix(N, lmax, pos, mie, k, out);
    if (ncell < 1) return;
    const int rmax = lmax_to_rmax(lmax);
    const int D = 2 * rmax * N;
    cd* agg = reinterpret_cast<cd*>(out);
    const cd* M = reinterpret_cast<const cd*>(mie);
    std::vector<cd> phase(ncell);
    for (int c = 0; c < ncell; c++)
        phase[c] = std::exp(cd(0, -k * (khat[0] * cells[3 * c] + khat[1] * cells[3 * c + 1] + khat[2] * cells[3 * c + 2])));
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) {
            std::vector<double> rad(ncell), theta(ncell), phi(ncell), tr(4 * size_t(ncell));
            for (int c = 0; c < ncell; c++) {
                const double dx = pos[3 * i] - (cells[3 * c] + pos[3 * j]);
                const double dy = pos[3 * i + 1] - (cells[3 * c + 1] + pos[3 * j + 1]);
                const double dz = pos[3 * i + 2] - (cells[3 * c + 2] + pos[3 * j + 2]);
                rad[c] = std::sqrt(dx * dx + dy * dy + dz * dz);
                theta[c] = std::acos(dz / rad[c]);
                phi[c] = std::atan2(dy, dx);
            }
            for (int n = 1; n <= lmax; n++)
                for (int m = -n; m <= n; m++)
                    for (int v = 1; v <= lmax; v++)
                        for (int u = -v; u <= v; u++) {
                            orc_vsh_translation(ncell, m, n, u, v, rad.data(), theta.data(), phi.data(), k, 0, tr.data());
                            cd sA = 0, sB = 0;
                            for (int c = 0; c < ncell; c++) {
                                sA += cd(tr[4 * c], tr[4 * c + 1]) * phase[c];
                                sB += cd(tr[4 * c + 2], tr[4 * c + 3]) * phase[c];
                            }
                            const cd tsum[2] = {sA, sB};
                            for (int a = 0; a < 2; a++)
                                for (int b = 0; b < 2; b++) {
                                    const long idx = long(i) * 2 * rmax + a * rmax + n * (n + 2) - n + m - 1;
                                    const long idy = long(j) * 2 * rmax + b * rmax + v * (v + 2) - v + u - 1;
                                    agg[idx * D + idy] += tsum[(a + b) % 2] * M[long(j) * 2 * lmax + b * lmax + v - 1];
                                }
                        }
        }
}

// interactions.solve_linear_system: cpp/src/interactions.cpp:347-368.
// method 0 = bicgstab (Eigen, tol/maxiter), 1 = exact (partial-pivot LU).
// T is the aggregate T-matrix WITHOUT the identity.  Returns iterations (bicgstab),
// 0 (exact) or -1 (singular).
int orc_solve_linear_system(int D, const double* T, const double* b, int method, double tol, int maxiter,
                            double* x, double* err_out) {
    std::vector<cd> A(size_t(D) * D);
    const cd* Tc = reinterpret_cast<const cd*>(T);
#pragma omp parallel for schedule(static)
    for (long e = 0; e < long(D) * D; e++) A[e] = Tc[e];
    for (int i = 0; i < D; i++) A[size_t(i) * D + i] += 1.0;
    if (method == 1) {
        if (err_out) *err_out = 0;
        return lu_solve(A.data(), D, reinterpret_cast<const cd*>(b), reinterpret_cast<cd*>(x));
    }
    return bicgstab_eigen(A.data(), D, reinterpret_cast<const cd*>(b), reinterpret_cast<cd*>(x), tol, maxiter,
                          err_out);
}

// solve_linear_system_preconditioned: cpp/src/interactions.cpp:321-345 (the exact
// branch ignores M).  Minv = M_inv_blocks [D][bs].
int orc_solve_linear_system_precond(int D, const double* T, const double* b, int method, const double* Minv, int bs,
                                    double tol, int maxiter, double* x, double* err_out) {
    if (method == 1) return orc_solve_linear_system(D, T, b, method, tol, maxiter, x, err_out);
    std::vector<cd> A(size_t(D) * D);
    const cd* Tc = reinterpret_cast<const cd*>(T);
#pragma omp parallel for schedule(static)
    for (long e = 0; e < long(D) * D; e++) A[e] = Tc[e];
    for (int i = 0; i < D; i++) A[size_t(i) * D + i] += 1.0;
    return bicgstab_eigen(A.data(), D, reinterpret_cast<const cd*>(b), reinterpret_cast<cd*>(x), tol, maxiter,
                          err_out, reinterpret_cast<const cd*>(Minv), bs);
}

// bicgstab_preconditioned_profiled (x0 = b, absolute |r| < tol):
// cpp/src/interactions.cpp:230-290.  A includes the identity.
int orc_bicgstab_precond(int D, const double* Aflat, const double* bflat, const double* Minv, int bs, int maxiter,
                         double tol, double* xflat, double* err_out) {
    const cd* A = reinterpret_cast<const cd*>(Aflat);
    const cd* b = reinterpret_cast<const cd*>(bflat);
    const cd* M = reinterpret_cast<const cd*>(Minv);
    std::vector<cd> x(b, b + D), Ax(D), r(D);
    gemv(A, D, x.data(), Ax.data());
    for (int e = 0; e < D; e++) r[e] = b[e] - Ax[e];
    double err = std::sqrt(sqnorm(r));
    int it = 0;
    if (err >= tol) {
        std::vector<cd> rh(r), v(D, 0.0), p(D, 0.0), ph(D), vi(D), s(D), sh(D), t(D);
        cd rho_prev = 1, alpha = 1, w_prev = 1;
        it = 1;
        while (true) {
            cd rho = dotc(rh, r);
            cd beta = (rho / rho_prev) * (alpha / w_prev);
            for (int e = 0; e < D; e++) p[e] = r[e] + beta * (p[e] - w_prev * v[e]);
            block_apply(M, bs, D, p, ph);
            gemv(A, D, ph.data(), vi.data());
            alpha = rho / dotc(rh, vi);
            for (int e = 0; e < D; e++) s[e] = r[e] - alpha * vi[e];
            block_apply(M, bs, D, s, sh);
            gemv(A, D, sh.data(), t.data());
            cd w = dotc(t, s) / dotc(t, t);
            for (int e = 0; e < D; e++) { x[e] += alpha * ph[e] + w * sh[e]; r[e] = s[e] - w * t[e]; }
            err = std::sqrt(sqnorm(r));
            if (err < tol || it > maxiter) break;
            rho_prev = rho; v = vi; w_prev = w;
            it++;
        }
    }
    if (err_out) *err_out = err;
    std::memcpy(xflat, x.data(), sizeof(cd) * D);
    return it;
}

// interactions.bicgstab (hand-written variant, x0 = b): cpp/src/interactions.cpp:98-150.
int orc_bicgstab_plain(int D, const double* Aflat, const double* bflat, int maxiter, double tol, double* xflat,
                       double* err_out) {
    const cd* A = reinterpret_cast<const cd*>(Aflat);
    const cd* b = reinterpret_cast<const cd*>(bflat);
    std::vector<cd> x(b, b + D), Ax(D), r(D);
    gemv(A, D, x.data(), Ax.data());
    for (int e = 0; e < D; e++) r[e] = b[e] - Ax[e];
    double err = std::sqrt(sqnorm(r));
    int it = 0;
    if (err >= tol) {
        std::vector<cd> rh(r), v(D, 0.0), p(D, 0.0), pi(D), vi(D), h(D), s(D), t(D);
        cd rho_prev = 1, alpha = 1, w_prev = 1;
        it = 1;
        while (true) {
            cd rho = dotc(rh, r);
            cd beta = (rho / rho_prev) * (alpha / w_prev);
            for (int e = 0; e < D; e++) pi[e] = r[e] + beta * (p[e] - w_prev * v[e]);
            gemv(A, D, pi.data(), vi.data());
            alpha = rho / dotc(rh, vi);
            for (int e = 0; e < D; e++) { h[e] = x[e] + alpha * pi[e]; s[e] = r[e] - alpha * vi[e]; }
            gemv(A, D, s.data(), t.data());
            cd w = dotc(t, s) / dotc(t, t);
            for (int e = 0; e < D; e++) { x[e] = h[e] + w * s[e]; r[e] = s[e] - w * t[e]; }
            err = std::sqrt(sqnorm(r));
            if (err < tol || it > maxiter) break;
            rho_prev = rho; v = vi; p = pi; w_prev = w;
            it++;
        }
    }
    if (err_out) *err_out = err;
    std::memcpy(xflat, x.data(), sizeof(cd) * D);
    return it;
}

// Row-block GEMV y = A x (cpp/src/interactions.cpp:70-92), used by timing legs.
void orc_gemv(int D, const double* A, const double* x, double* y) {
    gemv(reinterpret_cast<const cd*>(A), D, reinterpret_cast<const cd*>(x), reinterpret_cast<cd*>(y));
}

// flux.particle_cross_sections: cpp/src/flux.cpp:5-30.  out = [Cscat | Cabs | Cext], each 2*lmax.
void orc_particle_cross_sections(int rmax, const double* ps, const double* pi, const double* pr, double k, double* out) {
    const cd* p_scat = reinterpret_cast<const cd*>(ps);
    const cd* p_inc = reinterpret_cast<const cd*>(pi);
    const cd* p_src = reinterpret_cast<const cd*>(pr);
    int lmax = rmax_to_lmax(rmax);
    std::vector<double> Cext(2 * lmax, 0.0), Cabs(2 * lmax, 0.0);
    double f = 4 * kPi / (k * k);
    for (int n = 1; n <= lmax; n++)
        for (int m = -n; m <= n; m++)
            for (int a = 0; a < 2; a++) {
                int r = a * rmax + n * n + n + m - 1;
                int idx = a * lmax + n - 1;
                Cabs[idx] += f * (std::real(std::conj(p_inc[r]) * p_scat[r]) - std::norm(p_scat[r]));
                Cext[idx] += f * std::real(std::conj(p_src[r]) * p_scat[r]);
            }
    for (int i = 0; i < 2 * lmax; i++) {
        out[i] = Cext[i] - Cabs[i];
        out[2 * lmax + i] = Cabs[i];
        out[4 * lmax + i] = Cext[i];
    }
}

// flux.cluster_cross_sections: cpp/src/flux.cpp:32-57.
void orc_cluster_cross_sections(int rmax, const double* pc, const double* pr, double k, double* out) {
    const cd* p_cl = reinterpret_cast<const cd*>(pc);
    const cd* p_src = reinterpret_cast<const cd*>(pr);
    int lmax = rmax_to_lmax(rmax);
    std::vector<double> Cs(2 * lmax, 0.0), Ce(2 * lmax, 0.0);
    double f = 4 * kPi / (k * k);
    for (int n = 1; n <= lmax; n++)
        for (int m = -n; m <= n; m++)
            for (int a = 0; a < 2; a++) {
                int r = a * rmax + n * n + n + m - 1;
                int idx = a * lmax + n - 1;
                Cs[idx] += f * std::norm(p_cl[r]);
                Ce[idx] += f * std::real(std::conj(p_src[r]) * p_cl[r]);
            }
    for (int i = 0; i < 2 * lmax; i++) {
        out[i] = Cs[i];
        out[2 * lmax + i] = Ce[i] - Cs[i];
        out[4 * lmax + i] = Ce[i];
    }
}

// forces.force: cpp/src/forces.cpp:7-86.
void orc_force(int rmax, const double* psf, const double* pif, double k, double eps_b, double* F) {
    const cd* ps = reinterpret_cast<const cd*>(psf);
    const cd* pin = reinterpret_cast<const cd*>(pif);
    const cd *p = ps, *q = ps + rmax, *pi = pin, *qi = pin + rmax;
    int lmax = rmax_to_lmax(rmax);
    cd Fxy = 0, Fz = 0;
    double Axy = kPi / (k * k) * kEps0Gsl * eps_b;
    double Az = -2 * Axy;
    for (int n = 1; n <= lmax; n++)
        for (int m = -n; m <= n; m++) {
            int r = n * n + n + m - 1;
            if (m != n) {
                double f = Axy * std::sqrt(double((n + m + 1) * (n - m))) / double(n * (n + 1));
                int r1 = r + 1;
                Fxy += f * (2.0 * p[r] * std::conj(q[r1]) - p[r] * std::conj(qi[r1]) - pi[r] * std::conj(q[r1]) +
                            2.0 * q[r] * std::conj(p[r1]) - q[r] * std::conj(pi[r1]) - qi[r] * std::conj(p[r1]));
            }
            double f = Az * m / double(n * (n + 1));
            Fz += f * (2.0 * p[r] * std::conj(q[r]) - p[r] * std::conj(qi[r]) - pi[r] * std::conj(q[r]));
            if (n < lmax) {
                f = -Axy * std::sqrt((n + m + 2) * (n + m + 1) * n * (n + 2) / double((2 * n + 3) * (2 * n + 1))) / (n + 1);
                int r1 = (n + 1) * (n + 1) + (n + 1) + m;
                Fxy += f * (2.0 * p[r] * std::conj(p[r1]) - p[r] * std::conj(pi[r1]) - pi[r] * std::conj(p[r1]) +
                            2.0 * q[r] * std::conj(q[r1]) - q[r] * std::conj(qi[r1]) - qi[r] * std::conj(q[r1]));
                f = Axy * std::sqrt((n - m + 1) * (n - m + 2) * n * (n + 2) / double((2 * n + 3) * (2 * n + 1))) / (n + 1);
                r1 = (n + 1) * (n + 1) + (n + 1) + m - 2;
                Fxy += f * (2.0 * p[r1] * std::conj(p[r]) - p[r1] * std::conj(pi[r]) - pi[r1] * std::conj(p[r]) +
                            2.0 * q[r1] * std::conj(q[r]) - q[r1] * std::conj(qi[r]) - qi[r1] * std::conj(q[r]));
                f = Az * std::sqrt((n - m + 1) * (n + m + 1) * n * (n + 2) / double((2 * n + 3) * (2 * n + 1))) / (n + 1);
                r1 = (n + 1) * (n + 1) + (n + 1) + m - 1;
                Fz += f * (2.0 * p[r1] * std::conj(p[r]) - p[r1] * std::conj(pi[r]) - pi[r1] * std::conj(p[r]) +
                           2.0 * q[r1] * std::conj(q[r]) - q[r1] * std::conj(qi[r]) - qi[r1] * std::conj(q[r]));
            }
        }
    F[0] = Fxy.real();
    F[1] = Fxy.imag();
    F[2] = Fz.real();
}

// forces.torque: cpp/src/forces.cpp:88-137.
void orc_torque(int rmax, const double* psf, const double* pif, double k, double eps_b, double* T) {
    const cd* ps = reinterpret_cast<const cd*>(psf);
    const cd* pin = reinterpret_cast<const cd*>(pif);
    const cd *p = ps, *q = ps + rmax, *pi = pin, *qi = pin + rmax;
    int lmax = rmax_to_lmax(rmax);
    double A = -2 * kPi / (k * k * k) * kEps0Gsl * eps_b;
    T[0] = T[1] = T[2] = 0;
    for (int n = 1; n <= lmax; n++)
        for (int m = -n; m <= n; m++) {
            int r = n * n + n + m - 1;
            if (m != n) {
                double f = -A * std::sqrt(double((n - m) * (n + m + 1)));
                int r1 = r + 1;
                T[0] += f * std::real(p[r] * std::conj(p[r1]) + q[r] * std::conj(q[r1]) -
                                      0.5 * (p[r1] * std::conj(pi[r]) + p[r] * std::conj(pi[r1]) +
                                             q[r1] * std::conj(qi[r]) + q[r] * std::conj(qi[r1])));
                T[1] += f * std::imag(p[r] * std::conj(p[r1]) + q[r] * std::conj(q[r1]) +
                                      0.5 * (p[r1] * std::conj(pi[r]) - p[r] * std::conj(pi[r1]) +
                                             q[r1] * std::conj(qi[r]) - q[r] * std::conj(qi[r1])));
            }
            double f = A * m;
            T[2] += f * (std::norm(p[r]) + std::norm(q[r]) - std::real(p[r] * std::conj(pi[r]) + q[r] * std::conj(qi[r])));
        }
}

// forces.force_all / torque_all: cpp/src/forces.cpp:139-171 (OpenMP per particle).
void orc_force_all(int N, int rmax, const double* ps, const double* pi, double k, double eps_b, double* F) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) orc_force(rmax, ps + size_t(i) * 4 * rmax, pi + size_t(i) * 4 * rmax, k, eps_b, F + 3 * i);
}
void orc_torque_all(int N, int rmax, const double* ps, const double* pi, double k, double eps_b, double* T) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) orc_torque(rmax, ps + size_t(i) * 4 * rmax, pi + size_t(i) * 4 * rmax, k, eps_b, T + 3 * i);
}

// vsh_functions.Emn: cpp/src/vsh_functions.cpp:56-58.  out = {re, im}.
void orc_Emn(int m, int n, double* out) {
    cd e = Emn_fn(m, n);
    out[0] = e.real();
    out[1] = e.imag();
}

// vsh_functions.vsh_electric / vsh_magnetic: cpp/src/vsh_functions.cpp:60-98.  out = 3 complex.
void orc_vsh_electric(int n, int m, int mode, double rad, double theta, double phi, double k, double* out) {
    vsh_electric(n, m, mode, rad, theta, phi, k, reinterpret_cast<cd*>(out));
}
void orc_vsh_magnetic(int n, int m, int mode, double rad, double theta, double phi, double k, double* out) {
    vsh_magnetic(n, m, mode, rad, theta, phi, k, reinterpret_cast<cd*>(out));
}

// vsh_functions.expand_E_cluster: cpp/src/vsh_functions.cpp:100-143.
// pos [N,3], p [N, 2*rmax] c128, pts x/y/z [Npts] -> E [Npts, 3] c128.
void orc_expand_E_cluster(int N, int rmax, const double* pos, const double* pexp, int mode, int Npts, const double* x,
                          const double* y, const double* z, double k, double* Eout) {
    const cd* P = reinterpret_cast<const cd*>(pexp);
    cd* E = reinterpret_cast<cd*>(Eout);
    int lmax = rmax_to_lmax(rmax);
    cd factor = (mode == 0) ? cd(0, 1) : cd(0, -1);
#pragma omp parallel for schedule(dynamic, 16)
    for (int j = 0; j < Npts; j++) {
        cd acc[3] = {0, 0, 0};
        for (int i = 0; i < N; i++) {
            double xr = x[j] - pos[3 * i], yr = y[j] - pos[3 * i + 1], zr = z[j] - pos[3 * i + 2];
            double rad = std::sqrt(xr * xr + yr * yr + zr * zr);
            double th = std::acos(zr / rad), ph = std::atan2(yr, xr);
            for (int n = 1; n <= lmax; n++)
                for (int m = -n; m <= n; m++) {
                    cd em = Emn_fn(m, n);
                    int idx = n * (n + 2) - n + m - 1;
                    cd Es[3], Ec[3];
                    vsh_electric(n, m, mode, rad, th, ph, k, Es);
                    sph_to_cart_vec(Es, th, ph, Ec);
                    for (int c = 0; c < 3; c++) acc[c] += -factor * em * P[size_t(i) * 2 * rmax + idx] * Ec[c];
                    vsh_magnetic(n, m, mode, rad, th, ph, k, Es);
                    sph_to_cart_vec(Es, th, ph, Ec);
                    for (int c = 0; c < 3; c++) acc[c] += -factor * em * P[size_t(i) * 2 * rmax + idx + rmax] * Ec[c];
                }
        }
        for (int c = 0; c < 3; c++) E[size_t(j) * 3 + c] = acc[c];
    }
}

// decomposition.integrate_phase: cpp/src/decomposition.cpp:29-66 (trapezoid rule
// over theta then phi, trapz/trapz_2d :7-27).  rhat [3,Nx,Ny], p0 [2,rmax,Nx,Ny] c128.
void orc_integrate_phase(const double* rhat, const double* origin, double k, int rmax, int Nx, const double* theta,
                         int Ny, const double* phi, const double* p0f, double* out) {
    const cd* p0 = reinterpret_cast<const cd*>(p0f);
    cd* p = reinterpret_cast<cd*>(out);
    std::vector<cd> ph(size_t(Nx) * Ny);
    for (int i = 0; i < Nx; i++)
        for (int j = 0; j < Ny; j++) {
            size_t e = size_t(i) * Ny + j;
            double phase = -k * (rhat[e] * origin[0] + rhat[size_t(Nx) * Ny + e] * origin[1] +
                                 rhat[2 * size_t(Nx) * Ny + e] * origin[2]);
            ph[e] = std::exp(cd(0, phase));
        }
    auto trap = [](const double* xs, const cd* ys, int n, int stride) {
        cd s = 0;
        for (int i = 1; i < n; i++) s += (ys[size_t(i) * stride] + ys[size_t(i - 1) * stride]) * (xs[i] - xs[i - 1]) / 2.0;
        return s;
    };
    std::vector<cd> M(size_t(Nx) * Ny), zc(Ny);
    for (int a = 0; a < 2; a++)
        for (int r = 0; r < rmax; r++) {
            const cd* src = p0 + (size_t(a) * rmax + r) * Nx * Ny;
            for (size_t e = 0; e < size_t(Nx) * Ny; e++) M[e] = src[e] * ph[e];
            for (int c = 0; c < Ny; c++) zc[c] = trap(theta, M.data() + c, Nx, Ny);
            p[size_t(a) * rmax + r] = trap(phi, zc.data(), Ny, 1);
        }
}

}   // extern "C"
