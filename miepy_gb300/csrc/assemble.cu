// K1: translation-matrix assembler (replaces sphere_aggregate_tmatrix,
// cpp/src/interactions.cpp:370-415, and vsh_translation_insert_pair (Mie overload),
// cpp/src/vsh_translation.cpp:161-237).
//
// One CTA per group of PB particle pairs (grid-stride over the groups of all
// clusters of a batch).  Per group, in shared memory:
//   1. h_p(kr) by the upward j/y recurrence of spherical_hn_recursion
//      (cpp/src/special.cpp:90-111), one thread per pair; P_p^mu(cos theta) (no
//      Condon-Shortley phase, GSL_SF_LEGENDRE_NONE convention), one thread per
//      (pair, mu); e^{i mu phi} by powering e^{i phi}.  The angles enter only
//      through cos/sin of theta and phi, taken directly from the separation vector;
//   2. G[p][mu] = P_p^mu h_p e^{i mu phi} for all (p, |mu| <= p), in FP64.
// The packed double-float (mixed) path instead takes steps 1-2 from a separate pass,
// k_asm_gtab (below), with 32 pairs per CTA, and loads the group's G tables;
// then per pair, software-pipelined over the group (or, at lmax <= 5, for the whole
// group at once):
//   3. one thread per canonical tuple: A_t, B_t as real x complex FMA sums over
//      the per-lmax coefficient table (tables.cu);
//   4. coalesced block write: every entry of the B x B block looks up its tuple and
//      sign in the element map.  Packed output writes the (i, j) block only, without
//      Mie factors, in complex128 and/or complex64 hi / lo (sign flips are bit
//      operations).  Dense output writes the (i, j) and (j, i) blocks of the
//      reference's D x D matrix with the Mie factors of the column particle.

#include <algorithm>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace {

constexpr int kAsmThreads = 256;
constexpr int kAsmWideThreads = 512;

// 1/k for the Legendre recurrence (k = q - mu <= 2*lmax + 1)
__constant__ double c_inv_int[2 * GB_LMAX_MAX + 4] = {
    0.0, 1.0, 1.0 / 2, 1.0 / 3, 1.0 / 4, 1.0 / 5, 1.0 / 6, 1.0 / 7, 1.0 / 8, 1.0 / 9, 1.0 / 10, 1.0 / 11,
    1.0 / 12, 1.0 / 13, 1.0 / 14, 1.0 / 15, 1.0 / 16, 1.0 / 17, 1.0 / 18, 1.0 / 19, 1.0 / 20, 1.0 / 21,
    1.0 / 22, 1.0 / 23};

// Shared-memory layout of one CTA: the special functions of a group of PB pairs
// (launch-wide strides PM = 2 Lmax + 2 orders, MU = 4 Lmax + 1 azimuthal orders),
// then the tuple values of NB pairs: two (the one being written and the next) where
// they fit, one at large lmax, where two would cost occupancy.
struct AsmSmem {
    int PM, MU, M, PB, NB;
    size_t off_geo, off_h, off_P, off_e, off_G, off_Gs, off_T, off_Tf, off_Tl, total;
};

__host__ __device__ inline AsmSmem asm_layout(int L, int M, int PB, bool fp64_sums, bool want64, int NB,
                                               bool split = false, bool gsum = false) {
    AsmSmem s;
    s.PM = 2 * L + 2;
    s.MU = 4 * L + 1;
    s.M = M;
    s.PB = PB;
    s.NB = NB;
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t r = o; o += (bytes + 15) & ~size_t(15); return r; };
    // the double-float path reads its G tables (k_asm_gtab) and needs no special functions
    const size_t sf = fp64_sums ? 1 : 0;
    s.off_geo = take(sf * sizeof(double) * 8 * PB);
    s.off_h = take(sf * sizeof(double2) * s.PM * PB);
    s.off_e = take(sf * sizeof(double2) * s.MU * PB);
    s.off_P = take(sf * sizeof(double) * s.PM * s.PM * PB);
    s.off_G = take(16 * (size_t)s.PM * s.MU * PB);          // double2 (FP64 sums) or float4 (double-float)
    s.off_Gs = take(gsum ? sizeof(double2) * s.PM * s.MU : 0);   // lattice sums: the group's running G sum
    const size_t kinds = split ? 1 : 2;   // (A, B) per tuple, or one of them at a time
    s.off_T = take(fp64_sums ? sizeof(double2) * kinds * NB * M : 0);   // NB buffers of tuple values
    s.off_Tf = take(want64 ? sizeof(float2) * kinds * NB * M : 0);
    s.off_Tl = take(want64 ? sizeof(float2) * kinds * NB * M : 0);
    s.total = o;
    return s;
}

__device__ __forceinline__ double2 mul_ipow(double2 z, int k) {
    switch (k & 3) {
        case 0: return z;
        case 1: return make_double2(-z.y, z.x);
        case 2: return make_double2(-z.x, -z.y);
        default: return make_double2(z.y, -z.x);
    }
}
__device__ __forceinline__ float2 mul_ipowf(float2 z, int k) {
    switch (k & 3) {
        case 0: return z;
        case 1: return make_float2(-z.y, z.x);
        case 2: return make_float2(-z.x, -z.y);
        default: return make_float2(z.y, -z.x);
    }
}
__device__ __forceinline__ float2 bcf(float v) { return make_float2(v, v); }

// (sh, sl) += (ch + cl) * (g.hi + g.lo): double-float real x complex multiply-add
// on the FP32 pipes (packed f32x2), with nch = -ch given.  pn = RN(-ch gh) is the
// negated hi*hi product, fma(ch, gh, pn) its exact error; cross terms and the TwoSum
// error of sh + p = sh - pn go to the low word.  Written with subtractions so that
// no operand needs a sign flip.
__device__ __forceinline__ void df_rc_fma(float2& sh, float2& sl, float ch, float nch, float cl, float4 g) {
    const float2 gh = make_float2(g.x, g.y), gl = make_float2(g.z, g.w);
    const float2 pn = __fmul2_rn(bcf(nch), gh);
    float2 e = __ffma2_rn(bcf(ch), gh, pn);
    e = __ffma2_rn(bcf(ch), gl, e);
    e = __ffma2_rn(bcf(cl), gh, e);
    const float2 t = fsub2(sh, pn);
    const float2 bb = fsub2(t, sh);
    const float2 err = fsub2(fsub2(sh, fsub2(t, bb)), __fadd2_rn(pn, bb));   // (sh - (t - bb)) + (p - bb)
    sh = t;
    sl = __fadd2_rn(sl, __fadd2_rn(err, e));
}

// ------------------------------------------------------------ double-float --
// Double-float (h + l, |l| <= ulp(h)/2) arithmetic on the FP32 pipe for the
// special functions of the mixed path (GB300 issues an FP64 warp instruction about
// once per 64 cycles per SM sub-partition).  Products by the FMA error term,
// sums by TwoSum (Joldes, Muller, Popescu, ACM TOMS 44 (2017): DWTimesDW1 and
// AccurateDWPlusDW), relative error a few 2^-48.
struct DF { float h, l; };
struct DFC { DF re, im; };
__device__ __forceinline__ DF fast2sum(float a, float b) {
    const float s = a + b;
    return DF{s, b - (s - a)};
}
__device__ __forceinline__ DF two_sum(float a, float b) {
    const float s = a + b, bb = s - a;
    return DF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF df_of(double v) {   // FP64 -> double-float (2 conversions, 1 subtraction)
    const float h = __double2float_rn(v);
    return DF{h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    DF s = two_sum(a.h, b.h);
    const DF t = two_sum(a.l, b.l);
    s = fast2sum(s.h, s.l + t.h);
    return fast2sum(s.h, s.l + t.l);
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }
__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return fast2sum(p, e);
}
__device__ __forceinline__ DF df_mulf(DF a, float b) {   // by a float (small integers are exact)
    const float p = a.h * b;
    float e = fmaf(a.h, b, -p);
    e = fmaf(a.l, b, e);
    return fast2sum(p, e);
}
__device__ __forceinline__ DF df_divf(DF a, float b) {   // by a float: the remainder of a rounded quotient is exact
    const float q1 = a.h / b;
    const float r = fmaf(-q1, b, a.h) + a.l;
    return fast2sum(q1, r / b);
}
__device__ __forceinline__ DFC dfc_mul(DFC a, DFC b) {
    return DFC{df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im))), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
__device__ __forceinline__ float4 dfc_pack(DFC z) { return make_float4(z.re.h, z.im.h, z.re.l, z.im.l); }
__device__ __forceinline__ DFC dfc_unpack(float4 v) { return DFC{DF{v.x, v.z}, DF{v.y, v.w}}; }

__device__ __forceinline__ int find_sys(const long long* base, int nsys, long long g) {
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Planar interface at height z with normal-incidence reflection coefficient r0
// (the reflection matrix of interactions.cpp:464-512): pairs run over all (i, j),
// the translation goes from particle j to the mirror image of particle i.
struct Refl {
    double z = 0;
    double2 r0 = {0, 0};
};

// Periodic lattice (sphere_aggregate_tmatrix_periodic, interactions.py:153-186):
// block (i, j) gains sum_c e^{-i k khat.c} A(pos_i - pos_j - c) mie_j over the
// lattice cells c (cells [ncell][3], device).  Groups hold PB cells of one ordered
// pair (gpp groups per pair); each group sums its phase-weighted tuple values in
// shared memory and adds its block to the dense output with one atomic add per
// entry.
struct Latt {
    const double* cells = nullptr;
    int ncell = 0;
    int gpp = 1;   // groups per ordered pair, each over cpg consecutive cells in chunks of PB
    int cpg = 1;
    double kx = 0, ky = 0, kz = 0;
};

// FP64_SUMS: tuple sums in FP64 (complex128 or dense output); otherwise in
// double-float on the FP32 pipes, straight to the complex64 hi / lo outputs.
// MODE 0: the aggregate T-matrix; 1: the dense reflection matrix (Refl); 2: the
// lattice sums of a periodic cluster, added to a dense output (Latt).
// Occupancy: the double-float (mixed) path fits five CTAs per SM in 48 registers
// without spills; the FP64 paths keep three (at five they spill).
// TS: whole-group phases on the packed double-float path (lmax <= 5, one tuple-value
// buffer per pair of the group, NB = PB): the group's (tuple, pair) sums are spread
// evenly over the threads, then every block of the group is written after one
// barrier, each element-map code read once for all of them.
// SPLIT (MODE 0, one pair per group, one buffer): where one pair's A and B tuple
// values do not fit in shared memory together (lmax 10), the A sums are formed and
// their block elements written, then the B sums and theirs.
// NT: threads per CTA.  The pair-by-pair double-float path runs 512 (kAsmWideThreads)
// where its tuple buffers leave room for at most two CTAs per SM (lmax >= 8), so
// that the SM keeps 32 warps instead of 16; the packed FP64 and dense paths likewise
// where one CTA fits per SM (lmax >= 8: 16 warps instead of 8).
template <bool DENSE, bool FP64_SUMS, int MODE = 0, bool TS = false, bool SPLIT = false, int NT = kAsmThreads>
__global__ void __launch_bounds__(NT, FP64_SUMS ? (NT > kAsmThreads ? 1 : 3) : (NT > kAsmThreads ? 2 : 5))
k_assemble(const gb::SysDev* __restrict__ sys, int nsys, const long long* __restrict__ grp_base, long long ngroups,
           int Lmax, int Mmax, int PB, int NB, const double* __restrict__ pos, const double2* __restrict__ mie,
           double2* __restrict__ out128, float2* __restrict__ out64, float2* __restrict__ out64lo, long long dense_ld,
           Refl refl = Refl(), Latt latt = Latt()) {
    constexpr bool REFL = MODE == 1, LATT = MODE == 2;
    static_assert(MODE == 0 || (DENSE && FP64_SUMS), "reflection and lattice sums are dense FP64 outputs");
    static_assert(!TS || (!DENSE && !FP64_SUMS && MODE == 0), "whole-group phases serve the packed double-float path");
    static_assert(!SPLIT || (MODE == 0 && !TS), "split sums serve the pair-by-pair path of the aggregate");
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const bool want64 = out64 != nullptr || out64lo != nullptr;
    const AsmSmem lay = asm_layout(Lmax, Mmax, PB, FP64_SUMS, want64 && !DENSE, NB, SPLIT, LATT);
    double* geo = reinterpret_cast<double*>(smem + lay.off_geo);        // [PB][8]
    double2* hh = reinterpret_cast<double2*>(smem + lay.off_h);         // [PB][PM]
    double2* eph = reinterpret_cast<double2*>(smem + lay.off_e);        // [PB][MU]
    double* Pl = reinterpret_cast<double*>(smem + lay.off_P);           // [PB][PM][PM]
    double2* G64 = reinterpret_cast<double2*>(smem + lay.off_G);        // [PB][PM][MU]
    double2* Gs = reinterpret_cast<double2*>(smem + lay.off_Gs);        // [PM][MU] (lattice sums)
    float4* G32 = reinterpret_cast<float4*>(smem + lay.off_G);
    double2* Tv = reinterpret_cast<double2*>(smem + lay.off_T);
    float2* Tf = reinterpret_cast<float2*>(smem + lay.off_Tf);
    float2* Tl = reinterpret_cast<float2*>(smem + lay.off_Tl);
    const int PMs = lay.PM, MUs = lay.MU;   // launch-wide strides
    for (long long g = blockIdx.x; g < ngroups; g += gridDim.x) {
        const int s = find_sys(grp_base, nsys, g);
        const gb::SysDev S = sys[s];
        const int L = S.lmax, B = S.B, N = S.N;
        const int PM = 2 * L + 2, MU = 4 * L + 1;
        const long long gl = g - grp_base[s];
        const long long p_first = gl * (long long)PB;
        long long lat_pair = 0;   // lattice: the ordered pair (i, j) = (lat_pair / N, lat_pair % N) ...
        int lat_c0 = 0;           // ... the first cell of the chunk ...
        int lat_end = 0;          // ... and the end of the group's cells
        int np;
        if constexpr (LATT) {
            lat_pair = gl / latt.gpp;
            lat_c0 = (int)(gl - lat_pair * latt.gpp) * latt.cpg;
            lat_end = min(lat_c0 + latt.cpg, latt.ncell);
            np = min(PB, lat_end - lat_c0);
        } else {
            const long long Ptot = REFL ? (long long)N * N : S.P;   // all ordered pairs for the reflection
            np = (int)min((long long)PB, Ptot - p_first);
        }

        // lattice sums: phases 1a-1c for every chunk of PB cells of the group, each
        // chunk's phase-weighted G tables added to the running sum Gs; other modes run
        // them once
        for (bool first = true;; first = false) {
        // ---- phase 1a (FP64 paths; the double-float path reads the G tables of
        // k_asm_gtab): one thread per pair: geometry, then h_p(kr) by the upward
        // j/y recurrence of spherical_hn_recursion (cpp/src/special.cpp:90-111).  The
        // angles enter only through cos/sin of theta and phi, straight from the
        // separation vector (the reference goes through acos/atan2 and back).
        if (FP64_SUMS && tid < np) {
            int i, j;
            double lx = 0.0, ly = 0.0, lz = 0.0;   // lattice: the cell that holds the image of particle j
            if (LATT) {
                i = (int)(lat_pair / N);
                j = (int)(lat_pair % N);
                const double* c = latt.cells + 3 * (long long)(lat_c0 + tid);
                lx = c[0];
                ly = c[1];
                lz = c[2];
            } else if (REFL) {
                i = (int)((p_first + tid) / N);
                j = (int)((p_first + tid) % N);
            } else {
                pair_ij(p_first + tid, N, i, j);
            }
            const double* pi_ = pos + S.pos_off + 3 * (long long)i;
            const double* pj_ = pos + S.pos_off + 3 * (long long)j;
            const double zi = REFL ? 2.0 * refl.z - pi_[2] : pi_[2];   // mirror image of particle i
            const double dx = pi_[0] - (pj_[0] + lx), dy = pi_[1] - (pj_[1] + ly), dz = zi - (pj_[2] + lz);
            const double rho2 = dx * dx + dy * dy;
            const double rad = sqrt(rho2 + dz * dz);
            const double inv_r = 1.0 / rad;
            const double rho = sqrt(rho2);
            double cphi = 1.0, sphi = 0.0;                  // phi = atan2(dy, dx) = 0 on the z axis
            if (rho2 > 0.0) {
                const double inv_rho = 1.0 / rho;
                cphi = dx * inv_rho;
                sphi = dy * inv_rho;
            }
            double* ge = geo + 8 * tid;
            ge[0] = dz * inv_r;                             // cos(theta)
            ge[1] = rho * inv_r;                            // sin(theta) >= 0
            ge[2] = cphi;
            ge[3] = sphi;
            if (LATT) {   // the Bloch phase e^{-i k khat.c} of the cell
                double sp, cp;
                sincos(-S.k * (latt.kx * lx + latt.ky * ly + latt.kz * lz), &sp, &cp);
                ge[4] = cp;
                ge[5] = sp;
            }
            const double z = S.k * rad;
            const double inv_z = 1.0 / z;
            double sz, cz;
            sincos(z, &sz, &cz);
            double j0 = sz * inv_z, y0 = -cz * inv_z;
            double j1 = j0 * inv_z + y0, y1 = y0 * inv_z - j0;
            double2* h = hh + PMs * tid;
            h[0] = make_double2(j0, y0);
            h[1] = make_double2(j1, y1);
            for (int q = 2; q < PM; q++) {
                const double f = (2 * q - 1) * inv_z;
                const double jn = f * j1 - j0;
                const double yn = f * y1 - y0;
                j0 = j1; j1 = jn; y0 = y1; y1 = yn;
                h[q] = make_double2(jn, yn);
            }
        }
        if constexpr (FP64_SUMS) __syncthreads();
        // ---- phase 1b: P_q^mu(cos theta) (no Condon-Shortley phase), one thread per
        // (pair, mu); e^{i mu phi} by binary powering, one thread per (pair, mu >= 0).
        // The double-float path instead loads the group's G tables.
        if constexpr (FP64_SUMS) {
            for (int it = tid; it < np * PM; it += NT) {
                const int pp = it / PM, mu = it % PM;
                const double x = geo[8 * pp], u = geo[8 * pp + 1];
                double* P = Pl + (size_t)PMs * PMs * pp;
                double pmm = 1.0;
                for (int kk = 1; kk <= mu; kk++) pmm *= (2 * kk - 1) * u;
                P[mu * PMs + mu] = pmm;
                if (mu + 1 < PM) {
                    double pa = pmm, pb = x * (2 * mu + 1) * pmm;
                    P[(mu + 1) * PMs + mu] = pb;
                    for (int q = mu + 2; q < PM; q++) {
                        const double pc = ((2 * q - 1) * x * pb - (q + mu - 1) * pa) * c_inv_int[q - mu];
                        P[q * PMs + mu] = pc;
                        pa = pb;
                        pb = pc;
                    }
                }
            }
            for (int it = tid; it < np * (2 * L + 1); it += NT) {
                const int pp = it / (2 * L + 1), mu = it % (2 * L + 1);
                int e = mu;
                double2 acc = make_double2(1.0, 0.0), base = make_double2(geo[8 * pp + 2], geo[8 * pp + 3]);
                while (e) {
                    if (e & 1) acc = cmul(acc, base);
                    base = cmul(base, base);
                    e >>= 1;
                }
                eph[MUs * pp + 2 * L + mu] = acc;
                eph[MUs * pp + 2 * L - mu] = make_double2(acc.x, -acc.y);
            }
        } else {
            // the group's G tables, written by k_asm_gtab at the start of each pair's
            // own block in the output plane (entry p^2 + p + mu for |mu| <= p, as (re.hi,
            // im.hi), (re.lo, im.lo)); zeros where |mu| > p.  Read through L2 (the
            // kernel overwrites these words later, after the barrier that ends the sums).
            const float2* gsrc = out64lo ? out64lo : out64;
            const long long BBl = (long long)B * B;
            for (int it = tid; it < np * PM * MU; it += NT) {
                const int pp = it / (PM * MU), rem = it - pp * (PM * MU);
                const int q = rem / MU, mi = rem - q * MU, mu = mi - 2 * L;
                float4 gv = make_float4(0.f, 0.f, 0.f, 0.f);
                if ((mu < 0 ? -mu : mu) <= q) {
                    const float2* src = gsrc + S.mat_off + (p_first + pp) * BBl + 2 * (q * q + q + mu);
                    const float2 a = __ldcg(src), b = __ldcg(src + 1);
                    gv = make_float4(a.x, a.y, b.x, b.y);
                }
                G32[(size_t)PMs * MUs * pp + (size_t)q * MUs + mi] = gv;
            }
        }
        __syncthreads();
        // ---- phase 1c (FP64 paths): G[p][mu] = P_p^mu h_p e^{i mu phi} (negative mu
        // through the (-1)^mu (p-mu)!/(p+mu)! ratio)
        if constexpr (FP64_SUMS) {
            for (int it = tid; it < np * PM * MU; it += NT) {
                const int pp = it / (PM * MU), rem = it % (PM * MU);
                const int q = rem / MU, mi = rem % MU, mu = mi - 2 * L, am = mu < 0 ? -mu : mu;
                const size_t gi = (size_t)PMs * MUs * pp + (size_t)q * MUs + mi;
                double2 gval = make_double2(0.0, 0.0);
                if (am <= q) {
                    double P = Pl[(size_t)PMs * PMs * pp + q * PMs + am];
                    if (mu < 0) P *= S.neg_ratio[q * PM + am];
                    const double2 he = cmul(hh[PMs * pp + q], eph[MUs * pp + mi]);
                    gval = make_double2(P * he.x, P * he.y);
                }
                G64[gi] = gval;
            }
            __syncthreads();
        }
        if constexpr (LATT) {
            // the chunk's cells into the running sum, G = sum_c e^{-i k khat.c} G_c (the
            // tuple sums are linear in G), each thread its own entries
            for (int qm = tid; qm < PM * MU; qm += NT) {
                const int q = qm / MU, mi = qm - q * MU;
                double2 acc = first ? make_double2(0.0, 0.0) : Gs[(size_t)q * MUs + mi];
                for (int pp = 0; pp < np; pp++) {
                    const double2 ph = make_double2(geo[8 * pp + 4], geo[8 * pp + 5]);
                    const double2 gv = cmul(ph, G64[(size_t)PMs * MUs * pp + (size_t)q * MUs + mi]);
                    acc.x += gv.x;
                    acc.y += gv.y;
                }
                Gs[(size_t)q * MUs + mi] = acc;
            }
            __syncthreads();   // before the next chunk rewrites the cells' tables
            lat_c0 += PB;
            if (lat_c0 >= lat_end) break;
            np = min(PB, lat_end - lat_c0);
        } else {
            (void)first;
            break;
        }
        }

        // ---- phases 2 and 3, software-pipelined over the group's pairs: each thread
        // writes pair pp's block (phase 3) and then forms the tuple values of pair
        // pp + 1 (phase 2) into the other buffer, one barrier per pair.
        const int Mb = lay.M;   // tuple-buffer stride (launch-wide)
        constexpr int KINDS = SPLIT ? 1 : 2;
        // slot of tuple t's value of kind k (0: A, 1: B); kind 2 below means both
        auto slot = [](int t, int k) { return SPLIT ? t : 2 * t + k; };
        auto tuples = [&](int pp, int buf, int kind) {
            const size_t gbase = (size_t)PMs * MUs * pp;
            double2* tv = Tv + (size_t)buf * KINDS * Mb;
            float2* tf = Tf + (size_t)buf * KINDS * Mb;
            float2* tl = Tl + (size_t)buf * KINDS * Mb;
            const bool wantA = kind != 1, wantB = kind != 0;
            const int Q = L + 1;
            for (int it = tid; it < S.M; it += NT) {
                int t, mi, nv;
                int2 qq;
                if constexpr (FP64_SUMS) {
                    t = it;
                    const int4 e = S.nmvu[t];
                    qq = S.qab[t];
                    mi = (e.w - e.y) + 2 * L;
                    nv = e.x + e.z;
                } else {   // sorted order: the lanes of a warp run sums of equal length
                    const int4 f = S.tinfo[it];
                    t = f.x;
                    nv = f.y;
                    mi = f.z + 2 * L;
                    qq = make_int2(f.w & 255, f.w >> 8);
                }
                if constexpr (FP64_SUMS) {
                    const double* ca = S.cA + (size_t)t * Q;
                    const double* cb = S.cB + (size_t)t * Q;
                    double2 sa = make_double2(0.0, 0.0), sb = make_double2(0.0, 0.0);
                    for (int q = 0; wantA && q <= qq.x; q++) {
                        const double c = ca[q];
                        const double2 gv = G64[gbase + (size_t)(nv - 2 * q) * MUs + mi];
                        sa.x = fma(c, gv.x, sa.x);
                        sa.y = fma(c, gv.y, sa.y);
                    }
                    for (int q = 1; wantB && q <= qq.y; q++) {
                        const double c = cb[q];
                        const double2 gv = G64[gbase + (size_t)(nv - 2 * q + 1) * MUs + mi];
                        sb.x = fma(c, gv.x, sb.x);
                        sb.y = fma(c, gv.y, sb.y);
                    }
                    const double2 At = mul_ipow(sa, nv), Bt = mul_ipow(sb, nv + 1);
                    if (wantA) tv[slot(t, 0)] = At;
                    if (wantB) tv[slot(t, 1)] = Bt;
                    if (!DENSE && want64) {
                        const float2 ah = make_float2(__double2float_rn(At.x), __double2float_rn(At.y));
                        const float2 bh = make_float2(__double2float_rn(Bt.x), __double2float_rn(Bt.y));
                        if (wantA) {
                            tf[slot(t, 0)] = ah;
                            tl[slot(t, 0)] = make_float2(__double2float_rn(At.x - (double)ah.x),
                                                         __double2float_rn(At.y - (double)ah.y));
                        }
                        if (wantB) {
                            tf[slot(t, 1)] = bh;
                            tl[slot(t, 1)] = make_float2(__double2float_rn(Bt.x - (double)bh.x),
                                                         __double2float_rn(Bt.y - (double)bh.y));
                        }
                    }
                } else {
                    const float2* ca = S.cA2s + (size_t)it * Q;
                    const float2* cb = S.cB2s + (size_t)it * Q;
                    float2 ah = make_float2(0.f, 0.f), al = ah, bh = ah, bl = ah;
                    // the A and B sums interleaved: two independent double-float chains
                    const int qa = qq.x, qb = qq.y, qm = qa > qb ? qa : qb;
                    for (int q = 0; q <= qm; q++) {
                        if (wantA && q <= qa) {
                            const float2 c = ca[q];
                            df_rc_fma(ah, al, c.x, -c.x, c.y, G32[gbase + (size_t)(nv - 2 * q) * MUs + mi]);
                        }
                        if (wantB && q >= 1 && q <= qb) {
                            const float2 c = cb[q];
                            df_rc_fma(bh, bl, c.x, -c.x, c.y, G32[gbase + (size_t)(nv - 2 * q + 1) * MUs + mi]);
                        }
                    }
                    // normalise (Fast2Sum): hi = fl(h + l), lo = l - (hi - h)
                    const float2 a1 = __fadd2_rn(ah, al), b1 = __fadd2_rn(bh, bl);
                    const float2 a2 = fsub2(al, fsub2(a1, ah));
                    const float2 b2 = fsub2(bl, fsub2(b1, bh));
                    if (wantA) {
                        tf[slot(t, 0)] = mul_ipowf(a1, nv);
                        tl[slot(t, 0)] = mul_ipowf(a2, nv);
                    }
                    if (wantB) {
                        tf[slot(t, 1)] = mul_ipowf(b1, nv + 1);
                        tl[slot(t, 1)] = mul_ipowf(b2, nv + 1);
                    }
                }
            }
        };
        // the block elements of kind `kind` (2: all); element code (t << 2) | (is_B << 1)
        // | negate, its value at slot(t, is_B)
        auto write_block = [&](int pp, int buf, int kind) {
            const long long p = p_first + pp;
            const double2* tv = Tv + (size_t)buf * KINDS * Mb;
            const float2* tf = Tf + (size_t)buf * KINDS * Mb;
            const float2* tl = Tl + (size_t)buf * KINDS * Mb;
            const int BB = B * B;
            auto at = [&](int code) { return slot(code >> 2, (code >> 1) & 1); };
            auto skip = [&](int code) { return SPLIT && ((code >> 1) & 1) != kind; };
            if (!DENSE) {
                const long long base = S.mat_off + p * (long long)BB;
                if (!SPLIT && !FP64_SUMS && (base & 1) == 0 &&
                    ((reinterpret_cast<size_t>(out64) | reinterpret_cast<size_t>(out64lo)) & 15) == 0) {
                    // two elements per thread, 16-byte streaming stores (BB is even)
                    for (int e2 = tid; e2 < BB / 2; e2 += NT) {
                        const int2 code = __ldg(reinterpret_cast<const int2*>(S.elem_map) + e2);
                        const unsigned n0 = code.x & 1, n1 = code.y & 1;
                        const int t0 = code.x >> 1, t1 = code.y >> 1;
                        if (out64) {
                            const float2 a = tf[t0], b = tf[t1];
                            __stcs(reinterpret_cast<float4*>(out64 + base) + e2,
                                   make_float4(flipf(a.x, n0), flipf(a.y, n0), flipf(b.x, n1), flipf(b.y, n1)));
                        }
                        if (out64lo) {
                            const float2 a = tl[t0], b = tl[t1];
                            __stcs(reinterpret_cast<float4*>(out64lo + base) + e2,
                                   make_float4(flipf(a.x, n0), flipf(a.y, n0), flipf(b.x, n1), flipf(b.y, n1)));
                        }
                    }
                    return;
                }
                for (int e = tid; e < BB; e += NT) {
                    const int code = __ldg(S.elem_map + e);
                    if (skip(code)) continue;
                    const unsigned neg = code & 1;
                    if (FP64_SUMS && out128) {
                        const double2 v = tv[at(code)];
                        out128[base + e] = make_double2(flipd(v.x, neg), flipd(v.y, neg));
                    }
                    if (out64) {
                        const float2 v = tf[at(code)];
                        out64[base + e] = make_float2(flipf(v.x, neg), flipf(v.y, neg));
                    }
                    if (out64lo) {
                        const float2 v = tl[at(code)];
                        out64lo[base + e] = make_float2(flipf(v.x, neg), flipf(v.y, neg));
                    }
                }
            } else if (REFL) {
                // block (i, j) only: -r0 (-1)^(m+n+a+1) transfer mie(j, b, v)
                const int i = (int)(p / N), j = (int)(p % N);
                const double2* mj_ = mie + (long long)j * 2 * L;
                const int rmx = B / 2;
                for (int e = tid; e < BB; e += NT) {
                    const int R = e / B, C = e % B;
                    const int code = __ldg(S.elem_map + e);
                    const unsigned neg = code & 1;
                    double2 v = tv[code >> 1];
                    v = make_double2(flipd(v.x, neg), flipd(v.y, neg));
                    const int a = R / rmx, r = R - a * rmx;
                    int n = 1;   // r = n(n+2) - n + m - 1 = n^2 + n + m - 1, |m| <= n: n = floor(sqrt(r + 1))
                    while ((n + 1) * (n + 1) <= r + 1) n++;
                    const int m = r + 1 - n * n - n;
                    const double2 w = cmul(v, mj_[__ldg(S.miecol + C)]);
                    const unsigned sgn = (unsigned)((m + n + a + 1) & 1) ^ 1u;   // -(-1)^(m+n+a+1)
                    out128[((long long)i * B + R) * dense_ld + (long long)j * B + C] =
                        cmul(make_double2(flipd(refl.r0.x, sgn), flipd(refl.r0.y, sgn)), w);
                }
            } else {
                int i, j;
                pair_ij(p, N, i, j);
                const double2* mi_ = mie + (long long)i * 2 * L;
                const double2* mj_ = mie + (long long)j * 2 * L;
                for (int e = tid; e < BB; e += NT) {
                    const int R = e / B, C = e % B;
                    const int code = __ldg(S.elem_map + e);
                    if (skip(code)) continue;
                    const unsigned neg = code & 1;
                    double2 v = tv[at(code)];
                    v = make_double2(flipd(v.x, neg), flipd(v.y, neg));
                    const int col = __ldg(S.miecol + C);
                    const double2 vij = cmul(v, mj_[col]);
                    const unsigned sneg = ((unsigned)__ldg(S.rowinfo + R) >> 30 ^ (unsigned)__ldg(S.rowinfo + C) >> 30) & 1;
                    double2 vji = cmul(v, mi_[col]);
                    vji = make_double2(flipd(vji.x, sneg), flipd(vji.y, sneg));
                    out128[((long long)i * B + R) * dense_ld + (long long)j * B + C] = vij;
                    out128[((long long)j * B + R) * dense_ld + (long long)i * B + C] = vji;
                }
            }
        };
        if constexpr (LATT) {
            // the tuple values once from the group's summed G table (into the first
            // cell's slot), then the group's share of block (i, j), times mie(j, b, v),
            // added to the dense output
            for (int qm = tid; qm < PM * MU; qm += NT) {
                const int q = qm / MU, mi = qm - q * MU;
                G64[(size_t)q * MUs + mi] = Gs[(size_t)q * MUs + mi];
            }
            __syncthreads();
            tuples(0, 0, 2);
            __syncthreads();
            const int i = (int)(lat_pair / N), j = (int)(lat_pair % N);
            const double2* mj_ = mie + (long long)j * 2 * L;
            for (int e = tid; e < B * B; e += NT) {
                const int R = e / B, C = e % B;
                const int code = __ldg(S.elem_map + e);
                const unsigned neg = code & 1;
                double2 v = Tv[code >> 1];
                v = make_double2(flipd(v.x, neg), flipd(v.y, neg));
                const double2 w = cmul(v, mj_[__ldg(S.miecol + C)]);
                double* o = reinterpret_cast<double*>(out128 + ((long long)i * B + R) * dense_ld + (long long)j * B + C);
                atomicAdd(o, w.x);
                atomicAdd(o + 1, w.y);
            }
            __syncthreads();   // the next group rewrites the tables and the sums
            continue;
        }
        if constexpr (TS) {
            // the group's (tuple, pair) sums spread evenly over the threads: item it is
            // tuple it % M of pair it / M
            // (tuples in the sorted order of S.tinfo: the lanes of a warp run sums of
            // equal length)
            const int M = S.M;
            int i = tid, pp = 0;
            while (i >= M) { i -= M; pp++; }
            for (; pp < np;) {
                const int4 f = S.tinfo[i];
                const int t = f.x, nv = f.y, mi = f.z + 2 * L, qa = f.w & 255, qb = f.w >> 8;
                const int qm = qa > qb ? qa : qb;
                const float2* ca = S.cA2s + (size_t)i * (L + 1);
                const float2* cb = S.cB2s + (size_t)i * (L + 1);
                const float4* gp = G32 + (size_t)PMs * MUs * pp + (size_t)nv * MUs + mi;
                float2 ah = make_float2(0.f, 0.f), al = ah, bh = ah, bl = ah;
#pragma unroll
                for (int q = 0; q < 6; q++) {   // lmax <= 5: at most 6 terms per sum
                    if (q > qm) break;
                    if (q <= qa) {
                        const float2 c = ca[q];
                        df_rc_fma(ah, al, c.x, -c.x, c.y, gp[-2 * q * MUs]);
                    }
                    if (q >= 1 && q <= qb) {
                        const float2 c = cb[q];
                        df_rc_fma(bh, bl, c.x, -c.x, c.y, gp[(1 - 2 * q) * MUs]);
                    }
                }
                const float2 a1 = __fadd2_rn(ah, al), b1 = __fadd2_rn(bh, bl);
                const float2 a2 = fsub2(al, fsub2(a1, ah));
                const float2 b2 = fsub2(bl, fsub2(b1, bh));
                float2* tf = Tf + (size_t)pp * 2 * Mb;
                float2* tl = Tl + (size_t)pp * 2 * Mb;
                tf[2 * t] = mul_ipowf(a1, nv);
                tf[2 * t + 1] = mul_ipowf(b1, nv + 1);
                tl[2 * t] = mul_ipowf(a2, nv);
                tl[2 * t + 1] = mul_ipowf(b2, nv + 1);
                i += NT;
                while (i >= M) { i -= M; pp++; }
            }
            __syncthreads();
            const int BB = B * B;   // even: B = 2 rmax
            if ((S.mat_off & 1) == 0 && ((reinterpret_cast<size_t>(out64) | reinterpret_cast<size_t>(out64lo)) & 15) == 0) {
                // two elements per thread and 16-byte streaming stores (the blocks are
                // read by the next kernels from HBM: more than L2 holds)
                for (int e2 = tid; e2 < BB / 2; e2 += NT) {
                    const int2 code = __ldg(reinterpret_cast<const int2*>(S.elem_map) + e2);
                    const unsigned n0 = code.x & 1, n1 = code.y & 1;
                    const int t0 = code.x >> 1, t1 = code.y >> 1;
                    for (int pp = 0; pp < np; pp++) {
                        const long long at = S.mat_off + (p_first + pp) * (long long)BB + 2 * e2;
                        if (out64) {
                            const float2 a = Tf[(size_t)pp * 2 * Mb + t0], b = Tf[(size_t)pp * 2 * Mb + t1];
                            __stcs(reinterpret_cast<float4*>(out64 + at),
                                   make_float4(flipf(a.x, n0), flipf(a.y, n0), flipf(b.x, n1), flipf(b.y, n1)));
                        }
                        if (out64lo) {
                            const float2 a = Tl[(size_t)pp * 2 * Mb + t0], b = Tl[(size_t)pp * 2 * Mb + t1];
                            __stcs(reinterpret_cast<float4*>(out64lo + at),
                                   make_float4(flipf(a.x, n0), flipf(a.y, n0), flipf(b.x, n1), flipf(b.y, n1)));
                        }
                    }
                }
                __syncthreads();   // before the next group rewrites the tables and the buffers
                continue;
            }
            for (int el = tid; el < BB; el += NT) {
                const int code = __ldg(S.elem_map + el);
                const unsigned neg = code & 1;
                const int ti = code >> 1;
                for (int pp = 0; pp < np; pp++) {
                    const long long at = S.mat_off + (p_first + pp) * (long long)BB + el;
                    if (out64) {
                        const float2 v = Tf[(size_t)pp * 2 * Mb + ti];
                        out64[at] = make_float2(flipf(v.x, neg), flipf(v.y, neg));
                    }
                    if (out64lo) {
                        const float2 v = Tl[(size_t)pp * 2 * Mb + ti];
                        out64lo[at] = make_float2(flipf(v.x, neg), flipf(v.y, neg));
                    }
                }
            }
            __syncthreads();   // before the next group rewrites the tables and the buffers
            continue;
        }
        if constexpr (SPLIT) {   // one pair, one buffer: the A values and elements, then the B ones
            for (int pp = 0; pp < np; pp++)
                for (int kind = 0; kind < 2; kind++) {
                    tuples(pp, 0, kind);
                    __syncthreads();
                    write_block(pp, 0, kind);
                    __syncthreads();
                }
            continue;
        }
        tuples(0, 0, 2);
        __syncthreads();
        for (int pp = 0; pp < np; pp++) {
            write_block(pp, NB == 2 ? (pp & 1) : 0, 2);   // reads buffer pp & 1 (or the one buffer)
            if (pp + 1 < np) {
                if (NB == 1) __syncthreads();   // one buffer: every read of it done before it is refilled
                tuples(pp + 1, NB == 2 ? ((pp + 1) & 1) : 0, 2);
            }
            __syncthreads();
        }
    }
}

// Special functions of the packed double-float path, for PG pairs per CTA with the
// lanes of every phase busy (the assembler's groups hold only a few pairs, so these
// serial recurrences would leave most of its lanes idle):
//   A. one thread per pair: geometry (turned into double-float once) and h_p(kr) by
//      the upward j/y recurrence of spherical_hn_recursion (cpp/src/special.cpp:
//      90-111) in FP64;
//   B. one thread per (pair, mu): P_p^mu(cos theta) (no Condon-Shortley phase) and
//      e^{i mu phi} by binary powering, in double-float on the FP32 pipe
//      (Joldes-Muller-Popescu operations), and one per (pair, p) turning h_p into
//      double-float, on disjoint warps;
//   C. one thread per (pair, p, |mu|): G[p][+-mu] = P_p^|mu| h_p e^{+-i|mu|phi} for
//      |mu| <= p (negative mu through the (-1)^mu (p-mu)!/(p+mu)! ratio, held as a
//      double-float mantissa and an exact binary scaling).
// The table of pair p goes to the start of the pair's own block in the output plane
// (entry p^2 + p + mu as (re.hi, im.hi), (re.lo, im.lo): (2 lmax + 2)^2 entries fit in
// the B^2 words of a block at every lmax); the assembler CTA of the pair reads it back
// before it writes that block.
constexpr int kGtabThreads = 256;

struct GtabSmem {
    size_t off_geo, off_h, off_P, off_e, total;
};

__host__ __device__ inline GtabSmem gtab_layout(int L, int PG) {
    const int PM = 2 * L + 2, MU = 4 * L + 1;
    GtabSmem s;
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t r = o; o += (bytes + 15) & ~size_t(15); return r; };
    s.off_geo = take(sizeof(float2) * 4 * PG);             // cos theta, sin theta, cos phi, sin phi (double-float)
    s.off_h = take(sizeof(float4) * PM * PG);              // h_p as double-float complex
    s.off_P = take(sizeof(float2) * PM * PM * PG);         // P_p^mu [pair][p][mu] as double-float
    s.off_e = take(sizeof(float4) * MU * PG);              // e^{i mu phi}, mu = -2L..2L
    s.total = o;
    return s;
}

__global__ void __launch_bounds__(kGtabThreads)
k_asm_gtab(const gb::SysDev* __restrict__ sys, int nsys, const long long* __restrict__ grp_base, long long ngroups,
           int PG, const double* __restrict__ pos, float2* __restrict__ plane) {
    extern __shared__ __align__(16) unsigned char smem[];
    const long long g = blockIdx.x;
    if (g >= ngroups) return;
    const int tid = threadIdx.x;
    const int s = find_sys(grp_base, nsys, g);
    const gb::SysDev S = sys[s];
    const int L = S.lmax, N = S.N, PM = 2 * L + 2, MU = 4 * L + 1;
    const long long BB = (long long)S.B * S.B;
    const long long p_first = (g - grp_base[s]) * (long long)PG;
    const int np = (int)min((long long)PG, S.P - p_first);
    const GtabSmem lay = gtab_layout(L, PG);
    float2* geo = reinterpret_cast<float2*>(smem + lay.off_geo);
    float4* hh = reinterpret_cast<float4*>(smem + lay.off_h);
    float2* Pl = reinterpret_cast<float2*>(smem + lay.off_P);
    float4* eph = reinterpret_cast<float4*>(smem + lay.off_e);

    // ---- A: geometry (the angles enter only through cos/sin of theta and phi, taken
    // from the separation vector) and h_p(kr), one thread per pair
    if (tid < np) {
        int i, j;
        pair_ij(p_first + tid, N, i, j);
        const double* pi_ = pos + S.pos_off + 3 * (long long)i;
        const double* pj_ = pos + S.pos_off + 3 * (long long)j;
        const double dx = pi_[0] - pj_[0], dy = pi_[1] - pj_[1], dz = pi_[2] - pj_[2];
        const double rho2 = dx * dx + dy * dy;
        const double rad = sqrt(rho2 + dz * dz);
        const double inv_r = 1.0 / rad;
        const double rho = sqrt(rho2);
        double cphi = 1.0, sphi = 0.0;                  // phi = atan2(dy, dx) = 0 on the z axis
        if (rho2 > 0.0) {
            const double inv_rho = 1.0 / rho;
            cphi = dx * inv_rho;
            sphi = dy * inv_rho;
        }
        float2* ge = geo + 4 * tid;   // converted once here, not in every (pair, mu) thread
        const DF ct = df_of(dz * inv_r), st = df_of(rho * inv_r), cp = df_of(cphi), sp = df_of(sphi);
        ge[0] = make_float2(ct.h, ct.l);
        ge[1] = make_float2(st.h, st.l);
        ge[2] = make_float2(cp.h, cp.l);
        ge[3] = make_float2(sp.h, sp.l);
        const double z = S.k * rad;
        const double inv_z = 1.0 / z;
        double sz, cz;
        sincos(z, &sz, &cz);
        double j0 = sz * inv_z, y0 = -cz * inv_z;
        double j1 = j0 * inv_z + y0, y1 = y0 * inv_z - j0;
        // FP64 here; turned into double-float in place by the threads of phase B
        double2* h = reinterpret_cast<double2*>(hh) + PM * tid;
        h[0] = make_double2(j0, y0);
        h[1] = make_double2(j1, y1);
        for (int q = 2; q < PM; q++) {
            const double f = (2 * q - 1) * inv_z;
            const double jn = f * j1 - j0;
            const double yn = f * y1 - y0;
            j0 = j1; j1 = jn; y0 = y1; y1 = yn;
            h[q] = make_double2(jn, yn);
        }
    }
    __syncthreads();
    // ---- B: P_q^mu (threads from 0), e^{i mu phi} (threads from o1) and h_p into
    // double-float (threads from o2; o1 and o2 on warp boundaries, so that no warp
    // mixes two of the three)
    {
        const int n1 = np * PM, n2 = np * (2 * L + 1);
        const int o1 = (n1 + 31) & ~31, o2 = o1 + ((n2 + 31) & ~31);
        for (int it = tid; it < o2 + n1; it += kGtabThreads) {
            if (it >= o2) {   // each thread rewrites its own 16-byte slot
                const double2 hv = reinterpret_cast<const double2*>(hh)[it - o2];
                hh[it - o2] = dfc_pack(DFC{df_of(hv.x), df_of(hv.y)});
                continue;
            }
            if (it < n1) {
                const int pp = it / PM, mu = it - pp * PM;
                const DF x{geo[4 * pp].x, geo[4 * pp].y}, u{geo[4 * pp + 1].x, geo[4 * pp + 1].y};
                float2* P = Pl + (size_t)PM * PM * pp;
                DF pmm{1.f, 0.f};
                for (int kk = 1; kk <= mu; kk++) pmm = df_mulf(df_mul(pmm, u), (float)(2 * kk - 1));
                P[mu * PM + mu] = make_float2(pmm.h, pmm.l);
                if (mu + 1 < PM) {
                    DF pa = pmm, pb = df_mulf(df_mul(x, pmm), (float)(2 * mu + 1));
                    P[(mu + 1) * PM + mu] = make_float2(pb.h, pb.l);
                    for (int q = mu + 2; q < PM; q++) {
                        const DF t = df_add(df_mulf(df_mul(x, pb), (float)(2 * q - 1)), df_neg(df_mulf(pa, (float)(q + mu - 1))));
                        const DF pc = df_divf(t, (float)(q - mu));
                        P[q * PM + mu] = make_float2(pc.h, pc.l);
                        pa = pb;
                        pb = pc;
                    }
                }
            } else if (it >= o1 && it < o1 + n2) {
                const int k = it - o1, pp = k / (2 * L + 1), mu = k - pp * (2 * L + 1);
                int e = mu;
                DFC acc{DF{1.f, 0.f}, DF{0.f, 0.f}}, base{DF{geo[4 * pp + 2].x, geo[4 * pp + 2].y},
                                                          DF{geo[4 * pp + 3].x, geo[4 * pp + 3].y}};
                while (e) {
                    if (e & 1) acc = dfc_mul(acc, base);
                    base = dfc_mul(base, base);
                    e >>= 1;
                }
                eph[MU * pp + 2 * L + mu] = dfc_pack(acc);
                eph[MU * pp + 2 * L - mu] = dfc_pack(DFC{acc.re, df_neg(acc.im)});
            }
        }
    }
    __syncthreads();
    // ---- C: the table entries, one thread per (pair, p, |mu|) with |mu| <= min(p,
    // 2L) (orders |mu| > 2L, only at p = 2L + 1, occur in no tuple sum; e^{i mu phi}
    // is held for |mu| <= 2L): G(p, +-|mu|) from the four products of h_p and
    // e^{i|mu|phi}, h e = (t1 - t2, t3 + t4) and h conj(e) = (t1 + t2, t4 - t3)
    const int TRI = (2 * L + 1) * (2 * L + 2) / 2;   // entries with p <= 2L
    const int NE = TRI + 2 * L + 1;                 // and p = 2L + 1, |mu| <= 2L
    for (int it = tid; it < np * NE; it += kGtabThreads) {
        const int pp = it / NE, r2 = it - pp * NE;
        int q, am;
        if (r2 < TRI) {
            q = (int)((sqrtf(8.f * (float)r2 + 1.f) - 1.f) * 0.5f);
            if ((q + 1) * (q + 2) / 2 <= r2) q++;
            if (q * (q + 1) / 2 > r2) q--;
            am = r2 - q * (q + 1) / 2;
        } else {
            q = 2 * L + 1;
            am = r2 - TRI;
        }
        const float2 pv = Pl[(size_t)PM * PM * pp + q * PM + am];
        const DF P{pv.x, pv.y};
        const DFC h = dfc_unpack(hh[PM * pp + q]), e = dfc_unpack(eph[MU * pp + 2 * L + am]);
        const DF t1 = df_mul(h.re, e.re), t2 = df_mul(h.im, e.im), t3 = df_mul(h.re, e.im), t4 = df_mul(h.im, e.re);
        float2* dst = plane + S.mat_off + (p_first + pp) * BB + 2 * (q * q + q);
        {
            const DF gr = df_mul(P, df_add(t1, df_neg(t2))), gi = df_mul(P, df_add(t3, t4));
            dst[2 * am] = make_float2(gr.h, gi.h);
            dst[2 * am + 1] = make_float2(gr.l, gi.l);
        }
        if (am > 0) {   // mu = -|mu|: (-1)^mu (p-mu)!/(p+mu)! P_p^|mu| h_p e^{-i|mu|phi}
            const float4 rr = S.neg_ratio2[q * PM + am];
            DF Pn = df_mul(P, DF{rr.x, rr.y});
            if (rr.w != 0.f) {   // 2^e as a normal float: the scaling is one exact-rounded product
                Pn = DF{Pn.h * rr.w, Pn.l * rr.w};
            } else {
                const int ex = (int)rr.z;
                Pn = DF{ldexpf(Pn.h, ex), ldexpf(Pn.l, ex)};
            }
            const DF gr = df_mul(Pn, df_add(t1, t2)), gi = df_mul(Pn, df_add(t4, df_neg(t3)));
            dst[-2 * am] = make_float2(gr.h, gi.h);
            dst[-2 * am + 1] = make_float2(gr.l, gi.l);
        }
    }
}

__global__ void k_expand_mie(const gb::SysDev* __restrict__ sys, int nsys, const long long* __restrict__ mie_off,
                             const double2* __restrict__ mie, double2* __restrict__ tvec) {
    const int s = blockIdx.y;
    if (s >= nsys) return;
    const gb::SysDev S = sys[s];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < S.D; e += gridDim.x * blockDim.x) {
        const int pidx = e / S.B, R = e % S.B;
        tvec[S.t_off + e] = mie[mie_off[s] + (long long)pidx * 2 * S.lmax + S.miecol[R]];
    }
}

}   // namespace

namespace gb {

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return 148;
    if (!cached[dev]) {
        int c = 0;
        if (cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || c <= 0) c = 148;
        cached[dev] = c;
    }
    return cached[dev];
}

int make_sysdev(int nsys, const gb_system* sys, cudaStream_t stream, std::vector<SysDev>& out) {
    out.resize(nsys);
    long long tc_off = 0;
    for (int s = 0; s < nsys; s++) {
        const gb_system& a = sys[s];
        if (a.N < 1 || a.lmax < 1 || a.lmax > GB_LMAX_MAX)
            return gb_set_error(GB_BAD_ARG, "cluster %d: N=%d lmax=%d invalid", s, a.N, a.lmax);
        if (!(a.k > 0.0)) return gb_set_error(GB_BAD_ARG, "cluster %d: wavenumber must be positive", s);
        const Tables* T = nullptr;
        int st = get_tables(a.lmax, stream, &T);
        if (st) return st;
        SysDev& d = out[s];
        d.N = a.N;
        d.lmax = a.lmax;
        d.rmax = T->rmax;
        d.B = T->B;
        d.D = T->B * a.N;
        d.M = T->M;
        d.P = (long long)a.N * (a.N - 1) / 2;
        d.k = a.k;
        d.pos_off = a.pos_off;
        d.mat_off = a.mat_off;
        d.vec_off = a.vec_off;
        d.t_off = a.t_off;
        d.nmvu = T->nmvu;
        d.qab = T->qab;
        d.cA = T->cA;
        d.cB = T->cB;
        d.cA2 = T->cA2;
        d.cB2 = T->cB2;
        d.tinfo = T->tinfo;
        d.cA2s = T->cA2s;
        d.cB2s = T->cB2s;
        d.elem_map = T->elem_map;
        d.neg_ratio = T->neg_ratio;
        d.neg_ratio2 = T->neg_ratio2;
        d.rowinfo = T->rowinfo;
        d.miecol = T->miecol;
        d.tc_off = tc_off;
        tc_off += d.P * tc_block_bytes(d.B);
    }
    return GB_OK;
}

// Small per-call descriptor arrays travel through a ring of pinned host /
// device staging slots (per host thread and device).  A slot is reused only
// after the event recorded behind the kernels that read it has completed, so
// calls stay asynchronous.  Slots grow by doubling and never free a buffer while
// the thread lives (cudaFree and cudaFreeHost wait for the whole device, which
// would tie this thread to every other stream's work): outgrown buffers are
// parked and released when the thread exits.
struct Parked {
    std::vector<void*> host, dev;
    ~Parked() {
        for (void* p : host) cudaFreeHost(p);
        for (void* p : dev) cudaFree(p);
    }
};
static Parked& parked() {
    thread_local Parked p;
    return p;
}

struct StageSlot {
    void* host = nullptr;
    void* dev = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
    bool pending = false;
};
struct StageRing {
    int device = -1;
    int next = 0;
    StageSlot slot[16];
};

static StageRing& ring_for_thread() {
    thread_local StageRing r[8];
    int dev = 0;
    cudaGetDevice(&dev);
    return r[dev & 7];
}

int stage_acquire(const void* src, size_t bytes, cudaStream_t stream, void** dev_out, int* slot_out) {
    StageRing& R = ring_for_thread();
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    R.device = dev;
    const int k = R.next;
    R.next = (R.next + 1) % 16;
    StageSlot& S = R.slot[k];
    if (S.pending) {
        GB_CUDA_TRY(cudaEventSynchronize(S.done));
        S.pending = false;
    }
    if (!S.done) GB_CUDA_TRY(cudaEventCreateWithFlags(&S.done, cudaEventDisableTiming));
    if (S.cap < bytes) {
        size_t cap = std::max<size_t>(1 << 16, 2 * S.cap);
        while (cap < bytes) cap *= 2;
        if (S.host) parked().host.push_back(S.host);
        if (S.dev) parked().dev.push_back(S.dev);
        S.host = S.dev = nullptr;
        S.cap = 0;
        GB_CUDA_TRY(cudaHostAlloc(&S.host, cap, cudaHostAllocDefault));
        GB_CUDA_TRY(cudaMalloc(&S.dev, cap));
        S.cap = cap;
    }
    memcpy(S.host, src, bytes);
    GB_CUDA_TRY(cudaMemcpyAsync(S.dev, S.host, bytes, cudaMemcpyHostToDevice, stream));
    *dev_out = S.dev;
    *slot_out = k;
    return GB_OK;
}

void* host_readback(size_t bytes) {
    struct Buf {
        void* p = nullptr;
        size_t cap = 0;
    };
    thread_local Buf b[8];
    int dev = 0;
    cudaGetDevice(&dev);
    Buf& B = b[dev & 7];
    if (B.cap < bytes) {
        if (B.p) parked().host.push_back(B.p);
        B.p = nullptr;
        size_t cap = std::max<size_t>(1 << 16, 2 * B.cap);
        while (cap < bytes) cap *= 2;
        if (cudaHostAlloc(&B.p, cap, cudaHostAllocDefault) != cudaSuccess) {
            B.p = nullptr;
            B.cap = 0;
            return nullptr;
        }
        B.cap = cap;
    }
    return B.p;
}

int stage_release(int slot, cudaStream_t stream) {
    StageRing& R = ring_for_thread();
    StageSlot& S = R.slot[slot];
    GB_CUDA_TRY(cudaEventRecord(S.done, stream));
    S.pending = true;
    return GB_OK;
}

}   // namespace gb

namespace {

// One launch per lmax of the batch (each with its own tuple layout and pairs per
// group), so that small-lmax clusters of a ragged batch are not run with the
// shared-memory strides of the largest one.
int launch_assemble(int nsys, const gb_system* sys, const double* pos, const double* mie, double* out128,
                    float* out64, float* out64lo, long long dense_ld, bool dense, cudaStream_t stream,
                    const Refl* refl = nullptr, const Latt* latt = nullptr) {
    std::vector<gb::SysDev> all;
    int st = gb::make_sysdev(nsys, sys, stream, all);
    if (st) return st;
    const bool fp64_sums = dense || out128 != nullptr;
    const bool want64 = (out64 != nullptr || out64lo != nullptr) && !dense;
    std::vector<int> lmaxes;
    for (const gb::SysDev& d : all)
        if (std::find(lmaxes.begin(), lmaxes.end(), d.lmax) == lmaxes.end()) lmaxes.push_back(d.lmax);
    std::sort(lmaxes.begin(), lmaxes.end());
    for (int L : lmaxes) {
        std::vector<gb::SysDev> sd;
        for (const gb::SysDev& d : all)
            if (d.lmax == L) sd.push_back(d);
        const int ns = (int)sd.size();
        int Mmax = 0;
        long long total_pairs = 0;
        for (const gb::SysDev& d : sd) {
            Mmax = std::max(Mmax, d.M);
            total_pairs += (refl || latt) ? (long long)d.N * d.N : d.P;
        }
        if (total_pairs == 0) continue;
        // tuple buffers: two (pipelined pairs) when a one-pair group still fits the
        // CTA's shared-memory target, else one; pairs per group: the largest power of
        // two up to the cap whose tables keep the CTA within the target.  Targets: ~72
        // KB for the FP64 paths (three CTAs per SM), ~44 KB and at most 4 pairs for the
        // double-float path (five CTAs per SM: measured 0.31 ms against 0.35 ms with
        // three CTAs of 8 pairs at N = 200, lmax 4)
        const size_t target = fp64_sums ? 72 * 1024 : 44 * 1024;
        int NB = asm_layout(L, Mmax, 1, fp64_sums, want64, 2).total <= target ? 2 : 1;
        int PB = fp64_sums ? 32 : 4;
        while (PB > 1 && asm_layout(L, Mmax, PB, fp64_sums, want64, NB).total > target) PB >>= 1;
        // whole-group phases (packed double-float, lmax <= 5): one buffer per pair,
        // the most pairs up to 4 that keep the target (56 KB at lmax 5: two pairs, four
        // CTAs per SM; N = 200 in 0.424 ms against 0.451 ms pair by pair)
        bool ts = false;
        if (!dense && !refl && !latt && !fp64_sums && L <= 5) {
            int pb = 4;
            const size_t ts_target = L == 5 ? 56 * 1024 : target;
            while (pb > 1 && asm_layout(L, Mmax, pb, false, want64, pb).total > ts_target) pb--;
            if (pb >= 2) {
                ts = true;
                PB = NB = pb;
            }
        }
        // one pair's A and B tuple values together beyond a CTA's shared memory (lmax 10):
        // the split kernel forms and writes them one kind at a time
        const bool split = !ts && !refl && !latt && asm_layout(L, Mmax, PB, fp64_sums, want64, NB).total > 227 * 1024;
        if (split) PB = NB = 1;
        const AsmSmem lay = asm_layout(L, Mmax, PB, fp64_sums, want64, NB, split, latt != nullptr);
        const size_t smem = lay.total;
        if (smem > 227 * 1024) return gb_set_error(GB_UNSUPPORTED, "assembler needs %zu B of shared memory", smem);
        Latt lt = latt ? *latt : Latt();
        if (latt) {
            if (lt.ncell < 1) return GB_OK;
            // each group sums a range of whole chunks of PB cells (its tuple sums and
            // block additions once per range); enough groups to fill the SMs about
            // twice, at least one per ordered pair
            long long pairs = 0;
            for (const gb::SysDev& d : sd) pairs += (long long)d.N * d.N;
            const long long chunks = (lt.ncell + PB - 1) / PB;
            const long long want = 6LL * gb::sm_count();
            const long long g = std::min<long long>(chunks, std::max<long long>(1, (want + pairs - 1) / pairs));
            lt.cpg = (int)(((chunks + g - 1) / g) * PB);
            lt.gpp = (lt.ncell + lt.cpg - 1) / lt.cpg;
        }
        std::vector<long long> gbase(ns + 1, 0);
        for (int s = 0; s < ns; s++) {
            const long long np_s = refl ? (long long)sd[s].N * sd[s].N : sd[s].P;
            gbase[s + 1] = gbase[s] + (latt ? (long long)sd[s].N * sd[s].N * lt.gpp : (np_s + PB - 1) / PB);
        }
        const long long ngroups = gbase[ns];
        // the double-float path's G-table pass: PG pairs per CTA (the most, up to 32,
        // whose special functions fit in 48 KB of shared memory)
        int PG = 32;
        while (PG > 1 && gtab_layout(L, PG).total > 48 * 1024) PG >>= 1;
        std::vector<long long> gbase2(ns + 1, 0);
        for (int s = 0; s < ns; s++) gbase2[s + 1] = gbase2[s] + (fp64_sums ? 0 : (sd[s].P + PG - 1) / PG);
        // one staging upload: descriptors, then the group prefix sums of both passes
        std::vector<unsigned char> blob(sizeof(gb::SysDev) * ns + 2 * sizeof(long long) * (ns + 1));
        memcpy(blob.data(), sd.data(), sizeof(gb::SysDev) * ns);
        memcpy(blob.data() + sizeof(gb::SysDev) * ns, gbase.data(), sizeof(long long) * (ns + 1));
        memcpy(blob.data() + sizeof(gb::SysDev) * ns + sizeof(long long) * (ns + 1), gbase2.data(),
               sizeof(long long) * (ns + 1));
        void* dblob = nullptr;
        int slot = 0;
        st = gb::stage_acquire(blob.data(), blob.size(), stream, &dblob, &slot);
        if (st) return st;
        const gb::SysDev* dsys = reinterpret_cast<const gb::SysDev*>(dblob);
        const long long* dbase =
            reinterpret_cast<const long long*>(static_cast<unsigned char*>(dblob) + sizeof(gb::SysDev) * ns);

        // the pair-by-pair double-float path with room for at most two CTAs per SM
        // (lmax >= 8) runs 512 threads per CTA (N = 200, lmax 8: 2.94 ms against 3.25
        // ms; N = 60, lmax 9: 0.49 ms against 0.76 ms; more threads at lower lmax
        // measured slower), and so do the packed FP64 and dense paths with room for
        // one (lmax >= 8; packed N = 200, lmax 8: 8.37 ms against 9.93 ms; dense N = 60,
        // lmax 9: 2.29 ms against 2.98 ms)
        const bool wide = !split && !refl && !latt &&
                          (fp64_sums ? smem > 227 * 1024 / 2 : !ts && smem > 227 * 1024 / 3);
        const int nt = wide ? kAsmWideThreads : kAsmThreads;
        auto kfn = latt ? k_assemble<true, true, 2>
                        : refl ? k_assemble<true, true, 1>
                               : split ? (dense ? k_assemble<true, true, 0, false, true>
                                                : (fp64_sums ? k_assemble<false, true, 0, false, true>
                                                             : k_assemble<false, false, 0, false, true>))
                                       : (dense ? (wide ? k_assemble<true, true, 0, false, false, kAsmWideThreads>
                                                        : k_assemble<true, true>)
                                                : (fp64_sums ? (wide ? k_assemble<false, true, 0, false, false,
                                                                                  kAsmWideThreads>
                                                                     : k_assemble<false, true>)
                                                             : (ts ? k_assemble<false, false, 0, true>
                                                                   : (wide ? k_assemble<false, false, 0, false, false,
                                                                                        kAsmWideThreads>
                                                                           : k_assemble<false, false>))));
        GB_CUDA_TRY(gb::ensure_dynamic_smem(reinterpret_cast<const void*>(kfn), smem));
        int per_sm = 1;
        GB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, nt, smem));
        if (per_sm < 1) return gb_set_error(GB_UNSUPPORTED, "assembler does not fit on an SM (smem %zu B)", smem);
        // one group per CTA (no persistent loop): CTAs retire every few microseconds, so
        // kernels of higher-priority streams (other clusters' solves) are dispatched
        // between them instead of waiting for the whole assembly
        if (!fp64_sums && gbase2[ns] > 0) {
            // the G tables first (read back by the assembler CTA of each pair).  Running
            // them in chunks on a second stream beside the assembler measured slower
            // (0.232 ms with two chunks against 0.210 ms in one stream at N = 200, lmax 4).
            const size_t gsm = gtab_layout(L, PG).total;
            GB_CUDA_TRY(gb::ensure_dynamic_smem(reinterpret_cast<const void*>(k_asm_gtab), gsm));
            gb::note_launch();
            k_asm_gtab<<<(unsigned)std::min<long long>(gbase2[ns], 0x7fffffffLL), kGtabThreads, gsm, stream>>>(
                dsys, ns, dbase + (ns + 1), gbase2[ns], PG, pos, reinterpret_cast<float2*>(out64lo ? out64lo : out64));
            GB_CUDA_TRY(cudaGetLastError());
        }
        gb::note_launch();
        kfn<<<(unsigned)std::min<long long>(ngroups, 0x7fffffffLL), nt, smem, stream>>>(
            dsys, ns, dbase, ngroups, L, Mmax, PB, NB, pos, reinterpret_cast<const double2*>(mie),
            reinterpret_cast<double2*>(out128), reinterpret_cast<float2*>(out64), reinterpret_cast<float2*>(out64lo),
            dense_ld, refl ? *refl : Refl(), lt);
        GB_CUDA_TRY(cudaGetLastError());
        st = gb::stage_release(slot, stream);
        if (st) return st;
    }
    return GB_OK;
}

}   // namespace

extern "C" {

int gb_assemble_sphere_dense(int N, int lmax, const double* pos, const double* mie, double k, double* out,
                             void* stream) {
    if (!pos || !mie || !out) return gb_set_error(GB_BAD_ARG, "null pointer");
    if (N < 1 || lmax < 1 || lmax > GB_LMAX_MAX) return gb_set_error(GB_BAD_ARG, "N=%d lmax=%d invalid", N, lmax);
    const long long D = 2LL * lmax_to_rmax(lmax) * N;
    GB_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double2) * D * D, (cudaStream_t)stream));
    if (N == 1) return GB_OK;
    gb_system s{N, lmax, k, 0, 0, 0, 0};
    return launch_assemble(1, &s, pos, mie, out, nullptr, nullptr, D, true, (cudaStream_t)stream);
}

int gb_reflection_matrix_dense(int N, int lmax, const double* pos, const double* mie, double k, double r_re,
                               double r_im, double z, double* out, void* stream) {
    if (!pos || !mie || !out) return gb_set_error(GB_BAD_ARG, "null pointer");
    if (N < 1 || lmax < 1 || lmax > GB_LMAX_MAX) return gb_set_error(GB_BAD_ARG, "N=%d lmax=%d invalid", N, lmax);
    const long long D = 2LL * lmax_to_rmax(lmax) * N;
    GB_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double2) * D * D, (cudaStream_t)stream));
    gb_system s{N, lmax, k, 0, 0, 0, 0};
    Refl r;
    r.z = z;
    r.r0 = make_double2(r_re, r_im);
    return launch_assemble(1, &s, pos, mie, out, nullptr, nullptr, D, true, (cudaStream_t)stream, &r);
}

int gb_aggregate_periodic_dense(int N, int lmax, const double* pos, const double* mie, double k, const double* cells,
                                int ncell, double kx, double ky, double kz, double* out, void* stream) {
    if (!pos || !mie || !out || (ncell > 0 && !cells)) return gb_set_error(GB_BAD_ARG, "null pointer");
    if (N < 1 || lmax < 1 || lmax > GB_LMAX_MAX || ncell < 0)
        return gb_set_error(GB_BAD_ARG, "N=%d lmax=%d ncell=%d invalid", N, lmax, ncell);
    const long long D = 2LL * lmax_to_rmax(lmax) * N;
    GB_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double2) * D * D, (cudaStream_t)stream));
    gb_system s{N, lmax, k, 0, 0, 0, 0};
    if (N > 1) {
        const int e = launch_assemble(1, &s, pos, mie, out, nullptr, nullptr, D, true, (cudaStream_t)stream);
        if (e) return e;
    }
    Latt lt;
    lt.cells = cells;
    lt.ncell = ncell;
    lt.kx = kx;
    lt.ky = ky;
    lt.kz = kz;
    return launch_assemble(1, &s, pos, mie, out, nullptr, nullptr, D, true, (cudaStream_t)stream, nullptr, &lt);
}

int gb_assemble_sphere_packed(int N, int lmax, const double* pos, double k, double* out128, float* out64,
                              float* out64lo, void* stream) {
    if (!pos || (!out128 && !out64 && !out64lo)) return gb_set_error(GB_BAD_ARG, "null pointer");
    gb_system s{N, lmax, k, 0, 0, 0, 0};
    return launch_assemble(1, &s, pos, nullptr, out128, out64, out64lo, 0, false, (cudaStream_t)stream);
}

int gb_assemble_batch(int nsys, const gb_system* sys, const double* pos, double* mat128, float* mat64,
                      float* mat64lo, void* stream) {
    if (nsys < 1 || !sys || !pos || (!mat128 && !mat64 && !mat64lo))
        return gb_set_error(GB_BAD_ARG, "bad batch arguments");
    return launch_assemble(nsys, sys, pos, nullptr, mat128, mat64, mat64lo, 0, false, (cudaStream_t)stream);
}

int gb_expand_mie_batch(int nsys, const gb_system* sys, const int64_t* mie_off, const double* mie, double* tvec,
                        void* stream) {
    if (nsys < 1 || !sys || !mie_off || !mie || !tvec) return gb_set_error(GB_BAD_ARG, "bad arguments");
    cudaStream_t st_ = (cudaStream_t)stream;
    std::vector<gb::SysDev> sd;
    int st = gb::make_sysdev(nsys, sys, st_, sd);
    if (st) return st;
    std::vector<unsigned char> blob(sizeof(gb::SysDev) * nsys + sizeof(long long) * nsys);
    memcpy(blob.data(), sd.data(), sizeof(gb::SysDev) * nsys);
    memcpy(blob.data() + sizeof(gb::SysDev) * nsys, mie_off, sizeof(long long) * nsys);
    void* dblob = nullptr;
    int slot = 0;
    st = gb::stage_acquire(blob.data(), blob.size(), st_, &dblob, &slot);
    if (st) return st;
    int maxD = 0;
    for (auto& d : sd) maxD = std::max(maxD, d.D);
    dim3 grid((maxD + 255) / 256, nsys);
    gb::note_launch();
    k_expand_mie<<<grid, 256, 0, st_>>>(reinterpret_cast<const gb::SysDev*>(dblob), nsys,
                                        reinterpret_cast<const long long*>(static_cast<unsigned char*>(dblob) + sizeof(gb::SysDev) * nsys),
                                        reinterpret_cast<const double2*>(mie), reinterpret_cast<double2*>(tvec));
    GB_CUDA_TRY(cudaGetLastError());
    return gb::stage_release(slot, st_);
}

}   // extern "C"
