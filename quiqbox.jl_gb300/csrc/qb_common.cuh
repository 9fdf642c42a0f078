// Shared device definitions of the GB300 integral / Hartree–Fock path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define QB_PI 3.14159265358979323846
#define QB_SQRT_PI_HALF 0.88622692545275801365   // sqrt(pi)/2

// ---------------------------------------------------------------------------
// Boys function table.  Row k holds, for T_k = k/16 and every order m, the 8
// Taylor coefficients c_j = F_{m+j}(T_k) (-1)^j / j!, so that
//   F_m(T_k + d) = sum_j c_j d^j,  |d| <= 1/32   (relative error < 3e-17);
// after the rows, e^{-T_k} for every k (e^{-T} = e^{-T_k} e^{-d} with a degree-8
// Taylor polynomial of e^{-d}).
// Above T = QB_BOYS_TMAX the asymptotic F_0 = sqrt(pi/T)/2 (erfc(sqrt 50) ~ 2e-24)
// and the upward recursion F_{m+1} = ((2m+1) F_m - e^{-T}) / (2T) are used; for the
// orders m <= QB_BOYS_ASYM_NOEXP_M the e^{-T} term is dropped: its share of F_m is
// e^{-T} / (2T F_m) < 2e-15 for T >= 50.
#define QB_BOYS_DT_INV 16.0
#define QB_BOYS_DT 0.0625
#define QB_BOYS_TMAX 50.0
#define QB_BOYS_NROW 801      // T_k = 0 .. 50
#define QB_BOYS_NM 41         // orders m = 0 .. 40
#define QB_BOYS_NJ 8          // Taylor terms
#define QB_BOYS_EXP_OFF (QB_BOYS_NROW * QB_BOYS_NM * QB_BOYS_NJ)
#define QB_BOYS_TABLE_SIZE (QB_BOYS_EXP_OFF + QB_BOYS_NROW)
#define QB_BOYS_ASYM_NOEXP_M 6

// Primitive quartets with |K_ab K_cd| below this bound are skipped by the batched
// integral stores (the prefactor of every integral of the quartet is below 2.3 x this).
#define QB_PRIM_EPS 1e-20

// Primitive quartets whose primitive Schwarz factors multiply to less than this are
// skipped by the single-basis J/K kernels.  The key of a primitive pair (ab) is
// sqrt(max over components |(ab|ab)|) of the ratio-free shells, so by the Cauchy-Schwarz
// inequality every integral of a skipped primitive quartet is below this bound; with the
// per-function ratios (<= 3 per d pair) and at most 81 primitive quartets per quartet of
// 3-primitive shells, a contracted integral changes by < 7.3e-13.
#define QB_PRIM_EPS_Q 1e-15

// Largest total angular momentum of the generic (per-function) kernels.
#define QB_GEN_LTOT_MAX 32

__device__ __forceinline__ double qb_horner8(const double* __restrict__ c, double d) {
    const double2 c01 = __ldg(reinterpret_cast<const double2*>(c));
    const double2 c23 = __ldg(reinterpret_cast<const double2*>(c + 2));
    const double2 c45 = __ldg(reinterpret_cast<const double2*>(c + 4));
    const double2 c67 = __ldg(reinterpret_cast<const double2*>(c + 6));
    double r = fma(c67.y, d, c67.x);
    r = fma(r, d, c45.y);
    r = fma(r, d, c45.x);
    r = fma(r, d, c23.y);
    r = fma(r, d, c23.x);
    r = fma(r, d, c01.y);
    r = fma(r, d, c01.x);
    return r;
}

// e^{-d} for |d| <= 1/32: Taylor polynomial of degree 8 (truncation < 8e-20).
__device__ __forceinline__ double qb_exp_neg_small(double d) {
    double r = fma(d, 1.0 / 40320.0, -1.0 / 5040.0);
    r = fma(r, d, 1.0 / 720.0);
    r = fma(r, d, -1.0 / 120.0);
    r = fma(r, d, 1.0 / 24.0);
    r = fma(r, d, -1.0 / 6.0);
    r = fma(r, d, 0.5);
    r = fma(r, d, -1.0);
    return fma(r, d, 1.0);
}

// F[m] = pre * F_m(T) for m = 0..M (compile-time M).
template <int M>
__device__ __forceinline__ void qb_boys_scaled(double T, double pre, const double* __restrict__ tab,
                                               double (&F)[M + 1]) {
    if (T < QB_BOYS_TMAX) {
        const int k = __double2int_rn(T * QB_BOYS_DT_INV);
        const double d = fma(-(double)k, QB_BOYS_DT, T);
        const double* row = tab + (size_t)k * (QB_BOYS_NM * QB_BOYS_NJ);
        if (M <= 2) {
#pragma unroll
            for (int m = 0; m <= M; ++m) F[m] = pre * qb_horner8(row + m * QB_BOYS_NJ, d);
        } else {
            double f = pre * qb_horner8(row + M * QB_BOYS_NJ, d);
            const double e = (pre * __ldg(tab + QB_BOYS_EXP_OFF + k)) * qb_exp_neg_small(d);
            const double T2 = T + T;
            F[M] = f;
#pragma unroll
            for (int m = M - 1; m >= 0; --m) {
                f = fma(T2, f, e) * (1.0 / (2 * m + 1));
                F[m] = f;
            }
        }
    } else {
        const double ir = rsqrt(T);
        double f = pre * QB_SQRT_PI_HALF * ir;
        F[0] = f;
        if (M > 0) {
            const double i2T = 0.5 * ir * ir;
            if (M <= QB_BOYS_ASYM_NOEXP_M) {
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    f = f * ((double)(2 * m + 1) * i2T);
                    F[m + 1] = f;
                }
            } else {
                const double e = pre * exp(-T);
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    f = fma((double)(2 * m + 1), f, -e) * i2T;
                    F[m + 1] = f;
                }
            }
        }
    }
}

// Runtime-order variant for the generic kernels: F[0..M], M <= QB_GEN_LTOT_MAX.
__device__ __forceinline__ void qb_boys_scaled_rt(double T, double pre, const double* __restrict__ tab,
                                                  int M, double* F) {
    if (T < QB_BOYS_TMAX) {
        const int k = __double2int_rn(T * QB_BOYS_DT_INV);
        const double d = fma(-(double)k, QB_BOYS_DT, T);
        const double* row = tab + (size_t)k * (QB_BOYS_NM * QB_BOYS_NJ);
        double f = pre * qb_horner8(row + M * QB_BOYS_NJ, d);
        F[M] = f;
        if (M > 0) {
            const double e = (pre * __ldg(tab + QB_BOYS_EXP_OFF + k)) * qb_exp_neg_small(d);
            const double T2 = T + T;
            for (int m = M - 1; m >= 0; --m) {
                f = fma(T2, f, e) / (double)(2 * m + 1);
                F[m] = f;
            }
        }
    } else {
        const double ir = rsqrt(T);
        double f = pre * QB_SQRT_PI_HALF * ir;
        F[0] = f;
        if (M > 0) {
            const double e = (M <= QB_BOYS_ASYM_NOEXP_M) ? 0.0 : pre * exp(-T);
            const double i2T = 0.5 * ir * ir;
            for (int m = 0; m < M; ++m) {
                f = fma((double)(2 * m + 1), f, -e) * i2T;
                F[m + 1] = f;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Primitive pair of a shell pair (A, B), A the shell of higher angular momentum:
//   p = a + b, P = (aA + bB)/p, PA = P - A, oo2p = 1/(2p),
//   K = sqrt(2) pi^(5/4) c_a c_b exp(-ab/p |A-B|^2) / p
// so that the primitive ERI prefactor 2 pi^(5/2)/(p q sqrt(p+q)) K_AB K_CD ... equals
// K_ab K_cd / sqrt(p+q).  80 bytes, 16-byte aligned (five 128-bit loads).
struct __align__(16) PrimPair {
    double p, Px, Py, Pz, PAx, PAy, PAz, K, oo2p, pad;
};

__device__ __forceinline__ PrimPair qb_load_pair(const PrimPair* __restrict__ ptr) {
    const double2* q = reinterpret_cast<const double2*>(ptr);
    const double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3), e = __ldg(q + 4);
    PrimPair r;
    r.p = a.x; r.Px = a.y; r.Py = b.x; r.Pz = b.y; r.PAx = c.x; r.PAy = c.y; r.PAz = d.x; r.K = d.y;
    r.oo2p = e.x; r.pad = e.y;
    return r;
}

// Screening key of a primitive pair as a float, kept in the pad word (screening decisions
// in the FP32 pipe): |K| as built, replaced by the primitive Schwarz factor in the
// single-basis J/K engine (qb_prim_key_kernel).
__device__ __forceinline__ float qb_kabs(const PrimPair* __restrict__ p) {
    return __ldg(reinterpret_cast<const float*>(&p->pad));
}

// Shell pair (A, B) of a class list.
struct ShellPair {
    int fa, fb;        // first basis-function index of shells A and B
    int prim0, nprim;  // primitive pairs [prim0, prim0+nprim) in the PrimPair table
    double ABx, ABy, ABz;
    double Q;          // Schwarz factor sqrt(max |(ab|ab)|)
    int same;          // A == B (same shell)
    int pad;
};

// Generated per class (gen_eri.py): contracted block in SubshellXYZs order,
// index ((a*NB + b)*NC + c)*ND + d, without the per-function ratios.
template <int LA, int LB, int LC, int LD>
struct EriClass;

// Device-side status word: bit flags set by kernels that met an unexpected state.
#define QB_DEVERR_BAD_INDEX 1
