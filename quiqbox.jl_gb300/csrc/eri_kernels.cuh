// Class-templated ERI kernel: the fused J/K build of one angular-momentum class.
//
// The work of one class (bra pair class X, ket pair class Y) is the set of
// shell-pair couples (i, j), i over the bra list and j over the first cnt_i
// entries of the ket list, both lists sorted by descending Schwarz factor, so
// that Q_i Q_j >= threshold holds exactly on that prefix (and j <= i when
// X == Y, which makes every unordered couple appear once).  offs[i] is the
// exclusive prefix sum of cnt_i; one thread takes one couple.
#pragma once
#include "qb_common.cuh"

struct ClassWork {
    const ShellPair* __restrict__ bra;
    const ShellPair* __restrict__ ket;
    const long long* __restrict__ offs;   // nbra + 1 entries; offs[nbra] = total
    int nbra;
    int same;                              // bra class == ket class
};

struct JKArgs {
    const PrimPair* __restrict__ prims;
    const double* __restrict__ boys;
    const double* __restrict__ D;          // ratio-scaled density, column-major
    double* Jp;                            // J' accumulator (column-major nfun x nfun)
    double* Kp;                            // K' accumulator
    unsigned long long* primcount;         // primitive quartets evaluated (this class)
    int nfun;
};

__device__ __forceinline__ int qb_find_bra(const long long* __restrict__ offs, int n, long long t) {
    int lo = 0, hi = n;   // largest i with offs[i] <= t
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(offs + mid) <= t) lo = mid; else hi = mid;
    }
    return lo;
}

// One integral v = (ab|cd) into the six J'/K' accumulators (D blocks preloaded).
__device__ __forceinline__ void qb_digest(double v, int ab, int cd, int ac, int ad, int bc, int bd,
                                          const double* Dab, const double* Dcd, const double* Dac,
                                          const double* Dad, const double* Dbc, const double* Dbd, double* Jab,
                                          double* Jcd, double* Kac, double* Kad, double* Kbc, double* Kbd) {
    Jab[ab] = fma(Dcd[cd], v, Jab[ab]);
    Jcd[cd] = fma(Dab[ab], v, Jcd[cd]);
    Kac[ac] = fma(Dbd[bd], v, Kac[ac]);
    Kad[ad] = fma(Dbc[bc], v, Kad[ad]);
    Kbc[bc] = fma(Dad[ad], v, Kbc[bc]);
    Kbd[bd] = fma(Dac[ac], v, Kbd[bd]);
}

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) qb_jk_class_kernel(const ClassWork w, const JKArgs a) {
    using C = EriClass<LA, LB, LC, LD>;
    constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND;
    const long long total = __ldg(w.offs + w.nbra);
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned nprimq = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const int i = qb_find_bra(w.offs, w.nbra, t);
        const int j = (int)(t - __ldg(w.offs + i));
        const ShellPair P = w.bra[i];
        const ShellPair Q = w.ket[j];
        double I[C::NINT];
        C::block(a.prims + P.prim0, P.nprim, a.prims + Q.prim0, Q.nprim, P.ABx, P.ABy, P.ABz,
                 Q.ABx, Q.ABy, Q.ABz, a.boys, I, nprimq);
        const double deg = (P.same ? 1.0 : 2.0) * (Q.same ? 1.0 : 2.0) * ((w.same && i == j) ? 1.0 : 2.0);
        const int N = a.nfun;
        const double* __restrict__ D = a.D;
        double Dab[NA * NB], Dcd[NC * ND], Dac[NA * NC], Dad[NA * ND], Dbc[NB * NC], Dbd[NB * ND];
#pragma unroll
        for (int x = 0; x < NA; ++x)
#pragma unroll
            for (int y = 0; y < NB; ++y) Dab[x * NB + y] = __ldg(D + (P.fa + x) + (size_t)N * (P.fb + y));
#pragma unroll
        for (int x = 0; x < NC; ++x)
#pragma unroll
            for (int y = 0; y < ND; ++y) Dcd[x * ND + y] = __ldg(D + (Q.fa + x) + (size_t)N * (Q.fb + y));
#pragma unroll
        for (int x = 0; x < NA; ++x)
#pragma unroll
            for (int y = 0; y < NC; ++y) Dac[x * NC + y] = __ldg(D + (P.fa + x) + (size_t)N * (Q.fa + y));
#pragma unroll
        for (int x = 0; x < NA; ++x)
#pragma unroll
            for (int y = 0; y < ND; ++y) Dad[x * ND + y] = __ldg(D + (P.fa + x) + (size_t)N * (Q.fb + y));
#pragma unroll
        for (int x = 0; x < NB; ++x)
#pragma unroll
            for (int y = 0; y < NC; ++y) Dbc[x * NC + y] = __ldg(D + (P.fb + x) + (size_t)N * (Q.fa + y));
#pragma unroll
        for (int x = 0; x < NB; ++x)
#pragma unroll
            for (int y = 0; y < ND; ++y) Dbd[x * ND + y] = __ldg(D + (P.fb + x) + (size_t)N * (Q.fb + y));
        double Jab[NA * NB] = {}, Jcd[NC * ND] = {}, Kac[NA * NC] = {}, Kad[NA * ND] = {},
               Kbc[NB * NC] = {}, Kbd[NB * ND] = {};
        if constexpr (C::NINT <= 162) {
#pragma unroll
            for (int x = 0; x < NA; ++x)
#pragma unroll
                for (int y = 0; y < NB; ++y)
#pragma unroll
                    for (int z = 0; z < NC; ++z)
#pragma unroll
                        for (int u = 0; u < ND; ++u)
                            qb_digest(I[((x * NB + y) * NC + z) * ND + u], x * NB + y, z * ND + u, x * NC + z,
                                      x * ND + u, y * NC + z, y * ND + u, Dab, Dcd, Dac, Dad, Dbc, Dbd, Jab, Jcd, Kac,
                                      Kad, Kbc, Kbd);
        } else {
            // large blocks: rolled loops keep compile time and code size bounded
#pragma unroll 1
            for (int x = 0; x < NA; ++x)
#pragma unroll 1
                for (int y = 0; y < NB; ++y)
#pragma unroll 1
                    for (int z = 0; z < NC; ++z)
#pragma unroll 1
                        for (int u = 0; u < ND; ++u)
                            qb_digest(I[((x * NB + y) * NC + z) * ND + u], x * NB + y, z * ND + u, x * NC + z,
                                      x * ND + u, y * NC + z, y * ND + u, Dab, Dcd, Dac, Dad, Dbc, Dbd, Jab, Jcd, Kac,
                                      Kad, Kbc, Kbd);
        }
        double* Jp = a.Jp;
        double* Kp = a.Kp;
#pragma unroll
        for (int x = 0; x < NA; ++x)
#pragma unroll
            for (int y = 0; y < NB; ++y) atomicAdd(Jp + (P.fa + x) + (size_t)N * (P.fb + y), deg * Jab[x * NB + y]);
#pragma unroll
        for (int x = 0; x < NC; ++x)
#pragma unroll
            for (int y = 0; y < ND; ++y) atomicAdd(Jp + (Q.fa + x) + (size_t)N * (Q.fb + y), deg * Jcd[x * ND + y]);
#pragma unroll
        for (int x = 0; x < NA; ++x)
#pragma unroll
            for (int y = 0; y < NC; ++y) atomicAdd(Kp + (P.fa + x) + (size_t)N * (Q.fa + y), deg * Kac[x * NC + y]);
#pragma unroll
        for (int x = 0; x < NA; ++x)
#pragma unroll
            for (int y = 0; y < ND; ++y) atomicAdd(Kp + (P.fa + x) + (size_t)N * (Q.fb + y), deg * Kad[x * ND + y]);
#pragma unroll
        for (int x = 0; x < NB; ++x)
#pragma unroll
            for (int y = 0; y < NC; ++y) atomicAdd(Kp + (P.fb + x) + (size_t)N * (Q.fa + y), deg * Kbc[x * NC + y]);
#pragma unroll
        for (int x = 0; x < NB; ++x)
#pragma unroll
            for (int y = 0; y < ND; ++y) atomicAdd(Kp + (P.fb + x) + (size_t)N * (Q.fb + y), deg * Kbd[x * ND + y]);
    }
    unsigned long long cnt = nprimq;
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, d);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(a.primcount, cnt);
}

// Host-side launchers, one set per class (defined in the generated eri_class_*.cu).
struct ClassLaunchers {
    void (*jk)(const ClassWork&, const JKArgs&, int grid, cudaStream_t);
    int (*occupancy)(void);
    int la, lb, lc, ld;
};

#define QB_DEFINE_LAUNCHERS(LA, LB, LC, LD)                                                                  \
    static void qb_jk_launch_##LA##LB##LC##LD(const ClassWork& w, const JKArgs& a, int grid, cudaStream_t s) { \
        qb_jk_class_kernel<LA, LB, LC, LD><<<grid, 128, 0, s>>>(w, a);                                       \
    }                                                                                                        \
    static int qb_occ_##LA##LB##LC##LD(void) {                                                               \
        int nb = 0;                                                                                          \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, qb_jk_class_kernel<LA, LB, LC, LD>, 128, 0);       \
        return nb;                                                                                           \
    }
