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

// (ab|cd) block of one contracted shell quartet -> the six J'/K' blocks, scaled by the
// degeneracy factor, atomically added to the global accumulators.
template <class C>
__device__ __forceinline__ void qb_jk_digest(const ShellPair& P, const ShellPair& Q, double deg, const JKArgs& a,
                                             const double (&I)[C::NINT]) {
    constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND;
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
    double Jab[NA * NB] = {}, Jcd[NC * ND] = {}, Kac[NA * NC] = {}, Kad[NA * ND] = {}, Kbc[NB * NC] = {},
           Kbd[NB * ND] = {};
    if constexpr (C::NINT <= 162) {
#pragma unroll
        for (int x = 0; x < NA; ++x)
#pragma unroll
            for (int y = 0; y < NB; ++y)
#pragma unroll
                for (int z = 0; z < NC; ++z)
#pragma unroll
                    for (int u = 0; u < ND; ++u)
                        qb_digest(I[((x * NB + y) * NC + z) * ND + u], x * NB + y, z * ND + u, x * NC + z, x * ND + u,
                                  y * NC + z, y * ND + u, Dab, Dcd, Dac, Dad, Dbc, Dbd, Jab, Jcd, Kac, Kad, Kbc, Kbd);
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
                        qb_digest(I[((x * NB + y) * NC + z) * ND + u], x * NB + y, z * ND + u, x * NC + z, x * ND + u,
                                  y * NC + z, y * ND + u, Dab, Dcd, Dac, Dad, Dbc, Dbd, Jab, Jcd, Kac, Kad, Kbc, Kbd);
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

// One contracted quartet per thread (used for the classes whose per-warp accumulators
// do not fit in shared memory).
template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) qb_jk_class_kernel(const ClassWork w, const JKArgs a) {
    using C = EriClass<LA, LB, LC, LD>;
    const long long total = __ldg(w.offs + w.nbra);
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned nprimq = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const int i = qb_find_bra(w.offs, w.nbra, t);
        const int j = (int)(t - __ldg(w.offs + i));
        const ShellPair P = w.bra[i];
        const ShellPair Q = w.ket[j];
        double I[C::NINT];
        C::block(a.prims + P.prim0, P.nprim, a.prims + Q.prim0, Q.nprim, P.ABx, P.ABy, P.ABz, Q.ABx, Q.ABy, Q.ABz,
                 a.boys, I, nprimq);
        const double deg = (P.same ? 1.0 : 2.0) * (Q.same ? 1.0 : 2.0) * ((w.same && i == j) ? 1.0 : 2.0);
        qb_jk_digest<C>(P, Q, deg, a, I);
    }
    unsigned long long cnt = nprimq;
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, d);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(a.primcount, cnt);
}

#define QB_WARP_MAXNB 32       // bra primitive pairs whose ket counts are tabulated (more: recounted)
#define QB_WARP_MAXLEVEL 256   // primitive-quartet levels dealt out per pass

// Warp-cooperative variant: a warp takes G <= 32 contracted quartets (one per "owner"
// lane 0..G-1), pools all their significant primitive quartets and deals them out
// evenly over its 32 lanes in level order (the s-th primitive quartet of every owner,
// then the (s+1)-th, ...), so that the lanes of one round mostly serve distinct owners.
// Each lane adds its primitive quartet's VRR targets to the owner's accumulator row in
// shared memory as they are produced; the owners then run the HRR and the J/K
// digestion.  Lane utilisation no longer depends on how many primitive quartets
// survive the screening per contracted quartet, and the accumulators leave the
// register file.
template <int LA, int LB, int LC, int LD, int WPB, int G>
__global__ void __launch_bounds__(32 * WPB) qb_jk_warp_kernel(const ClassWork w, const JKArgs a) {
    using C = EriClass<LA, LB, LC, LD>;
    static_assert(G >= 1 && G <= 32, "owners per warp");
    constexpr int NTP = C::NT | 1;
    extern __shared__ double qb_dyn_smem[];
    __shared__ unsigned short s_cnt[WPB][G][QB_WARP_MAXNB];
    __shared__ int s_level[WPB][QB_WARP_MAXLEVEL + 1];
    __shared__ int s_prim0b[WPB][G], s_prim0k[WPB][G], s_nb[WPB][G], s_nk[WPB][G], s_tot[WPB][G];
    __shared__ unsigned char s_order[WPB][G];
    const unsigned FULL = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* acc = qb_dyn_smem + (size_t)warp * G * NTP;
    const long long total = __ldg(w.offs + w.nbra);
    const long long stride = (long long)gridDim.x * WPB * G;
    const float eps = (float)QB_PRIM_EPS;
    unsigned long long nprim_warp = 0;
    for (long long base = ((long long)blockIdx.x * WPB + warp) * G; base < total; base += stride) {
        const long long t = base + lane;
        const bool valid = lane < G && t < total;
        int i = 0, j = 0, mytot = 0;
        ShellPair P, Q;
        if (valid) {
            i = qb_find_bra(w.offs, w.nbra, t);
            j = (int)(t - __ldg(w.offs + i));
            P = w.bra[i];
            Q = w.ket[j];
            const PrimPair* bp = a.prims + P.prim0;
            const PrimPair* kp = a.prims + Q.prim0;
            // significant ket primitives per bra primitive: pairs are sorted by descending
            // |K|, so the counts are prefixes and the screening ends at the first miss
            if (Q.nprim > 0) {
                const float kmax_ket = qb_kabs(kp);
                for (int ib = 0; ib < P.nprim; ++ib) {
                    const float kb = qb_kabs(bp + ib);
                    if (kb * kmax_ket < eps) break;
                    int n = 1;
                    while (n < Q.nprim && kb * qb_kabs(kp + n) >= eps) ++n;
                    if (ib < QB_WARP_MAXNB) s_cnt[warp][lane][ib] = (unsigned short)n;
                    mytot += n;
                }
            }
            s_prim0b[warp][lane] = P.prim0;
            s_prim0k[warp][lane] = Q.prim0;
            s_nb[warp][lane] = P.nprim;
            s_nk[warp][lane] = Q.nprim;
        }
        // owners ranked by descending count (ties by lane)
        int rank = 0, maxtot = 0;
        for (int m = 0; m < G; ++m) {
            const int tm = __shfl_sync(FULL, mytot, m);
            rank += (tm > mytot) || (tm == mytot && m < lane);
            maxtot = max(maxtot, tm);
        }
        if (lane < G) {
            s_order[warp][rank] = (unsigned char)lane;
            s_tot[warp][rank] = mytot;
        }
        for (int e = lane; e < G * NTP; e += 32) acc[e] = 0.0;
        __syncwarp();
        // levels [l0, l1) at a time: s_level[s - l0] = sum_k (min(count_k, s) - min(count_k, l0))
        for (int l0 = 0; l0 < maxtot; l0 += QB_WARP_MAXLEVEL) {
            const int l1 = min(maxtot, l0 + QB_WARP_MAXLEVEL);
            for (int sl = l0 + lane; sl <= l1; sl += 32) {
                int v = 0;
                for (int k = 0; k < G; ++k) {
                    const int tk = s_tot[warp][k];
                    v += min(tk, sl) - min(tk, l0);
                }
                s_level[warp][sl - l0] = v;
            }
            __syncwarp();
            const int N = s_level[warp][l1 - l0];
            for (int r = lane; r < N; r += 32) {
                int lo = 0, hi = l1 - l0;   // s_level[lo] <= r < s_level[hi]
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (s_level[warp][mid] <= r) lo = mid; else hi = mid;
                }
                const int owner = s_order[warp][r - s_level[warp][lo]];
                // the owner's (l0 + lo)-th primitive quartet -> (bra ib, ket rem)
                int ib = 0, rem = l0 + lo;
                if (s_nb[warp][owner] <= QB_WARP_MAXNB) {
                    while (rem >= s_cnt[warp][owner][ib]) { rem -= s_cnt[warp][owner][ib]; ++ib; }
                } else {
                    const PrimPair* bp = a.prims + s_prim0b[warp][owner];
                    const PrimPair* kp = a.prims + s_prim0k[warp][owner];
                    const int nk = s_nk[warp][owner];
                    for (;;) {
                        const float kb = qb_kabs(bp + ib);
                        int n = 1;
                        while (n < nk && kb * qb_kabs(kp + n) >= eps) ++n;
                        if (rem < n) break;
                        rem -= n;
                        ++ib;
                    }
                }
                const PrimPair B = qb_load_pair(a.prims + s_prim0b[warp][owner] + ib);
                const PrimPair Kt = qb_load_pair(a.prims + s_prim0k[warp][owner] + rem);
                double* dst = acc + owner * NTP;
                C::prim(B, Kt, a.boys, [&](int k, double v) { atomicAdd(dst + k, v); });
            }
            if (lane == 0) nprim_warp += N;
            __syncwarp();
        }
        if (valid) {
            double I[C::NINT];
            C::hrr(acc + lane * NTP, P.ABx, P.ABy, P.ABz, Q.ABx, Q.ABy, Q.ABz, I);
            const double deg = (P.same ? 1.0 : 2.0) * (Q.same ? 1.0 : 2.0) * ((w.same && i == j) ? 1.0 : 2.0);
            qb_jk_digest<C>(P, Q, deg, a, I);
        }
        __syncwarp();
    }
    for (int d = 16; d > 0; d >>= 1) nprim_warp += __shfl_down_sync(FULL, nprim_warp, d);
    if (lane == 0 && nprim_warp) atomicAdd(a.primcount, nprim_warp);
}

// Host-side launchers, one set per class (defined in the generated eri_class_*.cu).
// Variant 0 runs one contracted quartet per thread (qb_jk_class_kernel); variant 1 the
// warp-cooperative kernel (qb_jk_warp_kernel), present when its accumulators fit in
// shared memory (warps_per_block > 0).
struct ClassLaunchers {
    void (*jk[2])(const ClassWork&, const JKArgs&, int grid, cudaStream_t);
    int (*occupancy[2])(void);   // resident blocks per SM (also sets the shared-memory limit)
    int la, lb, lc, ld;
    int warps_per_block;
    int preferred;               // default variant
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

#define QB_WARP_SMEM(LA, LB, LC, LD, WPB, G) \
    ((size_t)(WPB) * (G) * (EriClass<LA, LB, LC, LD>::NT | 1) * sizeof(double))

#define QB_DEFINE_WARP_LAUNCHERS(LA, LB, LC, LD, WPB, G)                                                      \
    static void qb_jkw_launch_##LA##LB##LC##LD(const ClassWork& w, const JKArgs& a, int grid, cudaStream_t s) { \
        qb_jk_warp_kernel<LA, LB, LC, LD, WPB, G>                                                               \
            <<<grid, 32 * (WPB), QB_WARP_SMEM(LA, LB, LC, LD, WPB, G), s>>>(w, a);                              \
    }                                                                                                        \
    static int qb_occw_##LA##LB##LC##LD(void) {                                                              \
        cudaFuncSetAttribute(qb_jk_warp_kernel<LA, LB, LC, LD, WPB, G>,                                          \
                             cudaFuncAttributeMaxDynamicSharedMemorySize,                                    \
                             (int)QB_WARP_SMEM(LA, LB, LC, LD, WPB, G));                                        \
        int nb = 0;                                                                                          \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, qb_jk_warp_kernel<LA, LB, LC, LD, WPB, G>, 32 * (WPB), \
                                                      QB_WARP_SMEM(LA, LB, LC, LD, WPB, G));                    \
        return nb;                                                                                           \
    }
