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
    const float4* __restrict__ prims32;    // (p, Px, Py, Pz) of prims in FP32
    const double* __restrict__ boys;
    const double* __restrict__ D;          // ratio-scaled density, column-major
    double* Jp;                            // J' accumulator (column-major nfun x nfun)
    double* Kp;                            // K' accumulator
    unsigned long long* primcount;         // primitive quartets evaluated (this class)
    int nfun;
    float prim_eps;                        // primitive-quartet threshold on the screening-key product
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
                 a.boys, I, nprimq, a.prim_eps);
        const double deg = (P.same ? 1.0 : 2.0) * (Q.same ? 1.0 : 2.0) * ((w.same && i == j) ? 1.0 : 2.0);
        qb_jk_digest<C>(P, Q, deg, a, I);
    }
    unsigned long long cnt = nprimq;
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, d);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(a.primcount, cnt);
}

#define QB_WARP_MAXNB 32       // bra primitive pairs whose ket counts are tabulated (more: recounted)
#define QB_WARP_MAXLEVEL 256   // primitive-quartet levels dealt out per pass
#define QB_WARP_WINDOW 128     // primitive quartets regrouped by Boys branch at a time

// Sum of the S accumulator rows of one owner (the HRR input).
template <int S>
struct QbRowSum {
    const double* p;
    int stride;
    __device__ __forceinline__ double operator[](int k) const {
        double v = p[k];
#pragma unroll
        for (int s = 1; s < S; ++s) v += p[s * stride + k];
        return v;
    }
};

// Column k*stride of an owner's S accumulator rows, summed (input of the bra HRR of one
// ket component: targets are stored e-major, k = e * NF + f).
template <int S>
struct QbColumnSum {
    const double* p;
    int stride, row;
    __device__ __forceinline__ double operator[](int k) const {
        double v = p[k * stride];
#pragma unroll
        for (int s = 1; s < S; ++s) v += p[s * row + k * stride];
        return v;
    }
};

// J/K digestion of one (ab|cd) block held in shared memory (Ib[ab * NCD + cd]) by a whole
// warp: every element of the six J'/K' blocks is summed by one lane over the other index
// pair (no reduction between lanes), scaled by the degeneracy factor and added to the
// global accumulators.  Same six products per integral as qb_jk_digest.
template <class C>
__device__ __forceinline__ void qb_jk_digest_warp(const ShellPair& P, const ShellPair& Q, double deg,
                                                  const JKArgs& a, const double* Ib, int lane) {
    constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND, NCD = NC * ND;
    const int N = a.nfun;
    const double* __restrict__ D = a.D;
    auto Dat = [&](int r, int c) { return __ldg(D + r + (size_t)N * c); };
    auto I = [&](int x, int y, int z, int u) { return Ib[(x * NB + y) * NCD + z * ND + u]; };
    for (int r = lane; r < NA * NB; r += 32) {   // J_ab = sum_cd (ab|cd) D_cd
        const int x = r / NB, y = r % NB;
        double s = 0.0;
        for (int z = 0; z < NC; ++z)
            for (int u = 0; u < ND; ++u) s = fma(Dat(Q.fa + z, Q.fb + u), I(x, y, z, u), s);
        atomicAdd(a.Jp + (P.fa + x) + (size_t)N * (P.fb + y), deg * s);
    }
    for (int r = lane; r < NC * ND; r += 32) {   // J_cd = sum_ab (ab|cd) D_ab
        const int z = r / ND, u = r % ND;
        double s = 0.0;
        for (int x = 0; x < NA; ++x)
            for (int y = 0; y < NB; ++y) s = fma(Dat(P.fa + x, P.fb + y), I(x, y, z, u), s);
        atomicAdd(a.Jp + (Q.fa + z) + (size_t)N * (Q.fb + u), deg * s);
    }
    for (int r = lane; r < NA * NC; r += 32) {   // K_ac = sum_bd (ab|cd) D_bd
        const int x = r / NC, z = r % NC;
        double s = 0.0;
        for (int y = 0; y < NB; ++y)
            for (int u = 0; u < ND; ++u) s = fma(Dat(P.fb + y, Q.fb + u), I(x, y, z, u), s);
        atomicAdd(a.Kp + (P.fa + x) + (size_t)N * (Q.fa + z), deg * s);
    }
    for (int r = lane; r < NA * ND; r += 32) {   // K_ad = sum_bc (ab|cd) D_bc
        const int x = r / ND, u = r % ND;
        double s = 0.0;
        for (int y = 0; y < NB; ++y)
            for (int z = 0; z < NC; ++z) s = fma(Dat(P.fb + y, Q.fa + z), I(x, y, z, u), s);
        atomicAdd(a.Kp + (P.fa + x) + (size_t)N * (Q.fb + u), deg * s);
    }
    for (int r = lane; r < NB * NC; r += 32) {   // K_bc = sum_ad (ab|cd) D_ad
        const int y = r / NC, z = r % NC;
        double s = 0.0;
        for (int x = 0; x < NA; ++x)
            for (int u = 0; u < ND; ++u) s = fma(Dat(P.fa + x, Q.fb + u), I(x, y, z, u), s);
        atomicAdd(a.Kp + (P.fb + y) + (size_t)N * (Q.fa + z), deg * s);
    }
    for (int r = lane; r < NB * ND; r += 32) {   // K_bd = sum_ac (ab|cd) D_ac
        const int y = r / ND, u = r % ND;
        double s = 0.0;
        for (int x = 0; x < NA; ++x)
            for (int z = 0; z < NC; ++z) s = fma(Dat(P.fa + x, Q.fa + z), I(x, y, z, u), s);
        atomicAdd(a.Kp + (P.fb + y) + (size_t)N * (Q.fb + u), deg * s);
    }
}

// Shared memory of one warp of the cooperative epilogue: (ab|f) and (ab|cd) of one quartet.
template <class C>
struct QbCoop {
    static constexpr int doubles = C::NA * C::NB * C::NF + C::NINT;
};

// Warp-cooperative variant: a warp takes G <= 32 contracted quartets (one per "owner"
// lane 0..G-1) and pools all their significant primitive quartets, dealt out evenly over
// its 32 lanes in level order (the s-th primitive quartet of every owner, then the
// (s+1)-th, ...).  REGROUP: every window of 128 pooled primitive quartets is first
// regrouped so that those on the Boys table branch (T < QB_BOYS_TMAX, decided in FP32)
// come before those on the asymptotic branch, and the warp runs one branch at a time.
// Lanes of a round that serve the same owner write different accumulator rows (their
// rank among them by __match_any_sync, capped at S-1) with atomicAdd; PLAIN: ranks
// 0..S-2, alone on their row, add without atomics.  The owners finally sum their rows
// and run the HRR and the J/K digestion.  Lane
// utilisation no longer depends on how many primitive quartets survive the screening
// per contracted quartet, and the accumulators leave the register file.  COOP: instead
// of each owner lane running its own HRR and digestion (hundreds of integrals per lane,
// spilled to local memory in the large classes), the warp takes the owners one at a
// time: the bra HRR with lanes over the ket components, the ket HRR with lanes over the
// bra function pairs, then qb_jk_digest_warp, all through shared memory.
template <int LA, int LB, int LC, int LD, int WPB, int G, int S, bool REGROUP, bool PLAIN, bool COOP>
__global__ void __launch_bounds__(32 * WPB) qb_jk_warp_kernel(const ClassWork w, const JKArgs a) {
    using C = EriClass<LA, LB, LC, LD>;
    static_assert(G >= 1 && G <= 32, "owners per warp");
    static_assert(S >= 1 && S <= 4, "accumulator rows per owner");
    static_assert(!PLAIN || S >= 2, "plain adds need a shared overflow row");
    constexpr int NTP = C::NT | 1;
    constexpr int ROW = G * NTP;                        // doubles between two rows of an owner
    constexpr int W = REGROUP ? QB_WARP_WINDOW : 32;    // items regrouped per window
    constexpr int NSUB = W / 32;
    constexpr int WS = REGROUP ? W : 1;
    extern __shared__ double qb_dyn_smem[];
    __shared__ unsigned short s_cnt[WPB][G][QB_WARP_MAXNB];
    __shared__ int s_level[WPB][QB_WARP_MAXLEVEL + 1];
    __shared__ int s_prim0b[WPB][G], s_prim0k[WPB][G], s_nb[WPB][G], s_nk[WPB][G], s_tot[WPB][G];
    __shared__ unsigned char s_order[WPB][G];
    __shared__ int s_wb[WPB][WS], s_wk[WPB][WS];        // window: bra / ket primitive-pair index
    __shared__ unsigned char s_wo[WPB][WS];              // window: owner
    const unsigned FULL = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lanes_below = (1u << lane) - 1u;
    constexpr int PER_WARP = S * ROW + (COOP ? QbCoop<C>::doubles : 0);
    double* acc = qb_dyn_smem + (size_t)warp * PER_WARP;
    const long long total = __ldg(w.offs + w.nbra);
    const long long stride = (long long)gridDim.x * WPB * G;
    const float eps = a.prim_eps;
    unsigned long long nprim_warp = 0;

    // the owner's q-th significant primitive quartet -> (bra, ket) primitive-pair indices
    auto decode = [&](int owner, int q, int& bpi, int& kpi) {
        int ib = 0, rem = q;
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
        bpi = s_prim0b[warp][owner] + ib;
        kpi = s_prim0k[warp][owner] + rem;
    };
    // one primitive quartet into the owner's accumulator rows (all lanes call it)
    auto accumulate = [&](bool act, int owner, int bpi, int kpi) {
        const unsigned same = __match_any_sync(FULL, act ? owner : 64 + lane);
        const int rank = __popc(same & lanes_below);
        if (act) {
            const bool plain = PLAIN && rank < S - 1;
            double* dst = acc + (size_t)min(rank, S - 1) * ROW + owner * NTP;
            const PrimPair B = qb_load_pair(a.prims + bpi);
            const PrimPair Kt = qb_load_pair(a.prims + kpi);
            C::prim(B, Kt, a.boys, [&](int k, double v) {
                if (plain) dst[k] += v;
                else atomicAdd(dst + k, v);
            });
        }
        __syncwarp();
    };

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
        for (int e = lane; e < S * ROW; e += 32) acc[e] = 0.0;
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
            // pooled item r -> (owner, owner's primitive-quartet index)
            auto item = [&](int r, int& owner, int& q) {
                int lo = 0, hi = l1 - l0;   // s_level[lo] <= r < s_level[hi]
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (s_level[warp][mid] <= r) lo = mid; else hi = mid;
                }
                owner = s_order[warp][r - s_level[warp][lo]];
                q = l0 + lo;
            };
            for (int w0 = 0; w0 < N; w0 += W) {
                const int nw = min(W, N - w0);
                if constexpr (REGROUP) {
                    // regroup the window: Boys table branch first, asymptotic branch after
                    int own[NSUB], bpi[NSUB], kpi[NSUB];
                    unsigned tab[NSUB], vmask[NSUB];
                    int ntab = 0;
#pragma unroll
                    for (int u = 0; u < NSUB; ++u) {
                        const bool act = 32 * u + lane < nw;
                        bool tb = false;
                        own[u] = 0; bpi[u] = 0; kpi[u] = 0;
                        if (act) {
                            int q;
                            item(w0 + 32 * u + lane, own[u], q);
                            decode(own[u], q, bpi[u], kpi[u]);
                            const float4 pb = __ldg(a.prims32 + bpi[u]);
                            const float4 pk = __ldg(a.prims32 + kpi[u]);
                            const float dx = pb.y - pk.y, dy = pb.z - pk.z, dz = pb.w - pk.w;
                            const float T = __fdividef(pb.x * pk.x, pb.x + pk.x) * (dx * dx + dy * dy + dz * dz);
                            tb = T < (float)QB_BOYS_TMAX;
                        }
                        tab[u] = __ballot_sync(FULL, tb);
                        vmask[u] = __ballot_sync(FULL, act);
                        ntab += __popc(tab[u]);
                    }
                    int seen_tab = 0, seen_asy = 0;
#pragma unroll
                    for (int u = 0; u < NSUB; ++u) {
                        const unsigned asy = vmask[u] & ~tab[u];
                        if (vmask[u] & (1u << lane)) {
                            const int pos = (tab[u] & (1u << lane)) ? seen_tab + __popc(tab[u] & lanes_below)
                                                                    : ntab + seen_asy + __popc(asy & lanes_below);
                            s_wb[warp][pos] = bpi[u];
                            s_wk[warp][pos] = kpi[u];
                            s_wo[warp][pos] = (unsigned char)own[u];
                        }
                        seen_tab += __popc(tab[u]);
                        seen_asy += __popc(asy);
                    }
                    __syncwarp();
#pragma unroll 1
                    for (int u = 0; u < NSUB; ++u) {
                        const int idx = 32 * u + lane;
                        if (32 * u >= nw) break;
                        const bool act = idx < nw;
                        accumulate(act, act ? s_wo[warp][idx] : 0, act ? s_wb[warp][idx] : 0,
                                   act ? s_wk[warp][idx] : 0);
                    }
                } else {
                    const bool act = lane < nw;
                    int owner = 0, bp = 0, kp = 0;
                    if (act) {
                        int q;
                        item(w0 + lane, owner, q);
                        decode(owner, q, bp, kp);
                    }
                    accumulate(act, owner, bp, kp);
                }
            }
            if (lane == 0) nprim_warp += N;
            __syncwarp();
        }
        if constexpr (COOP) {
            constexpr int NAB = C::NA * C::NB, NCD = C::NC * C::ND, NF = C::NF;
            double* Tb = acc + S * ROW;   // (ab|f) of the current owner, [ab][f]
            double* Ib = Tb + NAB * NF;   // (ab|cd), [ab][cd]
            const unsigned vmask = __ballot_sync(FULL, valid);   // owners 0..popc-1 (consecutive quartets)
            const int nown = __popc(vmask);
            for (int g = 0; g < nown; ++g) {
                const int ig = __shfl_sync(FULL, i, g), jg = __shfl_sync(FULL, j, g);
                const ShellPair Pg = w.bra[ig];
                const ShellPair Qg = w.ket[jg];
                for (int f = lane; f < NF; f += 32)
                    C::hrr_bra(QbColumnSum<S>{acc + g * NTP + f, NF, ROW}, Pg.ABx, Pg.ABy, Pg.ABz,
                               [&](int ab, double v) { Tb[ab * NF + f] = v; });
                __syncwarp();
                for (int ab = lane; ab < NAB; ab += 32)
                    C::hrr_ket(Tb + ab * NF, Qg.ABx, Qg.ABy, Qg.ABz, [&](int cd, double v) { Ib[ab * NCD + cd] = v; });
                __syncwarp();
                const double deg = (Pg.same ? 1.0 : 2.0) * (Qg.same ? 1.0 : 2.0) * ((w.same && ig == jg) ? 1.0 : 2.0);
                qb_jk_digest_warp<C>(Pg, Qg, deg, a, Ib, lane);
                __syncwarp();
            }
        } else {
            if (valid) {
                double I[C::NINT];
                C::hrr(QbRowSum<S>{acc + lane * NTP, ROW}, P.ABx, P.ABy, P.ABz, Q.ABx, Q.ABy, Q.ABz, I);
                const double deg = (P.same ? 1.0 : 2.0) * (Q.same ? 1.0 : 2.0) * ((w.same && i == j) ? 1.0 : 2.0);
                qb_jk_digest<C>(P, Q, deg, a, I);
            }
        }
        __syncwarp();
    }
    for (int d = 16; d > 0; d >>= 1) nprim_warp += __shfl_down_sync(FULL, nprim_warp, d);
    if (lane == 0 && nprim_warp) atomicAdd(a.primcount, nprim_warp);
}

// Reduce-scatter of eight values over the eight lanes of an aligned lane segment (j8 =
// lane & 7), staged through shared memory: every lane stores its eight values in its own
// row of the warp's staging area (rows of 9 doubles, so that the reads below spread over
// the banks), the warp synchronises, and lane j8 sums value j8 of the eight rows of its
// segment and adds the sum to row[j8].  Eight FP64 adds per eight values and no atomics;
// about half the instructions of a register-shuffle exchange (three halving stages).  Two staging areas alternate by batch parity, so
// one warp synchronisation per batch orders every store after the reads of the batch that
// last used the area.
__device__ __forceinline__ void qb_stage8_add(double* stage, double* row, int lane, int j8, double v0, double v1,
                                             double v2, double v3, double v4, double v5, double v6, double v7) {
    double* my = stage + lane * 9;
    my[0] = v0; my[1] = v1; my[2] = v2; my[3] = v3; my[4] = v4; my[5] = v5; my[6] = v6; my[7] = v7;
    __syncwarp();
    const double* sg = stage + (lane & ~7) * 9 + j8;
    const double s = ((sg[0] + sg[9]) + (sg[18] + sg[27])) + ((sg[36] + sg[45]) + (sg[54] + sg[63]));
    row[j8] += s;
}

#define QB_SEG_MAXNB 16   // bra primitive pairs whose ket counts the segmented kernel tabulates

// Segmented kernel (classes with many contracted targets).  A warp takes a batch of G <= 32
// contracted quartets ("owners"; G from the class's quartets per warp, at least four
// batches per warp), sorts them by their number of significant primitive quartets and
// runs them four at a time, one per 8-lane segment: in each round a segment's lanes
// evaluate eight of its owner's primitive quartets (lanes past the owner's count run a
// valid primitive quartet with a zero prefactor), and every group of eight VRR targets is
// reduce-scattered over the segment (qb_stage8_add) into the owner's shared-memory row, one
// plain add per lane and target: no atomics, so no compare-and-swap retries when many
// lanes serve one quartet, and no accumulator in registers or local memory.  Sorting makes
// the four owners of a wave need similar round counts.  After a wave the whole warp runs
// each owner's HRR and J/K digestion from shared memory (as the cooperative epilogue of
// qb_jk_warp_kernel).
template <class C>
struct QbSeg {
    static constexpr int NR = C::NSEGB * 8;   // row length: emission slots of the targets
    static constexpr int NI = C::NINT > C::NT ? C::NINT : C::NT;
    static constexpr int STAGE = 2 * 32 * 9;    // two staging areas of the reduce-scatter
    static constexpr int HRRBUF = C::NA * C::NB * C::NF + NI;
    // per warp: four rows, then the HRR buffers, which the staging areas share (the rounds
    // and the HRR phase of a wave never overlap)
    static constexpr int doubles = 4 * NR + (HRRBUF > STAGE ? HRRBUF : STAGE);
};

template <int LA, int LB, int LC, int LD, int WPB>
__global__ void __launch_bounds__(32 * WPB) qb_jk_seg_kernel(const ClassWork w, const JKArgs a) {
    using C = EriClass<LA, LB, LC, LD>;
    constexpr int GMAX = 32;
    constexpr int NR = QbSeg<C>::NR;
    constexpr int NAB = C::NA * C::NB, NCD = C::NC * C::ND, NF = C::NF, NT = C::NT;
    extern __shared__ double qb_dyn_smem[];
    __shared__ unsigned short s_cnt[WPB][GMAX][QB_SEG_MAXNB];
    __shared__ int s_prim0b[WPB][GMAX], s_prim0k[WPB][GMAX], s_nb[WPB][GMAX], s_nk[WPB][GMAX], s_tot[WPB][GMAX];
    __shared__ unsigned char s_order[WPB][GMAX];
    const unsigned FULL = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, seg = lane >> 3, j8 = lane & 7;
    double* rows = qb_dyn_smem + (size_t)warp * QbSeg<C>::doubles;
    double* Tb = rows + 4 * NR;    // (ab|f) of the current owner, [ab][f]
    double* Ib = Tb + NAB * NF;    // the owner's targets in (e, f) order, then its (ab|cd) block
    double* stage = Tb;            // reduce-scatter staging (two areas) during the rounds
    const long long total = __ldg(w.offs + w.nbra);
    const long long nwarps = (long long)gridDim.x * WPB;
    // owners per batch: a multiple of 4 in [4, 32], about a sixth of the quartets per warp
    const int G = (int)max(4LL, min((long long)GMAX, (total / nwarps / 6) & ~3LL));
    const long long stride = nwarps * G;
    const float eps = a.prim_eps;
    unsigned long long nprim = 0;

    auto decode = [&](int owner, int q, int& bpi, int& kpi) {
        int ib = 0, rem = q;
        if (s_nb[warp][owner] <= QB_SEG_MAXNB) {
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
        bpi = s_prim0b[warp][owner] + ib;
        kpi = s_prim0k[warp][owner] + rem;
    };

    for (long long base = ((long long)blockIdx.x * WPB + warp) * G; base < total; base += stride) {
        const long long t = base + lane;
        const bool valid = lane < G && t < total;
        int i = 0, j = 0, mytot = 0;
        if (valid) {
            i = qb_find_bra(w.offs, w.nbra, t);
            j = (int)(t - __ldg(w.offs + i));
            const ShellPair P = w.bra[i];
            const ShellPair Q = w.ket[j];
            const PrimPair* bp = a.prims + P.prim0;
            const PrimPair* kp = a.prims + Q.prim0;
            if (Q.nprim > 0) {
                const float kmax_ket = qb_kabs(kp);
                for (int ib = 0; ib < P.nprim; ++ib) {
                    const float kb = qb_kabs(bp + ib);
                    if (kb * kmax_ket < eps) break;
                    int n = 1;
                    while (n < Q.nprim && kb * qb_kabs(kp + n) >= eps) ++n;
                    if (ib < QB_SEG_MAXNB) s_cnt[warp][lane][ib] = (unsigned short)n;
                    mytot += n;
                }
            }
            s_prim0b[warp][lane] = P.prim0;
            s_prim0k[warp][lane] = Q.prim0;
            s_nb[warp][lane] = P.nprim;
            s_nk[warp][lane] = Q.nprim;
        }
        // valid owners (a prefix of the lanes) ranked by descending count, ties by lane:
        // positions 0..nown-1 of s_order are the valid owners
        int rank = 0;
        for (int m = 0; m < G; ++m) {
            const int tm = __shfl_sync(FULL, mytot, m);
            rank += (tm > mytot) || (tm == mytot && m < lane);
        }
        if (lane < G) {
            s_order[warp][rank] = (unsigned char)lane;
            s_tot[warp][rank] = mytot;
        }
        const int nown = __popc(__ballot_sync(FULL, valid));
        __syncwarp();
        for (int w0 = 0; w0 < nown; w0 += 4) {
            const int o = w0 + seg;
            const bool has = o < nown;
            const int ow = s_order[warp][has ? o : w0];
            const int tot = has ? s_tot[warp][o] : 0;
            const int rounds = (s_tot[warp][w0] + 7) >> 3;   // the wave's largest count
            for (int e = lane; e < 4 * NR; e += 32) rows[e] = 0.0;
            __syncwarp();
            double* row = rows + seg * NR;
            for (int r = 0; r < rounds; ++r) {
                const int q = r * 8 + j8;
                const bool act = q < tot;
                int bpi = s_prim0b[warp][ow], kpi = s_prim0k[warp][ow];
                if (act) decode(ow, q, bpi, kpi);
                PrimPair B = qb_load_pair(a.prims + bpi);
                const PrimPair Kt = qb_load_pair(a.prims + kpi);
                if (!act) B.K = 0.0;   // zero prefactor: every target of this lane is zero
                C::prim_seg(B, Kt, a.boys,
                            [&](int b, double v0, double v1, double v2, double v3, double v4, double v5, double v6,
                                double v7) {
                                qb_stage8_add(stage + (b & 1) * (32 * 9), row + 8 * b, lane, j8, v0, v1, v2, v3, v4,
                                              v5, v6, v7);
                            });
            }
            if (j8 == 0) nprim += tot;
            __syncwarp();
            const int nw = min(4, nown - w0);
            for (int g = 0; g < nw; ++g) {
                const int og = s_order[warp][w0 + g];
                const int ig = __shfl_sync(FULL, i, og), jg = __shfl_sync(FULL, j, og);
                const ShellPair Pg = w.bra[ig];
                const ShellPair Qg = w.ket[jg];
                const unsigned short* pos = C::seg_pos();
                const double* rg = rows + g * NR;
                for (int k = lane; k < NT; k += 32) Ib[k] = rg[pos[k]];
                __syncwarp();
                for (int f = lane; f < NF; f += 32)
                    C::hrr_bra(QbColumnSum<1>{Ib + f, NF, 0}, Pg.ABx, Pg.ABy, Pg.ABz,
                               [&](int ab, double v) { Tb[ab * NF + f] = v; });
                __syncwarp();
                for (int ab = lane; ab < NAB; ab += 32)
                    C::hrr_ket(Tb + ab * NF, Qg.ABx, Qg.ABy, Qg.ABz, [&](int cd, double v) { Ib[ab * NCD + cd] = v; });
                __syncwarp();
                const double deg = (Pg.same ? 1.0 : 2.0) * (Qg.same ? 1.0 : 2.0) * ((w.same && ig == jg) ? 1.0 : 2.0);
                qb_jk_digest_warp<C>(Pg, Qg, deg, a, Ib, lane);
                __syncwarp();
            }
        }
        __syncwarp();
    }
    for (int d = 16; d > 0; d >>= 1) nprim += __shfl_down_sync(FULL, nprim, d);
    if (lane == 0 && nprim) atomicAdd(a.primcount, nprim);
}

// Host-side launchers, one set per class (defined in the generated eri_class_*.cu).
// Variant 0 runs one contracted quartet per thread (qb_jk_class_kernel); variants 1..4
// are configurations of the warp-cooperative kernel, variant 5 the segmented kernel (null
// where not compiled).
#define QB_NVARIANT 6
typedef void (*QbSchwarzLaunch)(const ShellPair* pairs, int n, const PrimPair* prims, const double* boys,
                                const double* ratio, double* Q, cudaStream_t s);
typedef void (*QbPrimKeyLaunch)(const ShellPair* pairs, int n, PrimPair* prims, const double* boys, unsigned* keymax,
                                cudaStream_t s);
struct ClassLaunchers {
    void (*jk[QB_NVARIANT])(const ClassWork&, const JKArgs&, int grid, cudaStream_t);
    int (*occupancy[QB_NVARIANT])(void);   // resident blocks per SM (also sets the shared-memory limit)
    int la, lb, lc, ld;
    int preferred;                         // default variant
    QbSchwarzLaunch schwarz;               // diagonal classes (ab|ab): Schwarz factors of pair class (a, b)
    QbPrimKeyLaunch primkey;               // diagonal classes: primitive Schwarz keys of pair class (a, b)
};

// Schwarz factors Q_ab = max over components sqrt|(ab|ab)| of one pair class from the
// class's own quartet code with every primitive quartet: the shell integrals times the per-function ratios r_a r_b of
// the basis weights (weights factor as ratio(function) x coefficient(primitive)).
template <int LA, int LB>
__global__ void __launch_bounds__(128) qb_schwarz_class_kernel(const ShellPair* __restrict__ pairs, int n,
                                                               const PrimPair* __restrict__ prims,
                                                               const double* __restrict__ boys,
                                                               const double* __restrict__ ratio,
                                                               double* __restrict__ Q) {
    using C = EriClass<LA, LB, LA, LB>;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const ShellPair P = pairs[k];
    double I[C::NINT];
    unsigned cnt = 0;
    // every primitive quartet (no |K_ab K_cd| cut-off): a distant pair's (ab|ab) is tiny, yet
    // Q_ab Q_cd with a compact (cd) can still pass the quartet threshold
    C::block(prims + P.prim0, P.nprim, prims + P.prim0, P.nprim, P.ABx, P.ABy, P.ABz, P.ABx, P.ABy, P.ABz, boys, I,
             cnt, 0.0);
    double mx = 0.0;
    for (int x = 0; x < C::NA; ++x)
        for (int y = 0; y < C::NB; ++y) {
            const double r = __ldg(ratio + P.fa + x) * __ldg(ratio + P.fb + y);
            mx = fmax(mx, fabs(I[((x * C::NB + y) * C::NA + x) * C::NB + y]) * r * r);
        }
    Q[k] = sqrt(mx);
}

// Primitive Schwarz factors of one pair class: for every kept primitive pair (ab) of every
// shell pair, key = sqrt(max over components |(ab|ab)|) of the ratio-free shells (the
// class's own quartet code on the one primitive quartet (ab|ab)), stored as the pair's
// FP32 screening key; keymax receives the largest key (positive floats order as their bits).
template <int LA, int LB>
__global__ void __launch_bounds__(128) qb_prim_key_kernel(const ShellPair* __restrict__ pairs, int n,
                                                          PrimPair* prims, const double* __restrict__ boys,
                                                          unsigned* keymax) {
    using C = EriClass<LA, LB, LA, LB>;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const ShellPair P = pairs[k];
    float kmax = 0.f;
    for (int u = 0; u < P.nprim; ++u) {
        PrimPair* pp = prims + P.prim0 + u;
        double I[C::NINT];
        unsigned cnt = 0;
        C::block(pp, 1, pp, 1, P.ABx, P.ABy, P.ABz, P.ABx, P.ABy, P.ABz, boys, I, cnt, 0.f);
        double mx = 0.0;
        for (int x = 0; x < C::NA; ++x)
            for (int y = 0; y < C::NB; ++y) mx = fmax(mx, fabs(I[((x * C::NB + y) * C::NA + x) * C::NB + y]));
        const float key = (float)sqrt(mx);
        reinterpret_cast<float*>(&pp->pad)[0] = key;
        kmax = fmaxf(kmax, key);
    }
    atomicMax(keymax, __float_as_uint(kmax));
}

#define QB_DEFINE_SCHWARZ_LAUNCHER(LA, LB)                                                                     \
    static void qb_schwarz_launch_##LA##LB##LA##LB(const ShellPair* p, int n, const PrimPair* prims,           \
                                                   const double* boys, const double* ratio, double* Q,         \
                                                   cudaStream_t s) {                                           \
        if (n > 0) qb_schwarz_class_kernel<LA, LB><<<(n + 127) / 128, 128, 0, s>>>(p, n, prims, boys, ratio, Q); \
    }                                                                                                          \
    static void qb_primkey_launch_##LA##LB##LA##LB(const ShellPair* p, int n, PrimPair* prims,                 \
                                                   const double* boys, unsigned* keymax, cudaStream_t s) {     \
        if (n > 0) qb_prim_key_kernel<LA, LB><<<(n + 127) / 128, 128, 0, s>>>(p, n, prims, boys, keymax);     \
    }

#define QB_DEFINE_LAUNCHERS(LA, LB, LC, LD)                                                                  \
    static void qb_jk_launch_##LA##LB##LC##LD(const ClassWork& w, const JKArgs& a, int grid, cudaStream_t s) { \
        qb_jk_class_kernel<LA, LB, LC, LD><<<grid, 128, 0, s>>>(w, a);                                       \
    }                                                                                                        \
    static int qb_occ_##LA##LB##LC##LD(void) {                                                               \
        int nb = 0;                                                                                          \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, qb_jk_class_kernel<LA, LB, LC, LD>, 128, 0);       \
        return nb;                                                                                           \
    }

#define QB_WARP_SMEM(LA, LB, LC, LD, WPB, G, S, COOP)                                   \
    ((size_t)(WPB) * ((S) * (G) * (EriClass<LA, LB, LC, LD>::NT | 1) +                     \
                      ((COOP) ? QbCoop<EriClass<LA, LB, LC, LD>>::doubles : 0)) * sizeof(double))

// Warp-kernel configuration V of class LA LB LC LD.
#define QB_DEFINE_WARP_LAUNCHERS(V, LA, LB, LC, LD, WPB, G, S, RG, PL, CO)                                   \
    static void qb_jkw##V##_launch_##LA##LB##LC##LD(const ClassWork& w, const JKArgs& a, int grid,          \
                                                    cudaStream_t s) {                                        \
        qb_jk_warp_kernel<LA, LB, LC, LD, WPB, G, S, RG, PL, CO>                                             \
            <<<grid, 32 * (WPB), QB_WARP_SMEM(LA, LB, LC, LD, WPB, G, S, CO), s>>>(w, a);                    \
    }                                                                                                        \
    static int qb_occw##V##_##LA##LB##LC##LD(void) {                                                         \
        cudaFuncSetAttribute(qb_jk_warp_kernel<LA, LB, LC, LD, WPB, G, S, RG, PL, CO>,                        \
                             cudaFuncAttributeMaxDynamicSharedMemorySize,                                    \
                             (int)QB_WARP_SMEM(LA, LB, LC, LD, WPB, G, S, CO));                              \
        int nb = 0;                                                                                          \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb,                                                   \
                                                      qb_jk_warp_kernel<LA, LB, LC, LD, WPB, G, S, RG, PL, CO>, \
                                                      32 * (WPB), QB_WARP_SMEM(LA, LB, LC, LD, WPB, G, S, CO)); \
        return nb;                                                                                           \
    }

#define QB_SEG_SMEM(LA, LB, LC, LD, WPB) ((size_t)(WPB) * QbSeg<EriClass<LA, LB, LC, LD>>::doubles * sizeof(double))

// Segmented-kernel configuration V of class LA LB LC LD (WPB warps per block).
#define QB_DEFINE_SEG_LAUNCHERS(V, LA, LB, LC, LD, WPB)                                                      \
    static void qb_jkw##V##_launch_##LA##LB##LC##LD(const ClassWork& w, const JKArgs& a, int grid,          \
                                                    cudaStream_t s) {                                        \
        qb_jk_seg_kernel<LA, LB, LC, LD, WPB><<<grid, 32 * (WPB), QB_SEG_SMEM(LA, LB, LC, LD, WPB), s>>>(w, a); \
    }                                                                                                        \
    static int qb_occw##V##_##LA##LB##LC##LD(void) {                                                         \
        cudaFuncSetAttribute(qb_jk_seg_kernel<LA, LB, LC, LD, WPB>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             (int)QB_SEG_SMEM(LA, LB, LC, LD, WPB));                                         \
        int nb = 0;                                                                                          \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, qb_jk_seg_kernel<LA, LB, LC, LD, WPB>, 32 * (WPB),   \
                                                      QB_SEG_SMEM(LA, LB, LC, LD, WPB));                     \
        return nb;                                                                                           \
    }
