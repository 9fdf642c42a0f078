// Batched closed-shell Hartree–Fock: hundreds of independent small molecules
// (4-256 functions each, s and p shells) solved together on one GPU.
//
// The reference solves one molecule per runHartreeFock call (src/HartreeFock.jl:953-1046),
// building the full N^4 ERI tensor up front (initializeHartreeFock, :178-210) and
// contracting it with the density every iteration (getGcore, :305-319).  Here all
// molecules share each launch:
//   integrals (once): one-body S and H = T + V for every molecule in one kernel; the
//     shell pairs of all molecules (never across molecules) with their Schwarz factors,
//     grouped by pair class and sorted per molecule by Q; per angular-momentum class a
//     work list of canonical shell quartets with Q_ab Q_cd >= schwarz; the generated
//     HGP class code evaluates every listed quartet once and stores its integral block
//     (structure of arrays, coalesced).
//   SCF iterations (CUDA graph, several iterations per launch): per class one kernel
//     digests the stored blocks of every unconverged molecule into its J' and K'
//     accumulators (the fused digestion of the direct J/K path); then one thread block
//     per molecule builds F = H + 2J - K and the energy, applies Pulay DIIS in the
//     orthonormal basis X = S^{-1/2} (getOrthonormalization(:Symmetric),
//     HartreeFock.jl:39-42), diagonalises X^T F X by Jacobi rotations started from the
//     previous eigenvectors (a nearly diagonal matrix after the first iterations, so a
//     few sweeps suffice), and forms the new density and the convergence tests.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>
#include "qb_internal.h"
#include "qb_dense.cuh"
#include "eri_class_0000.cuh"
#include "eri_class_1000.cuh"
#include "eri_class_1010.cuh"
#include "eri_class_1100.cuh"
#include "eri_class_1110.cuh"
#include "eri_class_1111.cuh"

#define QB_TRY(expr)                  \
    do {                              \
        const int _rc = (expr);       \
        if (_rc != QB_OK) return _rc; \
    } while (0)
#define QB_CUDA(ctx, call) QB_TRY(qb_cuda_check((ctx), (call), #call))

#define QB_BATCH_MAXN 256
#define QB_BATCH_DIIS 15                   // largest DIIS subspace (defaultDIISsize, HartreeFock.jl:16)
#define QB_BATCH_SLOTS (QB_BATCH_DIIS + 1) // history slots: the subspace plus the entry being added
#define QB_BATCH_RESET 4e-13               // resetThreshold = 1000 getAtolVal(Float64) (HartreeFock.jl:1337)
#define QB_BATCH_NCLASS 6
#define QB_BATCH_THREADS 256

namespace {

struct BatchWork {           // one class: quartets t in [0, offs[nbra])
    const ShellPair* bra;    // bra pairs (pair class X)
    const ShellPair* ket;    // ket pairs (pair class Y); same array as bra when X == Y
    const long long* offs;   // nbra + 1 exclusive prefix of quartets per bra
    const int* kstart;       // first ket (index into ket) of each bra's molecule segment
    int nbra;
    int same;                // X == Y
};

// A contiguous range of one class's stored quartets, all of one molecule (bra pairs are
// sorted by molecule, and every bra's kets lie in its own molecule): the digest of an
// iteration visits a chunk only while its molecule iterates.
struct DigestChunk {
    long long t0, t1;        // quartets [t0, t1)
    int b0, b1;              // bras [b0, b1) own them (offs[b0] <= t0, offs[b1] >= t1)
    int mol, pad;
};
#define QB_DIGEST_CHUNK 2048        // quartets per digest block of a molecule with much work in a class
#define QB_DIGEST_CHUNK_SMALL 512   // ... and of the others (enough blocks to spread a straggler)

struct MolDev {
    int n, nocc, conv, iter;   // conv: 0 iterating, 1 converged, 2 stopped at max_iter, 3 failed
    int dlen, sweeps;          // DIIS subspace: dlist[0..dlen) slot ids, oldest first
    int iter0, restarted;      // iterations before a restart from the core-Hamiltonian guess
    int dlist[QB_BATCH_SLOTS];
    double dEs[QB_BATCH_SLOTS];   // per-spin energy of each slot's entry
    double E, Eprev, dE, rmsD;
    double *S, *H, *X, *F, *D, *Dt, *Do, *Jp, *Kp, *Cp, *W1, *W2, *W3, *W4, *W5, *W6;
    double *Fh, *Eh, *B, *eps, *wt;
    const double* ratio;
};

struct StepParams {
    double thr_e, thr_d;
    int max_iter, diis, sweeps, eig;   // eig 0: tridiagonal occupied-subspace solver, 1: Jacobi
    int fallback;                      // > 0: restart from the core-Hamiltonian guess after this many
};

// ---------------------------------------------------------------------------
// Visiting order of a class's quartets for the store kernel: by primitive-pair product
// (bucket 15 - floor(log2(nprim_bra * nprim_ket)), largest first), so that the lanes of a
// warp evaluate quartets of similar primitive counts (mixed bases pair 1- and 36-primitive
// shell pairs; a warp waits for its longest lane).  Counting sort: histogram, exclusive
// scan, scatter (order within a bucket is arbitrary; every quartet keeps its own slot).
#define QB_COST_BUCKETS 16
__device__ __forceinline__ int qb_cost_bucket(const BatchWork& w, long long t) {
    const int i = qb_find_bra(w.offs, w.nbra, t);
    const int j = __ldg(w.kstart + i) + (int)(t - __ldg(w.offs + i));
    const unsigned c = (unsigned)max(1, w.bra[i].nprim) * (unsigned)max(1, w.ket[j].nprim);
    return QB_COST_BUCKETS - 1 - min(QB_COST_BUCKETS - 1, 31 - __clz(c));
}

__global__ void qb_batch_cost_hist_kernel(const BatchWork w, unsigned* __restrict__ hist) {
    __shared__ unsigned h[QB_COST_BUCKETS];
    if (threadIdx.x < QB_COST_BUCKETS) h[threadIdx.x] = 0;
    __syncthreads();
    const long long total = __ldg(w.offs + w.nbra);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x)
        atomicAdd(&h[qb_cost_bucket(w, t)], 1u);
    __syncthreads();
    if (threadIdx.x < QB_COST_BUCKETS && h[threadIdx.x]) atomicAdd(hist + threadIdx.x, h[threadIdx.x]);
}

__global__ void qb_batch_cost_scan_kernel(unsigned* hist) {   // counts -> exclusive prefix (one thread)
    unsigned acc = 0;
    for (int b = 0; b < QB_COST_BUCKETS; ++b) {
        const unsigned v = hist[b];
        hist[b] = acc;
        acc += v;
    }
}

__global__ void qb_batch_cost_scatter_kernel(const BatchWork w, unsigned* __restrict__ cursor,
                                             unsigned* __restrict__ perm) {
    const long long total = __ldg(w.offs + w.nbra);
    const int lane = threadIdx.x & 31;
    for (long long t0 = (long long)blockIdx.x * blockDim.x; t0 < total; t0 += (long long)gridDim.x * blockDim.x) {
        const long long t = t0 + threadIdx.x;
        const bool act = t < total;
        const int b = act ? qb_cost_bucket(w, t) : QB_COST_BUCKETS + lane;   // inactive lanes: unique keys
        const unsigned same = __match_any_sync(0xffffffffu, b);
        const int leader = __ffs(same) - 1;
        unsigned base = 0;
        if (act && lane == leader) base = atomicAdd(cursor + b, (unsigned)__popc(same));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (act) perm[base + __popc(same & ((1u << lane) - 1u))] = (unsigned)t;
    }
}

// ---------------------------------------------------------------------------
template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) qb_batch_store_kernel(const BatchWork w, const PrimPair* __restrict__ prims,
                                                             const double* __restrict__ boys, double* __restrict__ out,
                                                             unsigned long long* primcount,
                                                             const unsigned* __restrict__ perm) {
    using C = EriClass<LA, LB, LC, LD>;
    const long long total = __ldg(w.offs + w.nbra);
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned nprimq = 0;
    for (long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += stride) {
        const long long t = __ldg(perm + u);   // quartets visited in cost order, stored in place
        const int i = qb_find_bra(w.offs, w.nbra, t);
        const int j = __ldg(w.kstart + i) + (int)(t - __ldg(w.offs + i));
        const ShellPair P = w.bra[i];
        const ShellPair Q = w.ket[j];
        double I[C::NINT];
        C::block(prims + P.prim0, P.nprim, prims + Q.prim0, Q.nprim, P.ABx, P.ABy, P.ABz, Q.ABx, Q.ABy, Q.ABz, boys,
                 I, nprimq);
#pragma unroll
        for (int k = 0; k < C::NINT; ++k) out[(size_t)k * total + t] = I[k];
    }
    unsigned long long cnt = nprimq;
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, d);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(primcount, cnt);
}

// One thread block per chunk; the blocks of converged molecules return after one read.
template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) qb_batch_digest_kernel(const BatchWork w, const DigestChunk* __restrict__ chunks,
                                                              const double* __restrict__ in,
                                                              const MolDev* __restrict__ mols) {
    using C = EriClass<LA, LB, LC, LD>;
    const DigestChunk ch = chunks[blockIdx.x];
    const MolDev& M = mols[ch.mol];
    if (M.conv) return;
    const long long total = __ldg(w.offs + w.nbra);
    const JKArgs a{nullptr, nullptr, nullptr, M.Dt, M.Jp, M.Kp, nullptr, M.n};
    for (long long t = ch.t0 + threadIdx.x; t < ch.t1; t += blockDim.x) {
        int i = ch.b0, hi = ch.b1;   // largest i in [b0, b1) with offs[i] <= t
        while (hi - i > 1) {
            const int mid = (i + hi) >> 1;
            if (__ldg(w.offs + mid) <= t) i = mid; else hi = mid;
        }
        const int j = __ldg(w.kstart + i) + (int)(t - __ldg(w.offs + i));
        const ShellPair P = w.bra[i];
        const ShellPair Q = w.ket[j];
        double I[C::NINT];
#pragma unroll
        for (int k = 0; k < C::NINT; ++k) I[k] = __ldg(in + (size_t)k * total + t);
        const double deg = (P.same ? 1.0 : 2.0) * (Q.same ? 1.0 : 2.0) * ((w.same && i == j) ? 1.0 : 2.0);
        qb_jk_digest<C>(P, Q, deg, a, I);
    }
}

// X = S^{-1/2} by the eigen-decomposition of S; C' = I; D = D' = 0, or with an initial
// density D0 (already in D): D' = S^{1/2} D0 S^{1/2}, D~ = ratio-scaled D0, and the SCF
// starts at iteration 1 (the first step builds F from D0).
__global__ void __launch_bounds__(QB_BATCH_THREADS) qb_batch_orth_kernel(MolDev* mols, int* failed, int have_d0) {
    __shared__ QbJacobiSmem<QB_BATCH_MAXN> jsm;
    MolDev& M = mols[blockIdx.x];
    const int n = M.n, nn = n * n, tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < nn; i += nt) M.W3[i] = M.S[i];
    __syncthreads();
    const int used = qb_cta_jacobi<QB_BATCH_MAXN>(n, M.W3, M.W1, nullptr, M.eps, M.wt, M.W2, 60, jsm);
    __shared__ int bad;
    (void)used;
    if (tid == 0) bad = !(M.eps[0] > 1e-10) ? 1 : 0;   // (near) linearly dependent basis
    __syncthreads();
    if (bad) {
        if (tid == 0) {
            M.conv = 3;
            atomicAdd(failed, 1);
        }
        return;
    }
    // W2 = V diag(s^{-1/2}); X = W2 V^T
    for (int i = tid; i < nn; i += nt) M.W2[i] = M.W1[i] / sqrt(M.eps[i / n]);
    __syncthreads();
    qb_cta_gemm(false, true, n, n, n, 1.0, M.W2, n, M.W1, n, 0.0, M.X, n);
    for (int i = tid; i < nn; i += nt) {
        M.Cp[i] = ((i % n) == (i / n)) ? 1.0 : 0.0;
        M.Jp[i] = 0.0;
        M.Kp[i] = 0.0;
        if (!have_d0) {
            M.D[i] = 0.0;
            M.Dt[i] = 0.0;
            M.Do[i] = 0.0;
        }
    }
    __syncthreads();
    if (have_d0) {
        // S^{1/2} = S X (W1), D' = W1 D0 W1^T
        qb_cta_gemm(false, false, n, n, n, 1.0, M.S, n, M.X, n, 0.0, M.W1, n);
        qb_cta_gemm(false, false, n, n, n, 1.0, M.W1, n, M.D, n, 0.0, M.W2, n);
        qb_cta_gemm(false, true, n, n, n, 1.0, M.W2, n, M.W1, n, 0.0, M.Do, n);
        for (int idx = tid; idx < nn; idx += nt) {
            const int i = idx % n, j = idx / n;
            M.Dt[idx] = M.D[idx] * M.ratio[i] * M.ratio[j];
        }
        if (tid == 0) M.iter = 1;
    }
}

// Pulay DIIS coefficients c (m entries) from the error Gram matrix B (ld QB_BATCH_SLOTS) of
// the slots in idx: minimise c^T B c subject to sum c = 1 (DIIScore with v = 0,
// HartreeFock.jl:1301-1315; the minimiser the constraint solvers converge to) via the
// bordered linear system, Gaussian elimination with partial pivoting (largest |pivot|,
// lowest row on ties; singular below 1e-14 after scaling by max B_ii) by one warp: lane i
// holds row i in shared memory A and the rows of each elimination step update in
// parallel.  Every lane of the warp calls it; the result is warp-uniform; false if singular.
__device__ bool qb_diis_coeffs_warp(int m, const double* B, const int* idx, double* c,
                                    double (*A)[QB_BATCH_SLOTS + 2]) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, n = m + 1;
    double scale = 0.0;
    for (int i = 0; i < m; ++i) scale = fmax(scale, fabs(B[idx[i] * QB_BATCH_SLOTS + idx[i]]));
    if (!(scale > 0.0)) return false;
    if (lane < n) {
        for (int j = 0; j < n; ++j)
            A[lane][j] = lane < m ? (j < m ? B[idx[lane] * QB_BATCH_SLOTS + idx[j]] / scale : 1.0) : (j < m ? 1.0 : 0.0);
        A[lane][n] = lane < m ? 0.0 : 1.0;   // right-hand side
    }
    __syncwarp();
    for (int k = 0; k < n; ++k) {
        double v = (lane >= k && lane < n) ? fabs(A[lane][k]) : -1.0;
        int pi = lane;
        for (int o = 16; o > 0; o >>= 1) {
            const double v2 = __shfl_xor_sync(FULL, v, o);
            const int p2 = __shfl_xor_sync(FULL, pi, o);
            if (v2 > v || (v2 == v && p2 < pi)) {
                v = v2;
                pi = p2;
            }
        }
        if (!(v > 1e-14)) return false;
        if (pi != k && lane <= n) {
            const double t = A[k][lane];
            A[k][lane] = A[pi][lane];
            A[pi][lane] = t;
        }
        __syncwarp();
        if (lane > k && lane < n) {
            const double f = A[lane][k] / A[k][k];
            for (int j = k; j < n; ++j) A[lane][j] -= f * A[k][j];
            A[lane][n] -= f * A[k][n];
        }
        __syncwarp();
    }
    if (lane == 0) {
        for (int i = n - 1; i >= 0; --i) {
            double t = A[i][n];
            for (int j = i + 1; j < n; ++j) t -= A[i][j] * A[j][n];
            A[i][n] = t / A[i][i];
        }
        for (int i = 0; i < m; ++i) c[i] = A[i][n];
    }
    __syncwarp();
    return true;
}

// One SCF iteration of one molecule per thread block (blocks ordered by size, largest first).
__global__ void __launch_bounds__(QB_BATCH_THREADS) qb_batch_step_kernel(MolDev* mols, const int* __restrict__ order,
                                                                         const StepParams prm, int* active) {
    __shared__ QbJacobiSmem<QB_BATCH_MAXN> jsm;
    __shared__ QbEigSmem<QB_BATCH_MAXN> esm;
    __shared__ double red[33];
    __shared__ double s_c[QB_BATCH_SLOTS];
    __shared__ int s_idx[QB_BATCH_SLOTS], s_ok;
    __shared__ double s_diis[QB_BATCH_SLOTS][QB_BATCH_SLOTS + 2];
    MolDev& M = mols[order[blockIdx.x]];
    if (M.conv) return;
    const int n = M.n, nn = n * n, tid = threadIdx.x, nt = blockDim.x;
    const int it = M.iter;
    const double* r = M.ratio;
    double E = 0.0;
    if (it == 0) {
        // core-Hamiltonian guess (also after a restart: drop what the digest accumulated)
        for (int i = tid; i < nn; i += nt) {
            M.F[i] = M.H[i];
            M.Jp[i] = 0.0;
            M.Kp[i] = 0.0;
        }
        __syncthreads();
    } else {
        // F = H + 2J - K (libint-convention accumulators, per-function ratios), energy of D
        double e = 0.0;
        for (int idx = tid; idx < nn; idx += nt) {
            const int i = idx % n, j = idx / n;
            const double rr = r[i] * r[j];
            const double J = 0.25 * rr * (M.Jp[i + n * j] + M.Jp[j + n * i]);
            const double K = 0.125 * rr * (M.Kp[i + n * j] + M.Kp[j + n * i]);
            const double f = M.H[idx] + 2.0 * J - K;
            M.F[idx] = f;
            e += M.D[idx] * (M.H[idx] + f);
        }
        E = qb_cta_sum(e, red);   // also a barrier: all reads of J', K' are done
        for (int i = tid; i < nn; i += nt) {
            M.Jp[i] = 0.0;
            M.Kp[i] = 0.0;
        }
        __syncthreads();
    }
    // F' = X^T F X  (W2)
    qb_cta_gemm(false, false, n, n, n, 1.0, M.F, n, M.X, n, 0.0, M.W1, n);
    qb_cta_gemm_sym(true, false, n, n, M.X, n, M.W1, n, M.W2, n);
    if (it > 0 && prm.diis > 1) {
        // DIIS subspace of (F', e', E) entries (initializeHFcore, HartreeFock.jl:1335-1394):
        // the entry of this density joins, then either the subspace restarts from the
        // previous entry (energy rise above resetThreshold) or, when over size, the entry of
        // highest energy leaves; F' is then extrapolated with the Pulay coefficients.
        if (tid == 0) {
            unsigned used_mask = 0;
            for (int k = 0; k < M.dlen; ++k) used_mask |= 1u << M.dlist[k];
            int slot = 0;
            while (used_mask & (1u << slot)) ++slot;
            s_idx[0] = slot;
        }
        __syncthreads();
        const int slot = s_idx[0];
        double* Fs = M.Fh + (size_t)slot * nn;
        double* Es = M.Eh + (size_t)slot * nn;
        // e' = F' D' - D' F' = X^T (F D S - S D F) X (getEresidual, :1298-1299)
        qb_cta_gemm(false, false, n, n, n, 1.0, M.W2, n, M.Do, n, 0.0, M.W1, n);
        for (int idx = tid; idx < nn; idx += nt) {
            const int i = idx % n, j = idx / n;
            Es[idx] = M.W1[i + n * j] - M.W1[j + n * i];
            Fs[idx] = M.W2[idx];
        }
        __syncthreads();
        const int len0 = M.dlen;
        for (int k = tid >> 5; k <= len0; k += nt >> 5) {   // one warp per Gram-matrix entry
            const int other = (k < len0) ? M.dlist[k] : slot;
            const double* Ek = M.Eh + (size_t)other * nn;
            double dot = 0.0;
            for (int idx = tid & 31; idx < nn; idx += 32) dot = fma(Es[idx], Ek[idx], dot);
            dot = qb_group_sum(dot, 32);
            if ((tid & 31) == 0) {
                M.B[slot * QB_BATCH_SLOTS + other] = dot;
                M.B[other * QB_BATCH_SLOTS + slot] = dot;
            }
        }
        __syncthreads();
        if (tid == 0) {
            M.dEs[slot] = 0.5 * E;   // per-spin energy of the entry
            M.dlist[M.dlen++] = slot;
            const int L = M.dlen;
            if (L > 2 && M.dEs[M.dlist[L - 1]] - M.dEs[M.dlist[L - 2]] > QB_BATCH_RESET) {
                M.dlist[0] = M.dlist[L - 2];   // keepOnly! of the second-to-last entry
                M.dlen = 1;
            } else if (L > prm.diis) {
                int pi = 0;
                for (int k = 1; k < L; ++k)
                    if (M.dEs[M.dlist[k]] > M.dEs[M.dlist[pi]]) pi = k;
                for (int k = pi; k + 1 < L; ++k) M.dlist[k] = M.dlist[k + 1];
                M.dlen = L - 1;
            }
            const int m = M.dlen;
            for (int k = 0; k < m; ++k) s_idx[k] = M.dlist[k];
            s_ok = m;
        }
        __syncthreads();
        const int m = s_ok;
        if (tid < 32) {   // Pulay coefficients by warp 0
            bool ok = true;
            if (m == 1) {
                if (tid == 0) s_c[0] = 1.0;
            } else {
                ok = qb_diis_coeffs_warp(m, M.B, s_idx, s_c, s_diis);
            }
            if (!ok && tid == 0) {   // singular system: extrapolate with the newest entry only
                for (int k = 0; k < m; ++k) s_c[k] = 0.0;
                s_c[m - 1] = 1.0;
            }
        }
        __syncthreads();
        for (int idx = tid; idx < nn; idx += nt) {
            double f = 0.0;
            for (int k = 0; k < m; ++k) f = fma(s_c[k], M.Fh[(size_t)s_idx[k] * nn + idx], f);
            M.W2[idx] = f;
        }
        __syncthreads();
    }
    int used = 0;
    if (prm.eig == 0) {
        // occupied eigenvectors Y of F' (W1, n x nocc): Householder + bisection + inverse
        // iteration; D' = Y Y^T (W3) and D = (X Y)(X Y)^T (W2)
        const int k = M.nocc;
        double *Aw = M.W3, *Yw = M.W1;
        for (int i = tid; i < nn; i += nt) Aw[i] = M.W2[i];
        __syncthreads();
        qb_cta_lowest_eig<QB_BATCH_MAXN>(n, k, Aw, Yw, M.eps, M.W4, M.W5, M.W6, M.wt, esm);
        qb_cta_gemm_sym(false, true, n, k, Yw, n, Yw, n, M.W3, n);
        qb_cta_gemm(false, false, n, k, n, 1.0, M.X, n, Yw, n, 0.0, M.W4, n);
        qb_cta_gemm_sym(false, true, n, k, M.W4, n, M.W4, n, M.W2, n);
    } else {
        // rotate into the previous eigenvectors, A = C'^T F' C' (W3), and diagonalise;
        // eigenvectors to off(A) <= 1e-12 ||A||: the density they give is exact far below
        // the 1e-8 density threshold, and the warm start usually needs a single sweep
        qb_cta_gemm(false, false, n, n, n, 1.0, M.W2, n, M.Cp, n, 0.0, M.W1, n);
        qb_cta_gemm(true, false, n, n, n, 1.0, M.Cp, n, M.W1, n, 0.0, M.W3, n);
        used = qb_cta_jacobi<QB_BATCH_MAXN>(n, M.W3, M.W1, M.Cp, M.eps, M.wt, M.W2, prm.sweeps, jsm, 1e-24);
        for (int i = tid; i < nn; i += nt) M.Cp[i] = M.W1[i];
        __syncthreads();
        // D' = C'_occ C'_occ^T (W3); D = X D' X^T (W2)
        qb_cta_gemm(false, true, n, n, M.nocc, 1.0, M.Cp, n, M.Cp, n, 0.0, M.W3, n);
        qb_cta_gemm(false, false, n, n, n, 1.0, M.X, n, M.W3, n, 0.0, M.W1, n);
        qb_cta_gemm(false, true, n, n, n, 1.0, M.W1, n, M.X, n, 0.0, M.W2, n);
    }
    double dd = 0.0;
    for (int idx = tid; idx < nn; idx += nt) {
        const double d = M.W2[idx] - M.D[idx];
        dd += d * d;
    }
    dd = qb_cta_sum(dd, red);
    const double rms = 2.0 * sqrt(dd) / n;   // RMS change of the total density 2D
    for (int idx = tid; idx < nn; idx += nt) {
        const int i = idx % n, j = idx / n;
        const double d = M.W2[idx];
        M.D[idx] = d;
        M.Dt[idx] = d * r[i] * r[j];
        M.Do[idx] = M.W3[idx];
    }
    __syncthreads();
    if (tid == 0) {
        M.sweeps += used < 0 ? prm.sweeps : used;   // Jacobi sweeps (0 with the tridiagonal solver)
        // convergence of the entry of this step (E of D, and D against the density before
        // it), as runHartreeFockCore compares consecutive steps (HartreeFock.jl:1160-1175)
        int conv = 0;
        if (it > 0) {
            M.dE = E - M.Eprev;
            if (it >= 2 && fabs(M.dE) <= prm.thr_e && M.rmsD <= prm.thr_d) conv = 1;
            M.E = E;
            M.Eprev = E;
        }
        M.rmsD = rms;   // change of the density handed to the next step
        M.iter = it + 1;
        const int spent = M.iter0 + M.iter;
        if (!conv && prm.fallback > 0 && !M.restarted && M.iter >= prm.fallback && spent < prm.max_iter) {
            // the supplied initial density has not converged: start again from F = H with an
            // empty DIIS subspace (the next step ignores D and the J'/K' of this iteration)
            M.iter0 = spent;
            M.iter = 0;
            M.dlen = 0;
            M.restarted = 1;
        } else if (!conv && spent >= prm.max_iter) {
            conv = 2;
        }
        M.conv = conv;
        if (!conv) atomicAdd(active, 1);
    }
}

template <int LA, int LB, int LC, int LD>
void launch_store(const BatchWork& w, const PrimPair* prims, const double* boys, double* out,
                  unsigned long long* pc, const unsigned* perm, int grid, cudaStream_t s) {
    qb_batch_store_kernel<LA, LB, LC, LD><<<grid, 128, 0, s>>>(w, prims, boys, out, pc, perm);
}
template <int LA, int LB, int LC, int LD>
void launch_digest(const BatchWork& w, const DigestChunk* chunks, const double* in, const MolDev* mols, int grid,
                   cudaStream_t s) {
    qb_batch_digest_kernel<LA, LB, LC, LD><<<grid, 128, 0, s>>>(w, chunks, in, mols);
}

struct ClassDef {
    int la, lb, lc, ld, nint;
    void (*store)(const BatchWork&, const PrimPair*, const double*, double*, unsigned long long*, const unsigned*, int,
                  cudaStream_t);
    void (*digest)(const BatchWork&, const DigestChunk*, const double*, const MolDev*, int, cudaStream_t);
};

const ClassDef kClasses[QB_BATCH_NCLASS] = {
    {0, 0, 0, 0, EriClass<0, 0, 0, 0>::NINT, launch_store<0, 0, 0, 0>, launch_digest<0, 0, 0, 0>},
    {1, 0, 0, 0, EriClass<1, 0, 0, 0>::NINT, launch_store<1, 0, 0, 0>, launch_digest<1, 0, 0, 0>},
    {1, 0, 1, 0, EriClass<1, 0, 1, 0>::NINT, launch_store<1, 0, 1, 0>, launch_digest<1, 0, 1, 0>},
    {1, 1, 0, 0, EriClass<1, 1, 0, 0>::NINT, launch_store<1, 1, 0, 0>, launch_digest<1, 1, 0, 0>},
    {1, 1, 1, 0, EriClass<1, 1, 1, 0>::NINT, launch_store<1, 1, 1, 0>, launch_digest<1, 1, 1, 0>},
    {1, 1, 1, 1, EriClass<1, 1, 1, 1>::NINT, launch_store<1, 1, 1, 1>, launch_digest<1, 1, 1, 1>},
};

int pc_of(int la, int lb) { return la * (la + 1) / 2 + lb; }

}  // namespace

// ---------------------------------------------------------------------------
extern "C" void qb_batch_config_default(qb_batch_config* cfg) {
    if (!cfg) return;
    cfg->conv_energy = 1e-10;
    cfg->conv_density = 1e-8;
    cfg->max_iter = 200;
    cfg->diis_size = QB_BATCH_DIIS;
    cfg->schwarz = 1e-14;
    cfg->iters_per_graph = 4;
    cfg->initial_density = nullptr;
    cfg->jacobi_sweeps = 0;
    cfg->eigensolver = 0;
    cfg->fallback_iter = 0;
}

int qb_batch_rhf_run(qb_ctx* ctx, int nmol, const qb_basis* bases, const int* nnuc, const double* Z,
                     const double* R, const int* nocc, const qb_batch_config* cfg_in, qb_batch_result* res) {
    if (nmol <= 0 || !bases || !nnuc || !Z || !R || !nocc || !res)
        return qb_set_error(ctx, QB_ERR_ARG, "bad batched SCF arguments");
    qb_batch_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else qb_batch_config_default(&cfg);
    if (cfg.diis_size < 1 || cfg.diis_size > QB_BATCH_DIIS || cfg.max_iter < 1 || cfg.iters_per_graph < 1 ||
        cfg.fallback_iter < 0 ||
        !(cfg.schwarz >= 0.0) || !(cfg.conv_energy > 0.0) || !(cfg.conv_density > 0.0))
        return qb_set_error(ctx, QB_ERR_DOMAIN, "bad batched SCF configuration");
    cudaStream_t s = ctx->stream;
    // ---- concatenate the bases, detect shells per molecule
    std::vector<int> fo(nmol + 1, 0), nf(nmol), nuc0(nmol + 1, 0);
    std::vector<int> fp(1, 0), ijk;
    std::vector<double> cen, al, w;
    for (int m = 0; m < nmol; ++m) {
        const qb_basis& b = bases[m];
        if (!b.fun_ptr || !b.center || !b.ijk || !b.alpha || !b.weight)
            return qb_set_error(ctx, QB_ERR_ARG, "null basis array");
        if (b.nfun < 1 || b.nfun > QB_BATCH_MAXN) return qb_set_error(ctx, QB_ERR_DIM, "batched SCF: 1 <= nfun <= 256");
        if (nocc[m] < 1 || nocc[m] > b.nfun) return qb_set_error(ctx, QB_ERR_DIM, "batched SCF: bad occupation");
        if (nnuc[m] < 1) return qb_set_error(ctx, QB_ERR_DIM, "batched SCF: molecule without nuclei");
        nf[m] = b.nfun;
        fo[m + 1] = fo[m] + b.nfun;
        nuc0[m + 1] = nuc0[m] + nnuc[m];
        const int np = b.fun_ptr[b.nfun];
        if (b.fun_ptr[0] != 0 || np <= 0) return qb_set_error(ctx, QB_ERR_ARG, "bad function pointers");
        const int base = fp.back();
        for (int f = 0; f < b.nfun; ++f) {
            if (b.fun_ptr[f + 1] <= b.fun_ptr[f]) return qb_set_error(ctx, QB_ERR_ARG, "bad function pointers");
            fp.push_back(base + b.fun_ptr[f + 1]);
        }
        for (int p = 0; p < np; ++p) {
            if (!(b.alpha[p] > 0.0) || !std::isfinite(b.alpha[p]) || !std::isfinite(b.weight[p]))
                return qb_set_error(ctx, QB_ERR_DOMAIN, "bad exponent or weight");
            for (int x = 0; x < 3; ++x) {
                if (!std::isfinite(b.center[3 * p + x])) return qb_set_error(ctx, QB_ERR_DOMAIN, "non-finite centre");
                cen.push_back(b.center[3 * p + x]);
                if (b.ijk[3 * p + x] < 0) return qb_set_error(ctx, QB_ERR_DOMAIN, "negative Cartesian power");
                ijk.push_back(b.ijk[3 * p + x]);
            }
            al.push_back(b.alpha[p]);
            w.push_back(b.weight[p]);
        }
    }
    const int F = fo[nmol];
    std::vector<HostShell> shells;
    std::vector<int> sh0(nmol + 1, 0), shell_mol;
    std::vector<double> ratio(F, 1.0);
    for (int m = 0; m < nmol; ++m) {
        if (!qb_detect_shells(fo[m], fo[m + 1], fp.data(), cen.data(), ijk.data(), al.data(), w.data(), shells,
                              ratio.data()))
            return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "batched SCF: basis of molecule " + std::to_string(m) +
                                                             " is not made of Cartesian shells");
        sh0[m + 1] = (int)shells.size();
        shell_mol.resize(shells.size(), m);
    }
    for (const HostShell& sh : shells)
        if (sh.L > 1) return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "batched SCF supports s and p shells");
    // local ratios per molecule start at ratio.data() + fo[m]
    // ---- device copies of the basis and nuclei
    DevArray<int> d_fp, d_ijk, d_fo, d_nf, d_nuc0, d_order;
    DevArray<double> d_cen, d_al, d_w, d_ratio, d_Z, d_R;
    DevArray<long long> d_poff, d_mo;
    QB_CUDA(ctx, d_fp.ensure(fp.size()));
    QB_CUDA(ctx, d_ijk.ensure(ijk.size()));
    QB_CUDA(ctx, d_cen.ensure(cen.size()));
    QB_CUDA(ctx, d_al.ensure(al.size()));
    QB_CUDA(ctx, d_w.ensure(w.size()));
    QB_CUDA(ctx, d_ratio.ensure(F));
    QB_CUDA(ctx, cudaMemcpyAsync(d_fp.p, fp.data(), fp.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_ijk.p, ijk.data(), ijk.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_cen.p, cen.data(), cen.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_al.p, al.data(), al.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_w.p, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_ratio.p, ratio.data(), F * sizeof(double), cudaMemcpyHostToDevice, s));
    const GenDevBasis gb{d_fp.p, d_cen.p, d_ijk.p, d_al.p, d_w.p, F};
    const int ntot_nuc = nuc0[nmol];
    for (int c = 0; c < ntot_nuc; ++c)
        if (!std::isfinite(Z[c]) || !std::isfinite(R[3 * c]) || !std::isfinite(R[3 * c + 1]) ||
            !std::isfinite(R[3 * c + 2]))
            return qb_set_error(ctx, QB_ERR_DOMAIN, "non-finite nuclear charge or position");
    QB_CUDA(ctx, d_Z.ensure(ntot_nuc));
    QB_CUDA(ctx, d_R.ensure(3 * (size_t)ntot_nuc));
    QB_CUDA(ctx, cudaMemcpyAsync(d_Z.p, Z, ntot_nuc * sizeof(double), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_R.p, R, 3 * ntot_nuc * sizeof(double), cudaMemcpyHostToDevice, s));
    // ---- per-molecule matrix storage
    std::vector<long long> mo(nmol + 1, 0), poff(nmol + 1, 0), vo(nmol + 1, 0);
    for (int m = 0; m < nmol; ++m) {
        mo[m + 1] = mo[m] + (long long)nf[m] * nf[m];
        poff[m + 1] = poff[m] + (long long)nf[m] * (nf[m] + 1) / 2;
        vo[m + 1] = vo[m] + nf[m];
    }
    const long long NN = mo[nmol];
    const int nmat = 16 + 2 * QB_BATCH_SLOTS;
    DevArray<double> d_mats, d_vecs, d_B;
    QB_CUDA(ctx, d_mats.ensure((size_t)nmat * NN));
    QB_CUDA(ctx, d_vecs.ensure(2 * (size_t)vo[nmol]));
    QB_CUDA(ctx, d_B.ensure((size_t)nmol * QB_BATCH_SLOTS * QB_BATCH_SLOTS));
    QB_CUDA(ctx, cudaMemsetAsync(d_B.p, 0, (size_t)nmol * QB_BATCH_SLOTS * QB_BATCH_SLOTS * sizeof(double), s));
    std::vector<MolDev> hm(nmol);
    for (int m = 0; m < nmol; ++m) {
        MolDev& M = hm[m];
        std::memset(&M, 0, sizeof(M));
        M.n = nf[m];
        M.nocc = nocc[m];
        double* mat[16];
        for (int k = 0; k < 16; ++k) mat[k] = d_mats.p + (size_t)k * NN + mo[m];
        M.S = mat[0]; M.H = mat[1]; M.X = mat[2]; M.F = mat[3]; M.D = mat[4]; M.Dt = mat[5]; M.Do = mat[6];
        M.Jp = mat[7]; M.Kp = mat[8]; M.Cp = mat[9]; M.W1 = mat[10]; M.W2 = mat[11]; M.W3 = mat[12];
        M.W4 = mat[13]; M.W5 = mat[14]; M.W6 = mat[15];
        M.Fh = d_mats.p + 16 * (size_t)NN + (size_t)QB_BATCH_SLOTS * mo[m];
        M.Eh = d_mats.p + (16 + QB_BATCH_SLOTS) * (size_t)NN + (size_t)QB_BATCH_SLOTS * mo[m];
        M.B = d_B.p + (size_t)m * QB_BATCH_SLOTS * QB_BATCH_SLOTS;
        M.eps = d_vecs.p + vo[m];
        M.wt = d_vecs.p + vo[nmol] + vo[m];
        M.ratio = d_ratio.p + fo[m];
    }
    DevArray<MolDev> d_mols;
    QB_CUDA(ctx, d_mols.ensure(nmol));
    QB_CUDA(ctx, cudaMemcpyAsync(d_mols.p, hm.data(), nmol * sizeof(MolDev), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, d_fo.ensure(nmol + 1));
    QB_CUDA(ctx, d_nf.ensure(nmol));
    QB_CUDA(ctx, d_nuc0.ensure(nmol + 1));
    QB_CUDA(ctx, d_poff.ensure(nmol + 1));
    QB_CUDA(ctx, d_mo.ensure(nmol + 1));
    QB_CUDA(ctx, cudaMemcpyAsync(d_fo.p, fo.data(), (nmol + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_nf.p, nf.data(), nmol * sizeof(int), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_nuc0.p, nuc0.data(), (nmol + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_poff.p, poff.data(), (nmol + 1) * sizeof(long long), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_mo.p, mo.data(), (nmol + 1) * sizeof(long long), cudaMemcpyHostToDevice, s));

    cudaEvent_t ev0, ev1, ev2;
    QB_CUDA(ctx, cudaEventCreate(&ev0));
    QB_CUDA(ctx, cudaEventCreate(&ev1));
    QB_CUDA(ctx, cudaEventCreate(&ev2));
    QB_CUDA(ctx, cudaEventRecord(ev0, s));
    // ---- one-body S and H
    if (qb_gen_onebody_batch(gb, nmol, poff[nmol], d_poff.p, d_fo.p, d_nf.p, d_mo.p, d_nuc0.p, d_Z.p, d_R.p,
                             ctx->boys.p, hm[0].S - mo[0], hm[0].H - mo[0], ctx->status.p, s) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "batched one-body kernel");
    // ---- shell pairs of every molecule, grouped by pair class
    const int npc = 3;   // ss, ps, pp
    std::vector<std::vector<ShellPair>> by(npc);
    std::vector<std::vector<PairSlot>> slots_by(npc);
    for (int m = 0; m < nmol; ++m)
        for (int a = sh0[m]; a < sh0[m + 1]; ++a)
            for (int b = sh0[m]; b <= a; ++b) {
                const HostShell* A = &shells[a];
                const HostShell* B = &shells[b];
                if (B->L > A->L) std::swap(A, B);
                const int pc = pc_of(A->L, B->L);
                ShellPair sp;
                sp.fa = A->f0;
                sp.fb = B->f0;
                sp.nprim = A->K * B->K;
                sp.prim0 = (int)slots_by[pc].size();   // local slot offset, rebased below
                sp.ABx = A->c[0] - B->c[0];
                sp.ABy = A->c[1] - B->c[1];
                sp.ABz = A->c[2] - B->c[2];
                sp.Q = 0.0;
                sp.same = (a == b);
                sp.pad = m;
                for (int i = 0; i < A->K; ++i)
                    for (int j = 0; j < B->K; ++j)
                        slots_by[pc].push_back(PairSlot{a, b, A->prim0 + i, B->prim0 + j});
                by[pc].push_back(sp);
            }
    std::vector<ShellPair> pairs;
    std::vector<PairSlot> slots;
    std::vector<int> pc_off(npc + 1, 0);
    for (int pc = 0; pc < npc; ++pc) {
        pc_off[pc] = (int)pairs.size();
        const int base = (int)slots.size();
        for (ShellPair sp : by[pc]) {
            sp.prim0 += base;
            pairs.push_back(sp);
        }
        slots.insert(slots.end(), slots_by[pc].begin(), slots_by[pc].end());
    }
    pc_off[npc] = (int)pairs.size();
    const int npair = (int)pairs.size(), nslot = (int)slots.size();
    DevArray<PairSlot> d_slots;
    DevArray<ShellPair> d_pairs;
    DevArray<PrimPair> d_prims;
    DevArray<float4> d_prims32;
    DevArray<int> d_nkept;
    DevArray<unsigned long long> d_kmax, d_primcount;
    DevArray<double> d_Q;
    QB_CUDA(ctx, d_slots.ensure(nslot));
    QB_CUDA(ctx, d_pairs.ensure(npair));
    QB_CUDA(ctx, d_prims.ensure(nslot));
    QB_CUDA(ctx, d_prims32.ensure(nslot));
    QB_CUDA(ctx, d_nkept.ensure(npair));
    QB_CUDA(ctx, d_kmax.ensure(1));
    QB_CUDA(ctx, d_primcount.ensure(1));
    QB_CUDA(ctx, d_Q.ensure(npair));
    QB_CUDA(ctx, cudaMemcpyAsync(d_slots.p, slots.data(), nslot * sizeof(PairSlot), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_pairs.p, pairs.data(), npair * sizeof(ShellPair), cudaMemcpyHostToDevice, s));
    // prim pairs: the slot centres/exponents/weights index the concatenated primitive arrays
    if (qb_build_prim_pairs(s, d_slots.p, nslot, d_cen.p, d_al.p, d_w.p, d_pairs.p, npair, d_prims.p, d_prims32.p,
                            d_nkept.p, d_kmax.p) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "batched primitive pairs");
    {
        std::vector<int> nkept(npair);
        QB_CUDA(ctx, cudaMemcpyAsync(nkept.data(), d_nkept.p, npair * sizeof(int), cudaMemcpyDeviceToHost, s));
        QB_CUDA(ctx, cudaStreamSynchronize(s));
        for (int k = 0; k < npair; ++k) pairs[k].nprim = nkept[k];
        QB_CUDA(ctx, cudaMemcpyAsync(d_pairs.p, pairs.data(), npair * sizeof(ShellPair), cudaMemcpyHostToDevice, s));
    }
    for (int pc = 0; pc < npc; ++pc) {
        const int n = pc_off[pc + 1] - pc_off[pc];
        if (n == 0) continue;
        const ShellPair* pp = d_pairs.p + pc_off[pc];
        double* q = d_Q.p + pc_off[pc];
        const int g = (n + 127) / 128;
        if (pc == 0) qb_schwarz_class_kernel<0, 0><<<g, 128, 0, s>>>(pp, n, d_prims.p, ctx->boys.p, d_ratio.p, q);
        else if (pc == 1) qb_schwarz_class_kernel<1, 0><<<g, 128, 0, s>>>(pp, n, d_prims.p, ctx->boys.p, d_ratio.p, q);
        else qb_schwarz_class_kernel<1, 1><<<g, 128, 0, s>>>(pp, n, d_prims.p, ctx->boys.p, d_ratio.p, q);
        QB_CUDA(ctx, cudaGetLastError());
    }
    QB_TRY(qb_check_status(ctx));
    {
        std::vector<double> Q(npair);
        QB_CUDA(ctx, cudaMemcpyAsync(Q.data(), d_Q.p, npair * sizeof(double), cudaMemcpyDeviceToHost, s));
        QB_CUDA(ctx, cudaStreamSynchronize(s));
        for (int k = 0; k < npair; ++k) pairs[k].Q = Q[k];
    }
    // sort each pair class by (molecule, Q descending); molecule segments; local function indices
    std::vector<std::vector<int>> seg(npc, std::vector<int>(nmol + 1, 0));
    for (int pc = 0; pc < npc; ++pc) {
        auto b0 = pairs.begin() + pc_off[pc], b1 = pairs.begin() + pc_off[pc + 1];
        std::stable_sort(b0, b1, [](const ShellPair& x, const ShellPair& y) {
            return x.pad != y.pad ? x.pad < y.pad : x.Q > y.Q;
        });
        std::vector<int> cnt(nmol, 0);
        for (auto it = b0; it != b1; ++it) ++cnt[it->pad];
        for (int m = 0; m < nmol; ++m) seg[pc][m + 1] = seg[pc][m] + cnt[m];
    }
    for (ShellPair& sp : pairs) {
        sp.fa -= fo[sp.pad];
        sp.fb -= fo[sp.pad];
    }
    QB_CUDA(ctx, cudaMemcpyAsync(d_pairs.p, pairs.data(), npair * sizeof(ShellPair), cudaMemcpyHostToDevice, s));
    // ---- quartet work lists per class
    std::vector<long long> h_offs;
    std::vector<int> h_kstart;
    std::vector<size_t> offs_at(QB_BATCH_NCLASS), ks_at(QB_BATCH_NCLASS), eri_at(QB_BATCH_NCLASS + 1, 0);
    std::vector<long long> total(QB_BATCH_NCLASS, 0);
    const double thr = cfg.schwarz;
    for (int c = 0; c < QB_BATCH_NCLASS; ++c) {
        const ClassDef& cd = kClasses[c];
        const int X = pc_of(cd.la, cd.lb), Y = pc_of(cd.lc, cd.ld);
        const int nbra = pc_off[X + 1] - pc_off[X];
        offs_at[c] = h_offs.size();
        ks_at[c] = h_kstart.size();
        long long acc = 0;
        for (int i = 0; i < nbra; ++i) {
            const ShellPair& P = pairs[pc_off[X] + i];
            const int m = P.pad;
            int ks = seg[Y][m], ke = seg[Y][m + 1];
            if (X == Y) ke = std::min(ke, i + 1);
            // kets in [ks, ke) are sorted by descending Q: count those with Q_P Q_K >= thr
            int lo = ks, hi = ke;
            while (lo < hi) {
                const int mid = (lo + hi) / 2;
                if (P.Q * pairs[pc_off[Y] + mid].Q >= thr) lo = mid + 1; else hi = mid;
            }
            h_offs.push_back(acc);
            h_kstart.push_back(ks);
            acc += std::max(0, lo - ks);
        }
        h_offs.push_back(acc);
        total[c] = acc;
        eri_at[c + 1] = eri_at[c] + (size_t)acc * cd.nint;
    }
    DevArray<long long> d_offs;
    DevArray<int> d_kstart;
    DevArray<double> d_eri;
    QB_CUDA(ctx, d_offs.ensure(h_offs.size()));
    QB_CUDA(ctx, d_kstart.ensure(h_kstart.size()));
    QB_CUDA(ctx, d_eri.ensure(eri_at[QB_BATCH_NCLASS]));
    QB_CUDA(ctx, cudaMemcpyAsync(d_offs.p, h_offs.data(), h_offs.size() * sizeof(long long), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(d_kstart.p, h_kstart.data(), h_kstart.size() * sizeof(int), cudaMemcpyHostToDevice,
                                 s));
    QB_CUDA(ctx, cudaMemsetAsync(d_primcount.p, 0, sizeof(unsigned long long), s));
    BatchWork work[QB_BATCH_NCLASS];
    long long max_total = 1;
    for (int c = 0; c < QB_BATCH_NCLASS; ++c) max_total = std::max(max_total, total[c]);
    if (max_total >= (1LL << 32)) return qb_set_error(ctx, QB_ERR_DIM, "batched SCF: over 2^32 quartets in one class");
    DevArray<unsigned> d_perm, d_hist;   // visiting order of one class (reused), bucket counters
    QB_CUDA(ctx, d_perm.ensure((size_t)max_total));
    QB_CUDA(ctx, d_hist.ensure(QB_COST_BUCKETS));
    for (int c = 0; c < QB_BATCH_NCLASS; ++c) {
        const ClassDef& cd = kClasses[c];
        const int X = pc_of(cd.la, cd.lb), Y = pc_of(cd.lc, cd.ld);
        work[c] = BatchWork{d_pairs.p + pc_off[X], d_pairs.p + pc_off[Y], d_offs.p + offs_at[c], d_kstart.p + ks_at[c],
                            pc_off[X + 1] - pc_off[X], X == Y};
        if (total[c] == 0) continue;
        const int grid = (int)std::min<long long>((total[c] + 127) / 128, (long long)ctx->nsm * 16);
        QB_CUDA(ctx, cudaMemsetAsync(d_hist.p, 0, QB_COST_BUCKETS * sizeof(unsigned), s));
        qb_batch_cost_hist_kernel<<<grid, 128, 0, s>>>(work[c], d_hist.p);
        qb_batch_cost_scan_kernel<<<1, 1, 0, s>>>(d_hist.p);
        qb_batch_cost_scatter_kernel<<<grid, 128, 0, s>>>(work[c], d_hist.p, d_perm.p);
        cd.store(work[c], d_prims.p, ctx->boys.p, d_eri.p + eri_at[c], d_primcount.p, d_perm.p, grid, s);
    }
    QB_CUDA(ctx, cudaGetLastError());
    // ---- digest chunks: per class and molecule, runs of at most QB_DIGEST_CHUNK quartets
    // (QB_DIGEST_CHUNK_SMALL for a molecule with fewer than 128 such runs in the class: its
    // late iterations then still spread over many SMs)
    std::vector<DigestChunk> h_chunks;
    std::vector<size_t> chunk_at(QB_BATCH_NCLASS + 1, 0);
    for (int c = 0; c < QB_BATCH_NCLASS; ++c) {
        chunk_at[c] = h_chunks.size();
        const ClassDef& cd = kClasses[c];
        const int X = pc_of(cd.la, cd.lb);
        const long long* off = h_offs.data() + offs_at[c];
        for (int m = 0; m < nmol; ++m) {
            const int s0 = seg[X][m], s1 = seg[X][m + 1];
            const long long chunk = (off[s1] - off[s0]) >= 128LL * QB_DIGEST_CHUNK ? QB_DIGEST_CHUNK
                                                                                   : QB_DIGEST_CHUNK_SMALL;
            for (long long t0 = off[s0]; t0 < off[s1]; t0 += chunk) {
                const long long t1 = std::min<long long>(t0 + chunk, off[s1]);
                // bras owning [t0, t1): largest b with off[b] <= t0, one past the largest with off[b] <= t1 - 1
                const int b0 = (int)(std::upper_bound(off + s0, off + s1, t0) - off) - 1;
                const int b1 = (int)(std::upper_bound(off + s0, off + s1, t1 - 1) - off);
                h_chunks.push_back(DigestChunk{t0, t1, b0, b1, m, 0});
            }
        }
    }
    chunk_at[QB_BATCH_NCLASS] = h_chunks.size();
    DevArray<DigestChunk> d_chunks;
    QB_CUDA(ctx, d_chunks.ensure(std::max<size_t>(1, h_chunks.size())));
    if (!h_chunks.empty())
        QB_CUDA(ctx, cudaMemcpyAsync(d_chunks.p, h_chunks.data(), h_chunks.size() * sizeof(DigestChunk),
                                     cudaMemcpyHostToDevice, s));
    // ---- X = S^{-1/2}
    DevArray<int> d_counters;   // [0] failed, [1] active
    QB_CUDA(ctx, d_counters.ensure(2));
    QB_CUDA(ctx, cudaMemsetAsync(d_counters.p, 0, 2 * sizeof(int), s));
    if (cfg.initial_density)
        QB_CUDA(ctx, cudaMemcpyAsync(d_mats.p + 4 * (size_t)NN, cfg.initial_density, NN * sizeof(double),
                                     cudaMemcpyDefault, s));   // host or device memory
    qb_batch_orth_kernel<<<nmol, QB_BATCH_THREADS, 0, s>>>(d_mols.p, d_counters.p, cfg.initial_density ? 1 : 0);
    QB_CUDA(ctx, cudaGetLastError());
    QB_CUDA(ctx, cudaEventRecord(ev1, s));
    QB_TRY(qb_check_status(ctx));
    // ---- SCF iterations, several per CUDA-graph launch
    std::vector<int> order(nmol);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return nf[a] > nf[b]; });
    QB_CUDA(ctx, d_order.ensure(nmol));
    QB_CUDA(ctx, cudaMemcpyAsync(d_order.p, order.data(), nmol * sizeof(int), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaStreamSynchronize(s));
    const StepParams prm{cfg.conv_energy, cfg.conv_density, cfg.max_iter, cfg.diis_size,
                         cfg.jacobi_sweeps > 0 ? std::min(cfg.jacobi_sweeps, 60) : 60, cfg.eigensolver ? 1 : 0,
                         cfg.initial_density && cfg.fallback_iter > 0 ? cfg.fallback_iter : 0};
    int* d_active = d_counters.p + 1;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    QB_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < cfg.iters_per_graph; ++k) {
        cudaMemsetAsync(d_active, 0, sizeof(int), s);
        for (int c = 0; c < QB_BATCH_NCLASS; ++c) {
            const int nch = (int)(chunk_at[c + 1] - chunk_at[c]);
            if (nch == 0) continue;
            kClasses[c].digest(work[c], d_chunks.p + chunk_at[c], d_eri.p + eri_at[c], d_mols.p, nch, s);
        }
        qb_batch_step_kernel<<<nmol, QB_BATCH_THREADS, 0, s>>>(d_mols.p, d_order.p, prm, d_active);
    }
    const cudaError_t cap = cudaStreamEndCapture(s, &graph);
    QB_CUDA(ctx, cap);
    QB_CUDA(ctx, cudaGraphInstantiate(&exec, graph, 0));
    int launches = 0, active = nmol;
    const int max_launch = (cfg.max_iter + cfg.iters_per_graph - 1) / cfg.iters_per_graph + 1;
    int rc = QB_OK;
    while (active > 0 && launches < max_launch) {
        rc = qb_cuda_check(ctx, cudaGraphLaunch(exec, s), "graph launch");
        if (rc != QB_OK) break;
        ++launches;
        rc = qb_cuda_check(ctx, cudaMemcpyAsync(&active, d_active, sizeof(int), cudaMemcpyDeviceToHost, s),
                           "active count");
        if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaStreamSynchronize(s), "SCF graph");
        if (rc != QB_OK) break;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    QB_TRY(rc);
    QB_CUDA(ctx, cudaEventRecord(ev2, s));
    QB_CUDA(ctx, cudaMemcpyAsync(hm.data(), d_mols.p, nmol * sizeof(MolDev), cudaMemcpyDeviceToHost, s));
    if (res->density)
        QB_CUDA(ctx, cudaMemcpyAsync(res->density, d_mats.p + 4 * (size_t)NN, NN * sizeof(double), cudaMemcpyDeviceToHost, s));
    unsigned long long nprimq = 0;
    QB_CUDA(ctx, cudaMemcpyAsync(&nprimq, d_primcount.p, sizeof(nprimq), cudaMemcpyDeviceToHost, s));
    QB_CUDA(ctx, cudaStreamSynchronize(s));
    float ms1 = 0.f, ms2 = 0.f;
    cudaEventElapsedTime(&ms1, ev0, ev1);
    cudaEventElapsedTime(&ms2, ev1, ev2);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaEventDestroy(ev2);
    QB_TRY(qb_check_status(ctx));
    long long nq = 0;
    for (int c = 0; c < QB_BATCH_NCLASS; ++c) nq += total[c];
    res->ms_integrals = ms1;
    res->ms_scf = ms2;
    res->quartets = nq;
    res->prim_quartets = (int64_t)nprimq;
    res->eri_doubles = (int64_t)eri_at[QB_BATCH_NCLASS];
    res->graph_launches = launches;
    int failed = 0;
    for (int m = 0; m < nmol; ++m) {
        if (res->energy) res->energy[m] = hm[m].E;
        if (res->iterations) res->iterations[m] = hm[m].iter0 + hm[m].iter;
        if (res->restarted) res->restarted[m] = hm[m].restarted;
        if (res->converged) res->converged[m] = hm[m].conv == 1 ? 1 : 0;
        if (res->jacobi_sweeps) res->jacobi_sweeps[m] = hm[m].sweeps;
        failed += hm[m].conv == 3;
    }
    if (failed) return qb_set_error(ctx, QB_ERR_DOMAIN, "batched SCF: overlap matrix not positive definite");
    return QB_OK;
}
