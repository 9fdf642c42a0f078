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
#include "qb_diis_solvers.cuh"
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

#define QB_BATCH_POOL 32   // entry slots of a molecule: history (<= 15) and DIIS subspace (<= 16) share them
#define QB_BATCH_HIST 15   // history kept for the next method's start: max(3, DIISsize) entries

struct MolDev {
    int n, nocc, conv, iter;   // conv: 0 iterating, 1 converged, 2 stopped, 3 failed; iter: step-kernel calls
    int steps, stage, nstep, phase;   // SCF steps (the reference's i), method index, steps of the method,
                                      // phase 0: the digested density is a step's entry, 1: a DD half step
    int hlen, slen, ne, nde;   // history / subspace lengths, energies seen (Etots), energy changes seen
    int iter0, restarted, sweeps, stale;   // stale: the history's last entry is not the digested density
    int hlist[QB_BATCH_HIST + 1], slist[QB_BATCH_DIIS + 2];   // slot ids, oldest first
    double sE[QB_BATCH_POOL];       // per-spin energy of each slot's entry
    double c[QB_BATCH_DIIS + 2];    // the method's coefficient vector (carried between its steps)
    double Er[32], dEr[4];          // last total energies (Etots) and energy changes (rings)
    double E, Eprev, dE, rmsD, dF;
    double *S, *H, *X, *Sh, *F, *D, *Dt, *Do, *Jp, *Kp, *Cp, *W1, *W2, *W3, *W4, *W5, *W6;
    double *Fs, *Ds, *Es;           // per slot: F (AO), D (AO), e' = X^T (F D S - S D F) X
    double *Gee, *Gdf;              // pool x pool: <e'_a, e'_b>, <D_a, F_b>
    double *eps, *wt;
    const double* ratio;
};

struct StepParams {
    int nmethod;
    int method[8];
    double interval[8];
    int solver[8];
    double r1, r2, osc, damp;          // secondaryConvRatio, oscillateThreshold, dampStrength
    int max_iter, diis, early_stop;
    int sweeps, eig;                   // eig 0: tridiagonal occupied-subspace solver, 1: Jacobi
    int fallback;                      // > 0: restart from the core-Hamiltonian guess after this many iterations
    int need_df;                       // some method is EDIIS or ADIIS: keep the <D_a, F_b> Gram entries
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
                 I, nprimq, (float)QB_PRIM_EPS_Q);
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
    // S^{1/2} = S X (orthonormal-basis densities D' = S^{1/2} D S^{1/2})
    qb_cta_gemm(false, false, n, n, n, 1.0, M.S, n, M.X, n, 0.0, M.Sh, n);
    if (have_d0) {
        qb_cta_gemm(false, false, n, n, n, 1.0, M.Sh, n, M.D, n, 0.0, M.W2, n);
        qb_cta_gemm(false, true, n, n, n, 1.0, M.W2, n, M.Sh, n, 0.0, M.Do, n);
        for (int idx = tid; idx < nn; idx += nt) {
            const int i = idx % n, j = idx / n;
            M.Dt[idx] = M.D[idx] * M.ratio[i] * M.ratio[j];
        }
        if (tid == 0) M.iter = 1;   // the supplied density is the first entry (initializeSCF)
    }
}

// Pulay DIIS coefficients c (m entries) minimising c^T B c with sum c = 1, B the error Gram
// matrix of the pool slots idx (leading dimension QB_BATCH_POOL): DIIScore with v = 0
// (HartreeFock.jl:1301-1315) solved exactly, the solution CMsolver! gives (:1445-1477),
// via the bordered linear system by one warp: Gaussian elimination with partial pivoting
// (largest |pivot|, lowest row on ties; singular below 1e-14 after scaling by max B_ii),
// lane i holding row i in shared memory A.  Every lane calls it; false if singular.
__device__ bool qb_diis_coeffs_warp(int m, const double* B, const int* idx, double* c,
                                    double (*A)[QB_BATCH_DIIS + 3]) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, n = m + 1;
    double scale = 0.0;
    for (int i = 0; i < m; ++i) scale = fmax(scale, fabs(B[idx[i] * QB_BATCH_POOL + idx[i]]));
    if (!(scale > 0.0)) return false;
    if (lane < n) {
        for (int j = 0; j < n; ++j)
            A[lane][j] = lane < m ? (j < m ? B[idx[lane] * QB_BATCH_POOL + idx[j]] / scale : 1.0) : (j < m ? 1.0 : 0.0);
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

// eigenvectors of the occupied orbitals of F' (in W2, orthonormal basis, destroyed) -> the
// density D' = Y Y^T (W3) and D = (X Y)(X Y)^T (W2)
__device__ int qb_batch_density(MolDev& M, const StepParams& prm, QbJacobiSmem<QB_BATCH_MAXN>& jsm,
                                QbEigSmem<QB_BATCH_MAXN>& esm) {
    const int n = M.n, nn = n * n, tid = threadIdx.x, nt = blockDim.x;
    int used = 0;
    if (prm.eig == 0) {
        const int k = M.nocc;
        double *Aw = M.W3, *Yw = M.W1;
        for (int i = tid; i < nn; i += nt) Aw[i] = M.W2[i];
        __syncthreads();
        qb_cta_lowest_eig<QB_BATCH_MAXN>(n, k, Aw, Yw, M.eps, M.W4, M.W5, M.W6, M.wt, esm);
        qb_cta_gemm_sym(false, true, n, k, Yw, n, Yw, n, M.W3, n);
        qb_cta_gemm(false, false, n, k, n, 1.0, M.X, n, Yw, n, 0.0, M.W4, n);
        qb_cta_gemm_sym(false, true, n, k, M.W4, n, M.W4, n, M.W2, n);
    } else {
        // rotate into the previous eigenvectors, A = C'^T F' C' (W3), and diagonalise
        qb_cta_gemm(false, false, n, n, n, 1.0, M.W2, n, M.Cp, n, 0.0, M.W1, n);
        qb_cta_gemm(true, false, n, n, n, 1.0, M.Cp, n, M.W1, n, 0.0, M.W3, n);
        used = qb_cta_jacobi<QB_BATCH_MAXN>(n, M.W3, M.W1, M.Cp, M.eps, M.wt, M.W2, prm.sweeps, jsm, 1e-24);
        for (int i = tid; i < nn; i += nt) M.Cp[i] = M.W1[i];
        __syncthreads();
        qb_cta_gemm(false, true, n, n, M.nocc, 1.0, M.Cp, n, M.Cp, n, 0.0, M.W3, n);
        qb_cta_gemm(false, false, n, n, n, 1.0, M.X, n, M.W3, n, 0.0, M.W1, n);
        qb_cta_gemm(false, true, n, n, n, 1.0, M.W1, n, M.X, n, 0.0, M.W2, n);
    }
    __syncthreads();
    return used < 0 ? prm.sweeps : used;
}

// the next density to digest: D (AO) with its ratio-scaled copy, and D' (orthonormal)
__device__ void qb_batch_set_density(MolDev& M, const double* Dao, const double* Dorth) {
    const int n = M.n, nn = n * n, tid = threadIdx.x, nt = blockDim.x;
    for (int idx = tid; idx < nn; idx += nt) {
        const int i = idx % n, j = idx / n;
        const double d = Dao[idx];
        M.D[idx] = d;
        M.Dt[idx] = d * M.ratio[i] * M.ratio[j];
        M.Do[idx] = Dorth[idx];
    }
    __syncthreads();
}

__device__ __forceinline__ int qb_stage_len(int method, int diis) {   // max(HFinterMatStoreSizes..., cache size)
    return method == QB_SCF_DD ? 3 : (diis > 3 ? diis : 3);
}

// isOscillateConverged (src/Tools.jl:291-315), minimum-seeking, minLen 10, maxRemains 15, on
// the ring of the last total energies
__device__ bool qb_osc_converged(const MolDev& M, double tar) {
    const int len = M.ne;
    if (len < 10) return false;
    const int slice = min(15, len / 3 + 1);
    if (slice < 2) return false;
    double v[15];
    for (int k = 0; k < slice; ++k) v[k] = M.Er[(len - slice + k) & 31];
    for (int i = 1; i < slice; ++i) {   // insertion sort
        const double t = v[i];
        int j = i - 1;
        while (j >= 0 && v[j] > t) {
            v[j + 1] = v[j];
            --j;
        }
        v[j + 1] = t;
    }
    const int nv = slice / 2 + 1;
    double mean = 0.0;
    for (int k = 0; k < nv; ++k) mean += v[k];
    mean /= nv;
    double var = 0.0;
    for (int k = 0; k < nv; ++k) var += (v[k] - mean) * (v[k] - mean);
    const double sd = nv > 1 ? sqrt(var / (nv - 1)) : 0.0;
    return sd <= 0.8 * tar && fabs(v[0] - M.Er[(len - 1) & 31]) <= tar;
}

// start of a method (initializeHFcore, HartreeFock.jl:1335-1360): a DIIS-type method takes
// the last min(DIISsize, history) entries as its subspace, coefficients 1, 2, ..., m
__device__ void qb_stage_init(MolDev& M, const StepParams& prm) {
    M.nstep = 0;
    M.slen = 0;
    if (M.stage >= prm.nmethod || prm.method[M.stage] == QB_SCF_DD) return;
    const int init = min(prm.diis, M.hlen);
    for (int k = 0; k < init; ++k) {
        M.slist[k] = M.hlist[M.hlen - init + k];
        M.c[k] = (double)(k + 1);
    }
    M.slen = init;
}

// One SCF step of one molecule per thread block (blocks ordered by size, largest first),
// following runHartreeFockCore (src/HartreeFock.jl:1049-1228) method by method: the
// digested density's Fock matrix either finishes a DD half step (directDiag, :1245-1270) or
// is a step's entry (C, D, F, E) that joins the history and the DIIS subspace (:1361-1390),
// is tested for convergence (:1160-1175), oscillation and early termination (:1177-1203),
// after which the next step of the current method starts.
__global__ void __launch_bounds__(QB_BATCH_THREADS) qb_batch_step_kernel(MolDev* mols, const int* __restrict__ order,
                                                                         const StepParams prm, int* active) {
    __shared__ QbJacobiSmem<QB_BATCH_MAXN> jsm;
    __shared__ QbEigSmem<QB_BATCH_MAXN> esm;
    __shared__ double red[33];
    __shared__ double s_B[QB_BATCH_DIIS * QB_BATCH_DIIS], s_v[QB_BATCH_DIIS];
    __shared__ int s_idx[QB_BATCH_POOL], s_slot, s_nlive, s_act, s_stale, s_needF;
    __shared__ double s_diis[QB_BATCH_DIIS + 2][QB_BATCH_DIIS + 3];
    extern __shared__ __align__(16) unsigned char s_dyn[];   // the coefficient solver's state
    QbDiisWork& sw = *reinterpret_cast<QbDiisWork*>(s_dyn);
    MolDev& M = mols[order[blockIdx.x]];
    if (M.conv) return;
    const int n = M.n, nn = n * n, tid = threadIdx.x, nt = blockDim.x;
    const double* r = M.ratio;
    const int it = M.iter;
    if (it == 0) {
        // core-Hamiltonian guess (also after a restart): F = H; drop what the digest accumulated
        for (int i = tid; i < nn; i += nt) {
            M.F[i] = M.H[i];
            M.Jp[i] = 0.0;
            M.Kp[i] = 0.0;
        }
        __syncthreads();
        qb_cta_gemm(false, false, n, n, n, 1.0, M.F, n, M.X, n, 0.0, M.W1, n);
        qb_cta_gemm_sym(true, false, n, n, M.X, n, M.W1, n, M.W2, n);
        const int used = qb_batch_density(M, prm, jsm, esm);
        qb_batch_set_density(M, M.W2, M.W3);
        if (tid == 0) {
            M.sweeps += used;
            M.iter = 1;
            M.phase = 0;
            M.steps = 0;
            M.stage = 0;
            M.nstep = 0;
            M.hlen = M.slen = M.ne = M.nde = 0;
            M.stale = 0;
            atomicAdd(active, 1);
        }
        return;
    }
    // F = H + 2J - K of the digested density (libint-convention accumulators, per-function
    // ratios) and E = tr(D (H + F)) (getE, :339-342, summed over the two equal spins)
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
    const double E = qb_cta_sum(e, red);   // also a barrier: all reads of J', K' are done
    for (int i = tid; i < nn; i += nt) {
        M.Jp[i] = 0.0;
        M.Kp[i] = 0.0;
    }
    __syncthreads();
    // F' = X^T F X (W2)
    qb_cta_gemm(false, false, n, n, n, 1.0, M.F, n, M.X, n, 0.0, M.W1, n);
    qb_cta_gemm_sym(true, false, n, n, M.X, n, M.W1, n, M.W2, n);
    if (M.phase == 1) {
        // second half of a DD step: the entry's density from the eigenvectors of F(D damped)
        const int used = qb_batch_density(M, prm, jsm, esm);
        qb_batch_set_density(M, M.W2, M.W3);
        if (tid == 0) {
            M.sweeps += used;
            M.phase = 0;
            M.iter = it + 1;
            atomicAdd(active, 1);
        }
        return;
    }
    // ---- the entry (D, F, E) of a step: a free pool slot, its e', the Gram entries
    if (tid == 0) {
        unsigned used_mask = 0;
        for (int k = 0; k < M.hlen; ++k) used_mask |= 1u << M.hlist[k];
        for (int k = 0; k < M.slen; ++k) used_mask |= 1u << M.slist[k];
        int slot = 0;
        while (slot < QB_BATCH_POOL - 1 && (used_mask & (1u << slot))) ++slot;
        s_slot = slot;
        int nl = 0;
        for (int k = 0; k < QB_BATCH_POOL; ++k)
            if ((used_mask | (1u << slot)) & (1u << k)) s_idx[nl++] = k;
        s_nlive = nl;
    }
    __syncthreads();
    const int slot = s_slot;
    double* Fs = M.Fs + (size_t)slot * nn;
    double* Ds = M.Ds + (size_t)slot * nn;
    double* Es = M.Es + (size_t)slot * nn;
    // e' = F' D' - D' F' = X^T (F D S - S D F) X (getEresidual, :1298-1299)
    qb_cta_gemm(false, false, n, n, n, 1.0, M.W2, n, M.Do, n, 0.0, M.W1, n);
    double dd = 0.0;
    const int last = M.hlen > 0 ? M.hlist[M.hlen - 1] : -1;
    const double* Dlast = last >= 0 ? M.Ds + (size_t)last * nn : nullptr;
    for (int idx = tid; idx < nn; idx += nt) {
        const int i = idx % n, j = idx / n;
        Es[idx] = M.W1[i + n * j] - M.W1[j + n * i];
        Fs[idx] = M.F[idx];
        Ds[idx] = M.D[idx];
        if (Dlast) {
            const double t = M.D[idx] - Dlast[idx];
            dd += t * t;
        }
    }
    dd = qb_cta_sum(dd, red);
    const double rmsD = 2.0 * sqrt(dd) / n;   // RMS change of the total density 2D (rmsOf, src/Tools.jl:588)
    const int nl = s_nlive;
    // one warp per Gram entry: <e'_new, e'_o> always, <D, F> both ways only when a method of the
    // strategy (EDIIS, ADIIS) uses them
    const int nkind = prm.need_df ? 3 : 1;
    for (int k = tid >> 5; k < nkind * nl; k += nt >> 5) {
        const int o = s_idx[k % nl], kind = k / nl;
        const double* a = kind == 0 ? Es : (kind == 1 ? Ds : M.Ds + (size_t)o * nn);
        const double* b = kind == 0 ? M.Es + (size_t)o * nn : (kind == 1 ? M.Fs + (size_t)o * nn : Fs);
        double dot = 0.0;
        for (int idx = tid & 31; idx < nn; idx += 32) dot = fma(a[idx], b[idx], dot);
        dot = qb_group_sum(dot, 32);
        if ((tid & 31) == 0) {
            if (kind == 0) {
                M.Gee[slot * QB_BATCH_POOL + o] = dot;
                M.Gee[o * QB_BATCH_POOL + slot] = dot;
            } else if (kind == 1) {
                M.Gdf[slot * QB_BATCH_POOL + o] = dot;   // <D_slot, F_o>
            } else {
                M.Gdf[o * QB_BATCH_POOL + slot] = dot;   // <D_o, F_slot>
            }
        }
    }
    __syncthreads();
    // ---- bookkeeping of the step (thread 0), with the RMS(FDS - SDF) test deferred to the
    // few steps whose other criteria make it matter
    const bool first = (M.hlen == 0);
    const int method = prm.method[min(M.stage, prm.nmethod - 1)];
    const double bp = prm.interval[min(M.stage, prm.nmethod - 1)];
    const bool endM = M.stage == prm.nmethod - 1;
    const double fluc = fmax(10 * bp, 1.5e-3), dEosc = fmax(bp, prm.osc);
    const double dE = first ? 0.0 : E - M.Eprev;
    if (tid == 0) {
        int need = 0;
        if (!first) {
            if (fabs(dE) <= bp && rmsD <= prm.r2 * bp) need = 1;
            if (M.nstep > 1 && M.steps > 10 && dE > fluc && prm.osc > 0 && endM) need = 1;
        }
        s_needF = need;
    }
    __syncthreads();
    double dF = -1.0;
    if (s_needF) {   // getErrorNrms (:1230-1237): RMS(F D S - S D F) in the AO basis
        qb_cta_gemm(false, false, n, n, n, 1.0, M.D, n, M.S, n, 0.0, M.W1, n);
        qb_cta_gemm(false, false, n, n, n, 1.0, M.F, n, M.W1, n, 0.0, M.W4, n);
        double ss = 0.0;
        for (int idx = tid; idx < nn; idx += nt) {
            const int i = idx % n, j = idx / n;
            const double t = M.W4[i + n * j] - M.W4[j + n * i];
            ss += t * t;
        }
        dF = sqrt(qb_cta_sum(ss, red)) / n;
    }
    if (tid == 0) {
        M.sE[slot] = 0.5 * E;   // per-spin energy of the entry
        // the entry joins the subspace of a DIIS-type method when one of its own steps made it
        if (!first && method != QB_SCF_DD && M.nstep >= 1) {
            M.slist[M.slen] = slot;
            M.c[M.slen] = 1.0;
            const int L = ++M.slen;
            if (L > 2 && M.sE[M.slist[L - 1]] - M.sE[M.slist[L - 2]] > QB_BATCH_RESET) {
                M.slist[0] = M.slist[L - 2];   // keepOnly! of the second-to-last entry
                M.c[0] = M.c[L - 2];
                M.slen = 1;
            } else if (L > prm.diis) {
                int pi = 0;
                for (int k = 1; k < L; ++k)
                    if (M.sE[M.slist[k]] > M.sE[M.slist[pi]]) pi = k;
                for (int k = pi; k + 1 < L; ++k) {
                    M.slist[k] = M.slist[k + 1];
                    M.c[k] = M.c[k + 1];
                }
                M.slen = L - 1;
            }
        }
        // history (updateHFtempInfo!, :463-477), truncated to the method's memory length
        const int len = qb_stage_len(method, prm.diis);
        while (M.hlen >= len) {
            for (int k = 0; k + 1 < M.hlen; ++k) M.hlist[k] = M.hlist[k + 1];
            --M.hlen;
        }
        M.hlist[M.hlen++] = slot;
        M.Er[M.ne & 31] = E;
        ++M.ne;
        M.stale = 0;
        bool done = false;
        if (first) {
            M.Eprev = E;
            M.dE = 0.0;
            M.rmsD = 0.0;
            qb_stage_init(M, prm);
        } else {
            M.dE = dE;
            M.rmsD = rmsD;
            M.dF = dF;
            M.dEr[M.nde & 3] = dE;
            ++M.nde;
            M.Eprev = E;
            // convergence of the method (:1168-1175): |dE| and RMS(dD) gated by RMS(FDS - SDF)
            // (a failed gate zeroes both thresholds, which dE = dD = 0 still meets)
            bool conv = (fabs(dE) <= bp && rmsD <= prm.r2 * bp && dF <= prm.r1 * bp) || (dE == 0.0 && rmsD == 0.0);
            bool stop = false;
            if (!conv && M.nstep > 1 && M.steps > 10 && dE > fluc) {
                bool isOsc = false;
                if (prm.osc > 0) {
                    isOsc = qb_osc_converged(M, 10 * dEosc);
                    if (isOsc && fabs(dE) <= dEosc &&
                        (endM ? (dF >= 0 && dF <= prm.r1 * dEosc && rmsD <= prm.r2 * dEosc) : true))
                        conv = true;   // converged to an oscillation
                }
                if (!conv && prm.early_stop && !isOsc) {
                    bool raising = M.nde >= 4;
                    for (int j = 0; j < 4 && raising; ++j)
                        if (!(M.dEr[(M.nde - 1 - j) & 3] > 10 * fluc)) raising = false;
                    if (raising) {   // terminateSCF!: roll the last steps back, end the method
                        const int rb = min(4, max(M.hlen - 1, 0));
                        M.hlen -= rb;
                        M.ne -= rb;
                        M.steps -= rb;
                        M.stale = rb > 0;
                        M.Eprev = M.Er[(M.ne - 1) & 31];
                        stop = true;
                    }
                }
            }
            if (conv || stop) {
                if (endM) {
                    M.conv = conv ? 1 : 2;
                    done = true;
                } else {
                    ++M.stage;
                    qb_stage_init(M, prm);
                }
            }
        }
        if (!done && M.iter0 + M.steps >= prm.max_iter) {   // i < maxStep || break (:1144)
            M.conv = 2;
            done = true;
        }
        if (!done && prm.fallback > 0 && !M.restarted && M.steps >= prm.fallback && M.iter0 + M.steps < prm.max_iter) {
            // the supplied initial density has not converged: start again from F = H
            M.iter0 += M.steps;
            M.iter = 0;
            M.restarted = 1;
            done = true;   // the next call makes the core-Hamiltonian guess
            atomicAdd(active, 1);
        }
        s_act = done ? 0 : 1;
        s_stale = M.stale;
        if (!done) {
            ++M.steps;
            ++M.nstep;
        }
    }
    __syncthreads();
    if (!s_act) return;   // stopped (the finish kernel takes the history's last entry) or restarting
    const int meth = prm.method[M.stage];
    const int lst = M.hlist[M.hlen - 1];
    if (s_stale) {
        // after a rollback the step starts from an earlier entry: its F' (W2), D (AO) and D' (Do)
        qb_cta_gemm(false, false, n, n, n, 1.0, M.Fs + (size_t)lst * nn, n, M.X, n, 0.0, M.W1, n);
        qb_cta_gemm_sym(true, false, n, n, M.X, n, M.W1, n, M.W2, n);
        qb_cta_gemm(false, false, n, n, n, 1.0, M.Sh, n, M.Ds + (size_t)lst * nn, n, 0.0, M.W1, n);
        qb_cta_gemm(false, true, n, n, n, 1.0, M.W1, n, M.Sh, n, 0.0, M.Do, n);
        for (int i = tid; i < nn; i += nt) M.D[i] = M.Ds[(size_t)lst * nn + i];
        __syncthreads();
    }
    int used = 0;
    if (meth == QB_SCF_DD) {
        // directDiag: D_damped = (1 - lambda) D(eigenvectors of F_last) + lambda D_last, then its Fock matrix
        for (int i = tid; i < nn; i += nt) M.W5[i] = M.Do[i];   // D'_last
        __syncthreads();
        used = qb_batch_density(M, prm, jsm, esm);
        const double lam = prm.damp;
        for (int idx = tid; idx < nn; idx += nt) {
            const int i = idx % n, j = idx / n;
            const double d = (1.0 - lam) * M.W2[idx] + lam * M.D[idx];
            M.D[idx] = d;
            M.Dt[idx] = d * r[i] * r[j];
            M.Do[idx] = (1.0 - lam) * M.W3[idx] + lam * M.W5[idx];
        }
        __syncthreads();
        if (tid == 0) M.phase = 1;
    } else {
        // DIIS / EDIIS / ADIIS (DIIScore :1301-1315, EDIIScore :1273-1285, ADIIScore :1287-1296)
        const int m = M.slen;
        if (tid == 0) {
            for (int k = 0; k < m; ++k) s_idx[k] = M.slist[k];
        }
        __syncthreads();
        const int L = m - 1;
        for (int q = tid; q < m * m; q += nt) {
            const int i = q % m, j = q / m;
            const int a = s_idx[i], b = s_idx[j], l = s_idx[L];
            double bv;
            if (meth == QB_SCF_DIIS) {
                bv = M.Gee[a * QB_BATCH_POOL + b];
            } else if (meth == QB_SCF_EDIIS) {
                bv = -(M.Gdf[a * QB_BATCH_POOL + a] - M.Gdf[a * QB_BATCH_POOL + b] - M.Gdf[b * QB_BATCH_POOL + a] +
                       M.Gdf[b * QB_BATCH_POOL + b]);
            } else {
                bv = M.Gdf[a * QB_BATCH_POOL + b] - M.Gdf[a * QB_BATCH_POOL + l] - M.Gdf[l * QB_BATCH_POOL + b] +
                     M.Gdf[l * QB_BATCH_POOL + l];
            }
            s_B[i + m * j] = bv;
            if (j == 0) {
                s_v[i] = meth == QB_SCF_DIIS ? 0.0
                                             : (meth == QB_SCF_EDIIS ? M.sE[a]
                                                                     : M.Gdf[a * QB_BATCH_POOL + l] - M.Gdf[l * QB_BATCH_POOL + l]);
            }
        }
        __syncthreads();
        const int sv = prm.solver[M.stage];
        if (m == 1) {
            if (tid == 0) M.c[0] = 1.0;
        } else if (sv == QB_DIIS_LCM && meth == QB_SCF_DIIS) {
            if (tid < 32) {
                const bool ok = qb_diis_coeffs_warp(m, M.Gee, s_idx, M.c, s_diis);
                if (!ok && tid == 0) {   // singular system: extrapolate with the newest entry only
                    for (int k = 0; k < m; ++k) M.c[k] = 0.0;
                    M.c[m - 1] = 1.0;
                }
            }
        } else if (tid < 32) {
            if (sv == QB_DIIS_LCM) qb_cm_solve(sw, m, meth != QB_SCF_DIIS, s_B, m, s_v, M.c);
            else qb_diis_iterative_solve(sw, sv, meth != QB_SCF_DIIS, m, s_B, m, s_v, M.c);
        }
        __syncthreads();
        // F = sum_k c_k F_k (AO) -> F' = X^T F X
        for (int idx = tid; idx < nn; idx += nt) {
            double f = 0.0;
            for (int k = 0; k < m; ++k) f = fma(M.c[k], M.Fs[(size_t)s_idx[k] * nn + idx], f);
            M.W3[idx] = f;
        }
        __syncthreads();
        qb_cta_gemm(false, false, n, n, n, 1.0, M.W3, n, M.X, n, 0.0, M.W1, n);
        qb_cta_gemm_sym(true, false, n, n, M.X, n, M.W1, n, M.W2, n);
        used = qb_batch_density(M, prm, jsm, esm);
        qb_batch_set_density(M, M.W2, M.W3);
    }
    if (tid == 0) {
        M.sweeps += used;
        M.iter = it + 1;
        atomicAdd(active, 1);
    }
}

// After the iterations: each molecule's result is its history's last entry.
__global__ void qb_batch_finish_kernel(MolDev* mols) {
    MolDev& M = mols[blockIdx.x];
    if (M.conv == 3 || M.hlen == 0) return;
    const int nn = M.n * M.n;
    const double* Dfin = M.Ds + (size_t)M.hlist[M.hlen - 1] * nn;
    for (int i = threadIdx.x; i < nn; i += blockDim.x) M.D[i] = Dfin[i];
    if (threadIdx.x == 0) M.E = 2.0 * M.sE[M.hlist[M.hlen - 1]];
}

// Loop condition of the SCF graph: another pass while some molecule iterates, at most
// `cap` passes in all.
__global__ void qb_batch_cond_kernel(cudaGraphConditionalHandle handle, const int* active, int* passes, int cap) {
    const int p = ++(*passes);
    cudaGraphSetConditional(handle, (*active > 0 && p < cap) ? 1u : 0u);
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
    cfg->nmethod = 0;   // one DIIS method at conv_energy with exact (Lagrange-multiplier) coefficients
    for (int l = 0; l < 8; ++l) {
        cfg->method[l] = QB_SCF_DIIS;
        cfg->interval[l] = 0.0;
        cfg->solver[l] = QB_DIIS_LBFGS;
    }
    cfg->secondary_ratio[0] = 1000.0;
    cfg->secondary_ratio[1] = 1000.0;
    cfg->oscillate_threshold = 5e-6;
    cfg->early_stop = 1;
    cfg->damp_strength = 0.75;
    cfg->digest_chunk = 0;
}

int qb_batch_rhf_run(qb_ctx* ctx, int nmol, const qb_basis* bases, const int* nnuc, const double* Z,
                     const double* R, const int* nocc, const qb_batch_config* cfg_in, qb_batch_result* res) {
    if (nmol <= 0 || !bases || !nnuc || !Z || !R || !nocc || !res)
        return qb_set_error(ctx, QB_ERR_ARG, "bad batched SCF arguments");
    qb_batch_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else qb_batch_config_default(&cfg);
    if (cfg.diis_size < 1 || cfg.diis_size > QB_BATCH_DIIS || cfg.max_iter < 1 || cfg.iters_per_graph < 1 ||
        cfg.fallback_iter < 0 || cfg.digest_chunk < 0 ||
        !(cfg.schwarz >= 0.0) || !(cfg.conv_energy > 0.0) || !(cfg.conv_density > 0.0))
        return qb_set_error(ctx, QB_ERR_DOMAIN, "bad batched SCF configuration");
    if (cfg.nmethod < 0 || cfg.nmethod > 8) return qb_set_error(ctx, QB_ERR_ARG, "nmethod must be 0..8");
    for (int l = 0; l < cfg.nmethod; ++l) {
        if (cfg.method[l] < QB_SCF_DD || cfg.method[l] > QB_SCF_ADIIS || !(cfg.interval[l] >= 0.0))
            return qb_set_error(ctx, QB_ERR_ARG, "bad SCF method or threshold");
        if (cfg.solver[l] < QB_DIIS_LBFGS || cfg.solver[l] > QB_DIIS_LCM)
            return qb_set_error(ctx, QB_ERR_ARG, "unknown DIIS coefficient solver");
    }
    if (cfg.nmethod > 0 && (!(cfg.damp_strength >= 0.0 && cfg.damp_strength <= 1.0) ||
                            !(cfg.secondary_ratio[0] > 0.0) || !(cfg.secondary_ratio[1] > 0.0)))
        return qb_set_error(ctx, QB_ERR_DOMAIN, "bad damping or secondary convergence ratio");
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
    const int nbase = 17;   // S, H, X, S^1/2, F, D, Dt, D', J', K', C', 6 work matrices
    const int nmat = nbase + 3 * QB_BATCH_POOL;
    DevArray<double> d_mats, d_vecs, d_G;
    QB_CUDA(ctx, d_mats.ensure((size_t)nmat * NN));
    QB_CUDA(ctx, d_vecs.ensure(2 * (size_t)vo[nmol]));
    QB_CUDA(ctx, d_G.ensure((size_t)nmol * 2 * QB_BATCH_POOL * QB_BATCH_POOL));
    QB_CUDA(ctx, cudaMemsetAsync(d_G.p, 0, (size_t)nmol * 2 * QB_BATCH_POOL * QB_BATCH_POOL * sizeof(double), s));
    std::vector<MolDev> hm(nmol);
    for (int m = 0; m < nmol; ++m) {
        MolDev& M = hm[m];
        std::memset(&M, 0, sizeof(M));
        M.n = nf[m];
        M.nocc = nocc[m];
        double* mat[17];
        for (int k = 0; k < 17; ++k) mat[k] = d_mats.p + (size_t)k * NN + mo[m];
        M.S = mat[0]; M.H = mat[1]; M.X = mat[2]; M.F = mat[3]; M.D = mat[4]; M.Dt = mat[5]; M.Do = mat[6];
        M.Jp = mat[7]; M.Kp = mat[8]; M.Cp = mat[9]; M.W1 = mat[10]; M.W2 = mat[11]; M.W3 = mat[12];
        M.W4 = mat[13]; M.W5 = mat[14]; M.W6 = mat[15]; M.Sh = mat[16];
        M.Fs = d_mats.p + (size_t)nbase * NN + (size_t)QB_BATCH_POOL * mo[m];
        M.Ds = d_mats.p + (size_t)(nbase + QB_BATCH_POOL) * NN + (size_t)QB_BATCH_POOL * mo[m];
        M.Es = d_mats.p + (size_t)(nbase + 2 * QB_BATCH_POOL) * NN + (size_t)QB_BATCH_POOL * mo[m];
        M.Gee = d_G.p + (size_t)m * 2 * QB_BATCH_POOL * QB_BATCH_POOL;
        M.Gdf = M.Gee + QB_BATCH_POOL * QB_BATCH_POOL;

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
    // primitive Schwarz keys (as in the single-basis J/K engine): each primitive pair's
    // screening key becomes its own Schwarz factor, the primitives of a shell pair are
    // re-sorted by it and the negligible ones dropped; the stores then skip primitive
    // quartets whose keys multiply to < QB_PRIM_EPS_Q
    {
        DevArray<unsigned> d_keymax;
        QB_CUDA(ctx, d_keymax.ensure(1));
        QB_CUDA(ctx, cudaMemsetAsync(d_keymax.p, 0, sizeof(unsigned), s));
        for (int pc = 0; pc < npc; ++pc) {
            const int n = pc_off[pc + 1] - pc_off[pc];
            if (n == 0) continue;
            const ShellPair* pp = d_pairs.p + pc_off[pc];
            const int g = (n + 127) / 128;
            if (pc == 0) qb_prim_key_kernel<0, 0><<<g, 128, 0, s>>>(pp, n, d_prims.p, ctx->boys.p, d_keymax.p);
            else if (pc == 1) qb_prim_key_kernel<1, 0><<<g, 128, 0, s>>>(pp, n, d_prims.p, ctx->boys.p, d_keymax.p);
            else qb_prim_key_kernel<1, 1><<<g, 128, 0, s>>>(pp, n, d_prims.p, ctx->boys.p, d_keymax.p);
            QB_CUDA(ctx, cudaGetLastError());
        }
        if (qb_compact_prim_keys(s, d_pairs.p, npair, d_prims.p, d_prims32.p, nslot, d_keymax.p,
                                 (float)QB_PRIM_EPS_Q, d_nkept.p) != 0)
            return qb_cuda_check(ctx, cudaGetLastError(), "batched primitive Schwarz keys");
        std::vector<int> nkept(npair);
        QB_CUDA(ctx, cudaMemcpyAsync(nkept.data(), d_nkept.p, npair * sizeof(int), cudaMemcpyDeviceToHost, s));
        QB_CUDA(ctx, cudaStreamSynchronize(s));
        for (int k = 0; k < npair; ++k) pairs[k].nprim = nkept[k];
    }
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
    // ---- digest chunks: per class and molecule, runs of at most `big` quartets (`small` for
    // a molecule with fewer than 128 such runs in the class: its late iterations then still
    // spread over many SMs).  The sizes are tuned on this batch: one digest pass of every
    // class timed per candidate pair before the iterations start (the densities are zeroed
    // for it, and J', K' after it).
    std::vector<DigestChunk> h_chunks;
    std::vector<size_t> chunk_at(QB_BATCH_NCLASS + 1, 0);
    auto build_chunks = [&](long long big, long long small) {
        h_chunks.clear();
        for (int c = 0; c < QB_BATCH_NCLASS; ++c) {
            chunk_at[c] = h_chunks.size();
            const ClassDef& cd = kClasses[c];
            const int X = pc_of(cd.la, cd.lb);
            const long long* off = h_offs.data() + offs_at[c];
            for (int m = 0; m < nmol; ++m) {
                const int s0 = seg[X][m], s1 = seg[X][m + 1];
                const long long chunk = (off[s1] - off[s0]) >= 128LL * big ? big : small;
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
    };
    static const long long kChunkCand[3][2] = {{QB_DIGEST_CHUNK / 2, QB_DIGEST_CHUNK_SMALL / 2},
                                               {QB_DIGEST_CHUNK, QB_DIGEST_CHUNK_SMALL},
                                               {2 * QB_DIGEST_CHUNK, 2 * QB_DIGEST_CHUNK_SMALL}};
    // size the chunk table for the finest split that may be used
    if (cfg.digest_chunk > 0 && cfg.digest_chunk < kChunkCand[0][0])
        build_chunks(cfg.digest_chunk, std::max(1LL, (long long)cfg.digest_chunk / 4));
    else
        build_chunks(kChunkCand[0][0], kChunkCand[0][1]);
    DevArray<DigestChunk> d_chunks;
    QB_CUDA(ctx, d_chunks.ensure(std::max<size_t>(1, h_chunks.size())));
    int best_cand = 1;
    if (cfg.digest_chunk > 0) {
        best_cand = -1;   // fixed by the caller
    } else {
        QB_CUDA(ctx, cudaMemsetAsync(d_mats.p + 5 * (size_t)NN, 0, NN * sizeof(double), s));   // D~
        float best_ms = -1.f;
        for (int k = 0; k < 3; ++k) {
            build_chunks(kChunkCand[k][0], kChunkCand[k][1]);
            if (h_chunks.empty()) break;
            QB_CUDA(ctx, cudaMemcpyAsync(d_chunks.p, h_chunks.data(), h_chunks.size() * sizeof(DigestChunk),
                                         cudaMemcpyHostToDevice, s));
            float ms = 0.f;   // one pass each: the stored integrals exceed L2, nothing to warm
            QB_CUDA(ctx, cudaEventRecord(ctx->ev_start, s));
            for (int c = 0; c < QB_BATCH_NCLASS; ++c) {
                const int nch = (int)(chunk_at[c + 1] - chunk_at[c]);
                if (nch > 0)
                    kClasses[c].digest(work[c], d_chunks.p + chunk_at[c], d_eri.p + eri_at[c], d_mols.p, nch, s);
            }
            QB_CUDA(ctx, cudaEventRecord(ctx->ev_stop, s));
            QB_CUDA(ctx, cudaEventSynchronize(ctx->ev_stop));
            QB_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
            if (best_ms < 0.f || ms < best_ms) {
                best_ms = ms;
                best_cand = k;
            }
        }
        QB_CUDA(ctx, cudaMemsetAsync(d_mats.p + 7 * (size_t)NN, 0, 2 * NN * sizeof(double), s));   // J', K'
    }
    const long long chunk_big = best_cand >= 0 ? kChunkCand[best_cand][0] : (long long)cfg.digest_chunk;
    const long long chunk_small = best_cand >= 0 ? kChunkCand[best_cand][1] : std::max(1LL, chunk_big / 4);
    build_chunks(chunk_big, chunk_small);
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
    StepParams prm;
    std::memset(&prm, 0, sizeof(prm));
    if (cfg.nmethod == 0) {   // SCFconfig((:DIIS,), (conv_energy,), Dict(1=>[:solver=>:LCM])), RMS(dD) <= conv_density
        prm.nmethod = 1;
        prm.method[0] = QB_SCF_DIIS;
        prm.interval[0] = cfg.conv_energy;
        prm.solver[0] = QB_DIIS_LCM;
        prm.r1 = 1e6;
        prm.r2 = cfg.conv_density / cfg.conv_energy;
        prm.osc = 5e-6;
        prm.early_stop = 1;
        prm.damp = 0.75;
    } else {
        prm.nmethod = cfg.nmethod;
        for (int l = 0; l < cfg.nmethod; ++l) {
            prm.method[l] = cfg.method[l];
            prm.interval[l] = cfg.interval[l];
            prm.solver[l] = cfg.solver[l];
        }
        prm.r1 = cfg.secondary_ratio[0];
        prm.r2 = cfg.secondary_ratio[1];
        prm.osc = cfg.oscillate_threshold;
        prm.early_stop = cfg.early_stop;
        prm.damp = cfg.damp_strength;
    }
    for (int l = 0; l < prm.nmethod; ++l)
        if (prm.method[l] == QB_SCF_EDIIS || prm.method[l] == QB_SCF_ADIIS) prm.need_df = 1;
    prm.max_iter = cfg.max_iter;
    prm.diis = std::max(2, cfg.diis_size);
    prm.sweeps = cfg.jacobi_sweeps > 0 ? std::min(cfg.jacobi_sweeps, 60) : 60;
    prm.eig = cfg.eigensolver ? 1 : 0;
    prm.fallback = cfg.initial_density && cfg.fallback_iter > 0 ? cfg.fallback_iter : 0;
    int* d_active = d_counters.p + 1;
    DevArray<int> d_passes;
    QB_CUDA(ctx, d_passes.ensure(1));
    QB_CUDA(ctx, cudaMemsetAsync(d_passes.p, 0, sizeof(int), s));
    // one SCF pass: the digest of every iterating molecule's density, then its step
    auto pass = [&](cudaStream_t st) {
        cudaMemsetAsync(d_active, 0, sizeof(int), st);
        for (int c = 0; c < QB_BATCH_NCLASS; ++c) {
            const int nch = (int)(chunk_at[c + 1] - chunk_at[c]);
            if (nch == 0) continue;
            kClasses[c].digest(work[c], d_chunks.p + chunk_at[c], d_eri.p + eri_at[c], d_mols.p, nch, st);
        }
        qb_batch_step_kernel<<<nmol, QB_BATCH_THREADS, sizeof(QbDiisWork), st>>>(d_mols.p, d_order.p, prm, d_active);
    };
    QB_CUDA(ctx, cudaFuncSetAttribute(qb_batch_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(QbDiisWork)));
    // every molecule needs at most 2 passes per SCF step, plus the guesses (a restart doubles them)
    const int cap = 2 * cfg.max_iter + 8;
    int launches = 0;
    int rc = QB_OK;
    {
        // the whole iteration in one launch: a graph whose conditional while-node repeats the
        // pass until no molecule iterates (or `cap` passes)
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaGraphConditionalHandle handle;
        bool ok = cudaGraphCreate(&graph, 0) == cudaSuccess &&
                  cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault) == cudaSuccess;
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cudaGraphNode_t node;
        if (ok) {
            cp.conditional.handle = handle;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            ok = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp) == cudaSuccess;
        }
        if (ok) {
            ok = cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) {
                pass(s);
                qb_batch_cond_kernel<<<1, 1, 0, s>>>(handle, d_active, d_passes.p, cap);
                cudaGraph_t body = nullptr;
                ok = cudaStreamEndCapture(s, &body) == cudaSuccess;
            }
        }
        if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
        if (ok) {
            rc = qb_cuda_check(ctx, cudaGraphLaunch(exec, s), "SCF graph launch");
            launches = 1;
            if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaStreamSynchronize(s), "SCF graph");
        } else {
            cudaGetLastError();   // conditional nodes unavailable: fall back to host-driven launches
        }
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (!ok && rc == QB_OK) {
            // several passes per captured graph, the host checking between launches
            cudaGraph_t g2 = nullptr;
            cudaGraphExec_t e2 = nullptr;
            QB_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            for (int k = 0; k < cfg.iters_per_graph; ++k) pass(s);
            QB_CUDA(ctx, cudaStreamEndCapture(s, &g2));
            QB_CUDA(ctx, cudaGraphInstantiate(&e2, g2, 0));
            int active = nmol;
            const int max_launch = (cap + cfg.iters_per_graph - 1) / cfg.iters_per_graph;
            while (active > 0 && launches < max_launch) {
                rc = qb_cuda_check(ctx, cudaGraphLaunch(e2, s), "graph launch");
                if (rc != QB_OK) break;
                ++launches;
                rc = qb_cuda_check(ctx, cudaMemcpyAsync(&active, d_active, sizeof(int), cudaMemcpyDeviceToHost, s),
                                   "active count");
                if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaStreamSynchronize(s), "SCF graph");
                if (rc != QB_OK) break;
            }
            cudaGraphExecDestroy(e2);
            cudaGraphDestroy(g2);
        }
    }
    QB_TRY(rc);
    qb_batch_finish_kernel<<<nmol, 256, 0, s>>>(d_mols.p);
    QB_CUDA(ctx, cudaGetLastError());
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
    res->digest_chunk = (int)chunk_big;
    int failed = 0;
    for (int m = 0; m < nmol; ++m) {
        if (res->energy) res->energy[m] = hm[m].E;
        if (res->iterations) res->iterations[m] = hm[m].iter0 + hm[m].steps;
        if (res->restarted) res->restarted[m] = hm[m].restarted;
        if (res->converged) res->converged[m] = hm[m].conv == 1 ? 1 : 0;
        if (res->jacobi_sweeps) res->jacobi_sweeps[m] = hm[m].sweeps;
        failed += hm[m].conv == 3;
    }
    if (failed) return qb_set_error(ctx, QB_ERR_DOMAIN, "batched SCF: overlap matrix not positive definite");
    return QB_OK;
}
