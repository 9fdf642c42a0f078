// Dense linear algebra run by one thread block (CTA): the small matrices of the SCF
// (N <= a few hundred) live in global memory / L2 and every thread of the block takes
// part.  Column-major storage throughout.
#pragma once
#include <cuda_runtime.h>

// Block-wide sum of one double per thread; every thread gets the result.  red must hold
// 33 doubles of shared memory.
__device__ __forceinline__ double qb_cta_sum(double v, double* red) {
    const int tid = threadIdx.x, nw = (blockDim.x + 31) >> 5;
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    __syncthreads();   // the previous call's readers are done with red
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    double t = 0.0;    // every thread sums the warp totals in the same order
    for (int k = 0; k < nw; ++k) t += red[k];
    return t;
}

// Lanes per row for a dot product per row of `rows` rows over nt threads: the largest
// power of two <= min(32, nt / rows) (1 when rows >= nt / 2).
__device__ __forceinline__ int qb_group_lanes(int nt, int rows) {
    int L = 1;
    while (L < 32 && 2 * L * rows <= nt) L <<= 1;
    return L;
}

// Sum over aligned groups of L lanes (L a power of two <= 32); every lane of the warp
// must call it.
__device__ __forceinline__ double qb_group_sum(double v, int L) {
    for (int o = L >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// C = alpha op(A) op(B) + beta C, op(A) m x k, op(B) k x n.  beta == 0 ignores C's contents.
// Ends with a block barrier.
static __device__ void qb_cta_gemm(bool tA, bool tB, int m, int n, int k, double alpha, const double* A, int lda,
                                   const double* B, int ldb, double beta, double* C, int ldc) {
    for (int idx = threadIdx.x; idx < m * n; idx += blockDim.x) {
        const int i = idx % m, j = idx / m;
        double s = 0.0;
        if (!tA && !tB) {
            for (int p = 0; p < k; ++p) s = fma(A[i + (size_t)lda * p], B[p + (size_t)ldb * j], s);
        } else if (tA && !tB) {
            for (int p = 0; p < k; ++p) s = fma(A[p + (size_t)lda * i], B[p + (size_t)ldb * j], s);
        } else if (!tA && tB) {
            for (int p = 0; p < k; ++p) s = fma(A[i + (size_t)lda * p], B[j + (size_t)ldb * p], s);
        } else {
            for (int p = 0; p < k; ++p) s = fma(A[p + (size_t)lda * i], B[j + (size_t)ldb * p], s);
        }
        C[i + (size_t)ldc * j] = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * C[i + (size_t)ldc * j]);
    }
    __syncthreads();
}

// C = op(A) op(B) (n x n, k inner) for a product known to be symmetric (X^T (F X), Y Y^T,
// (X Y)(X Y)^T): each entry i <= j is computed once and written to both (i, j) and (j, i).
// Ends with a block barrier.
static __device__ void qb_cta_gemm_sym(bool tA, bool tB, int n, int k, const double* A, int lda, const double* B,
                                       int ldb, double* C, int ldc) {
    const int npair = n * (n + 1) / 2;
    for (int idx = threadIdx.x; idx < npair; idx += blockDim.x) {
        // idx -> (i, j), j >= i, packed column by column (FP32 estimate, exact after the
        // corrections: 8 idx + 1 < 2^24 for n <= 2048)
        int j = (int)((sqrtf(8.0f * (float)idx + 1.0f) - 1.0f) * 0.5f);
        while (j * (j + 1) / 2 > idx) --j;
        while ((j + 1) * (j + 2) / 2 <= idx) ++j;
        const int i = idx - j * (j + 1) / 2;
        double s = 0.0;
        if (!tA && !tB) {
            for (int p = 0; p < k; ++p) s = fma(A[i + (size_t)lda * p], B[p + (size_t)ldb * j], s);
        } else if (tA && !tB) {
            for (int p = 0; p < k; ++p) s = fma(A[p + (size_t)lda * i], B[p + (size_t)ldb * j], s);
        } else if (!tA && tB) {
            for (int p = 0; p < k; ++p) s = fma(A[i + (size_t)lda * p], B[j + (size_t)ldb * p], s);
        } else {
            for (int p = 0; p < k; ++p) s = fma(A[p + (size_t)lda * i], B[j + (size_t)ldb * p], s);
        }
        C[i + (size_t)ldc * j] = s;
        C[j + (size_t)ldc * i] = s;
    }
    __syncthreads();
}

// Shared-memory scratch of qb_cta_jacobi for matrices up to MAXN.
template <int MAXN>
struct QbJacobiSmem {
    double cs[MAXN / 2], sn[MAXN / 2];
    int pp[MAXN / 2], qq[MAXN / 2];
    int pos[MAXN];
    double red[33];
    int rotated;
};

// Eigen-decomposition of the symmetric n x n matrix A (destroyed) by the cyclic Jacobi
// method with parallel round-robin ordering (each round rotates n/2 disjoint (p, q)
// planes).  V (n x n) receives the eigenvectors in columns, w the eigenvalues, both
// in ascending order; wtmp (n) and Vtmp (n x n) are scratch.  If Vin is non-null the
// rotations are applied to a copy of Vin instead of the identity (V = Vin * rotations:
// eigenvectors of Vin A Vin^T for orthogonal Vin).  A plane (p, q) is rotated only while
// |a_pq| > 1e-15 sqrt(|a_pp a_qq|) (below that the rotation changes nothing at double
// precision); converged when off(A)^2 <= tol2 ||A||^2 (default 1e-30), when a sweep rotated no plane, or
// when off(A)^2 <= 1e-24 ||A||^2 stopped shrinking (rounding level: it fell by less than
// 4x in the last sweep).  At most maxsweep sweeps; returns the number used, or -1 if not
// converged (off(A) is then still reported small enough by the caller's own test).
template <int MAXN>
__device__ int qb_cta_jacobi(int n, double* A, double* V, const double* Vin, double* w, double* wtmp, double* Vtmp,
                             int maxsweep, QbJacobiSmem<MAXN>& sm, double tol2 = 1e-30) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int m = n + (n & 1);
    const int half = m / 2;
    for (int i = tid; i < n * n; i += nt) V[i] = Vin ? Vin[i] : (((i % n) == (i / n)) ? 1.0 : 0.0);
    __syncthreads();
    int used = -1;
    double off_prev = 0.0;
    for (int sweep = 0; sweep <= maxsweep; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = tid; i < n * n; i += nt) {
            const double a = A[i];
            tot += a * a;
            if ((i % n) != (i / n)) off += a * a;
        }
        off = qb_cta_sum(off, sm.red);   // block-uniform
        tot = qb_cta_sum(tot, sm.red);
        const int rotated = sm.rotated;   // every thread reads the flag before it is reset
        __syncthreads();
        if (off <= tol2 * tot || off == 0.0 || (sweep > 0 && rotated == 0) ||
            (sweep > 0 && off <= 1e-24 * tot && off > 0.25 * off_prev)) {
            used = sweep;
            break;
        }
        off_prev = off;
        if (sweep == maxsweep) break;
        for (int i = tid; i < m; i += nt) sm.pos[i] = i;
        if (tid == 0) sm.rotated = 0;
        __syncthreads();
        for (int round = 0; round < m - 1; ++round) {
            for (int k = tid; k < half; k += nt) {
                int p = sm.pos[k], q = sm.pos[m - 1 - k];
                if (p > q) { const int t = p; p = q; q = t; }
                double c = 1.0, s = 0.0;
                if (q < n) {
                    const double apq = A[p + (size_t)n * q];
                    const double app = A[p + (size_t)n * p], aqq = A[q + (size_t)n * q];
                    if (fabs(apq) > 1e-300 && fabs(apq) > 1e-15 * sqrt(fabs(app * aqq))) {
                        const double theta = (aqq - app) / (2.0 * apq);
                        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        c = 1.0 / sqrt(t * t + 1.0);
                        s = t * c;
                        sm.rotated = 1;
                    }
                }
                sm.pp[k] = p; sm.qq[k] = q; sm.cs[k] = c; sm.sn[k] = s;
            }
            __syncthreads();
            // columns p, q of A and V
            for (int idx = tid; idx < half * n; idx += nt) {
                const int k = idx / n, r = idx % n;
                const int p = sm.pp[k], q = sm.qq[k];
                if (q >= n || sm.sn[k] == 0.0) continue;
                const double c = sm.cs[k], s = sm.sn[k];
                const double ap = A[r + (size_t)n * p], aq = A[r + (size_t)n * q];
                A[r + (size_t)n * p] = c * ap - s * aq;
                A[r + (size_t)n * q] = s * ap + c * aq;
                const double vp = V[r + (size_t)n * p], vq = V[r + (size_t)n * q];
                V[r + (size_t)n * p] = c * vp - s * vq;
                V[r + (size_t)n * q] = s * vp + c * vq;
            }
            __syncthreads();
            // rows p, q of A
            for (int idx = tid; idx < half * n; idx += nt) {
                const int k = idx / n, col = idx % n;
                const int p = sm.pp[k], q = sm.qq[k];
                if (q >= n || sm.sn[k] == 0.0) continue;
                const double c = sm.cs[k], s = sm.sn[k];
                const double ap = A[p + (size_t)n * col], aq = A[q + (size_t)n * col];
                A[p + (size_t)n * col] = c * ap - s * aq;
                A[q + (size_t)n * col] = s * ap + c * aq;
            }
            __syncthreads();
            if (tid == 0) {   // rotate positions 1..m-1
                const int last = sm.pos[m - 1];
                for (int i = m - 1; i > 1; --i) sm.pos[i] = sm.pos[i - 1];
                sm.pos[1] = last;
            }
            __syncthreads();
        }
    }
    // ascending order (stable by index)
    for (int i = tid; i < n; i += nt) wtmp[i] = A[i + (size_t)n * i];
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
        const double wi = wtmp[i];
        int r = 0;
        for (int j = 0; j < n; ++j) {
            const double wj = wtmp[j];
            r += (wj < wi) || (wj == wi && j < i);
        }
        w[r] = wi;
        for (int row = 0; row < n; ++row) Vtmp[row + (size_t)n * r] = V[row + (size_t)n * i];
    }
    __syncthreads();
    for (int i = tid; i < n * n; i += nt) V[i] = Vtmp[i];
    __syncthreads();
    return used;
}

// ---------------------------------------------------------------------------
// Lowest eigenpairs of a symmetric matrix by one thread block: Householder
// tridiagonalisation, FP32 bisection on Sturm counts for the k lowest eigenvalues (the
// FP32 pipe is ~64x the FP64 one on this GPU), FP64 Rayleigh-quotient inverse iteration
// with a pivoted tridiagonal LU for the eigenvectors, Gram-Schmidt within clusters of
// close eigenvalues, and the back-transformation by the stored reflectors.  About
// (4/3) n^3 + 2 n^2 k FMAs against ~4 n^3 per Jacobi sweep.
template <int MAXN>
struct QbEigSmem {
    double d[MAXN], e[MAXN], lam[MAXN], dots[MAXN];
    double lamr[MAXN];           // eigenvalue estimates after the FP64 refinement
    float lamw[MAXN];            // half width of each eigenvalue's FP32 bracket
    float df[MAXN], e2f[MAXN];   // d and e^2 in FP32 for the Sturm counts
    double red[33];
    double bounds[3];
};

// A (n x n, column-major, destroyed) -> d, e; reflector k (unit vector, length n-k-1)
// stored in A[k+1 .. n-1, k].  p is n doubles of scratch.
template <int MAXN>
__device__ void qb_cta_tridiag(int n, double* A, double* p, QbEigSmem<MAXN>& sm) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int k = 0; k + 2 < n; ++k) {
        const int m = n - k - 1;
        double* x = A + (k + 1) + (size_t)n * k;
        double s = 0.0;
        for (int i = tid; i < m; i += nt) s += x[i] * x[i];
        s = qb_cta_sum(s, sm.red);
        const double x0 = x[0];
        const double alpha = (s > 0.0) ? -copysign(sqrt(s), x0) : 0.0;
        const double vn2 = 2.0 * s - 2.0 * x0 * alpha;
        const bool refl = s > 0.0 && vn2 > 0.0;
        if (tid == 0) {
            sm.d[k] = A[k + (size_t)n * k];
            sm.e[k] = refl ? alpha : x0;
        }
        __syncthreads();   // x0 read by every thread before x is overwritten
        if (!refl) {
            for (int i = tid; i < m; i += nt) x[i] = 0.0;
            __syncthreads();
            continue;
        }
        const double inv = 1.0 / sqrt(vn2);
        for (int i = tid; i < m; i += nt) x[i] = (i == 0 ? x0 - alpha : x[i]) * inv;
        __syncthreads();
        double* S = A + (k + 1) + (size_t)n * (k + 1);
        // p = S x: L lanes per row (shorter dependent chains), row i's total on its first lane
        const int L = qb_group_lanes(nt, m);
        double K = 0.0;
        for (int i0 = 0; i0 < m; i0 += nt / L) {
            const int i = i0 + tid / L, sub = tid % L;
            double acc = 0.0;
            if (i < m)
                for (int j = sub; j < m; j += L) acc = fma(S[i + (size_t)n * j], x[j], acc);
            acc = qb_group_sum(acc, L);
            if (i < m && sub == 0) {
                p[i] = acc;
                K += x[i] * acc;
            }
        }
        K = qb_cta_sum(K, sm.red);
        for (int i0 = 0; i0 < m; i0 += nt / L) {
            const int i = i0 + tid / L;
            if (i < m && tid % L == 0) p[i] -= K * x[i];
        }
        __syncthreads();
        for (int idx = tid; idx < m * m; idx += nt) {
            const int i = idx % m, j = idx / m;
            S[i + (size_t)n * j] -= 2.0 * (x[i] * p[j] + p[i] * x[j]);
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (n >= 2) {
            sm.d[n - 2] = A[(n - 2) + (size_t)n * (n - 2)];
            sm.e[n - 2] = A[(n - 1) + (size_t)n * (n - 2)];
        }
        sm.d[n - 1] = A[(n - 1) + (size_t)n * (n - 1)];
    }
    __syncthreads();
}

// number of eigenvalues of the tridiagonal (d, e) below x, in FP32 (pivots of the LDL^T
// factorisation of T - x I from df = d and e2f = e^2; a pivot smaller than `tiny` is
// replaced by -tiny and counted as negative, which keeps the count consistent when x
// hits a pivot exactly)
__device__ __forceinline__ int qb_sturm_f(int n, const float* df, const float* e2f, float x, float tiny) {
    float q = df[0] - x;
    if (fabsf(q) <= tiny) q = -tiny;
    int c = q < 0.f;
    for (int j = 1; j < n; ++j) {
        q = (df[j] - x) - __fdividef(e2f[j - 1], q);
        if (fabsf(q) <= tiny) q = -tiny;
        c += q < 0.f;
    }
    return c;
}

// the same count in FP64 (for eigenvalues the FP32 brackets cannot separate)
__device__ __forceinline__ int qb_sturm_d(int n, const double* d, const double* e, double x, double tiny) {
    double q = d[0] - x;
    if (fabs(q) <= tiny) q = -tiny;
    int c = q < 0.0;
    for (int j = 1; j < n; ++j) {
        q = (d[j] - x) - e[j - 1] * e[j - 1] / q;
        if (fabs(q) <= tiny) q = -tiny;
        c += q < 0.0;
    }
    return c;
}

// The multiplier of an LU row carries the row's swap flag in its lowest mantissa bit (a
// one-ulp change of the multiplier).
__device__ __forceinline__ double qb_flagged(double f, bool swap) {
    return __longlong_as_double((__double_as_longlong(f) & ~1LL) | (swap ? 1LL : 0LL));
}
__device__ __forceinline__ bool qb_flag(double f) { return __double_as_longlong(f) & 1LL; }

// LU of T - lam I (T tridiagonal d, e) by Gaussian elimination with partial pivoting: rows
// j and j + 1 swap when |e_j| exceeds the pivot, a zero pivot becomes `pert`.  Per row j
// the reciprocal pivot u0i, the superdiagonal u1 and the flagged multiplier fm; the second
// superdiagonal of a swapped row is e_{j+1} (of an unswapped row 0).  Arrays strided by ld.
static __device__ void qb_tridiag_factor(int n, const double* d, const double* e, double lam, double pert,
                                         double* u0i, double* u1, double* fm, int ld) {
    double m0 = d[0] - lam, m1 = n > 1 ? e[0] : 0.0;
    for (int j = 0; j + 1 < n; ++j) {
        const double l = e[j], a = d[j + 1] - lam, b = (j + 2 < n) ? e[j + 1] : 0.0;
        if (fabs(l) > fabs(m0)) {
            const double f = m0 / l;
            u0i[(size_t)ld * j] = 1.0 / l;
            u1[(size_t)ld * j] = a;
            fm[(size_t)ld * j] = qb_flagged(f, true);
            m0 = m1 - f * a;
            m1 = -f * b;
        } else {
            if (m0 == 0.0) m0 = pert;
            const double f = l / m0;
            u0i[(size_t)ld * j] = 1.0 / m0;
            u1[(size_t)ld * j] = m1;
            fm[(size_t)ld * j] = qb_flagged(f, false);
            m0 = a - f * m1;
            m1 = b;
        }
    }
    if (m0 == 0.0) m0 = pert;
    u0i[(size_t)ld * (n - 1)] = 1.0 / m0;
    u1[(size_t)ld * (n - 1)] = 0.0;
    fm[(size_t)ld * (n - 1)] = 0.0;
}

// y <- (T - lam I)^{-1} y with the factors of qb_tridiag_factor (same stride ld).
static __device__ void qb_tridiag_apply(int n, const double* e, const double* u0i, const double* u1,
                                        const double* fm, double* y, int ld) {
    double cur = y[0];
    for (int j = 0; j + 1 < n; ++j) {
        const double f = fm[(size_t)ld * j], nxt = y[(size_t)ld * (j + 1)];
        const bool sw = qb_flag(f);
        const double a = sw ? nxt : cur, b = sw ? cur : nxt;
        y[(size_t)ld * j] = a;
        cur = b - f * a;
    }
    y[(size_t)ld * (n - 1)] = cur;
    double z1 = 0.0, z2 = 0.0;   // z_{j+1}, z_{j+2}
    for (int j = n - 1; j >= 0; --j) {
        double s = y[(size_t)ld * j] - u1[(size_t)ld * j] * z1;
        if (j + 2 < n && qb_flag(fm[(size_t)ld * j])) s -= e[j + 1] * z2;
        const double z = s * u0i[(size_t)ld * j];
        y[(size_t)ld * j] = z;
        z2 = z1;
        z1 = z;
    }
}

// k lowest eigenpairs of the symmetric n x n matrix A (destroyed): eigenvalues in w[0..k),
// eigenvectors in the columns of Y (n x k, column-major).  B0, B1, B2 are n x k scratch
// and p n doubles of scratch.  Eigenvalue i (and its vector) belongs to lane i / 4 of warp
// i % 4, which spreads the serial per-eigenvalue work over the four SM sub-partitions;
// the inverse-iteration vectors and LU factors are interleaved (entry j of vector i at
// j k + i) so that a warp's lanes read neighbouring addresses.
template <int MAXN>
__device__ void qb_cta_lowest_eig(int n, int k, double* A, double* Y, double* w, double* B0, double* B1, double* B2,
                                  double* p, QbEigSmem<MAXN>& sm) {
    const int tid = threadIdx.x, nt = blockDim.x;
    qb_cta_tridiag<MAXN>(n, A, p, sm);
    for (int j = tid; j < n; j += nt) {
        sm.df[j] = (float)sm.d[j];
        const float ef = j + 1 < n ? (float)sm.e[j] : 0.0f;
        sm.e2f[j] = ef * ef;
    }
    if (tid == 0) {   // Gershgorin interval and the scale of T
        double lo = 0.0, hi = 0.0;
        for (int i = 0; i < n; ++i) {
            const double r = (i > 0 ? fabs(sm.e[i - 1]) : 0.0) + (i + 1 < n ? fabs(sm.e[i]) : 0.0);
            lo = (i == 0) ? sm.d[i] - r : fmin(lo, sm.d[i] - r);
            hi = (i == 0) ? sm.d[i] + r : fmax(hi, sm.d[i] + r);
        }
        const double nrm = fmax(fabs(lo), fabs(hi)) + 1e-300;
        sm.bounds[0] = lo - 1e-6 * nrm;
        sm.bounds[1] = hi + 1e-6 * nrm;
        sm.bounds[2] = nrm;
    }
    __syncthreads();
    const double nrm = sm.bounds[2];
    const double pert = 1e-16 * nrm;
    // eigenvalue i by a group of G lanes: FP32 multisection on Sturm counts (each round
    // splits the bracket into G + 1 parts), then the group's first lane runs the inverse
    // iteration for eigenvector i
    const int G = min(8, qb_group_lanes(nt, k));
    const int ngrp = nt / G, lane = tid & 31, sub = tid % G;
    const float tiny = (float)(1e-30 * nrm) + 1e-30f;
    const float absres = (float)(1e-13 * nrm);
    double* Yt = B0;   // interleaved vectors; B1, B2 and Y hold the interleaved LU factors
    const int kb = k < n ? k + 1 : k;   // one eigenvalue beyond the occupied ones: the gap above them
    for (int i0 = 0; i0 < kb; i0 += ngrp) {
        const int i = i0 + tid / G;
        float lo = (float)sm.bounds[0], hi = (float)sm.bounds[1];
        bool frozen = i >= kb;
        for (int round = 0; round < 64; ++round) {
            if (__all_sync(0xffffffffu, frozen)) break;
            const float step = (hi - lo) / (float)(G + 1);
            const float x = fminf(lo + step * (float)(sub + 1), hi);
            const bool above = !frozen && qb_sturm_f(n, sm.df, sm.e2f, x, tiny) > i;
            const unsigned gm = (__ballot_sync(0xffffffffu, above) >> (lane & ~(G - 1))) & ((1u << G) - 1u);
            if (!frozen) {
                const int s = gm ? __ffs(gm) - 1 : G;   // first point above eigenvalue i
                const float nlo = s > 0 ? fminf(lo + step * (float)s, hi) : lo;
                const float nhi = s < G ? fminf(lo + step * (float)(s + 1), hi) : hi;
                lo = nlo;
                hi = nhi;
                frozen = !(hi - lo > 2.4e-7f * fmaxf(fabsf(lo), fabsf(hi)) + absres);
            }
        }
        if (i < kb && sub == 0) {
            sm.lam[i] = 0.5 * ((double)lo + (double)hi);
            sm.lamw[i] = 0.5f * (hi - lo) + absres;
        }
    }
    __syncthreads();
    // a gap between the highest occupied eigenvalue and the next one below the FP32
    // resolution: the occupied eigenvalues of that boundary cluster (each within its FP32
    // bracket of the next) are bisected again in FP64, so that inverse iteration separates
    // the occupied vectors from the unoccupied neighbour.  Clusters inside the occupied
    // set need no such care (Gram-Schmidt below orthogonalises them).
    __shared__ int s_lo;
    if (tid == 0) {
        s_lo = k;
        if (kb > k) {
            int j = k - 1;
            auto near = [&](int a) {   // eigenvalues a and a + 1 within their FP32 brackets
                return sm.lam[a + 1] - sm.lam[a] <= 4.0 * ((double)sm.lamw[a] + (double)sm.lamw[a + 1]);
            };
            while (j >= 0 && near(j)) {
                s_lo = j;
                --j;
            }
        }
    }
    __syncthreads();
    for (int i = tid; i < k; i += nt) {
        sm.lamr[i] = sm.lam[i];
        if (i < s_lo) continue;
        const double wi = 4.0 * (double)sm.lamw[i];
        const double tinyd = 1e-300 + 1e-290 * nrm;
        double lo = sm.lam[i] - 2.0 * wi, hi = sm.lam[i] + 2.0 * wi;
        if (!(qb_sturm_d(n, sm.d, sm.e, lo, tinyd) <= i && qb_sturm_d(n, sm.d, sm.e, hi, tinyd) > i)) {
            lo = sm.bounds[0];   // the FP32 bracket missed the eigenvalue: start from Gershgorin
            hi = sm.bounds[1];
        }
        for (int it = 0; it < 120 && hi - lo > 4.0 * 2.220446049250313e-16 * nrm; ++it) {
            const double mid = 0.5 * (lo + hi);
            if (qb_sturm_d(n, sm.d, sm.e, mid, tinyd) > i) hi = mid;
            else lo = mid;
        }
        sm.lamr[i] = 0.5 * (lo + hi);
    }
    __syncthreads();
    for (int i = tid; i < k; i += nt) sm.lam[i] = sm.lamr[i];
    __syncthreads();
    // inverse iteration at the fixed FP32 shift (within ~1e-7 ||T|| of the eigenvalue):
    // components of eigenvalues further than 1e-4 ||T|| shrink by >= 1e3 per step, so four
    // steps leave <= 1e-12 of them; an eigenvalue within 1e-4 ||T|| of a neighbour (a
    // cluster, orthogonalised below) takes six, which also separates pairs whose shifts
    // differ by a few FP32 ulps
    for (int i0 = 0; i0 < k; i0 += ngrp) {
        const int i = i0 + tid / G;
        if (i < k && sub == 0) {
            const double lam = sm.lam[i];
            const bool clustered = (i > 0 && lam - sm.lam[i - 1] <= 1e-4 * nrm) ||
                                   (i + 1 < k && sm.lam[i + 1] - lam <= 1e-4 * nrm);
            double* y = Yt + i;
            for (int j = 0; j < n; ++j) {   // deterministic start vector, distinct per eigenvalue
                const unsigned h = (unsigned)(j * 2654435761u) ^ (unsigned)(i * 40503u + 17u);
                y[(size_t)k * j] = 1.0 + 0.25 * ((double)(h & 0xffff) / 65536.0 - 0.5);
            }
            qb_tridiag_factor(n, sm.d, sm.e, lam, pert, B1 + i, B2 + i, Y + i, k);
            for (int s = 0; s < (clustered ? 6 : 4); ++s) {
                qb_tridiag_apply(n, sm.e, B1 + i, B2 + i, Y + i, y, k);
                double nn2 = 0.0;
                for (int j = 0; j < n; ++j) nn2 = fma(y[(size_t)k * j], y[(size_t)k * j], nn2);
                const double inv = 1.0 / sqrt(nn2);
                for (int j = 0; j < n; ++j) y[(size_t)k * j] *= inv;
            }
        }
    }
    __syncthreads();
    for (int idx = tid; idx < n * k; idx += nt) {   // Y (column-major) <- the interleaved vectors
        const int j = idx % n, i = idx / n;
        Y[idx] = Yt[(size_t)k * j + i];
    }
    __syncthreads();
    // Gram-Schmidt within clusters (|lam_i - lam_j| <= 1e-4 ||T||: the eigenvalues inverse
    // iteration cannot separate), normalisation
    for (int i = 1; i < k; ++i) {
        // vectors without a close predecessor are already normalised and need nothing
        if (sm.lam[i] - sm.lam[i - 1] > 1e-4 * nrm) continue;
        double* yi = Y + (size_t)n * i;
        for (int pass = 0; pass < 2; ++pass)   // twice: vectors of one cluster can be nearly parallel
            for (int j = 0; j < i; ++j) {
                if (fabs(sm.lam[i] - sm.lam[j]) > 1e-4 * nrm) continue;
                const double* yj = Y + (size_t)n * j;
                double dot = 0.0;
                for (int r = tid; r < n; r += nt) dot += yi[r] * yj[r];
                dot = qb_cta_sum(dot, sm.red);
                for (int r = tid; r < n; r += nt) yi[r] -= dot * yj[r];
                __syncthreads();
            }
        double nn2 = 0.0;
        for (int r = tid; r < n; r += nt) nn2 += yi[r] * yi[r];
        nn2 = qb_cta_sum(nn2, sm.red);
        const double inv = 1.0 / sqrt(nn2);
        for (int r = tid; r < n; r += nt) yi[r] *= inv;
        __syncthreads();
    }
    for (int i = tid; i < k; i += nt) {   // eigenvalue = Rayleigh quotient of the final vector
        const double* y = Y + (size_t)n * i;
        double rq = 0.0;
        for (int j = 0; j < n; ++j) {
            double ty = sm.d[j] * y[j];
            if (j > 0) ty += sm.e[j - 1] * y[j - 1];
            if (j + 1 < n) ty += sm.e[j] * y[j + 1];
            rq += y[j] * ty;
        }
        w[i] = rq;
    }
    __syncthreads();
    // back-transformation: Y <- H_0 H_1 ... H_{n-3} Y
    const int LB = qb_group_lanes(nt, k);
    for (int kk = n - 3; kk >= 0; --kk) {
        const int m = n - kk - 1;
        const double* v = A + (kk + 1) + (size_t)n * kk;
        for (int c0 = 0; c0 < k; c0 += nt / LB) {   // LB lanes per column
            const int c = c0 + tid / LB, sb = tid % LB;
            double dot = 0.0;
            if (c < k) {
                const double* yc = Y + (size_t)n * c + kk + 1;
                for (int r = sb; r < m; r += LB) dot = fma(v[r], yc[r], dot);
            }
            dot = qb_group_sum(dot, LB);
            if (c < k && sb == 0) sm.dots[c] = dot;
        }
        __syncthreads();
        for (int idx = tid; idx < m * k; idx += nt) {
            const int r = idx % m, c = idx / m;
            Y[(size_t)n * c + kk + 1 + r] -= 2.0 * v[r] * sm.dots[c];
        }
        __syncthreads();
    }
}
