// Dense linear algebra run by one thread block (CTA): the small matrices of the SCF
// (N <= a few hundred) live in global memory / L2 and every thread of the block takes
// part.  Column-major storage throughout.
#pragma once
#include <cuda_runtime.h>

// Block-wide sum of one double per thread; every thread gets the result.  red must hold
// 33 doubles of shared memory.
__device__ __forceinline__ double qb_cta_sum(double v, double* red) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int k = 0; k < (nt + 31) / 32; ++k) t += red[k];
        red[32] = t;
    }
    __syncthreads();
    return red[32];
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
// precision); converged when off(A)^2 <= 1e-30 ||A||^2, when a sweep rotated no plane, or
// when off(A)^2 <= 1e-24 ||A||^2 stopped shrinking (rounding level: it fell by less than
// 4x in the last sweep).  At most maxsweep sweeps; returns the number used, or -1 if not
// converged (off(A) is then still reported small enough by the caller's own test).
template <int MAXN>
__device__ int qb_cta_jacobi(int n, double* A, double* V, const double* Vin, double* w, double* wtmp, double* Vtmp,
                             int maxsweep, QbJacobiSmem<MAXN>& sm) {
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
        if (off <= 1e-30 * tot || off == 0.0 || (sweep > 0 && rotated == 0) ||
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
