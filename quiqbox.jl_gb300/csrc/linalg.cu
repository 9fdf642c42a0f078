// Dense FP64 kernels of the SCF driver: GEMM, Jacobi eigensolver, reductions,
// the J/K finalisation and the DIIS coefficient solve.
#include <cuda_runtime.h>
#include "qb_internal.h"
#include "qb_dense.cuh"
#include "qb_diis_solvers.cuh"

// ---------------------------------------------------------------------------
// C = alpha op(A) op(B) + beta C, column-major, 32x32 tiles in shared memory,
// each thread computing a 2x2 block.
#define GT 32
__global__ void qb_gemm_kernel(int tA, int tB, int m, int n, int k, double alpha, const double* __restrict__ A,
                               int lda, const double* __restrict__ B, int ldb, double beta, double* C, int ldc) {
    __shared__ double As[GT][GT + 1];
    __shared__ double Bs[GT][GT + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;   // 16 x 16
    const int row0 = blockIdx.x * GT, col0 = blockIdx.y * GT;
    double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    for (int kk = 0; kk < k; kk += GT) {
        for (int r = ty; r < GT; r += 16)
            for (int c = tx; c < GT; c += 16) {
                // As[r][c] = op(A)(row0 + r, kk + c); Bs[r][c] = op(B)(kk + r, col0 + c)
                const int ar = row0 + r, ac = kk + c;
                double av = 0.0;
                if (ar < m && ac < k) av = tA ? A[ac + (size_t)lda * ar] : A[ar + (size_t)lda * ac];
                As[r][c] = av;
                const int br = kk + r, bc = col0 + c;
                double bv = 0.0;
                if (br < k && bc < n) bv = tB ? B[bc + (size_t)ldb * br] : B[br + (size_t)ldb * bc];
                Bs[r][c] = bv;
            }
        __syncthreads();
#pragma unroll 8
        for (int q = 0; q < GT; ++q) {
            const double a0 = As[tx][q], a1 = As[tx + 16][q];
            const double b0 = Bs[q][ty], b1 = Bs[q][ty + 16];
            acc[0][0] = fma(a0, b0, acc[0][0]);
            acc[0][1] = fma(a0, b1, acc[0][1]);
            acc[1][0] = fma(a1, b0, acc[1][0]);
            acc[1][1] = fma(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            const int r = row0 + tx + 16 * i, c = col0 + ty + 16 * j;
            if (r < m && c < n) {
                double* dst = C + r + (size_t)ldc * c;
                *dst = alpha * acc[i][j] + (beta == 0.0 ? 0.0 : beta * *dst);
            }
        }
}

void qb_gemm(cudaStream_t s, int transA, int transB, int m, int n, int k, double alpha, const double* A, int lda,
             const double* B, int ldb, double beta, double* C, int ldc) {
    dim3 block(16, 16), grid((m + GT - 1) / GT, (n + GT - 1) / GT);
    qb_gemm_kernel<<<grid, block, 0, s>>>(transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

// ---------------------------------------------------------------------------
// Cyclic two-sided Jacobi eigensolver (one thread block, matrix in global
// memory / L2), parallel round-robin ordering: each round rotates n/2 disjoint
// (p, q) planes.  At most 60 sweeps; status bit 2 is set if it did not reach
// off(A)^2 <= 1e-30 ||A||^2.  Eigenvalues ascending, eigenvectors in columns.
#define QB_EIGH_MAXN 1024
__global__ void __launch_bounds__(1024) qb_jacobi_kernel(int n, double* A, double* V, double* w, double* wtmp,
                                                         double* Vtmp, int* status) {
    __shared__ QbJacobiSmem<QB_EIGH_MAXN> sm;
    const int used = qb_cta_jacobi<QB_EIGH_MAXN>(n, A, V, nullptr, w, wtmp, Vtmp, 59, sm);
    if (used < 0 && threadIdx.x == 0) atomicOr(status, 2);
}

// k lowest eigenpairs of a symmetric matrix (the batched SCF's solver) for testing and for
// callers that need only part of the spectrum; one thread block, n <= 1024.
__global__ void __launch_bounds__(256) qb_lowest_eig_kernel(int n, int k, double* A, double* Y, double* w,
                                                            double* B, double* p) {
    __shared__ QbEigSmem<QB_EIGH_MAXN> sm;
    qb_cta_lowest_eig<QB_EIGH_MAXN>(n, k, A, Y, w, B, B + (size_t)n * k, B + 2 * (size_t)n * k, p, sm);
}

int qb_lowest_eig(cudaStream_t s, int n, int k, double* A, double* Y, double* w, double* work) {
    if (n < 1 || n > QB_EIGH_MAXN || k < 1 || k > n) return -1;
    qb_lowest_eig_kernel<<<1, 256, 0, s>>>(n, k, A, Y, w, work, work + 3 * (size_t)n * k);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// w (n), V (n x n) from symmetric A; work needs 2 n^2 + n doubles.
int qb_eigh(cudaStream_t s, int n, const double* A, double* w, double* V, double* work, int* status) {
    if (n > QB_EIGH_MAXN) return -1;
    double* Aw = work;
    double* Vt = work + (size_t)n * n;
    double* wt = work + 2 * (size_t)n * n;
    cudaMemcpyAsync(Aw, A, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    const int threads = n <= 32 ? 64 : (n <= 128 ? 256 : 1024);
    qb_jacobi_kernel<<<1, threads, 0, s>>>(n, Aw, V, w, wt, Vt, status);
    return 0;
}

// ---------------------------------------------------------------------------
__global__ void qb_axpby_kernel(long long n, double a, const double* x, double b, const double* y, double* z) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = a * x[i] + (y ? b * y[i] : 0.0);
}
void qb_axpby(cudaStream_t s, long long n, double a, const double* x, double b, const double* y, double* z) {
    if (n > 0) qb_axpby_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, a, x, b, y, z);
}

__global__ void qb_fill_kernel(long long n, double v, double* x) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = v;
}
void qb_fill(cudaStream_t s, long long n, double v, double* x) {
    if (n > 0) qb_fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, v, x);
}

// Deterministic single-block dot product.
__global__ void __launch_bounds__(1024) qb_dot_kernel(long long n, const double* x, const double* y, double* out) {
    __shared__ double red[32];
    double acc = 0.0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) acc = fma(x[i], y[i], acc);
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
        *out = t;
    }
}
void qb_dot(cudaStream_t s, long long n, const double* x, const double* y, double* out) {
    qb_dot_kernel<<<1, 1024, 0, s>>>(n, x, y, out);
}

// A[i,j] = A[j,i] for i > j: the upper triangle wins (Hermitian(A) in the reference).
__global__ void qb_symmetrize_upper_kernel(int n, double* A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i < n && i > j) A[i + (size_t)n * j] = A[j + (size_t)n * i];
}
void qb_symmetrize_upper(cudaStream_t s, int n, double* A) {
    dim3 grid((n + 127) / 128, n);
    qb_symmetrize_upper_kernel<<<grid, 128, 0, s>>>(n, A);
}

// Flip the sign of every column whose first entry is negative (HartreeFock.jl:51-53).
__global__ void qb_sign_kernel(int n, double* C) {
    const int j = blockIdx.x;
    const bool flip = C[(size_t)n * j] < 0.0;
    if (!flip) return;
    for (int i = threadIdx.x; i < n; i += blockDim.x) C[i + (size_t)n * j] = -C[i + (size_t)n * j];
}
void qb_scale_columns_sign(cudaStream_t s, int n, double* C) { qb_sign_kernel<<<n, 128, 0, s>>>(n, C); }

// out = U diag(f(w)) U^T, f = w^-1/2 (kind 0), w^1/2 (kind 1), 1/w (kind 2); work n x n.
__global__ void qb_scale_cols_kernel(int n, const double* U, const double* w, int kind, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= n) return;
    const double x = w[j];
    const double f = kind == 0 ? 1.0 / sqrt(x) : (kind == 1 ? sqrt(x) : 1.0 / x);
    out[i + (size_t)n * j] = U[i + (size_t)n * j] * f;
}
void qb_diag_func(cudaStream_t s, int n, const double* U, const double* w, int kind, double* out, double* work) {
    dim3 grid((n + 127) / 128, n);
    qb_scale_cols_kernel<<<grid, 128, 0, s>>>(n, U, w, kind, work);
    qb_gemm(s, 0, 1, n, n, n, 1.0, work, n, U, n, 0.0, out, n);
}

// J = r r^T o (Jp + Jp^T)/4,  K = r r^T o (Kp + Kp^T)/8  (r = per-function ratios, or 1)
__global__ void qb_jk_finalize_kernel(int n, const double* __restrict__ r, const double* __restrict__ Jp,
                                      const double* __restrict__ Kp, double* J, double* K) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= n) return;
    const size_t a = i + (size_t)n * j, b = j + (size_t)n * i;
    const double s = r ? r[i] * r[j] : 1.0;
    if (J) J[a] = s * 0.25 * (Jp[a] + Jp[b]);
    if (K) K[a] = s * 0.125 * (Kp[a] + Kp[b]);
}
void qb_jk_finalize(cudaStream_t s, int n, const double* ratio, const double* Jp, const double* Kp, double* J,
                    double* K) {
    dim3 grid((n + 127) / 128, n);
    qb_jk_finalize_kernel<<<grid, 128, 0, s>>>(n, ratio, Jp, Kp, J, K);
}

// Dt = r r^T o D and dmax = max |D_ij| (non-negative doubles order like their bit patterns).
__global__ void qb_prescale_kernel(int n, const double* __restrict__ r, const double* __restrict__ D, double* Dt,
                                   unsigned long long* dmax) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    double a = 0.0;
    if (i < n) {
        const size_t k = i + (size_t)n * j;
        const double v = D[k];
        Dt[k] = r ? r[i] * r[j] * v : v;
        a = fabs(v);
    }
    for (int d = 16; d > 0; d >>= 1) a = fmax(a, __shfl_down_sync(0xffffffffu, a, d));
    if ((threadIdx.x & 31) == 0) atomicMax(dmax, (unsigned long long)__double_as_longlong(a));
}
void qb_density_prescale(cudaStream_t s, int n, const double* ratio, const double* D, double* Dt, double* dmax) {
    dim3 grid((n + 127) / 128, n);
    qb_prescale_kernel<<<grid, 128, 0, s>>>(n, ratio, D, Dt, reinterpret_cast<unsigned long long*>(dmax));
}

// Generalised Wolfsberg–Helmholz one-body matrix: 3 S_ij (H_ii + H_jj) / 8 (HartreeFock.jl:235-254)
__global__ void qb_gwh_kernel(int n, const double* S, const double* H, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= n) return;
    out[i + (size_t)n * j] = 3.0 * S[i + (size_t)n * j] * (H[i + (size_t)n * i] + H[j + (size_t)n * j]) / 8.0;
}
void qb_gwh(cudaStream_t s, int n, const double* S, const double* H, double* out) {
    dim3 grid((n + 127) / 128, n);
    qb_gwh_kernel<<<grid, 128, 0, s>>>(n, S, H, out);
}

// out = sum_i c[i] * mats[i]  (mats: device array of m device pointers)
__global__ void qb_lincomb_kernel(long long len, int m, const double* const* mats, const double* c, double* out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    double acc = 0.0;
    for (int i = 0; i < m; ++i) acc = fma(c[i], mats[i][k], acc);
    out[k] = acc;
}
void qb_lincomb(cudaStream_t s, long long len, int m, const double* const* mats, const double* c, double* out) {
    if (len > 0) qb_lincomb_kernel<<<(unsigned)((len + 255) / 256), 256, 0, s>>>(len, m, mats, c, out);
}

// ---------------------------------------------------------------------------
// DIIS coefficient problem: the Lagrange-multiplier solver (qb_cm_solve, CMsolver!,
// HartreeFock.jl:1445-1477) or the iterative ones (qb_diis_iterative_solve), one warp,
// its state in shared memory.
#define QB_DIIS_MAX 16
__global__ void qb_diis_cm_kernel(int m, int convex, const double* B, const double* v, double* c, int* status) {
    __shared__ QbDiisWork sw;
    if (threadIdx.x < 32 && blockIdx.x == 0) {
        const bool ok = qb_cm_solve(sw, m, convex, B, m, v, c);
        if (!ok && threadIdx.x == 0) atomicOr(status, 4);
    }
}

// L-BFGS-B / SPG solve by one warp (qb_diis_solvers.cuh); c holds the starting point.
__global__ void qb_diis_iter_kernel(int solver, int convex, int m, const double* B, const double* v, double* c,
                                    int* iters) {
    __shared__ QbDiisWork sw;
    if (threadIdx.x < 32 && blockIdx.x == 0) {
        const int it = qb_diis_iterative_solve(sw, solver, convex, m, B, m, v, c);
        if (iters && threadIdx.x == 0) *iters = it;
    }
}

int qb_diis_solve(cudaStream_t s, int m, int convex, int solver, const double* B, const double* v, double* c,
                  int* iters, int* status) {
    if (m < 1 || m > QB_DIIS_MAX || m > QB_DS_N) return -1;
    if (solver == QB_DIIS_LCM) qb_diis_cm_kernel<<<1, 32, 0, s>>>(m, convex, B, v, c, status);
    else qb_diis_iter_kernel<<<1, 32, 0, s>>>(solver, convex, m, B, v, c, iters);
    return 0;
}
