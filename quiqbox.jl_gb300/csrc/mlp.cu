// Kernels of the learned initial guess: a small MLP (BF16 weights and activations, FP32
// accumulation) that predicts minimal-basis density blocks of atom pairs.  Forward and
// backward passes are built from these primitives by quiqbox.jl_gb300/guess.py:
//   GEMM (tensor cores, mma.sync m16n8k16 BF16 -> FP32), GELU forward/backward, FP32 ->
//   BF16 conversion (optionally transposed), BF16 transpose, column sums (bias
//   gradients), masked mean-squared error with its gradient, Adam on FP32 master weights.
// Every entry point takes device pointers and a cudaStream_t (as void*); sizes that
// break a kernel's tiling are rejected with QB_ERR_DIM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include "qb_internal.h"

namespace {

constexpr int GM = 64, GN = 64, GK = 32, GPAD = 8;

__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C (M x N, fp32, row-major) = A (M x K, bf16, row-major) * B^T (B: N x K, bf16, row-major)
// [+ bias]; 64 x 64 block tile, 4 warps of 32 x 32, K steps of 32 through shared memory.
__global__ void __launch_bounds__(128) qb_bf16_gemm_nt_kernel(int M, int N, int K, const __nv_bfloat16* __restrict__ A,
                                                              const __nv_bfloat16* __restrict__ B,
                                                              const float* __restrict__ bias, float* __restrict__ C) {
    __shared__ __align__(16) __nv_bfloat16 As[GM][GK + GPAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[GN][GK + GPAD];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int m0 = blockIdx.y * GM, n0 = blockIdx.x * GN;
    const int g = lane >> 2, t = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
    for (int k0 = 0; k0 < K; k0 += GK) {
        for (int c = tid; c < GM * GK / 8; c += 128) {
            const int r = c / (GK / 8), col = (c % (GK / 8)) * 8;
            *reinterpret_cast<uint4*>(&As[r][col]) =
                *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * K + k0 + col);
            *reinterpret_cast<uint4*>(&Bs[r][col]) =
                *reinterpret_cast<const uint4*>(B + (size_t)(n0 + r) * K + k0 + col);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int mi = 0; mi < 2; ++mi) {
                const int r = wm + mi * 16;
                af[mi][0] = *reinterpret_cast<const uint32_t*>(&As[r + g][kk + 2 * t]);
                af[mi][1] = *reinterpret_cast<const uint32_t*>(&As[r + g + 8][kk + 2 * t]);
                af[mi][2] = *reinterpret_cast<const uint32_t*>(&As[r + g][kk + 2 * t + 8]);
                af[mi][3] = *reinterpret_cast<const uint32_t*>(&As[r + g + 8][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) {
                const int c = wn + ni * 8;
                bfr[ni][0] = *reinterpret_cast<const uint32_t*>(&Bs[c + g][kk + 2 * t]);
                bfr[ni][1] = *reinterpret_cast<const uint32_t*>(&Bs[c + g][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) mma_bf16_16816(acc[mi][ni], af[mi], bfr[ni]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
            const int row = m0 + wm + mi * 16 + g, col = n0 + wn + ni * 8 + 2 * t;
            const float b0 = bias ? bias[col] : 0.f, b1 = bias ? bias[col + 1] : 0.f;
            C[(size_t)row * N + col] = acc[mi][ni][0] + b0;
            C[(size_t)row * N + col + 1] = acc[mi][ni][1] + b1;
            C[(size_t)(row + 8) * N + col] = acc[mi][ni][2] + b0;
            C[(size_t)(row + 8) * N + col + 1] = acc[mi][ni][3] + b1;
        }
}

// GELU(z) = z Phi(z) = z (1 + erf(z / sqrt 2)) / 2
__global__ void qb_gelu_fwd_kernel(long long n, const float* __restrict__ z, __nv_bfloat16* __restrict__ a) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float x = z[i];
        a[i] = __float2bfloat16_rn(0.5f * x * (1.0f + erff(x * 0.70710678118654752f)));
    }
}

// d GELU / dz = Phi(z) + z phi(z)
__global__ void qb_gelu_bwd_kernel(long long n, const float* __restrict__ z, const float* __restrict__ da,
                                   float* __restrict__ dz) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float x = z[i];
        const float Phi = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
        const float phi = 0.39894228040143268f * expf(-0.5f * x * x);
        dz[i] = da[i] * (Phi + x * phi);
    }
}

// y = bf16(x) (rows x cols), or its transpose (cols x rows)
__global__ void qb_f32_to_bf16_kernel(int rows, int cols, const float* __restrict__ x, __nv_bfloat16* __restrict__ y,
                                      int transpose) {
    const long long n = (long long)rows * cols;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i / cols), c = (int)(i % cols);
        const __nv_bfloat16 v = __float2bfloat16_rn(x[i]);
        if (transpose) y[(size_t)c * rows + r] = v;
        else y[i] = v;
    }
}

__global__ void qb_bf16_transpose_kernel(int rows, int cols, const __nv_bfloat16* __restrict__ x,
                                         __nv_bfloat16* __restrict__ y) {
    const long long n = (long long)rows * cols;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i / cols), c = (int)(i % cols);
        y[(size_t)c * rows + r] = x[i];
    }
}

// out[j] = sum_i x[i][j]; one thread per column, rows summed in order
__global__ void qb_colsum_kernel(int rows, int cols, const float* __restrict__ x, float* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    float s = 0.f;
    for (int i = 0; i < rows; ++i) s += x[(size_t)i * cols + j];
    out[j] = s;
}

// masked MSE: dy = 2 w (y - t) / wsum, loss += sum w (y - t)^2 / wsum
__global__ void qb_mse_kernel(long long n, const float* __restrict__ y, const float* __restrict__ t,
                              const float* __restrict__ w, float inv_wsum, float* __restrict__ dy, float* loss) {
    float acc = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float d = y[i] - t[i];
        const float wd = w[i] * d;
        dy[i] = 2.0f * wd * inv_wsum;
        acc += wd * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc != 0.f) atomicAdd(loss, acc * inv_wsum);
}

// Adam (bias-corrected) on FP32 master weights; refreshes the BF16 copy
__global__ void qb_adam_kernel(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                               float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                               float eps, float c1, float c2) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16_rn(wi);
    }
}

int grid_for(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g < 4096 ? (g > 0 ? g : 1) : 4096);
}

int launched() { return cudaGetLastError() == cudaSuccess ? QB_OK : QB_ERR_CUDA; }

}  // namespace

extern "C" {

int qb_bf16_gemm_nt(int M, int N, int K, const void* A, const void* B, const float* bias, float* C, void* stream) {
    if (M <= 0 || N <= 0 || K <= 0 || M % GM || N % GN || K % GK) return QB_ERR_DIM;
    if (!A || !B || !C) return QB_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return QB_ERR_ARG;
    dim3 grid(N / GN, M / GM);
    qb_bf16_gemm_nt_kernel<<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        M, N, K, static_cast<const __nv_bfloat16*>(A), static_cast<const __nv_bfloat16*>(B), bias, C);
    return launched();
}

int qb_gelu_forward(int64_t n, const float* z, void* a, void* stream) {
    if (n < 0 || (n > 0 && (!z || !a))) return QB_ERR_ARG;
    if (n) qb_gelu_fwd_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        n, z, static_cast<__nv_bfloat16*>(a));
    return launched();
}

int qb_gelu_backward(int64_t n, const float* z, const float* da, float* dz, void* stream) {
    if (n < 0 || (n > 0 && (!z || !da || !dz))) return QB_ERR_ARG;
    if (n) qb_gelu_bwd_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(n, z, da, dz);
    return launched();
}

int qb_f32_to_bf16(int rows, int cols, const float* x, void* y, int transpose, void* stream) {
    if (rows < 0 || cols < 0 || ((long long)rows * cols > 0 && (!x || !y))) return QB_ERR_ARG;
    const long long n = (long long)rows * cols;
    if (n) qb_f32_to_bf16_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        rows, cols, x, static_cast<__nv_bfloat16*>(y), transpose);
    return launched();
}

int qb_bf16_transpose(int rows, int cols, const void* x, void* y, void* stream) {
    if (rows < 0 || cols < 0 || ((long long)rows * cols > 0 && (!x || !y))) return QB_ERR_ARG;
    const long long n = (long long)rows * cols;
    if (n) qb_bf16_transpose_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        rows, cols, static_cast<const __nv_bfloat16*>(x), static_cast<__nv_bfloat16*>(y));
    return launched();
}

int qb_colsum(int rows, int cols, const float* x, float* out, void* stream) {
    if (rows < 0 || cols <= 0 || !out || (rows > 0 && !x)) return QB_ERR_ARG;
    qb_colsum_kernel<<<(cols + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(rows, cols, x, out);
    return launched();
}

int qb_mse_grad(int64_t n, const float* y, const float* t, const float* w, float wsum, float* dy, float* loss,
                void* stream) {
    if (n < 0 || !(wsum > 0.f) || (n > 0 && (!y || !t || !w || !dy || !loss))) return QB_ERR_ARG;
    if (n) qb_mse_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(n, y, t, w, 1.0f / wsum, dy,
                                                                                      loss);
    return launched();
}

int qb_adam_step(int64_t n, float* w, const float* g, float* m, float* v, void* w_bf16, float lr, float b1, float b2,
                 float eps, int step, void* stream) {
    if (n < 0 || step < 1 || (n > 0 && (!w || !g || !m || !v))) return QB_ERR_ARG;
    const float c1 = 1.0f / (1.0f - powf(b1, (float)step)), c2 = 1.0f / (1.0f - powf(b2, (float)step));
    if (n) qb_adam_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        n, w, g, m, v, static_cast<__nv_bfloat16*>(w_bf16), lr, b1, b2, eps, c1, c2);
    return launched();
}

}  // extern "C"
