// Allocation-free direct J/K entry point (qb_jk_noalloc).
//
// Some callers cannot allocate device memory themselves: code running inside a
// host framework that owns every device allocation (a Julia GC-managed pool, a
// serving runtime with a fixed memory budget), or code that must not allocate
// between CUDA-graph captures.  For them this file offers one J/K build that
// calls no cudaMalloc / cudaFree: the caller passes device pointers for the
// basis arrays, the density and the outputs; the kernels' scratch (the J' and
// K' accumulators and a status word) lives in the file-scope device array below,
// and the Boys table in a second one.  Both stay allocated on every GPU that
// loads the library until the process exits.
#include <cmath>
#include <cstring>
#include <mutex>
#include "qb_internal.h"

#define QB_NOALLOC_MAXN 512   // largest basis (nfun) the scratch array holds

// J' (N^2) + K' (N^2) + status (one int, in its own 256-byte slot)
static __device__ __align__(256) double qb_noalloc_scratch[2 * QB_NOALLOC_MAXN * QB_NOALLOC_MAXN + 32];
static __device__ __align__(256) double qb_noalloc_boys[QB_BOYS_TABLE_SIZE];

namespace {

struct NoAllocDevice {
    bool ready = false;
    double* scratch = nullptr;   // device address of qb_noalloc_scratch
    double* boys = nullptr;      // device address of qb_noalloc_boys
    int nsm = 0;
};

constexpr int kMaxDevices = 64;
NoAllocDevice g_dev[kMaxDevices];
std::mutex g_mutex;
double g_boys_host[QB_BOYS_TABLE_SIZE];   // static staging, no heap

// Bad basis data set status bits instead of reaching the integral kernels.  The
// function pointers are checked first (their last entry bounds the primitive arrays);
// the primitives only once the pointers are known to be consistent.
__global__ void qb_noalloc_check_fp_kernel(const int* __restrict__ fp, int nfun, int* status) {
    if (threadIdx.x == 0 && fp[0] != 0) atomicOr(status, 1);
    for (int f = threadIdx.x; f < nfun; f += blockDim.x)
        if (fp[f + 1] <= fp[f]) atomicOr(status, 1);
}

__global__ void qb_noalloc_check_prims_kernel(const int* __restrict__ fp, int nfun, const int* __restrict__ ijk,
                                              const double* __restrict__ alpha, int* status) {
    const int np = fp[nfun];
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
        const int l = ijk[3 * p] + ijk[3 * p + 1] + ijk[3 * p + 2];
        if (ijk[3 * p] < 0 || ijk[3 * p + 1] < 0 || ijk[3 * p + 2] < 0 || l > 12) atomicOr(status, 2);
        if (!(alpha[p] > 0.0)) atomicOr(status, 4);
    }
}

int read_status(const int* status, cudaStream_t s, int* st) {
    if (cudaMemcpyAsync(st, status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return QB_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return QB_ERR_CUDA;
    return QB_OK;
}

int setup_device(int dev) {
    std::lock_guard<std::mutex> lock(g_mutex);
    NoAllocDevice& d = g_dev[dev];
    if (d.ready) return QB_OK;
    static bool table_built = false;
    if (!table_built) {
        qb_fill_boys_table(g_boys_host);
        table_built = true;
    }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, qb_noalloc_scratch) != cudaSuccess) return QB_ERR_CUDA;
    d.scratch = static_cast<double*>(p);
    if (cudaGetSymbolAddress(&p, qb_noalloc_boys) != cudaSuccess) return QB_ERR_CUDA;
    d.boys = static_cast<double*>(p);
    if (cudaMemcpyToSymbol(qb_noalloc_boys, g_boys_host, sizeof(g_boys_host)) != cudaSuccess) return QB_ERR_CUDA;
    if (cudaDeviceGetAttribute(&d.nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return QB_ERR_CUDA;
    d.ready = true;
    return QB_OK;
}

}  // namespace

extern "C" int qb_jk_noalloc(const qb_basis* dbasis, const double* dD, double* dJ, double* dK, void* stream) {
    if (!dbasis) return QB_ERR_ARG;
    const int n = dbasis->nfun;
    if (n < 1 || n > QB_NOALLOC_MAXN) return QB_ERR_DIM;
    if (!dbasis->fun_ptr || !dbasis->center || !dbasis->ijk || !dbasis->alpha || !dbasis->weight || !dD || !dJ ||
        !dK)
        return QB_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return QB_ERR_CUDA;
    const int rc = setup_device(dev);
    if (rc != QB_OK) return rc;
    const NoAllocDevice& d = g_dev[dev];
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t nn = (size_t)n * n;
    double* Jp = d.scratch;
    double* Kp = d.scratch + nn;
    int* status = reinterpret_cast<int*>(d.scratch + 2 * (size_t)QB_NOALLOC_MAXN * QB_NOALLOC_MAXN);
    // the array keeps the previous call's contents: clear what accumulates
    if (cudaMemsetAsync(d.scratch, 0, 2 * nn * sizeof(double), s) != cudaSuccess) return QB_ERR_CUDA;
    if (cudaMemsetAsync(status, 0, sizeof(int), s) != cudaSuccess) return QB_ERR_CUDA;
    int st = 0;
    qb_noalloc_check_fp_kernel<<<1, 256, 0, s>>>(dbasis->fun_ptr, n, status);
    if (read_status(status, s, &st) != QB_OK) return QB_ERR_CUDA;
    if (st & 1) return QB_ERR_ARG;
    qb_noalloc_check_prims_kernel<<<1, 256, 0, s>>>(dbasis->fun_ptr, n, dbasis->ijk, dbasis->alpha, status);
    if (read_status(status, s, &st) != QB_OK) return QB_ERR_CUDA;
    if (st & 2) return QB_ERR_UNSUPPORTED;
    if (st & 4) return QB_ERR_DOMAIN;
    const GenDevBasis gb{dbasis->fun_ptr, dbasis->center, dbasis->ijk, dbasis->alpha, dbasis->weight, n};
    if (qb_gen_eri(gb, 1, d.boys, nullptr, dD, Jp, Kp, status, d.nsm, s) != 0) return QB_ERR_CUDA;
    qb_jk_finalize(s, n, nullptr, Jp, Kp, dJ, dK);
    if (cudaGetLastError() != cudaSuccess) return QB_ERR_CUDA;
    if (read_status(status, s, &st) != QB_OK) return QB_ERR_CUDA;
    return st ? QB_ERR_UNSUPPORTED : QB_OK;
}
