// Host-side internals of the GB300 integral / Hartree–Fock library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "qb_common.cuh"
#include "eri_kernels.cuh"
#include "quiqbox_gb300.h"

#define QB_NSTREAM 4
#define QB_MAX_CLASS 32
#define QB_MAX_PC 8

struct GenDevBasis {
    const int* fp;
    const double* cen;
    const int* ijk;
    const double* alpha;
    const double* w;
    int nfun;
};

// generic.cu
int qb_gen_onebody_batch(const GenDevBasis& gb, int nmol, long long npair_total, const long long* poff,
                         const int* fo, const int* nf, const long long* mo, const int* nuc0, const double* dZ,
                         const double* dR, const double* boys, double* S, double* H, int* status, cudaStream_t s);
int qb_gen_adjoint_eri(const GenDevBasis& gb, int n, int ng, const double* P, const double* boys, double* Jx,
                       double* Kx, int* status, int nsm, cudaStream_t s);
int qb_gen_multipole(const GenDevBasis& gb, const double* C, const int* deg, double* M, int* status, cudaStream_t s);
int qb_gen_onebody(const GenDevBasis& gb, int flags, int nnuc, const double* dZ, const double* dR,
                   const double* boys, double* S, double* T, double* V, int* status, cudaStream_t s);
int qb_gen_eri(const GenDevBasis& gb, int mode, const double* boys, double* eri, const double* D, double* Jp,
               double* Kp, int* status, int nsm, cudaStream_t s);
int qb_boys_device(int n, const double* dT, int M, int path, const double* boys, double* dout, cudaStream_t s);
int qb_gen_eri_list(const GenDevBasis& gb, const double* boys, long long nq, const int* dq, double* out,
                    int* status, cudaStream_t s);

// generated eri_dispatch.cu
extern const int QB_NCLASS;
extern const int QB_LMAX_SHELL;
extern const double QB_CLASS_PRIM_FLOPS[];
extern const double QB_CLASS_CONTR_FLOPS[];
extern const int QB_CLASS_NINT[];
void qb_get_class_launchers(ClassLaunchers* out);
void qb_fill_boys_table(double* tab);   // QB_BOYS_TABLE_SIZE doubles, no allocation

// Growable device array.
template <class T>
struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        const size_t c = count ? count : 1;
        cudaError_t e = cudaMalloc(&p, c * sizeof(T));
        if (e == cudaSuccess) n = c;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct HostShell {
    double c[3];
    int L, K;
    int prim0;   // into the shell-primitive arrays (alpha, coef)
    int f0;      // first function
};

// Primitive-pair slot: shells and shell-primitive indices (into the flattened basis).
struct PairSlot {
    int sa, sb, pa, pb;
};
int qb_build_prim_pairs(cudaStream_t s, const PairSlot* d_slots, int nslot, const double* d_cen,
                        const double* d_alpha, const double* d_w, const ShellPair* d_pairs, int npair,
                        PrimPair* d_prims, float4* d_prims32, int* d_nkept, unsigned long long* d_kmax);
int qb_compact_prim_keys(cudaStream_t s, const ShellPair* d_pairs, int npair, PrimPair* d_prims, float4* d_prims32,
                         int nslot, const unsigned* d_keymax, float eps, int* d_nkept);

int qb_jk_autotune_device(qb_ctx* ctx, int repeats, int* chosen);
int qb_jk_class_times_device(qb_ctx* ctx, int repeats, float* ms);
int qb_jk_quartets_device(qb_ctx* ctx, long long nq, const int* pq, double* dJ, double* dK);
int qb_lowest_eig(cudaStream_t s, int n, int k, double* A, double* Y, double* w, double* work);
int qb_batch_rhf_run(qb_ctx* ctx, int nmol, const qb_basis* bases, const int* nnuc, const double* Z,
                     const double* R, const int* nocc, const qb_batch_config* cfg, qb_batch_result* res);

bool qb_detect_shells(int f_begin, int f_end, const int* fp, const double* cen, const int* ijk, const double* al,
                      const double* w, std::vector<HostShell>& shells, double* ratio);

struct qb_ctx {
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t streams[QB_NSTREAM] = {};
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr, ev_fork = nullptr;
    cudaEvent_t ev_join[QB_NSTREAM] = {};
    std::string err;

    DevArray<double> boys;
    DevArray<int> status;

    // flattened basis (host copy for change detection + device copy)
    bool basis_valid = false;
    int nfun = 0, nprim = 0;
    std::vector<int> h_fp, h_ijk;
    std::vector<double> h_cen, h_alpha, h_w;
    DevArray<int> d_fp, d_ijk;
    DevArray<double> d_cen, d_alpha, d_w;

    // shell structure
    bool shell_path = false;
    std::vector<HostShell> shells;
    std::vector<double> h_ratio;
    DevArray<double> d_ratio;
    bool pairs_valid = false;
    int npc = 0;
    int pc_off[QB_MAX_PC + 1] = {};
    std::vector<ShellPair> h_pairs;      // sorted by pair class then descending Q
    DevArray<ShellPair> d_pairs;
    DevArray<PrimPair> d_prims;
    DevArray<float4> d_prims32;   // (p, Px, Py, Pz) of d_prims in FP32 (Boys-branch grouping)
    DevArray<double> d_Q;                 // per pair, sorted like d_pairs
    DevArray<long long> d_npref;          // per pair class: exclusive prefix of nprim (segment of size n+1)
    int npref_off[QB_MAX_PC + 1] = {};

    // classes
    ClassLaunchers launch[QB_MAX_CLASS];
    int nclass = 0;
    int occ[QB_MAX_CLASS] = {};
    int variant[QB_MAX_CLASS] = {};   // launcher variant per class (0 per-thread, 1 warp-cooperative)
    float class_ms[QB_MAX_CLASS] = {};   // device time of each class kernel alone (autotuner / class timing; 0: unknown)
    float prim_eps = (float)QB_PRIM_EPS_Q;   // primitive-quartet threshold of the J/K class kernels
    int class_bra[QB_MAX_CLASS] = {}, class_ket[QB_MAX_CLASS] = {};
    long long offs_off[QB_MAX_CLASS + 1] = {};
    DevArray<long long> d_offs;
    DevArray<long long> d_one_offs;       // {0, 1}: the work list of one quartet
    DevArray<long long> d_stats;          // 2 per class: quartets, primitive quartets (upper bound)
    DevArray<unsigned long long> d_primcount;   // per class: primitive quartets evaluated

    // J/K buffers
    double schwarz = 1e-12;
    bool jk_prepared = false;
    DevArray<double> d_D, d_Dt, d_Jp, d_Kp, d_J, d_K, d_dmax;
    float ms_last = 0.f;
    int last_execute_shell = 0;

    // scratch for the integral APIs
    DevArray<double> d_m0, d_m1, d_m2, d_nucZ, d_nucR, d_big;
    DevArray<int> d_quart;
};

// engine.cu
int qb_set_error(qb_ctx* ctx, int code, const std::string& msg);
int qb_cuda_check(qb_ctx* ctx, cudaError_t e, const char* where);
int qb_set_basis(qb_ctx* ctx, const qb_basis* basis);
int qb_ensure_pairs(qb_ctx* ctx);
int qb_jk_device(qb_ctx* ctx, const double* dD, double* dJ, double* dK, double schwarz, cudaStream_t s);
int qb_onebody_device(qb_ctx* ctx, int flags, int nnuc, const double* Z, const double* R, double* dS,
                      double* dT, double* dV);
int qb_check_status(qb_ctx* ctx);
GenDevBasis qb_gen_basis(qb_ctx* ctx);

// linalg.cu (device matrices are column-major n x n unless stated)
void qb_gemm(cudaStream_t s, int transA, int transB, int m, int n, int k, double alpha, const double* A,
             int lda, const double* B, int ldb, double beta, double* C, int ldc);
int qb_eigh(cudaStream_t s, int n, const double* A, double* w, double* V, double* work, int* status);
void qb_axpby(cudaStream_t s, long long n, double a, const double* x, double b, const double* y, double* z);
void qb_fill(cudaStream_t s, long long n, double v, double* x);
void qb_dot(cudaStream_t s, long long n, const double* x, const double* y, double* out);
void qb_symmetrize_upper(cudaStream_t s, int n, double* A);
void qb_scale_columns_sign(cudaStream_t s, int n, double* C);
void qb_diag_func(cudaStream_t s, int n, const double* U, const double* w, int kind, double* out, double* work);
void qb_jk_finalize(cudaStream_t s, int n, const double* ratio, const double* Jp, const double* Kp, double* J,
                    double* K);
void qb_density_prescale(cudaStream_t s, int n, const double* ratio, const double* D, double* Dt, double* dmax);
void qb_gwh(cudaStream_t s, int n, const double* S, const double* H, double* out);
int qb_diis_solve(cudaStream_t s, int m, int convex, int solver, const double* B, const double* v, double* c,
                  int* iters, int* status);
void qb_lincomb(cudaStream_t s, long long len, int m, const double* const* mats, const double* c, double* out);
