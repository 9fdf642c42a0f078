// Hartree–Fock SCF driver on the GPU.
//
// Follows runHartreeFock / runHartreeFockCore (src/HartreeFock.jl:953-1228):
// symmetric orthogonalisation X = S^-1/2 (:39-42), Fock diagonalisation with
// the sign convention of solveFockMatrix (:46-56), getD / getE (:296-342),
// getCDFE (:392-403), the DD core (:1245-1270) and the DIIS / EDIIS / ADIIS
// cores (:1273-1394) with subspace reset and eviction and the per-method DIIS
// coefficient solver (L-BFGS-B by default, SPG or Lagrange multipliers, solved on the
// device, the coefficient vector carried between steps as the reference's `cs`), the CoreH / GWH / SAD /
// Direct guesses (:195-293) with breakCoeffSymmetry (:71-140), and the
// convergence, oscillation and early-stop rules (:1142-1203).  Every matrix
// operation runs as a CUDA kernel of this library; the two-electron part is the
// direct J/K build (no stored ERI tensor): G = 2J(D) - K(D) for RHF,
// G^s = J(Da+Db) - K(D^s) for UHF.  The host only sequences kernels and reads
// back the scalars that steer the iteration (energies and residual norms).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <numeric>
#include <string>
#include <vector>
#include "qb_internal.h"
#include "qb_diis_solvers.cuh"

#define QB_TRY(expr)                  \
    do {                              \
        const int _rc = (expr);       \
        if (_rc != QB_OK) return _rc; \
    } while (0)
#define QB_CUDA(ctx, call) QB_TRY(qb_cuda_check((ctx), (call), #call))

namespace {

constexpr double kAtolVal = 4e-16;   // getAtolVal(Float64) (src/Arithmetic.jl:42)

// Pool of n x n device matrices.
struct MatPool {
    size_t nn = 0;
    std::vector<double*> all, free_;
    ~MatPool() {
        for (double* p : all) cudaFree(p);
    }
    double* get() {
        if (!free_.empty()) {
            double* p = free_.back();
            free_.pop_back();
            return p;
        }
        double* p = nullptr;
        if (cudaMalloc(&p, nn * sizeof(double)) != cudaSuccess) return nullptr;
        all.push_back(p);
        return p;
    }
    void put(double* p) {
        if (p) free_.push_back(p);
    }
};

__global__ void residual_kernel(int n, const double* M, double* e) {   // e = M - M^T
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i < n) e[i + (size_t)n * j] = M[i + (size_t)n * j] - M[j + (size_t)n * i];
}

// Gram matrix G_ij = <P_i, Q_j> for pointer arrays (one block per entry).
__global__ void gram_kernel(int m, long long len, const double* const* P, const double* const* Q, double* G) {
    const int i = blockIdx.x, j = blockIdx.y;
    __shared__ double red[32];
    double acc = 0.0;
    for (long long k = threadIdx.x; k < len; k += blockDim.x) acc = fma(P[i][k], Q[j][k], acc);
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
        G[i + m * j] = t;
    }
}

// B and v of the DIIS variants from the Gram matrix G (G_ij = <R_i,R_j> for DIIS,
// <D_i,F_j> for EDIIS / ADIIS) and the energies E (HartreeFock.jl:1273-1315).
__global__ void diis_system_kernel(int m, int method, const double* G, const double* E, double* B, double* v) {
    const int i = threadIdx.x, j = threadIdx.y;
    if (i >= m || j >= m) return;
    const int L = m - 1;
    double b;
    if (method == QB_SCF_DIIS) {
        b = G[i + m * j];
    } else if (method == QB_SCF_EDIIS) {
        b = -(G[i + m * i] - G[i + m * j] - G[j + m * i] + G[j + m * j]);
    } else {
        b = G[i + m * j] - G[i + m * L] - G[L + m * j] + G[L + m * L];
    }
    B[i + m * j] = b;
    if (j == 0) {
        if (method == QB_SCF_DIIS) v[i] = 0.0;
        else if (method == QB_SCF_EDIIS) v[i] = E[i];
        else v[i] = G[i + m * L] - G[L + m * L];
    }
}

// breakCoeffSymmetryCore column step (HartreeFock.jl:84-97): per column j of o1
// (even j) or o2 (odd j), the largest-magnitude entry (first on ties) is negated
// into -v^2 when |v| is 1 within sqrt(eps), else zeroed and the column renormalised.
__global__ void break_sym_kernel(int n, double* o1, double* o2) {
    const int j = blockIdx.x;
    double* col = ((j & 1) == 0 ? o1 : o2) + (size_t)n * j;
    if (threadIdx.x != 0) return;
    int idx = 0;
    double mag = fabs(col[0]);
    for (int i = 1; i < n; ++i)
        if (fabs(col[i]) > mag) { mag = fabs(col[i]); idx = i; }
    const double val = col[idx];
    if (fabs(mag - 1.0) < 1.4901161193847656e-08) {
        col[idx] *= -val;
    } else {
        col[idx] = 0.0;
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += col[i] * col[i];
        s = sqrt(s);
        for (int i = 0; i < n; ++i) col[i] /= s;
    }
}

struct Entry {        // one SCF step of one spin sector
    double *C = nullptr, *D = nullptr, *F = nullptr;
    double E = 0.0;
};

struct DiisItem {
    double *D = nullptr, *F = nullptr, *R = nullptr;
    double E = 0.0;
};

struct Scf {
    qb_ctx* ctx;
    cudaStream_t s;
    int n;
    size_t nn;
    int nspin;
    int N[2];
    double schwarz;
    MatPool pool;
    double *S = nullptr, *H = nullptr, *X = nullptr;
    double *t1 = nullptr, *t2 = nullptr, *t3 = nullptr, *eigw = nullptr, *eigwork = nullptr, *J = nullptr,
           *K = nullptr, *scal = nullptr, *gram = nullptr, *B = nullptr, *v = nullptr, *c = nullptr,
           *E_d = nullptr;
    const double** ptrs_d = nullptr;
    const double** ptrs2_d = nullptr;
    std::vector<std::unique_ptr<double, void (*)(void*)>> owned;

    double* alloc(size_t count) {
        double* p = nullptr;
        if (cudaMalloc(&p, count * sizeof(double)) != cudaSuccess) return nullptr;
        owned.emplace_back(p, [](void* q) { cudaFree(q); });
        return p;
    }

    int init(qb_ctx* c_, int n_) {
        ctx = c_;
        s = ctx->stream;
        n = n_;
        nn = (size_t)n * n;
        pool.nn = nn;
        S = alloc(nn); H = alloc(nn); X = alloc(nn); t1 = alloc(nn); t2 = alloc(nn); t3 = alloc(nn);
        J = alloc(nn); K = alloc(nn); eigw = alloc(n); eigwork = alloc(2 * nn + n);
        scal = alloc(16); gram = alloc(QB_MAX_CLASS * QB_MAX_CLASS); B = alloc(256); v = alloc(16); c = alloc(16);
        E_d = alloc(16);
        void* p1 = nullptr;
        void* p2 = nullptr;
        if (cudaMalloc(&p1, 64 * sizeof(double*)) != cudaSuccess || cudaMalloc(&p2, 64 * sizeof(double*)) != cudaSuccess)
            return qb_set_error(ctx, QB_ERR_NOMEM, "SCF pointer tables");
        owned.emplace_back((double*)p1, [](void* q) { cudaFree(q); });
        owned.emplace_back((double*)p2, [](void* q) { cudaFree(q); });
        ptrs_d = (const double**)p1;
        ptrs2_d = (const double**)p2;
        if (!S || !H || !X || !t1 || !t2 || !t3 || !J || !K || !eigw || !eigwork || !scal || !gram || !B || !v ||
            !c || !E_d)
            return qb_set_error(ctx, QB_ERR_NOMEM, "SCF device buffers");
        return QB_OK;
    }

    double* mat() { return pool.get(); }
    void drop(double* p) { pool.put(p); }

    int eig_status() { return qb_check_status(ctx); }

    // host read of device scalars
    int read(const double* d, double* h, int cnt) {
        QB_CUDA(ctx, cudaMemcpyAsync(h, d, cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
        QB_CUDA(ctx, cudaStreamSynchronize(s));
        return QB_OK;
    }

    // C = X eigvecs(X^T F X) with sign stabilisation; optional eigenvalues into w_out
    int solve_fock(const double* Xm, const double* F, double* C, double* w_out = nullptr) {
        qb_gemm(s, 0, 0, n, n, n, 1.0, F, n, Xm, n, 0.0, t1, n);
        qb_gemm(s, 1, 0, n, n, n, 1.0, Xm, n, t1, n, 0.0, t2, n);
        qb_symmetrize_upper(s, n, t2);
        if (qb_eigh(s, n, t2, w_out ? w_out : eigw, t3, eigwork, ctx->status.p) != 0)
            return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "eigensolver limited to n <= 1024");
        qb_gemm(s, 0, 0, n, n, n, 1.0, Xm, n, t3, n, 0.0, C, n);
        qb_scale_columns_sign(s, n, C);
        return qb_cuda_check(ctx, cudaGetLastError(), "solve_fock");
    }

    void density(const double* C, int nocc, double* D) {
        if (nocc > 0) qb_gemm(s, 0, 1, n, n, nocc, 1.0, C, n, C, n, 0.0, D, n);
        else cudaMemsetAsync(D, 0, nn * sizeof(double), s);
    }

    // F^s = H + G^s(D) for every sector
    int fock(double* const* D, double* const* F) {
        if (nspin == 1) {
            QB_TRY(qb_jk_device(ctx, D[0], J, K, schwarz, s));
            qb_axpby(s, nn, 2.0, J, -1.0, K, F[0]);
            qb_axpby(s, nn, 1.0, F[0], 1.0, H, F[0]);
        } else {
            QB_TRY(qb_jk_device(ctx, D[0], J, K, schwarz, s));
            qb_axpby(s, nn, 1.0, H, -1.0, K, F[0]);     // F0 = H - K(Da)
            qb_axpby(s, nn, 1.0, J, 0.0, nullptr, t3);  // t3 = J(Da)
            QB_TRY(qb_jk_device(ctx, D[1], J, K, schwarz, s));
            qb_axpby(s, nn, 1.0, H, -1.0, K, F[1]);     // F1 = H - K(Db)
            qb_axpby(s, nn, 1.0, t3, 1.0, J, t3);       // t3 = J(Da + Db)
            qb_axpby(s, nn, 1.0, F[0], 1.0, t3, F[0]);
            qb_axpby(s, nn, 1.0, F[1], 1.0, t3, F[1]);
        }
        return qb_cuda_check(ctx, cudaGetLastError(), "fock");
    }

    // E^s = <D, H + F>/2 into scal[k]
    void energy(const double* F, const double* D, int k) {
        qb_axpby(s, nn, 1.0, H, 1.0, F, t1);
        qb_dot(s, nn, D, t1, scal + k);
        qb_axpby(s, 1, 0.5, scal + k, 0.0, nullptr, scal + k);
    }

    // RMS(FDS - SDF) into scal[k]; optionally keep X^T e X in R
    void residual(const double* F, const double* D, int k, double* R) {
        qb_gemm(s, 0, 0, n, n, n, 1.0, D, n, S, n, 0.0, t1, n);
        qb_gemm(s, 0, 0, n, n, n, 1.0, F, n, t1, n, 0.0, t2, n);
        dim3 grid((n + 127) / 128, n);
        residual_kernel<<<grid, 128, 0, s>>>(n, t2, t1);
        qb_dot(s, nn, t1, t1, scal + k);
        if (R) {
            qb_gemm(s, 0, 0, n, n, n, 1.0, t1, n, X, n, 0.0, t2, n);
            qb_gemm(s, 1, 0, n, n, n, 1.0, X, n, t2, n, 0.0, R, n);
        }
    }

    int break_symmetry_core(const double* C1, const double* C2, double* out1, double* out2) {
        // inv(Hermitian(X)) = U diag(1/w) U^T
        cudaMemcpyAsync(t2, X, nn * sizeof(double), cudaMemcpyDeviceToDevice, s);
        qb_symmetrize_upper(s, n, t2);
        if (qb_eigh(s, n, t2, eigw, t3, eigwork, ctx->status.p) != 0)
            return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "eigensolver limited to n <= 1024");
        double* inv = mat();
        double* o1 = mat();
        double* o2 = mat();
        if (!inv || !o1 || !o2) return qb_set_error(ctx, QB_ERR_NOMEM, "SCF matrices");
        qb_diag_func(s, n, t3, eigw, 2, inv, t1);
        qb_gemm(s, 0, 0, n, n, n, 1.0, inv, n, C1, n, 0.0, o1, n);
        qb_gemm(s, 0, 0, n, n, n, 1.0, inv, n, C2, n, 0.0, o2, n);
        break_sym_kernel<<<n, 32, 0, s>>>(n, o1, o2);
        qb_gemm(s, 0, 0, n, n, n, 1.0, X, n, o1, n, 0.0, out1, n);
        qb_gemm(s, 0, 0, n, n, n, 1.0, X, n, o2, n, 0.0, out2, n);
        drop(inv); drop(o1); drop(o2);
        return qb_cuda_check(ctx, cudaGetLastError(), "breakCoeffSymmetry");
    }
};

struct Trace {
    std::deque<Entry> steps;
};

struct RunState {
    std::vector<Trace> t;
    std::deque<double*> Dtots;
    std::vector<double> Etots;
};

struct StepOut {
    Entry e[2];
    double* Dtot = nullptr;
    double Etot = 0.0;
};

// getCDFE (HartreeFock.jl:392-403) from Fock matrices F[k]
int cdfe(Scf& sc, double* const* Fin, StepOut& out) {
    double* Dn[2] = {nullptr, nullptr};
    double* Fn[2] = {nullptr, nullptr};
    for (int k = 0; k < sc.nspin; ++k) {
        out.e[k].C = sc.mat();
        out.e[k].D = sc.mat();
        out.e[k].F = sc.mat();
        if (!out.e[k].C || !out.e[k].D || !out.e[k].F) return qb_set_error(sc.ctx, QB_ERR_NOMEM, "SCF matrices");
        QB_TRY(sc.solve_fock(sc.X, Fin[k], out.e[k].C));
        sc.density(out.e[k].C, sc.N[k], out.e[k].D);
        Dn[k] = out.e[k].D;
        Fn[k] = out.e[k].F;
    }
    QB_TRY(sc.fock(Dn, Fn));
    for (int k = 0; k < sc.nspin; ++k) sc.energy(Fn[k], Dn[k], k);
    double Eh[2];
    QB_TRY(sc.read(sc.scal, Eh, sc.nspin));
    for (int k = 0; k < sc.nspin; ++k) out.e[k].E = Eh[k];
    out.Dtot = sc.mat();
    if (!out.Dtot) return qb_set_error(sc.ctx, QB_ERR_NOMEM, "SCF matrices");
    if (sc.nspin == 1) qb_axpby(sc.s, sc.nn, 2.0, Dn[0], 0.0, nullptr, out.Dtot);
    else qb_axpby(sc.s, sc.nn, 1.0, Dn[0], 1.0, Dn[1], out.Dtot);
    out.Etot = sc.nspin == 1 ? 2 * Eh[0] : Eh[0] + Eh[1];
    return qb_cuda_check(sc.ctx, cudaGetLastError(), "getCDFE");
}

// updateHFtempInfo! (HartreeFock.jl:463-477)
void push_step(Scf& sc, size_t maxLen, RunState& st, StepOut& r) {
    for (int k = 0; k < sc.nspin; ++k) {
        auto& q = st.t[k].steps;
        while (q.size() >= maxLen) {
            sc.drop(q.front().C); sc.drop(q.front().D); sc.drop(q.front().F);
            q.pop_front();
        }
        q.push_back(r.e[k]);
    }
    while (st.Dtots.size() >= maxLen) {
        sc.drop(st.Dtots.front());
        st.Dtots.pop_front();
    }
    st.Dtots.push_back(r.Dtot);
    st.Etots.push_back(r.Etot);
}

void pop_steps(Scf& sc, RunState& st, int count) {   // popHFtempInfo! (:479-494)
    for (auto& tr : st.t)
        for (int c = 0; c < count && !tr.steps.empty(); ++c) {
            sc.drop(tr.steps.back().C); sc.drop(tr.steps.back().D); sc.drop(tr.steps.back().F);
            tr.steps.pop_back();
        }
    for (int c = 0; c < count && !st.Dtots.empty(); ++c) {
        sc.drop(st.Dtots.back());
        st.Dtots.pop_back();
        st.Etots.pop_back();
    }
}

int error_norm(Scf& sc, RunState& st, double* out) {   // getErrorNrms (:1230-1237)
    for (int k = 0; k < sc.nspin; ++k) sc.residual(st.t[k].steps.back().F, st.t[k].steps.back().D, k, nullptr);
    double v[2];
    QB_TRY(sc.read(sc.scal, v, sc.nspin));
    double acc = 0.0;
    for (int k = 0; k < sc.nspin; ++k) acc += std::sqrt(v[k]) / std::sqrt((double)sc.nn);
    *out = acc / sc.nspin;
    return QB_OK;
}

double stdev(const std::vector<double>& v) {
    const double m = std::accumulate(v.begin(), v.end(), 0.0) / v.size();
    double s = 0.0;
    for (double x : v) s += (x - m) * (x - m);
    return std::sqrt(s / (v.size() - 1));
}

bool oscillate_converged(const std::vector<double>& seq, double tar, int minLen, int maxRemains) {   // Tools.jl:291-315
    const int len = (int)seq.size();
    if (len < minLen) return false;
    const int slice = std::min(maxRemains, len / 3 + 1);
    std::vector<double> tail(seq.end() - slice, seq.end());
    if (tail.size() < 2) return false;
    std::sort(tail.begin(), tail.end());
    std::vector<double> valleys(tail.begin(), tail.begin() + (tail.size() / 2 + 1));
    const double target = *std::min_element(valleys.begin(), valleys.end());
    return stdev(valleys) <= 0.8 * tar && std::fabs(target - seq.back()) <= tar;
}

struct Core {
    int method;
    int solver = QB_DIIS_LBFGS;   // coefficient solver (defaultDIISsolver, :17)
    double damp = 0.75;
    int diis_size = 15;
    double reset = 1000 * kAtolVal;
    std::vector<std::vector<DiisItem>> sub;   // per spin
    std::vector<std::vector<double>> cs;      // per spin: coefficient vector, starting point of the next solve
};

void drop_item(Scf& sc, DiisItem& it) {
    sc.drop(it.D); sc.drop(it.F); sc.drop(it.R);
    it.D = it.F = it.R = nullptr;
}

int add_item(Scf& sc, Core& core, int k, const double* D, const double* F, double E) {
    DiisItem it;
    it.D = sc.mat();
    it.F = sc.mat();
    if (!it.D || !it.F) return qb_set_error(sc.ctx, QB_ERR_NOMEM, "SCF matrices");
    cudaMemcpyAsync(it.D, D, sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, sc.s);
    cudaMemcpyAsync(it.F, F, sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, sc.s);
    if (core.method == QB_SCF_DIIS) {
        it.R = sc.mat();
        if (!it.R) return qb_set_error(sc.ctx, QB_ERR_NOMEM, "SCF matrices");
        sc.residual(F, D, 15, it.R);
    }
    it.E = E;
    core.sub[k].push_back(it);
    return QB_OK;
}

int run_core(Scf& sc, Core& core, RunState& st, StepOut& out) {
    double* Fn[2] = {nullptr, nullptr};
    if (core.method == QB_SCF_DD) {   // directDiag (:1245-1270)
        double* Dn[2] = {nullptr, nullptr};
        for (int k = 0; k < sc.nspin; ++k) {
            double* C = sc.mat();
            Dn[k] = sc.mat();
            Fn[k] = sc.mat();
            if (!C || !Dn[k] || !Fn[k]) return qb_set_error(sc.ctx, QB_ERR_NOMEM, "SCF matrices");
            QB_TRY(sc.solve_fock(sc.X, st.t[k].steps.back().F, C));
            sc.density(C, sc.N[k], Dn[k]);
            qb_axpby(sc.s, sc.nn, 1.0 - core.damp, Dn[k], core.damp, st.t[k].steps.back().D, Dn[k]);
            sc.drop(C);
        }
        QB_TRY(sc.fock(Dn, Fn));
        const int rc = cdfe(sc, Fn, out);
        for (int k = 0; k < sc.nspin; ++k) { sc.drop(Dn[k]); sc.drop(Fn[k]); }
        return rc;
    }
    for (int k = 0; k < sc.nspin; ++k) {
        auto& sub = core.sub[k];
        const int m = (int)sub.size();
        std::vector<const double*> P(m), Q(m);
        std::vector<double> E(m);
        for (int i = 0; i < m; ++i) {
            P[i] = core.method == QB_SCF_DIIS ? sub[i].R : sub[i].D;
            Q[i] = core.method == QB_SCF_DIIS ? sub[i].R : sub[i].F;
            E[i] = sub[i].E;
        }
        QB_CUDA(sc.ctx, cudaMemcpyAsync(sc.ptrs_d, P.data(), m * sizeof(double*), cudaMemcpyHostToDevice, sc.s));
        QB_CUDA(sc.ctx, cudaMemcpyAsync(sc.ptrs2_d, Q.data(), m * sizeof(double*), cudaMemcpyHostToDevice, sc.s));
        QB_CUDA(sc.ctx, cudaMemcpyAsync(sc.E_d, E.data(), m * sizeof(double), cudaMemcpyHostToDevice, sc.s));
        QB_CUDA(sc.ctx, cudaMemcpyAsync(sc.c, core.cs[k].data(), m * sizeof(double), cudaMemcpyHostToDevice, sc.s));
        gram_kernel<<<dim3(m, m), 256, 0, sc.s>>>(m, (long long)sc.nn, sc.ptrs_d, sc.ptrs2_d, sc.gram);
        diis_system_kernel<<<1, dim3(16, 16), 0, sc.s>>>(m, core.method, sc.gram, sc.E_d, sc.B, sc.v);
        if (qb_diis_solve(sc.s, m, core.method != QB_SCF_DIIS, core.solver, sc.B, sc.v, sc.c, nullptr,
                          sc.ctx->status.p) != 0)
            return qb_set_error(sc.ctx, QB_ERR_ARG, "DIIS subspace size or solver out of range");
        std::vector<const double*> Fp(m);
        for (int i = 0; i < m; ++i) Fp[i] = sub[i].F;
        QB_CUDA(sc.ctx, cudaMemcpyAsync(sc.ptrs_d, Fp.data(), m * sizeof(double*), cudaMemcpyHostToDevice, sc.s));
        Fn[k] = sc.mat();
        if (!Fn[k]) return qb_set_error(sc.ctx, QB_ERR_NOMEM, "SCF matrices");
        qb_lincomb(sc.s, (long long)sc.nn, m, sc.ptrs_d, sc.c, Fn[k]);
        QB_CUDA(sc.ctx, cudaMemcpyAsync(core.cs[k].data(), sc.c, m * sizeof(double), cudaMemcpyDeviceToHost, sc.s));
        // the pointer table is reused by the next sector: finish this one first
        QB_CUDA(sc.ctx, cudaStreamSynchronize(sc.s));
    }
    QB_TRY(cdfe(sc, Fn, out));
    for (int k = 0; k < sc.nspin; ++k) sc.drop(Fn[k]);
    for (int k = 0; k < sc.nspin; ++k) {
        auto& sub = core.sub[k];
        auto& c = core.cs[k];
        QB_TRY(add_item(sc, core, k, out.e[k].D, out.e[k].F, out.e[k].E));
        c.push_back(1.0);
        const size_t L = sub.size();
        if (L > 2 && sub[L - 1].E - sub[L - 2].E > core.reset) {   // keepOnly! of the second-to-last
            DiisItem keep = sub[L - 2];
            for (size_t i = 0; i < L; ++i)
                if (i != L - 2) drop_item(sc, sub[i]);
            sub.assign(1, keep);
            c.assign(1, c[L - 2]);
        } else if ((int)L > core.diis_size) {
            size_t pi = 0;
            for (size_t i = 1; i < L; ++i)
                if (sub[i].E > sub[pi].E) pi = i;
            drop_item(sc, sub[pi]);
            sub.erase(sub.begin() + pi);
            c.erase(c.begin() + pi);
        }
    }
    return qb_check_status(sc.ctx);
}

struct CoreResult {
    int converged;
    int steps;
    double dE, dD, dF;
};

// runHartreeFockCore (HartreeFock.jl:1049-1228)
int scf_core(Scf& sc, double* const* C0, const qb_scf_config& cfg, const int* methods, const double* intervals,
             const int* solvers, int nmeth, int maxStep, RunState& st, CoreResult& res) {
    st.t.assign(sc.nspin, Trace{});
    {   // initializeSCF (:526-542)
        StepOut r;
        double* Dn[2] = {nullptr, nullptr};
        double* Fn[2] = {nullptr, nullptr};
        for (int k = 0; k < sc.nspin; ++k) {
            r.e[k].C = sc.mat();
            r.e[k].D = sc.mat();
            r.e[k].F = sc.mat();
            if (!r.e[k].C || !r.e[k].D || !r.e[k].F) return qb_set_error(sc.ctx, QB_ERR_NOMEM, "SCF matrices");
            cudaMemcpyAsync(r.e[k].C, C0[k], sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, sc.s);
            sc.density(r.e[k].C, sc.N[k], r.e[k].D);
            Dn[k] = r.e[k].D;
            Fn[k] = r.e[k].F;
        }
        QB_TRY(sc.fock(Dn, Fn));
        for (int k = 0; k < sc.nspin; ++k) sc.energy(Fn[k], Dn[k], k);
        double Eh[2];
        QB_TRY(sc.read(sc.scal, Eh, sc.nspin));
        for (int k = 0; k < sc.nspin; ++k) r.e[k].E = Eh[k];
        r.Dtot = sc.mat();
        if (sc.nspin == 1) qb_axpby(sc.s, sc.nn, 2.0, Dn[0], 0.0, nullptr, r.Dtot);
        else qb_axpby(sc.s, sc.nn, 1.0, Dn[0], 1.0, Dn[1], r.Dtot);
        r.Etot = sc.nspin == 1 ? 2 * Eh[0] : Eh[0] + Eh[1];
        st.Etots.clear();
        st.Dtots.clear();
        push_step(sc, 1 << 20, st, r);
    }
    std::vector<double> dEs = {0.0}, dDrms = {0.0}, dFrms;
    double e0;
    QB_TRY(error_norm(sc, st, &e0));
    dFrms.push_back(e0);
    const double ratio1 = cfg.secondary_ratio[0], ratio2 = cfg.secondary_ratio[1], oscThr = cfg.oscillate_threshold;
    const int HFminItr = 10, oscSize = 15;
    int converged = 1, i = 0;
    for (int l = 0; l < nmeth; ++l) {
        const bool endM = (l == nmeth - 1);
        const double bp = intervals[l];
        const size_t len = methods[l] == QB_SCF_DD ? 3 : (size_t)std::max(3, cfg.diis_size);
        Core core;
        core.method = methods[l];
        core.damp = cfg.damp_strength;
        core.diis_size = cfg.diis_size;
        core.solver = solvers[l];
        if (core.method != QB_SCF_DD) {   // initializeHFcore for DIIS types (:1335-1360)
            core.sub.resize(sc.nspin);
            core.cs.resize(sc.nspin);
            const size_t init = std::min<size_t>(core.diis_size, st.t[0].steps.size());
            for (int k = 0; k < sc.nspin; ++k) {
                for (size_t x = 0; x < init; ++x) core.cs[k].push_back((double)(x + 1));   // collect(OneTo(init))
                auto& q = st.t[k].steps;
                for (size_t x = q.size() - init; x < q.size(); ++x) QB_TRY(add_item(sc, core, k, q[x].D, q[x].F, q[x].E));
            }
        }
        const double fluc = std::max(10 * bp, 1.5e-3);
        const double dFbp = ratio1 * bp, dDbp = ratio2 * bp;
        const double dEosc = std::max(bp, oscThr), dFosc = ratio1 * dEosc, dDosc = ratio2 * dEosc;
        converged = 0;
        int nstep = 0;
        int rc = QB_OK;
        while (true) {
            if (!(i < maxStep)) break;
            ++i;
            ++nstep;
            StepOut r;
            rc = run_core(sc, core, st, r);
            if (rc != QB_OK) break;
            push_step(sc, len, st, r);
            dEs.push_back(st.Etots.back() - st.Etots[st.Etots.size() - 2]);
            qb_axpby(sc.s, sc.nn, 1.0, st.Dtots.back(), -1.0, st.Dtots[st.Dtots.size() - 2], sc.t1);
            qb_dot(sc.s, sc.nn, sc.t1, sc.t1, sc.scal + 8);
            double dd;
            rc = sc.read(sc.scal + 8, &dd, 1);
            if (rc != QB_OK) break;
            dDrms.push_back(std::sqrt(dd) / std::sqrt((double)sc.nn));
            double ef;
            rc = error_norm(sc, st, &ef);
            if (rc != QB_OK) break;
            dFrms.push_back(ef);
            const double dE = dEs.back(), dD = dDrms.back(), dF = dFrms.back(), adE = std::fabs(dE);
            double th0 = bp, th1 = dDbp;
            if (dF > dFbp) th0 = th1 = 0.0;
            if (adE <= th0 && dD <= th1) { converged = 1; break; }
            if (nstep > 1 && i > HFminItr && dE > fluc) {
                bool isOsc = false;
                if (oscThr > 0) {
                    isOsc = oscillate_converged(st.Etots, 10 * dEosc, HFminItr, oscSize);
                    if (isOsc && adE <= dEosc && (endM ? (dF <= dFosc && dD <= dDosc) : true)) {
                        converged = 2;
                        break;
                    }
                }
                if (cfg.early_stop && !isOsc) {
                    bool raising = true;
                    for (int j = 0; j <= HFminItr / 3; ++j)
                        if (!(dEs[dEs.size() - 1 - j] > 10 * fluc)) raising = false;
                    if (raising) {
                        const int memLen = (int)st.t[0].steps.size();
                        const int rb = std::min(HFminItr / 3 + 1, std::max(memLen - 1, 0));
                        pop_steps(sc, st, rb);
                        i -= rb;
                        break;
                    }
                }
            }
        }
        for (auto& sub : core.sub)
            for (auto& it : sub) drop_item(sc, it);
        if (rc != QB_OK) return rc;
    }
    res.converged = converged;
    res.steps = i;
    res.dE = dEs.back();
    res.dD = dDrms.back();
    res.dF = dFrms.back();
    return QB_OK;
}

void release_state(Scf& sc, RunState& st) {
    for (auto& tr : st.t)
        for (auto& e : tr.steps) { sc.drop(e.C); sc.drop(e.D); sc.drop(e.F); }
    for (double* p : st.Dtots) sc.drop(p);
    st.t.clear();
    st.Dtots.clear();
}

}  // namespace

extern "C" void qb_scf_config_default(qb_scf_config* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->uhf = 0;
    cfg->guess = QB_GUESS_SAD;
    cfg->nmethod = 3;   // SCFconfig() = ((:DD, :ADIIS, :DIIS), (5e-3, 1e-4, 1e-9)) (:27)
    cfg->method[0] = QB_SCF_DD;
    cfg->method[1] = QB_SCF_ADIIS;
    cfg->method[2] = QB_SCF_DIIS;
    cfg->interval[0] = 5e-3;
    cfg->interval[1] = 1e-4;
    cfg->interval[2] = 1e-9;
    cfg->secondary_ratio[0] = 1000.0;
    cfg->secondary_ratio[1] = 1000.0;
    cfg->oscillate_threshold = 5e-6;
    cfg->max_step = 200;
    cfg->early_stop = 1;
    cfg->diis_size = 15;
    cfg->damp_strength = 0.75;
    cfg->schwarz = 1e-14;
    for (int l = 0; l < 8; ++l) cfg->solver[l] = QB_DIIS_LBFGS;   // defaultDIISsolver (:17)
}

extern "C" int qb_diis_coefficients(qb_ctx* ctx, int solver, int convex, int m, const double* B, const double* v,
                                    double* c, int* iterations) {
    if (!ctx || !B || !c) return qb_set_error(ctx, QB_ERR_ARG, "null argument");
    if (m < 1 || m > 15) return qb_set_error(ctx, QB_ERR_DOMAIN, "DIIS subspace size must be 1..15");
    if (solver < QB_DIIS_LBFGS || solver > QB_DIIS_LCM) return qb_set_error(ctx, QB_ERR_ARG, "unknown solver");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return qb_set_error(ctx, QB_ERR_CUDA, "cudaSetDevice");
    cudaStream_t s = ctx->stream;
    const size_t bytes = (size_t)m * m * sizeof(double) + 2 * (size_t)m * sizeof(double) + sizeof(double);
    double* buf = nullptr;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) return qb_set_error(ctx, QB_ERR_NOMEM, "DIIS buffers");
    double *dB = buf, *dv = buf + (size_t)m * m, *dc = dv + m;
    int* dit = reinterpret_cast<int*>(dc + m);
    std::vector<double> vz(m, 0.0);
    int rc = QB_OK;
    rc = qb_cuda_check(ctx, cudaMemcpyAsync(dB, B, (size_t)m * m * sizeof(double), cudaMemcpyHostToDevice, s), "B");
    if (rc == QB_OK)
        rc = qb_cuda_check(ctx, cudaMemcpyAsync(dv, v ? v : vz.data(), m * sizeof(double), cudaMemcpyHostToDevice, s), "v");
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaMemcpyAsync(dc, c, m * sizeof(double), cudaMemcpyHostToDevice, s), "c");
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaMemsetAsync(dit, 0, sizeof(int), s), "iterations");
    if (rc == QB_OK && qb_diis_solve(s, m, convex != 0, solver, dB, dv, dc, dit, ctx->status.p) != 0)
        rc = qb_set_error(ctx, QB_ERR_ARG, "DIIS solve");
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaMemcpyAsync(c, dc, m * sizeof(double), cudaMemcpyDeviceToHost, s), "c");
    int it = 0;
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaMemcpyAsync(&it, dit, sizeof(int), cudaMemcpyDeviceToHost, s), "iters");
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaStreamSynchronize(s), "DIIS solve");
    cudaFree(buf);
    if (rc != QB_OK) return rc;
    if (iterations) *iterations = solver == QB_DIIS_LCM ? 0 : it;
    return qb_check_status(ctx);
}

extern "C" int qb_run_hartree_fock(qb_ctx* ctx, const qb_basis* basis, int nnuc, const double* Z, const double* R,
                                   int n_alpha, int n_beta, const qb_scf_config* cfg, qb_scf_result* res) {
    if (!ctx || !cfg || !res) return qb_set_error(ctx, QB_ERR_ARG, "null argument");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return qb_set_error(ctx, QB_ERR_CUDA, "cudaSetDevice");
    QB_TRY(qb_set_basis(ctx, basis));
    const int n = ctx->nfun;
    if (cfg->nmethod < 1 || cfg->nmethod > 8) return qb_set_error(ctx, QB_ERR_ARG, "nmethod must be 1..8");
    for (int l = 0; l < cfg->nmethod; ++l)
        if (cfg->method[l] < 0 || cfg->method[l] > 3 || !(cfg->interval[l] >= 0.0) && !std::isnan(cfg->interval[l]))
            return qb_set_error(ctx, QB_ERR_ARG, "bad SCF method or threshold");
    for (int l = 0; l < cfg->nmethod; ++l)
        if (cfg->solver[l] < QB_DIIS_LBFGS || cfg->solver[l] > QB_DIIS_LCM)
            return qb_set_error(ctx, QB_ERR_ARG, "unknown DIIS coefficient solver");
    if (cfg->diis_size < 2 || cfg->diis_size > 15) return qb_set_error(ctx, QB_ERR_DOMAIN, "DIISsize must be 2..15");
    if (!(cfg->damp_strength >= 0.0 && cfg->damp_strength <= 1.0))
        return qb_set_error(ctx, QB_ERR_DOMAIN, "dampStrength must be in [0, 1]");
    if (cfg->max_step < 1) return qb_set_error(ctx, QB_ERR_DOMAIN, "maxStep must be positive");
    if (n_alpha < 0 || n_beta < 0) return qb_set_error(ctx, QB_ERR_DOMAIN, "negative occupation");
    const int nspin = cfg->uhf ? 2 : 1;
    if (!cfg->uhf && n_alpha != n_beta)
        return qb_set_error(ctx, QB_ERR_ARG, "closed-shell HF needs equal spin occupations");
    const int total = n_alpha + n_beta;
    if (total <= (cfg->uhf ? 0 : 1))   // runHartreeFock (:988-990)
        return qb_set_error(ctx, QB_ERR_DOMAIN, "too few electrons for this HF type");
    if (n < std::max(n_alpha, n_beta)) return qb_set_error(ctx, QB_ERR_DOMAIN, "basis smaller than occupation");
    if (n > 1024) return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "SCF supports at most 1024 basis functions");
    if (cfg->guess == QB_GUESS_SAD && (nnuc <= 0 || !Z || !R)) return qb_set_error(ctx, QB_ERR_ARG, "SAD needs nuclei");

    Scf sc;
    QB_TRY(sc.init(ctx, n));
    sc.nspin = nspin;
    sc.N[0] = n_alpha;
    sc.N[1] = n_beta;
    sc.schwarz = cfg->schwarz;
    cudaStream_t s = ctx->stream;
    // one-electron part and orthogonalisation (initializeHartreeFock, :178-210)
    double* T = sc.mat();
    double* V = sc.mat();
    if (!T || !V) return qb_set_error(ctx, QB_ERR_NOMEM, "SCF matrices");
    QB_TRY(qb_onebody_device(ctx, 1 | 2 | 4, nnuc, Z, R, sc.S, T, V));
    qb_axpby(s, sc.nn, 1.0, T, 1.0, V, sc.H);
    QB_TRY(qb_check_status(ctx));
    cudaMemcpyAsync(sc.t2, sc.S, sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, s);
    qb_symmetrize_upper(s, n, sc.t2);
    if (qb_eigh(s, n, sc.t2, sc.eigw, sc.t3, sc.eigwork, ctx->status.p) != 0)
        return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "eigensolver limited to n <= 1024");
    {
        std::vector<double> w(n);
        QB_TRY(sc.read(sc.eigw, w.data(), n));
        if (!(w[0] > 0.0)) return qb_set_error(ctx, QB_ERR_DOMAIN, "overlap matrix is not positive definite");
    }
    qb_diag_func(s, n, sc.t3, sc.eigw, 0, sc.X, sc.t1);

    // initial coefficients
    double* C0[2] = {sc.mat(), nspin == 2 ? sc.mat() : nullptr};
    if (!C0[0] || (nspin == 2 && !C0[1])) return qb_set_error(ctx, QB_ERR_NOMEM, "SCF matrices");
    if (cfg->guess == QB_GUESS_DIRECT) {
        if (!cfg->C0) return qb_set_error(ctx, QB_ERR_DIM, "Direct guess needs coefficient matrices");
        for (int k = 0; k < nspin; ++k)
            QB_CUDA(ctx, cudaMemcpyAsync(C0[k], cfg->C0 + (size_t)k * sc.nn, sc.nn * sizeof(double),
                                         cudaMemcpyHostToDevice, s));
    } else if (cfg->guess == QB_GUESS_COREH || cfg->guess == QB_GUESS_GWH) {
        const double* Hg = sc.H;
        double* G = nullptr;
        if (cfg->guess == QB_GUESS_GWH) {
            G = sc.mat();
            qb_gwh(s, n, sc.S, sc.H, G);
            Hg = G;
        }
        QB_TRY(sc.solve_fock(sc.X, Hg, C0[0]));
        if (G) sc.drop(G);
        if (nspin == 2) {
            double* Cc = sc.mat();
            cudaMemcpyAsync(Cc, C0[0], sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, s);
            QB_TRY(sc.break_symmetry_core(Cc, Cc, C0[0], C0[1]));
            sc.drop(Cc);
        }
    } else if (cfg->guess == QB_GUESS_SAD) {   // (:266-293)
        double* Da = sc.mat();
        double* Db = sc.mat();
        double* Hs = sc.mat();
        double* Va = sc.mat();
        cudaMemsetAsync(Da, 0, sc.nn * sizeof(double), s);
        cudaMemsetAsync(Db, 0, sc.nn * sizeof(double), s);
        cudaMemcpyAsync(Hs, sc.H, sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, s);
        const int nspin0 = sc.nspin;
        sc.nspin = 2;
        for (int c = 0; c < nnuc; ++c) {
            QB_TRY(qb_onebody_device(ctx, 4, 1, Z + c, R + 3 * c, nullptr, nullptr, Va));
            qb_axpby(s, sc.nn, 1.0, T, 1.0, Va, sc.H);
            // CoreH guess of the atom with the overlap in place of X, then breakCoeffSymmetry
            double* Cg = sc.mat();
            double* Ca[2] = {sc.mat(), sc.mat()};
            QB_TRY(sc.solve_fock(sc.S, sc.H, Cg));
            {
                double* Xs = sc.X;
                sc.X = sc.S;
                const int rc = sc.break_symmetry_core(Cg, Cg, Ca[0], Ca[1]);
                sc.X = Xs;
                QB_TRY(rc);
            }
            sc.drop(Cg);
            RunState st;
            CoreResult cr;
            const int m3 = QB_SCF_ADIIS, sv = QB_DIIS_LBFGS;   // getDefaultSCFconfigForSAD (:262-264)
            const double iv = std::max(1e-2, 10 * kAtolVal);
            qb_scf_config acfg = *cfg;
            acfg.secondary_ratio[0] = acfg.secondary_ratio[1] = 1000.0;
            acfg.oscillate_threshold = 5e-6;
            acfg.early_stop = 1;
            acfg.diis_size = 15;
            QB_TRY(scf_core(sc, Ca, acfg, &m3, &iv, &sv, 1, 50, st, cr));
            qb_axpby(s, sc.nn, 1.0, Da, 1.0, st.t[0].steps.back().D, Da);
            qb_axpby(s, sc.nn, 1.0, Db, 1.0, st.t[1].steps.back().D, Db);
            release_state(sc, st);
            sc.drop(Ca[0]);
            sc.drop(Ca[1]);
        }
        sc.nspin = nspin0;
        cudaMemcpyAsync(sc.H, Hs, sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, s);
        qb_axpby(s, sc.nn, 1.0 / nnuc, Da, 0.0, nullptr, Da);
        qb_axpby(s, sc.nn, 1.0 / nnuc, Db, 0.0, nullptr, Db);
        if (nspin == 1) {
            qb_axpby(s, sc.nn, 0.5, Da, 0.5, Db, Da);
            double* Dl[1] = {Da};
            double* Fl[1] = {Va};
            QB_TRY(sc.fock(Dl, Fl));
            QB_TRY(sc.solve_fock(sc.X, Va, C0[0]));
        } else {
            double* Dl[2] = {Da, Db};
            double* Fl[2] = {Va, Hs};
            QB_TRY(sc.fock(Dl, Fl));
            QB_TRY(sc.solve_fock(sc.X, Va, C0[0]));
            QB_TRY(sc.solve_fock(sc.X, Hs, C0[1]));
            // breakCoeffSymmetry(UHF, X, (C1, C2)) (:108-119): only when the sectors nearly agree
            cudaMemcpyAsync(sc.t2, sc.X, sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, s);
            qb_symmetrize_upper(s, n, sc.t2);
            qb_eigh(s, n, sc.t2, sc.eigw, sc.t3, sc.eigwork, ctx->status.p);
            double* inv = sc.mat();
            qb_diag_func(s, n, sc.t3, sc.eigw, 2, inv, sc.t1);
            qb_axpby(s, sc.nn, 1.0, C0[0], -1.0, C0[1], Va);
            qb_gemm(s, 0, 0, n, n, n, 1.0, inv, n, Va, n, 0.0, Hs, n);
            qb_dot(s, sc.nn, Hs, Hs, sc.scal + 9);
            double d2;
            QB_TRY(sc.read(sc.scal + 9, &d2, 1));
            sc.drop(inv);
            if (std::sqrt(d2) / std::sqrt((double)sc.nn) < 0.1) {
                double* c1 = sc.mat();
                double* c2 = sc.mat();
                cudaMemcpyAsync(c1, C0[0], sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, s);
                cudaMemcpyAsync(c2, C0[1], sc.nn * sizeof(double), cudaMemcpyDeviceToDevice, s);
                QB_TRY(sc.break_symmetry_core(c1, c2, C0[0], C0[1]));
                sc.drop(c1);
                sc.drop(c2);
            }
        }
        sc.drop(Da); sc.drop(Db); sc.drop(Hs); sc.drop(Va);
    } else {
        return qb_set_error(ctx, QB_ERR_ARG, "unknown initial-guess method");
    }
    sc.drop(T);
    sc.drop(V);
    QB_TRY(qb_check_status(ctx));

    RunState st;
    CoreResult cr;
    QB_TRY(scf_core(sc, C0, *cfg, cfg->method, cfg->interval, cfg->solver, cfg->nmethod, cfg->max_step, st, cr));
    // results (HFfinalInfo, :803-819)
    res->E_elec = st.Etots.back();
    double enn = 0.0;   // nucRepulsion (src/Particles.jl:197-210)
    for (int a = 0; a < nnuc; ++a)
        for (int b = a + 1; b < nnuc; ++b) {
            const double dx = R[3 * a] - R[3 * b], dy = R[3 * a + 1] - R[3 * b + 1], dz = R[3 * a + 2] - R[3 * b + 2];
            enn += Z[a] * Z[b] / std::sqrt(dx * dx + dy * dy + dz * dz);
        }
    res->E_nuc = enn;
    res->converged = cr.converged;
    res->steps = cr.steps;
    res->dE = cr.dE;
    res->rms_dD = cr.dD;
    res->rms_FDS = cr.dF;
    for (int k = 0; k < nspin; ++k) {
        const Entry& e = st.t[k].steps.back();
        if (res->C) QB_CUDA(ctx, cudaMemcpyAsync(res->C + k * sc.nn, e.C, sc.nn * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (res->D) QB_CUDA(ctx, cudaMemcpyAsync(res->D + k * sc.nn, e.D, sc.nn * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (res->F) QB_CUDA(ctx, cudaMemcpyAsync(res->F + k * sc.nn, e.F, sc.nn * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (res->eps) {
            double* Ct = sc.mat();
            QB_TRY(sc.solve_fock(sc.X, e.F, Ct, sc.eigw));   // getOrbitalOccupations (:708-750)
            QB_CUDA(ctx, cudaMemcpyAsync(res->eps + k * n, sc.eigw, n * sizeof(double), cudaMemcpyDeviceToHost, s));
            QB_CUDA(ctx, cudaStreamSynchronize(s));
            sc.drop(Ct);
        }
    }
    QB_CUDA(ctx, cudaStreamSynchronize(s));
    release_state(sc, st);
    sc.drop(C0[0]);
    if (C0[1]) sc.drop(C0[1]);
    QB_TRY(qb_check_status(ctx));
    return cr.converged ? QB_OK : qb_set_error(ctx, QB_ERR_NOT_CONVERGED, "SCF stopped without convergence");
}
