// C ABI entry points (include/quiqbox_gb300.h).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include "qb_internal.h"

std::vector<double> qb_build_boys_table();

#define QB_TRY(expr)                  \
    do {                              \
        const int _rc = (expr);       \
        if (_rc != QB_OK) return _rc; \
    } while (0)
#define QB_CUDA(ctx, call) QB_TRY(qb_cuda_check((ctx), (call), #call))

static int enter(qb_ctx* ctx) {
    if (!ctx) return QB_ERR_ARG;
    ctx->err.clear();
    return qb_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
}

extern "C" {

int qb_create(qb_ctx** out, int device) {
    if (!out) return QB_ERR_ARG;
    *out = nullptr;
    qb_ctx* ctx = new (std::nothrow) qb_ctx();
    if (!ctx) return QB_ERR_NOMEM;
    ctx->device = device;
    int rc = qb_cuda_check(ctx, cudaSetDevice(device), "cudaSetDevice");
    cudaDeviceProp prop;
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    if (rc == QB_OK) {
        ctx->nsm = prop.multiProcessorCount;
        rc = qb_cuda_check(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream");
    }
    for (int k = 0; rc == QB_OK && k < QB_NSTREAM; ++k) {
        rc = qb_cuda_check(ctx, cudaStreamCreateWithFlags(&ctx->streams[k], cudaStreamNonBlocking), "stream");
        if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaEventCreateWithFlags(&ctx->ev_join[k], cudaEventDisableTiming), "event");
    }
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaEventCreate(&ctx->ev_start), "event");
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaEventCreate(&ctx->ev_stop), "event");
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming), "event");
    if (rc == QB_OK) {
        const std::vector<double> tab = qb_build_boys_table();
        rc = qb_cuda_check(ctx, ctx->boys.ensure(tab.size()), "Boys table");
        if (rc == QB_OK)
            rc = qb_cuda_check(ctx, cudaMemcpy(ctx->boys.p, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice),
                               "Boys table upload");
    }
    if (rc == QB_OK) rc = qb_cuda_check(ctx, ctx->status.ensure(1), "status word");
    if (rc == QB_OK) rc = qb_cuda_check(ctx, cudaMemset(ctx->status.p, 0, sizeof(int)), "status word");
    if (rc == QB_OK) {
        ctx->nclass = QB_NCLASS;
        qb_get_class_launchers(ctx->launch);
        // Variant per class: the generator's measured preference.  QB_JK_VARIANT overrides
        // it for tuning: "thread" (variant 0 everywhere), "warp" (variant 1 wherever
        // compiled), or one character per class, '0'..'5' (a variant that is not compiled
        // for a class falls back to the preference).
        const char* ov = getenv("QB_JK_VARIANT");
        for (int c = 0; c < ctx->nclass; ++c) {
            const ClassLaunchers& L = ctx->launch[c];
            int v = L.preferred;
            if (ov) {
                if (!strcmp(ov, "thread")) v = 0;
                else if (!strcmp(ov, "warp")) v = L.jk[1] ? 1 : 0;
                else if (strlen(ov) == (size_t)ctx->nclass && ov[c] >= '0' && ov[c] < '0' + QB_NVARIANT &&
                         L.jk[ov[c] - '0'])
                    v = ov[c] - '0';
            }
            if (!L.jk[v]) v = 0;
            ctx->variant[c] = v;
            ctx->occ[c] = L.occupancy[v]();
        }
        // QB_JK_PRIM_EPS overrides the primitive-quartet threshold of the J/K class kernels
        // (validation of the primitive screening; 0 evaluates every primitive quartet)
        if (const char* pe = getenv("QB_JK_PRIM_EPS")) {
            char* end = nullptr;
            const double v = strtod(pe, &end);
            if (end != pe && v >= 0.0) ctx->prim_eps = (float)v;
        }
        rc = qb_cuda_check(ctx, cudaGetLastError(), "kernel occupancy query");
    }
    if (rc != QB_OK) {
        // keep the context so that qb_last_error() can report why
        *out = ctx;
        return rc;
    }
    *out = ctx;
    return QB_OK;
}

void qb_destroy(qb_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int k = 0; k < QB_NSTREAM; ++k) {
        if (ctx->streams[k]) { cudaStreamSynchronize(ctx->streams[k]); cudaStreamDestroy(ctx->streams[k]); }
        if (ctx->ev_join[k]) cudaEventDestroy(ctx->ev_join[k]);
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    ctx->boys.release(); ctx->status.release();
    ctx->d_fp.release(); ctx->d_ijk.release(); ctx->d_cen.release(); ctx->d_alpha.release(); ctx->d_w.release();
    ctx->d_ratio.release(); ctx->d_pairs.release(); ctx->d_prims.release(); ctx->d_prims32.release(); ctx->d_Q.release(); ctx->d_npref.release();
    ctx->d_offs.release(); ctx->d_stats.release(); ctx->d_primcount.release();
    ctx->d_D.release(); ctx->d_Dt.release(); ctx->d_Jp.release(); ctx->d_Kp.release(); ctx->d_J.release();
    ctx->d_K.release(); ctx->d_dmax.release();
    ctx->d_m0.release(); ctx->d_m1.release(); ctx->d_m2.release(); ctx->d_nucZ.release(); ctx->d_nucR.release();
    ctx->d_big.release(); ctx->d_quart.release();
    delete ctx;
}

const char* qb_last_error(const qb_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int qb_device_info(qb_ctx* ctx, int* sm_count, int* cc_major, int* cc_minor) {
    QB_TRY(enter(ctx));
    cudaDeviceProp prop;
    QB_CUDA(ctx, cudaGetDeviceProperties(&prop, ctx->device));
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (cc_major) *cc_major = prop.major;
    if (cc_minor) *cc_minor = prop.minor;
    return QB_OK;
}

static int onebody_api(qb_ctx* ctx, const qb_basis* basis, int flags, int nnuc, const double* Z, const double* R,
                       double* out) {
    QB_TRY(enter(ctx));
    if (!out) return qb_set_error(ctx, QB_ERR_ARG, "null output");
    QB_TRY(qb_set_basis(ctx, basis));
    const size_t nn = (size_t)ctx->nfun * ctx->nfun;
    QB_CUDA(ctx, ctx->d_m0.ensure(nn));
    QB_CUDA(ctx, ctx->d_m1.ensure(nn));
    double* S = (flags & 1) ? ctx->d_m0.p : nullptr;
    double* T = (flags & 2) ? ctx->d_m0.p : nullptr;
    double* V = (flags & 4) ? ((flags & 2) ? ctx->d_m1.p : ctx->d_m0.p) : nullptr;
    QB_TRY(qb_onebody_device(ctx, flags, nnuc, Z, R, S, T, V));
    if ((flags & 6) == 6) qb_axpby(ctx->stream, nn, 1.0, ctx->d_m0.p, 1.0, ctx->d_m1.p, ctx->d_m0.p);
    QB_CUDA(ctx, cudaMemcpyAsync(out, ctx->d_m0.p, nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return qb_check_status(ctx);
}

int qb_overlaps(qb_ctx* ctx, const qb_basis* basis, double* S) { return onebody_api(ctx, basis, 1, 0, nullptr, nullptr, S); }
int qb_elec_kinetics(qb_ctx* ctx, const qb_basis* basis, double* T) {
    return onebody_api(ctx, basis, 2, 0, nullptr, nullptr, T);
}
int qb_nuc_attractions(qb_ctx* ctx, const qb_basis* basis, int nnuc, const double* Z, const double* R, double* V) {
    return onebody_api(ctx, basis, 4, nnuc, Z, R, V);
}
int qb_core_hamiltonian(qb_ctx* ctx, const qb_basis* basis, int nnuc, const double* Z, const double* R, double* H) {
    return onebody_api(ctx, basis, 6, nnuc, Z, R, H);
}

int qb_multipole_moments(qb_ctx* ctx, const qb_basis* basis, const double* center, const int* degrees, double* M) {
    QB_TRY(enter(ctx));
    if (!M || !center || !degrees) return qb_set_error(ctx, QB_ERR_ARG, "null argument");
    for (int k = 0; k < 3; ++k) {
        if (!std::isfinite(center[k])) return qb_set_error(ctx, QB_ERR_DOMAIN, "non-finite multipole centre");
        if (degrees[k] < 0) return qb_set_error(ctx, QB_ERR_DOMAIN, "negative multipole degree");
    }
    QB_TRY(qb_set_basis(ctx, basis));
    const size_t nn = (size_t)ctx->nfun * ctx->nfun;
    QB_CUDA(ctx, ctx->d_m0.ensure(nn));
    if (qb_gen_multipole(qb_gen_basis(ctx), center, degrees, ctx->d_m0.p, ctx->status.p, ctx->stream) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "multipole kernel");
    QB_CUDA(ctx, cudaMemcpyAsync(M, ctx->d_m0.p, nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return qb_check_status(ctx);
}

int qb_adjoint_jk(qb_ctx* ctx, const qb_basis* basis, int n, const double* P, double* Jx, double* Kx) {
    QB_TRY(enter(ctx));
    if (!basis || !P || !Jx || !Kx) return qb_set_error(ctx, QB_ERR_ARG, "null argument");
    if (n < 1 || n >= basis->nfun) return qb_set_error(ctx, QB_ERR_DIM, "need 1 <= n < nfun (extra functions after n)");
    QB_TRY(qb_set_basis(ctx, basis));
    const int ng = ctx->nfun - n;
    const size_t nn = (size_t)n * n, gn = (size_t)ng * n;
    QB_CUDA(ctx, ctx->d_m0.ensure(nn));
    QB_CUDA(ctx, ctx->d_m1.ensure(2 * gn));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_m0.p, P, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    QB_CUDA(ctx, cudaMemsetAsync(ctx->d_m1.p, 0, 2 * gn * sizeof(double), ctx->stream));
    if (qb_gen_adjoint_eri(qb_gen_basis(ctx), n, ng, ctx->d_m0.p, ctx->boys.p, ctx->d_m1.p, ctx->d_m1.p + gn,
                           ctx->status.p, ctx->nsm, ctx->stream) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "adjoint ERI kernel");
    QB_CUDA(ctx, cudaMemcpyAsync(Jx, ctx->d_m1.p, gn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaMemcpyAsync(Kx, ctx->d_m1.p + gn, gn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return qb_check_status(ctx);
}

int qb_eigh_lowest(qb_ctx* ctx, int n, int k, const double* A, double* w, double* Y) {
    QB_TRY(enter(ctx));
    if (!A || !w || !Y) return qb_set_error(ctx, QB_ERR_ARG, "null argument");
    if (n < 1 || n > 1024 || k < 1 || k > n) return qb_set_error(ctx, QB_ERR_DIM, "need 1 <= k <= n <= 1024");
    const size_t nn = (size_t)n * n, nk = (size_t)n * k;
    QB_CUDA(ctx, ctx->d_m0.ensure(nn));
    QB_CUDA(ctx, ctx->d_m1.ensure(nk + k + 3 * nk + n));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_m0.p, A, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    double* dY = ctx->d_m1.p;
    double* dw = dY + nk;
    if (qb_lowest_eig(ctx->stream, n, k, ctx->d_m0.p, dY, dw, dw + k) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "eigensolver kernel");
    QB_CUDA(ctx, cudaMemcpyAsync(Y, dY, nk * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaMemcpyAsync(w, dw, k * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QB_OK;
}

int qb_elec_repulsions(qb_ctx* ctx, const qb_basis* basis, double* eri) {
    QB_TRY(enter(ctx));
    if (!eri) return qb_set_error(ctx, QB_ERR_ARG, "null output");
    QB_TRY(qb_set_basis(ctx, basis));
    const size_t n = ctx->nfun, n4 = n * n * n * n;
    QB_CUDA(ctx, ctx->d_big.ensure(n4));
    if (qb_gen_eri(qb_gen_basis(ctx), 0, ctx->boys.p, ctx->d_big.p, nullptr, nullptr, nullptr, ctx->status.p,
                   ctx->nsm, ctx->stream) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "generic ERI kernel");
    QB_CUDA(ctx, cudaMemcpyAsync(eri, ctx->d_big.p, n4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return qb_check_status(ctx);
}

int qb_elec_repulsion_list(qb_ctx* ctx, const qb_basis* basis, int64_t nq, const int* quartets, double* out) {
    QB_TRY(enter(ctx));
    if (nq < 0 || (nq > 0 && (!quartets || !out))) return qb_set_error(ctx, QB_ERR_ARG, "bad quartet list");
    QB_TRY(qb_set_basis(ctx, basis));
    if (nq == 0) return QB_OK;
    for (int64_t q = 0; q < 4 * nq; ++q)
        if (quartets[q] < 0 || quartets[q] >= ctx->nfun) return qb_set_error(ctx, QB_ERR_DIM, "quartet index out of range");
    QB_CUDA(ctx, ctx->d_quart.ensure(4 * (size_t)nq));
    QB_CUDA(ctx, ctx->d_big.ensure((size_t)nq));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_quart.p, quartets, 4 * nq * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    if (qb_gen_eri_list(qb_gen_basis(ctx), ctx->boys.p, nq, ctx->d_quart.p, ctx->d_big.p, ctx->status.p, ctx->stream) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "ERI list kernel");
    QB_CUDA(ctx, cudaMemcpyAsync(out, ctx->d_big.p, nq * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return qb_check_status(ctx);
}

int qb_boys(qb_ctx* ctx, int n, const double* T, int M, int path, double* F) {
    QB_TRY(enter(ctx));
    if (n < 0 || (n > 0 && (!T || !F))) return qb_set_error(ctx, QB_ERR_ARG, "bad Boys arguments");
    if (path != 0 && path != 1) return qb_set_error(ctx, QB_ERR_ARG, "Boys path must be 0 or 1");
    if (M < 0 || M > (path == 0 ? 8 : QB_GEN_LTOT_MAX)) return qb_set_error(ctx, QB_ERR_DIM, "Boys order out of range");
    for (int i = 0; i < n; ++i)
        if (!(T[i] >= 0.0) || !std::isfinite(T[i])) return qb_set_error(ctx, QB_ERR_DOMAIN, "Boys argument must be finite and >= 0");
    if (n == 0) return QB_OK;
    QB_CUDA(ctx, ctx->d_m0.ensure((size_t)n));
    QB_CUDA(ctx, ctx->d_big.ensure((size_t)n * (M + 1)));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_m0.p, T, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (qb_boys_device(n, ctx->d_m0.p, M, path, ctx->boys.p, ctx->d_big.p, ctx->stream) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "Boys kernel");
    QB_CUDA(ctx, cudaMemcpyAsync(F, ctx->d_big.p, (size_t)n * (M + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QB_OK;
}

int qb_run_rhf_batched(qb_ctx* ctx, int nmol, const qb_basis* bases, const int* nnuc, const double* Z,
                       const double* R, const int* nocc, const qb_batch_config* cfg, qb_batch_result* res) {
    QB_TRY(enter(ctx));
    return qb_batch_rhf_run(ctx, nmol, bases, nnuc, Z, R, nocc, cfg, res);
}

int qb_jk_prepare(qb_ctx* ctx, const qb_basis* basis, double schwarz) {
    QB_TRY(enter(ctx));
    if (!(schwarz >= 0.0)) return qb_set_error(ctx, QB_ERR_DOMAIN, "Schwarz threshold must be >= 0");
    QB_TRY(qb_set_basis(ctx, basis));
    if (ctx->shell_path) QB_TRY(qb_ensure_pairs(ctx));
    const size_t nn = (size_t)ctx->nfun * ctx->nfun;
    QB_CUDA(ctx, ctx->d_D.ensure(nn));
    QB_CUDA(ctx, ctx->d_J.ensure(nn));
    QB_CUDA(ctx, ctx->d_K.ensure(nn));
    ctx->schwarz = schwarz;
    ctx->jk_prepared = true;
    return QB_OK;
}

int qb_jk_upload_density(qb_ctx* ctx, const double* D) {
    QB_TRY(enter(ctx));
    if (!ctx->jk_prepared) return qb_set_error(ctx, QB_ERR_ARG, "call qb_jk_prepare first");
    if (!D) return qb_set_error(ctx, QB_ERR_ARG, "null density");
    const size_t nn = (size_t)ctx->nfun * ctx->nfun;
    return qb_cuda_check(ctx, cudaMemcpyAsync(ctx->d_D.p, D, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
                         "density upload");
}

int qb_jk_execute(qb_ctx* ctx) {
    QB_TRY(enter(ctx));
    if (!ctx->jk_prepared) return qb_set_error(ctx, QB_ERR_ARG, "call qb_jk_prepare first");
    QB_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
    QB_TRY(qb_jk_device(ctx, ctx->d_D.p, ctx->d_J.p, ctx->d_K.p, ctx->schwarz, ctx->stream));
    QB_CUDA(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
    return QB_OK;
}

int qb_jk_quartet_list(qb_ctx* ctx, int64_t nq, const int* pairs, double* J, double* K) {
    QB_TRY(enter(ctx));
    if (!ctx->jk_prepared) return qb_set_error(ctx, QB_ERR_ARG, "call qb_jk_prepare first");
    if (nq < 0 || (nq > 0 && !pairs)) return qb_set_error(ctx, QB_ERR_ARG, "bad quartet list");
    QB_TRY(qb_jk_quartets_device(ctx, (long long)nq, pairs, ctx->d_J.p, ctx->d_K.p));
    return qb_jk_download(ctx, J, K);
}

int qb_jk_autotune(qb_ctx* ctx, int repeats, int* variants) {
    QB_TRY(enter(ctx));
    return qb_jk_autotune_device(ctx, repeats, variants);
}

int qb_jk_class_times(qb_ctx* ctx, int repeats, float* ms) {
    QB_TRY(enter(ctx));
    if (!ms) return qb_set_error(ctx, QB_ERR_ARG, "null output");
    return qb_jk_class_times_device(ctx, repeats, ms);
}

int qb_jk_download(qb_ctx* ctx, double* J, double* K) {
    QB_TRY(enter(ctx));
    if (!ctx->jk_prepared) return qb_set_error(ctx, QB_ERR_ARG, "call qb_jk_prepare first");
    const size_t nn = (size_t)ctx->nfun * ctx->nfun;
    if (J) QB_CUDA(ctx, cudaMemcpyAsync(J, ctx->d_J.p, nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (K) QB_CUDA(ctx, cudaMemcpyAsync(K, ctx->d_K.p, nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return qb_check_status(ctx);
}

int qb_jk(qb_ctx* ctx, const qb_basis* basis, const double* D, double schwarz, double* J, double* K) {
    QB_TRY(qb_jk_prepare(ctx, basis, schwarz));
    QB_TRY(qb_jk_upload_density(ctx, D));
    QB_TRY(qb_jk_execute(ctx));
    return qb_jk_download(ctx, J, K);
}

int qb_jk_get_stats(qb_ctx* ctx, qb_jk_stats* st) {
    QB_TRY(enter(ctx));
    if (!st) return qb_set_error(ctx, QB_ERR_ARG, "null stats");
    std::memset(st, 0, sizeof(*st));
    st->shell_path = ctx->shell_path ? 1 : 0;
    st->nshell = (int)ctx->shells.size();
    st->npair = ctx->shell_path && ctx->pairs_valid ? ctx->pc_off[ctx->npc] : 0;
    st->nclass = ctx->nclass;
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop) == cudaSuccess) st->ms_last = ms;
    cudaGetLastError();
    if (!ctx->shell_path || !ctx->pairs_valid || !ctx->last_execute_shell) return QB_OK;
    std::vector<long long> stats(2 * ctx->nclass);
    std::vector<unsigned long long> prim(ctx->nclass);
    QB_CUDA(ctx, cudaMemcpy(stats.data(), ctx->d_stats.p, stats.size() * sizeof(long long), cudaMemcpyDeviceToHost));
    QB_CUDA(ctx, cudaMemcpy(prim.data(), ctx->d_primcount.p, prim.size() * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost));
    double flops = 0.0;
    for (int c = 0; c < ctx->nclass && c < 32; ++c) {
        st->class_quartets[c] = stats[2 * c];
        st->class_prim_quartets[c] = (int64_t)prim[c];
        st->quartets += stats[2 * c];
        st->prim_quartets += (int64_t)prim[c];
        st->class_l[c][0] = ctx->launch[c].la;
        st->class_l[c][1] = ctx->launch[c].lb;
        st->class_l[c][2] = ctx->launch[c].lc;
        st->class_l[c][3] = ctx->launch[c].ld;
        flops += (double)prim[c] * QB_CLASS_PRIM_FLOPS[c] + (double)stats[2 * c] * QB_CLASS_CONTR_FLOPS[c];
    }
    st->flops = flops;
    return QB_OK;
}

int qb_jk_pair_table(qb_ctx* ctx, int* npair, int* fa, int* fb, int* la, int* lb, double* Q) {
    QB_TRY(enter(ctx));
    if (!npair) return qb_set_error(ctx, QB_ERR_ARG, "null npair");
    if (!ctx->jk_prepared || !ctx->shell_path || !ctx->pairs_valid) {
        *npair = 0;
        return QB_OK;
    }
    const int n = (int)ctx->h_pairs.size();
    *npair = n;
    if (!fa && !fb && !la && !lb && !Q) return QB_OK;
    if (!fa || !fb || !la || !lb || !Q) return qb_set_error(ctx, QB_ERR_ARG, "null output array");
    int k = 0;
    for (int pc = 0; pc < ctx->npc; ++pc) {
        int a = 0;
        while ((a + 1) * (a + 2) / 2 <= pc) ++a;
        const int b = pc - a * (a + 1) / 2;
        for (; k < ctx->pc_off[pc + 1]; ++k) {
            const ShellPair& sp = ctx->h_pairs[k];
            fa[k] = sp.fa; fb[k] = sp.fb; la[k] = a; lb[k] = b; Q[k] = sp.Q;
        }
    }
    return QB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// FP64 FMA throughput: 8 independent dependency chains per thread.
__global__ void qb_dfma_peak_kernel(int iters, double seed, double* sink) {
    double a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
           a7 = a0 + 7;
    const double m = 0.999999999, c = 1e-9;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
            a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
        }
    }
    const double r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 12345.678) sink[0] = r;
}

// FP64 tensor-core (DMMA) throughput: mma.sync m8n8k4 f64 (256 FMAs per warp instruction),
// 8 independent accumulators per warp.
__global__ void qb_dmma_peak_kernel(int iters, double seed, double* sink) {
    const double a = seed + threadIdx.x * 1e-3, b = 0.999999 + threadIdx.x * 1e-9;
    double c[8][2];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        c[k][0] = k;
        c[k][1] = k + 0.5;
    }
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int k = 0; k < 8; ++k)
                asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                             : "+d"(c[k][0]), "+d"(c[k][1])
                             : "d"(a), "d"(b));
    }
    double r = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) r += c[k][0] + c[k][1];
    if (r == 12345.678) sink[0] = r;
}

extern "C" int qb_fp64_dmma_peak(qb_ctx* ctx, double* tflops) {
    QB_TRY(enter(ctx));
    if (!tflops) return qb_set_error(ctx, QB_ERR_ARG, "null output");
    DevArray<double> sink;
    QB_CUDA(ctx, sink.ensure(1));
    const int block = 256, grid = ctx->nsm * 8, iters = 1000;
    qb_dmma_peak_kernel<<<grid, block, 0, ctx->stream>>>(16, 1.0, sink.p);   // warm-up
    QB_CUDA(ctx, cudaGetLastError());
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        QB_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
        qb_dmma_peak_kernel<<<grid, block, 0, ctx->stream>>>(iters, 1.0 + rep, sink.p);
        QB_CUDA(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
        QB_CUDA(ctx, cudaEventSynchronize(ctx->ev_stop));
        float ms = 0.f;
        QB_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
        if (ms < best) best = ms;
    }
    const double flops = 512.0 * 4.0 * 8.0 * (double)iters * (double)(block / 32) * (double)grid;
    *tflops = flops / (best * 1e-3) / 1e12;
    sink.release();
    return QB_OK;
}

extern "C" int qb_fp64_peak(qb_ctx* ctx, double* tflops) {
    QB_TRY(enter(ctx));
    if (!tflops) return qb_set_error(ctx, QB_ERR_ARG, "null output");
    DevArray<double> sink;
    QB_CUDA(ctx, sink.ensure(1));
    const int block = 256, grid = ctx->nsm * 8, iters = 2048;
    qb_dfma_peak_kernel<<<grid, block, 0, ctx->stream>>>(16, 1.0, sink.p);   // warm-up
    QB_CUDA(ctx, cudaGetLastError());
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        QB_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
        qb_dfma_peak_kernel<<<grid, block, 0, ctx->stream>>>(iters, 1.0 + rep, sink.p);
        QB_CUDA(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
        QB_CUDA(ctx, cudaEventSynchronize(ctx->ev_stop));
        float ms = 0.f;
        QB_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
        if (ms < best) best = ms;
    }
    const double flops = 2.0 * 8.0 * 16.0 * (double)iters * (double)block * (double)grid;
    *tflops = flops / (best * 1e-3) / 1e12;
    sink.release();
    return QB_OK;
}
