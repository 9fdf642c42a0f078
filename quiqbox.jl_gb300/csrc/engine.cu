// Integral engine: basis upload, shell detection, shell pairs, Schwarz screening,
// class work lists and the fused ERI + J/K build.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>
#include "qb_internal.h"

int qb_set_error(qb_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int qb_cuda_check(qb_ctx* ctx, cudaError_t e, const char* where) {
    if (e == cudaSuccess) return QB_OK;
    const int code = (e == cudaErrorMemoryAllocation) ? QB_ERR_NOMEM : QB_ERR_CUDA;
    return qb_set_error(ctx, code, std::string(where) + ": " + cudaGetErrorString(e));
}

#define QB_TRY(expr)                                  \
    do {                                              \
        const int _rc = (expr);                       \
        if (_rc != QB_OK) return _rc;                 \
    } while (0)
#define QB_CUDA(ctx, call) QB_TRY(qb_cuda_check((ctx), (call), #call))

// ---------------------------------------------------------------------------
// Boys table: F_m(T_k), T_k = k/16, by the power series
//   F_m(T) = e^{-T} sum_i (2T)^i / ((2m+1)(2m+3)...(2m+2i+1))
// in extended precision, then stored as the Taylor coefficients of qb_common.cuh,
// followed by e^{-T_k}.  Writes QB_BOYS_TABLE_SIZE doubles; allocates nothing.
void qb_fill_boys_table(double* tab) {
    const int NM = QB_BOYS_NM, NJ = QB_BOYS_NJ, MT = NM + NJ - 1;
    long double F[QB_BOYS_NM + QB_BOYS_NJ];
    long double fact[QB_BOYS_NJ];
    fact[0] = 1.0L;
    for (int j = 1; j < NJ; ++j) fact[j] = fact[j - 1] * j;
    for (int k = 0; k < QB_BOYS_NROW; ++k) {
        const long double T = (long double)k / 16.0L;
        // top order by the series, then downward recursion (stable)
        long double term = 1.0L / (2 * MT + 1), sum = term;
        for (int i = 1; i < 100000; ++i) {
            term *= 2.0L * T / (2 * MT + 2 * i + 1);
            sum += term;
            if (term < sum * 1e-30L) break;
        }
        const long double ex = expl(-T);
        F[MT] = ex * sum;
        for (int m = MT; m > 0; --m) F[m - 1] = (2.0L * T * F[m] + ex) / (2 * m - 1);
        for (int m = 0; m < NM; ++m)
            for (int j = 0; j < NJ; ++j) {
                const long double c = F[m + j] / fact[j] * ((j & 1) ? -1.0L : 1.0L);
                tab[((size_t)k * NM + m) * NJ + j] = (double)c;
            }
        tab[QB_BOYS_EXP_OFF + k] = (double)ex;
    }
}

std::vector<double> qb_build_boys_table() {
    std::vector<double> tab(QB_BOYS_TABLE_SIZE);
    qb_fill_boys_table(tab.data());
    return tab;
}

// ---------------------------------------------------------------------------
static bool same_vec(const std::vector<double>& a, const double* b, size_t n) {
    return a.size() == n && (n == 0 || std::memcmp(a.data(), b, n * sizeof(double)) == 0);
}
static bool same_vec(const std::vector<int>& a, const int* b, size_t n) {
    return a.size() == n && (n == 0 || std::memcmp(a.data(), b, n * sizeof(int)) == 0);
}

static std::vector<std::array<int, 3>> cart_components(int L) {
    std::vector<std::array<int, 3>> out;
    for (int i = L; i >= 0; --i)
        for (int j = L - i; j >= 0; --j) out.push_back({i, j, L - i - j});
    return out;
}

// Groups the consecutive functions [f_begin, f_end) into Cartesian shells: same centre,
// exponents and primitive count, powers in SubshellXYZs order (src/Lexicons.jl:17-36),
// and weights that factor as ratio(function) * coefficient(primitive).  Appends the
// shells and writes ratio[f]; returns false (shells/ratios partially written) if the
// functions are not shell-structured or L > QB_LMAX_SHELL.
bool qb_detect_shells(int f_begin, int f_end, const int* fp, const double* cen, const int* ijk, const double* al,
                      const double* w, std::vector<HostShell>& shells, double* ratio) {
    int f = f_begin;
    while (f < f_end) {
        const int p0 = fp[f], K = fp[f + 1] - fp[f];
        bool ok = K > 0;
        int L = ok ? ijk[3 * p0] + ijk[3 * p0 + 1] + ijk[3 * p0 + 2] : -1;
        ok = ok && L <= QB_LMAX_SHELL;
        std::vector<std::array<int, 3>> comps;
        if (ok) comps = cart_components(L);
        const int nc = ok ? (int)comps.size() : 0;
        ok = ok && f + nc <= f_end;
        for (int c = 0; ok && c < nc; ++c) {
            const int g = f + c, q0 = fp[g];
            if (fp[g + 1] - q0 != K) { ok = false; break; }
            const double r = w[p0] != 0.0 ? w[q0] / w[p0] : 0.0;
            if (w[p0] == 0.0) { ok = false; break; }
            for (int k = 0; k < K && ok; ++k) {
                const int pa = p0 + k, pb = q0 + k;
                if (al[pa] != al[pb]) ok = false;
                for (int x = 0; x < 3; ++x) {
                    if (cen[3 * pb + x] != cen[3 * p0 + x]) ok = false;
                    if (ijk[3 * pb + x] != comps[c][x]) ok = false;
                }
                if (w[pa] == 0.0 || std::fabs(w[pb] - r * w[pa]) > 1e-13 * std::fabs(w[pb])) ok = false;
            }
            if (ok) ratio[g] = r;
        }
        if (!ok) return false;
        HostShell s;
        for (int x = 0; x < 3; ++x) s.c[x] = cen[3 * p0 + x];
        s.L = L;
        s.K = K;
        s.prim0 = p0;
        s.f0 = f;
        shells.push_back(s);
        f += nc;
    }
    return true;
}

static void detect_shells(qb_ctx* ctx) {
    ctx->shells.clear();
    ctx->h_ratio.assign(ctx->nfun, 1.0);
    ctx->shell_path = qb_detect_shells(0, ctx->nfun, ctx->h_fp.data(), ctx->h_cen.data(), ctx->h_ijk.data(),
                                       ctx->h_alpha.data(), ctx->h_w.data(), ctx->shells, ctx->h_ratio.data());
    if (!ctx->shell_path) {
        ctx->shells.clear();
        ctx->h_ratio.assign(ctx->nfun, 1.0);
    }
}

int qb_set_basis(qb_ctx* ctx, const qb_basis* b) {
    if (!ctx || !b || !b->fun_ptr) return qb_set_error(ctx, QB_ERR_ARG, "null basis");
    if (b->nfun <= 0) return qb_set_error(ctx, QB_ERR_DIM, "basis has no functions");
    const int nf = b->nfun;
    if (b->fun_ptr[0] != 0) return qb_set_error(ctx, QB_ERR_ARG, "fun_ptr[0] must be 0");
    for (int f = 0; f < nf; ++f)
        if (b->fun_ptr[f + 1] <= b->fun_ptr[f])
            return qb_set_error(ctx, QB_ERR_ARG, "every function needs at least one primitive");
    const int np = b->fun_ptr[nf];
    if (!b->center || !b->ijk || !b->alpha || !b->weight) return qb_set_error(ctx, QB_ERR_ARG, "null basis array");
    if (ctx->basis_valid && ctx->nfun == nf && same_vec(ctx->h_fp, b->fun_ptr, nf + 1) &&
        same_vec(ctx->h_cen, b->center, 3 * (size_t)np) && same_vec(ctx->h_ijk, b->ijk, 3 * (size_t)np) &&
        same_vec(ctx->h_alpha, b->alpha, np) && same_vec(ctx->h_w, b->weight, np))
        return QB_OK;
    for (int p = 0; p < np; ++p) {
        if (!(b->alpha[p] > 0.0) || !std::isfinite(b->alpha[p]) || !std::isfinite(b->weight[p]))
            return qb_set_error(ctx, QB_ERR_DOMAIN, "exponents must be positive and finite");
        int L = 0;
        for (int x = 0; x < 3; ++x) {
            if (b->ijk[3 * p + x] < 0) return qb_set_error(ctx, QB_ERR_DOMAIN, "negative Cartesian power");
            if (!std::isfinite(b->center[3 * p + x])) return qb_set_error(ctx, QB_ERR_DOMAIN, "non-finite centre");
            L += b->ijk[3 * p + x];
        }
        if (L > 12) return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "primitive angular momentum above 12");
    }
    ctx->basis_valid = false;
    ctx->pairs_valid = false;
    ctx->jk_prepared = false;
    for (int c = 0; c < QB_MAX_CLASS; ++c) ctx->class_ms[c] = 0.f;   // timings belong to the old basis
    ctx->nfun = nf;
    ctx->nprim = np;
    ctx->h_fp.assign(b->fun_ptr, b->fun_ptr + nf + 1);
    ctx->h_cen.assign(b->center, b->center + 3 * (size_t)np);
    ctx->h_ijk.assign(b->ijk, b->ijk + 3 * (size_t)np);
    ctx->h_alpha.assign(b->alpha, b->alpha + np);
    ctx->h_w.assign(b->weight, b->weight + np);
    QB_CUDA(ctx, ctx->d_fp.ensure(nf + 1));
    QB_CUDA(ctx, ctx->d_cen.ensure(3 * (size_t)np));
    QB_CUDA(ctx, ctx->d_ijk.ensure(3 * (size_t)np));
    QB_CUDA(ctx, ctx->d_alpha.ensure(np));
    QB_CUDA(ctx, ctx->d_w.ensure(np));
    cudaStream_t s = ctx->stream;
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_fp.p, b->fun_ptr, (nf + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_cen.p, b->center, 3 * np * sizeof(double), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_ijk.p, b->ijk, 3 * np * sizeof(int), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_alpha.p, b->alpha, np * sizeof(double), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_w.p, b->weight, np * sizeof(double), cudaMemcpyHostToDevice, s));
    detect_shells(ctx);
    QB_CUDA(ctx, ctx->d_ratio.ensure(nf));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_ratio.p, ctx->h_ratio.data(), nf * sizeof(double), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaStreamSynchronize(s));
    ctx->basis_valid = true;
    return QB_OK;
}

GenDevBasis qb_gen_basis(qb_ctx* ctx) {
    return GenDevBasis{ctx->d_fp.p, ctx->d_cen.p, ctx->d_ijk.p, ctx->d_alpha.p, ctx->d_w.p, ctx->nfun};
}

int qb_check_status(qb_ctx* ctx) {
    int st = 0;
    QB_CUDA(ctx, cudaMemcpyAsync(&st, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (st != 0) {
        cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream);
        return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "a kernel met an index beyond its limits (status " +
                                                         std::to_string(st) + ")");
    }
    return QB_OK;
}

// ---------------------------------------------------------------------------
// Shell pairs and primitive pairs.

__global__ void qb_primpair_kernel(const PairSlot* __restrict__ slots, int n, const double* __restrict__ cen,
                                   const double* __restrict__ alpha, const double* __restrict__ w,
                                   PrimPair* __restrict__ out, unsigned long long* __restrict__ kmax) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const PairSlot s = slots[k];
    const double a = alpha[s.pa], b = alpha[s.pb];
    const double* A = cen + 3 * s.pa;
    const double* B = cen + 3 * s.pb;
    const double p = a + b, ip = 1.0 / p;
    PrimPair r;
    r.p = p;
    r.Px = (a * A[0] + b * B[0]) * ip;
    r.Py = (a * A[1] + b * B[1]) * ip;
    r.Pz = (a * A[2] + b * B[2]) * ip;
    r.PAx = r.Px - A[0];
    r.PAy = r.Py - A[1];
    r.PAz = r.Pz - A[2];
    const double dx = A[0] - B[0], dy = A[1] - B[1], dz = A[2] - B[2];
    const double ab2 = dx * dx + dy * dy + dz * dz;
    // sqrt(2 pi^(5/2)) = sqrt(2) pi^(5/4)
    const double c0 = 5.9149671727956128778;
    r.K = c0 * w[s.pa] * w[s.pb] * exp(-a * b * ip * ab2) * ip;
    r.oo2p = 0.5 * ip;
    float* kf = reinterpret_cast<float*>(&r.pad);
    kf[0] = (float)fabs(r.K);
    kf[1] = 0.0f;
    out[k] = r;
    atomicMax(kmax, (unsigned long long)__double_as_longlong(fabs(r.K)));
}

// Per shell pair: sort its primitive pairs by descending |K| and drop those with
// |K| * max|K| < QB_PRIM_EPS (negligible against every partner); writes the kept count.
__global__ void qb_primpair_compact_kernel(const ShellPair* __restrict__ pairs, int npair, PrimPair* prims,
                                           const unsigned long long* __restrict__ kmax_bits, int* __restrict__ nkept) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npair) return;
    const ShellPair sp = pairs[k];
    const double kmax = __longlong_as_double((long long)*kmax_bits);
    PrimPair* pp = prims + sp.prim0;
    // insertion sort by |K| (at most a few dozen entries)
    for (int i = 1; i < sp.nprim; ++i) {
        const PrimPair x = pp[i];
        int j = i - 1;
        while (j >= 0 && fabs(pp[j].K) < fabs(x.K)) {
            pp[j + 1] = pp[j];
            --j;
        }
        pp[j + 1] = x;
    }
    int kept = 0;
    while (kept < sp.nprim && fabs(pp[kept].K) * kmax >= QB_PRIM_EPS) ++kept;
    nkept[k] = kept;
}

// Per shell pair: sort its kept primitive pairs by descending screening key (the pad
// float, here the primitive Schwarz factor) and keep those with key * max key >= eps
// (negligible against every partner); writes the kept count.
__global__ void qb_primpair_key_compact_kernel(const ShellPair* __restrict__ pairs, int npair, PrimPair* prims,
                                               const unsigned* __restrict__ keymax_bits, float eps,
                                               int* __restrict__ nkept) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npair) return;
    const ShellPair sp = pairs[k];
    const float kmax = __uint_as_float(*keymax_bits);
    PrimPair* pp = prims + sp.prim0;
    auto key = [](const PrimPair& x) { return reinterpret_cast<const float*>(&x.pad)[0]; };
    for (int i = 1; i < sp.nprim; ++i) {
        const PrimPair x = pp[i];
        int j = i - 1;
        while (j >= 0 && key(pp[j]) < key(x)) {
            pp[j + 1] = pp[j];
            --j;
        }
        pp[j + 1] = x;
    }
    int kept = 0;
    while (kept < sp.nprim && key(pp[kept]) * kmax >= eps) ++kept;
    nkept[k] = kept;
}

// FP32 copy (p, P) of every primitive pair, read by the warp-cooperative class kernels
// to group primitive quartets by Boys-function branch.
__global__ void qb_primpair_f32_kernel(const PrimPair* __restrict__ prims, int n, float4* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const PrimPair& r = prims[k];
    out[k] = make_float4((float)r.p, (float)r.Px, (float)r.Py, (float)r.Pz);
}

// After the primitive Schwarz keys are in place (qb_prim_key_kernel per pair class, their
// maximum in *d_keymax): sort and compact every shell pair's primitive pairs by key (nkept)
// and refresh the FP32 centres in the new order.
int qb_compact_prim_keys(cudaStream_t s, const ShellPair* d_pairs, int npair, PrimPair* d_prims, float4* d_prims32,
                         int nslot, const unsigned* d_keymax, float eps, int* d_nkept) {
    if (npair > 0)
        qb_primpair_key_compact_kernel<<<(npair + 127) / 128, 128, 0, s>>>(d_pairs, npair, d_prims, d_keymax, eps,
                                                                            d_nkept);
    if (nslot > 0) qb_primpair_f32_kernel<<<(nslot + 127) / 128, 128, 0, s>>>(d_prims, nslot, d_prims32);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Primitive pairs of every slot, sorted and compacted per shell pair (nkept), plus their
// FP32 centres.  d_kmax is scratch (one word).
int qb_build_prim_pairs(cudaStream_t s, const PairSlot* d_slots, int nslot, const double* d_cen,
                        const double* d_alpha, const double* d_w, const ShellPair* d_pairs, int npair,
                        PrimPair* d_prims, float4* d_prims32, int* d_nkept, unsigned long long* d_kmax) {
    if (cudaMemsetAsync(d_kmax, 0, sizeof(unsigned long long), s) != cudaSuccess) return -1;
    if (nslot > 0)
        qb_primpair_kernel<<<(nslot + 127) / 128, 128, 0, s>>>(d_slots, nslot, d_cen, d_alpha, d_w, d_prims, d_kmax);
    if (npair > 0)
        qb_primpair_compact_kernel<<<(npair + 127) / 128, 128, 0, s>>>(d_pairs, npair, d_prims, d_kmax, d_nkept);
    if (nslot > 0) qb_primpair_f32_kernel<<<(nslot + 127) / 128, 128, 0, s>>>(d_prims, nslot, d_prims32);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

static int pc_index(int la, int lb) { return la * (la + 1) / 2 + lb; }

int qb_ensure_pairs(qb_ctx* ctx) {
    if (ctx->pairs_valid) return QB_OK;
    if (!ctx->shell_path) return qb_set_error(ctx, QB_ERR_ARG, "basis is not shell-structured");
    const int ns = (int)ctx->shells.size();
    const int npc = (QB_LMAX_SHELL + 1) * (QB_LMAX_SHELL + 2) / 2;
    ctx->npc = npc;
    // pairs grouped by pair class, A = shell of higher L
    std::vector<std::vector<ShellPair>> by(npc);
    std::vector<std::vector<PairSlot>> slots_by(npc);
    for (int a = 0; a < ns; ++a)
        for (int b = 0; b <= a; ++b) {
            const HostShell* A = &ctx->shells[a];
            const HostShell* B = &ctx->shells[b];
            if (B->L > A->L) std::swap(A, B);
            const int pc = pc_index(A->L, B->L);
            ShellPair sp;
            sp.fa = A->f0;
            sp.fb = B->f0;
            sp.nprim = A->K * B->K;
            sp.prim0 = 0;   // set after layout
            sp.ABx = A->c[0] - B->c[0];
            sp.ABy = A->c[1] - B->c[1];
            sp.ABz = A->c[2] - B->c[2];
            sp.Q = 0.0;
            sp.same = (a == b);
            sp.pad = (int)slots_by[pc].size();   // local slot offset, replaced below
            for (int i = 0; i < A->K; ++i)
                for (int j = 0; j < B->K; ++j)
                    slots_by[pc].push_back(PairSlot{a, b, A->prim0 + i, B->prim0 + j});
            by[pc].push_back(sp);
        }
    std::vector<ShellPair> pairs;
    std::vector<PairSlot> slots;
    for (int pc = 0; pc < npc; ++pc) {
        ctx->pc_off[pc] = (int)pairs.size();
        const int base = (int)slots.size();
        for (auto sp : by[pc]) {
            sp.prim0 = base + sp.pad;
            sp.pad = 0;
            pairs.push_back(sp);
        }
        slots.insert(slots.end(), slots_by[pc].begin(), slots_by[pc].end());
    }
    ctx->pc_off[npc] = (int)pairs.size();
    const int npair = (int)pairs.size(), nslot = (int)slots.size();
    cudaStream_t s = ctx->stream;
    DevArray<PairSlot> d_slots;
    QB_CUDA(ctx, d_slots.ensure(nslot));
    QB_CUDA(ctx, ctx->d_prims.ensure(nslot));
    QB_CUDA(ctx, ctx->d_pairs.ensure(npair));
    QB_CUDA(ctx, ctx->d_Q.ensure(npair));
    QB_CUDA(ctx, cudaMemcpyAsync(d_slots.p, slots.data(), nslot * sizeof(PairSlot), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_pairs.p, pairs.data(), npair * sizeof(ShellPair), cudaMemcpyHostToDevice, s));
    DevArray<unsigned long long> d_kmax;
    DevArray<int> d_nkept;
    QB_CUDA(ctx, d_kmax.ensure(1));
    QB_CUDA(ctx, d_nkept.ensure(npair));
    QB_CUDA(ctx, ctx->d_prims32.ensure(nslot));
    if (qb_build_prim_pairs(s, d_slots.p, nslot, ctx->d_cen.p, ctx->d_alpha.p, ctx->d_w.p, ctx->d_pairs.p, npair,
                            ctx->d_prims.p, ctx->d_prims32.p, d_nkept.p, d_kmax.p) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "primitive pairs");
    {
        std::vector<int> nkept(npair);
        QB_CUDA(ctx, cudaMemcpyAsync(nkept.data(), d_nkept.p, npair * sizeof(int), cudaMemcpyDeviceToHost, s));
        QB_CUDA(ctx, cudaStreamSynchronize(s));
        for (int k = 0; k < npair; ++k) pairs[k].nprim = nkept[k];
        QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_pairs.p, pairs.data(), npair * sizeof(ShellPair), cudaMemcpyHostToDevice, s));
    }
    // Schwarz factors from the diagonal classes' own quartet code
    for (int pc = 0; pc < npc; ++pc) {
        int la = 0;
        while ((la + 1) * (la + 2) / 2 <= pc) ++la;
        const int lb = pc - la * (la + 1) / 2;
        const int n = ctx->pc_off[pc + 1] - ctx->pc_off[pc];
        if (n == 0) continue;
        QbSchwarzLaunch launch = nullptr;
        for (int c = 0; c < QB_NCLASS; ++c) {
            const ClassLaunchers& L = ctx->launch[c];
            if (L.la == la && L.lb == lb && L.lc == la && L.ld == lb) launch = L.schwarz;
        }
        if (!launch) return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "no diagonal class for a pair class");
        launch(ctx->d_pairs.p + ctx->pc_off[pc], n, ctx->d_prims.p, ctx->boys.p, ctx->d_ratio.p,
               ctx->d_Q.p + ctx->pc_off[pc], s);
        QB_CUDA(ctx, cudaGetLastError());
    }
    QB_TRY(qb_check_status(ctx));
    // Primitive Schwarz keys: each kept primitive pair's screening key becomes its own
    // Schwarz factor, the pair's primitives are re-sorted by it and the ones negligible
    // against every partner dropped; the FP32 centres follow the new order.
    {
        DevArray<unsigned> d_keymax;
        QB_CUDA(ctx, d_keymax.ensure(1));
        QB_CUDA(ctx, cudaMemsetAsync(d_keymax.p, 0, sizeof(unsigned), s));
        for (int pc = 0; pc < npc; ++pc) {
            int la = 0;
            while ((la + 1) * (la + 2) / 2 <= pc) ++la;
            const int lb = pc - la * (la + 1) / 2;
            const int n = ctx->pc_off[pc + 1] - ctx->pc_off[pc];
            if (n == 0) continue;
            QbPrimKeyLaunch launch = nullptr;
            for (int c = 0; c < QB_NCLASS; ++c) {
                const ClassLaunchers& L = ctx->launch[c];
                if (L.la == la && L.lb == lb && L.lc == la && L.ld == lb) launch = L.primkey;
            }
            if (!launch) return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "no diagonal class for a pair class");
            launch(ctx->d_pairs.p + ctx->pc_off[pc], n, ctx->d_prims.p, ctx->boys.p, d_keymax.p, s);
        }
        if (qb_compact_prim_keys(s, ctx->d_pairs.p, npair, ctx->d_prims.p, ctx->d_prims32.p, nslot, d_keymax.p,
                                 ctx->prim_eps, d_nkept.p) != 0)
            return qb_cuda_check(ctx, cudaGetLastError(), "primitive Schwarz keys");
        std::vector<int> nkept(npair);
        QB_CUDA(ctx, cudaMemcpyAsync(nkept.data(), d_nkept.p, npair * sizeof(int), cudaMemcpyDeviceToHost, s));
        QB_CUDA(ctx, cudaStreamSynchronize(s));
        for (int k = 0; k < npair; ++k) pairs[k].nprim = nkept[k];
    }
    std::vector<double> Q(npair);
    QB_CUDA(ctx, cudaMemcpyAsync(Q.data(), ctx->d_Q.p, npair * sizeof(double), cudaMemcpyDeviceToHost, s));
    QB_CUDA(ctx, cudaStreamSynchronize(s));
    d_slots.release();
    // sort each pair class by descending Q
    std::vector<ShellPair> sorted(npair);
    std::vector<double> Qs(npair);
    std::vector<long long> npref;
    for (int pc = 0; pc < npc; ++pc) {
        const int o = ctx->pc_off[pc], n = ctx->pc_off[pc + 1] - o;
        std::vector<int> idx(n);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return Q[o + x] > Q[o + y]; });
        ctx->npref_off[pc] = (int)npref.size();
        long long acc = 0;
        for (int k = 0; k < n; ++k) {
            ShellPair sp = pairs[o + idx[k]];
            sp.Q = Q[o + idx[k]];
            sorted[o + k] = sp;
            Qs[o + k] = sp.Q;
            npref.push_back(acc);
            acc += sp.nprim;
        }
        npref.push_back(acc);
    }
    ctx->npref_off[npc] = (int)npref.size();
    ctx->h_pairs = sorted;
    QB_CUDA(ctx, ctx->d_npref.ensure(npref.size()));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_pairs.p, sorted.data(), npair * sizeof(ShellPair), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_Q.p, Qs.data(), npair * sizeof(double), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_npref.p, npref.data(), npref.size() * sizeof(long long),
                                 cudaMemcpyHostToDevice, s));
    // class work-list layout
    long long off = 0;
    for (int c = 0; c < ctx->nclass; ++c) {
        const ClassLaunchers& L = ctx->launch[c];
        ctx->class_bra[c] = pc_index(L.la, L.lb);
        ctx->class_ket[c] = pc_index(L.lc, L.ld);
        ctx->offs_off[c] = off;
        off += (ctx->pc_off[ctx->class_bra[c] + 1] - ctx->pc_off[ctx->class_bra[c]]) + 1;
    }
    ctx->offs_off[ctx->nclass] = off;
    QB_CUDA(ctx, ctx->d_offs.ensure(off));
    QB_CUDA(ctx, ctx->d_stats.ensure(2 * QB_MAX_CLASS));
    QB_CUDA(ctx, ctx->d_primcount.ensure(QB_MAX_CLASS));
    QB_CUDA(ctx, cudaStreamSynchronize(s));
    ctx->pairs_valid = true;
    return QB_OK;
}

// ---------------------------------------------------------------------------
struct CountPlan {
    int nclass;
    int bra_off[QB_MAX_CLASS], nbra[QB_MAX_CLASS], ket_off[QB_MAX_CLASS], nket[QB_MAX_CLASS];
    int same[QB_MAX_CLASS], npref_off[QB_MAX_CLASS];
    long long offs_off[QB_MAX_CLASS];
};

// One block per class: per bra pair the number of surviving ket pairs (binary
// search in the descending Q list), its exclusive prefix sum, and the class
// totals of shell quartets and primitive quartets.
__global__ void __launch_bounds__(1024) qb_count_kernel(const CountPlan plan, const ShellPair* __restrict__ pairs,
                                                        const double* __restrict__ Q,
                                                        const long long* __restrict__ npref,
                                                        const double* __restrict__ dmax, double thr,
                                                        long long* __restrict__ offs, long long* __restrict__ stats) {
    const int c = blockIdx.x;
    const int nb = plan.nbra[c], nk = plan.nket[c];
    const int bo = plan.bra_off[c], ko = plan.ket_off[c];
    long long* o = offs + plan.offs_off[c];
    const double dm = dmax ? *dmax : 1.0;
    const bool all = !(thr > 0.0);
    __shared__ long long wsum[32];
    __shared__ long long s_carry, s_pq;
    if (threadIdx.x == 0) { s_carry = 0; s_pq = 0; }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int base = 0; base < nb; base += blockDim.x) {
        const int i = base + threadIdx.x;
        long long cnt = 0, pq = 0;
        if (i < nb) {
            int hi = nk;
            if (!all) {
                const double qi = Q[bo + i];
                if (!(qi > 0.0) || !(dm > 0.0)) {
                    hi = 0;
                } else {
                    const double t = thr / (dm * qi);
                    int lo = 0;
                    hi = nk;
                    while (lo < hi) {   // first j with Q[j] < t
                        const int mid = (lo + hi) >> 1;
                        if (Q[ko + mid] >= t) lo = mid + 1; else hi = mid;
                    }
                    hi = lo;
                }
            }
            if (plan.same[c] && hi > i + 1) hi = i + 1;
            cnt = hi;
            pq = (long long)pairs[bo + i].nprim * npref[plan.npref_off[c] + hi];
        }
        // block-wide inclusive scan of cnt
        long long v = cnt;
        for (int d = 1; d < 32; d <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= d) v += y;
        }
        if (lane == 31) wsum[warp] = v;
        long long pqw = pq;
        for (int d = 16; d > 0; d >>= 1) pqw += __shfl_down_sync(0xffffffffu, pqw, d);
        __syncthreads();
        if (warp == 0) {
            long long x = lane < nw ? wsum[lane] : 0;
            for (int d = 1; d < 32; d <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= d) x += y;
            }
            if (lane < nw) wsum[lane] = x;
        }
        __syncthreads();
        const long long before = (warp > 0 ? wsum[warp - 1] : 0) + s_carry;
        if (i < nb) o[i] = before + v - cnt;
        if (lane == 0) atomicAdd((unsigned long long*)&s_pq, (unsigned long long)pqw);
        __syncthreads();
        if (threadIdx.x == 0) s_carry += wsum[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        o[nb] = s_carry;
        stats[2 * c] = s_carry;
        stats[2 * c + 1] = s_pq;
    }
}

int qb_jk_device(qb_ctx* ctx, const double* dD, double* dJ, double* dK, double thr, cudaStream_t s) {
    const int n = ctx->nfun;
    const size_t nn = (size_t)n * n;
    QB_CUDA(ctx, ctx->d_Dt.ensure(nn));
    QB_CUDA(ctx, ctx->d_Jp.ensure(nn));
    QB_CUDA(ctx, ctx->d_Kp.ensure(nn));
    QB_CUDA(ctx, ctx->d_dmax.ensure(1));
    QB_CUDA(ctx, cudaMemsetAsync(ctx->d_Jp.p, 0, nn * sizeof(double), s));
    QB_CUDA(ctx, cudaMemsetAsync(ctx->d_Kp.p, 0, nn * sizeof(double), s));
    QB_CUDA(ctx, cudaMemsetAsync(ctx->d_dmax.p, 0, sizeof(double), s));
    const bool shell = ctx->shell_path;
    qb_density_prescale(s, n, shell ? ctx->d_ratio.p : nullptr, dD, ctx->d_Dt.p, ctx->d_dmax.p);
    ctx->last_execute_shell = shell;
    if (!shell) {
        if (qb_gen_eri(qb_gen_basis(ctx), 1, ctx->boys.p, nullptr, ctx->d_Dt.p, ctx->d_Jp.p, ctx->d_Kp.p,
                       ctx->status.p, ctx->nsm, s) != 0)
            return qb_cuda_check(ctx, cudaGetLastError(), "generic J/K launch");
        qb_jk_finalize(s, n, nullptr, ctx->d_Jp.p, ctx->d_Kp.p, dJ, dK);
        return qb_cuda_check(ctx, cudaGetLastError(), "J/K finalize");
    }
    QB_TRY(qb_ensure_pairs(ctx));
    CountPlan plan;
    plan.nclass = ctx->nclass;
    for (int c = 0; c < ctx->nclass; ++c) {
        const int X = ctx->class_bra[c], Y = ctx->class_ket[c];
        plan.bra_off[c] = ctx->pc_off[X];
        plan.nbra[c] = ctx->pc_off[X + 1] - ctx->pc_off[X];
        plan.ket_off[c] = ctx->pc_off[Y];
        plan.nket[c] = ctx->pc_off[Y + 1] - ctx->pc_off[Y];
        plan.same[c] = (X == Y);
        plan.npref_off[c] = ctx->npref_off[Y];
        plan.offs_off[c] = ctx->offs_off[c];
    }
    qb_count_kernel<<<ctx->nclass, 1024, 0, s>>>(plan, ctx->d_pairs.p, ctx->d_Q.p, ctx->d_npref.p, ctx->d_dmax.p,
                                                  thr, ctx->d_offs.p, ctx->d_stats.p);
    QB_CUDA(ctx, cudaGetLastError());
    QB_CUDA(ctx, cudaMemsetAsync(ctx->d_primcount.p, 0, QB_MAX_CLASS * sizeof(unsigned long long), s));
    QB_CUDA(ctx, cudaEventRecord(ctx->ev_fork, s));
    for (int k2 = 0; k2 < QB_NSTREAM; ++k2) QB_CUDA(ctx, cudaStreamWaitEvent(ctx->streams[k2], ctx->ev_fork, 0));
    // Launch order and streams: the longest class kernels first (their measured times, once
    // the autotuner or the class timing has run; else by class, highest angular momentum
    // first), each on the stream with the least queued time, so that the short kernels fill
    // the GPU while the last long ones finish.
    int order[QB_MAX_CLASS];
    int ncls = 0;
    for (int c = ctx->nclass - 1; c >= 0; --c)
        if (plan.nbra[c] > 0 && plan.nket[c] > 0) order[ncls++] = c;
    std::stable_sort(order, order + ncls, [&](int a, int b) { return ctx->class_ms[a] > ctx->class_ms[b]; });
    float queued[QB_NSTREAM] = {};
    for (int k = 0; k < ncls; ++k) {
        const int c = order[k];
        ClassWork w{ctx->d_pairs.p + plan.bra_off[c], ctx->d_pairs.p + plan.ket_off[c],
                    ctx->d_offs.p + plan.offs_off[c], plan.nbra[c], plan.same[c]};
        const int grid = ctx->nsm * std::max(1, ctx->occ[c]);
        JKArgs args{ctx->d_prims.p, ctx->d_prims32.p, ctx->boys.p, ctx->d_Dt.p, ctx->d_Jp.p, ctx->d_Kp.p, ctx->d_primcount.p + c, n, ctx->prim_eps};
        int st = k % QB_NSTREAM;
        if (ctx->class_ms[c] > 0.f) {
            st = 0;
            for (int j = 1; j < QB_NSTREAM; ++j)
                if (queued[j] < queued[st]) st = j;
            queued[st] += ctx->class_ms[c];
        }
        ctx->launch[c].jk[ctx->variant[c]](w, args, grid, ctx->streams[st]);
    }
    QB_CUDA(ctx, cudaGetLastError());
    for (int j = 0; j < QB_NSTREAM; ++j) {
        QB_CUDA(ctx, cudaEventRecord(ctx->ev_join[j], ctx->streams[j]));
        QB_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_join[j], 0));
    }
    qb_jk_finalize(s, n, ctx->d_ratio.p, ctx->d_Jp.p, ctx->d_Kp.p, dJ, dK);
    return qb_cuda_check(ctx, cudaGetLastError(), "J/K finalize");
}

// J/K restricted to an explicit list of canonical shell quartets (pair indices into the
// pair table, bra pair class >= ket pair class, ket index <= bra index within one class):
// each quartet is one launch of its class's production kernel (the context's variant)
// over a one-bra, one-ket work list, accumulated into the same J'/K' and finalised as a
// full build is.  For parity tests of the class kernels on chosen quartets.
int qb_jk_quartets_device(qb_ctx* ctx, long long nq, const int* pq, double* dJ, double* dK) {
    cudaStream_t s = ctx->stream;
    const int n = ctx->nfun;
    const size_t nn = (size_t)n * n;
    if (!ctx->shell_path) return qb_set_error(ctx, QB_ERR_UNSUPPORTED, "the basis is not on the shell path");
    QB_TRY(qb_ensure_pairs(ctx));
    const int npair = ctx->pc_off[ctx->npc];
    auto pc_of = [&](int p) {
        int pc = 0;
        while (pc + 1 <= ctx->npc && ctx->pc_off[pc + 1] <= p) ++pc;
        return pc;
    };
    std::vector<int> cls(nq);
    for (long long q = 0; q < nq; ++q) {
        const int P = pq[2 * q], Q = pq[2 * q + 1];
        if (P < 0 || P >= npair || Q < 0 || Q >= npair) return qb_set_error(ctx, QB_ERR_ARG, "pair index out of range");
        const int X = pc_of(P), Y = pc_of(Q);
        int c = -1;
        for (int k = 0; k < ctx->nclass; ++k)
            if (ctx->class_bra[k] == X && ctx->class_ket[k] == Y) c = k;
        if (c < 0 || (X == Y && Q > P)) return qb_set_error(ctx, QB_ERR_ARG, "quartet not in canonical order");
        cls[q] = c;
    }
    QB_CUDA(ctx, ctx->d_Dt.ensure(nn));
    QB_CUDA(ctx, ctx->d_Jp.ensure(nn));
    QB_CUDA(ctx, ctx->d_Kp.ensure(nn));
    QB_CUDA(ctx, ctx->d_dmax.ensure(1));
    QB_CUDA(ctx, ctx->d_one_offs.ensure(2));
    const long long one[2] = {0, 1};
    QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_one_offs.p, one, sizeof(one), cudaMemcpyHostToDevice, s));
    QB_CUDA(ctx, cudaMemsetAsync(ctx->d_Jp.p, 0, nn * sizeof(double), s));
    QB_CUDA(ctx, cudaMemsetAsync(ctx->d_Kp.p, 0, nn * sizeof(double), s));
    QB_CUDA(ctx, cudaMemsetAsync(ctx->d_dmax.p, 0, sizeof(double), s));
    QB_CUDA(ctx, cudaMemsetAsync(ctx->d_primcount.p, 0, QB_MAX_CLASS * sizeof(unsigned long long), s));
    qb_density_prescale(s, n, ctx->d_ratio.p, ctx->d_D.p, ctx->d_Dt.p, ctx->d_dmax.p);
    ctx->last_execute_shell = false;   // the class statistics of qb_jk_get_stats stay those of a full build
    for (long long q = 0; q < nq; ++q) {
        const int P = pq[2 * q], Q = pq[2 * q + 1], c = cls[q];
        const ClassWork w{ctx->d_pairs.p + P, ctx->d_pairs.p + Q, ctx->d_one_offs.p, 1, P == Q ? 1 : 0};
        const JKArgs args{ctx->d_prims.p, ctx->d_prims32.p, ctx->boys.p, ctx->d_Dt.p, ctx->d_Jp.p, ctx->d_Kp.p,
                          ctx->d_primcount.p + c, n, ctx->prim_eps};
        ctx->launch[c].jk[ctx->variant[c]](w, args, 1, s);
    }
    QB_CUDA(ctx, cudaGetLastError());
    qb_jk_finalize(s, n, ctx->d_ratio.p, ctx->d_Jp.p, ctx->d_Kp.p, dJ, dK);
    return qb_cuda_check(ctx, cudaGetLastError(), "J/K finalize");
}

// Autotuner: after one J/K build on the current basis and density (work lists in place),
// time every compiled kernel variant of every class with work on the same list (CUDA events
// on the context stream, best of `repeats`) and keep the fastest per class.
int qb_jk_autotune_device(qb_ctx* ctx, int repeats, int* chosen) {
    if (!ctx->jk_prepared) return qb_set_error(ctx, QB_ERR_ARG, "call qb_jk_prepare first");
    cudaStream_t s = ctx->stream;
    QB_TRY(qb_jk_device(ctx, ctx->d_D.p, ctx->d_J.p, ctx->d_K.p, ctx->schwarz, s));
    QB_CUDA(ctx, cudaStreamSynchronize(s));
    if (!ctx->shell_path) return QB_OK;
    const int n = ctx->nfun;
    for (int c = 0; c < ctx->nclass; ++c) {
        const ClassLaunchers& L = ctx->launch[c];
        const int X = ctx->class_bra[c], Y = ctx->class_ket[c];
        const int nbra = ctx->pc_off[X + 1] - ctx->pc_off[X], nket = ctx->pc_off[Y + 1] - ctx->pc_off[Y];
        if (chosen) chosen[c] = ctx->variant[c];
        if (nbra == 0 || nket == 0) continue;
        int nvar = 0;
        for (int v = 0; v < QB_NVARIANT; ++v) nvar += L.jk[v] != nullptr;
        if (nvar < 2) continue;
        const ClassWork w{ctx->d_pairs.p + ctx->pc_off[X], ctx->d_pairs.p + ctx->pc_off[Y],
                          ctx->d_offs.p + ctx->offs_off[c], nbra, X == Y};
        const JKArgs args{ctx->d_prims.p, ctx->d_prims32.p, ctx->boys.p, ctx->d_Dt.p, ctx->d_Jp.p, ctx->d_Kp.p,
                          ctx->d_primcount.p + c, n, ctx->prim_eps};
        float best = 0.f;
        int best_v = ctx->variant[c], best_occ = ctx->occ[c];
        for (int v = 0; v < QB_NVARIANT; ++v) {
            if (!L.jk[v]) continue;
            const int occ = L.occupancy[v]();
            const int grid = ctx->nsm * std::max(1, occ);
            float t = 0.f;
            for (int r = 0; r < std::max(1, repeats); ++r) {
                QB_CUDA(ctx, cudaEventRecord(ctx->ev_start, s));
                L.jk[v](w, args, grid, s);
                QB_CUDA(ctx, cudaEventRecord(ctx->ev_stop, s));
                QB_CUDA(ctx, cudaEventSynchronize(ctx->ev_stop));
                float ms = 0.f;
                QB_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
                t = (r == 0) ? ms : std::min(t, ms);
            }
            if (best == 0.f || t < best) {
                best = t;
                best_v = v;
                best_occ = occ;
            }
        }
        ctx->variant[c] = best_v;
        ctx->occ[c] = best_occ;
        ctx->class_ms[c] = best;
        if (chosen) chosen[c] = best_v;
    }
    QB_CUDA(ctx, cudaGetLastError());
    // the timing runs accumulated into J'/K': leave the context's J and K consistent
    return qb_jk_device(ctx, ctx->d_D.p, ctx->d_J.p, ctx->d_K.p, ctx->schwarz, s);
}

// Per-class device time: every class kernel of the current work lists launched alone with
// its current variant on the context stream (CUDA events, best of `repeats`); then one
// build, so that J and K stay those of the density.
int qb_jk_class_times_device(qb_ctx* ctx, int repeats, float* ms) {
    if (!ctx->jk_prepared) return qb_set_error(ctx, QB_ERR_ARG, "call qb_jk_prepare first");
    cudaStream_t s = ctx->stream;
    QB_TRY(qb_jk_device(ctx, ctx->d_D.p, ctx->d_J.p, ctx->d_K.p, ctx->schwarz, s));
    QB_CUDA(ctx, cudaStreamSynchronize(s));
    for (int c = 0; c < ctx->nclass; ++c) ms[c] = 0.f;
    if (!ctx->shell_path) return QB_OK;
    const int n = ctx->nfun;
    for (int c = 0; c < ctx->nclass; ++c) {
        const ClassLaunchers& L = ctx->launch[c];
        const int X = ctx->class_bra[c], Y = ctx->class_ket[c];
        const int nbra = ctx->pc_off[X + 1] - ctx->pc_off[X], nket = ctx->pc_off[Y + 1] - ctx->pc_off[Y];
        if (nbra == 0 || nket == 0) continue;
        const ClassWork w{ctx->d_pairs.p + ctx->pc_off[X], ctx->d_pairs.p + ctx->pc_off[Y],
                          ctx->d_offs.p + ctx->offs_off[c], nbra, X == Y};
        const JKArgs args{ctx->d_prims.p, ctx->d_prims32.p, ctx->boys.p, ctx->d_Dt.p, ctx->d_Jp.p, ctx->d_Kp.p,
                          ctx->d_primcount.p + c, n, ctx->prim_eps};
        const int grid = ctx->nsm * std::max(1, ctx->occ[c]);
        float best = 0.f;
        for (int r = 0; r < std::max(1, repeats); ++r) {
            QB_CUDA(ctx, cudaEventRecord(ctx->ev_start, s));
            L.jk[ctx->variant[c]](w, args, grid, s);
            QB_CUDA(ctx, cudaEventRecord(ctx->ev_stop, s));
            QB_CUDA(ctx, cudaEventSynchronize(ctx->ev_stop));
            float t = 0.f;
            QB_CUDA(ctx, cudaEventElapsedTime(&t, ctx->ev_start, ctx->ev_stop));
            best = (r == 0) ? t : std::min(best, t);
        }
        ms[c] = best;
        ctx->class_ms[c] = best;
    }
    QB_CUDA(ctx, cudaGetLastError());
    return qb_jk_device(ctx, ctx->d_D.p, ctx->d_J.p, ctx->d_K.p, ctx->schwarz, s);
}

int qb_onebody_device(qb_ctx* ctx, int flags, int nnuc, const double* Z, const double* R, double* dS, double* dT,
                      double* dV) {
    cudaStream_t s = ctx->stream;
    const double* dZ = nullptr;
    const double* dR = nullptr;
    if (flags & 4) {
        if (nnuc <= 0 || !Z || !R) return qb_set_error(ctx, QB_ERR_ARG, "nuclear attraction needs nuclei");
        for (int c = 0; c < nnuc; ++c)
            if (!std::isfinite(Z[c]) || !std::isfinite(R[3 * c]) || !std::isfinite(R[3 * c + 1]) ||
                !std::isfinite(R[3 * c + 2]))
                return qb_set_error(ctx, QB_ERR_DOMAIN, "non-finite nuclear charge or position");
        QB_CUDA(ctx, ctx->d_nucZ.ensure(nnuc));
        QB_CUDA(ctx, ctx->d_nucR.ensure(3 * (size_t)nnuc));
        QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_nucZ.p, Z, nnuc * sizeof(double), cudaMemcpyHostToDevice, s));
        QB_CUDA(ctx, cudaMemcpyAsync(ctx->d_nucR.p, R, 3 * nnuc * sizeof(double), cudaMemcpyHostToDevice, s));
        dZ = ctx->d_nucZ.p;
        dR = ctx->d_nucR.p;
    }
    if (qb_gen_onebody(qb_gen_basis(ctx), flags, nnuc, dZ, dR, ctx->boys.p, dS, dT, dV, ctx->status.p, s) != 0)
        return qb_cuda_check(ctx, cudaGetLastError(), "one-body kernel");
    return QB_OK;
}
