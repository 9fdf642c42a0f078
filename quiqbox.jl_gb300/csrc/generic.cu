// Generic per-function integral kernels (any Cartesian powers per primitive).
//
// These cover every basis the reference accepts on its Gaussian path: each
// contracted function is an arbitrary list of primitives, each with its own
// centre, exponent, Cartesian powers and effective weight
// (src/Integration/Framework.jl:505-554 contracts exactly such lists).  They use
// McMurchie–Davidson Hermite expansions (J. Comput. Phys. 26, 218 (1978)):
// per-axis coefficients E^{ij}_t and Hermite Coulomb integrals R_{tuv}.  The
// shell-structured bases of the hot path go through the generated HGP class
// kernels instead (eri_kernels.cuh); these kernels serve one-electron matrices,
// the ERI tensor / J-K of non-shell bases and arbitrary angular momentum.
#include <cuda_runtime.h>
#include "qb_common.cuh"
#include "qb_internal.h"

#define GEN_LF_MAX 12          // largest Cartesian power sum of one primitive
#define GEN_E_MAX (2 * GEN_LF_MAX + 3)
#define GEN_BOX_MAX 800        // (Lx+1)(Ly+1)(Lz+1) of a quartet
#define GEN_LTOT_ERI 24        // largest total angular momentum of a quartet

struct GenBasis {
    const int* __restrict__ fp;
    const double* __restrict__ cen;
    const int* __restrict__ ijk;
    const double* __restrict__ alpha;
    const double* __restrict__ w;
    int nfun;
};

// Hermite expansion of x_A^i x_B^j about P: e[0..i+j] = E^{ij}_t (the factor
// exp(-mu X_AB^2) is applied by the caller).  Returns i+j+1.
__device__ __forceinline__ int md_expand(int i, int j, double XPA, double XPB, double oo2p, double* e) {
    e[0] = 1.0;
    int len = 1;
    for (int s = 0; s < i + j; ++s) {
        const double X = s < i ? XPA : XPB;
        e[len] = 0.0;
        double prev = 0.0;
        for (int t = 0; t <= len; ++t) {
            const double cur = e[t];
            const double nxt = (t + 1 <= len) ? e[t + 1] : 0.0;
            e[t] = oo2p * prev + X * cur + (t + 1) * nxt;
            prev = cur;
        }
        ++len;
    }
    return len;
}

// Hermite Coulomb integrals R^{(0)}_{tuv}(alpha; X,Y,Z) for t<=Lx, u<=Ly, v<=Lz, from
// F[n] = F_n(alpha R^2) scaled by the prefactor.  Result in r0 (box-indexed).
__device__ void md_hermite_R(int Lx, int Ly, int Lz, double alpha, double X, double Y, double Z,
                             const double* F, double* r0, double* r1) {
    const int nx = Lx + 1, ny = Ly + 1, nz = Lz + 1;
    const int N = Lx + Ly + Lz;
    double* cur = (N % 2 == 0) ? r0 : r1;
    double* prv = (N % 2 == 0) ? r1 : r0;
    double m2a = 1.0;
    for (int n = 0; n < N; ++n) m2a *= -2.0 * alpha;
    for (int n = N; n >= 0; --n) {
        // swap roles: level n goes into cur, level n+1 is in prv
        for (int t = 0; t < nx; ++t)
            for (int u = 0; u < ny; ++u)
                for (int v = 0; v < nz; ++v) {
                    if (t + u + v > N - n) continue;
                    const int id = (t * ny + u) * nz + v;
                    double val;
                    if (t + u + v == 0) {
                        val = m2a * F[n];
                    } else if (t > 0) {
                        val = X * prv[((t - 1) * ny + u) * nz + v];
                        if (t > 1) val += (t - 1) * prv[((t - 2) * ny + u) * nz + v];
                    } else if (u > 0) {
                        val = Y * prv[(t * ny + u - 1) * nz + v];
                        if (u > 1) val += (u - 1) * prv[(t * ny + u - 2) * nz + v];
                    } else {
                        val = Z * prv[(t * ny + u) * nz + v - 1];
                        if (v > 1) val += (v - 1) * prv[(t * ny + u) * nz + v - 2];
                    }
                    cur[id] = val;
                }
        if (n > 0) {
            m2a /= -2.0 * alpha;
            double* tmp = cur; cur = prv; prv = tmp;
        }
    }
}

__device__ __forceinline__ void tri_decode(long long n, int& i, int& j) {   // n -> (i >= j)
    long long a = (long long)((sqrt(8.0 * (double)n + 1.0) - 1.0) * 0.5);
    while (a * (a + 1) / 2 > n) --a;
    while ((a + 1) * (a + 2) / 2 <= n) ++a;
    i = (int)a;
    j = (int)(n - a * (a + 1) / 2);
}

// One-electron integrals of the function pair (fi, fj): flags 1 overlap, 2 kinetic,
// 4 nuclear attraction (nuclei Z, Rn).  Returns false (status bit set) on unsupported
// angular momentum.
__device__ bool qb_onebody_pair(const GenBasis& b, int fi, int fj, int flags, int nnuc, const double* __restrict__ Z,
                                const double* __restrict__ Rn, const double* __restrict__ boys, double& s_out,
                                double& t_out, double& v_out, int* status) {
    double s_acc = 0.0, t_acc = 0.0, v_acc = 0.0;
    double ex[GEN_E_MAX], ey[GEN_E_MAX], ez[GEN_E_MAX], F[GEN_LTOT_ERI + 1];
    double r0[GEN_BOX_MAX], r1[GEN_BOX_MAX];
    for (int pa = b.fp[fi]; pa < b.fp[fi + 1]; ++pa) {
        for (int pb = b.fp[fj]; pb < b.fp[fj + 1]; ++pb) {
            const double a = b.alpha[pa], be = b.alpha[pb];
            const double* A = b.cen + 3 * pa;
            const double* B = b.cen + 3 * pb;
            const int* la = b.ijk + 3 * pa;
            const int* lb = b.ijk + 3 * pb;
            if (la[0] + lb[0] > 2 * GEN_LF_MAX || la[1] + lb[1] > 2 * GEN_LF_MAX ||
                la[2] + lb[2] > 2 * GEN_LF_MAX) {
                atomicOr(status, QB_DEVERR_BAD_INDEX);
                return false;
            }
            const double p = a + be, oo2p = 0.5 / p, mu = a * be / p;
            double P[3], PA[3], PB[3], AB2 = 0.0;
            for (int k = 0; k < 3; ++k) {
                P[k] = (a * A[k] + be * B[k]) / p;
                PA[k] = P[k] - A[k];
                PB[k] = P[k] - B[k];
                AB2 += (A[k] - B[k]) * (A[k] - B[k]);
            }
            const double K = exp(-mu * AB2) * b.w[pa] * b.w[pb];
            const double sp = sqrt(QB_PI / p);
            if (flags & 3) {
                // 1D overlaps S_{i, j+s} for s = -2, 0, +2 on each axis (kinetic needs the shifts)
                double s1[3][3];
                for (int k = 0; k < 3; ++k) {
                    for (int s = 0; s < 3; ++s) {
                        const int jj = lb[k] + 2 * (s - 1);
                        if (jj < 0) { s1[k][s] = 0.0; continue; }
                        double e[GEN_E_MAX];
                        md_expand(la[k], jj, PA[k], PB[k], oo2p, e);
                        s1[k][s] = e[0] * sp;
                    }
                }
                const double Sx = s1[0][1], Sy = s1[1][1], Sz = s1[2][1];
                if (flags & 1) s_acc += K * Sx * Sy * Sz;
                if (flags & 2) {
                    double Tk[3];
                    for (int k = 0; k < 3; ++k) {
                        const int j = lb[k];
                        Tk[k] = -0.5 * (j * (j - 1) * s1[k][0] - 2.0 * be * (2 * j + 1) * s1[k][1] +
                                        4.0 * be * be * s1[k][2]);
                    }
                    t_acc += K * (Tk[0] * Sy * Sz + Sx * Tk[1] * Sz + Sx * Sy * Tk[2]);
                }
            }
            if (flags & 4) {
                const int nx = md_expand(la[0], lb[0], PA[0], PB[0], oo2p, ex);
                const int ny = md_expand(la[1], lb[1], PA[1], PB[1], oo2p, ey);
                const int nz = md_expand(la[2], lb[2], PA[2], PB[2], oo2p, ez);
                const int Lt = nx + ny + nz - 3;
                if (nx * ny * nz > GEN_BOX_MAX || Lt > GEN_LTOT_ERI) {
                    atomicOr(status, QB_DEVERR_BAD_INDEX);
                    return false;
                }
                double vsum = 0.0;
                for (int c = 0; c < nnuc; ++c) {
                    const double PC[3] = {P[0] - Rn[3 * c], P[1] - Rn[3 * c + 1], P[2] - Rn[3 * c + 2]};
                    const double R2 = PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2];
                    qb_boys_scaled_rt(p * R2, 1.0, boys, Lt, F);
                    md_hermite_R(nx - 1, ny - 1, nz - 1, p, PC[0], PC[1], PC[2], F, r0, r1);
                    double acc = 0.0;
                    for (int t = 0; t < nx; ++t)
                        for (int u = 0; u < ny; ++u) {
                            const double eu = ex[t] * ey[u];
                            for (int v = 0; v < nz; ++v) acc += eu * ez[v] * r0[(t * ny + u) * nz + v];
                        }
                    vsum += Z[c] * acc;
                }
                v_acc -= K * (2.0 * QB_PI / p) * vsum;
            }
        }
    }
    s_out = s_acc;
    t_out = t_acc;
    v_out = v_acc;
    return true;
}

// One-electron matrices: one thread per function pair i >= j.
// flags: 1 overlap, 2 kinetic, 4 nuclear attraction.  Outputs column-major, both triangles.
__global__ void qb_onebody_kernel(const GenBasis b, int flags, int nnuc, const double* __restrict__ Z,
                                  const double* __restrict__ Rn, const double* __restrict__ boys,
                                  double* S, double* T, double* V, int* status) {
    const long long npair = (long long)b.nfun * (b.nfun + 1) / 2;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npair) return;
    int fi, fj;
    tri_decode(n, fi, fj);
    double s_acc, t_acc, v_acc;
    if (!qb_onebody_pair(b, fi, fj, flags, nnuc, Z, Rn, boys, s_acc, t_acc, v_acc, status)) return;
    const size_t N = b.nfun;
    if (flags & 1) { S[fi + N * fj] = s_acc; S[fj + N * fi] = s_acc; }
    if (flags & 2) { T[fi + N * fj] = t_acc; T[fj + N * fi] = t_acc; }
    if (flags & 4) { V[fi + N * fj] = v_acc; V[fj + N * fi] = v_acc; }
}

// Batched overlap and core Hamiltonian of many molecules whose bases are concatenated
// in b: molecule m owns functions [fo[m], fo[m] + nf[m]), nuclei [nuc0[m], nuc0[m+1]),
// its function pairs are [poff[m], poff[m+1]) of the global pair index, and its
// matrices start at S + mo[m], H + mo[m] (nf[m] x nf[m], column-major).
__global__ void qb_onebody_batch_kernel(const GenBasis b, int nmol, const long long* __restrict__ poff,
                                        const int* __restrict__ fo, const int* __restrict__ nf,
                                        const long long* __restrict__ mo, const int* __restrict__ nuc0,
                                        const double* __restrict__ Z, const double* __restrict__ Rn,
                                        const double* __restrict__ boys, double* S, double* H, int* status) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= poff[nmol]) return;
    int lo = 0, hi = nmol;   // poff[lo] <= g < poff[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (poff[mid] <= g) lo = mid; else hi = mid;
    }
    const int m = lo;
    int i, j;
    tri_decode(g - poff[m], i, j);
    double s, t, v;
    const int c0 = nuc0[m];
    if (!qb_onebody_pair(b, fo[m] + i, fo[m] + j, 7, nuc0[m + 1] - c0, Z + c0, Rn + 3 * c0, boys, s, t, v, status))
        return;
    const size_t n = nf[m];
    double* Sm = S + mo[m];
    double* Hm = H + mo[m];
    Sm[i + n * j] = s;
    Sm[j + n * i] = s;
    Hm[i + n * j] = t + v;
    Hm[j + n * i] = t + v;
}

// Multipole-moment matrix M_ij = <i| prod_k (x_k - C_k)^{n_k} |j>: one thread per function
// pair i >= j.  Per axis, (x - C)^n = sum_q binom(n, q) (B - C)^q (x - B)^{n-q} raises the
// right primitive's power, and each term is a 1D overlap E^{i, j+n-q}_0 sqrt(pi/p).
__global__ void qb_multipole_kernel(const GenBasis b, double Cx, double Cy, double Cz, int nx, int ny, int nz,
                                    double* __restrict__ M, int* status) {
    const long long npair = (long long)b.nfun * (b.nfun + 1) / 2;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npair) return;
    int fi, fj;
    tri_decode(n, fi, fj);
    const double C[3] = {Cx, Cy, Cz};
    const int deg[3] = {nx, ny, nz};
    double acc = 0.0;
    double e[GEN_E_MAX];
    for (int pa = b.fp[fi]; pa < b.fp[fi + 1]; ++pa) {
        for (int pb = b.fp[fj]; pb < b.fp[fj + 1]; ++pb) {
            const double a = b.alpha[pa], be = b.alpha[pb];
            const double* A = b.cen + 3 * pa;
            const double* B = b.cen + 3 * pb;
            const int* la = b.ijk + 3 * pa;
            const int* lb = b.ijk + 3 * pb;
            const double p = a + be, oo2p = 0.5 / p, mu = a * be / p;
            const double sp = sqrt(QB_PI / p);
            double AB2 = 0.0, prod = 1.0;
            for (int k = 0; k < 3; ++k) {
                const double Pk = (a * A[k] + be * B[k]) / p;
                AB2 += (A[k] - B[k]) * (A[k] - B[k]);
                if (la[k] + lb[k] + deg[k] > GEN_E_MAX - 1) {
                    atomicOr(status, QB_DEVERR_BAD_INDEX);
                    return;
                }
                const double BC = B[k] - C[k];
                double sum = 0.0, pw = 1.0, binom = 1.0;
                for (int q = 0; q <= deg[k]; ++q) {
                    md_expand(la[k], lb[k] + deg[k] - q, Pk - A[k], Pk - B[k], oo2p, e);
                    sum += binom * pw * e[0];
                    pw *= BC;
                    binom = binom * (deg[k] - q) / (q + 1);
                }
                prod *= sum * sp;
            }
            acc += exp(-mu * AB2) * b.w[pa] * b.w[pb] * prod;
        }
    }
    const size_t N = b.nfun;
    M[fi + N * fj] = acc;
    M[fj + N * fi] = acc;
}

// Contracted ERI (ij|kl) of four functions by McMurchie–Davidson.
__device__ double md_eri(const GenBasis& b, int fi, int fj, int fk, int fl, const double* __restrict__ boys,
                         int* status) {
    double ebx[GEN_E_MAX], eby[GEN_E_MAX], ebz[GEN_E_MAX];
    double ekx[GEN_E_MAX], eky[GEN_E_MAX], ekz[GEN_E_MAX];
    double F[GEN_LTOT_ERI + 1], r0[GEN_BOX_MAX], r1[GEN_BOX_MAX];
    double res = 0.0;
    for (int pa = b.fp[fi]; pa < b.fp[fi + 1]; ++pa)
        for (int pb = b.fp[fj]; pb < b.fp[fj + 1]; ++pb) {
            const double a = b.alpha[pa], be = b.alpha[pb];
            const double* A = b.cen + 3 * pa;
            const double* B = b.cen + 3 * pb;
            const int* la = b.ijk + 3 * pa;
            const int* lb = b.ijk + 3 * pb;
            const double p = a + be, oo2p = 0.5 / p, mu = a * be / p;
            double P[3], AB2 = 0.0;
            for (int k = 0; k < 3; ++k) {
                P[k] = (a * A[k] + be * B[k]) / p;
                AB2 += (A[k] - B[k]) * (A[k] - B[k]);
            }
            const double Kab = exp(-mu * AB2) * b.w[pa] * b.w[pb] / p;
            if (Kab == 0.0) continue;
            const int bx = md_expand(la[0], lb[0], P[0] - A[0], P[0] - B[0], oo2p, ebx);
            const int by = md_expand(la[1], lb[1], P[1] - A[1], P[1] - B[1], oo2p, eby);
            const int bz = md_expand(la[2], lb[2], P[2] - A[2], P[2] - B[2], oo2p, ebz);
            for (int pc = b.fp[fk]; pc < b.fp[fk + 1]; ++pc)
                for (int pd = b.fp[fl]; pd < b.fp[fl + 1]; ++pd) {
                    const double c = b.alpha[pc], de = b.alpha[pd];
                    const double* Cc = b.cen + 3 * pc;
                    const double* Dd = b.cen + 3 * pd;
                    const int* lc = b.ijk + 3 * pc;
                    const int* ld = b.ijk + 3 * pd;
                    const double q = c + de, oo2q = 0.5 / q, nu = c * de / q;
                    double Q[3], CD2 = 0.0;
                    for (int k = 0; k < 3; ++k) {
                        Q[k] = (c * Cc[k] + de * Dd[k]) / q;
                        CD2 += (Cc[k] - Dd[k]) * (Cc[k] - Dd[k]);
                    }
                    const double Kcd = exp(-nu * CD2) * b.w[pc] * b.w[pd] / q;
                    if (Kcd == 0.0) continue;
                    const int kx = md_expand(lc[0], ld[0], Q[0] - Cc[0], Q[0] - Dd[0], oo2q, ekx);
                    const int ky = md_expand(lc[1], ld[1], Q[1] - Cc[1], Q[1] - Dd[1], oo2q, eky);
                    const int kz = md_expand(lc[2], ld[2], Q[2] - Cc[2], Q[2] - Dd[2], oo2q, ekz);
                    const int Lx = bx + kx - 2, Ly = by + ky - 2, Lz = bz + kz - 2;
                    if ((Lx + 1) * (Ly + 1) * (Lz + 1) > GEN_BOX_MAX || Lx + Ly + Lz > GEN_LTOT_ERI) {
                        atomicOr(status, QB_DEVERR_BAD_INDEX);
                        return 0.0;
                    }
                    const double rho = p * q / (p + q);
                    const double PQ[3] = {P[0] - Q[0], P[1] - Q[1], P[2] - Q[2]};
                    const double R2 = PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2];
                    const double pre = 2.0 * pow(QB_PI, 2.5) / sqrt(p + q) * Kab * Kcd;
                    qb_boys_scaled_rt(rho * R2, pre, boys, Lx + Ly + Lz, F);
                    md_hermite_R(Lx, Ly, Lz, rho, PQ[0], PQ[1], PQ[2], F, r0, r1);
                    const int ny = Ly + 1, nz = Lz + 1;
                    double acc = 0.0;
                    for (int t = 0; t < bx; ++t)
                        for (int u = 0; u < by; ++u)
                            for (int v = 0; v < bz; ++v) {
                                const double eb = ebx[t] * eby[u] * ebz[v];
                                double inner = 0.0;
                                for (int tt = 0; tt < kx; ++tt)
                                    for (int uu = 0; uu < ky; ++uu)
                                        for (int vv = 0; vv < kz; ++vv) {
                                            const double sgn = ((tt + uu + vv) & 1) ? -1.0 : 1.0;
                                            inner += sgn * ekx[tt] * eky[uu] * ekz[vv] *
                                                     r0[((t + tt) * ny + (u + uu)) * nz + (v + vv)];
                                        }
                                acc += eb * inner;
                            }
                    res += acc;
                }
        }
    return res;
}

// Canonical function quartets (i>=j, k>=l, ij>=kl).  mode 0: tensor 8-fold scatter,
// mode 1: J/K digestion into Jp/Kp (see eri_kernels.cuh for the accumulator convention).
__global__ void qb_eri_generic_kernel(const GenBasis b, const double* __restrict__ boys, int mode,
                                      double* eri, const double* __restrict__ D, double* Jp, double* Kp,
                                      int* status) {
    const long long np = (long long)b.nfun * (b.nfun + 1) / 2;
    const long long total = np * (np + 1) / 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const size_t N = b.nfun;
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < total; n += stride) {
        int P, Q, i, j, k, l;
        tri_decode(n, P, Q);
        tri_decode(P, i, j);
        tri_decode(Q, k, l);
        const double v = md_eri(b, i, j, k, l, boys, status);
        if (mode == 0) {
            eri[i + N * (j + N * (k + N * l))] = v; eri[j + N * (i + N * (k + N * l))] = v;
            eri[i + N * (j + N * (l + N * k))] = v; eri[j + N * (i + N * (l + N * k))] = v;
            eri[k + N * (l + N * (i + N * j))] = v; eri[l + N * (k + N * (i + N * j))] = v;
            eri[k + N * (l + N * (j + N * i))] = v; eri[l + N * (k + N * (j + N * i))] = v;
        } else {
            const double g = v * (i != j ? 2.0 : 1.0) * (k != l ? 2.0 : 1.0) * (P != Q ? 2.0 : 1.0);
            atomicAdd(Jp + i + N * j, D[k + N * l] * g);
            atomicAdd(Jp + k + N * l, D[i + N * j] * g);
            atomicAdd(Kp + i + N * k, D[j + N * l] * g);
            atomicAdd(Kp + j + N * l, D[i + N * k] * g);
            atomicAdd(Kp + i + N * l, D[j + N * k] * g);
            atomicAdd(Kp + j + N * k, D[i + N * l] * g);
        }
    }
}

// Explicit list of function quartets (ij|kl) -> out[q].
__global__ void qb_eri_list_kernel(const GenBasis b, const double* __restrict__ boys, long long nq,
                                   const int* __restrict__ quartets, double* out, int* status) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int* t = quartets + 4 * q;
    out[q] = md_eri(b, t[0], t[1], t[2], t[3], boys, status);
}

// Adjoint (backward) pass of the two-electron energy: functions [n, n + ng) of the
// basis are extra single primitives g (derivatives of the basis functions' primitives),
// functions [0, n) the basis itself with the total density P (n x n).  For every g, every
// nu and every canonical pair lambda >= sigma the integral (g nu | lambda sigma) is
// recomputed (nothing stored) and digested into
//   Jx[g][nu]     = sum_{lambda sigma} (g nu | lambda sigma) P_{lambda sigma}
//   Kx[g][lambda] = sum_{nu sigma}     (g nu | lambda sigma) P_{nu sigma}.
__global__ void qb_adjoint_eri_kernel(const GenBasis b, int n, int ng, const double* __restrict__ P,
                                      const double* __restrict__ boys, double* Jx, double* Kx, int* status) {
    const long long npair = (long long)n * (n + 1) / 2;
    const long long total = (long long)ng * n * npair;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long pr = t % npair;
        const long long rest = t / npair;
        const int nu = (int)(rest % n), g = (int)(rest / n);
        int lam, sig;
        tri_decode(pr, lam, sig);
        const double I = md_eri(b, n + g, nu, lam, sig, boys, status);
        if (I == 0.0) continue;
        const double w = (lam == sig) ? 1.0 : 2.0;
        atomicAdd(Jx + (size_t)g * n + nu, w * I * P[lam + (size_t)n * sig]);
        atomicAdd(Kx + (size_t)g * n + lam, I * P[nu + (size_t)n * sig]);
        if (lam != sig) atomicAdd(Kx + (size_t)g * n + sig, I * P[nu + (size_t)n * lam]);
    }
}

int qb_gen_adjoint_eri(const GenDevBasis& gb, int n, int ng, const double* P, const double* boys, double* Jx,
                       double* Kx, int* status, int nsm, cudaStream_t s) {
    GenBasis b{gb.fp, gb.cen, gb.ijk, gb.alpha, gb.w, gb.nfun};
    const long long total = (long long)ng * n * ((long long)n * (n + 1) / 2);
    const int block = 64;
    long long grid = (total + block - 1) / block;
    const long long cap = (long long)nsm * 32;
    if (grid > cap) grid = cap;
    if (grid > 0) qb_adjoint_eri_kernel<<<(unsigned)grid, block, 0, s>>>(b, n, ng, P, boys, Jx, Kx, status);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---------------------------------------------------------------------------
int qb_gen_onebody(const GenDevBasis& gb, int flags, int nnuc, const double* dZ, const double* dR,
                   const double* boys, double* S, double* T, double* V, int* status, cudaStream_t s) {
    GenBasis b{gb.fp, gb.cen, gb.ijk, gb.alpha, gb.w, gb.nfun};
    const long long npair = (long long)gb.nfun * (gb.nfun + 1) / 2;
    const int block = 64;
    const long long grid = (npair + block - 1) / block;
    if (grid > 0) qb_onebody_kernel<<<(unsigned)grid, block, 0, s>>>(b, flags, nnuc, dZ, dR, boys, S, T, V, status);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int qb_gen_onebody_batch(const GenDevBasis& gb, int nmol, long long npair_total, const long long* poff,
                         const int* fo, const int* nf, const long long* mo, const int* nuc0, const double* dZ,
                         const double* dR, const double* boys, double* S, double* H, int* status, cudaStream_t s) {
    GenBasis b{gb.fp, gb.cen, gb.ijk, gb.alpha, gb.w, gb.nfun};
    const int block = 64;
    const long long grid = (npair_total + block - 1) / block;
    if (grid > 0)
        qb_onebody_batch_kernel<<<(unsigned)grid, block, 0, s>>>(b, nmol, poff, fo, nf, mo, nuc0, dZ, dR, boys, S, H,
                                                                status);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int qb_gen_multipole(const GenDevBasis& gb, const double* C, const int* deg, double* M, int* status, cudaStream_t s) {
    GenBasis b{gb.fp, gb.cen, gb.ijk, gb.alpha, gb.w, gb.nfun};
    const long long npair = (long long)gb.nfun * (gb.nfun + 1) / 2;
    const int block = 64;
    const long long grid = (npair + block - 1) / block;
    if (grid > 0)
        qb_multipole_kernel<<<(unsigned)grid, block, 0, s>>>(b, C[0], C[1], C[2], deg[0], deg[1], deg[2], M, status);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int qb_gen_eri(const GenDevBasis& gb, int mode, const double* boys, double* eri, const double* D, double* Jp,
               double* Kp, int* status, int nsm, cudaStream_t s) {
    GenBasis b{gb.fp, gb.cen, gb.ijk, gb.alpha, gb.w, gb.nfun};
    const long long np = (long long)gb.nfun * (gb.nfun + 1) / 2;
    const long long total = np * (np + 1) / 2;
    const int block = 64;
    long long grid = (total + block - 1) / block;
    const long long cap = (long long)nsm * 16;
    if (grid > cap) grid = cap;
    if (grid > 0) qb_eri_generic_kernel<<<(unsigned)grid, block, 0, s>>>(b, boys, mode, eri, D, Jp, Kp, status);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int qb_gen_eri_list(const GenDevBasis& gb, const double* boys, long long nq, const int* dq, double* out,
                    int* status, cudaStream_t s) {
    GenBasis b{gb.fp, gb.cen, gb.ijk, gb.alpha, gb.w, gb.nfun};
    const int block = 64;
    const long long grid = (nq + block - 1) / block;
    if (grid > 0) qb_eri_list_kernel<<<(unsigned)grid, block, 0, s>>>(b, boys, nq, dq, out, status);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---------------------------------------------------------------------------
// Boys sequences F_0..F_M(T_i) by the device evaluators: path 0 the compile-time-order
// version of the class kernels (M <= 8), path 1 the runtime-order version of the
// generic kernels (M <= QB_GEN_LTOT_MAX).
template <int M>
__device__ void qb_boys_one(double T, const double* tab, double* out) {
    double F[M + 1];
    qb_boys_scaled<M>(T, 1.0, tab, F);
#pragma unroll
    for (int m = 0; m <= M; ++m) out[m] = F[m];
}

__global__ void qb_boys_kernel(int n, const double* __restrict__ T, int M, int path, const double* __restrict__ tab,
                               double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double* o = out + (size_t)i * (M + 1);
    if (path == 1) {
        double F[QB_GEN_LTOT_MAX + 1];
        qb_boys_scaled_rt(T[i], 1.0, tab, M, F);
        for (int m = 0; m <= M; ++m) o[m] = F[m];
        return;
    }
    switch (M) {
        case 0: qb_boys_one<0>(T[i], tab, o); break;
        case 1: qb_boys_one<1>(T[i], tab, o); break;
        case 2: qb_boys_one<2>(T[i], tab, o); break;
        case 3: qb_boys_one<3>(T[i], tab, o); break;
        case 4: qb_boys_one<4>(T[i], tab, o); break;
        case 5: qb_boys_one<5>(T[i], tab, o); break;
        case 6: qb_boys_one<6>(T[i], tab, o); break;
        case 7: qb_boys_one<7>(T[i], tab, o); break;
        default: qb_boys_one<8>(T[i], tab, o); break;
    }
}

int qb_boys_device(int n, const double* dT, int M, int path, const double* boys, double* dout, cudaStream_t s) {
    if (n > 0) qb_boys_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, dT, M, path, boys, dout);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
